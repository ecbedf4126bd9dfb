"""GB300-native fill-and-composite path with z2d's painter.fill /
SurfaceCompositor API (host-side mirror; compute runs in libz2dgpu.so)."""
from . import abi  # noqa: F401
from .path import Path, nodes_array  # noqa: F401
from .surface import Surface  # noqa: F401
from .types import (Color, FillOptions, Gradient, Operation, Param, Pattern, Pixel,  # noqa: F401
                    wrap_dither)
