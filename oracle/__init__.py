"""CPU oracle for the z2d fill/composite path -- TEST INFRASTRUCTURE ONLY.

A C++ restatement of z2d's CPU code (z2d_oracle.cpp) plus its ctypes
binding.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use it, always as the checker, never as the thing measured or shipped.
"""
from .binding import Oracle, build_oracle, load_oracle  # noqa: F401
