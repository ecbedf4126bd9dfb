"""Writes glyphs_inter_regular.json: simple-glyph outlines of the test font
in the z2d source tree (src/internal/test-fonts/Inter-Regular.subset.ttf),
decoded from its 'glyf' table as Glyph.zig's runOutline reads them
(src/internal/Glyph.zig:620-700: end points, flags with repeats, x then y
deltas), with unitsPerEm ('head') and the advances ('hmtx').  The device
path builder's tests replay them; run from the repository root:

    python tests/golden/extract_glyphs.py [z2d source tree]
"""
import json
import os
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def tables(data):
    n = struct.unpack_from(">H", data, 4)[0]
    out = {}
    for i in range(n):
        tag, _, off, length = struct.unpack_from(">4sIII", data, 12 + 16 * i)
        out[tag.decode()] = (off, length)
    return out


def simple_glyph(data, off):
    n_contours = struct.unpack_from(">h", data, off)[0]
    if n_contours <= 0:
        return None  # empty or composite
    p = off + 10
    ends = list(struct.unpack_from(f">{n_contours}H", data, p))
    p += 2 * n_contours
    n_instr = struct.unpack_from(">H", data, p)[0]
    p += 2 + n_instr
    n_pts = ends[-1] + 1
    flags = []
    while len(flags) < n_pts:
        f = data[p]
        p += 1
        flags.append(f)
        if f & 8:
            r = data[p]
            p += 1
            flags.extend([f] * r)
    flags = flags[:n_pts]
    xs, ys, cur = [], [], 0
    for f in flags:
        if f & 2:
            d = data[p]
            p += 1
            cur += d if f & 16 else -d
        elif not f & 16:
            cur += struct.unpack_from(">h", data, p)[0]
            p += 2
        xs.append(cur)
    cur = 0
    for f in flags:
        if f & 4:
            d = data[p]
            p += 1
            cur += d if f & 32 else -d
        elif not f & 32:
            cur += struct.unpack_from(">h", data, p)[0]
            p += 2
        ys.append(cur)
    return {"points": [[x, y, f & 1] for x, y, f in zip(xs, ys, flags)], "ends": ends}


def main():
    tree = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(HERE), "..", "..", "reference")
    path = os.path.join(tree, "src", "internal", "test-fonts", "Inter-Regular.subset.ttf")
    data = open(path, "rb").read()
    t = tables(data)
    upem = struct.unpack_from(">H", data, t["head"][0] + 18)[0]
    loca_long = struct.unpack_from(">h", data, t["head"][0] + 50)[0] == 1
    n_glyphs = struct.unpack_from(">H", data, t["maxp"][0] + 4)[0]
    n_hmetrics = struct.unpack_from(">H", data, t["hhea"][0] + 34)[0]
    loca = [struct.unpack_from(">I" if loca_long else ">H", data, t["loca"][0] + (4 if loca_long else 2) * i)[0]
            * (1 if loca_long else 2) for i in range(n_glyphs + 1)]
    glyphs = []
    # glyph 56 ('a', the outline Glyph.zig's tests check) first, then the
    # font's other simple glyphs in index order
    for gi in [56] + [i for i in range(1, n_glyphs) if i != 56]:
        if len(glyphs) >= 24:
            break
        if loca[gi + 1] == loca[gi]:
            continue
        g = simple_glyph(data, t["glyf"][0] + loca[gi])
        if g is None:
            continue
        adv = struct.unpack_from(">H", data, t["hmtx"][0] + 4 * min(gi, n_hmetrics - 1))[0]
        glyphs.append(dict(index=gi, advance=adv, **g))
    out = {"font": "src/internal/test-fonts/Inter-Regular.subset.ttf", "units_per_em": upem, "glyphs": glyphs}
    with open(os.path.join(HERE, "glyphs_inter_regular.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"{len(glyphs)} glyphs, units_per_em {upem}")


if __name__ == "__main__":
    main()
