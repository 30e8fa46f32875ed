"""Generate the SVG fixtures under tests/golden/ from vkvg's own parser.

    python tests/golden/make_svg_golden.py

Each fixture (svg_<name>.npz) is what vkvg's SVG walk reads from nanoSVG's
parse of one seeded document (vkvg_gb300.scenes.svg_document): the image
size and, per shape, its id, paint types and colours, visibility, opacity,
stroke width, bounds and every path's cubic points and closed flag.  The
parse is the reference's vendored nanoSVG (src/nsvg/nanosvg.h of vkvg),
compiled here by oracle/build_ref.py, so this script runs only where the
reference tree is present; the fixtures let the library's parser be checked
against it anywhere.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import nsvg_ref  # noqa: E402
from vkvg_gb300 import scenes  # noqa: E402


def documents():
    out = [("seed%d" % s, scenes.svg_document(seed=s, n_shapes=40)) for s in (1, 2, 3, 4)]
    out += [("quirks%d" % s, scenes.svg_document(seed=s, n_shapes=40, quirks=True)) for s in (5, 6)]
    return out


def pack(width, height, shapes):
    """shape records -> arrays"""
    ids = np.zeros((len(shapes), 64), np.uint8)
    u = np.zeros((len(shapes), 6), np.uint32)
    f = np.zeros((len(shapes), 6), np.float32)
    npts, closed, pts = [], [], []
    for i, sh in enumerate(shapes):
        ids[i, :len(sh["id"])] = np.frombuffer(sh["id"], np.uint8)
        u[i] = [sh["fill_type"], sh["fill_color"], sh["stroke_type"], sh["stroke_color"], sh["visible"],
                len(sh["paths"])]
        f[i] = [sh["opacity"], sh["stroke_width"]] + list(sh["bounds"])
        for p, c in sh["paths"]:
            npts.append(len(p))
            closed.append(int(c))
            pts.append(p)
    return {"size": np.float32([width, height]), "ids": ids, "u": u, "f": f,
            "path_npts": np.array(npts, np.uint32), "path_closed": np.array(closed, np.uint8),
            "points": np.concatenate(pts).astype(np.float32) if pts else np.zeros((0, 2), np.float32)}


def unpack(g):
    """a fixture's arrays -> shape records (as vkvg_gb300.Svg.shapes())"""
    out, k = [], 0
    for i in range(len(g["u"])):
        u, f = g["u"][i], g["f"][i]
        paths = []
        for _ in range(int(u[5])):
            n = int(g["path_npts"][k])
            start = int(g["path_npts"][:k].sum())
            paths.append((g["points"][start:start + n], bool(g["path_closed"][k])))
            k += 1
        out.append({"id": bytes(g["ids"][i]).rstrip(b"\0"), "fill_type": int(u[0]), "fill_color": int(u[1]),
                    "stroke_type": int(u[2]), "stroke_color": int(u[3]), "visible": bool(u[4]), "opacity": f[0],
                    "stroke_width": f[1], "bounds": f[2:6].copy(), "paths": paths})
    return out


def main():
    for name, text in documents():
        path = os.path.join(HERE, "svg_%s.npz" % name)
        np.savez_compressed(path, **pack(*nsvg_ref.parse(text)))
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
