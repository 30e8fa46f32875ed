"""Generate the golden fixtures under tests/golden/ from the oracle.

    python tests/golden/make_golden.py

vkvg's tree holds no numeric fixtures or golden images for the path (its
gunit PNGs are missing) and vkvg cannot run here, so these fixtures are the
oracle's outputs on small seeded scenes, committed so that any change of the
oracle or of the GPU library against them is caught.  Per scene (<name>.npz):
the final image (write_to_memory, unpremultiplied RGBA8), each draw's kind,
the flattened points of fill and clip draws, the vertices and indices of
stroke draws, and a SHA-256 digest of every fill, stroke and clip draw's
per-sample winding / covering-triangle counts (int32 [height][width][samples],
little endian).  Draws are the fills, strokes, paints, clears and clip paths;
the stencil operations of reset_clip / save / restore (kinds 7 and up) are
left out, as the library splits them differently.  The oracle runs with its
portable math (the kernels' math).

    python tests/golden/make_golden.py [scene name ...]   # default: all
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle_bind as ob  # noqa: E402
import parity_util as pu  # noqa: E402
from vkvg_gb300 import scenes  # noqa: E402


def golden_scenes():
    return [scenes.plain_small(n_polys=12, size=96, seed=0),
            scenes.curve_heavy(n_paths=10, size=128, seed=1, n_min=3, n_max=6),
            scenes.api_mix(n_items=24, size=160, seed=5),
            scenes.gradient_mix(n_items=14, size=144, seed=9),
            scenes.clip_mix(n_items=10, size=128, seed=13),
            scenes.gradient_mix(n_items=14, size=144, seed=9, radial=True),
            scenes.surface_mix(n_items=12, size=128, seed=23)]

STENCIL_OPS = 7
FILL_KINDS = (0, 1, 5, 6)


def _cat(parts, dtype, width):
    if not parts:
        return np.zeros((0,) + ((width,) if width else ()), dtype), np.zeros(1, np.uint32)
    off = np.zeros(len(parts) + 1, np.uint32)
    off[1:] = np.cumsum([len(p) for p in parts])
    return np.concatenate([np.asarray(p, dtype) for p in parts]), off


def digest(cov):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(cov, "<i4").tobytes()).digest(), np.uint8)


def capture(sc):
    L = ob.lib()
    L.vko_set_math_mode(0)
    surf, ctx = pu.run_oracle(ob, sc)
    W, H, S = sc["width"], sc["height"], sc["samples"]
    every = ctx.draws()
    idx = [i for i, d in enumerate(every) if d["kind"] < STENCIL_OPS]
    draws = [every[i] for i in idx]
    kinds = np.array([d["kind"] for d in draws], np.uint32)
    fpts = [d["points"] for d in draws if d["kind"] in FILL_KINDS]
    sv = [d["verts"] for d in draws if d["kind"] == 2]
    si = [d["inds"] for d in draws if d["kind"] == 2]
    cov = np.zeros((len(draws), 32), np.uint8)
    for j, (i, d) in enumerate(zip(idx, draws)):
        if d["kind"] in FILL_KINDS + (2,):
            cov[j] = digest(ctx.coverage(i, W, H, S))
    out = {"image": surf.image(), "kinds": kinds, "cov_sha256": cov}
    out["fill_pts"], out["fill_pts_off"] = _cat(fpts, np.float32, 2)
    out["stroke_verts"], out["stroke_verts_off"] = _cat(sv, np.float32, 2)
    out["stroke_inds"], out["stroke_inds_off"] = _cat(si, np.uint32, 0)
    ctx.destroy()
    surf.destroy()
    return out


def main():
    only = set(sys.argv[1:])
    for sc in golden_scenes():
        if only and sc["name"] not in only:
            continue
        path = os.path.join(HERE, sc["name"] + ".npz")
        np.savez_compressed(path, **capture(sc))
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
