"""GPU parity: every stage of the sm_103a pipeline against the CPU oracle on
the same seeded inputs, through the C ABI.

Bar: flattened points, stroke vertices and indices bit-exact (the kernels and
the oracle share the portable math and fp32 op order), per-sample winding /
covering-triangle counts bit-exact, and the final samples and image
bit-exact (integer UNORM8 blending on both sides)."""
import numpy as np
import pytest

import parity_util as pu
from vkvg_gb300 import scenes

pytestmark = pytest.mark.gpu


def small_scenes():
    out = [
        scenes.plain_small(n_polys=12, size=96, seed=0),
        scenes.curve_heavy(n_paths=10, size=128, seed=1, n_min=3, n_max=6),
    ]
    for o in out:
        o["samples"] = 4
    return out


@pytest.mark.parametrize("fn", range(6))
def test_pmath_device_matches_host(gb, fn):
    rng = np.random.default_rng(100 + fn)
    a = rng.uniform(-50, 50, 100000).astype(np.float32)
    b = rng.uniform(-50, 50, 100000).astype(np.float32)
    if fn in (1, 4):
        a = rng.uniform(-1.1, 1.1, 100000).astype(np.float32)
    h = gb.pmath(fn, a, b, device=False)
    d = gb.pmath(fn, a, b, device=True)
    assert np.array_equal(h.view(np.uint32), d.view(np.uint32))


@pytest.mark.parametrize("idx", [0, 1])
def test_geometry_bit_exact(gb, vko, idx):
    sc = small_scenes()[idx]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0  # device status word
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]


@pytest.mark.parametrize("idx", [0, 1])
def test_coverage_bit_exact(gb, vko, idx):
    sc = small_scenes()[idx]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    n = int(ctx.debug_counts()[2])
    for i in range(n):
        g = ctx.debug_coverage(i)
        o = octx.coverage(i, sc["width"], sc["height"], sc["samples"], mode=0)
        assert np.array_equal(g, o), "draw %d: %d samples differ" % (i, int((g != o).sum()))


@pytest.mark.parametrize("idx", [0, 1])
def test_image_bit_exact(gb, vko, idx):
    sc = small_scenes()[idx]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_curve_heavy_full_size_bit_exact(gb, vko):
    """The full 1024x1024, 2,048-path benchmark scene: every stroke/fill draw's
    geometry and the final 4x MSAA samples equal the oracle's."""
    import os

    sc = scenes.curve_heavy()
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc, threads=os.cpu_count() or 1)
    assert ctx.debug_counts()[5] == 0
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())
