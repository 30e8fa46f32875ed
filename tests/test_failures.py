"""Failure detection and reporting, in forms that fault no GPU.

vkvg reports its own failures through status codes: creation failures return
static status sentinels instead of objects (src/vkvg_internal.h:104-109,
src/vkvg_context.c:74-82), calls on an object in error are no-ops
(src/vkvg_context.c:332-334), and a GPU that does not finish in time gives
VKVG_STATUS_TIMEOUT (src/vkvg_context_internal.c:407-419).  Here:

* an allocation failure is injected on the host (the next device buffer
  growth fails as cudaMalloc would): creation returns the NO_MEMORY sentinel,
  a flush sets the context's status to NO_MEMORY and later calls are no-ops;
* the row-form raster's staging waits are given a limit of a few polls, so
  they run out as a lost copy would: the kernel stops its tiles, waits (with
  the normal limit) for the copies it issued, sets a status bit, and the host
  reports VKVG_STATUS_DEVICE_ERROR;
* the subdivision work cap per cubic is lowered below what a long curve
  needs: the curve is cut short and the flush reports DEVICE_ERROR.

After each, with the setting restored, the same process renders a scene equal
to the oracle's, so the CUDA context stayed usable."""
import numpy as np
import pytest

import parity_util as pu
from vkvg_gb300 import scenes

pytestmark = pytest.mark.gpu

NO_MEMORY, INVALID_SURFACE, DEVICE_ERROR = 1, 19, 16


@pytest.fixture
def inject(gb):
    L = gb.lib()
    yield lambda what, v: L.vkvg_gb300_debug_inject(what, v)
    for what in (0, 1, 2):
        L.vkvg_gb300_debug_inject(what, 0)
    L.vkvg_gb300_debug_set_raster_form(-1)


def _still_renders(gb, vko):
    sc = scenes.curve_heavy(n_paths=6, size=96, seed=11, n_min=3, n_max=5)
    dev, surf, ctx = pu.run_gpu(gb, sc, debug=False)
    assert ctx.status() == 0
    osurf, _ = pu.run_oracle(vko, sc)
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())


def _record(ctx):
    scenes.play(ctx, scenes.curve_heavy(n_paths=4, size=64, seed=2, n_min=3, n_max=5)["ops"])


def test_allocation_failure_at_creation(gb, vko, inject):
    L = gb.lib()
    dev = gb.Device(samples=4)
    inject(0, 1)
    s = L.vkvg_surface_create(dev.h, 64, 64)
    assert s and L.vkvg_surface_status(s) == NO_MEMORY  # the sentinel, never null
    L.vkvg_surface_destroy(s)  # a no-op on the sentinel
    assert L.vkvg_surface_status(s) == NO_MEMORY
    c = L.vkvg_create(s)
    assert c and L.vkvg_status(c) == INVALID_SURFACE
    surf = gb.Surface(dev, 64, 64)
    inject(0, 1)
    c = L.vkvg_create(surf.h)
    assert c and L.vkvg_status(c) == NO_MEMORY
    L.vkvg_move_to(c, 1.0, 2.0)  # calls on the sentinel do nothing
    assert L.vkvg_status(c) == NO_MEMORY
    _still_renders(gb, vko)


def test_allocation_failure_at_flush(gb, vko, inject):
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, 64, 64)
    ctx = surf.context()
    ctx.set_line_width(5.0)
    _record(ctx)
    inject(0, 1)
    ctx.flush()
    assert ctx.status() == NO_MEMORY
    # the context is in error: calls are no-ops, getters return defaults
    ctx.set_line_width(9.0)
    assert ctx.status() == NO_MEMORY
    assert ctx.get_line_width() == 0.0
    _still_renders(gb, vko)


@pytest.mark.parametrize("form,limit", [(3, 1), (4, 1), (4, 4)])
def test_raster_wait_limit_reports_device_error(gb, vko, inject, form, limit):
    gb.lib().vkvg_gb300_debug_set_raster_form(form)
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, 300, 200)
    ctx = surf.context()
    scenes.play(ctx, scenes.curve_heavy(n_paths=40, size=300, seed=5, n_min=4, n_max=12)["ops"])
    inject(1, limit)
    ctx.flush()
    assert ctx.status() == DEVICE_ERROR
    inject(1, 0)
    _still_renders(gb, vko)


def test_curve_work_cap_reports_device_error(gb, vko, inject):
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, 512, 512)
    ctx = surf.context()
    ctx.move_to(5.0, 5.0)
    ctx.curve_to(900.0, -300.0, -400.0, 900.0, 500.0, 500.0)  # hundreds of subdivision nodes
    ctx.close_path()
    ctx.fill()
    inject(2, 16)
    ctx.flush()
    assert ctx.status() == DEVICE_ERROR
    inject(2, 0)
    _still_renders(gb, vko)
