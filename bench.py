#!/usr/bin/env python
"""Benchmark of the vkvg path hot path on GB300.

Workload (one step = one frame): the curve-heavy scene - a 1024x1024 RGBA8
surface at 4x MSAA painted white, then 2,048 closed paths of U{4..64} cubic
Beziers with control points uniform in [0,1024)^2 (seed 1), each filled
(even-odd / non-zero alternating, alpha U[0.3,1)) and stroked (width U[1,8),
joins and caps cycled, every 4th path dashed [10,5]).  Synthetic seeded data
(vkvg_gb300/scenes.py); no public dataset exists for this path.

value  - paths/s with the recorded command buffers resident in HBM
         (vkvg_gb300_frame_execute: flatten -> stroke -> setup/binning ->
         raster/composite), device time from CUDA events on the library's
         stream, L2 flushed (a 256 MiB buffer is zeroed) before every step.
e2e    - paths/s through the public C API from host memory: each step replays
         the scene's vkvg_* calls (vkvg_gb300_replay_stream), flushes (H2D copy
         + kernels) and reads the image back (vkvg_surface_write_to_memory);
         wall-clock time.
roofline - the raster/composite kernel (dominant; the row form in half
         bands) against the measured HBM copy bandwidth; algorithmic bytes =
         8 B per flattened point and per stroke vertex read once, plus the
         RGBA8 surface read and written.  frame_frac applies the whole-frame
         count (8 B per input control point, 4 B per command word, 16 B per
         flattened point and per stroke vertex - written once, read once - and
         8 B per pixel) to the whole frame time.  The raster kernel is
         instruction-issue bound, not HBM bound: roofline.issue sets its warp
         instructions per launch (ncu, full-size launch, from the committed
         summary profiles/raster_rows_curve_heavy_1024.md) over its CUDA-event
         time against the SM issue peak (SMs x 4 schedulers x the SM clock
         sampled during the run).
cpu_baseline - the CPU restatement of vkvg's path code (oracle/): the
         headline figure on a bounded sample of the same scene (the first 256
         paths on the full surface, all host threads, median of 3), plus
         one-core and all-core medians on bounded samples of the other
         configurations (cpu_baseline.configs).

svg    - SVG ingestion through vkvg's SVG API (include/vkvg-svg.h): a seeded
         600-shape document parsed once, then rendered, flushed and read back
         per step (host timer); reported beside the headline.
analytic.glyphs - the 4096x4096 glyph construction in the differentiable
         analytic mode (tiled), forward and forward + backward (CUDA events).

`--impl reference` times that CPU implementation alone (vkvg itself cannot be
built or run here: no Vulkan stack and its vkh / glutess submodules are empty).
Multi-GPU: replicas only (one independent frame per GPU).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--paths", type=int, default=2048)
    p.add_argument("--size", type=int, default=1024)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-batch", action="store_true", help="skip the uneven-batch comparison")
    p.add_argument("--no-analytic", action="store_true", help="skip the differentiable analytic-coverage workload")
    p.add_argument("--no-glyphs", action="store_true", help="skip the 4096x4096 glyph workload")
    p.add_argument("--svg-shapes", type=int, default=600, help="shapes of the SVG ingestion workload (0: skip)")
    p.add_argument("--glyph-size", type=int, default=4096,
                   help="side of the glyph workload; smaller sides keep its density (profiling crops)")
    p.add_argument("--analytic-glyphs-only", action="store_true",
                   help="run only the glyph scene's analytic forward + backward and print its entry (profiling)")
    p.add_argument("--adam-steps", type=int, default=200, help="Adam steps of the differentiable workload")
    return p.parse_args()


def sm_max_mhz():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["sm_max_mhz"])
    except Exception:
        return 2070.0


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def reduce_max(x, dist, device):
    """max of a per-rank float over all ranks (x itself without a process group)"""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """units of all replicas per second of the slowest replica"""
    return units_per_rank * world / seconds


def cpu_sample(n_paths, size, threads, reps=1):
    """Time the CPU restatement on the first n_paths paths of the scene."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    from vkvg_gb300 import scenes

    sc = scenes.curve_heavy(n_paths=n_paths, size=size, seed=1)
    L = ob.lib()
    L.vko_set_math_mode(0)
    L.vko_set_raster_mode(0)
    L.vko_set_threads(threads)
    times = []
    for _ in range(reps):
        surf = ob.OracleSurface(size, size, 4)
        ctx = surf.context()
        t0 = time.perf_counter()
        scenes.play(ctx, sc["ops"])
        ctx.flush()
        times.append(time.perf_counter() - t0)
        ctx.destroy()
        surf.destroy()
    return n_paths / min(times), min(times)


def analytic_glyph_bench(a, gb, torch, np, flush, tile=128, cpu=False):
    """The large glyph configuration in the differentiable analytic mode
    (4096x4096 fp32 canvas, 200,000 quadratic outlines elevated to cubics,
    20,000 closed strokes, seed 5; the target is the same construction from
    seed 6): the tiled evaluation (tiles of `tile` pixels, every tile's area
    planes resident), forward and forward + backward timed with CUDA events
    (median of 3 after 2 warm-ups, L2 flushed), the device memory the scene
    holds, and the gradient of the outline control points (on-curve and
    off-curve points, through the elevation's transpose)."""
    from vkvg_gb300 import scenes

    t0 = time.perf_counter()
    scene, par, quad = scenes.analytic_glyph_scene(seed=5)
    tscene, tpar, _ = scenes.analytic_glyph_scene(seed=6)
    gen_s = time.perf_counter() - t0
    # the target: the seed-6 draw of the construction, rendered by its own scene
    T = gb.Analytic(tscene, tile=tile)
    td = {k: torch.tensor(v, device="cuda") for k, v in tpar.items()}
    canvas, _ = T.forward(td["ctrl"], td["colors"], td["widths"])
    target = canvas.clone()
    assert T.sync() == 0
    T.destroy()
    del td, canvas, T
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    A = gb.Analytic(scene, tile=tile)
    d = {k: torch.tensor(v, device="cuda") for k, v in par.items()}
    A.forward(d["ctrl"], d["colors"], d["widths"], target)
    grads = A.backward()
    assert A.sync() == 0
    free1, _ = torch.cuda.mem_get_info()
    st = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(2):
            flush()
            fn()
        ts = []
        for _ in range(3):
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    fwd_ms = timed(lambda: A.forward(d["ctrl"], d["colors"], d["widths"], target))

    def fb():
        A.forward(d["ctrl"], d["colors"], d["widths"], target)
        A.backward(grads=grads)

    fb_ms = timed(fb)
    A.set_timing(True)
    fb()
    phases = [float(x) for x in A.timing()]
    A.set_timing(False)
    assert A.sync() == 0
    loss = float(A.loss.item())
    gP, gQ = scenes.elevate_adjoint(quad, grads[0].cpu().numpy())
    out = {"workload": "analytic fp32 4096x4096 (seed 5; target seed 6): 200000 quadratic outlines with holes "
                       "(fill), 20000 closed strokes, %d cubic segments after elevation, tiles of %d px" %
                       (len(scene["seg_kind"]), tile),
           "fwd_ms": fwd_ms, "fwd_bwd_ms": fb_ms, "fwd_bwd_over_fwd": fb_ms / fwd_ms, "loss": loss,
           "phase_ms": {"flatten_and_tiles": phases[0], "cover": phases[1], "composite": phases[2],
                        "composite_adjoint": phases[3], "cover_adjoint": phases[4], "flatten_adjoint": phases[5]},
           "layers": int(A.nlayers), "device_bytes": int(free0 - free1), "scene_build_s": gen_s,
           "outline_grad_norm": {"on_curve": float(np.linalg.norm(gP)), "off_curve": float(np.linalg.norm(gQ))},
           "timing": "CUDA events on the scene's stream, L2 flushed before each, median of 3",
           "checked": "tests/test_analytic.py: tiled == whole canvas; the construction on a 192x192 crop against the "
                      "FP64 reference; outline gradients on a 128x128 crop against FP64 central differences"}
    A.destroy()
    if cpu:
        out["grad_error_crop"] = glyph_crop_fd(gb, torch, np, scenes)
    return out


def glyph_crop_fd(gb, torch, np, scenes, n=24):
    """The glyph construction on a 128x128 crop (200 outlines, 20 strokes,
    tiles of 64): the GPU gradients of n random outline coordinates
    (on-curve and off-curve points, through the quadratic elevation)
    against FP64 central differences of the CPU reference at h = 1e-3 px
    (coordinates whose differences at h and 10 h disagree, a flattening that
    changes within h, are replaced by the next draw)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import analytic_ref as ar

    scene, par, quad = scenes.analytic_glyph_scene(n_outlines=200, n_strokes=20, size=128)
    tscene, tpar, _ = scenes.analytic_glyph_scene(seed=6, n_outlines=200, n_strokes=20, size=128)
    target, _ = ar.Reference(tscene).forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    R = ar.Reference(scene)
    A = gb.Analytic(scene, tile=64)
    d = {k: torch.tensor(v, device="cuda") for k, v in par.items()}
    A.forward(d["ctrl"], d["colors"], d["widths"], torch.tensor(target.astype(np.float32), device="cuda"))
    gc = A.backward()[0].cpu().numpy().astype(np.float64)
    assert A.sync() == 0
    A.destroy()
    gP, gQ = scenes.elevate_adjoint(quad, gc)

    def fd(which, k, axis, h):
        out = []
        for sgn in (1.0, -1.0):
            P, Q = quad["P"].astype(np.float64), quad["Q"].astype(np.float64)
            (P if which == 0 else Q)[k, axis] += sgn * h
            out.append(R.forward(scenes.elevate(quad, P, Q), par["colors"], par["widths"], target)[1])
        return (out[0] - out[1]) / (2 * h)

    rng = np.random.default_rng(7)
    rows, skipped = [], 0
    while len(rows) < n:
        which, k, axis = int(rng.integers(2)), int(rng.integers(len(quad["P"]))), int(rng.integers(2))
        f1, f2 = fd(which, k, axis, 1e-3), fd(which, k, axis, 1e-2)
        if abs(f1 - f2) > 2e-3 * max(abs(f1), 1e-9):
            skipped += 1
            continue
        rows.append(((gP if which == 0 else gQ)[k, axis], f1))
    an, ref = np.array(rows).T
    err = np.abs(an - ref) / np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return {"max_rel": float(err.max()), "median_rel": float(np.median(err)), "coordinates": n,
            "not_smooth_replaced": skipped, "h_px": 1e-3,
            "rel": "|g - fd| / max(|fd|, 1e-3 max|fd|)", "crop": "128x128, 200 outlines, 20 strokes, tiles of 64"}


def cpu_scene_time(sc, threads, reps=3):
    """median wall time of the CPU restatement rendering one scene (its
    sources included) with the given raster worker threads"""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    import parity_util as pu

    L = ob.lib()
    L.vko_set_math_mode(0)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        surf, ctx = pu.run_oracle(ob, sc, raster_mode=0, threads=threads)
        times.append(time.perf_counter() - t0)
        ctx.destroy()
        surf.destroy()
    return statistics.median(times)


def cpu_configs(threads):
    """one-core and all-core medians (3 repetitions) of the CPU restatement on
    bounded samples of every single-GPU configuration"""
    from vkvg_gb300 import scenes

    cases = []
    cases.append(("small_polygons", scenes.plain_small(), "the whole configuration: 512x512, 64 polygons"))
    cases.append(("curve_heavy", scenes.curve_heavy(n_paths=32), "first 32 of 2048 paths, full 1024x1024 surface"))
    bs = scenes.batch_streams(seed=2, n_surfaces=2, max_paths=240, min_paths=60, max_segs=400, max_side=512)
    for b in bs:
        b["samples"] = 4
        b["ops"] = scenes.decode(b["cmds"], b["args"])
    cases.append(("batch_uneven", bs, "2 generated surfaces of the batch's construction, sides <= 512"))
    g = scenes.glyph_scene(n_outlines=3125, n_strokes=312, size=512)
    cases.append(("glyphs", g, "512x512 crop of the glyph construction at the same density (3,125 outlines, "
                               "312 strokes)"))
    out = {}
    for name, sc, sample in cases:
        scs = sc if isinstance(sc, list) else [sc]
        paths = sum(x["paths"] for x in scs)
        e = {"sample": sample, "paths": paths}
        for label, th in (("one_core", 1), ("all_cores", threads)):
            t = sum(cpu_scene_time(x, th) for x in scs)
            e[label + "_paths_per_s"] = paths / t
        out[name] = e
    return out


def analytic_bench(a, gb, torch, np, flush, cpu):
    """The differentiable analytic-coverage workload: a 256x256 fp32 canvas on
    white, 128 closed paths of 8 cubics (seed 3), NON_ZERO fill + stroke in a
    premultiplied colour, MSE against the same render of an independent
    seed-4 path set.  Times the forward, forward + backward, and Adam steps
    (lr 0.5 px for control points), all through the C ABI on device memory;
    e2e adds the host copies of parameters and gradients.  With cpu, also
    times the FP64 CPU reference's forward + backward and checks the GPU
    gradient against it and against FP64 central differences."""
    import ctypes as C

    from vkvg_gb300 import scenes

    scene, par = scenes.analytic_scene(seed=3)
    _, tpar = scenes.analytic_scene(seed=4)
    A = gb.Analytic(scene)
    dev = {k: torch.tensor(v, device="cuda") for k, v in par.items()}
    tdev = {k: torch.tensor(v, device="cuda") for k, v in tpar.items()}
    canvas, _ = A.forward(tdev["ctrl"], tdev["colors"], tdev["widths"])
    target = canvas.clone()
    st = torch.cuda.current_stream()
    A.forward(dev["ctrl"], dev["colors"], dev["widths"], target)
    grads = A.backward()

    def fwd():
        A.forward(dev["ctrl"], dev["colors"], dev["widths"], target)

    def fwd_bwd():
        fwd()
        A.backward(grads=grads)

    def timed(fn, n):
        for _ in range(max(3, a.warmup)):
            fn()
        ts = []
        for _ in range(n):
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    n = max(10, a.steps)
    t_f = timed(fwd, n)
    t_fb = timed(fwd_bwd, n)
    A.set_timing(True)
    fwd_bwd()
    phases = [float(x) for x in A.timing()]
    A.set_timing(False)
    assert A.sync() == 0
    # Adam on all parameters: lr 0.5 px (control points), 0.01 (colours,
    # clamped to [0,1]), 0.05 px (widths, clamped to [0.1,16])
    p = {k: v.clone() for k, v in dev.items()}
    m = {k: torch.zeros_like(v) for k, v in p.items()}
    v_ = {k: torch.zeros_like(v) for k, v in p.items()}
    lr = {"ctrl": (0.5, -1e4, 1e4), "colors": (0.01, 0.0, 1.0), "widths": (0.05, 0.1, 16.0)}
    losses = torch.zeros(a.adam_steps, device="cuda")
    torch.cuda.synchronize()
    l0 = gb.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for i in range(1, a.adam_steps + 1):
        A.forward(p["ctrl"], p["colors"], p["widths"], target)
        losses[i - 1].copy_(A.loss[0])
        g = A.backward(grads=grads)
        for k, gk in zip(("ctrl", "colors", "widths"), g):
            A.adam(p[k], gk, m[k], v_[k], i, *lr[k])
    e1.record(st)
    e1.synchronize()
    adam_ms = e0.elapsed_time(e1) / a.adam_steps
    launches = (gb.kernel_launches() - l0) / a.adam_steps
    assert A.sync() == 0
    ls = losses.cpu().numpy()
    # end to end: host parameters in, host gradients out, every step
    hp = {k: torch.tensor(v).pin_memory() for k, v in par.items()}
    hg = [torch.empty(t.shape, dtype=torch.float32).pin_memory() for t in grads]
    hl = torch.empty(1, dtype=torch.float32).pin_memory()

    def e2e_step():
        for k in dev:
            dev[k].copy_(hp[k], non_blocking=True)
        A.forward(dev["ctrl"], dev["colors"], dev["widths"], target)
        hl.copy_(A.loss, non_blocking=True)
        gg = A.backward(grads=grads)
        for h, d in zip(hg, gg):
            h.copy_(d, non_blocking=True)
        st.synchronize()

    for _ in range(3):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(n):
        e2e_step()
    e2e_ms = (time.perf_counter() - t0) / n * 1e3
    h2d = sum(t.numel() * 4 for t in hp.values())
    d2h = sum(t.numel() * 4 for t in hg) + 4
    pts, _ = A.points()
    npx, nl = 256 * 256, A.nlayers
    nchunk = (nl + 15) // 16
    # algorithmic bytes of the compositing adjoint: areas read and their
    # gradients written (4 B per layer-pixel each), chunk checkpoints read
    # (16 B per chunk-pixel), canvas and target read (32 B per pixel)
    cb_bytes = npx * (8 * nl + 16 * nchunk + 32)
    out = {"workload": "analytic fp32 256x256, 128 closed paths x 8 cubics (seed 3), NON_ZERO fill + stroke w U[0.5,4), "
                       "MSE vs the seed-4 render", "layers": nl, "flattened_points": int(len(pts)),
           "fwd_ms": t_f, "fwd_bwd_ms": t_fb, "fwd_bwd_over_fwd": t_fb / t_f,
           "phase_ms": {"flatten": phases[0], "cover": phases[1], "composite": phases[2],
                        "composite_adjoint": phases[3], "cover_adjoint": phases[4], "flatten_adjoint": phases[5]},
           "adam_steps": a.adam_steps, "adam_ms_per_step": adam_ms, "loss_first": float(ls[0]),
           "loss_last": float(ls[-1]), "gpu_launches_per_step": launches,
           "e2e": {"ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "roofline": {"kernel": "ak_composite_bwd", "bound": "hbm", "algorithmic_bytes": cb_bytes,
                        "achieved": cb_bytes / (phases[3] / 1e3) / 1e9, "unit": "GB/s"},
           "timing": "CUDA events on the scene's stream, L2 flushed (256 MiB write) before each fwd / fwd+bwd "
                     "iteration; the Adam loop runs unflushed, as a training loop does"}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import analytic_ref as ar

        R = ar.Reference(scene)
        tgt = target.cpu().numpy().astype(np.float64)
        t0 = time.perf_counter()
        _, rc, rcol, rw = R.backward(par["ctrl"], par["colors"], par["widths"], tgt)
        cpu_s = time.perf_counter() - t0
        A.forward(dev["ctrl"], dev["colors"], dev["widths"], target)
        gg = [x.cpu().numpy().astype(np.float64) for x in A.backward()]
        assert A.sync() == 0
        rel = {k: float(np.linalg.norm(a_ - b_) / np.linalg.norm(b_))
               for k, a_, b_ in zip(("ctrl", "colors", "widths"), gg, (rc, rcol, rw))}
        rng = np.random.default_rng(3)
        grp = np.concatenate([np.zeros(160), np.ones(80), 2 * np.ones(80)]).astype(np.uint32)
        idx = np.concatenate([rng.choice(2 * R.nctrl, 160, replace=False), rng.choice(4 * R.npaths, 80, replace=False),
                              rng.choice(R.npaths, 80, replace=False)]).astype(np.uint32)
        fd, fd2, ok = R.fd(par["ctrl"], par["colors"], par["widths"], tgt, grp, idx, h=1e-3, h2=1e-4)
        floor = 1e-3 * np.abs(fd).max()
        ok &= np.abs(fd2 - fd) / np.maximum(np.abs(fd), floor) < 2e-4
        keep = np.zeros(len(grp), bool)
        for gq, want in ((0, 128), (1, 64), (2, 64)):
            keep[np.nonzero((grp == gq) & ok)[0][:want]] = True
        an = np.array([gg[0].reshape(-1)[i] if k == 0 else gg[1].reshape(-1)[i] if k == 1 else gg[2][i]
                       for k, i in zip(grp, idx)])
        err = np.abs(an[keep] - fd[keep]) / np.maximum(np.abs(fd[keep]), floor)
        out["cpu_baseline"] = {"fwd_bwd_ms": cpu_s * 1e3, "cores": 1, "kind": "port",
                               "sample": "one forward + backward of the same scene, FP64 CPU reference"}
        out["grad_error"] = {"vs_fp64_reference_rel_l2": rel, "vs_fp64_fd_h1e-3_max_rel": float(err.max()),
                             "vs_fp64_fd_median_rel": float(np.median(err)), "fd_params": int(keep.sum()),
                             "fd_not_smooth_replaced": int((~ok[:np.nonzero(keep)[0].max() + 1]).sum()),
                             "rel": "|g - fd| / max(|fd|, 1e-3 max|fd|)"}
        R.close()
    A.destroy()
    return out


def small_polygon_bench(a, gb, L, np, flush):
    """The small polygon configuration as stated (512x512, MSAA 4, seed 0):
    64 closed self-intersecting polygons of 3-32 vertices, each filled
    NON_ZERO in an opaque colour then stroked black, width 4, miter (10),
    butt.  Device-resident frames (median of 20, L2 flushed before each) and
    end to end through the API (replay + flush + write_to_memory)."""
    import ctypes as C

    from vkvg_gb300 import scenes

    sc = scenes.plain_small()
    cm, ar = scenes.encode(sc["ops"])
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, sc["width"], sc["height"])
    ctx = surf.context()
    assert L.vkvg_gb300_replay_stream(ctx.h, cm.ctypes.data_as(C.c_void_p), len(cm), ar.ctypes.data_as(C.c_void_p),
                                      len(ar)) == 0
    frame = L.vkvg_gb300_frame_capture(ctx.h)
    timing = np.zeros(8, np.float32)
    for _ in range(3):
        flush()
        assert L.vkvg_gb300_frame_execute(frame, surf.h) == 0
    ms, stages = [], []
    for _ in range(20):
        flush()
        assert L.vkvg_gb300_frame_execute(frame, surf.h) == 0
        L.vkvg_gb300_frame_timing(frame, timing.ctypes.data_as(C.c_void_p))
        ms.append(float(timing[4]))
        stages.append(timing[:4].copy())
    med = statistics.median(ms)
    img = np.zeros((sc["height"], sc["width"], 4), np.uint8)
    ectx = surf.context()
    e = []
    for _ in range(10):
        t0 = time.perf_counter()
        L.vkvg_gb300_replay_stream(ectx.h, cm.ctypes.data_as(C.c_void_p), len(cm), ar.ctypes.data_as(C.c_void_p),
                                   len(ar))
        ectx.flush()
        L.vkvg_surface_write_to_memory(surf.h, img.ctypes.data_as(C.c_void_p))
        e.append(time.perf_counter() - t0)
    e_ms = statistics.median(e) * 1e3
    st = np.median(np.array(stages), axis=0)
    out = {"workload": "small polygons 512x512 msaa4 (seed 0): 64 self-intersecting polygons, NON_ZERO fill + "
                       "black width-4 miter stroke", "paths_per_s": 64 / (med / 1e3), "ms_per_frame": med,
           "mpx_per_s": 512 * 512 / (med / 1e3) / 1e6,
           "stage_ms": {"flatten": float(st[0]), "stroke": float(st[1]), "setup_bin": float(st[2]),
                        "raster": float(st[3])},
           "e2e": {"ms_per_step": e_ms, "paths_per_s": 64 / (e_ms / 1e3),
                   "note": "replay of the recorded calls + vkvg_flush + write_to_memory, host timer, median of 10"},
           "timing": "CUDA events on the library's stream, L2 flushed before each frame, median of 20"}
    L.vkvg_gb300_frame_destroy(frame)
    ectx.destroy()
    ctx.destroy()
    surf.destroy()
    dev.destroy()
    return out


def glyph_bench(a, gb, L, np, flush):
    """The large glyph scene (4096x4096, MSAA 4, seed 5): 200,000 quadratic
    glyph outlines with holes (NON_ZERO) and 20,000 round-join strokes under
    one linear gradient, recorded through vkvg's API (command-stream replay),
    then timed as device-resident frames and end to end."""
    import ctypes as C

    from vkvg_gb300 import scenes

    t0 = time.perf_counter()
    side = a.glyph_size  # a crop keeps the scene's density
    dens = (side / 4096.0) ** 2
    g = scenes.glyph_streams(seed=5, size=side, n_outlines=int(200000 * dens), n_strokes=int(20000 * dens))
    gen_s = time.perf_counter() - t0
    cm, ar = g["cmds"], g["args"]
    size = g["width"]
    x0, y0, x1, y1, stops = g["gradient"]
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, size, size)
    ctx = surf.context()

    def record(c):
        c.set_source_rgb(1.0, 1.0, 1.0)
        c.paint()
        c.set_source_linear(float(x0), float(y0), float(x1), float(y1), [tuple(float(v) for v in st) for st in stops])
        st = L.vkvg_gb300_replay_stream(c.h, cm.ctypes.data_as(C.c_void_p), len(cm), ar.ctypes.data_as(C.c_void_p),
                                        len(ar))
        assert st == 0, st

    record(ctx)
    frame = L.vkvg_gb300_frame_capture(ctx.h)
    assert frame
    timing = np.zeros(8, np.float32)
    for _ in range(2):
        flush()
        assert L.vkvg_gb300_frame_execute(frame, surf.h) == 0
    n = 3
    tot = np.zeros(5)
    for _ in range(n):
        flush()
        assert L.vkvg_gb300_frame_execute(frame, surf.h) == 0
        L.vkvg_gb300_frame_timing(frame, timing.ctypes.data_as(C.c_void_p))
        tot += timing[:5]
    ms = tot[4] / n
    stats = np.zeros(16, np.uint64)
    L.vkvg_gb300_frame_stats(frame, stats.ctypes.data_as(C.c_void_p))
    img = np.zeros((size, size, 4), np.uint8)
    ectx = surf.context()

    def e2e():
        record(ectx)
        L.vkvg_flush(ectx.h)
        assert L.vkvg_surface_write_to_memory(surf.h, img.ctypes.data_as(C.c_void_p)) == 0

    e2e()
    t0 = time.perf_counter()
    for _ in range(2):
        e2e()
    e_ms = (time.perf_counter() - t0) / 2 * 1e3
    paths = g["outlines"] + g["strokes"]
    out = {"workload": "glyphs %dx%d msaa4 (seed 5): %d quadratic outlines with holes (NON_ZERO), %d round-join "
                       "strokes, %d quads, one linear gradient" % (size, size, g["outlines"], g["strokes"], g["quads"]),
           "paths_per_s": paths / (ms / 1e3), "ms_per_frame": ms, "mpx_per_s": size * size / (ms / 1e3) / 1e6,
           "stage_ms": {"flatten": tot[0] / n, "stroke": tot[1] / n, "setup_bin": tot[2] / n, "raster": tot[3] / n},
           "flattened_points": int(stats[1]), "stroke_vertices": int(stats[2]), "bin_units": int(stats[5]),
           "e2e": {"ms_per_step": e_ms, "paths_per_s": paths / (e_ms / 1e3),
                   "note": "replay of the recorded calls + vkvg_flush + write_to_memory, host timer"},
           "scene_build_s": gen_s, "timing": "CUDA events on the library's stream, L2 flushed before each frame"}
    # the same frame as a batch of one surface: sizing, tuning, then timed
    # replays of its CUDA graph
    tgt = gb.Surface(dev, size, size)
    bt = L.vkvg_gb300_batch_create((C.c_void_p * 1)(frame), (C.c_void_p * 1)(tgt.h), 1)
    if bt:
        for _ in range(16):  # sizing, fourteen tuning runs, graph capture
            flush()
            assert L.vkvg_gb300_batch_execute(bt) == 0
        bms = []
        bi = np.zeros(9, np.float32)
        for _ in range(3):
            flush()
            assert L.vkvg_gb300_batch_execute(bt) == 0
            L.vkvg_gb300_batch_timing(bt, bi.ctypes.data_as(C.c_void_p))
            bms.append(float(bi[0]))
        out["batch"] = {"ms_per_frame": statistics.median(bms), "graph_replay": bool(bi[1]),
                        "tile_px": int(bi[8]), "equal_to_frame": bool(np.array_equal(tgt.samples_rgba(),
                                                                                       surf.samples_rgba())),
                        "timing": "CUDA events around the graph launch, L2 flushed before each, median of 3"}
        L.vkvg_gb300_batch_destroy(bt)
    tgt.destroy()
    L.vkvg_gb300_frame_destroy(frame)
    ectx.destroy()
    ctx.destroy()
    surf.destroy()
    dev.destroy()
    return out


def run_reference(a, rank):
    """CPU implementation of the path (the oracle port), all host threads.
    Each step renders the whole frame (all paths of the scene on the full
    surface) when the run's steps fit in about five minutes at the speed a
    64-path probe shows; otherwise the first n paths, n as large as fits."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    _, t64 = cpu_sample(64, a.size, threads)
    per_path = t64 / 64
    budget = 300.0 / max(1, a.steps + a.warmup)
    n_paths = a.paths if per_path * a.paths <= budget else max(64, int(budget / per_path))
    for _ in range(a.warmup):
        cpu_sample(n_paths, a.size, threads)
    t = 0.0
    for _ in range(a.steps):
        _, dt = cpu_sample(n_paths, a.size, threads)
        t += dt
    value = n_paths * a.steps / t
    line = {
        "impl": "reference", "metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000.0 * t / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32/int64/u8", "data": "synthetic",
        "config": {"workload": "curve_heavy_%dx%d_msaa4" % (a.size, a.size), "paths_per_frame": a.paths,
                   "sample": "first %d paths of the scene per step" % n_paths, "same_config": n_paths == a.paths},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                         "sample": "first %d of %d paths, full %dx%d surface" % (n_paths, a.paths, a.size, a.size)},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "vkvg itself is unavailable on this box (Vulkan-only; vkh/glutess submodules empty); the timed "
                "CPU implementation restates its path geometry and raster state",
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank)
        return

    import ctypes as C

    import numpy as np
    import torch

    import vkvg_gb300 as gb
    from vkvg_gb300 import scenes

    torch.cuda.set_device(local)
    if a.analytic_glyphs_only:
        buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        gb._build.build()
        print(json.dumps(analytic_glyph_bench(a, gb, torch, np, buf.zero_, cpu=not a.no_cpu)))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    gb._build.build()
    L = gb.lib()
    sc = scenes.curve_heavy(n_paths=a.paths, size=a.size, seed=1)
    cmds, args = scenes.encode(sc["ops"])
    cptr, aptr = cmds.ctypes.data_as(C.c_void_p), args.ctypes.data_as(C.c_void_p)

    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, a.size, a.size)
    ctx = surf.context()
    st = L.vkvg_gb300_replay_stream(ctx.h, cptr, len(cmds), aptr, len(args))
    assert st == 0, st
    frame = L.vkvg_gb300_frame_capture(ctx.h)
    assert frame
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def l2_flush():
        flush.zero_()
        torch.cuda.synchronize()

    timing = np.zeros(8, np.float32)
    stats = np.zeros(16, np.uint64)
    for _ in range(a.warmup):
        l2_flush()
        assert L.vkvg_gb300_frame_execute(frame, surf.h) == 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    l0 = gb.kernel_launches()
    tot = np.zeros(5)
    for _ in range(a.steps):
        l2_flush()
        assert L.vkvg_gb300_frame_execute(frame, surf.h) == 0
        L.vkvg_gb300_frame_timing(frame, timing.ctypes.data_as(C.c_void_p))
        tot += timing[:5]
    launches = gb.kernel_launches() - l0
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    L.vkvg_gb300_frame_stats(frame, stats.ctypes.data_as(C.c_void_p))
    ms = reduce_max(tot[4] / a.steps, dist, "cuda")
    paths = a.paths  # each path is filled and stroked (two draws)
    value = whole_job_rate(paths, world, ms / 1000.0)

    # ---- end to end through the C API with host buffers
    img = np.zeros((a.size, a.size, 4), np.uint8)
    iptr = img.ctypes.data_as(C.c_void_p)
    ectx = surf.context()

    def e2e_step():
        s = L.vkvg_gb300_replay_stream(ectx.h, cptr, len(cmds), aptr, len(args))
        assert s == 0, s
        L.vkvg_flush(ectx.h)
        assert L.vkvg_surface_write_to_memory(surf.h, iptr) == 0

    for _ in range(a.warmup):
        e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e_steps = max(3, a.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e_steps):
        e2e_step()
    e_t = reduce_max((time.perf_counter() - t0) / e_steps, dist, "cuda")
    e2e_value = whole_job_rate(paths, world, e_t)
    h2d = int(stats[12])
    d2h = a.size * a.size * 4

    # ---- SVG ingestion through vkvg's SVG API (include/vkvg-svg.h): parse a
    # seeded tiger-scale document, then render it on a surface of its size and
    # read the image back, every step
    svg = None
    if a.svg_shapes > 0:
        text = scenes.svg_document(seed=7, n_shapes=a.svg_shapes, size=a.size)
        t0 = time.perf_counter()
        doc = gb.Svg(text)
        parse_ms = (time.perf_counter() - t0) * 1000.0
        sw, sh = doc.dimensions()
        nshapes = int(L.vkvg_gb300_svg_shape_count(doc.h))
        ssurf = gb.Surface(dev, sw, sh)
        sctx = ssurf.context()
        simg = np.zeros((sh, sw, 4), np.uint8)

        def svg_step():
            doc.render(sctx)
            L.vkvg_flush(sctx.h)
            assert L.vkvg_surface_write_to_memory(ssurf.h, simg.ctypes.data_as(C.c_void_p)) == 0

        for _ in range(2):
            svg_step()
        torch.cuda.synchronize()
        s_steps = 5
        t0 = time.perf_counter()
        for _ in range(s_steps):
            svg_step()
        s_t = (time.perf_counter() - t0) / s_steps
        svg = {"workload": "seeded SVG document (svg_document seed 7), %d shapes, %dx%d, 4x MSAA" % (nshapes, sw, sh),
               "bytes": len(text), "parse_ms": parse_ms, "render_e2e_ms": s_t * 1000.0,
               "shapes_per_s": nshapes / s_t, "note": "host timer around vkvg_svg_render + vkvg_flush + "
                                                      "write_to_memory; not the headline metric"}
        sctx.destroy()
        ssurf.destroy()
        doc.destroy()

    # ---- the uneven batch (64 surfaces, Pareto path counts): its frames one
    # after another (the plain form), then as one batch job
    batch = None
    if not a.no_batch and world == 1:
        bs = scenes.batch_streams(seed=2)
        bframes, bsurf, bctx, btarget = [], [], [], []
        for s_ in bs:
            s1 = gb.Surface(dev, s_["width"], s_["height"])
            s2 = gb.Surface(dev, s_["width"], s_["height"])
            c1 = s1.context()
            assert L.vkvg_gb300_replay_stream(c1.h, s_["cmds"].ctypes.data_as(C.c_void_p), len(s_["cmds"]),
                                              s_["args"].ctypes.data_as(C.c_void_p), len(s_["args"])) == 0
            bframes.append(L.vkvg_gb300_frame_capture(c1.h))
            bsurf.append(s1)
            bctx.append(c1)
            btarget.append(s2)
        bpaths = sum(s_["paths"] for s_ in bs)

        def plain_pass():
            for fr, s1 in zip(bframes, bsurf):
                assert L.vkvg_gb300_frame_execute(fr, s1.h) == 0

        plain_pass()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            plain_pass()
        torch.cuda.synchronize()
        plain_s = (time.perf_counter() - t0) / 3
        fa = (C.c_void_p * len(bframes))(*bframes)
        ta = (C.c_void_p * len(btarget))(*[s2.h for s2 in btarget])
        bt = L.vkvg_gb300_batch_create(fa, ta, len(bframes))
        assert bt
        for _ in range(16):  # sizing, fourteen tuning runs, graph capture
            assert L.vkvg_gb300_batch_execute(bt) == 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            assert L.vkvg_gb300_batch_execute(bt) == 0
        batch_s = (time.perf_counter() - t0) / 5
        bt_info = np.zeros(9, np.float32)
        L.vkvg_gb300_batch_timing(bt, bt_info.ctypes.data_as(C.c_void_p))
        same = all(np.array_equal(s1.samples_rgba(), s2.samples_rgba()) for s1, s2 in zip(bsurf[:8], btarget[:8]))
        batch = {"workload": "64 surfaces, side log-U[256,2048], Pareto(1.2) paths in [100,20000], segments "
                             "log-U[3,2000] (70%% cubic, 20%% line, 10%% arc), seed 2: %d paths, %.1f Mpx" %
                             (bpaths, sum(s_["width"] * s_["height"] for s_ in bs) / 1e6),
                 "plain_ms": plain_s * 1e3, "plain_paths_per_s": bpaths / plain_s, "batch_ms": batch_s * 1e3,
                 "batch_paths_per_s": bpaths / batch_s, "speedup": plain_s / batch_s,
                 "graph_replay": bool(bt_info[1]), "tuned_stage_min": int(bt_info[2]),
                 "tuned_heaviest_first": bool(bt_info[3]), "tuned_tile_px": int(bt_info[8]),
                 "work_items": int(bt_info[4]),
                 "first_8_surfaces_equal_to_plain": same,
                 "note": "host timer, device-resident frames; the plain form executes the 64 captured frames one "
                         "after another"}
        L.vkvg_gb300_batch_destroy(bt)
        for fr, c1, s1, s2 in zip(bframes, bctx, bsurf, btarget):
            L.vkvg_gb300_frame_destroy(fr)
            c1.destroy()
            s1.destroy()
            s2.destroy()

    # ---- the differentiable analytic-coverage workload
    analytic = None
    if not a.no_analytic and world == 1:
        analytic = analytic_bench(a, gb, torch, np, l2_flush, cpu=rank == 0 and not a.no_cpu)
        if not a.no_glyphs:
            analytic["glyphs"] = analytic_glyph_bench(a, gb, torch, np, l2_flush, cpu=rank == 0 and not a.no_cpu)

    # ---- the small polygon configuration as stated
    small = small_polygon_bench(a, gb, L, np, l2_flush) if world == 1 else None

    # ---- the large glyph scene (4096x4096, 200k quadratic outlines + 20k strokes)
    glyphs = None
    if not a.no_glyphs and world == 1:
        glyphs = glyph_bench(a, gb, L, np, l2_flush)

    # ---- roofline of the raster/composite kernel
    peak, peak_kind = hbm_peak()
    nflat, nsv = int(stats[1]), int(stats[2])
    raster_bytes = 8 * nflat + 8 * nsv + 8 * a.size * a.size
    raster_ms = tot[3] / a.steps
    achieved = raster_bytes / (raster_ms / 1000.0) / 1e9
    n_ctrl = len(args) // 2
    frame_bytes = 8 * n_ctrl + 4 * len(cmds) + 16 * nflat + 16 * nsv + 8 * a.size * a.size
    prof = {}
    tfile = os.path.join(ROOT, "profiles", "raster_rows_curve_heavy_1024.md")
    if os.path.exists(tfile):
        for ln in open(tfile):
            k, _, v = ln.partition(":")
            if k.strip() in ("dram_bytes_per_launch", "issue_slots_busy_pct", "alu_pipe_active_pct",
                             "warp_inst_per_launch"):
                try:
                    prof[k.strip()] = float(v.split()[0])
                except (ValueError, IndexError):
                    pass
    traffic = int(prof["dram_bytes_per_launch"]) if "dram_bytes_per_launch" in prof else None
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clk["sm_mhz"] if clk else sm_max_mhz()
    issue_peak = sms * 4 * sm_mhz * 1e6  # warp instructions per second, one per scheduler per cycle
    issue = {"bound": "sm issue", "unit": "warp inst/s", "peak": issue_peak, "sms": sms, "sm_mhz": sm_mhz,
             "issue_slots_busy_pct": prof.get("issue_slots_busy_pct"),
             "alu_pipe_active_pct": prof.get("alu_pipe_active_pct"),
             "source": "ncu summary in profiles/raster_rows_curve_heavy_1024.md"}
    if "warp_inst_per_launch" in prof:
        issue["warp_inst_per_launch"] = prof["warp_inst_per_launch"]
        issue["achieved"] = prof["warp_inst_per_launch"] / (raster_ms / 1000.0)
        issue["frac"] = issue["achieved"] / issue_peak

    line = {
        "metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32/int64/u8", "data": "synthetic (seeded scene generator, seed 1)",
        "config": {"workload": "curve_heavy_%dx%d_msaa4" % (a.size, a.size), "paths_per_frame": paths,
                   "cubics_per_path": "U{4..64}", "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed before each step (256 MiB write)",
                   "flattened_points": nflat, "stroke_vertices": nsv, "stroke_triangles": int(stats[10]),
                   "fill_edges": int(stats[4]), "bin_units": int(stats[5])},
        "stage_ms": {"flatten": tot[0] / a.steps, "stroke": tot[1] / a.steps, "setup_bin": tot[2] / a.steps,
                     "raster": raster_ms},
        "mpx_per_s": a.size * a.size * world / (ms / 1000.0) / 1e6,
        "e2e": {"value": e2e_value, "unit": "paths/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e_t * 1000.0},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "gb_raster_rows (row form, half bands)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "algorithmic_bytes": raster_bytes, "frame_bytes": frame_bytes,
                     "frame_frac": frame_bytes / (ms / 1000.0) / 1e9 / peak, "issue": issue},
        "clocks": clk,
    }
    if small:
        line["small_polygons"] = small
    if batch:
        line["batch"] = batch
    if glyphs:
        line["glyphs"] = glyphs
    if svg:
        line["svg"] = svg
    if analytic:
        analytic["roofline"]["peak"] = peak
        analytic["roofline"]["frac"] = analytic["roofline"]["achieved"] / peak
        line["analytic"] = analytic
    if rank == 0 and not a.no_cpu:
        threads = os.cpu_count() or 1
        ts = [cpu_sample(256, a.size, threads)[1] for _ in range(3)]
        v = 256 / statistics.median(ts)
        line["cpu_baseline"] = {"value": v, "unit": "paths/s", "cores": threads, "kind": "port",
                                "sample": "first 256 of %d paths, full %dx%d surface, 4x MSAA, median of 3" %
                                          (paths, a.size, a.size),
                                "configs": cpu_configs(threads)}
    L.vkvg_gb300_frame_destroy(frame)
    ectx.destroy()
    ctx.destroy()
    surf.destroy()
    dev.destroy()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
