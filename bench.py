#!/usr/bin/env python
"""Benchmark of the GB300 span mesher: MeshBuffer::generate_for_box on one
octree span of 512^3 cells (513^3 = 135,005,697 corners), Mandelbulb P=8,
max_iters 15, bailout 2.5, over [-1.2, 1.2]^3 (widened by one cell per side,
src/mesh/buffer.rs:64-67).  One step = one full mesh: distance estimator at
every corner, surface-cell compaction, vertex placement with the reference's
six-sample normals, and the quad index list.

Prints one JSON line.  `value` = corners processed per second (whole job,
all ranks) with outputs left in HBM, timed with CUDA events on the mesher's
stream; `e2e` = the same through cg_generate_for_box into pinned host buffers
(device-to-host copies inside the timed region).  `--impl reference` times
the CPU restatement of the reference's mesher (the reference itself, Rust and
x86-only, cannot be built here) on all host cores.
"""
import argparse
import concurrent.futures as cf
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DE pts/s fwd & fwd+adjoint vs FD normals, 1 GB300, % FP32 peak"
UNIT = "pts/s"
RES = 512
SHAPE = dict(power=8, max_iters=15, bailout=2.5)
WORKLOAD = ("single octree span, 512^3 cells / 513^3 = 135,005,697 corners, Mandelbulb P=8 "
            "max_iters 15 bailout 2.5, span [-1.2,1.2]^3; DE + surface cells + vertices with "
            "FD normals + quad indices")
FLOPS_PER_STEP = 76   # P=8 iteration: magnitude, dr, polynomial, + p (each op = 1 flop)
FLOPS_PER_ESCAPE = 6  # the final magnitude of an escaping point
FLOPS_PER_POINT = 4   # ln(r) * r, * 0.5, / dr
LAUNCHES_PER_MESH = 12  # k_de_grid_brick (sign words fused), k_cells, 3x scan, k_vertex_list,
#                         k_place, k_quad_count, 3x scan, k_quad_emit (ncu launch list: 12 per mesh)


# ---------------------------------------------------------------- measured peaks
def fp32_peak(packed: bool = False) -> float:
    """FP32 flop/s of this GPU (2 per FMA) from the FFMA-chain probe in
    libcantucci_bench.so (benchmark instrumentation, not the C ABI)."""
    from cantucci_gb300 import build
    L = C.CDLL(build.build_bench())
    L.cgb_fp32_peak.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]
    L.cgb_fp32_peak.restype = C.c_int
    out = C.c_double()
    rc = L.cgb_fp32_peak(20000, 1 if packed else 0, C.byref(out))
    if rc != 0:
        raise RuntimeError("FP32 peak probe failed with CUDA error %d" % rc)
    return out.value


def ncu_record(kernel: str, res: int, pdir: str = None, digest: str = None):
    """The ncu figures of `kernel` at `res` recorded for THIS build, or None.
    A profile summary under profiles/ carries a line
        bench-record: digest=<16 hex> kernel=<name> res=<n> dram_bytes=<b> ...
    whose digest is the library build digest the capture ran on; a record of
    another build (any changed source) is ignored.  `pdir` and `digest`
    default to profiles/ and the built library's digest."""
    if digest is None:
        from cantucci_gb300 import build
        stamp = os.path.join(build.LIB_DIR, ".digest")
        try:
            digest = open(stamp).read().strip()
        except OSError:
            return None
    digest = digest[:16]
    pdir = pdir or os.path.join(ROOT, "profiles")
    for name in sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []:
        if not name.endswith(".md"):
            continue
        for line in open(os.path.join(pdir, name)):
            if "bench-record:" not in line:
                continue
            kv = dict(t.split("=", 1) for t in line.split("bench-record:", 1)[1].split()
                      if "=" in t)
            if (kv.get("digest") == digest and kv.get("kernel") == kernel
                    and kv.get("res") == str(res)):
                return kv
    return None


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # nvidia-smi takes a moment to print its first sample; the timed
        # region starts only once sampling runs.
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- CPU side
def leaf_spans(depth: int = 3):
    """The octree leaves of [-1.2,1.2]^3 at `depth` (create_spans order)."""
    from cantucci_gb300.api import Span, create_spans
    level = [Span(*__import__("cantucci_gb300.workloads", fromlist=["x"]).SPAN_C1)]
    for _ in range(depth):
        level = [c for s in level for c in create_spans(s)]
    return level


def cpu_mesh_sample(stride: int = 1, threads: int = None):
    """The reference's CPU path on a bounded sample of the same workload: the
    512 depth-3 octree leaves of the span (res 64 each, the same cell size as
    res 512 over the whole span), every `stride`-th leaf, one leaf per worker
    thread as ShapeMesh's thread pool runs them (src/mesh/mod.rs:58-63,141).
    Returns (corners/s, threads, corners, seconds, sample text)."""
    import numpy as np
    import oracle
    threads = threads or (os.cpu_count() or 1)
    leaves = leaf_spans(3)[::stride]
    shape = oracle.mandelbulb(**SHAPE)
    oracle.lib()

    def one(sp):
        span = np.concatenate([sp.start, sp.end]).astype(np.float32)
        r = oracle.generate_for_box(shape, span, 64, nthreads=1, vcap=64 ** 3, icap=18 * 64 ** 3)
        assert r["rc"] == 0
        return 65 ** 3

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        pts = sum(ex.map(one, leaves))
    dt = time.perf_counter() - t0
    which = ("all 512 depth-3 octree leaves of the span" if stride == 1 else
             "%d of the 512 depth-3 octree leaves of the span (every %dth)" % (len(leaves), stride))
    text = ("%s, res 64 each (%d corners), oracle C restatement of generate_for_box, one leaf "
            "per thread" % (which, pts))
    return pts / dt, threads, pts, dt, text


def run_reference(args, rank, world):
    """--impl reference: the CPU mesher on all host cores, rank 0 only."""
    if rank != 0:
        return
    stride = 1  # all 512 leaves: the whole span at the cell size of res 512
    for _ in range(args.warmup):
        cpu_mesh_sample(stride)
    rates, secs, pts, threads, text = [], 0.0, 0, 0, ""
    for _ in range(args.steps):
        r, threads, p, dt, text = cpu_mesh_sample(stride)
        rates.append(r)
        secs += dt
        pts += p
    value = pts / secs
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "res": RES},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": text + " (the Rust reference is x86-64 only: its Vec3 "
                                          "uses SSE4.1; this is its C restatement, "
                                          "bit-identical to a C++ translation of its own "
                                          "source on x86-64)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU extras
def _time_cuda(fn, reps=3, warm=1, stream=None):
    """Mean CUDA-event milliseconds of fn() over `reps` runs after `warm`."""
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    s = stream or torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        fn()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def extra_batched(dev, cpu=True):
    """4096 seeded octree spans (res 8..64): one batch replayed from a CUDA
    graph vs one cg_generate_for_box_device call per span."""
    import numpy as np
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import workloads as W
    from cantucci_gb300.batch import BatchMesher
    spans, res, power, iters = W.batched_spans(4096, seed=0)
    shape = cg.Mandelbulb(power, iters, 2.5)
    corners = int(np.sum((res.astype(np.int64) + 1) ** 3))
    b = BatchMesher(spans, res, vertex_cap=1 << 24, index_cap=6 << 24, device=dev)
    default_tuning = b.tuning
    ms_default = _time_cuda(lambda: b.run(shape, graph=True), reps=5, warm=2)
    t0 = time.perf_counter()
    tuned = b.autotune(shape, reps=3)
    tune_s = time.perf_counter() - t0
    ms_graph = _time_cuda(lambda: b.run(shape, graph=True), reps=5, warm=2)
    ms_direct = _time_cuda(lambda: b.run(shape, graph=False), reps=3, warm=1)
    out = b.run(shape, graph=True)
    _, tot = out.host()
    cpu_s, threads, same = None, os.cpu_count() or 1, None
    if cpu:
        # the CPU builder (oracle restatement of generate_for_box) on every
        # span, one span per host thread, and index lists compared on a sample
        import oracle
        oshape = oracle.mandelbulb(power, iters, 2.5)
        oracle.lib()

        def cpu_one(j):
            return oracle.generate_for_box(oshape, spans[j].astype(np.float32), int(res[j]),
                                           nthreads=1, vcap=int(res[j]) ** 3,
                                           icap=18 * int(res[j]) ** 3)
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            cpu_res = list(ex.map(cpu_one, range(len(res))))
        cpu_s = time.perf_counter() - t0
        same = sum(int(np.array_equal(out.mesh(j)[1], cpu_res[j]["indices"]))
                   for j in range(0, len(res), 16))
    m = cg.Mesher(dev)
    v = torch.empty((64 ** 3, 7), dtype=torch.float32, device=dev)
    i = torch.empty(18 * 64 ** 3, dtype=torch.int32, device=dev)
    t0 = time.perf_counter()
    for sp, r in zip(spans, res):
        m.generate_device(cg.Span(sp[:3], sp[3:]), shape, int(r), v, i, strict=False)
    seq_s = time.perf_counter() - t0
    m.close()
    # every power and max_iters the workload draws from, same spans and tuning
    draws = {}
    for P in (6, 8, 10):
        for it in (10, 15, 20):
            sh = cg.Mandelbulb(P, it, 2.5)
            ms = _time_cuda(lambda: b.run(sh, graph=True), reps=3, warm=1)
            _, t = b.run(sh, graph=True).host()
            draws["p%d_i%d" % (P, it)] = {"graph_ms": ms, "spans_per_s": 4096 / (ms * 1e-3),
                                          "corners_per_s": corners / (ms * 1e-3),
                                          "vertices": int(t[0]), "quads": int(t[1])}
    b.close()
    return {"workload": "4096 spans, centres on the 0.8-1.15 shell, edge 2^-k k in 3..7, res in "
                        "{8,16,32,64}, power %d, max_iters %d, seed 0" % (power, iters),
            "corners": corners, "vertices": int(tot[0]), "quads": int(tot[1]),
            "graph_ms": ms_graph, "direct_ms": ms_direct, "graph_ms_default_tuning": ms_default,
            "default_tuning": default_tuning, "tuning": tuned["tuning"],
            "autotune_s": tune_s,
            "cpu_builder_s": cpu_s, "cpu_builder_threads": threads,
            "cpu_builder_spans_per_s": 4096 / cpu_s if cpu_s else None,
            "speedup_vs_cpu_builder": cpu_s / (ms_graph * 1e-3) if cpu_s else None,
            "index_lists_equal_cpu_builder": ("%d of %d sampled spans" %
                                              (same, len(range(0, len(res), 16)))
                                              if cpu_s else None),
            "spans_per_s": 4096 / (ms_graph * 1e-3), "corners_per_s": corners / (ms_graph * 1e-3),
            "per_span_launches_s": seq_s, "per_span_spans_per_s": 4096 / seq_s,
            "speedup_vs_per_span": seq_s / (ms_graph * 1e-3),
            "every_draw": draws,
            "every_draw_note": "the same 4096 spans and tuned launch shapes for each power "
                               "{6, 8, 10} x max_iters {10, 15, 20}; P != 8 runs the "
                               "reference's trig path (acosf/atan2f/sinf/cosf)"}


def band_points(shape, n, seed=1, oversample=6):
    """n points drawn uniformly in [-1.2,1.2]^3, moved by 8 sphere-trace steps
    along random unit directions, kept where |DE| < 1e-3."""
    import numpy as np
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    keep = []
    have = 0
    while have < n:
        m = oversample * n
        p = torch.rand((m, 3), generator=g, device="cuda") * 2.4 - 1.2
        d = torch.randn((m, 3), generator=g, device="cuda")
        d = d / d.norm(dim=1, keepdim=True)
        for _ in range(8):
            p = p + d * shape.batch_min_distance_from(p)[:, None]
        de = shape.batch_min_distance_from(p)
        k = p[torch.isfinite(de) & (de.abs() < 1e-3)]
        keep.append(k)
        have += k.shape[0]
    return torch.cat(keep)[:n].contiguous()


def extra_normals(dev, n=16 << 20, cpu=True):
    """Adjoint normals vs six-evaluation central differences on 16M band
    points (polar form, power 8, max_iters 15), with angular errors against
    the FP64 forward-mode oracle on a 2000-point subsample."""
    import numpy as np
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300.autograd import de_grad, fd_grad
    from cantucci_gb300 import _ffi
    lib = _ffi.load()
    shape = cg.MandelbulbPolar(8.0, 15, 2.5)
    pts = band_points(shape, n)
    ms_fwd = _time_cuda(lambda: shape.batch_min_distance_from(pts), reps=2)
    ms_adj = _time_cuda(lambda: de_grad(pts, 8.0), reps=2)
    _ffi.check(lib.cg_set_option(b"adjoint_recompute", 1))
    try:
        ms_adj_fr = _time_cuda(lambda: de_grad(pts, 8.0), reps=2)
    finally:
        _ffi.check(lib.cg_set_option(b"adjoint_recompute", 0))
    ms_tan = _time_cuda(lambda: de_grad(pts, 8.0, mode="tangent", with_power=False), reps=2)
    ms_tan4 = _time_cuda(lambda: de_grad(pts, 8.0, mode="tangent"), reps=2)
    ms_tanf = _time_cuda(lambda: de_grad(pts, 8.0, mode="tangent", with_power=False, fast=True),
                         reps=2)
    ms_fd = _time_cuda(lambda: fd_grad(pts, shape, 1e-4), reps=2)
    out = {"workload": "%d points in |DE| < 1e-3 (uniform in [-1.2,1.2]^3, 8 sphere-trace steps "
                       "along random directions), polar Mandelbulb power 8, max_iters 15" % n,
           "forward_pts_per_s": n / (ms_fwd * 1e-3),
           "fwd_adjoint_pts_per_s": n / (ms_adj * 1e-3),
           "fwd_tangent_normals_pts_per_s": n / (ms_tan * 1e-3),
           "fwd_tangent_all_pts_per_s": n / (ms_tan4 * 1e-3),
           "fd6_pts_per_s": n / (ms_fd * 1e-3),
           "adjoint_vs_fd6_speedup": ms_fd / ms_adj,
           "fwd_adjoint_fast_recompute_pts_per_s": n / (ms_adj_fr * 1e-3),
           "adjoint_fast_recompute_vs_fd6_speedup": ms_fd / ms_adj_fr,
           "tangent_normals_vs_fd6_speedup": ms_fd / ms_tan,
           "tangent_all_vs_fd6_speedup": ms_fd / ms_tan4,
           "fwd_tangent_fast_normals_pts_per_s": n / (ms_tanf * 1e-3),
           "tangent_fast_normals_vs_fd6_speedup": ms_fd / ms_tanf,
           "modes": "adjoint = reverse mode with checkpoint recompute (DE, grad, d/dpower, "
                    "d/drotation; checkpoint every 5 steps, tape in shared memory); "
                    "adjoint_fast_recompute = the same with each segment recomputed from its "
                    "exact checkpoint in the fast polar arithmetic (cg_set_option "
                    "adjoint_recompute 1); tangent_normals = forward mode along x, y, z (DE, "
                    "grad, d/drotation); tangent_all = forward mode with the power direction too"}
    if not cpu:
        return out
    try:
        import oracle
        sub = pts[:2000]
        ref = oracle.de_grad_f64(oracle.mandelbulb_polar(8.0, 15, 2.5), sub.cpu().numpy())
        a = de_grad(sub, 8.0).cpu().numpy().astype(np.float64)
        _ffi.check(lib.cg_set_option(b"adjoint_recompute", 1))
        try:
            afr = de_grad(sub, 8.0).cpu().numpy().astype(np.float64)
        finally:
            _ffi.check(lib.cg_set_option(b"adjoint_recompute", 0))
        t = de_grad(sub, 8.0, mode="tangent", with_power=False).cpu().numpy().astype(np.float64)
        tf = de_grad(sub, 8.0, mode="tangent", with_power=False,
                     fast=True).cpu().numpy().astype(np.float64)
        f = fd_grad(sub, shape, 1e-4).cpu().numpy().astype(np.float64)

        def ang(x, y):
            x = x / np.linalg.norm(x, axis=1, keepdims=True)
            y = y / np.linalg.norm(y, axis=1, keepdims=True)
            return np.degrees(np.arccos(np.clip(np.sum(x * y, axis=1), -1, 1)))
        ok = np.all(np.isfinite(ref[:, 1:4]), axis=1)
        def stats(e):
            return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)),
                    "frac_le_0.1": float(np.mean(e <= 0.1))}
        out["angle_deg_vs_fp64"] = {
            "adjoint": stats(ang(a[ok, 1:4], ref[ok, 1:4])),
            "adjoint_fast_recompute": stats(ang(afr[ok, 1:4], ref[ok, 1:4])),
            "tangent": stats(ang(t[ok, 1:4], ref[ok, 1:4])),
            "tangent_fast": stats(ang(tf[ok, 1:4], ref[ok, 1:4])),
            "fd6_h1e-4": stats(ang(f[ok], ref[ok, 1:4]))}
        # no step size brings the f32 central difference to the adjoint's error
        for h in (1e-2, 1e-3, 3e-4, 3e-5, 1e-5):
            fh = fd_grad(sub, shape, h).cpu().numpy().astype(np.float64)
            out["angle_deg_vs_fp64"]["fd6_h%g" % h] = stats(ang(fh[ok], ref[ok, 1:4]))
    except Exception as e:  # the oracle is only a checker here
        out["angle_deg_vs_fp64"] = "unavailable: %s" % e
    return out


def extra_depth_fit(dev, steps=300):
    """1024x1024 depth map of power 8.3 rotated (0.2, 0.1, 0); fit power and
    rotation from (8.0, 0) with Adam (lr 1e-2) on per-pixel L1 depth loss."""
    import torch
    from cantucci_gb300 import fit
    cam = fit.camera(1024, 1024, 2.5, 60.0)
    target = fit.render(8.3, (0.2, 0.1, 0.0), cam)
    ms_fwd = _time_cuda(lambda: fit.render(8.3, (0.2, 0.1, 0.0), cam, out=target), reps=3)
    scratch = torch.empty_like(target)
    ms_fast = _time_cuda(lambda: fit.render(8.3, (0.2, 0.1, 0.0), cam, out=scratch, fast=True),
                         reps=3)
    power = torch.tensor(8.0, requires_grad=True)
    rot = torch.zeros(3, requires_grad=True)
    depth = fit.depth_render(power, rot, cam)
    loss = fit.l1_loss(depth, target)
    ms_bwd = _time_cuda(lambda: torch.autograd.grad(loss, [power, rot], retain_graph=True),
                        reps=3)
    t0 = time.perf_counter()
    p, r, losses = fit.fit(target, cam, steps=steps, lr=1e-2, fast=True)
    fit_s = time.perf_counter() - t0
    # the same steps as plain Adam on the masked depth loss, for comparison
    p0, r0, losses0 = fit.fit(target, cam, steps=steps, lr=1e-2, fast=True, surface_weight=0.0,
                              cap=0.0, anneal=False)
    return {"workload": "1024x1024 depth map, camera at 2.5, fov 60 deg, <= 256 steps, eps 1e-4 "
                        "pixel footprint, polar Mandelbulb power 8.3 rot (0.2, 0.1, 0), "
                        "max_iters 15; Adam %d steps lr 1e-2 from power 8.0, rot 0" % steps,
            "forward_pixels_per_s": 1024 * 1024 / (ms_fwd * 1e-3),
            "forward_fast_pixels_per_s": 1024 * 1024 / (ms_fast * 1e-3),
            "fit_march": "fast estimator (exact gradient)",
            "fit_objective": "depth L1 over pixels hit in both maps + mean |DE| at the target's "
                             "surface points; both gradients without the chaotic outliers "
                             "(|dt/dtheta| > 2, |dDE/dtheta| > 1); lr 1e-2 cosine-annealed",
            "backward_pixels_per_s": 1024 * 1024 / (ms_bwd * 1e-3),
            "fit_seconds": fit_s, "recovered_power": p, "recovered_rotation": r,
            "error_power": abs(p - 8.3),
            "error_rotation": [abs(a - b) for a, b in zip(r, (0.2, 0.1, 0.0))],
            "loss_first": losses[0], "loss_last": losses[-1],
            "plain_adam_masked_depth": {"recovered_power": p0, "recovered_rotation": r0,
                                        "loss_last": losses0[-1]}}


def extra_de_variants(dev, res=RES):
    """The step-1 DE alone (cg_de_span_grid, no sign words) on the 513^3
    span in several numerics: the exact P=8 polynomial (bit-faithful), the
    same polynomial FMA-contracted with approximate division and square root
    (not bit-faithful), the real-power polar form at power 8.0 (the
    reference's GLSL estimator, transcendental-bound), and P=6 through the
    reference's trig path and through the trig-free complex-power form.  Flop rates use the
    exact path's algorithmic count (76 per iteration, the exact path's
    iteration totals) for both P=8 variants."""
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import _ffi, workloads as W
    lib = _ffi.load()
    span = cg.Span(*W.SPAN_C1)
    n = res + 1
    out = torch.empty((n, n, n), dtype=torch.float32, device=dev)
    exact = cg.Mandelbulb(**SHAPE)
    steps_c, esc_c = C.c_uint64(), C.c_uint64()
    _ffi.check(lib.cg_span_grid_work(C.byref(exact._cshape()), C.byref(span.to_c()), res,
                                     C.byref(steps_c), C.byref(esc_c)))
    flops = FLOPS_PER_STEP * steps_c.value + FLOPS_PER_ESCAPE * esc_c.value + FLOPS_PER_POINT * n ** 3
    peak = fp32_peak(False)
    res_out = {"workload": "%d^3 corners of [-1.2,1.2]^3 widened, max_iters 15" % n,
               "fp32_peak_tflops": peak / 1e12}
    p6 = cg.Mandelbulb(6, 15, 2.5)
    for name, shape in (("exact_p8", exact), ("fast_p8", exact.fast()),
                        ("polar_p8.0", cg.MandelbulbPolar(8.0, 15, 2.5)),
                        ("polar_p8.0_fast", cg.MandelbulbPolar(8.0, 15, 2.5).fast()),
                        ("trig_p6", p6), ("trig_free_p6", p6.fast())):
        ms = _time_cuda(lambda: shape.span_grid(span, res, out=out), reps=5, warm=2)
        e = {"ms": ms, "pts_per_s": n ** 3 / (ms * 1e-3)}
        if name in ("exact_p8", "fast_p8"):
            e["tflops"] = flops / (ms * 1e-3) / 1e12
            e["frac_of_fp32_peak"] = e["tflops"] * 1e12 / peak
        res_out[name] = e
    return res_out


def _mesh_normals(dev, shape, workload, res, oshape=None):
    """The span mesher at res with the reference's six-sample normals and
    with analytic (forward-mode) normals: same vertices, DE values and
    indices; stage times, and with `oshape` (CPU legs only) the angle of
    both normals to the FP64 gradient at 2000 sampled vertices."""
    import numpy as np
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import workloads as W
    span = cg.Span(*W.SPAN_C1)
    vcap, icap = res ** 3 // 16, 18 * res ** 3 // 16
    v = torch.empty((vcap, 7), dtype=torch.float32, device=dev)
    i = torch.empty(icap, dtype=torch.int32, device=dev)
    out = {"workload": workload}
    verts = {}
    m = cg.Mesher(dev)
    try:
        for mode in ("fd", "analytic"):
            m.set_normals(mode)
            m.generate_device(span, shape, res, v, i, strict=False)
            tms = []
            for _ in range(3):
                nv, ni, tm = m.generate_device(span, shape, res, v, i, strict=False)
                tms.append(tm)
            out[mode] = {"step1_ms": min(t.first_ms for t in tms),
                         "step2_ms": min(t.second_ms for t in tms),
                         "step3_ms": min(t.third_ms for t in tms),
                         "mesh_ms": min(t.first_ms + t.second_ms + t.third_ms for t in tms),
                         "vertices": nv, "indices": ni}
            verts[mode] = v[:nv].cpu().numpy()
    finally:
        m.close()
    out["step2_speedup"] = out["fd"]["step2_ms"] / out["analytic"]["step2_ms"]
    out["mesh_speedup"] = out["fd"]["mesh_ms"] / out["analytic"]["mesh_ms"]
    out["same_positions_de"] = bool(np.array_equal(
        verts["fd"][:, [0, 1, 2, 6]].view(np.uint32),
        verts["analytic"][:, [0, 1, 2, 6]].view(np.uint32)))
    if oshape is not None:
        import oracle
        rng = np.random.default_rng(5)
        sel = rng.choice(len(verts["fd"]), size=min(2000, len(verts["fd"])), replace=False)
        g = oracle.de_grad_f64(oshape, verts["fd"][sel, :3])[:, 1:4]
        ok = np.all(np.isfinite(g), axis=1)
        for mode in ("fd", "analytic"):
            nrm = verts[mode][sel][ok, 3:6].astype(np.float64)
            gg = g[ok] / np.linalg.norm(g[ok], axis=1, keepdims=True)
            c = np.sum(nrm / np.linalg.norm(nrm, axis=1, keepdims=True) * gg, axis=1)
            ang = np.degrees(np.arccos(np.clip(c, -1, 1)))
            out[mode]["angle_deg_vs_fp64"] = {"median": float(np.median(ang)),
                                              "frac_le_0.1": float(np.mean(ang <= 0.1))}
    return out


def extra_polar_mesh_normals(dev, res=RES):
    """Six-sample vs analytic normals on the polar Mandelbulb (power 8.0)."""
    import cantucci_gb300 as cg
    return _mesh_normals(dev, cg.MandelbulbPolar(8.0, 15, 2.5),
                         "polar Mandelbulb power 8.0, max_iters 15, %d^3 corners" % (res + 1), res)


def extra_p8_mesh_normals(dev, res=RES, cpu=True):
    """Six-sample vs analytic normals on the reference's Mandelbulb<8> (the
    polynomial differentiated in dual numbers)."""
    import cantucci_gb300 as cg
    oshape = None
    if cpu:
        import oracle
        oshape = oracle.mandelbulb(**SHAPE)
    return _mesh_normals(dev, cg.Mandelbulb(**SHAPE),
                         "Mandelbulb P=8 max_iters 15, %d^3 corners" % (res + 1), res, oshape)


def extra_fp64_check(dev, res=RES, stride=67):
    """Distances of the 513^3 span against the FP64 oracle on every 67th
    corner (~2M points): sign agreement, the share within 1e-5 relative and
    1e-6 absolute, and how many of the points outside 1e-5 relative escape
    at a different iteration than in FP64."""
    import numpy as np
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import _ffi, workloads as W
    import oracle
    shape = cg.Mandelbulb(**SHAPE)
    span = cg.Span(*W.SPAN_C1)
    n = res + 1
    d32 = shape.span_grid(span, res).reshape(-1)
    idx = torch.arange(0, n ** 3, stride, device=d32.device)
    d32 = d32[idx].cpu().numpy().astype(np.float64)
    # corner coordinates exactly as the kernels form them (f32, v / res exact)
    rf = np.float32(res)
    st = (span.start + -((span.end - span.start) / rf)).astype(np.float32)
    en = (span.end + (span.end - span.start) / rf).astype(np.float32)
    across = (en - st).astype(np.float32)
    ii = idx.cpu().numpy()
    v = np.stack([ii // (n * n), (ii // n) % n, ii % n], 1).astype(np.float32)
    pts = (st + across * (v * (np.float32(1.0) / rf))).astype(np.float32)
    pd = torch.as_tensor(pts).to(dev)
    state = torch.empty((len(pts), 4), dtype=torch.float32, device=dev)
    _ffi.check(_ffi.load().cg_mandelbulb_state(C.byref(shape._cshape()), C.c_void_p(pd.data_ptr()),
                                               len(pts), C.c_void_p(state.data_ptr()), None))
    steps32 = state.cpu().numpy()[:, 2].view(np.uint32)
    d64, steps64 = oracle.de_f64(oracle.mandelbulb(**SHAPE), pts, with_steps=True)
    fin = np.isfinite(d64) & np.isfinite(d32)
    rel_ok = np.abs(d32 - d64) <= 1e-5 * np.abs(d64)
    out_rel = fin & ~rel_ok
    frac = float(np.mean(rel_ok[fin]))
    return {"workload": "every %dth corner of the 513^3 span (%d points)" % (stride, len(pts)),
            "sign_agreement": float(np.mean(np.signbit(d32[fin]) == np.signbit(d64[fin]))),
            "target": ">= 99.9% within 1e-5 relative of FP64, the rest confined to points "
                      "whose escape step differs",
            "target_met": bool(frac >= 0.999 or
                               int(out_rel.sum()) == int((out_rel & (steps32 != steps64)).sum())),
            "target_note": "the reference's own f32 loop, reproduced here bit for bit, does not "
                           "meet it: most points outside 1e-5 escape at the same step as FP64",
            "frac_within_1e-5_rel": frac,
            "frac_within_1e-6_abs": float(np.mean(np.abs(d32[fin] - d64[fin]) <= 1e-6)),
            "outside_1e-5_rel": int(out_rel.sum()),
            "outside_with_other_escape_step": int((out_rel & (steps32 != steps64)).sum()),
            "non_finite": int((~fin).sum())}


def extra_small_span(dev, reps=50):
    """Config 1: the 65^3-corner span (res 64, the reference's leaf
    resolution) meshed alone, device outputs and pinned host outputs: a
    latency-bound call (8 kernels on 274,625 corners: the scans fit one tile)."""
    import numpy as np
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import workloads as W
    span = cg.Span(*W.SPAN_C1)
    shape = cg.Mandelbulb(**SHAPE)
    res = 64
    m = cg.Mesher(dev)
    v = torch.empty((res ** 3 // 4, 7), dtype=torch.float32, device=dev)
    i = torch.empty(18 * res ** 3 // 4, dtype=torch.int32, device=dev)
    vh = torch.empty((res ** 3 // 4, 7), dtype=torch.float32, pin_memory=True)
    ih = torch.empty(18 * res ** 3 // 4, dtype=torch.int32, pin_memory=True)
    vnp = vh.numpy().view(cg.VERTEX_DTYPE).reshape(-1)
    inp = ih.numpy().view(np.uint32)
    try:
        for _ in range(5):
            m.generate_device(span, shape, res, v, i)
            m.generate(span, shape, res, vertices=vnp, indices=inp)
        t0 = time.perf_counter()
        for _ in range(reps):
            nv, ni, _ = m.generate_device(span, shape, res, v, i)
        dev_s = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            m.generate(span, shape, res, vertices=vnp, indices=inp)
        host_s = (time.perf_counter() - t0) / reps
    finally:
        m.close()
    n = (res + 1) ** 3
    return {"workload": "single span [-1.2,1.2]^3 at res 64 (274,625 corners), P=8, max_iters 15",
            "vertices": nv, "indices": ni,
            "device_call_ms": 1e3 * dev_s, "device_corners_per_s": n / dev_s,
            "host_call_ms": 1e3 * host_s, "host_corners_per_s": n / host_s,
            "timing": "host wall clock per synchronous call, %d calls" % reps}


def extra_lod(dev, cpu=True, updates=24):
    """The level-of-detail driver on a camera flight towards the surface:
    the camera moves from 3.0 to 1.25 from the origin along -y over 24
    updates (each one waits for its batched run), res-64 leaves as in the
    reference.  Reports the leaves meshed, the time per update, and the CPU
    builder's time for the same jobs (one job per host thread)."""
    import numpy as np
    import cantucci_gb300 as cg
    from cantucci_gb300.lod import Camera, ShapeMesh
    shape = cg.Mandelbulb(**SHAPE)
    sm = ShapeMesh(shape, resolution=64, device=dev)
    jobs, times, splits = [], [], 0
    seen = set()
    try:
        for k in range(updates):
            y = -3.0 + (3.0 - 1.25) * k / (updates - 1)
            cam = Camera(position=(0.05, y, 0.08), direction=(0.0, 1.0, 0.03))
            t0 = time.perf_counter()
            st = sm.update(cam, wait=True)
            times.append(time.perf_counter() - t0)
            splits += st["splits"]
            for leaf in sm.leaves():
                key = tuple(leaf.start.tolist()) + tuple(leaf.end.tolist())
                if leaf.status == 1 and key not in seen:
                    seen.add(key)
                    jobs.append(np.concatenate([leaf.start, leaf.end]).astype(np.float32))
        final = sm.leaves()
    finally:
        sm.close()
    out = {"workload": "camera from y=-3.0 to y=-1.25 over %d updates, Mandelbulb P=8 "
                       "max_iters 15, res-64 leaves" % updates,
           "updates": updates, "leaves_meshed": len(jobs), "splits": splits,
           "final_leaves": len(final), "max_depth": max(l.depth for l in final),
           "update_ms_mean": 1e3 * float(np.mean(times)),
           "update_ms_max": 1e3 * float(np.max(times)),
           "gpu_leaves_per_s": len(jobs) / float(np.sum(times))}
    if cpu and jobs:
        import oracle
        oshape = oracle.mandelbulb(**SHAPE)
        oracle.lib()
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            list(ex.map(lambda sp: oracle.generate_for_box(oshape, sp, 64, nthreads=1,
                                                           vcap=64 ** 3, icap=18 * 64 ** 3),
                        jobs))
        cpu_s = time.perf_counter() - t0
        out["cpu_builder_s"] = cpu_s
        out["cpu_leaves_per_s"] = len(jobs) / cpu_s
        out["speedup_vs_cpu_builder"] = out["gpu_leaves_per_s"] / out["cpu_leaves_per_s"]
    return out


def extra_root_crossings(dev, res=RES):
    """The 513^3 span meshed with the reference's lerped crossings and with
    root-found crossings (4 Illinois steps per crossing edge): mesh time and
    the median |DE| at the vertices."""
    import numpy as np
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import workloads as W
    span = cg.Span(*W.SPAN_C1)
    shape = cg.Mandelbulb(**SHAPE)
    vcap, icap = res ** 3 // 16, 18 * res ** 3 // 16
    v = torch.empty((vcap, 7), dtype=torch.float32, device=dev)
    i = torch.empty(icap, dtype=torch.int32, device=dev)
    out = {"workload": "Mandelbulb P=8 max_iters 15, %d^3 corners" % (res + 1)}
    m = cg.Mesher(dev)
    try:
        for mode in ("lerp", "root"):
            m.set_crossings(mode, 4)
            m.generate_device(span, shape, res, v, i, strict=False)
            best = None
            for _ in range(3):
                nv, ni, tm = m.generate_device(span, shape, res, v, i, strict=False)
                ms = tm.first_ms + tm.second_ms + tm.third_ms
                best = ms if best is None else min(best, ms)
            de = v[:nv, 6].abs()
            de = de[torch.isfinite(de)]
            out[mode] = {"mesh_ms": best, "vertices": nv,
                         "median_abs_de_at_vertex": float(de.median())}
    finally:
        m.close()
    out["de_ratio"] = out["root"]["median_abs_de_at_vertex"] / out["lerp"]["median_abs_de_at_vertex"]
    return out


def extra_dual_contouring(dev, res=RES):
    """The 513^3 span with the reference's centroid placement and with the
    dual-contouring vertex (one forward-mode gradient per crossing, a 3x3
    QEF per cell), with linear and with root-found (4 Illinois steps)
    crossings: mesh time and the median |DE| at the vertices."""
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import workloads as W
    span = cg.Span(*W.SPAN_C1)
    shape = cg.Mandelbulb(**SHAPE)
    vcap, icap = res ** 3 // 16, 18 * res ** 3 // 16
    v = torch.empty((vcap, 7), dtype=torch.float32, device=dev)
    i = torch.empty(icap, dtype=torch.int32, device=dev)
    out = {"workload": "Mandelbulb P=8 max_iters 15, %d^3 corners" % (res + 1)}
    m = cg.Mesher(dev)
    try:
        for name, placement, crossings in (("centroid", "centroid", "lerp"),
                                           ("qef", "qef", "lerp"),
                                           ("qef_root", "qef", "root")):
            m.set_placement(placement)
            m.set_crossings(crossings, 4)
            m.generate_device(span, shape, res, v, i, strict=False)
            best, best2 = None, None
            for _ in range(3):
                nv, ni, tm = m.generate_device(span, shape, res, v, i, strict=False)
                ms = tm.first_ms + tm.second_ms + tm.third_ms
                if best is None or ms < best:
                    best, best2 = ms, tm.second_ms
            de = v[:nv, 6].abs()
            de = de[torch.isfinite(de)]
            out[name] = {"mesh_ms": best, "step2_ms": best2, "vertices": nv,
                         "median_abs_de_at_vertex": float(de.median())}
    finally:
        m.close()
    for name in ("qef", "qef_root"):
        out[name]["de_ratio"] = (out[name]["median_abs_de_at_vertex"]
                                 / out["centroid"]["median_abs_de_at_vertex"])
    return out


def extra_fast_numerics(dev, res=RES):
    """The 513^3 span meshed with the exact estimator (the reference's bits)
    and with CG_NUMERICS_FAST (FMA-contracted P=8 polynomial, approximate
    division and square roots): mesh time, counts and the fraction of
    corners whose sign agrees with the exact grid."""
    import torch
    import cantucci_gb300 as cg
    from cantucci_gb300 import workloads as W
    span = cg.Span(*W.SPAN_C1)
    shape = cg.Mandelbulb(**SHAPE)
    vcap, icap = res ** 3 // 16, 18 * res ** 3 // 16
    v = torch.empty((vcap, 7), dtype=torch.float32, device=dev)
    i = torch.empty(icap, dtype=torch.int32, device=dev)
    out = {"workload": "Mandelbulb P=8 max_iters 15, %d^3 corners" % (res + 1)}
    signs = {}
    m = cg.Mesher(dev)
    try:
        for mode in ("exact", "fast"):
            m.set_numerics(mode)
            m.generate_device(span, shape, res, v, i, strict=False)
            best = None
            for _ in range(3):
                nv, ni, tm = m.generate_device(span, shape, res, v, i, strict=False)
                ms = tm.first_ms + tm.second_ms + tm.third_ms
                if best is None or ms < best[0]:
                    best = (ms, tm.first_ms, tm.second_ms)
            signs[mode] = torch.signbit(m.last_dists())
            out[mode] = {"mesh_ms": best[0], "step1_ms": best[1], "step2_ms": best[2],
                         "corners_per_s": (res + 1) ** 3 / (best[0] * 1e-3),
                         "vertices": nv, "quads": ni // 6}
    finally:
        m.close()
    out["sign_agreement"] = float((signs["exact"] == signs["fast"]).float().mean())
    out["speedup"] = out["exact"]["mesh_ms"] / out["fast"]["mesh_ms"]
    return out


def extra_leaf_pool(dev, threads=(1, 2, 4, 8, 16)):
    """The reference's call pattern for the same 512 depth-3 leaves the CPU
    baseline meshes (res 64 each): a native thread pool of T threads, each
    with its own mesher, each call the blocking generate_for_box into
    pageable vectors, as ShapeMesh's thread pool calls it
    (src/mesh/mod.rs:141-148); the C++ driver cg_leaf_pool.  Pinned and
    device outputs for comparison.  Whole-job leaves/s per T."""
    import numpy as np
    from cantucci_gb300 import build
    exe = build.build_leaf_pool()
    leaves = leaf_spans(3)
    spans = np.array([np.concatenate([l.start, l.end]) for l in leaves], np.float32)
    fd, path = tempfile.mkstemp(suffix=".f32")
    os.close(fd)
    spans.tofile(path)
    env = dict(os.environ)
    if dev != 0:  # the driver meshes on its device 0
        env["CUDA_VISIBLE_DEVICES"] = str(dev)
    out = {"workload": "512 depth-3 leaves of [-1.2,1.2]^3 at res 64 (140,608,000 corners), "
                       "Mandelbulb P=8 max_iters 15; native threads (C++), one cg_mesher each",
           "host_cores": os.cpu_count()}
    try:
        for mode in ("pageable", "pinned", "device"):
            r = subprocess.run([exe, path, mode, "3"] + [str(t) for t in threads],
                               capture_output=True, text=True, timeout=600, env=env)
            if r.returncode != 0:
                out[mode] = {"error": (r.stderr or r.stdout)[-300:]}
                continue
            rows = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
            out[mode] = {"threads_%d" % row["threads"]: {
                "leaves_per_s": row["leaves_per_s"], "ms_per_leaf": row["ms_per_leaf"],
                "corners_per_s": row["leaves_per_s"] * 65 ** 3, "failed": row["failed"]}
                for row in rows}
    finally:
        os.unlink(path)
    return out


def run_extras(args, dev):
    """The other configurations.  The oracle runs only in CPU legs (the CPU
    builder's timing and the accuracy checks against FP64), which
    --no-cpu-baseline switches off together with the cpu_baseline leg."""
    cpu = not args.no_cpu_baseline
    out = {}
    legs = [("small_span", lambda: extra_small_span(dev)),
            ("de_variants", lambda: extra_de_variants(dev)),
            ("batched_spans", lambda: extra_batched(dev, cpu)),
            ("normals", lambda: extra_normals(dev, cpu=cpu)),
            ("polar_mesh_normals", lambda: extra_polar_mesh_normals(dev)),
            ("p8_mesh_normals", lambda: extra_p8_mesh_normals(dev, cpu=cpu)),
            ("root_crossings", lambda: extra_root_crossings(dev)),
            ("dual_contouring", lambda: extra_dual_contouring(dev)),
            ("fast_numerics", lambda: extra_fast_numerics(dev)),
            ("lod", lambda: extra_lod(dev, cpu)),
            ("leaf_pool", lambda: extra_leaf_pool(dev)),
            ("depth_fit", lambda: extra_depth_fit(dev, args.fit_steps))]
    if cpu:
        legs.insert(1, ("fp64_check", lambda: extra_fp64_check(dev)))
    if args.only_extra:
        legs = [(n, f) for n, f in legs if n == args.only_extra]
    for name, fn in legs:
        try:
            out[name] = fn()
        except Exception as e:  # report, never hide the headline number
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
    return out


# ---------------------------------------------------------------- GPU side
def max_over_ranks(seconds: float, world: int, device) -> float:
    """The slowest rank's time (an all-reduce MAX; NCCL on GPUs, gloo on CPU).
    Replicas: each rank meshes its own copy of the workload, nothing else is
    exchanged."""
    if world <= 1:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def _measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import cantucci_gb300 as cg
    from cantucci_gb300 import _ffi, workloads as W

    torch.cuda.set_device(local_rank)
    lib = _ffi.load()
    dev = local_rank
    shape = cg.Mandelbulb(**SHAPE)
    span = cg.Span(*W.SPAN_C1)
    res = args.res
    _ffi.check(lib.cg_set_option(b"de_grid_kernel", args.de_kernel))
    n_pts = (res + 1) ** 3
    mesher = cg.Mesher(dev)
    sp = C.c_void_p()
    _ffi.check(lib.cg_mesher_stream(mesher.handle, C.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value, device=dev)

    # Size the outputs from a first (untimed) mesh.
    vcap, icap = max(res ** 3 // 16, 4096), max(18 * res ** 3 // 16, 65536)
    verts_d = torch.empty((vcap, 7), dtype=torch.float32, device=dev)
    idx_d = torch.empty(icap, dtype=torch.int32, device=dev)
    nv, ni, _ = mesher.generate_device(span, shape, res, verts_d, idx_d, strict=False)
    lerp_panic = mesher.last_status == _ffi.CG_ELERP

    def step_device():
        return mesher.generate_device(span, shape, res, verts_d, idx_d, strict=False)

    # Clocks are sampled from the warm-up through the end-to-end run, which
    # brackets the timed region.
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(dev)).split(",")[0])
                          if os.environ.get("CUDA_VISIBLE_DEVICES", "").isdigit() else dev)
    clocks.start()
    for _ in range(args.warmup):
        step_device()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stage = []
    e0.record(stream)
    for _ in range(args.steps):
        _, _, tm = step_device()
        stage.append((tm.first_ms, tm.second_ms, tm.third_ms))
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    t_max = max_over_ranks(ms * 1e-3, world, dev)
    value = world * n_pts * args.steps / t_max

    # End to end: the C ABI with host (pinned) output buffers.
    verts_h = torch.empty((vcap, 7), dtype=torch.float32, pin_memory=True)
    idx_h = torch.empty(icap, dtype=torch.int32, pin_memory=True)
    verts_np = verts_h.numpy().view(cg.VERTEX_DTYPE).reshape(-1)
    idx_np = idx_h.numpy().view(np.uint32)
    mesher.generate(span, shape, res, vertices=verts_np, indices=idx_np, strict=False)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        mesher.generate(span, shape, res, vertices=verts_np, indices=idx_np, strict=False)
    f1.record(stream)
    f1.synchronize()
    e2e_s = max_over_ranks(f0.elapsed_time(f1) * 1e-3, world, dev)
    clk = clocks.stop()
    e2e = {"value": world * n_pts * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": C.sizeof(_ffi.CgSpan) + C.sizeof(_ffi.CgShape),
           "d2h_bytes_per_step": nv * 28 + ni * 4 + 16,
           "gpu_launches_per_step": LAUNCHES_PER_MESH + 1,
           "note": "inputs are the span and shape (kernel parameters); outputs are the mesh, "
                   "the vertices stored by k_place into the pinned buffer, the indices copied "
                   "there by k_copy_words beside it"}

    # Roofline of the dominant kernel (k_de_grid): algorithmic flops from the
    # rotate steps actually executed, over its CUDA-event time per launch.
    steps_c, esc_c = C.c_uint64(), C.c_uint64()
    _ffi.check(lib.cg_span_grid_work(C.byref(shape._cshape()), C.byref(span.to_c()), res,
                                     C.byref(steps_c), C.byref(esc_c)))
    flops = (FLOPS_PER_STEP * steps_c.value + FLOPS_PER_ESCAPE * esc_c.value +
             FLOPS_PER_POINT * n_pts)
    de_ms = statistics.mean(s[0] for s in stage)
    achieved = flops / (de_ms * 1e-3) / 1e12
    peak_tf = fp32_peak(False) / 1e12
    peak2_tf = fp32_peak(True) / 1e12
    roofline = {
        "bound": "fp32",
        "kernel": {0: "k_de_grid_brick", 1: "k_de_grid", 2: "k_de_grid_brick",
                   3: "k_de_grid_p8x2"}[args.de_kernel],
        "achieved": achieved, "peak": peak_tf,
        "unit": "TFLOP/s", "frac": achieved / peak_tf, "traffic": None,
        "peak_source": "measured in this run: FFMA chains, 2 flop per FFMA (FP32 pipe peak; "
                       "not in MEASURED_PEAKS.json)",
        "peak_packed_f32x2": peak2_tf,
        "algorithmic_flops_per_launch": flops,
        "mean_steps_per_point": steps_c.value / n_pts,
        "flop_model": "76 per P=8 iteration + 6 per escape + 4 per point (add/sub/mul/div/sqrt"
                      " = 1 each, as the reference writes them; FMA never used)",
        "ops_frac_of_issue_peak": 2.0 * achieved / peak_tf,
        "ops_note": "each reference op is one FP32-pipe instruction (bit-exact => no FMA), so "
                    "the pipe's op peak is half its FMA flop peak",
    }
    rec = ncu_record(roofline["kernel"], res)
    if args.traffic is not None:
        roofline["traffic"] = args.traffic
        roofline["traffic_source"] = "--traffic (DRAM bytes per launch from an ncu capture)"
    elif rec is not None:
        roofline["traffic"] = float(rec["dram_bytes"])
        # pipe utilisation of the same launch in the same ncu capture
        roofline["ncu_pipe_active"] = {k: float(rec[k]) for k in ("fma", "alu", "xu", "issue")
                                       if k in rec}
        roofline["traffic_source"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one "
                                      "launch in an ncu capture of this build (digest %s)"
                                      % rec["digest"])
    else:
        roofline["traffic_source"] = "no ncu capture of this build: traffic not measured"
    # The same kernel against HBM: it writes one f32 distance per corner and
    # the packed sign words (one bit per corner, rows padded to 32 bits).
    grid_bytes = 4 * n_pts + 4 * (res + 1) ** 2 * ((res + 1 + 31) // 32)
    hbm_peak = _measured_hbm_gbs()
    roofline["hbm_view"] = {
        "algorithmic_bytes_per_launch": grid_bytes,
        "achieved_gbs": grid_bytes / (de_ms * 1e-3) / 1e9,
        "peak_gbs": hbm_peak, "frac": (grid_bytes / (de_ms * 1e-3) / 1e9 / hbm_peak
                                       if hbm_peak else None),
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)" if hbm_peak else None,
    }

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "res": res, "corners": n_pts,
                   "l2": "no flush: each step's working set (1.1 GB grids) exceeds the 129 MB L2",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "numerics": "exact (bit-identical loop state to the reference)"},
        "stages_ms": {"first": statistics.mean(s[0] for s in stage),
                      "second": statistics.mean(s[1] for s in stage),
                      "third": statistics.mean(s[2] for s in stage)},
        "mesh": {"vertices": nv, "indices": ni, "reference_would_panic": lerp_panic,
                 "panic_note": "at res 512 four corners in the y=0 plane evaluate to NaN "
                               "(x underflows, rxy8 = 0) next to outside corners, so a lerp "
                               "factor is NaN and src/math.rs:19 asserts; the mesh is "
                               "completed with factor 0 there, like the oracle"},
        "de_kernel_pts_per_s": n_pts / (de_ms * 1e-3),
        "cells_per_s": world * res ** 3 * args.steps / t_max,
        "roofline": roofline, "e2e": e2e, "clocks": clk,
        "gpu_launches": LAUNCHES_PER_MESH * args.steps,
    }
    if rank == 0 and not args.no_extras:
        line["extras"] = run_extras(args, dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, threads, p, dt, text = cpu_mesh_sample(1)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": text, "seconds": dt}
    if rank == 0:
        print(json.dumps(line), flush=True)
    mesher.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--res", type=int, default=RES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--de-kernel", type=int, default=0, choices=[0, 1, 2, 3],
                    help="step-1 kernel: 0 auto (2x4x4 bricks), 1 linear, 2 bricks, 3 packed "
                         "f32x2 (all bit-identical)")
    ap.add_argument("--fit-steps", type=int, default=300,
                    help="Adam steps of the depth-map fit extra")
    ap.add_argument("--only-extra", default=None,
                    help="run just this one of the extra measurements (e.g. depth_fit)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched, normals and depth-map measurements")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per k_de_grid launch from an ncu capture")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
