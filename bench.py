"""Headline benchmark: cone FP+BP GUPS at 512^3 / 1024 angles on GB300.

One step = one forward projection A(x) and one matched backprojection A.T(y)
of the cone-beam workload (volume 512^3 on the unit cube, ts.cone(size=sqrt2,
cone_angle=0.5), 1024 angles over 2 pi, detector 512 x 768), with inputs
resident in HBM. GUPS = (U_FP + U_BP) / time / 1e9 with U = 512^3 * 1024
voxel-angle updates per projection.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs the same workload on its own GPU
(independent replicas, no collective on the data path; weak scaling) and rank
0 prints one JSON line with the whole-job value (all ranks' updates over the
slowest rank's time).

``--impl reference`` times the reference implementation of this path on the
host cores. The reference (tomosipo) is pure Python around ASTRA's GPU
projector and has no CPU implementation of its own, and ASTRA is not
installed, so that arm runs the project's FP64 CPU oracle (oracle/) with all
host threads on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cone FP+BP GUPS at 512^3/1024 angles"
# Workloads: the headline one (the metric's) and small ones of the same
# geometry family for profiler captures: volume 256^3, 360 angles, 256x384;
# and the headline's volume and detector with 64 angles over 2 pi, whose
# kernels run with the headline's per-angle launch shapes.
WORKLOADS = {"headline": (512, 1024, (512, 768)), "c2": (256, 360, (256, 384)),
             "cone512_64": (512, 64, (512, 768))}
N, ANGLES, DET = WORKLOADS["headline"]
HBM_FALLBACK_GBS = 6800.0
BYTES_PER_UPDATE = 4  # one fp32 voxel operand per voxel-angle update


def metric_name():
    """The headline metric; the c2 profiling workload names its own size."""
    return METRIC if (N, ANGLES) == (512, 1024) else f"cone FP+BP GUPS at {N}^3/{ANGLES} angles"


def workload_geometry(ts):
    vg = ts.volume(shape=N, size=1)
    pg = ts.cone(angles=ANGLES, shape=DET, size=np.sqrt(2), cone_angle=0.5)
    return vg, pg


def config(extra=None):
    c = {
        "workload": f"cone FP+BP, volume {N}^3 unit cube, ts.cone(size=sqrt2, cone_angle=0.5), "
        f"{ANGLES} angles over 2pi, detector {DET[0]}x{DET[1]}, fp32, matched (exact-transpose) BP",
        "volume": [N, N, N],
        "angles": ANGLES,
        "detector": list(DET),
        "phantom": "20 seeded random ellipsoids, densities U[0.1,1] (seed 2)",
        "l2": f"no L2 flush; every step streams a {4 * N ** 3 / 1e9:.2f} GB volume and a "
        f"{4 * DET[0] * DET[1] * ANGLES / 1e9:.2f} GB sinogram (L2 is 129 MB)",
    }
    if extra:
        c.update(extra)
    return c


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while running."""

    FIELDS = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []
        self._thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
        except OSError:
            self.proc = None
            return
        self._thread = threading.Thread(target=self._read, daemon=True)
        self._thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._thread:
            self._thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {
            "sm_mhz": statistics.median(sm),
            "sm_max_mhz": max(smax),
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


# --------------------------------------------------------------------------- CPU baseline
def cpu_baseline_sample(threads=None, angles=None, keep=False):
    """Time the FP64 oracle (FP + matched BP) on a subset of the workload's angles.

    Returns (GUPS, dict) for the updates processed: 512^3 * n_angles per
    projection. With ``keep`` the dict also holds the sample's input volume
    (float32), angle indices and the oracle's FP and BP, for the parity check.
    """
    import tomosipo_gb300 as ts
    from oracle import oracle as orc

    threads = threads or (os.cpu_count() or 1)
    vg, pg = workload_geometry(ts)
    # one angle per thread, at least 8: about 10-20 s of CPU work
    n_angles = angles or max(8, min(threads, 32))
    idx = np.arange(0, ANGLES, ANGLES // n_angles)[:n_angles]
    sub = pg[:: ANGLES // n_angles][:n_angles]
    rng = np.random.default_rng(2)
    x = rng.random(vg.shape, dtype=np.float32)
    t0 = time.perf_counter()
    y = orc.fp(vg, sub, x, threads=threads)
    t1 = time.perf_counter()
    bp = orc.bp_matched(vg, sub, y, threads=threads)
    t2 = time.perf_counter()
    updates = 2 * N ** 3 * sub.num_angles
    gups = updates / (t2 - t0) / 1e9
    info = {
        "cores": threads,
        "sample": f"FP + matched BP of {sub.num_angles} of the {ANGLES} angles (every "
        f"{ANGLES // n_angles}th) at full {N}^3 / {DET[0]}x{DET[1]} size; fp64 oracle; "
        f"FP {t1 - t0:.2f} s, BP {t2 - t1:.2f} s; a full {ANGLES}-angle FP + BP step "
        f"extrapolates to {(t2 - t0) * ANGLES / sub.num_angles:.0f} s",
    }
    if keep:
        info["arrays"] = (x, idx, y, bp)
    return gups, info


def _rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def parity_vs_oracle(torch, A, device, arrays):
    """The GPU's full-size operator against the CPU baseline's oracle outputs.

    FP: the sample's angle slices of A(x). BP: A.T of a sinogram holding the
    oracle's FP (as float32) on the sample's angles and zeros on all others.
    Adjointness: <A x, y_s> against <x, A.T y_s>, dot products in float64.
    """
    x, idx, y_ref, bp_ref = arrays
    idx_t = torch.as_tensor(idx, device=device)
    y = A(torch.from_numpy(x).to(device))
    y_gpu = y.index_select(1, idx_t).cpu().numpy()
    ys = torch.zeros(A.range_shape, device=device)
    y_in = y_ref.astype(np.float32)
    ys[:, idx_t] = torch.from_numpy(y_in).to(device)
    bp_gpu = A.T(ys).cpu().numpy()
    lhs = float(np.dot(y_gpu.astype(np.float64).ravel(), y_in.astype(np.float64).ravel()))
    rhs = float(np.dot(x.astype(np.float64).ravel(), bp_gpu.astype(np.float64).ravel()))
    adj = abs(lhs - rhs) / (np.linalg.norm(y_gpu.astype(np.float64)) *
                            np.linalg.norm(y_in.astype(np.float64)))
    del y, ys
    torch.cuda.empty_cache()
    return {"fp_rel_l2": _rel_l2(y_gpu, y_ref), "bp_rel_l2": _rel_l2(bp_gpu, bp_ref),
            "adjoint": adj, "gate": "rel_l2 <= 1e-5, adjoint <= 1e-6",
            "angles": f"{len(idx)} of {ANGLES} (every {ANGLES // len(idx)}th), full-size operator"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from tomosipo_gb300._build import build_oracle

    build_oracle()
    vals = []
    info = None
    # each step one bounded sample: 16 of the 1024 angles (about 3 s on 16
    # cores), 8 when more than 40 steps are asked for
    angles = 16 if args.steps + args.warmup <= 40 else 8
    for _ in range(max(0, args.warmup)):
        cpu_baseline_sample(angles=angles)
    for _ in range(args.steps):
        v, info = cpu_baseline_sample(angles=angles)
        vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference",
        "metric": metric_name(),
        "value": value,
        "unit": "GUPS",
        "n_gpus": 0,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "dtype": "f64",
        "data": "synthetic",
        "config": config({"parallelism": f"replicas x{world}" if world > 1 else "single GPU"}),
        "arm": "reference CPU path: FP64 oracle on the host cores (tomosipo has no CPU "
               "projector; ASTRA not installable offline)",
        "cpu_baseline": {"value": value, "unit": "GUPS", "cores": info["cores"],
                         "kind": "port", "sample": info["sample"]},
        "e2e": {"value": value, "unit": "GUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "vs_baseline": None,
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- GPU arm
def phantom_gpu(torch, device, n, count=8, seed=0):
    """Sum of ``count`` seeded ellipsoids on an n^3 grid (densities U[0.1, 1])."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    ax = torch.linspace(-1, 1, n, device=device)
    x = torch.zeros((n, n, n), device=device)
    for _ in range(count):
        c = (torch.rand(3, generator=g) - 0.5).tolist()
        r = (torch.rand(3, generator=g) * 0.35 + 0.1).tolist()
        rho = float(torch.rand(1, generator=g)) * 0.9 + 0.1
        for z0 in range(0, n, 64):
            zz = ax[z0:z0 + 64, None, None]
            m = (((zz - c[0]) / r[0]) ** 2 + ((ax[None, :, None] - c[1]) / r[1]) ** 2
                 + ((ax[None, None, :] - c[2]) / r[2]) ** 2)
            x[z0:z0 + 64] += rho * (m <= 1)
    return x


def noisy_projection(torch, A, x, seed):
    """y = A(x) + N(0, 0.01 max(A(x))) (seeded)."""
    y = A(x)
    g = torch.Generator(device="cpu").manual_seed(seed)
    return y + 0.01 * float(y.max()) * torch.randn(y.shape, generator=g).to(y.device)


def bench_batched_sirt(torch, ts, device, n_jobs=64, iterations=30, seed=3):
    """64 independent jobs (64^3..256^3, parallel or cone, 60-720 angles, detector
    side x 1.5 side, noisy data): batched SIRT vs looping the plain operator."""
    from tomosipo_gb300.sirt import BatchedSirt, autotune_jobs, sirt

    rng = np.random.default_rng(seed)
    jobs, updates = [], 0
    for i in range(n_jobs):
        n = int(rng.choice([64, 96, 128, 192, 256]))
        cone = bool(rng.random() < 0.5)
        angles = int(rng.integers(60, 721))
        vg = ts.volume(shape=n, size=1)
        pg = (ts.cone(angles=angles, shape=(n, 3 * n // 2), size=np.sqrt(2), cone_angle=0.5) if cone
              else ts.parallel(angles=angles, shape=(n, 3 * n // 2), size=(1, 1.5)))
        A = ts.operator(vg, pg)
        y = noisy_projection(torch, A, phantom_gpu(torch, device, n, seed=seed * 1000 + i), i)
        jobs.append((A, y))
        updates += 2 * n ** 3 * angles * iterations
    torch.cuda.synchronize()
    # forward schedules from the autotuner, one run per job shape (timed apart);
    # both paths below use them
    t0 = time.perf_counter()
    tuning = autotune_jobs([j[0] for j in jobs], device)
    t_tune = time.perf_counter() - t0
    # warm both paths once on the smallest job
    small = min(jobs, key=lambda j: j[1].numel())
    sirt(small[0], small[1], 1)
    BatchedSirt([small]).run(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_each = []
    for A, y in jobs:
        t1 = time.perf_counter()
        sirt(A, y, iterations)
        torch.cuda.synchronize()
        plain_each.append(time.perf_counter() - t1)
    t_plain = time.perf_counter() - t0

    def batched(js):
        t1 = time.perf_counter()
        b = BatchedSirt(js)
        b.run(iterations, graph=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t1
        b.close()
        return dt

    t_batch = batched(jobs)
    # per size class: the small jobs (side <= 128) and the large ones, each
    # batched on its own, against the same jobs' plain-loop times
    classes = {}
    for name, pick in (("side_le_128", lambda A: A.domain_shape[0] <= 128),
                       ("side_gt_128", lambda A: A.domain_shape[0] > 128)):
        idx = [i for i, (A, _) in enumerate(jobs) if pick(A)]
        if not idx:
            continue
        tb = batched([jobs[i] for i in idx])
        tp = sum(plain_each[i] for i in idx)
        classes[name] = {"jobs": len(idx), "batched_s": tb, "plain_loop_s": tp,
                         "solves_per_s": len(idx) / tb, "plain_loop_solves_per_s": len(idx) / tp,
                         "speedup_vs_plain_loop": tp / tb}
    return {
        "config": f"{n_jobs} jobs, sides from {{64,96,128,192,256}}, parallel/cone 50/50, "
                  f"60-720 angles, {iterations} iterations, y = A(x) + N(0, 0.01 max) (seed {seed}); "
                  "forward schedules from the autotuner (one run per job shape, timed apart "
                  "as autotune_s); times include computing R and C",
        "solves_per_s": n_jobs / t_batch,
        "plain_loop_solves_per_s": n_jobs / t_plain,
        "speedup_vs_plain_loop": t_plain / t_batch,
        "batched_s": t_batch,
        "plain_loop_s": t_plain,
        "autotune_s": t_tune,
        "autotuned_shapes": len(tuning),
        "gups": updates / t_batch / 1e9,
        "size_classes": classes,
    }


def bench_general_bp(torch, ts, device, steps, n=256, angles=360, det=(256, 384)):
    """FP + matched BP of a scan whose detector is tilted out of the z axis (a
    cone scan rotated 0.4 rad about (1, 0.3, -0.2)): every angle takes the
    general backprojector (the forward projector is the same kernel as for any
    geometry). Volume n^3, ``angles`` angles, detector ``det``."""
    vg = ts.volume(shape=n, size=1)
    R = ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.4)
    pg = R * ts.cone(angles=angles, shape=det, size=np.sqrt(2), cone_angle=0.5).to_vec()
    A = ts.operator(vg, pg)
    st = A.projector.stats(device.index)
    x = phantom_gpu(torch, device, n, count=8, seed=6)
    y = torch.empty(A.range_shape, device=device)
    v = torch.empty(A.domain_shape, device=device)
    A(x, out=y)
    A.T(y, out=v)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    for e in ev:
        e[0].record()
        A(x, out=y)
        e[1].record()
        A.T(y, out=v)
        e[2].record()
    torch.cuda.synchronize()
    fp = statistics.mean(e[0].elapsed_time(e[1]) for e in ev)
    bp = statistics.mean(e[1].elapsed_time(e[2]) for e in ev)
    # the same backprojection with one thread per voxel (tuning bp_general = 1)
    kernel = A.projector.get_tuning(device.index)["bp_general"]
    A.projector.set_tuning(device.index, bp_general=1)
    v1 = torch.empty_like(v)
    A.T(y, out=v1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        A.T(y, out=v1)
    e1.record()
    torch.cuda.synchronize()
    bp_voxel = e0.elapsed_time(e1) / steps
    A.projector.set_tuning(device.index, bp_general=kernel)
    same = bool(torch.equal(v, v1))
    U = n ** 3 * angles
    peak, _ = measured_peak_hbm()
    return {"config": f"cone {n}^3, {angles} angles, detector {det[0]}x{det[1]}, tilted 0.4 rad "
                      f"about (1, 0.3, -0.2): {st['general_bp_angles']} of {angles} angles on the "
                      "general backprojector",
            "fp_ms": fp, "general_bp_ms": bp,
            "bp_gups": U / (bp / 1e3) / 1e9, "fp_gups": U / (fp / 1e3) / 1e9,
            "bp_roofline_frac": BYTES_PER_UPDATE * U / (bp / 1e3) / 1e9 / peak,
            "bp_kernel": "voxel boxes staging each angle's detector region (bp_general 0)"
                         if kernel == 0 else "one thread per voxel (bp_general 1)",
            "per_voxel_kernel_bp_ms": bp_voxel,
            "per_voxel_kernel_equal": same}


def bench_fdk(torch, ts, device, x, y, steps):
    """FDK reconstruction (tomosipo's ``fdk``: cosine weights, ramp filter on the
    device FFT, bilinear backprojection with FDK weights) of the headline scan's
    sinogram ``y`` of phantom ``x`` (512^3, 1024 angles over 2 pi, 512 x 768)."""
    from tomosipo_gb300.fdk import fdk_backproject, fdk_constants, fdk_filter
    from tomosipo_gb300.projector import create_projector

    vg, pg = workload_geometry(ts)
    proj = create_projector(vg, pg)
    w = fdk_constants(vg, pg)[2]
    out = torch.zeros(tuple(vg.shape), device=device)
    q = fdk_filter(vg, pg, y)
    fdk_backproject(proj, out, q, w, False)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    for e in ev:
        e[0].record()
        q = fdk_filter(vg, pg, y)
        e[1].record()
        fdk_backproject(proj, out, q, w, False)
        e[2].record()
    torch.cuda.synchronize()
    filt = statistics.mean(e[0].elapsed_time(e[1]) for e in ev)
    bp = statistics.mean(e[1].elapsed_time(e[2]) for e in ev)
    U = N ** 3 * ANGLES
    # reconstruction error on the central half cube (cone-beam FDK is exact on
    # the central plane only; the phantom's ellipsoids span the volume)
    c = slice(N // 4, 3 * N // 4)
    err = float(torch.linalg.vector_norm(out[c, c, c] - x[c, c, c]) / torch.linalg.vector_norm(x[c, c, c]))
    return {"config": f"FDK of the {N}^3 / {ANGLES}-angle / {DET[0]}x{DET[1]} cone scan "
                      "(full circle), sinogram in HBM",
            "ms": filt + bp, "filter_ms": filt, "backprojection_ms": bp,
            "backprojection_gups": U / (bp / 1e3) / 1e9,
            "rel_error_central_half_cube": err}


def bench_supersampling(torch, ts, device, steps, n=256, angles=360, det=(256, 384), d=2):
    """Detector supersampling d: FP averages d x d rays per pixel and the matched
    BP is its exact transpose (both on the d-times finer detector), against the
    same operator without supersampling. Cone n^3, ``angles`` angles, ``det``."""
    vg = ts.volume(shape=n, size=1)
    pg = ts.cone(angles=angles, shape=det, size=np.sqrt(2), cone_angle=0.5)
    x = phantom_gpu(torch, device, n, count=8, seed=7)
    out = {}
    for ss in (1, d):
        A = ts.operator(vg, pg, detector_supersampling=ss)
        y = torch.empty(A.range_shape, device=device)
        v = torch.empty(A.domain_shape, device=device)
        A(x, out=y)
        A.T(y, out=v)
        torch.cuda.synchronize()
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
        for e in ev:
            e[0].record()
            A(x, out=y)
            e[1].record()
            A.T(y, out=v)
            e[2].record()
        torch.cuda.synchronize()
        out[ss] = (statistics.mean(e[0].elapsed_time(e[1]) for e in ev),
                   statistics.mean(e[1].elapsed_time(e[2]) for e in ev))
    U = n ** 3 * angles
    return {"config": f"cone {n}^3, {angles} angles, detector {det[0]}x{det[1]}, "
                      f"detector_supersampling={d} ({d}x{d} rays per pixel)",
            "fp_ms": out[d][0], "bp_ms": out[d][1],
            "plain_fp_ms": out[1][0], "plain_bp_ms": out[1][1],
            "gups_per_coarse_update": 2 * U / ((out[d][0] + out[d][1]) / 1e3) / 1e9,
            "gups_per_fine_update": 2 * U * d * d / ((out[d][0] + out[d][1]) / 1e3) / 1e9}


def helical_cone_vec(ts, n, angles, rows, cols, rng, jitter_voxels=0.5):
    """Helical cone_vec around z for an n^3 unit-cube volume: source/detector at
    2 sqrt2 from the axis (the detector through it), detector sqrt2 x sqrt2*cols/rows
    wide, 1.5 turns rising 0.5 per turn, per-angle source and detector jitter
    N(0, jitter_voxels voxel)."""
    turns, pitch, dist = 1.5, 0.5, 2 * np.sqrt(2)
    t = np.linspace(0, 2 * np.pi * turns, angles, endpoint=False)
    rise = pitch * (t / (2 * np.pi) - turns / 2)
    c, s = np.cos(t), np.sin(t)
    vox = 1.0 / n
    src = np.stack([rise, -c * dist, s * dist], 1) + rng.normal(0, jitter_voxels * vox, (angles, 3))
    det = np.stack([rise, 0 * t, 0 * t], 1) + rng.normal(0, jitter_voxels * vox, (angles, 3))
    sv = np.sqrt(2) / rows
    su = np.sqrt(2) * (cols / rows) / cols
    dv = np.stack([np.full(angles, sv), 0 * t, 0 * t], 1)
    du = np.stack([0 * t, s * su, c * su], 1)
    return ts.cone_vec(shape=(rows, cols), src_pos=src, det_pos=det, det_v=dv, det_u=du)


def serving_requests(torch, ts, device, n_requests, rate, iterations, seed):
    """Poisson arrivals (mean ``rate``/s) of SIRT requests on helical cone_vec
    scans: sides from {128, 256, 384, 512}, 256-1024 angles, detector side x
    min(1.5 side, 768), noisy data (seeded). Returns (requests, updates)."""
    from tomosipo_gb300.serving import Request

    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    reqs, updates = [], 0
    for i in range(n_requests):
        n = int(rng.choice([128, 256, 384, 512]))
        angles = int(rng.integers(256, 1025))
        rows, cols = n, min(3 * n // 2, 768)
        pg = helical_cone_vec(ts, n, angles, rows, cols, rng)
        A = ts.operator(ts.volume(shape=n, size=1), pg)
        y = noisy_projection(torch, A, phantom_gpu(torch, device, n, seed=seed * 1000 + i), i)
        reqs.append(Request(i, A, y, iterations, float(arrivals[i])))
        updates += 2 * n ** 3 * angles * iterations
    torch.cuda.synchronize()
    return reqs, updates


def bench_serving(torch, ts, device, n_requests=64, rate=20.0, iterations=20, seed=5,
                  stable_requests=16, stable_load=0.5):
    """Serving loop over Poisson-arrival SIRT requests on helical cone_vec scans.

    First the workload's own arrival rate (20/s, far above what one GPU can
    serve, so a backlog builds and latency is mostly queueing); the completion
    rate under that backlog is the server's capacity. Then a second request
    set arriving at ``stable_load`` x that capacity, where queues stay short."""
    from tomosipo_gb300.serving import SirtServer, latency_stats

    reqs, updates = serving_requests(torch, ts, device, n_requests, rate, iterations, seed)
    server = SirtServer()  # shortest remaining work first (the default)
    t0 = time.perf_counter()
    res = server.run(reqs)
    wall = time.perf_counter() - t0
    st = latency_stats(res)
    del reqs, res
    torch.cuda.empty_cache()
    capacity = st.get("solves_per_s") or 0.0
    stable = None
    if stable_requests and capacity > 0:
        srate = stable_load * capacity
        reqs2, _ = serving_requests(torch, ts, device, stable_requests, srate, iterations, seed + 1)
        st2 = latency_stats(SirtServer().run(reqs2))
        stable = dict(st2, arrival_rate_per_s=srate,
                      note=f"{stable_requests} requests of the same mix arriving at "
                           f"{stable_load} x the measured capacity")
        del reqs2
        torch.cuda.empty_cache()
    return {
        "config": f"{n_requests} requests, Poisson arrivals {rate}/s, sides from "
                  "{128,256,384,512}, 256-1024 angles, helical cone_vec (1.5 turns, pitch 0.5) "
                  f"with N(0, 0.5 voxel) source/detector jitter, detector side x min(1.5 side, 768), "
                  f"{iterations} iterations, admission by free HBM (seed {seed})",
        "n_requests": st.get("n_requests"),
        "completed": st["completed"],
        "p50_latency_s": st.get("p50_s"),
        "p99_latency_s": st.get("p99_s"),
        "queue_p50_s": st.get("queue_p50_s"),
        "queue_p99_s": st.get("queue_p99_s"),
        "service_p50_s": st.get("service_p50_s"),
        "service_p99_s": st.get("service_p99_s"),
        "solves_per_s": st.get("solves_per_s"),
        "offered_rate_per_s": rate,
        "offered_load_vs_capacity": rate / capacity if capacity else None,
        "max_concurrent_jobs": server.max_concurrent,
        "steps": server.steps,
        "gups": updates / wall / 1e9,
        "policy": "srpt: per step a work budget of one iteration of the largest job, least "
                  "remaining work first, several iterations for small jobs",
        "stable_rate": stable,
    }


def bench_lpd(torch, ts, device, batch=8, n=128, angles=128, iterations=10, channels=32,
              steps=3, warmup=2):
    """One training step (forward, backward, SGD update) of the unrolled learned
    primal-dual: cone 128^3, 128 angles, detector 128 x 192, bf16 convolutions,
    fp32 projector, iterations recomputed (checkpointed) in the backward pass."""
    from tomosipo_gb300.lpd import LearnedPrimalDual3d

    vg = ts.volume(shape=n, size=1)
    pg = ts.cone(angles=angles, shape=(n, 3 * n // 2), size=np.sqrt(2), cone_angle=0.5)
    A = ts.operator(vg, pg)
    torch.manual_seed(0)
    net = LearnedPrimalDual3d(A, n_iters=iterations, channels=channels).to(device)
    opt = torch.optim.SGD(net.parameters(), lr=1e-4)
    x = torch.stack([phantom_gpu(torch, device, n, count=8, seed=40 + i) for i in range(batch)])[:, None]
    g = torch.stack([A(x[i, 0]) for i in range(batch)])[:, None]

    def step():
        opt.zero_grad(set_to_none=True)
        loss = (net(g) - x).square().mean()
        loss.backward()
        opt.step()
        return loss

    # cuDNN picks each 3D convolution's algorithm by timing the candidates on
    # the first call of each shape (the warm-up steps); restored afterwards
    bench_mode = torch.backends.cudnn.benchmark
    torch.backends.cudnn.benchmark = True
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        loss = step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    torch.backends.cudnn.benchmark = bench_mode
    # projector work per step: forward 2 x (FP + BP) per iteration (recomputed),
    # backward one BP and one FP per iteration, each over the batch
    updates = iterations * 3 * 2 * batch * n ** 3 * angles
    # The projector's own time: the batched FP and BP calls the network makes
    # (one call over the batch each), timed alone on the same operator and shapes.
    xb = x.detach().reshape(batch, n, n, n).contiguous()
    yb = torch.empty((batch, *A.range_shape), device=device)
    vb = torch.empty_like(xb)
    A._apply_batch(xb, yb)
    A.T._apply_batch(yb, vb)
    torch.cuda.synchronize()
    pe = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    reps = 5
    pe[0].record()
    for _ in range(reps):
        A._apply_batch(xb, yb)
    pe[1].record()
    for _ in range(reps):
        A.T._apply_batch(yb, vb)
    pe[2].record()
    torch.cuda.synchronize()
    fp_call_ms = pe[0].elapsed_time(pe[1]) / reps
    bp_call_ms = pe[1].elapsed_time(pe[2]) / reps
    proj_ms = iterations * 3 * (fp_call_ms + bp_call_ms)
    return {
        "config": f"batch {batch}, cone {n}^3, {angles} angles, detector {n}x{3 * n // 2}, "
                  f"{iterations} unrolled iterations, 3-layer 3D CNN with {channels} channels, "
                  "bf16 convolutions, fp32 projector, checkpointed iterations, SGD step",
        "ms_per_step": ms,
        "samples_per_s": batch * 1e3 / ms,
        "projector_gups_in_step": updates / (ms / 1e3) / 1e9,
        "projector_gups_in_step_note": "projector updates per step / whole training step time "
                                       "(convolutions included)",
        "projector_fp_batch_ms": fp_call_ms,
        "projector_bp_batch_ms": bp_call_ms,
        "projector_ms_per_step": proj_ms,
        "projector_share_of_step": proj_ms / ms,
        "projector_gups": updates / (proj_ms / 1e3) / 1e9,
        "projector_note": f"one batched FP and one batched BP call over the {batch} slices, timed "
                          f"alone ({reps} calls each); {3 * iterations} of each per step",
        "peak_mem_gb": torch.cuda.max_memory_allocated(device) / 1e9,
        "loss": float(loss.detach()),
    }


def bench_bilinear_pair(torch, ts, device, x, steps):
    """FP + the bilinear (ASTRA-style) BP on the headline workload."""
    vg, pg = workload_geometry(ts)
    A = ts.operator(vg, pg, backprojector="bilinear")
    y = torch.empty(A.range_shape, device=device)
    v = torch.empty(A.domain_shape, device=device)
    A(x, out=y)
    A.T(y, out=v)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    for e in ev:
        e[0].record()
        A(x, out=y)
        e[1].record()
        A.T(y, out=v)
        e[2].record()
    torch.cuda.synchronize()
    fp = statistics.mean(e[0].elapsed_time(e[1]) for e in ev)
    bp = statistics.mean(e[1].elapsed_time(e[2]) for e in ev)
    return {"fp_ms": fp, "bp_bilinear_ms": bp,
            "gups": 2 * N ** 3 * ANGLES / ((fp + bp) / 1e3) / 1e9}


def max_over_ranks(value, world, device=None):
    """The largest of every rank's value (the slowest rank's time); the value
    itself for one rank. Works over NCCL (CUDA device) and gloo (CPU)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gups(world, updates_per_rank_step, steps, seconds):
    """GUPS of the whole job: every rank's updates over the slowest rank's time."""
    return world * updates_per_rank_step * steps / seconds / 1e9


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    import __graft_entry__

    __graft_entry__.build()
    import tomosipo_gb300 as ts

    device = torch.device("cuda", local_rank)
    torch.cuda.set_device(device)
    vg, pg = workload_geometry(ts)
    A = ts.operator(vg, pg)
    if args.fp_copies != "auto":
        A.projector.set_tuning(device.index, fp_pair_layout=int(args.fp_copies == "pairs"))
    if args.bp_kernel != "auto":
        A.projector.set_tuning(device.index, bp_kernel=int(args.bp_kernel == "zlane"))
    x = phantom_gpu(torch, device, N, count=20, seed=2)
    y = torch.empty(A.range_shape, device=device)
    v = torch.empty(A.domain_shape, device=device)
    stats = A.projector.stats(device.index)
    U = N ** 3 * ANGLES

    def barrier():
        if world > 1:
            dist.barrier()

    def step():
        A(x, out=y)
        A.T(y, out=v)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream(device)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    clocks = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        A(x, out=y)
        ev[i][1].record(stream)
        A.T(y, out=v)
        ev[i][2].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    clock_info = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    fp_ms = [e[0].elapsed_time(e[1]) for e in ev]
    bp_ms = [e[1].elapsed_time(e[2]) for e in ev]

    total_ms = max_over_ranks(total_ms, world, device)
    ms_per_step = total_ms / args.steps
    value = whole_job_gups(world, 2 * U, args.steps, total_ms / 1e3)

    # End to end through the public API with page-locked host buffers
    # (ts.host_buffer: huge-page backed, so DMA keeps its rate on a host that
    # other processes have used): every step copies the volume in, projects,
    # copies the sinogram out, copies it back in, backprojects and copies the
    # volume out (A(x_host), A.T(y_host)).
    e2e = None
    if not args.no_e2e:
        xh = ts.host_buffer(A.domain_shape)
        xh.copy_(x.cpu())
        yh = ts.host_buffer(A.range_shape)
        vh = ts.host_buffer(A.domain_shape)
        for _ in range(max(1, args.warmup)):
            A(xh, out=yh)
            A.T(yh, out=vh)
        torch.cuda.synchronize()
        # the host's own copy rate just before the timed leg: one plain upload
        # and download of the volume buffer (0.54 GB each), so a slow end-to-end
        # number can be told apart from a pipeline that fails to hide copies
        xd = torch.empty_like(x)
        cev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        cev[0].record(stream)
        xd.copy_(xh, non_blocking=True)
        cev[1].record(stream)
        vh.copy_(xd, non_blocking=True)
        cev[2].record(stream)
        torch.cuda.synchronize()
        vol_gb = 4 * N ** 3 / 1e9
        copy_rate = {"h2d_gbs": round(vol_gb / (cev[0].elapsed_time(cev[1]) / 1e3), 1),
                     "d2h_gbs": round(vol_gb / (cev[1].elapsed_time(cev[2]) / 1e3), 1),
                     "what": "one plain copy of the volume buffer each way before the timed leg "
                             "(full rate on this host type: about 210 up, 192 down)"}
        del xd
        barrier()
        from tomosipo_gb300.projector import TransferTimeline, record_transfers

        timeline = TransferTimeline()
        t0 = time.perf_counter()
        calls = []  # both calls return with their results on the host
        with record_transfers(timeline):
            for _ in range(args.steps):
                ta = time.perf_counter()
                A(xh, out=yh)
                tb = time.perf_counter()
                A.T(yh, out=vh)
                calls.append((tb - ta, time.perf_counter() - tb))
        torch.cuda.synchronize()
        dt = max_over_ranks(time.perf_counter() - t0, world, device)
        barrier()
        spans = {k: v / args.steps for k, v in timeline.summary().items()}
        breakdown = {f"{k}_ms": round(v, 3) for k, v in sorted(spans.items())}
        # device time of each leg not covered by its kernels: the transfers
        # (and gaps) the chunked pipeline leaves exposed
        breakdown["fp_exposed_ms"] = round(spans.get("fp_leg", 0) - spans.get("fp", 0), 3)
        breakdown["bp_exposed_ms"] = round(spans.get("bp_leg", 0) - spans.get("bp", 0), 3)
        vol_b = 4 * N ** 3
        sino_b = 4 * DET[0] * DET[1] * ANGLES
        e2e = {
            "value": whole_job_gups(world, 2 * U, args.steps, dt),
            "unit": "GUPS",
            "h2d_bytes_per_step": vol_b + sino_b,
            "d2h_bytes_per_step": sino_b + vol_b,
            "ms_per_step": 1e3 * dt / args.steps,
            "fp_ms": 1e3 * statistics.median(c[0] for c in calls),
            "bp_ms": 1e3 * statistics.median(c[1] for c in calls),
            "per_step_device_ms": breakdown,
            "host_copy_rate": copy_rate,
            "path": "ts.operator A(x_host)->y_host, A.T(y_host)->x_host, page-locked huge-page host buffers (ts.host_buffer)",
        }

    if rank != 0:
        return 0

    peak, peak_kind = measured_peak_hbm()
    bp_avg = statistics.mean(bp_ms) / 1e3
    fp_avg = statistics.mean(fp_ms) / 1e3
    bp_kernel = A.projector.get_tuning(device.index)["bp_kernel"]
    bp_name = ("bp_matched (column-major weight pass + z-lane gather + transpose)" if bp_kernel
               else "bp_matched (weight pass + voxel-pair gather)")
    dom_name, dom_t, dom_key = (bp_name, bp_avg, f"bp_matched_kernel{bp_kernel}_bytes_per_call")
    if fp_avg > bp_avg:
        dom_name, dom_t, dom_key = ("fp (layout copies + ray kernel)", fp_avg, "fp_bytes_per_call")
    achieved = BYTES_PER_UPDATE * U / dom_t / 1e9
    # DRAM bytes per call of the dominant kernels, from the committed summary of
    # a one-pass ncu capture (gpu__time_duration, dram__bytes_read/write) of
    # this same workload; other workloads have none.
    traffic = traffic_source = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if (N, ANGLES) == (512, 1024) and os.path.exists(tpath):
        try:
            with open(tpath) as f:
                tj = json.load(f)
            traffic = tj.get(dom_key)
            traffic_source = tj.get("source") if traffic is not None else None
        except (OSError, ValueError):
            traffic = None
    batched = serving = lpd = bilinear = general = fdk = supersampling = None
    if not args.no_bilinear:
        bilinear = bench_bilinear_pair(torch, ts, device, x, args.steps)
        general = bench_general_bp(torch, ts, device, args.steps)
        fdk = bench_fdk(torch, ts, device, x, y, min(args.steps, 5))
        supersampling = bench_supersampling(torch, ts, device, min(args.steps, 5))
    if not args.no_lpd:
        lpd = bench_lpd(torch, ts, device)
    if not args.no_sirt:
        batched = bench_batched_sirt(torch, ts, device, n_jobs=args.sirt_jobs)
        serving = bench_serving(torch, ts, device, n_requests=args.serve_requests,
                                stable_requests=args.serve_stable_requests)
    cpu = parity = None
    if world == 1 and not args.no_cpu_baseline:
        gups, info = cpu_baseline_sample(keep=True)
        cpu = {"value": gups, "unit": "GUPS", "cores": info["cores"], "kind": "port",
               "sample": info["sample"]}
        parity = parity_vs_oracle(torch, A, device, info.pop("arrays"))
    line = {
        "metric": metric_name(),
        "value": value,
        "unit": "GUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": config(dict({"parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
                              **({"fp_copies": args.fp_copies} if args.fp_copies != "auto" else {}),
                              **({"bp_kernel": args.bp_kernel} if args.bp_kernel != "auto" else {}))),
        "fp_ms": statistics.mean(fp_ms),
        "bp_ms": statistics.mean(bp_ms),
        "roofline": {
            "bound": "hbm",
            "kernel": dom_name,
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_kind": peak_kind,
            "traffic": traffic,
            "traffic_source": traffic_source,
            "algorithmic_bytes": f"{BYTES_PER_UPDATE} B per voxel-angle update x {N}^3 x {ANGLES}",
            "step_frac": BYTES_PER_UPDATE * value * 1e9 / world / peak / 1e9,
        },
        "cpu_baseline": cpu,
        "parity": parity,
        "e2e": e2e,
        "batched_sirt": batched,
        "serving": serving,
        "learned_primal_dual": lpd,
        "fp_plus_bilinear_bp": bilinear,
        "tilted_detector_general_bp": general,
        "fdk": fdk,
        "detector_supersampling": supersampling,
        "gpu_launches": args.steps * (stats["fp_launches"] + stats["bp_matched_launches"]),
        "clocks": clock_info,
        "plan": stats,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-sirt", action="store_true", help="skip the batched SIRT and serving parts")
    p.add_argument("--no-lpd", action="store_true", help="skip the learned primal-dual step")
    p.add_argument("--no-bilinear", action="store_true",
                   help="skip the FP + bilinear BP pair, the tilted-detector, FDK and "
                   "detector-supersampling timings")
    p.add_argument("--sirt-jobs", type=int, default=64)
    p.add_argument("--serve-requests", type=int, default=64)
    p.add_argument("--serve-stable-requests", type=int, default=16)
    p.add_argument("--workload", choices=sorted(WORKLOADS), default="headline",
                   help="headline = the metric's 512^3/1024 workload; c2 = 256^3/360 and "
                   "cone512_64 = 512^3/64 (profiling)")
    p.add_argument("--fp-copies", choices=["auto", "single", "pairs"], default="auto",
                   help="forward projector's volume copies (tuning fp_pair_layout; auto = the "
                   "projector's default): to profile the headline's single-voxel copies on "
                   "the c2 workload")
    p.add_argument("--bp-kernel", choices=["auto", "pairs", "zlane"], default="auto",
                   help="matched backprojector (tuning bp_kernel; auto = the projector's default: "
                   "z-lane warps from 448 voxels along z): to profile the voxel-pair kernel")
    args = p.parse_args()
    global N, ANGLES, DET
    N, ANGLES, DET = WORKLOADS[args.workload]
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        return run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
