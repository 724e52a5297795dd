"""Benchmark: 3D type-1 NUFFT throughput (NU pts/s) at tol 1e-5, FP32.

Workload (the metric's configuration): N = 256^3 modes, M = 1e8 points drawn
80% from 8 isotropic Gaussians (sigma 0.3, centres uniform in [-pi,pi)^3,
wrapped periodically) and 20% uniform, complex64 strengths N(0,1), iflag +1.
Synthetic, seeded inputs of those shapes stand in for user data.

A step is one execute of the planned transform on resident device inputs
(spread -> FFT -> deconvolve), timed with CUDA events on the plan's stream.
``value`` is the planned+batched form (ntransf strength vectors sharing the
points, one CUDA-graph replay per step). Beside it:
  * ``plain``: one transform planned by the reference library's heuristic
    (planner 1: its bin sizes, method, subproblem size and ES kernel), no
    batching, no graph -- the plain GPU form;
  * ``plain_engine``: one transform with this engine's own planning;
  * ``e2e``: the batched transform through the host-pointer C ABI
    (finufftf_execute) with pinned host buffers, copies inside the timed region;
  * ``accuracy``: relative l2 error on 1e3 sampled modes (a seeded 10x10x10
    grid of mode indices) against an FP64 direct sum, for the engine and for
    the CPU restatement of FINUFFT on the same inputs at the same tol;
  * ``cpu_baseline``: that CPU restatement (OpenMP, all host cores) timed on
    the full workload (the 4 vectors over all 1e8 points);
  * ``configs``: the other workloads (C1 1D FP64, C2 2D type 2 x16, C4 4096
    uneven 2D problems, C5 3D type 3, C3 in FP64 at tol 1e-12), each with its
    throughput, its error on sampled outputs against FP64 direct sums, the CPU
    restatement's error on the same inputs and the ratio of the two.
Inputs (800 MB of strengths per vector, a 1 GB fine grid per vector) exceed
the 129 MB L2, so no flush is needed.

--impl reference times the CPU restatement of FINUFFT's algorithm (the oracle
port, PSWF kernel, OpenMP spreading + threaded FFT) on the host cores: each
step is the full workload, the 4 strength vectors over all 1e8 points. Under torchrun
each rank runs an independent replica (the transform does not shard); value
sums the replicas.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_MODES = (256, 256, 256)
M_FULL = 100_000_000
TOL = 1e-5
METRIC = "3D type-1 NU pts/s @tol 1e-5: planned+batched vs plain GPU vs CPU FINUFFT"
WORKLOAD = ("3D type 1, 256^3 modes, M=1e8 clustered (8 Gaussians sigma 0.3 + 20% uniform), "
            "complex64, tol 1e-5, iflag +1")


def clustered_points(M, seed, rng_dev="cpu"):
    """80% from 8 Gaussians (sigma 0.3, wrapped) + 20% uniform on [-pi,pi)^3."""
    import torch

    g = torch.Generator(device=rng_dev).manual_seed(seed)
    dev = torch.device(rng_dev)
    ncl = int(0.8 * M)
    centres = (torch.rand(8, 3, generator=g, device=dev, dtype=torch.float64) * 2 - 1) * np.pi
    which = torch.randint(0, 8, (ncl,), generator=g, device=dev)
    pts = torch.empty(3, M, dtype=torch.float32, device=dev)
    cl = centres[which].T + 0.3 * torch.randn(3, ncl, generator=g, device=dev, dtype=torch.float64)
    cl = torch.remainder(cl + np.pi, 2 * np.pi) - np.pi
    pts[:, :ncl] = cl.to(torch.float32)
    pts[:, ncl:] = ((torch.rand(3, M - ncl, generator=g, device=dev, dtype=torch.float64) * 2 - 1)
                    * np.pi).to(torch.float32)
    return pts


def strengths(n, M, seed, dev, dtype=None):
    import torch

    dtype = dtype or torch.float32
    g = torch.Generator(device=dev).manual_seed(seed)
    z = torch.randn(n, M, 2, generator=g, device=dev, dtype=dtype)
    return z.view(torch.complex64 if dtype == torch.float32 else torch.complex128)[..., 0]


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_over_ranks(ms, world, device):
    """per-rank step times -> the slowest rank's (MAX over ranks; identity at N=1)"""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_value(units_per_rank, world, ms):
    """whole-job throughput: every rank processes units_per_rank per step (replicas)"""
    return world * units_per_rank / (ms * 1e-3)


def time_steps(fn, stream, steps, warmup):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps  # ms per step


# fallback denominators where MEASURED_PEAKS.json is absent: one earlier
# measurement on a GB300 (STREAM-style copy; cuBLAS bf16 burst)
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def measured_peak(key):
    """(peak, source): from MEASURED_PEAKS.json at the repository root, else the
    fallback figure"""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key]), "MEASURED_PEAKS.json %s (of measured)" % key
    except (OSError, KeyError, ValueError, TypeError):
        return FALLBACK_PEAKS.get(key), "fallback %s (no MEASURED_PEAKS.json)" % key


# DRAM bytes (read + write) per point per transform of the default 3D spread
# kernel (int32 fixed-point tile), from the ncu capture at the same point
# density (1.25e7 clustered points on a 256^3 grid: 987 MB read + 141 MB
# written); scaled by points and transforms to one launch of this workload
SPREAD_DRAM_BYTES_PER_POINT = (987e6 + 141e6) / 12.5e6


# ------------------------------------------------------------------ accuracy ----
def sample_axes(n_modes, per_axis, seed):
    """seeded mode indices per array axis (row-major): their product grid is the
    sample (per_axis ** dim modes)"""
    g = np.random.default_rng(seed)
    return [np.sort(g.choice(n, size=min(per_axis, n), replace=False)) for n in n_modes]


def direct_type1_grid(coords, c, n_modes, axes_idx, isign, dev, chunk=1 << 20):
    """FP64 direct type-1 sums f[k] = sum_j c_j exp(i isign k.x_j) on the
    product grid of the given per-axis mode indices (modes k = idx - n//2;
    coords[a] pairs with array axis a), on the GPU: the exponential separates
    over axes, so each chunk of points is one complex GEMM."""
    import torch

    dim = len(n_modes)
    ks = [torch.tensor(idx - n // 2, dtype=torch.float64, device=dev)
          for idx, n in zip(axes_idx, n_modes)]
    L = [len(k) for k in ks]
    out = torch.zeros(int(np.prod(L)), dtype=torch.complex128, device=dev)
    M = coords[0].numel()
    for j0 in range(0, M, chunk):
        j1 = min(M, j0 + chunk)
        E = [torch.polar(torch.ones(1, dtype=torch.float64, device=dev),
                         isign * ks[a][:, None] * coords[a][j0:j1].to(torch.float64)[None, :])
             for a in range(dim)]
        w = c[j0:j1].to(torch.complex128)
        if dim == 1:
            out += E[0] @ w
        elif dim == 2:
            out += (E[0] @ (E[1] * w[None, :]).T).reshape(-1)
        else:
            P = (E[1][:, None, :] * (E[2] * w[None, :])[None, :, :]).reshape(L[1] * L[2], -1)
            out += (E[0] @ P.T).reshape(-1)
    return out.reshape(L)


def take_grid(f, axes_idx):
    """f restricted to the product grid of per-axis indices"""
    import torch

    if isinstance(f, np.ndarray):
        return f[np.ix_(*axes_idx)]
    idx = [torch.as_tensor(a, device=f.device) for a in axes_idx]
    for a, ix in enumerate(idx):
        f = f.index_select(a, ix)
    return f


def cpu_model():
    """the host CPU's model name and logical core count (lscpu; /proc/cpuinfo
    when lscpu is missing)"""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if name is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    name = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"model": name, "logical_cores": os.cpu_count()}


def rel_l2(a, b):
    import torch

    a = torch.as_tensor(a).to(torch.complex128).reshape(-1).cpu()
    b = torch.as_tensor(b).to(torch.complex128).reshape(-1).cpu()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def acc_entry(gpu_err, cpu_err, sample):
    return {"gpu_rel_l2": gpu_err, "cpu_rel_l2": cpu_err,
            "ratio_gpu_over_cpu": (gpu_err / cpu_err) if cpu_err else None, "sample": sample}


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    return O


def cpu_type1_3d(pts_np, c_np, tol, dtype):
    """CPU restatement (oracle port of FINUFFT's CPU algorithm, PSWF kernel,
    OpenMP) of the metric transform on the strength vectors c_np[k] sharing the
    points: (modes array of vector 0, setpts s, execute s of all vectors, threads)."""
    O = _oracle()
    c_np = np.atleast_2d(c_np)
    plan = O.CpuPlan(1, list(N_MODES[::-1]), +1, tol, dtype=dtype)
    t0 = time.perf_counter()
    plan.setpts([pts_np[2], pts_np[1], pts_np[0]])  # fastest axis first
    t1 = time.perf_counter()
    f0 = None
    for k in range(c_np.shape[0]):
        f = plan.execute(c_np[k])
        f0 = f if f0 is None else f0
    t2 = time.perf_counter()
    return f0, t1 - t0, t2 - t1, plan.threads


# --------------------------------------------------------------- metric (C3) ----
def run_gpu(args):
    import torch
    import torch.distributed as dist

    import finufft_gb300 as fg

    global N_MODES
    rank, world, local = dist_info()
    if args.nmodes:
        N_MODES = (args.nmodes,) * 3
    plan_kw = {}
    if args.variant >= 0:
        plan_kw["spread_variant"] = args.variant
    plan_kw["planner"] = args.planner
    if args.bins:
        bx, by, bz = (int(v) for v in args.bins.split(","))
        plan_kw.update(gpu_binsizex=bx, gpu_binsizey=by, gpu_binsizez=bz)
    if args.maxsub:
        plan_kw["gpu_maxsubprobsize"] = args.maxsub
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    M = args.m
    pts = clustered_points(M, 1234 + 3 + rank, rng_dev="cuda").to(dev)
    x, y, z = pts[0].contiguous(), pts[1].contiguous(), pts[2].contiguous()
    nt = args.ntransf
    c = strengths(nt, M, 99 + rank, dev)
    stream = torch.cuda.Stream(device=dev)
    c0 = c[0].contiguous()

    def single(kw):
        p = fg.Plan(1, N_MODES, n_trans=1, eps=TOL, dtype="complex64",
                    gpu_stream=stream.cuda_stream, **kw)
        t0 = time.perf_counter()
        p.setpts(x, y, z)
        torch.cuda.synchronize()
        ts = time.perf_counter() - t0
        f = torch.empty(N_MODES, dtype=torch.complex64, device=dev)
        ms = time_steps(lambda: p.execute(c0, out=f), stream, args.steps, args.warmup)
        p.stage_times(True)
        p.execute(c0, out=f)
        torch.cuda.synchronize()
        st = p.stage_times(True)
        info = p.info()
        del p
        torch.cuda.empty_cache()
        return ms, st, info, ts, f

    # plain GPU form: one transform, the reference library's heuristic planning
    plain_kw = dict(plan_kw)
    plain_kw["planner"] = 1
    if args.only == "batched":
        ms_plain = st_plain = info_plain = f_plain = None
    else:
        ms_plain, st_plain, info_plain, _, f_plain = single(plain_kw)
    if args.only == "plain":
        print(json.dumps({"plain_ms": ms_plain, "stage_ms": st_plain, "M": M,
                          "nsub": info_plain.nsub, "bins": list(info_plain.bins)}))
        return
    # this engine's fixed default planning (planner 0), one transform
    eng_kw = dict(plan_kw)
    eng_kw["planner"] = 0
    if args.only != "batched":
        ms_eng, st_eng, info_eng, setpts_s, f_eng = single(eng_kw)
    if args.only == "engine":
        print(json.dumps({"engine_ms": ms_eng, "stage_ms": st_eng, "M": M,
                          "nsub": info_eng.nsub, "bins": list(info_eng.bins)}))
        return

    # planned + batched form: nt vectors sharing the points, graph replay
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bplan = fg.Plan(1, N_MODES, n_trans=nt, eps=TOL, dtype="complex64",
                    gpu_stream=stream.cuda_stream, gpu_maxbatchsize=nt, **plan_kw)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    bplan.setpts(x, y, z)
    torch.cuda.synchronize()
    makeplan_s, bsetpts_s = t1 - t0, time.perf_counter() - t1
    fkb = torch.empty((nt,) + N_MODES, dtype=torch.complex64, device=dev)
    bplan.execute(c, out=fkb)
    torch.cuda.synchronize()
    bplan.graph_capture(c, fkb)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms_batched = time_steps(bplan.graph_launch, stream, args.steps, args.warmup)
    bplan.stage_times(True)
    bplan.execute(c, out=fkb)
    torch.cuda.synchronize()
    stb = bplan.stage_times(True)
    binfo = bplan.info()
    if args.only == "batched":
        print(json.dumps({"batched_ms": ms_batched, "stage_ms": stb, "M": M, "ntransf": nt,
                          "nsub": binfo.nsub, "bins": list(binfo.bins)}))
        return

    # e2e through the reference-facing host-pointer C ABI (finufftf_makeplan /
    # setpts / execute) with pinned host arrays: every step copies the nt strength
    # vectors in and the nt mode arrays out, pipelined over the plan's batches
    # (the call is synchronous: wall clock around it)
    import ctypes

    from finufft_gb300 import _lib

    lib = _lib.load()
    fo = _lib.FinufftOpts()
    lib.finufft_default_opts(ctypes.byref(fo))
    hplan = ctypes.c_void_p()
    hm = (ctypes.c_int64 * 3)(*reversed(N_MODES))
    assert lib.finufftf_makeplan(1, 3, hm, 1, nt, TOL, ctypes.byref(hplan), ctypes.byref(fo)) == 0
    # C order: the fastest mode axis (last array axis) pairs with the first coordinate
    hx, hy, hz = (a.cpu().numpy() for a in (x, y, z))
    assert lib.finufftf_setpts(hplan, M, hz.ctypes.data, hy.ctypes.data, hx.ctypes.data, 0,
                               None, None, None) == 0
    hc = torch.empty((nt, M), dtype=torch.complex64, pin_memory=True)
    hc.copy_(c.cpu())
    hf = torch.empty((nt,) + N_MODES, dtype=torch.complex64, pin_memory=True)

    def e2e_step():
        assert lib.finufftf_execute(hplan, hc.data_ptr(), hf.data_ptr()) == 0

    for _ in range(2):
        e2e_step()
    # each step timed on its own (wall clock around the synchronous call); the
    # value is the mean over the steps
    n_e2e = max(1, args.steps)
    e2e_ms = []
    for _ in range(n_e2e):
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    ms_e2e = float(np.mean(e2e_ms))
    e2e_err = float(torch.linalg.norm(hf[0].to(dev) - fkb[0]) / torch.linalg.norm(fkb[0]))
    lib.finufftf_destroy(hplan)
    del hc, hf

    # the reference cuFINUFFT compiled for this GPU, same inputs, default options
    ref_gpu = reference_gpu_type1(x, y, z, c, nt, stream, args, dev)

    # roofline of the dominant kernel (spread): shared-memory adds
    ns = binfo.ns
    atom_per_launch = float(M) * nt * 2 * ns ** 3
    spread_ms = stb[0]
    achieved = atom_per_launch / (spread_ms * 1e-3)
    # peak: the measured rate of the shared-memory add the kernel issues (native
    # int32 for the fixed-point tile, else the f32 compare-and-swap loop)
    fixed = bool(getattr(binfo, "spread_fixed", 0))
    peak = fg.smem_atomic_peak(dev.index, i32=fixed)
    kname = {0: "spread_tile3_kernel", 1: "spread_tile3w_kernel", 2: "spread_tile3m_kernel",
             3: "spread_tile3v_kernel"}.get(binfo.spread_variant, "spread_global_kernel")
    # algorithmic HBM bytes of one spread launch (nt transforms): coordinates and
    # strengths read once (3*4 + 2*4 B per point per transform), fine grid written
    nf_cells = int(np.prod(list(binfo.nf)))
    hbm_bytes = float(M) * (12 + 8 * nt) + nf_cells * 8.0 * nt
    hbm_ach = hbm_bytes / (spread_ms * 1e-3)
    hbm_peak, hbm_src = measured_peak("hbm_gbs")
    traffic = SPREAD_DRAM_BYTES_PER_POINT * M * nt if kname == "spread_tile3v_kernel" else None

    ms_batched, ms_plain, ms_e2e = reduce_over_ranks([ms_batched, ms_plain, ms_e2e], world, dev)
    if rank != 0:
        dist.barrier() if world > 1 else None
        return

    # accuracy: 1e3 sampled modes against an FP64 direct sum, and the CPU
    # restatement of FINUFFT (same inputs, same tol), which is also the timed
    # CPU baseline (one execute of one vector over all points)
    ax = sample_axes(N_MODES, 10, 5)
    ref = direct_type1_grid([x, y, z], c0, N_MODES, ax, +1, dev)
    acc = {"batched": rel_l2(take_grid(fkb[0], ax), ref),
           "plain": rel_l2(take_grid(f_plain, ax), ref),
           "plain_engine": rel_l2(take_grid(f_eng, ax), ref)}
    del f_plain, f_eng
    cpu_line = None
    if not args.no_cpu and world == 1:
        del bplan
        torch.cuda.empty_cache()
        f_cpu, cs, ce, thr = cpu_type1_3d(np.stack([hx, hy, hz]), c.cpu().numpy(), TOL,
                                          np.complex64)
        acc["cpu"] = rel_l2(take_grid(f_cpu, ax), ref)
        cpu_line = {"value": M * nt / ce, "unit": "NU pts/s", "cores": thr, "kind": "port",
                    "sample": "the full metric workload: one execute (spread, FFT, "
                              "deconvolution) of the %d strength vectors over all %d points, "
                              "timed in full (%.2f s; setpts sort %.2f s outside)"
                              % (nt, M, ce, cs),
                    "execute_s": ce, "setpts_s": cs, "host": cpu_model()}
    value = job_value(M * nt, world, ms_batched)
    out = {
        "metric": METRIC, "value": value, "unit": "NU pts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batched,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clustered points, N(0,1) strengths)",
        "config": {"workload": WORKLOAD, "ntransf_batched": nt, "M": M, "N": list(N_MODES),
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas",
                   "ns": ns, "nf": list(binfo.nf), "bins": list(binfo.bins),
                   "nsub": binfo.nsub, "kernel": "PSWF" if binfo.kernel_form == 2 else "ES",
                   "planner": {0: "engine default", 1: "reference heuristic", 2: "learned",
                               3: "autotuned"}.get(args.planner),
                   "planner_used": binfo.planner_used, "planned_slot": binfo.planned_slot,
                   "upsampfac": binfo.upsampfac, "spread_variant": binfo.spread_variant,
                   "maxsubprobsize": binfo.maxsubprobsize},
        "plain": {"value": job_value(M, world, ms_plain), "ms_per_step": ms_plain,
                  "planner": "reference heuristic (cuFINUFFT 2.6: ES kernel, method 2, "
                             "bins from the shared-memory budget, 1024-point subproblems)",
                  "stage_ms": {"spread": st_plain[0], "fft": st_plain[1], "deconv": st_plain[2]},
                  "bins": list(info_plain.bins), "spread_variant": info_plain.spread_variant},
        "value_over_plain": ms_plain * nt / ms_batched,
        "plain_engine": {"value": job_value(M, world, ms_eng), "ms_per_step": ms_eng,
                         "stage_ms": {"spread": st_eng[0], "fft": st_eng[1], "deconv": st_eng[2]}},
        "batched_stage_ms": {"spread": stb[0], "fft": stb[1], "deconv": stb[2]},
        "setpts_s": setpts_s,
        # the reference perftest's amortized figure (perftest/cuda/cuperftest.cu:401):
        # points over makeplan + setpts + one execute, batched plan
        "amortized": {"value": job_value(M * nt, world, (makeplan_s + bsetpts_s) * 1e3 + ms_batched),
                      "unit": "NU pts/s", "makeplan_s": makeplan_s, "setpts_s": bsetpts_s},
        "accuracy": {"rel_l2_vs_fp64_direct": acc,
                     "sample": "1e3 modes: seeded 10x10x10 grid of mode indices, vector 0",
                     "ratio_batched_over_cpu": (acc["batched"] / acc["cpu"]) if "cpu" in acc else None},
        "reference_gpu": ref_gpu,
        "e2e": {"value": job_value(M * nt, world, ms_e2e), "unit": "NU pts/s",
                "h2d_bytes_per_step": nt * M * 8, "d2h_bytes_per_step": nt * int(np.prod(N_MODES)) * 8,
                "api": "finufftf_execute (host pointers, pinned)", "rel_diff_vs_device_api": e2e_err,
                "steps": n_e2e, "step_ms": {"mean": ms_e2e, "median": float(np.median(e2e_ms)),
                                            "min": float(np.min(e2e_ms)),
                                            "max": float(np.max(e2e_ms))}},
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "smem_atomic", "achieved": achieved / 1e9,
                     "peak": (peak / 1e9) if peak else None,
                     "unit": "G shared-memory adds/s (achieved: 2*ns^3 updates per point)",
                     "frac": (achieved / peak) if peak else None, "traffic": traffic,
                     "kernel": kname, "per_launch": atom_per_launch,
                     "tile": "int32 fixed point" if fixed else "f32",
                     "peak_source": ("measured by gbnufft_smem_atomic_rate_i32 on this GPU" if fixed
                                     else "measured by gbnufft_smem_atomic_rate on this GPU")},
        "roofline_hbm": {"bound": "hbm", "achieved": hbm_ach / 1e9, "peak": hbm_peak,
                         "unit": "GB/s", "frac": (hbm_ach / 1e9 / hbm_peak) if hbm_peak else None,
                         "traffic": traffic, "kernel": kname,
                         "algorithmic_bytes_per_launch": hbm_bytes,
                         "peak_source": hbm_src},
        "clocks": clk.summary(),
    }
    if cpu_line:
        out["cpu_baseline"] = cpu_line
    if not args.no_configs and world == 1:
        x = y = z = pts = c = c0 = fkb = None
        torch.cuda.empty_cache()
        out["configs"] = {}
        for name in ("c1", "c2", "c4", "c5", "c3f64"):
            try:
                out["configs"][name] = CONFIGS[name](args, dev, stream, with_cpu=not args.no_cpu)
            except Exception as e:  # a failed side config must not hide the metric line
                out["configs"][name] = {"error": "%s: %s" % (type(e).__name__, e)}
            torch.cuda.empty_cache()
    print(json.dumps(out))
    if world > 1:
        dist.barrier()


# ------------------------------------------------------ the other workloads ----
REF_GPU_LIB = os.path.join(ROOT, "baseline", "_ref", "cufinufft", "libcufinufft_ref.so")


def reference_gpu_type1(x, y, z, c, nt, stream, args, dev):
    """The reference cuFINUFFT (its src/cuda compiled for sm_103a by
    oracle/Makefile target ref-gpu) on the same device inputs through its own C
    API with default options: one vector, and the nt vectors as one plan
    (its batching). Execute timed with CUDA events on the same stream."""
    import ctypes

    import torch

    from finufft_gb300 import _lib

    if not os.path.exists(REF_GPU_LIB):
        return {"unavailable": "reference cuFINUFFT not built for this GPU (oracle/Makefile "
                               "targets ref-gpu-src, ref-gpu)"}
    try:
        L = ctypes.CDLL(REF_GPU_LIB)  # its own namespace: RTLD_LOCAL
        P = ctypes.c_void_p
        L.cufinufft_default_opts.argtypes = [ctypes.POINTER(_lib.CufinufftOpts)]
        L.cufinufftf_makeplan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                          ctypes.POINTER(P), ctypes.POINTER(_lib.CufinufftOpts)]
        L.cufinufftf_setpts.argtypes = [P, ctypes.c_int64, P, P, P, ctypes.c_int, P, P, P]
        L.cufinufftf_execute.argtypes = [P, P, P]
        L.cufinufftf_destroy.argtypes = [P]
        out = {"library": "reference cuFINUFFT (src/cuda) built for sm_103a, default options"}
        M = x.numel()
        N = list(N_MODES)
        for name, ntr in (("plain", 1), ("batched", nt)):
            o = _lib.CufinufftOpts()
            L.cufinufft_default_opts(ctypes.byref(o))
            o.gpu_stream = stream.cuda_stream
            plan = P()
            nm = (ctypes.c_int64 * 3)(N[2], N[1], N[0])  # x fastest
            rc = L.cufinufftf_makeplan(1, 3, nm, 1, ntr, TOL, ctypes.byref(plan), ctypes.byref(o))
            if rc != 0:
                out[name] = {"error": "makeplan %d" % rc}
                continue
            # its fastest axis is the last array axis: pass (z, y, x)
            t0 = time.perf_counter()
            rc = L.cufinufftf_setpts(plan, M, z.data_ptr(), y.data_ptr(), x.data_ptr(), 0, None,
                                     None, None)
            torch.cuda.synchronize()
            setpts_s = time.perf_counter() - t0
            cc = c[0].contiguous() if ntr == 1 else c
            fk = torch.empty((ntr,) + tuple(N), dtype=torch.complex64, device=dev)
            ms = time_steps(lambda: L.cufinufftf_execute(plan, cc.data_ptr(), fk.data_ptr()),
                            stream, max(1, args.steps // 2), min(args.warmup, 2))
            ent = {"value": M * ntr / (ms * 1e-3), "ms_per_step": ms, "setpts_s": setpts_s}
            if ntr == 1:
                ax = sample_axes(N_MODES, 10, 5)
                ref = direct_type1_grid([x, y, z], c[0], N_MODES, ax, +1, dev)
                ent["rel_l2_vs_fp64_direct"] = rel_l2(take_grid(fk[0], ax), ref)
            out[name] = ent
            L.cufinufftf_destroy(plan)
            del fk
            torch.cuda.empty_cache()
        return out
    except Exception as e:  # the baseline must not take the metric line down
        return {"error": "%s: %s" % (type(e).__name__, e)}


def cfg_c1(args, dev, stream, with_cpu=True):
    """C1: 1D type 1 FP64, M = N = 1e6, tol 1e-9 (the reference's CPU-runnable case)"""
    import torch

    import finufft_gb300 as fg

    M, N, tol = 1_000_000, 1_000_000, 1e-9
    g = torch.Generator(device="cuda").manual_seed(11)
    x = (torch.rand(M, generator=g, device="cuda", dtype=torch.float64) * 2 - 1) * np.pi
    c = torch.randn(M, 2, generator=g, device="cuda", dtype=torch.float64).view(torch.complex128)[:, 0]
    p = fg.Plan(1, (N,), eps=tol, dtype="complex128", gpu_stream=stream.cuda_stream)
    p.setpts(x)
    f = torch.empty(N, dtype=torch.complex128, device=dev)
    ms = time_steps(lambda: p.execute(c, out=f), stream, args.steps, args.warmup)
    ax = sample_axes((N,), 1000, 7)
    ref = direct_type1_grid([x], c, (N,), ax, +1, dev)
    out = {"workload": "1D type 1 FP64, M=N=1e6 uniform, tol 1e-9", "value": M / (ms * 1e-3),
           "unit": "NU pts/s", "ms_per_step": ms}
    gerr = rel_l2(take_grid(f, ax), ref)
    cerr = None
    if with_cpu:
        O = _oracle()
        cp = O.CpuPlan(1, [N], +1, tol, dtype=np.complex128)
        cp.setpts([x.cpu().numpy()])
        t0 = time.perf_counter()
        fc = cp.execute(c.cpu().numpy())
        out["cpu_value"] = M / (time.perf_counter() - t0)
        out["cpu_cores"] = cp.threads
        cerr = rel_l2(take_grid(fc, ax), ref)
    out["accuracy"] = acc_entry(gerr, cerr, "1e3 sampled modes, FP64 direct sum")
    return out


def cfg_c2(args, dev, stream, with_cpu=True):
    """C2: 2D type 2 FP32, N = 1024^2, 16 vectors, M = 1e7, tol 1e-5, iflag -1"""
    import torch

    import finufft_gb300 as fg

    M, nt, N, tol = 10_000_000, 16, (1024, 1024), 1e-5
    g = torch.Generator(device="cuda").manual_seed(12)
    x, y = ((torch.rand(2, M, generator=g, device="cuda", dtype=torch.float64) * 2 - 1)
            * np.pi).to(torch.float32)
    fk = torch.randn(nt, *N, 2, generator=g, device="cuda").view(torch.complex64)[..., 0]
    f0 = fk[0].contiguous()

    def single(kw):
        p = fg.Plan(2, N, eps=tol, isign=-1, gpu_stream=stream.cuda_stream, **kw)
        p.setpts(x, y)
        cc = torch.empty(M, dtype=torch.complex64, device=dev)
        ms = time_steps(lambda: p.execute(f0, out=cc), stream, args.steps, args.warmup)
        return ms, cc

    ms_plain, c_plain = single({"planner": 1})
    ms1, c1 = single({})
    pb = fg.Plan(2, N, n_trans=nt, eps=tol, isign=-1, gpu_stream=stream.cuda_stream,
                 gpu_maxbatchsize=nt, planner=args.planner)
    pb.setpts(x, y)
    cb = torch.empty(nt, M, dtype=torch.complex64, device=dev)
    pb.execute(fk, out=cb)
    torch.cuda.synchronize()
    pb.graph_capture(cb, fk)
    msb = time_steps(pb.graph_launch, stream, args.steps, args.warmup)
    pb.stage_times(True)
    pb.execute(fk, out=cb)
    torch.cuda.synchronize()
    st = pb.stage_times(True)
    nf = pb.info().nf
    interp_bytes = nt * nf[0] * nf[1] * 8 + M * 2 * 4 + nt * M * 8
    # accuracy on 1e3 sampled targets, vector 0: c_j = sum_k f_k exp(-i k.x_j)
    sel = torch.as_tensor(np.random.default_rng(13).choice(M, 1000, replace=False), device=dev)
    k0 = torch.arange(N[0], dtype=torch.float64, device=dev) - N[0] // 2
    k1 = torch.arange(N[1], dtype=torch.float64, device=dev) - N[1] // 2
    one = torch.ones(1, dtype=torch.float64, device=dev)
    E0 = torch.polar(one, -k0[:, None] * x[sel].to(torch.float64)[None, :])
    E1 = torch.polar(one, -k1[:, None] * y[sel].to(torch.float64)[None, :])
    ref = ((f0.to(torch.complex128) @ E1) * E0).sum(0)
    out = {"workload": "2D type 2 FP32, N=1024^2, 16 vectors, M=1e7 uniform, tol 1e-5",
           "value": M * nt / (msb * 1e-3), "unit": "NU pts/s", "ms_per_step": msb,
           "plain": {"value": M / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                     "planner": "reference heuristic"},
           "plain_engine": {"value": M / (ms1 * 1e-3), "ms_per_step": ms1},
           "batched_stage_ms": {"interp": st[0], "fft": st[1], "amplify": st[2], "total": st[3]},
           "interp_hbm_GBps_algorithmic": interp_bytes / (st[0] * 1e-3) / 1e9}
    gerr = rel_l2(cb[0][sel], ref)
    cerr = None
    if with_cpu:
        O = _oracle()
        cp = O.CpuPlan(2, list(N[::-1]), -1, tol, dtype=np.complex64)
        cp.setpts([y.cpu().numpy(), x.cpu().numpy()])  # fastest axis first
        cc = cp.execute(f0.cpu().numpy())
        cerr = rel_l2(cc[sel.cpu().numpy()], ref)
    out["accuracy"] = acc_entry(gerr, cerr, "1e3 sampled targets of vector 0, FP64 direct sum")
    out["accuracy"]["plain_rel_l2"] = rel_l2(c_plain[sel], ref)
    return out


def cfg_c4(args, dev, stream, with_cpu=True):
    """C4: 4096 uneven 2D type-1 FP32 problems in one batched plan, tol 1e-6"""
    import ctypes

    import torch

    import finufft_gb300 as fg
    from finufft_gb300 import _lib

    tol = 1e-6
    g = torch.Generator(device="cuda").manual_seed(14)
    rng = np.random.default_rng(4)
    nprob = 4096
    Ns = np.round(np.exp(rng.uniform(np.log(32), np.log(256), (nprob, 2)))).astype(np.int64)
    Ms = np.round(np.exp(rng.uniform(np.log(1e3), np.log(1e5), nprob))).astype(np.int64)
    Mt = int(Ms.sum())
    xy = ((torch.rand(2, Mt, generator=g, device="cuda", dtype=torch.float64) * 2 - 1)
          * np.pi).to(torch.float32)
    c = torch.randn(Mt, 2, generator=g, device="cuda").view(torch.complex64)[:, 0]
    nm = np.concatenate([Ns, np.ones((nprob, 1), np.int64)], axis=1).ravel()
    lib = fg.load_library()
    plan = ctypes.c_void_p()
    o = _lib.default_opts()
    o.gpu_stream = stream.cuda_stream
    ext = None
    if args.variant >= 0:  # tuning runs: the 2D spread variant of the batch
        ext = _lib.default_ext_opts()
        ext.spread_variant = args.variant
    assert lib.cufinufftf_batch_makeplan(1, 2, nprob, nm.ctypes.data_as(
        ctypes.POINTER(ctypes.c_int64)), 1, tol, ctypes.byref(plan), ctypes.byref(o),
        ctypes.byref(ext) if ext is not None else None) == 0
    t0 = time.perf_counter()
    assert lib.cufinufftf_batch_setpts(plan, Ms.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                       xy[0].data_ptr(), xy[1].data_ptr(), None) == 0
    torch.cuda.synchronize()
    setpts_s = time.perf_counter() - t0
    nmodes = Ns[:, 0] * Ns[:, 1]
    fk = torch.empty(int(nmodes.sum()), dtype=torch.complex64, device=dev)
    ms = time_steps(lambda: lib.cufinufftf_batch_execute(plan, c.data_ptr(), fk.data_ptr()),
                    stream, args.steps, args.warmup)
    lib.cufinufftf_batch_destroy(plan)
    torch.cuda.synchronize()
    # per-problem times: a sample of problems run alone through single plans
    per = []
    off = np.concatenate([[0], np.cumsum(Ms)])
    moff = np.concatenate([[0], np.cumsum(nmodes)])
    for pidx in rng.choice(nprob, size=min(256, nprob), replace=False):
        a, b = off[pidx], off[pidx + 1]
        sp = fg.Plan(1, (int(Ns[pidx, 1]), int(Ns[pidx, 0])), eps=tol,
                     gpu_stream=stream.cuda_stream)
        sp.setpts(xy[1, a:b].contiguous(), xy[0, a:b].contiguous())
        cc = c[a:b].contiguous()
        per.append(time_steps(lambda: sp.execute(cc), stream, 3, 1))
    out = {"workload": "4096 uneven 2D type 1 FP32, N/side log-uniform [32,256], M "
                       "log-uniform [1e3,1e5], tol 1e-6, one batched plan",
           "value": Mt / (ms * 1e-3), "unit": "NU pts/s", "ms_per_step": ms, "M_total": Mt,
           "setpts_s": setpts_s,
           "per_problem_ms_single_plans": {"p50": float(np.percentile(per, 50)),
                                           "p99": float(np.percentile(per, 99)),
                                           "sample": len(per)},
           "batched_ms_per_problem": ms / nprob}
    # accuracy: 64 seeded problems, 16 sampled modes each (1024 modes)
    fk_h = fk.cpu().numpy()
    xy_h = xy.cpu().numpy()
    c_h = c.cpu().numpy()
    O = _oracle()
    got, want, cpu = [], [], []
    for pidx in np.random.default_rng(15).choice(nprob, 64, replace=False):
        a, b = off[pidx], off[pidx + 1]
        n0, n1 = int(Ns[pidx, 0]), int(Ns[pidx, 1])  # C order: n0 fastest (pairs with x)
        kidx = np.random.default_rng(int(pidx)).choice(n0 * n1, 16, replace=False)
        fprob = fk_h[moff[pidx]:moff[pidx + 1]]
        ref = O.dirft1([xy_h[0, a:b], xy_h[1, a:b]], c_h[a:b], 1, [n0, n1], kidx=kidx)
        got.append(fprob[kidx])
        want.append(ref)
        if with_cpu:
            cp = O.CpuPlan(1, [n0, n1], +1, tol, dtype=np.complex64)
            cp.setpts([xy_h[0, a:b], xy_h[1, a:b]])
            cpu.append(cp.execute(c_h[a:b]).ravel()[kidx])
    want = np.concatenate(want)
    out["accuracy"] = acc_entry(rel_l2(np.concatenate(got), want),
                                rel_l2(np.concatenate(cpu), want) if cpu else None,
                                "64 seeded problems x 16 sampled modes, FP64 direct sums")
    return out


def direct_type3(xs, c, ss_sel, isign, dev, chunk=20000):
    """FP64 direct type-3 sums at a few targets (GPU): f_k = sum_j c_j exp(i isign s_k.x_j)"""
    import torch

    X = torch.stack([a.to(torch.float64) for a in xs])
    S = torch.stack([a.to(torch.float64) for a in ss_sel])
    out = torch.zeros(S.shape[1], dtype=torch.complex128, device=dev)
    one = torch.ones(1, dtype=torch.float64, device=dev)
    for j0 in range(0, X.shape[1], chunk):
        ph = isign * (S.T @ X[:, j0:j0 + chunk])
        out += torch.polar(one, ph) @ c[j0:j0 + chunk].to(torch.complex128)
    return out


def cfg_c5(args, dev, stream, with_cpu=True):
    """C5: 3D type 3 FP32, M = K = 1e7, sources in box (1,2,4), targets in box
    (200,100,50), tol 1e-6; error on 1e4 sampled targets"""
    import torch

    import finufft_gb300 as fg

    M = K = 10_000_000
    tol = 1e-6
    g = torch.Generator(device="cuda").manual_seed(16)
    hs = torch.tensor([1.0, 2.0, 4.0], device="cuda", dtype=torch.float64)[:, None]
    ht = torch.tensor([200.0, 100.0, 50.0], device="cuda", dtype=torch.float64)[:, None]
    xs = ((torch.rand(3, M, generator=g, device="cuda", dtype=torch.float64) * 2 - 1) * hs).to(torch.float32)
    ss = ((torch.rand(3, K, generator=g, device="cuda", dtype=torch.float64) * 2 - 1) * ht).to(torch.float32)
    c = torch.randn(M, 2, generator=g, device="cuda").view(torch.complex64)[:, 0]
    res = {}
    for name, kw in (("plain", {"planner": 1}), ("engine", {"planner": 0}),
                     ("planned", {"planner": args.planner})):
        p = fg.Plan(3, 3, eps=tol, gpu_stream=stream.cuda_stream, **kw)
        p.setpts(xs[0], xs[1], xs[2], s=ss[0], t=ss[1], u=ss[2])
        f = torch.empty(K, dtype=torch.complex64, device=dev)
        ms = time_steps(lambda: p.execute(c, out=f), stream, args.steps, args.warmup)
        res[name] = (ms, f, p.info())
        del p
    sel = torch.as_tensor(np.random.default_rng(17).choice(K, 10000, replace=False), device=dev)
    ref = direct_type3([xs[0], xs[1], xs[2]], c, [ss[0][sel], ss[1][sel], ss[2][sel]], +1, dev)
    ms, f, info = res["planned"]
    out = {"workload": "3D type 3 FP32, M=K=1e7, boxes (1,2,4) x (200,100,50), tol 1e-6",
           "value": (M + K) / (ms * 1e-3), "unit": "NU pts/s (M+K)", "ms_per_step": ms,
           "planner": args.planner, "planner_used": info.planner_used,
           "planned_slot": info.planned_slot,
           "plain": {"value": (M + K) / (res["plain"][0] * 1e-3), "ms_per_step": res["plain"][0],
                     "planner": "reference heuristic",
                     "rel_l2": rel_l2(res["plain"][1][sel], ref)},
           "engine_default": {"value": (M + K) / (res["engine"][0] * 1e-3),
                              "ms_per_step": res["engine"][0],
                              "upsampfac": res["engine"][2].upsampfac,
                              "rel_l2": rel_l2(res["engine"][1][sel], ref)},
           "upsampfac": info.upsampfac, "ns": info.ns, "nf": list(info.nf),
           "inner_nf": list(info.inner_nf)}
    gerr = rel_l2(f[sel], ref)
    cerr = None
    if with_cpu:
        O = _oracle()
        cp = O.CpuPlan(3, 3, +1, tol, dtype=np.complex64, sigma=info.upsampfac)
        xh = xs.cpu().numpy()
        sh = ss.cpu().numpy()
        cp.setpts([xh[0], xh[1], xh[2]], [sh[0], sh[1], sh[2]])
        fc = cp.execute(c.cpu().numpy())
        cerr = rel_l2(fc[sel.cpu().numpy()], ref)
    out["accuracy"] = acc_entry(gerr, cerr, "1e4 sampled targets, FP64 direct sum")
    return out


def cfg_c3f64(args, dev, stream, with_cpu=True):
    """C3 in double precision at tol 1e-12: throughput on the full 1e8 points;
    errors on 1e3 sampled modes of a 1e7-point subset (engine and CPU
    restatement on the same subset)"""
    import torch

    import finufft_gb300 as fg

    M = args.m
    pts = clustered_points(M, 1234 + 3, rng_dev="cuda").to(torch.float64)
    gd = torch.Generator(device="cuda").manual_seed(99)
    c = torch.randn(M, 2, generator=gd, device="cuda", dtype=torch.float64).view(torch.complex128)[:, 0]
    x, y, z = (pts[d].contiguous() for d in range(3))
    kw = {"spread_variant": args.variant} if args.variant >= 0 else {}
    p = fg.Plan(1, N_MODES, eps=1e-12, dtype="complex128", gpu_stream=stream.cuda_stream, **kw)
    p.setpts(x, y, z)
    f = torch.empty(N_MODES, dtype=torch.complex128, device=dev)
    ms = time_steps(lambda: p.execute(c, out=f), stream, min(args.steps, 3), min(args.warmup, 1))
    p.stage_times(True)
    p.execute(c, out=f)
    torch.cuda.synchronize()
    st = p.stage_times(True)
    info = p.info()
    out = {"workload": "3D type 1 FP64, 256^3 modes, M=1e8 clustered, tol 1e-12",
           "value": M / (ms * 1e-3), "unit": "NU pts/s", "ms_per_step": ms,
           "stage_ms": {"spread": st[0], "fft": st[1], "deconv": st[2]}, "ns": info.ns,
           "spread_variant": info.spread_variant}
    # accuracy on a subset (the CPU restatement at ns=13 in FP64 is slow on 1e8)
    ms_sub = min(M, 10_000_000)
    xs_, ys_, zs_, cs_ = x[:ms_sub].contiguous(), y[:ms_sub].contiguous(), z[:ms_sub].contiguous(), c[:ms_sub].contiguous()
    del p
    ps = fg.Plan(1, N_MODES, eps=1e-12, dtype="complex128", gpu_stream=stream.cuda_stream)
    ps.setpts(xs_, ys_, zs_)
    fs = ps.execute(cs_)
    torch.cuda.synchronize()
    ax = sample_axes(N_MODES, 10, 5)
    ref = direct_type1_grid([xs_, ys_, zs_], cs_, N_MODES, ax, +1, dev)
    gerr = rel_l2(take_grid(fs, ax), ref)
    del ps, fs, f
    torch.cuda.empty_cache()
    cerr = None
    if with_cpu:
        fc, _, _, _ = cpu_type1_3d(np.stack([a.cpu().numpy() for a in (xs_, ys_, zs_)]),
                                   cs_.cpu().numpy(), 1e-12, np.complex128)
        cerr = rel_l2(take_grid(fc, ax), ref)
    out["accuracy"] = acc_entry(gerr, cerr, "1e3 modes (10x10x10 grid) of the first %d points"
                                % ms_sub)
    return out


def cfg_c3t2(args, dev, stream, with_cpu=True):
    """3D type 2 on the metric's points and sizes (the adjoint direction)"""
    import torch

    import finufft_gb300 as fg

    M = args.m
    pts = clustered_points(M, 1234 + 3, rng_dev="cuda")
    g = torch.Generator(device="cuda").manual_seed(18)
    fk = torch.randn(*N_MODES, 2, generator=g, device="cuda").view(torch.complex64)[..., 0]
    p = fg.Plan(2, N_MODES, eps=TOL, isign=-1, gpu_stream=stream.cuda_stream,
                interp_mode=args.interp_mode)
    p.setpts(pts[0].contiguous(), pts[1].contiguous(), pts[2].contiguous())
    cc = torch.empty(M, dtype=torch.complex64, device=dev)
    ms = time_steps(lambda: p.execute(fk, out=cc), stream, args.steps, args.warmup)
    p.stage_times(True)
    p.execute(fk, out=cc)
    torch.cuda.synchronize()
    st = p.stage_times(True)
    return {"workload": "3D type 2 FP32, 256^3 modes, M=1e8 clustered, tol 1e-5",
            "value": M / (ms * 1e-3), "unit": "NU pts/s", "ms_per_step": ms,
            "stage_ms": {"interp": st[0], "fft": st[1], "amplify": st[2]}}


CONFIGS = {"c1": cfg_c1, "c2": cfg_c2, "c4": cfg_c4, "c5": cfg_c5, "c3f64": cfg_c3f64,
           "c3t2": cfg_c3t2}


def run_config(args):
    """One secondary configuration as its own JSON line (not the metric line)."""
    import torch

    global N_MODES
    if args.nmodes:  # smaller grids for profiling runs of c3f64 / c3t2
        N_MODES = (args.nmodes,) * 3
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    out = {"config_name": args.config, "n_gpus": 1, "data": "synthetic (seeded)"}
    out.update(CONFIGS[args.config](args, dev, stream, with_cpu=not args.no_cpu))
    print(json.dumps(out))


# -------------------------------------------------------------- reference arm ----
def run_reference(args):
    """CPU FINUFFT restatement on the host cores, same metric and workload: each
    step executes the ntransf strength vectors over all 1e8 points."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    import torch

    O = _oracle()
    M = args.m
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    pts = clustered_points(M, 1234 + 3, rng_dev=dev).cpu().numpy()
    nt = args.ntransf
    cs = strengths(nt, M, 99, dev).cpu().numpy()
    plan = O.CpuPlan(1, list(N_MODES[::-1]), +1, TOL, dtype=np.complex64)
    t0 = time.perf_counter()
    plan.setpts([pts[2], pts[1], pts[0]])
    setpts_s = time.perf_counter() - t0

    def step():
        for k in range(nt):
            plan.execute(cs[k])

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    ms = float(np.mean(times)) * 1e3
    v = M * nt / (ms * 1e-3)
    out = {"metric": METRIC, "value": v, "unit": "NU pts/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic (seeded clustered points, N(0,1) strengths)",
           "config": {"workload": WORKLOAD, "ntransf_batched": nt, "M": M, "N": list(N_MODES),
                      "parallelism": "host cores (OpenMP)"},
           "cpu_baseline": {"kind": "port", "cores": plan.threads,
                            "sample": "every step: the full workload, one execute (spread, FFT, "
                                      "deconvolution) of each of the %d strength vectors over "
                                      "all %d points; setpts sort %.2f s outside the steps"
                                      % (nt, M, setpts_s),
                            "value": v, "unit": "NU pts/s", "host": cpu_model()},
           "step_s": {"min": min(times), "max": max(times), "median": float(np.median(times))},
           "e2e": {"value": v, "unit": "NU pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--m", type=int, default=M_FULL)
    ap.add_argument("--ntransf", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU restatement legs")
    ap.add_argument("--no-configs", action="store_true", help="skip the nested workloads")
    ap.add_argument("--config", default="c3", choices=["c1", "c2", "c3", "c3f64", "c3t2", "c4", "c5"],
                    help="c3 (default) is the metric line; the others print their own line")
    ap.add_argument("--nmodes", type=int, default=0, help="modes per side (profiling cases)")
    ap.add_argument("--bins", default="", help="bin sizes x,y,z (default: the planner's)")
    ap.add_argument("--maxsub", type=int, default=0, help="max points per subproblem")
    ap.add_argument("--variant", type=int, default=-1, help="3D spread variant (tuning runs)")
    ap.add_argument("--interp-mode", type=int, default=0,
                    help="type-2 interpolation schedule of --config c3t2 (0 auto, 1 gather, "
                         "2 block tiles, 3 TMA tiles)")
    ap.add_argument("--planner", type=int, default=2,
                    help="planner of the planned forms (2 learned, 3 autotuned, 0 fixed default)")
    ap.add_argument("--only", default="", choices=["", "plain", "engine", "batched"],
                    help="time only one form (profiling runs): a single-transform plan "
                         "(plain, engine) or the batched plan")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config != "c3":
        run_config(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
