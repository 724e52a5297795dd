"""Benchmark: 3D type-1 NUFFT throughput (NU pts/s) at tol 1e-5, FP32.

Workload (the metric's configuration): N = 256^3 modes, M = 1e8 points drawn
80% from 8 isotropic Gaussians (sigma 0.3, centres uniform in [-pi,pi)^3,
wrapped periodically) and 20% uniform, complex64 strengths N(0,1), iflag +1.
Synthetic, seeded inputs of those shapes stand in for user data.

A step is one execute of the planned transform on resident device inputs
(spread -> FFT -> deconvolve), timed with CUDA events on the plan's stream.
``value`` is the planned+batched form (ntransf strength vectors sharing the
points, one CUDA-graph replay per step); the plain form (one transform,
default options) is reported beside it. ``e2e`` times the same batched
transform through the public API with host buffers: pinned H2D of the step's
strengths, execute, D2H of the modes. Inputs (800 MB of strengths per vector,
a 1 GB fine grid per vector) exceed the 129 MB L2, so no flush is needed.

--impl reference times the CPU restatement of FINUFFT's algorithm (the
oracle port, PSWF kernel, OpenMP spreading + threaded FFT) on the host cores.
Under torchrun each rank runs an independent replica (the transform does not
shard); value sums the replicas.
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


def strengths(n, M, seed, dev):
    import torch

    g = torch.Generator(device=dev).manual_seed(seed)
    return torch.randn(n, M, 2, generator=g, device=dev, dtype=torch.float32).view(torch.complex64)[..., 0]


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
    if args.planner:
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
    res = {}

    # plain GPU form: one transform, default options (reference heuristic planning)
    plain = fg.Plan(1, N_MODES, n_trans=1, eps=TOL, dtype="complex64",
                    gpu_stream=stream.cuda_stream, **plan_kw)
    t0 = time.perf_counter()
    plain.setpts(x, y, z)
    torch.cuda.synchronize()
    setpts_s = time.perf_counter() - t0
    fk1 = torch.empty(N_MODES, dtype=torch.complex64, device=dev)
    c0 = c[0].contiguous()
    ms_plain = time_steps(lambda: plain.execute(c0, out=fk1), stream, args.steps, args.warmup)
    plain.stage_times(True)
    plain.execute(c0, out=fk1)
    torch.cuda.synchronize()
    st = plain.stage_times(True)
    info = plain.info()
    if args.only == "plain":
        print(json.dumps({"plain_ms": ms_plain, "stage_ms": st, "M": M, "nsub": info.nsub,
                          "bins": list(info.bins)}))
        return
    del plain
    torch.cuda.empty_cache()

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
    n_e2e = max(1, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        e2e_step()
    ms_e2e = (time.perf_counter() - t0) * 1e3 / n_e2e
    e2e_err = float(torch.linalg.norm(hf[0].to(dev) - fkb[0]) / torch.linalg.norm(fkb[0]))
    lib.finufftf_destroy(hplan)

    # accuracy on sampled modes against an FP64 direct sum (GPU, torch FP64)
    err = sampled_error(x, y, z, c[0], fkb[0], dev, nsample=args.err_modes, seed=5)

    # roofline of the dominant kernel (spread): shared-memory atomic updates
    ns = info.ns
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
    hbm_peak = measured_peak("hbm_gbs")
    traffic = SPREAD_DRAM_BYTES_PER_POINT * M * nt if kname == "spread_tile3v_kernel" else None

    ms_batched, ms_plain, ms_e2e = reduce_over_ranks([ms_batched, ms_plain, ms_e2e], world, dev)
    if rank != 0:
        dist.barrier() if world > 1 else None
        return
    value = job_value(M * nt, world, ms_batched)
    out = {
        "metric": METRIC, "value": value, "unit": "NU pts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batched,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clustered points, N(0,1) strengths)",
        "config": {"workload": "3D type 1, 256^3 modes, M=1e8 clustered (8 Gaussians sigma 0.3 "
                               "+ 20% uniform), complex64, tol 1e-5, iflag +1",
                   "ntransf_batched": nt, "M": M, "N": list(N_MODES),
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas",
                   "ns": ns, "nf": list(info.nf), "bins": list(info.bins),
                   "nsub": info.nsub},
        "plain": {"value": job_value(M, world, ms_plain), "ms_per_step": ms_plain,
                  "stage_ms": {"spread": st[0], "fft": st[1], "deconv": st[2]}},
        "batched_stage_ms": {"spread": stb[0], "fft": stb[1], "deconv": stb[2]},
        "setpts_s": setpts_s,
        # the reference perftest's amortized figure (perftest/cuda/cuperftest.cu:401):
        # points over makeplan + setpts + one execute, batched plan
        "amortized": {"value": job_value(M * nt, world, (makeplan_s + bsetpts_s) * 1e3 + ms_batched),
                      "unit": "NU pts/s", "makeplan_s": makeplan_s, "setpts_s": bsetpts_s},
        "rel_l2_err_sampled": err,
        "e2e": {"value": job_value(M * nt, world, ms_e2e), "unit": "NU pts/s",
                "h2d_bytes_per_step": nt * M * 8, "d2h_bytes_per_step": nt * int(np.prod(N_MODES)) * 8,
                "api": "finufftf_execute (host pointers, pinned)", "rel_diff_vs_device_api": e2e_err},
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
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu and world == 1:
        out["cpu_baseline"] = cpu_baseline(args.cpu_sample, 1)
    print(json.dumps(out))
    if world > 1:
        dist.barrier()


# DRAM bytes (read + write) per point per transform of the default 3D spread
# kernel, from an ncu capture at the same point density (1.25e7 clustered
# points on a 256^3 grid: 950.2 MB read + 132.4 MB written); scaled by points
# and transforms to one launch of this workload
SPREAD_DRAM_BYTES_PER_POINT = (950.213e6 + 132.354e6) / 12.5e6


def measured_peak(key):
    """a peak from MEASURED_PEAKS.json at the repository root (None if absent)"""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key])
    except (OSError, KeyError, ValueError):
        return None


def sampled_error(x, y, z, c, fk, dev, nsample=64, seed=5):
    """rel l2 error of nsample modes against an FP64 direct sum on the GPU."""
    import torch

    g = np.random.default_rng(seed)
    ks = [g.integers(0, n, nsample) for n in N_MODES]  # row-major indices
    got = fk[ks[0], ks[1], ks[2]].to(torch.complex128)
    modes = torch.tensor(np.stack([k - n // 2 for k, n in zip(ks, N_MODES)]),
                         dtype=torch.float64, device=dev)  # (3, S): axis0 <-> x
    X = torch.stack([x, y, z]).to(torch.float64)
    cc = c.to(torch.complex128)
    ref = torch.zeros(nsample, dtype=torch.complex128, device=dev)
    chunk = 4_000_000
    for j0 in range(0, X.shape[1], chunk):
        ph = modes.T @ X[:, j0:j0 + chunk]
        ref += (torch.polar(torch.ones_like(ph), ph) * cc[j0:j0 + chunk]).sum(dim=1)
    return float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))


def cpu_baseline(m_sample, seed):
    """CPU restatement of FINUFFT (oracle port) on a bounded sample: the spread
    of m_sample points is timed and scaled to M=1e8; FFT and deconvolution of
    the full 512^3 grid are timed as they are."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    pts = clustered_points(m_sample, 1234 + 3).numpy()
    rng = np.random.default_rng(seed)
    c = (rng.standard_normal(m_sample) + 1j * rng.standard_normal(m_sample)).astype(np.complex64)
    plan = O.CpuPlan(1, list(N_MODES), +1, TOL, dtype=np.complex64)
    plan.setpts([pts[2], pts[1], pts[0]])
    t0 = time.perf_counter()
    plan.execute(c)
    t_full = time.perf_counter() - t0
    # isolate the spread share: run again with no points to time FFT + deconvolution
    empty = O.CpuPlan(1, list(N_MODES), +1, TOL, dtype=np.complex64)
    empty.setpts([np.zeros(1, np.float32)] * 3)
    t0 = time.perf_counter()
    empty.execute(np.zeros(1, np.complex64))
    t_fixed = time.perf_counter() - t0
    t_spread = max(t_full - t_fixed, 1e-9)
    t_est = t_spread * (M_FULL / m_sample) + t_fixed
    return {"value": M_FULL / t_est, "unit": "NU pts/s", "cores": plan.threads, "kind": "port",
            "sample": "spread of %d clustered points timed and scaled to 1e8; 512^3 FFT + "
                      "deconvolution timed in full (%.2f s spread, %.2f s fixed)"
                      % (m_sample, t_spread, t_fixed)}


def _timed(fn, stream, steps, warmup):
    return time_steps(fn, stream, steps, warmup)


def run_config(args):
    """Secondary configurations (one JSON line each; not the metric line)."""
    import torch

    import finufft_gb300 as fg

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    g = torch.Generator(device="cuda").manual_seed(11)
    out = {"config_name": args.config, "n_gpus": 1, "data": "synthetic (seeded)"}
    if args.config == "c1":
        # 1D type 1, FP64: M = N = 1e6, tol 1e-9
        M, N = 1_000_000, 1_000_000
        x = (torch.rand(M, generator=g, device="cuda", dtype=torch.float64) * 2 - 1) * np.pi
        c = torch.randn(M, 2, generator=g, device="cuda", dtype=torch.float64).view(torch.complex128)[:, 0]
        p = fg.Plan(1, (N,), eps=1e-9, dtype="complex128", gpu_stream=stream.cuda_stream)
        p.setpts(x)
        f = torch.empty(N, dtype=torch.complex128, device=dev)
        ms = _timed(lambda: p.execute(c, out=f), stream, args.steps, args.warmup)
        out.update({"workload": "1D type 1 FP64, M=N=1e6, tol 1e-9", "value": M / (ms * 1e-3),
                    "unit": "NU pts/s", "ms_per_step": ms})
    elif args.config == "c2":
        # 2D type 2 batched: N = 1024^2, ntransf 16, M = 1e7, tol 1e-5, iflag -1
        M, nt, N = 10_000_000, 16, (1024, 1024)
        x, y = ((torch.rand(2, M, generator=g, device="cuda", dtype=torch.float64) * 2 - 1)
                * np.pi).to(torch.float32)
        fk = torch.randn(nt, *N, 2, generator=g, device="cuda").view(torch.complex64)[..., 0]
        p1 = fg.Plan(2, N, eps=1e-5, isign=-1, gpu_stream=stream.cuda_stream)
        p1.setpts(x, y)
        c1 = torch.empty(M, dtype=torch.complex64, device=dev)
        f0 = fk[0].contiguous()
        ms1 = _timed(lambda: p1.execute(f0, out=c1), stream, args.steps, args.warmup)
        pb = fg.Plan(2, N, n_trans=nt, eps=1e-5, isign=-1, gpu_stream=stream.cuda_stream,
                     gpu_maxbatchsize=nt)
        pb.setpts(x, y)
        cb = torch.empty(nt, M, dtype=torch.complex64, device=dev)
        pb.execute(fk, out=cb)
        torch.cuda.synchronize()
        pb.graph_capture(cb, fk)
        msb = _timed(pb.graph_launch, stream, args.steps, args.warmup)
        pb.stage_times(True)
        pb.execute(fk, out=cb)
        torch.cuda.synchronize()
        st = pb.stage_times(True)
        # interp roofline: grid bytes read per transform + coordinates + output
        nf = pb.info().nf
        interp_bytes = nt * nf[0] * nf[1] * 8 + M * 2 * 4 + nt * M * 8
        out.update({"workload": "2D type 2 FP32, N=1024^2, 16 vectors, M=1e7, tol 1e-5",
                    "value": M * nt / (msb * 1e-3), "unit": "NU pts/s", "ms_per_step": msb,
                    "plain": {"value": M / (ms1 * 1e-3), "ms_per_step": ms1},
                    "batched_stage_ms": {"interp": st[0], "fft": st[1], "amplify": st[2],
                                         "total": st[3]},
                    "interp_hbm_GBps_algorithmic": interp_bytes / (st[0] * 1e-3) / 1e9})
    elif args.config == "c4":
        # 4096 uneven 2D type 1 problems, tol 1e-6, one batched plan
        import ctypes

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
        from finufft_gb300 import _lib

        o = _lib.default_opts()
        o.gpu_stream = stream.cuda_stream
        assert lib.cufinufftf_batch_makeplan(1, 2, nprob, nm.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int64)), 1, 1e-6, ctypes.byref(plan), ctypes.byref(o), None) == 0
        t0 = time.perf_counter()
        assert lib.cufinufftf_batch_setpts(plan, Ms.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                           xy[0].data_ptr(), xy[1].data_ptr(), None) == 0
        torch.cuda.synchronize()
        setpts_s = time.perf_counter() - t0
        fk = torch.empty(int((Ns[:, 0] * Ns[:, 1]).sum()), dtype=torch.complex64, device=dev)
        ms = _timed(lambda: lib.cufinufftf_batch_execute(plan, c.data_ptr(), fk.data_ptr()),
                    stream, args.steps, args.warmup)
        lib.cufinufftf_batch_destroy(plan)
        # per-problem times: a sample of problems run alone through single plans
        per = []
        off = np.concatenate([[0], np.cumsum(Ms)])
        for pidx in rng.choice(nprob, size=min(256, nprob), replace=False):
            a, b = off[pidx], off[pidx + 1]
            sp = fg.Plan(1, (int(Ns[pidx, 1]), int(Ns[pidx, 0])), eps=1e-6,
                         gpu_stream=stream.cuda_stream)
            sp.setpts(xy[1, a:b].contiguous(), xy[0, a:b].contiguous())
            cc = c[a:b].contiguous()
            per.append(_timed(lambda: sp.execute(cc), stream, 3, 1))
        out.update({"workload": "4096 uneven 2D type 1 FP32, N/side log-uniform [32,256], M "
                                "log-uniform [1e3,1e5], tol 1e-6, one batched plan",
                    "value": Mt / (ms * 1e-3), "unit": "NU pts/s", "ms_per_step": ms,
                    "M_total": Mt, "setpts_s": setpts_s,
                    "per_problem_ms_single_plans": {"p50": float(np.percentile(per, 50)),
                                                    "p99": float(np.percentile(per, 99)),
                                                    "sample": len(per)},
                    "batched_ms_per_problem": ms / nprob})
    elif args.config == "c3t2":
        # 3D type 2 on the metric's points and sizes (the adjoint direction)
        M = args.m
        pts = clustered_points(M, 1234 + 3, rng_dev="cuda")
        fk = torch.randn(*N_MODES, 2, generator=g, device="cuda").view(torch.complex64)[..., 0]
        p = fg.Plan(2, N_MODES, eps=TOL, isign=-1, gpu_stream=stream.cuda_stream)
        p.setpts(pts[0].contiguous(), pts[1].contiguous(), pts[2].contiguous())
        cc = torch.empty(M, dtype=torch.complex64, device=dev)
        ms = _timed(lambda: p.execute(fk, out=cc), stream, args.steps, args.warmup)
        p.stage_times(True)
        p.execute(fk, out=cc)
        torch.cuda.synchronize()
        st = p.stage_times(True)
        out.update({"workload": "3D type 2 FP32, 256^3 modes, M=1e8 clustered, tol 1e-5",
                    "value": M / (ms * 1e-3), "unit": "NU pts/s", "ms_per_step": ms,
                    "stage_ms": {"interp": st[0], "fft": st[1], "amplify": st[2]}})
    elif args.config == "c3f64":
        # the metric's workload in double precision at tol 1e-12 (ns = 13)
        M = args.m
        pts = clustered_points(M, 1234 + 3, rng_dev="cuda").to(torch.float64)
        gd = torch.Generator(device="cuda").manual_seed(99)
        c = torch.randn(M, 2, generator=gd, device="cuda", dtype=torch.float64).view(torch.complex128)[:, 0]
        x, y, z = (pts[d].contiguous() for d in range(3))
        p = fg.Plan(1, N_MODES, eps=1e-12, dtype="complex128", gpu_stream=stream.cuda_stream)
        p.setpts(x, y, z)
        f = torch.empty(N_MODES, dtype=torch.complex128, device=dev)
        ms = _timed(lambda: p.execute(c, out=f), stream, min(args.steps, 3), min(args.warmup, 1))
        p.stage_times(True)
        p.execute(c, out=f)
        torch.cuda.synchronize()
        st = p.stage_times(True)
        err = sampled_error(x, y, z, c, f, dev, nsample=32, seed=5)
        info = p.info()
        out.update({"workload": "3D type 1 FP64, 256^3 modes, M=1e8 clustered, tol 1e-12",
                    "value": M / (ms * 1e-3), "unit": "NU pts/s", "ms_per_step": ms,
                    "stage_ms": {"spread": st[0], "fft": st[1], "deconv": st[2]},
                    "rel_l2_err_sampled": err, "ns": info.ns, "spread_variant": info.spread_variant})
    elif args.config == "c5":
        # 3D type 3: M = K = 1e7, sources in box (1,2,4), targets in box (200,100,50)
        M = K = 10_000_000
        hs = torch.tensor([1.0, 2.0, 4.0], device="cuda", dtype=torch.float64)[:, None]
        ht = torch.tensor([200.0, 100.0, 50.0], device="cuda", dtype=torch.float64)[:, None]
        xs = ((torch.rand(3, M, generator=g, device="cuda", dtype=torch.float64) * 2 - 1) * hs).to(torch.float32)
        ss = ((torch.rand(3, K, generator=g, device="cuda", dtype=torch.float64) * 2 - 1) * ht).to(torch.float32)
        c = torch.randn(M, 2, generator=g, device="cuda").view(torch.complex64)[:, 0]
        p = fg.Plan(3, 3, eps=1e-6, gpu_stream=stream.cuda_stream)
        p.setpts(xs[0], xs[1], xs[2], s=ss[0], t=ss[1], u=ss[2])
        f = torch.empty(K, dtype=torch.complex64, device=dev)
        ms = _timed(lambda: p.execute(c, out=f), stream, args.steps, args.warmup)
        # error on 256 sampled targets against an FP64 direct sum
        nchk, blk = 256, 500_000
        idx = torch.randint(0, K, (nchk,), generator=g, device="cuda")
        S = ss[:, idx].to(torch.float64)
        X = xs.to(torch.float64)
        ref = torch.zeros(nchk, dtype=torch.complex128, device=dev)
        for j0 in range(0, M, blk):
            ph = S.T @ X[:, j0:j0 + blk]
            ref += (torch.polar(torch.ones_like(ph), ph) * c[j0:j0 + blk].to(torch.complex128)).sum(1)
        err = float(torch.linalg.norm(f[idx].to(torch.complex128) - ref) / torch.linalg.norm(ref))
        info = p.info()
        out.update({"workload": "3D type 3 FP32, M=K=1e7, boxes (1,2,4) x (200,100,50), tol 1e-6",
                    "value": (M + K) / (ms * 1e-3), "unit": "NU pts/s (M+K)", "ms_per_step": ms,
                    "rel_l2_err_sampled": err, "upsampfac": info.upsampfac, "ns": info.ns,
                    "nf": list(info.nf), "inner_nf": list(info.inner_nf)})
    print(json.dumps(out))


def run_reference(args):
    """CPU FINUFFT restatement on the host cores, same metric and config."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    vals = []
    for s in range(args.warmup + args.steps):
        cb = cpu_baseline(args.cpu_sample, s)
        if s >= args.warmup:
            vals.append(cb)
    v = float(np.median([c["value"] for c in vals]))
    out = {"metric": METRIC, "value": v, "unit": "NU pts/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": M_FULL / v * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic (seeded clustered points, N(0,1) strengths)",
           "config": {"workload": "3D type 1, 256^3 modes, M=1e8 clustered (8 Gaussians sigma 0.3 "
                                  "+ 20% uniform), complex64, tol 1e-5, iflag +1"},
           "cpu_baseline": {"kind": "port", "cores": vals[-1]["cores"], "sample": vals[-1]["sample"],
                            "value": v, "unit": "NU pts/s"},
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
    ap.add_argument("--cpu-sample", type=int, default=4_000_000)
    ap.add_argument("--err-modes", type=int, default=32)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--config", default="c3", choices=["c1", "c2", "c3", "c3f64", "c3t2", "c4", "c5"],
                    help="c3 (default) is the metric line; the others print their own line")
    ap.add_argument("--nmodes", type=int, default=0, help="modes per side (profiling cases)")
    ap.add_argument("--bins", default="", help="bin sizes x,y,z (default: the planner's)")
    ap.add_argument("--maxsub", type=int, default=0, help="max points per subproblem")
    ap.add_argument("--variant", type=int, default=-1, help="3D spread variant (tuning runs)")
    ap.add_argument("--planner", type=int, default=0, help="1: reference heuristic planning")
    ap.add_argument("--only", default="", choices=["", "plain"],
                    help="plain: time only the single-transform plan (profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config != "c3":
        run_config(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
