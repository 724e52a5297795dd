"""Sweep generator of the learned planner: timing and error sweeps that the
engine runs on synthetic point clouds.

Each sample draws a problem (dimension 2 or 3, type 1/2/3, precision, tol,
sizes, a point cloud mixing uniform points with a random number of Gaussian
clusters of random widths) and runs every candidate plan shape of the
planner's table (gbnufft_planner_candidate: upsampling factor x bins /
subproblem size / spread variant, one slot being the reference library's
heuristic) through the C ABI: makeplan, setpts, one warm-up execute, then the
median of three executes timed with CUDA events on the plan's stream, and the
relative error of 16 sampled outputs against an FP64 direct sum. The problem's
features come from gbnufft_point_features, the same device code the planner
runs at setpts. Output: an .npz of features, per-slot times (NaN where a slot
is unused or its plan fails) and errors.

Usage: python -m finufft_gb300.planner_sweep --out sweeps.npz --samples 2000 --budget 900
"""
import argparse
import ctypes
import math
import time

import numpy as np


def width_center(lo, hi):
    """half-width and centre of [lo, hi], centred only when that shrinks the
    half-width by more than 10% (the engine's type-3 rule)"""
    w, c = (hi - lo) / 2, (hi + lo) / 2
    if abs(c) < 0.1 * w:
        w += abs(c)
        c = 0.0
    return w, c


def draw_problem(rng):
    dim = int(rng.choice([2, 3], p=[0.4, 0.6]))
    ty = int(rng.choice([1, 2, 3], p=[0.5, 0.25, 0.25]))
    dbl = bool(rng.random() < 0.2)
    tol = float(10 ** rng.uniform(-12 if dbl else -6.5, -2))
    M = int(10 ** rng.uniform(4, 7))
    if ty == 3:
        K = int(10 ** rng.uniform(4, 6.7))
        X = rng.uniform(0.5, 5.0, dim)
        S = 10 ** rng.uniform(0.3, 2.2 if dim == 3 else 2.8, dim) / X
        return dict(dim=dim, type=ty, dbl=dbl, tol=tol, M=M, K=K, X=X, S=S,
                    ntr=int(rng.choice([1, 1, 2, 4])))
    lo, hi = (16, 180) if dim == 3 else (32, 1600)
    n = [int(10 ** rng.uniform(math.log10(lo), math.log10(hi))) for _ in range(dim)]
    return dict(dim=dim, type=ty, dbl=dbl, tol=tol, M=M, n=n, ntr=int(rng.choice([1, 1, 2, 4])))


def draw_points(rng, dim, M, half=None):
    """uniform plus Gaussian clusters (wrapped); half: box half-widths (type 3)"""
    fcl = 0.0 if rng.random() < 0.3 else rng.uniform(0.2, 1.0)
    ncl = int(rng.integers(1, 17))
    width = 10 ** rng.uniform(-2, 0)
    nc = int(fcl * M)
    x = rng.uniform(-np.pi, np.pi, (dim, M))
    if nc:
        cen = rng.uniform(-np.pi, np.pi, (ncl, dim))
        x[:, :nc] = (cen[rng.integers(0, ncl, nc)].T + width * rng.standard_normal((dim, nc)))
        x[:, :nc] = np.remainder(x[:, :nc] + np.pi, 2 * np.pi) - np.pi
    if half is not None:
        x = x / np.pi * np.asarray(half)[:, None]
    return x


def run(args):
    import torch

    import finufft_gb300 as fg
    from finufft_gb300 import _lib

    lib = _lib.load()
    nf_, h_, k_, nw_ = (ctypes.c_int() for _ in range(4))
    lib.gbnufft_planner_dims(ctypes.byref(nf_), ctypes.byref(h_), ctypes.byref(k_), ctypes.byref(nw_))
    NF, K = nf_.value, k_.value
    rng = np.random.default_rng(args.seed)
    dev = torch.device("cuda")
    stream = torch.cuda.Stream()
    feats, times, errs, metas = [], [], [], []
    t_start = time.time()
    for it in range(args.samples):
        if time.time() - t_start > args.budget:
            break
        p = draw_problem(rng)
        dim, ty, dbl = p["dim"], p["type"], p["dbl"]
        rdt = torch.float64 if dbl else torch.float32
        cdt = torch.complex128 if dbl else torch.complex64
        M = p["M"]
        xs = draw_points(rng, dim, M, p["X"] if ty == 3 else None)
        x = [torch.tensor(a, dtype=rdt, device=dev) for a in xs]
        if ty == 3:
            s = (rng.uniform(-1, 1, (dim, p["K"])) * p["S"][:, None])
            sv = [torch.tensor(a, dtype=rdt, device=dev) for a in s]
            nout = p["K"]
        else:
            nm = tuple(p["n"])
            nout = int(np.prod(nm))
        ntr = p["ntr"]
        # features (the planner's conventions)
        shift = np.full(3, -np.pi)
        scale = np.full(3, 0.5 / np.pi)
        xsp = 0.0
        if ty == 3:
            for d in range(dim):
                X, C = width_center(float(xs[d].min()), float(xs[d].max()))
                Sd, _ = width_center(float(s[d].min()), float(s[d].max()))
                X = X if X > 0 else 1.0
                shift[d], scale[d] = C - X, 0.5 / X
                xsp += math.log10(X * Sd + 1.0) / dim
        feat = np.zeros(NF, np.float32)
        ptr = [a.data_ptr() for a in x] + [None] * (3 - dim)
        assert lib.gbnufft_point_features(dim, ty, int(dbl), M, ptr[0], ptr[1], ptr[2],
                                          shift.ctypes.data, scale.ctypes.data, float(nout),
                                          p["tol"], min(ntr, 8), 10 ** xsp - 1.0,
                                          feat.ctypes.data, None) == 0
        # inputs and a 16-output FP64 check
        if ty == 2:
            data = torch.randn((ntr,) + nm + (2,), dtype=rdt, device=dev).view(cdt)[..., 0]
        else:
            data = torch.randn(ntr, M, 2, dtype=rdt, device=dev).view(cdt)[..., 0]
        sel = torch.as_tensor(rng.choice(nout if ty != 2 else M, 16, replace=False), device=dev)
        ref = direct_ref(p, x, sv if ty == 3 else None, data[0], sel, dev)
        t_row = np.full(K, np.nan)
        e_row = np.full(K, np.nan)
        for k in range(K):
            sig, bins, maxsub, var, refh = (ctypes.c_double(), (ctypes.c_int * 3)(),
                                            ctypes.c_int(), ctypes.c_int(), ctypes.c_int())
            if lib.gbnufft_planner_candidate(dim, int(dbl), k, ctypes.byref(sig), bins,
                                             ctypes.byref(maxsub), ctypes.byref(var),
                                             ctypes.byref(refh)) != 0:
                continue
            kw = dict(upsampfac=sig.value, kernel_form=2, gpu_kerevalmeth=0,
                      gpu_stream=stream.cuda_stream, gpu_maxbatchsize=min(ntr, 8))
            if refh.value:
                kw["planner"] = 1
            else:
                b = list(bins)
                kw.update(gpu_binsizex=b[0], gpu_binsizey=b[1], gpu_binsizez=b[2],
                          gpu_maxsubprobsize=maxsub.value, spread_variant=var.value)
            try:
                plan = fg.Plan(ty, dim if ty == 3 else nm, n_trans=ntr, eps=p["tol"],
                               dtype="complex128" if dbl else "complex64",
                               isign=-1 if ty == 2 else 1, **kw)
                if ty == 3:
                    plan.setpts(*x, **dict(zip("stu", sv)))
                else:
                    plan.setpts(*x)
                out = plan.execute(data)
                torch.cuda.synchronize()
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                ms = []
                for _ in range(3):
                    ev[0].record(stream)
                    plan.execute(data, out=out)
                    ev[1].record(stream)
                    torch.cuda.synchronize()
                    ms.append(ev[0].elapsed_time(ev[1]))
                t_row[k] = float(np.median(ms))
                got = (out[0] if ntr > 1 else out).reshape(-1)[sel].to(torch.complex128)
                e_row[k] = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
                del plan, out
            except Exception:  # a slot whose plan cannot be built for this problem
                pass
        feats.append(feat)
        times.append(t_row)
        errs.append(e_row)
        metas.append([dim, ty, int(dbl), p["tol"], M, nout, ntr])
        if args.verbose and it % 50 == 0:
            print(it, time.time() - t_start, feat[:7], np.nanargmin(t_row) if np.isfinite(t_row).any() else -1,
                  flush=True)
    np.savez(args.out, features=np.array(feats), times=np.array(times), errors=np.array(errs),
             meta=np.array(metas))
    print("samples", len(feats), "seconds", time.time() - t_start)


def direct_ref(p, x, s, c0, sel, dev):
    """FP64 direct sums at the selected outputs (modes, targets or points)"""
    import torch

    dim, ty = p["dim"], p["type"]
    one = torch.ones(1, dtype=torch.float64, device=dev)
    X = torch.stack([a.to(torch.float64) for a in x])
    if ty == 3:
        S = torch.stack([a.to(torch.float64) for a in s])[:, sel]
        return (torch.polar(one, S.T @ X) @ c0.to(torch.complex128))
    nm = p["n"]
    if ty == 1:
        idx = np.unravel_index(sel.cpu().numpy(), tuple(nm))
        k = torch.tensor(np.stack([i - n // 2 for i, n in zip(idx, nm)]), dtype=torch.float64,
                         device=dev)
        return torch.polar(one, k.T @ X) @ c0.to(torch.complex128)
    # type 2 at the selected points: sum over all modes
    grids = torch.meshgrid(*[torch.arange(n, dtype=torch.float64, device=dev) - n // 2 for n in nm],
                           indexing="ij")
    kk = torch.stack([g.reshape(-1) for g in grids])
    return torch.polar(one, -(X[:, sel].T @ kk)) @ c0.reshape(-1).to(torch.complex128)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="planner_sweeps.npz")
    ap.add_argument("--samples", type=int, default=2000)
    ap.add_argument("--budget", type=float, default=900.0, help="seconds")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--verbose", action="store_true")
    run(ap.parse_args())


if __name__ == "__main__":
    main()
