"""Trains the learned planner on the engine's own sweeps and writes the model
that the library compiles in (csrc/planner_weights.inc).

The 2x64 MLP (tanh hidden layers) maps standardised problem features to the
standardised log10 execute time of every candidate slot; training minimises
the squared error over the slots each sample timed (minibatch Adam), in the
library's hand-written CUDA training kernels (gbnufft_planner_train). 20% of
the samples are held out: the report gives, on them, the time of the slot the
model picks (among the slots the sample timed) over the fastest slot, beside
the same ratio for the engine's fixed default slot and the reference
heuristic's slot, and the measured FP64 errors of the picked plans against tol.

Usage: python -m finufft_gb300.planner_train sweeps.npz --out csrc/planner_weights.inc
"""
import argparse
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_sweeps(paths):
    F, T, E, Mt = [], [], [], []
    for p in paths:
        d = np.load(p)
        F.append(d["features"])
        T.append(d["times"])
        E.append(d["errors"])
        Mt.append(d["meta"])
    return np.concatenate(F), np.concatenate(T), np.concatenate(E), np.concatenate(Mt)


def forward_np(w, x, NF, H, K):
    """the MLP on the host (float64), same layout as the library's kernels"""
    o = 0
    W1 = w[o:o + H * NF].reshape(H, NF); o += H * NF
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    W3 = w[o:o + K * H].reshape(K, H); o += K * H
    b3 = w[o:o + K]
    a1 = np.tanh(x @ W1.T + b1)
    a2 = np.tanh(a1 @ W2.T + b2)
    return a2 @ W3.T + b3


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("sweeps", nargs="+")
    ap.add_argument("--out", default=os.path.join(HERE, "csrc", "planner_weights.inc"))
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=128)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--wd", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--report", default="")
    args = ap.parse_args()

    from finufft_gb300 import _lib

    lib = _lib.load()
    nf_, h_, k_, nw_ = (ctypes.c_int() for _ in range(4))
    lib.gbnufft_planner_dims(ctypes.byref(nf_), ctypes.byref(h_), ctypes.byref(k_), ctypes.byref(nw_))
    NF, H, K, NW = nf_.value, h_.value, k_.value, nw_.value
    F, T, E, meta = load_sweeps(args.sweeps)
    ok = np.isfinite(T) & (T > 0)
    keep = ok.sum(1) >= 2
    F, T, E, meta, ok = F[keep], T[keep], E[keep], meta[keep], ok[keep]
    n = len(F)
    rng = np.random.default_rng(args.seed)
    perm = rng.permutation(n)
    ntest = max(1, n // 5)
    test, train = perm[:ntest], perm[ntest:]
    mean = F[train].mean(0)
    std = F[train].std(0)
    std[std < 1e-6] = 1.0
    Y = np.where(ok, np.log10(np.where(ok, T, 1.0)), 0.0)
    ymean = float(Y[train][ok[train]].mean())
    ystd = float(Y[train][ok[train]].std())
    X = ((F - mean) / std).astype(np.float32)
    Yn = ((Y - ymean) / ystd).astype(np.float32)
    Mk = ok.astype(np.float32)
    # Glorot-uniform initialisation
    w = np.zeros(NW, np.float32)
    o = 0
    for fan_in, fan_out in ((NF, H), (H, H), (H, K)):
        lim = np.sqrt(6.0 / (fan_in + fan_out))
        w[o:o + fan_in * fan_out] = rng.uniform(-lim, lim, fan_in * fan_out)
        o += fan_in * fan_out + fan_out
    loss = np.zeros(args.epochs, np.float32)
    xt, yt, mt = (np.ascontiguousarray(a[train]) for a in (X, Yn, Mk))
    rc = lib.gbnufft_planner_train(len(train), xt.ctypes.data, yt.ctypes.data, mt.ctypes.data,
                                   args.epochs, args.batch, args.lr, args.wd, args.seed,
                                   w.ctypes.data, loss.ctypes.data)
    assert rc == 0, rc
    pred = forward_np(w.astype(np.float64), X.astype(np.float64), NF, H, K)
    # the slots the library may take for each sample (its analytic rejection
    # rule, gbnufft_planner_valid); the report picks among these, as the
    # library does at setpts
    allowed = np.zeros_like(ok)
    vflag = ctypes.c_int()
    for i in range(n):
        for k in range(K):
            if lib.gbnufft_planner_valid(int(meta[i, 1]), int(meta[i, 0]), int(meta[i, 2]),
                                         float(meta[i, 3]), k, ctypes.byref(vflag)) == 0:
                allowed[i, k] = bool(vflag.value)
    use = ok & allowed
    test = np.array([i for i in test if use[i].any()])

    def pick_ratio(idx, choose):
        r = []
        for i in idx:
            valid = np.where(use[i])[0]
            k = choose(i, valid)
            r.append(T[i, k] / T[i, valid].min())
        return np.array(r)

    # the library's choice: the fastest predicted allowed slot, but the default
    # slot 0 unless the other is predicted PLANNER_KEEP_DEFAULT (1.037) times faster
    keep = np.log10(1.037) / ystd  # that ratio in standardised units

    def choose(i, v):
        k = v[np.argmin(pred[i, v])]
        if k != 0 and 0 in v and pred[i, 0] - pred[i, k] <= keep:
            k = 0
        return k

    learned = pick_ratio(test, choose)
    default = pick_ratio(test, lambda i, v: 0 if 0 in v else v[0])
    reference = pick_ratio(test, lambda i, v: 3 if 3 in v else v[0])
    chosen = [choose(i, np.where(use[i])[0]) for i in test]
    err_over_tol = np.array([E[i, k] / meta[i, 3] for i, k in zip(test, chosen)])
    rep = {
        "samples": int(n), "train": int(len(train)), "test": int(len(test)),
        "note": "held-out picks among the timed slots the library's rejection rule allows",
        "loss_first_last": [float(loss[0]), float(loss[-1])],
        "heldout_time_over_best": {
            "learned": {"mean": float(learned.mean()), "median": float(np.median(learned)),
                        "p90": float(np.percentile(learned, 90))},
            "engine_default_slot0": {"mean": float(default.mean()),
                                     "median": float(np.median(default))},
            "reference_heuristic_slot3": {"mean": float(reference.mean()),
                                          "median": float(np.median(reference))}},
        "heldout_error_over_tol_of_picked": {
            "median": float(np.nanmedian(err_over_tol)),
            "p90": float(np.nanpercentile(err_over_tol, 90)),
            "max": float(np.nanmax(err_over_tol))},
    }
    print(json.dumps(rep, indent=1))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(rep, f, indent=1)
    lo = F.min(0) - 0.25 * np.abs(F.min(0)) - 0.5
    hi = F.max(0) + 0.25 * np.abs(F.max(0)) + 0.5
    def lit(v):
        t = "%.9g" % v
        return (t if any(ch in t for ch in ".en") else t + ".0") + "f"

    fmt = lambda a: ", ".join(lit(v) for v in a)
    lines = [
        "// Trained weights of the learned planner (2x64 MLP), written by",
        "// python -m finufft_gb300.planner_train from %d engine sweeps (%d held out)." % (n, ntest),
        "// Held-out picked-slot time / fastest slot time: mean %.3f (engine default slot %.3f,"
        % (learned.mean(), default.mean()),
        "// reference heuristic slot %.3f)." % reference.mean(),
        "#define GBN_PLANNER_TRAINED 1",
        "static const float kPlannerMean[PLANNER_NF] = {%s};" % fmt(mean),
        "static const float kPlannerStd[PLANNER_NF] = {%s};" % fmt(std),
        "static const float kPlannerLo[PLANNER_NF] = {%s};" % fmt(lo),
        "static const float kPlannerHi[PLANNER_NF] = {%s};" % fmt(hi),
        "static const float kPlannerYMean = %s, kPlannerYStd = %s;" % (lit(ymean), lit(ystd)),
        "__device__ float g_planner_w[PLANNER_NW] = {",
    ]
    for i in range(0, NW, 8):
        lines.append("    " + fmt(w[i:i + 8]) + ",")
    lines.append("};")
    with open(args.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", args.out)


if __name__ == "__main__":
    main()
