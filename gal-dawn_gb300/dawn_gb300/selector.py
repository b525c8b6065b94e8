"""Learned per-level variant selector: data collection, training, evaluation.

The selector is a 9 x 32 x 32 x 3 ReLU MLP that the per-level decide
kernels evaluate on the device (csrc/selector.cuh).  It predicts log2 of a
level's duration in microseconds for three variants (0 sparse push, 1
bitmap pull, 2 dense push) and the level runs the smallest prediction.

Training data is the library's own trace: a traversal is run once per
forced variant with tracing on (dawn_trace_enable), which times every
level's kernels with CUDA events.  Levels are direction-independent (the
vertices a level discovers do not depend on how it is expanded), so the
three runs see the same frontier at every level and give every variant's
time for the same state.  The direction heuristics are the fallback (no
weights loaded) and the yardstick: ``evaluate`` times held-out graphs under
both and reports the ratio.

    python -m dawn_gb300.selector collect --split train --out data_train.npz
    python -m dawn_gb300.selector train data_train.npz --out weights.json
    python -m dawn_gb300.selector evaluate weights.json --split heldout
"""

import argparse
import json
import os
import sys
import time

import numpy as np

from . import abi, gen

N_IN, N_HID, N_OUT = 9, 32, 3
N_WEIGHTS = N_HID * N_IN + N_HID + N_HID * N_HID + N_HID + N_OUT * N_HID + N_OUT
PUSH, PULL, DENSE = 0, 1, 2
FORCE = {PUSH: 1, PULL: 2, DENSE: 3}  # DAWN_OPT_FORCE_VARIANT values
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "selector_weights.json")

assert N_WEIGHTS == 1475


def _f(x):
    return np.asarray(x, np.float64).astype(np.float32)


def _lg1p(x):
    return np.log2(np.float32(1.0) + np.maximum(_f(x), np.float32(0.0)))


def features(n, m, nf, mf, mu, level, prev_nf, nsrc):
    """The nine inputs of csrc/selector.cuh sel_features (single precision),
    vectorised."""
    n, m = _f(n), _f(m)
    nf, mf = _f(nf), _f(mf)
    ln, lm = _lg1p(n), _lg1p(m)
    x = np.stack([
        _lg1p(nf) / ln,
        _lg1p(mf) / lm,
        _lg1p(mu) / lm,
        np.broadcast_to(ln / np.float32(32.0), nf.shape),
        np.broadcast_to(_lg1p(m / np.maximum(n, np.float32(1.0))) / np.float32(8.0), nf.shape),
        _lg1p(level) / np.float32(12.0),
        _lg1p(prev_nf) / ln,
        _lg1p(mf / np.maximum(nf, np.float32(1.0))) / np.float32(16.0),
        np.broadcast_to(_f(nsrc) / np.float32(256.0), nf.shape),
    ], axis=-1)
    return x.astype(np.float32)


def _levels(recs):
    """(run, level) -> (frontier, frontier_edges, unvisited_edges, body ms)."""
    out = {}
    for r in recs:
        if r["level"] < 1 or "decide" in r["kernel"]:
            continue
        key = (r["run"], r["level"])
        f = out.get(key)
        if f is None:
            out[key] = [r["frontier"], r["frontier_edges"], r["unvisited_edges"], r["ms"]]
        else:
            f[3] += r["ms"]
    return out


def collect_one(dg, n, m, sources, batched, variants=None):
    """Rows (X, Y) of one traversal: Y[:, c] = log2(us) of variant c at that
    level, NaN where the traversal family has no such variant."""
    variants = variants or ([PUSH, PULL, DENSE] if batched else [PUSH, PULL])
    kind = abi.VARIANT_BITSET if batched else abi.VARIANT_DO
    per_var = {}
    for v in variants:
        dg.set_option(abi.OPT_FORCE_VARIANT, FORCE[v])
        dg.trace(True)
        dg.bfs_stats(sources, variant=kind)
        dg.trace(False)
        per_var[v] = _levels(dg.trace_read())
    dg.set_option(abi.OPT_FORCE_VARIANT, 0)
    keys = sorted(per_var[variants[0]])
    prev = {}
    for (run, lv) in keys:
        prev[(run, lv + 1)] = per_var[variants[0]][(run, lv)][0]
    rows_x, rows_y = [], []
    nb = len(sources) if batched else 1
    if batched:
        per = 64 * (4 if nb > 128 else 2 if nb > 64 else 1)
    for (run, lv) in keys:
        if lv < 2 or any((run, lv) not in per_var[v] for v in variants):
            continue
        fr, fe, ue, _ = per_var[variants[0]][(run, lv)]
        nsrc = min(per, nb - run * per) if batched else 1
        x = features(n, m, fr, fe, ue, lv, prev.get((run, lv), 0), nsrc)
        y = np.full(N_OUT, np.nan, np.float32)
        for v in variants:
            y[v] = np.log2(max(per_var[v][(run, lv)][3], 1e-4) * 1e3)
        rows_x.append(x)
        rows_y.append(y)
    return np.array(rows_x, np.float32).reshape(-1, N_IN), np.array(rows_y, np.float32).reshape(-1, N_OUT)


# --- the mixed family ---------------------------------------------------------

def family(split):
    """Seeded graph specs of the mixed family: RMAT scales 20-24 with a in
    [0.45, 0.65] (b = c = (1 - a - 0.05) / 2), the 2048 x 2048 4-neighbour
    grid and the 2^21-point kNN graph with k = 8.  'train' and 'heldout'
    draw different seeds (and different RMAT parameters)."""
    if split == "train":
        rng = np.random.default_rng(101)
        specs = [("rmat", int(s), float(a), int(rng.integers(1, 2**31)))
                 for s, a in ((20, 0.45), (20, 0.55), (20, 0.65), (21, 0.50), (21, 0.60), (22, 0.57))]
        specs += [("grid", 2048, 0.0, 1), ("knn", 21, 0.0, int(rng.integers(1, 2**31)))]
    elif split == "heldout":
        rng = np.random.default_rng(202)
        specs = [("rmat", int(s), float(a), int(rng.integers(1, 2**31)))
                 for s, a in ((20, 0.60), (21, 0.45), (22, 0.65), (23, 0.52), (24, 0.57))]
        specs += [("grid", 2048, 0.0, 2), ("knn", 21, 0.0, int(rng.integers(1, 2**31)))]
    else:
        raise ValueError(split)
    return specs


def build(spec):
    kind, size, a, seed = spec
    if kind == "rmat":
        d = 0.05
        b = c = (1.0 - a - d) / 2.0
        return gen.rmat(size, 16, a, b, c, seed=seed)
    if kind == "grid":
        return gen.grid(size, size, seed=seed)
    return gen.knn(1 << size, 8, seed=seed)


def spec_name(spec):
    kind, size, a, seed = spec
    return f"rmat{size}-a{a:.2f}" if kind == "rmat" else (f"grid{size}" if kind == "grid" else f"knn2^{size}")


def collect(split, batches=((64, 11), (64, 12), (64, 13), (256, 14)), nsrc_single=8, max_rows_per_run=64,
            log=print):
    """Traced forced-variant runs over the split's graphs: batched traversals
    of the given (sources, seed) batches and single-source traversals of
    nsrc_single sources.  Long traversals (grid, kNN) are thinned to
    max_rows_per_run levels per batch or source."""
    xs, ys, tags = [], [], []
    for spec in family(split):
        g = build(spec)
        runs = [(True, gen.sources(g, k, seed=spec[3] % 1000 + s)) for k, s in batches]
        runs.append((False, gen.sources(g, nsrc_single, seed=spec[3] % 1000 + 3)))
        with abi.Graph(g) as dg:
            for batched, ss in runs:
                t0 = time.time()
                x, y = collect_one(dg, g.n, g.m, ss, batched)
                cap = max_rows_per_run * (-(-len(ss) // 256) if batched else len(ss))
                if len(x) > cap:
                    keep = np.linspace(0, len(x) - 1, cap).astype(int)
                    x, y = x[keep], y[keep]
                xs.append(x)
                ys.append(y)
                tag = f"{spec_name(spec)}/{'bitset' if batched else 'single'}"
                tags += [tag] * len(x)
                log(f"{tag} ({len(ss)} sources): {len(x)} rows, {time.time() - t0:.1f}s")
        del g
    return np.concatenate(xs), np.concatenate(ys), np.array(tags)


# --- training (numpy, full-batch Adam on the squared error of the known entries) --

def init_params(rng):
    def he(fan_in, shape):
        return (rng.standard_normal(shape) * np.sqrt(2.0 / fan_in)).astype(np.float64)
    return [he(N_IN, (N_HID, N_IN)), np.zeros(N_HID), he(N_HID, (N_HID, N_HID)), np.zeros(N_HID),
            he(N_HID, (N_OUT, N_HID)), np.zeros(N_OUT)]


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = p
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    return h1, h2, h2 @ W3.T + b3


def train(x, y, epochs=4000, lr=3e-3, seed=0, log=print):
    rng = np.random.default_rng(seed)
    p = init_params(rng)
    p[5] = np.nanmean(y, axis=0)
    mask = ~np.isnan(y)
    yt = np.where(mask, y, 0.0)
    m = [np.zeros_like(a) for a in p]
    v = [np.zeros_like(a) for a in p]
    x = x.astype(np.float64)
    cnt = max(mask.sum(), 1)
    for t in range(1, epochs + 1):
        h1, h2, out = forward(p, x)
        err = np.where(mask, out - yt, 0.0)
        loss = float((err ** 2).sum() / cnt)
        g_out = 2.0 * err / cnt
        gW3 = g_out.T @ h2
        gb3 = g_out.sum(0)
        g_h2 = (g_out @ p[4]) * (h2 > 0)
        gW2 = g_h2.T @ h1
        gb2 = g_h2.sum(0)
        g_h1 = (g_h2 @ p[2]) * (h1 > 0)
        gW1 = g_h1.T @ x
        gb1 = g_h1.sum(0)
        grads = [gW1, gb1, gW2, gb2, gW3, gb3]
        for i, gr in enumerate(grads):
            m[i] = 0.9 * m[i] + 0.1 * gr
            v[i] = 0.999 * v[i] + 0.001 * gr * gr
            p[i] -= lr * (m[i] / (1 - 0.9 ** t)) / (np.sqrt(v[i] / (1 - 0.999 ** t)) + 1e-8)
        if log and (t % 1000 == 0 or t == 1):
            log(f"epoch {t}: mse {loss:.4f}")
    return p, loss


def flatten(p):
    w = np.concatenate([a.reshape(-1) for a in p]).astype(np.float32)
    assert w.size == N_WEIGHTS
    return w


def unflatten(w):
    w = np.asarray(w, np.float64)
    shapes = [(N_HID, N_IN), (N_HID,), (N_HID, N_HID), (N_HID,), (N_OUT, N_HID), (N_OUT,)]
    out, o = [], 0
    for s in shapes:
        k = int(np.prod(s))
        out.append(w[o:o + k].reshape(s))
        o += k
    return out


def pick(w, x, allowed=(PUSH, PULL, DENSE)):
    _, _, out = forward(unflatten(w), np.asarray(x, np.float64))
    masked = np.full_like(out, np.inf)
    for c in allowed:
        masked[:, c] = out[:, c]
    return masked.argmin(1)


def save(w, path, meta):
    with open(path, "w") as f:
        json.dump({"layout": "W1[32][9] b1[32] W2[32][32] b2[32] W3[3][32] b3[3]", "outputs":
                   ["sparse push", "bitmap pull", "dense push"], "target": "log2(level microseconds)",
                   "meta": meta, "weights": [float(v) for v in w]}, f, indent=0)


def load(path=DEFAULT_WEIGHTS):
    with open(path) as f:
        d = json.load(f)
    w = np.array(d["weights"], np.float32)
    if w.size != N_WEIGHTS:
        raise ValueError(f"{path}: {w.size} weights, expected {N_WEIGHTS}")
    return w


# --- evaluation: selector against the direction heuristics on held-out graphs --

def evaluate(w, split="heldout", nsrc=64, reps=3, margins=(250,), log=print):
    """Device time of each held-out traversal under the direction heuristic
    and under the selector (one row per margin, in thousandths of log2)."""
    import torch
    rows = []
    for spec in family(split):
        g = build(spec)
        srcs = gen.sources(g, nsrc, seed=spec[3] % 1000 + 5)
        s = torch.cuda.Stream()
        with abi.Graph(g, stream=s.cuda_stream) as dg:
            d = torch.empty((nsrc, g.n), dtype=torch.int32, device="cuda")
            for variant, name in ((abi.VARIANT_BITSET, "bitset"), (abi.VARIANT_DO, "single")):
                k = nsrc if variant == abi.VARIANT_BITSET else 8

                def best_of():
                    best = None
                    for _ in range(reps):
                        st = dg.bfs_device(srcs[:k], d.data_ptr(), variant=variant)
                        best = st.device_ms if best is None else min(best, st.device_ms)
                    return best, st
                dg.set_selector(None)
                h_ms, h_st = best_of()
                for margin in margins:
                    dg.set_selector(w)
                    dg.set_option(abi.OPT_SELECTOR_MARGIN, margin)
                    l_ms, l_st = best_of()
                    row = {"graph": spec_name(spec), "family": name, "sources": k, "margin": margin,
                           "heuristic_ms": round(h_ms, 4), "learned_ms": round(l_ms, 4),
                           "speedup": round(h_ms / l_ms, 3),
                           "gteps_learned": round(l_st.edges_traversed / l_ms / 1e6, 1),
                           "levels_push_pull": [l_st.push_levels, l_st.pull_levels],
                           "heuristic_push_pull": [h_st.push_levels, h_st.pull_levels]}
                    rows.append(row)
                    log(json.dumps(row))
                dg.set_selector(None)
        del g
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m dawn_gb300.selector")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--split", default="train")
    c.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("data", nargs="+")
    t.add_argument("--out", default=DEFAULT_WEIGHTS)
    t.add_argument("--epochs", type=int, default=4000)
    e = sub.add_parser("evaluate")
    e.add_argument("weights", nargs="?", default=DEFAULT_WEIGHTS)
    e.add_argument("--split", default="heldout")
    e.add_argument("--out")
    e.add_argument("--margins", default="250", help="comma-separated margins (thousandths of log2)")
    a = ap.parse_args(argv)
    if a.cmd == "collect":
        x, y, tags = collect(a.split)
        np.savez_compressed(a.out, x=x, y=y, tags=tags)
        print(f"{len(x)} rows -> {a.out}")
    elif a.cmd == "train":
        xs, ys, tags = [], [], []
        for path in a.data:
            z = np.load(path)
            xs.append(z["x"])
            ys.append(z["y"])
            tags += list(z["tags"])
        x, y = np.concatenate(xs), np.concatenate(ys)
        p, loss = train(x, y, epochs=a.epochs)
        w = flatten(p)
        # how often the trained choice is the measured fastest, and the time it
        # gives up against always taking the fastest
        best = np.nanargmin(np.where(np.isnan(y), np.inf, y), axis=1)
        allowed_rows = [(PUSH, PULL, DENSE) if not np.isnan(r[DENSE]) else (PUSH, PULL) for r in y]
        chosen = np.array([pick(w, x[i:i + 1], al)[0] for i, al in enumerate(allowed_rows)])
        t_best = np.exp2(np.take_along_axis(y, best[:, None], 1)[:, 0]).sum()
        t_sel = np.exp2(np.take_along_axis(y, chosen[:, None], 1)[:, 0]).sum()
        meta = {"rows": int(len(x)), "mse_log2us": round(loss, 5), "agree_with_fastest": round(float(
            np.mean(chosen == best)), 4), "time_vs_fastest": round(float(t_sel / t_best), 4),
            "sources": sorted(set(tags))}
        save(w, a.out, meta)
        print(json.dumps(meta))
    else:
        w = load(a.weights)
        rows = evaluate(w, a.split, margins=[int(v) for v in a.margins.split(",")])
        if a.out:
            with open(a.out, "w") as f:
                json.dump(rows, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
