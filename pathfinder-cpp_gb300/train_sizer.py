"""Train the learned per-path sizer on the GPU and write its weight file.

    python pathfinder-cpp_gb300/train_sizer.py --out pathfinder-cpp_gb300/weights/sizer.bin

1. Training paths come from the single-scene generators (the 240-path cubic generator at
   every batched canvas side, the large mixed scene, the glyph scene, stroked scenes whose
   stroke outlines the upload builds) and from seeded SVG documents parsed by pf_svg_parse,
   about 2 M paths by default.  Each scene is rendered with the exact two-pass frame; its
   per-path features and exact leaf-line / fill counts are the inputs and labels
   (targets are log1p of the counts).
2. The MLP (12 -> 64 -> 64 -> 2, bf16 weights, fp32 accumulation) is trained with the
   library's own forward / backward / Adam kernels on standardised features; the
   standardisation is then folded into the first layer so the frame feeds raw features.
3. It is evaluated on a held-out mixed 8,192-path scene at 4096 x 4096 (seed 7): per-path
   overflow rate and over-allocation at the chosen margins, and the learned frame against
   the exact frame (identical output, time of each).
A JSON report is written next to the weights.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import pfcuda  # noqa: E402
import scenes as S  # noqa: E402

# parameter layout of the sizer (matches csrc/pf_sizer.cu)
N_IN, HIDDEN, N_OUT = 12, 64, 2


def _fold_standardisation(params: np.ndarray, mu: np.ndarray, sd: np.ndarray) -> np.ndarray:
    p = params.astype(np.float64).copy()
    w1 = p[:HIDDEN * N_IN].reshape(HIDDEN, N_IN)
    b1 = p[HIDDEN * N_IN:HIDDEN * N_IN + HIDDEN]
    b1 -= (w1 * (mu / sd)[None, :]).sum(1)
    w1 /= sd[None, :]
    return p.astype(np.float32)


def training_scenes(target_paths: int, seed0: int = 100):
    """Yield scenes from the three generators until about target_paths paths."""
    import svg_docs
    n = 0
    k = 0
    sides = (256, 512, 1024, 2048)
    while n < target_paths:
        kind = k % 6
        if kind in (0, 1):
            sc = S.plain_small(seed=seed0 + k, n_paths=2048, side=sides[(k // 6) % 4])
        elif kind == 2:
            sc = S.large_single(seed=seed0 + k, n_paths=20000, side=4096)
        elif kind == 3:
            sc = S.glyphs(seed=seed0 + k, n_paths=60000, side=2048)
        elif kind == 4:
            sc = S.stroked(seed=seed0 + k, n_paths=4096, side=sides[(k // 6) % 4], dash_share=0.3,
                           fill_share=0.2)
        else:
            sc = pfcuda.parse_svg(svg_docs.random_document(50_000 + k, n_shapes=(256, 1024, 4096)[(k // 6) % 3]))
        n += sc.n_paths
        k += 1
        yield sc


def collect(r: pfcuda.Renderer, scs):
    feats, labels = [], []
    for sc in scs:
        r.upload(sc)
        r.render()
        feats.append(r.path_features(sc.n_paths))
        leaves, fills = r.path_counts(sc.n_paths)
        labels.append(np.stack([leaves, fills], axis=1))
    return np.concatenate(feats), np.concatenate(labels)


def evaluate(r: pfcuda.Renderer, sc, mul: float, add: float, pool: float, repeats: int = 3):
    """Budgets vs exact counts on one scene, and the learned frame against the exact one."""
    r.upload(sc)
    r.render()
    feat = r.path_features(sc.n_paths)
    leaves, fills = r.path_counts(sc.n_paths)
    pred = r.sizer_predict(feat)
    budget = np.ceil(np.maximum(np.expm1(pred[:, 0]), 0) * mul + add)
    fill_est = np.ceil(np.maximum(np.expm1(pred[:, 1]), 0) * mul + add)
    over = leaves > budget
    spill = np.maximum(leaves - budget, 0).sum()
    r.sizer_margin(mul, add, pool)
    times = {}
    for name, fn in (("exact", r.render), ("learned", r.render_learned)):
        fn()
        t = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            st = fn()
            t.append(time.perf_counter() - t0)
        times[name] = {"ms": 1e3 * min(t), "syncs": st["host_syncs"], "launches": st["kernel_launches"],
                       "overflow": st["overflow"]}
    canon_l = r.canon(0)
    img_l = r.image(0)
    r.render()
    canon_e = r.canon(0)
    img_e = r.image(0)
    same = all(np.array_equal(canon_l[k], canon_e[k]) for k in canon_e) and np.array_equal(img_l, img_e)
    rel_err = np.abs(np.expm1(pred) - np.stack([leaves, fills], 1)) / np.maximum(np.stack([leaves, fills], 1), 1)
    return {
        "paths": int(sc.n_paths),
        "path_overflow_rate": float(over.mean()),
        "leaf_over_allocation": float((budget.sum() + pool * budget.sum()) / max(leaves.sum(), 1)),
        "fill_over_allocation": float(fill_est.sum() / max(fills.sum(), 1)),
        "spilled_leaves": int(spill),
        "pool_slots": int(pool * budget.sum()),
        "median_rel_err_leaves": float(np.median(rel_err[:, 0])),
        "median_rel_err_fills": float(np.median(rel_err[:, 1])),
        "frames": times,
        "learned_equals_exact": bool(same),
    }


def held_out_batches_():
    """Batches unlike any training scene's seeds: the benchmark's kinds at a smaller count."""
    import svg_docs
    yield "batched_64", S.batched(n_scenes=64, first_seed=9000)
    yield "batched_stroked_64", S.batched_stroked(n_scenes=64, first_seed=9100)
    rng = np.random.default_rng(9200)
    sizes = np.exp(rng.uniform(np.log(16), np.log(1024), 64)).astype(int)
    yield "svg_64", [pfcuda.parse_svg(svg_docs.random_document(9200 + i, n_shapes=int(sizes[i]))) for i in range(64)]


def evaluate_batch(r: pfcuda.Renderer, scs, repeats: int = 3):
    """The learned frame over a batch: overflow (frame redone exactly) and equality with the exact frame."""
    r.upload(scs)
    r.render()
    exact = [r.image(i) for i in range(len(scs))]
    over = [r.render_learned()["overflow"] for _ in range(repeats)]
    same = all(np.array_equal(r.image(i), exact[i]) for i in range(len(scs)))
    paths_over, pool_used = r.sizer_last_frame()
    return {"scenes": len(scs), "paths": int(sum(s.n_paths for s in scs)), "frames_redone_exactly": int(sum(over)),
            "paths_over_budget": int(paths_over), "spill_pool_slots_used": int(pool_used),
            "learned_equals_exact": bool(same)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "sizer.bin"))
    ap.add_argument("--paths", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--mul", type=float, default=1.15)
    ap.add_argument("--add", type=float, default=4.0)
    ap.add_argument("--pool", type=float, default=0.10)
    args = ap.parse_args()

    t0 = time.perf_counter()
    r = pfcuda.Renderer()
    x, counts = collect(r, training_scenes(args.paths))
    y = np.log1p(counts.astype(np.float32))
    t_collect = time.perf_counter() - t0
    # hold out 2 % of the training paths to watch generalisation
    rng = np.random.default_rng(0)
    perm = rng.permutation(len(x))
    n_val = max(1, len(x) // 50)
    val, tr = perm[:n_val], perm[n_val:]
    mu, sd = x[tr].mean(0), x[tr].std(0) + 1e-6
    r.sizer_init(seed=1)
    t1 = time.perf_counter()
    losses = r.sizer_train((x[tr] - mu) / sd, y[tr], epochs=args.epochs, batch=args.batch, lr=args.lr, seed=3)
    t_train = time.perf_counter() - t1
    r.set_sizer_params(_fold_standardisation(r.sizer_params(), mu, sd))
    r.sizer_margin(args.mul, args.add, args.pool)
    val_pred = r.sizer_predict(x[val])
    val_mse = float(((val_pred - y[val]) ** 2).mean())
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    r.sizer_save(args.out)

    held_out = evaluate(r, S.mixed(seed=7, n_paths=8192, side=4096), args.mul, args.add, args.pool)
    held_out_batches = {name: evaluate_batch(r, scs) for name, scs in held_out_batches_()}
    report = {
        "training_paths": int(len(tr)), "validation_paths": int(n_val), "epochs": args.epochs,
        "batch": args.batch, "lr": args.lr, "epoch_mse": [float(v) for v in losses],
        "validation_mse": val_mse, "collect_s": t_collect, "train_s": t_train,
        "margin": {"mul": args.mul, "add": args.add, "pool": args.pool},
        "held_out_mixed_8192_4096": held_out,
        "held_out_batches": held_out_batches,
    }
    with open(os.path.splitext(args.out)[0] + "_report.json", "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report))
    r.close()


if __name__ == "__main__":
    main()
