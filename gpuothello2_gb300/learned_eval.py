"""What the learned move orderer gains: train it, then solve the same
positions with and without it.

  python -m gpuothello2_gb300.learned_eval [--train N] [--eval N] [--empties E]
                                           [--epochs K] [--min-empties M]

1. training positions: seed 3, 12..14 empties, labelled with the solver's
   own best moves (exact search);
2. training: the library's GPU kernels (gpo_mlp_train, Adam, BF16 weights
   with FP32 accumulation);
3. evaluation: seed 4 positions at E empties (DEPTH = E), solved twice --
   fastest-first root ordering, then the network ordering the roots of
   positions with >= M empties.  Scores must be identical; the line reports
   the node counts, positions/s of both runs and how often the network's
   highest-scoring empty square is the solver's best move on held-out
   positions.

Defaults are the full-size learned-ordering configuration: 4,194,304
training positions, 262,144 evaluation positions at 18 empties.  Prints one
JSON line.
"""
import argparse
import json
import sys
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=1 << 22)
    ap.add_argument("--eval", type=int, default=1 << 18)
    ap.add_argument("--empties", type=int, default=18)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--min-empties", type=int, default=14)
    args = ap.parse_args(argv)

    import gpuothello2_gb300 as g

    t0 = time.perf_counter()
    tp, to = g.generate(3, args.train, 12, 14)
    _, labels, _, _, _ = g.solve(tp, to, 14, best=True)
    t_label = time.perf_counter() - t0
    t0 = time.perf_counter()
    w, hist = g.mlp_train(tp, to, labels, g.mlp_init(3), epochs=args.epochs, batch=2048,
                          lr=1e-3, seed=1)
    t_train = time.perf_counter() - t0

    # held-out top-1 agreement, the network's best empty square
    hp, ho = g.generate(33, 8192, 12, 14)
    _, hb, _, _, _ = g.solve(hp, ho, 14, best=True)
    z = g.mlp_forward(w, hp, ho)
    hits = total = 0
    for i in range(len(hp)):
        if hb[i] >= 64:
            continue
        occ = int(hp[i]) | int(ho[i])
        masked = np.where([(occ >> k) & 1 == 0 for k in range(64)], z[i], -np.inf)
        total += 1
        hits += int(np.argmax(masked)) == int(hb[i])

    ep, eo = g.generate(4, args.eval, args.empties, args.empties)
    runs = {}
    for name, learned in (("fastest_first", 0), ("learned", 1)):
        if learned:
            g.mlp_load(w)
        try:
            t0 = time.perf_counter()
            sc, _, _, st, _ = g.solve(ep, eo, args.empties, use_learned=learned,
                                      learned_min_empties=args.min_empties)
            dt = time.perf_counter() - t0
        finally:
            if learned:
                g.mlp_load(None)
        runs[name] = {"scores": sc, "nodes": int(st.nodes), "seconds": dt,
                      "positions_per_s": args.eval / dt, "learned_calls": int(st.learned_calls)}
    same = bool(np.array_equal(runs["fastest_first"]["scores"], runs["learned"]["scores"]))
    for r in runs.values():
        del r["scores"]
    line = {
        "train_positions": args.train, "label_s": t_label, "train_s": t_train,
        "loss_accuracy_per_epoch": hist,
        "heldout_top1": hits / max(1, total),
        "eval_positions": args.eval, "empties": args.empties,
        "min_empties": args.min_empties, "scores_identical": same,
        "runs": runs,
        "node_ratio": runs["learned"]["nodes"] / max(1, runs["fastest_first"]["nodes"]),
    }
    print(json.dumps(line), flush=True)
    return 0 if same else 1


if __name__ == "__main__":
    sys.exit(main())
