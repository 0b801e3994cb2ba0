"""Train the learned move orderer, and measure what it gains.

  python -m gpuothello2_gb300.learned_eval train [--train N] [--epochs K] [--out FILE]
  python -m gpuothello2_gb300.learned_eval eval [--weights FILE] [--eval N] [--empties E]
                                                [--min-empties M]

train: positions of seed 3 at 12..14 empties (default 4,194,304, the
learned-ordering configuration) labelled with the solver's own best moves
(exact search on the GPU), then the library's GPU training kernels
(gpo_mlp_train: BF16 tensor-core products, FP32 accumulation, Adam) for K
epochs; writes the FP32 weights (gpo_mlp_param_count floats, little endian)
to FILE and prints one JSON line with the loss and accuracy per epoch and
the held-out top-1 agreement with the solver's best move at 14 and 16
empties next to the fastest-first rule's.

eval: positions of seed 4 at E empties (DEPTH = E) solved twice with the
same options -- fastest-first ordering, then the network ordering every
node with >= M empties in the top two plies -- scores must be identical;
prints node counts, kernel times and their ratios.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "orderer.f32")


def _top1(g, w, empties, n=4096):
    """Held-out top-1 agreement with the solver's best move: the network's
    highest-scoring legal move, and the fastest-first rule's choice (fewest
    opponent replies, corners first on ties)."""
    p, o = g.generate(33, n, empties, empties)
    _, best, _, _, _ = g.solve(p, o, empties, best=True)
    z = g.mlp_forward(w, p, o)
    hits = ff = total = 0
    for i in range(n):
        b = int(best[i])
        if b >= 64:
            continue
        P, O = int(p[i]), int(o[i])
        moves = [k for k in range(64) if _legal(P, O, k)]
        if not moves:
            continue
        total += 1
        hits += moves[int(np.argmax(z[i, moves]))] == b
        ff += min(moves, key=lambda k: _ff_key(P, O, k)) == b
    return hits / max(1, total), ff / max(1, total)


_DIRS = ((0, 1), (0, -1), (1, 0), (-1, 0), (1, 1), (1, -1), (-1, 1), (-1, -1))


def _flips(P, O, sq):
    out = 0
    for dr, dc in _DIRS:
        r, c, run = sq // 8 + dr, sq % 8 + dc, 0
        while 0 <= r < 8 and 0 <= c < 8 and (O >> (r * 8 + c)) & 1:
            run |= 1 << (r * 8 + c)
            r, c = r + dr, c + dc
        if 0 <= r < 8 and 0 <= c < 8 and (P >> (r * 8 + c)) & 1:
            out |= run
    return out


def _legal(P, O, sq):
    return not ((P | O) >> sq) & 1 and _flips(P, O, sq) != 0


def _ff_key(P, O, sq):
    f = _flips(P, O, sq)
    cP, cO = O ^ f, P ^ f ^ (1 << sq)
    replies = sum(1 for k in range(64) if _legal(cP, cO, k))
    return 2 * replies + (0 if sq in (0, 7, 56, 63) else 1)


def train(args):
    import gpuothello2_gb300 as g

    t0 = time.perf_counter()
    tp, to = g.generate(3, args.train, 12, 14)
    _, labels, _, _, _ = g.solve(tp, to, 14, best=True)
    t_label = time.perf_counter() - t0
    t0 = time.perf_counter()
    w, hist = g.mlp_train(tp, to, labels, g.mlp_init(3), epochs=args.epochs, batch=args.batch,
                          lr=args.lr, seed=1)
    t_train = time.perf_counter() - t0
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.asarray(w, np.float32).tofile(args.out)
    acc = {}
    for e in (14, 16):
        learned, ff = _top1(g, w, e, 2048)
        acc[str(e)] = {"learned": learned, "fastest_first": ff}
    print(json.dumps({"train_positions": args.train, "epochs": args.epochs, "batch": args.batch,
                      "lr": args.lr, "label_s": t_label, "train_s": t_train,
                      "loss_accuracy_per_epoch": hist, "heldout_top1": acc,
                      "weights": args.out, "params": int(len(w))}), flush=True)
    return 0


def evaluate(args):
    import gpuothello2_gb300 as g

    w = np.fromfile(args.weights, dtype=np.float32)
    ep, eo = g.generate(4, args.eval, args.empties, args.empties)
    runs = {}
    scores = {}
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
        scores[name] = sc
        runs[name] = {"nodes": int(st.nodes), "kernel_ms": st.kernel_ms, "seconds": dt,
                      "positions_per_s": args.eval / dt, "frontier": int(st.learned_calls)}
    same = bool(np.array_equal(scores["fastest_first"], scores["learned"]))
    print(json.dumps({
        "eval_positions": args.eval, "empties": args.empties, "min_empties": args.min_empties,
        "weights": args.weights, "scores_identical": same, "runs": runs,
        "node_ratio": runs["learned"]["nodes"] / max(1, runs["fastest_first"]["nodes"]),
        "time_ratio": runs["learned"]["seconds"] / max(1e-9, runs["fastest_first"]["seconds"]),
    }), flush=True)
    return 0 if same else 1


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--train", type=int, default=1 << 22)
    t.add_argument("--epochs", type=int, default=8)
    t.add_argument("--batch", type=int, default=4096)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--out", default=DEFAULT_WEIGHTS)
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=DEFAULT_WEIGHTS)
    e.add_argument("--eval", type=int, default=1 << 15)
    e.add_argument("--empties", type=int, default=18)
    e.add_argument("--min-empties", type=int, default=14)
    args = ap.parse_args(argv)
    return train(args) if args.cmd == "train" else evaluate(args)


if __name__ == "__main__":
    sys.exit(main())
