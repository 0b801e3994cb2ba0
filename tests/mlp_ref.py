"""CPU reference of the learned move orderer (mlp.cu) -- the checker for its
forward and backward kernels.  numpy FP32 arithmetic with BF16 rounding
applied exactly where the GPU rounds (weights, hidden activations, the
back-propagated deltas), so the two agree to FP32 summation-order error."""
import numpy as np

N_IN, N_H, N_OUT = 192, 256, 64
SHAPES = [("W1", (N_IN, N_H)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)),
          ("W3", (N_H, N_OUT)), ("b3", (N_OUT,))]


def unpack(w):
    out, off = {}, 0
    dt = np.float64 if np.asarray(w).dtype == np.float64 else np.float32
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = np.asarray(w[off:off + size], dt).reshape(shape)
        off += size
    assert off == len(w)
    return out


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def features(player, opp, legal):
    bits = np.arange(64, dtype=np.uint64)
    cols = [((np.asarray(a, np.uint64)[:, None] >> bits) & 1) for a in (player, opp, legal)]
    return np.concatenate(cols, axis=1).astype(np.float32)


def forward(w, X, round_weights=True):
    q = unpack(w) if round_weights else {k: np.asarray(v, np.float64) for k, v in unpack(w).items()}
    r = bf16 if round_weights else (lambda a: np.asarray(a, np.float64))
    H1 = r(np.maximum(X @ r(q["W1"]) + q["b1"], 0))
    H2 = r(np.maximum(H1 @ r(q["W2"]) + q["b2"], 0))
    Z = H2 @ r(q["W3"]) + q["b3"]
    return H1, H2, Z


def loss_and_gradients(w, X, legal, label, rnd=True):
    q = unpack(w) if rnd else {k: np.asarray(v, np.float64) for k, v in unpack(w).items()}
    r = bf16 if rnd else (lambda a: np.asarray(a, np.float64))
    H1, H2, Z = forward(w, X, round_weights=rnd)
    n = len(X)
    mask = ((np.asarray(legal, np.uint64)[:, None] >> np.arange(64, dtype=np.uint64)) & 1).astype(bool)
    use = np.array([lg != 0 and 0 <= y < 64 and mask[i, y] for i, (lg, y) in enumerate(zip(legal, label))])
    Zm = np.where(mask, Z, -np.inf)
    mx = Zm.max(axis=1, keepdims=True)
    mx[~np.isfinite(mx)] = 0
    e = np.where(mask, np.exp(Z - mx), 0.0)
    P = e / np.maximum(e.sum(axis=1, keepdims=True), 1e-30)
    onehot = np.zeros_like(P)
    for i, y in enumerate(label):
        if use[i]:
            onehot[i, y] = 1.0
    D3 = r(np.where(use[:, None] & mask, (P - onehot) / n, 0.0))
    loss = -sum(np.log(P[i, y]) for i, y in enumerate(label) if use[i]) / n
    W2, W3 = r(q["W2"]), r(q["W3"])
    D2 = r((D3 @ W3.T) * (H2 > 0))
    D1 = r((D2 @ W2.T) * (H1 > 0))
    g = {"W3": H2.T @ D3, "b3": D3.sum(0), "W2": H1.T @ D2, "b2": D2.sum(0),
         "W1": X.T @ D1, "b1": D1.sum(0)}
    flat = np.concatenate([np.asarray(g[name], np.float64).ravel() for name, _ in SHAPES])
    return loss, flat
