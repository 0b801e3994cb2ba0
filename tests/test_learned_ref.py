"""The CPU reference of the learned orderer (tests/mlp_ref.py) is itself
checked against finite differences, without rounding (float64)."""
import numpy as np

from tests import mlp_ref


def test_reference_gradient_matches_finite_differences(oracle):
    rng = np.random.default_rng(0)
    n_params = sum(int(np.prod(s)) for _, s in mlp_ref.SHAPES)
    w = rng.normal(0, 0.1, n_params)
    p, o = oracle.generate(3, 24, 12, 14)
    legal = np.array([oracle.L.orc_mobility(int(a), int(b)) for a, b in zip(p, o)], np.uint64)
    label = np.array([int(np.log2(int(m) & -int(m))) if m else 65 for m in legal])
    X = mlp_ref.features(p, o, legal).astype(np.float64)

    def loss_at(wv):
        q = mlp_ref.unpack(wv.astype(np.float64))
        H1 = np.maximum(X @ q["W1"] + q["b1"], 0)
        H2 = np.maximum(H1 @ q["W2"] + q["b2"], 0)
        Z = H2 @ q["W3"] + q["b3"]
        total = 0.0
        for i, y in enumerate(label):
            m = [k for k in range(64) if (int(legal[i]) >> k) & 1]
            if y >= 64 or not m:
                continue
            zs = Z[i, m]
            total -= Z[i, y] - (zs.max() + np.log(np.exp(zs - zs.max()).sum()))
        return total / len(X)

    _, g = mlp_ref.loss_and_gradients(w, X, legal, label, rnd=False)
    for idx in rng.choice(n_params, 40, replace=False):
        e = np.zeros(n_params)
        e[idx] = 1e-6
        fd = (loss_at(w + e) - loss_at(w - e)) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 + 1e-4 * abs(fd), idx
