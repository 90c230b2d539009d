"""The MLP oracle's FP64 gradients against central finite differences."""
import numpy as np

from oracle import mlp_ref


def test_mlp_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    M, d, H, C = 6, 5, 4, 7
    X = rng.standard_normal((M, d))
    y = rng.integers(0, C, M)
    P = {"W1": rng.standard_normal((H, d)) * 0.5, "b1": rng.standard_normal(H) * 0.1,
         "W2": rng.standard_normal((H, H)) * 0.5, "b2": rng.standard_normal(H) * 0.1,
         "W3": rng.standard_normal((C, H)) * 0.5, "b3": rng.standard_normal(C) * 0.1}

    def L(p):
        lr, _ = mlp_ref.loss_and_grads(X, y, p["W1"], p["b1"], p["W2"], p["b2"], p["W3"], p["b3"],
                                       bf=False)
        return lr.mean()

    _, g = mlp_ref.loss_and_grads(X, y, P["W1"], P["b1"], P["W2"], P["b2"], P["W3"], P["b3"], bf=False)
    eps = 1e-6
    for name, w in P.items():
        num = np.zeros_like(w)
        it = np.nditer(w, flags=["multi_index"])
        for _ in it:
            i = it.multi_index
            old = w[i]
            w[i] = old + eps
            lp = L(P)
            w[i] = old - eps
            lm = L(P)
            w[i] = old
            num[i] = (lp - lm) / (2 * eps)
        assert np.allclose(g[name], num, rtol=1e-5, atol=1e-7), name


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38], np.float32)
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == -2.5
