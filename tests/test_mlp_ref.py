"""CPU checks of the presize MLP reference (the checker of the GPU training
and inference kernels): its gradient against central finite differences and
its BF16 rounding."""
import numpy as np

from oracle import mlp_ref


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.2, mlp_ref.N_PARAMS)
    X = rng.uniform(0, 1.5, (40, mlp_ref.IN))
    t = rng.uniform(0, 6, 40)
    _, g = mlp_ref.loss_grad(p, X, t, huber=0.7)
    idx = rng.choice(mlp_ref.N_PARAMS, 60, replace=False)
    idx = np.concatenate([idx, [mlp_ref.N_PARAMS - 1, 0, 4096]])
    eps = 1e-6
    for k in idx:
        q = p.copy()
        q[k] += eps
        lp, _ = mlp_ref.loss_grad(q, X, t, huber=0.7)
        q[k] -= 2 * eps
        lm, _ = mlp_ref.loss_grad(q, X, t, huber=0.7)
        assert abs((lp - lm) / (2 * eps) - g[k]) < 1e-6 + 1e-5 * abs(g[k]), k


def test_parameter_count_and_layout():
    assert mlp_ref.N_PARAMS == 20865
    p = np.arange(mlp_ref.N_PARAMS, dtype=np.float64)
    w = mlp_ref.unpack(p)
    assert w["w1"][1, 0] == 32 and w["b1"][0] == 4096 and w["w2"][0, 0] == 4224
    assert w["b3"][0] == mlp_ref.N_PARAMS - 1
    assert np.array_equal(mlp_ref.pack(w), p)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 0.0, 65504.0], np.float32)
    b = mlp_ref.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 1.5 * 2^-8 rounds up
    assert b[0] == 1.0 and b[1] == 1.0 and b[2] == 1.0078125 and b[3] == 1.0078125
    assert b[4] == np.float32(-3.140625) and b[5] == 0.0 and b[6] == 65536.0
