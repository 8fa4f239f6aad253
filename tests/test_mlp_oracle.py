"""CPU checks of the learned-restart network's oracle and packing (no GPU)."""
import numpy as np
import pytest

from oracle import mlp_oracle


def test_bf16_rounding_is_round_to_nearest_even():
    torch = pytest.importorskip("torch")
    a = np.random.default_rng(0).normal(size=20000).astype(np.float32) * 100
    a[:4] = [1.00390625, 1.01171875, -1.00390625, 3.0e-39]  # ties to even and a subnormal
    ref = torch.from_numpy(a).to(torch.bfloat16).float().numpy()
    assert np.array_equal(mlp_oracle.bf16(a).astype(np.float32), ref)


def test_parameter_packing_matches_the_library_layout():
    from reprobus_gb300 import mlp
    n = mlp.nparams()
    assert n == 64 * 256 + 256 + 2 * (256 * 256 + 256) + 256 * 64 + 64
    p = np.arange(n, dtype=np.float32)
    for (W, b), (Wo, bo) in zip(mlp.unpack(p), mlp_oracle.unpack(p)):
        assert np.array_equal(W, Wo) and np.array_equal(b, bo)


def test_oracle_gradient_matches_finite_differences():
    """The oracle's backward pass, with BF16 rounding switched off, against
    central differences of its own loss (float64)."""
    rng = np.random.default_rng(1)
    p = (rng.normal(size=sum(i * o + o for i, o in mlp_oracle.DIMS)) * 0.05).astype(np.float64)
    norm = np.concatenate([np.zeros(64), np.ones(64), np.zeros(64), np.ones(64)])
    X = rng.normal(size=(8, 64))
    Y = rng.normal(size=(8, 64))
    saved = mlp_oracle.bf16
    mlp_oracle.bf16 = lambda a: np.asarray(a, dtype=np.float64)
    try:
        _, g = mlp_oracle.loss_and_grads(p, norm, X, Y)
        for k in rng.choice(p.size, 12, replace=False):
            e = np.zeros_like(p)
            e[k] = 1e-6
            lp, _ = mlp_oracle.loss_and_grads(p + e, norm, X, Y)
            lm, _ = mlp_oracle.loss_and_grads(p - e, norm, X, Y)
            assert abs((lp - lm) / 2e-6 - g[k]) <= 1e-5 * max(1.0, abs(g[k])), k
    finally:
        mlp_oracle.bf16 = saved
