"""GPU checks of the tensor-core (tcgen05) kernels of the learned restart:
the BF16 GEMM against an FP32 product of the same BF16 operands."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(lib_built):
    from reprobus_gb300 import chem
    L = chem.load_library()
    L.reprobus_tc_gemm_test.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3 + [ctypes.c_void_p] * 2
    return L


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 256, 128), (200, 64, 256), (384, 48, 64)])
def test_tc_gemm_matches_fp32_product(lib, M, N, K):
    g = torch.Generator().manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    C = torch.full((M, N), float("nan"), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.reprobus_tc_gemm_test(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, err.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0 and int(err.item()) == 0
    ref = A.float() @ B.float().T
    assert torch.allclose(C, ref, rtol=1e-4, atol=1e-3 * float(ref.abs().max())), float((C - ref).abs().max())


@pytest.fixture(scope="module")
def mlp_mod(lib_built):
    from reprobus_gb300 import mlp
    return mlp


def _batch(B, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(B, 64)).astype(np.float32) * 3 + 1
    Y = rng.normal(size=(B, 64)).astype(np.float32)
    return X, Y


def _norm(seed):
    rng = np.random.default_rng(seed)
    n = np.concatenate([rng.normal(size=64) * 0.5 + 1, rng.uniform(1, 4, 64), rng.normal(size=64) * 0.1,
                        rng.uniform(0.5, 2, 64), np.zeros(64)]).astype(np.float32)
    return n


def test_mlp_gradients_match_the_cpu_oracle(mlp_mod):
    from oracle import mlp_oracle
    net = mlp_mod.Mlp(batch_cap=512, seed=3)
    p, _ = net.get_params()
    p[:] += np.random.default_rng(4).normal(size=p.size).astype(np.float32) * 0.01  # non-zero biases
    norm = _norm(5)
    net.set_params(p, norm)
    X, Y = _batch(384, 6)
    g, loss = net.grads(torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda())
    loss_ref, g_ref = mlp_oracle.loss_and_grads(p, norm, X, Y)
    assert abs(loss - loss_ref) <= 2e-3 * loss_ref
    o = 0
    for i, n in mlp_oracle.DIMS:
        for size in (i * n, n):
            a, b = g[o:o + size].astype(np.float64), g_ref[o:o + size]
            assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-12, (i, n, size)
            o += size
    net.close()


def test_mlp_inference_kernel_matches_the_cpu_oracle(mlp_mod):
    from oracle import mlp_oracle
    net = mlp_mod.Mlp(batch_cap=128, seed=7)
    p, _ = net.get_params()
    p[:] += np.random.default_rng(8).normal(size=p.size).astype(np.float32) * 0.01
    norm = _norm(9)
    net.set_params(p, norm)
    X, _ = _batch(1000, 10)  # ragged: 7 full tiles of 128 and one of 104 rows
    Yg = torch.zeros(1000, 64, device="cuda")
    net.forward(torch.from_numpy(X).cuda(), Yg)
    ref = mlp_oracle.forward(p, norm, X)
    got = Yg.cpu().numpy()
    scale = np.abs(ref[:, :57]).max()
    assert np.abs(got[:, 57:]).max() == 0.0
    assert np.abs(got[:, :57] - ref[:, :57]).max() <= 2e-2 * scale
    net.close()


def test_mlp_training_fits_a_smooth_map(mlp_mod):
    net = mlp_mod.Mlp(batch_cap=1024, seed=11)
    rng = np.random.default_rng(12)
    X = rng.uniform(-2, 2, size=(65536, 64)).astype(np.float32)
    M = rng.normal(size=(64, 64)).astype(np.float32) / 8
    Y = np.tanh(X @ M).astype(np.float32)
    Y[:, 57:] = 0
    Xt, Yt = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    net.set_params(None, mlp_mod.normalisation(Xt, Yt))
    hist = mlp_mod.train(net, Xt, Yt, steps=600, batch=1024, lr=2e-3)
    assert np.mean(hist[-20:]) < 0.15 * np.mean(hist[:5])
    net.close()
