"""K-d1: FP32 X stage vs the CPU path (genericAddProduct_32fc_conj looped over products)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _cpu_vis(orc, spec):
    C, S, K = spec.shape
    P = S * (S + 1) // 2
    vis = np.zeros((C, P), np.complex64)
    for i in range(S):
        for j in range(i + 1):
            acc = np.zeros(C, np.complex64)
            for k in range(K):
                orc.addproduct(np.ascontiguousarray(spec[:, i, k]), np.ascontiguousarray(spec[:, j, k]), acc, True)
            vis[:, orc.tri_index(i, j)] = acc
    return vis


@pytest.mark.parametrize("S,C,K", [(1, 4, 5), (2, 16, 64), (5, 8, 33), (70, 3, 40), (130, 2, 17)])
def test_xmac_vs_cpu(cg, orc, S, C, K):
    rng = np.random.default_rng(S * 100 + K)
    spec = (rng.standard_normal((C, S, K)) + 1j * rng.standard_normal((C, S, K))).astype(np.complex64)
    P = S * (S + 1) // 2
    vis = np.zeros((C, P), np.complex64)
    cg.xmac(spec, S, C, K, vis)
    ref = _cpu_vis(orc, spec)
    assert np.linalg.norm(vis - ref) / np.linalg.norm(ref) < TOL
    # autos are real and non-negative
    for i in range(S):
        a = vis[:, orc.tri_index(i, i)]
        assert np.all(a.real >= 0) and np.abs(a.imag).max() <= 1e-5 * np.abs(a.real).max()


def test_xmac_accumulate(cg):
    rng = np.random.default_rng(7)
    C, S, K = 4, 9, 16
    spec = (rng.standard_normal((C, S, K)) + 1j * rng.standard_normal((C, S, K))).astype(np.complex64)
    P = S * (S + 1) // 2
    v1 = np.zeros((C, P), np.complex64)
    cg.xmac(spec, S, C, K, v1)
    v2 = v1.copy()
    cg.xmac(spec, S, C, K, v2, accumulate=True)
    assert np.allclose(v2, 2 * v1, rtol=1e-6, atol=1e-5)
