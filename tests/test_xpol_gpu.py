"""Cross-polarisation spectrometer (two sources + cross spectrum) vs the restated
TaskCoreIPP::doMaths with num_sources = 2."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _two_recordings(nsub, T, seed, rho=0.4):
    """Two interleaved 2-bit recordings whose subbands share a common signal."""
    import synth

    rng = np.random.default_rng(seed)
    common = rng.standard_normal((T, nsub)).astype(np.float32)
    recs = []
    for _ in range(2):
        x = np.sqrt(rho) * common + np.sqrt(1 - rho) * rng.standard_normal((T, nsub)).astype(np.float32)
        recs.append(synth.pack2bit(synth.quantize_mark5b(x).reshape(-1)))
    return recs


@pytest.mark.parametrize("nsub,N,overlap,K,nspec,ch0,ch1", [(4, 1024, 2, 4, 3, 1, 1), (8, 4096, 1, 3, 2, 0, 5),
                                                            (16, 2048, 4, 2, 2, 15, 3), (1, 8192, 2, 2, 1, 0, 0)])
def test_xpol_vs_oracle(cg, orc, nsub, N, overlap, K, nspec, ch0, ch1):
    T = N * K * nspec
    r0, r1 = _two_recordings(nsub, T, seed=N + nsub)
    tb = 32
    p = cg.spec_params(N, overlap, 2, K, nspec, nsub, r0.size, tonebins=tb, rotatorlen=tb, fs_hz=32e6)
    power = np.zeros((2, nspec, N // 2 + 1), np.float32)
    xpol = np.zeros((nspec, N // 2 + 1), np.complex64)
    bins = np.zeros((2, nspec, tb), np.complex64)
    cg.spectrometer_xpol(p, r0, r1, ch0, ch1, power, xpol, bins)
    x0 = orc.unpack2bit(r0, T, nsub, orc.MARK5B_LUT)[ch0]
    x1 = orc.unpack2bit(r1, T, nsub, orc.MARK5B_LUT)[ch1]
    rp, rx, rb = orc.spectrometer_xpol(x0, x1, N, overlap, 2, K, tb, tb, 0.0, 32e6)
    assert _rel(power, rp) < TOL
    assert _rel(xpol, rx) < TOL
    assert np.all(xpol[:, 0].imag == 0) and np.all(xpol[:, -1].imag == 0)
    for s in range(2):
        if np.linalg.norm(rb[s]) == 0:
            assert np.all(bins[s] == 0)           # this source folds no window
        else:
            assert _rel(bins[s], rb[s]) < TOL
    # cross spectrum coherence of the shared signal (same channel index -> same common component)
    if ch0 == ch1:
        coh = np.abs(xpol[:, 1:-1]).sum() / np.sqrt(power[0, :, 1:-1].sum() * power[1, :, 1:-1].sum())
        assert coh > 0.2


def test_xpol_framed_and_device(cg, orc):
    """Framed Mark5B recordings on the device give the same spectra as their payloads."""
    import torch

    import synth

    nsub, N, K, nspec = 16, 2048, 4, 2
    T = N * K * nspec
    r0, r1 = _two_recordings(nsub, T, seed=9)
    pad = (-r0.size) % 10000
    f0 = synth.mark5b_frames(np.concatenate([r0, np.zeros(pad, np.uint8)]), prefix=40)
    f1 = synth.mark5b_frames(np.concatenate([r1, np.zeros(pad, np.uint8)]), prefix=40)
    pa = cg.spec_params(N, 2, 2, K, nspec, nsub, r0.size)
    a_pow = np.zeros((2, nspec, N // 2 + 1), np.float32)
    a_x = np.zeros((nspec, N // 2 + 1), np.complex64)
    cg.spectrometer_xpol(pa, r0, r1, 2, 7, a_pow, a_x)
    pf = cg.spec_params(N, 2, 2, K, nspec, nsub, f0.size, layout=cg.SPEC_MARK5B_FRAMED)
    b_pow = torch.zeros((2, nspec, N // 2 + 1), dtype=torch.float32, device="cuda")
    b_x = torch.zeros((nspec, N // 2 + 1), dtype=torch.complex64, device="cuda")
    cg.spectrometer_xpol(pf, torch.from_numpy(f0).cuda(), torch.from_numpy(f1).cuda(), 2, 7, b_pow, b_x)
    assert np.array_equal(a_pow, b_pow.cpu().numpy())
    assert np.array_equal(a_x, b_x.cpu().numpy())


def test_xpol_rejects(cg):
    r = np.zeros(1024 * 4, np.uint8)
    p = cg.spec_params(1024, 2, 2, 2, 1, 4, r.size)
    with pytest.raises(cg.CellspeError):
        cg.spectrometer_xpol(p, r, r, 0, 4, np.zeros((2, 1, 513), np.float32), np.zeros((1, 513), np.complex64))
    p = cg.spec_params(65536, 2, 2, 1, 1, 1, 65536 // 4)
    with pytest.raises(cg.CellspeError):
        cg.spectrometer_xpol(p, r, r, 0, 0, np.zeros((2, 1, 32769), np.float32), np.zeros((1, 32769), np.complex64))
