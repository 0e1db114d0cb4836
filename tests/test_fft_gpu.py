"""K-b: batched C2C / R2C FFTs vs the FP64 DFT and the FP32 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5   # relative L2, FP32 transform vs FP64 / vs the FP32 CPU path


@pytest.mark.parametrize("n", [16, 32, 64, 256, 1024, 4096, 16384])
def test_c2c_vs_fp64(cg, orc, n):
    rng = np.random.default_rng(n)
    batch = 3
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    out = np.zeros_like(x)
    cg.fft_c2c(x, out, n, batch)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < TOL
    cpu = np.stack([orc.cfft_f32(r) for r in x])
    assert np.linalg.norm(out - cpu) / np.linalg.norm(cpu) < TOL


@pytest.mark.parametrize("n", [32, 128, 1024, 2048, 8192, 32768])
def test_r2c_vs_fp64(cg, orc, n):
    rng = np.random.default_rng(n + 1)
    batch = 5
    x = rng.standard_normal((batch, n)).astype(np.float32)
    out = np.zeros((batch, n // 2 + 1), np.complex64)
    cg.fft_r2c(x, out, n, batch)
    ref = np.fft.rfft(x.astype(np.float64), axis=1)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < TOL
    assert np.all(out[:, 0].imag == 0) and np.all(out[:, -1].imag == 0)
    cpu = np.stack([orc.rfft_f32(r) for r in x])
    assert np.linalg.norm(out - cpu) / np.linalg.norm(cpu) < TOL


def test_fft_impulse_and_tone_known_answers(cg):
    n = 1024
    x = np.zeros((2, n), np.complex64)
    x[0, 0] = 1.0                                   # impulse -> flat
    x[1] = np.exp(2j * np.pi * 37 * np.arange(n) / n)  # tone -> bin 37, height n
    out = np.zeros_like(x)
    cg.fft_c2c(x, out, n, 2)
    assert np.allclose(out[0], 1.0, atol=1e-6)
    assert abs(out[1, 37] - n) < 1e-3 and np.abs(np.delete(out[1], 37)).max() < 1e-3


def test_fft_large_batch_device(cg):
    import torch

    n, batch = 2048, 4099
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((batch, n), device="cuda", generator=g)
    out = torch.zeros((batch, n // 2 + 1), dtype=torch.complex64, device="cuda")
    cg.fft_r2c(x, out, n, batch)
    ref = torch.fft.rfft(x.double(), dim=1)
    err = (torch.linalg.norm(out.to(torch.complex128) - ref) / torch.linalg.norm(ref)).item()
    assert err < TOL


@pytest.mark.parametrize("n,batch", [(32, 3), (2048, 5), (32768, 2)])
def test_fft_r2c_perm_packing(cg, n, batch):
    """IPP Perm rows as TaskCoreIPP::doMaths reads them (TaskCoreIPP.cpp:438-439:
    element 0 the DC bin, element 1 the Nyquist bin, then Re/Im pairs of bins
    1..n/2-1), against an FP64 real FFT; host and device buffers."""
    import torch

    rng = np.random.default_rng(n + batch)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    out = np.zeros((batch, n), np.float32)
    cg.fft_r2c_perm(x, out)
    X = np.fft.rfft(x.astype(np.float64), axis=1)
    ref = np.empty((batch, n))
    ref[:, 0] = X[:, 0].real
    ref[:, 1] = X[:, n // 2].real
    ref[:, 2::2] = X[:, 1:n // 2].real
    ref[:, 3::2] = X[:, 1:n // 2].imag
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-5
    xd, od = torch.from_numpy(x).cuda(), torch.zeros((batch, n), dtype=torch.float32, device="cuda")
    cg.fft_r2c_perm(xd, od)
    assert np.array_equal(od.cpu().numpy(), out)
