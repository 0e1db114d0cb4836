"""Full FX path (K-a + K-b + K-c + K-d1) vs the oracle: FP32 CPU path and FP64 model."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5   # FP32 GPU path vs the FP32 CPU path / FP64 model, relative L2


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("S,N,K", [(3, 512, 40), (2, 1024, 64), (4, 2048, 40), (3, 4096, 9), (5, 8192, 4),
                                   (2, 32768, 2), (3, 2048, 13)])
def test_fx_fp32_vs_cpu_path(cg, orc, S, N, K):
    import synth

    raw = synth.stations_offset_binary(S, N * K, rho=0.2, lags=np.arange(S) % 4, seed=S + N)
    p = cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_BASELINE_MAJOR)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis)
    ref = orc.fx_fp32(raw, S, N, K)
    assert _rel(vis, ref) < TOL


def test_config1_lag_known_answer(cg, orc):
    """Config 1: 2 stations, 2^22 samples each, 1024-pt FFT, station 2 lags by 3 samples.

    V_10 = X_1 conj(X_0) with x_1(t) = c(t - 3) has phase -2 pi 3 k / N; its
    lag spectrum (inverse FFT over channels) peaks at lag +3.
    """
    import synth

    S, N, K = 2, 1024, 4096
    raw = synth.stations_offset_binary(S, N * K, rho=0.1, lags=[0, 3], seed=1)
    p = cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_BASELINE_MAJOR)
    vis = np.zeros((3, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis)
    cross = vis[orc.tri_index(1, 0)].astype(np.complex128)
    k = np.arange(N // 2)
    derot = (cross * np.exp(2j * np.pi * 3 * k / N))[16:-16].reshape(-1, 16).sum(axis=1)
    assert np.abs(np.angle(derot)).max() < 0.15
    lag = np.fft.ifft(cross, n=N)
    assert int(np.argmax(np.abs(lag))) == 3
    coh = np.abs(cross) / np.sqrt(vis[0].real * vis[2].real)
    assert 0.06 < np.median(coh) < 0.12                        # 2-bit coherence ~ 0.88 rho


def test_fx_delay_model_vs_oracle(cg, orc):
    import synth

    S, N, K = 3, 2048, 24
    fs, lo = 32e6, 8.4e9
    margin = 4096
    T = N * K + 2 * margin
    raw = synth.stations_offset_binary(S, T, rho=0.3, seed=9)
    rng = np.random.default_rng(4)
    poly = np.zeros((S, 4))
    poly[:, 0] = rng.uniform(-40e-6, 40e-6, S)     # +-1280 samples
    poly[:, 1] = rng.uniform(-3e-6, 3e-6, S)
    poly[:, 2] = rng.uniform(-1e-9, 1e-9, S)
    p = cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_BASELINE_MAJOR, start_sample=margin,
                     fs_hz=fs, lo_hz=lo)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis, delay_poly=poly)
    shift, ph0, dph = orc.delay_state_f64(poly, N, K, fs, lo)
    c = np.arange(N // 2)
    phasor = np.exp(1j * (ph0.astype(np.float32)[:, :, None].astype(np.float64) +
                          c[None, None, :] * dph.astype(np.float32)[:, :, None].astype(np.float64))).astype(np.complex64)
    ref = orc.fx_fp32(raw, S, N, K, start_sample=margin, shift=shift, phasor=phasor)
    assert _rel(vis, ref) < TOL
    # and against the FP64 model
    X = orc.fx_spectra_f64(raw, S, N, K, margin, shift, ph0, dph)
    pairs = [(i, j) for i in range(S) for j in range(i + 1)]
    ref64 = orc.fx_vis_f64(X, pairs)
    assert _rel(vis, ref64) < TOL


def test_fx_layouts_memory_and_accumulate(cg):
    import torch

    import synth

    S, N, K = 6, 1024, 16
    raw = synth.stations_offset_binary(S, N * K, rho=0.1, seed=3)
    P, C = S * (S + 1) // 2, N // 2
    vb = np.zeros((P, C), np.complex64)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_BASELINE_MAJOR), raw, vb)
    vc = np.zeros((C, P), np.complex64)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_CHANNEL_MAJOR), raw, vc)
    assert np.array_equal(vb, vc.T)
    d_raw = torch.from_numpy(raw).cuda()
    d_vis = torch.zeros((C, P), dtype=torch.complex64, device="cuda")
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1]), d_raw, d_vis)
    assert np.array_equal(d_vis.cpu().numpy(), vc)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], accumulate=True), raw, vc)
    assert np.allclose(vc, 2 * d_vis.cpu().numpy(), rtol=1e-6, atol=1e-4)


def test_fx_rejects_bad_jobs(cg):
    raw = np.zeros((2, 1024), np.uint8)
    vis = np.zeros((3, 512), np.complex64)
    with pytest.raises(cg.CellspeError) as e:     # unsupported FFT size
        cg.fx_correlate(cg.fx_params(2, 1000, 1, 1024), raw, vis)
    assert e.value.code == cg.ERR_ARG
    with pytest.raises(cg.CellspeError) as e:     # segments past the end of the data
        cg.fx_correlate(cg.fx_params(2, 1024, 5, 1024), raw, vis)
    assert e.value.code == cg.ERR_ARG
    cg.lib().cellspe_set_hbm_budget(1 << 10)      # admission control
    try:
        with pytest.raises(cg.CellspeError) as e:
            cg.fx_correlate(cg.fx_params(2, 1024, 4, 1024), raw, vis)
        assert e.value.code == cg.ERR_NOMEM
    finally:
        cg.lib().cellspe_set_hbm_budget(0)


def test_xf_lags_match_backward_fft(cg, orc):
    """zerocorr lags (examples/zerocorr.c:391, 626-645): FFTW_BACKWARD of the visibilities, scaled 1/n."""
    import synth

    S, N, K = 2, 1024, 512
    raw = synth.stations_offset_binary(S, N * K, rho=0.2, lags=[0, 6], seed=21)
    vis = np.zeros((3, N // 2), np.complex64)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_BASELINE_MAJOR), raw, vis)
    lags = np.zeros_like(vis)
    cg.vis_lags(vis, lags, scale=1.0 / K)
    ref = np.fft.ifft(vis.astype(np.complex128), axis=1) * (N // 2) / K
    assert np.linalg.norm(lags - ref) / np.linalg.norm(ref) < 1e-5
    # x_1(t) = c(t - 6): V_10(k) = |C|^2 exp(-2 pi i k 6 / N) over the N/2 channels,
    # whose backward transform peaks at lag index 6 / 2 = 3 (two samples per index)
    cross = lags[orc.tri_index(1, 0)]
    assert int(np.argmax(np.abs(cross))) == 3
    assert np.abs(cross[3]) > 5 * np.abs(np.delete(cross, 3)).max()


@pytest.mark.parametrize("mode", ["tc", "fp32"])
def test_fx_host_buffers_streamed_match_device(cg, mode):
    """Host-buffer jobs of 64 MB or more move their input in blocks of inputs and
    their channel-major visibilities in blocks of channels on a copy stream,
    overlapping the F and X stages: bit-identical to the device-buffer run."""
    import torch

    import synth

    S, N, K = 128, 2048, 2048
    x_mode = cg.X_TC_FP16 if mode == "tc" else cg.X_FP32
    d_raw = synth.device_stations(S, N * K, 0.1, seed=12)
    raw = d_raw.cpu().numpy()
    assert raw.nbytes >= 64 << 20
    P, C = S * (S + 1) // 2, N // 2
    d_vis = torch.empty((C, P), dtype=torch.complex64, device="cuda")
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=x_mode), d_raw, d_vis)
    ref = d_vis.cpu().numpy()
    h_vis = np.zeros((C, P), np.complex64)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=x_mode), raw, h_vis)
    assert np.array_equal(h_vis, ref)
    vb = np.zeros((P, C), np.complex64)              # baseline-major: streamed in only
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=x_mode, vis_order=cg.VIS_BASELINE_MAJOR), raw, vb)
    assert np.array_equal(vb, ref.T)


def test_direct_call_waits_for_prior_default_stream_work(cg):
    """A synchronous call on device buffers sees the data that work queued just
    before it on the default stream writes (the library's streams are
    non-blocking; each call first waits on the device for that stream)."""
    import torch

    import synth

    S, N, K = 64, 2048, 1024
    P, C = S * (S + 1) // 2, N // 2
    src = synth.device_stations(S, N * K, 0.1, seed=13)
    p = cg.fx_params(S, N, K, src.shape[1])
    want = torch.empty((C, P), dtype=torch.complex64, device="cuda")
    cg.fx_correlate(p, src, want)
    for _ in range(3):
        raw = torch.zeros_like(src)
        busy = torch.randn((4096, 4096), device="cuda")
        for _ in range(8):                       # keep the default stream busy for a while
            busy = busy @ busy.T / 4096.0
        raw.copy_(src)                           # queued behind the products, not yet done
        vis = torch.empty((C, P), dtype=torch.complex64, device="cuda")
        cg.fx_correlate(p, raw, vis)
        assert torch.equal(vis, want)


@pytest.mark.parametrize("mode", ["tc", "fp32"])
@pytest.mark.parametrize("K", [160, 104])
def test_fx_w2048_schedules_identical(cg, mode, K, monkeypatch):
    """The 2048-point F stage's CTA schedules, between which the autotuner
    picks by time alone, compute the same values: every forced schedule gives
    bit-identical visibilities (K = 160: whole 32-segment tiles; K = 104: a
    partial last tile and the planar layout)."""
    import torch

    import synth

    S, N = 16, 2048
    x_mode = cg.X_TC_FP16 if mode == "tc" else cg.X_FP32
    raw = synth.device_stations(S, N * K, 0.2, seed=17)
    P, C = S * (S + 1) // 2, N // 2
    outs = []
    for v in "12345":
        monkeypatch.setenv("CELLSPE_FSTAGE_VARIANT", v)
        vis = torch.empty((C, P), dtype=torch.complex64, device="cuda")
        cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=x_mode), raw, vis)
        outs.append(vis)
    for o in outs[1:]:
        assert torch.equal(o, outs[0])


@pytest.mark.parametrize("N,K", [(512, 40), (512, 128), (1024, 40), (1024, 128), (4096, 24), (8192, 16), (16384, 8),
                                 (32768, 8)])
def test_fx_warp_fstages_delay_model(cg, orc, N, K, monkeypatch):
    """The warp four-step F stages other than N = 2048: N = 512 and 1024 (a
    half-warp per segment, 16 or 32 points per lane; 64-segment tiles in FP16, 32
    in FP32 at N = 1024: K = 40 a partial tile, K = 128 full ones) and
    N = 4096 ... 32768 (N/2048 warps per segment, each a 1024-point transform of
    every (N/2048)-th point, then radix-N/2048 columns and the real-FFT split in
    registers).  FP32 path against the oracle's FP32 path with the same delay
    model and against the CTA-wide Stockham F stage; the tensor-core path (K a
    multiple of 8) against the same job through the Stockham F stage."""
    import synth

    S = 3
    fs, lo = 32e6, 8.4e9
    margin = 4096
    raw = synth.stations_offset_binary(S, N * K + 2 * margin, rho=0.3, seed=N + 7)
    rng = np.random.default_rng(N)
    poly = np.zeros((S, 4))
    poly[:, 0] = rng.uniform(-40e-6, 40e-6, S)
    poly[:, 1] = rng.uniform(-3e-6, 3e-6, S)
    kw = dict(vis_order=cg.VIS_BASELINE_MAJOR, start_sample=margin, fs_hz=fs, lo_hz=lo)
    P = S * (S + 1) // 2
    vis = np.zeros((P, N // 2), np.complex64)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], **kw), raw, vis, delay_poly=poly)
    shift, ph0, dph = orc.delay_state_f64(poly, N, K, fs, lo)
    c = np.arange(N // 2)
    phasor = np.exp(1j * (ph0.astype(np.float32)[:, :, None].astype(np.float64) +
                          c[None, None, :] * dph.astype(np.float32)[:, :, None].astype(np.float64))).astype(np.complex64)
    ref = orc.fx_fp32(raw, S, N, K, start_sample=margin, shift=shift, phasor=phasor)
    assert _rel(vis, ref) < TOL
    tc = np.zeros_like(vis)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, **kw), raw, tc, delay_poly=poly)
    monkeypatch.setenv("CELLSPE_FSTAGE_GENERIC", "1")
    gen = np.zeros_like(vis)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], **kw), raw, gen, delay_poly=poly)
    assert _rel(vis, gen) < 2e-6
    gtc = np.zeros_like(vis)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, **kw), raw, gtc, delay_poly=poly)
    assert _rel(tc, gtc) < 1e-3
    assert _rel(tc, ref) < 1e-3
