"""K-d2: tcgen05 FP16 X stage.

Two bars: (1) on FP16 inputs the tensor-core result equals the FP64 product of
the same FP16 values up to FP32 accumulation (relative 1e-5); (2) through the
full FX path it is within 1e-3 relative amplitude and 0.05 degree phase of the
FP64 oracle, the precision the engine promises for the tensor-core path.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fp64_vis(xr, xi):
    """xr, xi: [C][S][K] float64 -> V[C][P] with p = i(i+1)/2 + j."""
    X = xr + 1j * xi
    C, S, _ = X.shape
    full = np.einsum("csk,ctk->cst", X, np.conj(X))
    ii, jj = np.tril_indices(S)
    order = np.argsort(ii * (ii + 1) // 2 + jj)
    return full[:, ii[order], jj[order]]


@pytest.mark.parametrize("S,C,K", [(8, 3, 64), (128, 2, 96), (130, 2, 40), (256, 1, 128), (300, 2, 32)])
def test_xmac_f16_exact_inputs(cg, S, C, K):
    rng = np.random.default_rng(S + K)
    spec = rng.standard_normal((C, 2, S, K)).astype(np.float16)
    P = S * (S + 1) // 2
    vis = np.zeros((C, P), np.complex64)
    cg.xmac_f16(spec, S, C, K, vis)
    ref = _fp64_vis(spec[:, 0].astype(np.float64), spec[:, 1].astype(np.float64))
    err = np.linalg.norm(vis - ref) / np.linalg.norm(ref)
    assert err < 1e-5, err
    # lower triangle written, autos real
    ii = np.array([i for i in range(S) for _ in range(i + 1)])
    jj = np.array([j for i in range(S) for j in range(i + 1)])
    autos = vis[:, ii == jj]
    assert np.abs(autos.imag).max() <= 1e-5 * np.abs(autos.real).max()


@pytest.mark.parametrize("S", [40, 200])
def test_xmac_f16_accumulate(cg, S):
    """accumulate adds to the visibilities; S = 200 has diagonal tiles past the
    single-tile size (Im = M - M^T staged in the epilogue) and an edge tile."""
    rng = np.random.default_rng(1)
    C, K = 2, 64
    spec = rng.standard_normal((C, 2, S, K)).astype(np.float16)
    vis = np.zeros((C, S * (S + 1) // 2), np.complex64)
    cg.xmac_f16(spec, S, C, K, vis)
    v2 = vis.copy()
    cg.xmac_f16(spec, S, C, K, v2, accumulate=True)
    assert np.allclose(v2, 2 * vis, rtol=1e-6, atol=1e-4)


def test_fx_tc_accumulate_channel_grouped(cg):
    """FX with accumulate on the default N = 2048 tensor-core path (channel-grouped
    spectra, diagonal tiles past 128 inputs): a second call adds the same
    visibilities."""
    import synth

    S, N, K = 160, 2048, 64
    raw = synth.stations_offset_binary(S, N * K, rho=0.2, seed=41)
    P, C = S * (S + 1) // 2, N // 2
    vis = np.zeros((C, P), np.complex64)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16), raw, vis)
    v2 = vis.copy()
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, accumulate=True), raw, v2)
    assert np.allclose(v2, 2 * vis, rtol=1e-6, atol=1e-4)


def _fx_pair(cg, raw, S, N, K, mode, **kw):
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=mode, vis_order=cg.VIS_BASELINE_MAJOR, **kw)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis, delay_poly=kw.get("delay_poly"))
    return vis


@pytest.mark.parametrize("S,N,K,rho", [(64, 2048, 256, 0.02), (32, 8192, 64, 0.5), (200, 1024, 128, 0.3)])
def test_fx_tc_vs_fp64_oracle(cg, orc, S, N, K, rho):
    import synth

    raw = synth.stations_offset_binary(S, N * K, rho=rho, seed=S * 7 + N)
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=cg.VIS_BASELINE_MAJOR)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis)
    # FP64 oracle on a seeded subset of products and channels, full K
    rng = np.random.default_rng(0)
    inputs = sorted(rng.choice(S, size=min(S, 12), replace=False))
    chans = sorted(rng.choice(N // 2, size=32, replace=False))
    X = orc.fx_spectra_f64(raw, S, N, K, inputs=inputs, channels=chans)
    pairs = [(a, b) for a in range(len(inputs)) for b in range(a + 1)]
    ref = orc.fx_vis_f64(X, pairs)
    got = np.stack([vis[orc.tri_index(inputs[a], inputs[b])][chans] for a, b in pairs])
    amp_err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert amp_err.max() < 1e-3, amp_err.max()
    # phase over channels whose |V| is above the thermal-noise floor
    # 3 sqrt(V_ii V_jj / K) (below it the phase is noise, not signal)
    auto = {a: ref[pairs.index((a, a))].real for a in range(len(inputs))}
    floor = np.stack([3 * np.sqrt(auto[a] * auto[b] / K) for a, b in pairs])
    mask = np.abs(ref) > floor
    phase_deg = np.degrees(np.abs(np.angle(got * np.conj(ref))))[mask]
    assert phase_deg.max() < 0.05, phase_deg.max()
    if rho >= 0.3:
        cross = np.array([a != b for a, b in pairs])
        assert mask[cross].mean() > 0.5      # the phase bar really covers cross products
    # and agrees with the FP32 CUDA-core path
    v32 = np.zeros_like(vis)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_FP32, vis_order=cg.VIS_BASELINE_MAJOR),
                    raw, v32)
    rel = np.linalg.norm(vis - v32, axis=1) / np.linalg.norm(v32, axis=1)
    assert rel.max() < 1e-3


def test_fx_tc_channel_scale(cg):
    """A per-(input, channel) scale before the FP16 cast is undone in the epilogue."""
    import synth

    S, N, K = 16, 1024, 64
    raw = synth.stations_offset_binary(S, N * K, rho=0.1, seed=3)
    base = _fx_pair(cg, raw, S, N, K, cg.X_TC_FP16)
    scale = np.random.default_rng(2).uniform(0.01, 0.05, (S, N // 2)).astype(np.float32)
    scaled = _fx_pair(cg, raw, S, N, K, cg.X_TC_FP16, channel_scale=scale)
    rel = np.linalg.norm(scaled - base) / np.linalg.norm(base)
    assert rel < 1e-3


def _tc_bars(orc, vis, X, pairs, K, sel=None, chans=None, cross_coverage=True):
    """1e-3 relative amplitude per product, 0.05 deg phase above the 3-sigma noise floor."""
    ref = orc.fx_vis_f64(X, pairs)
    got = vis if sel is None else np.stack([vis[p][chans] for p in sel])
    amp_err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert amp_err.max() < 1e-3, amp_err.max()
    auto = {a: ref[pairs.index((a, a))].real for a, b in pairs if a == b}
    floor = np.stack([3 * np.sqrt(auto[a] * auto[b] / K) for a, b in pairs])
    mask = np.abs(ref) > floor
    cross = np.array([a != b for a, b in pairs])
    if cross_coverage:
        assert mask[cross].mean() > 0.5
    phase_deg = np.degrees(np.abs(np.angle(got * np.conj(ref))))[mask]
    assert phase_deg.max() < 0.05, phase_deg.max()


@pytest.fixture(params=["0", "1"], ids=["warp-fft", "tc-fstage"])
def fstage_engine(request, monkeypatch):
    """N = 2048 FP16 spectra from the warp FFT (default) or the tensor-core F stage."""
    monkeypatch.setenv("CELLSPE_FSTAGE_TC", request.param)
    return request.param


@pytest.mark.parametrize("S,K,rho", [(24, 64, 0.5), (9, 72, 0.6), (40, 136, 0.4)])
def test_fx_tc_fstage_2048_vs_fp64(cg, orc, S, K, rho, fstage_engine):
    """N = 2048 with either F stage (tensor-core one: units of 8 segments over 9
    to 40 inputs; the X stage needs K % 8 == 0)."""
    import synth

    N = 2048
    raw = synth.stations_offset_binary(S, N * K, rho=rho, lags=np.arange(S) % 3, seed=S + K)
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=cg.VIS_BASELINE_MAJOR)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis)
    inputs = list(range(min(S, 8)))
    X = orc.fx_spectra_f64(raw, S, N, K, inputs=inputs)
    pairs = [(a, b) for a in range(len(inputs)) for b in range(a + 1)]
    sel = [orc.tri_index(inputs[a], inputs[b]) for a, b in pairs]
    _tc_bars(orc, vis, X, pairs, K, sel=sel, chans=slice(None))


def test_fx_tc_fstage_2048_delay_model(cg, orc, fstage_engine):
    """Integer shifts (start offsets at every sample alignment) and the fringe /
    fractional-delay phasor in the tensor-core F stage's epilogue."""
    import synth

    S, N, K = 5, 2048, 40
    fs, lo = 32e6, 8.4e9
    margin = 4096
    raw = synth.stations_offset_binary(S, N * K + 2 * margin, rho=0.5, seed=21)
    rng = np.random.default_rng(6)
    poly = np.zeros((S, 4))
    poly[:, 0] = rng.uniform(-40e-6, 40e-6, S)
    poly[:, 1] = rng.uniform(-2e-3, 2e-3, S)          # fast rates: the shift walks through alignments
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=cg.VIS_BASELINE_MAJOR,
                     start_sample=margin, fs_hz=fs, lo_hz=lo)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis, delay_poly=poly)
    shift, ph0, dph = orc.delay_state_f64(poly, N, K, fs, lo)
    assert len(set((shift.ravel() + margin) % 64)) > 20          # many sample alignments
    X = orc.fx_spectra_f64(raw, S, N, K, margin, shift, ph0, dph)
    pairs = [(i, j) for i in range(S) for j in range(i + 1)]
    # the random delays decorrelate the inputs: the phase bar covers the autos
    _tc_bars(orc, vis, X, pairs, K, cross_coverage=False)


@pytest.fixture(params=["0", "1", "2"], ids=["warp-fft", "tc32-fstage", "tc32-specialised"])
def fstage32(request, monkeypatch):
    """N = 2048 k-blocked FP16 spectra from the warp FFT or the 32-segment
    tensor-core F stage (real-input symmetry, k1 = 32 row via pass 2'), in its
    lockstep and its warp-specialised form."""
    monkeypatch.setenv("CELLSPE_FSTAGE_TC32", request.param)
    return request.param


@pytest.mark.parametrize("S,K,rho", [(24, 64, 0.5), (9, 96, 0.6), (40, 128, 0.4), (130, 64, 0.6)])
def test_fx_tc32_fstage_vs_fp64(cg, orc, S, K, rho, fstage32):
    """Every channel (the direct, mirrored and k1 = 32 families) of the
    tensor-core F stage through the full FX path: all products of the first 8
    inputs against the FP64 oracle, and the whole matrix against the FP32 path."""
    import synth

    N = 2048
    raw = synth.stations_offset_binary(S, N * K, rho=rho, lags=np.arange(S) % 5, seed=S * 3 + K)
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=cg.VIS_BASELINE_MAJOR)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis)
    inputs = list(range(min(S, 8)))
    X = orc.fx_spectra_f64(raw, S, N, K, inputs=inputs)
    pairs = [(a, b) for a in range(len(inputs)) for b in range(a + 1)]
    sel = [orc.tri_index(inputs[a], inputs[b]) for a, b in pairs]
    _tc_bars(orc, vis, X, pairs, K, sel=sel, chans=slice(None))
    v32 = np.zeros_like(vis)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_FP32, vis_order=cg.VIS_BASELINE_MAJOR),
                    raw, v32)
    rel = np.linalg.norm(vis - v32, axis=1) / np.linalg.norm(v32, axis=1)
    assert rel.max() < 1e-3


def test_fx_tc32_fstage_delay_model_and_scale(cg, orc, fstage32):
    """Integer shifts at every sample alignment, the fringe / fractional-delay
    phasor on all three channel families, and a per-(input, channel) scale."""
    import synth

    S, N, K = 5, 2048, 64
    fs, lo = 32e6, 8.4e9
    margin = 4096
    raw = synth.stations_offset_binary(S, N * K + 2 * margin, rho=0.5, seed=23)
    rng = np.random.default_rng(7)
    poly = np.zeros((S, 4))
    poly[:, 0] = rng.uniform(-40e-6, 40e-6, S)
    poly[:, 1] = rng.uniform(-2e-3, 2e-3, S)
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=cg.VIS_BASELINE_MAJOR,
                     start_sample=margin, fs_hz=fs, lo_hz=lo)
    vis = np.zeros((S * (S + 1) // 2, N // 2), np.complex64)
    cg.fx_correlate(p, raw, vis, delay_poly=poly)
    shift, ph0, dph = orc.delay_state_f64(poly, N, K, fs, lo)
    X = orc.fx_spectra_f64(raw, S, N, K, margin, shift, ph0, dph)
    pairs = [(i, j) for i in range(S) for j in range(i + 1)]
    _tc_bars(orc, vis, X, pairs, K, cross_coverage=False)
    scale = np.random.default_rng(3).uniform(0.01, 0.05, (S, N // 2)).astype(np.float32)
    ps = cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=cg.VIS_BASELINE_MAJOR,
                      start_sample=margin, fs_hz=fs, lo_hz=lo, channel_scale=scale)
    vs = np.zeros_like(vis)
    cg.fx_correlate(ps, raw, vs, delay_poly=poly)
    assert np.linalg.norm(vs - vis) / np.linalg.norm(vis) < 1e-3
