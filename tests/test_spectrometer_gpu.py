"""K-e + K-pcal: GPU spectrometer vs the restated TaskCoreIPP::doMaths."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _oracle(orc, words, nsub, N, overlap, window, K, tonebins=0, rotatorlen=0, offset=0.0, fs=1.0):
    raw = words.view(np.uint8)
    nsamp = raw.size * 4 // nsub
    planes = orc.unpack2bit(raw, nsamp, nsub, orc.MARK5B_LUT)
    pw, pc = [], []
    for c in range(nsub):
        p, b = orc.spectrometer(planes[c], N, overlap, window, K, tonebins, rotatorlen, offset, fs)
        pw.append(p)
        pc.append(b)
    return np.stack(pw), (np.stack(pc) if tonebins else None)


@pytest.mark.parametrize("nsub,N,overlap,window,K,nspec", [
    (16, 1024, 2, 2, 8, 2), (4, 4096, 1, 0, 4, 1), (1, 2048, 4, 1, 3, 2), (8, 32768, 2, 2, 2, 1),
    (4, 65536, 2, 2, 3, 1),
    # the warp four-step kernel of N = 32768 / 65536 with every other window and overlap
    (4, 65536, 1, 1, 2, 2), (4, 32768, 4, 3, 2, 1), (1, 65536, 4, 5, 2, 1), (1, 32768, 1, 0, 3, 2),
    (1, 65536, 2, 4, 2, 1)])
def test_spectrometer_vs_oracle(cg, orc, nsub, N, overlap, window, K, nspec):
    import synth

    T = N * K * nspec
    words, _ = synth.mark5b_subbands(nsub, T, fs_hz=32e6, seed=N + nsub, n_channels=N // 2)
    if nsub < 16:  # repack to nsub channels per sample time
        raw8 = words.view(np.uint8)
        codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nsub)], axis=1)
        words = synth.pack2bit(codes.reshape(-1)).view(np.uint8)
    raw = np.ascontiguousarray(words).view(np.uint8)
    p = cg.spec_params(N, overlap, window, K, nspec, nsub, raw.size)
    power = np.zeros((nsub, nspec, N // 2 + 1), np.float32)
    cg.spectrometer(p, raw, power)
    ref, _ = _oracle(orc, raw, nsub, N, overlap, window, K)
    assert ref.shape == power.shape
    assert np.linalg.norm(power - ref) / np.linalg.norm(ref) < TOL


def test_spectrometer_pcal_and_sines_known_answer(cg, orc):
    """Config-2 shape in miniature: 16 subbands, 32 MS/s, 1 MHz comb, 3 sines."""
    import synth

    nsub, N, K, fs = 16, 4096, 64, 32e6
    T = N * K
    words, truth = synth.mark5b_subbands(nsub, T, fs_hz=fs, seed=2, n_channels=N // 2, pcal_amp=0.3)
    raw = words.view(np.uint8)
    tb, ntones = 32, 16
    p = cg.spec_params(N, 2, 2, K, 1, nsub, raw.size, tonebins=tb, rotatorlen=tb, ntones=ntones, offset_hz=0.0,
                       fs_hz=fs)
    power = np.zeros((nsub, 1, N // 2 + 1), np.float32)
    bins = np.zeros((nsub, 1, tb), np.complex64)
    tones = np.zeros((nsub, 1, ntones), np.complex64)
    cg.spectrometer(p, raw, power, bins, tones)
    ref_p, ref_b = _oracle(orc, raw, nsub, N, 2, 2, K, tb, tb, 0.0, fs)
    assert np.linalg.norm(power - ref_p) / np.linalg.norm(ref_p) < TOL
    assert np.linalg.norm(bins - ref_b) / np.linalg.norm(ref_b) < TOL
    for c in range(nsub):
        ref_t = orc.pcal_tones(ref_b[c, 0], ntones)
        assert np.linalg.norm(tones[c, 0] - ref_t) / np.linalg.norm(ref_t) < TOL
        # injected comb phases (cosine at k MHz, phase phi -> tone phase phi).
        # Thermal noise and 2-bit intermodulation of the harmonic comb leave a
        # few degrees per tone at this length; a wrong sign or bin would be off
        # by tens of degrees.
        ph = np.angle(tones[c, 0, 1:ntones])
        d = np.degrees(np.abs(np.angle(np.exp(1j * (ph - truth["tone_phase"][c, : ntones - 1])))))
        assert d.max() < 15.0 and d.mean() < 6.0
        # the sine with the highest frequency resolution lands at its bin
        for f in truth["sine_f"][c]:
            kbin = int(round(f / fs * N))
            assert power[c, 0, kbin] > 3 * np.median(power[c, 0])


def test_spectrometer_pcal_offset_rotator(cg, orc):
    import synth

    nsub, N, K, fs = 4, 4096, 4, 32.768e6
    words, _ = synth.mark5b_subbands(16, N * K, fs_hz=fs, seed=5, n_channels=N // 2)
    codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nsub)], axis=1)
    raw = synth.pack2bit(codes.reshape(-1))
    tb, L = 32, 4096        # spacing 1.024 MHz, offset 8 kHz
    p = cg.spec_params(N, 2, 2, K, 1, nsub, raw.size, tonebins=tb, rotatorlen=L, ntones=16, offset_hz=8e3, fs_hz=fs)
    power = np.zeros((nsub, 1, N // 2 + 1), np.float32)
    bins = np.zeros((nsub, 1, tb), np.complex64)
    cg.spectrometer(p, raw, power, bins)
    _, ref_b = _oracle(orc, raw, nsub, N, 2, 2, K, tb, L, 8e3, fs)
    assert np.linalg.norm(bins - ref_b) / np.linalg.norm(ref_b) < TOL


@pytest.mark.parametrize("overlap,K,nspec", [(2, 4, 3), (4, 3, 4), (1, 5, 2)])
def test_spectrometer_pcal_running_fft_count(cg, orc, overlap, K, nspec):
    """Several spectra in one call: the phase-cal fold follows the FFT count
    that runs on across the spectra of one doMaths call, so with an odd
    number of overlapped FFTs per spectrum later spectra fold other windows."""
    import synth

    nsub, N, fs = 4, 2048, 32e6
    words, _ = synth.mark5b_subbands(16, N * K * nspec, fs_hz=fs, seed=40 + overlap, n_channels=N // 2, pcal_amp=0.3)
    codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nsub)], axis=1)
    raw = synth.pack2bit(codes.reshape(-1))
    tb = 32
    p = cg.spec_params(N, overlap, 2, K, nspec, nsub, raw.size, tonebins=tb, rotatorlen=tb, ntones=16, offset_hz=0.0,
                       fs_hz=fs)
    power = np.zeros((nsub, nspec, N // 2 + 1), np.float32)
    bins = np.zeros((nsub, nspec, tb), np.complex64)
    cg.spectrometer(p, raw, power, bins)
    ref_p, ref_b = _oracle(orc, raw, nsub, N, overlap, 2, K, tb, tb, 0.0, fs)
    assert np.linalg.norm(power - ref_p) / np.linalg.norm(ref_p) < TOL
    for s in range(nspec):
        assert np.linalg.norm(bins[:, s] - ref_b[:, s]) / np.linalg.norm(ref_b[:, s]) < TOL


def test_spectrometer_planes_layout_and_device(cg):
    import torch

    import synth

    nsub, N, K = 4, 1024, 4
    words, _ = synth.mark5b_subbands(16, N * K, fs_hz=32e6, seed=8, n_channels=N // 2)
    codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nsub)], axis=1)
    inter = synth.pack2bit(codes.reshape(-1))
    planes = np.concatenate([synth.pack2bit(codes[:, c]) for c in range(nsub)])
    a = np.zeros((nsub, 1, N // 2 + 1), np.float32)
    cg.spectrometer(cg.spec_params(N, 2, 2, K, 1, nsub, inter.size), inter, a)
    b = torch.zeros((nsub, 1, N // 2 + 1), dtype=torch.float32, device="cuda")
    cg.spectrometer(cg.spec_params(N, 2, 2, K, 1, nsub, planes.size, layout=cg.SPEC_PLANES),
                    torch.from_numpy(planes).cuda(), b)
    assert np.array_equal(a, b.cpu().numpy())


def test_spectrometer_config2_shape(cg, orc):
    """The Mark5B spectrometer configuration's shape (16 subbands, N = 65536,
    overlap 2, cosine^2, PCal at 1 MHz) on 64 FFT lengths per subband of random
    2-bit codes; two subbands checked against the oracle."""
    nsub, N, K, fs = 16, 65536, 64, 32e6
    raw = np.random.default_rng(12).integers(0, 256, N * K * nsub // 4, dtype=np.uint8)
    p = cg.spec_params(N, 2, 2, K, 1, nsub, raw.size, tonebins=32, rotatorlen=32, ntones=16, fs_hz=fs)
    power = np.zeros((nsub, 1, N // 2 + 1), np.float32)
    bins = np.zeros((nsub, 1, 32), np.complex64)
    cg.spectrometer(p, raw, power, bins)
    planes = orc.unpack2bit(raw, N * K, nsub, orc.MARK5B_LUT)
    for c in (0, 11):
        ref, ref_b = orc.spectrometer(planes[c], N, 2, 2, K, 32, 32, 0.0, fs)
        assert np.linalg.norm(power[c] - ref) / np.linalg.norm(ref) < TOL
        assert np.linalg.norm(bins[c] - ref_b) / np.linalg.norm(ref_b) < TOL


def test_spectrometer_interleaved_equals_planes_full_size(cg):
    """The Mark5B spectrometer input at full size (16 subbands x 2^25 samples, 128 MiB in
    device memory, N = 65536, overlap 2, cosine^2): the interleaved layout, which goes
    through the on-device corner turn, gives the same spectra bit for bit as the
    per-subband 2-bit planes built here from the same words with torch bit operations."""
    import torch

    nsub, N, T = 16, 65536, 1 << 25
    K = T // N
    g = torch.Generator(device="cuda").manual_seed(25)
    raw = torch.randint(0, 256, (T * nsub // 4,), dtype=torch.uint8, device="cuda", generator=g)
    words = raw.view(torch.int32).to(torch.int64)                # one 32-bit word per sample time
    shifts = torch.arange(0, 8, 2, device="cuda", dtype=torch.int64)
    planes = torch.cat([(((words >> (2 * c)) & 3).view(-1, 4) << shifts).sum(dim=1).to(torch.uint8)
                        for c in range(nsub)])
    del words
    a = torch.zeros((nsub, 1, N // 2 + 1), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    cg.spectrometer(cg.spec_params(N, 2, 2, K, 1, nsub, raw.numel()), raw, a)
    cg.spectrometer(cg.spec_params(N, 2, 2, K, 1, nsub, planes.numel(), layout=cg.SPEC_PLANES), planes, b)
    torch.cuda.synchronize()
    assert torch.isfinite(a).all() and float(a.abs().max()) > 0
    assert torch.equal(a, b)


@pytest.mark.parametrize("slope_deg", [5.0, 0.0])
def test_pcal_unit_test_recipe_through_the_gpu(cg, slope_deg):
    """The reference's phase-cal known answer (PCal.cpp:879-951) through
    cellspe_spectrometer's phase-cal fold and tone transform: tones at
    t * 1 MHz in a 16 MHz band (fs = 32 MS/s, offset 0, 32 bins, 16 tones) with
    phase t * slope, data[n] = sum_t sin(pi n t spacing / bw + t slope); the
    extracted tone t must read -90 deg + t slope within 0.1 deg.

    The engine's input is 2-bit; the recipe's data is real-valued.  The fold
    and the tone transform are linear in the samples, so the data go in as a
    16-bit integer (2000 x data + 32768) split into eight base-4 digit planes,
    each run as a 2-bit recording whose custom level table is that digit's
    weight {0, 1, 2, 3} x 4^b; the eight tone sets add up to the tones of the
    16-bit samples (rounding at 1/4000 of a tone amplitude; the constant
    offset lands on the DC tone only, which has no phase and is not checked,
    as in the reference)."""
    import synth

    fs, bw, spacing = 32e6, 16e6, 1e6
    tb, ntones = 32, 16
    N, K = 4096, 32
    n = np.arange(N * K, dtype=np.float64)
    data = np.zeros(n.size)
    for t in range(ntones):
        data += np.sin(np.pi * n * (t * spacing) / bw + t * np.pi * slope_deg / 180)
    v = (np.rint(data * 2000.0) + 32768).astype(np.int64)
    assert v.min() >= 0 and v.max() < 65536
    tones = np.zeros(ntones, np.complex128)
    for b in range(8):
        digits = ((v >> (2 * b)) & 3).astype(np.uint8)
        raw = synth.pack2bit(digits)
        levels = (np.arange(4) * float(4 ** b)).astype(np.float32)
        p = cg.spec_params(N, 1, 0, K, 1, 1, raw.size, layout=cg.SPEC_PLANES, tonebins=tb, rotatorlen=tb,
                           ntones=ntones, offset_hz=0.0, fs_hz=fs)
        p.custom_levels = levels.ctypes.data
        power = np.zeros((1, 1, N // 2 + 1), np.float32)
        bins = np.zeros((1, 1, tb), np.complex64)
        tn = np.zeros((1, 1, ntones), np.complex64)
        cg.spectrometer(p, raw, power, bins, tn)
        tones += tn[0, 0]
    phase = np.degrees(np.angle(tones[1:]))
    expect = -90.0 + slope_deg * np.arange(1, ntones)
    err = np.abs((phase - expect + 180) % 360 - 180)
    assert err.max() < 0.1, err
