"""The oracle pinned to the reference: golden vectors, live reference, known answers."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("fmt,nch", [("Mark5B_512_16_2", 16), ("Mark5B_256_8_2", 8), ("Mark5B_128_4_2", 4)])
def test_unpack_matches_mark5access_golden(orc, fmt, nch):
    g = np.load(GOLD / "mark5b_unpack.npz")
    raw, ref = g[f"{fmt}_raw"], g[f"{fmt}_out"]
    mine = orc.unpack2bit(raw, ref.shape[1], nch, orc.MARK5B_LUT)
    assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))


def test_unpack_matches_live_mark5access(orc):
    if not orc.have_ref():
        pytest.skip("reference tree not compiled here")
    rng = np.random.default_rng(5)
    for fmt, nch in [(b"Mark5B-1024-16-2", 16), (b"Mark5B-256-8-2", 8), (b"Mark5B-128-4-2", 4)]:
        n = 4096
        raw = rng.integers(0, 256, n * nch // 4, dtype=np.uint8)
        ref = np.zeros(nch * n, np.float32)
        c = ctypes.c_int()
        rc = orc.ref_mark5().ref_mark5_unpack(fmt, raw.ctypes.data, n, ref.ctypes.data, ctypes.byref(c))
        assert rc == n
        mine = orc.unpack2bit(raw, n, nch, orc.MARK5B_LUT)
        assert np.array_equal(mine.view(np.uint32), ref.reshape(nch, n).view(np.uint32))


FRAMED_LEVELS = np.array([-3.3359, 1.0, -1.0, 3.3359, 0.0], np.float32)


@pytest.mark.parametrize("fmt,nch", [("Mark5B_512_16_2", 16), ("Mark5B_256_8_2", 8), ("Mark5B_128_4_2", 4)])
def test_framed_mark5b_golden(orc, fmt, nch):
    """Header strip + fill-pattern blanking + end-of-data rule vs the library's own decode."""
    g = np.load(GOLD / "mark5b_framed.npz")
    fr = g["framed"]
    assert orc.lib().orc_mark5b_find_first_frame(fr.ctypes.data, fr.size) == 137
    for k, ns in enumerate(g[f"{fmt}_nsamp"]):
        good, out = orc.mark5b_decode_framed(fr, nch, int(ns))
        assert good == int(g[f"{fmt}_rc{k}"])
        assert np.array_equal(out.view(np.uint32), FRAMED_LEVELS[g[f"{fmt}_codes{k}"]].view(np.uint32))


def test_framed_mark5b_live_reference(orc):
    if not orc.have_ref():
        pytest.skip("reference tree not compiled here")
    import synth

    rng = np.random.default_rng(17)
    for fmt, nch in [(b"Mark5B-512-16-2", 16), (b"Mark5B-256-8-2", 8), (b"Mark5B-128-4-2", 4)]:
        nf, pre = 6, int(rng.integers(0, 3000))
        fr = synth.mark5b_frames(rng.integers(0, 256, nf * 10000, dtype=np.uint8), prefix=pre,
                                 first_frame=int(rng.integers(0, 6400)))
        for f in range(nf):
            a = int(rng.integers(0, 2501)) * 4
            kind = int(rng.integers(0, 4))
            if kind == 1:
                synth.mark5b_fill(fr, f, 0, a, pre)
            elif kind == 2:
                synth.mark5b_fill(fr, f, a, 10000, pre)
        spf = 10000 // (nch // 4)
        for ns in (int(rng.integers(1, nf * spf)), (nf - 1) * spf, nf * spf):
            rc, ref, off = orc.ref_mark5_decode_memory(fmt, fr, ns)
            good, mine = orc.mark5b_decode_framed(fr, nch, ns)
            assert off == pre and good == rc
            assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))


VDIF_LEVELS = np.array([-3.3359, -1.0, 1.0, 3.3359, 0.0], np.float32)
VDIF_GOLDEN = {"v4ch": (4, 128), "v8ch_legacy": (8, 256), "v16ch_granularity": (16, 8192), "v1ch_day": (1, 128),
               "v2ch_legacy": (2, 64)}


@pytest.mark.parametrize("name", sorted(VDIF_GOLDEN))
def test_framed_vdif_golden(orc, name):
    """VDIF validation (invalid bit, header time, fill) + legacy headers + end-of-data rule
    vs the library's own decode of the same bytes."""
    nch, mbps = VDIF_GOLDEN[name]
    g = np.load(GOLD / "vdif_framed.npz")
    fr = g[f"{name}_framed"]
    for k, ns in enumerate(g[f"{name}_nsamp"]):
        good, out = orc.vdif_decode_framed(fr, nch, mbps, int(ns))
        assert good == int(g[f"{name}_rc{k}"])
        assert np.array_equal(out.view(np.uint32), VDIF_LEVELS[g[f"{name}_codes{k}"]].view(np.uint32))


def test_vdif_golden_covers_each_blanking_rule():
    """The fixtures hold what they are meant to: an invalid-bit frame 0 that stays
    (frame 0 is not validated), blanked invalid / time-glitch / fill frames, and the
    frame the library blanks because its frame time is not a whole number of ns."""
    g = np.load(GOLD / "vdif_framed.npz")

    def blanked(name, nch, db):
        spf = db * 4 // nch
        c = g[f"{name}_codes1"]
        return [bool((c[:, f * spf:(f + 1) * spf] == 4).all()) for f in range(c.shape[1] // spf)]

    assert blanked("v4ch", 4, 2000) == [False, False, True, True, False, True, True]
    assert blanked("v16ch_granularity", 16, 2000)[8] and not any(blanked("v16ch_granularity", 16, 2000)[4:8])
    assert blanked("v1ch_day", 1, 1024) == [False, False, False, False, True]


def test_vdif_first_frame_time_every_epoch(orc):
    """The calendar-computed reference epochs against the library's table, all 64."""
    import synth

    want = np.load(GOLD / "vdif_framed.npz")["epoch_times"]
    for e in range(64):
        fr = synth.vdif_frames(np.zeros(2 * 1024, np.uint8), 1024, 4, 128, ref_epoch=e, seconds=5 * 86400 + 7,
                               first_frame=3)
        assert orc.vdif_first_time(fr, 128) == tuple(int(v) for v in want[e]), e
        if orc.have_ref():
            assert orc.ref_mark5_stream_time(b"VDIF_1024-128-4-2", fr) == tuple(int(v) for v in want[e])


def test_framed_vdif_live_reference(orc):
    if not orc.have_ref():
        pytest.skip("reference tree not compiled here")
    import synth

    rng = np.random.default_rng(23)
    for db, nch, mbps, legacy in [(8000, 4, 512, False), (8000, 16, 2048, True), (8000, 1, 128, False),
                                  (8000, 2, 256, False), (8000, 8, 8192, False), (1024, 4, 1024, False),
                                  (5000, 8, 4000, True), (8192, 16, 4096, False)]:
        hs = 16 if legacy else 32
        fb, nf = db + hs, 9
        fr = synth.vdif_frames(rng.integers(0, 256, nf * db, dtype=np.uint8), db, nch, mbps, legacy=legacy,
                               ref_epoch=int(rng.integers(0, 64)), seconds=int(rng.integers(0, 1 << 30)),
                               first_frame=int(rng.integers(0, 8)))
        for f in rng.choice(nf, 4, replace=False):
            kind = int(rng.integers(0, 4))
            if kind == 0:
                synth.vdif_set_invalid(fr, int(f), fb)
            elif kind == 1:
                fr[int(f) * fb + 4] ^= 1
            elif kind == 2:
                synth.vdif_fill(fr, int(f), fb, hs, 0, 8)
            else:
                synth.vdif_fill(fr, int(f), fb, hs, db - 8, db)
        spf = db * 4 // nch
        fmt = f"VDIF_{db}-{mbps}-{nch}-2".encode()
        for ns in (3 * spf + 16, (nf - 1) * spf, nf * spf, nf * spf - 4):
            rc, ref, off = orc.ref_mark5_decode_memory(fmt, fr, ns)
            good, mine = orc.vdif_decode_framed(fr, nch, mbps, ns)
            assert off == 0 and good == rc, (fmt, ns)
            assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32)), (fmt, ns)


def test_generic_mac_golden(orc):
    g = np.load(GOLD / "generic_mac.npz")
    acc = g["acc0"].copy()
    orc.addproduct(g["a"], g["b"], acc, conj=False)
    assert np.array_equal(acc.view(np.uint32), g["mac"].view(np.uint32))
    acc = g["acc0"].copy()
    orc.addproduct(g["a"], g["b"], acc, conj=True)
    assert np.array_equal(acc.view(np.uint32), g["mac_conj"].view(np.uint32))


def test_generic_mac_live_reference(orc):
    if not orc.have_ref():
        pytest.skip("reference tree not compiled here")
    rng = np.random.default_rng(3)
    a = (rng.standard_normal(777) + 1j * rng.standard_normal(777)).astype(np.complex64)
    b = (rng.standard_normal(777) + 1j * rng.standard_normal(777)).astype(np.complex64)
    for conj, name in [(True, "ref_addproduct_32fc_conj"), (False, "ref_addproduct_32fc")]:
        acc0 = (rng.standard_normal(777) + 1j * rng.standard_normal(777)).astype(np.complex64)
        mine, ref = acc0.copy(), acc0.copy()
        orc.addproduct(a, b, mine, conj)
        getattr(orc.ref_generic(), name)(a.ctypes.data, b.ctypes.data, ref.ctypes.data, 777)
        assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))


def test_twobit_and_msb_first_tables(orc):
    # TwoBitUnpacker (DataUnpackers.cpp:174-227): channel c of a 4-channel byte
    # sits at shift 2c, value map_rev[code].
    raw = np.arange(256, dtype=np.uint8)
    out = orc.unpack2bit(raw, 256, 4, orc.TWOBIT_LUT)
    for c in range(4):
        codes = (raw >> (2 * c)) & 3
        assert np.array_equal(out[c], orc.TWOBIT_LUT[codes])
    # single channel MSB first: sample 0 in bits 7:6
    out = orc.unpack2bit(raw, 1024, 1, orc.TWOBIT_LUT, msb_first=True)[0].reshape(256, 4)
    for j in range(4):
        assert np.array_equal(out[:, j], orc.TWOBIT_LUT[(raw >> (6 - 2 * j)) & 3])


@pytest.mark.parametrize("n", [32, 1024, 4096])
def test_fft_vs_fp64(orc, n):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    ref = np.fft.fft(x.astype(np.complex128))
    assert np.linalg.norm(orc.cfft_f32(x) - ref) / np.linalg.norm(ref) < 1e-6
    r = rng.standard_normal(2 * n).astype(np.float32)
    ref = np.fft.rfft(r.astype(np.float64))
    assert np.linalg.norm(orc.rfft_f32(r) - ref) / np.linalg.norm(ref) < 1e-6


def test_spectrometer_known_tone(orc):
    # A pure tone at bin 100 of a 1024-point FFT: the power peaks there.
    N, K = 1024, 8
    n = np.arange(N * K)
    x = np.cos(2 * np.pi * 100 * n / N).astype(np.float32)
    power, _ = orc.spectrometer(x, N, 2, 2, K)
    assert power.shape == (1, N // 2 + 1)
    assert int(np.argmax(power[0])) == 100
    # 1/core_overlapped_ffts scaling: overlapped FFTs = 2K-1 (swspectrometer.cpp:231)
    w = orc.window(2, N)
    expect = (np.abs(np.sum(w * np.cos(2 * np.pi * 100 * np.arange(N) / N) * np.exp(-2j * np.pi * 100 * np.arange(N) / N))) ** 2)
    assert power[0, 100] == pytest.approx(expect, rel=1e-3)


def test_pcal_unit_test_recipe(orc):
    """PCal.cpp:879-951: tones with phase -90 deg + 5 deg per tone, checked to 0.1 deg.

    Offset 0 (PCalExtractorTrivial); tone 0 is DC and has no phase, so tones
    1..N_tones-1 are checked.
    """
    bw, spacing = 16e6, 1e6
    fs = 2 * bw
    nbins = int(fs / spacing)
    ntones = int(bw // spacing)
    nsamp = nbins * 4096
    n = np.arange(nsamp)
    data = np.zeros(nsamp)
    for t in range(ntones):
        data += np.sin(np.pi * n * (t * spacing) / bw + t * np.pi * 5 / 180)
    # fold the real samples into Nbins (TaskCoreIPP::extract_PCal with a unit rotator)
    bins = np.zeros(nbins, np.complex64)
    for b in range(nbins):
        bins[b] = data[b::nbins].sum()
    tones = orc.pcal_tones(bins, ntones)
    phase = np.degrees(np.angle(tones[1:]))
    expect = -90.0 + 5.0 * np.arange(1, ntones)
    assert np.all(np.abs((phase - expect + 180) % 360 - 180) < 0.1)


def test_streamed_subset_model_equals_full_fp64_model(orc):
    """fx_vis_subset_f64 (exact DFT at chosen channels, streamed over segments,
    used for the full-size checks) equals the FP64 rfft model on the same
    inputs, delay state included; vis_errors reads zero error off it."""
    import synth

    S, N, K, margin = 5, 1024, 40, 4096
    raw = synth.stations_offset_binary(S, N * K + 2 * margin, rho=0.5, seed=21)
    rng = np.random.default_rng(6)
    poly = np.zeros((S, 4))
    poly[:, 0] = rng.uniform(-40e-6, 40e-6, S)
    poly[:, 1] = rng.uniform(-2e-3, 2e-3, S)
    shift, ph0, dph = orc.delay_state_f64(poly, N, K, 32e6, 8.4e9)
    X = orc.fx_spectra_f64(raw, S, N, K, margin, shift, ph0, dph)
    pairs = [(i, j) for i in range(S) for j in range(i + 1)]
    full = orc.fx_vis_f64(X, pairs)
    ch, inp = [0, 3, 17, 100, 511], [1, 2, 4]
    V, autos = orc.fx_vis_subset_f64(raw[inp], N, K, ch, margin, shift[inp], ph0[inp], dph[inp], chunk=16)
    for a in range(3):
        for b in range(a + 1):
            ref = full[pairs.index((inp[a], inp[b]))][ch]
            assert np.abs(V[a, b] - ref).max() <= 1e-12 * np.abs(ref).max()
    err = orc.vis_errors(V, V, autos, K)
    assert err["max_rel_amp"] == 0 and err["max_phase_deg"] == 0 and err["products"] == 6
