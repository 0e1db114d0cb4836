"""Framed Mark5B input on the GPU: header strip, fill-pattern blanking, spectrometer on framed data.

The oracle is the restated mark5_stream_decode (pinned to the compiled
mark5access library and its golden vectors in test_oracle_golden.py)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
LEVELS = np.array([-3.3359, 1.0, -1.0, 3.3359, 0.0], np.float32)


def _framed(rng, nch, nf, prefix, fill_every=3):
    import synth

    fr = synth.mark5b_frames(rng.integers(0, 256, nf * 10000, dtype=np.uint8), prefix=prefix,
                             first_frame=int(rng.integers(0, 6000)))
    for f in range(0, nf, fill_every):
        a = int(rng.integers(0, 2501)) * 4
        kind = int(rng.integers(0, 4))
        if kind == 0:
            synth.mark5b_fill(fr, f, 0, a, prefix)
        elif kind == 1:
            synth.mark5b_fill(fr, f, a, 10000, prefix)
        elif kind == 2:
            synth.mark5b_fill(fr, f, 0, 10000, prefix)
    return fr


@pytest.mark.parametrize("fmt,nch", [("Mark5B_512_16_2", 16), ("Mark5B_256_8_2", 8), ("Mark5B_128_4_2", 4)])
def test_decode_matches_golden(cg, fmt, nch):
    g = np.load(GOLD / "mark5b_framed.npz")
    fr = g["framed"]
    for k, ns in enumerate(g[f"{fmt}_nsamp"]):
        out = np.zeros((nch, int(ns)), np.float32)
        info = cg.mark5b_decode(fr, nch, int(ns), out)
        assert info.good_samples == int(g[f"{fmt}_rc{k}"])
        assert np.array_equal(out.view(np.uint32), LEVELS[g[f"{fmt}_codes{k}"]].view(np.uint32))
        assert (info.first_frame_offset, info.frames) == (137, 8)
        assert (info.mjd, info.seconds, info.frame_number) == (56789, 43210, 0)


@pytest.mark.parametrize("nch", [16, 8, 4])
def test_decode_vs_oracle_host_and_device(cg, orc, nch):
    import torch

    rng = np.random.default_rng(100 + nch)
    nf, pre = 97, int(rng.integers(0, 5000))
    fr = _framed(rng, nch, nf, pre)
    spf = 10000 // (nch // 4)
    for ns in (int(rng.integers(1, nf * spf)), (nf - 1) * spf, nf * spf + 5):
        good, ref = orc.mark5b_decode_framed(fr, nch, ns)
        out = np.zeros((nch, ns), np.float32)
        info = cg.mark5b_decode(fr, nch, ns, out)
        assert info.good_samples == good and info.first_frame_offset == pre and info.frames == nf
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
        d = torch.zeros((nch, ns), dtype=torch.float32, device="cuda")
        info = cg.mark5b_decode(torch.from_numpy(fr).cuda(), nch, ns, d)
        assert info.good_samples == good
        assert np.array_equal(d.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_decode_leaves_samples_past_the_last_frame(cg):
    import synth

    rng = np.random.default_rng(8)
    fr = synth.mark5b_frames(rng.integers(0, 256, 3 * 10000, dtype=np.uint8))
    ns = 3 * 2500 + 100
    out = np.full((16, ns), 7.0, np.float32)
    info = cg.mark5b_decode(fr, 16, ns, out)
    assert info.good_samples == -1
    assert np.all(out[:, 7500:] == 7.0) and np.all(out[:, :7500] != 7.0)


def test_decode_without_frames_raises(cg):
    junk = np.zeros(3 * 10016, np.uint8)
    with pytest.raises(cg.CellspeError) as e:
        cg.mark5b_decode(junk, 16, 100, np.zeros((16, 100), np.float32))
    assert e.value.code == cg.ERR_ARG


@pytest.mark.parametrize("nch", [16, 4])
def test_deframe_payload_and_mask(cg, orc, nch):
    rng = np.random.default_rng(30 + nch)
    nf, pre = 41, 333
    fr = _framed(rng, nch, nf, pre, fill_every=2)
    info = cg.mark5b_deframe(fr, nch)
    assert info.frames == nf and info.first_frame_offset == pre
    spf = 10000 // (nch // 4)
    pay = np.zeros(nf * 10000, np.uint8)
    mask = np.zeros((nf * spf + 31) // 32, np.uint32)
    cg.mark5b_deframe(fr, nch, 0, pay, mask)
    frames = fr[pre:pre + nf * 10016].reshape(nf, 10016)
    assert np.array_equal(pay, frames[:, 16:].reshape(-1))
    _, ref = orc.mark5b_decode_framed(fr, nch, nf * spf - 1)
    valid = np.unpackbits(mask.view(np.uint8), bitorder="little")[: nf * spf - 1].astype(bool)
    assert np.array_equal(valid, ref[0] != 0.0)


def _spec_oracle(orc, fr, nch, N, overlap, K, nspec, tb, fs):
    good, planes = orc.mark5b_decode_framed(fr, nch, N * K * nspec)
    pw, pc = [], []
    for c in range(nch):
        p, b = orc.spectrometer(planes[c], N, overlap, 2, K, tb, tb, 0.0, fs)
        pw.append(p)
        pc.append(b)
    return np.stack(pw), np.stack(pc)


@pytest.mark.parametrize("nch,N,overlap,K,nspec", [(16, 4096, 2, 4, 2), (8, 2048, 1, 6, 3), (4, 8192, 2, 3, 1)])
def test_spectrometer_on_framed_input_vs_oracle(cg, orc, nch, N, overlap, K, nspec):
    import synth

    fs, tb = 32e6, 32
    T = N * K * nspec
    spf = 10000 // (nch // 4)
    nf = -(-T // spf) + 1
    words, _ = synth.mark5b_subbands(16, nf * spf, fs_hz=fs, seed=nch + N, n_channels=N // 2, pcal_amp=0.3)
    codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nch)], axis=1)
    payload = synth.pack2bit(codes.reshape(-1))
    rng = np.random.default_rng(nch)
    pre = 77
    fr = synth.mark5b_frames(payload, prefix=pre)
    for f in range(1, nf, 2):
        a = int(rng.integers(1, 2500)) * 4
        synth.mark5b_fill(fr, f, 0, a, pre) if f % 4 == 1 else synth.mark5b_fill(fr, f, a, 10000, pre)
    p = cg.spec_params(N, overlap, 2, K, nspec, nch, fr.size, layout=cg.SPEC_MARK5B_FRAMED, tonebins=tb,
                       rotatorlen=tb, ntones=16, fs_hz=fs)
    power = np.zeros((nch, nspec, N // 2 + 1), np.float32)
    bins = np.zeros((nch, nspec, tb), np.complex64)
    cg.spectrometer(p, fr, power, bins)
    ref_p, ref_b = _spec_oracle(orc, fr, nch, N, overlap, K, nspec, tb, fs)
    assert np.linalg.norm(power - ref_p) / np.linalg.norm(ref_p) < 1e-5
    assert np.linalg.norm(bins - ref_b) / np.linalg.norm(ref_b) < 1e-5


@pytest.mark.parametrize("nch,N,K,fill", [(16, 65536, 4, (3, 4)), (4, 32768, 2, (2,))])
def test_long_fft_framed_spectrometer_with_blanked_and_clean_windows(cg, orc, nch, N, K, fill):
    """N = 32768 / 65536 run the warp four-step power kernel, which applies the
    blanking mask only to windows that contain a blanked sample: fill in a
    few frames gives both kinds of window in one call (16 channels, N = 65536:
    only the first of 7 overlapped windows touches frames 3 and 4)."""
    import synth

    fs, tb, nspec, overlap = 32e6, 32, 1, 2
    T = N * K * nspec
    spf = 10000 // (nch // 4)
    nf = -(-T // spf) + 1
    words, _ = synth.mark5b_subbands(16, nf * spf, fs_hz=fs, seed=nch + N + 1, n_channels=N // 2, pcal_amp=0.3)
    codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nch)], axis=1)
    payload = synth.pack2bit(codes.reshape(-1))
    pre = 77
    fr = synth.mark5b_frames(payload, prefix=pre)
    for f in fill:
        synth.mark5b_fill(fr, f, 0, 10000, pre)
    p = cg.spec_params(N, overlap, 2, K, nspec, nch, fr.size, layout=cg.SPEC_MARK5B_FRAMED, tonebins=tb,
                       rotatorlen=tb, ntones=16, fs_hz=fs)
    power = np.zeros((nch, nspec, N // 2 + 1), np.float32)
    bins = np.zeros((nch, nspec, tb), np.complex64)
    cg.spectrometer(p, fr, power, bins)
    ref_p, ref_b = _spec_oracle(orc, fr, nch, N, overlap, K, nspec, tb, fs)
    assert np.linalg.norm(power - ref_p) / np.linalg.norm(ref_p) < 1e-5
    assert np.linalg.norm(bins - ref_b) / np.linalg.norm(ref_b) < 1e-5


def test_framed_spectrometer_equals_payload_spectrometer_at_scale(cg):
    """Size-independent property: with no fill, framed input gives bit-identical
    spectra to the stripped payload through the interleaved layout (16 ch,
    2^22 sample times, 16 MiB of payload, on the device)."""
    import torch

    import synth

    nch, N, K, nspec = 16, 65536, 16, 4
    T = N * K * nspec
    nf = -(-T // 2500)
    g = torch.Generator(device="cuda").manual_seed(5)
    payload = torch.randint(0, 256, (nf * 10000,), dtype=torch.uint8, device="cuda", generator=g)
    hdr = synth.mark5b_frames(np.zeros(nf * 10000, np.uint8)).reshape(nf, 10016)[:, :16]
    fr = torch.empty((nf, 10016), dtype=torch.uint8, device="cuda")
    fr[:, :16] = torch.from_numpy(hdr).cuda()
    fr[:, 16:] = payload.view(nf, 10000)
    fr = fr.reshape(-1)
    a = torch.zeros((nch, nspec, N // 2 + 1), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    cg.spectrometer(cg.spec_params(N, 2, 2, K, nspec, nch, fr.numel(), layout=cg.SPEC_MARK5B_FRAMED), fr, a)
    usable = (T * 4) // 16 * 16
    cg.spectrometer(cg.spec_params(N, 2, 2, K, nspec, nch, usable), payload[:usable].contiguous(), b)
    assert torch.equal(a, b)
