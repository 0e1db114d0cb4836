"""Framed VDIF input on the GPU: header model, frame validation and blanking, spectrometer.

The oracle is the restated mark5access memory-stream decode (pinned to the
compiled library and its golden vectors in test_oracle_golden.py)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
LEVELS = np.array([-3.3359, -1.0, 1.0, 3.3359, 0.0], np.float32)
GOLDEN = {"v4ch": (4, 128, 2000, 32), "v8ch_legacy": (8, 256, 2000, 16), "v16ch_granularity": (16, 8192, 2000, 32),
          "v1ch_day": (1, 128, 1024, 32), "v2ch_legacy": (2, 64, 1000, 16)}


def _stream(rng, db, nch, mbps, nf, legacy=False, edits=8):
    """Random payload, random epoch/seconds/first frame, `edits` random frame edits."""
    import synth

    hs = 16 if legacy else 32
    fb = db + hs
    fr = synth.vdif_frames(rng.integers(0, 256, nf * db, dtype=np.uint8), db, nch, mbps, legacy=legacy,
                           ref_epoch=int(rng.integers(0, 64)), seconds=int(rng.integers(0, 1 << 30)),
                           first_frame=int(rng.integers(0, 50)))
    for f in rng.choice(nf, min(edits, nf), replace=False):
        f = int(f)
        kind = int(rng.integers(0, 4))
        if kind == 0:
            synth.vdif_set_invalid(fr, f, fb)
        elif kind == 1:
            fr[f * fb + 4] ^= 1
        elif kind == 2:
            synth.vdif_fill(fr, f, fb, hs, 0, 8)
        else:
            synth.vdif_fill(fr, f, fb, hs, db - 8, db)
    return fr


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_decode_matches_golden(cg, name):
    nch, mbps, db, hs = GOLDEN[name]
    g = np.load(GOLD / "vdif_framed.npz")
    fr = g[f"{name}_framed"]
    for k, ns in enumerate(g[f"{name}_nsamp"]):
        out = np.zeros((nch, int(ns)), np.float32)
        info = cg.vdif_decode(fr, nch, mbps, int(ns), out)
        assert info.good_samples == int(g[f"{name}_rc{k}"])
        assert np.array_equal(out.view(np.uint32), LEVELS[g[f"{name}_codes{k}"]].view(np.uint32))
        assert (info.frame_bytes, info.header_bytes, info.frames) == (db + hs, hs, fr.size // (db + hs))


def test_info_fields(cg):
    import synth

    fr = synth.vdif_frames(np.zeros(4 * 8000, np.uint8), 8000, 16, 2048, ref_epoch=40, seconds=86400 * 3 + 61,
                           first_frame=10, thread=7, station=0x4142)
    info = cg.vdif_decode(fr, 16, 2048, 100, np.zeros((16, 100), np.float32))
    assert (info.mjd, info.seconds, info.frame_number) == (58849 + 3, 61, 10)   # epoch 40 = 2020-01-01
    assert info.ns == 10 * 31250 and info.nchan_header == 16
    assert (info.thread_id, info.station_id, info.blanked_frames) == (7, 0x4142, 0)


def test_first_frame_time_at_every_reference_epoch(cg):
    """info.mjd/seconds/ns against the library's own reading of the first header."""
    import synth

    want = np.load(GOLD / "vdif_framed.npz")["epoch_times"]
    for e in range(64):
        fr = synth.vdif_frames(np.zeros(2 * 1024, np.uint8), 1024, 4, 128, ref_epoch=e, seconds=5 * 86400 + 7,
                               first_frame=3)
        info = cg.vdif_decode(fr, 4, 128, 16, np.zeros((4, 16), np.float32))
        assert (info.mjd, info.seconds, info.ns) == tuple(int(v) for v in want[e]), e


@pytest.mark.parametrize("db,nch,mbps,legacy", [(8000, 4, 512, False), (8000, 16, 2048, True), (8192, 1, 1024, False),
                                                (1000, 2, 64, False), (8000, 8, 8192, False), (5000, 16, 4000, True)])
def test_decode_vs_oracle_host_and_device(cg, orc, db, nch, mbps, legacy):
    import torch

    rng = np.random.default_rng(db + nch + mbps)
    nf = 61
    fr = _stream(rng, db, nch, mbps, nf, legacy)
    spf = db * 4 // nch
    gran = 4 // nch if nch < 4 else 1
    for ns in (int(rng.integers(1, nf * spf // gran)) * gran, (nf - 1) * spf, nf * spf + 4 * gran):
        good, ref = orc.vdif_decode_framed(fr, nch, mbps, ns)
        out = np.zeros((nch, ns), np.float32)
        info = cg.vdif_decode(fr, nch, mbps, ns, out)
        assert info.good_samples == good and info.frames == nf
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
        d = torch.zeros((nch, ns), dtype=torch.float32, device="cuda")
        info = cg.vdif_decode(torch.from_numpy(fr).cuda(), nch, mbps, ns, d)
        assert info.good_samples == good
        assert np.array_equal(d.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    oks = [orc.vdif_frame_ok(fr, mbps, f) for f in range(nf)]
    assert info.blanked_frames == nf - sum(oks)


def test_decode_leaves_samples_past_the_last_frame(cg):
    import synth

    fr = synth.vdif_frames(np.full(3 * 8000, 0x1B, np.uint8), 8000, 4, 512)
    ns = 3 * 8000 + 100
    out = np.full((4, ns), 7.0, np.float32)
    info = cg.vdif_decode(fr, 4, 512, ns, out)
    assert info.good_samples == -1
    assert np.all(out[:, 24000:] == 7.0) and np.all(out[:, :24000] != 7.0)


def test_decode_rejects_bad_requests(cg):
    import synth

    fr = synth.vdif_frames(np.zeros(2 * 8000, np.uint8), 8000, 4, 512)
    for args in [(fr[:8032], 4, 512, 100),    # one frame only
                 (fr, 3, 512, 100),            # nchan
                 (fr, 4, 0, 100),              # Mbps
                 (fr, 1, 128, 6)]:             # 1 channel: multiple of 4 samples
        with pytest.raises(cg.CellspeError) as e:
            cg.vdif_decode(args[0], args[1], args[2], args[3], np.zeros((args[1], args[3]), np.float32))
        assert e.value.code == cg.ERR_ARG


@pytest.mark.parametrize("nch,legacy", [(16, False), (4, True), (1, False)])
def test_deframe_payload_and_mask(cg, orc, nch, legacy):
    rng = np.random.default_rng(40 + nch)
    db, mbps, nf = 8000, 512, 33
    fr = _stream(rng, db, nch, mbps, nf, legacy, edits=12)
    info = cg.vdif_deframe(fr, nch, mbps)
    hs = 16 if legacy else 32
    assert info.frames == nf and info.header_bytes == hs
    spf = db * 4 // nch
    pay = np.zeros(nf * db, np.uint8)
    mask = np.zeros((nf * spf + 31) // 32, np.uint32)
    cg.vdif_deframe(fr, nch, mbps, 0, pay, mask)
    frames = fr.reshape(nf, db + hs)
    assert np.array_equal(pay[db:], frames[1:, hs:].reshape(-1))
    assert np.array_equal(pay[:db], fr[32:32 + db])          # frame 0 read from byte 32
    _, ref = orc.vdif_decode_framed(fr, nch, mbps, nf * spf - 4)
    valid = np.unpackbits(mask.view(np.uint8), bitorder="little")[: nf * spf - 4].astype(bool)
    assert np.array_equal(valid, ref[0] != 0.0)


def _spec_oracle(orc, fr, nch, mbps, N, overlap, K, nspec, tb, fs):
    good, planes = orc.vdif_decode_framed(fr, nch, mbps, N * K * nspec)
    pw, pc = [], []
    for c in range(nch):
        p, b = orc.spectrometer(planes[c], N, overlap, 2, K, tb, tb, 0.0, fs)
        pw.append(p)
        pc.append(b)
    return np.stack(pw), np.stack(pc)


@pytest.mark.parametrize("nch,N,overlap,K,nspec,legacy", [(16, 4096, 2, 4, 2, False), (8, 2048, 1, 6, 3, True),
                                                          (4, 8192, 2, 3, 1, False), (1, 4096, 2, 2, 2, False)])
def test_spectrometer_on_vdif_vs_oracle(cg, orc, nch, N, overlap, K, nspec, legacy):
    import synth

    fs, tb, db = 16e6, 32, 8000
    mbps = int(fs * 2 * nch / 1e6)
    T = N * K * nspec
    spf = db * 4 // nch
    nf = -(-T // spf) + 2
    words, _ = synth.mark5b_subbands(16, nf * spf, fs_hz=fs, seed=nch + N, n_channels=N // 2, pcal_amp=0.3)
    codes = np.stack([(words >> np.uint32(2 * c)) & np.uint32(3) for c in range(nch)], axis=1)
    payload = synth.pack2bit(codes.reshape(-1))
    rng = np.random.default_rng(nch)
    fr = synth.vdif_frames(payload, db, nch, mbps, legacy=legacy, first_frame=3)
    hs = 16 if legacy else 32
    for f in range(1, nf, 3):
        synth.vdif_set_invalid(fr, f, db + hs) if rng.integers(0, 2) else synth.vdif_fill(fr, f, db + hs, hs, 0, 8)
    p = cg.spec_params(N, overlap, 2, K, nspec, nch, fr.size, layout=cg.SPEC_VDIF_FRAMED, levels=cg.LEVELS_VDIF,
                       tonebins=tb, rotatorlen=tb, ntones=16, fs_hz=fs)
    power = np.zeros((nch, nspec, N // 2 + 1), np.float32)
    bins = np.zeros((nch, nspec, tb), np.complex64)
    cg.spectrometer(p, fr, power, bins)
    ref_p, ref_b = _spec_oracle(orc, fr, nch, mbps, N, overlap, K, nspec, tb, fs)
    assert np.linalg.norm(power - ref_p) / np.linalg.norm(ref_p) < 1e-5
    assert np.linalg.norm(bins - ref_b) / np.linalg.norm(ref_b) < 1e-5


def test_vdif_spectrometer_equals_payload_spectrometer_at_scale(cg):
    """Size-independent property: with every frame valid, VDIF input gives
    bit-identical spectra to its payload through the interleaved layout (16 ch,
    2^22 sample times, 16 MiB of payload, 8192-byte payloads, on the device)."""
    import torch

    import synth

    nch, N, K, nspec, db = 16, 65536, 16, 4, 8192
    T = N * K * nspec
    nf = T * 4 // db + 1
    g = torch.Generator(device="cuda").manual_seed(6)
    payload = torch.randint(0, 256, (nf * db,), dtype=torch.uint8, device="cuda", generator=g)
    payload.view(nf, db)[:, :8] = 0x55        # no fill word can start a payload
    payload.view(nf, db)[:, -8:] = 0x55
    fs = 64e6
    mbps = int(fs * 2 * nch / 1e6)
    hdr = synth.vdif_frames(np.zeros(nf * db, np.uint8), db, nch, mbps).reshape(nf, db + 32)[:, :32]
    fr = torch.empty((nf, db + 32), dtype=torch.uint8, device="cuda")
    fr[:, :32] = torch.from_numpy(hdr).cuda()
    fr[:, 32:] = payload.view(nf, db)
    fr = fr.reshape(-1)
    a = torch.zeros((nch, nspec, N // 2 + 1), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    cg.spectrometer(cg.spec_params(N, 2, 2, K, nspec, nch, fr.numel(), layout=cg.SPEC_VDIF_FRAMED,
                                   levels=cg.LEVELS_VDIF, fs_hz=fs), fr, a)
    usable = (T * 4) // 16 * 16
    cg.spectrometer(cg.spec_params(N, 2, 2, K, nspec, nch, usable, levels=cg.LEVELS_VDIF), payload[:usable].contiguous(), b)
    assert torch.equal(a, b)


def test_xpol_on_vdif_equals_payload_xpol(cg):
    """Two framed VDIF sources through cellspe_spectrometer_xpol give bit-identical
    auto and cross spectra to their payloads through the interleaved layout when
    every frame is valid."""
    import synth

    nch, N, K, nspec, db, fs = 4, 4096, 4, 2, 8000, 32e6
    mbps = int(fs * 2 * nch / 1e6)
    spf = db * 4 // nch
    nf = -(-N * K * nspec // spf) + 1
    rng = np.random.default_rng(77)
    pays, frs = [], []
    for _ in range(2):
        pay = rng.integers(0, 256, nf * db, dtype=np.uint8)
        pay.reshape(nf, db)[:, :8] = 0x55              # no fill word can start or end a payload
        pay.reshape(nf, db)[:, -8:] = 0x55
        pays.append(pay)
        frs.append(synth.vdif_frames(pay, db, nch, mbps))
    nb = N // 2 + 1
    out = []
    for layout, bufs in ((cg.SPEC_VDIF_FRAMED, frs), (cg.SPEC_INTERLEAVED, pays)):
        p = cg.spec_params(N, 2, 2, K, nspec, nch, bufs[0].size, layout=layout, levels=cg.LEVELS_VDIF, fs_hz=fs)
        power = np.zeros((2, nspec, nb), np.float32)
        xpol = np.zeros((nspec, nb), np.complex64)
        cg.spectrometer_xpol(p, bufs[0], bufs[1], 1, 2, power, xpol)
        out.append((power, xpol))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
