"""Seeded synthetic 2-bit sources (the engine's test-pattern inputs).

The reference's own drivers fill their raw buffers with synthetic patterns
(minicorrelator_ppu.c:131-133, (17*i+3*j) % 256); no recorded data ships with
it.  These generators produce the inputs of the benchmark configurations:

* ``stations_offset_binary`` -- S inputs that share a N(0,1) sky signal with
  correlation rho, each with its own integer lag, quantised at +-0.98 sigma
  to offset-binary codes 0..3 (levels -3.336, -1, +1, +3.336), 4 samples per
  byte, sample 0 in bits 1:0.
* ``mark5b_subbands`` -- nsub subbands of noise + phase-cal comb + narrowband
  sinusoids, quantised to Mark5B sign/magnitude codes and interleaved
  2 bits per channel into 32-bit words (mark5_format_mark5b.c:1852-1915).
* ``device_stations`` -- the same statistics as stations_offset_binary,
  generated on the GPU with torch (for the 512-input configuration whose
  4.3 G samples would take minutes on the host).
* ``device_delayed_stations`` -- a sky signal seen through per-input cubic
  geometric delays with fringe rotation (the 16-station configuration), so
  that delay-corrected visibilities are coherent.
* ``mark5b_frames`` / ``mark5b_fill`` -- a payload byte stream wrapped into
  Mark5B frames (16-byte header + 10000-byte payload) and fill-pattern
  (0x11223344) zones written over parts of payloads, the way a recorder marks
  missing data.
"""
from __future__ import annotations

import numpy as np

THRESH = 0.98
OFFSET_BINARY_LEVELS = np.array([-3.336, -1.0, 1.0, 3.336], np.float32)


def quantize_offset_binary(x: np.ndarray) -> np.ndarray:
    """Codes 0..3 for x < -t, -t <= x < 0, 0 <= x < t, x >= t."""
    return (np.searchsorted(np.array([-THRESH, 0.0, THRESH]), x, side="right")).astype(np.uint8)


def quantize_mark5b(x: np.ndarray) -> np.ndarray:
    """Mark5B code l with value lut[l], lut = {-H, +1, -1, +H}."""
    ob = quantize_offset_binary(x)
    return np.array([0, 2, 1, 3], np.uint8)[ob]


def pack2bit(codes: np.ndarray) -> np.ndarray:
    """Pack the last axis of 2-bit codes, 4 per byte, first code in bits 1:0."""
    c = codes.reshape(*codes.shape[:-1], -1, 4).astype(np.uint8)
    return (c[..., 0] | (c[..., 1] << 2) | (c[..., 2] << 4) | (c[..., 3] << 6)).astype(np.uint8)


def stations_offset_binary(S: int, T: int, rho: float, lags=None, seed: int = 1) -> np.ndarray:
    """uint8 [S][T/4].  Input s sees x_s(t) = sqrt(rho) c(t - lag_s) + sqrt(1-rho) n_s(t)."""
    assert T % 64 == 0
    rng = np.random.Generator(np.random.Philox(seed))
    lags = np.zeros(S, np.int64) if lags is None else np.asarray(lags, np.int64)
    pad = int(lags.max(initial=0)) + 1
    common = rng.standard_normal(T + pad).astype(np.float32)
    out = np.empty((S, T // 4), np.uint8)
    a, b = np.float32(np.sqrt(rho)), np.float32(np.sqrt(1.0 - rho))
    for s in range(S):
        n = rng.standard_normal(T).astype(np.float32)
        sig = common[pad - lags[s] : pad - lags[s] + T]   # c(t - lag)
        out[s] = pack2bit(quantize_offset_binary(a * sig + b * n))
    return out


def mark5b_subbands(nsub: int, T: int, fs_hz: float, seed: int = 2, pcal_spacing_hz: float = 1e6,
                    pcal_amp: float = 0.05, n_sines: int = 3, snr_db: float = 10.0, n_channels: int = 32768,
                    chunk: int = 1 << 22):
    """Mark5B-style payload (uint32 words, T of them) and the injected truth.

    Per subband: N(0,1) noise + phase-cal comb at k*spacing (k = 1..fs/2/spacing-1)
    with amplitude pcal_amp and seeded phases + n_sines sinusoids at seeded
    frequencies with A^2/2 = 10^(snr_db/10) / n_channels (SNR per channel).
    """
    assert T % chunk == 0 or T < chunk
    chunk = min(chunk, T)
    rng = np.random.Generator(np.random.Philox(seed))
    ntone = int(fs_hz / 2 / pcal_spacing_hz)
    tone_k = np.arange(1, ntone)
    tone_phase = rng.uniform(0, 2 * np.pi, (nsub, tone_k.size))
    sine_f = rng.uniform(0.05, 0.45, (nsub, n_sines)) * fs_hz
    sine_phase = rng.uniform(0, 2 * np.pi, (nsub, n_sines))
    sine_amp = np.sqrt(2 * 10 ** (snr_db / 10) / n_channels)
    words = np.zeros(T, np.uint32)
    for t0 in range(0, T, chunk):
        t = (np.arange(t0, t0 + chunk, dtype=np.float64)) / fs_hz
        for c in range(nsub):
            x = rng.standard_normal(chunk)
            for i, k in enumerate(tone_k):
                x += pcal_amp * np.cos(2 * np.pi * k * pcal_spacing_hz * t + tone_phase[c, i])
            for i in range(n_sines):
                x += sine_amp * np.cos(2 * np.pi * sine_f[c, i] * t + sine_phase[c, i])
            code = quantize_mark5b(x.astype(np.float32)).astype(np.uint32)
            words[t0 : t0 + chunk] |= code << np.uint32(2 * c)
    truth = dict(tone_k=tone_k, tone_phase=tone_phase, sine_f=sine_f, sine_phase=sine_phase)
    return words, truth


def device_stations(S: int, T: int, rho: float, seed: int, device="cuda", chunk: int = 1 << 24):
    """torch uint8 [S][T/4] on the device, offset-binary codes (no lags)."""
    import torch

    assert T % chunk == 0 or T < chunk
    chunk = min(chunk, T)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = torch.empty((S, T // 4), dtype=torch.uint8, device=device)
    a, b = float(np.sqrt(rho)), float(np.sqrt(1.0 - rho))
    thr = torch.tensor([-THRESH, 0.0, THRESH], device=device)
    shifts = torch.tensor([0, 2, 4, 6], dtype=torch.uint8, device=device)
    for t0 in range(0, T, chunk):
        common = torch.randn(chunk, generator=g, device=device)
        for s0 in range(0, S, 64):
            s1 = min(S, s0 + 64)
            n = torch.randn((s1 - s0, chunk), generator=g, device=device)
            x = a * common + b * n
            codes = torch.bucketize(x, thr, right=True).to(torch.uint8).view(s1 - s0, -1, 4)
            packed = (codes << shifts).sum(dim=-1, dtype=torch.uint8)
            out[s0:s1, t0 // 4 : (t0 + chunk) // 4] = packed
    return out


def geometric_delay_state(poly, N: int, K: int, fs_hz: float, lo_hz: float):
    """Per (input, segment) delay seen by the sky signal, in FP64.

    tau(t) = sum_m poly[s, m] t^m at the segment centre t = (k N + N/2) / fs:
    integer sample shift round(tau fs), fringe phase 2 pi (lo tau mod 1) and
    the per-channel phase step 2 pi (fs / N) (tau - shift / fs) -- the delay
    model the engine's header (cellspe_fx_correlate) defines.
    """
    poly = np.asarray(poly, np.float64)
    t = (np.arange(K, dtype=np.float64) * N + N / 2) / fs_hz
    tau = np.zeros((poly.shape[0], K))
    for m in range(poly.shape[1] - 1, -1, -1):
        tau = tau * t[None, :] + poly[:, m:m + 1]
    shift = np.rint(tau * fs_hz).astype(np.int64)
    cyc = lo_hz * tau
    phase0 = 2 * np.pi * (cyc - np.floor(cyc))
    dphase = 2 * np.pi * (fs_hz / N) * (tau - shift / fs_hz)
    return shift, phase0, dphase


def device_delayed_stations(S: int, N: int, K: int, poly, fs_hz: float, lo_hz: float, rho: float, seed: int,
                            margin: int, device="cuda", chunk: int = 128):
    """A common sky signal seen by S inputs through a delay model (torch uint8 [S][(N K + 2 margin) / 4]).

    Each N-sample segment k is synthesised in the frequency domain: channel c
    of input s carries sqrt(rho) S_k(c) exp(-i (phase0 + c dphase)) +
    sqrt(1 - rho) n_{s,k}(c) (complex N(0,1) spectra, the sky at RF lo + c fs/N
    delayed by tau_s(t_k)), is brought to the time domain by an inverse real
    FFT, quantised to offset-binary 2-bit codes at +-0.98 sigma and written at
    sample margin + k N + shift[s, k], where the delay model's segment k
    starts.  The engine's delay correction therefore makes the inputs coherent
    again (|V_ij| ~ 0.88 rho per sample); samples no segment covers are noise.
    """
    import torch

    shift, phase0, dphase = geometric_delay_state(poly, N, K, fs_hz, lo_hz)
    lo_s, hi_s = int(shift.min()), int(shift.max())
    assert margin + lo_s >= 0 and margin + hi_s + N * K <= N * K + 2 * margin, "margin too small for the delays"
    Tt = N * K + 2 * margin
    assert Tt % 4 == 0
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    thr = torch.tensor([-THRESH, 0.0, THRESH], device=device)
    codes = torch.bucketize(torch.randn((S, Tt), generator=g, device=device), thr, right=True).to(torch.uint8)
    C = N // 2 + 1
    c = torch.arange(C, dtype=torch.float64, device=device)
    a, b = float(np.sqrt(rho)), float(np.sqrt(1.0 - rho))
    sh_d = torch.from_numpy(shift).to(device)
    p0_d = torch.from_numpy(phase0).to(device)
    dp_d = torch.from_numpy(dphase).to(device)
    n_idx = torch.arange(N, dtype=torch.int64, device=device)
    for k0 in range(0, K, chunk):
        k1 = min(K, k0 + chunk)
        kc = k1 - k0
        sky = torch.complex(torch.randn((kc, C), generator=g, device=device),
                            torch.randn((kc, C), generator=g, device=device)) * (0.5 ** 0.5)
        noise = torch.complex(torch.randn((S, kc, C), generator=g, device=device),
                              torch.randn((S, kc, C), generator=g, device=device)) * (0.5 ** 0.5)
        ph = p0_d[:, k0:k1, None] + c[None, None, :] * dp_d[:, k0:k1, None]          # FP64 phases
        rot = torch.polar(torch.ones_like(ph), -ph).to(torch.complex64)
        Y = a * sky[None] * rot + b * noise
        x = torch.fft.irfft(Y, n=N, dim=-1) * float(np.sqrt(N))                      # ~N(0,1) per sample
        q = torch.bucketize(x, thr, right=True).to(torch.uint8)
        start = margin + (torch.arange(k0, k1, device=device) * N)[None, :] + sh_d[:, k0:k1]   # [S][kc]
        idx = (start[:, :, None] + n_idx[None, None, :]).reshape(S, -1)
        codes.scatter_(1, idx, q.reshape(S, -1))
    shifts = torch.tensor([0, 2, 4, 6], dtype=torch.uint8, device=device)
    return (codes.view(S, -1, 4) << shifts).sum(dim=-1, dtype=torch.uint8)


MARK5B_FRAME = 10016
MARK5B_PAYLOAD = 10000


def _bcd(v: int, digits: int) -> int:
    out = 0
    for d in range(digits):
        out |= (v % 10) << (4 * d)
        v //= 10
    return out


def mark5b_frames(payload: np.ndarray, prefix: int = 0, first_frame: int = 0, seconds: int = 43210,
                  mjd_digits: int = 789, frames_per_second: int = 6400) -> np.ndarray:
    """Wrap payload bytes (a multiple of 10000) into Mark5B frames.

    Header words (little-endian): sync 0xABADDEED; frame number within the
    second in bits 0..14 of word 1; BCD time code JJJSSSSS in word 2 (last three
    MJD digits, seconds of day); word 3 zero.  ``prefix`` zero bytes precede the
    first frame.
    """
    payload = np.ascontiguousarray(payload, np.uint8).reshape(-1, MARK5B_PAYLOAD)
    nf = payload.shape[0]
    frames = np.zeros((nf, MARK5B_FRAME), np.uint8)
    hdr = np.zeros((nf, 4), np.uint32)
    n = first_frame + np.arange(nf)
    hdr[:, 0] = 0xABADDEED
    hdr[:, 1] = (n % frames_per_second).astype(np.uint32) & 0x7FFF
    for f in range(nf):
        sec = seconds + int(n[f] // frames_per_second)
        hdr[f, 2] = (_bcd(mjd_digits, 3) << 20) | _bcd(sec, 5)
    frames[:, :16] = hdr.view(np.uint8).reshape(nf, 16)
    frames[:, 16:] = payload
    return np.concatenate([np.zeros(prefix, np.uint8), frames.reshape(-1)])


def mark5b_fill(framed: np.ndarray, frame: int, start: int, end: int, prefix: int = 0) -> None:
    """Overwrite payload bytes [start, end) of one frame with the fill pattern
    (32-bit words 0x11223344; start and end multiples of 4)."""
    assert start % 4 == 0 and end % 4 == 0 and 0 <= start <= end <= MARK5B_PAYLOAD
    o = prefix + frame * MARK5B_FRAME + 16
    framed[o + start:o + end] = np.tile(np.array([0x44, 0x33, 0x22, 0x11], np.uint8), (end - start) // 4)


def vdif_frames(payload: np.ndarray, databytes: int = 8000, nchan: int = 4, mbps: int = 512,
                legacy: bool = False, seconds: int = 7654321, ref_epoch: int = 40, first_frame: int = 0,
                thread: int = 0, station: int = 0x4D62) -> np.ndarray:
    """Wrap payload bytes (a multiple of ``databytes``) into VDIF frames.

    Header words (little-endian, VDIF 1.0): word 0 = seconds from the reference
    epoch (bits 0..29), legacy flag (bit 30), invalid flag (bit 31, clear);
    word 1 = frame number within the second (bits 0..23), reference epoch
    (bits 24..29, half years since 2000); word 2 = frame length in 8-byte
    units (bits 0..23), log2(nchan) (bits 24..28); word 3 = bits per sample - 1
    (bits 26..30, 2-bit samples: 1), thread (bits 16..25), station (bits
    0..15); words 4..7 (non-legacy) zero.  Frames per second follow from mbps:
    mbps * 1e6 / (8 * databytes), which must be a whole number here.
    """
    hsize = 16 if legacy else 32
    fps = mbps * 1_000_000 // (8 * databytes)
    assert fps * 8 * databytes == mbps * 1_000_000, "frame rate must be whole"
    assert (databytes + hsize) % 8 == 0
    payload = np.ascontiguousarray(payload, np.uint8).reshape(-1, databytes)
    nf = payload.shape[0]
    n = first_frame + np.arange(nf, dtype=np.int64)
    hdr = np.zeros((nf, hsize // 4), np.uint32)
    hdr[:, 0] = ((seconds + n // fps) & 0x3FFFFFFF).astype(np.uint32) | (np.uint32(1 << 30) if legacy else 0)
    hdr[:, 1] = ((n % fps) & 0xFFFFFF).astype(np.uint32) | np.uint32((ref_epoch & 0x3F) << 24)
    hdr[:, 2] = np.uint32(((databytes + hsize) // 8) | ((nchan.bit_length() - 1) << 24))
    hdr[:, 3] = np.uint32((1 << 26) | ((thread & 0x3FF) << 16) | (station & 0xFFFF))
    frames = np.concatenate([hdr.view(np.uint8).reshape(nf, hsize), payload], axis=1)
    return frames.reshape(-1)


def vdif_set_invalid(framed: np.ndarray, frame: int, framebytes: int) -> None:
    """Set the invalid-data bit (word 0 bit 31) of one VDIF frame."""
    framed[frame * framebytes + 3] |= 0x80


def vdif_fill(framed: np.ndarray, frame: int, framebytes: int, hsize: int, start: int, end: int) -> None:
    """Overwrite payload bytes [start, end) of one VDIF frame with the fill
    pattern (32-bit words 0x11223344; start and end multiples of 4)."""
    assert start % 4 == 0 and end % 4 == 0 and 0 <= start <= end <= framebytes - hsize
    o = frame * framebytes + hsize
    framed[o + start:o + end] = np.tile(np.array([0x44, 0x33, 0x22, 0x11], np.uint8), (end - start) // 4)
