"""CPU oracle for the FX correlator / spectrometer hot path.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg use this package, and only as the checker or
as the timed CPU baseline.  The product library (``cellspe-tasklib_gb300``)
never imports it and has no CPU fallback.

Contents
--------
* ``lib()``         -- ctypes handle on ``oracle/liboracle.so``, the plain-C
                       restatement (``cellspe_oracle.c``).
* ``ref_mark5()``   -- the reference's own mark5access 1.4.3, compiled from the
                       reference tree into ``oracle/_ref`` (this container only).
* ``ref_generic()`` -- the reference's GENERIC kernels of ``architecture.h``.
* FP64 numpy models: ``fx_spectra_f64``, ``fx_vis_f64``, ``delay_state_f64``.

Parity status: the 2-bit decode, the framed Mark5B and VDIF memory-stream
decodes (header strip, validation, blanking, end-of-data rule) and the
complex MAC are pinned bit-for-bit to the reference (mark5access,
architecture.h GENERIC), live and through the golden vectors in tests/golden.  The FFT is not
pinned by the reference (FFTW/IPP/Cell SDK absent): it is checked against an
FP64 DFT and analytic known answers.  The phase-cal fold is pinned by the
reference's own PCal unit-test recipe (tone phase within 0.1 degree).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"

_lib = None
_ref_m5 = None
_ref_gen = None

f32p = ctypes.POINTER(ctypes.c_float)


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def build(ref_tree: str | None = None) -> None:
    """Compile liboracle.so (always) and oracle/_ref from the reference tree
    ``ref_tree`` (else the CELLSPE_REFERENCE_TREE environment variable) when
    one is given and exists; without one only the restatement is built."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    ref_tree = ref_tree or os.environ.get("CELLSPE_REFERENCE_TREE")
    if ref_tree and Path(ref_tree).is_dir():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={ref_tree}"], check=True)
        (REF_DIR / "reference_tree.txt").write_text(str(Path(ref_tree).resolve()))


def reference_tree() -> Path | None:
    """The reference tree oracle/_ref was built from (None where it was not built)."""
    f = REF_DIR / "reference_tree.txt"
    if not f.exists():
        return None
    p = Path(f.read_text().strip())
    return p if p.is_dir() else None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        so = HERE / "liboracle.so"
        if not so.exists():
            build()
        _lib = ctypes.CDLL(str(so))
        V, I, L = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        _lib.orc_unpack2bit.argtypes = [V, L, I, I, V, V]
        _lib.orc_addproduct_32fc.argtypes = [V, V, V, I]
        _lib.orc_addproduct_32fc_conj.argtypes = [V, V, V, I]
        _lib.orc_cfft_f32.argtypes = [V, V, I]
        _lib.orc_cfft_f64.argtypes = [V, V, I]
        _lib.orc_rfft_f32.argtypes = [V, V, I]
        _lib.orc_spectrometer.argtypes = [V, L, V, V, V]
        _lib.orc_spectrometer.restype = I
        _lib.orc_spectrometer_xpol.argtypes = [V, V, L, V, V, V, V]
        _lib.orc_spectrometer_xpol.restype = I
        _lib.orc_spec_window.argtypes = [I, I, V]
        _lib.orc_pcal_tones.argtypes = [V, I, I, V]
        _lib.orc_fx_fp32.argtypes = [V, L, I, I, I, L, V, V, V, I, V, I]
        _lib.orc_fx_fstage_fp32.argtypes = [V, L, I, I, I, L, V, V, V, I, V, I]
        _lib.orc_mark5b_find_first_frame.argtypes = [V, L]
        _lib.orc_mark5b_valid_range.argtypes = [V, ctypes.POINTER(I), ctypes.POINTER(I)]
        _lib.orc_mark5b_decode_framed.argtypes = [V, L, I, L, V]
        _lib.orc_mark5b_decode_framed.restype = L
        _lib.orc_vdif_frame_ok.argtypes = [V, L, I, L]
        _lib.orc_vdif_decode_framed.argtypes = [V, L, I, I, L, V]
        _lib.orc_vdif_decode_framed.restype = L
        _lib.orc_vdif_first_time.argtypes = [V, L, I, V, V, V]
    return _lib


def have_ref() -> bool:
    return (REF_DIR / "libref_mark5.so").exists() and (REF_DIR / "libref_generic.so").exists()


def ref_mark5() -> ctypes.CDLL:
    global _ref_m5
    if _ref_m5 is None:
        _ref_m5 = ctypes.CDLL(str(REF_DIR / "libref_mark5.so"))
        _ref_m5.ref_mark5_unpack.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    return _ref_m5


def ref_mark5_decode_memory(fmt: bytes, framed: np.ndarray, nsamp: int):
    """The reference's framed decode (mark5access memory stream + mark5_stream_decode)."""
    m5 = ref_mark5()
    m5.ref_mark5_decode_memory.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)]
    buf = np.ascontiguousarray(framed, np.uint8).copy()
    nch = int(fmt.split(b"-")[2])
    out = np.zeros((nch, nsamp), np.float32)
    c, off = ctypes.c_int(), ctypes.c_int()
    rc = m5.ref_mark5_decode_memory(fmt, buf.ctypes.data, buf.size, nsamp, out.ctypes.data, ctypes.byref(c),
                                    ctypes.byref(off))
    return rc, out, off.value


def mark5b_decode_framed(framed: np.ndarray, nchan: int, nsamp: int):
    framed = np.ascontiguousarray(framed, np.uint8)
    out = np.zeros((nchan, nsamp), np.float32)
    good = lib().orc_mark5b_decode_framed(_ptr(framed), framed.size, nchan, nsamp, _ptr(out))
    return good, out


def vdif_decode_framed(framed: np.ndarray, nchan: int, mbps: int, nsamp: int):
    """(good samples or -1/-2/-3, out[nchan][nsamp]) of a framed VDIF buffer."""
    framed = np.ascontiguousarray(framed, np.uint8)
    out = np.zeros((nchan, nsamp), np.float32)
    good = lib().orc_vdif_decode_framed(_ptr(framed), framed.size, nchan, mbps, nsamp, _ptr(out))
    return good, out


def vdif_first_time(framed: np.ndarray, mbps: int):
    """(mjd, seconds, ns) of frame 0 as the memory stream reads it."""
    framed = np.ascontiguousarray(framed, np.uint8)
    t = (ctypes.c_int * 3)()
    rc = lib().orc_vdif_first_time(_ptr(framed), framed.size, mbps, ctypes.byref(t, 0), ctypes.byref(t, 4),
                                   ctypes.byref(t, 8))
    assert rc == 0
    return tuple(t)


def ref_mark5_stream_time(fmt: bytes, framed: np.ndarray):
    """(mjd, seconds, ns) of the first frame as the compiled library reads it."""
    m5 = ref_mark5()
    m5.ref_mark5_stream_time.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint] + [ctypes.c_void_p] * 3
    buf = np.ascontiguousarray(framed, np.uint8).copy()
    t = (ctypes.c_int * 3)()
    rc = m5.ref_mark5_stream_time(fmt, buf.ctypes.data, buf.size, ctypes.byref(t, 0), ctypes.byref(t, 4),
                                  ctypes.byref(t, 8))
    assert rc == 0, rc
    return tuple(t)


def vdif_frame_ok(framed: np.ndarray, mbps: int, frame: int) -> int:
    framed = np.ascontiguousarray(framed, np.uint8)
    return lib().orc_vdif_frame_ok(_ptr(framed), framed.size, mbps, frame)


def ref_generic() -> ctypes.CDLL:
    global _ref_gen
    if _ref_gen is None:
        _ref_gen = ctypes.CDLL(str(REF_DIR / "libref_generic.so"))
        for name in ("ref_addproduct_32fc", "ref_addproduct_32fc_conj", "ref_mul_32fc",
                     "ref_mul_32fc_conj"):
            getattr(_ref_gen, name).argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int]
    return _ref_gen


# ---------------------------------------------------------------------------
# thin wrappers over the C restatement
# ---------------------------------------------------------------------------
MARK5B_LUT = np.array([-3.3359, 1.0, -1.0, 3.3359], np.float32)       # mark5_format_mark5b.c:63
TWOBIT_LUT = np.array([1.0, -1.0, 3.3359, -3.3359], np.float32)       # DataUnpackers.cpp:195
OFFSET_BINARY_LUT = np.array([-3.336, -1.0, 1.0, 3.336], np.float32)  # synthetic configs


def unpack2bit(raw: np.ndarray, nsamp: int, nchan: int, lut, msb_first: bool = False) -> np.ndarray:
    raw = np.ascontiguousarray(raw, np.uint8)
    lut = np.ascontiguousarray(lut, np.float32)
    out = np.empty((nchan, nsamp), np.float32)
    lib().orc_unpack2bit(_ptr(raw), nsamp, nchan, int(msb_first), _ptr(lut), _ptr(out))
    return out


def addproduct(a, b, acc, conj: bool):
    fn = lib().orc_addproduct_32fc_conj if conj else lib().orc_addproduct_32fc
    fn(_ptr(a), _ptr(b), _ptr(acc), a.size)
    return acc


def rfft_f32(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty(x.size // 2 + 1, np.complex64)
    lib().orc_rfft_f32(_ptr(x), _ptr(out), x.size)
    return out


def cfft_f32(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.complex64)
    out = np.empty_like(x)
    lib().orc_cfft_f32(_ptr(x), _ptr(out), x.size)
    return out


class SpecCfg(ctypes.Structure):
    _fields_ = [("fft_points", ctypes.c_int), ("overlap", ctypes.c_int), ("window", ctypes.c_int),
                ("ffts_per_spectrum", ctypes.c_int), ("pcal_tonebins", ctypes.c_int),
                ("pcal_rotatorlen", ctypes.c_int), ("pcal_offset_hz", ctypes.c_double),
                ("sample_rate_hz", ctypes.c_double)]


def spectrometer(samples: np.ndarray, N: int, overlap: int, window: int, K: int,
                 tonebins: int = 0, rotatorlen: int = 0, offset_hz: float = 0.0,
                 fs_hz: float = 1.0):
    samples = np.ascontiguousarray(samples, np.float32)
    cfg = SpecCfg(N, overlap, window, K, tonebins, rotatorlen, offset_hz, fs_hz)
    nspec_max = max(1, samples.size // (N * K))
    power = np.zeros((nspec_max, N // 2 + 1), np.float32)
    pc = np.zeros((nspec_max, max(tonebins, 1)), np.complex64)
    n = lib().orc_spectrometer(_ptr(samples), samples.size, ctypes.byref(cfg), _ptr(power),
                               _ptr(pc) if tonebins else None)
    return power[:n], (pc[:n] if tonebins else None)


def spectrometer_xpol(s0: np.ndarray, s1: np.ndarray, N: int, overlap: int, window: int, K: int,
                      tonebins: int = 0, rotatorlen: int = 0, offset_hz: float = 0.0, fs_hz: float = 1.0):
    """Two sources: (power [2][nspec][N/2+1], xpol [nspec][N/2+1], pcal [2][nspec][tonebins] or None)."""
    s0 = np.ascontiguousarray(s0, np.float32)
    s1 = np.ascontiguousarray(s1, np.float32)
    assert s0.size == s1.size
    cfg = SpecCfg(N, overlap, window, K, tonebins, rotatorlen, offset_hz, fs_hz)
    nspec = s0.size // (N * K)
    power = np.zeros((2, nspec, N // 2 + 1), np.float32)
    xpol = np.zeros((nspec, N // 2 + 1), np.complex64)
    pc = np.zeros((2, nspec, max(tonebins, 1)), np.complex64)
    n = lib().orc_spectrometer_xpol(_ptr(s0), _ptr(s1), s0.size, ctypes.byref(cfg), _ptr(power), _ptr(xpol),
                                    _ptr(pc) if tonebins else None)
    assert n == nspec
    return power, xpol, (pc if tonebins else None)


def window(kind: int, n: int) -> np.ndarray:
    w = np.empty(n, np.float32)
    lib().orc_spec_window(kind, n, _ptr(w))
    return w


def pcal_tones(bins: np.ndarray, ntones: int) -> np.ndarray:
    bins = np.ascontiguousarray(bins, np.complex64)
    out = np.empty(ntones, np.complex64)
    lib().orc_pcal_tones(_ptr(bins), bins.size, ntones, _ptr(out))
    return out


def fx_fp32(raw, S, N, K, start_sample=0, shift=None, phasor=None, lut=OFFSET_BINARY_LUT,
            msb_first=False, nthreads=1):
    """FP32 CPU FX path; returns vis[P][C] complex64 (baseline-major)."""
    raw = np.ascontiguousarray(raw, np.uint8).reshape(S, -1)
    C = N // 2
    P = S * (S + 1) // 2
    vis = np.zeros((P, C), np.complex64)
    sh = None if shift is None else np.ascontiguousarray(shift, np.int32)
    ph = None if phasor is None else np.ascontiguousarray(phasor, np.complex64)
    lut = np.ascontiguousarray(lut, np.float32)
    lib().orc_fx_fp32(_ptr(raw), raw.shape[1], S, N, K, start_sample,
                      _ptr(sh) if sh is not None else None,
                      _ptr(ph) if ph is not None else None, _ptr(lut), int(msb_first),
                      _ptr(vis), nthreads)
    return vis


def fx_fstage_fp32(raw, S, N, K, start_sample=0, shift=None, phasor=None,
                   lut=OFFSET_BINARY_LUT, msb_first=False, nthreads=1):
    raw = np.ascontiguousarray(raw, np.uint8).reshape(S, -1)
    C = N // 2
    out = np.empty((S, K, C), np.complex64)
    sh = None if shift is None else np.ascontiguousarray(shift, np.int32)
    ph = None if phasor is None else np.ascontiguousarray(phasor, np.complex64)
    lut = np.ascontiguousarray(lut, np.float32)
    lib().orc_fx_fstage_fp32(_ptr(raw), raw.shape[1], S, N, K, start_sample,
                             _ptr(sh) if sh is not None else None,
                             _ptr(ph) if ph is not None else None, _ptr(lut), int(msb_first),
                             _ptr(out), nthreads)
    return out


# ---------------------------------------------------------------------------
# FP64 models
# ---------------------------------------------------------------------------
def unpack_segments_f64(raw, S, N, K, start_sample, shift, lut, msb_first=False,
                        inputs=None):
    """Decoded samples [len(inputs)][K][N] in float64 (exact: table values)."""
    raw = np.ascontiguousarray(raw, np.uint8).reshape(S, -1)
    inputs = range(S) if inputs is None else inputs
    lut = np.asarray(lut, np.float32).astype(np.float64)
    out = np.empty((len(inputs), K, N), np.float64)
    n = np.arange(N, dtype=np.int64)
    for ii, s in enumerate(inputs):
        for k in range(K):
            st = start_sample + k * N + (0 if shift is None else int(shift[s, k]))
            f = st + n
            b = raw[s, f >> 2]
            sh = (6 - 2 * (f & 3)) if msb_first else (2 * (f & 3))
            out[ii, k] = lut[(b >> sh) & 3]
    return out


def fx_spectra_f64(raw, S, N, K, start_sample=0, shift=None, phase0=None, dphase=None,
                   lut=OFFSET_BINARY_LUT, msb_first=False, inputs=None, channels=None):
    """FP64 F stage: X[s][k][c] = rfft(x)[c] * exp(i*(phase0[s,k] + c*dphase[s,k]))."""
    inputs = list(range(S)) if inputs is None else list(inputs)
    x = unpack_segments_f64(raw, S, N, K, start_sample, shift, lut, msb_first, inputs)
    X = np.fft.rfft(x, axis=-1)[..., : N // 2]
    if channels is not None:
        X = X[..., channels]
        c = np.asarray(channels, np.float64)
    else:
        c = np.arange(N // 2, dtype=np.float64)
    if phase0 is not None:
        p0 = np.asarray(phase0, np.float64)[inputs][:, :, None]
        dp = np.asarray(dphase, np.float64)[inputs][:, :, None]
        X = X * np.exp(1j * (p0 + c[None, None, :] * dp))
    return X


def fx_vis_f64(X: np.ndarray, pairs):
    """V[p][c] = sum_k X_i[k][c] * conj(X_j[k][c]) for (i, j) in pairs (indices into X)."""
    out = np.empty((len(pairs), X.shape[-1]), np.complex128)
    for n, (i, j) in enumerate(pairs):
        out[n] = np.einsum("kc,kc->c", X[i], np.conj(X[j]))
    return out


def delay_state_f64(poly: np.ndarray, N: int, K: int, fs_hz: float, lo_hz: float):
    """Per (input, segment) integer shift, fringe phase and per-channel phase step.

    tau(t) = sum_m poly[s, m] t^m at the segment centre t = (k*N + N/2)/fs.
    shift = round(tau*fs); frac = tau - shift/fs.
    phase0 = 2*pi*lo*tau (reduced mod 2*pi); dphase = 2*pi*(fs/N)*frac.
    The correction multiplies channel c by exp(i*(phase0 + c*dphase)).
    """
    poly = np.asarray(poly, np.float64)
    S = poly.shape[0]
    t = (np.arange(K, dtype=np.float64) * N + N / 2) / fs_hz
    tau = np.zeros((S, K))
    for m in range(poly.shape[1] - 1, -1, -1):
        tau = tau * t[None, :] + poly[:, m : m + 1]
    shift = np.rint(tau * fs_hz).astype(np.int64)
    frac = tau - shift / fs_hz
    cyc = lo_hz * tau
    phase0 = 2 * np.pi * (cyc - np.floor(cyc))
    dphase = 2 * np.pi * (fs_hz / N) * frac
    return shift.astype(np.int32), phase0, dphase


def tri_index(i: int, j: int) -> int:
    return i * (i + 1) // 2 + j


def _decode_rows(raw_row: np.ndarray, first: np.ndarray, N: int, lut64: np.ndarray, msb_first: bool):
    """Samples [len(first)][N] of one input whose segments start at sample first[k]."""
    f = first[:, None] + np.arange(N, dtype=np.int64)[None, :]
    b = raw_row[f >> 2]
    sh = (6 - 2 * (f & 3)) if msb_first else (2 * (f & 3))
    return lut64[(b >> sh.astype(np.uint8)) & 3]


def fx_vis_subset_f64(raw_rows, N: int, K: int, channels, start_sample: int = 0, shift=None, phase0=None,
                      dphase=None, lut=OFFSET_BINARY_LUT, msb_first: bool = False, chunk: int = 256):
    """FP64 visibilities of a subset of inputs and channels, streamed over segments.

    raw_rows: uint8 [n][bytes] -- the raw bytes of the chosen inputs (row a of
    the result's inputs is raw_rows[a]); shift / phase0 / dphase: [n][K] rows
    of the delay state of those inputs (or None).  Spectra are an exact DFT at
    the chosen channels, X[c] = sum_t x[t] exp(-2 pi i c t / N) with the
    argument reduced in integers, multiplied by exp(i (phase0 + c dphase)) as
    the engine's model defines (fx_spectra_f64), and accumulated as
    V[a][b][c] = sum_k X_a[k][c] conj(X_b[k][c]) for b <= a.  Memory stays at
    one chunk of segments, so K = 4096 at N = 8192 is a few seconds per input.
    Returns (V [n][n][len(channels)] complex128 with the lower triangle and the
    diagonal filled, autos [n][len(channels)] float64).
    """
    raw_rows = np.ascontiguousarray(raw_rows, np.uint8)
    n = raw_rows.shape[0]
    ch = np.asarray(channels, np.int64)
    t = np.arange(N, dtype=np.int64)
    W = np.exp(-2j * np.pi * ((t[:, None] * ch[None, :]) % N) / N)           # [N][nc]
    lut64 = np.asarray(lut, np.float32).astype(np.float64)
    V = np.zeros((n, n, ch.size), np.complex128)
    for k0 in range(0, K, chunk):
        k1 = min(K, k0 + chunk)
        ks = np.arange(k0, k1, dtype=np.int64)
        X = np.empty((n, k1 - k0, ch.size), np.complex128)
        for a in range(n):
            first = start_sample + ks * N + (0 if shift is None else np.asarray(shift[a][k0:k1], np.int64))
            X[a] = _decode_rows(raw_rows[a], first, N, lut64, msb_first) @ W
            if phase0 is not None:
                p0 = np.asarray(phase0[a][k0:k1], np.float64)[:, None]
                dp = np.asarray(dphase[a][k0:k1], np.float64)[:, None]
                X[a] *= np.exp(1j * (p0 + ch[None, :].astype(np.float64) * dp))
        for a in range(n):
            V[a, : a + 1] += np.einsum("kc,bkc->bc", X[a], np.conj(X[: a + 1]))
    autos = np.stack([V[a, a].real for a in range(n)])
    return V, autos


def vis_errors(got, ref, autos, K: int):
    """Errors of visibilities against an FP64 reference, the engine's bars.

    got, ref: [n][n][nc] (lower triangle + diagonal used); autos: [n][nc].
    * amplitude: max over products of ||got - ref||_2 / ||ref||_2 over channels;
    * phase: max |arg(got conj(ref))| in degrees over (product, channel) whose
      |ref| is above the thermal-noise floor 3 sqrt(V_aa V_bb / K);
    * the number of cross products (b < a) with at least one channel above it.
    """
    n = ref.shape[0]
    amp, ph, cross_cov, cells = 0.0, 0.0, 0, 0
    for a in range(n):
        for b in range(a + 1):
            r, g = ref[a, b], got[a, b]
            amp = max(amp, float(np.linalg.norm(g - r) / np.linalg.norm(r)))
            floor = 3 * np.sqrt(autos[a] * autos[b] / K)
            m = np.abs(r) > floor
            if m.any():
                ph = max(ph, float(np.degrees(np.abs(np.angle(g[m] * np.conj(r[m])))).max()))
                cells += int(m.sum())
                cross_cov += int(a != b)
    return {"max_rel_amp": amp, "max_phase_deg": ph, "phase_cells": cells, "cross_products_above_floor": cross_cov,
            "products": n * (n + 1) // 2, "cross_products": n * (n - 1) // 2}


# ---------------------------------------------------------------------------
# Cell control blocks (restated from the SPE programs)
# ---------------------------------------------------------------------------
MC_PARTNER = (1, 3, 4)      # minicorrelator_spu.c:302-304: partners rank+1, rank+3, rank+4 (mod 6)


def minicorrelator_slots_f64(raws, ffts_total: int, ffts_to_integrate: int):
    """The minicorrelator SPE job (minicorrelator_spu.c:326-481, 835-866) as the
    engine defines it: station s = raws[s] (ffts_total x 256 bytes of 2-bit
    offset-binary samples), one 2048-sample segment per time period (two
    1024-sample FFT buffers), blocks of ffts_to_integrate / 2 segments.
    Returns (autos[s][b][1024], slots{slot: [b][1024]}) of FP64 complex sums,
    slot s + 6 m < 15 holding X_s conj(X_o), o = (s + MC_PARTNER[m]) % 6."""
    S, N = 6, 2048
    K = ffts_total // 2
    Kb = ffts_to_integrate // 2
    blocks = ffts_total // ffts_to_integrate
    raw = np.stack([np.asarray(r, np.uint8) for r in raws])
    X = fx_spectra_f64(raw, S, N, K)                       # [S][K][1024]
    X = X[:, : blocks * Kb].reshape(S, blocks, Kb, N // 2)
    autos = np.einsum("sbkc,sbkc->sbc", X, np.conj(X))
    slots = {}
    for s in range(S):
        for m, off in enumerate(MC_PARTNER):
            slot = s + S * m
            if slot < 15:
                o = (s + off) % S
                slots[slot] = np.einsum("bkc,bkc->bc", X[s], np.conj(X[o]))
    return autos, slots


def cell_spectrometer_f64(buffers, N: int, K: int, overlap: int, spr: int = 1, levels=None):
    """The Cell spectrometer SPE task (spectrometer_spu.c:96-205) over a
    sequence of raw buffers, one task each, as the engine defines it: FFT f
    of a buffer starts at byte f*d, d = (N/spr)//overlap, for
    f < min(len//d - 1, (len - N/spr)//d + 1); samples byte - 127.5 (spr 1)
    or 2-bit LSB-first codes through `levels` (spr 4); window
    sin^2(pi i/(N-1)) (calc_cos_window_function, :286-312); |X_k|^2 / K of
    the N-point FFT summed over K FFTs, the running spectrum carried from one
    task to the next; each finished spectrum as N {power, 0} pairs.
    Returns one list of spectra ([N][2] float64 arrays) per task."""
    w = np.sin(np.pi * np.arange(N) / (N - 1)) ** 2
    rb = N // spr
    d = rb // overlap
    acc = np.zeros(N)
    n = 0
    out = []
    lv = None if levels is None else np.asarray(levels, np.float64)
    for buf in buffers:
        buf = np.asarray(buf, np.uint8)
        B = buf.size
        nfft = min(B // d - 1 if B >= 2 * d else 0, (B - rb) // d + 1 if B >= rb else 0)
        spectra = []
        for f in range(nfft):
            chunk = buf[f * d: f * d + rb]
            if spr == 1:
                x = chunk.astype(np.float64) - 127.5
            else:
                codes = (chunk[:, None] >> (2 * np.arange(4))[None, :]) & 3
                x = lv[codes.reshape(-1)]
            X = np.fft.fft(x * w)
            acc += np.abs(X) ** 2 / K
            n += 1
            if n == K:
                spectra.append(np.stack([acc, np.zeros(N)], axis=1))
                acc = np.zeros(N)
                n = 0
        out.append(spectra)
    return out


# ---------------------------------------------------------------------------
# PCal library (spectrometer/src/IA-32/PhaseCal/PCal.cpp)
# ---------------------------------------------------------------------------
def pcal_config(bw: float, spacing: float, offset: int):
    """PCal::getNew's choice (PCal.cpp:92-112) and each extractor's derived
    sizes: (kind, nbins, rotlen, ntones, first, step); kind 0 Trivial,
    1 Shifting, 2 ImplicitShift."""
    from math import floor, gcd

    fs = int(2 * bw)
    sp = int(spacing)
    Np = fs // gcd(sp, fs)
    if offset == 0:
        return 0, Np, 1, int(floor(bw / spacing)), 0, 1
    No = fs // gcd(int(offset), fs)
    ntones = int(floor((bw - offset) / spacing)) + 1
    if No % Np == 0:
        return 2, No, 1, ntones, int(floor(No * offset / fs)), int(floor(No * (spacing / fs)))
    return 1, Np, No, ntones, 0, int(floor(Np * (spacing / fs)))


def pcal_extract_f64(pieces, bw: float, spacing: float, offset: int, sampleoffset: int = 0):
    """The PCal extractors' result in FP64 for a sequence of pieces, each
    (samples, new_sampleoffset or None): sample n after an offset o lands in
    bin (o + n) mod nbins (Trivial PCal.cpp:235-253, ImplicitShift :610-628),
    mixed by exp(-2 pi i offset (o + n) / fs) first for Shifting (:421-462,
    every sample counted); then the DFT of the bins divided by nbins and the
    picked bins (:301-315, :477-507, :669-688).  Returns (tones, samplecount),
    tones past the last bin < nbins omitted."""
    kind, nbins, rotlen, ntones, first, step = pcal_config(bw, spacing, offset)
    fs = 2 * bw
    acc = np.zeros(nbins, np.complex128)
    pos = sampleoffset
    count = 0
    for samples, new_off in pieces:
        if new_off is not None:
            pos = new_off
        x = np.asarray(samples, np.float64)
        n = pos + np.arange(x.size, dtype=np.int64)
        if kind == 1:
            r = (int(offset) * (n % int(fs))) % int(fs)
            x = x * np.exp(-2j * np.pi * r / fs)
        np.add.at(acc, n % nbins, x)
        pos += x.size
        count += x.size
    bins = [first + t * step for t in range(ntones) if first + t * step < nbins]
    b = np.arange(nbins)
    tones = np.array([np.sum(acc * np.exp(-2j * np.pi * ((k * b) % nbins) / nbins)) / nbins for k in bins])
    return tones, count
