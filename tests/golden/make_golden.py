"""Generate the golden vectors in this folder from the reference itself.

Runs in the build container only (it needs the reference tree): the
reference's mark5access 1.4.3 and its architecture.h GENERIC kernels are
compiled from the reference sources by ``make -C oracle ref`` into
oracle/_ref/, and this script calls them on the reference's own test inputs:

* mark5access examples/test_unpacker.c:121 -- byte buffer (i % 11) + 2*(i % 121),
  decoded with mark5_unpack() for three Mark5B 2-bit formats.
* the same test_unpacker byte pattern as payload of a framed Mark5B stream
  (16-byte headers, 10000-byte payloads, fill-pattern zones at frame starts,
  ends, a whole frame, 4-byte stragglers), decoded through the library's
  memory stream and mark5_stream_decode() -- header strip plus blanking.
  Stored as level indices (0..3 = lut2bit entry, 4 = blanked 0.0).
* framed VDIF streams (mark5access format_vdif.c) with the same byte pattern
  as payload: 32-byte and legacy 16-byte headers, 1 to 16 channels, frames
  marked invalid, a frame whose header time breaks the sequence, fill words
  at payload starts and ends, a day boundary, and a bit rate whose frame time
  is not a whole number of ns; decoded through the library's memory stream
  with the format "VDIF_<payload>-<Mbps>-<nchan>-2".  Stored as level
  indices (0..3 = VDIF lut entry, 4 = blanked 0.0).
* minitest-cell.cpp:131-138 -- the MAC validation ramp
  (in1 = 0.5i - 0.5i*j, in2 = 0.15 i^2 - 0.25j, acc = 1 + 1.5j), run through
  genericAddProduct_32fc, genericAddProduct_32fc_conj and genericMul_32fc.

Usage:  python tests/golden/make_golden.py <reference tree>
"""
import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
import oracle  # noqa: E402


FRAMED_FILL = [(1, 0, 2000), (2, 7000, 10000), (3, 0, 10000), (4, 0, 1004), (5, 5004, 10000), (6, 4, 400)]
FRAMED_PREFIX, FRAMED_FRAMES = 137, 8
LEVELS = np.array([-3.3359, 1.0, -1.0, 3.3359, 0.0], np.float32)


def framed_input():
    """Framed Mark5B bytes with fill zones; payload = test_unpacker.c:121 pattern."""
    sys.path.insert(0, str(HERE.parent.parent / "cellspe-tasklib_gb300"))
    import synth

    n = FRAMED_FRAMES * 10000
    pay = np.array([(i % 11) + 2 * (i % 121) for i in range(n)], dtype=np.uint8)
    fr = synth.mark5b_frames(pay, prefix=FRAMED_PREFIX)
    for f, a, b in FRAMED_FILL:
        synth.mark5b_fill(fr, f, a, b, FRAMED_PREFIX)
    return fr


def framed_cases():
    fr = framed_input()
    out = {"framed": fr}
    for fmt, nch in [("Mark5B-512-16-2", 16), ("Mark5B-256-8-2", 8), ("Mark5B-128-4-2", 4)]:
        spf = 10000 // (nch // 4)
        nsamps = np.array([3 * spf + 17, (FRAMED_FRAMES - 1) * spf, FRAMED_FRAMES * spf])
        key = fmt.replace("-", "_")
        out[f"{key}_nsamp"] = nsamps
        for k, ns in enumerate(nsamps):
            rc, dec, off = oracle.ref_mark5_decode_memory(fmt.encode(), fr, int(ns))
            assert off == FRAMED_PREFIX, off
            idx = np.searchsorted(np.sort(LEVELS), dec)
            codes = np.argsort(LEVELS)[idx].astype(np.uint8)
            assert np.array_equal(LEVELS[codes], dec)
            out[f"{key}_rc{k}"] = np.array(rc)
            out[f"{key}_codes{k}"] = codes
    return out


VDIF_LEVELS = np.array([-3.3359, -1.0, 1.0, 3.3359, 0.0], np.float32)
# name: (payload bytes, Mbps, nchan, legacy, ref epoch, seconds, first frame, frames, edits)
# edits: ("invalid", f) | ("time", f) (frame number + 1) | ("fill0", f) | ("fill1", f)
VDIF_CASES = {
    "v4ch": (2000, 128, 4, False, 40, 7654321, 0, 8,
             [("invalid", 0), ("invalid", 3), ("time", 5), ("fill0", 2), ("fill1", 6)]),
    "v8ch_legacy": (2000, 256, 8, True, 21, 123456, 17, 8, [("invalid", 2), ("fill0", 4)]),
    "v16ch_granularity": (2000, 8192, 16, False, 5, 99999, 0, 10, [("fill1", 3)]),
    "v1ch_day": (1024, 128, 1, False, 63, 2 * 86400 - 1, 15622, 6, [("invalid", 4)]),
    "v2ch_legacy": (1000, 64, 2, True, 0, 500, 7990, 6, [("fill1", 1)]),
}


def vdif_input(name):
    sys.path.insert(0, str(HERE.parent.parent / "cellspe-tasklib_gb300"))
    import synth

    db, mbps, nch, legacy, ep, sec, f0, nf, edits = VDIF_CASES[name]
    pay = np.array([(i % 11) + 2 * (i % 121) for i in range(nf * db)], dtype=np.uint8)
    fr = synth.vdif_frames(pay, db, nch, mbps, legacy=legacy, seconds=sec, ref_epoch=ep, first_frame=f0)
    hs = 16 if legacy else 32
    fb = db + hs
    for kind, f in edits:
        if kind == "invalid":
            synth.vdif_set_invalid(fr, f, fb)
        elif kind == "time":
            fr[f * fb + 4] = (int(fr[f * fb + 4]) + 1) & 0xFF
        elif kind == "fill0":
            synth.vdif_fill(fr, f, fb, hs, 0, 8)
        elif kind == "fill1":
            synth.vdif_fill(fr, f, fb, hs, db - 8, db)
    return fr


def vdif_epochs():
    """Library-read first-frame time of 2-frame streams at each of the 64 reference epochs."""
    sys.path.insert(0, str(HERE.parent.parent / "cellspe-tasklib_gb300"))
    import synth

    times = []
    for e in range(64):
        fr = synth.vdif_frames(np.zeros(2 * 1024, np.uint8), 1024, 4, 128, ref_epoch=e, seconds=5 * 86400 + 7,
                               first_frame=3)
        times.append(oracle.ref_mark5_stream_time(b"VDIF_1024-128-4-2", fr))
    return np.array(times, np.int64)


def vdif_cases():
    out = {"epoch_times": vdif_epochs()}
    for name, (db, mbps, nch, legacy, ep, sec, f0, nf, edits) in VDIF_CASES.items():
        fr = vdif_input(name)
        out[f"{name}_framed"] = fr
        spf = db * 4 // nch
        nsamps = np.array([3 * spf + 16, (nf - 1) * spf, nf * spf])
        out[f"{name}_nsamp"] = nsamps
        fmt = f"VDIF_{db}-{mbps}-{nch}-2".encode()
        for k, ns in enumerate(nsamps):
            rc, dec, off = oracle.ref_mark5_decode_memory(fmt, fr, int(ns))
            assert off == 0, off
            idx = np.searchsorted(np.sort(VDIF_LEVELS), dec)
            codes = np.argsort(VDIF_LEVELS)[idx].astype(np.uint8)
            assert np.array_equal(VDIF_LEVELS[codes], dec)
            out[f"{name}_rc{k}"] = np.array(rc)
            out[f"{name}_codes{k}"] = codes
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference tree>")
    oracle.build(sys.argv[1])
    assert oracle.have_ref(), "oracle/_ref was not built"
    m5 = oracle.ref_mark5()
    out = {}
    for fmt, nch in [("Mark5B-512-16-2", 16), ("Mark5B-256-8-2", 8), ("Mark5B-128-4-2", 4)]:
        n = 1000
        raw = np.array([(i % 11) + 2 * (i % 121) for i in range(n * nch // 4)], dtype=np.uint8)
        dec = np.zeros(nch * n, np.float32)
        c = ctypes.c_int()
        rc = m5.ref_mark5_unpack(fmt.encode(), raw.ctypes.data, n, dec.ctypes.data, ctypes.byref(c))
        assert rc == n and c.value == nch, (fmt, rc, c.value)
        key = fmt.replace("-", "_")
        out[f"{key}_raw"] = raw
        out[f"{key}_out"] = dec.reshape(nch, n)
    np.savez_compressed(HERE / "mark5b_unpack.npz", **out)

    np.savez_compressed(HERE / "mark5b_framed.npz", **framed_cases())
    np.savez_compressed(HERE / "vdif_framed.npz", **vdif_cases())

    gen = oracle.ref_generic()
    n = 1024   # twicenumchannels in minitest-cell.cpp
    i = np.arange(n, dtype=np.float64)
    a = (0.5 * i - 0.5j * i).astype(np.complex64)
    b = (0.15 * i * i - 0.25j).astype(np.complex64)
    acc0 = np.full(n, 1.0 + 1.5j, np.complex64)
    acc = acc0.copy()
    gen.ref_addproduct_32fc(a.ctypes.data, b.ctypes.data, acc.ctypes.data, n)
    accc = acc0.copy()
    gen.ref_addproduct_32fc_conj(a.ctypes.data, b.ctypes.data, accc.ctypes.data, n)
    mul = np.zeros(n, np.complex64)
    gen.ref_mul_32fc(a.ctypes.data, b.ctypes.data, mul.ctypes.data, n)
    np.savez_compressed(HERE / "generic_mac.npz", a=a, b=b, acc0=acc0, mac=acc, mac_conj=accc, mul=mul)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
