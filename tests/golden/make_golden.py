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
* minitest-cell.cpp:131-138 -- the MAC validation ramp
  (in1 = 0.5i - 0.5i*j, in2 = 0.15 i^2 - 0.25j, acc = 1 + 1.5j), run through
  genericAddProduct_32fc and genericAddProduct_32fc_conj.

Usage:  python tests/golden/make_golden.py
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


def main():
    oracle.build(with_ref=True)
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
    np.savez_compressed(HERE / "generic_mac.npz", a=a, b=b, acc0=acc0, mac=acc, mac_conj=accc)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
