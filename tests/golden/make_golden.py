"""Generate the golden vectors in this folder from the reference itself.

Runs in the build container only (it needs the reference tree): the
reference's mark5access 1.4.3 and its architecture.h GENERIC kernels are
compiled from the reference sources by ``make -C oracle ref`` into
oracle/_ref/, and this script calls them on the reference's own test inputs:

* mark5access examples/test_unpacker.c:121 -- byte buffer (i % 11) + 2*(i % 121),
  decoded with mark5_unpack() for three Mark5B 2-bit formats.
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
