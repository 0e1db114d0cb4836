"""K-a: GPU 2-bit unpack is bit-exact with the oracle (itself pinned to mark5access)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("fmt,nch", [("Mark5B_512_16_2", 16), ("Mark5B_256_8_2", 8), ("Mark5B_128_4_2", 4)])
def test_unpack_golden_mark5b(cg, fmt, nch):
    g = np.load(GOLD / "mark5b_unpack.npz")
    raw, ref = g[f"{fmt}_raw"], g[f"{fmt}_out"]
    out = np.zeros_like(ref)
    cg.unpack2bit(raw, ref.shape[1], nch, out, levels=cg.LEVELS_MARK5B)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("nch", [1, 2, 4, 8, 16])
@pytest.mark.parametrize("nsamp", [0, 1, 7, 64, 1000, 65536 + 12])
@pytest.mark.parametrize("levels", ["MARK5B", "TWOBIT", "OFFSET_BINARY"])
def test_unpack_random_vs_oracle(cg, orc, nch, nsamp, levels):
    rng = np.random.default_rng(nch * 1000 + nsamp)
    nbytes = max(16, (nsamp * nch * 2 + 7) // 8)
    raw = rng.integers(0, 256, nbytes, dtype=np.uint8)
    lut = {"MARK5B": orc.MARK5B_LUT, "TWOBIT": orc.TWOBIT_LUT, "OFFSET_BINARY": orc.OFFSET_BINARY_LUT}[levels]
    out = np.full((nch, max(nsamp, 1)), np.nan, np.float32)[:, :nsamp].copy()
    cg.unpack2bit(raw, nsamp, nch, out, levels=getattr(cg, "LEVELS_" + levels))
    ref = orc.unpack2bit(raw, nsamp, nch, lut)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_unpack_msb_first_and_device_memory(cg, orc):
    import torch

    rng = np.random.default_rng(1)
    raw = rng.integers(0, 256, 4096, dtype=np.uint8)
    ref = orc.unpack2bit(raw, 16384, 1, orc.TWOBIT_LUT, msb_first=True)
    d_raw = torch.from_numpy(raw).cuda()
    d_out = torch.zeros((1, 16384), dtype=torch.float32, device="cuda")
    cg.unpack2bit(d_raw, 16384, 1, d_out, levels=cg.LEVELS_TWOBIT, msb_first=True)
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_unpack_custom_levels(cg, orc):
    raw = np.arange(256, dtype=np.uint8).repeat(4)
    lut = np.array([0.5, -7.0, 2.25, 1e-3], np.float32)
    out = np.zeros((4, 1024), np.float32)
    cg.unpack2bit(raw, 1024, 4, out, custom_levels=lut)
    assert np.array_equal(out, orc.unpack2bit(raw, 1024, 4, lut))


def test_unpack_rejects_bad_arguments(cg):
    raw = np.zeros(64, np.uint8)
    out = np.zeros((3, 16), np.float32)
    with pytest.raises(cg.CellspeError) as e:
        cg.unpack2bit(raw, 16, 3, out)
    assert e.value.code == cg.ERR_ARG
