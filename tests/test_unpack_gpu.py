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


def _code_counts(raw: np.ndarray, nch: int) -> np.ndarray:
    """Per-channel histogram of the 2-bit codes in an LSB-first stream, from byte histograms.

    Field p (0..3) of byte b holds code (b >> 2p) & 3; with nch >= 4 channels a sample time
    spans nch/4 bytes and byte phase ph carries channels 4ph .. 4ph+3, with fewer channels
    field p belongs to channel p mod nch."""
    codes = (np.arange(256)[:, None] >> (2 * np.arange(4))[None, :]) & 3
    bpt = max(nch // 4, 1)
    cnt = np.zeros((nch, 4), np.int64)
    for ph in range(bpt):
        h = np.bincount(raw[ph::bpt], minlength=256)
        for p in range(4):
            c = 4 * ph + p if nch >= 4 else p % nch
            cnt[c] += np.bincount(codes[:, p], weights=h, minlength=4).astype(np.int64)
    return cnt


@pytest.mark.parametrize("nch,nsamp", [
    pytest.param(16, 1 << 25, id="m5b16_full"),     # Mark5B spectrometer input: 16 subbands x 2^25 samples
    pytest.param(1, 1 << 29, id="single_full"),     # one channel, the same 128 MiB of raw bytes
    pytest.param(16, 1 << 23, id="m5b16_small"),    # profiling-sized cases (512 MiB out, above L2)
    pytest.param(1, 1 << 27, id="single_small"),
])
def test_unpack_large_exact_and_rate(cg, orc, nch, nsamp):
    """Full-size unpack from device memory: every level count per channel equals the code
    histogram of the raw bytes, sampled 64 KiB blocks equal the oracle bit for bit, each call
    is one vector-kernel launch; prints the rate of the blocking call (algorithmic bytes
    0.25 B in + 4 B out per field)."""
    import time

    import torch

    nbytes = nsamp * nch // 4
    g = torch.Generator(device="cuda").manual_seed(nch * 7919 + nsamp.bit_length())
    d_raw = torch.randint(0, 256, (nbytes,), dtype=torch.uint8, device="cuda", generator=g)
    d_out = torch.full((nch, nsamp), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    times = []
    for it in range(7):
        n0 = cg.kernel_launches()
        t0 = time.perf_counter()
        cg.unpack2bit(d_raw, nsamp, nch, d_out, levels=cg.LEVELS_MARK5B)
        times.append(time.perf_counter() - t0)
        assert cg.kernel_launches() - n0 == 1
    raw = d_raw.cpu().numpy()
    lut = torch.tensor(orc.MARK5B_LUT, dtype=torch.float32, device="cuda")
    got = torch.stack([(d_out == lut[k]).sum(dim=1) for k in range(4)], dim=1).cpu().numpy()
    assert np.array_equal(got, _code_counts(raw, nch))
    blk = 1 << 16
    tpb = blk * 4 // nch
    for b in (0, (nbytes // 2) // blk * blk, nbytes - blk):
        t = b * 4 // nch
        ref = orc.unpack2bit(raw[b:b + blk], tpb, nch, orc.MARK5B_LUT)
        assert np.array_equal(d_out[:, t:t + tpb].cpu().numpy().view(np.uint32), ref.view(np.uint32))
    best = min(times[2:])
    gbs = nsamp * nch * 4.25 / best / 1e9
    print(f"\nunpack2bit nch={nch} nsamp={nsamp}: best blocking call {best * 1e3:.3f} ms, "
          f"median {sorted(times[2:])[2] * 1e3:.3f} ms, {gbs:.0f} GB/s algorithmic")
