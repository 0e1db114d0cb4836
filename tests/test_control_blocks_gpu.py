"""The reference's Cell control blocks through the C ABI (cellspe_control_blocks.h).

* cellspe_minicorrelator_run on the six `control_block`s of the reference's
  6-station setup (minicorrelator_ppu.c:131-148): every SPE's autocorrelation
  blocks and its baseline slots (rank, rank + 6, rank + 12 < 15, partners
  rank + 1, 3, 4 mod 6) against the FP64 restatement, at the FP32 path's
  1e-5 relative error; the control blocks handed over in a shuffled order
  (spe_num, not the array index, names the station).
* cellspe_cell_spectrometer_task on a `control_block_t` task sequence
  (TaskCoreCell.cpp:34-116): 8-bit and 2-bit samples, overlap 1, 2 and 4,
  spectra that span two tasks (the SPE keeps its partial spectrum), the
  reported spectra and FFT counts, and terminate_flag releasing the state.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _planar(buf, blocks):
    v = buf.reshape(blocks, 2, 1024)
    return v[:, 0] + 1j * v[:, 1]


@pytest.mark.parametrize("ffts_total,integ", [(64, 16), (96, 32), (4096, 4096)])
def test_minicorrelator_control_blocks(cg, orc, ffts_total, integ):
    rng = np.random.default_rng(ffts_total + integ)
    raws = [rng.integers(0, 256, ffts_total * 256, dtype=np.uint8) for _ in range(6)]
    blocks = ffts_total // integ
    autos = [np.zeros(blocks * 2048, np.float32) for _ in range(6)]
    slots = [np.full(blocks * 2048, np.nan, np.float32) for _ in range(15)]
    order = [3, 0, 5, 1, 4, 2]                      # array position i holds SPE order[i]
    cbs = []
    for rank in order:
        cb = cg.ControlBlock()
        cb.rawdata_src.p = raws[rank].ctypes.data
        cb.autocorrelation_out.p = autos[rank].ctypes.data
        for b in range(15):
            cb.baselines_out[b].p = slots[b].ctypes.data
        cb.spe_num, cb.num_spes = rank, 6
        cb.ffts_total, cb.ffts_to_integrate = ffts_total, integ
        cbs.append(cb)
    cg.minicorrelator_run(cbs)
    ref_auto, ref_slots = orc.minicorrelator_slots_f64(raws, ffts_total, integ)
    for s in range(6):
        got = _planar(autos[s], blocks)
        assert _rel(got, ref_auto[s]) < TOL, s
        assert np.abs(got.imag).max() <= 1e-6 * np.abs(got.real).max()
    assert sorted(ref_slots) == list(range(15))
    for slot, ref in ref_slots.items():
        assert _rel(_planar(slots[slot], blocks), ref) < TOL, slot
    # the reference's slot assignment: slot 9 is (3, 0), the conjugate of slot 6's (0, 3)
    np.testing.assert_allclose(_planar(slots[9], blocks), np.conj(_planar(slots[6], blocks)), rtol=1e-6, atol=1e-3)


def test_minicorrelator_rejects_bad_blocks(cg):
    cbs = [cg.ControlBlock() for _ in range(6)]
    with pytest.raises(cg.CellspeError) as e:
        cg.minicorrelator_run(cbs[:5])
    assert e.value.code == cg.ERR_ARG
    raw = np.zeros(64 * 256, np.uint8)
    out = np.zeros(4 * 2048, np.float32)
    for i, cb in enumerate(cbs):
        cb.rawdata_src.p = raw.ctypes.data
        cb.autocorrelation_out.p = out.ctypes.data
        for b in range(15):
            cb.baselines_out[b].p = out.ctypes.data
        cb.spe_num, cb.num_spes, cb.ffts_total, cb.ffts_to_integrate = i % 5, 6, 64, 16   # rank 0 twice
    with pytest.raises(cg.CellspeError) as e:
        cg.minicorrelator_run(cbs)
    assert "permutation" in str(e.value)
    for i, cb in enumerate(cbs):
        cb.spe_num, cb.ffts_to_integrate = i, 15                                           # odd
    with pytest.raises(cg.CellspeError) as e:
        cg.minicorrelator_run(cbs)
    assert "even" in str(e.value)


def _cell_tasks(cg, buffers, N, K, overlap, spr, levels=None):
    task = cg.CellSpectrometerTask(levels)
    outs, stats = [], []
    try:
        for buf in buffers:
            cap = (len(buf) // max(1, (N // spr) // overlap) // K + 2) * N * 2
            dst = np.full(cap, np.nan, np.float32)
            cb = cg.ControlBlockT()
            cb.fft_points, cb.fft_points_log2 = N, N.bit_length() - 1
            cb.overlap_factor, cb.integrate_ffts, cb.samples_per_rawbyte = overlap, K, spr
            cb.rawif_src.p = buf.ctypes.data
            cb.rawif_bytecount = len(buf)
            cb.spectrum_dst.p = dst.ctypes.data
            st = task.run(cb)
            outs.append(dst[: st[1] * 2 * N].reshape(st[1], N, 2))
            stats.append(st)
    finally:
        task.close()
    assert task.state.value is None
    return outs, stats


@pytest.mark.parametrize("N,K,overlap,spr,sizes", [
    (1024, 5, 2, 1, [40000, 23000, 61000]),          # 8-bit, spectra across task boundaries
    (256, 16, 1, 1, [4096, 4096]),                   # overlap 1: the SPE's loop leaves the last FFT out
    (2048, 3, 4, 4, [30000, 9000]),                  # 2-bit, overlap 4
    (32768, 2, 2, 1, [200000]),                      # largest FFT
])
def test_cell_spectrometer_task_sequence(cg, orc, N, K, overlap, spr, sizes):
    rng = np.random.default_rng(N + K)
    bufs = [rng.integers(0, 256, n, dtype=np.uint8) for n in sizes]
    levels = np.array([1.0, -1.0, 3.3359, -3.3359], np.float32)       # TwoBitUnpacker map_rev
    outs, stats = _cell_tasks(cg, bufs, N, K, overlap, spr)
    ref = orc.cell_spectrometer_f64(bufs, N, K, overlap, spr, levels)
    d = (N // spr) // overlap
    for t, (buf, got, want, st) in enumerate(zip(bufs, outs, ref, stats)):
        B = len(buf)
        nfft = min(B // d - 1 if B >= 2 * d else 0, (B - N // spr) // d + 1 if B >= N // spr else 0)
        assert st[2] == nfft and st[1] == len(want), (t, st)
        assert st[0] > 0
        if want:
            w = np.stack(want)
            assert _rel(got, w) < TOL, t
            assert (got[..., 1] == 0).all()
            np.testing.assert_array_equal(got[:, 1:N // 2, 0], got[:, N - 1:N // 2:-1, 0])   # k and N - k


def test_cell_spectrometer_task_argument_checks(cg):
    task = cg.CellSpectrometerTask()
    cb = cg.ControlBlockT()
    cb.fft_points, cb.integrate_ffts, cb.overlap_factor, cb.samples_per_rawbyte = 1000, 4, 2, 1
    with pytest.raises(cg.CellspeError) as e:
        task.run(cb)
    assert e.value.code == cg.ERR_ARG and "power of two" in str(e.value)
    cb.fft_points, cb.samples_per_rawbyte = 1024, 2
    with pytest.raises(cg.CellspeError) as e:
        task.run(cb)
    assert "samples_per_rawbyte" in str(e.value)
    task.close()
    assert task.state.value is None


def test_cell_spectrometer_task_short_and_empty_buffers(cg, orc):
    """Buffers shorter than two hops give no FFT (the SPE's loop bound), an
    empty buffer none either; the partial spectrum of earlier tasks carries over
    untouched, and the spectrum destination is not written."""
    N, K, overlap = 1024, 3, 2
    rng = np.random.default_rng(21)
    bufs = [rng.integers(0, 256, n, dtype=np.uint8) for n in (5000, 1023, 0, 600, 9000)]
    outs, stats = _cell_tasks(cg, bufs, N, K, overlap, 1)
    ref = orc.cell_spectrometer_f64(bufs, N, K, overlap, 1)
    for t, (got, want, st) in enumerate(zip(outs, ref, stats)):
        assert st[1] == len(want), (t, st)
        if want:
            assert _rel(got, np.stack(want)) < TOL
    assert [s[2] for s in stats] == [8, 0, 0, 0, 16]      # floor(B / 512) - 1, none below two hops
