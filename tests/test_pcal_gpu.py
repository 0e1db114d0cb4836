"""The PCal library on the GPU (cellspe_pcal.h) against the reference's own
known answer and the FP64 restatement.

* The reference's PCal unit test (PCal.cpp:879-951: `test 32000 16e6 1e6
  510e3 0`): 16 tones with phases -90 + 5 x tone degrees, extracted from the
  32000 samples, then the same data from sample 3 on after
  adjustSampleOffset(sampleoffset + 32000 + 3); every tone within 0.1 degree.
  Run for the method getNew picks there (ImplicitShift), for a Shifting case
  (offset 128 Hz, 10^6 samples: whole cycles of the mixed-down image) and
  with a non-zero sample offset.
* Each method against pcal_extract_f64 on noise cut into pieces of random
  length, with a gap announced by adjust_sample_offset, from host and from
  device memory: FP32 accumulation within 2e-5 relative of FP64; the piece
  boundaries do not change the result beyond that.
* getNew's choice and sizes, clear/finalise semantics, argument errors.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tones_signal(bw, sp, off, nt, so, N):
    n = np.arange(N, dtype=np.float64) + so
    x = np.zeros(N)
    for t in range(nt):
        x += np.sin(np.pi * n * (off + t * sp) / bw + t * np.pi * 5 / 180)
    return x.astype(np.float32)


def _phase_err(tones):
    ph = np.degrees(np.angle(tones))
    want = -90.0 + 5.0 * np.arange(len(tones))
    return float(np.abs((ph - want + 180.0) % 360.0 - 180.0).max())


@pytest.mark.parametrize("bw,sp,off,so,N,kind", [
    (16e6, 1e6, 510000, 0, 32000, 2),       # the reference's example command line
    (16e6, 1e6, 510000, 7, 32000, 2),       # non-zero sample offset
    (16e6, 1e6, 128, 0, 1000000, 1),        # getNew picks Shifting
])
def test_pcal_reference_unit_test_recipe(cg, bw, sp, off, so, N, kind):
    pc = cg.Pcal(bw, sp, off, so)
    assert pc.kind == kind
    nt = pc.length
    data = _tones_signal(bw, sp, off, nt, so, N)
    pc.extract(data)
    pc.adjust_sample_offset(so + N + 3)       # skip_some_data (PCal.cpp:916-920)
    pc.extract(data[3:])
    tones, count = pc.final()
    assert count == 2 * N - 3
    assert _phase_err(tones) < 0.1
    assert pc.seconds == pytest.approx(count / (2 * bw))
    pc.close()


@pytest.mark.parametrize("bw,sp,off", [(16e6, 1e6, 0), (16e6, 1e6, 510000), (16e6, 1e6, 128), (8e6, 5e5, 10000)])
@pytest.mark.parametrize("device", [False, True])
def test_pcal_pieces_vs_fp64(cg, orc, bw, sp, off, device):
    import torch

    rng = np.random.default_rng(int(off) + 17)
    cuts = np.sort(rng.choice(np.arange(1, 300000), size=6, replace=False))
    x = rng.standard_normal(300000).astype(np.float32)
    pieces = [(p, None) for p in np.split(x, cuts)]
    pieces[3] = (pieces[3][0], 123457)        # a gap: sample offset moved before piece 3
    pc = cg.Pcal(bw, sp, off, 11)
    kind, nbins, _, ntones, _, _ = orc.pcal_config(bw, sp, off)
    assert (pc.kind, pc.nbins, pc.length) == (kind, nbins, ntones)
    for p, new_off in pieces:
        if new_off is not None:
            pc.adjust_sample_offset(new_off)
        pc.extract(torch.from_numpy(p).cuda() if device else p)
    got, count = pc.final()
    want, wcount = orc.pcal_extract_f64(pieces, bw, sp, off, 11)
    assert count == wcount == x.size
    got = got[: len(want)]
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 2e-5
    # the same stream in one piece per offset run gives the same tones
    pc2 = cg.Pcal(bw, sp, off, 11)
    pc2.extract(np.concatenate([p for p, _ in pieces[:3]]))
    pc2.adjust_sample_offset(123457)
    pc2.extract(np.concatenate([p for p, _ in pieces[3:]]))
    got2, _ = pc2.final()
    assert np.linalg.norm(got2[: len(want)] - got) / np.linalg.norm(want) < 2e-5


def test_pcal_finalise_clear_and_errors(cg):
    pc = cg.Pcal(16e6, 1e6, 510000)
    x = _tones_signal(16e6, 1e6, 510000, pc.length, 0, 32000)
    pc.extract(x)
    a, n = pc.final()
    b, m = pc.final()                         # cached: same tones, same count
    assert n == m == 32000 and np.array_equal(a, b)
    with pytest.raises(cg.CellspeError) as e:
        pc.extract(x)                         # the reference returns false once finalised
    assert e.value.code == cg.ERR_ARG
    pc.clear()
    pc.adjust_sample_offset(0)
    pc.extract(x)
    c, k = pc.final()
    assert k == 32000 and np.allclose(c, a, rtol=1e-6, atol=1e-7)
    with pytest.raises(cg.CellspeError):
        cg.Pcal(16.25, 1e6, 0)                # 2 x bandwidth not a whole number of Hz
    with pytest.raises(cg.CellspeError):
        cg.Pcal(16e6, 0.0, 0)


def test_pcal_empty_pieces_and_single_samples(cg, orc):
    """Pieces of length 0 change nothing; a stream fed one sample at a time
    equals the same stream in one piece (the bin and rotator indices advance
    per sample), for every method."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal(700).astype(np.float32)
    for off in (0, 510000, 128):
        one = cg.Pcal(16e6, 1e6, off, 5)
        one.extract(x)
        a, n = one.final()
        many = cg.Pcal(16e6, 1e6, off, 5)
        many.extract(np.zeros(0, np.float32))
        for v in x[:40]:
            many.extract(np.array([v], np.float32))
        many.extract(np.zeros(0, np.float32))
        many.extract(x[40:])
        b, m = many.final()
        assert n == m == x.size
        want, _ = orc.pcal_extract_f64([(x, None)], 16e6, 1e6, off, 5)
        assert np.linalg.norm(a[: len(want)] - want) / np.linalg.norm(want) < 2e-5
        assert np.linalg.norm(b[: len(want)] - want) / np.linalg.norm(want) < 2e-5
