"""TaskCoreCUDA, the swspectrometer plug-in, driven the way TaskDispatcher drives
its platform cores (cellspe_taskcore_spectrometer), against the oracle's
restatement of TaskCoreIPP::doMaths on the decoded channel.

* one source, 16 channels, mark5access levels (Mk5B), cosine^2 window,
  phase-cal, two cores, several spectra per raw buffer: every spectrum and
  every phase-cal vector as the oracle computes it per raw buffer (the
  reference's FFT count, which picks the phase-cal windows, restarts with
  each doMaths call);
* two sources (TwoBitUnpacker levels, decreasing channel order, Hann window)
  with their cross product;
* one spectrum spanning two raw buffers: each core's sub-spectrum is added
  into the common spectrum on the GPU by combineResults;
* settings the plug-in does not take fail in join(), and the dispatcher
  reports the plug-in's message.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5

TWOBIT = np.array([1.0, -1.0, 3.3359, -3.3359], np.float32)       # TwoBitUnpacker map_rev
MARK5B = np.array([-3.3359, 1.0, -1.0, 3.3359], np.float32)       # mark5access lut


def _decode(raw, nchan, chan, lut, increasing=True):
    """Channel `chan` of interleaved 2-bit data, as TwoBitUnpacker / mark5access read it."""
    step = nchan // 4
    byte = chan // 4 if increasing else step - 1 - chan // 4
    shift = 2 * (chan % 4) if increasing else 6 - 2 * (chan % 4)
    b = raw.reshape(-1, step)[:, byte]
    return lut[(b >> shift) & 3].astype(np.float32)


def _integ(K, N, fs=32e6):
    """FFTIntegrationTimeSec for K FFTs of N points (a tenth of an FFT more, so
    that the FP32 product fs * T / N does not round below K)."""
    return (K + 0.1) * N / fs


def _cfg(cg, **kw):
    c = cg.TaskcoreConfig()
    defaults = dict(num_cores=2, fft_points=4096, integ_seconds=_integ(8, 4096), overlap=2, window=2,
                    source_channels=16, channel1=1, channel2=1, channelorder_increasing=1, sourceformat=7,
                    samplingfreq=32e6, extract_pcal=0, pcal_offset_hz=0.0, pcal_harmonics_hz=1e6, num_sources=1,
                    calc_xpol=0, max_rawbuf_bytes=1 << 20)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(c, k, v)
    return c


def test_taskcore_single_source_pcal_two_cores(cg, orc):
    N, K, nch, ch = 4096, 8, 16, 5
    spec_bytes = K * N * nch // 4                     # 128 KiB per spectrum
    per_buf = (1 << 20) // 2 // spec_bytes            # 4 spectra per raw buffer and core
    nspec = 3 * per_buf
    raw = np.random.default_rng(7).integers(0, 256, nspec * spec_bytes, dtype=np.uint8)
    cfg = _cfg(cg, channel1=ch + 1, extract_pcal=1)
    nb = N // 2 + 1
    sinks, n = cg.taskcore_spectrometer(cfg, raw, sink_bytes=(nspec * nb * 4, 0, 0, nspec * 32 * 8, 0))
    assert n == nspec
    power = sinks[0].view(np.float32).reshape(nspec, nb)
    pcal = sinks[3].view(np.complex64).reshape(nspec, 32)
    x = _decode(raw, nch, ch, MARK5B)
    for b in range(nspec // per_buf):                 # one doMaths call per raw buffer
        seg = x[b * per_buf * K * N:(b + 1) * per_buf * K * N]
        ref_p, ref_c = orc.spectrometer(seg, N, 2, 2, K, 32, 32, 0.0, 32e6)
        got_p, got_c = power[b * per_buf:(b + 1) * per_buf], pcal[b * per_buf:(b + 1) * per_buf]
        assert np.linalg.norm(got_p - ref_p) / np.linalg.norm(ref_p) < TOL
        assert np.linalg.norm(got_c - ref_c) / np.linalg.norm(ref_c) < TOL


def test_taskcore_two_sources_cross_product(cg, orc):
    N, K, nch = 2048, 4, 4
    cfg = _cfg(cg, num_cores=1, fft_points=N, integ_seconds=_integ(K, N), window=4, source_channels=nch,
               channel1=2, channel2=4, channelorder_increasing=0, sourceformat=0, num_sources=2, calc_xpol=1,
               max_rawbuf_bytes=K * N * 2)              # two spectra per raw buffer (one in the last)
    nspec = 5
    rng = np.random.default_rng(8)
    s0 = rng.integers(0, 256, nspec * K * N * nch // 4, dtype=np.uint8)
    s1 = rng.integers(0, 256, s0.size, dtype=np.uint8)
    nb = N // 2 + 1
    sinks, n = cg.taskcore_spectrometer(cfg, s0, s1, sink_bytes=(nspec * nb * 4, nspec * nb * 4, nspec * nb * 8, 0, 0))
    assert n == nspec
    got0 = sinks[0].view(np.float32).reshape(nspec, nb)
    got1 = sinks[1].view(np.float32).reshape(nspec, nb)
    gotx = sinks[2].view(np.complex64).reshape(nspec, nb)
    x0 = _decode(s0, nch, 1, TWOBIT, increasing=False)
    x1 = _decode(s1, nch, 3, TWOBIT, increasing=False)
    for sp in range(nspec):
        sl = slice(sp * K * N, (sp + 1) * K * N)
        power, xpol, _ = orc.spectrometer_xpol(x0[sl], x1[sl], N, 2, 4, K)
        assert np.linalg.norm(got0[sp] - power[0, 0]) / np.linalg.norm(power[0, 0]) < TOL
        assert np.linalg.norm(got1[sp] - power[1, 0]) / np.linalg.norm(power[1, 0]) < TOL
        assert np.linalg.norm(gotx[sp] - xpol[0]) / np.linalg.norm(xpol[0]) < TOL


def test_taskcore_spectrum_over_two_buffers_combined_on_gpu(cg, orc):
    """averaged_ffts = 16 with 8 KiB of raw buffer per core: the reference's
    sizing gives 2 raw buffers per spectrum of 8 FFTs each (core_overlapped_ffts
    15); the written spectrum is the sum of the two cores' sub-spectra, each
    scaled by 1/15, and so are the phase-cal bins."""
    N, nch = 2048, 4
    cfg = _cfg(cg, fft_points=N, integ_seconds=_integ(16, N), source_channels=nch, channel1=3, sourceformat=2,
               extract_pcal=1, max_rawbuf_bytes=16 << 10)
    Kc = 8
    nspec = 3
    raw = np.random.default_rng(9).integers(0, 256, nspec * 2 * Kc * N * nch // 4, dtype=np.uint8)
    nb = N // 2 + 1
    sinks, n = cg.taskcore_spectrometer(cfg, raw, sink_bytes=(nspec * nb * 4, 0, 0, nspec * 32 * 8, 0))
    assert n == nspec
    power = sinks[0].view(np.float32).reshape(nspec, nb)
    pcal = sinks[3].view(np.complex64).reshape(nspec, 32)
    x = _decode(raw, nch, 2, TWOBIT)
    for sp in range(nspec):
        parts = [orc.spectrometer(x[(2 * sp + h) * Kc * N:(2 * sp + h + 1) * Kc * N], N, 2, 2, Kc, 32, 32, 0.0, 32e6)
                 for h in range(2)]
        ref_p = parts[0][0][0] + parts[1][0][0]
        ref_c = parts[0][1][0] + parts[1][1][0]
        assert np.linalg.norm(power[sp] - ref_p) / np.linalg.norm(ref_p) < TOL
        assert np.linalg.norm(pcal[sp] - ref_c) / np.linalg.norm(ref_c) < TOL


def test_taskcore_rejects_unsupported_settings(cg):
    cfg = _cfg(cg, source_channels=2, num_cores=1)
    raw = np.zeros(8 * 4096 * 2 // 4 * 2, np.uint8)
    with pytest.raises(cg.CellspeError) as e:
        cg.taskcore_spectrometer(cfg, raw, sink_bytes=(1 << 20, 0, 0, 0, 0))
    assert "source_channels" in str(e.value)
