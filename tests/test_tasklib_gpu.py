"""The celldsp_* task runtime and spe* wrappers on the GPU (minitest-cell.cpp cases)."""
import ctypes
import struct
import threading
import time
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture()
def rt(cg):
    L = cg.lib()
    assert L.celldsp_start() == 0
    yield L
    L.celldsp_setBehaviour(cg.BEHAV_DEFAULT)
    assert L.celldsp_stop() == 0


def test_start_stop_refcount(cg, rt):
    assert rt.celldsp_start() == 0      # second client
    assert rt.celldsp_stop() == 0       # still running for the first
    assert rt.speNOP() == 0


def test_mac_matches_reference_golden(cg, rt):
    """minitest-cell.cpp:131-161: speAddProduct_32fc == genericAddProduct_32fc, bit for bit."""
    g = np.load(GOLD / "generic_mac.npz")
    a, b, acc = g["a"].copy(), g["b"].copy(), g["acc0"].copy()
    assert rt.speAddProduct_32fc(a.ctypes.data, b.ctypes.data, acc.ctypes.data, a.size) == 0
    assert np.array_equal(acc.view(np.uint32), g["mac"].view(np.uint32))
    t = cg.new_task(cg.TASK_MAC_CONJ)
    acc = g["acc0"].copy()
    cg.add_in(t, a); cg.add_in(t, b); cg.add_out(t, acc)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0 and t.completed_flag == cg.TASK_OK
    assert np.array_equal(acc.view(np.uint32), g["mac_conj"].view(np.uint32))


def test_iocheck_values(cg, rt):
    out = np.zeros(8, np.float32)
    t = cg.new_task(cg.TASK_IOTEST)
    cg.add_out(t, out)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0
    assert np.allclose(out[:4], [0.1, 2.3, 4.5, 6.7])


def test_fft_continuable_and_single(cg, rt):
    rng = np.random.default_rng(0)
    for n in (32, 1024):
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
        out = np.zeros_like(x)
        spe = ctypes.c_int(-1)
        assert rt.speFFT_init(n, ctypes.byref(spe)) == 0 and spe.value >= 0
        assert rt.speFFT_exec(x.ctypes.data, out.ctypes.data, n, ctypes.byref(spe)) == 0
        assert rt.speFFT_destroy(ctypes.byref(spe)) == 0 and spe.value == -1
        ref = np.fft.fft(x.astype(np.complex128))
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-5
        out2 = np.zeros_like(x)
        assert rt.speFFT_singleexec(x.ctypes.data, out2.ctypes.data, n) == 0
        assert np.array_equal(out, out2)


def test_sincos_family(cg, rt):
    arg = np.linspace(-10, 10, 1000).astype(np.float32)
    out = np.zeros(1000, np.complex64)
    assert rt.speSinCosAccurate(arg.ctypes.data, out.ctypes.data, 1000) == 0
    assert np.abs(out - np.exp(1j * arg.astype(np.float64))).max() < 2e-6
    nrm = np.linspace(-1, 1, 1000).astype(np.float32)
    assert rt.speSinCosAccurateNorm(nrm.ctypes.data, out.ctypes.data, 1000) == 0
    assert np.abs(out - np.exp(2j * np.pi * nrm.astype(np.float64))).max() < 2e-6
    gen = np.zeros(4096, np.complex64)
    assert rt.speSinCosGenerator(ctypes.c_float(0.1), ctypes.c_float(0.23), gen.ctypes.data, 4096) == 0
    ph = np.float64(np.float32(0.1)) + np.arange(4096) * np.float64(np.float32(0.23))
    assert np.abs(gen - np.exp(1j * ph)).max() < 1e-6


def test_unknown_command_and_injected_failure(cg, rt):
    t = cg.new_task(999)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 1
    assert t.completed_flag == cg.TASK_UNKOWNCOMMAND
    slot = rt.celldsp_getFreeSPE()
    assert slot >= 0
    assert rt.cellspe_debug_inject_failure(slot, 1) == 0
    t = cg.new_task(cg.TASK_NOP)
    assert rt.celldsp_startTask(slot, ctypes.byref(t)) == 0
    assert rt.celldsp_waitTask(slot) == cg.TASK_GENERICERROR
    assert t.completed_flag == cg.TASK_GENERICERROR
    assert rt.celldsp_startTask(slot, ctypes.byref(t)) == 0     # next one runs normally
    assert rt.celldsp_waitTask(slot) == cg.TASK_OK
    rt.celldsp_setFreeSPE(slot)
    assert rt.celldsp_startTask(slot, ctypes.byref(t)) == -1    # not reserved
    assert rt.celldsp_waitTask(slot) == -1                      # nothing started: no hang


def test_task_chain_and_tick_count(cg, rt):
    a = np.ones(1 << 16, np.complex64)
    acc1 = np.zeros_like(a)
    acc2 = np.zeros_like(a)
    t1, t2 = cg.new_task(cg.TASK_MAC), cg.new_task(cg.TASK_MAC)
    cg.add_in(t1, a); cg.add_in(t1, a); cg.add_out(t1, acc1)
    cg.add_in(t2, a); cg.add_in(t2, a); cg.add_out(t2, acc2)
    t1.next_task = ctypes.addressof(t2)
    assert rt.celldsp_executeTask(ctypes.byref(t1)) == 0
    assert t1.completed_flag == 0 and t2.completed_flag == 0
    assert np.all(acc1 == 1) and np.all(acc2 == 1)
    assert t1.tick_count > 0


def test_blocking_behaviour(cg, rt):
    slots = [rt.celldsp_getFreeSPE() for _ in range(cg.MAX_SLOTS)]
    assert sorted(slots) == list(range(cg.MAX_SLOTS))
    assert rt.celldsp_getFreeSPE() == -1                        # non-blocking: none left
    rt.celldsp_setBehaviour(cg.BEHAV_BLOCKING)
    got = []
    th = threading.Thread(target=lambda: got.append(rt.celldsp_getFreeSPE()))
    th.start()
    time.sleep(0.2)
    assert not got                                               # waiting
    rt.celldsp_setFreeSPE(slots[2])
    th.join(timeout=5)
    assert got == [slots[2]]
    for s in slots:
        rt.celldsp_setFreeSPE(s)


def test_difx_process(cg, rt):
    """exec_difxprocess semantics (cellspe-tasklib-dsp.cpp:609-698), lower sideband."""
    rng = np.random.default_rng(2)
    nch = 64
    nfft = 2 * nch
    x = (rng.standard_normal(nfft) + 1j * rng.standard_normal(nfft)).astype(np.complex64)
    mult = np.exp(1j * rng.uniform(0, 6.28, nch + 4)).astype(np.complex64)
    fftout = np.zeros(nch + 4, np.complex64)
    conj = np.zeros(nch + 4, np.complex64)
    auto = np.full(nch + 4, 0.5, np.complex64)
    assert rt.speDIFX_process(x.ctypes.data, mult.ctypes.data, fftout.ctypes.data, conj.ctypes.data,
                              auto.ctypes.data, nfft, nfft, 0) == 0
    X = np.fft.fft(x.astype(np.complex128))
    band = X[:nch] * mult[:nch]
    assert np.linalg.norm(fftout[:nch] - band) / np.linalg.norm(band) < 1e-5
    assert np.allclose(auto[:nch].real, 0.5 + np.abs(band) ** 2, rtol=1e-5)


def test_fx_and_spectrometer_through_tasks(cg, orc, rt):
    import synth

    S, N, K = 3, 1024, 8
    raw = synth.stations_offset_binary(S, N * K, rho=0.2, seed=12)
    p = cg.fx_params(S, N, K, raw.shape[1], vis_order=cg.VIS_BASELINE_MAJOR)
    vis = np.zeros((6, N // 2), np.complex64)
    t = cg.new_task(cg.TASK_FX_CORRELATE)
    cg.add_in_struct(t, p); cg.add_in(t, raw); cg.add_out(t, vis)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0
    ref = orc.fx_fp32(raw, S, N, K)
    assert np.linalg.norm(vis - ref) / np.linalg.norm(ref) < 1e-5

    words, _ = synth.mark5b_subbands(16, 1024 * 4, fs_hz=32e6, seed=3, n_channels=512)
    rawm = words.view(np.uint8)
    sp = cg.spec_params(1024, 2, 2, 4, 1, 16, rawm.size)
    power = np.zeros((16, 1, 513), np.float32)
    t = cg.new_task(cg.TASK_SPECTROMETER)
    cg.add_in_struct(t, sp); cg.add_in(t, rawm); cg.add_out(t, power)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0
    direct = np.zeros_like(power)
    cg.spectrometer(cg.spec_params(1024, 2, 2, 4, 1, 16, rawm.size), rawm, direct)
    assert np.array_equal(power, direct)


def test_unpack_task_per_channel_outputs(cg, orc, rt):
    raw = np.random.default_rng(1).integers(0, 256, 2 * 256, dtype=np.uint8)
    outs = [np.zeros(256, np.float32) for _ in range(8)]      # at most 8 vectors per task
    t = cg.new_task(cg.TASK_UNPACK)
    cg.add_in(t, raw)
    for o in outs:
        cg.add_out(t, o)
    t.subcontext[0] = 256          # nsamp_lo
    t.subcontext[1] = 0
    t.subcontext[2] = 8            # nchan
    t.subcontext[3] = cg.LEVELS_MARK5B
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0
    ref = orc.unpack2bit(raw, 256, 8, orc.MARK5B_LUT)
    assert all(np.array_equal(outs[c], ref[c]) for c in range(8))


def test_mulc_addc_tasks(cg, rt):
    """CELLDSP_TASK_MULC / ADDC (cellspe-tasklib-dsp.h:30-31: out = in1 * in2,
    out = in1 + in2).  The reference's SPU loop accepts both without computing
    (cellspe-tasklib.cpp:502-505); the product is the generic genericMul_32fc
    (architecture.h:270-278), compiled from the reference for the golden
    vector, and matches it bit for bit; the sum is one correctly rounded FP32
    add per component."""
    g = np.load(GOLD / "generic_mac.npz")
    a, b = g["a"].copy(), g["b"].copy()
    out = np.full_like(a, np.nan)
    t = cg.new_task(cg.TASK_MULC)
    cg.add_in(t, a); cg.add_in(t, b); cg.add_out(t, out)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0 and t.completed_flag == cg.TASK_OK
    assert np.array_equal(out.view(np.uint32), g["mul"].view(np.uint32))
    out = np.full_like(a, np.nan)
    t = cg.new_task(cg.TASK_ADDC)
    cg.add_in(t, a); cg.add_in(t, b); cg.add_out(t, out)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0 and t.completed_flag == cg.TASK_OK
    ref = (a.view(np.float32) + b.view(np.float32)).view(np.complex64)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def _difx_expect(x, mult, nch, band_off_pts, auto0):
    X = np.concatenate([np.fft.fft(x.astype(np.complex128)), np.zeros(band_off_pts + nch, np.complex128)])
    band = X[band_off_pts:band_off_pts + nch] * mult[:nch]
    return band, auto0 + np.abs(band) ** 2


def test_difx_process_upper_sideband(cg, rt):
    """exec_difxprocess with useUpperOrLower = 1 (cellspe-tasklib-dsp.cpp:663-668):
    the band starts outputvector_lengths[0] bytes into the FFT output.  As a
    task whose output 0 holds numchannels points that is the upper half of the
    FFT, X[nch .. 2 nch); through speDIFX_process, whose output 0 holds
    numchannels + 4 points (:334-338), the reference's window runs 4 points
    past the FFT, which read as zeros here."""
    rng = np.random.default_rng(3)
    nch = 64
    nfft = 2 * nch
    x = (rng.standard_normal(nfft) + 1j * rng.standard_normal(nfft)).astype(np.complex64)
    mult = np.exp(1j * rng.uniform(0, 6.28, nch + 4)).astype(np.complex64)
    # the task form: output 0 of numchannels points -> the upper half
    fftout = np.zeros(nch, np.complex64)
    conj = np.zeros(nch, np.complex64)
    auto = np.full(nch, 0.25, np.complex64)
    t = cg.new_task(cg.TASK_DIFXPROCESS)
    cg.add_in(t, x); cg.add_in(t, mult[:nch].copy())
    cg.add_out(t, fftout); cg.add_out(t, conj); cg.add_out(t, auto)
    t.subcontext[0] = nfft
    t.subcontext[2] = 1            # useUpperOrLower
    t.subcontext[3] = nfft         # twicenumchannels
    t.subcontext[4] = nch          # numchannels
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0 and t.completed_flag == cg.TASK_OK
    band, acc = _difx_expect(x, mult, nch, nch, 0.25)
    assert np.linalg.norm(fftout - band) / np.linalg.norm(band) < 1e-5
    assert np.allclose(auto.real, acc, rtol=1e-5)
    # the wrapper form: window at (nch + 4) points
    fftout = np.zeros(nch + 4, np.complex64)
    conj = np.zeros(nch + 4, np.complex64)
    auto = np.full(nch + 4, 0.5, np.complex64)
    assert rt.speDIFX_process(x.ctypes.data, mult.ctypes.data, fftout.ctypes.data, conj.ctypes.data,
                              auto.ctypes.data, nfft, nfft, 1) == 0
    band, acc = _difx_expect(x, mult, nch, nch + 4, 0.5)
    assert np.linalg.norm(fftout[:nch] - band) / np.linalg.norm(band) < 1e-5
    assert np.allclose(auto[:nch].real, acc, rtol=1e-5)


def test_rfft_task(cg, rt):
    """CELLDSP_TASK_RFFT: rows of N reals -> N/2+1 bins each (genericFFTexec_R,
    architecture.h:563-600: FFTW r2c, forward, unscaled)."""
    rng = np.random.default_rng(4)
    for n, rows in ((64, 3), (4096, 5)):
        x = rng.standard_normal((rows, n)).astype(np.float32)
        out = np.zeros((rows, n // 2 + 1), np.complex64)
        t = cg.new_task(cg.TASK_RFFT)
        cg.add_in(t, x); cg.add_out(t, out)
        t.subcontext[0] = n
        assert rt.celldsp_executeTask(ctypes.byref(t)) == 0 and t.completed_flag == cg.TASK_OK
        ref = np.fft.rfft(x.astype(np.float64), axis=1)
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-5


def test_xmac_task(cg, rt):
    """CELLDSP_TASK_XMAC: V_ij = sum_k X_i conj(X_j) over precomputed spectra
    (genericAddProduct_32fc_conj, architecture.h:427-433, for every product),
    then once more with accumulate set (read-modify-write output)."""
    rng = np.random.default_rng(5)
    S, C, K = 6, 4, 40
    spec = (rng.standard_normal((C, S, K)) + 1j * rng.standard_normal((C, S, K))).astype(np.complex64)
    P = S * (S + 1) // 2
    vis = np.zeros((C, P), np.complex64)
    prm = cg.XmacParams(S, C, K, 0)
    t = cg.new_task(cg.TASK_XMAC)
    cg.add_in_struct(t, prm); cg.add_in(t, spec); cg.add_out(t, vis)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0 and t.completed_flag == cg.TASK_OK
    X = spec.astype(np.complex128)
    ii, jj = np.tril_indices(S)
    order = np.argsort(ii * (ii + 1) // 2 + jj)
    ref = np.einsum("csk,ctk->cst", X, np.conj(X))[:, ii[order], jj[order]]
    assert np.linalg.norm(vis - ref) / np.linalg.norm(ref) < 1e-5
    prm2 = cg.XmacParams(S, C, K, 1)
    t = cg.new_task(cg.TASK_XMAC)
    cg.add_in_struct(t, prm2); cg.add_in(t, spec); cg.add_out(t, vis)
    assert rt.celldsp_executeTask(ctypes.byref(t)) == 0
    assert np.linalg.norm(vis - 2 * ref) / np.linalg.norm(2 * ref) < 1e-5


def test_continuable_tasks(cg, rt):
    """celldsp_startContinuableTask / continueTask / stopContinuableTask
    (cellspe-tasklib.cpp:364-412): the first task reserves a slot and runs
    there, later tasks run on the same slot, stop frees it and sets -1.  A
    failing first task frees the slot again and returns 1 (!vecNoErr)."""
    n = 512
    init = cg.new_task(cg.TASK_FFT_INIT)
    init.subcontext[0] = n
    spe = ctypes.c_int(-1)
    assert rt.celldsp_startContinuableTask(ctypes.byref(init), ctypes.byref(spe)) == 0
    assert 0 <= spe.value < cg.MAX_SLOTS
    rng = np.random.default_rng(6)
    for _ in range(3):
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
        out = np.zeros_like(x)
        t = cg.new_task(cg.TASK_FFT_EXEC)
        cg.add_in(t, x); cg.add_out(t, out)
        t.subcontext[0] = n
        assert rt.celldsp_continueTask(ctypes.byref(t), ctypes.byref(spe)) == 0
        ref = np.fft.fft(x.astype(np.complex128))
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-5
    # an FFT_EXEC of another length than the slot was prepared for fails
    bad = cg.new_task(cg.TASK_FFT_EXEC)
    xb = np.zeros(256, np.complex64)
    cg.add_in(bad, xb); cg.add_out(bad, xb)
    bad.subcontext[0] = 256
    assert rt.celldsp_continueTask(ctypes.byref(bad), ctypes.byref(spe)) == 1
    assert rt.celldsp_stopContinuableTask(ctypes.byref(spe)) == 0 and spe.value == -1
    # a first task that fails leaves no slot reserved
    before = [rt.celldsp_getFreeSPE() for _ in range(cg.MAX_SLOTS)]
    for s in before:
        rt.celldsp_setFreeSPE(s)
    init_bad = cg.new_task(cg.TASK_FFT_INIT)
    init_bad.subcontext[0] = 3                           # not a power of two
    spe2 = ctypes.c_int(-1)
    assert rt.celldsp_startContinuableTask(ctypes.byref(init_bad), ctypes.byref(spe2)) == 1
    after = [rt.celldsp_getFreeSPE() for _ in range(cg.MAX_SLOTS)]
    assert sorted(after) == list(range(cg.MAX_SLOTS))
    for s in after:
        rt.celldsp_setFreeSPE(s)


def test_cxx_caller_through_mangled_names(tmp_path):
    """A C++ caller built against the reference's declarations runs the
    minitest-cell.cpp MAC through the mangled speAddProduct_32fc: bit for bit
    the reference's genericAddProduct_32fc (golden vector)."""
    import subprocess

    from test_abi import build_cxx_caller

    exe = build_cxx_caller(tmp_path)
    g = np.load(GOLD / "generic_mac.npz")
    inp, out = tmp_path / "in.bin", tmp_path / "acc.bin"
    np.concatenate([g["a"], g["b"], g["acc0"]]).astype(np.complex64).tofile(inp)
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    acc = np.fromfile(out, np.complex64)
    assert np.array_equal(acc.view(np.uint32), g["mac"].view(np.uint32))
