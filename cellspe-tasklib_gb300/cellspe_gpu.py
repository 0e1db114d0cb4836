"""Python mirror of the engine's C ABI (include/cellspe_gpu.h, cellspe-tasklib*.h).

The product is ``libcellspe_gpu.so``; this module only binds it with ctypes
so that tests and the benchmark call exactly what a C/C++ caller calls.
Arrays may be numpy arrays (host memory: the engine stages them through the
GPU) or torch CUDA tensors (device memory, used in place).  There is no CPU
implementation here: if the library is missing or the GPU is unusable every
call raises ``CellspeError``.
"""
from __future__ import annotations

import ctypes
import os
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
LIB_PATH = PKG / "libcellspe_gpu.so"

# ---- constants (cellspe_gpu.h, cellspe-tasklib*.h) --------------------------
MEM_HOST, MEM_DEVICE = 0, 1
OK, ERR_ARG, ERR_UNSUPPORTED, ERR_NOMEM, ERR_CUDA, ERR_INJECTED = range(6)
LEVELS_MARK5B, LEVELS_TWOBIT, LEVELS_OFFSET_BINARY, LEVELS_VDIF = 0, 1, 2, 3
UNPACK_MSB_FIRST = 0x100
X_FP32, X_TC_FP16, X_INT8 = 0, 1, 2
VIS_CHANNEL_MAJOR, VIS_BASELINE_MAJOR = 0, 1
SPEC_INTERLEAVED, SPEC_PLANES, SPEC_MARK5B_FRAMED, SPEC_VDIF_FRAMED = 0, 1, 2, 3
MARK5B_FRAME, MARK5B_PAYLOAD = 10016, 10000

TASK_INCOMPLETE, TASK_OK, TASK_GENERICERROR, TASK_UNKOWNCOMMAND = 0xFFFF, 0, 1, 2
TASK_FLAG_DEVPTR = 0x40000000
BEHAV_BLOCKING, BEHAV_DEFAULT = 1, 0
MAX_SLOTS = 4
(TASK_NOP, TASK_MAC, TASK_MULC, TASK_ADDC, TASK_IOTEST, TASK_IOBENCH, TASK_FFT_INIT, TASK_FFT_FREE,
 TASK_FFT_EXEC, TASK_FFT_EXEC_DYN, TASK_SINCOS, TASK_SINCOS_NORM, TASK_SINCOS_GENERTR, TASK_UNPACK,
 TASK_RUNALL, TASK_DMASIMULATION, TASK_DIFXPROCESS, TASK_MAC_CONJ, TASK_RFFT, TASK_FX_CORRELATE,
 TASK_SPECTROMETER, TASK_XMAC, TASK_SIGTERM) = range(23)


class CellspeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cellspe error {code}: {msg}")
        self.code = code


# ---- ctypes mirrors of the C structs ----------------------------------------
class CellDSPTask(ctypes.Structure):
    """CellDSPTask_t (cellspe-tasklib.h); 256 bytes, next_task at offset 240."""
    _fields_ = [
        ("command", ctypes.c_uint32),
        ("completed_flag", ctypes.c_uint16),
        ("_pad0", ctypes.c_uint16),
        ("tick_count", ctypes.c_uint32),
        ("num_input_vectors", ctypes.c_uint32),
        ("inputvector_ptrs", ctypes.c_uint64 * 8),
        ("inputvector_lengths", ctypes.c_uint32 * 8),
        ("num_output_vectors", ctypes.c_uint32),
        ("_pad1", ctypes.c_uint32),
        ("outputvector_ptrs", ctypes.c_uint64 * 8),
        ("outputvector_lengths", ctypes.c_uint32 * 8),
        ("subcontext", ctypes.c_uint32 * 5),
        ("_pad2", ctypes.c_uint32),
        ("next_task", ctypes.c_uint64),
        ("_pad3", ctypes.c_uint64 * 1),
    ]


assert ctypes.sizeof(CellDSPTask) == 256


class FxParams(ctypes.Structure):
    _fields_ = [("n_inputs", ctypes.c_int), ("fft_points", ctypes.c_int), ("n_segments", ctypes.c_int),
                ("x_mode", ctypes.c_int), ("vis_order", ctypes.c_int), ("levels", ctypes.c_int),
                ("bytes_per_input", ctypes.c_longlong), ("start_sample", ctypes.c_longlong),
                ("sample_rate_hz", ctypes.c_double), ("lo_freq_hz", ctypes.c_double),
                ("accumulate", ctypes.c_int), ("memory", ctypes.c_int),
                ("custom_levels", ctypes.c_void_p), ("channel_scale", ctypes.c_void_p)]


class SpecParams(ctypes.Structure):
    _fields_ = [("fft_points", ctypes.c_int), ("overlap", ctypes.c_int), ("window", ctypes.c_int),
                ("ffts_per_spectrum", ctypes.c_int), ("n_spectra", ctypes.c_int),
                ("n_subbands", ctypes.c_int), ("input_layout", ctypes.c_int), ("levels", ctypes.c_int),
                ("raw_bytes", ctypes.c_longlong), ("pcal_tonebins", ctypes.c_int),
                ("pcal_rotatorlen", ctypes.c_int), ("pcal_ntones", ctypes.c_int),
                ("pcal_offset_hz", ctypes.c_double), ("sample_rate_hz", ctypes.c_double),
                ("memory", ctypes.c_int), ("custom_levels", ctypes.c_void_p)]


class ServiceConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_longlong), ("max_streams", ctypes.c_int), ("batch_inputs", ctypes.c_int),
                ("priority_samples", ctypes.c_longlong), ("large_samples", ctypes.c_longlong)]


class ServiceStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_longlong), ("failed", ctypes.c_longlong), ("queued", ctypes.c_longlong),
                ("running", ctypes.c_int), ("max_running", ctypes.c_int), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("p99_queue_ms", ctypes.c_double), ("budget_bytes", ctypes.c_longlong),
                ("batched_jobs", ctypes.c_longlong), ("batched_launches", ctypes.c_longlong)]


class Mark5bInfo(ctypes.Structure):
    _fields_ = [("first_frame_offset", ctypes.c_longlong), ("frames", ctypes.c_longlong),
                ("good_samples", ctypes.c_longlong), ("mjd", ctypes.c_int), ("seconds", ctypes.c_int),
                ("frame_number", ctypes.c_int), ("reserved", ctypes.c_int)]


class VdifInfo(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_longlong), ("good_samples", ctypes.c_longlong),
                ("blanked_frames", ctypes.c_longlong), ("frame_bytes", ctypes.c_int),
                ("header_bytes", ctypes.c_int), ("mjd", ctypes.c_int), ("seconds", ctypes.c_int),
                ("ns", ctypes.c_int), ("frame_number", ctypes.c_int), ("nchan_header", ctypes.c_int),
                ("thread_id", ctypes.c_int), ("station_id", ctypes.c_int), ("reserved", ctypes.c_int)]


class Addr64(ctypes.Union):
    """addr64 (cellspe_control_blocks.h)."""
    _fields_ = [("ull", ctypes.c_ulonglong), ("ui", ctypes.c_uint * 2), ("p", ctypes.c_void_p)]


class ControlBlock(ctypes.Structure):
    """control_block of the minicorrelator (cellspe_control_blocks.h): 256 bytes, 128-byte aligned."""
    _fields_ = [("rawdata_src", Addr64), ("autocorrelation_out", Addr64), ("baselines_out", Addr64 * 15),
                ("fmultipliers_src", Addr64), ("syncline", Addr64), ("spe_num", ctypes.c_int),
                ("num_spes", ctypes.c_int), ("ffts_total", ctypes.c_uint), ("ffts_to_integrate", ctypes.c_uint),
                ("spe_ls_listOnPPU", Addr64), ("spe_sig_listOnPPU", Addr64), ("_pad", ctypes.c_ubyte * 72)]


class ControlBlockT(ctypes.Structure):
    """control_block_t of the Cell spectrometer (cellspe_control_blocks.h): 128 bytes."""
    _fields_ = [("rank", ctypes.c_uint), ("terminate_flag", ctypes.c_uint), ("fft_points", ctypes.c_uint),
                ("fft_points_log2", ctypes.c_uint), ("overlap_factor", ctypes.c_uint),
                ("integrate_ffts", ctypes.c_uint), ("samples_per_rawbyte", ctypes.c_uint), ("_pad0", ctypes.c_uint),
                ("rawif_src", Addr64), ("rawif_bytecount", ctypes.c_uint), ("_pad1", ctypes.c_uint),
                ("spectrum_dst", Addr64), ("_pad2", ctypes.c_ubyte * 72)]


class XmacParams(ctypes.Structure):
    _fields_ = [("S", ctypes.c_int), ("C", ctypes.c_int), ("K", ctypes.c_int), ("accumulate", ctypes.c_int)]


assert ctypes.sizeof(FxParams) == 80 and ctypes.sizeof(SpecParams) == 88 and ctypes.sizeof(Mark5bInfo) == 40
assert ctypes.sizeof(VdifInfo) == 64


# ---- library loading ----------------------------------------------------------
_lib = None


def declared_functions() -> list[str]:
    """Names of every function declared in include/*.h."""
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:celldsp|spe|cellspe)\w*)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


TASKCORE_LIB_PATH = PKG / "libcellspe_taskcore.so"
_taskcore = None


class TaskcoreConfig(ctypes.Structure):
    """cellspe_taskcore_config (taskcore/cellspe_taskcore.h)."""
    _fields_ = [("num_cores", ctypes.c_int), ("fft_points", ctypes.c_int), ("integ_seconds", ctypes.c_double),
                ("overlap", ctypes.c_int), ("window", ctypes.c_int), ("source_channels", ctypes.c_int),
                ("channel1", ctypes.c_int), ("channel2", ctypes.c_int), ("channelorder_increasing", ctypes.c_int),
                ("sourceformat", ctypes.c_int), ("samplingfreq", ctypes.c_double), ("extract_pcal", ctypes.c_int),
                ("pcal_offset_hz", ctypes.c_double), ("pcal_harmonics_hz", ctypes.c_double),
                ("num_sources", ctypes.c_int), ("calc_xpol", ctypes.c_int), ("max_rawbuf_bytes", ctypes.c_longlong)]


def taskcore_lib() -> ctypes.CDLL:
    """libcellspe_taskcore.so: the TaskCoreCUDA plug-in and its in-memory dispatcher."""
    global _taskcore
    if _taskcore is None:
        if not TASKCORE_LIB_PATH.exists():
            raise CellspeError(ERR_CUDA, f"{TASKCORE_LIB_PATH.name} is not built; run __graft_entry__.build()")
        L = ctypes.CDLL(str(TASKCORE_LIB_PATH))
        V, LLP = ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)
        L.cellspe_taskcore_spectrometer.argtypes = [V, V, V, ctypes.c_longlong, ctypes.POINTER(V), LLP, LLP, LLP]
        L.cellspe_taskcore_spectrometer.restype = ctypes.c_int
        L.cellspe_taskcore_last_error.restype = ctypes.c_char_p
        _taskcore = L
    return _taskcore


def taskcore_spectrometer(cfg: TaskcoreConfig, src0: np.ndarray, src1=None, sink_bytes=(0, 0, 0, 0, 0)):
    """Runs cellspe_taskcore_spectrometer on host recordings; returns (sinks as uint8 arrays, spectra count)."""
    L = taskcore_lib()
    src0 = np.ascontiguousarray(src0, np.uint8)
    if src1 is not None:
        src1 = np.ascontiguousarray(src1, np.uint8)
        assert src1.size == src0.size
    sinks = [np.zeros(max(int(n), 1), np.uint8) for n in sink_bytes]
    ptrs = (ctypes.c_void_p * 5)(*[s.ctypes.data if n else None for s, n in zip(sinks, sink_bytes)])
    caps = (ctypes.c_longlong * 5)(*[int(n) for n in sink_bytes])
    used = (ctypes.c_longlong * 5)()
    nspec = ctypes.c_longlong()
    rc = L.cellspe_taskcore_spectrometer(ctypes.byref(cfg), src0.ctypes.data,
                                         src1.ctypes.data if src1 is not None else None, src0.size, ptrs, caps,
                                         used, ctypes.byref(nspec))
    if rc != 0:
        raise CellspeError(ERR_CUDA, L.cellspe_taskcore_last_error().decode())
    return [s[: used[i]] for i, s in enumerate(sinks)], nspec.value


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise CellspeError(ERR_CUDA, f"{LIB_PATH.name} is not built; run __graft_entry__.build()")
        L = ctypes.CDLL(str(LIB_PATH))
        V, I, LL, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
        sig = {
            "cellspe_last_error": ([], ctypes.c_char_p),
            "cellspe_device_count": ([], I),
            "cellspe_set_hbm_budget": ([LL], I),
            "cellspe_get_hbm_budget": ([], LL),
            "cellspe_host_alloc": ([ctypes.c_size_t], V),
            "cellspe_host_free": ([V], None),
            "cellspe_device_alloc": ([ctypes.c_size_t], V),
            "cellspe_device_free": ([V], None),
            "cellspe_memcpy": ([V, V, ctypes.c_size_t, I], I),
            "cellspe_debug_inject_failure": ([I, I], I),
            "cellspe_kernel_launches": ([], LL),
            "cellspe_last_stage_times": ([ctypes.POINTER(ctypes.c_float), I], I),
            "cellspe_unpack2bit": ([V, LL, I, I, V, V, I], I),
            "cellspe_fft_c2c": ([V, V, I, LL, I], I),
            "cellspe_fft_r2c": ([V, V, I, LL, I], I),
            "cellspe_fft_r2c_perm": ([V, V, I, LL, I], I),
            "cellspe_xmac": ([V, I, I, I, V, I, I], I),
            "cellspe_vis_lags": ([V, V, LL, I, D, I], I),
            "cellspe_xmac_f16": ([V, I, I, I, V, I, I], I),
            "cellspe_xmac_i8": ([V, V, I, I, I, V, I, I], I),
            "cellspe_fx_correlate": ([V, V, V, V], I),
            "cellspe_fx_workspace_bytes": ([V], LL),
            "cellspe_fx_correlate_async": ([V, V, V, V, V], I),
            "cellspe_release_workspace": ([], I),
            "cellspe_spectrometer": ([V, V, V, V, V], I),
            "cellspe_spectrometer_workspace_bytes": ([V], LL),
            "cellspe_spectrometer_noalloc": ([V, V, V, V, V, V], I),
            "cellspe_accumulate_f32": ([V, V, LL, I], I),
            "cellspe_mark5b_decode": ([V, LL, I, LL, V, I, V], I),
            "cellspe_spectrometer_xpol": ([V, V, V, I, I, V, V, V], I),
            "cellspe_mark5b_deframe": ([V, LL, I, LL, V, V, I, V], I),
            "cellspe_vdif_decode": ([V, LL, I, I, LL, V, I, V], I),
            "cellspe_vdif_deframe": ([V, LL, I, I, LL, V, V, I, V], I),
            "cellspe_minicorrelator_run": ([V, I], I),
            "cellspe_cell_spectrometer_task": ([ctypes.POINTER(V), V, V, V], I),
            "cellspe_pcal_new": ([D, D, I, ctypes.c_ulonglong], V),
            "cellspe_pcal_free": ([V], None),
            "cellspe_pcal_kind": ([V], I),
            "cellspe_pcal_length": ([V], I),
            "cellspe_pcal_nbins": ([V], LL),
            "cellspe_pcal_seconds": ([V], D),
            "cellspe_pcal_clear": ([V], I),
            "cellspe_pcal_adjust_sample_offset": ([V, ctypes.c_ulonglong], I),
            "cellspe_pcal_extract": ([V, V, LL, I], I),
            "cellspe_pcal_final": ([V, V], LL),
            "cellspe_service_create": ([V], V),
            "cellspe_service_submit": ([V, V, V, V, V, ctypes.POINTER(ctypes.c_longlong)], I),
            "cellspe_service_wait": ([V, ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)], I),
            "cellspe_service_get_stats": ([V, V], I),
            "cellspe_service_destroy": ([V], None),
            "celldsp_start": ([], I), "celldsp_stop": ([], I),
            "celldsp_getFreeSPE": ([], I), "celldsp_setFreeSPE": ([I], I),
            "celldsp_startTask": ([I, V], I), "celldsp_waitTask": ([I], I),
            "celldsp_executeTask": ([V], I),
            "celldsp_startContinuableTask": ([V, V], I), "celldsp_continueTask": ([V, V], I),
            "celldsp_stopContinuableTask": ([V], I),
            "celldsp_setBehaviour": ([ctypes.c_uint], None), "celldsp_getBehaviour": ([], ctypes.c_uint),
            "speNOP": ([], I), "speRunAllCheck": ([], I), "speIOCheck": ([], I), "speIOSimulation": ([], I),
            "speIOBench": ([V, ctypes.c_uint, I], I), "speIOBenchStreamed": ([V, ctypes.c_uint, I, I], I),
            "speAddProduct_32fc": ([V, V, V, I], I),
            "speFFT_init": ([I, V], I), "speFFT_exec": ([V, V, I, V], I), "speFFT_destroy": ([V], I),
            "speFFT_singleexec": ([V, V, I], I),
            "speDIFX_process": ([V, V, V, V, V, I, I, I], I),
            "speSinCosGenerator": ([ctypes.c_float, ctypes.c_float, V, I], I),
            "speSinCosAccurate": ([V, V, I], I), "speSinCosAccurateNorm": ([V, V, I], I),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def stage_times() -> list[float]:
    buf = (ctypes.c_float * 4)()
    _check(lib().cellspe_last_stage_times(buf, 4))
    return list(buf)


def kernel_launches() -> int:
    return int(lib().cellspe_kernel_launches())


def last_error() -> str:
    return (lib().cellspe_last_error() or b"").decode()


def _check(rc: int):
    if rc != 0:
        raise CellspeError(rc, last_error())


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _ptr(x):
    """(pointer, memory kind) of a numpy array or torch CUDA tensor."""
    if x is None:
        return None, None
    if _is_torch_cuda(x):
        assert x.is_contiguous()
        return ctypes.c_void_p(x.data_ptr()), MEM_DEVICE
    assert isinstance(x, np.ndarray) and x.flags.c_contiguous, "need a C-contiguous numpy array"
    return ctypes.c_void_p(x.ctypes.data), MEM_HOST


def _mem(*xs) -> int:
    kinds = {_ptr(x)[1] for x in xs if x is not None}
    if len(kinds) != 1:
        raise CellspeError(ERR_ARG, "mix of host and device buffers in one call")
    return kinds.pop()


# ---- direct entry points --------------------------------------------------------
def unpack2bit(raw, nsamp: int, nchan: int, out, levels: int = LEVELS_MARK5B, custom_levels=None,
               msb_first: bool = False):
    fmt = levels | (UNPACK_MSB_FIRST if msb_first else 0)
    cl = None
    if custom_levels is not None:
        cl = np.ascontiguousarray(custom_levels, np.float32)
    _check(lib().cellspe_unpack2bit(_ptr(raw)[0], nsamp, nchan, fmt,
                                    ctypes.c_void_p(cl.ctypes.data) if cl is not None else None,
                                    _ptr(out)[0], _mem(raw, out)))
    return out


def fft_c2c(x, out, n: int, batch: int):
    _check(lib().cellspe_fft_c2c(_ptr(x)[0], _ptr(out)[0], n, batch, _mem(x, out)))
    return out


def fft_r2c(x, out, n: int, batch: int):
    _check(lib().cellspe_fft_r2c(_ptr(x)[0], _ptr(out)[0], n, batch, _mem(x, out)))
    return out


def fft_r2c_perm(x, out):
    """cellspe_fft_r2c_perm: rows of n reals -> IPP Perm-packed rows of n floats."""
    n = x.shape[-1]
    batch = (x.size if isinstance(x, np.ndarray) else x.numel()) // n
    _check(lib().cellspe_fft_r2c_perm(_ptr(x)[0], _ptr(out)[0], n, batch, _mem(x, out)))
    return out


def xmac(spectra, S: int, C: int, K: int, vis, accumulate: bool = False):
    _check(lib().cellspe_xmac(_ptr(spectra)[0], S, C, K, _ptr(vis)[0], int(accumulate), _mem(spectra, vis)))
    return vis


def vis_lags(vis, lags, scale: float = 1.0):
    """vis, lags: complex64 [P][C] (baseline-major)."""
    P, C = vis.shape[0], vis.shape[-1]
    _check(lib().cellspe_vis_lags(_ptr(vis)[0], _ptr(lags)[0], P, C, scale, _mem(vis, lags)))
    return lags


def xmac_f16(spectra_f16, S: int, C: int, K: int, vis, accumulate: bool = False):
    """spectra_f16: float16 [C][2][S][K] (Re plane, Im plane)."""
    _check(lib().cellspe_xmac_f16(_ptr(spectra_f16)[0], S, C, K, _ptr(vis)[0], int(accumulate),
                                  _mem(spectra_f16, vis)))
    return vis


def xmac_i8(planes, scale, S: int, C: int, K: int, vis, accumulate: bool = False):
    """INT8 X stage on planes int8 [C][2][S][K] and scale float [S][C]."""
    _check(lib().cellspe_xmac_i8(_ptr(planes)[0], _ptr(scale)[0], S, C, K, _ptr(vis)[0], int(accumulate),
                                 _mem(planes, scale, vis)))


def fx_params(S, N, K, bytes_per_input, x_mode=X_FP32, vis_order=VIS_CHANNEL_MAJOR,
              levels=LEVELS_OFFSET_BINARY, start_sample=0, fs_hz=0.0, lo_hz=0.0, accumulate=False,
              memory=MEM_HOST, custom_levels=None, channel_scale=None) -> FxParams:
    p = FxParams(S, N, K, x_mode, vis_order, levels, bytes_per_input, start_sample, fs_hz, lo_hz,
                 int(accumulate), memory, None, None)
    p._keep = (custom_levels, channel_scale)
    if custom_levels is not None:
        p.custom_levels = custom_levels.ctypes.data
    if channel_scale is not None:
        p.channel_scale = _ptr(channel_scale)[0].value
    return p


def fx_correlate(params: FxParams, raw, vis, delay_poly=None):
    params.memory = _mem(raw, vis)
    _check(lib().cellspe_fx_correlate(ctypes.byref(params), _ptr(raw)[0],
                                      _ptr(delay_poly)[0] if delay_poly is not None else None,
                                      _ptr(vis)[0]))
    return vis


def fx_correlate_async(params: FxParams, raw, vis, stream_ptr: int, delay_poly=None):
    params.memory = MEM_DEVICE
    _check(lib().cellspe_fx_correlate_async(ctypes.byref(params), _ptr(raw)[0],
                                            _ptr(delay_poly)[0] if delay_poly is not None else None,
                                            _ptr(vis)[0], ctypes.c_void_p(stream_ptr)))


def spec_params(N, overlap, window, K, nspec, nsub, raw_bytes, layout=SPEC_INTERLEAVED,
                levels=LEVELS_MARK5B, tonebins=0, rotatorlen=0, ntones=0, offset_hz=0.0, fs_hz=0.0,
                memory=MEM_HOST) -> SpecParams:
    return SpecParams(N, overlap, window, K, nspec, nsub, layout, levels, raw_bytes, tonebins, rotatorlen,
                      ntones, offset_hz, fs_hz, memory, None)


def spectrometer(params: SpecParams, raw, power, pcal_bins=None, pcal_tones=None):
    params.memory = _mem(raw, power)
    _check(lib().cellspe_spectrometer(ctypes.byref(params), _ptr(raw)[0], _ptr(power)[0],
                                      _ptr(pcal_bins)[0] if pcal_bins is not None else None,
                                      _ptr(pcal_tones)[0] if pcal_tones is not None else None))
    return power


def spectrometer_xpol(params: SpecParams, raw0, raw1, channel0: int, channel1: int, power, xpol, pcal_bins=None):
    """cellspe_spectrometer_xpol: power [2][n][N/2+1], xpol [n][N/2+1] complex, pcal [2][n][T]."""
    params.memory = _mem(raw0, raw1, power, xpol)
    _check(lib().cellspe_spectrometer_xpol(ctypes.byref(params), _ptr(raw0)[0], _ptr(raw1)[0], channel0, channel1,
                                           _ptr(power)[0], _ptr(xpol)[0],
                                           _ptr(pcal_bins)[0] if pcal_bins is not None else None))
    return power, xpol


def mark5b_decode(framed, nchan: int, nsamp: int, out) -> Mark5bInfo:
    """cellspe_mark5b_decode: framed Mark5B bytes -> out[nchan][nsamp] float32 (0.0 where blanked)."""
    info = Mark5bInfo()
    nbytes = framed.numel() if _is_torch_cuda(framed) else framed.size
    _check(lib().cellspe_mark5b_decode(_ptr(framed)[0], nbytes, nchan, nsamp, _ptr(out)[0], _mem(framed, out),
                                       ctypes.byref(info)))
    return info


def vdif_decode(framed, nchan: int, mbps: int, nsamp: int, out) -> VdifInfo:
    """cellspe_vdif_decode: framed VDIF bytes -> out[nchan][nsamp] float32 (0.0 where blanked)."""
    info = VdifInfo()
    nbytes = framed.numel() if _is_torch_cuda(framed) else framed.size
    _check(lib().cellspe_vdif_decode(_ptr(framed)[0], nbytes, nchan, mbps, nsamp, _ptr(out)[0], _mem(framed, out),
                                     ctypes.byref(info)))
    return info


def vdif_deframe(framed, nchan: int, mbps: int, frames: int = 0, payload=None, valid_mask=None) -> VdifInfo:
    """cellspe_vdif_deframe: the payloads the decoder reads, back to back (+ validity bit per
    sample time).  With payload None only the frame checks run (info.frames tells the size)."""
    info = VdifInfo()
    nbytes = framed.numel() if _is_torch_cuda(framed) else framed.size
    _check(lib().cellspe_vdif_deframe(_ptr(framed)[0], nbytes, nchan, mbps, frames,
                                      _ptr(payload)[0] if payload is not None else None,
                                      _ptr(valid_mask)[0] if valid_mask is not None else None,
                                      _mem(framed, payload, valid_mask), ctypes.byref(info)))
    return info


def mark5b_deframe(framed, nchan: int, frames: int = 0, payload=None, valid_mask=None) -> Mark5bInfo:
    """cellspe_mark5b_deframe: payload bytes back to back (+ validity bit per sample time).
    With payload None only the frame search runs (info.frames tells the size)."""
    info = Mark5bInfo()
    nbytes = framed.numel() if _is_torch_cuda(framed) else framed.size
    _check(lib().cellspe_mark5b_deframe(_ptr(framed)[0], nbytes, nchan, frames,
                                        _ptr(payload)[0] if payload is not None else None,
                                        _ptr(valid_mask)[0] if valid_mask is not None else None,
                                        _mem(framed, payload, valid_mask), ctypes.byref(info)))
    return info


def minicorrelator_run(blocks) -> None:
    """cellspe_minicorrelator_run on an array of 6 ControlBlock (host buffers)."""
    arr = (ControlBlock * len(blocks))(*blocks)
    _check(lib().cellspe_minicorrelator_run(ctypes.addressof(arr), len(blocks)))


PCAL_TRIVIAL, PCAL_SHIFTING, PCAL_IMPLICIT_SHIFT = 0, 1, 2


class Pcal:
    """A PCal extractor (cellspe_pcal.h): PCal::getNew and its methods."""

    def __init__(self, bandwidth_hz: float, spacing_hz: float, offset_hz: int, sampleoffset: int = 0):
        self.h = lib().cellspe_pcal_new(bandwidth_hz, spacing_hz, int(offset_hz), int(sampleoffset))
        if not self.h:
            raise CellspeError(ERR_ARG, last_error())

    kind = property(lambda self: lib().cellspe_pcal_kind(self.h))
    length = property(lambda self: lib().cellspe_pcal_length(self.h))
    nbins = property(lambda self: lib().cellspe_pcal_nbins(self.h))
    seconds = property(lambda self: lib().cellspe_pcal_seconds(self.h))

    def clear(self):
        _check(lib().cellspe_pcal_clear(self.h))

    def adjust_sample_offset(self, sampleoffset: int):
        _check(lib().cellspe_pcal_adjust_sample_offset(self.h, int(sampleoffset)))

    def extract(self, samples):
        if _is_torch_cuda(samples):
            _check(lib().cellspe_pcal_extract(self.h, samples.data_ptr(), samples.numel(), MEM_DEVICE))
        else:
            x = np.ascontiguousarray(samples, np.float32)
            _check(lib().cellspe_pcal_extract(self.h, x.ctypes.data, x.size, MEM_HOST))

    def final(self, out=None):
        """(tones complex64 [length], samples integrated); tones the reference
        leaves unwritten keep `out`'s values (zeros by default)."""
        out = np.zeros(self.length, np.complex64) if out is None else out
        n = lib().cellspe_pcal_final(self.h, out.ctypes.data)
        if n < 0:
            _check(-n)
        return out, n

    def close(self):
        if self.h:
            lib().cellspe_pcal_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CellSpectrometerTask:
    """One Cell-spectrometer SPE context: run(cb) per task, close() sends terminate_flag."""

    def __init__(self, levels4=None):
        self.state = ctypes.c_void_p(None)
        self.levels = None if levels4 is None else np.ascontiguousarray(levels4, np.float32)

    def run(self, cb: ControlBlockT):
        stats = (ctypes.c_uint * 3)()
        lv = None if self.levels is None else self.levels.ctypes.data
        _check(lib().cellspe_cell_spectrometer_task(ctypes.byref(self.state), ctypes.addressof(cb), lv, stats))
        return list(stats)

    def close(self):
        cb = ControlBlockT()
        cb.terminate_flag = 1
        _check(lib().cellspe_cell_spectrometer_task(ctypes.byref(self.state), ctypes.addressof(cb), None, None))


def spectrometer_noalloc(params: SpecParams, raw, power, pcal_bins=None, pcal_tones=None, stream: int = 0):
    """cellspe_spectrometer_noalloc: device tensors only, asynchronous on `stream`."""
    params.memory = MEM_DEVICE
    _check(lib().cellspe_spectrometer_noalloc(ctypes.byref(params), _ptr(raw)[0], _ptr(power)[0],
                                              _ptr(pcal_bins)[0] if pcal_bins is not None else None,
                                              _ptr(pcal_tones)[0] if pcal_tones is not None else None,
                                              ctypes.c_void_p(stream)))
    return power


class Service:
    """cellspe_service_*: continuous-batching correlation service."""

    def __init__(self, hbm_budget_bytes: int = 0, max_streams: int = 0, priority_samples: int = 0,
                 large_samples: int = 0, batch_inputs: int = 0):
        cfg = ServiceConfig(hbm_budget_bytes, max_streams, batch_inputs, priority_samples, large_samples)
        self._h = lib().cellspe_service_create(ctypes.byref(cfg))
        if not self._h:
            raise CellspeError(ERR_CUDA, last_error())
        self._keep = {}

    def submit(self, params: FxParams, raw, vis, delay_poly=None) -> int:
        params.memory = _mem(raw, vis)
        jid = ctypes.c_longlong()
        _check(lib().cellspe_service_submit(self._h, ctypes.byref(params), _ptr(raw)[0],
                                            _ptr(delay_poly)[0] if delay_poly is not None else None,
                                            _ptr(vis)[0], ctypes.byref(jid)))
        self._keep[jid.value] = (params, raw, vis, delay_poly)
        return jid.value

    def wait(self, job_id: int) -> float:
        lat = ctypes.c_double()
        rc = lib().cellspe_service_wait(self._h, job_id, ctypes.byref(lat))
        self._keep.pop(job_id, None)
        _check(rc)
        return lat.value

    def stats(self) -> dict:
        st = ServiceStats()
        _check(lib().cellspe_service_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServiceStats._fields_}

    def close(self):
        if self._h:
            lib().cellspe_service_destroy(self._h)
            self._h = None


# ---- task API ------------------------------------------------------------------
def new_task(command: int) -> CellDSPTask:
    t = CellDSPTask()
    t.command = command
    return t


def add_in(t: CellDSPTask, arr) -> None:
    p, _ = _ptr(arr)
    n = arr.nbytes if isinstance(arr, np.ndarray) else arr.numel() * arr.element_size()
    t.inputvector_ptrs[t.num_input_vectors] = p.value
    t.inputvector_lengths[t.num_input_vectors] = n
    t.num_input_vectors += 1


def add_in_struct(t: CellDSPTask, s: ctypes.Structure) -> None:
    t.inputvector_ptrs[t.num_input_vectors] = ctypes.addressof(s)
    t.inputvector_lengths[t.num_input_vectors] = ctypes.sizeof(s)
    t.num_input_vectors += 1


def add_out(t: CellDSPTask, arr) -> None:
    p, _ = _ptr(arr)
    n = arr.nbytes if isinstance(arr, np.ndarray) else arr.numel() * arr.element_size()
    t.outputvector_ptrs[t.num_output_vectors] = p.value
    t.outputvector_lengths[t.num_output_vectors] = n
    t.num_output_vectors += 1
