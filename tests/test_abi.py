"""The C-ABI library loads and exports every symbol the headers declare (no GPU calls)."""
import ctypes
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_all_declared_symbols():
    import cellspe_gpu

    if not cellspe_gpu.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    names = cellspe_gpu.declared_functions()
    assert len(names) >= 40
    out = subprocess.run(["nm", "-D", "--defined-only", str(cellspe_gpu.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    lib = ctypes.CDLL(str(cellspe_gpu.LIB_PATH))
    for n in names:
        assert getattr(lib, n)


def test_task_descriptor_layout_matches_header(tmp_path):
    """CellDSPTask_t keeps the reference's field offsets (cellspe-tasklib.h:62-86)."""
    import cellspe_gpu

    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "cellspe_gpu.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(CellDSPTask_t), offsetof(CellDSPTask_t, completed_flag),
   offsetof(CellDSPTask_t, inputvector_ptrs), offsetof(CellDSPTask_t, outputvector_ptrs),
   offsetof(CellDSPTask_t, subcontext), offsetof(CellDSPTask_t, next_task), sizeof(cellspe_fx_params),
   sizeof(cellspe_spec_params), sizeof(cellspe_service_config), offsetof(cellspe_service_config, priority_samples),
   sizeof(cellspe_service_stats), sizeof(cellspe_vdif_info));
 return 0; }''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    vals = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    T = cellspe_gpu.CellDSPTask
    assert vals == [ctypes.sizeof(T), T.completed_flag.offset, T.inputvector_ptrs.offset,
                    T.outputvector_ptrs.offset, T.subcontext.offset, T.next_task.offset,
                    ctypes.sizeof(cellspe_gpu.FxParams), ctypes.sizeof(cellspe_gpu.SpecParams),
                    ctypes.sizeof(cellspe_gpu.ServiceConfig), cellspe_gpu.ServiceConfig.priority_samples.offset,
                    ctypes.sizeof(cellspe_gpu.ServiceStats), ctypes.sizeof(cellspe_gpu.VdifInfo)]
    assert vals[0] == 256 and vals[5] == 240


def test_command_enum_keeps_reference_values():
    import cellspe_gpu as cg

    # cellspe-tasklib-dsp.h:27-46: the original commands keep their values,
    # SIGTERM stays last.
    assert (cg.TASK_NOP, cg.TASK_MAC, cg.TASK_FFT_EXEC_DYN, cg.TASK_UNPACK, cg.TASK_DIFXPROCESS) == (0, 1, 9, 13, 16)
    assert cg.TASK_SIGTERM == max(cg.TASK_MAC_CONJ, cg.TASK_XMAC, cg.TASK_SPECTROMETER) + 1
    hdr = (ROOT / "include" / "cellspe-tasklib-dsp.h").read_text()
    body = hdr[hdr.index("enum CellDspCommandEnum"): hdr.index("};", hdr.index("enum CellDspCommandEnum"))]
    names = [l.split(",")[0].split("=")[0].split("/*")[0].strip() for l in body.splitlines()
             if l.strip().startswith("CELLDSP_TASK_")]
    assert names[-1] == "CELLDSP_TASK_SIGTERM" and len(names) == 23


def test_no_cpu_fallback_without_gpu():
    """Without a usable GPU the engine fails loudly instead of computing on the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import numpy as np

    import cellspe_gpu as cg

    raw = np.zeros(64, np.uint8)
    out = np.zeros(256, np.float32)
    with pytest.raises(cg.CellspeError) as e:
        cg.unpack2bit(raw, 256, 1, out)
    assert e.value.code == cg.ERR_CUDA


# A caller compiled against the reference's own declarations (cellspe-tasklib.h:
# 122-133, cellspe-tasklib-dsp.h:79-94: C++ linkage, fc32 an unnamed-struct
# typedef) links against the C++-mangled names; these are the declarations.
CXX_CALLER = r'''
#include <cstdio>
#include <cstring>
struct CellDSPTask_tt;
typedef CellDSPTask_tt CellDSPTask_t;
typedef struct { float re; float im; } fc32;
typedef fc32 cf32;
int celldsp_start(); int celldsp_stop(); int celldsp_getFreeSPE(); int celldsp_setFreeSPE(int targetSPE);
int celldsp_startTask(int targetSPE, CellDSPTask_t* task); int celldsp_waitTask(int targetSPE);
int celldsp_executeTask(CellDSPTask_t* task); int celldsp_startContinuableTask(CellDSPTask_t* task, int* speID);
int celldsp_continueTask(CellDSPTask_t* task, int* speID); int celldsp_stopContinuableTask(int* speID);
void celldsp_setBehaviour(unsigned int flags); unsigned int celldsp_getBehaviour();
int speNOP(); int speRunAllCheck(); int speIOCheck(); int speIOSimulation();
int speIOBench(void* buffer, unsigned int bufbytes, int spes);
int speIOBenchStreamed(void* buffer, unsigned int bufbytes, int spes, int stream_length);
int speAddProduct_32fc(fc32* src, fc32* src2, fc32* accumulator, int length);
int speFFT_init(int fft_len, int* speID); int speFFT_exec(void* in, void* out, int fft_len, int* speID);
int speFFT_destroy(int* speID); int speFFT_singleexec(void* in, void* out, int fft_len);
int speDIFX_process(void*, void*, void*, void*, void*, int nfft, int twicenumchannels, int useUpperOrLower);
int speSinCosGenerator(float startphase, float increment, fc32* cos_sin_out, int numiter);
int speSinCosAccurate(float* argument, cf32* cos_sin_out, int argumentcount);
int speSinCosAccurateNorm(float* normalizedargument, cf32* cos_sin_out, int argumentcount);
volatile int use_all = 0;
int main(int argc, char** argv) {
  if (use_all) {   // referenced so that every name must resolve at link time
    celldsp_getFreeSPE(); celldsp_setFreeSPE(0); celldsp_startTask(0, 0); celldsp_waitTask(0);
    celldsp_executeTask(0); celldsp_startContinuableTask(0, 0); celldsp_continueTask(0, 0);
    celldsp_stopContinuableTask(0); speRunAllCheck(); speIOCheck(); speIOSimulation(); speIOBench(0, 0, 0);
    speIOBenchStreamed(0, 0, 0, 0); speFFT_init(0, 0); speFFT_exec(0, 0, 0, 0); speFFT_destroy(0);
    speFFT_singleexec(0, 0, 0); speDIFX_process(0, 0, 0, 0, 0, 0, 0, 0); speSinCosGenerator(0, 0, 0, 0);
    speSinCosAccurate(0, 0, 0); speSinCosAccurateNorm(0, 0, 0);
  }
  celldsp_setBehaviour(1u); unsigned b = celldsp_getBehaviour(); celldsp_setBehaviour(0u);
  std::printf("behaviour %u\n", b);
  if (argc > 2) {  // on a GPU: a MAC through the mangled names; in: a, b, acc; out: acc
    const int n = 1024; static fc32 a[n], c[n], acc[n];
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(a, sizeof a, 1, f) != 1 || std::fread(c, sizeof c, 1, f) != 1 ||
        std::fread(acc, sizeof acc, 1, f) != 1) return 3;
    std::fclose(f);
    if (celldsp_start() != 0 || speNOP() != 0) return 2;
    int rc = speAddProduct_32fc(a, c, acc, n);
    celldsp_stop();
    f = std::fopen(argv[2], "wb"); std::fwrite(acc, sizeof acc, 1, f); std::fclose(f);
    return rc;
  }
  return 0;
}
'''


def build_cxx_caller(tmp_path):
    import cellspe_gpu

    src = tmp_path / "caller.cpp"
    src.write_text(CXX_CALLER)
    exe = tmp_path / "caller"
    subprocess.run(["g++", "-std=c++17", str(src), "-o", str(exe), "-L", str(cellspe_gpu.PKG), "-lcellspe_gpu",
                    f"-Wl,-rpath,{cellspe_gpu.PKG}"], check=True)
    return exe


def test_cxx_linkage_aliases_link_and_run(tmp_path):
    """celldsp_* and spe* under their C++-mangled names, for callers already
    compiled against the reference's headers."""
    import cellspe_gpu

    if not cellspe_gpu.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    exe = build_cxx_caller(tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert out.startswith("behaviour ")          # (the runtime is not started: no GPU work here)
    syms = subprocess.run(["nm", "-D", "--defined-only", str(cellspe_gpu.LIB_PATH)], capture_output=True, text=True,
                          check=True).stdout
    assert "_Z17celldsp_startTaskiP14CellDSPTask_tt" in syms and "_Z18speAddProduct_32fcP4fc32S0_S0_i" in syms


def test_control_block_layouts_match_reference(tmp_path):
    """control_block (minicorrelator.h:107-119) and control_block_t
    (cell_spectrometer.h:104-115): member offsets of the reference's
    declarations on LP64 (addr64 is 8 bytes, the first member and the struct
    128-byte aligned), from the C header and from the ctypes mirror."""
    import cellspe_gpu as cg

    src = tmp_path / "cb.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "cellspe_control_blocks.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(control_block), _Alignof(control_block),
   offsetof(control_block, rawdata_src), offsetof(control_block, autocorrelation_out),
   offsetof(control_block, baselines_out), offsetof(control_block, fmultipliers_src), offsetof(control_block, syncline),
   offsetof(control_block, spe_num), offsetof(control_block, num_spes), offsetof(control_block, ffts_total),
   offsetof(control_block, ffts_to_integrate), offsetof(control_block, spe_ls_listOnPPU),
   offsetof(control_block, spe_sig_listOnPPU));
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(control_block_t), _Alignof(control_block_t),
   offsetof(control_block_t, rank), offsetof(control_block_t, terminate_flag), offsetof(control_block_t, fft_points),
   offsetof(control_block_t, fft_points_log2), offsetof(control_block_t, overlap_factor),
   offsetof(control_block_t, integrate_ffts), offsetof(control_block_t, samples_per_rawbyte),
   offsetof(control_block_t, rawif_src), offsetof(control_block_t, rawif_bytecount),
   offsetof(control_block_t, spectrum_dst));
 return 0; }''')
    exe = tmp_path / "cb"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    cb, cbt = (list(map(int, ln.split())) for ln in lines)
    assert cb == [256, 128, 0, 8, 16, 136, 144, 152, 156, 160, 164, 168, 176]
    assert cbt == [128, 128, 0, 4, 8, 12, 16, 20, 24, 32, 40, 48]
    C, T = cg.ControlBlock, cg.ControlBlockT
    assert [ctypes.sizeof(C), C.rawdata_src.offset, C.autocorrelation_out.offset, C.baselines_out.offset,
            C.fmultipliers_src.offset, C.syncline.offset, C.spe_num.offset, C.num_spes.offset, C.ffts_total.offset,
            C.ffts_to_integrate.offset, C.spe_ls_listOnPPU.offset, C.spe_sig_listOnPPU.offset] == [cb[0]] + cb[2:]
    assert [ctypes.sizeof(T), T.rank.offset, T.terminate_flag.offset, T.fft_points.offset, T.fft_points_log2.offset,
            T.overlap_factor.offset, T.integrate_ffts.offset, T.samples_per_rawbyte.offset, T.rawif_src.offset,
            T.rawif_bytecount.offset, T.spectrum_dst.offset] == [cbt[0]] + cbt[2:]
