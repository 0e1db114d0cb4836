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
