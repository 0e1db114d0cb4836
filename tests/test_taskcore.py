"""TaskCoreCUDA, the swspectrometer plug-in: build and interface checks (no GPU).

* The plug-in and its dispatcher library are built and export the plug-in
  class and the in-memory dispatcher.
* Where the reference tree is at hand (the container that compiled
  oracle/_ref from it), TaskCoreCUDA.cpp also compiles against the
  spectrometer's own TaskCore.h / Settings.h / Buffer.h
  (spectrometer/src), and the stand-in headers give swspect_settings_t,
  Buffer and TaskCore the same layout as the originals: same size and the
  same offset for every member, and the same vtable slot order.
"""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "cellspe-tasklib_gb300"
TC = PKG / "taskcore"

FIELDS = """num_cores fft_points fft_integ_seconds fft_overlap_factor wf_type bits_per_sample
channelorder_increasing seconds_to_skip source_channels use_channel_file1 use_channel_file2 samplingfreq
pcaloffsethz pcalharmonicshz max_rawbuf_size extract_PCal calc_Xpol costas_loop use_live_plot
basefilename1_pattern basefilename2_pattern sources sinks pcalsinks num_sources num_sinks num_xpols
sourceformat sourceformat_str sinkformat rawbuffers outbuffers outbuffersXpol outbuffersPCal basefilename1
basefilename2 dt df averaged_ffts averaged_overlapped_ffts fft_overlap_points fft_ssb_points
rawbytes_per_channelsample raw_fullfft_bytes raw_overlap_bytes fft_bytes fft_bytes_ssb fft_bytes_xpol
rawbuf_size max_spectra_per_buffer max_specffts_per_buffer max_buffers_per_spectrum core_overlapped_ffts
core_averaged_ffts pcal_tonebins pcal_rotatorlen pcal_pulses pcal_pulses_per_fft pcal_result_bytes logIO log
tlog""".split()

LAYOUT = r'''
#include <cstdio>
#include "TaskCore.h"
#include "Buffer.h"
struct Probe : TaskCore {
  void prepare(swspect_settings_t*) override {}
  int run(Buffer**, Buffer**, Buffer**, Buffer**) override { return 0; }
};
int main() {
  static swspect_settings_t s;
  const char* b = (const char*)&s;
  std::printf("size %zu\n", sizeof(swspect_settings_t));
%FIELDS%
  std::printf("Buffer %zu\n", sizeof(Buffer));
  std::printf("enums %d %d %d %d\n", (int)Blackman, (int)Mk5B, (int)Maxim, (int)Binary);
  // vtable slot of each virtual method: pointer-to-member values encode it
  typedef int (TaskCore::*RunFn)(Buffer**, Buffer**, Buffer**, Buffer**);
  RunFn r = &TaskCore::run; int (TaskCore::*j)() = &TaskCore::join; int (TaskCore::*f)() = &TaskCore::finalize;
  int (TaskCore::*c)(Buffer**, Buffer**) = &TaskCore::combineResults; void (TaskCore::*z)(Buffer*) = &TaskCore::resetBuffer;
  void (TaskCore::*p)(swspect_settings_t*) = &TaskCore::prepare;
  size_t v[6]; std::memcpy(&v[0], &p, 8); std::memcpy(&v[1], &r, 8); std::memcpy(&v[2], &j, 8);
  std::memcpy(&v[3], &f, 8); std::memcpy(&v[4], &c, 8); std::memcpy(&v[5], &z, 8);
  std::printf("vslots %zu %zu %zu %zu %zu %zu\n", v[0], v[1], v[2], v[3], v[4], v[5]);
  Probe pr; (void)pr;
  return 0;
}
'''


def _layout(tmp_path, incdir: Path, tag: str) -> str:
    body = "\n".join(f'  std::printf("{f} %td\\n", (const char*)&s.{f} - b);' for f in FIELDS)
    src = tmp_path / f"layout_{tag}.cpp"
    src.write_text(LAYOUT.replace("%FIELDS%", body).replace("#include <cstdio>", "#include <cstdio>\n#include <cstring>"))
    exe = tmp_path / f"layout_{tag}"
    subprocess.run(["g++", "-std=c++17", "-w", "-I", str(incdir), str(src), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def test_taskcore_library_exports_the_plugin():
    import cellspe_gpu

    lib = PKG / "libcellspe_taskcore.so"
    if not lib.exists():
        import __graft_entry__

        __graft_entry__.build()
    out = subprocess.run(["nm", "-DC", "--defined-only", str(lib)], capture_output=True, text=True,
                         check=True).stdout
    for sym in ("TaskCoreCUDA::prepare(swspect_settings_tt*)", "TaskCoreCUDA::run(Buffer**, Buffer**, Buffer**, Buffer**)",
                "TaskCoreCUDA::join()", "TaskCoreCUDA::combineResults(Buffer**, Buffer**)",
                "TaskCoreCUDA::finalize()", "TaskCoreCUDA::resetBuffer(Buffer*)",
                "cellspe_taskcore_spectrometer", "cellspe_taskcore_last_error"):
        assert sym in out, sym
    assert cellspe_gpu.taskcore_lib()


def _reference_src():
    import oracle

    tree = oracle.reference_tree()
    if tree is None or not (tree / "spectrometer" / "src" / "TaskCore.h").exists():
        pytest.skip("the reference tree is not at hand here")
    return tree / "spectrometer" / "src"


def test_plugin_compiles_against_the_reference_headers():
    ref = _reference_src()
    for src in (TC / "TaskCoreCUDA.cpp", TC / "taskcore_dispatch.cpp"):
        subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", str(ref), "-I", str(TC),
                        "-I", str(ROOT / "include"), str(src)], check=True)


def test_stand_in_headers_keep_the_reference_layout(tmp_path):
    ref = _reference_src()
    mine = _layout(tmp_path, TC / "compat", "compat")
    theirs = _layout(tmp_path, ref, "reference")
    assert mine == theirs
    assert "size " in mine and len(mine.splitlines()) == len(FIELDS) + 4
