"""Build recipe for libcellspe_gpu.so (sm_103a only).

Every .cu / .cpp under csrc/ is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked
into ``libcellspe_gpu.so`` next to this file (static CUDA runtime, C ABI of
include/*.h).  Objects go to _build/<host machine>/ (git-ignored), so objects
of another host architecture are never linked; the library and the programs
are relinked when the stamp of this host's last link is missing or older
than an object.  Rebuilds only what changed (by mtime against the sources
and headers).  The swspectrometer plug-in (taskcore/: TaskCoreCUDA and its
in-memory dispatcher) is host C++ over that library's C ABI, built with g++
into libcellspe_taskcore.so.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build" / platform.machine()
LIB = PKG / "libcellspe_gpu.so"
STAMP = OUT / "linked.stamp"            # this host's last link of LIB and the programs
APPS = sorted((CSRC / "apps").glob("*.cpp"))
TASKCORE = PKG / "taskcore"
TASKCORE_LIB = PKG / "libcellspe_taskcore.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
          "--expt-relaxed-constexpr"]


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))


def _stale(obj: Path, src: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = OUT / (src.name + ".o")
    cmd = [NVCC, *ARCH, *COMMON, "-c", str(src), "-o", str(obj)]
    if verbose_ptxas and src.suffix == ".cu":
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"nvcc failed on {src.name}")
    if verbose_ptxas:
        (OUT / (src.name + ".ptxas.txt")).write_text(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    deps = _headers()
    todo = [s for s in srcs if force or verbose_ptxas or _stale(OUT / (s.name + ".o"), s, deps)]
    with ThreadPoolExecutor(max_workers=max(2, min(len(todo) or 1, os.cpu_count() or 4))) as ex:
        list(ex.map(lambda s: _compile(s, verbose_ptxas), todo))
    objs = [OUT / (s.name + ".o") for s in srcs]
    relink = (force or bool(todo) or not LIB.exists() or not STAMP.exists()
              or any(o.stat().st_mtime > STAMP.stat().st_mtime for o in objs))
    if relink:
        cmd = [NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    for src in APPS:                 # entry-point programs linked against the library
        exe = PKG / src.stem
        if relink or not exe.exists() or exe.stat().st_mtime < max(src.stat().st_mtime, LIB.stat().st_mtime):
            cmd = ["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                   "-L", str(PKG), "-lcellspe_gpu", "-Wl,-rpath,$ORIGIN", "-lpthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError(f"link failed for {src.name}")
    # the swspectrometer plug-in (TaskCoreCUDA) and its in-memory dispatcher,
    # compiled against the stand-in spectrometer headers
    tc_srcs = sorted(TASKCORE.glob("*.cpp"))
    tc_deps = tc_srcs + list(TASKCORE.glob("*.h")) + list((TASKCORE / "compat").glob("*.h")) + [LIB]
    if relink or not TASKCORE_LIB.exists() or TASKCORE_LIB.stat().st_mtime < max(d.stat().st_mtime for d in tc_deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-I", str(TASKCORE / "compat"),
               "-I", str(TASKCORE), "-I", str(ROOT / "include"), *map(str, tc_srcs), "-o", str(TASKCORE_LIB),
               "-L", str(PKG), "-lcellspe_gpu", "-Wl,-rpath,$ORIGIN", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("build failed for libcellspe_taskcore.so")
    if relink:
        STAMP.touch()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
