"""Build the GB300 DEAC engine in-tree.

Produces, under deac-cpp_gb300/:
  lib/libdeac_gb300.so        the C-ABI library (include/deac_gb300.h)
  lib/libdeac_gb300_debug.so  test aids (include/deac_gb300_debug.h)
  bin/deac.e                  the deac.e command-line front end

Device code is compiled for sm_103a only, with --fmad=false (every fused
multiply-add in the kernels is an explicit fma()), host code with
-ffp-contract=off for the same reason.  Translation units compile in
parallel; a full build takes well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libdeac_gb300.so"
DEBUG_LIB = PKG / "lib" / "libdeac_gb300_debug.so"  # test aids (deac_debug.cu), apart from the engine
EXE = PKG / "bin" / "deac.e"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out))
        elif out and out.strip() and os.environ.get("DEAC_BUILD_VERBOSE"):
            print(out)
    if failed:
        msg = "\n".join(f"$ {' '.join(c)}\n{out}" for c, out in failed)
        raise RuntimeError(f"build failed:\n{msg}")


def _stale(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    EXE.parent.mkdir(exist_ok=True)
    inc = ["-I", str(REPO / "include"), "-I", str(CSRC)]
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + [REPO / "include" / "deac_gb300.h"]
    nv = nvcc()
    cu_flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                       "-Xptxas", "-warn-spills"] + inc
    if ptxas_verbose:
        cu_flags += ["-Xptxas", "-v"]
    objs, cmds = [], []
    debug_obj = BUILD / "deac_debug.o"
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".o")
        if obj != debug_obj:
            objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append([nv] + cu_flags + ["-c", str(src), "-o", str(obj)])
    host_srcs = [CSRC / "deac_model.cpp"]
    for src in host_srcs:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"] + inc +
                        ["-c", str(src), "-o", str(obj)])
    if verbose:
        for c in cmds:
            print("$", " ".join(c))
    _run_all(cmds)
    links = []
    if force or cmds or _stale(LIB, objs):
        links.append([nv] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lpthread"])
    if force or _stale(DEBUG_LIB, [debug_obj]):
        links.append([nv] + ARCH + ["-shared", "-o", str(DEBUG_LIB), str(debug_obj)])
    _run_all(links)
    main_src = CSRC / "deac_main.cpp"
    if force or _stale(EXE, [main_src, LIB, REPO / "include" / "deac_gb300.h"]):
        _run_all([["g++", "-O2", "-std=c++17", "-Wall"] + inc + [str(main_src), "-o", str(EXE),
                   "-L", str(LIB.parent), "-ldeac_gb300", "-Wl,-rpath,$ORIGIN/../lib"]])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
    print(EXE)
