"""In-tree build of the native parts (no cmake, no pip install).

  lib/libgpuothello2.so  CUDA kernels + C ABI (include/gpuothello2.h), sm_103a
  bin/solver             C++ CLI `solver INPUT OUTPUT DEPTH` over the C ABI
  bin/gen_boards         C++ board-file generator over the C ABI
  bin/diff_results       C++ result-file differ keyed by board (host only)
  oracle/lib/liboracle.so  CPU oracle (test infrastructure, not the product)
  oracle/lib/libthink_host.so, libbatched_emu.so  csrc/think.cuh and batched.cu
                         compiled for the CPU (built on demand by the tests)
  oracle/_ref/refsolve, refthink  the reference's own search and think mode
                         built for the CPU, only where the reference sources
                         are present (x86-64)

Translation units are compiled in parallel; a unit is rebuilt only when a
source it depends on (same directory headers included) is newer.
"""
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG, "lib")
BIN_DIR = os.path.join(PKG, "bin")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libgpuothello2.so")
SOLVER_BIN = os.path.join(BIN_DIR, "solver")
GEN_BIN = os.path.join(BIN_DIR, "gen_boards")
DIFF_BIN = os.path.join(BIN_DIR, "diff_results")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "lib", "liboracle.so")
# test infrastructure, built on demand by the CPU tests: csrc/think.cuh
# compiled for the host, and batched.cu under the SIMT emulation
THINK_HOST_LIB = os.path.join(ORACLE_DIR, "lib", "libthink_host.so")
BATCHED_EMU_LIB = os.path.join(ORACLE_DIR, "lib", "libbatched_emu.so")
REF_BIN = os.path.join(ORACLE_DIR, "_ref", "refsolve")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]

CU_SOURCES = ["plain.cu", "batched.cu", "prep.cu", "capi.cu", "noalloc.cu", "mlp.cu", "think.cu"]
INTPEAK_LIB = os.path.join(LIB_DIR, "libgpo_intpeak.so")


def _headers(d):
    return [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cuh", ".h"))]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd, log=None):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("build step failed: %s" % os.path.basename(cmd[-1]))
    if log is not None:
        log.append(r.stderr)
    return r


def build_library(verbose=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    hdrs = _headers(CSRC) + [os.path.join(INCLUDE, "gpuothello2.h")]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs + [__file__]):
            jobs.append([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with ThreadPoolExecutor(len(jobs)) as ex:
            list(ex.map(lambda c: _run(c, logs), jobs))
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    src = os.path.join(CSRC, "intpeak.cu")
    if _stale(INTPEAK_LIB, [src, __file__]):
        _run([NVCC] + NVCC_FLAGS + ["-shared", src, "-o", INTPEAK_LIB])
    if verbose:
        for lg in logs:
            sys.stderr.write(lg)
    return LIB


def build_host():
    os.makedirs(BIN_DIR, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    common = [os.path.join(HOST, "boardfile.cpp")]
    deps = common + _headers(HOST) + [os.path.join(INCLUDE, "gpuothello2.h"), LIB]
    flags = ["-std=c++17", "-O2", "-Wall", "-I", INCLUDE, "-I", HOST]
    link = ["-L", LIB_DIR, "-lgpuothello2", "-Wl,-rpath,$ORIGIN/../lib", "-pthread"]
    jobs = []
    for main, out in (("solver_main.cpp", SOLVER_BIN), ("gen_main.cpp", GEN_BIN)):
        src = os.path.join(HOST, main)
        if _stale(out, [src] + deps):
            jobs.append([cxx] + flags + [src] + common + ["-o", out] + link)
    # the result differ is host code only (no GPU library)
    src = os.path.join(HOST, "diff_main.cpp")
    if _stale(DIFF_BIN, [src] + common + _headers(HOST)):
        jobs.append([cxx] + flags + [src] + common + ["-o", DIFF_BIN])
    if jobs:
        with ThreadPoolExecutor(len(jobs)) as ex:
            list(ex.map(_run, jobs))
    return SOLVER_BIN


def build_oracle():
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(ORACLE_DIR, "oracle.c")
    if _stale(ORACLE_LIB, [src, os.path.join(ORACLE_DIR, "oracle.h")]):
        _run(["gcc", "-O2", "-std=c11", "-Wall", "-shared", "-fPIC", "-pthread", src, "-o",
              ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_think_host():
    """tests/think_host.cpp: the think-mode search and evaluator header
    compiled for the CPU, for tests only."""
    os.makedirs(os.path.dirname(THINK_HOST_LIB), exist_ok=True)
    src = os.path.join(ROOT, "tests", "think_host.cpp")
    deps = [src, os.path.join(CSRC, "think.cuh"), os.path.join(CSRC, "evalfile.h"),
            os.path.join(ROOT, "include", "gpuothello2.h")]
    if _stale(THINK_HOST_LIB, deps):
        _run(["g++", "-std=c++17", "-O2", "-Wall", "-shared", "-fPIC", src, "-o",
              THINK_HOST_LIB])
    return THINK_HOST_LIB


_LAUNCH = re.compile(r"(\w+)<<<(.*?)>>>\(")


def _emu_sources():
    """Copies of the kernel files with their <<<...>>> launches rewritten to
    simt_launch(kernel, simt_cfg(...), args), in oracle/lib/emu/."""
    emu_dir = os.path.join(ORACLE_DIR, "lib", "emu")
    os.makedirs(emu_dir, exist_ok=True)
    for name in ("batched.cu", "prep.cu", "plain.cu"):
        src = os.path.join(CSRC, name)
        dst = os.path.join(emu_dir, name.replace(".cu", "_emu.cu"))
        text = _LAUNCH.sub(r"simt_launch(\1, simt_cfg(\2), ", open(src).read())
        text = text.replace('#include "', '#include "%s/' % CSRC)
        if not os.path.exists(dst) or open(dst).read() != text:
            with open(dst, "w") as f:
                f.write(text)
    return emu_dir


def build_batched_emu():
    """tests/batched_emu.cpp: the batched search kernel's source run on CPU
    threads (tests/simt/simt_prelude.h), for tests only."""
    os.makedirs(os.path.dirname(BATCHED_EMU_LIB), exist_ok=True)
    emu_dir = _emu_sources()
    src = os.path.join(ROOT, "tests", "batched_emu.cpp")
    simt = os.path.join(ROOT, "tests", "simt")
    deps = [src, os.path.join(simt, "simt_prelude.h"), os.path.join(simt, "cuda_runtime.h")]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    if _stale(BATCHED_EMU_LIB, deps):
        _run(["g++", "-std=c++20", "-O2", "-pthread", "-shared", "-fPIC", "-include",
              os.path.join(simt, "simt_prelude.h"), "-I", simt, "-I", emu_dir, src, "-o",
              BATCHED_EMU_LIB])
    return BATCHED_EMU_LIB


PIPELINE_EMU_LIB = os.path.join(ORACLE_DIR, "lib", "libpipeline_emu.so")


def build_pipeline_emu():
    """tests/pipeline_emu.cpp: the C-ABI layer and every solve kernel run on
    CPU threads (tests only), from the rewritten copies of _emu_sources."""
    emu_dir = _emu_sources()
    src = os.path.join(ROOT, "tests", "pipeline_emu.cpp")
    simt = os.path.join(ROOT, "tests", "simt")
    deps = [src, os.path.join(simt, "simt_prelude.h"), os.path.join(simt, "cuda_runtime.h"),
            os.path.join(ROOT, "include", "gpuothello2.h")]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    if _stale(PIPELINE_EMU_LIB, deps):
        _run(["g++", "-std=c++20", "-O2", "-pthread", "-shared", "-fPIC", "-include",
              os.path.join(simt, "simt_prelude.h"), "-I", simt, "-I", emu_dir, "-I", CSRC, src,
              "-o", PIPELINE_EMU_LIB])
    return PIPELINE_EMU_LIB


def build_reference():
    """The reference's search compiled for the CPU (oracle/ref_build.sh);
    a no-op where the reference sources or an x86-64 host are absent."""
    script = os.path.join(ORACLE_DIR, "ref_build.sh")
    subprocess.run(["bash", script], check=True, capture_output=True)
    return REF_BIN if os.path.exists(REF_BIN) else None


def build_all(verbose=False):
    with ThreadPoolExecutor(3) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference)
        f_lib.result()
        f_orc.result()
        f_ref.result()
    build_host()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
