"""Build the native parts in-tree with nvcc/g++ (no cmake).

Products:
  libfluid_gb300/libsph_gb300.so  - the C ABI (include/sph_c.h) + sm_103a kernels
  libfluid_gb300/libfluid.so      - C++ FluidSystem drop-in (include/fluidsystem.h)
  libfluid_gb300/bin/fluidtest    - fluidtest-equivalent driver (.geo export)
  oracle/liboracle.so             - CPU oracle (test infrastructure only)

Every device compile targets sm_103a only:
  -gencode arch=compute_103a,code=sm_103a -lineinfo
Host code is compiled with -ffp-contract=off so that float results do not
depend on the host architecture's fused multiply-add.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
INCLUDE = os.path.join(ROOT, "include")


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


CUDA = _cuda_home()
NVCC = os.path.join(CUDA, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                        "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}", f"-I{CSRC}",
             f"-I{os.path.join(CUDA, 'include')}"]

KERNEL_SOURCES = ["sph_kernels.cu", "sph_noalloc.cu"]
HOST_SOURCES = ["engine.cpp", "capi.cpp", "capi_batch.cpp", "server.cpp", "geo.cpp"]

LIB_SPH = os.path.join(PKG, "libsph_gb300.so")
LIB_FLUID = os.path.join(PKG, "libfluid.so")
LIB_ORACLE = os.path.join(ROOT, "oracle", "liboracle.so")
BIN_DIR = os.path.join(PKG, "bin")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                hs.append(os.path.join(d, f))
    return hs


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _compile(src: str, obj: str) -> str:
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = [CXX] + CXX_FLAGS + ["-c", src, "-o", obj]
    _run(cmd)
    return obj


def build(force: bool = False, verbose: bool = False) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN_DIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for name in KERNEL_SOURCES + HOST_SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + hdrs):
            jobs.append((src, obj))
    oracle_src = os.path.join(ROOT, "oracle", "oracle.cpp")
    need_oracle = force or not _newer(LIB_ORACLE, [oracle_src])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        futs = [ex.submit(_compile, s, o) for s, o in jobs]
        if need_oracle:
            futs.append(ex.submit(_run, [CXX, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
                                         "-shared", "-Wall", oracle_src, "-o", LIB_ORACLE]))
        for f in futs:
            f.result()
    if force or jobs or not os.path.exists(LIB_SPH):
        _run([NVCC] + GENCODE + ["-shared", "-o", LIB_SPH] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    # C++ FluidSystem drop-in over the C ABI
    fs_src = os.path.join(CSRC, "fluidsystem.cpp")
    if os.path.exists(fs_src) and (force or not _newer(LIB_FLUID, [fs_src, LIB_SPH] + hdrs)):
        _run([CXX] + CXX_FLAGS + ["-shared", fs_src, "-o", LIB_FLUID, f"-L{PKG}", "-lsph_gb300",
                                  "-Wl,-rpath,$ORIGIN"])
    drv_src = os.path.join(CSRC, "fluidtest_main.cpp")
    drv = os.path.join(BIN_DIR, "fluidtest")
    if os.path.exists(drv_src) and (force or not _newer(drv, [drv_src, LIB_FLUID] + hdrs)):
        _run([CXX] + CXX_FLAGS + [drv_src, "-o", drv, f"-L{PKG}", "-lfluid", "-lsph_gb300",
                                  "-Wl,-rpath,$ORIGIN/.."])
    build_reference_runner(force=force)
    if verbose:
        print(f"built {LIB_SPH}, {LIB_ORACLE}")
    return {"sph": LIB_SPH, "fluid": LIB_FLUID, "oracle": LIB_ORACLE}


REF_DIR = os.path.join(ROOT, "oracle", "_ref")
REF_CUBIN = os.path.join(REF_DIR, "libfluid_ref.cubin")
REF_RUNNER = os.path.join(REF_DIR, "ref_runner")


def build_reference_runner(force: bool = False) -> bool:
    """Oracle pins: the reference's own device code as a cubin (built only
    where the reference tree is present, by oracle/ref_build.sh) and the host
    runner that drives it (oracle/ref_runner.cu, built wherever the cubin
    is).  Test infrastructure; returns False when the cubin is unavailable."""
    script = os.path.join(ROOT, "oracle", "ref_build.sh")
    deps = [os.path.join(ROOT, "oracle", "ref_unity.cu"), os.path.join(ROOT, "oracle", "ref_compat", "helper_math.h"),
            script]
    if force or not _newer(REF_CUBIN, deps):
        r = subprocess.run(["bash", script], capture_output=True, text=True)
        if r.returncode not in (0, 2):
            raise RuntimeError("reference device build failed:\n" + r.stdout + r.stderr)
    if not os.path.exists(REF_CUBIN):
        return False
    src = os.path.join(ROOT, "oracle", "ref_runner.cu")
    if force or not _newer(REF_RUNNER, [src]):
        _run([NVCC, "-O2", "-std=c++17"] + GENCODE + [src, "-o", REF_RUNNER,
                                                      f"-L{os.path.join(CUDA, 'lib64', 'stubs')}", "-lcuda"])
    return True


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
