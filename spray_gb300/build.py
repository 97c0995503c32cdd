"""Builds libspray_gpu.so in-tree: CUDA sources for sm_103a with nvcc, host
sources with g++, compiled in parallel and linked against the static CUDA
runtime.  Floating-point contraction is disabled on both compilers so host
and device produce the same bits for the shared scalar code."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libspray_gpu.so"
FILM = PKG / "spray_gpu_film"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["sched.cu", "trace.cu", "shade.cu", "tracer.cu", "insitu.cu", "bvh_build.cu", "noalloc.cu",
              "rounds.cu", "mlp.cu", "mlp_api.cu"]
CPP_SOURCES = ["bvh.cpp", "host_scene.cpp", "host_api.cpp"]

CXXFLAGS = ["-O2", "-fPIC", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-Wall",
            "-Wno-unused-function"]
NVCCFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                    "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off"]


def _needs(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


EXTRA_DEFINES = [d for d in os.environ.get("SPRAY_BUILD_DEFINES", "").split() if d]


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every translation unit that changed and link the library.

    SPRAY_BUILD_DEFINES (space-separated -D flags) sets tuning constants."""
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "spray_gpu.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _needs(o, [s] + headers):
            jobs.append([NVCC] + NVCCFLAGS + EXTRA_DEFINES + ["-c", str(s), "-o", str(o)])
    for src in CPP_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _needs(o, [s] + headers):
            jobs.append(["g++"] + CXXFLAGS + EXTRA_DEFINES + ["-c", str(s), "-o", str(o)])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(" ".join(j) + "\n" + (out or ""))
        if p.returncode != 0:
            failed.append(j[-3] if len(j) > 3 else str(j))
    if failed:
        raise RuntimeError("compilation failed: " + ", ".join(failed))
    if force or jobs or not LIB.exists() or _needs(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = ["g++", "-shared", "-o", str(tmp)] + [str(o) for o in objs] + [
            "-L" + str(CUDA_HOME / "lib64"), "-lcudart_static", "-lrt", "-ldl", "-lpthread", "-fopenmp"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout)
        os.replace(tmp, LIB)
    film_src = CSRC / "film_main.cpp"
    if force or not FILM.exists() or _needs(FILM, [film_src, LIB]):
        # no contraction here either: the default camera's distance is an a*b + c
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(FILM), str(film_src), "-L" + str(PKG),
               "-lspray_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("film app link failed:\n" + r.stdout)
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    if LIB.exists():
        LIB.unlink()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
