"""Build recipe for libmbg.so and the MaBoSSG command line (no cmake).

Host C++ is compiled with g++, the ahead-of-time kernels with nvcc for sm_103a only, all in
parallel; the shared library links the CUDA runtime statically and NVRTC dynamically, so it loads
on a machine without a GPU driver (calls then return MBG_ERR_CUDA). The device headers the NVRTC
program needs are embedded into the library as string literals.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
GEN = os.path.join(CSRC, "_gen")
LIB = os.path.join(PKG, "lib", "libmbg.so")
CLI = os.path.join(PKG, "bin", "MaBoSSG")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["parser.cpp", "model.cpp", "codegen.cpp", "jit.cpp", "sim.cpp", "batch.cpp", "surrogate.cpp",
                "output.cpp", "capi.cpp", "devmem.cpp"]
DEVICE_SOURCES = ["sim_aot.cu", "sim_aot_hash.cu", "window_table.cu", "noalloc.cu", "mlp.cu", "mlp_tc.cu",
                  "mlp_train.cu"]
JIT_HEADERS = ["sim_types.h", "philox.h", "sim_core.cuh", "sim_thread.cuh"]


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def embed_jit_headers():
    os.makedirs(GEN, exist_ok=True)
    parts = []
    for h in JIT_HEADERS:
        with open(os.path.join(CSRC, "device", h)) as f:
            text = f.read()
        if ")MBGSRC\"" in text:
            raise RuntimeError(f"{h} contains the raw-string delimiter")
        parts.append(f'R"MBGSRC(\n// ---- {h}\n{text}\n)MBGSRC"')
    body = ("// generated by upmabossg_gb300/build.py from csrc/device headers; do not edit\n"
            f"static const char* const kJitHeaders[] = {{\n" + ",\n".join(parts) + "\n};\n"
            f"static const int kJitHeaderCount = {len(parts)};\n")
    out = os.path.join(GEN, "jit_src.inc")
    old = open(out).read() if os.path.exists(out) else None
    if old != body:
        with open(out, "w") as f:
            f.write(body)


def build(verbose: bool = False, jobs: int = 0) -> str:
    embed_jit_headers()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    cuda_inc = os.path.join(CUDA, "include")
    jobs_list = []
    objs = []
    for src in HOST_SOURCES:
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        jobs_list.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                          f"-I{cuda_inc}", f"-I{INCLUDE}", "-c", os.path.join(CSRC, "host", src), "-o", o])
    for src in DEVICE_SOURCES:
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        jobs_list.append([NVCC] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                                          "-Xptxas", "-v", f"-I{INCLUDE}", "-c",
                                          os.path.join(CSRC, "device", src), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(lambda c: _run(c, verbose), jobs_list))
    ptxas = [l for log in logs for l in log.splitlines() if "registers" in l or "spill" in l]
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs +
         [f"-L{os.path.join(CUDA, 'lib64')}", "-lnvrtc", "-Xlinker", f"-rpath={os.path.join(CUDA, 'lib64')}"],
         verbose)
    os.replace(tmp, LIB)
    _run(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", os.path.join(CSRC, "cli", "main.cpp"), "-o", CLI + ".tmp",
          f"-L{os.path.dirname(LIB)}", "-lmbg", "-Wl,-rpath,$ORIGIN/../lib"], verbose)
    os.replace(CLI + ".tmp", CLI)
    if verbose:
        print("\n".join(ptxas))
    return LIB


def clean():
    for p in (OBJ, GEN, os.path.dirname(LIB), os.path.dirname(CLI)):
        shutil.rmtree(p, ignore_errors=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
