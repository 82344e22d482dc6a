"""Reference-kernel harness (baseline measurement only): the reference MaBoSSG's own device kernels,
compiled unmodified from its sources (build_kernels.sh, run where the reference checkout is), driven
by refgpu.cu, a restatement of the reference's host path. Nothing in upmabossg_gb300 imports this.

    python -m baseline.refgpu <workload> [n_traj]   # times the reference kernels, prints JSON
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
FATBINS = os.path.join(ROOT, "baseline", "_ref")
LIB = os.path.join(ROOT, "baseline", "_ref", "librefgpu.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def kernels_present() -> bool:
    return all(os.path.exists(os.path.join(FATBINS, f + ".fatbin"))
               for f in ("simulation", "final_states", "window_average_small"))


def build(verbose=False) -> str:
    """Compiles the harness (the reference's CUB/thrust host path restated, for sm_103 as the
    reference's build targets a GB300) against the product's parser sources."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    host = os.path.join(ROOT, "upmabossg_gb300", "csrc", "host")
    cmd = [os.path.join(CUDA, "bin", "nvcc"), "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           "-gencode", "arch=compute_103,code=sm_103", "-o", LIB + ".tmp", os.path.join(HERE, "refgpu.cu"),
           os.path.join(host, "parser.cpp"), os.path.join(host, "model.cpp"),
           f"-L{os.path.join(CUDA, 'lib64')}", "-lnvrtc", "-lnvJitLink",
           "-Xlinker", f"-rpath={os.path.join(CUDA, 'lib64')}"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.rg_run.restype = ctypes.c_void_p
        L.rg_run.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_char_p,
                             ctypes.c_size_t]
        L.rg_free.argtypes = [ctypes.c_void_p]
        L.rg_link_check.restype = ctypes.c_size_t
        L.rg_link_check.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.rg_dims.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_times.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_windows.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.rg_final.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.rg_fixed_count.restype = ctypes.c_size_t
        L.rg_fixed_count.argtypes = [ctypes.c_void_p]
        L.rg_fixed.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefResult:
    """One run of the reference kernels: timings, transitions, window sums (windows x 2^outputs),
    TH sums, final-state counts, fixed points (reference order) and their counts."""

    def __init__(self, h):
        L = lib()
        d = np.zeros(6, np.int32)
        L.rg_dims(h, _p(d))
        self.n, self.words, self.outputs, self.windows, self.discrete, self.iterations = (int(x) for x in d)
        t = np.zeros(5, np.float64)
        L.rg_times(h, _p(t))
        self.sim_ms, self.compile_ms, self.count_ms = float(t[0]), float(t[1]), float(t[2])
        self.transitions, self.n_traj = int(t[3]), int(t[4])
        S = 1 << self.outputs
        self.window_sums = np.zeros((self.windows, S), np.float32)
        self.th_sums = np.zeros(self.windows, np.float32)
        L.rg_windows(h, _p(self.window_sums), _p(self.th_sums))
        self.final_counts = np.zeros(S, np.int32)
        L.rg_final(h, _p(self.final_counts))
        nf = L.rg_fixed_count(h)
        self.fixed_states = np.zeros((nf, self.words), np.uint32)
        self.fixed_counts = np.zeros(nf, np.int32)
        if nf:
            L.rg_fixed(h, _p(self.fixed_states), _p(self.fixed_counts))


def link_check(bnd: str, cfg: str) -> int:
    """Generates the model's rate source in the reference's layout and links it with the reference
    kernels (NVRTC + nvJitLink, no GPU): the linked cubin's size."""
    err = ctypes.create_string_buffer(4096)
    n = lib().rg_link_check(bnd.encode(), cfg.encode(), FATBINS.encode(), err, 4096)
    if not n:
        raise RuntimeError("reference kernels: " + err.value.decode())
    return int(n)


def run(bnd: str, cfg: str, n_traj: int = 0) -> RefResult:
    if not kernels_present():
        raise FileNotFoundError("reference kernels not built: sh baseline/refgpu/build_kernels.sh <reference checkout>")
    err = ctypes.create_string_buffer(4096)
    h = lib().rg_run(bnd.encode(), cfg.encode(), FATBINS.encode(), n_traj, err, 4096)
    if not h:
        raise RuntimeError("reference kernels: " + err.value.decode())
    try:
        return RefResult(h)
    finally:
        lib().rg_free(h)
