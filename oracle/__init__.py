"""ctypes binding of the host FP64 oracle: TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module. The
product (``upmabossg_gb300``) never imports or links it, and it shares no code with the product:
the oracle library is built by ``build()`` from oracle.cpp and its own front end (front.h: parser,
expression evaluation, Philox streams, fixed-point rules).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.cpp")]


def build(verbose: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", LIB] + SOURCES
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return LIB


class _Opts(ctypes.Structure):
    _fields_ = [
        ("n_traj", ctypes.c_uint64),
        ("traj_base", ctypes.c_uint64),
        ("seed", ctypes.c_uint64),
        ("use_cfg_seed", ctypes.c_int),
        ("frac_bits", ctypes.c_int),
        ("threads", ctypes.c_int),
        ("max_steps", ctypes.c_uint32),
        ("keep_trajectories", ctypes.c_int),
        ("redraw_period", ctypes.c_uint32),
        ("legacy_final", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_run.restype = ctypes.c_void_p
        L.orc_run.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_Opts), ctypes.c_char_p,
                              ctypes.c_size_t]
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_dims.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 4
        L.orc_counters.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_hist_nnz.restype = ctypes.c_size_t
        L.orc_hist_nnz.argtypes = [ctypes.c_void_p]
        L.orc_hist_get.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_th.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_final.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_trajectories.argtypes = [ctypes.c_void_p] * 6
        L.orc_seconds.restype = ctypes.c_double
        L.orc_seconds.argtypes = [ctypes.c_void_p]
        L.orc_threads.restype = ctypes.c_int
        L.orc_threads.argtypes = [ctypes.c_void_p]
        L.orc_philox.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class OracleResult:
    """Results of one oracle run, copied into numpy arrays."""

    COUNTERS = ("transitions", "finished", "fixed", "step_limit", "pick_ties", "time_ties", "steps")

    def __init__(self, handle, n_traj, keep):
        L = lib()
        n, w, no, k = (ctypes.c_int() for _ in range(4))
        L.orc_dims(handle, ctypes.byref(n), ctypes.byref(w), ctypes.byref(no), ctypes.byref(k))
        self.n, self.words, self.n_out, self.windows = n.value, w.value, no.value, k.value
        self.n_traj = n_traj
        c = np.zeros(7, np.uint64)
        L.orc_counters(handle, _ptr(c))
        self.counters = {name: int(v) for name, v in zip(self.COUNTERS, c)}
        nnz = L.orc_hist_nnz(handle)
        self.hist_window = np.zeros(nnz, np.uint32)
        self.hist_state = np.zeros(nnz, np.uint32)
        self.hist_value = np.zeros(nnz, np.float64)
        if nnz:
            L.orc_hist_get(handle, _ptr(self.hist_window), _ptr(self.hist_state), _ptr(self.hist_value))
        self.th = np.zeros(self.windows, np.float64)
        L.orc_th(handle, _ptr(self.th))
        self.final = np.zeros(1 << self.n_out, np.float64)
        L.orc_final(handle, _ptr(self.final))
        self.seconds = L.orc_seconds(handle)
        self.threads = L.orc_threads(handle)
        if keep:
            self.states = np.zeros((n_traj, self.words), np.uint32)
            self.times = np.zeros(n_traj, np.float64)
            self.transitions = np.zeros(n_traj, np.uint32)
            self.status = np.zeros(n_traj, np.uint8)
            self.ties = np.zeros(n_traj, np.uint8)
            L.orc_trajectories(handle, _ptr(self.states), _ptr(self.times), _ptr(self.transitions),
                               _ptr(self.status), _ptr(self.ties))

    def dense_hist(self):
        """windows x 2^n_out array of time sums (continuous) or counts (discrete)."""
        h = np.zeros((self.windows, 1 << self.n_out), np.float64)
        h[self.hist_window, self.hist_state] = self.hist_value
        return h


def run(bnd: str, cfg: str, *, frac_bits: int = 0, n_traj: int = 0, seed=None, traj_base: int = 0,
        threads: int = 0, max_steps: int = 0, keep_trajectories: bool = False,
        legacy_final: bool = False, redraw_period: int = 0) -> OracleResult:
    L = lib()
    o = _Opts()
    o.n_traj = n_traj
    o.traj_base = traj_base
    o.seed = 0 if seed is None else int(seed)
    o.use_cfg_seed = 1 if seed is None else 0
    o.frac_bits = frac_bits
    o.threads = threads
    o.max_steps = max_steps
    o.keep_trajectories = 1 if keep_trajectories else 0
    o.legacy_final = 1 if legacy_final else 0
    o.redraw_period = redraw_period
    err = ctypes.create_string_buffer(1024)
    h = L.orc_run(bnd.encode(), cfg.encode(), ctypes.byref(o), err, 1024)
    if not h:
        raise RuntimeError("oracle: " + err.value.decode())
    try:
        if n_traj == 0:
            n, w, no, k = (ctypes.c_int() for _ in range(4))
            c = np.zeros(7, np.uint64)
            L.orc_counters(h, _ptr(c))
            n_traj = int(c[1] + c[2] + c[3])
        return OracleResult(h, n_traj, keep_trajectories)
    finally:
        L.orc_free(h)


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    lib().orc_philox(_ptr(c), _ptr(k), _ptr(out))
    return out
