"""GB300-native MaBoSS-style Boolean network simulator (ctypes binding of libmbg.so).

The product is the C ABI in include/mbg.h (libmbg.so) and the ``MaBoSSG`` command line; this
module is a thin Python binding used by the tests and the benchmark. It loads the in-tree
library and fails loudly if it has not been built: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libmbg.so")
CLI_PATH = os.path.join(PKG, "bin", "MaBoSSG")

LAYOUT_AUTO, LAYOUT_THREAD, LAYOUT_WARP = 0, 1, 2
STATUS = {0: "OK", 1: "ARG", 2: "IO", 3: "PARSE", 4: "MODEL", 5: "CUDA", 6: "JIT", 7: "NOMEM", 8: "DEVICE",
          9: "STATE"}

# Every symbol include/mbg.h declares.
EXPORTS = (
    "mbg_last_error", "mbg_version", "mbg_device_count", "mbg_model_parse_files", "mbg_model_parse_strings",
    "mbg_model_destroy", "mbg_model_info_get", "mbg_model_node_name", "mbg_model_outputs", "mbg_model_rate",
    "mbg_model_jit_check",
    "mbg_sim_opts_default", "mbg_sim_create", "mbg_sim_destroy", "mbg_sim_run", "mbg_sim_summary",
    "mbg_sim_probtraj", "mbg_sim_probtraj_raw", "mbg_sim_final_states", "mbg_sim_fixed_points",
    "mbg_sim_trajectories", "mbg_write_probtraj_csv", "mbg_write_fp_csv", "mbg_print_results",
    "mbg_fixed_points_aggregate_noalloc",
)


class MbgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


class ModelInfo(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_int32), ("words", ctypes.c_int32), ("outputs", ctypes.c_int32),
                ("windows", ctypes.c_int32), ("discrete_time", ctypes.c_int32), ("frac_bits", ctypes.c_int32),
                ("max_regulators", ctypes.c_int32), ("palette_nodes", ctypes.c_int32),
                ("max_time", ctypes.c_double), ("time_tick", ctypes.c_double),
                ("sample_count", ctypes.c_uint64), ("seed", ctypes.c_uint64)]


class SimOpts(ctypes.Structure):
    _fields_ = [("n_traj", ctypes.c_uint64), ("traj_base", ctypes.c_uint64), ("seed", ctypes.c_uint64),
                ("use_cfg_seed", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("record_trajectories", ctypes.c_int32), ("device", ctypes.c_int32),
                ("max_steps", ctypes.c_uint32), ("block_size", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("thread_cutoff", ctypes.c_int32)]


class RunSummary(ctypes.Structure):
    _fields_ = [("trajectories", ctypes.c_uint64), ("transitions", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("finished", ctypes.c_uint64), ("fixed_points", ctypes.c_uint64),
                ("step_limited", ctypes.c_uint64), ("errors", ctypes.c_uint64),
                ("fixed_point_states", ctypes.c_uint64), ("device_error", ctypes.c_uint32),
                ("layout", ctypes.c_int32), ("sim_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("jit_ms", ctypes.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None


def lib():
    """The loaded libmbg.so; raises if the library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MbgError(5, f"{LIB_PATH} is missing: run upmabossg_gb300/build.py (or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, u64, dp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p
        sig = {
            "mbg_last_error": (ctypes.c_char_p, []),
            "mbg_version": (ctypes.c_char_p, []),
            "mbg_device_count": (ctypes.c_int, []),
            "mbg_model_parse_files": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp)]),
            "mbg_model_parse_strings": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp)]),
            "mbg_model_destroy": (None, [vp]),
            "mbg_model_info_get": (ctypes.c_int, [vp, ctypes.POINTER(ModelInfo)]),
            "mbg_model_node_name": (ctypes.c_char_p, [vp, i32]),
            "mbg_model_outputs": (i32, [vp, dp, i32]),
            "mbg_model_rate": (ctypes.c_int, [vp, i32, dp, ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_double)]),
            "mbg_model_jit_check": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
            "mbg_sim_opts_default": (None, [ctypes.POINTER(SimOpts)]),
            "mbg_sim_create": (ctypes.c_int, [vp, ctypes.POINTER(SimOpts), ctypes.POINTER(vp)]),
            "mbg_sim_destroy": (None, [vp]),
            "mbg_sim_run": (ctypes.c_int, [vp, vp]),
            "mbg_sim_summary": (ctypes.c_int, [vp, ctypes.POINTER(RunSummary)]),
            "mbg_sim_probtraj": (ctypes.c_int, [vp, dp, dp]),
            "mbg_sim_probtraj_raw": (ctypes.c_int, [vp, dp, dp]),
            "mbg_sim_final_states": (ctypes.c_int, [vp, dp]),
            "mbg_sim_fixed_points": (ctypes.c_int, [vp, dp, dp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
            "mbg_sim_trajectories": (ctypes.c_int, [vp, dp, dp, dp, dp]),
            "mbg_write_probtraj_csv": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_write_fp_csv": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_print_results": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_fixed_points_aggregate_noalloc": (ctypes.c_int, [vp, ctypes.c_uint32, i32, vp, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(st):
    if st != 0:
        raise MbgError(st, lib().mbg_last_error().decode(errors="replace"))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def device_count() -> int:
    return lib().mbg_device_count()


class Model:
    """A parsed and compiled .bnd/.cfg model (driver::parse of the reference)."""

    def __init__(self, handle):
        self._h = handle
        info = ModelInfo()
        _check(lib().mbg_model_info_get(self._h, ctypes.byref(info)))
        self.info = info
        L = lib()
        self.names = [L.mbg_model_node_name(self._h, i).decode() for i in range(info.nodes)]
        out = np.zeros(max(1, info.outputs), np.int32)
        L.mbg_model_outputs(self._h, _p(out), info.outputs)
        self.outputs = [int(x) for x in out[:info.outputs]]

    @classmethod
    def from_files(cls, bnd_path, cfg_path):
        h = ctypes.c_void_p()
        _check(lib().mbg_model_parse_files(os.fsencode(bnd_path), os.fsencode(cfg_path), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_strings(cls, bnd, cfg):
        h = ctypes.c_void_p()
        _check(lib().mbg_model_parse_strings(bnd.encode(), cfg.encode(), ctypes.byref(h)))
        return cls(h)

    def rate(self, node: int, state) -> tuple:
        """(fixed-point rate, real rate) of `node` in the full state (sequence of 0/1 per node)."""
        st = np.ascontiguousarray(np.asarray(state, dtype=np.uint8))
        if st.size != self.info.nodes:
            raise ValueError("state needs one entry per node")
        q = ctypes.c_uint64()
        r = ctypes.c_double()
        _check(lib().mbg_model_rate(self._h, int(node), _p(st), ctypes.byref(q), ctypes.byref(r)))
        return q.value, r.value

    def jit_check(self) -> float:
        ms = ctypes.c_double()
        _check(lib().mbg_model_jit_check(self._h, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if self._h:
            lib().mbg_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """One simulation handle: trajectories, seed, layout; results after run()."""

    def __init__(self, model: Model, n_traj=0, seed=None, layout=LAYOUT_AUTO, record_trajectories=False,
                 max_steps=0, traj_base=0, device=0, block_size=0, blocks_per_sm=0, thread_cutoff=0):
        o = SimOpts()
        lib().mbg_sim_opts_default(ctypes.byref(o))
        o.n_traj = int(n_traj)
        o.traj_base = int(traj_base)
        if seed is not None:
            o.seed = int(seed)
            o.use_cfg_seed = 0
        o.layout = layout
        o.record_trajectories = 1 if record_trajectories else 0
        o.max_steps = int(max_steps)
        o.device = device
        o.block_size = block_size
        o.blocks_per_sm = blocks_per_sm
        o.thread_cutoff = thread_cutoff
        self.model = model
        h = ctypes.c_void_p()
        _check(lib().mbg_sim_create(model._h, ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self.n_traj = int(n_traj) or int(model.info.sample_count)

    def run(self, stream=None):
        _check(lib().mbg_sim_run(self._h, ctypes.c_void_p(stream) if stream else None))
        return self

    def summary(self) -> dict:
        s = RunSummary()
        _check(lib().mbg_sim_summary(self._h, ctypes.byref(s)))
        return s.as_dict()

    def probtraj(self):
        info = self.model.info
        P = np.zeros((info.windows, 1 << info.outputs), np.float64)
        TH = np.zeros(info.windows, np.float64)
        _check(lib().mbg_sim_probtraj(self._h, _p(P), _p(TH)))
        return P, TH

    def probtraj_raw(self):
        info = self.model.info
        P = np.zeros((info.windows, 1 << info.outputs), np.uint64)
        TH = np.zeros(info.windows, np.uint64)
        _check(lib().mbg_sim_probtraj_raw(self._h, _p(P), _p(TH)))
        return P, TH

    def final_states(self):
        F = np.zeros(1 << self.model.info.outputs, np.float64)
        _check(lib().mbg_sim_final_states(self._h, _p(F)))
        return F

    def fixed_points(self):
        n = ctypes.c_size_t()
        _check(lib().mbg_sim_fixed_points(self._h, None, None, 0, ctypes.byref(n)))
        W = self.model.info.words
        states = np.zeros((n.value, W), np.uint32)
        probs = np.zeros(n.value, np.float64)
        if n.value:
            _check(lib().mbg_sim_fixed_points(self._h, _p(states), _p(probs), n.value, ctypes.byref(n)))
        return states, probs

    def trajectories(self):
        W = self.model.info.words
        st = np.zeros((self.n_traj, W), np.uint32)
        t = np.zeros(self.n_traj, np.float64)
        tr = np.zeros(self.n_traj, np.uint32)
        s = np.zeros(self.n_traj, np.uint8)
        _check(lib().mbg_sim_trajectories(self._h, _p(st), _p(t), _p(tr), _p(s)))
        return st, t, tr, s

    def write_csv(self, prefix):
        _check(lib().mbg_write_probtraj_csv(self._h, os.fsencode(prefix)))
        _check(lib().mbg_write_fp_csv(self._h, os.fsencode(prefix)))

    def print_results(self, path="-"):
        _check(lib().mbg_print_results(self._h, os.fsencode(path)))

    def close(self):
        if self._h:
            lib().mbg_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
