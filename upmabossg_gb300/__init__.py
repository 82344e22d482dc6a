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

LAYOUT_AUTO, LAYOUT_THREAD, LAYOUT_WARP, LAYOUT_LANE, LAYOUT_LANE_GLOBAL = 0, 1, 2, 3, 4
STATUS = {0: "OK", 1: "ARG", 2: "IO", 3: "PARSE", 4: "MODEL", 5: "CUDA", 6: "JIT", 7: "NOMEM", 8: "DEVICE",
          9: "STATE"}

# Every symbol include/mbg.h declares.
EXPORTS = (
    "mbg_last_error", "mbg_version", "mbg_device_count", "mbg_model_parse_files", "mbg_model_parse_strings",
    "mbg_model_destroy", "mbg_model_info_get", "mbg_model_node_name", "mbg_model_outputs", "mbg_model_rate",
    "mbg_model_with_rate_scales", "mbg_model_parse_files_overrides", "mbg_model_with_mutations",
    "mbg_model_jit_check", "mbg_model_layout_check", "mbg_model_from_arrays",
    "mbg_sim_opts_default", "mbg_sim_create", "mbg_sim_destroy", "mbg_sim_run", "mbg_sim_summary",
    "mbg_sim_probtraj", "mbg_sim_probtraj_raw", "mbg_sim_probtraj_sparse", "mbg_sim_final_states",
    "mbg_sim_final_states_sparse", "mbg_sim_fixed_points",
    "mbg_sim_trajectories", "mbg_write_probtraj_csv", "mbg_write_fp_csv", "mbg_print_results",
    "mbg_write_final_states_csv", "mbg_fixed_points_aggregate_noalloc",
    "mbg_batch_opts_default", "mbg_batch_create", "mbg_batch_destroy", "mbg_batch_run", "mbg_batch_summary",
    "mbg_batch_instance_summary", "mbg_batch_probtraj", "mbg_batch_probtraj_raw", "mbg_batch_window_probs", "mbg_batch_final_states",
    "mbg_batch_fixed_points", "mbg_batch_class_count", "mbg_batch_class", "mbg_batch_class_timings",
    "mbg_surrogate_create", "mbg_surrogate_destroy", "mbg_surrogate_train", "mbg_surrogate_predict",
    "mbg_surrogate_param_count", "mbg_surrogate_get_params", "mbg_surrogate_set_params", "mbg_surrogate_gradients",
    "mbg_surrogate_set_tensor_path", "mbg_surrogate_time_forward", "mbg_surrogate_predict_column",
    "mbg_device_l2_atomic_rate",
)


class BatchOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_steps", ctypes.c_uint32), ("block_size", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("autotune", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("lane_variant", ctypes.c_int32)]


class BatchClassTiming(ctypes.Structure):
    _fields_ = [("layout", ctypes.c_int32), ("block_size", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("kernel_ms", ctypes.c_double)]


class BatchClassInfo(ctypes.Structure):
    _fields_ = [("max_nodes", ctypes.c_int32), ("instances", ctypes.c_int32), ("trajectories", ctypes.c_uint64),
                ("layout", ctypes.c_int32), ("block_size", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("grid", ctypes.c_int32), ("kernel_ms", ctypes.c_double), ("timings", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


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


class ModelRun(ctypes.Structure):
    _fields_ = [("max_time", ctypes.c_double), ("time_tick", ctypes.c_double), ("sample_count", ctypes.c_uint64),
                ("seed", ctypes.c_uint64), ("discrete_time", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class SimOpts(ctypes.Structure):
    _fields_ = [("n_traj", ctypes.c_uint64), ("traj_base", ctypes.c_uint64), ("seed", ctypes.c_uint64),
                ("use_cfg_seed", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("record_trajectories", ctypes.c_int32), ("device", ctypes.c_int32),
                ("max_steps", ctypes.c_uint32), ("block_size", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("thread_cutoff", ctypes.c_int32),
                ("lane_update", ctypes.c_int32), ("window_table", ctypes.c_int32),
                ("window_hash_bits", ctypes.c_int32), ("redraw_period", ctypes.c_uint32)]


class RunSummary(ctypes.Structure):
    _fields_ = [("trajectories", ctypes.c_uint64), ("transitions", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("finished", ctypes.c_uint64), ("fixed_points", ctypes.c_uint64),
                ("step_limited", ctypes.c_uint64), ("errors", ctypes.c_uint64),
                ("fixed_point_states", ctypes.c_uint64), ("device_error", ctypes.c_uint32),
                ("layout", ctypes.c_int32), ("sim_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("jit_ms", ctypes.c_double), ("block_size", ctypes.c_int32), ("grid_size", ctypes.c_int32),
                ("lane_update", ctypes.c_int32), ("window_table", ctypes.c_int32),
                ("window_hash_bits", ctypes.c_int32), ("window_reruns", ctypes.c_int32),
                ("window_entries", ctypes.c_uint64)]

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
            "mbg_model_from_arrays": (ctypes.c_int, [i32, ctypes.POINTER(ctypes.c_char_p), vp, vp, vp, ctypes.c_int64,
                                                     vp, vp, vp, vp, vp, ctypes.POINTER(ModelRun),
                                                     ctypes.POINTER(vp)]),
            "mbg_model_parse_files_overrides": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                                               ctypes.POINTER(vp)]),
            "mbg_model_with_mutations": (ctypes.c_int, [vp, dp, dp, i32, ctypes.POINTER(vp)]),
            "mbg_model_destroy": (None, [vp]),
            "mbg_model_info_get": (ctypes.c_int, [vp, ctypes.POINTER(ModelInfo)]),
            "mbg_model_node_name": (ctypes.c_char_p, [vp, i32]),
            "mbg_model_outputs": (i32, [vp, dp, i32]),
            "mbg_model_rate": (ctypes.c_int, [vp, i32, dp, ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_double)]),
            "mbg_model_jit_check": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
            "mbg_model_layout_check": (ctypes.c_int, [vp]),
            "mbg_model_with_rate_scales": (ctypes.c_int, [vp, dp, dp, ctypes.POINTER(vp)]),
            "mbg_sim_opts_default": (None, [ctypes.POINTER(SimOpts)]),
            "mbg_sim_create": (ctypes.c_int, [vp, ctypes.POINTER(SimOpts), ctypes.POINTER(vp)]),
            "mbg_sim_destroy": (None, [vp]),
            "mbg_sim_run": (ctypes.c_int, [vp, vp]),
            "mbg_sim_summary": (ctypes.c_int, [vp, ctypes.POINTER(RunSummary)]),
            "mbg_sim_probtraj": (ctypes.c_int, [vp, dp, dp]),
            "mbg_sim_probtraj_raw": (ctypes.c_int, [vp, dp, dp]),
            "mbg_device_l2_atomic_rate": (ctypes.c_int, [i32, ctypes.c_uint32, dp]),
            "mbg_sim_probtraj_sparse": (ctypes.c_int, [vp, dp, dp, dp, ctypes.c_size_t,
                                                        ctypes.POINTER(ctypes.c_size_t)]),
            "mbg_sim_final_states": (ctypes.c_int, [vp, dp]),
            "mbg_sim_final_states_sparse": (ctypes.c_int, [vp, dp, dp, ctypes.c_size_t,
                                                            ctypes.POINTER(ctypes.c_size_t)]),
            "mbg_sim_fixed_points": (ctypes.c_int, [vp, dp, dp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
            "mbg_sim_trajectories": (ctypes.c_int, [vp, dp, dp, dp, dp]),
            "mbg_write_probtraj_csv": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_write_fp_csv": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_write_final_states_csv": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_print_results": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "mbg_fixed_points_aggregate_noalloc": (ctypes.c_int, [vp, ctypes.c_uint32, i32, vp, vp, vp, vp]),
            "mbg_batch_opts_default": (None, [ctypes.POINTER(BatchOpts)]),
            "mbg_batch_create": (ctypes.c_int, [dp, i32, dp, dp, ctypes.POINTER(BatchOpts), ctypes.POINTER(vp)]),
            "mbg_batch_destroy": (None, [vp]),
            "mbg_batch_run": (ctypes.c_int, [vp, vp]),
            "mbg_batch_summary": (ctypes.c_int, [vp, ctypes.POINTER(RunSummary)]),
            "mbg_batch_instance_summary": (ctypes.c_int, [vp, i32, ctypes.POINTER(RunSummary)]),
            "mbg_batch_probtraj": (ctypes.c_int, [vp, i32, dp, dp]),
            "mbg_batch_probtraj_raw": (ctypes.c_int, [vp, i32, dp, dp]),
            "mbg_batch_window_probs": (ctypes.c_int, [vp, i32, dp]),
            "mbg_batch_final_states": (ctypes.c_int, [vp, i32, dp]),
            "mbg_batch_fixed_points": (ctypes.c_int, [vp, i32, dp, dp, ctypes.c_size_t,
                                                      ctypes.POINTER(ctypes.c_size_t)]),
            "mbg_batch_class_count": (ctypes.c_int, [vp, ctypes.POINTER(i32)]),
            "mbg_batch_class": (ctypes.c_int, [vp, i32, ctypes.POINTER(BatchClassInfo)]),
            "mbg_batch_class_timings": (ctypes.c_int, [vp, i32, ctypes.POINTER(BatchClassTiming), i32,
                                                       ctypes.POINTER(i32)]),
            "mbg_surrogate_create": (ctypes.c_int, [i32, i32, i32, i32, i32, u64, i32, ctypes.POINTER(vp)]),
            "mbg_surrogate_destroy": (None, [vp]),
            "mbg_surrogate_train": (ctypes.c_int, [vp, dp, dp, ctypes.c_int64, i32, i32, ctypes.c_float, u64,
                                                   ctypes.POINTER(ctypes.c_float)]),
            "mbg_surrogate_predict": (ctypes.c_int, [vp, dp, ctypes.c_int64, dp, dp]),
            "mbg_surrogate_predict_column": (ctypes.c_int, [vp, dp, ctypes.c_int64, i32, dp, dp]),
            "mbg_surrogate_param_count": (ctypes.c_int64, [vp]),
            "mbg_surrogate_get_params": (ctypes.c_int, [vp, i32, dp]),
            "mbg_surrogate_set_params": (ctypes.c_int, [vp, i32, dp]),
            "mbg_surrogate_gradients": (ctypes.c_int, [vp, i32, dp, dp, i32, ctypes.POINTER(ctypes.c_float), dp]),
            "mbg_surrogate_set_tensor_path": (ctypes.c_int, [vp, i32]),
            "mbg_surrogate_time_forward": (ctypes.c_int, [vp, i32, i32, ctypes.POINTER(ctypes.c_double)]),
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


def l2_atomic_rate(distinct: int, device: int = 0) -> float:
    """Measured u64 atomic adds per second into `distinct` L2-resident addresses."""
    r = ctypes.c_double()
    _check(lib().mbg_device_l2_atomic_rate(device, distinct, ctypes.byref(r)))
    return r.value


def device_count() -> int:
    return lib().mbg_device_count()


class Model:
    """A parsed and compiled .bnd/.cfg model (driver::parse of the reference)."""

    def __init__(self, handle, like=None):
        """`like`: a model this one was derived from (rate scales, mutants), whose node names and
        output nodes it shares; they are copied instead of read through the handle."""
        self._h = handle
        info = ModelInfo()
        _check(lib().mbg_model_info_get(self._h, ctypes.byref(info)))
        self.info = info
        if like is not None:
            self.names = list(like.names)
            self.outputs = list(like.outputs)
            return
        L = lib()
        self.names = [L.mbg_model_node_name(self._h, i).decode() for i in range(info.nodes)]
        out = np.zeros(max(1, info.outputs), np.int32)
        L.mbg_model_outputs(self._h, _p(out), info.outputs)
        self.outputs = [int(x) for x in out[:info.outputs]]

    @classmethod
    def from_files(cls, bnd_path, cfg_path, overrides=None):
        """Parse the model files; `overrides` (cfg statements, e.g. "$k = 2; max_time = 50;") are
        applied after the cfg file and replace its values."""
        h = ctypes.c_void_p()
        if overrides:
            _check(lib().mbg_model_parse_files_overrides(os.fsencode(bnd_path), os.fsencode(cfg_path),
                                                         overrides.encode(), ctypes.byref(h)))
        else:
            _check(lib().mbg_model_parse_files(os.fsencode(bnd_path), os.fsencode(cfg_path), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_strings(cls, bnd, cfg):
        h = ctypes.c_void_p()
        _check(lib().mbg_model_parse_strings(bnd.encode(), cfg.encode(), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, regulators, logic, rate_up, rate_down, istate, is_output=None, names=None, max_time=10.0,
                    time_tick=0.1, sample_count=1000000, seed=0, discrete=False):
        """A model from arrays (mbg_model_from_arrays): regulators[i] lists node i's regulators,
        logic[i] its truth table over them (2^k entries of 0/1, entry idx = sum_j state(reg_j) << j);
        the node turns on at rate_up[i] while off with logic 1, off at rate_down[i] while on with
        logic 0. is_output (default: every node) marks the non-internal nodes."""
        n = len(regulators)
        reg_off = np.zeros(n + 1, np.int32)
        for i, r in enumerate(regulators):
            reg_off[i + 1] = reg_off[i] + len(r)
        regs = np.ascontiguousarray(np.concatenate([np.asarray(r, np.int32) for r in regulators])
                                    if reg_off[-1] else np.zeros(1, np.int32), dtype=np.int32)
        words, logic_off = [], np.zeros(n, np.int64)
        for i, (r, t) in enumerate(zip(regulators, logic)):
            t = np.asarray(t, np.uint8).ravel()
            if t.size != 1 << len(r):
                raise ValueError(f"node {i}: truth table needs {1 << len(r)} entries")
            logic_off[i] = len(words)
            bits = np.zeros(((t.size + 31) // 32) * 32, np.uint8)
            bits[:t.size] = t != 0
            w = (bits.reshape(-1, 32).astype(np.uint64) << np.arange(32, dtype=np.uint64)).sum(axis=1)
            words.extend(int(x) for x in w)
        logic_w = np.ascontiguousarray(np.array(words, np.uint32))
        up = np.ascontiguousarray(np.asarray(rate_up, np.float64))
        down = np.ascontiguousarray(np.asarray(rate_down, np.float64))
        ist = np.ascontiguousarray(np.asarray(istate, np.float64))
        if not (up.size == down.size == ist.size == n) or (is_output is not None and len(is_output) != n):
            raise ValueError("one rate_up, rate_down, istate (and is_output) entry per node")
        outs = None if is_output is None else np.ascontiguousarray(np.asarray(is_output, np.uint8))
        cnames = None
        if names is not None:
            if len(names) != n:
                raise ValueError("one name per node")
            cnames = (ctypes.c_char_p * n)(*[s.encode() for s in names])
        run = ModelRun(max_time, time_tick, sample_count, seed, 1 if discrete else 0, 0)
        h = ctypes.c_void_p()
        _check(lib().mbg_model_from_arrays(n, cnames, _p(reg_off), _p(regs), _p(logic_w), logic_w.size, _p(logic_off),
                                           _p(up), _p(down), _p(ist), _p(outs), ctypes.byref(run), ctypes.byref(h)))
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

    def with_rate_scales(self, up=None, down=None) -> "Model":
        """Copy with node i's up rates times up[i] and down rates times down[i] (no re-parse)."""
        u = None if up is None else np.ascontiguousarray(np.asarray(up, dtype=np.float64))
        d = None if down is None else np.ascontiguousarray(np.asarray(down, dtype=np.float64))
        for a in (u, d):
            if a is not None and a.size != self.info.nodes:
                raise ValueError("one scale per node")
        h = ctypes.c_void_p()
        _check(lib().mbg_model_with_rate_scales(self._h, _p(u), _p(d), ctypes.byref(h)))
        return Model(h, like=self)

    def with_mutations(self, mutants) -> "Model":
        """Mutant copy: `mutants` maps node names (or indices) to "ON"/"OFF" (or 1/0); each such
        node starts at that value and never leaves it."""
        idx, val = [], []
        for k, v in dict(mutants).items():
            i = self.names.index(k) if isinstance(k, str) else int(k)
            if isinstance(v, str):
                if v.upper() not in ("ON", "OFF"):
                    raise ValueError(f"mutant value {v!r}: expected ON or OFF")
                v = 1 if v.upper() == "ON" else 0
            idx.append(i)
            val.append(int(v))
        n = np.ascontiguousarray(np.asarray(idx, dtype=np.int32))
        w = np.ascontiguousarray(np.asarray(val, dtype=np.int32))
        h = ctypes.c_void_p()
        _check(lib().mbg_model_with_mutations(self._h, _p(n), _p(w), len(idx), ctypes.byref(h)))
        return Model(h, like=self)

    def layout_check(self):
        """Checks the model's device tables on the host (raises MbgError on an index out of range)."""
        _check(lib().mbg_model_layout_check(self._h))

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
                 max_steps=0, traj_base=0, device=0, block_size=0, blocks_per_sm=0, thread_cutoff=0,
                 lane_update=0, window_table=0, window_hash_bits=0, redraw_period=0):
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
        o.lane_update = lane_update
        o.window_table = window_table
        o.window_hash_bits = window_hash_bits
        o.redraw_period = redraw_period
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

    def probtraj_sparse(self):
        """The reached window bins only: (bins, raw sums, probabilities), bins increasing, each
        bin = window * 2^outputs + output state."""
        n = ctypes.c_size_t()
        _check(lib().mbg_sim_probtraj_sparse(self._h, None, None, None, 0, ctypes.byref(n)))
        bins = np.empty(n.value, np.uint64)  # every entry is written
        sums = np.empty(n.value, np.uint64)
        probs = np.empty(n.value, np.float64)
        _check(lib().mbg_sim_probtraj_sparse(self._h, _p(bins), _p(sums), _p(probs), n.value, ctypes.byref(n)))
        return bins, sums, probs

    def tr_entropy(self):
        """Per-window transition entropy."""
        TH = np.zeros(self.model.info.windows, np.float64)
        _check(lib().mbg_sim_probtraj(self._h, None, _p(TH)))
        return TH

    def final_states(self):
        F = np.empty(1 << self.model.info.outputs, np.float64)  # every entry is written
        _check(lib().mbg_sim_final_states(self._h, _p(F)))
        return F

    def final_states_sparse(self):
        """The reached final output states only: (states, probabilities), states increasing."""
        n = ctypes.c_size_t()
        _check(lib().mbg_sim_final_states_sparse(self._h, None, None, 0, ctypes.byref(n)))
        states = np.empty(n.value, np.uint64)  # every entry is written
        probs = np.empty(n.value, np.float64)
        _check(lib().mbg_sim_final_states_sparse(self._h, _p(states), _p(probs), n.value, ctypes.byref(n)))
        return states, probs

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

    def write_csv(self, prefix, final_states=False):
        _check(lib().mbg_write_probtraj_csv(self._h, os.fsencode(prefix)))
        _check(lib().mbg_write_fp_csv(self._h, os.fsencode(prefix)))
        if final_states:
            _check(lib().mbg_write_final_states_csv(self._h, os.fsencode(prefix)))

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


class Batch:
    """Many instances (models, trajectory counts, seeds) run in one graph-captured launch."""

    def __init__(self, models, n_traj=None, seeds=None, device=0, max_steps=0, block_size=0, blocks_per_sm=0,
                 autotune=False, layout=0, lane_variant=0):
        o = BatchOpts()
        lib().mbg_batch_opts_default(ctypes.byref(o))
        o.device, o.max_steps, o.block_size, o.blocks_per_sm = device, max_steps, block_size, blocks_per_sm
        o.autotune = 1 if autotune else 0
        o.layout = layout
        o.lane_variant = lane_variant
        self.models = list(models)
        handles = (ctypes.c_void_p * len(self.models))(*[m._h for m in self.models])
        nt = None if n_traj is None else np.ascontiguousarray(np.asarray(n_traj, dtype=np.uint64))
        sd = None if seeds is None else np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
        h = ctypes.c_void_p()
        _check(lib().mbg_batch_create(ctypes.cast(handles, ctypes.c_void_p), len(self.models), _p(nt), _p(sd),
                                      ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self.n_traj = [int(x) for x in nt] if nt is not None else [int(m.info.sample_count) for m in self.models]

    def run(self, stream=None):
        _check(lib().mbg_batch_run(self._h, ctypes.c_void_p(stream) if stream else None))
        return self

    def summary(self, instance=None) -> dict:
        s = RunSummary()
        if instance is None:
            _check(lib().mbg_batch_summary(self._h, ctypes.byref(s)))
        else:
            _check(lib().mbg_batch_instance_summary(self._h, int(instance), ctypes.byref(s)))
        return s.as_dict()

    def classes(self):
        """Size classes with their launch shapes and, after an autotuned run, every timed shape."""
        n = ctypes.c_int32()
        _check(lib().mbg_batch_class_count(self._h, ctypes.byref(n)))
        out = []
        for c in range(n.value):
            k = BatchClassInfo()
            _check(lib().mbg_batch_class(self._h, c, ctypes.byref(k)))
            t = (BatchClassTiming * max(1, k.timings))()
            cnt = ctypes.c_int32()
            _check(lib().mbg_batch_class_timings(self._h, c, t, k.timings, ctypes.byref(cnt)))
            out.append({"max_nodes": k.max_nodes, "instances": k.instances, "trajectories": k.trajectories,
                        "layout": {LAYOUT_LANE: "lane", LAYOUT_WARP: "warp", LAYOUT_LANE_GLOBAL: "lane_global"}.get(k.layout, k.layout),
                        "block_size": k.block_size, "variant": k.variant, "grid": k.grid,
                        "kernel_ms": k.kernel_ms,
                        "timings": [{"layout": {LAYOUT_LANE: "lane", LAYOUT_WARP: "warp", LAYOUT_LANE_GLOBAL: "lane_global"}.get(x.layout, x.layout),
                                     "block_size": x.block_size, "variant": x.variant, "kernel_ms": x.kernel_ms}
                                    for x in t[:cnt.value]]})
        return out

    def probtraj(self, i):
        info = self.models[i].info
        P = np.zeros((info.windows, 1 << info.outputs), np.float64)
        TH = np.zeros(info.windows, np.float64)
        _check(lib().mbg_batch_probtraj(self._h, int(i), _p(P), _p(TH)))
        return P, TH

    def window_probs(self, window=-1):
        """One window of every instance (negative: from each instance's last window), gathered on
        the device: an instances x 2^outputs array when all instances have the same outputs, else a
        list of per-instance arrays."""
        sizes = [1 << m.info.outputs for m in self.models]
        out = np.empty(sum(sizes), np.float64)  # every entry is written
        _check(lib().mbg_batch_window_probs(self._h, int(window), _p(out)))
        if len(set(sizes)) <= 1:
            return out.reshape(len(sizes), sizes[0] if sizes else 0)
        return np.split(out, np.cumsum(sizes)[:-1])

    def probtraj_raw(self, i):
        info = self.models[i].info
        P = np.zeros((info.windows, 1 << info.outputs), np.uint64)
        TH = np.zeros(info.windows, np.uint64)
        _check(lib().mbg_batch_probtraj_raw(self._h, int(i), _p(P), _p(TH)))
        return P, TH

    def final_states(self, i):
        F = np.zeros(1 << self.models[i].info.outputs, np.float64)
        _check(lib().mbg_batch_final_states(self._h, int(i), _p(F)))
        return F

    def fixed_points(self, i):
        n = ctypes.c_size_t()
        _check(lib().mbg_batch_fixed_points(self._h, int(i), None, None, 0, ctypes.byref(n)))
        W = self.models[i].info.words
        states = np.zeros((n.value, W), np.uint32)
        probs = np.zeros(n.value, np.float64)
        if n.value:
            _check(lib().mbg_batch_fixed_points(self._h, int(i), _p(states), _p(probs), n.value, ctypes.byref(n)))
        return states, probs

    def close(self):
        if self._h:
            lib().mbg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    """Ensemble of BF16 MLPs screening sweep points (mbg_surrogate_*)."""

    def __init__(self, in_dim, out_dim, hidden=512, hidden_layers=3, ensemble=4, seed=0, device=0, tcgen05=True):
        h = ctypes.c_void_p()
        _check(lib().mbg_surrogate_create(in_dim, hidden, hidden_layers, out_dim, ensemble, seed, device,
                                          ctypes.byref(h)))
        self._h = h
        self.set_tensor_path(tcgen05)
        self.in_dim, self.out_dim, self.hidden, self.hidden_layers = in_dim, out_dim, hidden, hidden_layers
        self.ensemble = ensemble

    def set_tensor_path(self, tcgen05: bool):
        """Forward products on the tcgen05 tensor cores (True) or on the mma.sync kernel (False)."""
        _check(lib().mbg_surrogate_set_tensor_path(self._h, 1 if tcgen05 else 0))
        self.tcgen05 = bool(tcgen05)

    def time_forward(self, rows, reps=10):
        """Device milliseconds of one forward pass of every member over `rows` rows."""
        ms = ctypes.c_double()
        _check(lib().mbg_surrogate_time_forward(self._h, int(rows), int(reps), ctypes.byref(ms)))
        return ms.value

    def param_count(self):
        return int(lib().mbg_surrogate_param_count(self._h))

    def train(self, x, y, epochs=50, batch=256, lr=1e-3, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = ctypes.c_float()
        _check(lib().mbg_surrogate_train(self._h, _p(x), _p(y), len(x), epochs, batch, lr, seed, ctypes.byref(loss)))
        return loss.value

    def predict(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        probs = np.zeros((len(x), self.out_dim), np.float32)
        spread = np.zeros(len(x), np.float32)
        _check(lib().mbg_surrogate_predict(self._h, _p(x), len(x), _p(probs), _p(spread)))
        return probs, spread

    def predict_column(self, x, column):
        """Ensemble-mean probability of output state `column` and the spread, per row."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        score = np.zeros(len(x), np.float32)
        spread = np.zeros(len(x), np.float32)
        _check(lib().mbg_surrogate_predict_column(self._h, _p(x), len(x), int(column), _p(score), _p(spread)))
        return score, spread

    def params(self, member=0):
        out = np.zeros(self.param_count(), np.float32)
        _check(lib().mbg_surrogate_get_params(self._h, member, _p(out)))
        return out

    def set_params(self, member, params):
        params = np.ascontiguousarray(params, dtype=np.float32)
        _check(lib().mbg_surrogate_set_params(self._h, member, _p(params)))

    def gradients(self, member, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_float()
        _check(lib().mbg_surrogate_gradients(self._h, member, _p(x), _p(y), len(x), ctypes.byref(loss), _p(g)))
        return loss.value, g

    def close(self):
        if self._h:
            lib().mbg_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shard_range(n_traj: int, rank: int, world: int):
    """(first trajectory id, count) of `rank`'s share of n_traj trajectories over `world` ranks.
    Trajectories are keyed by id, so the union of the shards equals one run over all ids."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank outside the world")
    q, r = divmod(int(n_traj), world)
    return rank * q + min(rank, r), q + (1 if rank < r else 0)
