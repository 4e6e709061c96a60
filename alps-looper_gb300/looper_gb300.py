"""Python binding of the GB300 loop-cluster engine (ctypes over include/looper_gpu.h).

`LoopWorker` mirrors looper's path-integral worker plug-in (path_integral.C:57-124): it is
constructed from the worker's parameters, `run()` performs one sweep of update + measurement,
`is_thermalized()` / `progress()` report the schedule, `save()` / `load()` checkpoint the
configuration and `set_beta()` / `weight_parameter()` / `log_weight()` are the exchange Monte
Carlo hooks.  `Batch` runs many independent chains in one arena.

There is no CPU fallback: importing this module fails if the CUDA library is missing.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liblooper_gb300.so")

CHAIN, SQUARE, CUBIC = 1, 2, 3
LATTICES = {"chain lattice": CHAIN, "chain": CHAIN, "square lattice": SQUARE, "square": SQUARE,
            "simple cubic lattice": CUBIC, "cubic": CUBIC}
RECORD_WORDS = 32
NUM_OBS = 19

ERRORS = {0: "LG_OK", -1: "LG_EINVAL", -2: "LG_ENOMEM", -3: "LG_EDEVICE", -4: "LG_EUNSUPPORTED",
          -5: "LG_EITERCAP", -6: "LG_EBUDGET", -7: "LG_ECORRUPT", -8: "LG_ENOTREADY"}


class LoopError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("lattice", ctypes.c_int), ("L", ctypes.c_int), ("T", ctypes.c_double),
                ("beta", ctypes.c_double), ("J", ctypes.c_double), ("Jz", ctypes.c_double),
                ("Jxy", ctypes.c_double), ("h", ctypes.c_double),
                ("force_scatter", ctypes.c_double), ("sweeps", ctypes.c_uint64),
                ("thermalization", ctypes.c_int64), ("seed", ctypes.c_uint64),
                ("init_spins", ctypes.c_int), ("disable_improved_estimator", ctypes.c_int),
                ("measure_correlations", ctypes.c_int), ("measure_structure_factor", ctypes.c_int),
                ("initial_site", ctypes.c_int), ("spin2", ctypes.c_int),
                ("algorithm", ctypes.c_int)]


class Obs(ctypes.Structure):
    _fields_ = [("count", ctypes.c_uint64), ("beta", ctypes.c_double), ("volume", ctypes.c_double),
                ("improved", ctypes.c_int), ("mean", ctypes.c_double * NUM_OBS),
                ("error", ctypes.c_double * NUM_OBS), ("tau", ctypes.c_double * NUM_OBS)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_double), ("sweeps_per_tick", ctypes.c_int),
                ("rebuild_interval_s", ctypes.c_double), ("max_active", ctypes.c_int),
                ("lanes", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int), ("t_submit", ctypes.c_double),
                ("t_start", ctypes.c_double), ("t_finish", ctypes.c_double),
                ("sweeps", ctypes.c_uint64), ("sites", ctypes.c_int64), ("obs", Obs)]


class Shape(ctypes.Structure):
    """Launch shape of an arena (lg_shape): changes speed only, never a result."""
    _fields_ = [("insert_k", ctypes.c_double), ("narrow_k", ctypes.c_double),
                ("acc_tile", ctypes.c_int), ("cl_tile", ctypes.c_int),
                ("union_warps", ctypes.c_int), ("resident", ctypes.c_int),
                ("union_mode", ctypes.c_int)]

    def as_dict(self):
        return {"insert_k": self.insert_k, "narrow_k": self.narrow_k, "acc_tile": self.acc_tile,
                "cl_tile": self.cl_tile, "union_warps": self.union_warps,
                "resident": self.resident, "union_mode": self.union_mode}


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("rejected", ctypes.c_uint64), ("rebuilds", ctypes.c_uint64),
                ("site_sweeps", ctypes.c_int64), ("queued", ctypes.c_int64),
                ("active_bytes", ctypes.c_double), ("elapsed_s", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("looper_gb300: %s is missing; build it with "
                              "python alps-looper_gb300/build.py" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, u64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64
        sig = {
            "lg_params_default": (None, [vp]),
            "lg_params_parse": (ctypes.c_int, [ctypes.c_char_p, vp]),
            "lg_obs_name": (ctypes.c_char_p, [ctypes.c_int]),
            "lg_value_name": (ctypes.c_char_p, [ctypes.c_int]),
            "lg_value_mask": (ctypes.c_int, [vp, vp]),
            "lg_keep_values": (ctypes.c_int, [vp, ctypes.c_int]),
            "lg_fetch_values": (ctypes.c_int, [vp, vp, i64, vp]),
            "lg_create": (ctypes.c_int, [vp, vp]),
            "lg_destroy": (ctypes.c_int, [vp]),
            "lg_run": (ctypes.c_int, [vp, i64]),
            "lg_is_thermalized": (ctypes.c_int, [vp]),
            "lg_progress": (ctypes.c_double, [vp]),
            "lg_observables": (ctypes.c_int, [vp, vp]),
            "lg_save": (ctypes.c_int, [vp, vp, vp]),
            "lg_load": (ctypes.c_int, [vp, vp, ctypes.c_size_t]),
            "lg_set_beta": (ctypes.c_int, [vp, ctypes.c_double]),
            "lg_correlations": (ctypes.c_int, [vp, ctypes.c_int, vp, vp]),
            "lg_correlation_sums": (ctypes.c_int, [vp, ctypes.c_int, vp, vp]),
            "lg_weight_parameter": (ctypes.c_double, [vp]),
            "lg_log_weight": (ctypes.c_double, [ctypes.c_double, ctypes.c_double]),
            "lg_last_error": (ctypes.c_int, [vp, ctypes.c_size_t]),
            "lg_get_state": (ctypes.c_int, [vp, vp, vp, vp, i64, vp]),
            "lg_set_state": (ctypes.c_int, [vp, vp, vp, vp, i64, u64]),
            "lg_fetch_records": (ctypes.c_int, [vp, vp, i64, vp]),
            "lg_keep_records": (ctypes.c_int, [vp, ctypes.c_int]),
            "lg_set_iteration_cap": (ctypes.c_int, [vp, ctypes.c_int]),
            "lg_validate_sweeps": (ctypes.c_int, [vp, i64]),
            "lg_batch_validate_sweeps": (ctypes.c_int, [vp, i64]),
            "lg_uf_label": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, i64, vp, vp, vp, i64, vp, vp]),
            "lg_uf_label_static": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, i64, vp, vp, vp, vp, vp, vp]),
            "lg_batch_create": (ctypes.c_int, [ctypes.c_int, vp, vp]),
            "lg_batch_destroy": (ctypes.c_int, [vp]),
            "lg_batch_run": (ctypes.c_int, [vp, i64]),
            "lg_batch_observables": (ctypes.c_int, [vp, ctypes.c_int, vp]),
            "lg_batch_size": (ctypes.c_int, [vp]),
            "lg_batch_stats": (ctypes.c_int, [vp, vp, vp]),
            "lg_batch_chain": (vp, [vp, ctypes.c_int]),
            "lg_time_sweeps": (ctypes.c_int, [vp, i64, ctypes.c_size_t, vp]),
            "lg_batch_time_sweeps": (ctypes.c_int, [vp, i64, ctypes.c_size_t, vp]),
            "lg_profile_sweeps": (ctypes.c_int, [vp, i64, ctypes.c_size_t, vp, vp]),
            "lg_batch_profile_sweeps": (ctypes.c_int, [vp, i64, ctypes.c_size_t, vp, vp]),
            "lg_autotune": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_size_t, vp, vp, ctypes.c_size_t]),
            "lg_batch_autotune": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_size_t, vp, vp, ctypes.c_size_t]),
            "lg_batch_get_shape": (ctypes.c_int, [vp, vp]),
            "lg_batch_set_shape": (ctypes.c_int, [vp, vp]),
            "lg_get_shape": (ctypes.c_int, [vp, vp]),
            "lg_set_shape": (ctypes.c_int, [vp, vp]),
            "lg_num_kernels": (ctypes.c_int, []),
            "lg_kernel_name": (ctypes.c_char_p, [ctypes.c_int]),
            "lg_exchange_chain_seed": (u64, [u64, ctypes.c_int]),
            "lg_exchange_create": (ctypes.c_int, [vp, ctypes.c_int, vp, vp]),
            "lg_exchange_destroy": (ctypes.c_int, [vp]),
            "lg_exchange_run": (ctypes.c_int, [vp, i64, ctypes.c_int]),
            "lg_exchange_observables": (ctypes.c_int, [vp, ctypes.c_int, vp]),
            "lg_exchange_state": (ctypes.c_int, [vp, vp, vp, vp]),
            "lg_exchange_chain": (vp, [vp, ctypes.c_int]),
            "lg_server_config_default": (None, [vp]),
            "lg_request_bytes": (ctypes.c_double, [vp]),
            "lg_server_create": (ctypes.c_int, [vp, vp]),
            "lg_server_submit": (ctypes.c_int, [vp, vp, vp]),
            "lg_server_poll": (ctypes.c_int, [vp, vp, ctypes.c_int, vp]),
            "lg_server_wait": (ctypes.c_int, [vp, ctypes.c_double]),
            "lg_server_get_stats": (ctypes.c_int, [vp, vp]),
            "lg_server_destroy": (ctypes.c_int, [vp]),
            "lg_kernel_launches": (u64, []),
            "lg_copy_bytes": (None, [vp, vp]),
            "lg_version": (ctypes.c_char_p, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().lg_last_error(buf, 1024)
    return buf.value.decode()


def check(rc):
    if rc != 0:
        raise LoopError(rc, last_error())
    return rc


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_params(**kw) -> Params:
    """Parameters with the worker's key names: LATTICE, L, T, BETA, J, Jz, Jxy, h, SWEEPS,
    THERMALIZATION, SEED, FORCE_SCATTER, INITIAL_SPINS, DISABLE_IMPROVED_ESTIMATOR (lower-case
    aliases accepted), and the correlation switches MEASURE_CORRELATIONS (MEASURE[Correlations]),
    MEASURE_STRUCTURE_FACTOR (MEASURE[Structure Factor]) and INITIAL_SITE, and local_S (1/2, 1,
    3/2: the site spin)."""
    p = Params()
    lib().lg_params_default(ctypes.byref(p))
    for k, v in kw.items():
        key = k.upper() if k.upper() in ("LATTICE", "BETA", "SWEEPS", "THERMALIZATION", "SEED", "ALGORITHM",
                                         "FORCE_SCATTER", "INITIAL_SPINS",
                                         "DISABLE_IMPROVED_ESTIMATOR", "MEASURE_CORRELATIONS",
                                         "MEASURE_STRUCTURE_FACTOR", "INITIAL_SITE") else k
        if key == "LATTICE":
            p.lattice = LATTICES[v] if isinstance(v, str) else int(v)
        elif key == "L":
            p.L = int(v)
        elif key == "T":
            p.T = float(v)
        elif key == "BETA":
            p.beta = float(v)
        elif key in ("J", "Jz", "Jxy", "h"):
            setattr(p, key, float(v))
        elif key == "SWEEPS":
            p.sweeps = int(v)
        elif key == "THERMALIZATION":
            p.thermalization = int(v)
        elif key == "SEED":
            p.seed = int(v)
        elif key == "FORCE_SCATTER":
            p.force_scatter = float(v)
        elif key == "INITIAL_SPINS":
            p.init_spins = 1 if v in ("random", 1, True) else 0
        elif key == "DISABLE_IMPROVED_ESTIMATOR":
            p.disable_improved_estimator = 1 if v else 0
        elif key in ("MEASURE_CORRELATIONS", "MEASURE[Correlations]"):
            p.measure_correlations = 1 if v else 0
        elif key in ("MEASURE_STRUCTURE_FACTOR", "MEASURE[Structure Factor]"):
            p.measure_structure_factor = 1 if v else 0
        elif key == "INITIAL_SITE":
            p.initial_site = int(v)
        elif key == "ALGORITHM":
            p.algorithm = 1 if str(v).lower() in ("sse", "loop; sse", "1") else 0
        elif key in ("local_S", "LOCAL_S"):
            p.spin2 = int(round(2 * float(v)))
        else:
            raise KeyError(k)
    return p


def parse_params(text: str) -> Params:
    p = Params()
    lib().lg_params_default(ctypes.byref(p))
    check(lib().lg_params_parse(text.encode(), ctypes.byref(p)))
    return p


NUM_VALUES = 37  # LG_NUM_VALUES


def value_name(i):
    return lib().lg_value_name(i).decode()


def obs_names():
    return [lib().lg_obs_name(i).decode() for i in range(NUM_OBS)]


def _obs_dict(o: Obs):
    names = obs_names()
    return {n: (o.mean[i], o.error[i]) for i, n in enumerate(names)} | {
        "count": o.count, "improved": bool(o.improved)}


def _time(fn, h, n, flush_bytes):
    ms = np.zeros(max(int(n), 1), dtype=np.float32)
    check(fn(h, int(n), int(flush_bytes), _p(ms)))
    return ms[:int(n)]


def _profile(fn, h, n, flush_bytes):
    k = lib().lg_num_kernels()
    out = np.zeros(k, dtype=np.float64)
    v = ctypes.c_int64()
    check(fn(h, int(n), int(flush_bytes), _p(out), ctypes.byref(v)))
    names = [lib().lg_kernel_name(i).decode() for i in range(k)]
    return dict(zip(names, out.tolist())), v.value


def _autotune(fn, h, trial, flush_bytes):
    sh = Shape()
    buf = ctypes.create_string_buffer(8192)
    check(fn(h, int(trial), int(flush_bytes), ctypes.byref(sh), buf, 8192))
    return sh.as_dict(), buf.value.decode()


class LoopWorker:
    """One chain: looper's "loop; path integral" worker on the GPU."""

    def __init__(self, params: Params | None = None, _handle=None, _owner=None, **kw):
        self._owner = _owner
        if _handle is not None:
            self._h = ctypes.c_void_p(_handle)
            self._own = False
        else:
            if params is None:
                params = make_params(**kw)
            h = ctypes.c_void_p()
            check(lib().lg_create(ctypes.byref(params), ctypes.byref(h)))
            self._h = h
            self._own = True
        self.params = params

    def close(self):
        if getattr(self, "_own", False) and self._h:
            lib().lg_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsweeps: int = 1):
        check(lib().lg_run(self._h, int(nsweeps)))

    CORR_KINDS = {"Spin Correlations": 0, "Staggered Spin Correlations": 1,
                  "Spin Structure Factor": 2}

    def correlations(self, kind="Spin Correlations"):
        """(mean, error) arrays of N entries: "Spin Correlations", "Staggered Spin Correlations"
        (entry i = displacement, or the site with INITIAL_SITE, of site index i) or "Spin
        Structure Factor" (entry i = momentum 2 pi (x, y, z) / L of site index i)."""
        k = self.CORR_KINDS[kind] if isinstance(kind, str) else int(kind)
        n = self.num_sites()
        mean = np.zeros(n)
        err = np.zeros(n)
        check(lib().lg_correlations(self._h, k, _p(mean), _p(err)))
        return mean, err

    def correlation_sums(self, which=0):
        """Exact integer sums over the measured sweeps (which = 0: sum_i m_i m_{i+r} per
        displacement r; 1: m_o m_j per site j for INITIAL_SITE o) and the sweep count."""
        n = self.num_sites()
        out = np.zeros(n, dtype=np.int64)
        ns = ctypes.c_int64()
        check(lib().lg_correlation_sums(self._h, int(which), _p(out), ctypes.byref(ns)))
        return out, ns.value

    def validate_sweeps(self, n: int):
        """n sweeps with structural checks between the kernels (raises on a failed check)."""
        check(lib().lg_validate_sweeps(self._h, int(n)))

    def set_iteration_cap(self, cap: int):
        """Test seam: union-find retries per union (0: default; < 0: none, forcing
        LG_EITERCAP)."""
        check(lib().lg_set_iteration_cap(self._h, int(cap)))

    def is_thermalized(self) -> bool:
        return bool(lib().lg_is_thermalized(self._h))

    def progress(self) -> float:
        return lib().lg_progress(self._h)

    def observables(self):
        o = Obs()
        check(lib().lg_observables(self._h, ctypes.byref(o)))
        return _obs_dict(o)

    def set_beta(self, beta: float):
        check(lib().lg_set_beta(self._h, float(beta)))

    def weight_parameter(self) -> float:
        return lib().lg_weight_parameter(self._h)

    @staticmethod
    def log_weight(gw: float, beta: float) -> float:
        return lib().lg_log_weight(float(gw), float(beta))

    def save(self) -> bytes:
        n = ctypes.c_size_t(0)
        check(lib().lg_save(self._h, None, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        check(lib().lg_save(self._h, buf, ctypes.byref(n)))
        return buf.raw[:n.value]

    def load(self, blob: bytes):
        blob = bytes(blob)  # read in place (lg_load copies nothing it keeps)
        check(lib().lg_load(self._h, ctypes.c_char_p(blob), len(blob)))

    def time_sweeps(self, n, flush_bytes=0):
        """Device time (ms) of each of n sweeps, L2 flushed between sweeps."""
        return _time(lib().lg_time_sweeps, self._h, n, flush_bytes)

    def profile_sweeps(self, n, flush_bytes=0):
        """Per-stage device time (ms, summed over n sweeps) and operators processed."""
        return _profile(lib().lg_profile_sweeps, self._h, n, flush_bytes)

    def autotune(self, trial_sweeps=4, flush_bytes=0):
        """Pick the fastest launch shape for this chain; returns (shape dict, report text)."""
        return _autotune(lib().lg_autotune, self._h, trial_sweeps, flush_bytes)

    @property
    def shape(self):
        sh = Shape()
        check(lib().lg_get_shape(self._h, ctypes.byref(sh)))
        return sh.as_dict()

    @shape.setter
    def shape(self, d):
        sh = Shape()
        check(lib().lg_get_shape(self._h, ctypes.byref(sh)))
        for k, v in d.items():
            setattr(sh, k, v)
        check(lib().lg_set_shape(self._h, ctypes.byref(sh)))

    # ---- test seams ----
    def num_sites(self):
        """Simulated sites: L^dim, times 2S virtual sites per site for S > 1/2."""
        L = self.params.L
        return L ** self.params.lattice * max(1, self.params.spin2)

    def state(self):
        N = self.num_sites()
        spins = np.zeros(N, dtype=np.int32)
        n = ctypes.c_int64()
        check(lib().lg_get_state(self._h, _p(spins), None, None, 0, ctypes.byref(n)))
        bonds = np.zeros(max(n.value, 1), dtype=np.int32)
        times = np.zeros(max(n.value, 1), dtype=np.float64)
        check(lib().lg_get_state(self._h, _p(spins), _p(bonds), _p(times), n.value, ctypes.byref(n)))
        return spins, bonds[:n.value].copy(), times[:n.value].copy()

    def set_state(self, spins, bonds, times, sweep):
        spins = np.ascontiguousarray(spins, dtype=np.int32)
        bonds = np.ascontiguousarray(bonds, dtype=np.int32)
        times = np.ascontiguousarray(times, dtype=np.float64)
        check(lib().lg_set_state(self._h, _p(spins), _p(bonds), _p(times), len(bonds), int(sweep)))

    def keep_records(self, on=True):
        check(lib().lg_keep_records(self._h, 1 if on else 0))

    def fetch_records(self, cap=1 << 20):
        out = np.zeros(cap * RECORD_WORDS, dtype=np.uint64)
        n = ctypes.c_int64()
        check(lib().lg_fetch_records(self._h, _p(out), cap, ctypes.byref(n)))
        return out[:n.value * RECORD_WORDS].reshape(n.value, RECORD_WORDS).copy()

    def value_names(self):
        """The ObservableSet keys this chain's sweeps push (lg_value_mask), in LG_VAL order."""
        m = ctypes.c_uint64()
        check(lib().lg_value_mask(self._h, ctypes.byref(m)))
        return [value_name(i) for i in range(NUM_VALUES) if m.value >> i & 1]

    def keep_values(self, on=True):
        check(lib().lg_keep_values(self._h, 1 if on else 0))

    def fetch_values(self, cap=1 << 16):
        """Per-sweep values of the measurement sweeps since the last fetch: {name: array}."""
        out = np.zeros(cap * NUM_VALUES, dtype=np.float64)
        n = ctypes.c_int64()
        check(lib().lg_fetch_values(self._h, _p(out), cap, ctypes.byref(n)))
        rows = out[:n.value * NUM_VALUES].reshape(n.value, NUM_VALUES)
        m = ctypes.c_uint64()
        check(lib().lg_value_mask(self._h, ctypes.byref(m)))
        return {value_name(i): rows[:, i].copy() for i in range(NUM_VALUES) if m.value >> i & 1}


class Batch:
    """Many independent chains (possibly of different sizes and temperatures) in one arena."""

    def __init__(self, params_list):
        arr = (Params * len(params_list))(*params_list)
        h = ctypes.c_void_p()
        check(lib().lg_batch_create(len(params_list), arr, ctypes.byref(h)))
        self._h = h
        self.params = list(params_list)

    def close(self):
        if self._h:
            lib().lg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return lib().lg_batch_size(self._h)

    def run(self, nsweeps: int = 1):
        check(lib().lg_batch_run(self._h, int(nsweeps)))

    def observables(self, i):
        o = Obs()
        check(lib().lg_batch_observables(self._h, i, ctypes.byref(o)))
        return _obs_dict(o)

    def stats(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        check(lib().lg_batch_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def validate_sweeps(self, n: int):
        """n sweeps of the arena with structural checks between the kernels."""
        check(lib().lg_batch_validate_sweeps(self._h, int(n)))

    def time_sweeps(self, n, flush_bytes=0):
        return _time(lib().lg_batch_time_sweeps, self._h, n, flush_bytes)

    def profile_sweeps(self, n, flush_bytes=0):
        return _profile(lib().lg_batch_profile_sweeps, self._h, n, flush_bytes)

    def autotune(self, trial_sweeps=4, flush_bytes=0):
        """Pick the fastest launch shape; returns (shape dict, report text)."""
        return _autotune(lib().lg_batch_autotune, self._h, trial_sweeps, flush_bytes)

    @property
    def shape(self):
        sh = Shape()
        check(lib().lg_batch_get_shape(self._h, ctypes.byref(sh)))
        return sh.as_dict()

    @shape.setter
    def shape(self, d):
        sh = Shape()
        check(lib().lg_batch_get_shape(self._h, ctypes.byref(sh)))
        for k, v in d.items():
            setattr(sh, k, v)
        check(lib().lg_batch_set_shape(self._h, ctypes.byref(sh)))

    def chain(self, i) -> LoopWorker:
        h = lib().lg_batch_chain(self._h, i)
        if not h:
            raise IndexError(i)
        return LoopWorker(self.params[i], _handle=h, _owner=self)


class Exchange:
    """Exchange Monte Carlo (parallel tempering) over a ladder of inverse temperatures."""

    def __init__(self, params: Params, betas):
        self.params = params
        self.betas = [float(b) for b in betas]
        arr = (ctypes.c_double * len(self.betas))(*self.betas)
        h = ctypes.c_void_p()
        check(lib().lg_exchange_create(ctypes.byref(params), len(self.betas), arr, ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().lg_exchange_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsweeps: int, interval: int = 1):
        check(lib().lg_exchange_run(self._h, int(nsweeps), int(interval)))

    def observables(self, t):
        o = Obs()
        check(lib().lg_exchange_observables(self._h, int(t), ctypes.byref(o)))
        return _obs_dict(o)

    def state(self):
        """(chain_of_temp, attempts, accepts) as numpy arrays."""
        n = len(self.betas)
        cot = np.zeros(n, dtype=np.int32)
        att = np.zeros(max(n - 1, 1), dtype=np.uint64)
        acc = np.zeros(max(n - 1, 1), dtype=np.uint64)
        check(lib().lg_exchange_state(self._h, _p(cot), _p(att), _p(acc)))
        return cot, att[:n - 1], acc[:n - 1]

    def chain(self, c) -> "LoopWorker":
        h = lib().lg_exchange_chain(self._h, int(c))
        if not h:
            raise IndexError(c)
        p = Params.from_buffer_copy(self.params)
        p.seed = chain_seed(self.params.seed, c)
        return LoopWorker(p, _handle=h, _owner=self)


def chain_seed(seed: int, i: int) -> int:
    """SEED of chain i of an exchange ladder created with SEED = seed."""
    return int(lib().lg_exchange_chain_seed(int(seed), int(i)))


def request_bytes(params: Params) -> float:
    """Device bytes the server's admission control expects a request to need."""
    return lib().lg_request_bytes(ctypes.byref(params))


class Server:
    """Request server with continuous batching (lg_server_*)."""

    def __init__(self, budget_bytes=None, sweeps_per_tick=None, rebuild_interval_s=None,
                 max_active=None, lanes=None):
        c = ServerConfig()
        lib().lg_server_config_default(ctypes.byref(c))
        if budget_bytes is not None:
            c.budget_bytes = float(budget_bytes)
        if sweeps_per_tick is not None:
            c.sweeps_per_tick = int(sweeps_per_tick)
        if rebuild_interval_s is not None:
            c.rebuild_interval_s = float(rebuild_interval_s)
        if max_active is not None:
            c.max_active = int(max_active)
        if lanes is not None:
            c.lanes = int(lanes)
        h = ctypes.c_void_p()
        check(lib().lg_server_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h

    def submit(self, params: Params) -> int:
        i = ctypes.c_uint64()
        check(lib().lg_server_submit(self._h, ctypes.byref(params), ctypes.byref(i)))
        return i.value

    def poll(self, cap=4096):
        arr = (Result * cap)()
        n = ctypes.c_int()
        check(lib().lg_server_poll(self._h, arr, cap, ctypes.byref(n)))
        out = []
        for r in arr[:n.value]:
            out.append({"id": r.id, "status": r.status, "t_submit": r.t_submit,
                        "t_start": r.t_start, "t_finish": r.t_finish, "sweeps": r.sweeps,
                        "sites": r.sites, "obs": _obs_dict(r.obs) if r.status == 0 else None})
        return out

    def wait(self, timeout_s=600.0):
        check(lib().lg_server_wait(self._h, float(timeout_s)))

    def stats(self):
        st = ServerStats()
        check(lib().lg_server_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self._h:
            lib().lg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uf_label(lattice, L, bonds, graphs):
    """Reference-numbered cluster labels of a time-ordered configuration, on the GPU."""
    bonds = np.ascontiguousarray(bonds, dtype=np.int32)
    graphs = np.ascontiguousarray(graphs, dtype=np.int32)
    cap = L ** lattice + len(bonds) + 1
    lab = np.zeros(cap, dtype=np.int32)
    nf, nc = ctypes.c_int64(), ctypes.c_int64()
    check(lib().lg_uf_label(int(lattice), int(L), len(bonds), _p(bonds), _p(graphs), _p(lab), cap,
                            ctypes.byref(nf), ctypes.byref(nc)))
    return lab[:nf.value].copy(), nc.value


def uf_label_static(lattice, L, nops, d_bonds, d_graphs, d_labels, stream=0):
    """Allocation-free labelling: device pointers in and out (see lg_uf_label_static)."""
    nf, nc = ctypes.c_int64(), ctypes.c_int64()
    check(lib().lg_uf_label_static(int(lattice), int(L), int(nops), ctypes.c_void_p(d_bonds),
                                   ctypes.c_void_p(d_graphs), ctypes.c_void_p(d_labels),
                                   ctypes.byref(nf), ctypes.byref(nc), ctypes.c_void_p(stream)))
    return nf.value, nc.value


CHECKPOINT_BLOCK = 1 << 20


def checkpoint_checksum(blob) -> int:
    """The checksum lg_save stores in a checkpoint's last 8 bytes, computed over everything before
    them: FNV-1a (64-bit) of each 1 MiB block, over its 64-bit little-endian words and then its
    remaining bytes, and FNV-1a of those block hashes in order.  For tools that edit a blob."""
    body = bytes(blob)[:-8]
    mask = (1 << 64) - 1

    def fnv(data):
        h = 1469598103934665603
        n8 = len(data) // 8 * 8
        words = np.frombuffer(data[:n8], dtype="<u8").tolist()
        for w in words:
            h = ((h ^ w) * 1099511628211) & mask
        for x in data[n8:]:
            h = ((h ^ x) * 1099511628211) & mask
        return h

    h = 1469598103934665603
    for b0 in range(0, len(body), CHECKPOINT_BLOCK):
        h = ((h ^ fnv(body[b0:b0 + CHECKPOINT_BLOCK])) * 1099511628211) & mask
    return h


def kernel_launches() -> int:
    return lib().lg_kernel_launches()


def copy_bytes():
    """(host -> device, device -> host) bytes copied by the library so far."""
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    lib().lg_copy_bytes(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def version() -> str:
    return lib().lg_version().decode()


def exported_symbols():
    """Names declared in include/looper_gpu.h."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "looper_gpu.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(lg_[a-z_0-9]+)\s*\(", text)))
