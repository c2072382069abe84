"""Python binding of the GB300 DQMC sweep library (ctypes over include/dqmc_gb300.h).

The names follow the reference's operator interface (dqmc-framework:
DqmcWalker, Model, MeasureHandler): a Batch is a set of independent walkers,
each the equivalent of one reference MPI rank's DqmcWalker + Model + Lattice.
The CUDA library is the only compute path: if libdqmc_gb300.so is missing or
no GPU is present, calls raise instead of falling back to the CPU.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libdqmc_gb300.so")

REPULSIVE, ATTRACTIVE = 0, 1
SQUARE, CUBIC = 0, 1
RNG_MINSTD, RNG_PHILOX = 0, 1
FP64, MIXED = 0, 1
OBS_NAMES = [
    "filling_number", "double_occupancy", "kinetic_energy", "momentum_distribution",
    "local_spin_corr", "spin_density_structure_factor", "charge_density_structure_factor",
    "s_wave_pairing_corr", "equaltime_sign",
]
NUM_OBS = len(OBS_NAMES)

# every symbol include/dqmc_gb300.h declares
EXPORTS = [
    "dqmc_last_error", "dqmc_abi_version", "dqmc_batch_create", "dqmc_batch_destroy", "dqmc_set_stream",
    "dqmc_synchronize", "dqmc_fields_random", "dqmc_set_fields", "dqmc_get_fields", "dqmc_init_greens",
    "dqmc_sweep_0_to_beta", "dqmc_sweep_beta_to_0", "dqmc_get_green", "dqmc_get_config_sign",
    "dqmc_get_wrap_error", "dqmc_get_accept_count", "dqmc_get_status", "dqmc_get_observables",
    "dqmc_clear_observables", "dqmc_trace_count", "dqmc_trace_get", "dqmc_trace_clear", "dqmc_batch_info",
    "dqmc_profile_enable", "dqmc_profile_read", "dqmc_microbench_fp64", "dqmc_get_observables_all",
    "dqmc_product_check", "dqmc_product_device_noalloc", "dqmc_launch_count", "dqmc_tuning",
    "dqmc_sweep_dynamic", "dqmc_get_dynamic", "dqmc_clear_dynamic", "dqmc_get_green_dynamic", "dqmc_get_dynamic_obs",
    "dqmc_get_dynamic_r", "dqmc_measure_bins", "dqmc_set_green", "dqmc_set_wait_limit", "dqmc_tuning_products",
]
KCLASSES = ["segment", "push", "greens", "measure", "product", "metropolis", "dynamic", "dynamic_stab"]


class DqmcError(RuntimeError):
    pass


class _Desc(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int), ("L", ctypes.c_int), ("hopping_t", ctypes.c_double),
        ("onsite_u", ctypes.c_double), ("mu", ctypes.c_double), ("beta", ctypes.c_double),
        ("Lt", ctypes.c_int), ("pace", ctypes.c_int), ("checkerboard", ctypes.c_int),
        ("momentum_index", ctypes.c_int), ("seed", ctypes.c_uint64), ("lattice", ctypes.c_int),
    ]


class _Opts(ctypes.Structure):
    _fields_ = [("rng", ctypes.c_int), ("precision", ctypes.c_int), ("trace", ctypes.c_int),
                ("graphs", ctypes.c_int), ("hbm", ctypes.c_int)]


_lib = None


def load() -> ctypes.CDLL:
    """Load libdqmc_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise DqmcError(f"{LIB_PATH} not built: run __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, i8p, i64p, ip = (ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int8),
                             ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int))
    c = ctypes.c_int
    sig = {
        "dqmc_last_error": (ctypes.c_char_p, []), "dqmc_abi_version": (c, []),
        "dqmc_batch_create": (c, [ctypes.POINTER(_Desc), c, ctypes.POINTER(_Opts), ctypes.POINTER(vp)]),
        "dqmc_batch_destroy": (c, [vp]), "dqmc_set_stream": (c, [vp, vp]), "dqmc_synchronize": (c, [vp]),
        "dqmc_fields_random": (c, [vp, c]), "dqmc_set_fields": (c, [vp, c, i8p]),
        "dqmc_get_fields": (c, [vp, c, i8p]), "dqmc_init_greens": (c, [vp]),
        "dqmc_sweep_0_to_beta": (c, [vp, c]), "dqmc_sweep_beta_to_0": (c, [vp, c]),
        "dqmc_get_green": (c, [vp, c, c, dp]), "dqmc_get_config_sign": (c, [vp, c, dp]),
        "dqmc_get_wrap_error": (c, [vp, c, dp]), "dqmc_get_accept_count": (c, [vp, c, i64p]),
        "dqmc_get_status": (c, [vp, c, ip]), "dqmc_get_observables": (c, [vp, c, dp, i64p]),
        "dqmc_clear_observables": (c, [vp]), "dqmc_trace_count": (c, [vp, ip]),
        "dqmc_trace_get": (c, [vp, c, c, c, dp]), "dqmc_trace_clear": (c, [vp]),
        "dqmc_batch_info": (c, [vp, ip, i64p]),
        "dqmc_profile_enable": (c, [vp, c]), "dqmc_profile_read": (c, [vp, c, dp, i64p]),
        "dqmc_microbench_fp64": (c, [dp]), "dqmc_get_observables_all": (c, [vp, dp, i64p]),
        "dqmc_product_check": (c, [c, dp, dp, dp]),
        "dqmc_product_device_noalloc": (c, [c, vp, vp, vp, vp]),
        "dqmc_launch_count": (c, [vp, i64p]),
        "dqmc_tuning": (c, [vp, ip, ip, ip, ip, ip, ctypes.POINTER(ctypes.c_float)]),
        "dqmc_sweep_dynamic": (c, [vp, ip, c]), "dqmc_get_dynamic": (c, [vp, c, dp, i64p]),
        "dqmc_clear_dynamic": (c, [vp]), "dqmc_get_green_dynamic": (c, [vp, c, c, c, dp]),
        "dqmc_get_dynamic_obs": (c, [vp, c, dp, dp, dp]),
        "dqmc_get_dynamic_r": (c, [vp, c, dp]),
        "dqmc_measure_bins": (c, [vp, c, c, c, dp]),
        "dqmc_set_green": (c, [vp, c, c, dp]),
        "dqmc_set_wait_limit": (c, [vp, c]),
        "dqmc_tuning_products": (c, [vp, ip, ip, ip, ctypes.POINTER(ctypes.c_float)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise DqmcError(f"status {rc}: {load().dqmc_last_error().decode()}")


@dataclass
class WalkerDesc:
    """Parameters of one walker (Model::set_model_params + Lattice + DqmcWalker)."""
    model: int = REPULSIVE
    L: int = 4
    t: float = 1.0
    U: float = 4.0
    mu: float = 0.0
    beta: float = 4.0
    Lt: int = 80
    pace: int = 10
    checkerboard: bool = False
    momentum_index: int = -1
    seed: int = 0
    lattice: int = SQUARE

    @property
    def N(self) -> int:
        return self.L ** (3 if self.lattice == CUBIC else 2)

    def _c(self) -> _Desc:
        return _Desc(self.model, self.L, self.t, abs(self.U), self.mu, self.beta, self.Lt, self.pace,
                     int(self.checkerboard), self.momentum_index, self.seed, self.lattice)


class Batch:
    """A batch of independent walkers on the current CUDA device."""

    def __init__(self, walkers, rng=RNG_MINSTD, precision=FP64, trace=False, graphs=True, hbm=False):
        L = load()
        self.walkers = list(walkers)
        arr = (_Desc * len(self.walkers))(*[w._c() for w in self.walkers])
        opts = _Opts(rng, precision, int(trace), int(graphs), int(hbm))
        h = ctypes.c_void_p()
        _check(L.dqmc_batch_create(arr, len(self.walkers), ctypes.byref(opts), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().dqmc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.walkers)

    # --- set-up ------------------------------------------------------------
    def set_stream(self, stream_ptr: int):
        _check(load().dqmc_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def synchronize(self):
        _check(load().dqmc_synchronize(self.h))

    def fields_random(self, w: int):
        """Model::set_bosonic_fields_to_random with the walker's own engine."""
        _check(load().dqmc_fields_random(self.h, w))

    def _walker(self, w: int) -> "WalkerDesc":
        if not 0 <= w < len(self.walkers):
            raise IndexError(f"walker {w} outside the batch of {len(self.walkers)}")
        return self.walkers[w]

    def set_fields(self, w: int, fields):
        """Walker w's fields, [Lt][N] of +1/-1 (the library reads exactly Lt * N bytes)."""
        d = self._walker(w)
        f = np.ascontiguousarray(fields, dtype=np.int8)
        if f.size != d.Lt * d.N:
            raise ValueError(f"fields of walker {w}: {f.size} values, expected Lt * N = {d.Lt * d.N}")
        _check(load().dqmc_set_fields(self.h, w, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))

    def fields(self, w: int) -> np.ndarray:
        d = self._walker(w)
        f = np.zeros((d.Lt, d.N), dtype=np.int8)
        _check(load().dqmc_get_fields(self.h, w, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return f

    def init_greens(self):
        """initial_svd_stacks + initial_greens_functions + initial_config_sign."""
        _check(load().dqmc_init_greens(self.h))

    # --- sweeps --------------------------------------------------------------
    def sweep_0_to_beta(self, measure: bool = False):
        _check(load().dqmc_sweep_0_to_beta(self.h, int(measure)))

    def sweep_beta_to_0(self, measure: bool = False):
        _check(load().dqmc_sweep_beta_to_0(self.h, int(measure)))

    # --- accessors -------------------------------------------------------------
    def green(self, w: int, spin: int) -> np.ndarray:
        N = self._walker(w).N
        g = np.zeros((N, N), order="F")
        _check(load().dqmc_get_green(self.h, w, spin, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return g

    def set_green(self, w: int, spin: int, g):
        """Overwrite walker w's equal-time G of one spin (restart and test hook)."""
        N = self._walker(w).N
        g = np.asfortranarray(g, dtype=np.float64)
        if g.shape != (N, N):
            raise ValueError(f"G of walker {w}: shape {g.shape}, expected ({N}, {N})")
        _check(load().dqmc_set_green(self.h, w, spin, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def config_sign(self, w: int) -> float:
        v = ctypes.c_double()
        _check(load().dqmc_get_config_sign(self.h, w, ctypes.byref(v)))
        return v.value

    def wrap_error(self, w: int) -> float:
        v = ctypes.c_double()
        _check(load().dqmc_get_wrap_error(self.h, w, ctypes.byref(v)))
        return v.value

    def accept_count(self, w: int) -> int:
        v = ctypes.c_int64()
        _check(load().dqmc_get_accept_count(self.h, w, ctypes.byref(v)))
        return v.value

    def status(self, w: int) -> int:
        v = ctypes.c_int()
        _check(load().dqmc_get_status(self.h, w, ctypes.byref(v)))
        return v.value

    def observables(self, w: int):
        s = np.zeros(NUM_OBS)
        c = np.zeros(NUM_OBS, dtype=np.int64)
        _check(load().dqmc_get_observables(self.h, w, s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           c.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return s, c

    def observables_all(self):
        n = len(self.walkers)
        s = np.zeros((n, NUM_OBS))
        c = np.zeros((n, NUM_OBS), dtype=np.int64)
        _check(load().dqmc_get_observables_all(self.h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               c.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return s, c

    def measure_bins(self, nbins: int, bin_size: int, sweeps_between: int = 0) -> np.ndarray:
        """Dqmc::measure with device-side binning: [walker][bin][NUM_OBS] normalised bins."""
        out = np.zeros((len(self.walkers), nbins, NUM_OBS))
        _check(load().dqmc_measure_bins(self.h, nbins, bin_size, sweeps_between,
                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def clear_observables(self):
        _check(load().dqmc_clear_observables(self.h))

    def trace(self, w: int) -> np.ndarray:
        n = ctypes.c_int()
        _check(load().dqmc_trace_count(self.h, ctypes.byref(n)))
        N = self._walker(w).N
        out = np.zeros((n.value, 2, N, N))
        for k in range(n.value):
            for s in range(2):
                g = np.zeros((N, N), order="F")
                _check(load().dqmc_trace_get(self.h, w, k, s, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
                out[k, s] = g
        return out

    def trace_clear(self):
        _check(load().dqmc_trace_clear(self.h))

    def set_wait_limit(self, limit: int):
        """Test hook: iteration limit of the tensor-core products' operand waits (-1: default)."""
        _check(load().dqmc_set_wait_limit(self.h, int(limit)))

    def profile_enable(self, on: bool = True):
        _check(load().dqmc_profile_enable(self.h, int(on)))

    def profile_read(self) -> dict:
        out = {}
        for k, name in enumerate(KCLASSES):
            ms = ctypes.c_double()
            n = ctypes.c_int64()
            _check(load().dqmc_profile_read(self.h, k, ctypes.byref(ms), ctypes.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def sweep_dynamic(self, taus):
        """DqmcWalker::sweep_for_dynamic_greens + G(k, tau) at the listed tau (fields fixed)."""
        self._taus = [int(t) for t in taus]
        arr = (ctypes.c_int * max(1, len(self._taus)))(*self._taus)
        _check(load().dqmc_sweep_dynamic(self.h, arr, len(self._taus)))

    def dynamic(self, w: int):
        """(sums, counts) of sign * G(k, tau) per listed tau for walker w."""
        n = len(getattr(self, "_taus", []))
        s = np.zeros(max(n, 1))
        c = (ctypes.c_int64 * max(n, 1))()
        _check(load().dqmc_get_dynamic(self.h, w, s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), c))
        return s[:n], np.array(list(c))[:n]

    def dynamic_obs(self, w: int):
        """(dos, chi, rho) sums per listed tau for walker w: density of states, local
        dynamic spin susceptibility and the superfluid-stiffness contribution of that tau."""
        n = len(getattr(self, "_taus", []))
        d, c, r = (np.zeros(max(n, 1)) for _ in range(3))
        P = ctypes.POINTER(ctypes.c_double)
        _check(load().dqmc_get_dynamic_obs(self.h, w, d.ctypes.data_as(P), c.ctypes.data_as(P), r.ctypes.data_as(P)))
        return d[:n], c[:n], r[:n]

    def dynamic_r(self, w: int) -> np.ndarray:
        """[tau][r] sums of sign * 0.5 sum_i (G_up + G_dn)(i + r, i) / N per displacement r."""
        n = len(getattr(self, "_taus", []))
        out = np.zeros((max(n, 1), self._walker(w).N))
        _check(load().dqmc_get_dynamic_r(self.h, w, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out[:n]

    def dynamic_greens_k(self, w: int, momenta) -> np.ndarray:
        """G(k,tau) sums [k][tau] for the momenta (kx, ky) or (kx, ky, kz) (measure_greens_functions):
        sum_r cos(-k.r) S(r)."""
        d = self._walker(w)
        L = d.L
        r = np.arange(d.N)
        coords = [r % L, (r // L) % L, r // (L * L)]
        ff = np.array([np.cos(-sum(c * k for c, k in zip(coords, kv))) for kv in momenta])  # [k][r]
        return ff @ self.dynamic_r(w).T

    def clear_dynamic(self):
        _check(load().dqmc_clear_dynamic(self.h))

    def green_dynamic(self, w: int, which: int, spin: int) -> np.ndarray:
        """G(beta, 0) (which 0) or G(0, beta) (which 1) after the last dynamic half-sweep."""
        N = self._walker(w).N
        g = np.zeros((N, N), order="F")
        _check(load().dqmc_get_green_dynamic(self.h, w, which, spin, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return g

    def tuning(self) -> dict:
        """The autotuner's picks and every candidate's time: the Metropolis update kind (delayed
        block k, tc_flush 0-3) and the tensor-core products' tile shape (product_tile 0: 128 x 32
        tiles up to N = 256 and 128 x 64 above, 1: the other way round)."""
        kd, tc, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ck = (ctypes.c_int * 8)()
        ct = (ctypes.c_int * 8)()
        cm = (ctypes.c_float * 8)()
        _check(load().dqmc_tuning(self.h, ctypes.byref(kd), ctypes.byref(tc), ctypes.byref(n), ck, ct, cm))
        sh, ns = ctypes.c_int(), ctypes.c_int()
        cs = (ctypes.c_int * 2)()
        csm = (ctypes.c_float * 2)()
        _check(load().dqmc_tuning_products(self.h, ctypes.byref(sh), ctypes.byref(ns), cs, csm))
        return {"kd": kd.value, "tc_flush": tc.value,
                "candidates": [{"kd": ck[i], "tc_flush": ct[i], "ms_per_slice": cm[i]} for i in range(n.value)],
                "product_tile": sh.value,
                "product_candidates": [{"tile": cs[i], "ms_per_slice": csm[i]} for i in range(ns.value)]}

    def launch_count(self) -> int:
        v = ctypes.c_int64()
        _check(load().dqmc_launch_count(self.h, ctypes.byref(v)))
        return v.value

    def updates_per_half_sweep(self) -> int:
        nw = ctypes.c_int()
        u = ctypes.c_int64()
        _check(load().dqmc_batch_info(self.h, ctypes.byref(nw), ctypes.byref(u)))
        return u.value


def product_check(a, b):
    """C = A B through the mixed-precision product engine (column-major doubles)."""
    a = np.asfortranarray(a, dtype=np.float64)
    b = np.asfortranarray(b, dtype=np.float64)
    n = a.shape[0]
    c = np.zeros((n, n), order="F")
    dp = ctypes.POINTER(ctypes.c_double)
    _check(load().dqmc_product_check(n, a.ctypes.data_as(dp), b.ctypes.data_as(dp), c.ctypes.data_as(dp)))
    return c


def microbench_fp64() -> float:
    """Measured FP64 FMA throughput of the current device in GFLOP/s."""
    v = ctypes.c_double()
    _check(load().dqmc_microbench_fp64(ctypes.byref(v)))
    return v.value


def write_bin(sums, counts):
    """MeasureHandler::normalize_stats for one bin (measure_handler.cpp:170-189):
    observables divided by count and by the mean sign; the sign bin is |<sign>|."""
    sums = np.asarray(sums, dtype=np.float64)
    counts = np.asarray(counts, dtype=np.float64)
    sign = sums[-1] / counts[-1]
    out = sums / (counts * sign)
    out[-1] = abs(sign)
    return out
