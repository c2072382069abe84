"""ctypes front-end of the CPU oracle (test infrastructure only).

The oracle is a C++17 restatement of the reference DQMC sweep
(dqmc-framework: src/dqmc_walker.cpp, src/model/*.cpp,
src/checkerboard/square.cpp, src/svd_stack.cpp,
include/utils/numerical_stable.hpp, src/measure/measure_methods.cpp).
Only tests/, the smoke entry point and bench.py's CPU-baseline leg use it,
and only as the checker; the product path never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libdqmc_oracle.so")
SOURCES = [os.path.join(HERE, "dqmc_oracle.cpp")]

REPULSIVE, ATTRACTIVE = 0, 1
STACK_SVD, STACK_QRP = 0, 1
SQUARE, CUBIC = 0, 1
OBS_NAMES = [
    "filling_number", "double_occupancy", "kinetic_energy", "momentum_distribution",
    "local_spin_corr", "spin_density_structure_factor", "charge_density_structure_factor",
    "s_wave_pairing_corr", "equaltime_sign",
]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (FP contraction off so x86 and Arm agree)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "dqmc_oracle.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", LIB_PATH + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class Params(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int), ("L", ctypes.c_int), ("hopping_t", ctypes.c_double),
        ("onsite_u", ctypes.c_double), ("mu", ctypes.c_double), ("beta", ctypes.c_double),
        ("Lt", ctypes.c_int), ("pace", ctypes.c_int), ("checkerboard", ctypes.c_int),
        ("stack_kind", ctypes.c_int), ("momentum_index", ctypes.c_int),
        ("record_greens", ctypes.c_int), ("lattice", ctypes.c_int),
    ]


_lib = None


def _capsule_ptr(capsule) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, i8p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int8)
    sig = {
        "orc_create": (vp, [ctypes.POINTER(Params)]), "orc_destroy": (None, [vp]),
        "orc_space_size": (ctypes.c_int, [vp]), "orc_seed": (None, [vp, ctypes.c_uint]),
        "orc_draw_uniform": (ctypes.c_double, [vp]),
        "orc_set_uniforms": (None, [vp, dp, ctypes.c_size_t]),
        "orc_fields_random": (None, [vp]), "orc_set_fields": (None, [vp, i8p]),
        "orc_get_fields": (None, [vp, i8p]), "orc_init": (None, [vp]),
        "orc_sweep_0_to_beta": (None, [vp]), "orc_sweep_beta_to_0": (None, [vp]),
        "orc_sweep_dynamic": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
        "orc_get_dynamic": (None, [vp, dp, ctypes.POINTER(ctypes.c_int64)]),
        "orc_get_green_dynamic": (None, [vp, ctypes.c_int, ctypes.c_int, dp]),
        "orc_get_dynamic_obs": (None, [vp, dp, dp, dp]),
        "orc_get_dynamic_r": (None, [vp, dp]),
        "orc_measure": (None, [vp]), "orc_write_bin": (None, [vp, ctypes.c_int, dp]),
        "orc_get_accumulators": (None, [vp, dp, ctypes.POINTER(ctypes.c_int)]),
        "orc_get_green": (None, [vp, ctypes.c_int, dp]),
        "orc_set_green": (None, [vp, ctypes.c_int, dp]),
        "orc_wrap_error": (ctypes.c_double, [vp]), "orc_config_sign": (ctypes.c_double, [vp]),
        "orc_set_config_sign": (None, [vp, ctypes.c_double]),
        "orc_accept_count": (ctypes.c_int64, [vp]), "orc_trace_count": (ctypes.c_int, [vp]),
        "orc_trace_get": (None, [vp, ctypes.c_int, ctypes.c_int, dp]),
        "orc_trace_clear": (None, [vp]), "orc_trace_enable": (None, [vp, ctypes.c_int]),
        "orc_update_ratio": (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int]),
        "orc_update_greens": (None, [vp, ctypes.c_int, ctypes.c_int]),
        "orc_mult_B": (None, [vp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int]),
        "orc_mult_expK": (None, [vp, ctypes.c_int, dp]),
        "orc_get_expK": (None, [vp, ctypes.c_int, dp]), "orc_alpha": (ctypes.c_double, [vp]),
        "orc_svd": (None, [ctypes.c_int, dp, dp, dp, dp]),
        "orc_qrp_udt": (None, [ctypes.c_int, dp, dp, dp, dp]),
        "orc_greens_from_udv": (None, [ctypes.c_int, dp, dp, dp, dp]),
        "orc_num_k_stars": (ctypes.c_int, [vp]), "orc_m_point_index": (ctypes.c_int, [vp]),
        "orc_fourier_factor": (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int]),
        "orc_space_dim": (ctypes.c_int, [vp]),
        "orc_nearest_neighbour": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
        "orc_displacement": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
        "orc_k_star": (None, [vp, ctypes.c_int, dp]),
        "orc_set_lapack": (None, [vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def use_scipy_lapack(on: bool = True) -> bool:
    """Route the oracle's dgemm/dgesvd to scipy's bundled BLAS/LAPACK."""
    L = lib()
    if not on:
        L.orc_set_lapack(None, None)
        return False
    try:
        import scipy.linalg.cython_blas as cb
        import scipy.linalg.cython_lapack as cl
    except Exception:
        return False
    L.orc_set_lapack(_capsule_ptr(cb.__pyx_capi__["dgemm"]), _capsule_ptr(cl.__pyx_capi__["dgesvd"]))
    return True


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i8p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))


class Walker:
    """One reference walker (model + lattice + DqmcWalker + equal-time measure)."""

    def __init__(self, model=REPULSIVE, L=4, t=1.0, U=4.0, mu=0.0, beta=4.0, Lt=80, pace=10,
                 checkerboard=False, stack=STACK_SVD, momentum_index=-1, record=True, lattice=SQUARE):
        self.p = Params(model, L, t, abs(U), mu, beta, Lt, pace, int(checkerboard), stack,
                        momentum_index, int(record), lattice)
        self.h = lib().orc_create(ctypes.byref(self.p))
        if not self.h:
            raise ValueError("oracle: parameters rejected (lattice type, side, or checkerboard off the square lattice)")
        self.N = L ** (3 if lattice == CUBIC else 2)
        self.Lt = Lt
        self._u = None

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # rng / fields
    def seed(self, s: int):
        lib().orc_seed(self.h, s)

    def uniforms(self, n: int) -> np.ndarray:
        return np.array([lib().orc_draw_uniform(self.h) for _ in range(n)])

    def inject_uniforms(self, u):
        if u is None:
            self._u = None
            lib().orc_set_uniforms(self.h, None, 0)
            return
        self._u = np.ascontiguousarray(u, dtype=np.float64)
        lib().orc_set_uniforms(self.h, _dp(self._u), self._u.size)

    def fields_random(self):
        lib().orc_fields_random(self.h)

    def set_fields(self, f):
        f = np.ascontiguousarray(f, dtype=np.int8).reshape(self.Lt, self.N)
        lib().orc_set_fields(self.h, _i8p(f))

    def fields(self) -> np.ndarray:
        f = np.zeros((self.Lt, self.N), dtype=np.int8)
        lib().orc_get_fields(self.h, _i8p(f))
        return f

    # walker
    def init(self):
        lib().orc_init(self.h)

    def sweep_0_to_beta(self):
        lib().orc_sweep_0_to_beta(self.h)

    def sweep_beta_to_0(self):
        lib().orc_sweep_beta_to_0(self.h)

    def measure(self):
        lib().orc_measure(self.h)

    def sweep_dynamic(self, taus):
        """sweep_for_dynamic_greens + G(k, tau) at the listed tau (fields fixed)."""
        self._taus = [int(t) for t in taus]
        arr = (ctypes.c_int * len(self._taus))(*self._taus)
        if lib().orc_sweep_dynamic(self.h, arr, len(self._taus)) != 0:
            raise RuntimeError("sweep_dynamic needs the stacks of t = 0 (after init or sweep_beta_to_0)")

    def dynamic(self):
        """(sums, counts) of sign * G(k, tau) per listed tau."""
        n = len(self._taus)
        s = np.zeros(n)
        c = (ctypes.c_int64 * n)()
        lib().orc_get_dynamic(self.h, _dp(s), c)
        return s, np.array(list(c))

    def dynamic_obs(self):
        """(dos, chi, rho) sums per listed tau: density of states, dynamic spin
        susceptibility and the superfluid-stiffness contribution of that tau."""
        n = len(self._taus)
        d, c, r = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().orc_get_dynamic_obs(self.h, _dp(d), _dp(c), _dp(r))
        return d, c, r

    def dynamic_r(self) -> np.ndarray:
        """[tau][r] sums of sign * 0.5 sum_i (G_up + G_dn)(i + r, i) / N."""
        out = np.zeros((len(self._taus), self.N))
        lib().orc_get_dynamic_r(self.h, _dp(out))
        return out

    def green_dynamic(self, which: int, spin: int) -> np.ndarray:
        """which 0: G(t, 0), 1: G(0, t) after the last dynamic sweep (t = beta)."""
        g = np.zeros((self.N, self.N), order="F")
        lib().orc_get_green_dynamic(self.h, which, spin, _dp(g))
        return g

    def write_bin(self) -> np.ndarray:
        out = np.zeros(len(OBS_NAMES))
        lib().orc_write_bin(self.h, 0, _dp(out))
        return out

    def accumulators(self):
        s = np.zeros(len(OBS_NAMES))
        c = (ctypes.c_int * len(OBS_NAMES))()
        lib().orc_get_accumulators(self.h, _dp(s), c)
        return s, np.array(list(c))

    def green(self, spin: int) -> np.ndarray:
        g = np.zeros((self.N, self.N), order="F")
        lib().orc_get_green(self.h, spin, _dp(g))
        return g

    def set_green(self, spin: int, g):
        g = np.asfortranarray(g, dtype=np.float64)
        lib().orc_set_green(self.h, spin, _dp(g))

    @property
    def wrap_error(self) -> float:
        return lib().orc_wrap_error(self.h)

    @property
    def sign(self) -> float:
        return lib().orc_config_sign(self.h)

    @sign.setter
    def sign(self, s: float):
        lib().orc_set_config_sign(self.h, float(s))

    @property
    def accepts(self) -> int:
        return lib().orc_accept_count(self.h)

    @property
    def alpha(self) -> float:
        return lib().orc_alpha(self.h)

    def trace(self, on=True):
        lib().orc_trace_enable(self.h, int(on))

    def trace_clear(self):
        lib().orc_trace_clear(self.h)

    def trace_get(self):
        n = lib().orc_trace_count(self.h)
        out = np.zeros((n, 2, self.N, self.N))
        for k in range(n):
            for s in range(2):
                g = np.zeros((self.N, self.N), order="F")
                lib().orc_trace_get(self.h, k, s, _dp(g))
                out[k, s] = g
        return out

    # model pieces
    def ratio(self, eff_t: int, i: int) -> float:
        return lib().orc_update_ratio(self.h, eff_t, i)

    def update_greens(self, eff_t: int, i: int):
        lib().orc_update_greens(self.h, eff_t, i)

    def mult_B(self, which: int, m, t: int, spin: int) -> np.ndarray:
        m = np.asfortranarray(m, dtype=np.float64).copy(order="F")
        lib().orc_mult_B(self.h, which, _dp(m), t, spin)
        return m

    def mult_expK(self, which: int, m) -> np.ndarray:
        m = np.asfortranarray(m, dtype=np.float64).copy(order="F")
        lib().orc_mult_expK(self.h, which, _dp(m))
        return m

    def dense(self, which: int) -> np.ndarray:
        m = np.zeros((self.N, self.N), order="F")
        lib().orc_get_expK(self.h, which, _dp(m))
        return m

    def num_k_stars(self) -> int:
        return lib().orc_num_k_stars(self.h)

    def m_point(self) -> int:
        return lib().orc_m_point_index(self.h)

    def fourier(self, disp: int, k: int) -> float:
        return lib().orc_fourier_factor(self.h, disp, k)

    def space_dim(self) -> int:
        return lib().orc_space_dim(self.h)

    def nearest_neighbour(self, i: int, direction: int) -> int:
        """LatticeBase::NearestNeighbour: direction < 2 dim, +x, +y (, +z), -x, -y (, -z)."""
        if not 0 <= direction < 2 * self.space_dim() or not 0 <= i < self.N:
            raise IndexError("site or direction out of range")
        return lib().orc_nearest_neighbour(self.h, i, direction)

    def displacement(self, i: int, j: int) -> int:
        if not (0 <= i < self.N and 0 <= j < self.N):
            raise IndexError("site out of range")
        return lib().orc_displacement(self.h, i, j)

    def k_star(self, k: int) -> np.ndarray:
        if not 0 <= k < self.num_k_stars():
            raise IndexError("k star out of range")
        out = np.zeros(3)
        lib().orc_k_star(self.h, k, _dp(out))
        return out[: self.space_dim()]


def svd(a):
    a = np.asfortranarray(a, dtype=np.float64)
    n = a.shape[0]
    u, s, v = np.zeros((n, n), order="F"), np.zeros(n), np.zeros((n, n), order="F")
    lib().orc_svd(n, _dp(a), _dp(u), _dp(s), _dp(v))
    return u, s, v


def qrp_udt(a):
    a = np.asfortranarray(a, dtype=np.float64)
    n = a.shape[0]
    u, d, t = np.zeros((n, n), order="F"), np.zeros(n), np.zeros((n, n), order="F")
    lib().orc_qrp_udt(n, _dp(a), _dp(u), _dp(d), _dp(t))
    return u, d, t


def greens_from_udv(u, d, f):
    u = np.asfortranarray(u, dtype=np.float64)
    f = np.asfortranarray(f, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    n = u.shape[0]
    g = np.zeros((n, n), order="F")
    lib().orc_greens_from_udv(n, _dp(u), _dp(d), _dp(f), _dp(g))
    return g


def analyse(bins: np.ndarray):
    """Mean and error over bins (include/measure/observable.h:179-193)."""
    bins = np.asarray(bins, dtype=np.float64)
    nb = bins.shape[0]
    mean = bins.sum(axis=0) / nb
    err = np.sqrt(np.maximum((bins ** 2).sum(axis=0) / nb - mean ** 2, 0.0)) / np.sqrt(nb - 1)
    return mean, err


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
