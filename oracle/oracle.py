"""ctypes binding of oracle/h4_oracle.c, the CPU restatement of the reference
GraviDy Hermite4 CPU path (src/include/cpu/Hermite4CPU.cpp,
src/include/Hermite4.cpp, src/include/utils/NbodyUtils.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
baseline.  Parity of the restatement with the reference is pinned by the
golden fixtures under tests/golden/ (made by the reference sources compiled
unmodified, see tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libh4oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

D_TIME_MIN = 2.0 ** -23
D_TIME_MAX = 0.125
ETA_S = np.float32(0.01)


class OrcSystem(C.Structure):
    _fields_ = [
        ("n", C.c_uint), ("e2", C.c_double), ("eta", C.c_float),
        ("dt_min", C.c_double), ("dt_max", C.c_double),
        ("r", C.c_void_p), ("v", C.c_void_p), ("f", C.c_void_p), ("old", C.c_void_p),
        ("a2", C.c_void_p), ("a3", C.c_void_p), ("t", C.c_void_p), ("dt", C.c_void_p),
        ("move", C.c_void_p), ("p", C.c_void_p), ("epot_i", C.c_void_p),
        ("max_mass", C.c_double),
    ]


class RunStats(C.Structure):
    _fields_ = [("itime", C.c_double), ("atime", C.c_double),
                ("iterations", C.c_longlong), ("nsteps", C.c_longlong),
                ("interactions", C.c_longlong), ("e_ini", C.c_double),
                ("e_last", C.c_double)]


def build() -> str:
    """Compile the restatement (make -C oracle port); returns the .so path."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(OrcSystem)
        vp, d, f, u = C.c_void_p, C.c_double, C.c_float, C.c_uint
        sig = {
            "orc_e2_from_softening": (d, [f]),
            "orc_create": (P, [u, d, f, vp, vp]),
            "orc_destroy": (None, [P]),
            "orc_set_dt_limits": (None, [P, d, d]),
            "orc_set_threads": (C.c_int, [C.c_int]),
            "orc_find_particles_to_move": (u, [P, d]),
            "orc_next_integration_time": (None, [P, C.POINTER(d)]),
            "orc_init_dt": (None, [P, C.POINTER(d), f, d]),
            "orc_save_old_acc_jrk": (None, [P, u]),
            "orc_init_acc_jrk": (None, [P]),
            "orc_update_acc_jrk": (None, [P, u]),
            "orc_predicted_pos_vel": (None, [P, d]),
            "orc_correction_pos_vel": (None, [P, d, u]),
            "orc_get_timestep_normal": (d, [P, u, f]),
            "orc_normalize_dt": (d, [P, d, d, d]),
            "orc_get_energy": (d, [P, C.POINTER(d), C.POINTER(d)]),
            "orc_forces_for": (None, [u, vp, d, u, vp, vp]),
            "orc_block_step": (u, [P, C.POINTER(d), C.POINTER(d)]),
            "orc_integrate": (C.c_int, [P, f, f, C.POINTER(RunStats), vp, C.c_int]),
            "orc_fnv1a": (C.c_ulonglong, [vp, C.c_size_t, C.c_ulonglong]),
            "orc_total_mass": (f, [P]),
            "orc_center_of_density": (None, [P, vp]),
            "orc_mass_radii": (None, [P, vp, f, C.POINTER(d), C.POINTER(d), vp]),
            "orc_nbody_attributes": (None, [P, d, f, vp, vp]),
            "orc_state_hash": (C.c_ulonglong, [P]),
            "orc_state_record": (None, [P, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def e2_from_softening(softening: float) -> float:
    return lib().orc_e2_from_softening(C.c_float(softening))


def set_threads(n: int) -> int:
    return lib().orc_set_threads(n)


def fnv1a(arr: np.ndarray) -> int:
    a = np.ascontiguousarray(arr)
    return lib().orc_fnv1a(a.ctypes.data, a.nbytes, 14695981039346656037)


PRED_DTYPE = np.dtype({"names": ["r", "v", "m"], "formats": [("<f8", 3), ("<f8", 3), "<f4"],
                       "offsets": [0, 24, 48], "itemsize": 56})


def pack_double4(pos: np.ndarray, w: np.ndarray | None = None) -> np.ndarray:
    out = np.zeros((len(pos), 4), dtype=np.float64)
    out[:, :3] = pos
    if w is not None:
        out[:, 3] = w
    return out


class Oracle:
    """One system in the CPU restatement; mirrors the Hermite4CPU methods."""

    def __init__(self, mass, pos, vel, e2: float, eta: float = 0.01,
                 dt_min: float = D_TIME_MIN, dt_max: float = D_TIME_MAX):
        L = lib()
        self.n = len(mass)
        r4 = np.ascontiguousarray(pack_double4(pos, np.asarray(mass, np.float32).astype(np.float64)))
        v4 = np.ascontiguousarray(pack_double4(vel))
        self._s = L.orc_create(self.n, float(e2), C.c_float(eta), r4.ctypes.data, v4.ctypes.data)
        if not self._s:
            raise MemoryError("orc_create failed")
        L.orc_set_dt_limits(self._s, dt_min, dt_max)

    def close(self):
        if self._s:
            lib().orc_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- views on the C arrays -------------------------------------------------
    def _view(self, field, shape, dtype):
        s = self._s.contents
        addr = getattr(s, field)
        cnt = int(np.prod(shape))
        buf = (C.c_char * (cnt * np.dtype(dtype).itemsize)).from_address(addr)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    @property
    def r(self): return self._view("r", (self.n, 4), np.float64)
    @property
    def v(self): return self._view("v", (self.n, 4), np.float64)
    @property
    def f(self): return self._view("f", (self.n, 6), np.float64)
    @property
    def old(self): return self._view("old", (self.n, 6), np.float64)
    @property
    def a2(self): return self._view("a2", (self.n, 3), np.float64)
    @property
    def a3(self): return self._view("a3", (self.n, 3), np.float64)
    @property
    def t(self): return self._view("t", (self.n,), np.float64)
    @property
    def dt(self): return self._view("dt", (self.n,), np.float64)
    @property
    def move(self): return self._view("move", (self.n,), np.uint32)
    @property
    def p(self): return self._view("p", (self.n,), PRED_DTYPE)

    # -- Hermite4 methods -------------------------------------------------------
    def init_acc_jrk(self): lib().orc_init_acc_jrk(self._s)

    def init_dt(self, itime: float = 0.0, eta: float = 0.01):
        a = C.c_double(1.0e10)
        lib().orc_init_dt(self._s, C.byref(a), C.c_float(eta), itime)
        return a.value

    def find_particles_to_move(self, itime: float) -> int:
        return lib().orc_find_particles_to_move(self._s, itime)

    def save_old_acc_jrk(self, nact: int): lib().orc_save_old_acc_jrk(self._s, nact)
    def predicted_pos_vel(self, itime: float): lib().orc_predicted_pos_vel(self._s, itime)
    def update_acc_jrk(self, nact: int): lib().orc_update_acc_jrk(self._s, nact)
    def correction_pos_vel(self, itime: float, nact: int): lib().orc_correction_pos_vel(self._s, itime, nact)

    def next_integration_time(self) -> float:
        a = C.c_double(0.0)
        lib().orc_next_integration_time(self._s, C.byref(a))
        return a.value

    def energy(self):
        k, p = C.c_double(), C.c_double()
        e = lib().orc_get_energy(self._s, C.byref(k), C.byref(p))
        return e, k.value, p.value

    def block_step(self, itime: float, atime: float):
        it, at = C.c_double(itime), C.c_double(atime)
        nact = lib().orc_block_step(self._s, C.byref(it), C.byref(at))
        return nact, it.value, at.value

    def integrate(self, t_end: float, interval: float = 0.125, max_rows: int = 4096):
        rows = np.zeros((max_rows, 4))
        st = RunStats()
        k = lib().orc_integrate(self._s, C.c_float(t_end), C.c_float(interval), C.byref(st),
                                rows.ctypes.data, max_rows)
        return st, rows[:k].copy()

    def total_mass(self) -> float:
        return lib().orc_total_mass(self._s)

    def center_of_density(self) -> np.ndarray:
        out = np.zeros(3)
        lib().orc_center_of_density(self._s, out.ctypes.data)
        return out

    def mass_radii(self, center, total_mass: float):
        c = np.ascontiguousarray(center, dtype=np.float64)
        core, half = C.c_double(), C.c_double()
        lag = np.zeros(6)
        lib().orc_mass_radii(self._s, c.ctypes.data, C.c_float(total_mass), C.byref(core), C.byref(half),
                             lag.ctypes.data)
        return core.value, half.value, lag

    def nbody_attributes(self, e_ini: float, total_mass: float, cod_state: np.ndarray) -> np.ndarray:
        """[r_virial, t_cr, r_cl, dt_cl, r_core, t_rlx, r_hm, cod.x, cod.y, cod.z];
        cod_state is updated in place (NbodyUtils::cod)."""
        out = np.zeros(10)
        lib().orc_nbody_attributes(self._s, e_ini, C.c_float(total_mass), cod_state.ctypes.data, out.ctypes.data)
        return out

    def state_hash(self) -> int:
        return lib().orc_state_hash(self._s)

    def state_record(self) -> np.ndarray:
        out = np.zeros((self.n, 15))
        lib().orc_state_record(self._s, out.ctypes.data)
        return out


def forces_for(pred: np.ndarray, e2: float, move: np.ndarray) -> np.ndarray:
    """acc/jerk of the listed particles against all others (no state)."""
    p = np.ascontiguousarray(pred, dtype=PRED_DTYPE)
    mv = np.ascontiguousarray(move, dtype=np.uint32)
    out = np.zeros((len(mv), 6))
    lib().orc_forces_for(len(p), p.ctypes.data, float(e2), len(mv), mv.ctypes.data, out.ctypes.data)
    return out


def make_predictors(mass, pos, vel) -> np.ndarray:
    p = np.zeros(len(mass), dtype=PRED_DTYPE)
    p["r"] = pos
    p["v"] = vel
    p["m"] = np.asarray(mass, np.float32)
    return p
