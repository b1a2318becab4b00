"""Python mirror of the reference's Hermite4GPU integrator interface.

``NbodySystem`` holds what src/include/NbodySystem.hpp:98-134 holds for the
hot path (n, e2, eta, integration and log times, host arrays h_r, h_v, ...),
``Hermite4GPU`` has the reference's method names
(src/include/gpu/Hermite4GPU.cuh:100-144, src/include/Hermite4.hpp:60-63)
and drives the C ABI of include/gravidy_gb300.h.  Device state is
authoritative; the host arrays are refreshed by ``sync_host()`` (for logs and
snapshots), as the reference's arrays would be after its copies.
"""
from __future__ import annotations

import ctypes as C
import sys
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .io import EnergyLog, InputData, read_input_file

D_TIME_MIN = 2.0 ** -23   # common.hpp:122
D_TIME_MAX = 0.125        # common.hpp:129
ETA_S = np.float32(0.01)  # common.hpp:114
ETA_N = np.float32(0.01)  # common.hpp:119
E_SOFT = 1e-4             # common.hpp:107

FORCES_DTYPE = np.dtype([("a", "<f8", 3), ("a1", "<f8", 3)])


def e2_from_softening(softening: float) -> float:
    """NbodySystem::e2 (NbodySystem.cpp:50): the float product, as double."""
    s = np.float32(softening)
    return float(np.float32(s * s))


@dataclass
class NbodySystem:
    """Particle system and run parameters (NbodySystem.hpp:98-134)."""
    mass: np.ndarray
    pos: np.ndarray
    vel: np.ndarray
    softening: float = E_SOFT
    eta: float = float(ETA_N)
    integration_time: float = 1.0
    interval_time: float = D_TIME_MAX
    ids: np.ndarray | None = None
    snapshot_time: float = 0.0
    iterations: int = 0
    e2_value: float | None = None   # exact e2 (a resumed run); else from softening
    h_r: np.ndarray = field(init=False)
    h_v: np.ndarray = field(init=False)

    def __post_init__(self):
        self.mass = np.asarray(self.mass, np.float32).astype(np.float64)
        n = len(self.mass)
        self.h_r = np.zeros((n, 4))
        self.h_r[:, :3] = self.pos
        self.h_r[:, 3] = self.mass
        self.h_v = np.zeros((n, 4))
        self.h_v[:, :3] = self.vel
        if self.ids is None:
            self.ids = np.arange(n, dtype=np.uint32)
        self.eta = float(np.float32(self.eta))
        self.integration_time = float(np.float32(self.integration_time))
        self.interval_time = float(np.float32(self.interval_time))

    @property
    def n(self) -> int:
        return len(self.mass)

    @property
    def e2(self) -> float:
        if self.e2_value is not None:
            return float(self.e2_value)
        return e2_from_softening(self.softening)

    @classmethod
    def from_input_file(cls, path: str, **kw) -> "NbodySystem":
        data: InputData = read_input_file(path)
        return cls(data.mass, data.pos, data.vel, ids=data.ids,
                   snapshot_time=data.snapshot_time, **kw)


class Hermite4GPU:
    """GPU block-timestep Hermite4 integrator with the reference's methods."""

    def __init__(self, ns: NbodySystem, mode: str = "fp64", dt_min: float = D_TIME_MIN,
                 dt_max: float = D_TIME_MAX):
        self.L = _lib.load()
        self.ns = ns
        self.n = ns.n
        self.mode = mode
        h = C.c_void_p()
        r4 = np.ascontiguousarray(ns.h_r, dtype=np.float64)
        v4 = np.ascontiguousarray(ns.h_v, dtype=np.float64)
        _lib.check(self.L.h4_create(C.byref(h), self.n, ns.e2, C.c_float(ns.eta),
                                    r4.ctypes.data, v4.ctypes.data, _lib.MODES[mode]))
        self.h = h
        if dt_min != D_TIME_MIN or dt_max != D_TIME_MAX:
            _lib.check(self.L.h4_set_dt_limits(self.h, dt_min, dt_max))
        self.interactions = 0
        self.nsteps = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.h4_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- the reference's methods ------------------------------------------------
    def init_acc_jrk(self):
        _lib.check(self.L.h4_init_acc_jrk(self.h))

    def init_dt(self, atime: float = 1.0e10, eta: float = float(ETA_S), itime: float = 0.0) -> float:
        a = C.c_double(atime)
        _lib.check(self.L.h4_init_dt(self.h, C.byref(a), C.c_float(eta), itime))
        return a.value

    def find_particles_to_move(self, itime: float) -> int:
        n = C.c_uint()
        _lib.check(self.L.h4_find_particles_to_move(self.h, itime, C.byref(n)))
        return n.value

    def save_old_acc_jrk(self, nact: int):
        _lib.check(self.L.h4_save_old_acc_jrk(self.h, nact))

    def predicted_pos_vel(self, itime: float):
        _lib.check(self.L.h4_predicted_pos_vel(self.h, itime))

    def update_acc_jrk(self, nact: int):
        _lib.check(self.L.h4_update_acc_jrk(self.h, nact))

    def correction_pos_vel(self, itime: float, nact: int):
        _lib.check(self.L.h4_correction_pos_vel(self.h, itime, nact))

    def next_integration_time(self) -> float:
        a = C.c_double()
        _lib.check(self.L.h4_next_integration_time(self.h, C.byref(a)))
        return a.value

    def get_energy_gpu(self) -> float:
        k, p, e = C.c_double(), C.c_double(), C.c_double()
        _lib.check(self.L.h4_get_energy(self.h, C.byref(k), C.byref(p), C.byref(e)))
        self.ekin, self.epot = k.value, p.value
        return e.value

    # -- fused paths ------------------------------------------------------------
    def step(self, atime: float):
        """One block step on the device; returns (nact, itime, next atime)."""
        a, it, n = C.c_double(atime), C.c_double(), C.c_uint()
        _lib.check(self.L.h4_step(self.h, C.byref(a), C.byref(it), C.byref(n)))
        return n.value, it.value, a.value

    def advance(self, t_stop: float, t_log: float, atime: float):
        """Device-resident block steps until itime >= t_stop or >= t_log."""
        a, it = C.c_double(atime), C.c_double()
        st = (C.c_double * 5)()
        _lib.check(self.L.h4_advance(self.h, t_stop, t_log, C.byref(a), C.byref(it), st))
        return it.value, a.value, int(st[0]), int(st[1]), int(st[2]), int(st[4])

    def integration(self, log: EnergyLog | None = None, fused: bool = True):
        """Hermite4GPU::integration (Hermite4GPU_integration.cpp:38-124):
        init, then block steps to ns.integration_time with an energy log row
        at t = 0 and every interval_time.  Returns the EnergyLog."""
        ns = self.ns
        log = log if log is not None else EnergyLog()
        t0 = time.perf_counter()
        itime = ns.snapshot_time
        self.init_acc_jrk()
        atime = self.init_dt(1.0e10, float(ETA_S), itime)
        e = self.get_energy_gpu()
        log.row(itime, ns.iterations, self.nsteps, e, time.perf_counter() - t0)
        out = 1
        t_end = ns.integration_time
        while itime < t_end:
            t_log = float(np.float32(np.float32(ns.interval_time) * np.float32(out)))
            if fused:
                itime, atime, steps, psteps, inter, last_nact = self.advance(t_end, t_log, atime)
                ns.iterations += steps
                self.nsteps += psteps
                self.interactions += inter
            else:
                itime = atime
                nact = self.find_particles_to_move(itime)
                self.save_old_acc_jrk(nact)
                self.predicted_pos_vel(itime)
                self.update_acc_jrk(nact)
                self.correction_pos_vel(itime, nact)
                self.interactions += nact * self.n
                atime = self.next_integration_time()
                ns.iterations += 1
                self.nsteps += nact
                last_nact = nact
            if itime >= t_log:
                # the reference logs before counting the step (Hermite4GPU_integration.cpp:102-121)
                it_log = ns.iterations - 1
                ns_log = self.nsteps - last_nact
                log.row(itime, it_log, ns_log, self.get_energy_gpu(), time.perf_counter() - t0,
                        self.interactions, 0.0)
                out += 1
        return log

    # -- state transfer -----------------------------------------------------------
    def download(self) -> dict:
        n = self.n
        out = {"r": np.zeros((n, 4)), "v": np.zeros((n, 4)), "f": np.zeros((n, 6)),
               "old": np.zeros((n, 6)), "a2": np.zeros((n, 3)), "a3": np.zeros((n, 3)),
               "t": np.zeros(n), "dt": np.zeros(n), "move": np.zeros(n, np.uint32)}
        _lib.check(self.L.h4_download(self.h, *[out[k].ctypes.data for k in
                                                ("r", "v", "f", "old", "a2", "a3", "t", "dt", "move")]))
        return out

    def download_predicted(self):
        pr, pv = np.zeros((self.n, 4)), np.zeros((self.n, 4))
        _lib.check(self.L.h4_download_predicted(self.h, pr.ctypes.data, pv.ctypes.data))
        return pr, pv

    def upload(self, r=None, v=None, f=None, old=None, t=None, dt=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (r, v, f, old, t, dt)]
        _lib.check(self.L.h4_upload(self.h, *[_lib.ptr(a) for a in arrs]))

    def restore(self, state: dict, atime: float):
        """Continue from a saved state (r, v, f, t, dt) with next block time
        atime, without recomputing forces or timesteps."""
        arrs = [np.ascontiguousarray(state[k], dtype=np.float64) for k in ("r", "v", "f", "t", "dt")]
        _lib.check(self.L.h4_restore(self.h, *[a.ctypes.data for a in arrs], float(atime)))

    def save_checkpoint(self, path: str, itime: float, atime: float, **scalars):
        from .checkpoint import write_checkpoint
        ns = self.ns
        sc = dict(e2=ns.e2, eta=ns.eta, itime=itime, atime=atime, iterations=ns.iterations,
                  nsteps=self.nsteps, interactions=self.interactions)
        sc.update(scalars)
        write_checkpoint(path, self.download(), sc, ns.ids)

    @classmethod
    def from_checkpoint(cls, path: str, mode: str = "fp64", **ns_kw):
        """(integrator, itime, atime, scalars) continuing the saved run."""
        from .checkpoint import read_checkpoint
        state, sc, ids = read_checkpoint(path)
        ns = NbodySystem(state["r"][:, 3], state["r"][:, :3], state["v"][:, :3], ids=ids,
                         eta=sc["eta"], e2_value=sc["e2"], **ns_kw)
        g = cls(ns, mode=mode)
        g.restore(state, sc["atime"])
        ns.iterations = int(sc["iterations"])
        g.nsteps = int(sc["nsteps"])
        g.interactions = int(sc["interactions"])
        return g, sc["itime"], sc["atime"], sc

    def sync_host(self):
        st = self.download()
        self.ns.h_r[:] = st["r"]
        self.ns.h_v[:] = st["v"]
        return st

    def forces_for(self, pr: np.ndarray, pv: np.ndarray, move: np.ndarray) -> np.ndarray:
        """acc/jerk of move[] against all particles, from given predictors
        (overwrites the handle's predicted arrays)."""
        pr = np.ascontiguousarray(pr, np.float64)
        pv = np.ascontiguousarray(pv, np.float64)
        mv = np.ascontiguousarray(move, np.uint32)
        out = np.zeros((len(mv), 6))
        _lib.check(self.L.h4_forces_for(self.h, pr.ctypes.data, pv.ctypes.data, len(mv),
                                        mv.ctypes.data, out.ctypes.data))
        return out

    def set_mixed_threshold(self, nact_threshold: int):
        _lib.check(self.L.h4_set_mixed_threshold(self.h, int(nact_threshold)))

    def set_force_mode(self, mode: str):
        _lib.check(self.L.h4_set_force_mode(self.h, _lib.MODES[mode]))
        self.mode = mode

    def last_timings(self):
        f, a = C.c_float(), C.c_float()
        _lib.check(self.L.h4_last_timings(self.h, C.byref(f), C.byref(a)))
        return f.value, a.value

    def phase_times(self) -> dict:
        """{phase: (device ms, calls)} with the reference's Gtime phase names."""
        ms = np.zeros(8)
        cnt = np.zeros(8, dtype=np.uint64)
        _lib.check(self.L.h4_phase_times(self.h, ms.ctypes.data, cnt.ctypes.data))
        return {self.L.h4_phase_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(8)}

    def nact_histogram(self) -> np.ndarray:
        out = np.zeros(32, dtype=np.uint64)
        _lib.check(self.L.h4_nact_histogram(self.h, out.ctypes.data))
        return out

    def kernel_launches(self) -> int:
        c = C.c_ulonglong()
        _lib.check(self.L.h4_kernel_launches(self.h, C.byref(c)))
        return c.value
