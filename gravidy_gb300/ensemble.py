"""Batched ensemble of independent N-body systems (C ABI h4_ens_*).

Each system is integrated exactly as a single system would be by
``Hermite4GPU.integration`` (its own block time, active set and timesteps);
all of them advance together in one persistent fused kernel per iteration,
replayed from a CUDA graph.  The tuning table (per (N, N_act) bucket: warp
items of 1-2 particles or block-tiled items of 16-512 particles, the j-chunk
length and the shared-memory j tile) comes from ``gravidy_gb300.autotune``.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _lib
from .hermite4 import ETA_S, e2_from_softening

NB_N, NB_A = 6, 8
TUNING_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "ensemble_gb300.json")


class Ensemble:
    def __init__(self, systems, mode: str = "fp64", tuning: str | dict | None = "default"):
        """systems: list of (mass, pos, vel, softening, eta)."""
        self.L = _lib.load()
        self.nsys = len(systems)
        self.n = np.array([len(s[0]) for s in systems], dtype=np.uint32)
        self.off = np.concatenate([[0], np.cumsum(self.n)]).astype(np.int64)
        total = int(self.off[-1])
        r = np.zeros((total, 4)); v = np.zeros((total, 4))
        e2 = np.zeros(self.nsys); eta = np.zeros(self.nsys, dtype=np.float32)
        for c, (m, p, vel, soft, et) in enumerate(systems):
            a, b = self.off[c], self.off[c + 1]
            r[a:b, :3] = p
            r[a:b, 3] = np.asarray(m, np.float32)
            v[a:b, :3] = vel
            e2[c] = e2_from_softening(soft)
            eta[c] = et
        self.total = total
        self.mode = mode
        h = C.c_void_p()
        _lib.check_ens(self.L.h4_ens_create(C.byref(h), self.nsys, self.n.ctypes.data, e2.ctypes.data,
                                            eta.ctypes.data, r.ctypes.data, v.ctypes.data, _lib.MODES[mode]))
        self.h = h
        if tuning == "default":
            tuning = TUNING_FILE if os.path.exists(TUNING_FILE) else None
        if tuning is not None:
            self.set_tuning(tuning)

    def close(self):
        if getattr(self, "h", None):
            self.L.h4_ens_destroy(self.h)
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

    def set_tuning(self, tuning):
        if isinstance(tuning, str):
            with open(tuning) as fh:
                tuning = json.load(fh)
        if "modes" in tuning:
            if self.mode not in tuning["modes"]:
                return
            tuning = tuning["modes"][self.mode]
        if self.mode == "mixed" and "jtile" not in tuning:
            return   # a table from before the block-tiled items were tuned: keep the built-in one
        ig = np.ascontiguousarray(np.array(tuning["ig"], dtype=np.uint32).reshape(-1))
        ch = np.ascontiguousarray(np.array(tuning["chunk"], dtype=np.uint32).reshape(-1))
        jt = np.ascontiguousarray(np.array(tuning.get("jtile", np.full(NB_N * NB_A, 256)),
                                           dtype=np.uint32).reshape(-1))
        assert ig.size == NB_N * NB_A and ch.size == NB_N * NB_A and jt.size == NB_N * NB_A
        _lib.check_ens(self.L.h4_ens_set_tuning(self.h, ig.ctypes.data, ch.ctypes.data, jt.ctypes.data))

    def set_dt_limits(self, dt_min, dt_max):
        _lib.check_ens(self.L.h4_ens_set_dt_limits(self.h, dt_min, dt_max))

    def init(self):
        _lib.check_ens(self.L.h4_ens_init(self.h))

    def advance(self, t_end):
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t_end, np.float64), (self.nsys,)))
        st = (C.c_double * 4)()
        _lib.check_ens(self.L.h4_ens_advance(self.h, t.ctypes.data, st))
        return {"steps": int(st[0]), "psteps": int(st[1]), "interactions": int(st[2]), "launches": int(st[3])}

    def energy(self):
        k = np.zeros(self.nsys); p = np.zeros(self.nsys)
        _lib.check_ens(self.L.h4_ens_energy(self.h, k.ctypes.data, p.ctypes.data))
        return k + p, k, p

    def download(self):
        N = self.total
        out = {"r": np.zeros((N, 4)), "v": np.zeros((N, 4)), "f": np.zeros((N, 6)), "t": np.zeros(N),
               "dt": np.zeros(N)}
        _lib.check_ens(self.L.h4_ens_download(self.h, *[out[k].ctypes.data for k in ("r", "v", "f", "t", "dt")]))
        return out

    def system_slice(self, c):
        return slice(int(self.off[c]), int(self.off[c + 1]))

    def stats(self):
        it = np.zeros(self.nsys); at = np.zeros(self.nsys)
        steps = np.zeros(self.nsys, np.uint64); ps = np.zeros(self.nsys, np.uint64)
        inter = np.zeros(self.nsys, np.uint64)
        _lib.check_ens(self.L.h4_ens_system_stats(self.h, it.ctypes.data, at.ctypes.data, steps.ctypes.data,
                                                  ps.ctypes.data, inter.ctypes.data))
        return {"itime": it, "atime": at, "steps": steps, "psteps": ps, "interactions": inter}

    def tune_force(self, nact: int, ig: int, chunk: int, jtile: int = 256) -> float:
        ms = C.c_float()
        _lib.check_ens(self.L.h4_ens_tune_force(self.h, nact, ig, chunk, jtile, C.byref(ms)))
        return ms.value

    def bucket_stats(self):
        """Block steps and interactions per (N bucket, N_act bucket) of the
        tuning table, since creation: arrays of shape (NB_N, NB_A)."""
        steps = np.zeros(NB_N * NB_A, np.uint64)
        inter = np.zeros(NB_N * NB_A, np.uint64)
        _lib.check_ens(self.L.h4_ens_bucket_stats(self.h, steps.ctypes.data, inter.ctypes.data))
        return steps.reshape(NB_N, NB_A), inter.reshape(NB_N, NB_A)

    def timings(self):
        ms = C.c_float(); n = C.c_ulonglong()
        _lib.check_ens(self.L.h4_ens_timings(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    PHASES = ("active_set", "prediction", "grav", "correction")

    def phase_times(self) -> dict:
        """Device ms per phase of the persistent kernel since creation."""
        ms = np.zeros(4)
        _lib.check_ens(self.L.h4_ens_phase_times(self.h, ms.ctypes.data))
        return dict(zip(self.PHASES, ms.tolist()))
