"""Helpers shared by the GPU parity tests."""
from __future__ import annotations

import numpy as np

from golden_util import case_dir, cases
from gravidy_gb300 import Hermite4GPU, NbodySystem, ics
from gravidy_gb300.io import read_input_file
from oracle import oracle as orc


def golden_system(name: str) -> NbodySystem:
    c = cases()[name]
    d = read_input_file(case_dir(name) + "/input.txt")
    return NbodySystem(d.mass, d.pos, d.vel, softening=c["softening"], eta=c["eta"],
                       integration_time=c["t_end"], interval_time=c["interval"])


def plummer_system(n: int, seed: int, imf: str = "equal", softening: float = 0.01,
                   eta: float = 0.01) -> NbodySystem:
    m, p, v = ics.plummer(n, seed, imf)
    return NbodySystem(m, p, v, softening=softening, eta=eta)


def oracle_for(ns: NbodySystem, **kw) -> orc.Oracle:
    return orc.Oracle(ns.mass, ns.pos, ns.vel, ns.e2, ns.eta, **kw)


def gpu_record(st: dict) -> np.ndarray:
    """State in the 15-double record layout of the reference trace."""
    n = len(st["t"])
    rec = np.zeros((n, 15))
    rec[:, 0:4] = st["r"]
    rec[:, 4:7] = st["v"][:, :3]
    rec[:, 7:13] = st["f"]
    rec[:, 13] = st["t"]
    rec[:, 14] = st["dt"]
    return rec


def state_hash(rec: np.ndarray) -> int:
    return orc.fnv1a(np.ascontiguousarray(rec))


def rel_err_vec(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-particle |a - b| / |b| of 3-vectors (rows)."""
    num = np.linalg.norm(a - b, axis=1)
    den = np.linalg.norm(b, axis=1)
    return num / np.where(den > 0, den, 1.0)
