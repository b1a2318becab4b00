"""The measured configurations, as seeded synthetic inputs.

C1  N = 1024 equal-mass Plummer, softening 0.01, eta 0.01, t = 0..1
C2  N = 65536 equal-mass Plummer, same units, t = 0..0.5 (block steps);
    all-active force sweep N = 4k..256k
C3  N = 65536 Plummer with a Salpeter IMF (slope -2.35, m in [0.1, 100],
    total mass 1), t = 0..1, FP64 vs mixed
C4  256 independent Plummer systems, seed per system, N log-uniform in
    [512, 16384], half equal-mass and half Salpeter, eps^2 = 1e-4, eta 0.01,
    each to t = 1 in the batched ensemble
C5  N = 1,048,576 Plummer + Salpeter, eps^2 = 1e-5 (softening 0.0031623),
    eta 0.02, t = 0..0.125
"""
from __future__ import annotations

import numpy as np

from . import ics
from .hermite4 import NbodySystem


def c1_system(seed: int = 1) -> NbodySystem:
    m, p, v = ics.plummer(1024, seed, "equal")
    return NbodySystem(m, p, v, softening=0.01, eta=0.01, integration_time=1.0)


def c2_system(n: int = 65536, seed: int = 1) -> NbodySystem:
    m, p, v = ics.plummer(n, seed, "equal")
    return NbodySystem(m, p, v, softening=0.01, eta=0.01, integration_time=0.5)


def c3_system(seed: int = 3) -> NbodySystem:
    m, p, v = ics.plummer(65536, seed, "salpeter")
    return NbodySystem(m, p, v, softening=0.01, eta=0.01, integration_time=1.0)


def c5_system(seed: int = 5) -> NbodySystem:
    m, p, v = ics.plummer(1 << 20, seed, "salpeter")
    return NbodySystem(m, p, v, softening=0.0031623, eta=0.02, integration_time=0.125)


def c4_sizes(nsys: int = 256, seed: int = 4, n_lo: int = 512, n_hi: int = 16384) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = rng.random(nsys)
    return np.round(n_lo * (n_hi / n_lo) ** u).astype(int)


def c4_systems(nsys: int = 256, seed: int = 4, rescale_energy: bool = True):
    """List of (mass, pos, vel, softening, eta) of the ensemble.  With
    ``rescale_energy`` every system is rescaled to E = -1/4 exactly, using the
    GPU ensemble energy kernel for the O(N^2) potential."""
    sizes = c4_sizes(nsys, seed)
    systems = []
    for s, n in enumerate(sizes):
        imf = "equal" if s % 2 == 0 else "salpeter"
        m, p, v = ics.plummer(int(n), seed * 100_000 + s, imf, exact_scaling_max_n=0)
        systems.append([m, p, v, 0.01, 0.01])
    if rescale_energy:
        from .ensemble import Ensemble
        with Ensemble([tuple(x) for x in systems], mode="fp64", tuning=None) as E:
            _, kin, pot = E.energy()
        for k, sd in enumerate(systems):
            sd[1] = sd[1] * (pot[k] / -0.5)
            sd[2] = sd[2] * np.sqrt(0.25 / kin[k])
    return [tuple(x) for x in systems]
