"""Seeded initial conditions in Henon units (G = M = 1, E = -1/4).

The reference reads its initial conditions from files of an external
repository that is not vendored (the ``input`` submodule).  These generators
produce the same kind of models from a seed:

* ``plummer``: the Plummer sphere sampled as in Aarseth, Henon & Wielen (1974,
  A&A 37, 183): radius from the cumulative mass fraction, isotropic
  directions, speed by von Neumann rejection on g(q) = q^2 (1 - q^2)^(7/2).
* ``salpeter_masses``: a power-law IMF dN/dm ~ m^-2.35 on [0.1, 100] by
  inverse-CDF sampling, renormalised to a total mass of one.

Positions and velocities are moved to the centre-of-mass frame and rescaled so
that the unsoftened energy of the sample (the energy definition of
src/include/utils/NbodyUtils.cpp:427-529) is exactly -1/4 with virial ratio
1/2.  For large N (above ``exact_scaling_max_n``) the analytic scaling of the
continuous model is used instead and the sample energy is only close to -1/4.
"""
from __future__ import annotations

import numpy as np

__all__ = ["plummer", "salpeter_masses", "energy", "write_input_file"]


def salpeter_masses(n: int, rng: np.random.Generator, alpha: float = 2.35,
                    m_lo: float = 0.1, m_hi: float = 100.0) -> np.ndarray:
    """Masses from dN/dm ~ m^-alpha on [m_lo, m_hi], normalised to sum 1."""
    u = rng.random(n)
    k = 1.0 - alpha
    m = (m_lo ** k + u * (m_hi ** k - m_lo ** k)) ** (1.0 / k)
    return m / m.sum()


def energy(pos: np.ndarray, vel: np.ndarray, mass: np.ndarray, chunk: int = 2048):
    """Unsoftened kinetic and potential energy (float64, chunked O(N^2))."""
    kin = 0.5 * float(np.sum(mass * np.sum(vel * vel, axis=1)))
    pot = 0.0
    n = len(mass)
    for i0 in range(0, n, chunk):
        i1 = min(n, i0 + chunk)
        d = pos[None, :, :] - pos[i0:i1, None, :]
        r = np.sqrt(np.sum(d * d, axis=2))
        idx = np.arange(i0, i1)
        mask = np.arange(n)[None, :] > idx[:, None]
        with np.errstate(divide="ignore"):
            term = np.where(mask, mass[None, :] / np.where(mask, r, 1.0), 0.0)
        pot -= float(np.sum(mass[i0:i1, None] * term))
    return kin, pot


def _isotropic(rng: np.random.Generator, mag: np.ndarray) -> np.ndarray:
    n = len(mag)
    z = (1.0 - 2.0 * rng.random(n)) * mag
    phi = 2.0 * np.pi * rng.random(n)
    rxy = np.sqrt(np.maximum(mag * mag - z * z, 0.0))
    return np.stack([rxy * np.cos(phi), rxy * np.sin(phi), z], axis=1)


def plummer(n: int, seed: int, imf: str = "equal", exact_scaling_max_n: int = 16384):
    """Return (mass[n], pos[n,3], vel[n,3]) of a seeded Plummer model.

    ``imf`` is "equal" (m = 1/n, exact in float for powers of two) or
    "salpeter".  Masses are returned already rounded to float32, the precision
    the reference keeps for masses (src/include/NbodySystem.cpp:174).
    """
    if n < 1:
        raise ValueError("n must be >= 1")
    rng = np.random.default_rng(seed)
    if imf == "equal":
        mass = np.full(n, 1.0 / n)
    elif imf == "salpeter":
        mass = salpeter_masses(n, rng)
    else:
        raise ValueError(f"unknown imf {imf!r}")
    mass = mass.astype(np.float32).astype(np.float64)

    # Radius from the enclosed mass fraction X (cut at X = 0.999, AHW74).
    x = rng.random(n) * 0.999
    x = np.maximum(x, 1e-300)
    r = 1.0 / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
    pos = _isotropic(rng, r)

    # Speed q * v_escape, q by rejection on q^2 (1 - q^2)^3.5 (max < 0.1).
    q = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        x4 = rng.random(len(todo))
        x5 = rng.random(len(todo))
        ok = 0.1 * x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
        q[todo[ok]] = x4[ok]
        todo = todo[~ok]
    ve = np.sqrt(2.0) * (1.0 + r * r) ** -0.25
    vel = _isotropic(rng, q * ve)

    mtot = mass.sum()
    pos -= (mass[:, None] * pos).sum(axis=0) / mtot
    vel -= (mass[:, None] * vel).sum(axis=0) / mtot

    if n >= 2 and n <= exact_scaling_max_n:
        kin, pot = energy(pos, vel, mass)
        # Rescale to U = -1/2, T = 1/4 (E = -1/4, virial ratio 1/2).
        pos *= pot / -0.5
        vel *= np.sqrt(0.25 / kin)
    else:
        # Continuous Plummer model with scale length 1: E = -3 pi / 64 (M = 1).
        # Lengths scale by 3 pi / 16 and speeds by its inverse square root.
        s = 3.0 * np.pi / 16.0
        pos *= s
        vel /= np.sqrt(s)
    return mass, pos, vel


def write_input_file(path: str, mass: np.ndarray, pos: np.ndarray, vel: np.ndarray) -> None:
    """Write the 8-column input format of src/include/NbodySystem.cpp:161-181.

    ``id m x y z vx vy vz``, one particle per line, with 17 significant
    digits so every double (and the float mass) round-trips exactly.
    """
    with open(path, "w") as fh:
        for i in range(len(mass)):
            fh.write("%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n" % (
                i, mass[i], pos[i, 0], pos[i, 1], pos[i, 2],
                vel[i, 0], vel[i, 1], vel[i, 2]))
