"""Cluster diagnostics of NbodyUtils (src/include/utils/NbodyUtils.cpp:59-328)
on the device state: center of density, core/half-mass/Lagrange radii, and
nbody_attributes with the reference's float/double arithmetic."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib

f32 = np.float32
LAGRANGE_RADII = (0.01, 0.05, 0.1, 0.2, 0.5, 0.75)


def total_mass(masses) -> float:
    """NbodySystem::total_mass: float sum in input order (NbodySystem.cpp:182)."""
    t = f32(0.0)
    for m in np.asarray(masses, dtype=np.float32):
        t = f32(t + m)
    return float(t)


def center_of_density(h4) -> np.ndarray:
    out = np.zeros(3)
    st = h4.L.h4_center_of_density(h4.h, out.ctypes.data)
    if st:
        raise _lib.H4Error(st, h4.L.h4_diag_last_error().decode())
    return out


def mass_radii(h4, center, tm: float):
    c = np.ascontiguousarray(center, dtype=np.float64)
    core, half = C.c_double(), C.c_double()
    lag = np.zeros(6)
    st = h4.L.h4_mass_radii(h4.h, c.ctypes.data, C.c_float(tm), C.byref(core), C.byref(half), lag.ctypes.data)
    if st:
        raise _lib.H4Error(st, h4.L.h4_diag_last_error().decode())
    return core.value, half.value, lag


def lagrange_radii(h4, tm: float):
    """NbodyUtils::lagrange_radii (:246-263): radii about a fresh center of
    density; returns (radii[6], cod)."""
    cod = center_of_density(h4)
    _, _, lag = mass_radii(h4, cod, tm)
    return lag, cod


def nbody_attributes(h4, e_ini: float, tm: float, cod_state: np.ndarray) -> dict:
    """NbodyUtils::nbody_attributes (:59-78).  cod_state is NbodyUtils::cod,
    updated in place: the core radius uses its value on entry."""
    n = h4.n
    r_virial = f32(float(f32(f32(-1.0) * f32(tm)) * f32(tm)) / (4 * e_ini))
    M = f32(tm)
    rv3 = f32(float(r_virial) * float(r_virial) * float(r_virial))
    ut = f32(math.sqrt(float(f32(rv3 / f32(M)))))
    t_cr = f32(2 * math.sqrt(2) * float(ut))
    r_cl = (4.0 * float(r_virial)) / n
    r_cl3 = f32(r_cl * r_cl * r_cl)
    dt_cl = 0.04 * math.sqrt(float(f32(r_cl3 * f32(n))))
    core, _, _ = mass_radii(h4, cod_state, tm)
    cod = center_of_density(h4)
    cod_state[:] = cod
    _, half, _ = mass_radii(h4, cod, tm)
    r_h = f32(half)
    num = f32(f32(f32(f32(n) * r_h) * r_h) * r_h)
    den = f32(f32(1.0) * f32(f32(tm) / f32(n)))
    a = f32(math.sqrt(float(f32(num / den))))
    b = f32(1.0 / math.log(0.11 * n))
    t_rh = f32(0.138 * float(a) * float(b))
    return {"r_virial": float(r_virial), "t_cr": float(t_cr), "r_cl": r_cl, "dt_cl": dt_cl, "r_core": core,
            "t_rlx": float(t_rh), "r_hm": float(r_h), "cod": cod}
