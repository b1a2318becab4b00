"""Exact checkpoints of a block-step integration.

The reference resumes from its ASCII snapshots (4 significant digits,
src/include/utils/Logger.cpp:84-85) and recomputes forces and timesteps
(OptionsParser.cpp:122-323, NbodySystem.cpp:106-147), with the first block
time taken from init_dt's CTIME (Hermite4.cpp:137-138).  A checkpoint here
holds the full state (positions with masses, velocities, acc/jerk, times,
timesteps) in binary and the loop's scalars, so a resumed run continues bit
for bit as the uninterrupted one.

Format (little endian): magic b"H4CHK001", u64 n, then 14 f64 scalars
(e2, eta, dt_min, dt_max, itime, atime, iterations, nsteps, interactions,
e_ini, e_tmp, output_factor, snapshot_number, t_end), then the arrays r[n,4],
v[n,4], f[n,6], t[n], dt[n] (f64), ids[n] (u32).
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"H4CHK001"
SCALARS = ("e2", "eta", "dt_min", "dt_max", "itime", "atime", "iterations", "nsteps", "interactions",
           "e_ini", "e_tmp", "output_factor", "snapshot_number", "t_end")


def write_checkpoint(path: str, state: dict, scalars: dict, ids: np.ndarray) -> None:
    n = len(state["t"])
    with open(path, "wb") as fh:
        fh.write(MAGIC)
        fh.write(struct.pack("<Q", n))
        fh.write(struct.pack("<14d", *[float(scalars.get(k, 0.0)) for k in SCALARS]))
        for k, shape in (("r", (n, 4)), ("v", (n, 4)), ("f", (n, 6)), ("t", (n,)), ("dt", (n,))):
            fh.write(np.ascontiguousarray(state[k], dtype="<f8").reshape(shape).tobytes())
        fh.write(np.ascontiguousarray(ids, dtype="<u4").tobytes())


def read_checkpoint(path: str):
    with open(path, "rb") as fh:
        if fh.read(8) != MAGIC:
            raise ValueError(f"{path}: not a checkpoint")
        (n,) = struct.unpack("<Q", fh.read(8))
        vals = struct.unpack("<14d", fh.read(14 * 8))
        scalars = dict(zip(SCALARS, vals))
        state = {}
        for k, shape in (("r", (n, 4)), ("v", (n, 4)), ("f", (n, 6)), ("t", (n,)), ("dt", (n,))):
            cnt = int(np.prod(shape))
            state[k] = np.frombuffer(fh.read(8 * cnt), dtype="<f8").reshape(shape).copy()
        ids = np.frombuffer(fh.read(4 * n), dtype="<u4").copy()
    return state, scalars, ids
