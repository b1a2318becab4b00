"""Input files and the energy log, in the reference's formats.

* ``read_input_file`` follows NbodySystem::read_input_file
  (src/include/NbodySystem.cpp:79-207): 8 whitespace-separated tokens per line
  ``id m x y z vx vy vz``; the mass is parsed with strtod and rounded to float
  (:174); a leading ``#`` line holding ``Time: t`` sets the snapshot time
  (:106-147), other ``#`` lines are comments; a line with a token count other
  than 8 stops the reading (:163-169) and the particles read so far are kept.
* ``EnergyLog`` writes the rows of Logger::print_energy_log
  (src/include/utils/Logger.cpp:324-391), header at t = 0 included.
"""
from __future__ import annotations

import math
import sys
from dataclasses import dataclass, field

import numpy as np

__all__ = ["InputData", "read_input_file", "EnergyLog", "KERNEL_FLOP_LOG"]

# Flops per interaction the reference's log column uses (common.hpp:331).
KERNEL_FLOP_LOG = 48.0


@dataclass
class InputData:
    ids: np.ndarray
    mass: np.ndarray          # float32 values held in float64
    pos: np.ndarray           # (n, 3) float64
    vel: np.ndarray           # (n, 3) float64
    snapshot_time: float = 0.0
    warnings: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return len(self.mass)


def _strtod(tok: str) -> float:
    """strtod on a whole token: the longest valid prefix, 0.0 if none."""
    try:
        return float(tok)
    except ValueError:
        for k in range(len(tok) - 1, 0, -1):
            try:
                return float(tok[:k])
            except ValueError:
                continue
        return 0.0


def _atoi(tok: str) -> int:
    s = tok.strip()
    k = 0
    if k < len(s) and s[k] in "+-":
        k += 1
    while k < len(s) and s[k].isdigit():
        k += 1
    try:
        return int(s[:k])
    except ValueError:
        return 0


def read_input_file(path: str) -> InputData:
    ids, mass, pos, vel = [], [], [], []
    got_time = False
    snapshot_time = 0.0
    warnings = []
    with open(path, "r") as fh:
        lines = fh.read().split("\n")
    # The reference's getline loop ends as soon as a read reaches EOF, so the
    # piece after the last '\n' (empty, or a line without its newline) is
    # never parsed.
    lines = lines[:-1]
    for line in lines:
        stripped = line.lstrip(" ")
        if stripped.startswith("#"):
            if not got_time:
                clean = line.replace("#", "").replace(":", "").lower()
                toks = clean.split()
                for k, tk in enumerate(toks):
                    if tk == "time" and k + 1 < len(toks):
                        snapshot_time = _strtod(toks[k + 1])
                        got_time = True
                        break
            continue
        toks = line.split()
        if len(toks) != 8:
            warnings.append(f"gravidy: wrong line format in {path}: only eight numbers per line are allowed")
            break
        ids.append(_atoi(toks[0]) & 0xFFFFFFFF)
        mass.append(float(np.float32(_strtod(toks[1]))))
        pos.append([_strtod(t) for t in toks[2:5]])
        vel.append([_strtod(t) for t in toks[5:8]])
    return InputData(np.array(ids, dtype=np.uint32), np.array(mass, dtype=np.float64),
                     np.array(pos, dtype=np.float64).reshape(-1, 3),
                     np.array(vel, dtype=np.float64).reshape(-1, 3),
                     snapshot_time, warnings)


class EnergyLog:
    """Energy log rows in the format of Logger::print_energy_log."""

    HEADER = "%-2s%10s%15s%15s%20s%15s%15s%16s%12s" % (
        "#", "IteTime", "Iter", "Nsteps", "Energy", "RelE", "CumE", "ElapsedTime", "GFLOPS")

    def __init__(self, stream=None):
        self.stream = stream if stream is not None else sys.stdout
        self.e_ini = None
        self.e_tmp = None
        self.rows = []

    def row(self, itime: float, iterations: int, nsteps: int, energy: float,
            elapsed: float, interactions: int = 0, update_time: float = 0.0) -> str:
        if self.e_ini is None:
            self.e_ini = energy
            self.e_tmp = energy
        rel = abs((energy - self.e_tmp) / self.e_tmp) if self.e_tmp != 0 else math.nan
        cum = abs((energy - self.e_ini) / self.e_ini) if self.e_ini != 0 else math.nan
        self.e_tmp = energy
        gflops = 0.0
        if itime != 0.0 and update_time > 0:
            gflops = KERNEL_FLOP_LOG * 1e-9 * interactions / update_time
        out = []
        if itime == 0.0:
            out.append(self.HEADER)
        out.append("%2s%10.3f%15d%15d%20.10e%15.6e%15.6e%16.6e%12.3f" % (
            "00", itime, iterations & 0xFFFFFFFF, nsteps & 0xFFFFFFFF, energy, rel, cum, elapsed, gflops))
        text = "\n".join(out)
        self.rows.append((itime, iterations, nsteps, energy, rel, cum))
        if self.stream is not False:
            print(text, file=self.stream)
        return text
