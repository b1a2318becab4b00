"""Readers for the fixtures in tests/golden/ (see tests/golden/make_golden.py)."""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases() -> dict:
    with open(os.path.join(GOLDEN, "cases.json")) as fh:
        return json.load(fh)


def case_dir(name: str) -> str:
    return os.path.join(GOLDEN, name)


def load_init(name: str, n: int):
    raw = np.fromfile(os.path.join(case_dir(name), "init.bin"), dtype="<f8")
    f = raw[: 6 * n].reshape(n, 6)
    dt = raw[6 * n: 7 * n]
    atime = raw[7 * n]
    return f, dt, atime


def load_steps(name: str):
    """[(step, itime, nact, fnv_move, fnv_state)], summary dict."""
    rows, summary = [], {}
    with open(os.path.join(case_dir(name), "steps.txt")) as fh:
        for line in fh:
            if line.startswith("#"):
                tok = line[1:].split()
                summary = {tok[k]: int(tok[k + 1]) for k in range(0, len(tok), 2)}
                continue
            s, it, nact, hm, hs = line.split()
            rows.append((int(s), float.fromhex(it), int(nact), int(hm, 16), int(hs, 16)))
    return rows, summary


def load_energy(name: str):
    out = []
    with open(os.path.join(case_dir(name), "energy.txt")) as fh:
        for line in fh:
            a, b = line.split()
            out.append((float.fromhex(a), float.fromhex(b)))
    return out


def load_state(name: str, tag: str, n: int) -> np.ndarray:
    return np.fromfile(os.path.join(case_dir(name), f"state_{tag}.bin"), dtype="<f8").reshape(n, 15)


def load_cli_log(name: str):
    """Deterministic columns of the reference program's energy log."""
    path = os.path.join(case_dir(name), "energy_log.txt")
    if not os.path.exists(path):
        return None
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                continue
            tok = line.split()
            rows.append((tok[1], tok[2], tok[3], tok[4], tok[5], tok[6]))
    return rows
