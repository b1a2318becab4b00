"""Autotuner of the ensemble force phase: particles per warp item (1, 2, 4)
and j-chunk length, per (N bucket, N_act bucket).

For every bucket it builds a homogeneous ensemble (about 2^20 particles in
systems of the bucket's N), forces the bucket's active count on every system,
times the force phase alone (h4_ens_tune_force, CUDA events) for each
candidate, and keeps the fastest.  The table is written as JSON, one table per
force mode, and read by ``gravidy_gb300.ensemble.Ensemble``.

    python -m gravidy_gb300.autotune --out gravidy_gb300/tuning/ensemble_gb300.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import ics
from .ensemble import NB_A, NB_N, Ensemble

N_REP = [512, 1024, 2048, 4096, 8192, 16384]
A_REP = [1, 3, 12, 48, 192, 768, 3072, 8192]      # one count inside each active bucket
IG_CAND = [1, 2, 4]
CHUNK_CAND = [64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384]


def tune(mode: str, total_particles: int = 1 << 20, reps: int = 3, verbose: bool = True) -> dict:
    ig_tab = np.full((NB_N, NB_A), 4, dtype=int)
    ch_tab = np.full((NB_N, NB_A), 1024, dtype=int)
    rate_tab = np.zeros((NB_N, NB_A))
    for b, n in enumerate(N_REP):
        k = max(1, min(256, total_particles // n))
        systems = []
        for s in range(k):
            m, p, v = ics.plummer(n, 10_000 + s, "equal", exact_scaling_max_n=0)
            systems.append((m, p, v, 0.01, 0.01))
        with Ensemble(systems, mode=mode, tuning=None) as E:
            for a, nact in enumerate(A_REP):
                nact = min(nact, n)
                best = None
                for ig in IG_CAND:
                    for chunk in CHUNK_CAND:
                        if chunk > 2 * n:
                            continue
                        t = E.tune_force(nact, ig, chunk)
                        if t < 50.0:   # repeat the short probes, keep the best
                            t = min([t] + [E.tune_force(nact, ig, chunk) for _ in range(reps - 1)])
                        if best is None or t < best[0]:
                            best = (t, ig, chunk)
                t, ig, chunk = best
                ig_tab[b, a], ch_tab[b, a] = ig, chunk
                rate_tab[b, a] = k * nact * n / (t * 1e-3)
                if verbose:
                    print(f"{mode} N={n:6d} nact={nact:6d} systems={k:4d}: ig={ig} chunk={chunk:6d} "
                          f"{t:8.4f} ms {rate_tab[b, a]:.3e} int/s", flush=True)
    return {"ig": ig_tab.tolist(), "chunk": ch_tab.tolist(), "interactions_per_s": rate_tab.tolist(),
            "n_rep": N_REP, "nact_rep": A_REP}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--modes", default="fp64,mixed")
    args = ap.parse_args()
    t0 = time.time()
    out = {"generated_by": "python -m gravidy_gb300.autotune", "modes": {}}
    for mode in args.modes.split(","):
        out["modes"][mode] = tune(mode)
    out["seconds"] = time.time() - t0
    with open(args.out, "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
