"""Autotuner of the ensemble force phase, per (N bucket, N_act bucket).

Tuned shape of a system's force work (include/gravidy_gb300.h, the tuning
table of h4_ens_set_tuning):
  * FP64 form: particles per warp item (1, 2, 4) x j-chunk length;
  * mixed form: warp items of 1 particle or a packed pair (lanes over j) x
    j-chunk length, or block-tiled items of 16 ... 512 particles (lanes over
    i, j tiles in shared memory) x j-chunk length x shared-memory j tile
    (128 or 256).

The tuning follows the workload's mixture: the C4 ensemble (256 Plummer
systems, N log-uniform in [512, 16384], half equal-mass, half Salpeter).  It
is first integrated for a short time with the default table, and the
library's per-bucket statistics (h4_ens_bucket_stats: block steps and
interactions per bucket) give each bucket's weight and its typical active
count (interaction-weighted mean).

Mixed form: the shape of an item decides how many items one block step
yields, and in the ensemble only the systems that step in the same iteration
share the GPU -- a step of one large system must still fill 152 SMs.  A probe
of many identical systems cannot see that, so the mixed table is tuned on the
mixture itself: coordinate descent over the buckets that carry at least
MIN_WEIGHT of the interactions, heaviest first, each candidate timed as the
device time of the C4 ensemble from t = 0 to EVAL_T (the same block steps
every time).  FP64 form: the FP64 warp items are small and FP64-pipe bound,
so a probe suffices -- for every bucket a homogeneous ensemble of that N
(about 2^20 particles, equal-mass and Salpeter systems alternating) with the
bucket's active count forced on every system (h4_ens_tune_force).

Ties go, deterministically, to the first candidate within TIE (descent) or
PROBE_TIE (probes) of the fastest -- the current choice first in the descent
-- so that a re-run reproduces the table.  Finally C4 runs (to t = 1 mixed, 0.125 FP64) with the default and the
tuned table and both device times are recorded.

    python -m gravidy_gb300.autotune --out gravidy_gb300/tuning/ensemble_gb300.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import ics, workloads
from .ensemble import NB_A, NB_N, Ensemble

N_REP = [512, 1024, 2048, 4096, 8192, 16384]
A_LO = [1, 2, 4, 16, 64, 256, 1024, 4096]          # first active count of each bucket
A_REP = [1, 3, 12, 48, 192, 768, 3072, 8192]       # count used where C4 gives none
TIE = 0.01            # the mixed descent: repeatable whole-C4 timings
PROBE_TIE = 0.03      # the FP64 probes: single short launches, noisier
CHUNKS = [64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384]


def candidates(mode: str, n: int, nact: int):
    """(ig, chunk, jtile) candidates of the FP64 probe tuning, in preference
    order (ties go to the first)."""
    out = []
    for ig in (4, 2, 1):
        for chunk in reversed(CHUNKS):
            if chunk <= 2 * n:
                out.append((ig, chunk, 256))
    return out


def mixed_candidates(n: int, a: int):
    """(ig, chunk, jtile) candidates of the mixed descent for N bucket n and
    active bucket a (A_LO[a] particles and more)."""
    out = []
    if a >= 5:      # 256 and more active: block-tiled items, wide to narrow
        for bti in (512, 256, 128, 64):
            for chunk in (512, 1024, 2048, 4096):
                out.append((bti, chunk, 256))
        out += [(512, 1024, 128), (256, 1024, 128)]
        out += [(2, 2048, 256), (2, 4096, 256)]
    elif a >= 3:    # 16 - 255 active: packed-pair warp items or narrow blocks
        for chunk in (512, 1024, 2048, 4096):
            out.append((2, chunk, 256))
        for bti in (128, 64, 32, 16):
            if bti <= 4 * A_LO[a + 1]:
                out += [(bti, 1024, 256), (bti, 2048, 256)]
    else:           # a handful active: warp items
        for ig in (2, 1):
            for chunk in (256, 512, 1024, 2048):
                out.append((ig, chunk, 256))
    return [c for c in out if c[1] <= 2 * n]


def record_mixture(mode: str, t_end: float = 0.25, verbose: bool = True):
    """Block steps and interactions per bucket of the C4 ensemble run to
    t_end with the default table."""
    systems = workloads.c4_systems(256, seed=4)
    with Ensemble(systems, mode=mode, tuning=None) as E:
        E.init()
        E.advance(t_end)
        steps, inter = E.bucket_stats()
    if verbose:
        print(f"{mode}: C4 mixture to t={t_end}: {int(steps.sum())} block steps, {float(inter.sum()):.3e} "
              f"interactions", flush=True)
    return steps.astype(np.float64), inter.astype(np.float64)


def probe_ensemble(mode: str, n: int, total_particles: int):
    k = max(1, min(256, total_particles // n))
    systems = []
    for s in range(k):
        m, p, v = ics.plummer(n, 10_000 + s, "equal" if s % 2 == 0 else "salpeter", exact_scaling_max_n=0)
        systems.append((m, p, v, 0.01, 0.01))
    return Ensemble(systems, mode=mode, tuning=None), k


def time_candidate(E, nact, cand, reps):
    ig, chunk, jt = cand
    t = E.tune_force(nact, ig, chunk, jt)
    if t < 50.0:   # repeat the short probes, keep the best
        t = min([t] + [E.tune_force(nact, ig, chunk, jt) for _ in range(reps - 1)])
    return t


# C4 run lengths: the mixture record, the descent's objective and the
# validation (the FP64 form runs about 22x longer than the mixed form)
RECORD_T = {"mixed": 0.25, "fp64": 0.0625}
VALIDATE_T = {"mixed": 1.0, "fp64": 0.125}
EVAL_T = 0.125        # the mixed descent: one cycle of the largest block timestep
MIN_WEIGHT = 0.005    # buckets carrying less of the interactions keep the default


def default_table(mode: str) -> dict:
    """The library's built-in table (default_tuning in h4_ensemble.cu)."""
    ch = [128, 128, 256, 512, 1024, 2048, 4096, 8192]
    mixed_ig = [1, 2, 2, 2, 2, 2, 512, 512]
    ig = [[(mixed_ig[a] if mode == "mixed" else 4) for a in range(NB_A)] for _ in range(NB_N)]
    chunk = [[(1024 if mode == "mixed" and mixed_ig[a] > 2 else ch[a]) for a in range(NB_A)] for _ in range(NB_N)]
    return {"ig": ig, "chunk": chunk, "jtile": [[256] * NB_A for _ in range(NB_N)]}


def c4_seconds(mode: str, systems, table: dict, t_end: float) -> float:
    with Ensemble(systems, mode=mode, tuning=table) as E:
        E.init()
        E.advance(t_end)
        ms, _ = E.timings()
    return ms * 1e-3


def tune_mixed(verbose: bool = True) -> dict:
    steps, inter = record_mixture("mixed", t_end=RECORD_T["mixed"], verbose=verbose)
    systems = workloads.c4_systems(256, seed=4)
    table = default_table("mixed")
    t_best = c4_seconds("mixed", systems, table, EVAL_T)
    if verbose:
        print(f"mixed: default table, C4 to t={EVAL_T}: {t_best:.4f} s", flush=True)
    order = sorted(((inter[b, a], b, a) for b in range(NB_N) for a in range(NB_A)), reverse=True)
    trace = []
    for w, b, a in order:
        if w < MIN_WEIGHT * inter.sum():
            break
        cur = (table["ig"][b][a], table["chunk"][b][a], table["jtile"][b][a])
        cands = [cur] + [c for c in mixed_candidates(N_REP[b], a) if c != cur]
        times = []
        for c in cands:
            if c == cur:
                times.append(t_best)
                continue
            trial = json.loads(json.dumps(table))
            trial["ig"][b][a], trial["chunk"][b][a], trial["jtile"][b][a] = c
            times.append(c4_seconds("mixed", systems, trial, EVAL_T))
        best = min(times)
        pick = next(i for i, t in enumerate(times) if t <= best * (1.0 + TIE))
        table["ig"][b][a], table["chunk"][b][a], table["jtile"][b][a] = cands[pick]
        t_best = times[pick]
        trace.append({"bucket": [b, a], "weight": float(w), "candidates": [list(c) for c in cands],
                      "seconds": times, "pick": list(cands[pick])})
        if verbose:
            print(f"mixed N<={N_REP[b]:6d} a={a} weight={w:.2e}: pick {cands[pick]} {t_best:.4f} s "
                  f"(best {best:.4f}, current was {times[0]:.4f})", flush=True)
    table.update({"c4_steps": steps.astype(int).tolist(), "c4_interactions": inter.tolist(),
                  "eval_t": EVAL_T, "descent": trace})
    return table


def tune(mode: str = "fp64", total_particles: int = 1 << 20, reps: int = 3, verbose: bool = True) -> dict:
    """FP64 probe tuning: per N bucket a homogeneous ensemble of about
    total_particles particles; per active bucket every candidate timed with
    the bucket's C4 active count forced on every system (best of reps)."""
    steps, inter = record_mixture(mode, t_end=RECORD_T[mode], verbose=verbose)
    ig_tab = np.zeros((NB_N, NB_A), dtype=int)
    ch_tab = np.zeros((NB_N, NB_A), dtype=int)
    jt_tab = np.full((NB_N, NB_A), 256, dtype=int)
    rate_tab = np.zeros((NB_N, NB_A))
    nact_tab = np.zeros((NB_N, NB_A), dtype=int)
    for b, n in enumerate(N_REP):
        E, k = probe_ensemble(mode, n, total_particles)
        with E:
            for a in range(NB_A):
                if steps[b, a] > 0:   # interaction-weighted mean active count of the bucket
                    nact = int(round(inter[b, a] / steps[b, a] / n))
                    nact = max(A_LO[a], min(nact, (A_LO[a + 1] - 1) if a + 1 < NB_A else nact))
                else:
                    nact = A_REP[a]
                nact = max(1, min(nact, n))
                nact_tab[b, a] = nact
                cands = candidates(mode, n, nact)
                times = [time_candidate(E, nact, c, reps) for c in cands]
                best = min(times)
                pick = next(i for i, t in enumerate(times) if t <= best * (1.0 + PROBE_TIE))
                ig, chunk, jt = cands[pick]
                ig_tab[b, a], ch_tab[b, a], jt_tab[b, a] = ig, chunk, jt
                rate_tab[b, a] = k * nact * n / (times[pick] * 1e-3)
                if verbose:
                    print(f"{mode} N={n:6d} nact={nact:6d} systems={k:4d} weight={inter[b, a]:.2e}: ig={ig} "
                          f"chunk={chunk:6d} jtile={jt} {times[pick]:8.4f} ms (best {best:8.4f}) "
                          f"{rate_tab[b, a]:.3e} int/s", flush=True)
    table = {"ig": ig_tab.tolist(), "chunk": ch_tab.tolist(), "jtile": jt_tab.tolist(),
             "interactions_per_s": rate_tab.tolist(), "n_rep": N_REP, "nact_probe": nact_tab.tolist(),
             "c4_steps": steps.astype(int).tolist(), "c4_interactions": inter.tolist()}
    return table


def validate_c4(mode: str, table: dict, t_end: float = 1.0) -> dict:
    """C4 to t_end with the default table and with `table`: device seconds."""
    systems = workloads.c4_systems(256, seed=4)
    out = {}
    for name, tuning in (("default", None), ("tuned", table)):
        with Ensemble(systems, mode=mode, tuning=tuning) as E:
            E.init()
            st = E.advance(t_end)
            ms, _ = E.timings()
        out[name] = {"device_seconds": ms * 1e-3, "interactions_per_s": st["interactions"] / (ms * 1e-3)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--modes", default="fp64,mixed")
    ap.add_argument("--no-validate", action="store_true")
    args = ap.parse_args()
    t0 = time.time()
    out = {"generated_by": "python -m gravidy_gb300.autotune", "modes": {}}
    for mode in args.modes.split(","):
        out["modes"][mode] = tune_mixed() if mode == "mixed" else tune(mode)
        if not args.no_validate:
            out["modes"][mode]["c4_validation"] = validate_c4(mode, out["modes"][mode], VALIDATE_T[mode])
            print(mode, "C4 validation:", out["modes"][mode]["c4_validation"], flush=True)
    out["seconds"] = time.time() - t0
    with open(args.out, "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
