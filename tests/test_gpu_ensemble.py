"""Batched ensemble (persistent fused kernel + graph) against per-system runs.

  * exact force mode: every system's final state is bit-identical to the
    oracle's (the reference CPU path restated) after the same block steps;
  * FP64 mode: same block-step counts and times as the single-system GPU
    path, states within 1e-9 (FP64 forces differ only in summation order);
  * mixed mode: |dE/E| of every system within 2x of its FP64 value (+1e-9),
    and its state within 1e-6 of the FP64 ensemble's after a short run (the
    mixed predictor works from an FP32 form of the corrected state).
"""
import numpy as np
import pytest

from gravidy_gb300 import Hermite4GPU, NbodySystem, ics
from gravidy_gb300.ensemble import Ensemble
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SIZES = [2, 33, 100, 257, 512, 1000, 1500]


def _systems(sizes, seed0=100):
    out = []
    for k, n in enumerate(sizes):
        imf = "salpeter" if k % 2 else "equal"
        m, p, v = ics.plummer(n, seed0 + k, imf)
        out.append((m, p, v, 0.01, 0.01))
    return out


def _oracle_run(sysdef, t_end):
    m, p, v, soft, eta = sysdef
    o = orc.Oracle(m, p, v, orc.e2_from_softening(soft), eta)
    o.init_acc_jrk()
    atime = o.init_dt(0.0, float(orc.ETA_S))
    itime, steps = 0.0, 0
    while itime < t_end:
        _, itime, atime = o.block_step(itime, atime)
        steps += 1
    return o, steps, itime


def test_ensemble_exact_mode_bit_identical_to_oracle():
    systems = _systems(SIZES)
    t_end = 0.0625
    with Ensemble(systems, mode="exact") as E:
        E.init()
        E.advance(t_end)
        st = E.download()
        stats = E.stats()
    for c, sd in enumerate(systems):
        o, steps, itime = _oracle_run(sd, t_end)
        sl = E.system_slice(c)
        assert int(stats["steps"][c]) == steps and stats["itime"][c] == itime, c
        assert np.array_equal(st["r"][sl], o.r), c
        assert np.array_equal(st["v"][sl][:, :3], o.v[:, :3]), c
        assert np.array_equal(st["f"][sl], o.f), c
        assert np.array_equal(st["dt"][sl], o.dt) and np.array_equal(st["t"][sl], o.t), c


def test_ensemble_fp64_matches_single_system_runs():
    systems = _systems(SIZES, seed0=300)
    t_end = 0.125
    with Ensemble(systems, mode="fp64") as E:
        E.init()
        E.advance(t_end)
        st = E.download()
        stats = E.stats()
        etot, _, _ = E.energy()
    for c, (m, p, v, soft, eta) in enumerate(systems):
        ns = NbodySystem(m, p, v, softening=soft, eta=eta)
        with Hermite4GPU(ns) as g:
            g.init_acc_jrk()
            atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
            itime, atime, steps, _, _, _ = g.advance(t_end, 1e30, atime)
            s1 = g.download()
            e1 = g.get_energy_gpu()
        sl = E.system_slice(c)
        assert int(stats["steps"][c]) == steps and stats["itime"][c] == itime, c
        assert np.abs(st["r"][sl] - s1["r"]).max() < 1e-9, c
        assert np.array_equal(st["dt"][sl], s1["dt"]), c
        assert abs(etot[c] - e1) < 1e-12 * abs(e1), c


def test_ensemble_fp64_many_chunk_steps_match_single_system_runs():
    """A 9000-particle system beside a small one: its steps of 1-3 active
    particles split the j range into 71 chunks of 128, so the corrector sums
    their partials by warps, 32 particles per group on the grid's last
    blocks.  Same steps and block times as the single-system runs, states
    within 1e-9 (FP64 sums in another order)."""
    systems = _systems([9000, 700], seed0=1900)
    t_end = 0.03125
    with Ensemble(systems, mode="fp64") as E:
        E.init()
        E.advance(t_end)
        st = E.download()
        stats = E.stats()
        steps_b, _ = E.bucket_stats()
    assert steps_b[5, 0] + steps_b[5, 1] > 0   # N in (8192, 16384], 1-3 active: the warp reduction ran
    for c, (m, p, v, soft, eta) in enumerate(systems):
        ns = NbodySystem(m, p, v, softening=soft, eta=eta)
        with Hermite4GPU(ns) as g:
            g.init_acc_jrk()
            atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
            itime, atime, steps, _, _, _ = g.advance(t_end, 1e30, atime)
            s1 = g.download()
        sl = E.system_slice(c)
        assert int(stats["steps"][c]) == steps and stats["itime"][c] == itime, c
        assert np.abs(st["r"][sl] - s1["r"]).max() < 1e-9, c


def test_ensemble_mixed_energy_error_close_to_fp64():
    systems = _systems([512, 1024, 2048, 700], seed0=500)
    t_end = 0.25
    res = {}
    for mode in ("fp64", "mixed"):
        with Ensemble(systems, mode=mode) as E:
            E.init()
            e0, _, _ = E.energy()
            E.advance(t_end)
            e1, _, _ = E.energy()
        res[mode] = np.abs((e1 - e0) / e0)
    print("dE/E fp64", res["fp64"], "mixed", res["mixed"])
    assert np.all(res["mixed"] <= 2 * res["fp64"] + 1e-9)


def test_ensemble_mixed_state_tracks_fp64():
    """Systems stepping with warp items (N <= 2000) and with block-tiled
    items (N = 6000, steps of 1024 and more active) to t = 1/16: positions
    and velocities of the mixed ensemble within 1e-6 of the FP64 ensemble's,
    relative to the system's largest |r| and |v|."""
    systems = _systems([700, 2000, 6000], seed0=1700)
    st = {}
    for mode in ("fp64", "mixed"):
        with Ensemble(systems, mode=mode) as E:
            E.init()
            E.advance(0.0625)
            st[mode] = E.download()
            sl = [E.system_slice(c) for c in range(len(systems))]
    for c in range(len(systems)):
        for k in ("r", "v"):
            a, b = st["fp64"][k][sl[c]][:, :3], st["mixed"][k][sl[c]][:, :3]
            err = np.abs(a - b).max() / np.abs(a).max()
            print(f"system {c} {k}: max deviation {err:.2e}")
            assert err < 1e-6, (c, k, err)


def test_ensemble_tune_probe_leaves_state_unchanged():
    systems = _systems([600, 900, 1200], seed0=700)
    with Ensemble(systems, mode="fp64") as E:
        E.init()
        E.advance(0.03125)
        a = E.download()
        sa = E.stats()
        for ig in (1, 2, 4):
            for chunk in (64, 512):
                assert E.tune_force(100, ig, chunk) > 0.0
        b = E.download()
        sb = E.stats()
        for k in a:
            assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(sa["itime"], sb["itime"])
        E.advance(0.0625)
        assert np.all(E.stats()["itime"] >= 0.0625)


def test_ensemble_energy_matches_oracle():
    systems = _systems([2, 37, 300], seed0=900)
    with Ensemble(systems, mode="fp64") as E:
        etot, ek, ep = E.energy()
    for c, (m, p, v, soft, eta) in enumerate(systems):
        o = orc.Oracle(m, p, v, orc.e2_from_softening(soft), eta)
        e, k, pp = o.energy()
        assert abs(ek[c] - k) <= 1e-12 * abs(k)
        assert abs(ep[c] - pp) <= 1e-12 * max(abs(pp), 1e-300)


def test_ensemble_mixed_forces_vs_oracle():
    """Initial forces of every system (all particles active: block-tiled items
    for N >= 2048, warp items below) within the mixed-form tolerance."""
    from h4_util import rel_err_vec
    systems = _systems([300, 700, 2048, 5000], seed0=1100)
    with Ensemble(systems, mode="mixed") as E:
        E.init()
        f = E.download()["f"]
    for c, (m, p, v, soft, eta) in enumerate(systems):
        want = orc.forces_for(orc.make_predictors(m, p, v), orc.e2_from_softening(soft),
                              np.arange(len(m), dtype=np.uint32))
        got = f[E.system_slice(c)]
        ea = rel_err_vec(got[:, :3], want[:, :3])
        ej = rel_err_vec(got[:, 3:], want[:, 3:])
        assert np.median(ea) < 1e-6 and ea.max() < 1e-4, (c, np.median(ea), ea.max())
        assert np.median(ej) < 1e-6 and ej.max() < 1e-4, (c, np.median(ej), ej.max())


def test_ensemble_mixed_forces_large_system_vs_oracle():
    """An ensemble holding a 16384-particle system (the top of C4's size
    range) beside smaller ones: initial forces (all particles active, so the
    large systems run as block-tiled items and the small one as warp items)
    on a sample of particles of every system against the oracle."""
    from h4_util import rel_err_vec
    systems = _systems([16384, 3000, 700], seed0=1500)
    with Ensemble(systems, mode="mixed") as E:
        E.init()
        f = E.download()["f"]
    for c, (m, p, v, soft, eta) in enumerate(systems):
        sample = np.unique(np.linspace(0, len(m) - 1, min(len(m), 1024)).astype(np.uint32))
        want = orc.forces_for(orc.make_predictors(m, p, v), orc.e2_from_softening(soft), sample)
        got = f[E.system_slice(c)][sample]
        ea = rel_err_vec(got[:, :3], want[:, :3])
        ej = rel_err_vec(got[:, 3:], want[:, 3:])
        print(f"N={len(m)}: acc median {np.median(ea):.2e} max {ea.max():.2e}; "
              f"jerk median {np.median(ej):.2e} max {ej.max():.2e}")
        assert np.median(ea) < 1e-6 and ea.max() < 1e-4, (c, np.median(ea), ea.max())
        assert np.median(ej) < 1e-6 and ej.max() < 1e-4, (c, np.median(ej), ej.max())


def test_ensemble_phase_timers():
    """Device time per phase of the persistent kernel (h4_ens_phase_times):
    every phase ran, and the phases add up to no more than the advance's
    CUDA-event time."""
    systems = _systems([600, 2100, 900], seed0=1300)
    with Ensemble(systems, mode="mixed") as E:
        E.init()
        p0 = E.phase_times()
        E.advance(0.03125)
        ms, _ = E.timings()
        p1 = E.phase_times()
    d = {k: p1[k] - p0[k] for k in p1}
    assert list(d) == ["active_set", "prediction", "grav", "correction"]
    assert all(v > 0.0 for v in d.values()), d
    assert sum(d.values()) <= ms * 1.02 + 0.05, (d, ms)
