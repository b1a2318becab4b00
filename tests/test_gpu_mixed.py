"""Mixed-precision form against the FP64 oracle.

Accuracy contract of the mixed form (reported, and bounded here):
  * per-particle relative error of acc and jerk: median below MIXED_MED_RTOL,
    maximum below MIXED_MAX_RTOL, against the FP64 oracle;
  * |dE/E| at t = 1 of the C1 run (N = 1024 Plummer) within 2x of the FP64
    run's value.
"""
import numpy as np
import pytest

from h4_util import golden_system, plummer_system, rel_err_vec
from gravidy_gb300 import EnergyLog, Hermite4GPU
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
MIXED_MED_RTOL = 1e-6
MIXED_MAX_RTOL = 1e-4


def _forces_case(n, nact, seed, threshold=None, softening=0.01):
    ns = plummer_system(n, seed=seed, imf="salpeter", softening=softening)
    rng = np.random.default_rng(seed + nact)
    move = np.sort(rng.choice(n, size=nact, replace=False)).astype(np.uint32)
    pr = np.zeros((n, 4)); pr[:, :3] = ns.pos; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = ns.vel
    want = orc.forces_for(orc.make_predictors(ns.mass, ns.pos, ns.vel), ns.e2, move)
    with Hermite4GPU(ns, mode="mixed") as g:
        if threshold is not None:
            g.set_mixed_threshold(threshold)
        got = g.forces_for(pr, pv, move)
    ea = rel_err_vec(got[:, :3], want[:, :3])
    ej = rel_err_vec(got[:, 3:], want[:, 3:])
    return ea, ej


@pytest.mark.parametrize("n,nact", [(65536, 1), (65536, 33), (65536, 1000), (65536, 4096),
                                    (65536, 65536), (5000, 5000), (1023, 17)])
def test_mixed_force_errors(n, nact):
    ea, ej = _forces_case(n, nact, seed=3)
    print(f"N={n} nact={nact}: acc median {np.median(ea):.2e} max {ea.max():.2e}; "
          f"jerk median {np.median(ej):.2e} max {ej.max():.2e}")
    assert np.median(ea) < MIXED_MED_RTOL and np.median(ej) < MIXED_MED_RTOL
    assert ea.max() < MIXED_MAX_RTOL and ej.max() < MIXED_MAX_RTOL


@pytest.mark.parametrize("threshold", [1, 1 << 30])
def test_mixed_both_shapes_agree(threshold):
    """Tiled (threshold 1) and warp-item (huge threshold) shapes both meet
    the mixed tolerance on the same case."""
    ea, ej = _forces_case(8192, 3000, seed=8, threshold=threshold)
    assert np.median(ea) < MIXED_MED_RTOL and ea.max() < MIXED_MAX_RTOL
    assert np.median(ej) < MIXED_MED_RTOL and ej.max() < MIXED_MAX_RTOL


def test_mixed_zero_softening_masks_self():
    n = 300
    ns = plummer_system(n, seed=4, softening=0.0)
    assert ns.e2 == 0.0
    move = np.arange(n, dtype=np.uint32)
    pr = np.zeros((n, 4)); pr[:, :3] = ns.pos; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = ns.vel
    want = orc.forces_for(orc.make_predictors(ns.mass, ns.pos, ns.vel), 0.0, move)
    for thr in (1, 1 << 30):
        with Hermite4GPU(ns, mode="mixed") as g:
            g.set_mixed_threshold(thr)
            got = g.forces_for(pr, pv, move)
        assert np.all(np.isfinite(got))
        assert np.median(rel_err_vec(got[:, :3], want[:, :3])) < MIXED_MED_RTOL


def test_mixed_c1_energy_error_within_2x_fp64():
    res = {}
    for mode in ("fp64", "mixed"):
        ns = golden_system("c1_plummer_n1024")
        with Hermite4GPU(ns, mode=mode) as g:
            log = g.integration(log=EnergyLog(stream=False))
        res[mode] = log.rows[-1][5]
    print("CumE at t=1:", res)
    assert res["mixed"] <= 2.0 * res["fp64"]


@pytest.mark.parametrize("threshold", [1, 1 << 30])
def test_mixed_forces_for_uses_the_given_predictors(threshold):
    """h4_forces_for in the mixed form packs its FP32 j data from the
    predictors it is given, not from the handle's last prediction: forces of
    perturbed predictors (not the state the handle holds) match the oracle's
    forces of the same predictors."""
    n, nact = 4000, 700
    ns = plummer_system(n, seed=12, imf="salpeter")
    rng = np.random.default_rng(12)
    pos = ns.pos + 1e-2 * rng.standard_normal(ns.pos.shape)
    vel = ns.vel * 1.3
    move = np.sort(rng.choice(n, size=nact, replace=False)).astype(np.uint32)
    pr = np.zeros((n, 4)); pr[:, :3] = pos; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = vel
    want = orc.forces_for(orc.make_predictors(ns.mass, pos, vel), ns.e2, move)
    with Hermite4GPU(ns, mode="mixed") as g:
        g.set_mixed_threshold(threshold)
        got = g.forces_for(pr, pv, move)
    ea = rel_err_vec(got[:, :3], want[:, :3])
    ej = rel_err_vec(got[:, 3:], want[:, 3:])
    assert np.median(ea) < MIXED_MED_RTOL and ea.max() < MIXED_MAX_RTOL
    assert np.median(ej) < MIXED_MED_RTOL and ej.max() < MIXED_MAX_RTOL


def test_switch_to_mixed_packs_current_predictors():
    """h4_set_force_mode into the mixed form between the methods of a block
    step: the force sum uses the j data of the current predictors."""
    ns = plummer_system(3000, seed=13, imf="salpeter")
    with Hermite4GPU(ns, mode="fp64") as a, Hermite4GPU(ns, mode="mixed") as b:
        for g in (a, b):
            g.init_acc_jrk()
        ta = a.init_dt()
        tb = b.init_dt()
        assert ta == tb
        for g, t in ((a, ta), (b, tb)):
            nact = g.find_particles_to_move(t)
            g.save_old_acc_jrk(nact)
            g.predicted_pos_vel(t)
        _lib_set = a.L.h4_set_force_mode
        assert _lib_set(a.h, 2) == 0     # fp64 -> mixed after the FP64-mode prediction
        nact = a.find_particles_to_move(ta)
        a.update_acc_jrk(nact)
        b.update_acc_jrk(nact)
        sa, sb = a.download(), b.download()
    act = sa["move"][:nact]
    assert np.array_equal(act, sb["move"][:nact])
    # the active particles' new forces (the others keep their initial forces,
    # FP64 in a and mixed in b)
    assert np.array_equal(sa["f"][act], sb["f"][act])


def test_mixed_salpeter_n16384_energy_error_within_2x_fp64():
    """The C3 configuration (Salpeter-IMF Plummer, softening 0.01, eta 0.01)
    at a quarter of its size and time: N = 16384 to t = 0.25 through the
    device-resident block-timestep loop in both forms; the mixed form's
    |dE/E| is within 2x of the FP64 form's."""
    res = {}
    for mode in ("fp64", "mixed"):
        ns = plummer_system(16384, seed=3, imf="salpeter")
        with Hermite4GPU(ns, mode=mode) as g:
            g.init_acc_jrk()
            atime = g.init_dt()
            e0 = g.get_energy_gpu()
            itime, atime, steps, _, _, _ = g.advance(0.25, 1e30, atime)
            e1 = g.get_energy_gpu()
        assert itime >= 0.25 and steps > 0
        res[mode] = abs((e1 - e0) / e0)
    print("N=16384 Salpeter, t=0.25, |dE/E|:", res)
    assert res["mixed"] <= 2.0 * res["fp64"]
