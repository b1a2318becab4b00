"""CUDA path (through the C ABI) against the oracle and the golden traces.

Tolerances (from the parity contract of the FP64 drop-in):
  * predictor, corrector, timesteps, active sets: bit-exact;
  * acc and jerk of the FP64 force kernel: per-particle relative error of the
    3-vector below 1e-12 (FORCE_RTOL);
  * the exact force mode: bit-exact forces, hence the reference's trace.
"""
import numpy as np
import pytest

from golden_util import cases, load_energy, load_init, load_steps
from h4_util import gpu_record, golden_system, oracle_for, plummer_system, rel_err_vec, state_hash
from gravidy_gb300 import Hermite4GPU
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
FORCE_RTOL = 1e-12
ENERGY_RTOL = 1e-12
CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_mode_reproduces_reference_trace(name):
    """Exact force mode + exact integrator kernels = the reference's traced
    state hashes at every recorded block step, and its final state."""
    c = CASES[name]
    ns = golden_system(name)
    rows, summary = load_steps(name)
    want = {r[0]: r for r in rows}
    with Hermite4GPU(ns, mode="exact") as g:
        g.init_acc_jrk()
        atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        f0, dt0, at0 = load_init(name, c["n"])
        st = g.download()
        assert np.array_equal(st["f"].view(np.uint64), f0.view(np.uint64))
        assert np.array_equal(st["dt"].view(np.uint64), dt0.view(np.uint64))
        assert atime == at0
        itime, step = 0.0, 0
        t_end = float(np.float32(c["t_end"]))
        while itime < t_end:
            nact, itime, atime = g.step(atime)
            if step in want:
                _, it, na, hm, hs = want[step]
                assert (itime, nact) == (it, na), f"step {step}"
                st = g.download()
                assert orc.fnv1a(st["move"][:nact]) == hm, f"active set, step {step}"
                assert state_hash(gpu_record(st)) == hs, f"state, step {step}"
            step += 1
        assert step == summary["steps"]


def test_fp64_init_forces_vs_oracle():
    ns = golden_system("c1_plummer_n1024")
    o = oracle_for(ns)
    o.init_acc_jrk()
    with Hermite4GPU(ns) as g:
        g.init_acc_jrk()
        f = g.download()["f"]
    assert rel_err_vec(f[:, :3], o.f[:, :3]).max() < FORCE_RTOL
    assert rel_err_vec(f[:, 3:], o.f[:, 3:]).max() < FORCE_RTOL


@pytest.mark.parametrize("n,nact", [(1000, 1), (1000, 31), (1000, 33), (4099, 4099), (4099, 7),
                                    (65536, 1), (65536, 37), (65536, 5000)])
def test_fp64_forces_random_active_sets(n, nact):
    ns = plummer_system(n, seed=11, imf="salpeter")
    rng = np.random.default_rng(n + nact)
    move = np.sort(rng.choice(n, size=nact, replace=False)).astype(np.uint32)
    # predictors = state plus small random displacement (independent positions)
    pr = np.zeros((n, 4)); pr[:, :3] = ns.pos + 1e-3 * rng.standard_normal((n, 3)); pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = ns.vel
    p = orc.make_predictors(ns.mass, pr[:, :3], pv[:, :3])
    want = orc.forces_for(p, ns.e2, move)
    with Hermite4GPU(ns) as g:
        got = g.forces_for(pr, pv, move)
    assert rel_err_vec(got[:, :3], want[:, :3]).max() < FORCE_RTOL
    assert rel_err_vec(got[:, 3:], want[:, 3:]).max() < FORCE_RTOL


def test_fp64_block_steps_bit_exact_levels_first_steps():
    """FP64 forces (not bit-identical) still give the reference's active sets
    and timestep levels bit for bit over the first 300 block steps of C1."""
    name = "c1_plummer_n1024"
    ns = golden_system(name)
    rows, _ = load_steps(name)
    o = oracle_for(ns)
    o.init_acc_jrk()
    oat = o.init_dt(0.0, float(orc.ETA_S))
    with Hermite4GPU(ns) as g:
        g.init_acc_jrk()
        atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        assert atime == oat
        oit = 0.0
        for step in range(300):
            nact, itime, atime = g.step(atime)
            onact, oit, oat = o.block_step(oit, oat)
            assert (nact, itime, atime) == (onact, oit, oat), f"step {step}"
            st = g.download()
            assert np.array_equal(st["move"][:nact], o.move[:nact])
            assert np.array_equal(st["dt"], o.dt), f"levels at step {step}"
            assert np.array_equal(st["t"], o.t)
            assert rows[step][2] == nact


def test_predictor_and_corrector_bit_exact_on_same_inputs():
    """Give the GPU and the oracle identical forces; the predictor and the
    corrector (with its timestep) then agree bit for bit."""
    ns = golden_system("c1_plummer_n1024")
    o = oracle_for(ns)
    o.init_acc_jrk()
    oat = o.init_dt(0.0, float(orc.ETA_S))
    with Hermite4GPU(ns, mode="exact") as g:
        g.init_acc_jrk()
        atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        oit = 0.0
        for step in range(40):
            # oracle step; GPU takes the same steps with the separate methods
            itime = atime
            nact = g.find_particles_to_move(itime)
            g.save_old_acc_jrk(nact)
            g.predicted_pos_vel(itime)
            onact, oit, oat = o.block_step(oit, oat)
            pr, pv = g.download_predicted()
            assert np.array_equal(pr[:, :3], o.p["r"]) and np.array_equal(pv[:, :3], o.p["v"])
            # the same forces as the oracle (uploaded), then the corrector
            st = g.download()
            f = st["f"].copy()
            f[o.move[:onact]] = o.f[o.move[:onact]]
            g.upload(f=f)
            g.correction_pos_vel(itime, nact)
            atime = g.next_integration_time()
            st = g.download()
            assert (nact, itime, atime) == (onact, oit, oat)
            assert np.array_equal(st["r"], o.r) and np.array_equal(st["v"][:, :3], o.v[:, :3])
            assert np.array_equal(st["a2"], o.a2) and np.array_equal(st["a3"], o.a3)
            assert np.array_equal(st["dt"], o.dt) and np.array_equal(st["t"], o.t)


@pytest.mark.parametrize("name", ["c1_plummer_n1024", "ragged_n33", "binary_n2", "single_n1"])
def test_energy_vs_oracle(name):
    ns = golden_system(name)
    o = oracle_for(ns)
    e_ref, k_ref, p_ref = o.energy()
    with Hermite4GPU(ns) as g:
        e = g.get_energy_gpu()
        assert abs(g.ekin - k_ref) <= ENERGY_RTOL * abs(k_ref)
        assert abs(g.epot - p_ref) <= ENERGY_RTOL * max(abs(p_ref), 1e-300)
        assert abs(e - e_ref) <= ENERGY_RTOL * abs(e_ref) * 10


def test_energy_at_log_times_matches_golden_exact_mode():
    name = "c1_plummer_n1024"
    energies = load_energy(name)
    ns = golden_system(name)
    with Hermite4GPU(ns, mode="exact") as g:
        log = g.integration(fused=True, log=__import__("gravidy_gb300").EnergyLog(stream=False))
    got = [(r[0], r[3]) for r in log.rows]
    assert len(got) == len(energies)
    for (t1, e1), (t2, e2) in zip(got, energies):
        assert t1 == t2
        assert abs(e1 - e2) <= 1e-13 * abs(e2)


def test_fp64_c1_energy_error_within_1e2_of_reference():
    """C1 (N=1024 Plummer to t=1): |dE/E| at t=1 within 1e-2 (relative) of
    the reference's value."""
    name = "c1_plummer_n1024"
    energies = load_energy(name)
    ref_cum = abs((energies[-1][1] - energies[0][1]) / energies[0][1])
    ns = golden_system(name)
    with Hermite4GPU(ns) as g:
        log = g.integration(fused=True, log=__import__("gravidy_gb300").EnergyLog(stream=False))
    cum = log.rows[-1][5]
    assert abs(cum - ref_cum) <= 1e-2 * ref_cum, (cum, ref_cum)


def test_advance_graph_equals_host_driven_steps():
    ns = golden_system("salpeter_n100")
    with Hermite4GPU(ns) as a, Hermite4GPU(ns) as b:
        for g in (a, b):
            g.init_acc_jrk()
        ta = a.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        tb = b.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        itime_b, steps_b, ps_b = 0.0, 0, 0
        while itime_b < 0.0625:
            nact, itime_b, tb = b.step(tb)
            steps_b += 1
            ps_b += nact
        itime_a, ta, steps_a, ps_a, inter_a, last = a.advance(0.0625, 1e30, ta)
        assert (itime_a, ta, steps_a, ps_a) == (itime_b, tb, steps_b, ps_b)
        sa, sb = a.download(), b.download()
        for k in ("r", "v", "f", "t", "dt"):
            assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.gpu
def test_phase_timers_count_host_driven_calls():
    """Per-phase device timers (the reference's Gtime phases, common.hpp:287-310)."""
    ns = plummer_system(2048, seed=5)
    with Hermite4GPU(ns) as g:
        g.init_acc_jrk()
        atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        steps = 6
        for _ in range(steps):
            itime = atime
            nact = g.find_particles_to_move(itime)
            g.save_old_acc_jrk(nact)
            g.predicted_pos_vel(itime)
            g.update_acc_jrk(nact)
            g.correction_pos_vel(itime, nact)
            atime = g.next_integration_time()
        g.get_energy_gpu()
        g.advance(atime + 2.0 ** -8, 1e30, atime)
        ph = g.phase_times()
    assert list(ph) == ["prediction", "update", "grav", "correction", "active_set",
                        "next_time", "energy", "advance"]
    for k in ("prediction", "update", "grav", "correction", "active_set", "next_time"):
        assert ph[k][1] == steps, k
        assert ph[k][0] > 0.0, k
    assert ph["energy"][1] == 1 and ph["advance"][1] == 1
    assert ph["grav"][0] <= ph["update"][0]


@pytest.mark.parametrize("limits", [(2.0 ** -9, 2.0 ** -6), (2.0 ** -14, 2.0 ** -12)])
def test_exact_mode_narrow_dt_limits_bit_exact(limits):
    """Narrow timestep bounds (h4_set_dt_limits, D_TIME_MIN/D_TIME_MAX of
    common.hpp:122,129) make most new timesteps hit a clamp of
    NbodyUtils::normalize_dt (NbodyUtils.cpp:371-424) and of init_dt
    (Hermite4.cpp:131-135); the exact mode still follows the oracle bit for
    bit through both."""
    dt_min, dt_max = limits
    ns = golden_system("salpeter_n100")
    o = oracle_for(ns, dt_min=dt_min, dt_max=dt_max)
    o.init_acc_jrk()
    oat = o.init_dt(0.0, float(orc.ETA_S))
    with Hermite4GPU(ns, mode="exact", dt_min=dt_min, dt_max=dt_max) as g:
        g.init_acc_jrk()
        atime = g.init_dt(1.0e10, float(orc.ETA_S), 0.0)
        assert atime == oat
        assert np.array_equal(g.download()["dt"], o.dt)
        oit = 0.0
        clamped = 0
        for step in range(120):
            nact, itime, atime = g.step(atime)
            onact, oit, oat = o.block_step(oit, oat)
            assert (nact, itime, atime) == (onact, oit, oat), f"step {step}"
            st = g.download()
            assert np.array_equal(st["dt"], o.dt) and np.array_equal(st["t"], o.t), f"step {step}"
            assert np.array_equal(st["r"], o.r), f"step {step}"
            clamped += int(np.sum((o.dt == dt_min) | (o.dt == dt_max)))
        assert clamped > 0   # the clamps were exercised
