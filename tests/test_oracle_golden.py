"""The CPU restatement (oracle/h4_oracle.c) against the reference itself.

The fixtures in tests/golden/ were written by the reference GraviDy sources
compiled unmodified (tests/golden/make_golden.py).  These tests pin the
restatement bit for bit: initial forces and timesteps, the active set and the
full state after every traced block step, the energies at every log time and
the final state, and the deterministic columns of the reference program's
own energy log.
"""
import numpy as np
import pytest

from golden_util import cases, load_cli_log, load_energy, load_init, load_state, load_steps, case_dir
from gravidy_gb300.io import EnergyLog, read_input_file
from oracle import oracle as orc

CASES = cases()


def _make(name):
    c = CASES[name]
    data = read_input_file(case_dir(name) + "/input.txt")
    assert data.n == c["n"]
    e2 = orc.e2_from_softening(c["softening"])
    return c, data, orc.Oracle(data.mass, data.pos, data.vel, e2, c["eta"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_init_forces_and_dt_bit_exact(name):
    c, data, o = _make(name)
    o.init_acc_jrk()
    atime = o.init_dt(0.0, float(orc.ETA_S))
    f, dt, at = load_init(name, c["n"])
    assert np.array_equal(o.f.view(np.uint64), f.view(np.uint64))
    assert np.array_equal(o.dt.view(np.uint64), dt.view(np.uint64))
    assert atime == at


@pytest.mark.parametrize("name", sorted(CASES))
def test_block_steps_trace_bit_exact(name):
    c, data, o = _make(name)
    rows, summary = load_steps(name)
    energies = load_energy(name)
    o.init_acc_jrk()
    atime = o.init_dt(0.0, float(orc.ETA_S))
    e0, _, _ = o.energy()
    assert (0.0, e0) == energies[0]
    want = {r[0]: r for r in rows}
    itime, step, out_factor, nsteps, k_e = 0.0, 0, 1, 0, 1
    t_end, interval = np.float32(c["t_end"]), np.float32(c["interval"])
    while itime < t_end:
        nact, itime, atime = o.block_step(itime, atime)
        if itime >= float(interval * np.float32(out_factor)):
            e, _, _ = o.energy()
            assert energies[k_e] == (itime, e), f"energy at log {k_e}"
            k_e += 1
            out_factor += 1
        nsteps += nact
        if step in want:
            s, it, na, hm, hs = want[step]
            assert it == itime and na == nact, f"step {step}"
            assert orc.fnv1a(o.move[:nact]) == hm, f"active set at step {step}"
            assert o.state_hash() == hs, f"state at step {step}"
        step += 1
    assert step == summary["steps"] and nsteps == summary["nsteps"]
    assert k_e == len(energies)
    final = load_state(name, "final", c["n"])
    assert np.array_equal(o.state_record().view(np.uint64), final.view(np.uint64))


@pytest.mark.parametrize("name", sorted(n for n in CASES if CASES[n].get("cli_returncode") == 0))
def test_energy_log_columns_match_reference_program(name):
    c, data, o = _make(name)
    st, rows = o.integrate(c["t_end"], c["interval"])
    log = EnergyLog(stream=False)
    mine = []
    for itime, it, ns, e in rows:
        text = log.row(itime, int(it), int(ns), e, 0.0).splitlines()[-1].split()
        mine.append(tuple(text[1:7]))
    ref = load_cli_log(name)
    assert mine == ref


def _attributes(name):
    rows = {}
    with open(case_dir(name) + "/attributes.txt") as fh:
        for line in fh:
            tok = line.split()
            rows[tok[0]] = [float.fromhex(t) for t in tok[1:]]
    return rows


@pytest.mark.parametrize("name", ["c1_plummer_n1024", "salpeter_n100", "ragged_n33"])
def test_diagnostics_bit_exact(name):
    """nbody_attributes and lagrange_radii (NbodyUtils.cpp:59-328) at t = 0
    and at the end, in the reference's call order (the core radius uses the
    center of density left by the previous call)."""
    c = CASES[name]
    want = _attributes(name)
    c_, data, o = _make(name)
    tm = o.total_mass()
    assert tm == want["total_mass"][0]
    cod_state = np.zeros(3)
    o.init_acc_jrk()
    atime = o.init_dt(0.0, float(orc.ETA_S))
    e0, _, _ = o.energy()
    for tag in ("t0", "end"):
        attr = o.nbody_attributes(e0, tm, cod_state)
        assert list(attr) == want[f"{tag}_attr"], tag
        cod = o.center_of_density()
        core, half, lag = o.mass_radii(cod, tm)
        assert list(lag) + list(cod) == want[f"{tag}_lagr"], tag
        cod_state[:] = cod
        if tag == "t0":
            itime = 0.0
            t_end = np.float32(c["t_end"])
            while itime < t_end:
                _, itime, atime = o.block_step(itime, atime)
