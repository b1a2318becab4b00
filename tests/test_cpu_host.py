"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared symbol, argument validation, the input format, the energy log
format, and the initial-condition generators."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from gravidy_gb300 import _lib, ics
from gravidy_gb300.hermite4 import e2_from_softening
from gravidy_gb300.io import EnergyLog, read_input_file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "gravidy_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(h4_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    syms = _declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)
    assert L.h4_abi_version() == 2


def test_create_validates_arguments_before_touching_the_device():
    L = _lib.load()
    h = C.c_void_p()
    r = np.zeros((4, 4)); v = np.zeros((4, 4))
    assert L.h4_create(C.byref(h), 0, 1e-4, C.c_float(0.01), r.ctypes.data, v.ctypes.data, 0) == 1
    assert L.h4_create(C.byref(h), (1 << 28) + 1, 1e-4, C.c_float(0.01), r.ctypes.data, v.ctypes.data, 0) == 1
    assert b"2^28" in L.h4_last_error()
    assert L.h4_create(C.byref(h), 4, -1.0, C.c_float(0.01), r.ctypes.data, v.ctypes.data, 0) == 1
    assert L.h4_create(C.byref(h), 4, 1e-4, C.c_float(0.01), None, v.ctypes.data, 0) == 1
    assert L.h4_create(C.byref(h), 4, 1e-4, C.c_float(0.01), r.ctypes.data, v.ctypes.data, 7) == 1
    r[2, 1] = np.nan
    assert L.h4_create(C.byref(h), 4, 1e-4, C.c_float(0.01), r.ctypes.data, v.ctypes.data, 0) == 5
    assert b"particle 2" in L.h4_last_error()
    assert L.h4_destroy(None) == 0
    assert L.h4_step(None, None, None, None) == 1


def test_e2_is_the_float_product():
    assert e2_from_softening(0.01) == float(np.float32(np.float32(0.01) * np.float32(0.01)))
    assert e2_from_softening(1e-4) != 1e-8


def test_reader_rounds_mass_to_float_and_stops_at_bad_line(tmp_path):
    p = tmp_path / "in.txt"
    p.write_text("# Time: 0.25\n# comment\n0 0.1 1 2 3 4 5 6\n1 0.3 1e-3 2 3 4 5 6\n2 0.5 1 2 3\n3 0.1 1 1 1 1 1 1\n")
    d = read_input_file(str(p))
    assert d.n == 2 and d.snapshot_time == 0.25
    assert d.mass[0] == float(np.float32(0.1)) and d.mass[1] == float(np.float32(0.3))
    assert d.pos[1, 0] == 1e-3 and d.warnings


def test_reader_drops_last_line_without_newline(tmp_path):
    p = tmp_path / "in.txt"
    p.write_text("0 0.5 1 2 3 4 5 6\n1 0.5 1 2 3 4 5 6")
    assert read_input_file(str(p)).n == 1


def test_energy_log_format():
    log = EnergyLog(stream=False)
    head = log.row(0.0, 0, 0, -0.25, 0.1).splitlines()
    assert head[0].split() == ["#", "IteTime", "Iter", "Nsteps", "Energy", "RelE", "CumE", "ElapsedTime", "GFLOPS"]
    row = log.row(0.125, 486, 28942, -0.25003355903, 0.48, 100, 1.0).split()
    assert row[:4] == ["00", "0.125", "486", "28942"]
    assert row[4] == "-2.5003355903e-01" and row[6] == "1.342361e-04"


@pytest.mark.parametrize("imf", ["equal", "salpeter"])
def test_plummer_henon_units(imf):
    m, p, v = ics.plummer(2000, 5, imf)
    assert abs(m.sum() - 1.0) < 1e-6
    assert np.all(m == m.astype(np.float32))
    k, u = ics.energy(p, v, m)
    assert abs(k + u + 0.25) < 1e-12 and abs(2 * k + u) < 1e-12
    assert np.abs((m[:, None] * p).sum(0)).max() < 1e-12
    if imf == "salpeter":
        mm = m / m.min()
        assert mm.max() > 50   # spans the [0.1, 100] range after normalisation


def test_plummer_is_seeded():
    a = ics.plummer(500, 9)
    b = ics.plummer(500, 9)
    c = ics.plummer(500, 10)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not np.array_equal(a[1], c[1])


def _header_defines():
    text = open(os.path.join(ROOT, "include", "gravidy_gb300.h")).read()
    return {k: int(v) for k, v in re.findall(r"#define\s+(H4_[A-Z0-9_]+)\s+\(?(\d+)", text)}


def test_header_constants_match_the_binding():
    """Constants of include/gravidy_gb300.h used by the Python side."""
    from gravidy_gb300 import ensemble
    d = _header_defines()
    assert d["H4_ENS_TUNE_NB_N"] == ensemble.NB_N and d["H4_ENS_TUNE_NB_A"] == ensemble.NB_A
    assert d["H4_PHASES"] == 8 and d["H4_BUILD_BOUNDS_CHECK"] == 1
    assert _lib.MODES == {"fp64": 0, "exact": 1, "mixed": 2}
    L = _lib.load()
    assert [L.h4_phase_name(k).decode() for k in range(d["H4_PHASES"])] == [
        "prediction", "update", "grav", "correction", "active_set", "next_time", "energy", "advance"]
    assert L.h4_phase_name(d["H4_PHASES"]) == b""
    assert L.h4_build_flags() in (0, d["H4_BUILD_BOUNDS_CHECK"])


def test_committed_tuning_table_is_well_formed():
    """gravidy_gb300/tuning/ensemble_gb300.json: one table per force form
    covering every (N, N_act) bucket (NB_N x NB_A entries).  FP64: ig in
    {1, 2, 4}, chunks multiples of 32.  Mixed: ig 1, 2 or 4 (warp items) or a
    power of two in [16, 512] (block-tiled items), j tiles of 128 or 256 and
    block-item chunks a whole number of tiles; the mixture weights the tuner
    recorded have the same shape."""
    import json
    from gravidy_gb300 import ensemble
    t = json.load(open(ensemble.TUNING_FILE))
    shape = (ensemble.NB_N, ensemble.NB_A)
    for mode in ("fp64", "mixed"):
        T = t["modes"][mode]
        ig = np.array(T["ig"])
        ch = np.array(T["chunk"])
        jt = np.array(T.get("jtile", np.full(shape, 256)))
        assert ig.shape == ch.shape == jt.shape == shape
        assert np.all(ch >= 32) and np.all(ch % 32 == 0)
        if mode == "fp64":
            assert set(np.unique(ig)) <= {1, 2, 4}
        else:
            assert "jtile" in T
            assert set(np.unique(ig)) <= {1, 2, 4, 16, 32, 64, 128, 256, 512}
            assert set(np.unique(jt)) <= {128, 256}
            block = ig >= 16
            assert np.all(ch[block] % jt[block] == 0)
            assert np.array(T["c4_interactions"]).shape == shape


def test_autotuner_candidates_are_valid_table_entries():
    """Every candidate the descent may write passes the same rules as the
    committed table (the library's tuning_valid), for both forms."""
    from gravidy_gb300 import autotune
    for mode in ("fp64", "mixed"):
        d = autotune.default_table(mode)
        assert np.array(d["ig"]).shape == (len(autotune.N_REP), len(autotune.A_LO))
        for b, n in enumerate(autotune.N_REP):
            for a in range(len(autotune.A_LO)):
                if mode == "fp64":
                    cands = autotune.fp64_candidates(n, a, d["chunk"][b][a])
                    assert cands and all(ig in (2, 4) for ig, _, _ in cands)
                else:
                    cands = autotune.mixed_candidates(n, a)
                for ig, chunk, jt in cands:
                    assert ig in (1, 2, 4, 16, 32, 64, 128, 256, 512) and jt in (128, 256)
                    assert chunk % 32 == 0 and chunk <= 2 * n
                    if ig >= 16:
                        assert mode == "mixed" and chunk % jt == 0


def test_autotuner_pick_rule():
    """The descent's pick: the current choice (listed first) stays unless a
    candidate beats it by more than the tie band; among candidates within
    the band of the fastest the earliest wins."""
    from gravidy_gb300.autotune import TIE, pick_within_tie
    assert pick_within_tie([1.0, 0.995, 0.999]) == 0            # within 1 %: keep the current
    assert pick_within_tie([1.0, 0.98, 0.985]) == 1             # beaten by 2 %: the first near-best
    assert pick_within_tie([1.0, 0.985, 0.98]) == 1             # 0.985 is within 1 % of 0.98
    assert pick_within_tie([1.0, 0.97, 0.95]) == 2
    assert pick_within_tie([1.0, 0.97, 0.95], tie=0.05) == 1   # 0.97 <= 0.95 * 1.05
    assert pick_within_tie([1.0, 0.97, 0.95], tie=0.06) == 0   # 1.0 <= 0.95 * 1.06
    times = [0.7791, 0.7817, 0.8027, 0.7660, 0.7718]
    assert pick_within_tie(times) == pick_within_tie(list(times)) == 3   # repeatable
    assert TIE == 0.01


def test_c4_sizes_are_seeded_and_in_range():
    from gravidy_gb300 import workloads
    a = workloads.c4_sizes(256, seed=7)
    b = workloads.c4_sizes(256, seed=7)
    assert np.array_equal(a, b) and len(a) == 256
    assert a.min() >= 512 and a.max() <= 16384
    assert not np.array_equal(a, workloads.c4_sizes(256, seed=8))
