"""The gravidy-gb300 program (C++ drop-in of the reference's main flow) on
the C1 input: its energy log against the reference program's own log."""
import os
import subprocess

import numpy as np
import pytest

from golden_util import case_dir, cases, load_cli_log
from gravidy_gb300.build import CLI, build_cli, build_library

pytestmark = pytest.mark.gpu


def _run(tmp_path, name, mode, extra=()):
    build_library()
    build_cli()
    c = cases()[name]
    out = os.path.join(str(tmp_path), "run")
    cmd = [CLI, "-i", os.path.join(case_dir(name), "input.txt"), "-s", repr(c["softening"]),
           "-e", repr(c["eta"]), "-t", repr(c["t_end"]), "-z", repr(c["interval"]), "-o", out,
           "--mode", mode, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = []
    for line in open(out + ".out.log"):
        if line.startswith("#"):
            continue
        t = line.split()
        rows.append((t[1], t[2], t[3], float(t[4]), float(t[5]), float(t[6])))
    return rows, out


@pytest.mark.parametrize("extra", [(), ("--host-steps",)])
def test_cli_exact_mode_energy_log_matches_reference(tmp_path, extra):
    name = "c1_plummer_n1024"
    rows, out = _run(tmp_path, name, "exact", extra)
    ref = load_cli_log(name)
    assert len(rows) == len(ref)
    for mine, theirs in zip(rows, ref):
        assert mine[:3] == theirs[:3]
        assert abs(mine[3] - float(theirs[3])) <= 1e-10 * abs(float(theirs[3]))
        assert abs(mine[5] - float(theirs[5])) <= 1e-5 * max(float(theirs[5]), 1e-12)
    # snapshots and info file in the reference's layout
    assert os.path.exists(out + ".out.info")
    snaps = sorted(f for f in os.listdir(tmp_path) if ".snapshot_" in f)
    assert len(snaps) == len(ref) + 1
    with open(os.path.join(tmp_path, snaps[0])) as fh:
        head = fh.readline()
        assert head.startswith("# Time:")
        assert len(fh.readline().split()) == 8


def test_cli_fp64_energy_error_matches_reference(tmp_path):
    name = "c1_plummer_n1024"
    rows, _ = _run(tmp_path, name, "fp64")
    ref = load_cli_log(name)
    assert [r[0] for r in rows] == [r[0] for r in ref]
    cum, cum_ref = rows[-1][5], float(ref[-1][5])
    assert abs(cum - cum_ref) <= 1e-2 * cum_ref


def test_cli_lagrange_radii_file(tmp_path):
    """-l writes the Lagrange radii at t = 0 and every output time in the
    reference's format; the t = 0 row equals the reference's values."""
    name = "c1_plummer_n1024"
    _, out = _run(tmp_path, name, "exact", ("-l",))
    rows = [l.split() for l in open(out + ".out.radii")]
    assert len(rows) == 1 + 8 and all(r[0] == "01" and len(r) == 8 for r in rows)
    want = None
    for line in open(os.path.join(case_dir(name), "attributes.txt")):
        if line.startswith("t0_lagr"):
            want = [float.fromhex(t) for t in line.split()[1:7]]
    assert [float(x) for x in rows[0][2:8]] == pytest.approx(want, rel=1e-5, abs=1e-6)


def test_cli_resume_from_info_file(tmp_path):
    """-r <out>.info (the reference's resume, OptionsParser.cpp:122-323):
    the run restarts at the info file's IntegrationTime from the snapshot the
    file names (a 4-digit counter) and logs to <input>.out.log.  In the exact
    mode its log equals the oracle's replay of the reference's loop
    (Hermite4GPU_integration.cpp:38-124) from that snapshot's state at that
    time: the same rows, iteration and step counters, energies to 1e-10.  The
    old info file is kept as <info>.old."""
    from gravidy_gb300.io import read_input_file
    from oracle import oracle as orc
    build_library()
    build_cli()
    name = "salpeter_n100"
    c = cases()[name]
    inp = tmp_path / "in.txt"
    inp.write_text(open(os.path.join(case_dir(name), "input.txt")).read())
    t1, t2, dz = 2.0 ** -4, 2.0 ** -3, 2.0 ** -11
    common = ["-s", repr(c["softening"]), "-e", repr(c["eta"]), "-z", repr(dz), "--mode", "exact"]
    r = subprocess.run([CLI, "-i", str(inp), "-t", repr(t1), "-o", str(tmp_path / "run"), *common],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    info = {l.split(":")[0].strip("# "): l.split(":", 1)[1].strip() for l in open(tmp_path / "run.out.info")}
    snap = tmp_path / f"run.out.snapshot_{int(info['SnapshotNumber']):04d}"
    assert snap.exists()
    r = subprocess.run([CLI, "-r", str(tmp_path / "run.out.info"), "-t", repr(t2), *common],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "run.out.info.old").exists()
    got = [l.split()[1:5] for l in open(str(inp) + ".out.log") if not l.startswith("#")]
    # the oracle, from the snapshot's state at the info file's time
    d = read_input_file(str(snap))
    o = orc.Oracle(d.mass, d.pos, d.vel, orc.e2_from_softening(c["softening"]), c["eta"])
    o.init_acc_jrk()
    itime = float(np.float32(t1))
    atime = o.init_dt(itime, float(orc.ETA_S))
    want = [(itime, 0, 0, o.energy()[0])]
    it, ns, k = 0, 0, 1
    while itime < float(np.float32(t2)):
        nact, itime, atime = o.block_step(itime, atime)
        if itime >= float(np.float32(np.float32(dz) * np.float32(k))):
            want.append((itime, it, ns, o.energy()[0]))
            k += 1
        ns += nact
        it += 1
    assert len(got) == len(want) > 1
    for g, w in zip(got, want):
        # the log prints the time with 3 decimals (0.0625 -> "0.062")
        assert abs(float(g[0]) - w[0]) <= 5e-4 + 1e-9 and (int(g[1]), int(g[2])) == (w[1], w[2])
        assert abs(float(g[3]) - w[3]) <= 1e-10 * abs(w[3])
