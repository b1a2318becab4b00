"""Exact checkpoint/resume: a run stopped at a log time and resumed from its
checkpoint ends in the bit-identical state of the uninterrupted run (Python
API and the gravidy-gb300 program, -r)."""
import os
import subprocess

import numpy as np
import pytest

from golden_util import case_dir, cases
from h4_util import golden_system
from gravidy_gb300 import Hermite4GPU
from gravidy_gb300.build import CLI, build_cli, build_library
from gravidy_gb300.checkpoint import read_checkpoint

pytestmark = pytest.mark.gpu


def test_python_checkpoint_resume_bit_identical(tmp_path):
    ns = golden_system("c1_plummer_n1024")
    with Hermite4GPU(ns) as g:
        g.init_acc_jrk()
        at = g.init_dt(1.0e10, 0.01, 0.0)
        it, at, *_ = g.advance(1.0, 1e30, at)
        want = g.download()
    ns = golden_system("c1_plummer_n1024")
    path = str(tmp_path / "c1.chk")
    with Hermite4GPU(ns) as g:
        g.init_acc_jrk()
        at = g.init_dt(1.0e10, 0.01, 0.0)
        it, at, *_ = g.advance(1.0, 0.5, at)
        assert 0.5 <= it < 1.0
        g.save_checkpoint(path, it, at)
    g2, it2, at2, sc = Hermite4GPU.from_checkpoint(path)
    with g2:
        assert it2 == it and at2 == at
        it3, at3, *_ = g2.advance(1.0, 1e30, at2)
        got = g2.download()
    for k in ("r", "v", "f", "t", "dt"):
        assert np.array_equal(got[k], want[k]), k


def _cli(args):
    build_library()
    build_cli()
    r = subprocess.run([CLI, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def test_cli_resume_bit_identical(tmp_path):
    c = cases()["c1_plummer_n1024"]
    inp = os.path.join(case_dir("c1_plummer_n1024"), "input.txt")
    common = ["-s", repr(c["softening"]), "-e", repr(c["eta"]), "-z", "0.125"]
    full = str(tmp_path / "full")
    _cli(["-i", inp, "-t", "1", "-o", full, *common])
    half = str(tmp_path / "half")
    _cli(["-i", inp, "-t", "0.5", "-o", half, *common])
    _cli(["-r", half + ".out.chk", "-t", "1", "-o", half, *common])
    a, sa, _ = read_checkpoint(full + ".out.chk")
    b, sb, _ = read_checkpoint(half + ".out.chk")
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert sa["iterations"] == sb["iterations"] and sa["nsteps"] == sb["nsteps"]
    rows = lambda p: [l.split()[:7] for l in open(p + ".out.log") if not l.startswith("#")]
    assert rows(full) == rows(half)
