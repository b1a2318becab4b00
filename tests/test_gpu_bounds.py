"""Bounds-checked build on ragged sizes (a stand-in for a memory checker).

The library is built a second time with -DH4_BOUNDS_CHECK: every kernel then
checks the index ranges it touches (active list, particle indices, j range,
partial-force area, ensemble system ranges) and a violation fails the call
instead of reading or writing out of bounds.  tests/bounds_scenarios.py runs
single systems in every force form and kernel shape, the allocation-free
entry point, diagnostics and ensembles at N = 1, 2, 31, 33, 257, 513, 1000,
1500, 2500 under both builds, in child processes; the checked build must report
no violation and give bit-identical results to the normal one.  The checked
build also runs one failing allocation-free call (an active list naming a
particle past n, which its checks refuse) and then a good one.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(lib_path):
    env = dict(os.environ, GRAVIDY_GB300_LIB=lib_path)
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_scenarios.py")], env=env, text=True,
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_bounds_checked_build_clean_and_identical():
    from gravidy_gb300.build import LIB, build_library
    bounds_lib = build_library(bounds_check=True)
    normal = _run(LIB)
    checked = _run(bounds_lib)
    assert normal["build_flags"] == 0
    assert checked["build_flags"] == 1
    assert set(checked["results"]) == set(normal["results"])
    diff = {k: (normal["results"][k], checked["results"][k]) for k in normal["results"]
            if normal["results"][k] != checked["results"][k]}
    assert not diff, diff
    # a failed allocation-free call leaves no error behind for the next call
    assert checked["checked_only"] == {"noalloc_recovers": True}
