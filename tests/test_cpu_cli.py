"""The gravidy-gb300 program's command line without a GPU: the reference's
flags are parsed (OptionsParser.cpp), bad input is refused with a message
and a non-zero status, and with no CUDA device the program stops cleanly
after a clear error instead of crashing."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from golden_util import case_dir
from gravidy_gb300 import _lib
from gravidy_gb300.build import CLI, build_cli, build_library


def _cli():
    build_library()
    if build_cli() is None:
        pytest.skip("no host sources")
    return CLI


def _run(*args):
    return subprocess.run([_cli(), *args], capture_output=True, text=True, timeout=120)


def test_usage_and_bad_arguments():
    r = _run()
    assert r.returncode != 0 and "--input" in r.stdout + r.stderr
    r = _run("-i", "/nonexistent/input.dat", "-t", "1")
    assert r.returncode != 0 and "cannot access" in r.stdout + r.stderr
    inp = os.path.join(case_dir("c1_plummer_n1024"), "input.txt")
    r = _run("-i", inp, "-t", "1", "--mode", "quad")
    assert r.returncode != 0 and "--mode" in r.stdout + r.stderr


def test_no_device_is_a_clean_error(tmp_path):
    L = _lib.load()
    h = C.c_void_p()
    r4 = np.zeros((2, 4)); r4[1, 0] = 1.0; r4[:, 3] = 0.5
    v4 = np.zeros((2, 4))
    if L.h4_create(C.byref(h), 2, 1e-4, C.c_float(0.01), r4.ctypes.data, v4.ctypes.data, 0) == 0:
        L.h4_destroy(h)
        pytest.skip("a CUDA device is present")
    inp = os.path.join(case_dir("c1_plummer_n1024"), "input.txt")
    r = _run("-i", inp, "-t", "0.125", "-o", str(tmp_path / "run"))
    assert r.returncode not in (0, -11, 139)   # an error status, not success and not SIGSEGV
    assert "CUDA" in r.stdout + r.stderr


def _info(path, **over):
    keys = {"NumberParticles": "33", "Softening": "0.05", "EtaTimestep": "0.01", "IntegrationTime": "0.0625",
            "PrintScreen": "0", "InputFilename": str(path / "in.txt"), "OutputFilename": str(path / "run.out"),
            "SnapshotNumber": "7"}
    keys.update(over)
    with open(path / "run.out.info", "w") as fh:
        for k, v in keys.items():
            fh.write(f"# {k + ':':<20}{v:>20}\n")
    return str(path / "run.out.info")


def test_resume_from_info_file_arguments(tmp_path):
    """-r <out>.info follows the reference's resume rules
    (OptionsParser.cpp:122-323) before any device work: -t is required and
    must exceed the info file's IntegrationTime, every key must be known, and
    the snapshot it names (4-digit counter) must exist."""
    info = _info(tmp_path)
    r = _run("-r", info)
    assert r.returncode != 0 and "'time'" in r.stderr
    r = _run("-r", info, "-t", "0.0625")
    assert r.returncode != 0 and "greater than the one" in r.stderr
    r = _run("-r", info, "-t", "0.125")
    assert r.returncode != 0 and "run.out.snapshot_0007" in r.stderr
    r = _run("-r", _info(tmp_path, Colour="blue"), "-t", "0.125")
    assert r.returncode != 0 and "Invalid option -- Colour" in r.stderr
