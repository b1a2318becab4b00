"""The C ABI from a plain C99 program (tests/c_abi/block_steps.c).

CPU: the header compiles as strict C99 (-pedantic -Werror), the program links
against libgravidy_gb300.so, and an invalid creation is refused with a status
and a message before any device work.  GPU: the program runs the reference's
block-step loop (Hermite4GPU_integration.cpp:81-99) through the C ABI and
ends bit-identical to the Python binding driving the same methods.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from gravidy_gb300.build import ROOT, build_library

HERE = os.path.dirname(os.path.abspath(__file__))


def _compile(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = build_library()
    exe = str(tmp_path / "block_steps")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-O2",
                        "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c_abi", "block_steps.c"),
                        "-L", os.path.dirname(lib), "-lgravidy_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}",
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c99_program_builds_and_gets_a_status_without_a_gpu(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("refused 1 ")


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_c99_program_matches_python_binding(tmp_path, mode):
    from gravidy_gb300 import Hermite4GPU, NbodySystem, ics
    exe = _compile(tmp_path)
    m, p, v = ics.plummer(1500, 77, "salpeter")
    ns = NbodySystem(m, p, v, softening=0.01, eta=0.01)
    state = tmp_path / "state.bin"
    with open(state, "wb") as fh:
        fh.write(struct.pack("<Idf", ns.n, ns.e2, ns.eta))
        fh.write(np.ascontiguousarray(ns.h_r, dtype=np.float64).tobytes())
        fh.write(np.ascontiguousarray(ns.h_v, dtype=np.float64).tobytes())
    t_end = 0.0625
    r = subprocess.run([exe, str(state), repr(t_end), mode], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    tok = r.stdout.split()
    got = {"steps": int(tok[1]), "itime": float.fromhex(tok[3]), "atime": float.fromhex(tok[5]),
           "energy": float.fromhex(tok[7]), "r0": [float.fromhex(x) for x in tok[9:12]]}
    with Hermite4GPU(ns, mode=mode) as g:
        g.init_acc_jrk()
        atime = g.init_dt(1.0e10, 0.01, 0.0)
        itime, steps = 0.0, 0
        while itime < t_end:
            itime = atime
            nact = g.find_particles_to_move(itime)
            g.save_old_acc_jrk(nact)
            g.predicted_pos_vel(itime)
            g.update_acc_jrk(nact)
            g.correction_pos_vel(itime, nact)
            atime = g.next_integration_time()
            steps += 1
        e = g.get_energy_gpu()
        r0 = g.download()["r"][0, :3].tolist()
    assert got == {"steps": steps, "itime": itime, "atime": atime, "energy": e, "r0": r0}
