"""Failure handling without faulting the GPU: non-finite state reported as a
status (and the device loop stopping), a failing system of an ensemble
stopping alone, and a bounded device wait running out on a flag that nothing
sets.  No test traps, faults or hangs the device; the context stays usable
after each."""
import ctypes as C

import numpy as np
import pytest

from gravidy_gb300 import Hermite4GPU, NbodySystem, _lib, ics
from gravidy_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu


def _system(n=256, seed=3):
    m, p, v = ics.plummer(n, seed)
    return NbodySystem(m, p, v, softening=0.01)


def test_nonfinite_state_is_reported_by_step_and_advance():
    for use_advance in (False, True):
        with Hermite4GPU(_system()) as g:
            g.init_acc_jrk()
            at = g.init_dt(1.0e10, 0.01, 0.0)
            st = g.download()
            st["v"][5, 0] = np.nan          # injected on the host
            g.upload(v=st["v"])
            with pytest.raises(_lib.H4Error) as ei:
                if use_advance:
                    g.advance(0.125, 1e30, at)
                else:
                    g.step(at)
            assert ei.value.status == 5     # H4_ERR_NONFINITE
    # the device is still usable
    with Hermite4GPU(_system()) as g:
        g.init_acc_jrk()
        at = g.init_dt(1.0e10, 0.01, 0.0)
        nact, it, at2 = g.step(at)
        assert nact > 0 and it == at


def test_ensemble_failing_system_stops_alone():
    good = []
    for k, n in enumerate((200, 300)):
        m, p, v = ics.plummer(n, 40 + k)
        good.append((m, p, v, 0.01, 0.01))
    # two coincident particles and no softening: non-finite forces
    m, p, v = ics.plummer(64, 49)
    p[1] = p[0]
    bad = (m, p, v, 0.0, 0.01)
    with Ensemble([good[0], bad, good[1]], mode="fp64") as E:
        E.init()
        with pytest.raises(_lib.H4Error) as ei:
            E.advance(0.0625)
        assert ei.value.status == 5
        st = E.stats()
    assert st["itime"][0] >= 0.0625 and st["itime"][2] >= 0.0625
    assert st["itime"][1] < 0.0625


def test_bounded_wait_times_out_and_context_survives():
    L = _lib.load()
    t = C.c_int(-1)
    _lib.check(L.h4_selftest_bounded_wait(0.2, C.byref(t)))
    assert t.value == 1
    with Hermite4GPU(_system(64)) as g:
        g.init_acc_jrk()
        assert np.all(np.isfinite(g.download()["f"]))
