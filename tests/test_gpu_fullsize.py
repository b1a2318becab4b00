"""Parity at the benchmark sizes, through properties that do not need a full
O(N^2) CPU reference:

  * N = 2^20 (C5) and N = 65536 (C2): acc/jerk of 512 sampled particles
    against the oracle's per-particle sums (the oracle does only the sampled
    rows, O(sample * N)), FP64 within 1e-12 and mixed within 1e-4;
  * momentum balance of the all-active force sum: sum_i m_i a_i and
    sum_i m_i a1_i vanish to rounding (Newton's third law), relative to
    sum_i m_i |a_i|;
  * a block step is deterministic: two runs give bit-identical states.
"""
import numpy as np
import pytest

from h4_util import rel_err_vec
from gravidy_gb300 import Hermite4GPU, NbodySystem, ics
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,imf,soft", [(1 << 20, "salpeter", 0.0031623), (65536, "equal", 0.01)])
def test_sampled_forces_at_full_size(n, imf, soft):
    m, p, v = ics.plummer(n, 5, imf)
    ns = NbodySystem(m, p, v, softening=soft)
    rng = np.random.default_rng(n)
    move = np.sort(rng.choice(n, size=512, replace=False)).astype(np.uint32)
    pr = np.zeros((n, 4)); pr[:, :3] = p; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = v
    want = orc.forces_for(orc.make_predictors(ns.mass, p, v), ns.e2, move)
    for mode, tol in (("fp64", 1e-12), ("mixed", 1e-4)):
        with Hermite4GPU(ns, mode=mode) as g:
            got = g.forces_for(pr, pv, move)
        assert rel_err_vec(got[:, :3], want[:, :3]).max() < tol, mode
        assert rel_err_vec(got[:, 3:], want[:, 3:]).max() < tol, mode


@pytest.mark.parametrize("n", [65536, 1 << 18])
def test_momentum_balance_all_active(n):
    m, p, v = ics.plummer(n, 7, "salpeter")
    ns = NbodySystem(m, p, v, softening=0.01)
    for mode, tol in (("fp64", 1e-12), ("mixed", 1e-5)):
        with Hermite4GPU(ns, mode=mode) as g:
            g.init_acc_jrk()
            f = g.download()["f"]
        w = ns.mass[:, None]
        for a in (f[:, :3], f[:, 3:]):
            net = np.abs((w * a).sum(axis=0)).max()
            scale = (w * np.abs(a)).sum()
            assert net < tol * scale, (mode, net / scale)


def test_block_steps_deterministic_at_65536():
    m, p, v = ics.plummer(65536, 9, "equal")
    ns = NbodySystem(m, p, v, softening=0.01)
    states = []
    for _ in range(2):
        with Hermite4GPU(ns) as g:
            g.init_acc_jrk()
            at = g.init_dt(1.0e10, 0.01, 0.0)
            g.advance(1.0 / 256, 1e30, at)
            states.append(g.download())
    for k in ("r", "v", "f", "dt", "t"):
        assert np.array_equal(states[0][k], states[1][k]), k
