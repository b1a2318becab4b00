"""Ragged-size scenarios run under the normal and the bounds-checked library.

Run as a child process (``python tests/bounds_scenarios.py``) with
GRAVIDY_GB300_LIB naming the library to load; prints one JSON object: the
library's build flags and, per scenario, a hash of every result.  The
bounds-checked build checks every index range its kernels touch and fails a
call that would have accessed memory out of bounds, so the scenarios passing
there with the same hashes as in the normal build means no kernel stepped
outside its arrays on these sizes and the checks changed no result.

Sizes are the ragged ones: N = 1, 2, 31, 33, 257, 1000 (none a multiple of a
tile or a chunk), active sets of 1, 31, 33 and all particles, the mixed
form on both of its kernel shapes, ensembles with systems below and above
the block-tiled threshold.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from gravidy_gb300 import Hermite4GPU, NbodySystem, _lib, diagnostics, ics  # noqa: E402
from gravidy_gb300.ensemble import Ensemble  # noqa: E402


def _h(*arrays) -> str:
    m = hashlib.sha256()
    for a in arrays:
        m.update(np.ascontiguousarray(a).tobytes())
    return m.hexdigest()[:16]


def _system(n, seed, imf="salpeter", softening=0.01):
    m, p, v = ics.plummer(n, seed, imf)
    return NbodySystem(m, p, v, softening=softening, eta=0.01)


def single(n, mode, seed, host_steps, t_end, threshold=None):
    ns = _system(n, seed)
    with Hermite4GPU(ns, mode=mode) as g:
        if threshold is not None:
            g.set_mixed_threshold(threshold)
        g.init_acc_jrk()
        atime = g.init_dt()
        for _ in range(host_steps):
            itime = atime
            nact = g.find_particles_to_move(itime)
            g.save_old_acc_jrk(nact)
            g.predicted_pos_vel(itime)
            g.update_acc_jrk(nact)
            g.correction_pos_vel(itime, nact)
            atime = g.next_integration_time()
        itime, atime, steps, ps, inter, _ = g.advance(t_end, 1e30, atime)
        e = g.get_energy_gpu()
        st = g.download()
        # chosen active sets through the allocating force entry point
        pr = np.zeros((n, 4)); pr[:, :3] = ns.pos; pr[:, 3] = ns.mass
        pv = np.zeros((n, 4)); pv[:, :3] = ns.vel
        extra = []
        for k in sorted({1, min(31, n), min(33, n), n}):
            move = np.linspace(0, n - 1, k).astype(np.uint32)
            extra.append(g.forces_for(pr, pv, np.unique(move)))
        diag = []
        if n >= 8:
            tm = diagnostics.total_mass(ns.mass)
            cod = diagnostics.center_of_density(g)
            diag = [cod, np.array(diagnostics.mass_radii(g, cod, tm)[2])]
        return _h(st["r"], st["v"], st["f"], st["t"], st["dt"], np.array([e, steps, ps, inter]), *extra, *diag)


def noalloc(n, seed):
    import torch
    ns = _system(n, seed)
    pr = np.zeros((n, 4)); pr[:, :3] = ns.pos; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = ns.vel
    L = _lib.load()
    dev = torch.device("cuda", 0)
    d_pr, d_pv = torch.from_numpy(pr).to(dev), torch.from_numpy(pv).to(dev)
    outs = []
    for k in sorted({1, min(33, n), n}):
        move = np.unique(np.linspace(0, n - 1, k).astype(np.uint32))
        d_move = torch.from_numpy(move.astype(np.int32)).to(dev)
        d_out = torch.zeros((len(move), 6), dtype=torch.float64, device=dev)
        st = L.h4_forces_noalloc(n, ns.e2, C.c_void_p(d_pr.data_ptr()), C.c_void_p(d_pv.data_ptr()), len(move),
                                 C.c_void_p(d_move.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                 C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
        if st != 0:
            raise _lib.H4Error(st, L.h4_forces_noalloc_error().decode())
        torch.cuda.synchronize()
        outs.append(d_out.cpu().numpy())
    return _h(*outs)


def noalloc_recovers(n, seed):
    """Bounds-checked build only: a call whose active list names a particle
    past n fails with H4_ERR_STATE (the kernels' own checks skip the access),
    and the next call with a valid list succeeds and matches a fresh one --
    the failure does not stick to the shared control block."""
    import torch
    ns = _system(n, seed)
    pr = np.zeros((n, 4)); pr[:, :3] = ns.pos; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = ns.vel
    L = _lib.load()
    dev = torch.device("cuda", 0)
    d_pr, d_pv = torch.from_numpy(pr).to(dev), torch.from_numpy(pv).to(dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def call(move):
        d_move = torch.from_numpy(move.astype(np.int32)).to(dev)
        d_out = torch.zeros((len(move), 6), dtype=torch.float64, device=dev)
        st = L.h4_forces_noalloc(n, ns.e2, C.c_void_p(d_pr.data_ptr()), C.c_void_p(d_pv.data_ptr()), len(move),
                                 C.c_void_p(d_move.data_ptr()), C.c_void_p(d_out.data_ptr()), stream)
        torch.cuda.synchronize()
        return st, d_out.cpu().numpy()

    good = np.arange(0, n, 3, dtype=np.uint32)
    st0, want = call(good)
    bad = good.copy()
    bad[len(bad) // 2] = n + 5
    st1, _ = call(bad)
    st2, got = call(good)
    return st0 == 0 and st1 == 4 and st2 == 0 and np.array_equal(got, want)


def ensemble(mode, sizes, t_end, seed0=300):
    systems = []
    for k, n in enumerate(sizes):
        m, p, v = ics.plummer(n, seed0 + k, "salpeter" if k % 2 else "equal")
        systems.append((m, p, v, 0.01, 0.01))
    with Ensemble(systems, mode=mode) as E:
        E.init()
        E.advance(t_end)
        st = E.download()
        en = E.energy()
        stats = E.stats()
        probe = E.tune_force(2100, 64, 512, 128) if mode == "mixed" else 0.0
    return _h(st["r"], st["v"], st["f"], st["t"], st["dt"], np.asarray(en), stats["steps"]), probe >= 0.0


def main():
    L = _lib.load()
    out = {"build_flags": int(L.h4_build_flags()), "library": _lib.library_path(), "results": {}}
    R = out["results"]
    for n in (1, 2, 31, 33, 257, 1000):
        R[f"fp64_n{n}"] = single(n, "fp64", 10 + n, 3, 2.0 ** -5)
    for n in (2, 33, 257):
        R[f"exact_n{n}"] = single(n, "exact", 20 + n, 2, 2.0 ** -6)
    # mixed: warp items only (threshold above N), tiled shape (threshold 1)
    for n in (31, 257, 1000):
        R[f"mixed_warp_n{n}"] = single(n, "mixed", 30 + n, 3, 2.0 ** -5, threshold=1 << 30)
        R[f"mixed_tiled_n{n}"] = single(n, "mixed", 30 + n, 3, 2.0 ** -5, threshold=1)
    ns0 = _system(1000, 44, softening=0.0)   # e2 = 0: the masked mixed kernels
    with Hermite4GPU(ns0, mode="mixed") as g:
        g.set_mixed_threshold(1)
        g.init_acc_jrk()
        R["mixed_e2zero_n1000"] = _h(g.download()["f"])
    for n in (33, 1000):
        R[f"noalloc_n{n}"] = noalloc(n, 50 + n)
    sizes = [2, 33, 257, 513, 1000, 1500, 2500]   # 2500: block-tiled items at init (mixed)
    for mode in ("fp64", "mixed", "exact"):
        R[f"ensemble_{mode}"] = ensemble(mode, sizes if mode != "exact" else sizes[:4], 2.0 ** -5)[0]
    if out["build_flags"] & 1:
        # failure paths that only the checked build can take without an
        # out-of-bounds access
        out["checked_only"] = {"noalloc_recovers": bool(noalloc_recovers(1000, 77))}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
