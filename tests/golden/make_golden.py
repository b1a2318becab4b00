"""Regenerate the golden fixtures from the reference GraviDy CPU path.

Run where the reference sources are present (the location named by REF in
oracle/Makefile; override with GRAVIDY_REF):

    python tests/golden/make_golden.py

It builds the reference sources unmodified (make -C oracle ref), writes each
case's seeded input file, and runs

* oracle/_ref/ref_harness : full-precision trace of the block-step loop
  (init.bin, steps.txt, energy.txt, state_final.bin), and
* oracle/_ref/gravidy_ref : the reference command-line program itself, whose
  energy log (<out>.log, src/include/utils/Logger.cpp:324-391) is kept.

Both run with OMP_NUM_THREADS=1, the setting under which the reference energy
sum is reproducible (its per-i partial sums are added with omp atomic,
src/include/utils/NbodyUtils.cpp:519-522).
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gravidy_gb300 import ics  # noqa: E402

# name: (n, seed, imf, softening, eta, t_end, interval, full-trace steps)
CASES = {
    "c1_plummer_n1024": (1024, 1, "equal", 0.01, 0.01, 1.0, 0.125, 300),
    "salpeter_n100": (100, 7, "salpeter", 0.01, 0.02, 0.25, 0.0625, 100000),
    "ragged_n33": (33, 3, "equal", 0.05, 0.01, 0.125, 0.03125, 100000),
    "binary_n2": (2, 5, "equal", 0.001, 0.01, 0.5, 0.125, 100000),
    "single_n1": (1, 9, "equal", 0.01, 0.01, 1e-5, 0.125, 100000),
}


def main() -> None:
    ref = os.environ.get("GRAVIDY_REF")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"] + ([f"REF={ref}"] if ref else []),
                   check=True)
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    cli = os.path.join(ROOT, "oracle", "_ref", "gravidy_ref")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    index = {}
    for name, (n, seed, imf, soft, eta, tend, interval, nfull) in CASES.items():
        d = os.path.join(HERE, name)
        shutil.rmtree(d, ignore_errors=True)
        os.makedirs(d)
        mass, pos, vel = ics.plummer(n, seed, imf)
        inp = os.path.join(d, "input.txt")
        ics.write_input_file(inp, mass, pos, vel)
        flags = ["-i", inp, "-s", repr(soft), "-e", repr(eta), "-t", repr(tend), "-z", repr(interval)]
        subprocess.run([harness, *flags, "-d", d, "-K", str(nfull)], check=True, env=env)
        index[name] = {"n": n, "seed": seed, "imf": imf, "softening": soft, "eta": eta,
                       "t_end": tend, "interval": interval, "full_trace_steps": nfull}
        tmp = os.path.join(d, "cli")
        os.makedirs(tmp)
        # The reference program needs at least a handful of particles: its
        # diagnostics (nbody_attributes, called before the first step) crash
        # with SIGSEGV for N=1, so that case keeps only the harness trace.
        rc = subprocess.run([cli, *flags, "-o", os.path.join(tmp, "run")], env=env,
                            stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode
        if rc == 0:
            shutil.copy(os.path.join(tmp, "run.out.log"), os.path.join(d, "energy_log.txt"))
        index[name]["cli_returncode"] = rc
        shutil.rmtree(tmp)
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(index, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
