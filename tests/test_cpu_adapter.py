"""The reference-side drop-in (gravidy_gb300/csrc/reference_adapter:
class Hermite4GB300 : public Hermite4) compiles and links against the
reference's own, unmodified headers and sources (gnu++98, as the reference
builds) and runs the reference's main flow: on a machine without a GPU it
stops cleanly at h4_create with the library's message."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
# location of the reference sources: the oracle recipe's default, or GRAVIDY_REF
REF_ARGS = [f"REF={os.environ['GRAVIDY_REF']}"] if os.environ.get("GRAVIDY_REF") else []


def _have_reference() -> bool:
    return subprocess.run(["make", "-s", "-C", ORACLE, "has-ref", *REF_ARGS], capture_output=True).returncode == 0


@pytest.mark.skipif(not _have_reference(), reason="reference sources not present")
def test_adapter_builds_against_reference_and_runs_main_flow(tmp_path):
    from gravidy_gb300.build import build_library
    build_library()
    subprocess.run(["make", "-s", "-C", ORACLE, "adapter", *REF_ARGS], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "gravidy_ref_gb300")
    inp = os.path.join(ROOT, "tests", "golden", "ragged_n33", "input.txt")
    r = subprocess.run([exe, "-i", inp, "-t", "0.0625", "-o", str(tmp_path / "run")], capture_output=True,
                       text=True, timeout=300)
    if r.returncode == 0:          # a GPU is present: the run completed
        assert os.path.exists(str(tmp_path / "run.out.log"))
    else:
        assert r.returncode == 1 and "h4_create" in r.stderr
