"""The reference's own GPU tests, run unchanged through the module swap.

tests/test_warp_physics.py, test_warp_propagation.py, test_warp_simulator.py and test_warp_lbm.py
of the reference (copied under baseline/_ref/tests by oracle/install_reference.py, beside the
reference's CPU package they compare against) run in a separate pytest process with
``direbm.warp`` aliased to ``direbm_gb300.warp`` (tests/_reference_swap.py).  Skipped when the
reference is not installed.
"""

import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF_TESTS = ROOT / "baseline" / "_ref" / "tests"
FILES = ["test_warp_physics.py", "test_warp_propagation.py", "test_warp_simulator.py", "test_warp_lbm.py"]

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(not all((REF_TESTS / f).exists() for f in FILES),
                    reason="the reference is not installed (python oracle/install_reference.py <reference>)")
def test_reference_gpu_tests_pass_unchanged_through_the_module_swap():
    cmd = [sys.executable, "-m", "pytest", "-q", "-p", "tests._reference_swap", "-p", "no:cacheprovider",
           "--rootdir", str(REF_TESTS), *[str(REF_TESTS / f) for f in FILES]]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    tail = (r.stdout + r.stderr)[-4000:]
    assert r.returncode == 0, tail
    assert " passed" in r.stdout and "skipped" not in r.stdout, tail
