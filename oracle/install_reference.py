"""Install the reference's CPU package (``direbm``) into ``baseline/_ref`` for the CPU baselines.

Test infrastructure: ``bench.py`` times the reference's own CPU simulator
(``direbm.reference.Simulator``) from this install when it is present, and
tests/test_gpu_reference_suite.py runs the reference's own GPU tests (copied beside the package)
against this library; nothing in the library imports it.  ``baseline/_ref`` is git-ignored but
travels with the repository to the GPU host.

The reference's CPU path is pure Python over numpy.  ``pip install --no-index --target`` is tried
first; the reference builds with the hatchling backend, which the offline wheelhouse does not
carry, so when pip fails the pure-Python package directory is placed under ``baseline/_ref``
unchanged -- what a wheel install of a pure-Python package amounts to.  The outcome is written to
``baseline/_ref/INSTALL.txt``.

    python oracle/install_reference.py <path to a checkout of the reference>
"""

from __future__ import annotations

import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
DEST = ROOT / "baseline" / "_ref"


def main(src: str) -> int:
    src_p = Path(src).resolve()
    if not (src_p / "direbm" / "__init__.py").exists():
        sys.exit(f"{src_p} holds no direbm package")
    DEST.mkdir(parents=True, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:  # the build may write into its source tree
        copy = Path(tmp) / "ref"
        shutil.copytree(src_p, copy)
        r = subprocess.run([sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation",
                            "--find-links", "/opt/wheelhouse", "--target", str(DEST), str(copy)],
                           capture_output=True, text=True)
    if r.returncode == 0:
        how = "pip install --no-index --target (succeeded)"
    else:
        tail = (r.stderr or r.stdout).strip().splitlines()[-1:] or ["?"]
        target = DEST / "direbm"
        if target.exists():
            shutil.rmtree(target)
        shutil.copytree(src_p / "direbm", target, ignore=shutil.ignore_patterns("__pycache__"))
        how = f"pip install failed ({tail[0]}); pure-Python package directory placed instead"
    # the reference's own tests, run unchanged against this library by tests/test_gpu_reference_suite.py
    tests = DEST / "tests"
    if tests.exists():
        shutil.rmtree(tests)
    shutil.copytree(src_p / "tests", tests, ignore=shutil.ignore_patterns("__pycache__"))
    (DEST / "INSTALL.txt").write_text(f"source: {src_p}\nmethod: {how}\ntests: copied to baseline/_ref/tests\n")
    print(how)
    return 0


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/install_reference.py <path to a checkout of the reference>")
    sys.exit(main(sys.argv[1]))
