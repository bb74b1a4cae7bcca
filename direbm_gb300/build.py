"""Build libdirebm_gb300.so (sm_103a) in-tree with nvcc.

Every translation unit under ``csrc/`` is compiled in parallel to an object file and the objects
are linked into ``direbm_gb300/_lib/libdirebm_gb300.so``.  Nothing is installed anywhere else.
The build is incremental: an object is rebuilt when its source or any header changed.

    python -m direbm_gb300.build          # build (or refresh) the library
    python -m direbm_gb300.build --ptxas  # also print ptxas register / spill / smem report
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
ROOT = PKG.parent
OUT_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_lib" / "obj"
LIB = OUT_DIR / "libdirebm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-O2",
    f"-I{ROOT / 'include'}",
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdirebm_gb300.so")
    return cand


def _stale(src: Path, obj: Path, headers) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in headers)


def build(ptxas: bool = False, verbose: bool = False) -> Path:
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    cc = nvcc()
    jobs = []
    for src in sources:
        obj = OBJ_DIR / (src.stem + ".o")
        if ptxas or _stale(src, obj, headers):
            cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    failed = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for src, r in ex.map(run, jobs):
                if verbose or ptxas:
                    sys.stderr.write(r.stderr)
                if r.returncode != 0:
                    failed.append((src, r.stderr))
    if failed:
        msg = "\n".join(f"--- {s.name}\n{e}" for s, e in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    objs = [str(OBJ_DIR / (s.stem + ".o")) for s in sources]
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ptxas", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(ptxas=a.ptxas, verbose=a.verbose))


if __name__ == "__main__":
    main()
