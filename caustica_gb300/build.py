"""Build the in-tree shared library ``libcaustica_gb300.so`` with nvcc.

One ``-gencode`` (sm_103a), one object per ``.cu`` compiled in parallel,
static CUDA runtime (the library then needs only the driver at run time, and
``ctypes`` can load it on a machine without a GPU). No CMake.

    python -m caustica_gb300.build          # or __graft_entry__.build()
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libcaustica_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# the size-specialised passes are split into several units per family (one
# length group each) so the parallel build finishes in about a minute
SOURCES = (["cg_kspace.cu", "cg_pennes.cu", "cg_post.cu", "cg_store.cu", "cg_fused_xy.cu", "cg_fast_yx.cu", "cg_fast_z.cu"]
           + [f"cg_fast_yx_{g}.cu" for g in "abcdef"] + [f"cg_fast_z_{g}.cu" for g in "abcdef"])


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: set NVCC or put the CUDA toolkit on PATH")


def _flags(verbose_ptxas: bool = False) -> list[str]:
    # host code keeps the reference's operation order: no fused multiply-add
    f = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off",
         f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr"]
    if verbose_ptxas:
        f.append("-Xptxas=-v")
    for var in ("CG_FAST_MINB_Y", "CG_FAST_MINB_X", "CG_FAST_MINB_XG", "CG_FAST_MINB_X20", "CG_FAST_MINB_Z", "CG_YP", "CG_YP20", "CG_XP", "CG_ZP"):
        if os.environ.get(var):
            f.append(f"-D{var}={int(os.environ[var])}")
    return f


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src, *CSRC.glob("*.cuh"), INCLUDE / "caustica_gb300.h", Path(__file__)]
    mt = obj.stat().st_mtime
    return any(d.stat().st_mtime > mt for d in deps if d.exists())


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = True) -> Path:
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = []
    for name in SOURCES:
        src = CSRC / name
        obj = BUILD / (name[:-3] + ".o")
        if force or _stale(obj, src):
            jobs.append([cc, *_flags(verbose_ptxas), "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(run, jobs))
    if not quiet:
        for log in logs:
            sys.stdout.write(log)
    objs = [str(BUILD / (n[:-3] + ".o")) for n in SOURCES]
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        run([cc, ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, quiet=False)
    print(LIB)
