"""Builds libaleator_gb300.so in-tree for sm_103a with nvcc.

Each translation unit under csrc/ is compiled in parallel
(``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo``) and linked into
``aleator_gb300/_build/libaleator_gb300.so``. ptxas resource usage
(``-Xptxas -v``) is kept in ``_build/ptxas.log``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libaleator_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["common.cu", "philox.cu", "grid.cu", "grid_cache.cpp", "cif.cpp", "lj.cu", "ewald.cu",
           "widom.cu", "gcmc.cu", "proposal.cu", "capi.cu", "probe.cu", "noalloc.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "aleator_gb300.h"]
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I", str(PKG.parent / "include")]

    def compile_one(src: str):
        s = CSRC / src
        o = BUILD / (src.rsplit(".", 1)[0] + ".o")
        if not force and not _stale(o, [s, *headers]):
            return o, ""
        cmd = [cc, *common, "-Xptxas", "-v", "-c", str(s), "-o", str(o)]
        if src.endswith(".cpp"):  # host code: the reference's IEEE sequence, no FMA contraction
            cmd = [cc, *common, "-x", "cu", "-Xcompiler", "-ffp-contract=off", "-c", str(s), "-o",
                   str(o)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return o, r.stderr

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    logs = "".join(f"== {SOURCES[i]}\n{r[1]}" for i, r in enumerate(results) if r[1])
    if logs:
        (BUILD / "ptxas.log").write_text(logs)
    objs = [str(r[0]) for r in results]
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        r = subprocess.run([cc, *ARCH, "-shared", "-o", str(tmp), *objs], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
