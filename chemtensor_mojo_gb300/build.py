"""Build recipe of libctdmrg.so (sm_103a only), in-tree.

Each ``csrc/*.cu`` is compiled by ``nvcc -gencode arch=compute_103a,code=sm_103a``
in parallel, then linked into ``chemtensor_mojo_gb300/libctdmrg.so``.  The
library links the CUDA runtime statically and needs no libcuda at link time
(the TMA descriptor encoder is fetched from the driver at run time).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libctdmrg.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _flags(debug: bool = False):
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-Xptxas", "-O3"] + ARCH
    if debug:
        f += ["-DCT_CHECKED=1"]
    return f


def _compile(src: Path, obj: Path, debug: bool, verbose: bool) -> None:
    cmd = [_nvcc(), "-c", str(src), "-o", str(obj)] + _flags(debug)
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def _stamp(debug: bool) -> str:
    """What the objects were built for: the host machine, the compiler and the flags."""
    r = subprocess.run([_nvcc(), "--version"], capture_output=True, text=True)
    tail = r.stdout.strip().splitlines()[-1] if r.stdout.strip() else ""
    return f"{platform.machine()}|{tail}|{' '.join(_flags(debug))}"


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    """Compile every kernel source and link libctdmrg.so; returns its path.

    Objects are reused by modification time only when ``_build/stamp`` names the same
    machine, compiler and flags; otherwise (a tree copied from another machine, a new
    toolkit, a debug build) everything is compiled again."""
    BUILD.mkdir(exist_ok=True)
    stamp_file = BUILD / "stamp"
    stamp = _stamp(debug)
    if not stamp_file.exists() or stamp_file.read_text() != stamp:
        force = True
    sources = sorted(CSRC.glob("*.cu"))
    headers = list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "ctdmrg.h"]
    newest_hdr = max(p.stat().st_mtime for p in headers if p.exists())
    jobs = []
    objs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_hdr):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, debug, verbose) for s, o in jobs]
            for f in futs:
                f.result()
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + ["-Xcompiler", "-fPIC",
                                                                                     "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, debug="--debug" in sys.argv))
