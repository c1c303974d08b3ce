"""Builds the sm_103a engine library in-tree: myquantlib_gb300/libmyql_gpu.so.

Every .cu / .cpp under csrc/ is compiled by nvcc in parallel (one -gencode,
sm_103a) and linked into one shared library that exports the C ABI declared in
include/myql_gpu.h.  Objects go to myquantlib_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmyql_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _flags() -> list[str]:
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
            f"-I{ROOT / 'include'}", f"-I{CSRC}", *ARCH]


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    cmd = [nvcc(), *_flags(), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


STAMP = BUILD / "stamp.txt"


def _fingerprint() -> str:
    h = hashlib.sha256()
    h.update(platform.machine().encode())
    h.update(" ".join(_flags()).encode())
    for p in _sources() + _headers():
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def up_to_date() -> bool:
    """True when the library was built on this machine type from these sources."""
    if not LIB.exists() or not STAMP.exists():
        return False
    return STAMP.read_text().strip() == _fingerprint()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    STAMP.write_text(_fingerprint())
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
