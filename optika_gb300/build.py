"""Build the in-tree C-ABI library ``optika_gb300/_lib/liboptika_gb300.so``.

Each CUDA translation unit is compiled for sm_103a in its own ``nvcc``
process (in parallel), then linked into one shared library.  Objects are
rebuilt only when a source or header is newer than the library.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess

PACKAGE = pathlib.Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PACKAGE / "_lib"
LIB = OUT_DIR / "liboptika_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[pathlib.Path]:
    return (
        sources()
        + sorted(CSRC.glob("*.cuh"))
        + sorted(CSRC.glob("*.h"))
        + sorted(INCLUDE.glob("*.h"))
        + [pathlib.Path(__file__)]
    )


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe is None:
        cand = pathlib.Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build optika_gb300")
    return exe


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _compile(src: pathlib.Path, obj: pathlib.Path) -> None:
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile every CUDA source and link the shared library."""
    if not force and up_to_date():
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    objs = []
    jobs = min(len(sources()), max(1, os.cpu_count() or 1))
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = []
        for src in sources():
            obj = OUT_DIR / (src.stem + ".o")
            objs.append(obj)
            futs.append(ex.submit(_compile, src, obj))
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        o.unlink(missing_ok=True)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
