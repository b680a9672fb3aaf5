"""Builds libncgb300.so in-tree with nvcc for sm_103a.

Every translation unit under ``csrc/`` is compiled in parallel to an object
file, then linked into ``_build/libncgb300.so`` (cudart static, NVRTC shared,
no link against libcuda: driver entry points are resolved at run time).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libncgb300.so"
INCLUDE = PKG.parent / "include"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cpp", ".cu"))


def _needs_rebuild() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.iterdir()) + list(INCLUDE.iterdir()) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the extension if any source is newer than the library."""
    if not force and not _needs_rebuild():
        return LIB
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    common = [ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
              "-I", str(INCLUDE), "-I", str(CSRC)]

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *common, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [nvcc, "-x", "cu", *common, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    libdir = home / "lib64"
    if not libdir.exists():
        libdir = home / "lib"
    tmp = BUILD / "libncgb300.so.tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-L", str(libdir), "-lnvrtc",
           "-Xlinker", f"-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
