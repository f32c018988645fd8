"""Build recipe for the engine's shared library (sm_103a only).

Compiles every translation unit under ``d4-pieces_gb300/csrc`` in parallel
(nvcc for ``.cu``, g++ for ``.cpp``) and links ``d4-pieces_gb300/lib/libd4e.so``
in-tree.  No cmake; one ``-gencode``; portable host flags (the same recipe
runs on x86_64 and aarch64 hosts).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # d4-pieces_gb300/
CSRC = PKG_ROOT / "csrc"
OBJ_DIR = PKG_ROOT / "_build"
LIB_DIR = PKG_ROOT / "lib"
LIB_PATH = LIB_DIR / "libd4e.so"
HOST_DIR = PKG_ROOT / "host"
EXAMPLE_PATH = LIB_DIR / "example_step"
FAMILY_EXAMPLE_PATH = LIB_DIR / "example_family"
INCLUDE = PKG_ROOT.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                     "-diag-suppress", "1444"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libd4e.so")
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp"))


def _needs_rebuild(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, headers: list[Path], verbose: bool) -> Path:
    obj = OBJ_DIR / (src.name + ".o")
    if not _needs_rebuild(obj, [src] + headers):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc()] + NVCC_FLAGS + ["-I", str(CSRC), "-I", str(INCLUDE), "-c", str(src),
                                        "-o", str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + [
            "-I", str(CSRC), "-I", str(INCLUDE), "-I", _cuda_include(), "-c", str(src),
            "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link libd4e.so; returns its path."""
    OBJ_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    if force:
        for o in OBJ_DIR.glob("*.o"):
            o.unlink()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, headers, verbose), srcs))
    if force or _needs_rebuild(LIB_PATH, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", str(LIB_PATH)] + [str(o) for o in objs]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    _build_example("example_step.cpp", EXAMPLE_PATH, ["searcher_cuda.h"], verbose)
    _build_example("example_family.cpp", FAMILY_EXAMPLE_PATH,
                   ["searcher_cuda.h", "board_family.h"], verbose)
    return LIB_PATH


def _build_example(name: str, out: Path, headers: list[str], verbose: bool) -> Path:
    """A C++ facade example driver, linked against libd4e.so."""
    src = HOST_DIR / name
    deps = [src, INCLUDE / "d4e.h", LIB_PATH] + [HOST_DIR / h for h in headers]
    if not _needs_rebuild(out, deps):
        return out
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-Wall", "-I", str(HOST_DIR),
           str(src), "-o", str(out), "-L", str(LIB_DIR), "-ld4e", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"example build failed ({name})\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
