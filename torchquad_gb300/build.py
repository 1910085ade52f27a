"""Builds the CUDA library ``torchquad_gb300/_lib/libtorchquad_gb300.so`` in-tree.

Each ``csrc/*.cu`` file is compiled for sm_103a only (GB300), in parallel, and
linked into one shared library against the shared CUDA runtime, so the
library and PyTorch in the same process use one runtime instance (streams
and the current device are shared).  Run ``python -m torchquad_gb300.build``.
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
OUT_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
LIB_NAME = "libtorchquad_gb300.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def nvcc_path() -> str:
    p = cuda_home() / "bin" / "nvcc"
    return str(p) if p.exists() else "nvcc"


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, extra: list[str]) -> Path:
    obj = OBJ_DIR / (src.stem + ".o")
    cmd = [
        nvcc_path(),
        "-c",
        str(src),
        "-o",
        str(obj),
        *ARCH_FLAGS,
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler",
        "-fPIC",
        "-I",
        str(INCLUDE),
        "-I",
        str(CSRC),
        *extra,
    ]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("TQ_BUILD_VERBOSE"):
        print(r.stderr, file=sys.stderr)
    return obj


def _stale() -> bool:
    lib = lib_path()
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile and link the library if any source is newer than it."""
    if not force and not _stale():
        return lib_path()
    OUT_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    extra = list(extra_flags or [])
    if verbose:
        extra += ["-Xptxas", "-v"]
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = OUT_DIR / (LIB_NAME + ".tmp")
    cmd = [
        nvcc_path(),
        "-shared",
        *ARCH_FLAGS,
        "-o",
        str(tmp),
        *map(str, objs),
        "-cudart",
        "shared",
        "-Xlinker",
        f"-rpath,{cuda_home() / 'lib64'}",
    ]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
