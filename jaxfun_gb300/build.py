"""Build the in-tree CUDA library ``jaxfun_gb300/_lib/libjaxfun_gb300.so``.

Each ``csrc/*.cu`` translation unit is compiled for sm_103a in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into one shared
library exposing the C ABI declared in ``include/jaxfun_gb300.h``.  Objects
are rebuilt only when a source or header is newer than the library.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUTDIR = PKG / "_lib"
LIBNAME = "libjaxfun_gb300.so"
GENCODE = "arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jaxfun_gb300")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(_sources()) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    deps.append(Path(__file__))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and return the path of the shared library."""
    OUTDIR.mkdir(exist_ok=True)
    lib = OUTDIR / LIBNAME
    if not force and not _stale(lib):
        return lib
    nvcc = nvcc_path()
    objdir = OUTDIR / "obj"
    objdir.mkdir(exist_ok=True)
    common = [
        "-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17",
        "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC),
        "--expt-relaxed-constexpr",
    ]

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        cmd = [nvcc, *common, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, "-gencode", GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    build_xla_ffi(nvcc, lib, verbose)
    return lib


def xla_include_dir() -> Path | None:
    """Directory holding xla/ffi/api/ffi.h: JFG_XLA_INCLUDE, else jaxlib's own
    include directory (jax.ffi.include_dir()) when JAX is installed."""
    cands = []
    if os.environ.get("JFG_XLA_INCLUDE"):
        cands.append(Path(os.environ["JFG_XLA_INCLUDE"]))
    import importlib.util

    if importlib.util.find_spec("jax") is not None:
        r = subprocess.run([sys.executable, "-c", "import jax.ffi; print(jax.ffi.include_dir())"],
                           capture_output=True, text=True)
        if r.returncode == 0 and r.stdout.strip():
            cands.append(Path(r.stdout.strip()))
    for c in cands:
        if (c / "xla" / "ffi" / "api" / "ffi.h").exists():
            return c
    return None


def build_xla_ffi(nvcc: str, lib: Path, verbose: bool = False) -> Path | None:
    """Compile the XLA FFI handlers (ffi/jfg_xla.cc) into _lib/libjfg_xla.so,
    linked against the C-ABI library, when XLA's FFI header is available;
    returns None (and builds nothing) otherwise."""
    inc = xla_include_dir()
    if inc is None:
        return None
    src = PKG / "ffi" / "jfg_xla.cc"
    out = OUTDIR / "libjfg_xla.so"
    cmd = [nvcc, "-x", "c++", "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared",
           "-I", str(INCLUDE), "-I", str(inc), str(src), "-o", str(out),
           "-L", str(OUTDIR), "-ljaxfun_gb300", "-lcudart", "-Xlinker", "-rpath=$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
