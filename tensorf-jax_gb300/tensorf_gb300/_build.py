"""Build the CUDA library ``libtensorf_gb300.so`` in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``) and the objects are linked
into one shared library next to this file. Rebuilds only what is out of date.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG_DIR = pathlib.Path(__file__).resolve().parent
SRC_DIR = PKG_DIR.parent / "csrc"
REPO_ROOT = PKG_DIR.parent.parent
INCLUDE_DIR = REPO_ROOT / "include"
BUILD_DIR = PKG_DIR.parent / "_build"
LIB_NAME = "libtensorf_gb300.so"
LIB_PATH = PKG_DIR / LIB_NAME

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
    f"-I{INCLUDE_DIR}",
    f"-I{SRC_DIR}",
]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return sorted(SRC_DIR.glob("*.cu"))


def _headers():
    return sorted(list(SRC_DIR.glob("*.cuh")) + list(SRC_DIR.glob("*.h")) + list(INCLUDE_DIR.glob("*.h")))


def _compile(src: pathlib.Path, extra) -> pathlib.Path:
    obj = BUILD_DIR / (src.stem + ".o")
    newest_dep = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep:
        return obj
    cmd = [_nvcc(), *NVCC_FLAGS, *extra, "-dc" if False else "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, extra_flags=()) -> pathlib.Path:
    """Compile every translation unit and link the shared library. Returns its path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra_flags)), srcs))
    newest_obj = max(o.stat().st_mtime for o in objs)
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < newest_obj:
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


def jax_ffi_available() -> bool:
    """True where jax with the FFI headers is importable (jaxlib >= 0.4.31)."""
    try:
        import jax.ffi  # noqa: F401

        return bool(jax.ffi.include_dir())
    except Exception:
        return False


def build_jax_shim(verbose: bool = False) -> pathlib.Path:
    """libtvm_jax_ffi.so: the XLA FFI handlers of csrc/jax/tvm_jax_ffi.cc, linked against
    the kernels' library. Needs jax.ffi."""
    import jax.ffi

    lib = build(verbose)
    src = SRC_DIR / "jax" / "tvm_jax_ffi.cc"
    out = PKG_DIR / "libtvm_jax_ffi.so"
    cmd = ["g++", "-std=c++17", "-O2", "-shared", "-fPIC", f"-I{jax.ffi.include_dir()}", f"-I{INCLUDE_DIR}",
           "-I/usr/local/cuda/include", str(src), str(lib), f"-Wl,-rpath,{PKG_DIR}", "-L/usr/local/cuda/lib64",
           "-lcudart", "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"building {out.name} failed:\n{res.stderr}")
    if verbose:
        print(f"built {out}", file=sys.stderr)
    return out


if __name__ == "__main__":
    build(verbose=True)
    if jax_ffi_available():
        build_jax_shim(verbose=True)
