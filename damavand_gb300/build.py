"""Builds libdamavand_gpu.so in-tree for sm_103a (GB300).

Each CUDA/C++ source compiles to an object in parallel under
damavand_gb300/_build/, then nvcc links them into
damavand_gb300/libdamavand_gpu.so with the CUDA runtime linked statically.
Objects are rebuilt when their source or any header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libdamavand_gpu.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-Wall", "--expt-relaxed-constexpr",
          f"-I{os.path.join(REPO_DIR, 'include')}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(REPO_DIR, "include", "*.h"))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep and not extra:
        return obj
    cmd = [_nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [_nvcc(), "-x", "cu", *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile all sources (in parallel) and link the shared library. Returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    extra = list(extra or [])
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if os.path.exists(LIB_PATH) and not extra and \
            os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(o) for o in objs):
        return LIB_PATH
    cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB_PATH, *objs, "-lpthread", "-ldl", "-lrt"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    _link_alias()
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


def _link_alias() -> None:
    """libdamavand-gpu.so -> libdamavand_gpu.so: the name the reference's build.rs
    links (`cargo:rustc-link-lib=dylib=damavand-gpu`)."""
    alias = os.path.join(PKG_DIR, "libdamavand-gpu.so")
    if os.path.islink(alias) or os.path.exists(alias):
        os.remove(alias)
    os.symlink(LIB_NAME, alias)


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
