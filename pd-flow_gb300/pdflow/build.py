"""Builds the solver's shared library, in tree, for sm_103a only.

    python -m pdflow.build          (from pd-flow_gb300/)

Each translation unit under csrc/ is compiled in parallel by nvcc with
`-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`; the objects are
linked into lib/libpdflow_gb300.so (a C ABI: include/pdflow.h).  The ptxas
resource report of every kernel (of all translation units, also those not
recompiled) is kept in lib/ptxas.log.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # pd-flow_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
LIBDIR = os.path.join(PKG_ROOT, "lib")
OBJDIR = os.path.join(LIBDIR, "_build")
LIB_PATH = os.path.join(LIBDIR, "libpdflow_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(REPO_ROOT, "include", "*.h")))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        rep = obj + ".ptxas"
        return obj, open(rep).read() if os.path.exists(rep) else ""
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
           "-Xptxas", "-v", "--expt-relaxed-constexpr", "-I", os.path.join(REPO_ROOT, "include"),
           "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    with open(obj + ".ptxas", "w") as f:
        f.write(r.stderr)
    return obj, r.stderr


def build(verbose: bool = False) -> str:
    """Compiles csrc/ into lib/libpdflow_gb300.so (incremental) and returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)     # every translation unit's report, fresh or kept
    with open(os.path.join(LIBDIR, "ptxas.log"), "w") as f:
        f.write(logs)
    if _stale(LIB_PATH, objs):
        cuda_lib = os.path.join(_cuda_home(), "lib64")
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", LIB_PATH, *objs,
               "-Xlinker", f"-rpath,{cuda_lib}", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose="-q" not in sys.argv)
