"""Build recipe for the native library ``tfce_mediation_gb300/_native/libtfce_gb300.so``.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into one
shared library with a plain C ABI (``include/tfce_gb300.h``).  No torch headers,
no cmake: nvcc + the host g++ only, so the same recipe runs on the x86_64 build
container and on the aarch64 GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUTDIR = os.path.join(PKG, "_native")
LIB = os.path.join(OUTDIR, "libtfce_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["capi.cu", "tfce_sweep.cu", "glm.cu", "glm_tc.cu", "fwer.cu", "mlp.cu", "rm_anova.cu", "gd_fwhm.cu", "geodesic.cu",
           "perm_stream.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tfce_mediation_gb300")


def _stale(extra=()) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "tfce_gb300.h")]
    deps += [os.path.abspath(__file__)] + list(extra)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUTDIR, exist_ok=True)
    objdir = os.path.join(OUTDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                    "-I", CSRC, "--expt-relaxed-constexpr"]
    if ptxas_verbose:
        flags += ["-Xptxas", "-v"]
    flags += os.environ.get("TFGB_NVCC_FLAGS", "").split()

    def compile_one(src: str) -> str:
        obj = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + flags
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
        if verbose or ptxas_verbose:
            sys.stderr.write(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
