"""ORACLE build recipe -- test infrastructure, not product code.

Compiles the reference's own code for the TFCE/GLM path from the sources where
they lie in a reference checkout, writing only into ``oracle/_ref/``.  The
checkout is ``$TFCE_REFERENCE_ROOT`` when that is set, else a directory named
``reference`` beside the repository's own directory:

* ``oracle/_ref/libref_tfce.so`` -- ``tfce_mediation/lib/fast_tfce.hpp``
  (the reference sweep) behind the C-ABI shim ``oracle/ref_tfce_shim.cpp``;
* ``oracle/_ref/libref_geodesic.so`` -- the header-only exact geodesic library
  ``tfce_mediation/lib/geodesic/`` behind ``oracle/ref_geodesic_shim.cpp``;
* ``oracle/_ref/tfce_mediation/{tfce,cynumstats,adjacency}*.so`` -- the
  reference's Cython modules ``tfce_mediation/tfce.pyx``,
  ``tfce_mediation/cynumstats.pyx`` and ``tfce_mediation/adjacency.pyx`` (the
  exact geodesic neighbour lists over ``lib/geodesic``), cythonized with language_level 2 (they use
  ``xrange``) into ``oracle/_ref/cython/`` and compiled as C++11, the flags
  ``tfce_mediation/setup.py:25-41`` gives them.

The reference's own setup.py needs numpy.distutils (removed in numpy 2), so it
is not used.  When the checkout is absent (the GPU machine) this is a no-op and the
tests that need ``oracle/_ref`` skip.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REPO = os.path.dirname(HERE)


def ref_root() -> str:
    """The reference checkout: $TFCE_REFERENCE_ROOT, else ``reference`` next
    to the repository directory (absent on machines without a checkout)."""
    env = os.environ.get("TFCE_REFERENCE_ROOT")
    return env if env else os.path.join(os.path.dirname(REPO), "reference")


def build_shim(ref: str) -> str | None:
    lib = os.path.join(ref, "tfce_mediation", "lib")
    if not os.path.isfile(os.path.join(lib, "fast_tfce.hpp")):
        return None
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libref_tfce.so")
    src = os.path.join(HERE, "ref_tfce_shim.cpp")
    if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(src):
        return so
    subprocess.check_call(["g++", "-O2", "-std=c++11", "-shared", "-fPIC", "-I", lib,
                           src, "-o", so])
    return so


def build_geodesic_shim(ref: str) -> str | None:
    """oracle/_ref/libref_geodesic.so: the reference's header-only exact
    geodesic library (tfce_mediation/lib/geodesic) behind
    oracle/ref_geodesic_shim.cpp."""
    lib = os.path.join(ref, "tfce_mediation", "lib", "geodesic")
    if not os.path.isfile(os.path.join(lib, "geodesic_algorithm_exact.h")):
        return None
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libref_geodesic.so")
    src = os.path.join(HERE, "ref_geodesic_shim.cpp")
    if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(src):
        return so
    subprocess.check_call(["g++", "-O2", "-std=c++11", "-shared", "-fPIC", "-w", "-I", lib, src, "-o", so])
    return so


def build_cython(ref: str) -> bool:
    pkg = os.path.join(ref, "tfce_mediation")
    if not os.path.isfile(os.path.join(pkg, "tfce.pyx")):
        return False
    try:
        import numpy
        from Cython.Build import cythonize
        from setuptools import Extension
        from setuptools.dist import Distribution
    except ImportError:
        return False
    dst = os.path.join(OUT, "tfce_mediation")
    os.makedirs(dst, exist_ok=True)
    init = os.path.join(dst, "__init__.py")
    if not os.path.exists(init):
        open(init, "w").close()
    have = [f for f in os.listdir(dst) if f.endswith(".so")]
    if all(any(f.startswith(m + ".") for f in have) for m in ("tfce", "cynumstats", "adjacency")):
        return True
    exts = [
        Extension("tfce_mediation.tfce", [os.path.join(pkg, "tfce.pyx")],
                  include_dirs=[os.path.join(pkg, "lib"), numpy.get_include()],
                  language="c++", extra_compile_args=["-std=c++11", "-O2", "-w"]),
        Extension("tfce_mediation.cynumstats", [os.path.join(pkg, "cynumstats.pyx")],
                  include_dirs=[numpy.get_include()],
                  language="c++", extra_compile_args=["-std=c++11", "-O2", "-w"]),
        Extension("tfce_mediation.adjacency", [os.path.join(pkg, "adjacency.pyx")],
                  include_dirs=[os.path.join(pkg, "lib"), numpy.get_include()],
                  language="c++", extra_compile_args=["-std=c++11", "-O2", "-w"]),
    ]
    exts = cythonize(exts, build_dir=os.path.join(OUT, "cython"), quiet=True,
                     compiler_directives={"language_level": 2})
    dist = Distribution({"name": "tfce_mediation_ref", "ext_modules": exts})
    cmd = dist.get_command_obj("build_ext")
    cmd.build_lib = OUT
    cmd.build_temp = os.path.join(OUT, "tmp")
    cmd.inplace = False
    cmd.ensure_finalized()
    cmd.run()
    return True


def build() -> dict:
    ref = ref_root()
    out = {"shim": None, "cython": False}
    if not os.path.isdir(ref):
        return out
    out["shim"] = build_shim(ref)
    try:
        out["geodesic"] = build_geodesic_shim(ref)
    except Exception as exc:  # pins the geodesic oracle only
        print(f"oracle/build_ref.py: geodesic shim not built: {exc}", file=sys.stderr)
    try:
        out["cython"] = build_cython(ref)
    except Exception as exc:  # the shim alone still pins the sweep
        print(f"oracle/build_ref.py: Cython modules not built: {exc}", file=sys.stderr)
    return out


if __name__ == "__main__":
    print(build())
