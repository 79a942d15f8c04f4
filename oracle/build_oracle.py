"""Build recipe for the CPU oracle (test infrastructure, see mesh_bem_oracle.c).

``build()`` compiles ``oracle/mesh_bem_oracle.c`` twice (double and float) with gcc and
links ``oracle/_build/libmeshbem_oracle.so``.  ``-ffp-contract=off`` keeps the results
identical between the x86 build host and the Arm GPU host.

``build_ref()`` (only where the reference checkout is present) compiles the reference's
own MoM kernel bodies (``src/mesh_BEM/cuda/mesh_MOM_3d.cu`` lines 7-565) as host C++,
read straight from the checkout through a pipe, behind ``ref_shim.h`` (macro shims for
``__device__``/``__global__``/thread indices) and ``ref_driver.inc`` (an OpenMP loop per
kernel).  The result, ``oracle/_ref/libref_mom.so``, is used to pin the restatement.
Nothing of the reference's source is written to disk.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD_DIR, "libmeshbem_oracle.so")
REF_LIB = os.path.join(REF_DIR, "libref_mom.so")
# the reference checkout (read-only); MESH_FERROFLUID_REF overrides where it lives
REF_ROOT = os.environ.get("MESH_FERROFLUID_REF", "/root/reference")
REF_CU = os.path.join(REF_ROOT, "src", "mesh_BEM", "cuda", "mesh_MOM_3d.cu")

_CFLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "mesh_bem_oracle.c")
    if not force and not _stale(LIB, [src, __file__]):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    objs = []
    for real, sfx in (("double", "f64"), ("float", "f32")):
        obj = os.path.join(BUILD_DIR, f"oracle_{sfx}.o")
        subprocess.check_call(
            ["gcc", *_CFLAGS, f"-DREAL={real}", f"-DSFX={sfx}",
             *(["-DORC_FLOAT"] if real == "float" else []), "-c", src, "-o", obj]
        )
        objs.append(obj)
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", tmp, *objs, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def reference_available() -> bool:
    return os.path.exists(REF_CU)


def build_ref(force: bool = False) -> str | None:
    """Host-compile the reference's kernel bodies; returns the .so path or None."""
    if not reference_available():
        return None
    shim = os.path.join(HERE, "ref_shim.h")
    driver = os.path.join(HERE, "ref_driver.inc")
    if not force and not _stale(REF_LIB, [shim, driver, __file__, REF_CU]):
        return REF_LIB
    os.makedirs(REF_DIR, exist_ok=True)
    with open(REF_CU, "r") as fh:
        lines = fh.read().split("\n")
    body = "\n".join(lines[6:565])  # lines 7..565: helpers and the three kernels
    unit = (
        f'#include "{shim}"\n#line 7 "{REF_CU}"\n' + body + f'\n#include "{driver}"\n'
    )
    tmp = REF_LIB + ".tmp"
    proc = subprocess.run(
        ["g++", "-x", "c++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off",
         "-shared", "-w", "-o", tmp, "-"],
        input=unit.encode(),
        capture_output=True,
    )
    if proc.returncode != 0:
        sys.stderr.write(proc.stderr.decode())
        raise RuntimeError("host build of the reference kernels failed")
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_ref(force=True))
