"""Build oracle/_ref/libmtref.so: the reference's own OpenCL kernels compiled as C++.

Test infrastructure only. Reads MambaTracer's kernel sources where they lie
(src/cl/kernel under the checkout that MT_REFERENCE_ROOT names, else the
default checkout location below), concatenates them in the order of
src/cl/kernel/CSource.java:18-38, applies mechanical rewrites (OpenCL vector
literals "(float4)(a, b, c, d)" become calls "clv_float4(a, b, c, d)", since C++
parses the former as a cast of a comma expression; the two below), and compiles the result
together with oracle/ref/ref_harness.cpp through the shim oracle/ref/clshim.h.

Everything it writes goes to oracle/_ref/ (git-ignored). When the reference tree
is absent (a machine without the reference sources), it does nothing and returns False.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

# Root of the MambaTracer checkout: MT_REFERENCE_ROOT, else where this build
# environment mounts it.
REF_ROOT = os.environ.get("MT_REFERENCE_ROOT") or "/root/reference"
REF_KERNELS = os.path.join(REF_ROOT, "src", "cl", "kernel")
# src/cl/kernel/CSource.java:18-38
TU_ORDER = [
    "Print.cl", "Util.cl", "SAT.cl", "RGBSpace.cl", "Sampling.cl", "Matrix.cl",
    "Geometry.cl", "Bsdf.cl", "Primitive.cl", "Material.cl", "NormalBVH.cl",
    "LightGrid.cl", "Light.cl", "LightConfiguration.cl", "Path.cl",
    "Initialize.cl", "Raytrace.cl", "Render.cl", "Compact.cl", "Image.cl",
]

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")

_VEC_LITERAL = re.compile(r"\((float|int)([234])\)\s*\(")
# getEnvironmentLight (Light.cl:129-137) and InitEnvironmentSAT (Initialize.cl:118-127)
# call setRegion on a fresh local SATRegion whose nu/nv are still unset, so the
# region is only filled in when stack garbage happens to exceed the map size. The
# rewrite starts such a local with nu = nv = INT_MAX, the value under which the
# reference's own bounds checks pass and the region covers the full map.
_UNSET_REGION = re.compile(r"SATRegion region;(\s*\n\s*setRegion\(&region)")
# "a.xyz = f(...).xyz;" (Raytrace.cl:170) assigns three lanes in OpenCL; the
# shim's swizzle proxies would copy all four, so the right-hand side is
# converted to a three-lane value first. Only operator-free right-hand sides
# ending in .xyz match.
_SWIZZLE_COPY = re.compile(r"\.xyz(\s*)=(\s*)([A-Za-z_][\w.\[\]]*(?:\([^;+*/]*\))?\.xyz)\s*;")


def write_tu() -> str:
    parts = []
    for name in TU_ORDER:
        path = os.path.join(REF_KERNELS, name)
        with open(path, "r", encoding="latin-1") as f:
            text = f.read()
        parts.append(f'#line 1 "{path}"\n')
        text = _VEC_LITERAL.sub(r"clv_\1\2(", text)
        text = _UNSET_REGION.sub(r"SATRegion region = clshim_unset_region();\1", text)
        text = _SWIZZLE_COPY.sub(r".xyz\1=\2(float3)(\3);", text)
        parts.append(text)
        parts.append("\n")
    os.makedirs(OUT, exist_ok=True)
    tu = os.path.join(OUT, "ref_tu.inc")
    with open(tu, "w") as f:
        f.write("".join(parts))
    return tu


def build(force: bool = False, verbose: bool = False) -> bool:
    if not os.path.isdir(REF_KERNELS):
        return False
    lib = os.path.join(OUT, "libmtref.so")
    harness = os.path.join(HERE, "ref_harness.cpp")
    shim = os.path.join(HERE, "clshim.h")
    newest_src = max(os.path.getmtime(p) for p in (harness, shim, __file__))
    if not force and os.path.exists(lib) and os.path.getmtime(lib) > newest_src:
        return True
    write_tu()
    # -O0: several reference functions flow off the end of a non-void function
    # (e.g. SET_INT, Util.cl:898-902); an optimising C++ compiler may assume
    # that path unreachable, which would change their behaviour.
    cmd = [
        "g++", "-std=c++20", "-O0", "-fPIC", "-shared", "-w", "-fpermissive",
        "-fwrapv", "-ffp-contract=off", "-fsingle-precision-constant",
        "-ftrivial-auto-var-init=zero", "-fno-unreachable-traps", "-I", HERE, "-I", OUT,
        harness, "-o", lib, "-lpthread",
    ]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr[-20000:])
        raise RuntimeError("building the reference oracle failed")
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv, verbose=True)
    print("built" if ok else "reference tree absent: skipped")
