#!/usr/bin/env python3
"""Build oracle/_ref/librtps_ref.so: the reference's own SPH kernels, run on the host.

TEST INFRASTRUCTURE.  The reference (RTPS / EnjaParticles) cannot run as
shipped: its host code needs a GL context and its kernels need an OpenCL
driver, and neither exists on these machines.  Its OpenCL C kernel sources are
plain arithmetic, though, so this recipe compiles them for the host with g++:

  1. copy the kernel sources the SPH step uses from the reference tree
     (rtpslib/system/common/cl_src, rtpslib/system/sph/cl_src) into a
     temporary directory laid out as the reference's build lays them out
     (cl_common/, cl_sph/; rtpslib/system/sph/CMakeLists.txt:3-11);
  2. rewrite four pieces of OpenCL-only syntax there, nothing else:
       `(float4)(a, b, c, d)` / `(int4)(...)` / `(float3)(...)` / `(int2)(...)`
           ->  `make_float4(...)` / `make_int4(...)` / `make_float3(...)` / `make_int2(...)`
       kernel-scope `__local T name[N];` arrays  ->  `static T name[N];`
       the identity swizzle `v.xyzw`  ->  `v`
       the implicit Triangle* -> float* argument conversion of one call in
       collision_tri.cl  ->  the same conversion as an explicit cast, with a
       barrier in front (the order of shared-memory reads and writes that the
       32-wide lockstep work-group gives on the GPU)
     (work-groups run one at a time, so a static array is the group's local
     memory);
  3. compile them with clshim.hpp (vector types, built-ins, barrier) and the
     ref_*.cpp drivers, plus the reference's host Domain.cpp / IV.cpp /
     structs.cpp unchanged (and its Hose.cpp, included unchanged by
     ref_hose.cpp; its RTPSSettings.cpp and a scratch copy of
     system/SPHSettings.cpp, included unchanged by ref_settings.cpp, the
     copy's SPH.h being sph_settings_shim.h), into oracle/_ref/librtps_ref.so.  -ffp-contract=off keeps
     every multiply and add separately rounded, as written.

The temporary copies are deleted; only the shared library is kept, under
oracle/_ref/ (git-ignored).  Nothing from the reference is written into the
repository.  Usage: python oracle/ref/build_ref.py [--reference DIR].
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
OUT_LIB = os.path.join(OUT_DIR, "librtps_ref.so")

COMMON = ["hash.cl", "cl_hash.h", "cl_structs.h", "cl_macros.h", "cellindices.cl", "permute.cl", "bitonic.cl",
          "gravity.cl", "indexmap.h", "classifycubes.cl", "constructhp.cl", "traversehp.cl"]
SPH = ["density.cl", "force.cl", "collision_wall.cl", "collision_tri.cl", "leapfrog.cl", "euler.cl", "colorfield.cl",
       "cl_sph_kernels.h", "cl_sph_neighbors.h", "cl_sph_structs.h", "cl_sph_collision.h", "cl_sph_macros.h"]
DRIVERS = ["ref_runtime.cpp", "ref_hash.cpp", "ref_bitonic.cpp", "ref_cellindices.cpp", "ref_permute.cpp",
           "ref_density.cpp", "ref_force.cpp", "ref_collision.cpp", "ref_leapfrog.cpp", "ref_domain.cpp",
           "ref_gravity.cpp", "ref_euler.cpp", "ref_collision_tri.cpp", "ref_hose.cpp",
           "ref_colorfield.cpp", "ref_marching_cubes.cpp", "ref_settings.cpp"]
# SPH::calculate / updateParams: compiled from a scratch copy beside which
# the shim below is written as SPH.h (the real SPH.h needs the OpenCL system)
SETTINGS_SRC = os.path.join("system", "SPHSettings.cpp")
SETTINGS_SHIM = "sph_settings_shim.h"

VEC_LITERAL = re.compile(r"\((float4|int4|float3|int2)\)\s*\(")
LOCAL_ARRAY = re.compile(r"^(\s*)__local(\s+\w+\s+\w+\s*\[)", re.M)
IDENTITY_SWIZZLE = re.compile(r"\.xyzw\b")
# collision_tri.cl passes its Triangle arrays where float* is declared; C
# converts the pointers implicitly, C++ needs the cast written out.  The same
# call refills the shared chunk of 220 triangles with no barrier after the
# previous chunk's reads: on the GPU the 32 work-items of a group run in
# lockstep, so every read of chunk k precedes every write of chunk k+1; the
# fibers here switch only at barriers, so the barrier that lockstep gives is
# written in front of the copy.
TRI_TO_FLOATS = "global_to_shared_tri(triangles_glob, triangles,"
TRI_TO_FLOATS_CPP = ("barrier(CLK_LOCAL_MEM_FENCE); "
                     "global_to_shared_tri((float*)triangles_glob, (float*)triangles,")


def rewrite(text):
    text = VEC_LITERAL.sub(lambda m: "make_%s(" % m.group(1), text)
    text = LOCAL_ARRAY.sub(r"\1static\2", text)
    text = IDENTITY_SWIZZLE.sub("", text)
    text = text.replace(TRI_TO_FLOATS, TRI_TO_FLOATS_CPP)
    return text


def build(reference, verbose=False):
    src_common = os.path.join(reference, "rtpslib", "system", "common", "cl_src")
    src_sph = os.path.join(reference, "rtpslib", "system", "sph", "cl_src")
    rtpslib = os.path.join(reference, "rtpslib")
    for d in (src_common, src_sph):
        if not os.path.isdir(d):
            raise FileNotFoundError(d)
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="rtps_ref_")
    try:
        for sub, names, src in (("cl_common", COMMON, src_common), ("cl_sph", SPH, src_sph)):
            os.makedirs(os.path.join(tmp, sub))
            for name in names:
                with open(os.path.join(src, name), "r", errors="replace") as f:
                    text = f.read()
                with open(os.path.join(tmp, sub, name), "w") as f:
                    f.write(rewrite(text))
        shutil.copyfile(os.path.join(rtpslib, SETTINGS_SRC), os.path.join(tmp, "SPHSettings.cpp"))
        shutil.copyfile(os.path.join(HERE, SETTINGS_SHIM), os.path.join(tmp, "SPH.h"))
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
               "-w", "-I", tmp, "-I", HERE, "-I", rtpslib]
        cmd += [os.path.join(HERE, d) for d in DRIVERS]
        cmd += [os.path.join(rtpslib, "domain", "Domain.cpp"), os.path.join(rtpslib, "domain", "IV.cpp"),
                os.path.join(rtpslib, "structs.cpp")]
        cmd += ["-o", OUT_LIB]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return OUT_LIB


def default_reference():
    """RTPS_REFERENCE_TREE when set, else a directory named `reference` beside
    the repository (None when neither exists)."""
    env = os.environ.get("RTPS_REFERENCE_TREE")
    if env:
        return env
    beside = os.path.join(os.path.dirname(os.path.dirname(ORACLE)), "reference")
    return beside if os.path.isdir(beside) else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=default_reference())
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    if not a.reference or not os.path.isdir(a.reference):
        print("reference tree not found (%s); nothing built" % a.reference)
        return 0
    print(build(a.reference, a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
