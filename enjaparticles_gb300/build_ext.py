"""Build librtps_sph.so in-tree with nvcc for sm_103a (no cmake).

Each translation unit compiles in parallel into enjaparticles_gb300/_build/,
then one link step writes enjaparticles_gb300/librtps_sph.so.  The same
sources compiled with -DSPH_CHECKED (every kernel index tested against its
array, failures reported as SPH_EBOUNDS) give librtps_sph_checked.so, in
_build_checked/.  Usage:
    python -m enjaparticles_gb300.build_ext [-v] [--ptxas-verbose] [--no-checked]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librtps_sph.so")
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "librtps_sph_checked.so")
DRIVER = os.path.join(PKG, "sph_bench")

SOURCES = ["sph_api.cu", "sph_sort.cu", "sph_cellsort.cu", "sph_cells.cu", "sph_density.cu", "sph_force.cu", "sph_integrate.cu",
           "sph_triangles.cu", "sph_surface.cu", "sph_batch.cu", "sph_noalloc.cu", "sph_adjoint.cu", "sph_params.cpp",
           "sph_hose.cpp"]
# Per-file flags: the density pass and the hose's host arithmetic rely on
# every multiply and add being rounded on its own (no contraction, on any host).
EXTRA = {"sph_density.cu": ["-fmad=false"], "sph_hose.cpp": ["-Xcompiler", "-ffp-contract=off"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, ptxas_verbose, checked=False):
    obj = os.path.join(BUILD_CHECKED if checked else BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    cmd = [nvcc(), "-c", path, "-o", obj, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fno-fast-math", "-I", os.path.join(PKG, "..", "include")]
    if checked:
        cmd += ["-DSPH_CHECKED"]
    if src.endswith(".cu"):
        cmd += ARCH + ["--expt-relaxed-constexpr"] + EXTRA.get(src, [])
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "c++"] + EXTRA.get(src, [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr, " ".join(cmd)


def _link(objs, lib):
    tmp = lib + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, lib)


def build(verbose=False, ptxas_verbose=False, checked=True):
    """Both libraries (the checked one unless checked=False), every
    translation unit of both compiled in one pool."""
    variants = [False, True] if checked else [False]
    for v in variants:
        os.makedirs(BUILD_CHECKED if v else BUILD, exist_ok=True)
    jobs = [(src, v) for v in variants for src in SOURCES]
    objs = {v: [] for v in variants}
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(max(os.cpu_count() or 8, 8), 16, len(jobs))) as ex:
        results = ex.map(lambda j: (j[1],) + _compile(j[0], ptxas_verbose and not j[1], j[1]), jobs)
        for v, src, obj, rc, out, cmd in results:
            if verbose:
                print(cmd)
            if out.strip() and (verbose or (ptxas_verbose and not v) or rc):
                logs.append("== %s%s\n%s" % (src, " (checked)" if v else "", out))
            if rc:
                raise RuntimeError("nvcc failed on %s%s:\n%s" % (src, " (checked)" if v else "", out))
            objs[v].append(obj)
    _link(objs[False], LIB)
    if checked:
        _link(objs[True], LIB_CHECKED)
    build_driver()
    for line in logs:
        print(line)
    return LIB


def build_driver():
    """The headless C++ driver (driver/sph_bench.cpp) over include/rtps_sph.hpp,
    linked against librtps_sph.so (found next to it at run time)."""
    src = os.path.join(PKG, "driver", "sph_bench.cpp")
    tmp = DRIVER + ".tmp"
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", src, "-o", tmp, "-I",
           os.path.join(PKG, "..", "include"), "-L", PKG, "-lrtps_sph", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("driver build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas-verbose" in sys.argv,
                checked="--no-checked" not in sys.argv))
