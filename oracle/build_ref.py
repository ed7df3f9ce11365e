#!/usr/bin/env python3
"""Compile the unmodified reference (Athena++ fork) CPU solver from its own sources.

Test infrastructure only: the binaries built here are the *reference* that the
CPU restatement in ``oracle/athena_oracle.c`` and the CUDA path are checked
against. Nothing in the product links or runs them.

The reference's own build system (``configure.py`` + ``Makefile.in``) is not
run. Instead this script

1. writes a ``defs.hpp`` of its own (the preprocessor settings that
   ``configure.py`` would have chosen: physics, Riemann solver, EOS, NGHOST,
   gravity; see ``src/defs.hpp.in`` and ``configure.py:364-423`` in the
   reference) into ``oracle/_ref/<name>/``;
2. compiles the same source list that ``Makefile.in:27-56`` names, with
   ``g++ -O3 -std=c++11`` (``configure.py:454``), straight from the read-only
   reference tree, objects and binary going to ``oracle/_ref/<name>/``;
3. optionally adds a harness problem generator from ``oracle/harness/``
   (own code) in place of a reference ``src/pgen/*.cpp``.

``oracle/_ref/`` is git-ignored. The reference tree is read from the directory
named by the environment variable ``ATHG_REFERENCE`` (default: the development
container's checkout). It is only present in the development container, so this
runs there (``build()`` skips it elsewhere).
"""
import argparse
import concurrent.futures as cf
import glob
import hashlib
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("ATHG_REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "_ref")

# name -> (pgen file, flux, mhd, nghost, self_gravity(0|2), omp, eos override)
CONFIGS = {
    "lw_hydro_hllc": ("linear_wave.cpp", "hllc", False, 2, 0, False, None),
    "lw_hydro_hlle": ("linear_wave.cpp", "hlle", False, 2, 0, False, None),
    "lw_mhd_hlld": ("linear_wave.cpp", "hlld", True, 2, 0, False, None),
    "lw_mhd_hlle": ("linear_wave.cpp", "hlle", True, 2, 0, False, None),
    "ot_mhd_hlld": ("orszag_tang.cpp", "hlld", True, 2, 0, False, None),
    "ot_mhd_hlld_omp": ("orszag_tang.cpp", "hlld", True, 2, 0, True, None),
    "blast_mhd_hlld": ("blast.cpp", "hlld", True, 4, 0, False, None),
    "blast_hydro_hllc": ("blast.cpp", "hllc", False, 4, 0, False, None),
    "blast_mhd_hlld_ng2": ("blast.cpp", "hlld", True, 2, 0, False, None),
    "blast_hydro_hllc_ng2": ("blast.cpp", "hllc", False, 2, 0, False, None),
    # harness: loads a raw state file written by the tests (own pgen)
    "state_mhd_hlld": ("harness:load_state.cpp", "hlld", True, 2, 0, False, None),
    "state_mhd_hlld_ng4": ("harness:load_state.cpp", "hlld", True, 4, 0, False, None),
    "state_hydro_hllc": ("harness:load_state.cpp", "hllc", False, 2, 0, False, None),
    "state_hydro_hlle": ("harness:load_state.cpp", "hlle", False, 2, 0, False, None),
    "state_mhd_hlle": ("harness:load_state.cpp", "hlle", True, 2, 0, False, None),
    "state_hydro_hllc_ng4": ("harness:load_state.cpp", "hllc", False, 4, 0, False, None),
    "state_hydro_lhllc": ("harness:load_state.cpp", "lhllc", False, 2, 0, False, None),
    "state_mhd_lhlld": ("harness:load_state.cpp", "lhlld", True, 2, 0, False, None),
    # multi-level (SMR) meshes from per-block states
    "smr_mhd_hlld": ("harness:load_blocks.cpp", "hlld", True, 2, 0, False, None),
    "smr_mhd_hlld_ng4": ("harness:load_blocks.cpp", "hlld", True, 4, 0, False, None),
    "smr_hydro_hllc": ("harness:load_blocks.cpp", "hllc", False, 2, 0, False, None),
    # multigrid self-gravity
    "poisson_mg": ("poisson.cpp", "hllc", False, 2, 2, False, None),
    "jeans_mg": ("jeans.cpp", "hllc", False, 2, 2, False, None),
    "sg_state_mhd_hlld": ("harness:load_state.cpp", "hlld", True, 2, 2, False, None),
    "sg_state_hydro": ("harness:load_state.cpp", "hllc", False, 2, 2, False, None),
    # FFT drivers (turbulence driving; FFT self-gravity, SELF_GRAVITY_ENABLED = 1), the
    # FFTW calls served by the test shim in harness/fftw3 (direct transforms)
    "turb_state_mhd_hlld": ("harness:load_state.cpp", "hlld", True, 2, 0, False, None),
    "turb_state_hydro_hllc": ("harness:load_state.cpp", "hllc", False, 2, 0, False, None),
    "fftgrav_state_hydro_hllc": ("harness:load_state.cpp", "hllc", False, 2, 1, False, None),
    "fftgrav_state_mhd_hlld": ("harness:load_state.cpp", "hlld", True, 2, 1, False, None),
}
FFT_BUILDS = {"turb_state_mhd_hlld", "turb_state_hydro_hllc", "fftgrav_state_hydro_hllc",
              "fftgrav_state_mhd_hlld"}
SHIM = os.path.join(HERE, "harness", "fftw3")
# the reference-side binding of the GB300 library (INTEGRATION.md's shim), compiled into the
# reference against its own headers and linked with the in-tree libathena_gb300.so
REPO = os.path.dirname(HERE)
PKG = os.path.join(REPO, "athena-gamma_gb300")
CONFIGS["shim_mhd_hlld"] = ("harness:shim_driver.cpp", "hlld", True, 2, 0, False, None)
LINKED = {"shim_mhd_hlld": {
    "srcs": [os.path.join(HERE, "harness", "gb300_shim.cpp")],
    "inc": [os.path.join(REPO, "include")],
    "ld": ["-L", PKG, "-lathena_gb300", "-Wl,-rpath," + PKG]}}


def source_list(pgen):
    s = []
    pat = ["src/*.cpp", "src/bvals/*.cpp", "src/bvals/cc/*.cpp", "src/bvals/cc/fft_grav/*.cpp",
           "src/bvals/cc/hydro/*.cpp", "src/bvals/cc/mg/*.cpp", "src/bvals/fc/*.cpp",
           "src/bvals/orbital/*.cpp", "src/bvals/utils/*.cpp", "src/coordinates/*.cpp",
           "src/fft/*.cpp", "src/field/*.cpp", "src/field/field_diffusion/*.cpp",
           "src/gravity/*.cpp", "src/hydro/*.cpp", "src/hydro/srcterms/*.cpp",
           "src/hydro/hydro_diffusion/*.cpp", "src/inputs/*.cpp", "src/mesh/*.cpp",
           "src/multigrid/*.cpp", "src/orbital_advection/*.cpp", "src/outputs/*.cpp",
           "src/reconstruct/*.cpp", "src/scalars/*.cpp", "src/task_list/*.cpp",
           "src/utils/*.cpp"]
    for p in pat:
        s += sorted(glob.glob(os.path.join(REF, p)))
    s.append(os.path.join(REF, "src/pgen/default_pgen.cpp"))
    if pgen.startswith("harness:"):
        s.append(os.path.join(HERE, "harness", pgen.split(":", 1)[1]))
    else:
        s.append(os.path.join(REF, "src/pgen", pgen))
    return s


def write_defs(d, pgen, flux, mhd, nghost, grav, omp, fft=False):
    with open(os.path.join(REF, "src/defs.hpp.in")) as f:
        t = f.read()
    sub = {
        "PROBLEM": pgen.replace("harness:", "").replace(".cpp", ""),
        "COORDINATE_SYSTEM": "cartesian",
        "RSOLVER": flux,
        "EQUATION_OF_STATE": "adiabatic",
        "GENERAL_EOS": "0",
        "EOS_TABLE_ENABLED": "0",
        "NON_BAROTROPIC_EOS": "1",
        "MAGNETIC_FIELDS_ENABLED": "1" if mhd else "0",
        "STS_ENABLED": "0",
        "SELF_GRAVITY_ENABLED": str(grav),
        "RELATIVISTIC_DYNAMICS": "0",
        "GENERAL_RELATIVITY": "0",
        "FRAME_TRANSFORMATIONS": "0",
        "SINGLE_PRECISION_ENABLED": "0",
        "H5_DOUBLE_PRECISION_ENABLED": "0",
        "FFT_OPTION": "FFT" if fft else "NO_FFT",
        "MPI_OPTION": "NOT_MPI_PARALLEL",
        "OPENMP_OPTION": "OPENMP_PARALLEL" if omp else "NOT_OPENMP_PARALLEL",
        "HDF5_OPTION": "NO_HDF5OUTPUT",
        "DEBUG_OPTION": "NOT_DEBUG",
        "EXCEPTION_HANDLING_OPTION": "ENABLE_EXCEPTIONS",
        "COMPILER_CHOICE": "g++",
        "COMPILER_COMMAND": "g++",
        "COMPILER_FLAGS": "-O3 -std=c++11",
        "NHYDRO_VARIABLES": "5",
        "NFIELD_VARIABLES": "3" if mhd else "0",
        "NWAVE_VALUE": "7" if mhd else "5",
        "NUMBER_PASSIVE_SCALARS": "0",
        "NUMBER_GHOST_CELLS": str(nghost),
    }
    for k, v in sub.items():
        t = t.replace("@" + k + "@", v)
    left = re.findall(r"@([A-Z_0-9]+)@", t)
    assert not left, "unsubstituted keys: %s" % left
    # sources include the header as "defs.hpp", "../defs.hpp" or "../../defs.hpp";
    # a nested include path makes each spelling resolve to the one generated file
    os.makedirs(os.path.join(d, "inc", "a", "b", "c"), exist_ok=True)
    p = os.path.join(d, "inc", "defs.hpp")
    old = open(p).read() if os.path.exists(p) else None
    if old != t:
        with open(p, "w") as f:
            f.write(t)


def build(name, jobs=8, verbose=False):
    pgen, flux, mhd, nghost, grav, omp, _ = CONFIGS[name]
    d = os.path.join(OUT, name)
    exe = os.path.join(d, "athena")
    fft = name in FFT_BUILDS
    write_defs(d, pgen, flux, mhd, nghost, grav, omp, fft)
    srcs = source_list(pgen)
    if fft:
        srcs.append(os.path.join(SHIM, "fftw3_dft.cpp"))
    extra = LINKED.get(name, {})
    srcs += extra.get("srcs", [])
    eos = os.path.join(REF, "src/eos", "adiabatic_mhd.cpp" if mhd else "adiabatic_hydro.cpp")
    srcs += [eos, os.path.join(REF, "src/eos/general/noop.cpp"),
             os.path.join(REF, "src/eos/eos_high_order.cpp"),
             os.path.join(REF, "src/eos/eos_scalars.cpp"),
             os.path.join(REF, "src/hydro/rsolvers", "mhd/" if mhd else "hydro/",
                          flux + ("_mhd" if (mhd and flux == "hlle") else "") + ".cpp")]
    inc = os.path.join(d, "inc")
    flags = ["-O3", "-std=c++11", "-I", inc, "-I", os.path.join(inc, "a"),
             "-I", os.path.join(inc, "a", "b"), "-I", os.path.join(inc, "a", "b", "c")]
    flags += ["-fopenmp"] if omp else []
    flags += ["-I", SHIM] if fft else []
    for d in extra.get("inc", []):
        flags += ["-I", d]
    if pgen.startswith("harness:"):
        flags += ["-I", os.path.join(REF, "src")]
    objdir = os.path.join(d, "obj")
    os.makedirs(objdir, exist_ok=True)
    defs_mtime = os.path.getmtime(os.path.join(inc, "defs.hpp"))

    def one(src):
        h = hashlib.md5(src.encode()).hexdigest()[:8]
        obj = os.path.join(objdir, os.path.basename(src)[:-4] + "_" + h + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) > max(defs_mtime, os.path.getmtime(src)):
            return obj
        cmd = ["g++"] + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (src, r.stderr[-3000:]))
        return obj

    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(one, srcs))
    if (not os.path.exists(exe)) or any(os.path.getmtime(o) > os.path.getmtime(exe) for o in objs):
        r = subprocess.run(["g++"] + flags + ["-o", exe] + objs + extra.get("ld", []),
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-3000:])
    if verbose:
        print("built", exe)
    return exe


def available():
    return os.path.isfile(os.path.join(REF, "src/defs.hpp.in"))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("names", nargs="*", default=[])
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    if not available():
        print("reference tree not present; nothing to build")
        sys.exit(0)
    for n in (a.names or list(CONFIGS)):
        if CONFIGS[n][0].startswith("harness:") and not os.path.exists(
                os.path.join(HERE, "harness", CONFIGS[n][0].split(":", 1)[1])):
            continue
        build(n, a.j, verbose=True)
