"""Test infrastructure: build the reference's own CPU code into oracle/_ref/ (never into the
reference tree) and link the harness oracle/ref_harness.cpp against it.

The reference is compiled from its sources where they lie, with g++ directly on its translation
units (not its Makefile): the configuration includes param.py generates are committed in the
reference, so no code generation runs. -O2 without -march, so that on x86-64 no FMA contraction
happens and the restatement in oracle/atsat_oracle.c (built with -ffp-contract=off) can be compared
with it bit for bit.

Usage: python oracle/build_ref.py [--ref PATH] [--jobs N]
The reference tree is PATH, else $ATSAT_REFERENCE, else /root/reference.
Produces oracle/_ref/ref_harness. Exits 0 without doing anything when the reference tree is absent.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def default_ref() -> str:
    """The reference tree: $ATSAT_REFERENCE when set, else where this container mounts it."""
    return os.environ.get("ATSAT_REFERENCE") or "/root/reference"

# The translation units of libatsat (the reference Makefile's LIB_OBJ, ATSAT_OBJ, XML_OBJ) and the
# command-line stream stub, which the harness needs instead of cli/sat.cpp's main().
SOURCES = [
    "lib/Array.cpp", "lib/Array_2D.cpp", "lib/Array_1D.cpp", "lib/Config.cpp", "lib/Utils.cpp",
    "lib/FFT.cpp",
    "planet/cSaturnModel.cpp", "planet/PrintMsg_Sat.cpp", "planet/RungeKutta_Sat_Turb.cpp",
    "planet/RHS_Sat_Turb.cpp", "planet/BC_Sat.cpp", "planet/ParaView_Sat.cpp",
    "planet/Thermo_Sat.cpp", "planet/Pressure_Sat.cpp", "planet/InitVelocity_Sat.cpp",
    "planet/InitVariables_Sat.cpp", "planet/Weather_Sat.cpp", "planet/FileIO_Sat.cpp",
    "planet/SaturationAdjustmentSat.cpp",
    "tinyxml2/tinyxml2.cpp", "cli/DefaultStream.cpp",
]
FLAGS = ["-O2", "-std=c++11", "-fopenmp", "-fPIC", "-w"]


def build(ref: str, jobs: int) -> str:
    if not os.path.isdir(os.path.join(ref, "planet")):
        print(f"build_ref: no reference tree at {ref}; nothing to build")
        return ""
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    inc = ["-I" + os.path.join(ref, d) for d in ("lib", "planet", "tinyxml2")]

    def cc(src):
        obj = os.path.join(objdir, src.replace("/", "_").replace(".cpp", ".o"))
        path = os.path.join(ref, src)
        if os.path.exists(obj) and os.path.getmtime(obj) > os.path.getmtime(path):
            return obj
        subprocess.run(["g++", *FLAGS, *inc, "-c", path, "-o", obj], check=True)
        return obj

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(cc, SOURCES))
    exe = os.path.join(OUT, "ref_harness")
    subprocess.run(["g++", *FLAGS, *inc, os.path.join(HERE, "ref_harness.cpp"), *objs,
                    "-o", exe], check=True)
    return exe


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=default_ref())
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    exe = build(a.ref, a.jobs)
    if exe:
        print(exe)


if __name__ == "__main__":
    sys.exit(main())
