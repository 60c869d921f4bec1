"""TEST INFRASTRUCTURE ONLY: builds the CPU oracle (and, where the reference
sources are present, the CPU build of the reference itself).

    python -m oracle.build            # oracle only
    python -m oracle.build --ref      # also oracle/_ref/libostr_ref.so
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "libostr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libostr_ref.so")
# The reference sources: NR_REFERENCE_DIR, else a checkout named "reference"
# beside this repository.
REFERENCE_DIR = os.environ.get(
    "NR_REFERENCE_DIR", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def oracle_cmd():
    return ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC",
            "-shared", "-o", ORACLE_SO, os.path.join(HERE, "ostr_oracle.cpp")]


def build_oracle() -> subprocess.Popen:
    os.makedirs(BUILD_DIR, exist_ok=True)
    return subprocess.Popen(oracle_cmd())


def reference_present() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_DIR, "Tomo_OSTR.cu"))


def build_reference() -> subprocess.Popen | None:
    if not reference_present():
        return None
    return subprocess.Popen(["bash", os.path.join(HERE, "build_ref.sh")])


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    procs = [build_oracle()]
    if "--ref" in argv:
        p = build_reference()
        if p is not None:
            procs.append(p)
    rc = 0
    for p in procs:
        rc |= p.wait()
    return rc


if __name__ == "__main__":
    sys.exit(main())
