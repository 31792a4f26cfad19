"""Build recipe for the CPU oracle (test infrastructure; never part of the product path).

Compiles oracle/omx_oracle.c (time domain) and oracle/fd_oracle.c (frequency-domain operator
and BiCGStab(L)) into oracle/liborc.so with gcc: -O2, OpenMP, and
-ffp-contract=off so that no multiply-add is contracted (the reference's gfortran -O3
build on a generic target emits none).

The reference itself is Fortran 2008 with a hard dependency on the external DFTB+ library;
there is no Fortran compiler in the build image, so nothing from the reference is compiled
here and oracle/_ref stays empty.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "omx_oracle.c")
SRC_FD = os.path.join(HERE, "fd_oracle.c")
OUT = os.path.join(HERE, "liborc.so")


def build(force=False):
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(
            os.path.getmtime(SRC), os.path.getmtime(SRC_FD), os.path.getmtime(os.path.join(HERE, "omx_oracle.h"))):
        return OUT
    tmp = OUT + ".tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c99",
           "-o", tmp, SRC, SRC_FD, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
