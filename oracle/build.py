"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/bsam_oracle.c into oracle/libbsam_oracle.so with FMA
contraction disabled (-ffp-contract=off) so that every multiply and add is
rounded separately, as in the reference Fortran built without fast-math.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bsam_oracle.c")
LIB = os.path.join(HERE, "libbsam_oracle.so")


def build_oracle(force=False):
    """Compile the oracle shared library if it is missing or stale."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "bsam_oracle.h")))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-variable",
           "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
