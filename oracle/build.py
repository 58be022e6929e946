"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/genfire_oracle.c`` into ``oracle/_build/libgenfire_oracle.so``
with gcc, OpenMP, and ``-ffp-contract=off`` so that FP32 selection arithmetic
is evaluated operation by operation, exactly as written.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "genfire_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgenfire_oracle.so")

CFLAGS = ["-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
          "-shared", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def build_oracle(force=False):
    """Compile the oracle if it is missing or older than its source; return the .so path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc"] + CFLAGS + ["-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
