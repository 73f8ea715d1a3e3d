"""Build recipe of the CPU oracle (test infrastructure: the CPU oracle the GPU product is tested against).

Compiles ``oracle/jf_oracle.c`` into ``oracle/_build/libjforacle.so`` with ``-ffp-contract=off`` so that
every floating-point operation is rounded on its own, as CPython rounds Python-level float arithmetic.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIBRARY = os.path.join(BUILD_DIR, "libjforacle.so")


def build(force: bool = False) -> str:
    source = os.path.join(HERE, "jf_oracle.c")
    header = os.path.join(HERE, "jf_oracle.h")
    if (not force and os.path.exists(LIBRARY)
            and os.path.getmtime(LIBRARY) >= max(os.path.getmtime(source), os.path.getmtime(header))):
        return LIBRARY
    os.makedirs(BUILD_DIR, exist_ok=True)
    temporary = LIBRARY + ".%d.tmp" % os.getpid()
    command = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off",
               "-fno-fast-math", "-Wall", "-o", temporary, source, "-lm"]
    subprocess.run(command, check=True)
    os.replace(temporary, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
