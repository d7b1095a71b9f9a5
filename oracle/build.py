"""Build recipe for the C oracle (test infrastructure; see mk_oracle.c).

``python oracle/build.py`` or ``oracle.build.build()`` compiles
``mk_oracle.c`` with gcc into ``oracle/_build/libmk_oracle.so``.  Portable
flags only (no -march=native) so the same recipe builds on x86_64 and
aarch64; -ffp-contract=off keeps every a*b+c as two roundings.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mk_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmk_oracle.so")


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-shared", "-fPIC", SRC, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
