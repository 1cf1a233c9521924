"""Build recipe for the C restatement of the reference interpolation (test/baseline infrastructure).

    python -m oracle.build_oracle

Compiles ``oracle/interp_oracle.c`` with gcc and OpenMP into
``oracle/_build/liboracle_interp.so`` (git-ignored). Portable flags only:
the same recipe runs on x86_64 and aarch64.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle_interp.so")
SRC = os.path.join(HERE, "interp_oracle.c")


def build(force: bool = False) -> str:
    if not force and os.path.isfile(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-o", OUT + ".tmp", SRC,
           "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
