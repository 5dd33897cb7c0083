"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``wb_oracle.c`` into ``oracle/libwb_oracle.so`` with gcc at -O2 and
``-ffp-contract=off`` so that no multiply-add is fused on either x86-64 or
aarch64 hosts (the reference's Cython C is built with gcc -O2 on x86-64, which
never fuses without -mfma).
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "wb_oracle.c")
LIB = os.path.join(HERE, "libwb_oracle.so")


def build(force=False):
    if (
        not force
        and os.path.exists(LIB)
        and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
    ):
        return LIB
    cmd = [
        os.environ.get("CC", "gcc"),
        "-O2",
        "-std=c99",
        "-D_GNU_SOURCE",
        "-ffp-contract=off",
        "-fno-fast-math",
        "-fPIC",
        "-shared",
        "-pthread",
        SRC,
        "-o",
        LIB + ".tmp",
        "-lm",
    ]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
