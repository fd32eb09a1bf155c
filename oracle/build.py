"""Build recipe for the oracle shared library (test infrastructure).

``gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC gbdx_oracle.c`` into
``oracle/_build/``.  -ffp-contract=off keeps x86-64 and aarch64 bit-identical.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def oracle_lib_path() -> str:
    return os.path.join(HERE, "_build", "libgbdx_oracle.so")


def build_oracle() -> str:
    out = oracle_lib_path()
    os.makedirs(os.path.dirname(out), exist_ok=True)
    src = os.path.join(HERE, "gbdx_oracle.c")
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC",
           "-shared", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle())
