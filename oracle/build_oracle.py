"""Build recipe for the CPU oracle (test infrastructure, never part of the product path).

Compiles oracle/pn_oracle.c into oracle/_build/libpn_oracle.so with gcc.  The flags pin
Julia's floating-point behaviour: no contraction of a*b+c into an FMA (gcc contracts by
default on aarch64), no fast-math.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpn_oracle.so")
SRCS = ["pn_oracle.c"]
DEPS = ["pn_oracle.c", "pn_oracle.h", "pn_oracle_body.h"]
CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-Wno-unused-function", "-Wno-maybe-uninitialized"]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in DEPS)


def build(force: bool = False) -> str:
    """Compile the oracle if its sources changed; return the library path."""
    if force or _stale():
        os.makedirs(OUT_DIR, exist_ok=True)
        cmd = ["gcc", *CFLAGS, *[os.path.join(HERE, s) for s in SRCS], "-lm", "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
