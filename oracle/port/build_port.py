"""Compile ``pdq_port.c`` into ``libpdq_port.so`` next to it (gcc, no cmake).

Test infrastructure: the C port is the timed CPU baseline and a second check
of the Python oracle.  Host code only (no intrinsics, no -march=native), so it
builds the same on x86-64 and aarch64.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pdq_port.c")
LIB = os.path.join(HERE, "libpdq_port.so")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-o", LIB + ".tmp", SRC, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"gcc failed:\n{res.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
