"""Host runs of kernel bodies: compile a harness from this directory with the
host C++ compiler (``cuda_runtime.h`` here stands in for the CUDA runtime),
under AddressSanitizer and UBSan where the toolchain has them."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def compile_harness(source, exe, sanitize="address,undefined"):
    """Compile ``tests/hostsim/<source>`` to ``exe`` (AddressSanitizer and
    UBSan, or ``sanitize="thread"`` for ThreadSanitizer); skips the test
    without g++."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-pthread", "-ffp-contract=off", "-fsanitize=" + sanitize, "-fno-sanitize-recover=all",
           "-I" + HERE, "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "probdiffeq_gb300", "csrc"),
           os.path.join(HERE, source), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0 and "sanitize" in res.stderr and sanitize == "thread":
        pytest.skip("no ThreadSanitizer runtime")
    if res.returncode != 0 and "sanitize" in res.stderr:
        cmd = [c for c in cmd if "sanitize" not in c]  # a toolchain without the sanitizer runtimes
        res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    return str(exe)


def run_harness(exe, path):
    """Run a compiled harness on an input file; returns its stdout lines."""
    res = subprocess.run([exe, str(path)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-4000:]
    return res.stdout.strip().splitlines()
