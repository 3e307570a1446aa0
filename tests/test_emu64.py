"""The integer-pipe binary64 arithmetic of hamers_gb300/csrc/hmr_emu64.cuh, bit for bit.

The emulated multiply, add and subtract stand in for native FP64 instructions in the face
kernels, so they must give the native results for every input.  The CPU test builds the header
for the host (tests/native/emu64_host_check.cpp) and compares it with the host's IEEE-754
operations on seeded operand families that reach every branch: typical and extreme exponents,
arbitrary bit patterns, exact products and rounding ties, cancellation, zeros.  The GPU test
runs the same comparison on the device against __dmul_rn / __dadd_rn / __dsub_rn.
"""
import ctypes
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "emu64_host_check.cpp")


def test_host_build_matches_ieee_double(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "emu64_host_check")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", SRC, "-o", exe])
    out = subprocess.run([exe, "2000000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-3000:]
    assert out.stdout.count(" 0 mismatches") == 20, out.stdout


@pytest.mark.gpu
def test_device_matches_native_instructions(cuda):
    from hamers_gb300 import build as B
    lib = ctypes.CDLL(B.PEAK_LIB)
    lib.hmr_emu64_check.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.hmr_emu64_check.restype = ctypes.c_int
    bad = (ctypes.c_ulonglong * 21)()
    assert lib.hmr_emu64_check(64, bad) == 0
    assert list(bad) == [0] * 21
