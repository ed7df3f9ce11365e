"""The mixed path's integer binary32/binary64 conversions and error-free sums
(athena-gamma_gb300/csrc/athg_numeric.h), compiled for the host and checked bit for bit
against the host's IEEE 754 casts and exact sums."""
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "athena-gamma_gb300", "csrc")


def test_numeric_helpers():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "numeric_check")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                               os.path.join(HERE, "numeric_check.cpp"), "-o", exe])
        out = subprocess.run([exe, "1000000"], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
