"""The integer-pipe FP64 add / multiply (arcanefem_gb300/csrc/afem_fp64_int.cuh)
against the host's IEEE binary64 arithmetic, bit for bit, on random normal
operands with equal, adjacent and distant exponents, near-equal magnitudes,
significands near 2 and exact cancellations."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integer_fp64_ops_match_ieee(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "fp64_int_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "arcanefem_gb300", "csrc"), os.path.join(ROOT, "tests", "fp64_int_check.cc"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for seed in (1, 2):
        out = subprocess.run([exe, "3000000", str(seed)], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stderr
        bad_mul, bad_add, bad_sub, fallbacks = map(int, out.stdout.split())
        assert (bad_mul, bad_add, bad_sub) == (0, 0, 0)
