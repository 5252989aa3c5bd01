"""CPU test of the integer-pipe format conversions (csrc/sf_convert.cuh): double -> float rounds to nearest even
and float -> double is exact, bit for bit equal to the compiler's casts on edge cases (zeros, halfway cases in
every binade, subnormal and overflowing results, infinities, NaN) and on 12 M seeded random values.  The device
code compiles the same functions."""
import os
import subprocess

from conftest import ROOT


def test_conversions_match_casts():
    src = os.path.join(ROOT, "tests", "cpp", "convert_check.cpp")
    out_dir = os.path.join(ROOT, "oracle", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "convert_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                           os.path.join(ROOT, "simferrofluid-cuda_gb300", "csrc"), src, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    bad, n = (int(v) for v in r.stdout.split()[-2:])
    assert r.returncode == 0 and bad == 0, r.stdout
    assert n > 12_000_000
