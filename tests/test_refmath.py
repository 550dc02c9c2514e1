"""The FP32 evaluations of the reference's double-promoted expressions
(flip3d_gb300/csrc/refmath.h) against the expressions themselves, on the host
with the same IEEE float operations the GPU uses."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_refmath_matches_reference_expressions(tmp_path):
    exe = tmp_path / "refmath_check"
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-o", str(exe),
                           os.path.join(ROOT, "tests", "native", "refmath_check.cpp")])
    out = subprocess.check_output([str(exe), "1000000"], text=True).strip().splitlines()[-1]
    fields = out.split()
    counts = {fields[i]: int(fields[i + 1]) for i in range(0, 14, 2)}
    assert all(v == 0 for v in counts.values()), out
