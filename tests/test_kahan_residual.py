"""The integer-pipe Kahan residual (rusty_particles_gb300/csrc/rp_kahan.h)
against FP64 hardware: built for the host and run on 20 million seeded cases
(integrator magnitudes, near cancellations, arbitrary exponents, raw bit
patterns with zeros, subnormals, inf and NaN); wherever it answers, its bits
must equal those of (t - s) - y."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_kahan_residual_bits_match_fp64(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "kahan_check"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-std=c++17", "-I",
                    os.path.join(ROOT, "rusty_particles_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "kahan_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "20000000", "11"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = r.stdout.split()
    fast = int(fields[fields.index("fast") + 1])
    assert fast > 10_000_000, r.stdout  # the integer path answers for most cases
