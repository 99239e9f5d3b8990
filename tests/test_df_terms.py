"""The compensated single-precision shape terms of the pair kernels
(corr_pc_gb300/csrc/pair_df.cuh), built for the host, against the
double-precision terms of pair_values.h (the reference's corels.cpp): every
cancelling field within 2^-40 of its bound for float32 positions, the
fixed-point conversion within half a quantum plus rounding, words in range."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "corr_pc_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_df_terms_match_double(tmp_path):
    exe = str(tmp_path / "df_terms")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(ROOT, "tests", "df_terms_driver.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "200000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("range ok") == 10, r.stdout
