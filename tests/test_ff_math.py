"""Accuracy of the float-float (two-FP32) arithmetic used by the mixed form
(atomistica_gb300/csrc/ff.h), compiled for the host and checked against long
double references (CPU only)."""

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ff_kernel_math(tmp_path):
    exe = str(tmp_path / "ff_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "atomistica_gb300", "csrc"),
                           "-I", "/usr/local/cuda/include",
                           os.path.join(ROOT, "tests", "cpp", "ff_check.cpp"), "-o", exe])
    e_exp, e_log, e_sin, e_cos, e_sqrt, e_rsqrt, e_rcp, e_mul = \
        [float(x) for x in subprocess.check_output([exe]).split()]
    assert e_exp < 2e-12      # relative, |t| < 30
    assert e_log < 2e-12      # absolute
    assert e_sin < 1e-11 and e_cos < 1e-11
    assert e_sqrt < 1e-13 and e_rsqrt < 1e-13 and e_rcp < 1e-13 and e_mul < 1e-13


def test_ff_tables_header_is_generated():
    # csrc/ff_tables.h is exactly the output of its generator
    # (csrc/gen_ff_tables.py: 60-digit arithmetic, integer rounding to FP32)
    import io
    import sys
    pytest.importorskip("mpmath")
    here = os.path.join(ROOT, "atomistica_gb300", "csrc")
    sys.path.insert(0, here)
    try:
        import gen_ff_tables
    finally:
        sys.path.remove(here)
    buf = io.StringIO()
    gen_ff_tables.main(buf)
    with open(os.path.join(here, "ff_tables.h")) as fh:
        assert fh.read() == buf.getvalue()
