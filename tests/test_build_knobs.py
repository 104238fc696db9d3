"""The stencil pass's compile-time knobs build in their non-default settings too (nvcc
cross-compiles for sm_103a without a GPU): the scalar arithmetic that the packed f32x2 forms
replace stays compilable, so the bit-for-bit comparison of the two builds can be repeated."""
import os
import shutil
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_scalar_arithmetic_build_compiles():
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("nvcc not available")
    sys.path.insert(0, os.path.join(ROOT, "proxy-geos-hc_gb300"))
    import build
    with tempfile.TemporaryDirectory() as d:
        cmd = [build.nvcc(), *build._flags("k_stencil.cu"), "-DSEM_STENCIL_PACKED=0", "-DSEM_STENCIL_PACKED_AXIS=0",
               "-c", os.path.join(build.CSRC, "k_stencil.cu"), "-o", os.path.join(d, "k_stencil.o")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
