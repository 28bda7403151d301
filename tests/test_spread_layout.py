"""The spread layout's index arithmetic, on the host (no GPU).

tests/spread_layout_check.cu is built with nvcc from the library's own
headers (spread_range, spread_cta_of, spread_group, make_spread_layout are
host-and-device functions) and run here: over random (nbeta, nseq, sequence
groups, replicas per CTA, CTAs) within the launch constraints it checks that
the groups' layouts hold every replica once, that each sequence has one
exchange owner whose slot is its ibeta = 0 replica, and that the owner waits
for exactly the CTAs that hold the sequence.  The same arithmetic runs in the
spread kernel, where a wrong count would end every wait in CMC_ERR_TIMEOUT.
"""
import os
import shutil
import subprocess

import pytest

from cuda_mcmc_gb300 import _build

HERE = os.path.dirname(os.path.abspath(__file__))


def test_spread_layout_index_arithmetic(tmp_path):
    nvcc = _build.nvcc()
    if shutil.which(nvcc) is None and not os.path.exists(nvcc):
        pytest.skip("nvcc not present")
    exe = str(tmp_path / "spread_layout_check")
    cmd = [nvcc, *_build.ARCH, "-O2", "-std=c++17", "-I", _build.CSRC, "-I", _build.INCLUDE,
           "--expt-relaxed-constexpr", os.path.join(HERE, "spread_layout_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert r.stdout.startswith("ok ") and int(r.stdout.split()[1]) >= 1000, r.stdout
