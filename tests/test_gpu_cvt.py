"""The integer-pipe conversions d2f_alu / f2d_alu (lh_internal.cuh), which every kernel of the
mixed form uses in place of the conversion instructions, against the hardware conversions on
the GPU: ties to even, the carry into the exponent, the overflow edge, subnormals, signed zeros,
infinities, NaN and random inputs (tests/cvt_check.cu states the contract)."""
import os
import subprocess

import pytest

from test_fft_host import nvcc

HERE = os.path.dirname(os.path.abspath(__file__))
pytestmark = pytest.mark.gpu


def test_conversions_match_hardware(cuda_ok, tmp_path):
    cc = nvcc()
    if cc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "cvt_check")
    subprocess.run([cc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    os.path.join(HERE, "cvt_check.cu"), "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    w = r.stdout.split()
    assert w[0] == "d2f" and w[3] == "f2d", r.stdout
    nd, bad_d, nf, bad_f = int(w[1]), int(w[2]), int(w[4]), int(w[5])
    assert nd > 400000 and nf > 400000
    assert bad_d == 0, r.stderr
    assert bad_f == 0, r.stderr
