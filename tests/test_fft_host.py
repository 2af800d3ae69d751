"""The shared-memory FFT's plan on the CPU (tests/fft_host_check.cu): every compiled length,
both layouts, both directions, FP64 and FP32, against a direct DFT in long double."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
LENGTHS = (24, 48, 72, 96, 144, 192, 288, 384, 576, 768, 1152)


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


def test_fft_plan_against_direct_dft(tmp_path):
    cc = nvcc()
    if cc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "fft_host_check")
    subprocess.run([cc, "-O2", "-std=c++17", "-x", "cu", os.path.join(HERE, "fft_host_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout
    rows = {int(r.split()[0]): [float(x) for x in r.split()[1:]] for r in out.strip().splitlines()}
    assert sorted(rows) == list(LENGTHS)
    for n, e in rows.items():
        assert max(e[:4]) < 1e-14, (n, e[:4])   # FP64: IL0 fwd/inv, IL1 fwd/inv
        assert max(e[4:]) < 2e-6, (n, e[4:])    # FP32


def test_register_dfts_against_direct_dft(tmp_path):
    """The register DFTs of the two-stage transform kernels (lh_regfft.cuh,
    tests/regfft_host_check.cu): every radix the plans use, both directions, FP64 and FP32,
    and the compile-time twiddle constants."""
    cc = nvcc()
    if cc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "regfft_host_check")
    subprocess.run([cc, "-O2", "-std=c++17", "-x", "cu", os.path.join(HERE, "regfft_host_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout.strip().splitlines()
    rows = {r.split()[0]: [float(x) for x in r.split()[1:]] for r in out}
    assert float(rows.pop("tw")[0]) < 1e-15
    assert {int(k) for k in rows} >= {2, 3, 4, 6, 8, 9, 12, 16, 18, 24, 32, 36, 48, 72}
    for n, e in rows.items():
        assert max(e[:2]) < 1e-15, (n, e)   # FP64 forward / inverse
        assert max(e[2:]) < 5e-7, (n, e)    # FP32


def test_inverse_z_pass_slot_order(tmp_path):
    """The inverse z passes' launch rows (zinv_slot, tests/slot_order_check.cu): a bijection
    onto the slots for every split of u and v slots, each row following the row that read a
    level it reads again."""
    cc = nvcc()
    if cc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "slot_order_check")
    subprocess.run([cc, "-O2", "-std=c++17", "-x", "cu", os.path.join(HERE, "slot_order_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok %d" % (161 * 161), out.stdout

