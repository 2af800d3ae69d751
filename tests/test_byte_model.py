"""bench.py's algorithmic byte model against the DRAM traffic that ncu measured per launch at
C1 (profiles/ncu_traffic_C1.txt): the transform kernels move their compulsory bytes and no
more (within 5 %: writes still in L2 when a kernel ends are not counted by ncu), and the
pressure step's traffic exceeds its count by the documented second read of u, w and v."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
from rnl_multiblock_nofft_gb300.workloads import workload_setup  # noqa: E402


@pytest.fixture(scope="module")
def c1():
    return workload_setup("C1"), bench.traffic_table()


@pytest.mark.parametrize("kernel", ["k_xpass_nl", "k_zinv_nl"])
def test_transform_kernels_move_their_compulsory_bytes(c1, kernel):
    s, table = c1
    alg = bench.algorithmic_bytes(s, kernel, "mixed")
    traffic = table[("C1", kernel, "mixed")]
    assert 0.95 < traffic / alg <= 1.0, (kernel, traffic / alg)


def test_pressure_traffic_is_its_count_plus_the_second_read(c1):
    s, table = c1
    alg = bench.algorithmic_bytes(s, "k_press", "mixed")
    traffic = table[("C1", "k_press", "mixed")]
    # per column level: the forward sweep reads u, w, v (complex128) and the factors dg1, dg2
    # (one double each) and writes psi; the backward sweep reads psi, p, u, w, v and dg3 and
    # writes p, u, w, v
    forward = 3 * 16 + 2 * 8 + 16
    backward = 5 * 16 + 8 + 4 * 16
    full = bench.column_levels(s, 2) * (forward + backward)
    assert alg < traffic <= full, (alg, traffic, full)


def test_solve_counts_per_column_level():
    s = workload_setup("C0")
    for form, uw, v in (("fp64", 208, 112), ("mixed", 144, 80)):
        assert bench.algorithmic_bytes(s, "k_helm_uw", form) == bench.column_levels(s, 2) * uw
        assert bench.algorithmic_bytes(s, "k_helm_v", form) == bench.column_levels(s, 1) * v
