"""Triad-list nonlinear form on the GPU (k_triad, through the C ABI) vs the CPU oracle's
restatement of ops_in_planes / nonlinInter (FOU3D.f90:1724-2088), same seeded inputs.
Lists: the complete enumeration, and seeded random subsets in shuffled order that
differ per file and per product (stand-ins for the reference's thresholded lists).
Bar: FP64 form within 1e-12 relative per step; mixed form within 1e-5."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.native import GpuChannel, LhError
from rnl_multiblock_nofft_gb300.triads import TriadLists
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

pytestmark = pytest.mark.gpu
FIELDS = ("u1", "u2", "u3", "p")


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def run_pair(name, lists, seed, precision, steps):
    s = workload_setup(name)
    tl = TriadLists.complete(s) if lists == "complete" else TriadLists.thinned(s, 0.7, seed=seed + 1)
    st = initial_field(s, seed)
    o = Oracle(s, triads=tl)
    o.set_state(*st)
    o.set_scalars(**initial_scalars(s))
    g = GpuChannel(s, precision, triads=tl)
    g.upload_state(*st)
    g.set_scalars(**initial_scalars(s))
    errs = []
    for _ in range(steps):
        o.step()
        g.step()
        g.synchronize()
        errs.append({f: relerr(b, a) for f, a, b in zip(FIELDS, o.get_state(), g.download_state())})
    return s, o, g, errs


@pytest.mark.parametrize("lists", ["complete", "thinned"])
def test_triad_fp64_matches_oracle(cuda_ok, lists):
    s, o, g, errs = run_pair("C0", lists, 31, "fp64", 2)
    for k, e in enumerate(errs):
        for f in FIELDS:
            assert e[f] < 1e-12 * (k + 1), (k, f, e[f])
    so, sg = o.scalars(), g.scalars()
    assert sg["t"] == pytest.approx(so["t"], rel=1e-14)
    assert sg["Qx"] == pytest.approx(so["Qx"], rel=1e-13)


def test_triad_small_channel(cuda_ok):
    # N 16: x-mode 8 and z-mode -8 carry data, exercising the linear-advection-only modes
    _, _, _, errs = run_pair("S", "thinned", 33, "fp64", 2)
    for k, e in enumerate(errs):
        for f in FIELDS:
            assert e[f] < 1e-12 * (k + 1), (k, f, e[f])


def test_triad_mixed_within_1e5(cuda_ok):
    _, _, _, errs = run_pair("C0", "thinned", 35, "mixed", 2)
    for e in errs:
        for f in ("u1", "u2", "u3"):
            assert e[f] < 1e-5, (f, e[f])


def test_triad_header_mismatch_rejected(cuda_ok):
    s = workload_setup("S")
    tl = TriadLists.complete(s)
    tl.nx += 1
    with pytest.raises(LhError, match="nx number"):
        GpuChannel(s, "fp64", triads=tl)
