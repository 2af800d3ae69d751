"""Statistics on the GPU (k_xstats, through the C ABI) vs the CPU oracle: plane sums
and tile-conditioned sums of stats.f90 after accumulating twice around a step.
Bar: FP64 form 1e-12 relative to the largest sum; mixed 1e-5."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.native import GpuChannel
from rnl_multiblock_nofft_gb300.workloads import (initial_field, initial_field_bands, initial_scalars,
                                                  workload_setup)

pytestmark = pytest.mark.gpu


def run(name, precision, seed):
    s = workload_setup(name)
    o = Oracle(s)
    g = GpuChannel(s, precision)
    if s.multiblock:
        f = initial_field_bands(s, seed)
        o.set_bands(f)
        g.upload_bands(f)
    else:
        f = initial_field(s, seed)
        o.set_state(*f)
        g.upload_state(*f)
    for x in (o, g):
        x.set_scalars(**initial_scalars(s))
        x.stats_accumulate()
        x.step()
        x.stats_accumulate()
    g.synchronize()
    return o.stats(), g.stats()


def close(a, b, tol):
    # relative to the largest sum (the energy scale): sums with a zero mean (V, UV) have
    # no scale of their own
    scale = max(np.abs(a).max(), 1e-300)
    for q in range(a.shape[0]):
        assert np.abs(a[q] - b[q]).max() <= tol * scale, (q, np.abs(a[q] - b[q]).max() / scale)


@pytest.mark.parametrize("name,precision,tol", [("SP", "fp64", 1e-12), ("MB", "fp64", 1e-12),
                                                ("SP", "mixed", 1e-5)])
def test_stats_match_oracle(cuda_ok, name, precision, tol):
    (po, co, io), (pg, cg, ig) = run(name, precision, 51)
    assert io == ig == 2
    close(po, pg, tol)
    if co is not None:
        assert cg is not None and cg.shape == co.shape
        close(co.reshape(9, -1), cg.reshape(9, -1), tol)
