"""The blow-up guard: a non-finite value in the uploaded state reaches dt and err through
the CFL and divergence maxima, and lh_synchronize reports LH_ENONFINITE (no GPU fault:
NaN arithmetic is ordinary input here)."""
import numpy as np
import pytest

from rnl_multiblock_nofft_gb300.abi import LH_ENONFINITE
from rnl_multiblock_nofft_gb300.native import GpuChannel, LhError
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_state_is_reported(cuda_ok, precision):
    s = workload_setup("S")
    st = initial_field(s, 90)
    st[0][3, 5] = np.nan
    g = GpuChannel(s, precision)
    g.upload_state(*st)
    g.set_scalars(**initial_scalars(s))
    g.step(1)
    with pytest.raises(LhError) as e:
        g.synchronize()
    assert e.value.code == LH_ENONFINITE


def test_finite_state_passes(cuda_ok):
    s = workload_setup("S")
    g = GpuChannel(s, "mixed")
    g.upload_state(*initial_field(s, 91))
    g.set_scalars(**initial_scalars(s))
    g.step(2)
    g.synchronize()
    assert np.isfinite(g.scalars()["err"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_v_reaches_dt_in_the_first_substep(cuda_ok, precision):
    # a NaN only in v reaches dt through the v maximum of the CFL limit; the guard fires
    # after lh_substep(1) alone, before the divergence of the third substep is formed
    s = workload_setup("S")
    st = initial_field(s, 92)
    st[1][4, 7] = np.nan
    g = GpuChannel(s, precision)
    g.upload_state(*st)
    g.set_scalars(**initial_scalars(s))
    g.substep(1)
    with pytest.raises(LhError) as e:
        g.synchronize()
    assert e.value.code == LH_ENONFINITE
    assert np.isnan(g.scalars()["dt"])
