"""Why the FP64 form keeps FP64 transforms: the oracle run with noise of amplitude eps on every
transform output (the size of a transform's rounding: ~1e-16 for FP64, ~1e-14 for a float-float
transform with 48-bit significands) against the same run without. The velocities move by about
eps, the pressure by ~1e3 eps (measured: 1.3e-13 at eps 1.1e-16, 1.1e-11 at eps 1e-14 on this
textured channel; 4.2e-13 and 3.6e-11 at the 256²×301 headline size), so a float-float
transform would put the pressure 10-40x outside the FP64 form's 1e-12 parity bar."""
import numpy as np
import pytest

import oracle as oracle_mod
from oracle import Oracle
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

FIELDS = ("u1", "u2", "u3", "p")


def one_step(s, st, eps):
    oracle_mod.set_transform_noise(eps)
    try:
        o = Oracle(s)
        o.set_state(*st)
        o.set_scalars(**initial_scalars(s))
        o.step()
        out = o.get_state()
        o.close()
    finally:
        oracle_mod.set_transform_noise(0.0)
    return out


def test_pressure_amplifies_transform_rounding():
    s = workload_setup("SP")
    st = initial_field(s, 1001)
    ref = one_step(s, st, 0.0)
    rel = {}
    for eps in (1.1e-16, 1e-14):
        got = one_step(s, st, eps)
        rel[eps] = {f: np.linalg.norm(a - b) / np.linalg.norm(b) for f, a, b in zip(FIELDS, got, ref)}
    # FP64-sized rounding keeps every field inside the FP64 form's 1e-12 bar
    assert max(rel[1.1e-16].values()) < 1e-12
    # float-float-sized rounding: the velocities stay inside, the pressure does not
    assert max(rel[1e-14][f] for f in ("u1", "u2", "u3")) < 1e-12
    assert rel[1e-14]["p"] > 5e-12
    # and the pressure's response is linear in eps, ~1e3 eps
    assert rel[1e-14]["p"] / rel[1.1e-16]["p"] == pytest.approx(1e-14 / 1.1e-16, rel=0.3)
