"""Multiblock channels on the CPU oracle: wall bands (1, 3) at a finer x/z resolution
than the core band (2). Long columns (the core's modes) span every level, short
columns (the wall bands' extra modes) only their band, with the band's boundary rows
(tridLU_3D.f90:257-329, start.f90:537-559) and plane transposes per band
(FOU3D.f90:1000-1098, 2295-2442). The reference's multiblock run needs three or more
MPI ranks and left no output, so these checks are structural: per-band state I/O,
the projection keeps every band divergence-free, the flow rate holds, and a
single-resolution channel gives the same step through the band layout."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.workloads import (initial_field, initial_field_bands, initial_scalars,
                                                  workload_setup)


def test_band_geometry():
    s = workload_setup("MB")
    assert s.multiblock and (s.N1c, s.N2c, s.G1c, s.G2c) == (16, 16, 24, 24)
    c1, c2, c3 = (s.band_cols(b) for b in (1, 2, 3))
    assert len(c2) == (s.N1c // 2 + 1) * s.N2c
    assert np.array_equal(c1, c3) and len(c1) + len(c2) == (s.N1 // 2 + 1) * s.N2
    assert np.intersect1d(c1, c2).size == 0
    # band 1 levels: jlim(ugrid, 1) = N(4,0)..N(4,1)+1
    assert s.band_levels(1, 2) == (0, int(s.N[3, 1]) + 1)
    assert s.band_levels(3, 1) == (int(s.N[2, 2]), s.nyv - 1)


def test_band_io_roundtrip():
    s = workload_setup("MB")
    f = initial_field_bands(s, 4)
    o = Oracle(s)
    o.set_bands(f)
    g = o.get_bands()
    for b in (1, 2, 3):
        for x, y in zip(f[b], g[b]):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("name", ["MB", "MBP"])
def test_multiblock_projection_and_flow_rate(name):
    s = workload_setup(name)
    o = Oracle(s)
    o.set_bands(initial_field_bands(s, 5))
    o.set_scalars(**initial_scalars(s))
    q0 = o.scalars()["QxT"]
    for _ in range(3):
        o.step()
        sc = o.scalars()
        assert sc["err"] < 1e-13                       # every band's columns divergence-free
        assert sc["Qx"] == pytest.approx(q0, rel=1e-13)  # constant flow rate
    st = o.get_bands()
    for b in (1, 3):                                   # short columns: v = 0 at both band ends
        assert np.abs(st[b][1][:, 0]).max() == 0 and np.abs(st[b][1][:, -1]).max() == 0
        assert np.isfinite(st[b][0]).all() and np.abs(st[b][0]).max() > 0


def test_single_resolution_band_layout_is_the_state_layout():
    s = workload_setup("S")
    st = initial_field(s, 6)
    a, b = Oracle(s), Oracle(s)
    a.set_state(*st)
    b.set_bands({2: st})
    for o in (a, b):
        o.set_scalars(**initial_scalars(s))
        o.step()
    x = a.get_state()
    y = b.get_bands()[2]
    for u, v in zip(x, y):
        assert np.array_equal(u, v)
