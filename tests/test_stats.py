"""Statistics of stats.f90 on the CPU oracle: the tile-conditioned sums (conddown/condup)
add up, over a tile, to the plane sums of the bottom level plus the mirrored top level
(V with its sign flipped), and the mean profile is the laminar profile's."""
import numpy as np

from oracle import Oracle
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup


def test_conditioned_sums_tile_the_planes():
    s = workload_setup("SP")
    o = Oracle(s)
    o.set_state(*initial_field(s, 3))
    o.set_scalars(**initial_scalars(s))
    o.step()
    o.stats_accumulate()
    pl, cd, ist = o.stats()
    assert ist == 1 and cd is not None
    nu, nv = s.nyu, s.nyv
    assert cd.shape[2:] == (s.G2 // s.p.ntilez, s.G1 // s.p.ntilex)
    n4, n3 = s.N[3], s.N[2]
    for j1 in range(1, int(n4[1] - n4[0]) + 1):
        for qty in (0, 1, 2, 3, 5):                   # U, U^2, W, W^2, UW
            top = pl[qty, nu - 1 - j1] if j1 <= n4[3] - n4[2] else 0.0
            ref = pl[qty, j1] + top
            assert abs(cd[qty, j1 - 1].sum() - ref) <= 1e-12 * max(1.0, abs(ref))
        top = pl[4, nu - 1 - j1] if j1 <= n4[3] - n4[2] else 0.0  # UV: V mirrored
        assert abs(cd[4, j1 - 1].sum() - (pl[4, j1] - top)) <= 1e-12 * max(1.0, abs(pl[4, j1]))
    for j1 in range(1, int(n3[1] - n3[0]) + 1):
        top = pl[6, nv - 1 - j1] if j1 <= n3[3] - n3[2] else 0.0
        assert abs(cd[6, j1 - 1].sum() - (pl[6, j1] - top)) <= 1e-12 * max(1.0, abs(pl[6, j1]))


def test_mean_profile():
    s = workload_setup("C0")
    o = Oracle(s)
    st = initial_field(s, 5)
    o.set_state(*st)
    o.set_scalars(**initial_scalars(s))
    o.stats_accumulate()
    pl, cd, ist = o.stats()
    assert cd is None
    pp = s.G1 * s.G2
    # the plane mean of u is its (0,0) mode
    assert np.allclose(pl[0, 1:-1] / pp, st[0][0, 1:-1].real, rtol=1e-12, atol=1e-14)
