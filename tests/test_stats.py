"""Statistics of stats.f90 on the CPU oracle: the tile-conditioned sums (conddown/condup)
add up, over a tile, to the plane sums of the bottom level plus the mirrored top level
(V with its sign flipped), and the mean profile is the laminar profile's. The pressure sums
are those of the physical pressure (a NumPy inverse transform of the state's p on the
dealiased grid), and its conditioned sums and those of omega_x tile the planes too."""
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


def physical(s, modes):
    """[ncol] modes of one level (kz row-major, N1/2+1 x-modes) -> the G2 x G1 physical plane:
    the spectrum zero-padded onto the dealiased grid, the inverse transforms unnormalised"""
    n1h = s.N1 // 2 + 1
    a = np.asarray(modes).reshape(s.N2, n1h)
    pad = np.zeros((s.G2, s.G1 // 2 + 1), np.complex128)
    pad[: s.N2 // 2, :n1h] = a[: s.N2 // 2]
    pad[s.G2 - s.N2 // 2:, :n1h] = a[s.N2 // 2:]
    return np.fft.irfft2(pad, s=(s.G2, s.G1), norm="forward")


def test_pressure_sums_are_the_physical_pressures():
    s = workload_setup("SP")
    o = Oracle(s)
    o.set_state(*initial_field(s, 3))
    o.set_scalars(**initial_scalars(s))
    o.step()
    o.stats_accumulate()
    pp, c4 = o.stats_pw()
    p = o.get_state()[3]
    assert pp.shape == (2, s.nyu - 2) == (2, p.shape[1])
    f = np.stack([physical(s, p[:, q]) for q in range(p.shape[1])])
    s1, s2 = f.sum(axis=(1, 2)), (f * f).sum(axis=(1, 2))
    assert np.abs(pp[0] - s1).max() <= 1e-12 * np.abs(s1).max()
    assert np.abs(pp[1] - s2).max() <= 1e-12 * np.abs(s2).max()
    # conditioned P: a bottom plane and its mirror at the top, summed per tile position
    dnz, dnx = c4.shape[2:]
    n4 = s.N[3]
    for j1 in (0, 3):
        qb, qt = j1, p.shape[1] - 1 - j1       # p levels N(4,0)+1+j1 and N(4,3)-j1
        both = (f[qb], f[qt])
        ref = sum(x.reshape(s.G2 // dnz, dnz, s.G1 // dnx, dnx).sum(axis=(0, 2)) for x in both)
        ref2 = sum((x * x).reshape(s.G2 // dnz, dnz, s.G1 // dnx, dnx).sum(axis=(0, 2)) for x in both)
        assert np.abs(c4[0, j1] - ref).max() <= 1e-12 * np.abs(ref).max()
        assert np.abs(c4[1, j1] - ref2).max() <= 1e-12 * np.abs(ref2).max()
    assert int(n4[1] - n4[0] - 1) <= c4.shape[1]


def test_conditioned_omega_x_tiles_the_planes():
    """omega_x conditioned on the dealiased grid: per level, the sum over the tile positions
    is the plane mean on the padded grid, (G1 G2 / N1 N2) x the unpadded plane sum of
    stats.f90, bottom plane plus mirrored top plane (xsign 1)"""
    s = workload_setup("SP")
    o = Oracle(s)
    o.set_state(*initial_field(s, 3))
    o.set_scalars(**initial_scalars(s))
    o.step()
    o.stats_accumulate()
    pl, _, _ = o.stats()
    pp, c4 = o.stats_pw()
    n3 = s.N[2]
    ratio = s.G1 * s.G2 / (s.N1 * s.N2)
    scale = ratio * np.abs(pl[9]).max()
    for j1 in range(int(n3[1] - n3[0]) + 1):
        qb, qt = int(n3[0] + j1 + s.dny), int(n3[3] + 1 - j1 + s.dny)
        assert abs(c4[2, j1].sum() - ratio * (pl[9, qb] + pl[9, qt])) <= 1e-12 * scale
    assert (c4[3] >= 0).all() and c4[3].max() > 0
