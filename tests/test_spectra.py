"""The remaining statistics of the statistics step on the CPU oracle, each against a NumPy
restatement from the state: spectra (spectra.f90), the omega_x plane sums (FOU3D.f90:300-327
+ stats.f90:56-63, inverse transform on the unpadded grid), the slip statistics at the wall
faces (sl_stats2.f90, inst_sl_stats.f90); and the host-side folding and file writers."""
import struct

import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.setup_grid import PGRID, UGRID, VGRID
from rnl_multiblock_nofft_gb300.statsfile import (fold_spectrum, read_records, write_slip_file,
                                                  write_spectra_file, write_stats_file)
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup


def oracle_twice(name, seed):
    """statistics accumulated before and after one step; the two states"""
    s = workload_setup(name)
    o = Oracle(s)
    o.set_state(*initial_field(s, seed))
    o.set_scalars(**initial_scalars(s))
    states = [o.get_state()]
    o.stats_accumulate()
    o.step()
    states.append(o.get_state())
    o.stats_accumulate()
    return s, o, states


def u2_itp(s, u2):
    """interp_v of the long columns over band 2's u levels (FOU3D.f90:427-474), [col][level]"""
    lo, hi = s.band_levels(2, UGRID)
    vlo, vhi = s.band_levels(2, VGRID)
    yu, yv = s.yu, s.yv
    out = np.zeros((u2.shape[0], hi - lo + 1), complex)
    for q in range(lo + 1, hi):
        out[:, q - lo] = ((yu[q] - yv[q - 1]) * u2[:, q] + (yv[q] - yu[q]) * u2[:, q - 1]) / (yv[q] - yv[q - 1])
    g0, g1 = s.gw_interp[1]
    i1, i2 = out[:, 1], out[:, hi - lo - 1]
    out[:, 0] = g0 * (u2[:, vlo] - i1) + i1
    out[:, hi - lo] = g1 * (u2[:, vhi] - i2) + i2
    return out


@pytest.mark.parametrize("name", ["C0", "SP"])
def test_spectra_sums(name):
    s, o, states = oracle_twice(name, 61)
    sp = o.spectra()
    lo, hi = s.band_levels(2, UGRID)
    vlo, vhi = s.band_levels(2, VGRID)
    plo, phi = s.band_levels(2, PGRID)
    ref = {k: 0.0 for k in sp}
    for u1, u2, u3, p in states:
        ref["U"] = ref["U"] + np.abs(u1[:, lo:hi + 1]) ** 2
        ref["W"] = ref["W"] + np.abs(u3[:, lo:hi + 1]) ** 2
        ref["V"] = ref["V"] + np.abs(u2[:, vlo:vhi + 1]) ** 2
        ref["P"] = ref["P"] + np.abs(p[:, plo - 1:phi]) ** 2
        v = u2_itp(s, u2)
        ref["UV"] = ref["UV"] + (u1[:, lo:hi + 1].real * v.real + u1[:, lo:hi + 1].imag * v.imag)
    for k in sp:
        assert sp[k].shape == ref[k].shape, k
        scale = np.abs(ref[k]).max()
        assert np.abs(sp[k] - ref[k]).max() <= 1e-13 * scale, k


def test_wx_plane_sums():
    s, o, states = oracle_twice("SP", 62)
    pl, _, ist = o.stats()
    assert ist == 2 and pl.shape[0] == 11
    n1, n2, n1h = s.N1, s.N2, s.N1 // 2 + 1
    kz = s.k1z.reshape(n2, 1)
    fy = s.dthdyv * s.ddthetavi
    ref_s, ref_s2 = np.zeros(s.nyv), np.zeros(s.nyv)
    for u1, u2, u3, p in states:
        for q in range(s.nyv):
            v = u2[:, q].reshape(n2, n1h)
            dw = (u3[:, q + 1] - u3[:, q]).reshape(n2, n1h) * fy[q]
            c = -(1j * kz) * v + dw
            a = np.fft.ifft(c, axis=0) * n2                 # z backward, unnormalised
            f = np.fft.irfft(a, n=n1, axis=1) * n1          # x backward real (Im of 0, N1/2 dropped)
            ref_s[q] += f.sum()
            ref_s2[q] += (f * f).sum()
    scale = ref_s2.max()
    assert np.abs(pl[10, : s.nyv] - ref_s2).max() <= 1e-12 * scale
    # the plane sum of omega_x is N1 N2 Re of its (0,0) mode: compare on the rms scale
    assert np.abs(pl[9, : s.nyv] - ref_s).max() <= 1e-12 * np.sqrt(scale * n1 * n2)


def test_slip_statistics():
    s, o, states = oracle_twice("C0", 63)
    acc = o.slip()
    inst = o.slip_planes()                                 # the state after the step
    n2, n1h = s.N2, s.N1 // 2 + 1
    jb, jt = s.band_levels(2, VGRID)
    fy = s.dthdyv * s.ddthetavi
    ref = np.zeros_like(acc)
    for u1, u2, u3, p in states:
        one = np.zeros_like(acc)
        for w, (q, sg) in enumerate(((jb, 1.0), (jt, -1.0))):
            yv, ya, yb = s.yv[q], s.yu[q], s.yu[q + 1]
            for f, u in ((0, u1), (2, u3)):
                one[w, f] = (((yv - ya) * u[:, q + 1] + (yb - yv) * u[:, q]) / (yb - ya)).reshape(n2, n1h)
                one[w, f + 1] = (sg * ((u[:, q + 1] - u[:, q]) * fy[q])).reshape(n2, n1h)
        ref += one
    scale = np.abs(ref).max()
    assert np.abs(acc - ref).max() <= 1e-13 * scale
    assert np.abs(inst - one).max() <= 1e-13 * scale


def test_fold_spectrum():
    s = workload_setup("S")
    n1h, n2 = s.N1c // 2 + 1, s.N2c
    rng = np.random.default_rng(5)
    sp = rng.random((n1h * n2, 3))
    b = fold_spectrum(s, sp)
    g = sp.reshape(n2, n1h, 3)
    assert b.shape == (3, n2 // 2 + 1, n1h)
    assert np.allclose(b[:, 0, 0], g[0, 0])                         # (0, 0): not doubled
    assert np.allclose(b[:, 0, 1:], 2 * g[0, 1:].T)                 # kz = 0: no partner row
    assert np.allclose(b[:, 3, 2], 2 * (g[3, 2] + g[n2 - 3, 2]))    # +kz and -kz, doubled
    assert np.allclose(b[:, n2 // 2, 2], g[n2 // 2, 2])             # |kz| = N2/2: one row, not doubled
    assert np.allclose(b[:, 3, 0], g[3, 0] + g[n2 - 3, 0])          # x-mode 0 not doubled


def test_files_roundtrip(tmp_path):
    s, o, _ = oracle_twice("SP", 64)
    pl, cd, ist = o.stats()
    sp = o.spectra()
    p = str(tmp_path / "spU.dat")
    write_spectra_file(p, s, sp["U"], ist, 0.5, -3e-3, 7)
    r = read_records(p)
    t, Re, alp, bet, mpgx = struct.unpack_from("<5d", r[0])
    assert (t, mpgx) == (0.5, -3e-3) and struct.unpack_from("<2i", r[0], 40) == (3, 7)
    assert np.array_equal(np.frombuffer(r[1], "<i4").reshape(5, 4).T, s.N)
    assert struct.unpack("<i", r[4])[0] == ist
    b = np.frombuffer(r[5], "<f8").reshape(-1, s.N2c // 2 + 1, s.N1c // 2 + 1)
    assert np.array_equal(b, fold_spectrum(s, sp["U"]))
    p = str(tmp_path / "stats.dat")
    write_stats_file(p, s, pl, cd, ist, 0.5, -3e-3, 7)
    r = read_records(p)
    assert len(r) == 5 + 13 + (13 if cd is not None else 0)
    assert np.array_equal(np.frombuffer(r[5], "<f8"), pl[0, : s.nyu])
    assert np.array_equal(np.frombuffer(r[16], "<f8"), pl[9, : s.nyv])
    assert not np.frombuffer(r[11], "<f8").any()                       # P without pw
    pp, c4 = o.stats_pw()
    write_stats_file(p, s, pl, cd, ist, 0.5, -3e-3, 7, pw=(pp, c4))
    r = read_records(p)
    assert np.array_equal(np.frombuffer(r[11], "<f8"), pp[0]) and np.array_equal(np.frombuffer(r[12], "<f8"), pp[1])
    if cd is not None:
        dnz, dnx = cd.shape[2:]
        n4, n3 = s.N[3], s.N[2]
        ncp, ncv = int(n4[1] - n4[0]) - 1, int(n3[1] - n3[0]) + 1
        assert np.array_equal(np.frombuffer(r[24], "<f8").reshape(ncp, dnz, dnx), c4[0, :ncp])
        assert np.array_equal(np.frombuffer(r[29], "<f8").reshape(ncv, dnz, dnx), c4[2, :ncv])
    p = str(tmp_path / "sl.dat")
    acc = o.slip()
    write_slip_file(p, s, acc, ist, 0.5, -3e-3, 7)
    r = read_records(p)
    x = np.frombuffer(r[3], "<f8").reshape(s.N2, s.N1 + 2)
    assert np.array_equal(x[:, 0::2] + 1j * x[:, 1::2], acc[0, 0] + acc[1, 0])
