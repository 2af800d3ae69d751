"""Host side of the statistics output: folding of the accumulated spectra and the writers of
the reference's statistics files.

The device accumulates (``lh_stats_accumulate``); these functions do what the reference's
rank 0 does when it writes (``flagwr``):

- ``fold_spectrum``: recvwrspec (spectra.f90:124-182). sp(level, long column) -> buffSP
  (0:N1/2, 1:N2/2+1, level) of the core band's modes: x-mode i, z index folded onto
  |kz| + 1, the contributions of +kz and -kz added, then doubled for i >= 1 and kz
  index <= N2/2. The reference *assigns* rank 0's own columns before adding the other
  ranks', so on one rank the -kz column overwrites the +kz one; every multi-rank run whose
  rank 0 holds no column pair (+kz, -kz) adds them, which is what is done here.
- ``write_spectra_file`` (write_spect + recvwrspec), ``write_stats_file`` (write_stats,
  stats.f90:252-440), ``write_slip_file`` (write_sl_stats, sl_stats2.f90:124-199) and
  ``write_slip_inst_file`` (inst_sl_stats.f90:1-82): Fortran unformatted sequential records,
  4-byte little-endian markers, like the plane files.

The pressure sums P, P^2 and the tile-conditioned P and omega_x sums come from
``lh_stats_get_pw`` (argument ``pw`` of ``write_stats_file``): the reference sums ``ppPL``,
which holds the spectral packing of p from the last record_out (FOU3D.f90:156-157), and
conditions ``wx``, allocated (N1+2) x N2 per plane, through an igal x kgal dummy
(stats.f90:91-92, 100-101); these are the physical pressure and omega_x on the dealiased
grid instead. Without ``pw`` those records are zeros. The values on the wall and ghost planes
of the velocity statistics are zeros (the reference sums the untransformed spectral packing
there).
"""
from __future__ import annotations

import struct

import numpy as np

from .setup_grid import ChannelSetup

# order of the sums in lh_stats_get's plane array
PLANE_QTY = ("U", "U2", "W", "W2", "UV", "UW", "V", "V2", "VW", "wx", "wx2")
COND_QTY = ("U", "U2", "W", "W2", "UV", "UW", "V", "V2", "VW")


def _rec(b: bytes) -> bytes:
    return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))


def _header(s: ChannelSetup, t: float, mpgx: float, it: int) -> bytes:
    p = s.p
    return _rec(struct.pack("<5d2i", t, p.Re, p.alp, p.bet, mpgx, 3, it) + bytes(88 * 4))


def _i4(a) -> bytes:
    return np.ascontiguousarray(np.asarray(a).T, dtype="<i4").tobytes()


def _f8(*arrays) -> bytes:
    return np.concatenate([np.atleast_1d(np.asarray(a, np.float64)).ravel() for a in arrays]).astype("<f8").tobytes()


def _grids(s: ChannelSetup) -> list:
    return [_rec(_f8(s.yu, s.dthetai, s.dthdyu)), _rec(_f8(s.yv, s.dthetai, s.dthdyv))]


def fold_spectrum(s: ChannelSetup, sp: np.ndarray) -> np.ndarray:
    """sp [long column][level] (columns in columns_long_list order) -> buffSP as the file
    holds it: [level][N2c/2+1][N1c/2+1] (x-mode fastest)."""
    n1h, n2 = s.N1c // 2 + 1, s.N2c
    sp = np.asarray(sp, np.float64)
    nl = sp.shape[1]
    grid = sp.reshape(n2, n1h, nl)               # long columns: kz rows 0..N2c-1, kx fastest
    out = np.zeros((nl, n2 // 2 + 1, n1h))
    for r in range(n2):
        kk = r if r < n2 // 2 else n2 - r        # |kz| (0-based folded index)
        out[:, kk, :] += grid[r].T
    out[:, : n2 // 2, 1:] *= 2.0
    return out


def write_spectra_file(path: str, s: ChannelSetup, sp: np.ndarray, istat: int, t: float, mpgx: float,
                       it: int) -> None:
    out = [_header(s, t, mpgx, it), _rec(_i4(s.N))] + _grids(s)
    out.append(_rec(struct.pack("<i", int(istat))))
    out.append(_rec(np.ascontiguousarray(fold_spectrum(s, sp), "<f8").tobytes()))
    with open(path, "wb") as f:
        f.write(b"".join(out))


def write_stats_file(path: str, s: ChannelSetup, plane: np.ndarray, cond, istat: int, t: float, mpgx: float,
                     it: int, pw=None) -> None:
    """plane [11][nyu] and cond [9][ncl][dnz][dnx] (or None) as lh_stats_get returns them;
    pw = (pplane [2][nyu - 2], cond4 [4][ncl + 1][dnz][dnx] or None) as lh_stats_get_pw
    returns them, or None (P records zero)."""
    nu, nv, npl = s.nyu, s.nyv, s.nyu - 2
    q = {k: plane[i] for i, k in enumerate(PLANE_QTY)}
    pp, c4 = pw if pw is not None else (np.zeros((2, npl)), None)
    recs = [q["U"][:nu], q["U2"][:nu], q["V"][:nv], q["V2"][:nv], q["W"][:nu], q["W2"][:nu], pp[0][:npl],
            pp[1][:npl], q["UV"][:nu], q["UW"][:nu], q["VW"][:nv], q["wx"][:nv], q["wx2"][:nv]]
    out = [_header(s, t, mpgx, it), _rec(_i4(s.Ngal))] + _grids(s)
    out.append(_rec(struct.pack("<i", int(istat))))
    out += [_rec(_f8(r)) for r in recs]
    if cond is not None:
        # xC(dnx, dnz, 0:Ny(grid,1)-Ny(grid,0)): level 0 is the wall/ghost plane
        n4, n3 = s.N[3], s.N[2]
        ncu, ncv, ncp = int(n4[1] - n4[0]) + 1, int(n3[1] - n3[0]) + 1, int(n4[1] - n4[0]) - 1
        c = {k: cond[i] for i, k in enumerate(COND_QTY)}
        dnz, dnx = cond.shape[2], cond.shape[3]

        def lv(a, n):
            o = np.zeros((n, dnz, dnx))
            m = min(n - 1, a.shape[0])
            o[1:1 + m] = a[:m]
            return o

        def lv0(qty, n):
            # conditioned P / omega_x: level j1 = 0 .. n - 1 from the wall, level 0 included
            o = np.zeros((n, dnz, dnx))
            if c4 is not None:
                m = min(n, c4.shape[1])
                o[:m] = c4[qty, :m]
            return o

        crecs = [lv(c["U"], ncu), lv(c["U2"], ncu), lv(c["V"], ncv), lv(c["V2"], ncv), lv(c["W"], ncu),
                 lv(c["W2"], ncu), lv0(0, ncp), lv0(1, ncp), lv(c["UV"], ncu), lv(c["UW"], ncu), lv(c["VW"], ncv),
                 lv0(2, ncv), lv0(3, ncv)]
        out += [_rec(np.ascontiguousarray(r, "<f8").tobytes()) for r in crecs]
    with open(path, "wb") as f:
        f.write(b"".join(out))


def _slip_plane(a: np.ndarray) -> bytes:
    """complex [N2][N1/2+1] -> real (N1+2, N2) column-major (re/im of each x-mode)"""
    n2, nh = a.shape
    buf = np.empty((n2, 2 * nh), "<f8")
    buf[:, 0::2] = a.real
    buf[:, 1::2] = a.imag
    return buf.tobytes()


def write_slip_file(path: str, s: ChannelSetup, slip: np.ndarray, istat: int, t: float, mpgx: float,
                    it: int) -> None:
    """slip [2 walls][4][N2][N1/2+1] accumulated: the file holds bottom + top of u1_itp,
    du1dy, u3_itp, du3dy (recvbreal adds the top rank's arrays to rank 0's)."""
    out = [_header(s, t, mpgx, it), _rec(_i4(s.N)), _rec(struct.pack("<i", int(istat)))]
    out += [_rec(_slip_plane(slip[0, f] + slip[1, f])) for f in range(4)]
    with open(path, "wb") as f:
        f.write(b"".join(out))


def write_slip_inst_file(path: str, s: ChannelSetup, planes: np.ndarray, t: float, mpgx: float,
                         it: int) -> None:
    """instantaneous planes [2][4][N2][N1/2+1]: per quantity the bottom then the top plane"""
    out = [_header(s, t, mpgx, it), _rec(_i4(s.N))]
    for f in range(4):
        out += [_rec(_slip_plane(planes[0, f])), _rec(_slip_plane(planes[1, f]))]
    with open(path, "wb") as f:
        f.write(b"".join(out))


def read_records(path: str) -> list:
    """The records of a Fortran unformatted sequential file (bytes each)."""
    with open(path, "rb") as f:
        raw = f.read()
    recs, off = [], 0
    while off < len(raw):
        (n,) = struct.unpack_from("<i", raw, off)
        recs.append(raw[off + 4: off + 4 + n])
        (n2,) = struct.unpack_from("<i", raw, off + 4 + n)
        if n2 != n:
            raise ValueError("corrupt record markers")
        off += 8 + n
    return recs
