"""Reader and writer of the reference's plane files (u1/u2/u3/p_NNNNxNNNNxNNNN_tTTTTT.dat).

Format (FOU3D.f90:2856-3073 `record_out`, start.f90:2444-2882 `read_in`): Fortran
unformatted sequential records with 4-byte little-endian length markers.

1. ``t, Re, alp, bet, mpgx`` (5 x real*8), ``nband, iter`` (2 x int32), 88 x int32 zeros
2. ``N(4, 0:nband+1)`` int32, column-major
3. ``y, dthetavi, dthdy`` of the field's grid (u/p: yu, v: yv)
4. one record per y-level: ``j, field_id, nx, nz`` (int32), ``y(j)`` (real*8), then the
   spectral plane ``buff(nx, nz)`` real*8 with nx = N1+2 (re/im of the kx-modes
   0..N1/2) and nz = N2 in the column ordering of k1F_z (`u_to_buff`, FOU3D.f90:3134-3163).

u and w carry levels N(4,0)..N(4,3)+1, v levels N(3,0)..N(3,3)+1, p levels
N(4,0)+1..N(4,3). Here a field is returned as a complex array ``[level, kz, kx]``.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np


@dataclass
class PlaneFile:
    t: float
    Re: float
    alp: float
    bet: float
    mpgx: float
    nband: int
    iter: int
    N: np.ndarray          # (4, nband+2)
    y: np.ndarray
    dthetavi: float
    dthdy: np.ndarray
    levels: np.ndarray     # reference level index j of each plane
    field_id: int
    data: np.ndarray       # complex128 [nlevels, N2, N1/2+1]


def _records(raw: bytes):
    off = 0
    while off < len(raw):
        (n,) = struct.unpack_from("<i", raw, off)
        yield raw[off + 4: off + 4 + n]
        (n2,) = struct.unpack_from("<i", raw, off + 4 + n)
        if n2 != n:
            raise ValueError("corrupt record markers")
        off += 8 + n


def read_planefile(path: str) -> PlaneFile:
    with open(path, "rb") as f:
        raw = f.read()
    recs = list(_records(raw))
    t, Re, alp, bet, mpgx = struct.unpack_from("<5d", recs[0], 0)
    nband, it = struct.unpack_from("<2i", recs[0], 40)
    N = np.frombuffer(recs[1], "<i4").reshape(nband + 2, 4).T.copy()
    hdr = np.frombuffer(recs[2], "<f8")
    ny = (hdr.size - 1) // 2
    y, dthetavi, dthdy = hdr[:ny].copy(), float(hdr[ny]), hdr[ny + 1:].copy()
    levels, planes, fid = [], [], None
    for r in recs[3:]:
        j, fid, nx, nz = struct.unpack_from("<4i", r, 0)
        buf = np.frombuffer(r, "<f8", offset=24).reshape(nz, nx)
        levels.append(j)
        planes.append(buf[:, 0::2] + 1j * buf[:, 1::2])
    return PlaneFile(t, Re, alp, bet, mpgx, nband, it, N, y, dthetavi, dthdy,
                     np.array(levels), fid, np.stack(planes))


def write_planefile(path: str, pf: PlaneFile) -> None:
    def rec(b: bytes) -> bytes:
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))

    out = [rec(struct.pack("<5d2i", pf.t, pf.Re, pf.alp, pf.bet, pf.mpgx, pf.nband, pf.iter)
               + bytes(88 * 4))]
    out.append(rec(np.ascontiguousarray(pf.N.T, dtype="<i4").tobytes()))
    out.append(rec(np.concatenate([pf.y, [pf.dthetavi], pf.dthdy]).astype("<f8").tobytes()))
    for lev, plane in zip(pf.levels, pf.data):
        nz, nh = plane.shape
        buf = np.empty((nz, 2 * nh), "<f8")
        buf[:, 0::2] = plane.real
        buf[:, 1::2] = plane.imag
        yj = pf.y[int(lev) - int(pf.levels[0])] if pf.y.size >= len(pf.levels) else 0.0
        out.append(rec(struct.pack("<4id", int(lev), pf.field_id, 2 * nh, nz, yj) + buf.tobytes()))
    with open(path, "wb") as f:
        f.write(b"".join(out))
