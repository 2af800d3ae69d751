"""Writer and reader of the reference's history file (hist_NNNNxNNNNxNNNN.dat).

Format (opened by start.f90:246-253, appended by record_out, FOU3D.f90:3064-3070): Fortran
unformatted sequential records with 4-byte little-endian length markers.

1. ``t, Re, alp, bet, mpgx`` (5 x real*8) and ``nband`` (int32), written when the file is
   created (a run that finds the file appends to it without a header);
2. ``N(4, 0:nband+1)`` int32, column-major;
3. one record per output step: ``flag_ctpress, iter`` (int32), then
   ``t, dtv, dtc, dt, err, Qx, QxT, mpgx, dgx, Umax, Uslip`` (real*8) when flag_ctpress == 0,
   ``t, dtv, dtc, dt, err, Qx, mpgx, Umax, Uslip`` when flag_ctpress == 1.

A record's values come from ``GpuChannel.history_record()`` (lh_history_record).
"""
from __future__ import annotations

import os
import struct

import numpy as np

from .planefile import _records
from .setup_grid import ChannelSetup

FIELDS_CT = ("t", "dtv", "dtc", "dt", "err", "Qx", "QxT", "mpgx", "dgx", "Umax", "Uslip")   # flag_ctpress 0
FIELDS_CP = ("t", "dtv", "dtc", "dt", "err", "Qx", "mpgx", "Umax", "Uslip")                 # flag_ctpress 1


def history_name(setup: ChannelSetup) -> str:
    """hist_<N(1,1)>x<N(2,1)>x<ny>.dat, the name start.f90 builds (the restart files' naming):
    the wall band's modes and ny = nn + 2 levels without the immersed region."""
    return f"hist_{setup.N1:04d}x{setup.N2:04d}x{setup.nn + 2:04d}.dat"


def _rec(b: bytes) -> bytes:
    n = struct.pack("<i", len(b))
    return n + b + n


def header_bytes(setup: ChannelSetup, t: float, mpgx: float, nband: int = 3) -> bytes:
    N = np.asarray(setup.N, dtype="<i4").T.copy()    # column-major N(4, 0:nband+1)
    return _rec(struct.pack("<5di", t, setup.p.Re, setup.p.alp, setup.p.bet, mpgx, nband)) + _rec(N.tobytes())


def record_bytes(rec: dict) -> bytes:
    fl = int(rec["flag_ctpress"])
    names = FIELDS_CT if fl == 0 else FIELDS_CP
    return _rec(struct.pack(f"<2i{len(names)}d", fl, int(rec["iter"]), *[float(rec[k]) for k in names]))


class HistoryFile:
    """Appends records to a history file; writes the two header records when the file is new
    (as start.f90 opens it: status 'new' with the header, or 'old' in append position)."""

    def __init__(self, path: str, setup: ChannelSetup, t: float, mpgx: float):
        self.path = path
        if not os.path.exists(path):
            with open(path, "wb") as f:
                f.write(header_bytes(setup, t, mpgx))

    def append(self, rec: dict) -> None:
        with open(self.path, "ab") as f:
            f.write(record_bytes(rec))
            f.flush()


def read_history(path: str):
    """(header dict, N (4, nband+2) int array, list of record dicts)."""
    with open(path, "rb") as f:
        recs = list(_records(f.read()))
    t, Re, alp, bet, mpgx, nband = struct.unpack("<5di", recs[0])
    N = np.frombuffer(recs[1], "<i4").reshape(nband + 2, 4).T.copy()
    out = []
    for r in recs[2:]:
        fl, it = struct.unpack_from("<2i", r, 0)
        names = FIELDS_CT if fl == 0 else FIELDS_CP
        vals = struct.unpack_from(f"<{len(names)}d", r, 8)
        d = dict(flag_ctpress=fl, iter=it, **dict(zip(names, vals)))
        out.append(d)
    return dict(t=t, Re=Re, alp=alp, bet=bet, mpgx=mpgx, nband=nband), N, out
