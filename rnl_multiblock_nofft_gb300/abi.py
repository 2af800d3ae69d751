"""ctypes mirror of include/lh.h (`lh_config`, `lh_scalars`) and the packing of a
ChannelSetup into an `lh_config`."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .setup_grid import UGRID, VGRID, ChannelSetup

LH_ABI_VERSION = 2
LH_OK, LH_EINVAL, LH_ENONFINITE, LH_ETIMEOUT, LH_ECUDA, LH_ENOMEM = 0, -1, -2, -3, -4, -5
LH_PREC_FP64, LH_PREC_MIXED = 0, 1
LH_NONLIN_PRODUCTS, LH_NONLIN_TRIADS = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_bp = C.POINTER(C.c_int8)


class LhConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("precision", C.c_int32),
        ("N1", C.c_int32), ("N2", C.c_int32), ("Ngal1", C.c_int32), ("Ngal2", C.c_int32),
        ("dny", C.c_int32), ("nn", C.c_int32),
        ("N3", C.c_int32 * 4), ("N4", C.c_int32 * 4),
        ("nyu", C.c_int32), ("nyv", C.c_int32),
        ("yu", _dp), ("yv", _dp), ("dthdyu", _dp), ("dthdyv", _dp),
        ("dyu2i", _dp), ("dyv2i", _dp), ("k1x", _dp), ("k2x", _dp), ("k1z", _dp), ("k2z", _dp),
        ("Re", C.c_double), ("CFL", C.c_double), ("dtv", C.c_double), ("ddthetavi", C.c_double),
        ("dthetavi", C.c_double), ("alp", C.c_double), ("bet", C.c_double), ("Kib", C.c_double),
        ("aRK", C.c_double * 3), ("bRK", C.c_double * 3), ("cRK", C.c_double * 3),
        ("dRK", C.c_double * 3), ("gRK", C.c_double * 3),
        ("gw", (C.c_double * 2) * 3), ("gw_interp", (C.c_double * 2) * 3),
        ("gw_bc_u1", C.c_double), ("gw_bc_u3", C.c_double),
        ("flag_ctpress", C.c_int32), ("ib_enable", C.c_int32),
        ("nib_u", C.c_int32), ("nib_v", C.c_int32),
        ("list_ib_u", _ip), ("list_ib_v", _ip), ("A_ib_u", _dp), ("A_ib_v", _dp),
        ("nonlin_form", C.c_int32), ("triad_nx", C.c_int32), ("triad_nz", C.c_int32),
        ("triad_nsets", C.c_int32), ("triad_off", _lp), ("triad_len", _lp), ("triad_data", _bp),
        ("triad_set_u", _ip), ("triad_set_v", _ip),
        ("N1c", C.c_int32), ("N2c", C.c_int32), ("Ngal1c", C.c_int32), ("Ngal2c", C.c_int32),
        ("ntilex", C.c_int32), ("ntilez", C.c_int32),
    ]


class LhScalars(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("dti", C.c_double), ("dtc", C.c_double),
                ("err", C.c_double), ("mpgx", C.c_double), ("QxT", C.c_double), ("Qx", C.c_double),
                ("iter", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class LhHistory(C.Structure):
    _fields_ = [("flag_ctpress", C.c_int32), ("iter", C.c_int32),
                ("t", C.c_double), ("dtv", C.c_double), ("dtc", C.c_double), ("dt", C.c_double),
                ("err", C.c_double), ("Qx", C.c_double), ("QxT", C.c_double), ("mpgx", C.c_double),
                ("dgx", C.c_double), ("Umax", C.c_double), ("Uslip", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


def _ptr(a: np.ndarray, typ):
    return a.ctypes.data_as(typ)


def make_config(s: ChannelSetup, precision: int = LH_PREC_FP64, triads=None):
    """Returns (LhConfig, keepalive) for a channel (single-resolution or multiblock).
    `triads` (a triads.TriadLists) selects the triad-list nonlinear form; None the
    FFT products."""
    keep = []

    def d(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return _ptr(a, _dp)

    def i32(a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        keep.append(a)
        return _ptr(a, _ip)

    c = LhConfig()
    c.abi_version = LH_ABI_VERSION
    c.precision = precision
    c.N1, c.N2 = s.N1, s.N2
    c.Ngal1, c.Ngal2 = s.G1, s.G2
    c.N1c, c.N2c, c.Ngal1c, c.Ngal2c = s.N1c, s.N2c, s.G1c, s.G2c
    if p_has_tiles(s):
        c.ntilex, c.ntilez = int(s.p.ntilex), int(s.p.ntilez)
    c.dny, c.nn = s.dny, s.nn
    for b in range(4):
        c.N3[b] = int(s.N[2, b])
        c.N4[b] = int(s.N[3, b])
    c.nyu, c.nyv = s.nyu, s.nyv
    c.yu, c.yv, c.dthdyu, c.dthdyv = d(s.yu), d(s.yv), d(s.dthdyu), d(s.dthdyv)
    c.dyu2i, c.dyv2i = d(s.dyu2i), d(s.dyv2i)
    c.k1x, c.k2x, c.k1z, c.k2z = d(s.k1x), d(s.k2x), d(s.k1z), d(s.k2z)
    p = s.p
    c.Re, c.CFL, c.dtv = p.Re, p.CFL, s.dtv
    c.ddthetavi = s.ddthetavi
    c.dthetavi = 0.0   # never assigned in the reference (declaration.f90:76); see dtc_calc
    c.alp, c.bet, c.Kib = p.alp, p.bet, p.Kib
    for k in range(3):
        c.aRK[k], c.bRK[k], c.cRK[k] = s.aRK[k], s.bRK[k], s.cRK[k]
        c.dRK[k], c.gRK[k] = s.dRK[k], s.gRK[k]
    for b in range(3):
        for e in range(2):
            c.gw[b][e] = s.gw[b, e]
            c.gw_interp[b][e] = s.gw_interp[b, e]
    c.gw_bc_u1, c.gw_bc_u3 = s.gw_bc_u1, s.gw_bc_u3
    c.flag_ctpress = p.flpress
    c.ib_enable = int(bool(p.ib_enable) and p.geometry_type == 2 and s.dny > 0)
    lu, lv = s.list_ib[UGRID], s.list_ib[VGRID]
    c.nib_u, c.nib_v = len(lu), len(lv)
    c.list_ib_u = i32(lu.reshape(-1) if len(lu) else np.zeros(6, np.int32))
    c.list_ib_v = i32(lv.reshape(-1) if len(lv) else np.zeros(6, np.int32))
    c.A_ib_u = d(s.A_ib[UGRID] if len(lu) else np.zeros(1))
    c.A_ib_v = d(s.A_ib[VGRID] if len(lv) else np.zeros(1))
    c.nonlin_form = LH_NONLIN_PRODUCTS
    if triads is not None:
        pk = triads.pack(s)
        c.nonlin_form = LH_NONLIN_TRIADS
        c.triad_nx, c.triad_nz = pk["nx"], pk["nz"]
        c.triad_nsets = len(pk["off"])
        for name, typ in (("off", _lp), ("len", _lp), ("data", _bp)):
            keep.append(pk[name])
        c.triad_off = _ptr(pk["off"], _lp)
        c.triad_len = _ptr(pk["len"], _lp)
        c.triad_data = _ptr(pk["data"], _bp)
        c.triad_set_u = i32(pk["set_u"])
        c.triad_set_v = i32(pk["set_v"])
    return c, keep


def p_has_tiles(s: ChannelSetup) -> bool:
    p = s.p
    return p.geometry_type == 2 and p.ntilex > 0 and p.ntilez > 0 and s.G1 % p.ntilex == 0 and s.G2 % p.ntilez == 0


def cfield_shape(s: ChannelSetup):
    """Host cfield shapes (ncols, nlevels) of u1, u2, u3, p (single-resolution
    channels; multiblock channels use ChannelSetup.band_shapes)."""
    return ((s.ncols, s.nyu), (s.ncols, s.nyv), (s.ncols, s.nyu), (s.ncols, s.nyu - 2))
