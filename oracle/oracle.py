"""ctypes wrapper of the CPU oracle (liblh_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from rnl_multiblock_nofft_gb300.abi import LhScalars, cfield_shape, make_config
from rnl_multiblock_nofft_gb300.setup_grid import ChannelSetup

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liblh_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "lh_oracle.c")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "liblh_oracle.so"],
                       check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp]
        L.orc_destroy.argtypes = [vp]
        for f in ("orc_set_band", "orc_get_band"):
            getattr(L, f).argtypes = [vp, C.c_int] + [dp] * 4
        for f in ("orc_set_state", "orc_get_state", "orc_get_nonlinear"):
            getattr(L, f).argtypes = [vp] + [dp] * (4 if f != "orc_get_nonlinear" else 3)
        L.orc_set_scalars.argtypes = [vp, vp]
        L.orc_get_scalars.argtypes = [vp, vp]
        L.orc_substep.argtypes = [vp, C.c_int]
        L.orc_step.argtypes = [vp]
        L.orc_four_to_phys.argtypes = [vp, dp, dp, C.c_int]
        L.orc_phys_to_four.argtypes = [vp, dp, dp, C.c_int]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_transform_noise.argtypes = [C.c_double]
        L.orc_stats_accumulate.argtypes = [vp]
        L.orc_stats_get.argtypes = [vp, dp, dp, C.POINTER(C.c_int64), C.POINTER(C.c_int)]
        L.orc_stats_reset.argtypes = [vp]
        L.orc_stats_get_pw.argtypes = [vp, dp, dp]
        L.orc_spectra_get.argtypes = [vp] + [dp] * 5 + [C.POINTER(C.c_int)] * 2
        L.orc_slip_get.argtypes = [vp, dp]
        L.orc_slip_planes.argtypes = [vp, dp]
        _lib = L
    return _lib


def set_transform_noise(eps: float) -> None:
    """Test hook of the oracle: noise of amplitude eps x (the line's largest modulus) on every
    transform output, process-wide (0 turns it off)."""
    lib().orc_set_transform_noise(float(eps))


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class Oracle:
    """One channel on the CPU oracle. State arrays use the host cfield layout
    (complex128 [ncols, nlevels])."""

    def __init__(self, setup: ChannelSetup, threads: int = 0, triads=None):
        """`triads` (a TriadLists) selects the triad-list nonlinear term."""
        self.s = setup
        L = lib()
        if threads:
            L.orc_set_threads(threads)
        cfg, self._keep = make_config(setup, triads=triads)
        self._cfg = cfg
        self.h = L.orc_create(C.byref(cfg))
        if not self.h:
            raise RuntimeError("orc_create failed")
        self.shapes = cfield_shape(setup)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    __del__ = close

    def set_state(self, u1, u2, u3, p):
        arrs = [np.ascontiguousarray(a, np.complex128) if a is not None else None for a in (u1, u2, u3, p)]
        for a, sh in zip(arrs, self.shapes):
            if a is not None and a.shape != sh:
                raise ValueError(f"shape {a.shape} != {sh}")
        lib().orc_set_state(self.h, *[_dptr(a) for a in arrs])

    def set_bands(self, bands: dict):
        """{band: (u1, u2, u3, p)} in the bands' cfield layouts (ChannelSetup.band_shapes)."""
        for b, arrs in bands.items():
            arrs = [np.ascontiguousarray(a, np.complex128) for a in arrs]
            for a, sh in zip(arrs, self.s.band_shapes(b)):
                if a.shape != sh:
                    raise ValueError(f"band {b}: shape {a.shape} != {sh}")
            if lib().orc_set_band(self.h, b, *[_dptr(a) for a in arrs]) != 0:
                raise ValueError("orc_set_band failed")

    def get_bands(self) -> dict:
        out = {}
        for b in (1, 2, 3):
            arrs = [np.zeros(sh, np.complex128) for sh in self.s.band_shapes(b)]
            lib().orc_get_band(self.h, b, *[_dptr(a) for a in arrs])
            out[b] = arrs
        return out

    def get_state(self):
        out = [np.zeros(sh, np.complex128) for sh in self.shapes]
        lib().orc_get_state(self.h, *[_dptr(a) for a in out])
        return out

    def get_nonlinear(self):
        sh = (self.shapes[0], self.shapes[1], self.shapes[2])
        out = [np.zeros(x, np.complex128) for x in sh]
        lib().orc_get_nonlinear(self.h, *[_dptr(a) for a in out])
        return out

    def set_scalars(self, **kw):
        s = LhScalars()
        for k, v in kw.items():
            setattr(s, k, v)
        lib().orc_set_scalars(self.h, C.byref(s))

    def scalars(self) -> dict:
        s = LhScalars()
        lib().orc_get_scalars(self.h, C.byref(s))
        return s.as_dict()

    def substep(self, kRK: int):
        if lib().orc_substep(self.h, kRK) != 0:
            raise RuntimeError("orc_substep failed")

    def step(self, n: int = 1):
        for _ in range(n):
            if lib().orc_step(self.h) != 0:
                raise RuntimeError("orc_step failed")

    def stats_accumulate(self):
        lib().orc_stats_accumulate(self.h)

    def stats_reset(self):
        lib().orc_stats_reset(self.h)

    def spectra(self) -> dict:
        """Accumulated sp(level, long column) of spectra.f90, as {"U", "V", "W", "UV", "P"}:
        arrays [long column][level of band 2]."""
        nl = (C.c_int * 5)()
        nlong = C.c_int()
        lib().orc_spectra_get(self.h, None, None, None, None, None, nl, C.byref(nlong))
        out = {k: np.zeros((nlong.value, nl[q])) for q, k in enumerate(("U", "V", "W", "UV", "P"))}
        lib().orc_spectra_get(self.h, *[_dptr(out[k]) for k in ("U", "V", "W", "UV", "P")], None, None)
        return out

    def slip(self) -> np.ndarray:
        """Accumulated slip statistics: complex [wall (bottom, top)][u1_itp, du1dy, u3_itp,
        du3dy][N2][N1/2+1]"""
        out = np.zeros((2, 4, self.s.N2, self.s.N1 // 2 + 1), np.complex128)
        lib().orc_slip_get(self.h, _dptr(out.view(np.float64)))
        return out

    def slip_planes(self) -> np.ndarray:
        """Instantaneous slip planes of the current state, laid out as slip()"""
        out = np.zeros((2, 4, self.s.N2, self.s.N1 // 2 + 1), np.complex128)
        lib().orc_slip_planes(self.h, _dptr(out.view(np.float64)))
        return out

    def stats(self):
        """(plane [11][nyu], cond [9][ncl][dnz][dnx] or None, istat)"""
        dims = (C.c_int * 3)()
        lib().orc_stats_get(self.h, None, None, None, dims)
        ncl, dnx, dnz = dims[0], dims[1], dims[2]
        plane = np.zeros((11, self.s.nyu))
        cond = np.zeros((9, ncl, dnz, dnx)) if dnx else None
        ist = C.c_int64()
        lib().orc_stats_get(self.h, _dptr(plane), _dptr(cond), C.byref(ist), dims)
        return plane, cond, ist.value

    def stats_pw(self):
        """(pressure plane sums [2][nyu - 2], conditioned P, P^2, omega_x, omega_x^2
        [4][ncl + 1][dnz][dnx] or None)"""
        dims = (C.c_int * 3)()
        lib().orc_stats_get(self.h, None, None, None, dims)
        ncl, dnx, dnz = dims[0], dims[1], dims[2]
        pplane = np.zeros((2, self.s.nyu - 2))
        cond = np.zeros((4, ncl + 1, dnz, dnx)) if dnx else None
        lib().orc_stats_get_pw(self.h, _dptr(pplane), _dptr(cond))
        return pplane, cond

    def four_to_phys(self, spec: np.ndarray) -> np.ndarray:
        spec = np.ascontiguousarray(spec, np.complex128)
        npl = spec.shape[0]
        phys = np.zeros((npl, self.s.G2, self.s.G1))
        lib().orc_four_to_phys(self.h, _dptr(spec.view(np.float64)), _dptr(phys), npl)
        return phys

    def phys_to_four(self, phys: np.ndarray) -> np.ndarray:
        phys = np.ascontiguousarray(phys, np.float64)
        npl = phys.shape[0]
        spec = np.zeros((npl, self.s.N2, self.s.N1 // 2 + 1), np.complex128)
        lib().orc_phys_to_four(self.h, _dptr(phys), _dptr(spec.view(np.float64)), npl)
        return spec
