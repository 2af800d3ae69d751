"""ctypes binding of the CUDA library (liblh.so, include/lh.h).

There is no CPU fallback: constructing a GpuChannel without the built library or
without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import LH_OK, LH_PREC_FP64, LH_PREC_MIXED, LhConfig, LhHistory, LhScalars, cfield_shape, make_config
from .setup_grid import ChannelSetup

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "liblh.so")
_lib = None

EXPORTS = ("lh_create", "lh_destroy", "lh_last_error", "lh_upload_state", "lh_download_state",
           "lh_upload_state_async", "lh_download_state_async", "lh_upload_band_async", "lh_download_band_async",
           "lh_upload_band", "lh_download_band", "lh_stats_accumulate", "lh_stats_reset", "lh_stats_dims",
           "lh_stats_get", "lh_stats_get_pw", "lh_spectra_dims", "lh_spectra_get", "lh_slip_get", "lh_slip_planes",
           "lh_set_scalars", "lh_get_scalars", "lh_substep", "lh_step", "lh_synchronize",
           "lh_device_state", "lh_stream", "lh_four_to_phys", "lh_phys_to_four", "lh_kernel_launches",
           "lh_profile_steps", "lh_four_to_phys_noalloc", "lh_autotune", "lh_batch_create", "lh_batch_step",
           "lh_batch_synchronize", "lh_batch_destroy", "lh_batch_stream", "lh_history_record", "lh_get_tuning")


class LhKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int32), ("total_ms", C.c_double)]


class LhError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lh error {code}: {msg}")
        self.code = code


def load(path: str = _LIB_PATH):
    """Load liblh.so and declare the signatures. Raises if the library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"native library not built: {path} (run __graft_entry__.build())")
    L = C.CDLL(path)
    vp, dp, i = C.c_void_p, C.POINTER(C.c_double), C.c_int
    L.lh_create.argtypes = [C.POINTER(LhConfig), C.POINTER(vp)]
    L.lh_destroy.argtypes = [vp]
    L.lh_last_error.argtypes = [vp]
    L.lh_last_error.restype = C.c_char_p
    L.lh_upload_state.argtypes = [vp, dp, dp, dp, dp]
    L.lh_download_state.argtypes = [vp, dp, dp, dp, dp]
    L.lh_upload_state_async.argtypes = [vp, dp, dp, dp, dp]
    L.lh_upload_band_async.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    L.lh_download_band_async.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    L.lh_download_state_async.argtypes = [vp, dp, dp, dp, dp]
    L.lh_upload_band.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    L.lh_stats_accumulate.argtypes = [vp]
    L.lh_stats_reset.argtypes = [vp]
    L.lh_stats_dims.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.lh_stats_get.argtypes = [vp, dp, dp, C.POINTER(C.c_int64)]
    L.lh_stats_get_pw.argtypes = [vp, dp, dp]
    L.lh_spectra_dims.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.lh_spectra_get.argtypes = [vp, dp, dp, dp, dp, dp]
    L.lh_slip_get.argtypes = [vp, dp]
    L.lh_slip_planes.argtypes = [vp, dp]
    L.lh_download_band.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    L.lh_set_scalars.argtypes = [vp, C.POINTER(LhScalars)]
    L.lh_get_scalars.argtypes = [vp, C.POINTER(LhScalars)]
    L.lh_history_record.argtypes = [vp, C.POINTER(LhHistory)]
    L.lh_substep.argtypes = [vp, i]
    L.lh_step.argtypes = [vp]
    L.lh_synchronize.argtypes = [vp]
    L.lh_device_state.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]
    L.lh_stream.argtypes = [vp]
    L.lh_stream.restype = vp
    L.lh_four_to_phys.argtypes = [vp, vp, vp, i]
    L.lh_phys_to_four.argtypes = [vp, vp, vp, i]
    L.lh_kernel_launches.argtypes = [vp]
    L.lh_kernel_launches.restype = C.c_int64
    L.lh_profile_steps.argtypes = [vp, i, C.POINTER(LhKernelTime), i, C.POINTER(i)]
    L.lh_four_to_phys_noalloc.argtypes = [i, i, i, i, vp, vp, i, vp, C.POINTER(C.c_char_p)]
    L.lh_autotune.argtypes = [vp]
    L.lh_get_tuning.argtypes = [vp, C.POINTER(C.c_int32)]
    L.lh_batch_create.argtypes = [C.POINTER(vp), i, C.POINTER(vp)]
    L.lh_batch_step.argtypes = [vp]
    L.lh_batch_synchronize.argtypes = [vp]
    L.lh_batch_destroy.argtypes = [vp]
    L.lh_batch_stream.argtypes = [vp]
    L.lh_batch_stream.restype = vp
    _lib = L
    return L


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class GpuChannel:
    """One channel whose RK3 substep runs on the GPU through the C ABI.

    State arrays on the host use the reference's cfield layout: complex128
    [ncols, nlevels] (level fastest), one column per (kx, kz) mode."""

    def __init__(self, setup: ChannelSetup, precision: str = "fp64", triads=None):
        """`triads` (triads.TriadLists) selects the as-run triad-list nonlinear term
        (ops_in_planes); None the pseudo-spectral products (ops_in_planes2)."""
        self.s = setup
        self.L = load()
        prec = {"fp64": LH_PREC_FP64, "mixed": LH_PREC_MIXED}[precision]
        self.precision = precision
        cfg, self._keep = make_config(setup, prec, triads=triads)
        self._cfg = cfg
        h = C.c_void_p()
        rc = self.L.lh_create(C.byref(cfg), C.byref(h))
        if rc != LH_OK:
            raise LhError(rc, "lh_create failed: " + self.L.lh_last_error(None).decode())
        self.h = h
        self.shapes = cfield_shape(setup)
        self._pending = []   # host arrays of queued asynchronous copies

    def _check(self, rc: int):
        if rc != LH_OK:
            raise LhError(rc, self.L.lh_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.lh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state ----
    def upload_state(self, u1, u2, u3, p):
        arrs = [np.ascontiguousarray(a, np.complex128) if a is not None else None for a in (u1, u2, u3, p)]
        for a, sh in zip(arrs, self.shapes):
            if a is not None and a.shape != sh:
                raise ValueError(f"shape {a.shape} != {sh}")
        self._check(self.L.lh_upload_state(self.h, *[_dptr(a) for a in arrs]))

    def download_state(self, out=None):
        """Returns (u1, u2, u3, p); `out` may supply C-contiguous complex128 arrays
        (e.g. views of pinned host memory) to receive them."""
        if out is None:
            out = [np.zeros(sh, np.complex128) for sh in self.shapes]
        for a, sh in zip(out, self.shapes):
            if a.shape != sh or a.dtype != np.complex128 or not a.flags.c_contiguous:
                raise ValueError("download buffers must be C-contiguous complex128 of the state shapes")
        self._check(self.L.lh_download_state(self.h, *[_dptr(a) for a in out]))
        return out

    def upload_state_async(self, u1, u2, u3, p):
        """Queued upload (lh_upload_state_async): the arrays must be C-contiguous complex128 of
        the state shapes, ideally page-locked; they are kept alive until synchronize()."""
        arrs = (u1, u2, u3, p)
        for a, sh in zip(arrs, self.shapes):
            if a.shape != sh or a.dtype != np.complex128 or not a.flags.c_contiguous:
                raise ValueError("upload buffers must be C-contiguous complex128 of the state shapes")
        self._pending.extend(arrs)
        self._check(self.L.lh_upload_state_async(self.h, *[_dptr(a) for a in arrs]))

    def download_state_async(self, out):
        """Queued download into `out` (lh_download_state_async); valid after synchronize()."""
        for a, sh in zip(out, self.shapes):
            if a.shape != sh or a.dtype != np.complex128 or not a.flags.c_contiguous:
                raise ValueError("download buffers must be C-contiguous complex128 of the state shapes")
        self._pending.extend(out)
        self._check(self.L.lh_download_state_async(self.h, *[_dptr(a) for a in out]))
        return out

    def upload_bands_async(self, bands: dict):
        """Queued per-band upload (lh_upload_band_async); arrays kept alive until synchronize()."""
        for b, arrs in bands.items():
            for a, sh in zip(arrs, self.s.band_shapes(b)):
                if a.shape != sh or a.dtype != np.complex128 or not a.flags.c_contiguous:
                    raise ValueError(f"band {b}: C-contiguous complex128 of shape {sh} expected")
            self._pending.extend(arrs)
            self._check(self.L.lh_upload_band_async(self.h, b, *[_dptr(a) for a in arrs]))

    def download_bands_async(self, out: dict):
        """Queued per-band download into `out` ({band: (u1, u2, u3, p)}); valid after synchronize()."""
        for b, arrs in out.items():
            for a, sh in zip(arrs, self.s.band_shapes(b)):
                if a.shape != sh or a.dtype != np.complex128 or not a.flags.c_contiguous:
                    raise ValueError(f"band {b}: C-contiguous complex128 of shape {sh} expected")
            self._pending.extend(arrs)
            self._check(self.L.lh_download_band_async(self.h, b, *[_dptr(a) for a in arrs]))
        return out

    def upload_bands(self, bands: dict):
        """{band: (u1, u2, u3, p)} in the bands' cfield layouts (ChannelSetup.band_shapes);
        the per-band upload of a multiblock channel (lh_upload_band)."""
        for b, arrs in bands.items():
            arrs = [np.ascontiguousarray(a, np.complex128) if a is not None else None for a in arrs]
            for a, sh in zip(arrs, self.s.band_shapes(b)):
                if a is not None and a.shape != sh:
                    raise ValueError(f"band {b}: shape {a.shape} != {sh}")
            self._check(self.L.lh_upload_band(self.h, b, *[_dptr(a) for a in arrs]))

    def download_bands(self) -> dict:
        out = {}
        for b in (1, 2, 3):
            arrs = [np.zeros(sh, np.complex128) for sh in self.s.band_shapes(b)]
            self._check(self.L.lh_download_band(self.h, b, *[_dptr(a) for a in arrs]))
            out[b] = arrs
        return out

    # ---- statistics (stats.f90, spectra.f90, sl_stats2.f90) ----
    def stats_accumulate(self):
        self._check(self.L.lh_stats_accumulate(self.h))

    def stats_reset(self):
        self._check(self.L.lh_stats_reset(self.h))

    def spectra(self) -> dict:
        """Accumulated sp(level, long column) as {"U", "V", "W", "UV", "P"}: arrays
        [long column][level of band 2]; see include/lh.h."""
        nl = (C.c_int * 5)()
        nlong = C.c_int()
        self._check(self.L.lh_spectra_dims(self.h, nl, C.byref(nlong)))
        keys = ("U", "V", "W", "UV", "P")
        out = {k: np.zeros((nlong.value, nl[q])) for q, k in enumerate(keys)}
        self._check(self.L.lh_spectra_get(self.h, *[_dptr(out[k]) for k in keys]))
        return out

    def slip(self) -> np.ndarray:
        """Accumulated slip statistics: complex [face (bottom, top)][u1, du1dy, u3, du3dy][N2][N1/2+1]"""
        out = np.zeros((2, 4, self.s.N2, self.s.N1 // 2 + 1), np.complex128)
        self._check(self.L.lh_slip_get(self.h, _dptr(out.view(np.float64))))
        return out

    def slip_planes(self) -> np.ndarray:
        """The slip planes of the current state, laid out as slip()"""
        out = np.zeros((2, 4, self.s.N2, self.s.N1 // 2 + 1), np.complex128)
        self._check(self.L.lh_slip_planes(self.h, _dptr(out.view(np.float64))))
        return out

    def stats(self):
        """(plane [11][nyu], cond [9][ncl][dnz][dnx] or None, istat); see include/lh.h."""
        ncl, dnx, dnz = C.c_int(), C.c_int(), C.c_int()
        self._check(self.L.lh_stats_dims(self.h, C.byref(ncl), C.byref(dnx), C.byref(dnz)))
        plane = np.zeros((11, self.s.nyu))
        cond = np.zeros((9, ncl.value, dnz.value, dnx.value)) if dnx.value else None
        ist = C.c_int64()
        self._check(self.L.lh_stats_get(self.h, _dptr(plane), _dptr(cond), C.byref(ist)))
        return plane, cond, ist.value

    def stats_pw(self):
        """(pressure plane sums [2][nyu - 2], conditioned P, P^2, omega_x, omega_x^2
        [4][ncl + 1][dnz][dnx] or None); see include/lh.h."""
        ncl, dnx, dnz = C.c_int(), C.c_int(), C.c_int()
        self._check(self.L.lh_stats_dims(self.h, C.byref(ncl), C.byref(dnx), C.byref(dnz)))
        pplane = np.zeros((2, self.s.nyu - 2))
        cond = np.zeros((4, ncl.value + 1, dnz.value, dnx.value)) if dnx.value else None
        self._check(self.L.lh_stats_get_pw(self.h, _dptr(pplane), _dptr(cond)))
        return pplane, cond

    def set_scalars(self, **kw):
        s = LhScalars()
        for k, v in kw.items():
            setattr(s, k, v)
        self._check(self.L.lh_set_scalars(self.h, C.byref(s)))

    def scalars(self) -> dict:
        s = LhScalars()
        self._check(self.L.lh_get_scalars(self.h, C.byref(s)))
        return s.as_dict()

    def history_record(self) -> dict:
        """The history-file record of the current state (lh_history_record)."""
        r = LhHistory()
        self._check(self.L.lh_history_record(self.h, C.byref(r)))
        return r.as_dict()

    # ---- time stepping ----
    def substep(self, kRK: int):
        self._check(self.L.lh_substep(self.h, kRK))

    def step(self, n: int = 1):
        for _ in range(n):
            self._check(self.L.lh_step(self.h))

    def synchronize(self):
        self._check(self.L.lh_synchronize(self.h))
        self._pending = []

    def kernel_launches(self) -> int:
        return int(self.L.lh_kernel_launches(self.h))

    def tuning(self) -> dict:
        """Block sizes and staging depths of the solve kernels (lh_get_tuning)."""
        a = (C.c_int32 * 6)()
        self._check(self.L.lh_get_tuning(self.h, a))
        return dict(threads_uw=a[0], threads_v=a[1], threads_p=a[2], stage_uw=a[3], stage_v=a[4], stage_p=a[5])

    def autotune(self):
        """Pick the block sizes of the column kernels for this channel (state restored)."""
        self._check(self.L.lh_autotune(self.h))

    def profile_steps(self, nsteps: int) -> dict:
        """{kernel name: (launches, total ms)} over `nsteps` eager steps."""
        buf = (LhKernelTime * 64)()
        n = C.c_int(0)
        self._check(self.L.lh_profile_steps(self.h, nsteps, buf, 64, C.byref(n)))
        return {buf[k].name.decode(): (buf[k].launches, buf[k].total_ms) for k in range(n.value)}

    def stream(self) -> int:
        return int(self.L.lh_stream(self.h) or 0)

    def device_state(self):
        ptrs = [C.c_void_p() for _ in range(4)]
        self._check(self.L.lh_device_state(self.h, *[C.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]

    # ---- leaves (device pointers, e.g. torch tensors' data_ptr()) ----
    def four_to_phys(self, spec_ptr: int, phys_ptr: int, nplanes: int):
        self._check(self.L.lh_four_to_phys(self.h, C.c_void_p(spec_ptr), C.c_void_p(phys_ptr), nplanes))

    def phys_to_four(self, phys_ptr: int, spec_ptr: int, nplanes: int):
        self._check(self.L.lh_phys_to_four(self.h, C.c_void_p(phys_ptr), C.c_void_p(spec_ptr), nplanes))


class GpuBatch:
    """Many independent channels (any sizes) advanced together: one RK3 step of
    every channel is one CUDA-graph launch (lh_batch_*). The GpuChannel objects
    stay owned by the caller and must outlive the batch."""

    def __init__(self, channels):
        self.channels = list(channels)
        self.L = load()
        arr = (C.c_void_p * len(self.channels))(*[c.h.value for c in self.channels])
        b = C.c_void_p()
        rc = self.L.lh_batch_create(arr, len(self.channels), C.byref(b))
        if rc != LH_OK:
            raise LhError(rc, (self.L.lh_last_error(None) or b"lh_batch_create failed").decode())
        self.b = b

    def step(self, n: int = 1):
        for _ in range(n):
            rc = self.L.lh_batch_step(self.b)
            if rc != LH_OK:
                raise LhError(rc, "lh_batch_step failed")

    def synchronize(self):
        rc = self.L.lh_batch_synchronize(self.b)
        if rc != LH_OK:
            raise LhError(rc, "lh_batch_synchronize failed")

    def stream(self) -> int:
        return int(self.L.lh_batch_stream(self.b) or 0)

    def close(self):
        if getattr(self, "b", None):
            self.L.lh_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
