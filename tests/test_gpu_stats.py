"""Statistics on the GPU (k_xstats, k_wx_stats, k_p_stats, k_cond_spec + k_cond_phys, k_spectra,
k_slip, through the C ABI) vs the CPU oracle after accumulating twice around a step: plane sums
and tile-conditioned sums of stats.f90 (omega_x and P by Parseval on the GPU, by the inverse
transform in the oracle; the conditioned P and omega_x from FP64 physical planes), the
spectra of spectra.f90 and the wall slip statistics of sl_stats2.f90 / inst_sl_stats.f90.
Bar: FP64 form 1e-12 relative to the largest sum of a kind; mixed 1e-5."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.native import GpuChannel
from rnl_multiblock_nofft_gb300.workloads import (initial_field, initial_field_bands, initial_scalars,
                                                  workload_setup)

pytestmark = pytest.mark.gpu


def run(name, precision, seed):
    s = workload_setup(name)
    o = Oracle(s)
    g = GpuChannel(s, precision)
    if s.multiblock:
        f = initial_field_bands(s, seed)
        o.set_bands(f)
        g.upload_bands(f)
    else:
        f = initial_field(s, seed)
        o.set_state(*f)
        g.upload_state(*f)
    for x in (o, g):
        x.set_scalars(**initial_scalars(s))
        x.stats_accumulate()
        x.step()
        x.stats_accumulate()
    g.synchronize()
    return o, g


def close(a, b, tol):
    # relative to the largest sum (the energy scale): sums with a zero mean (V, UV) have
    # no scale of their own
    scale = max(np.abs(a).max(), 1e-300)
    for q in range(a.shape[0]):
        assert np.abs(a[q] - b[q]).max() <= tol * scale, (q, np.abs(a[q] - b[q]).max() / scale)


@pytest.mark.parametrize("name,precision,tol", [("SP", "fp64", 1e-12), ("MB", "fp64", 1e-12),
                                                ("MBP", "fp64", 1e-12), ("SP", "mixed", 1e-5)])
def test_stats_match_oracle(cuda_ok, name, precision, tol):
    o, g = run(name, precision, 51)
    (po, co, io), (pg, cg, ig) = o.stats(), g.stats()
    assert io == ig == 2 and pg.shape == po.shape == (11, o.s.nyu)
    close(po[:9], pg[:9], tol)
    close(po[9:], pg[9:], tol)                      # omega_x, on its own scale
    if co is not None:
        assert cg is not None and cg.shape == co.shape
        close(co.reshape(9, -1), cg.reshape(9, -1), tol)
    # pressure sums (Parseval on the GPU, transform + point sums in the oracle) and the
    # conditioned P, omega_x sums; the mixed form's pressure is within 1e-4 of the oracle's
    (ppo, c4o), (ppg, c4g) = o.stats_pw(), g.stats_pw()
    tp = tol if precision == "fp64" else 3e-4
    assert ppg.shape == ppo.shape == (2, o.s.nyu - 2)
    close(ppo, ppg, tp)
    if c4o is not None:
        assert c4g is not None and c4g.shape == c4o.shape
        # the conditioned P sums cover the wall planes, where the posts are: the FP64 pressure
        # there agrees to ~5e-12 (the parity tests at size), and the tile sums of a field with
        # a near-zero mean keep that absolute error (measured 8.3e-12 of the largest sum)
        close(c4o[:2].reshape(2, -1), c4g[:2].reshape(2, -1), max(tp, 5e-11))
        close(c4o[2:].reshape(2, -1), c4g[2:].reshape(2, -1), tol)
    # spectra are quadratic in a field whose mixed-form error is up to 1e-5 of its own
    # scale: 3x the field bar (FP64: the same bar)
    so, sg = o.spectra(), g.spectra()
    tq = tol if precision == "fp64" else 3 * tol
    for k in so:
        assert sg[k].shape == so[k].shape, k
        close(so[k][None], sg[k][None], tq)
    # slip statistics: the state agrees to the parity bar on the scale of the whole field, so
    # that is their scale (the faces of a textured channel lie deep in the solid, where u is
    # small); the derivatives scale with dthdyv ddthetavi at the faces
    bands = o.get_bands() if o.s.multiblock else {2: o.get_state()}
    umax = {f: max(np.abs(a[f]).max() for a in bands.values() if a[f].size) for f in (0, 2)}
    q = o.s.band_levels(2, 1)
    fy = max(abs(o.s.dthdyv[q[0]]), abs(o.s.dthdyv[q[1]])) * o.s.ddthetavi
    lo, lg = o.slip(), g.slip()
    io_, ig_ = o.slip_planes(), g.slip_planes()
    for f in range(4):
        sc = 2 * umax[f & 2] * (fy if f in (1, 3) else 1.0)
        assert np.abs(lo[:, f] - lg[:, f]).max() <= tol * sc, f
        assert np.abs(io_[:, f] - ig_[:, f]).max() <= tol * sc / 2, f
