"""GPU (CUDA, through the C ABI) vs the CPU oracle on the same seeded inputs.
Bar: FP64 form within 1e-12 relative per step (L2 per field, and max-abs relative
to the field's max); mixed form within 1e-5 relative velocity error."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.native import GpuChannel
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

pytestmark = pytest.mark.gpu
FIELDS = ("u1", "u2", "u3", "p")
TOL64 = 1e-12


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def pair(name, seed, precision="fp64"):
    s = workload_setup(name)
    st = initial_field(s, seed)
    o = Oracle(s)
    o.set_state(*st)
    o.set_scalars(**initial_scalars(s))
    g = GpuChannel(s, precision)
    g.upload_state(*st)
    g.set_scalars(**initial_scalars(s))
    return s, o, g


def compare(o, g, tol, fields=FIELDS):
    a = o.get_state()
    b = g.download_state()
    out = {}
    for f, x, y in zip(FIELDS, a, b):
        if f not in fields:
            continue
        out[f] = relerr(y, x)
        assert out[f] < tol, (f, out[f])
    return out


def test_roundtrip_state(cuda_ok):
    s, o, g = pair("S", 11)
    a = o.get_state()
    b = g.download_state()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_initial_scalars(cuda_ok):
    s, o, g = pair("C0", 12)
    so, sg = o.scalars(), g.scalars()
    assert sg["Qx"] == pytest.approx(so["Qx"], rel=1e-14)
    assert sg["QxT"] == pytest.approx(so["QxT"], rel=1e-14)
    assert abs(sg["err"] - so["err"]) < 1e-15


@pytest.mark.parametrize("name", ["S", "C0"])
def test_substeps_fp64(cuda_ok, name):
    s, o, g = pair(name, 13)
    for k in (1, 2, 3):
        o.substep(k)
        g.substep(k)
        g.synchronize()
        compare(o, g, TOL64)
        so, sg = o.scalars(), g.scalars()
        assert sg["dt"] == pytest.approx(so["dt"], rel=1e-13)
        assert sg["mpgx"] == pytest.approx(so["mpgx"], rel=1e-12)


@pytest.mark.parametrize("name", ["C0", "M"])
def test_steps_fp64_graph(cuda_ok, name):
    s, o, g = pair(name, 14)
    for it in range(3):
        o.step()
        g.step()
        g.synchronize()
        compare(o, g, TOL64)
    so, sg = o.scalars(), g.scalars()
    assert sg["iter"] == so["iter"] == 3
    assert sg["t"] == pytest.approx(so["t"], rel=1e-13)
    assert sg["err"] < 1e-13


def test_posts_immersed_boundary_fp64(cuda_ok):
    s, o, g = pair("SP", 15)
    assert s.dny > 0 and len(s.list_ib[2]) > 0
    for it in range(2):
        o.step()
        g.step()
        g.synchronize()
        compare(o, g, TOL64)


def test_leaves_transforms(cuda_ok):
    import torch
    s, o, g = pair("C0", 16)
    rng = np.random.default_rng(3)
    npl = 5
    spec = rng.normal(size=(npl, s.N2, s.N1 // 2 + 1)) + 1j * rng.normal(size=(npl, s.N2, s.N1 // 2 + 1))
    ref = o.four_to_phys(spec)
    ds = torch.from_numpy(spec.view(np.float64).copy()).cuda()
    dp = torch.zeros((npl, s.G2, s.G1), dtype=torch.float64, device="cuda")
    g.four_to_phys(ds.data_ptr(), dp.data_ptr(), npl)
    g.synchronize()
    phys = dp.cpu().numpy()
    assert np.abs(phys - ref).max() / np.abs(ref).max() < 1e-13
    back_ref = o.phys_to_four(ref)
    db = torch.zeros_like(ds)
    g.phys_to_four(dp.data_ptr(), db.data_ptr(), npl)
    g.synchronize()
    back = db.cpu().numpy().view(np.complex128).reshape(back_ref.shape)
    assert np.abs(back - back_ref).max() / np.abs(back_ref).max() < 1e-13


def test_mixed_precision_error(cuda_ok):
    s, o, g = pair("C0", 17, precision="mixed")
    for it in range(5):
        o.step()
        g.step()
    g.synchronize()
    compare(o, g, 1e-5, fields=("u1", "u2", "u3"))
