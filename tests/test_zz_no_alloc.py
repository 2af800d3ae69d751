"""lh_four_to_phys_noalloc: the x/z inverse transform for callers that cannot call
cudaMalloc (hosts that own all device memory and so cannot create a handle). It
must give what the handle-based lh_four_to_phys gives, call after call, while its
working memory is the library's fixed device array. Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from rnl_multiblock_nofft_gb300 import abi, native
from rnl_multiblock_nofft_gb300.native import GpuChannel
from rnl_multiblock_nofft_gb300.workloads import workload_setup

pytestmark = pytest.mark.gpu
TOL = 1e-13   # the tolerance of the leaf-transform parity test
SCRATCH = 32 << 20


def noalloc(L, s, spec, phys, nplanes):
    err = C.c_char_p()
    rc = L.lh_four_to_phys_noalloc(s.N1, s.N2, s.G1, s.G2, C.c_void_p(spec.data_ptr()),
                                   C.c_void_p(phys.data_ptr()), nplanes, None, C.byref(err))
    return rc, (err.value or b"").decode()


@pytest.mark.parametrize("name", ["C0", "M"])
def test_noalloc_matches_handle_twice(cuda_ok, name):
    import torch
    s = workload_setup(name)
    g = GpuChannel(s, "fp64")
    L = native.load()
    rng = np.random.default_rng(7)
    npl = 6
    for call in range(2):   # two calls in a row: the shared array keeps the last call's contents
        spec = rng.normal(size=(npl, s.N2, s.N1 // 2 + 1)) + 1j * rng.normal(size=(npl, s.N2, s.N1 // 2 + 1))
        ds = torch.from_numpy(spec.view(np.float64).copy()).cuda()
        ref = torch.zeros((npl, s.G2, s.G1), dtype=torch.float64, device="cuda")
        out = torch.full((npl, s.G2, s.G1), float("nan"), dtype=torch.float64, device="cuda")
        g.four_to_phys(ds.data_ptr(), ref.data_ptr(), npl)
        g.synchronize()
        rc, msg = noalloc(L, s, ds, out, npl)
        assert rc == 0, msg
        torch.cuda.synchronize()
        a, b = ref.cpu().numpy(), out.cpu().numpy()
        assert np.isfinite(b).all()
        assert np.abs(b - a).max() / np.abs(a).max() < TOL, (call, np.abs(b - a).max())
    g.close()


def test_noalloc_rejects_oversize(cuda_ok):
    import torch
    s = workload_setup("C0")
    L = native.load()
    plane = 16 * s.G2 * (s.N1 // 2 + 1)
    too_many = SCRATCH // plane + 1
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc, msg = noalloc(L, s, d, d, too_many)
    assert rc == abi.LH_EINVAL
    assert "too many planes" in msg
