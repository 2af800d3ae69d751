"""Queued state I/O (lh_upload_state_async / lh_download_state_async): a chain of
upload -> step -> download, queued without host synchronisation and with the copies on
their own streams, gives the same states as the blocking calls, bit for bit."""
import numpy as np
import pytest
import torch

from rnl_multiblock_nofft_gb300.native import GpuChannel
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

pytestmark = pytest.mark.gpu


def pinned(shapes):
    return [torch.empty(tuple(sh) + (2,), dtype=torch.float64, pin_memory=True).numpy()
            .view(np.complex128)[..., 0] for sh in shapes]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_chain_matches_blocking(cuda_ok, precision):
    s = workload_setup("SP")
    inputs = [initial_field(s, 70 + k) for k in range(3)]
    # blocking reference: each input uploaded, one step, state read back
    g = GpuChannel(s, precision)
    ref = []
    for st in inputs:
        g.upload_state(*st)
        g.set_scalars(**initial_scalars(s))
        g.step(1)
        g.synchronize()
        ref.append(g.download_state())
    # queued: the three uploads, steps and downloads, one synchronisation at the end
    h = GpuChannel(s, precision)
    ins = [pinned(h.shapes) for _ in inputs]
    outs = [pinned(h.shapes) for _ in inputs]
    for buf, st in zip(ins, inputs):
        for d, a in zip(buf, st):
            d[...] = a
    for k in range(3):
        h.upload_state_async(*ins[k])
        h.set_scalars(**initial_scalars(s))
        h.step(1)
        h.download_state_async(outs[k])
    h.synchronize()
    for k in range(3):
        for a, b in zip(ref[k], outs[k]):
            assert np.array_equal(a, b), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_band_chain_matches_blocking(cuda_ok, precision):
    from rnl_multiblock_nofft_gb300.workloads import initial_field_bands
    s = workload_setup("MBP")
    inputs = [initial_field_bands(s, 80 + k) for k in range(3)]
    g = GpuChannel(s, precision)
    ref = []
    for bands in inputs:
        g.upload_bands(bands)
        g.set_scalars(**initial_scalars(s))
        g.step(1)
        g.synchronize()
        ref.append(g.download_bands())
    h = GpuChannel(s, precision)
    ins = [{b: pinned(s.band_shapes(b)) for b in (1, 2, 3)} for _ in inputs]
    outs = [{b: pinned(s.band_shapes(b)) for b in (1, 2, 3)} for _ in inputs]
    for buf, bands in zip(ins, inputs):
        for b in (1, 2, 3):
            for d, a in zip(buf[b], bands[b]):
                d[...] = a
    for k in range(3):
        h.upload_bands_async(ins[k])
        h.set_scalars(**initial_scalars(s))
        h.step(1)
        h.download_bands_async(outs[k])
    h.synchronize()
    for k in range(3):
        for b in (1, 2, 3):
            for a, c in zip(ref[k][b], outs[k][b]):
                assert np.array_equal(a, c), (k, b)
