"""Batches of channels of different sizes advanced by one graph launch per step,
and the block-size autotuner, against the CPU oracle."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.native import GpuBatch, GpuChannel
from rnl_multiblock_nofft_gb300.workloads import (ensemble_setups, initial_field, initial_scalars,
                                                  workload_setup)

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make(s, seed, prec="fp64"):
    st = initial_field(s, seed)
    o = Oracle(s)
    o.set_state(*st)
    o.set_scalars(**initial_scalars(s))
    g = GpuChannel(s, prec)
    g.upload_state(*st)
    g.set_scalars(**initial_scalars(s))
    return o, g


def test_batch_of_uneven_channels(cuda_ok):
    setups = [workload_setup("S"), workload_setup("C0"), workload_setup("SP")] + ensemble_setups(3, seed=77)
    pairs = [make(s, 300 + i) for i, s in enumerate(setups)]
    b = GpuBatch([g for _, g in pairs])
    for _ in range(2):
        b.step()
        for o, _ in pairs:
            o.step()
    b.synchronize()
    for o, g in pairs:   # bar: 1e-12 relative per step
        for x, y in zip(o.get_state(), g.download_state()):
            assert rel(y, x) < 2 * 1e-12
        assert g.scalars()["iter"] == 2
    b.close()


def test_autotune_keeps_state_and_parity(cuda_ok):
    s = workload_setup("M")
    o, g = make(s, 41)
    before = g.download_state()
    sc0 = g.scalars()
    g.autotune()
    after = g.download_state()
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    assert g.scalars()["t"] == sc0["t"]
    o.step(2)
    g.step(2)
    g.synchronize()
    for x, y in zip(o.get_state(), g.download_state()):
        assert rel(y, x) < 2 * 1e-12


def test_mixed_batch_matches_channels_stepped_alone(cuda_ok):
    """The mixed form in a batch: every channel's state after two batched steps equals (bit for bit)
    the same channel stepped on its own. The channels are created largest first, so a kernel
    attribute that one handle set for its own sizes could not serve an earlier, larger one."""
    setups = sorted(ensemble_setups(6, seed=91), key=lambda s: -s.nyu * s.ncols)
    alone, batched = [], []
    for i, s in enumerate(setups):
        st = initial_field(s, 500 + i)
        for lst in (alone, batched):
            g = GpuChannel(s, "mixed")
            g.upload_state(*st)
            g.set_scalars(**initial_scalars(s))
            lst.append(g)
    b = GpuBatch(batched)
    b.step(2)
    b.synchronize()
    for g in alone:
        g.step(2)
        g.synchronize()
    for ga, gb in zip(alone, batched):
        for x, y in zip(ga.download_state(), gb.download_state()):
            assert np.array_equal(x, y)
