"""Host set-up vs the y-grid, metrics and band limits stored in the reference's own
plane files (start.f90:693-1077 writes them; record_out stores them in each file)."""
import os

import numpy as np

from rnl_multiblock_nofft_gb300.setup_grid import ChannelParams, build_setup

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_ygrid_bit_exact():
    s = build_setup(ChannelParams())      # the reference's input.in (32x32x153 smooth)
    ic = np.load(os.path.join(GOLD, "ic_0032x0032x0153.npz"))
    assert np.array_equal(ic["yu"], s.yu)
    assert np.array_equal(ic["yv"], s.yv)
    assert np.array_equal(ic["dthdyu"], s.dthdyu)
    assert np.array_equal(ic["dthdyv"], s.dthdyv)
    assert np.array_equal(ic["N"], s.N)
    assert float(ic["dthetavi"]) == 0.0   # never assigned in the reference


def test_dtv_matches_history():
    import json
    s = build_setup(ChannelParams())
    h = json.load(open(os.path.join(GOLD, "hist_0032x0032x0153.json")))
    assert s.dtv == h[1]["dtv"]


def test_post_lists_shape():
    from rnl_multiblock_nofft_gb300.workloads import workload_setup
    s = workload_setup("SP")
    lu, lv = s.list_ib[2], s.list_ib[1]
    p = s.p
    per_tile = p.npeakx * p.npeakz * s.dny
    assert len(lu) == 2 * per_tile * p.ntilex * p.ntilez == len(lv)
    # lower tip layer of u interpolates from level 1 with u = 0 at yv(0)
    tip = lu[lu[:, 2] == 0]
    assert (tip[:, 5] == 1).all()
    assert (lu[:, 0] >= 1).all() and (lu[:, 0] <= s.G1).all() and (lu[:, 1] <= s.G2).all()
