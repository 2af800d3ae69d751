"""The reference's plane files (record_out / read_in, FOU3D.f90:2856-3073): a written file
reads back bit for bit, and the committed initial-state fixture is the cfield of the
reference's restart files (compared directly when LH_REFERENCE_DIR names a checkout)."""
import os
import struct

import numpy as np
import pytest

from rnl_multiblock_nofft_gb300.planefile import PlaneFile, read_planefile, write_planefile
from rnl_multiblock_nofft_gb300.setup_grid import ChannelParams, build_setup

GOLD = os.path.join(os.path.dirname(__file__), "golden")
REF_DIR = os.environ.get("LH_REFERENCE_DIR", "")


def test_roundtrip(tmp_path):
    rng = np.random.default_rng(4)
    N = np.arange(20, dtype=np.int32).reshape(4, 5)
    y = np.linspace(-1, 1, 7)
    data = rng.standard_normal((7, 6, 5)) + 1j * rng.standard_normal((7, 6, 5))
    pf = PlaneFile(0.25, 3250.0, 1.0, 2.0, -3e-3, 3, 12, N, y, 1.5, rng.random(7), np.arange(-1, 6), 2, data)
    p = str(tmp_path / "u2.dat")
    write_planefile(p, pf)
    back = read_planefile(p)
    assert (back.t, back.Re, back.alp, back.bet, back.mpgx, back.nband, back.iter) == (0.25, 3250.0, 1.0, 2.0, -3e-3, 3, 12)
    assert np.array_equal(back.N, N) and np.array_equal(back.y, y) and back.dthetavi == 1.5
    assert np.array_equal(back.levels, pf.levels) and back.field_id == 2
    assert np.array_equal(back.data, data)
    # record markers: every record framed by equal 4-byte lengths
    raw = open(p, "rb").read()
    off = nrec = 0
    while off < len(raw):
        (n,) = struct.unpack_from("<i", raw, off)
        assert struct.unpack_from("<i", raw, off + 4 + n)[0] == n
        off += 8 + n
        nrec += 1
    assert nrec == 3 + len(pf.levels)


def test_fixture_grid_is_the_setup_grid():
    ic = np.load(os.path.join(GOLD, "ic_0032x0032x0153.npz"))
    s = build_setup(ChannelParams())
    assert np.array_equal(ic["yu"], s.yu) and np.array_equal(ic["yv"], s.yv)
    assert ic["u1"].shape == (s.N2 * (s.N1 // 2 + 1), s.nyu) and ic["u2"].shape[1] == s.nyv


def test_fixture_matches_reference_restart_files():
    if not REF_DIR or not os.path.isdir(os.path.join(REF_DIR, "input")):
        pytest.skip("set LH_REFERENCE_DIR to a reference checkout to compare its restart files")
    ic = np.load(os.path.join(GOLD, "ic_0032x0032x0153.npz"))
    for f in ("u1", "u2", "u3", "p"):
        pf = read_planefile(os.path.join(REF_DIR, "input", f"{f}_0032x0032x0153_t00000.dat"))
        assert np.array_equal(np.ascontiguousarray(pf.data.reshape(pf.data.shape[0], -1).T), ic[f])
