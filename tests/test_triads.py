"""Triad-list nonlinear term (ops_in_planes + nonlinInter, FOU3D.f90:1724-2088): list
files, the complete enumeration, the plane -> file map, and the oracle's triad form
pinned two ways: against its own transform form (complete lists must give the same
products to round-off) and against the reference's golden run, whose lists 1-9 are
in tests/golden (the files for planes 10-76 are not in the reference)."""
import json
import os
import sys

import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.setup_grid import ChannelParams, build_setup
from rnl_multiblock_nofft_gb300.triads import (TriadFile, TriadLists, complete_list, plane_files,
                                               read_triad_file, write_triad_file)
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

GOLD = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLD)
from make_triad_fixture import load_fixture  # noqa: E402

FIELDS = ("u1", "u2", "u3", "p")
# directory of the reference checkout, when one is at hand (its 3e-9 lists files are compared)
REF_DIR = os.environ.get("LH_REFERENCE_DIR", "")


def test_complete_list_enumeration():
    a = complete_list(15, 15).astype(int)
    assert len(a) == 139905
    assert len(np.unique(a, axis=0)) == len(a)
    lt, kt = a[:, 0] + a[:, 2], a[:, 1] + a[:, 3]
    assert (lt >= 0).all() and (lt <= 15).all() and (kt >= 0).all() and (kt <= 15).all()
    assert not ((lt == 0) & (kt == 0)).any()
    assert not ((a[:, 0] == 0) & (a[:, 1] == 0)).any() and not ((a[:, 2] == 0) & (a[:, 3] == 0)).any()


def test_file_roundtrip(tmp_path):
    s = workload_setup("S")
    tl = TriadLists.thinned(s, 0.5, seed=3)
    j = sorted(tl.files)[0]
    tf = TriadFile(tl.nx, tl.nz, j, tl.files[j])
    p = str(tmp_path / "full_y01.dat")
    write_triad_file(p, tf)
    back = read_triad_file(p)
    assert (back.nx, back.nz, back.j) == (tf.nx, tf.nz, j)
    for a, b in zip(tf.lists, back.lists):
        assert np.array_equal(a, b)


def test_fixture_matches_reference_files():
    fx = load_fixture()
    lists_dir = os.path.join(REF_DIR, "3e-9")
    if not REF_DIR or not os.path.isdir(lists_dir):
        pytest.skip("set LH_REFERENCE_DIR to a reference checkout to compare its lists files")
    for j, lists in fx.items():
        tf = read_triad_file(os.path.join(lists_dir, f"full_y{j:02d}.dat"))
        assert (tf.nx, tf.nz, tf.j) == (15, 15, j)
        for a, b in zip(lists, tf.lists):
            assert len(a) == len(b)
            sa = set(map(tuple, a.tolist()))
            assert sa == set(map(tuple, b.tolist()))


def test_plane_files_symmetric():
    s = build_setup(ChannelParams())
    fu, fv = plane_files(s)
    # u planes 1..152 -> files 1..76, 76..1; v planes 1..151 -> 1..76, 75..1
    assert fu[0] == 0 and fu[-1] == 0 and fv[0] == 0 and fv[-1] == 0
    assert fu[1:-1].tolist() == list(range(1, 77)) + list(range(76, 0, -1))
    assert fv[1:-1].tolist() == list(range(1, 77)) + list(range(75, 0, -1))


def test_header_mismatch_rejected():
    s = workload_setup("S")
    with pytest.raises(ValueError):
        TriadLists.check_header(s, s.N1 // 2, s.N2 // 2 - 1)


def test_complete_lists_equal_transform_products():
    """Complete lists + linear advection + zeroth mode reproduce the 3/2-dealiased
    products on every mode except x-mode N1/2 and z-mode -N2/2 (the lists hold
    |kx| <= N1/2-1, |kz| <= N2/2-1)."""
    s = workload_setup("C0")
    f = initial_field(s, seed=1000)
    nus = []
    for tl in (None, TriadLists.complete(s)):
        o = Oracle(s, triads=tl)
        o.set_state(*f)
        o.set_scalars(**initial_scalars(s))
        o.substep(1)
        nus.append(o.get_nonlinear())
    N1h = s.N1 // 2 + 1
    for a, b in zip(*nus):
        keep = np.arange(s.N2) != s.N2 // 2
        a = a.reshape(s.N2, N1h, -1)[keep, : N1h - 1]
        b = b.reshape(s.N2, N1h, -1)[keep, : N1h - 1]
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()


# measured triad-form gaps to the golden run (lists 1-9 from the reference, complete
# lists for the planes whose files are missing), with 25 % headroom
TRIAD_GAP = {1: {"u1": 7.8e-5, "u2": 5.3e-4, "u3": 2.6e-3, "p": 1.4e-1},
             5: {"u1": 3.4e-4, "u2": 2.4e-3, "u3": 1.1e-2, "p": 1.52e-1}}
# the transform form's gaps (test_oracle_pin.py): the triad form must beat them
PRODUCT_GAP = {1: {"u1": 7.0e-4, "u2": 5.0e-3, "u3": 1.08e-2, "p": 3.4e-1},
               5: {"u1": 2.86e-3, "u2": 2.34e-2, "u3": 4.75e-2, "p": 3.67e-1}}


@pytest.fixture(scope="module")
def triad_run5():
    s = build_setup(ChannelParams())
    ic = np.load(os.path.join(GOLD, "ic_0032x0032x0153.npz"))
    comp = TriadLists.complete(s)
    tl = comp.with_files(TriadLists(comp.nx, comp.nz, load_fixture()))
    o = Oracle(s, triads=tl)
    o.set_state(*[ic[f] for f in FIELDS])
    o.set_scalars(t=0.0, mpgx=-3.0675e-3, iter=0)
    states, scal = [], []
    for _ in range(5):
        o.step()
        states.append(o.get_state())
        scal.append(o.scalars())
    return states, scal


def test_triad_flow_rate_and_cfl_history(triad_run5):
    _, scal = triad_run5
    h = json.load(open(os.path.join(GOLD, "hist_0032x0032x0153.json")))
    for k in range(5):
        assert scal[k]["t"] == h[k + 1]["t"]
        assert scal[k]["Qx"] == pytest.approx(h[k + 1]["Qx"], rel=1e-10)   # measured <= 2.4e-11
        assert scal[k]["dtc"] == pytest.approx(h[k + 1]["dtc"], rel=2e-4)  # measured <= 8.3e-5
        assert scal[k]["err"] < 1e-14


@pytest.mark.parametrize("it", [1, 5])
def test_triad_fields_closer_to_golden(triad_run5, it):
    states, _ = triad_run5
    g = np.load(os.path.join(GOLD, f"golden_it{it}.npz"))
    for f, a in zip(FIELDS, states[it - 1]):
        b = g[f].astype(np.complex128)
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel < 1.25 * TRIAD_GAP[it][f], (f, rel)
        assert rel < PRODUCT_GAP[it][f], (f, rel)


# the same gaps restricted to the planes whose list files are the reference's own (files y01-y09:
# planes 1-9 and their mirror planes 144-152) against the other planes, after 1 and 5 steps
# (measured, 25 % headroom): w is 9x closer there, p 3.8x (the pressure solve couples every level,
# so the missing lists above plane 9 still reach it), u and v ~20 % closer
TRIAD_GAP_OWN = {1: {"u1": 7.7e-5, "u2": 5.3e-4, "u3": 3.9e-4, "p": 5.6e-2},
                 5: {"u1": 3.5e-4, "u2": 2.3e-3, "u3": 2.2e-3, "p": 7.5e-2}}


@pytest.mark.parametrize("it", [1, 5])
def test_triad_gap_on_the_planes_with_the_references_lists(triad_run5, it):
    states, _ = triad_run5
    s = build_setup(ChannelParams())
    fu, fv = plane_files(s)
    g = np.load(os.path.join(GOLD, f"golden_it{it}.npz"))
    for f, a in zip(FIELDS, states[it - 1]):
        b = g[f].astype(np.complex128)
        files = np.asarray(fv if f == "u2" else fu)
        if f == "p":
            files = files[1:-1]
        own, other = (files >= 1) & (files <= 9), files > 9
        r_own = np.linalg.norm((a - b)[:, own]) / np.linalg.norm(b[:, own])
        r_other = np.linalg.norm((a - b)[:, other]) / np.linalg.norm(b[:, other])
        assert r_own < TRIAD_GAP_OWN[it][f], (f, r_own)
        assert r_own < r_other, (f, r_own, r_other)
    e = lambda f: states[it - 1][FIELDS.index(f)]
    files = np.asarray(fu)
    own, other = (files >= 1) & (files <= 9), files > 9
    w = g["u3"].astype(np.complex128)
    assert (np.linalg.norm((e("u3") - w)[:, own]) / np.linalg.norm(w[:, own])) * 5 < \
        np.linalg.norm((e("u3") - w)[:, other]) / np.linalg.norm(w[:, other])
