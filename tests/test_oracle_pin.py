"""Pins the CPU oracle against the reference's golden run (32x32x153 restart file,
5 iterations, tests/golden/). The reference produced those files with its truncated
triad-list nonlinear term (threshold 3e-9) from a restart field whose kx = 0 plane
is not Hermitian; the oracle restates the pseudo-spectral form. Scalars the goldens
expose are matched to the printed precision; fields are held to the measured gap."""
import json
import os

import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.setup_grid import ChannelParams, build_setup

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("u1", "u2", "u3", "p")


@pytest.fixture(scope="module")
def run5():
    s = build_setup(ChannelParams())
    ic = np.load(os.path.join(GOLD, "ic_0032x0032x0153.npz"))
    o = Oracle(s)
    o.set_state(*[ic[f] for f in FIELDS])
    o.set_scalars(t=0.0, mpgx=-3.0675e-3, iter=0)
    sc0 = o.scalars()
    states, scal = [], []
    for _ in range(5):
        o.step()
        states.append(o.get_state())
        scal.append(o.scalars())
    return sc0, states, scal


def test_initial_scalars_exact(run5):
    sc0, _, _ = run5
    h = json.load(open(os.path.join(GOLD, "hist_0032x0032x0153.json")))
    assert sc0["err"] == h[0]["err"]          # divergence of the restart field
    assert sc0["Qx"] == h[0]["Qx"]            # flow rate of mode (0,0)


def test_first_step_dt_and_cfl(run5):
    _, _, scal = run5
    h = json.load(open(os.path.join(GOLD, "hist_0032x0032x0153.json")))
    assert scal[0]["dtc"] == pytest.approx(h[1]["dtc"], rel=1e-14)   # CFL max over physical u, w
    for k in range(5):
        assert scal[k]["t"] == h[k + 1]["t"]                         # dt = 2.5 dtv, exact
        assert scal[k]["err"] < 1e-14                                 # projection: div ~ 1e-16


def test_flow_rate_history(run5):
    _, _, scal = run5
    h = json.load(open(os.path.join(GOLD, "hist_0032x0032x0153.json")))
    for k in range(5):
        assert scal[k]["Qx"] == pytest.approx(h[k + 1]["Qx"], rel=2e-8 * (k + 1))


# measured oracle-vs-golden relative L2 gaps (triad-list truncation + kx=0 handling),
# with 25 % headroom; they grow linearly with the number of steps
GAP_IT1 = {"u1": 7.1e-4, "u2": 5.1e-3, "u3": 1.1e-2, "p": 3.5e-1}
GAP_IT5 = {"u1": 2.9e-3, "u2": 2.4e-2, "u3": 4.8e-2, "p": 3.7e-1}


@pytest.mark.parametrize("it,gap", [(1, GAP_IT1), (5, GAP_IT5)])
def test_fields_within_measured_gap(run5, it, gap):
    _, states, _ = run5
    g = np.load(os.path.join(GOLD, f"golden_it{it}.npz"))
    for f, a in zip(FIELDS, states[it - 1]):
        b = g[f].astype(np.complex128)
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel < 1.25 * gap[f], (f, rel)
    # the mean flow (mode (0,0) of u) is pinned much tighter
    a0 = states[it - 1][0][0].real
    b0 = g["u1"][0].real
    assert np.abs(a0 - b0).max() / np.abs(b0).max() < 3e-4 * it
