"""lh_history_record (the scalar record of record_out, FOU3D.f90:3040-3070) on the GPU against
the oracle's state and scalars after two steps: Qx (flowrateIm), Umax (maxvel), the slip
velocity and the time-integration scalars; then the records written to a history file and
read back."""
import numpy as np
import pytest

from oracle import Oracle
from rnl_multiblock_nofft_gb300.historyfile import HistoryFile, history_name, read_history
from rnl_multiblock_nofft_gb300.native import GpuChannel
from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

pytestmark = pytest.mark.gpu


def expected(s, u1, sc):
    """The record from the oracle's state, restated from record_out / maxvel / flowrateIm."""
    u = u1[0].real                      # mode (0,0) of u1, level index j + dny
    d = s.dny
    j = np.arange(1, s.nn + 2)
    Qx = float(np.sum((s.yv[j + d] - s.yv[j - 1 + d]) * u[j + d]))
    Umax = max(0.0, float(np.max(u[d:d + s.nn + 3])))
    y0, y1 = s.yu[d], s.yu[1 + d]
    Uslip = (u[1 + d] * (-1.0 - y0) + u[d] * (y1 + 1.0)) / (y1 - y0)
    return dict(Qx=Qx, Umax=Umax, Uslip=Uslip, t=sc["t"], dt=sc["dt"], dtc=sc["dtc"], mpgx=sc["mpgx"],
                QxT=sc["QxT"], iter=sc["iter"])


@pytest.mark.parametrize("name", ["C0", "SP"])
def test_history_record_matches_oracle(cuda_ok, name, tmp_path):
    s = workload_setup(name)
    st = initial_field(s, 31)
    o = Oracle(s)
    o.set_state(*st)
    o.set_scalars(**initial_scalars(s))
    g = GpuChannel(s, "fp64")
    g.upload_state(*st)
    g.set_scalars(**initial_scalars(s))
    path = str(tmp_path / history_name(s))
    hf = HistoryFile(path, s, 0.0, s.p.mpgx)
    recs = []
    for it in range(2):
        o.step()
        g.step()
        g.synchronize()
        r = g.history_record()
        ex = expected(s, o.get_state()[0], o.scalars())
        assert r["iter"] == ex["iter"] == it + 1
        assert r["flag_ctpress"] == s.p.flpress
        for k in ("Qx", "Umax", "t", "dt", "dtc", "QxT"):
            assert r[k] == pytest.approx(ex[k], rel=1e-12, abs=1e-300), k
        # flowrate_corr's g = (QxT - Qx0) / Qx1 cancels about six digits (Qx0 is within ~1e-6 of
        # QxT), so mpgx carries round-off amplified ~1e6 times: the oracle's and the GPU's agree
        # to ~1e-10 relative
        assert r["mpgx"] == pytest.approx(ex["mpgx"], rel=1e-9)
        assert r["Uslip"] == pytest.approx(ex["Uslip"], rel=1e-9, abs=1e-14)
        assert r["dtv"] == s.dtv
        assert r["err"] < 1e-12
        if s.p.flpress == 0:
            assert np.isfinite(r["dgx"]) and r["dgx"] != 0.0
        hf.append(r)
        recs.append(r)
    _, _, back = read_history(path)
    assert len(back) == 2
    for a, b in zip(recs, back):
        for k in b:
            assert b[k] == a[k], k
