"""History file (hist_*.dat) writer and reader: the header and record layout of
start.f90:246-253 / FOU3D.f90:3064-3070, round trip of the reference run's records (the
golden fixture), and byte equality with the reference's own file when LH_REFERENCE_DIR names
a checkout."""
import json
import os

import numpy as np
import pytest

from rnl_multiblock_nofft_gb300.historyfile import (HistoryFile, header_bytes, history_name, read_history,
                                                    record_bytes)
from rnl_multiblock_nofft_gb300.planefile import _records
from rnl_multiblock_nofft_gb300.setup_grid import ChannelParams, build_setup

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("LH_REFERENCE_DIR", "")
# N(4, 0:4) of the reference's 32x32x153 run, as its history file stores it (column-major)
REF_N = [0, 0, 0, 0, 32, 32, 29, 30, 32, 32, 122, 122, 32, 32, 151, 152, -2, 0, 0, 0]


def golden_records():
    recs = json.load(open(os.path.join(HERE, "golden", "hist_0032x0032x0153.json")))
    return [dict(flag_ctpress=1, **r) for r in recs]


def test_header_layout_of_the_reference_case(tmp_path):
    s = build_setup(ChannelParams())
    assert history_name(s) == "hist_0032x0032x0153.dat"
    hb = header_bytes(s, 0.0, s.p.mpgx)
    recs = list(_records(hb))
    assert [len(r) for r in recs] == [44, 80]
    assert list(np.frombuffer(recs[1], "<i4")) == REF_N


def test_round_trip_of_the_golden_records(tmp_path):
    s = build_setup(ChannelParams())
    path = str(tmp_path / history_name(s))
    h = HistoryFile(path, s, 0.0, s.p.mpgx)
    recs = golden_records()
    for r in recs:
        h.append(r)
    HistoryFile(path, s, 99.0, 0.0)   # an existing file is appended to, not re-headed
    h.append(dict(recs[-1], flag_ctpress=0, QxT=1.5, dgx=-1e-6))
    hdr, N, got = read_history(path)
    assert hdr["Re"] == s.p.Re and hdr["t"] == 0.0 and hdr["nband"] == 3
    assert list(N.T.ravel()) == REF_N
    assert len(got) == len(recs) + 1
    for a, b in zip(recs, got):
        for k, v in a.items():
            assert b[k] == v, k
    assert got[-1]["QxT"] == 1.5 and got[-1]["dgx"] == -1e-6
    assert len(record_bytes(recs[0])) == 8 + 80 and len(record_bytes(got[-1])) == 8 + 96


def test_bytes_equal_the_reference_file():
    if not REF_DIR:
        pytest.skip("set LH_REFERENCE_DIR to a reference checkout to compare its history file")
    raw = open(os.path.join(REF_DIR, "output", "hist_0032x0032x0153.dat"), "rb").read()
    s = build_setup(ChannelParams())
    hb = header_bytes(s, 0.0, s.p.mpgx)
    assert raw[:len(hb)] == hb
    run = b"".join(record_bytes(r) for r in golden_records())   # iterations 0..5 of one run
    assert run in raw
