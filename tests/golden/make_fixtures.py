"""Extract the golden vectors of the reference's 32x32x153 case into small fixtures.

Reads (only when run by hand, in a checkout that has the reference):
  <ref>/input/{u1,u2,u3,p}_0032x0032x0153_t00000.dat     initial state (restart file)
  <ref>/output/{u1,u2,u3,p}_0032x0032x0153_t00052.dat    state after iteration 1
  <ref>/output/{u1,u2,u3,p}_0032x0032x0153_t00264.dat    state after iteration 5
  <ref>/output/hist_0032x0032x0153.dat                   history records (FOU3D.f90:3064-3070)
Writes next to this file:
  ic_0032x0032x0153.npz       complex128 cfield arrays + y-grid headers (float64, exact)
  golden_it1.npz, golden_it5.npz  complex64 cfield arrays (the tests compare at ~1e-3)
  hist_0032x0032x0153.json    the last history records of the run (iter 0..5)
Usage: python tests/golden/make_fixtures.py /path/to/reference
"""
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from rnl_multiblock_nofft_gb300.planefile import read_planefile  # noqa: E402


def cfield(pf):
    return np.ascontiguousarray(pf.data.reshape(pf.data.shape[0], -1).T)


def main(ref):
    fields = ("u1", "u2", "u3", "p")
    pfs = {f: read_planefile(os.path.join(ref, "input", f"{f}_0032x0032x0153_t00000.dat")) for f in fields}
    np.savez_compressed(os.path.join(HERE, "ic_0032x0032x0153.npz"),
                        **{f: cfield(pfs[f]) for f in fields},
                        yu=pfs["u1"].y, dthdyu=pfs["u1"].dthdy, yv=pfs["u2"].y, dthdyv=pfs["u2"].dthdy,
                        N=pfs["u1"].N, dthetavi=pfs["u1"].dthetavi)
    for it, tag in ((1, "00052"), (5, "00264")):
        g = {f: read_planefile(os.path.join(ref, "output", f"{f}_0032x0032x0153_t{tag}.dat")) for f in fields}
        np.savez_compressed(os.path.join(HERE, f"golden_it{it}.npz"),
                            **{f: cfield(g[f]).astype(np.complex64) for f in fields},
                            t=g["u1"].t, iter=g["u1"].iter)
    raw = open(os.path.join(ref, "output", "hist_0032x0032x0153.dat"), "rb").read()
    off, recs = 0, []
    while off < len(raw):
        (n,) = struct.unpack_from("<i", raw, off)
        r = raw[off + 4: off + 4 + n]
        off += 8 + n
        if n == 80:
            fl, it, t, dtv, dtc, dt, err, Qx, mpgx, Umax, Uslip = struct.unpack("<2i9d", r)
            recs.append(dict(iter=it, t=t, dtv=dtv, dtc=dtc, dt=dt, err=err, Qx=Qx, mpgx=mpgx, Umax=Umax, Uslip=Uslip))
    # the last run in the file: iterations 0..5 (consecutive), taken from the tail
    tail = {}
    for r in recs[::-1]:
        if r["iter"] in tail or r["iter"] > 5:
            if len(tail) == 6:
                break
            continue
        tail[r["iter"]] = r
    with open(os.path.join(HERE, "hist_0032x0032x0153.json"), "w") as f:
        json.dump([tail[k] for k in sorted(tail)], f, indent=1)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LH_REFERENCE_DIR", "")
    if not ref:
        sys.exit("usage: make_fixtures.py REFERENCE_CHECKOUT (or set LH_REFERENCE_DIR)")
    main(ref)
