"""Extract the reference's triad interaction lists that exist (files 1-9 of the 3e-9 set)
into a small fixture.

Every list of those files is a subset of the complete triad enumeration
(triads.complete_list), so each is stored as a bit mask over that enumeration;
the lists are rebuilt in enumeration order (the file's own order only changes the
order of the floating-point sums).

Reads (only when run by hand, in a checkout that has the reference):
  <ref>/3e-9/full_yNN.dat, NN = 01..09        (nonlinRead's files, start.f90:2983-3069)
Writes next to this file:
  triads_3e-9_y01-y09.npz   masks uint8 [9 files][9 types][bytes], lengths int64 [9][9],
                            headers int32 [9][3], sha256 of each source file
Usage: python tests/golden/make_triad_fixture.py /path/to/reference
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from rnl_multiblock_nofft_gb300.triads import complete_list, read_triad_file  # noqa: E402

FIXTURE = os.path.join(HERE, "triads_3e-9_y01-y09.npz")


def triad_keys(a: np.ndarray, nx: int, nz: int) -> np.ndarray:
    a = a.astype(np.int64)
    wx, wz = 2 * nx + 1, 2 * nz + 1
    return (((a[:, 0] + nx) * wz + (a[:, 1] + nz)) * wx + (a[:, 2] + nx)) * wz + (a[:, 3] + nz)


def main(ref):
    nx = nz = 15
    full = complete_list(nx, nz)
    fk = triad_keys(full, nx, nz)
    order = np.argsort(fk)
    masks, lens, heads, shas = [], [], [], []
    for j in range(1, 10):
        path = os.path.join(ref, "3e-9", f"full_y{j:02d}.dat")
        tf = read_triad_file(path)
        assert (tf.nx, tf.nz, tf.j) == (nx, nz, j)
        fm, fl = [], []
        for t in range(9):
            k = triad_keys(tf.lists[t], nx, nz)
            pos = np.searchsorted(fk, k, sorter=order)
            idx = order[np.minimum(pos, len(fk) - 1)]
            assert (fk[idx] == k).all(), "a listed triad is outside the complete enumeration"
            m = np.zeros(len(full), bool)
            m[idx] = True
            assert m.sum() == len(k), "duplicate triads"
            fm.append(np.packbits(m))
            fl.append(len(k))
        masks.append(fm)
        lens.append(fl)
        heads.append((tf.nx, tf.nz, tf.j))
        shas.append(hashlib.sha256(open(path, "rb").read()).hexdigest())
    np.savez_compressed(FIXTURE, masks=np.array(masks, np.uint8), lengths=np.array(lens, np.int64),
                        headers=np.array(heads, np.int32), sha256=np.array(shas))


def load_fixture():
    """{file number: nine int8 (L, 4) lists} rebuilt from the fixture."""
    z = np.load(FIXTURE)
    nx, nz = 15, 15
    full = complete_list(nx, nz)
    out = {}
    for f in range(z["masks"].shape[0]):
        j = int(z["headers"][f, 2])
        ls = []
        for t in range(9):
            m = np.unpackbits(z["masks"][f, t])[: len(full)].astype(bool)
            assert m.sum() == z["lengths"][f, t]
            ls.append(np.ascontiguousarray(full[m]))
        out[j] = ls
    return out


if __name__ == "__main__":
    main(sys.argv[1])
