"""Triad interaction lists of the as-run nonlinear term.

The reference computes the velocity products of its reduced (restricted nonlinear)
model not with transforms but as spectral convolutions over lists of "important"
triads (ops_in_planes + nonlinInter, FOU3D.f90:1724-2088). One lists file per plane
pair of the symmetric channel (nonlinRead, start.f90:2983-3069) holds nine lists, one
per product, in the order uu, uv, uw, vu, vv, vw, wu, wv, ww (the first letter is the
passive field, FOU3D.f90:1835). A triad (la, ka, lp, kp) adds u_a(la, ka) u_p(lp, kp)
to mode (la + lp, ka + kp) of the product and, mirrored, u_a(la, -ka) u_p(lp, -kp) to
(la + lp, -(ka + kp)); negative x-modes are conjugates of the stored ones.

File format (Fortran `access='stream'`, little-endian): int32[3] = N1/2-1, N2/2-1 and
the file number j; then nine records of int32 type, int32 L and int8 list(L, 4) stored
column-major (la[L], ka[L], lp[L], kp[L]).
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field

import numpy as np

TYPES = ("uu", "uv", "uw", "vu", "vv", "vw", "wu", "wv", "ww")
U_TYPES = (1, 3, 5, 7, 9)   # computed on u (cell-centre) planes, FOU3D.f90:1845-1849
V_TYPES = (2, 4, 6, 8)      # computed on v (face) planes, FOU3D.f90:1943-1946


@dataclass
class TriadFile:
    nx: int
    nz: int
    j: int
    lists: list = field(default_factory=list)   # 9 int8 arrays (L, 4): la, ka, lp, kp


def read_triad_file(path: str) -> TriadFile:
    """Reads one lists file (nonlinRead's record sequence, start.f90:3035-3064)."""
    with open(path, "rb") as f:
        data = f.read()
    nx, nz, j = struct.unpack_from("<3i", data, 0)
    off = 12
    lists = [None] * 9
    for _ in range(9):
        typ, L = struct.unpack_from("<2i", data, off)
        off += 8
        if not 1 <= typ <= 9 or L < 0 or off + 4 * L > len(data):
            raise ValueError(f"{path}: bad list record (type {typ}, length {L})")
        a = np.frombuffer(data, dtype=np.int8, count=4 * L, offset=off).reshape(4, L).T
        lists[typ - 1] = np.ascontiguousarray(a)
        off += 4 * L
    if any(x is None for x in lists):
        raise ValueError(f"{path}: a list type is missing")
    return TriadFile(nx, nz, j, lists)


def write_triad_file(path: str, tf: TriadFile) -> None:
    with open(path, "wb") as f:
        f.write(struct.pack("<3i", tf.nx, tf.nz, tf.j))
        for t in range(9):
            a = np.asarray(tf.lists[t], dtype=np.int8).reshape(-1, 4)
            f.write(struct.pack("<2i", t + 1, len(a)))
            f.write(np.ascontiguousarray(a.T).tobytes())


def complete_list(nx: int, nz: int) -> np.ndarray:
    """Every triad a lists file can hold: sources (la, ka), (lp, kp) with |l| <= nx,
    |k| <= nz, neither the (0, 0) mode (linear advection covers those, FOU3D.f90:1785-1800),
    target la + lp in 0..nx and ka + kp in 0..nz, not (0, 0) (the zeroth-mode loop covers
    it, FOU3D.f90:1755-1772). The reference's thresholded lists are subsets of this set.
    Order: target x-mode, target z-mode, la, ka."""
    la = np.arange(-nx, nx + 1)
    ka = np.arange(-nz, nz + 1)
    LA, KA = np.meshgrid(la, ka, indexing="ij")
    LA, KA = LA.ravel(), KA.ravel()
    out = []
    for lt in range(nx + 1):
        for kt in range(nz + 1):
            if lt == 0 and kt == 0:
                continue
            LP, KP = lt - LA, kt - KA
            ok = (np.abs(LP) <= nx) & (np.abs(KP) <= nz)
            ok &= ~((LA == 0) & (KA == 0)) & ~((LP == 0) & (KP == 0))
            out.append(np.stack([LA[ok], KA[ok], LP[ok], KP[ok]], axis=1))
    return np.concatenate(out).astype(np.int8)


def plane_files(s) -> tuple[np.ndarray, np.ndarray]:
    """File number (1-based, 0 = none) used by every u level and v level of a setup.

    nonlinRead reads file jread = j for j <= (Ngal(3)+1)/2, else Ngal(3)+1-j
    (start.f90:3019-3023), for the list index j; ops_in_planes takes index j-1 for
    u planes above the centre (FOU3D.f90:1838-1842) and j for v planes. Ngal(3) is the
    input's ny - 2 (start.f90:106-107)."""
    ng3 = int(s.nn)
    half = (ng3 + 1) // 2
    n3_0, n4_0 = int(s.N[2, 0]), int(s.N[3, 0])

    def jread(jidx):
        return jidx if jidx <= half else ng3 + 1 - jidx

    fu = np.zeros(s.nyu, np.int32)
    fv = np.zeros(s.nyv, np.int32)
    for q in range(1, s.nyu - 1):
        j = q + n4_0
        jidx = j - 1 if j > half else j
        fu[q] = jread(jidx)
    for q in range(1, s.nyv - 1):
        fv[q] = jread(q + n3_0)
    if (fu[1:-1] < 1).any() or (fv[1:-1] < 1).any():
        raise ValueError("triad lists exist for planes 1..(ny-1)/2 only: the immersed region "
                         "(dny > 0) has no lists file")
    return fu, fv


class TriadLists:
    """The lists of one channel: file number -> nine int8 (L, 4) arrays."""

    def __init__(self, nx: int, nz: int, files: dict):
        self.nx, self.nz = int(nx), int(nz)
        self.files = files

    @staticmethod
    def check_header(s, nx: int, nz: int):
        if nx != s.N1 // 2 - 1:
            raise ValueError("nx number does not agree between list and simulation")
        if nz != s.N2 // 2 - 1:
            raise ValueError("nz number does not agree between list and simulation")

    @classmethod
    def from_dir(cls, s, dirlist: str, heading: str = "full_y") -> "TriadLists":
        """Loads the files a setup needs, as nonlinRead does (dirlist + heading + 'NN.dat')."""
        fu, fv = plane_files(s)
        need = sorted(set(fu[1:-1].tolist()) | set(fv[1:-1].tolist()))
        files = {}
        nx = nz = None
        for j in need:
            tf = read_triad_file(os.path.join(dirlist, f"{heading}{j:02d}.dat"))
            cls.check_header(s, tf.nx, tf.nz)
            if tf.j != j:
                raise ValueError("something wrong with the j index of the list")
            nx, nz = tf.nx, tf.nz
            files[j] = tf.lists
        return cls(nx, nz, files)

    @classmethod
    def complete(cls, s) -> "TriadLists":
        """Complete lists (threshold zero) for every plane: all files share one list."""
        nx, nz = s.N1 // 2 - 1, s.N2 // 2 - 1
        full = complete_list(nx, nz)
        fu, fv = plane_files(s)
        need = sorted(set(fu[1:-1].tolist()) | set(fv[1:-1].tolist()))
        return cls(nx, nz, {j: [full] * 9 for j in need})

    @classmethod
    def thinned(cls, s, keep: float, seed: int) -> "TriadLists":
        """Seeded random subsets of the complete list, a different subset per file and
        type, in shuffled order: synthetic stand-ins for thresholded lists."""
        nx, nz = s.N1 // 2 - 1, s.N2 // 2 - 1
        full = complete_list(nx, nz)
        fu, fv = plane_files(s)
        need = sorted(set(fu[1:-1].tolist()) | set(fv[1:-1].tolist()))
        rng = np.random.default_rng(seed)
        files = {}
        for j in need:
            ls = []
            for _ in range(9):
                m = rng.random(len(full)) < keep
                sel = full[m]
                ls.append(np.ascontiguousarray(sel[rng.permutation(len(sel))]))
            files[j] = ls
        return cls(nx, nz, files)

    def with_files(self, other: "TriadLists") -> "TriadLists":
        """These lists, with the files of `other` replacing same-numbered ones."""
        files = dict(self.files)
        files.update(other.files)
        return TriadLists(self.nx, self.nz, files)

    def n_triads(self) -> int:
        return sum(len(a) for ls in self.files.values() for a in ls)

    def pack(self, s) -> dict:
        """Arrays for lh_config's triad fields. Identical list arrays are stored once."""
        fu, fv = plane_files(s)
        nums = sorted(self.files)
        index = {j: i for i, j in enumerate(nums)}
        off = np.zeros((len(nums), 9), np.int64)
        ln = np.zeros((len(nums), 9), np.int64)
        chunks, seen, pos = [], {}, 0
        for i, j in enumerate(nums):
            for t in range(9):
                a = self.files[j][t]
                key = id(a)
                if key not in seen:
                    seen[key] = pos
                    chunks.append(np.ascontiguousarray(np.asarray(a, np.int8).reshape(-1, 4).T).reshape(-1))
                    pos += len(a)
                off[i, t] = seen[key]
                ln[i, t] = len(a)
        data = np.concatenate(chunks) if chunks else np.zeros(4, np.int8)
        missing = [int(j) for j in set(fu[1:-1].tolist()) | set(fv[1:-1].tolist()) if j not in index]
        if missing:
            raise ValueError(f"lists files missing for planes {sorted(missing)}")
        set_u = np.array([index[int(j)] if j > 0 else -1 for j in fu], np.int32)
        set_v = np.array([index[int(j)] if j > 0 else -1 for j in fv], np.int32)
        return dict(nx=self.nx, nz=self.nz, off=off, len=ln, data=data, set_u=set_u, set_v=set_v)
