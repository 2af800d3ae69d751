"""Host-side set-up of one channel: the data the RK3 substep consumes.

This restates the set-up half of the reference (everything `start` computes
before the time loop) for a single process that owns every spectral column and
every physical plane:

* the stretched staggered y-grid and its metrics (start.f90:693-1077, `ygrid`);
* the Fourier wavenumbers k1F/k2F (start.f90:1079-1194, `def_k`);
* the Le & Moin RK3 coefficients and the viscous time-step limit
  (start.f90:418-456);
* the band limits N(3:4,0:3), `jlim` and the column list of the long columns
  (start.f90:1490-1734, `proc_lims_columns`);
* the ghost/interface weights `gridweighting*` (start.f90:537-559);
* the immersed-boundary lists of the square-post texture
  (boundary_post_coll.f90:1-474, called through `getbounds`, start.f90:1196-1488).

All arrays indexed by a y-level carry an offset: element ``[j + dny]`` holds the
reference's level ``j`` (levels start at ``N(3,0) = N(4,0) = -dny``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

UGRID, VGRID, PGRID = 2, 1, 3


def fpow(x: float, n: int) -> float:
    """``x**n`` for a real base and a run-time integer exponent, evaluated the
    way a Fortran run-time library does it (binary exponentiation), so the
    grid matches the reference bit for bit."""
    if n == 0:
        return 1.0
    neg = n < 0
    n = abs(n)
    result = None
    base = float(x)
    while n:
        if n & 1:
            result = base if result is None else result * base
        n >>= 1
        if n:
            base = base * base
    return 1.0 / result if neg else result


@dataclass
class ChannelParams:
    """The fields of the reference's ``input.in`` (start.f90:62-220) that the
    substep depends on. Names follow the input file."""
    Re: float = 3250.0
    alp: float = 1.0
    bet: float = 2.0
    Ngalx: tuple = (48, 48)       # (wall bands, core band)
    Ngalz: tuple = (48, 48)
    ny: int = 153
    dyq: float = 10.0
    pp: int = 5
    CFL: float = 0.7
    flpress: int = 1              # 0 constant flow rate, 1 constant pressure gradient
    mpgx: float = -3.0675e-3
    Kib: float = 1.0
    geometry_type: int = 0        # 0 smooth, 2 square posts (immersed boundaries)
    ntilex: int = 1
    ntilez: int = 1
    posth: float = 0.5            # post height / post spacing (input units)
    npeakx: int = 7
    npeakz: int = 7
    bslpu1: float = 0.0
    bslpu3: float = 0.0
    ib_enable: bool = True        # apply the immersed-boundary forcing when geometry_type == 2


@dataclass
class ChannelSetup:
    p: ChannelParams
    N: np.ndarray                 # (4, 5) int: N(1:4, 0:4) as in the reference
    Ngal: np.ndarray
    dny: int
    nn: int                       # N(3,nband) before the immersed region is added
    yu: np.ndarray
    yv: np.ndarray
    dthdyu: np.ndarray
    dthdyv: np.ndarray
    dyu2i: np.ndarray             # (3, nyu)
    dyv2i: np.ndarray             # (3, nyv)
    dtheta: float
    dthetai: float
    ddthetavi: float
    posth_abs: float
    k1x: np.ndarray               # imaginary part of k1F_x(i), i = 0..N1/2
    k2x: np.ndarray
    k1z: np.ndarray               # imaginary part of k1F_z(k), k = 1..N2 (0-based here)
    k2z: np.ndarray
    aRK: np.ndarray
    bRK: np.ndarray
    cRK: np.ndarray
    dRK: np.ndarray
    gRK: np.ndarray
    dtv: float
    gw: np.ndarray                # gridweighting(3, 2)
    gw_interp: np.ndarray         # gridweighting_interp(3, 2)
    gw_bc_u1: float
    gw_bc_u3: float
    jlim: np.ndarray              # (2, 3, 3): jlim(lo/hi, grid 1..3, band 1..3)
    list_ib: dict = field(default_factory=dict)   # grid -> (n, 6) int32 (i,k,j,i1,k1,j1)
    A_ib: dict = field(default_factory=dict)      # grid -> (n,) float64

    # ---- convenience sizes (single-resolution channels) ----
    @property
    def N1(self) -> int:
        return int(self.N[0, 1])

    @property
    def N2(self) -> int:
        return int(self.N[1, 1])

    @property
    def G1(self) -> int:
        return int(self.Ngal[0, 1])

    @property
    def G2(self) -> int:
        return int(self.Ngal[1, 1])

    @property
    def nyu(self) -> int:
        """u levels N(4,0) .. N(4,3)+1 (ghosts included)."""
        return int(self.N[3, 3] + 1 - self.N[3, 0] + 1)

    @property
    def nyv(self) -> int:
        """v levels N(3,0) .. N(3,3)+1 (walls included)."""
        return int(self.N[2, 3] + 1 - self.N[2, 0] + 1)

    @property
    def ncols(self) -> int:
        return (self.N1 // 2 + 1) * self.N2

    @property
    def multiblock(self) -> bool:
        return bool(self.N[0, 1] != self.N[0, 2] or self.N[1, 1] != self.N[1, 2])

    # ---- core band (band 2); equal to the above for one resolution ----
    @property
    def N1c(self) -> int:
        return int(self.N[0, 2])

    @property
    def N2c(self) -> int:
        return int(self.N[1, 2])

    @property
    def G1c(self) -> int:
        return int(self.Ngal[0, 2])

    @property
    def G2c(self) -> int:
        return int(self.Ngal[1, 2])

    def is_long(self) -> np.ndarray:
        """Per column of the wall-band mode grid (row kz index r = 0..N2-1 in k1F_z
        order, kx = 0..N1/2 fastest): True for the long columns (modes the core band
        also holds, start.f90:1596-1609), False for the short ones (wall bands only)."""
        N1h, N2 = self.N1 // 2 + 1, self.N2
        r = np.arange(N2)[:, None]
        kx = np.arange(N1h)[None, :]
        rz = (r < self.N2c // 2) | (r >= N2 - self.N2c // 2)
        return ((kx <= self.N1c // 2) & rz).reshape(-1)

    def band_cols(self, band: int) -> np.ndarray:
        """Columns of band 1..3 as indices into the wall-band mode grid, in the order of
        columns_i/k with one process (start.f90:1566-1609): row-major over (r, kx)."""
        lng = self.is_long()
        idx = np.arange(lng.size)
        return idx[lng] if band == 2 else idx[~lng]

    def band_levels(self, band: int, grid: int) -> tuple:
        """(lo, hi) array indices (j + dny) of jlim(1:2, grid, band)."""
        lo, hi = self.jlim[:, grid - 1, band - 1]
        return int(lo) + self.dny, int(hi) + self.dny

    def band_shapes(self, band: int):
        """Host cfield shapes of (u1, u2, u3, p) of one band: [columns][levels]."""
        nc = len(self.band_cols(band))
        out = []
        for grid in (UGRID, VGRID, UGRID, PGRID):
            lo, hi = self.band_levels(band, grid)
            out.append((nc, hi - lo + 1))
        return tuple(out)

    def mode_points(self) -> int:
        """Retained mode-points of one substep: sum over the nominal y-levels
        (``ny`` of the configuration, v levels 0..ny-1) of N1*N2 of the level's band."""
        if not self.multiblock:
            return int(self.N1 * self.N2 * self.p.ny)
        j = np.arange(self.p.ny)
        wall = (j <= self.N[2, 1]) | (j > self.N[2, 2])
        return int(np.where(wall, self.N1 * self.N2, self.N1c * self.N2c).sum())


def _ygrid(p: ChannelParams, N: np.ndarray, posth_abs: float):
    """start.f90:693-1077 (`ygrid`), including the order in which the smooth
    'wall grid' overwrites the immersed-region values."""
    nband = 3
    nn = int(N[2, nband]) + 1
    ppp = int(p.pp)
    dyq = float(p.dyq)
    qqq = nn / 2.0
    bbb = (dyq - 1.0) / (qqq * (1.0 - fpow(qqq, ppp - 1)
                                + dyq * ((1.0 - qqq) * fpow(qqq, ppp - 1) - fpow(1.0 - qqq, ppp))))
    aaa = (1.0 - bbb * fpow(qqq, ppp)) / qqq
    dtheta = 1.0
    dthetai = 1.0 / dtheta
    ddthetavi = 1.0 / dtheta
    dy0 = aaa * (1.0 - qqq) + bbb * fpow(1.0 - qqq, ppp) + 1.0

    if p.geometry_type == 2:
        dny = int(math.ceil(posth_abs / dy0))
        sumj = sum(range(-dny, 0))
        ddy = (posth_abs - dy0 * dny) / sumj
    else:
        dny = 0
        ddy = 0.0

    off = dny
    yu = np.zeros(nn + 2 * dny + 2)
    yv = np.zeros(nn + 2 * dny + 1)
    thu = np.zeros(nn + 2 * dny + 2)
    thv = np.zeros(nn + 2 * dny + 1)

    def U(j):
        return j + off

    posth = posth_abs if p.geometry_type == 2 else 0.0
    yv[U(-dny)] = -1.0 - posth
    yu[U(-dny)] = yv[U(-dny)] - dy0 * .5 - ddy * (-dny - .5) * 0.5
    for j in range(-dny + 1, 0):
        yv[U(j)] = yv[U(j - 1)] + dy0 + ddy * (j - 1)
        yu[U(j)] = yu[U(j - 1)] + dy0 + ddy * (j - 1.5)
    if dny > 0:
        yu[U(0)] = yu[U(-1)] + dy0 + ddy * (-1.5)
    else:
        yu[U(0)] = -2 - (aaa * (.5 - qqq) + bbb * fpow(.5 - qqq, ppp))
    for j in range(0, nn + 1):
        yv[U(j)] = aaa * (j - qqq) + bbb * fpow(j - qqq, ppp)
        yu[U(j + 1)] = aaa * (j + .5 - qqq) + bbb * fpow(j + .5 - qqq, ppp)
    for j in range(nn + 1, nn + dny + 1):
        yv[U(j)] = yv[U(j - 1)] + dy0 - ddy * (j - nn)
        yu[U(j)] = -yu[U(nn - j + 1)]
    yu[U(nn + dny + 1)] = -yu[U(-dny)]

    for j in range(-dny, 0):
        thv[U(j)] = dtheta / (dy0 + ddy * (j - .5))
        thu[U(j)] = dtheta / (dy0 + ddy * (j - 1.0))
    if dny > 0:
        thu[U(0)] = dtheta / (dy0 + ddy * (-1.0))
    else:
        thu[U(0)] = 1.0 / (aaa + ppp * bbb * fpow(.5 - qqq, ppp - 1))
    for j in range(0, nn + 1):
        thv[U(j)] = 1.0 / (aaa + ppp * bbb * fpow(j - qqq, ppp - 1))
        thu[U(j + 1)] = 1.0 / (aaa + ppp * bbb * fpow(j + .5 - qqq, ppp - 1))
    for j in range(nn + 1, nn + dny + 1):
        thv[U(j)] = dtheta / (dy0 - ddy * (j - nn + .5))
        thu[U(j)] = thu[U(nn - j + 1)]
    thu[U(nn + dny + 1)] = thu[U(-dny)]
    for j in range(0, -dny - 1, -1):
        thu[U(j)] = thu[U(-j + 1)]
    for j in range(-1, -dny - 1, -1):
        thv[U(j)] = thv[U(-j)]
    for j in range(nn + 1, nn + dny + 1):
        thu[U(j)] = thu[U(nn - j + 1)]
        thv[U(j)] = thv[U(nn - j)]
    thu[U(nn + dny + 1)] = thu[U(-dny)]

    # smooth 'wall grid' pass, which overwrites levels 0..nn+1 of yu and 0..nn of yv
    yu[U(0)] = aaa * (-1.0 + .5 - qqq) + bbb * fpow(-1.0 + .5 - qqq, ppp)
    for j in range(0, nn + 1):
        yv[U(j)] = aaa * (j - qqq) + bbb * fpow(j - qqq, ppp)
        yu[U(j + 1)] = aaa * (j + .5 - qqq) + bbb * fpow(j + .5 - qqq, ppp)
    thu[U(0)] = 1.0 / (aaa + ppp * bbb * fpow(-1.0 + .5 - qqq, ppp - 1))
    for j in range(0, nn + 1):
        thv[U(j)] = 1.0 / (aaa + ppp * bbb * fpow(j - qqq, ppp - 1))
        thu[U(j + 1)] = 1.0 / (aaa + ppp * bbb * fpow(j + .5 - qqq, ppp - 1))

    # second-order finite-difference coefficients
    nyu = yu.size
    nyv = yv.size
    du = np.zeros((3, nyu))
    dv = np.zeros((3, nyv))
    j = -dny
    du[0, U(j)] = 0.0
    du[1, U(j)] = -2.0 / (yu[U(j + 1)] - yu[U(j)]) ** 2
    du[2, U(j)] = 1.0 / (yu[U(j + 1)] - yu[U(j)]) ** 2
    dv[0, U(j)] = 0.0
    dv[1, U(j)] = -2.0 / (yv[U(j + 1)] - yv[U(j)]) ** 2
    dv[2, U(j)] = 1.0 / (yv[U(j + 1)] - yv[U(j)]) ** 2

    def inner(y, d, j):
        d[0, U(j)] = 2.0 / ((y[U(j)] - y[U(j - 1)]) * (y[U(j + 1)] - y[U(j - 1)]))
        d[1, U(j)] = -2.0 / ((y[U(j + 1)] - y[U(j)]) * (y[U(j)] - y[U(j - 1)]))
        d[2, U(j)] = 2.0 / ((y[U(j + 1)] - y[U(j)]) * (y[U(j + 1)] - y[U(j - 1)]))

    for j in range(-dny + 1, nn + dny):
        inner(yu, du, j)
        inner(yv, dv, j)
    j = nn + dny
    inner(yu, du, j)
    dv[0, U(j)] = 1.0 / (yv[U(j)] - yv[U(j - 1)]) ** 2
    dv[1, U(j)] = -2.0 / (yv[U(j)] - yv[U(j - 1)]) ** 2
    dv[2, U(j)] = 0.0
    j = nn + dny + 1
    du[0, U(j)] = 1.0 / (yu[U(j)] - yu[U(j - 1)]) ** 2
    du[1, U(j)] = -2.0 / (yu[U(j)] - yu[U(j - 1)]) ** 2
    du[2, U(j)] = 0.0
    return dict(dny=dny, yu=yu, yv=yv, thu=thu, thv=thv, du=du, dv=dv, dtheta=dtheta,
                dthetai=dthetai, ddthetavi=ddthetavi)


def _post_lists(p: ChannelParams, N: np.ndarray, Ngal: np.ndarray, nn: int, dny: int, yu, yv):
    """boundary_post_coll.f90:80-467: solid points of one tile of square posts on
    each wall, replicated over ntilex x ntilez tiles. Entries are
    (i, k, j, i1, k1, j1), 1-based physical-plane indices and reference y-levels;
    forcing at (i,k,j) is Kib/dt * (A * u(i1,k1,j1) - u(i,k,j))."""
    if Ngal[0, 1] % p.ntilez != 0 or Ngal[1, 1] % p.ntilez != 0:
        raise ValueError("Ngal must be a multiple of the number of tiles")
    dnx = int(Ngal[0, 1]) // p.ntilex
    dnz = int(Ngal[1, 1]) // p.ntilez
    npx, npz = p.npeakx, p.npeakz
    off = dny

    def corner_points():
        pts = []
        for i in range(1, (npx + 1) // 2 + 1):
            for k in range(1, (npz + 1) // 2 + 1):
                pts.append((i, k))
            for k in range((npz + 1) // 2 + 1, npz + 1):
                pts.append((i, dnz - npz + k))
        for i in range((npx + 1) // 2 + 1, npx + 1):
            ii = dnx - npx + i
            for k in range(1, (npz + 1) // 2 + 1):
                pts.append((ii, k))
            for k in range((npz + 1) // 2 + 1, npz + 1):
                pts.append((ii, dnz - npz + k))
        return pts

    pts = corner_points()
    lists = {UGRID: ([], []), VGRID: ([], [])}
    # lower wall: planes -dny+1 .. 0; the tip plane (j1 = 0) of u interpolates to j1+1
    low_u, low_v, low_Au = [], [], []
    for j in range(1, dny + 1):
        j1 = int(N[2, 0]) + j
        for (i, k) in pts:
            if j < dny:
                low_u.append((i, k, j1, i, k, j1)); low_Au.append(0.0)
            else:
                low_u.append((i, k, j1, i, k, j1 + 1))
                low_Au.append((yu[j1 + off] - yv[j1 + off]) / (yu[j1 + 1 + off] - yv[j1 + off]))
            low_v.append((i, k, j1, i, k, j1))
    up_u, up_v, up_Au = [], [], []
    for j in range(1, dny + 1):
        j1 = nn + j
        for (i, k) in pts:
            if j == 1:
                up_u.append((i, k, j1 + 1, i, k, j1))
                up_Au.append((yu[j1 + 1 + off] - yv[j1 + off]) / (yu[j1 + off] - yv[j1 + off]))
            else:
                up_u.append((i, k, j1 + 1, i, k, j1 + 1)); up_Au.append(0.0)
            up_v.append((i, k, j1, i, k, j1))

    def replicate(base, A):
        out, outA = [], []
        for ix in range(p.ntilex):
            for iz in range(p.ntilez):
                for (e, a) in zip(base, A):
                    i, k, j, i1, k1, j1 = e
                    out.append((i + dnx * ix, k + dnz * iz, j, i1 + dnx * ix, k1 + dnz * iz, j1))
                    outA.append(a)
        return out, outA

    lu, lAu = replicate(low_u, low_Au)
    uu, uAu = replicate(up_u, up_Au)
    lv, lAv = replicate(low_v, [0.0] * len(low_v))
    uv, uAv = replicate(up_v, [0.0] * len(up_v))
    list_ib = {UGRID: np.array(lu + uu, dtype=np.int32).reshape(-1, 6),
               VGRID: np.array(lv + uv, dtype=np.int32).reshape(-1, 6)}
    A_ib = {UGRID: np.array(lAu + uAu, dtype=np.float64),
            VGRID: np.array(lAv + uAv, dtype=np.float64)}
    return list_ib, A_ib


def build_setup(p: ChannelParams) -> ChannelSetup:
    nband = 3
    Ngal = np.zeros((4, nband + 2), dtype=np.int64)
    Ngal[0, 1] = p.Ngalx[0]; Ngal[0, 2] = p.Ngalx[1]; Ngal[0, 3] = p.Ngalx[0]; Ngal[0, 4] = -2
    Ngal[1, 1] = p.Ngalz[0]; Ngal[1, 2] = p.Ngalz[1]; Ngal[1, 3] = p.Ngalz[0]; Ngal[1, 4] = 0
    Ngal[2, nband] = p.ny - 2
    N = Ngal.copy()
    for b in range(1, nband + 1):
        N[0, b] = 2 * (Ngal[0, b] // 3)
        N[1, b] = 2 * (Ngal[1, b] // 3)

    Lz = 2.0 * math.pi / p.bet
    if p.geometry_type == 0:
        posth_abs = 0.0
        h_ny = .25
    elif p.geometry_type == 2:
        post_spacing = Lz / p.ntilez
        posth_abs = p.posth * post_spacing
        h_ny = 1.5 * posth_abs
    else:
        raise ValueError("geometry_type must be 0 (smooth) or 2 (square posts)")

    g = _ygrid(p, N, posth_abs)
    dny = g["dny"]
    yu, yv = g["yu"], g["yv"]
    off = dny
    nn = int(N[2, nband])
    N[2, 0] = -dny
    N[3, 0] = -dny
    # band limits (start.f90:1000-1050)
    j = int(N[2, 0])
    h = yu[0 + off] + h_ny
    while yu[j + off] < h:
        j += 1
    N[2, 1] = j
    N[2, nband - 1] = N[2, nband] - j
    N[2, nband] = nn + dny
    N[3, 1] = N[2, 1] + 1
    N[3, 2] = N[2, 2]
    N[3, 3] = N[2, 3] + 1
    for b in range(0, nband + 2):
        Ngal[2, b] = N[2, b]
        Ngal[3, b] = N[3, b]

    N1, N2 = int(N[0, 1]), int(N[1, 1])
    # def_k (start.f90:1079-1132): imaginary parts of k1F, and k2F
    k1x = np.array([p.alp * i for i in range(N1 // 2 + 1)])
    k2x = np.array([-(p.alp * i) ** 2 for i in range(N1 // 2 + 1)])
    k1z = np.zeros(N2)
    k2z = np.zeros(N2)
    for k in range(1, N2 // 2 + 1):
        k1z[k - 1] = p.bet * (k - 1)
        k2z[k - 1] = -(p.bet * (k - 1)) ** 2
    for k in range(N2 // 2 + 1, N2 + 1):
        k1z[k - 1] = -p.bet * (N2 - k + 1)
        k2z[k - 1] = -(p.bet * (N2 - k + 1)) ** 2

    aRK = np.array([4. / 15., 1. / 15., 1. / 6.])
    bRK = np.array([4. / 15., 1. / 15., 1. / 6.])
    gRK = np.array([8. / 15., 5. / 12., 3. / 4.])
    cRK = np.array([0., -17. / 60., -5. / 12.])
    dRK = np.array([8. / 15., 2. / 15., 1. / 3.])
    dtv = p.Re / (-k2x[N1 // 2] - k2z[N2 // 2 - 1]
                  + 4.0 / (yv[int(N[2, 0]) + 1 + off] - yv[int(N[2, 0]) + off]) ** 2)

    Y = lambda arr, jj: arr[int(jj) + off]
    gw = np.zeros((3, 2))
    gw[0, 0] = -(Y(yv, N[2, 0]) - Y(yu, N[3, 0])) / (Y(yv, N[2, 0]) - Y(yu, N[3, 0] + 1))
    gw[0, 1] = (Y(yu, N[3, 1] + 1) - Y(yv, N[2, 1] + 1)) / (Y(yv, N[2, 1] + 1) - Y(yu, N[3, 1]))
    gw[1, 0] = -(Y(yv, N[2, 0]) - Y(yu, N[3, 0])) / (Y(yv, N[2, 0]) - Y(yu, N[3, 0] + 1))
    gw[1, 1] = (Y(yu, N[3, 3] + 1) - Y(yv, N[2, 3] + 1)) / (Y(yv, N[2, 3] + 1) - Y(yu, N[3, 3]))
    gw[2, 0] = -(Y(yv, N[2, 2]) - Y(yu, N[3, 2])) / (Y(yv, N[2, 2]) - Y(yu, N[3, 2] + 1))
    gw[2, 1] = (Y(yu, N[3, 3] + 1) - Y(yv, N[2, 3] + 1)) / (Y(yv, N[2, 3] + 1) - Y(yu, N[3, 3]))
    thv = g["thv"]
    dd = g["ddthetavi"]
    gwbc = []
    for bsl in (p.bslpu1, p.bslpu3):
        s = bsl * dd * thv[0 + off] * (yu[1 + off] - yu[0 + off])
        gwbc.append(((yu[0 + off] - yv[0 + off]) + s) / ((yu[1 + off] - yv[0 + off]) + s))
    gwi = np.zeros((3, 2))
    gwi[0, 0] = (Y(yu, N[3, 0]) - Y(yu, N[3, 0] + 1)) / (Y(yv, N[2, 0]) - Y(yu, N[3, 0] + 1))
    gwi[1, 0] = gwi[0, 0]
    gwi[2, 0] = (Y(yu, N[3, 2]) - Y(yu, N[3, 2] + 1)) / (Y(yv, N[2, 2]) - Y(yu, N[3, 2] + 1))
    gwi[0, 1] = (Y(yu, N[3, 1] + 1) - Y(yu, N[3, 1])) / (Y(yv, N[2, 1] + 1) - Y(yu, N[3, 1]))
    gwi[1, 1] = (Y(yu, N[3, 3] + 1) - Y(yu, N[3, 3])) / (Y(yv, N[2, 3] + 1) - Y(yu, N[3, 3]))
    gwi[2, 1] = gwi[1, 1]

    # jlim (start.f90:1675-1709); index [lo/hi, grid-1, band-1]
    jlim = np.zeros((2, 3, 3), dtype=np.int64)
    jlim[:, UGRID - 1, 0] = (N[3, 0], N[3, 1] + 1)
    jlim[:, UGRID - 1, 1] = (N[3, 0], N[3, 3] + 1)
    jlim[:, UGRID - 1, 2] = (N[3, 2], N[3, 3] + 1)
    jlim[:, VGRID - 1, 0] = (N[2, 0], N[2, 1] + 1)
    jlim[:, VGRID - 1, 1] = (N[2, 0], N[2, 3] + 1)
    jlim[:, VGRID - 1, 2] = (N[2, 2], N[2, 3] + 1)
    jlim[:, PGRID - 1, 0] = (N[3, 0] + 1, N[3, 1])
    jlim[:, PGRID - 1, 1] = (N[3, 0] + 1, N[3, 3])
    jlim[:, PGRID - 1, 2] = (N[3, 2] + 1, N[3, 3])

    s = ChannelSetup(p=p, N=N, Ngal=Ngal, dny=dny, nn=nn, yu=yu, yv=yv,
                     dthdyu=g["thu"], dthdyv=g["thv"], dyu2i=g["du"], dyv2i=g["dv"],
                     dtheta=g["dtheta"], dthetai=g["dthetai"], ddthetavi=g["ddthetavi"],
                     posth_abs=posth_abs, k1x=k1x, k2x=k2x, k1z=k1z, k2z=k2z,
                     aRK=aRK, bRK=bRK, cRK=cRK, dRK=dRK, gRK=gRK, dtv=dtv,
                     gw=gw, gw_interp=gwi, gw_bc_u1=gwbc[0], gw_bc_u3=gwbc[1], jlim=jlim)
    if p.geometry_type == 2:
        s.list_ib, s.A_ib = _post_lists(p, N, Ngal, nn, dny, yu, yv)
    else:
        s.list_ib = {UGRID: np.zeros((0, 6), np.int32), VGRID: np.zeros((0, 6), np.int32)}
        s.A_ib = {UGRID: np.zeros(0), VGRID: np.zeros(0)}
    return s
