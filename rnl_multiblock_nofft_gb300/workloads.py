"""Named workloads and the seeded synthetic initial field.

No public dataset is involved. The reference's own initial condition (a 32x32x153
restart file) only exists at one size, so every workload starts from a seeded
synthetic field with the shapes of the reference's set-up:

* laminar parabolic u(y) with bulk velocity 1 (centreline 1.5);
* a random Fourier perturbation on the modes |(i, k)| <= kmax, wall envelope
  (1-y^2)^2, amplitude `amp` x centreline velocity, built so that the discrete
  divergence of the reference (littleharsh.f90:237-272) is zero to round-off:
  v is random, (u, w) = i (kx, kz) D / |k|^2 + (kz, -kx) phi, D = dv/dy at the
  centres; ghosts follow v_corr's extrapolation (littleharsh.f90:992-1044);
* p = 0.
"""
from __future__ import annotations

import math

import numpy as np

from .setup_grid import ChannelParams, ChannelSetup, build_setup


def re_tau_params(N: int, ny: int, re_tau: float = 180.0, Re: float = 3250.0, posts: bool = False,
                  post_period: int = 16, post_points: int = 8, post_height_plus: float = 6.0,
                  CFL: float = 0.5, flpress: int = 0, Nz: int | None = None) -> ChannelParams:
    """Reference-style parameters for an N x Nz x ny channel at a given Re_tau
    (u_tau^2 = -mpgx, so Re_tau = Re * sqrt(-mpgx)). With posts: square posts of
    post_points^2 physical points on a period of post_period points, protruding
    post_height_plus wall units (geometry_type 2, boundary_post_coll.f90)."""
    Nz = N if Nz is None else Nz
    G1, G2 = 3 * N // 2, 3 * Nz // 2
    p = ChannelParams(Re=Re, alp=1.0, bet=2.0, Ngalx=(G1, G1), Ngalz=(G2, G2), ny=ny, dyq=10.0, pp=5,
                      CFL=CFL, flpress=flpress, mpgx=-(re_tau / Re) ** 2, Kib=1.0)
    if posts:
        Lz = 2.0 * math.pi / p.bet
        p.geometry_type = 2
        p.ntilex = G1 // post_period
        p.ntilez = G2 // post_period
        p.npeakx = p.npeakz = post_points
        p.posth = (post_height_plus / re_tau) / (Lz / p.ntilez)
    return p


# Workloads: (params factory, description). "C1" is the one the throughput metric is quoted on.
WORKLOADS = {
    "C0": dict(N=32, ny=153, posts=False, flpress=0,
               desc="smooth channel N 32x32, ny 153, Re_tau 180, constant flow rate"),
    "C1": dict(N=256, ny=301, posts=True, flpress=0,
               desc="textured channel N 256x256, ny 301, Re_tau 180, 8x8-point posts on a 16-point period, 6 wall units high"),
    "C1s": dict(N=256, ny=301, posts=False, flpress=0,
                desc="smooth channel N 256x256, ny 301, Re_tau 180"),
    "S": dict(N=16, ny=41, posts=False, flpress=0, desc="small smooth channel N 16x16, ny 41"),
    "SP": dict(N=32, ny=65, posts=True, flpress=0, post_period=8, post_points=4, post_height_plus=20.0,
               desc="small textured channel N 32x32, ny 65, 4x4-point posts on an 8-point period"),
    "M": dict(N=64, ny=97, posts=False, flpress=0, desc="mid smooth channel N 64x64, ny 97"),
    "MP": dict(N=64, ny=97, posts=True, flpress=0, post_period=16, post_points=8, post_height_plus=12.0,
               desc="mid textured channel N 64x64, ny 97, posts"),
    "P": dict(N=192, ny=201, posts=False, flpress=0,
              desc="profiling case: smooth channel N 192x192, ny 201 (state 0.27 GB, above L2)"),
    "P384": dict(N=256, ny=97, posts=False, flpress=0,
                 desc="profiling case at the 384-point transforms: smooth channel N 256x256, ny 97 "
                      "(state 0.26 GB, above L2)"),
    "C4": dict(N=768, Nz=384, ny=385, re_tau=550.0, posts=True, post_period=24, post_points=12,
               post_height_plus=6.0, flpress=0, core=(384, 192),
               desc="multiblock channel: wall bands N 768x384, core band N 384x192, ny 385, Re_tau 550, "
                    "12x12-point posts on a 24-point period, 6 wall units high"),
    "MB": dict(N=32, ny=65, posts=False, flpress=0, core=(16, 16),
               desc="small multiblock channel: wall bands N 32x32, core band N 16x16, ny 65"),
    "MBP": dict(N=32, ny=65, posts=True, flpress=0, post_period=8, post_points=4, post_height_plus=20.0,
                core=(16, 16),
                desc="small multiblock channel with posts: wall bands N 32x32, core N 16x16, ny 65"),
}


def workload_params(name: str) -> ChannelParams:
    w = dict(WORKLOADS[name])
    w.pop("desc")
    N = w.pop("N")
    ny = w.pop("ny")
    core = w.pop("core", None)
    p = re_tau_params(N, ny, **w)
    if core is not None:
        p.Ngalx = (p.Ngalx[0], 3 * core[0] // 2)
        p.Ngalz = (p.Ngalz[0], 3 * core[1] // 2)
    return p


def workload_setup(name: str) -> ChannelSetup:
    return build_setup(workload_params(name))


def initial_field(s: ChannelSetup, seed: int, amp: float = 0.1, kmax: int = 8):
    """Returns (u1, u2, u3, p) in the host cfield layout, complex128 [ncols, nlevels]."""
    rng = np.random.default_rng(seed)
    N1h, N2 = s.N1 // 2 + 1, s.N2
    nu, nv = s.nyu, s.nyv
    off = s.dny
    yu, yv = s.yu, s.yv
    Uc = 1.5
    env_v = np.where(np.abs(yv) <= 1.0, (1.0 - yv ** 2) ** 2, 0.0)
    env_u = np.where(np.abs(yu) <= 1.0, (1.0 - yu ** 2) ** 2, 0.0)
    u1 = np.zeros((N2, N1h, nu), np.complex128)
    u3 = np.zeros((N2, N1h, nu), np.complex128)
    u2 = np.zeros((N2, N1h, nv), np.complex128)
    # mean flow
    u1[0, 0, :] = np.where(np.abs(yu) <= 1.0, Uc * (1.0 - yu ** 2), 0.0)
    modes = []
    for r in range(N2):
        kz_i = r if r < N2 // 2 else r - N2
        if r == N2 // 2:
            continue
        for i in range(N1h):
            if i == 0 and kz_i <= 0:
                continue  # kx = 0 plane is filled from kz > 0 by Hermitian symmetry
            if i * i + kz_i * kz_i > kmax * kmax:
                continue
            modes.append((r, i))
    th = s.dthdyu * s.ddthetavi
    for (r, i) in modes:
        kx, kz = s.k1x[i], s.k1z[r]
        k2 = kx * kx + kz * kz
        cv = (rng.normal() + 1j * rng.normal())
        cp = (rng.normal() + 1j * rng.normal())
        v = cv * env_v
        v[0] = 0.0
        v[-1] = 0.0
        D = np.zeros(nu, np.complex128)
        D[1:-1] = (v[1:] - v[:-1]) * th[1:-1]
        phi = cp * env_u
        u = 1j * kx * D / k2 + kz * phi
        w = 1j * kz * D / k2 - kx * phi
        u1[r, i] = u
        u3[r, i] = w
        u2[r, i] = v
        if i == 0:
            rr = (N2 - r) % N2
            u1[rr, 0] = np.conj(u)
            u3[rr, 0] = np.conj(w)
            u2[rr, 0] = np.conj(v)
    # amplitude: rms of the perturbation velocity ~ amp * Uc / 3 at the centre plane
    pert = np.concatenate([u1[:, :, nu // 2].ravel()[1:], u3[:, :, nu // 2].ravel(), u2[:, :, nv // 2].ravel()])
    energy = 2.0 * np.sum(np.abs(pert) ** 2)
    if energy > 0:
        scale = (amp * Uc / 3.0) / math.sqrt(energy / 3.0)
        mean = u1[0, 0].copy()
        u1 *= scale
        u3 *= scale
        u2 *= scale
        u1[0, 0] = mean
    # ghosts of u and w as v_corr leaves them
    u1[:, :, 0] = s.gw_bc_u1 * u1[:, :, 1]
    u1[:, :, -1] = s.gw_bc_u1 * u1[:, :, -2]
    u3[:, :, 0] = s.gw_bc_u3 * u3[:, :, 1]
    u3[:, :, -1] = s.gw_bc_u3 * u3[:, :, -2]
    p = np.zeros((N2 * N1h, nu - 2), np.complex128)
    return (u1.reshape(N2 * N1h, nu), u2.reshape(N2 * N1h, nv), u3.reshape(N2 * N1h, nu), p)


def _fine_field(s: ChannelSetup, seed: int, amp: float, kmax: int):
    """initial_field on the wall-band mode grid, all levels: (u1, u2, u3) [N2][N1h][lev]."""
    u1, u2, u3, _ = initial_field(s, seed, amp, kmax)
    N1h, N2 = s.N1 // 2 + 1, s.N2
    return (u1.reshape(N2, N1h, -1), u2.reshape(N2, N1h, -1), u3.reshape(N2, N1h, -1))


def initial_field_bands(s: ChannelSetup, seed: int, amp: float = 0.1, kmax: int = 8,
                        short_amp: float = 0.02) -> dict:
    """Per-band initial state {band: (u1, u2, u3, p)} in the bands' cfield layouts
    (ChannelSetup.band_shapes). Long columns (band 2) carry initial_field's laminar
    profile and perturbation; the short columns of bands 1 and 3 a divergence-free
    perturbation of relative amplitude `short_amp` confined to their band: v with the
    envelope (y - y_lo)^2 (y_hi - y)^2 between the band's end v levels (where v = 0),
    (u, w) built from it as in initial_field, ghosts from the band's boundary rows."""
    rng = np.random.default_rng(seed + 7919)
    u1f, u2f, u3f, _ = initial_field(s, seed, amp, kmax)
    lng = s.is_long()
    out = {}
    nu, nv = s.nyu, s.nyv
    th = s.dthdyu * s.ddthetavi
    for band in (1, 2, 3):
        cols = s.band_cols(band)
        shp = s.band_shapes(band)
        if band == 2:
            a = [u1f[cols], u2f[cols], u3f[cols]]
            (lo, hi) = s.band_levels(2, 2)
            out[band] = (a[0][:, lo:hi + 1], a[1], a[2][:, lo:hi + 1], np.zeros(shp[3], np.complex128))
            continue
        ulo, uhi = s.band_levels(band, 2)
        vlo, vhi = s.band_levels(band, 1)
        U1 = np.zeros((len(cols), nu), np.complex128)
        U3 = np.zeros_like(U1)
        U2 = np.zeros((len(cols), nv), np.complex128)
        yv = s.yv
        env = np.zeros(nv)
        env[vlo:vhi + 1] = (yv[vlo:vhi + 1] - yv[vlo]) ** 2 * (yv[vhi] - yv[vlo:vhi + 1]) ** 2
        env /= max(env.max(), 1e-300)
        yu = s.yu
        envu = np.clip((yu - yv[vlo]) * (yv[vhi] - yu), 0.0, None) ** 2
        envu /= max(envu.max(), 1e-300)
        N1h = s.N1 // 2 + 1
        for i, c in enumerate(cols):
            r, kx = divmod(int(c), N1h)
            if kx == 0 and r > s.N2 // 2:
                continue  # kx = 0 modes filled by Hermitian symmetry below
            k1x, k1z = s.k1x[kx], s.k1z[r]
            k2 = k1x * k1x + k1z * k1z
            v = short_amp * (rng.normal() + 1j * rng.normal()) * env
            D = np.zeros(nu, np.complex128)
            D[1:-1] = (v[1:] - v[:-1]) * th[1:-1]
            ph = np.zeros(nu, np.complex128)
            ph[ulo + 1:uhi] = (short_amp / math.sqrt(k2)) * (rng.normal() + 1j * rng.normal()) * envu[ulo + 1:uhi]
            U1[i] = 1j * k1x * D / k2 + k1z * ph
            U3[i] = 1j * k1z * D / k2 - k1x * ph
            U2[i] = v
        # kx = 0 columns: Hermitian partner of row r is row N2 - r
        pos = {int(c): i for i, c in enumerate(cols)}
        for i, c in enumerate(cols):
            r, kx = divmod(int(c), N1h)
            if kx == 0 and r > s.N2 // 2:
                j = pos.get((s.N2 - r) * N1h)
                if j is not None:
                    U1[i], U2[i], U3[i] = np.conj(U1[j]), np.conj(U2[j]), np.conj(U3[j])
        for U in (U1, U3):
            U[:, :ulo + 1] = 0.0
            U[:, uhi:] = 0.0
        # ghosts: wall ghosts from gridweighting_bc, interface ghosts from the band's BC row
        b = band - 1
        if band == 1:
            U1[:, ulo] = s.gw_bc_u1 * U1[:, ulo + 1]
            U3[:, ulo] = s.gw_bc_u3 * U3[:, ulo + 1]
            U1[:, uhi] = -s.gw[b, 1] * U1[:, uhi - 1]
            U3[:, uhi] = -s.gw[b, 1] * U3[:, uhi - 1]
        else:
            U1[:, uhi] = s.gw_bc_u1 * U1[:, uhi - 1]
            U3[:, uhi] = s.gw_bc_u3 * U3[:, uhi - 1]
            U1[:, ulo] = -s.gw[b, 0] * U1[:, ulo + 1]
            U3[:, ulo] = -s.gw[b, 0] * U3[:, ulo + 1]
        out[band] = (U1[:, ulo:uhi + 1], U2[:, vlo:vhi + 1], U3[:, ulo:uhi + 1], np.zeros(shp[3], np.complex128))
    return out


def initial_scalars(s: ChannelSetup) -> dict:
    return dict(t=0.0, dt=0.0, dti=0.0, dtc=0.0, mpgx=s.p.mpgx, iter=0, QxT=0.0)


def ensemble_params(n: int = 64, seed: int = 2000):
    """The batched ensemble: n independent channels with uneven grids drawn from a
    seed: N in {32, 48, 64, 96} (Nx = Nz), ny in {97, 129, 153}, Re_tau in [120, 300],
    square posts with a period of 8-24 physical points (a divisor of Ngal) and a solid
    fraction of 0.1-0.5, 6 wall units high. Channel c uses seed + c for its field."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n):
        N = int(rng.choice([32, 48, 64, 96]))
        ny = int(rng.choice([97, 129, 153]))
        re_tau = float(rng.uniform(120.0, 300.0))
        G = 3 * N // 2
        periods = [d for d in range(8, 25) if G % d == 0]
        period = int(rng.choice(periods))
        frac = float(rng.uniform(0.1, 0.5))
        npk = max(1, min(period - 1, int(round(period * math.sqrt(frac)))))
        p = re_tau_params(N, ny, re_tau=re_tau, posts=True, post_period=period, post_points=npk,
                          post_height_plus=6.0, flpress=0)
        out.append(p)
    return out


def ensemble_setups(n: int = 64, seed: int = 2000):
    return [build_setup(p) for p in ensemble_params(n, seed)]
