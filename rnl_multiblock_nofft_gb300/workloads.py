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
}


def workload_params(name: str) -> ChannelParams:
    w = dict(WORKLOADS[name])
    w.pop("desc")
    N = w.pop("N")
    ny = w.pop("ny")
    return re_tau_params(N, ny, **w)


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
