"""Seeded synthetic inputs of the channel workloads (no dataset is involved).

Axis convention of the solver (the reference's): i is wall-normal, j and k are
periodic.  The channel workloads are quoted with walls on y and x, z periodic,
lengths 2*pi x 2 x pi half-heights (h = 1 m), so here

    i <-> y (length 2, walls at y = -1 and +1),
    j <-> x (length 2*pi),  k <-> z (length pi).

Arrays are float32 with numpy shape (kmax, jmax, imax): i fastest, the dense
layout of include/dnsmc.h.

Fluctuation field (5 % "seeded Fourier" perturbation): with 8 modes per
direction,

    f(x, y, z) = sum_{m,n,l=1..8} a_mnl cos(2 pi m x / Lx + p_m)
                                        sin(n pi (y + 1) / 2)
                                        cos(2 pi l z / Lz + q_l),

a_mnl ~ N(0, 1) / (m^2 + n^2 + l^2), phases p, q ~ U[0, 2 pi) drawn from
numpy.random.default_rng(seed); f is scaled to max |f| = 1.  The sine factor
vanishes on both walls, so the walls keep their temperature.
"""
from __future__ import annotations

import math

import numpy as np

LX, LY, LZ = 2 * math.pi, 2.0, math.pi  # x, y (wall-normal), z in half-heights


def gauss_legendre_half(nq: int = 16):
    """Positive half of the 2*nq-point Gauss-Legendre rule on [-1, 1]: the
    g-points and weights of the reference's narrow-band tables
    (code/NarrowBand.h:201-207 lists these 16 values)."""
    x, w = np.polynomial.legendre.leggauss(2 * nq)
    m = x > 0
    return x[m].astype(np.float64), w[m].astype(np.float64)


def cell_centres(n: int, L: float) -> np.ndarray:
    return (np.arange(n) + 0.5) * (L / n)


def fourier_fluct(ni: int, nj: int, nk: int, seed: int, nmodes: int = 8) -> np.ndarray:
    """f of the module docstring on the cell centres, shape (nk, nj, ni)."""
    rng = np.random.default_rng(seed)
    m = np.arange(1, nmodes + 1)
    a = rng.standard_normal((nmodes, nmodes, nmodes))
    a /= (m[:, None, None] ** 2 + m[None, :, None] ** 2 + m[None, None, :] ** 2)
    px = rng.uniform(0, 2 * math.pi, nmodes)
    qz = rng.uniform(0, 2 * math.pi, nmodes)
    x = cell_centres(nj, LX)
    y = cell_centres(ni, LY) - 1.0
    z = cell_centres(nk, LZ)
    X = np.cos(2 * math.pi * m[:, None] * x[None, :] / LX + px[:, None])   # (m, nj)
    Y = np.sin(m[:, None] * math.pi * (y[None, :] + 1.0) / 2.0)            # (n, ni)
    Z = np.cos(2 * math.pi * m[:, None] * z[None, :] / LZ + qz[:, None])   # (l, nk)
    f = np.einsum("mnl,mj,ni,lk->kji", a, X, Y, Z, optimize=True)
    return np.ascontiguousarray(f / np.abs(f).max(), dtype=np.float64)


def channel_temperature(n: int, T_wall: float, T_rise: float, seed: int, amp: float = 0.05) -> np.ndarray:
    """T = (T_wall + T_rise (1 - y^2)) (1 + amp f), shape (n, n, n)."""
    y = cell_centres(n, LY) - 1.0
    base = T_wall + T_rise * (1.0 - y * y)
    f = fourier_fluct(n, n, n, seed)
    return np.ascontiguousarray(base[None, None, :] * (1.0 + amp * f), dtype=np.float32)


def grey_channel(n: int = 64, seed: int = 0) -> dict:
    """Grey channel: T = 300 + 700 (1 - y^2) K (+5 %), black walls at 300 K,
    kappa = 1 per half-height."""
    T = channel_temperature(n, 300.0, 700.0, seed)
    return dict(T=T, n=n, T_wall=300.0, kappa=1.0, L=(LY, LX, LZ))


def slab(n: int = 64, T: float = 1000.0) -> dict:
    """Isothermal slab: uniform T, kappa = 1, tau_L = 2 between black walls."""
    return dict(T=np.full((n, n, n), T, np.float32), n=n, kappa=1.0, L=(LY, LX, LZ))


def h2o_fraction(n: int, seed: int) -> np.ndarray:
    """x_H2O = 0.1 + 0.05 f with an independent fluctuation (seed + 1000)."""
    return np.ascontiguousarray(0.1 + 0.05 * fourier_fluct(n, n, n, seed + 1000), dtype=np.float32)


def ck_channel(n: int = 128, seed: int = 0) -> dict:
    """Correlated-k channel: T = 400 + 1400 (1 - y^2) K (+5 %), walls at 400 K,
    x_H2O = 0.1 + 0.05 f."""
    return dict(T=channel_temperature(n, 400.0, 1400.0, seed), x=h2o_fraction(n, seed), n=n, T_wall=400.0,
                L=(LY, LX, LZ))


def ck_table(nbands: int = 64, nq: int = 16, nT: int = 50, nX: int = 8, seed: int = 0,
             T_range=(300.0, 2500.0), X_range=(0.0, 0.3), nu_range=(150.0, 7500.0)) -> dict:
    """Synthetic narrow-band correlated-k table k(band, g, T, x) in 1/m.

    ln k = 2.0 * z with z ~ N(0, 1) smoothed along T (Gaussian filter, 3
    points), rescaled to unit variance, sorted ascending over g at every
    (band, T) -- so k is monotone in g -- times (x / 0.1)^p_band, p_band ~
    U[0.8, 1.2]; bands of equal width between nu_range.
    """
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((nbands, nq, nT))
    tt = np.arange(-9, 10)
    ker = np.exp(-0.5 * (tt / 3.0) ** 2)
    ker /= ker.sum()
    zs = np.empty_like(z)
    for b in range(nbands):
        for g in range(nq):
            zs[b, g] = np.convolve(np.pad(z[b, g], 9, mode="reflect"), ker, mode="valid")
    zs /= zs.std(axis=2, keepdims=True)
    zs = np.sort(zs, axis=1)
    p = rng.uniform(0.8, 1.2, nbands)
    X = np.linspace(X_range[0], X_range[1], nX)
    xf = (X[None, :] / 0.1) ** p[:, None]                                   # (band, nX)
    k = np.exp(2.0 * zs)[..., None] * xf[:, None, None, :]
    nu = np.linspace(nu_range[0], nu_range[1], nbands + 1)
    gq, wq = gauss_legendre_half(nq)
    return dict(k=k.astype(np.float32), wvc=(0.5 * (nu[1:] + nu[:-1])).astype(np.float32),
                dnu=np.diff(nu).astype(np.float32), wq=wq.astype(np.float32), gq=gq,
                T0=float(T_range[0]), dT=float((T_range[1] - T_range[0]) / (nT - 1)),
                X0=float(X_range[0]), dX=float((X_range[1] - X_range[0]) / (nX - 1)))


def particle_fraction(n: int, seed: int) -> np.ndarray:
    """Particle volume fraction fv = 1e-5 (1 + 0.5 f), f an independent
    fluctuation field (seed + 2000), shape (n, n, n)."""
    return np.ascontiguousarray(1e-5 * (1.0 + 0.5 * fourier_fluct(n, n, n, seed + 2000)), dtype=np.float32)


def particle_table(nbands: int = 64, seed: int = 0, diameter: float = 1e-5) -> dict:
    """Smooth synthetic particle optics per band: extinction efficiency
    Q_ext in [1.0, 2.2] and single-scattering albedo in [0.3, 0.9], both slowly
    varying with the band index (sums of two sinusoids with seeded phases);
    coefficients per unit volume fraction for spheres of the given diameter:
    a = 3 Q_abs / (2 d), s = 3 Q_sca / (2 d) [1/m]."""
    rng = np.random.default_rng(seed + 3000)
    u = np.linspace(0.0, 1.0, nbands)
    ph = rng.uniform(0, 2 * math.pi, 4)
    qext = 1.6 + 0.4 * np.sin(2 * math.pi * u + ph[0]) + 0.2 * np.sin(5 * math.pi * u + ph[1])
    alb = 0.6 + 0.2 * np.sin(2 * math.pi * u + ph[2]) + 0.1 * np.sin(3 * math.pi * u + ph[3])
    qext = np.clip(qext, 1.0, 2.2)
    alb = np.clip(alb, 0.3, 0.9)
    f = 1.5 / diameter
    return dict(absorption=(f * qext * (1 - alb)).astype(np.float32), scattering=(f * qext * alb).astype(np.float32),
                albedo=alb, qext=qext, g=0.6)


def lbl_spectrum(temperatures, fractions=(0.1,), nbands: int = 6, band_width: float = 25.0,
                 wv0: float = 1000.0, dwv: float = 0.01, lines_per_band: int = 40, seed: int = 0) -> dict:
    """Seeded synthetic line-by-line H2O-like absorption spectra (no spectral
    database is involved): Lorentz lines with log-normal strengths and
    random positions, line strengths S(T) = S0 (296 / T)^1.5
    exp(-1.4388 E'' (1/T - 1/296)) and half widths gamma = gamma0 (296 /
    T)^0.7 (1 + 4 x) per H2O mole fraction x, absorption coefficient
    k(nu) = 100 x sum S gamma / (pi ((nu - nu0)^2 + gamma^2)) [1/m], on a
    uniform grid of spacing dwv [1/cm] with `nbands` contiguous bands of
    `band_width` [1/cm].  Returns kappa [nT][nX][npts] (float64), the grid
    (wv0, dwv) and the band point ranges and edges."""
    rng = np.random.default_rng(seed)
    per = int(round(band_width / dwv))
    npts = nbands * per + 1
    nu = wv0 + dwv * np.arange(npts)
    nl = nbands * lines_per_band
    pos = wv0 + rng.uniform(0, nbands * band_width, nl)
    S0 = np.exp(rng.normal(np.log(1e-2), 2.0, nl))
    E = rng.uniform(0.0, 3000.0, nl)
    g0 = rng.uniform(0.02, 0.1, nl)
    T = np.asarray(temperatures, np.float64)
    X = np.asarray(fractions, np.float64)
    kappa = np.zeros((T.size, X.size, npts))
    for a, t in enumerate(T):
        S = S0 * (296.0 / t) ** 1.5 * np.exp(-1.4388 * E * (1.0 / t - 1.0 / 296.0))
        for b, x in enumerate(X):
            gam = g0 * (296.0 / t) ** 0.7 * (1.0 + 4.0 * x)
            k = np.zeros(npts)
            for i0 in range(0, nl, 64):
                sl = slice(i0, i0 + 64)
                d = nu[None, :] - pos[sl, None]
                k += (S[sl, None] * gam[sl, None] / (np.pi * (d * d + gam[sl, None] ** 2))).sum(0)
            kappa[a, b] = 100.0 * x * k + 1e-6
    first = np.arange(nbands, dtype=np.int64) * per
    count = np.full(nbands, per + 1, np.int32)
    wl = wv0 + band_width * np.arange(nbands)
    return dict(kappa=kappa, wv0=wv0, dwv=dwv, npts=npts, first=first, count=count, wv_left=wl,
                wv_right=wl + band_width, wvc=wl + 0.5 * band_width, T=T, X=X)
