"""Seeded initial conditions for the soft-force workloads.

All models are in Henon units (G = 1, M = 1, E = -1/4).  The reference ships
only an equal-mass Plummer generator
(src/particle_distribution_generator.hpp:173-251) and otherwise relies on an
external cluster generator, so the mass function, binaries and King model here
are this package's own, from their published definitions:

* Kroupa (2001) IMF: dN/dm ~ m^-1.3 on [0.08, 0.5), m^-2.3 on [0.5, 150] Msun,
  continuous at 0.5, masses normalised to a total of 1.
* Plummer (1911) sphere sampled as in the reference generator: radius from the
  inverse cumulative mass, cut at 22.8 Henon length units, speeds by the von
  Neumann rejection on q^2 (1 - q^2)^3.5, then scaled to r_scale = 3 pi / 16.
* Binaries: semi-major axis log-uniform, thermal eccentricity f(e) = 2e,
  isotropic orientation, uniform mean anomaly (Kepler's equation by Newton).
* King (1966) model with dimensionless central potential W0, integrated from
  Poisson's equation and sampled by rejection on the lowered Maxwellian.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

KROUPA_BREAKS = (0.08, 0.5, 150.0)
KROUPA_SLOPES = (1.3, 2.3)


def kroupa_masses(rng: np.random.Generator, n: int) -> np.ndarray:
    """Draws n masses (Msun) from the two-segment Kroupa IMF on [0.08, 150]."""
    m0, m1, m2 = KROUPA_BREAKS
    a1, a2 = KROUPA_SLOPES
    k1 = 1.0
    k2 = k1 * m1 ** (a2 - a1)  # continuity at m1
    w1 = k1 * (m1 ** (1 - a1) - m0 ** (1 - a1)) / (1 - a1)
    w2 = k2 * (m2 ** (1 - a2) - m1 ** (1 - a2)) / (1 - a2)
    seg = rng.random(n) < w1 / (w1 + w2)
    u = rng.random(n)
    out = np.empty(n)
    lo, hi, a = m0, m1, a1
    p = 1 - a
    out[seg] = (lo ** p + u[seg] * (hi ** p - lo ** p)) ** (1 / p)
    lo, hi, a = m1, m2, a2
    p = 1 - a
    out[~seg] = (lo ** p + u[~seg] * (hi ** p - lo ** p)) ** (1 / p)
    return out


def _isotropic(rng: np.random.Generator, n: int) -> np.ndarray:
    phi = 2.0 * np.pi * rng.random(n)
    cth = 2.0 * (rng.random(n) - 0.5)
    sth = np.sqrt(1.0 - cth * cth)
    return np.stack([sth * np.cos(phi), sth * np.sin(phi), cth], axis=1)


def plummer(rng: np.random.Generator, mass: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Plummer positions and velocities in Henon units for the given masses
    (any normalisation; the centre of mass is removed with these masses)."""
    n = mass.size
    r_scale = 3.0 * np.pi / 16.0
    r_cut = 22.8 / r_scale
    r = np.empty(0)
    while r.size < n:
        m = rng.random(2 * (n - r.size) + 16)
        m = m[m > 0]
        rr = 1.0 / np.sqrt(m ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr <= r_cut]])
    r = r[:n]
    pos = r[:, None] * _isotropic(rng, n)
    q = np.empty(0)
    while q.size < n:
        k = 2 * (n - q.size) + 16
        v_try = rng.random(k)
        v_crit = 0.1 * rng.random(k)
        ok = v_crit < v_try ** 2 * (1.0 - v_try ** 2) ** 3.5
        q = np.concatenate([q, v_try[ok]])
    q = q[:n]
    ve = np.sqrt(2.0) * (r * r + 1.0) ** -0.25
    vel = (ve * q)[:, None] * _isotropic(rng, n)
    w = mass / mass.sum()
    pos -= (w[:, None] * pos).sum(0)
    vel -= (w[:, None] * vel).sum(0)
    return pos * r_scale, vel / np.sqrt(r_scale)


def _kepler_E(M: np.ndarray, e: np.ndarray) -> np.ndarray:
    E = np.where(e < 0.8, M, np.pi * np.ones_like(M))
    for _ in range(60):
        f = E - e * np.sin(E) - M
        fp = 1.0 - e * np.cos(E)
        dE = f / fp
        E = E - dE
        if np.max(np.abs(dE)) < 1e-14:
            break
    return E


def split_binaries(rng: np.random.Generator, pos: np.ndarray, vel: np.ndarray, m1: np.ndarray,
                   m2: np.ndarray, a_lo: float = 1e-5, a_hi: float = 1e-2,
                   G: float = 1.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Replaces each centre of mass by a Keplerian pair (m1, m2).

    Returns positions, velocities and masses of the 2n components, primary
    then secondary for each pair."""
    n = m1.size
    mt = m1 + m2
    a = 10.0 ** rng.uniform(np.log10(a_lo), np.log10(a_hi), n)
    e = np.sqrt(rng.random(n))
    M = 2.0 * np.pi * rng.random(n)
    E = _kepler_E(M, e)
    cE, sE = np.cos(E), np.sin(E)
    sq = np.sqrt(1.0 - e * e)
    nmot = np.sqrt(G * mt / a ** 3)
    den = 1.0 - e * cE
    xr = np.stack([a * (cE - e), a * sq * sE, np.zeros(n)], axis=1)
    vr = np.stack([-a * nmot * sE / den, a * nmot * sq * cE / den, np.zeros(n)], axis=1)
    # Isotropic orientation: random inclination (cos i uniform), node and periapsis.
    inc = np.arccos(2.0 * rng.random(n) - 1.0)
    node = 2.0 * np.pi * rng.random(n)
    peri = 2.0 * np.pi * rng.random(n)

    def rot(v):
        # R = Rz(node) Rx(inc) Rz(peri)
        c, s = np.cos(peri), np.sin(peri)
        x1 = c * v[:, 0] - s * v[:, 1]
        y1 = s * v[:, 0] + c * v[:, 1]
        z1 = v[:, 2]
        c, s = np.cos(inc), np.sin(inc)
        y2 = c * y1 - s * z1
        z2 = s * y1 + c * z1
        c, s = np.cos(node), np.sin(node)
        return np.stack([c * x1 - s * y2, s * x1 + c * y2, z2], axis=1)

    xr, vr = rot(xr), rot(vr)
    f1 = (m2 / mt)[:, None]
    f2 = (m1 / mt)[:, None]
    p = np.empty((2 * n, 3))
    v = np.empty((2 * n, 3))
    m = np.empty(2 * n)
    p[0::2] = pos + f1 * xr
    p[1::2] = pos - f2 * xr
    v[0::2] = vel + f1 * vr
    v[1::2] = vel - f2 * vr
    m[0::2] = m1
    m[1::2] = m2
    return p, v, m


def king(rng: np.random.Generator, mass: np.ndarray, W0: float = 7.0) -> tuple[np.ndarray, np.ndarray]:
    """King (1966) model with central potential W0, scaled to Henon units
    (virial radius 1 for M = 1, G = 1) with the given masses."""
    from scipy.integrate import solve_ivp
    from scipy.special import erf

    def rho_of_w(w):
        w = np.maximum(w, 0.0)
        return np.exp(w) * erf(np.sqrt(w)) - np.sqrt(4.0 * w / np.pi) * (1.0 + 2.0 * w / 3.0)

    rho0 = rho_of_w(W0)

    # Dimensionless Poisson equation (King radius units): W'' + 2W'/r = -9 rho/rho0.
    def rhs(r, y):
        w, dw = y
        return [dw, -9.0 * rho_of_w(w) / rho0 - 2.0 * dw / r]

    def tidal(r, y):
        return y[0]

    tidal.terminal = True
    tidal.direction = -1
    r0 = 1e-6
    y0 = [W0 - 1.5 * r0 * r0, -3.0 * r0]
    sol = solve_ivp(rhs, (r0, 1e4), y0, events=tidal, dense_output=True, rtol=1e-10, atol=1e-12,
                    max_step=0.01)
    rt = sol.t_events[0][0] if sol.t_events[0].size else sol.t[-1]
    rg = np.linspace(r0, rt, 20000)
    wg = np.maximum(sol.sol(rg)[0], 0.0)
    dens = rho_of_w(wg)
    cum = np.concatenate([[0.0], np.cumsum(0.5 * (dens[1:] * rg[1:] ** 2 + dens[:-1] * rg[:-1] ** 2)
                                           * np.diff(rg))])
    cum /= cum[-1]
    n = mass.size
    r = np.interp(rng.random(n), cum, rg)
    w = np.maximum(np.interp(r, rg, wg), 0.0)
    pos = r[:, None] * _isotropic(rng, n)
    # Velocities: f(E) ~ exp(w - v^2/2) - 1 for v < sqrt(2w) (velocity unit sigma);
    # sample v from p(v) ~ v^2 (exp(w - v^2/2) - 1) by rejection with an
    # envelope at each particle's maximum.
    vmax = np.sqrt(2.0 * w)
    vv = np.zeros(n)
    todo = np.arange(n)
    # Envelope: the maximum of p over v on a grid of w values (p's maximum
    # grows with w), interpolated per particle with a 10% margin.
    xs = np.linspace(0.0, 1.0, 257)[1:]
    wgrid = np.linspace(0.0, float(w.max()) if n else 0.0, 2049)
    vgrid = np.sqrt(2.0 * wgrid)[:, None] * xs[None, :]
    pgrid = (vgrid ** 2 * (np.exp(wgrid[:, None] - 0.5 * vgrid ** 2) - 1.0)).max(axis=1)
    pmax_all = np.interp(w, wgrid, pgrid) * 1.10 + 1e-300
    while todo.size:
        vm = vmax[todo]
        ww = w[todo]
        pmax = pmax_all[todo]
        v_try = vm * rng.random(todo.size)
        p = v_try ** 2 * (np.exp(ww - 0.5 * v_try ** 2) - 1.0)
        ok = rng.random(todo.size) * pmax < p
        vv[todo[ok]] = v_try[ok]
        todo = todo[~ok]
    vel = vv[:, None] * _isotropic(rng, n)
    wgt = mass / mass.sum()
    pos -= (wgt[:, None] * pos).sum(0)
    vel -= (wgt[:, None] * vel).sum(0)
    # Scale to Henon units: E = -1/4 for M = 1 from the virial theorem
    # (|W| = 2K) with energies measured on the sampled particles.
    ke = 0.5 * float((wgt * (vel ** 2).sum(1)).sum())
    pe = _potential_energy_estimate(rng, pos, wgt)
    # With lengths scaled by L and speeds by V: K' = K V^2, W' = W / L.
    # Choose L with W' = -1/2 and V with K' = 1/4.
    L = pe / -0.5
    V = np.sqrt(0.25 / ke)
    return pos * L, vel * V


def _potential_energy_estimate(rng: np.random.Generator, pos: np.ndarray, w: np.ndarray,
                               n_sample: int = 4096) -> float:
    """Potential energy of a unit-mass system, estimated from a random subsample
    (exact for n <= n_sample)."""
    n = pos.shape[0]
    if n > n_sample:
        idx = rng.choice(n, n_sample, replace=False)
        p = pos[idx]
        m = np.full(n_sample, 1.0 / n_sample)
    else:
        p, m = pos, w
    pe = 0.0
    for s in range(0, p.shape[0], 512):
        d = p[s:s + 512, None, :] - p[None, :, :]
        r = np.sqrt((d * d).sum(-1))
        np.fill_diagonal(r[:, s:s + 512], np.inf)
        pe -= 0.5 * float((m[s:s + 512, None] * m[None, :] / r).sum())
    return pe


@dataclass
class Cluster:
    """Particles of one star cluster and the soft-force parameters PeTar would
    use for it (all radii in Henon units)."""
    pos: np.ndarray
    vel: np.ndarray
    mass: np.ndarray
    r_out: float
    r_in: float
    r_search: np.ndarray
    theta: float
    n_leaf_limit: int = 20
    n_group_limit: int = 512
    eps: float = 0.0
    G: float = 1.0

    @property
    def n(self) -> int:
        return self.mass.size


def make_plummer_cluster(seed: int, n_cm: int, r_out: float, binary_fraction: float = 0.0,
                         theta: float = 0.3, n_group_limit: int = 512) -> Cluster:
    """Plummer sphere of n_cm centres of mass with Kroupa masses; a fraction of
    them split into binaries.  r_in = 0.1 r_out and r_search = 1.5 r_out."""
    rng = np.random.default_rng(seed)
    n_bin = int(round(binary_fraction * n_cm))
    n_single = n_cm - n_bin
    m_single = kroupa_masses(rng, n_single)
    m1 = kroupa_masses(rng, n_bin)
    m2 = kroupa_masses(rng, n_bin)
    m_cm = np.concatenate([m_single, m1 + m2])
    pos, vel = plummer(rng, m_cm)
    mass = m_single
    if n_bin:
        # Binary orbits in Henon units need the masses in the same units.
        scale = 1.0 / m_cm.sum()
        bp, bv, bm = split_binaries(rng, pos[n_single:], vel[n_single:], m1 * scale, m2 * scale)
        pos = np.concatenate([pos[:n_single], bp])
        vel = np.concatenate([vel[:n_single], bv])
        mass = np.concatenate([m_single, bm / scale])
    mass = mass / mass.sum()
    rs = np.full(mass.size, 1.5 * r_out)
    return Cluster(pos=pos, vel=vel, mass=mass, r_out=r_out, r_in=0.1 * r_out, r_search=rs,
                   theta=theta, n_group_limit=n_group_limit)


def make_king_cluster(seed: int, n: int, r_out: float, W0: float = 7.0, theta: float = 0.4) -> Cluster:
    rng = np.random.default_rng(seed)
    mass = kroupa_masses(rng, n)
    mass /= mass.sum()
    pos, vel = king(rng, mass, W0)
    return Cluster(pos=pos, vel=vel, mass=mass, r_out=r_out, r_in=0.1 * r_out,
                   r_search=np.full(n, 1.5 * r_out), theta=theta)
