"""Seeded synthetic particle sets: an NFW host halo plus NFW subhalos.

The reference's own particle data (Via Lactea II snapshots read by
src/datareader.cpp) is not available, so maps are rendered from synthetic
sets with the reference's data shape: float32 position, mass, SPH density and
smoothing length per particle, positions in code length units of 1 kpc
(``Lbox_in_Mpc = 0.001``) and masses in Msun (``mass_to_Msun = 1``).

Generator (all draws from ``numpy.random.Generator(PCG64(seed))``):
  * host: NFW with r_s = 20 kpc, r200 = 400 kpc (c = 20), truncated at r200;
    radii from the inverse of the enclosed-mass profile
    mu(x) = ln(1+x) - x/(1+x); isotropic directions; rho_s chosen so the
    host's particles hold its mass inside r200;
  * subhalos: masses log-uniform in [1e6, 1e9] Msun, centres uniform in the
    300 kpc ball; they hold ``sub_frac`` of the particles, shared in
    proportion to subhalo mass; each an NFW with c = 20 and
    r200_sub = r200 * (M_sub / M_host)^(1/3), normalised to its particles;
  * density: rho = rho_NFW(r) * exp(N(0, 0.3)); smoothing length
    h = (32 m / (4 pi/3 rho))^(1/3) (the 32-neighbour SPH convention);
  * optional ``near_observer`` particles uniform within ``near_radius`` of
    the observer, with the host density there (the large-disc case);
  * the particle order is shuffled, so any prefix is an i.i.d. sample;
  * ``n_total`` draws the n particles as an i.i.d. sample of an n_total-
    particle set: densities (hence smoothing lengths) are normalised to the
    larger set's particle counts, so the sample has its per-particle disc
    statistics without generating it whole.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

RS_HOST = 20.0       # kpc
R200_HOST = 400.0    # kpc
CONC = 20.0
SUB_RMAX = 300.0     # kpc
OBS_DIST = 8.0       # kpc


def _mu(x):
    return np.log1p(x) - x / (1.0 + x)


def _inv_mu(q, c):
    """Solves mu(x) = q for x in [0, c] (q <= mu(c)), vectorised."""
    grid = np.concatenate([[0.0], np.geomspace(1e-6, c, 4096)])
    mg = _mu(grid)
    x = np.interp(q, mg, grid)
    for _ in range(4):  # Newton polish: mu'(x) = x / (1+x)^2
        d = x / (1.0 + x) ** 2
        step = np.where(d > 0, (_mu(x) - q) / np.maximum(d, 1e-300), 0.0)
        x = np.clip(x - step, 0.0, c)
    return x


def _iso(rng, n):
    u = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * math.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - u * u))
    return np.stack([s * np.cos(ph), s * np.sin(ph), u], axis=1)


def _nfw_sample(rng, n, rs, c, mass_in_r200, center, m):
    """n particles of an NFW halo truncated at c*rs; returns pos, rho, h."""
    mc = _mu(c)
    q = rng.uniform(0.0, 1.0, n) * mc
    x = _inv_mu(q, c)
    r = x * rs
    pos = center[None, :] + _iso(rng, n) * r[:, None]
    rho_s = mass_in_r200 / (4.0 * math.pi * rs ** 3 * mc)
    xs = np.maximum(x, 1e-6)
    rho = rho_s / (xs * (1.0 + xs) ** 2)
    rho = rho * np.exp(rng.normal(0.0, 0.3, n))
    h = np.cbrt(32.0 * m / (4.0 * math.pi / 3.0 * rho))
    return pos, rho, h


@dataclass
class Particles:
    """Float32 SoA particle set plus the observer set-up it was made for."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    m: np.ndarray
    rho: np.ndarray
    h: np.ndarray
    obs_pos: tuple = (0.0, 0.0, 0.0)
    centerpos: tuple = (0.0, 0.0, 0.0)
    align_vec: tuple = (0.0, 0.0, 1.0)
    particle_mass: float = 4.1e3
    meta: dict = field(default_factory=dict)

    def __len__(self):
        return int(self.x.shape[0])

    def as_dict(self):
        return {"x": self.x, "y": self.y, "z": self.z, "m": self.m, "rho": self.rho, "h": self.h}

    def subset(self, sl):
        return Particles(self.x[sl], self.y[sl], self.z[sl], self.m[sl], self.rho[sl], self.h[sl],
                         self.obs_pos, self.centerpos, self.align_vec, self.particle_mass,
                         dict(self.meta))


def default_observer():
    s = OBS_DIST / math.sqrt(3.0)
    return (s, s, s)


def nfw_halo(n: int, *, seed: int, n_sub: int = 0, sub_frac: float = 0.1,
             particle_mass: float = 4.1e3, near_observer: int = 0, near_radius: float = 0.5,
             obs_pos=None, shuffle: bool = True, n_total: int | None = None) -> Particles:
    """Builds an ``n``-particle set (see the module docstring)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    obs = np.array(obs_pos if obs_pos is not None else default_observer(), dtype=np.float64)
    m = float(particle_mass)
    n_near = int(near_observer)
    n_halo = n - n_near
    if n_halo < 0:
        raise ValueError("near_observer exceeds n")
    counts = np.zeros(0, dtype=np.int64)
    msub = np.zeros(0)
    if n_sub > 0:
        msub = 10.0 ** rng.uniform(6.0, 9.0, n_sub)
        share = msub / msub.sum() * (sub_frac * n_halo)
        counts = np.floor(share).astype(np.int64)
        rem = int(round(sub_frac * n_halo)) - int(counts.sum())
        if rem > 0:
            order = np.argsort(-(share - counts))
            counts[order[:rem]] += 1
    n_host = n_halo - int(counts.sum())
    # the set the particles are a sample of (itself unless n_total is given)
    grow = 1.0 if n_total is None else float(n_total) / float(n)
    m_host = n_host * m * grow

    pos_l, rho_l, h_l = [], [], []
    chunk = 1 << 22
    done = 0
    while done < n_host:
        k = min(chunk, n_host - done)
        p, r, h = _nfw_sample(rng, k, RS_HOST, CONC, m_host, np.zeros(3), m)
        pos_l.append(p); rho_l.append(r); h_l.append(h)
        done += k
    if n_sub > 0:
        centres = _iso(rng, n_sub) * (SUB_RMAX * np.cbrt(rng.uniform(0.0, 1.0, n_sub)))[:, None]
        for j in range(n_sub):
            k = int(counts[j])
            if k == 0:
                continue
            r200s = R200_HOST * (msub[j] / m_host) ** (1.0 / 3.0)
            p, r, h = _nfw_sample(rng, k, r200s / CONC, CONC, k * m * grow, centres[j], m)
            pos_l.append(p); rho_l.append(r); h_l.append(h)
    if n_near > 0:
        d = near_radius * np.cbrt(rng.uniform(0.0, 1.0, n_near))
        p = obs[None, :] + _iso(rng, n_near) * d[:, None]
        rr = np.linalg.norm(p, axis=1) / RS_HOST
        rho_s = m_host / (4.0 * math.pi * RS_HOST ** 3 * _mu(CONC))
        r = rho_s / (rr * (1.0 + rr) ** 2) * np.exp(rng.normal(0.0, 0.3, n_near))
        h = np.cbrt(32.0 * m / (4.0 * math.pi / 3.0 * r))
        pos_l.append(p); rho_l.append(r); h_l.append(h)

    pos = np.concatenate(pos_l) if pos_l else np.zeros((0, 3))
    rho = np.concatenate(rho_l) if rho_l else np.zeros(0)
    hs = np.concatenate(h_l) if h_l else np.zeros(0)
    if shuffle and n > 1:
        perm = rng.permutation(n)
        pos, rho, hs = pos[perm], rho[perm], hs[perm]
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return Particles(f(pos[:, 0]), f(pos[:, 1]), f(pos[:, 2]), np.full(n, m, dtype=np.float32),
                     f(rho), f(hs), tuple(obs.tolist()), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), m,
                     {"seed": seed, "n_sub": n_sub, "near_observer": n_near})


# Named workloads: the five configurations the benchmark and tests use.
def workload(name: str, *, scale: float = 1.0) -> tuple[Particles, int]:
    """Returns (particles, nside) for a named configuration.  ``scale``
    shrinks the particle count (tests use small scales)."""
    if name == "nfw1m_ns512":        # plain method, small
        n = max(64, int((1 << 20) * scale))
        return nfw_halo(n, seed=20240001), 512
    if name == "nfw16m_sub100_ns2048":
        n = max(64, int((1 << 24) * scale))
        return nfw_halo(n, seed=20240002, n_sub=100), 2048
    if name == "nfw134m_sub500_ns4096":
        n = max(64, int((1 << 27) * scale))
        m = 4.1e3 * (1 << 24) / (1 << 27)
        return nfw_halo(n, seed=20240003, n_sub=500, particle_mass=m,
                        near_observer=max(1, int(10000 * scale))), 4096
    if name == "nfw8m_sub50_batched":
        n = max(64, int((1 << 23) * scale))
        return nfw_halo(n, seed=20240004, n_sub=50), 1024
    if name == "nfw4m_sub20_adjoint":
        n = max(64, int((1 << 22) * scale))
        return nfw_halo(n, seed=20240005, n_sub=20), 512
    raise KeyError(name)


def batched_observers(k: int = 64, seed: int = 20240014, nsides=(256, 512, 1024)):
    """k observer positions uniform on the 8 kpc sphere, Nside cycling."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dirs = _iso(rng, k)
    return [(tuple((OBS_DIST * d).tolist()), int(nsides[i % len(nsides)])) for i, d in enumerate(dirs)]
