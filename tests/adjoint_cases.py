"""Shared set-up of the adjoint tests: a seeded NFW particle set, its oracle
parameters and the pixelwise loss of the adjoint workload,
    L = sum_p w_p (map_p - target_p)^2,  w_p = 1 / (target_p + eps),
target = the map of the same particles with positions jittered by 0.1 h,
so dL/dmap = 2 w (map - target)."""
import numpy as np

import oracle as O
from annmap import synth

FIELDS = ("x", "y", "z", "m", "rho", "h")
N_FULL = 1 << 22   # particles of the full adjoint workload


def make_case(n, nside, *, seed=11, n_sub=3, single_frac=0.0, skipped=0):
    """Particles whose smoothing lengths are those of an N_FULL-particle halo
    (h scales as n^(-1/3)), a fraction of them shrunk below a pixel
    (single-pixel deposits), and ``skipped`` of them masked or above the
    hires-mass threshold."""
    P = synth.nfw_halo(n, seed=seed, n_sub=n_sub)
    P.h *= np.float32((n / N_FULL) ** (1.0 / 3.0))
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    if single_frac > 0:
        idx = rng.choice(n, int(single_frac * n), replace=False)
        P.h[idx] *= np.float32(1e-3)
    if skipped:
        idx = rng.choice(n, skipped, replace=False)
        P.rho[idx[: skipped // 2]] = -1.0                      # masked
        P.m[idx[skipped // 2:]] = np.float32(P.particle_mass * 2.0)  # low resolution
    p = O.make_params(nside=nside, obs_pos=P.obs_pos, centerpos=P.centerpos,
                      align_vec=P.align_vec, particle_masses=(P.particle_mass,))
    return P, P.as_dict(), p


def jittered(P, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    d = P.as_dict()
    out = dict(d)
    for k in ("x", "y", "z"):
        out[k] = (d[k] + 0.1 * d["h"] * rng.standard_normal(len(P)).astype(np.float32)).astype(np.float32)
    return out


def loss_grad(mp, target):
    """(w, dL/dmap) of the weighted squared loss."""
    eps = 1e-3 * float(np.mean(target)) if np.mean(target) > 0 else 1.0
    w = 1.0 / (target + eps)
    return w, 2.0 * w * (mp - target)


def fd_check(p, parts, G, grad, rel_eps=1e-5):
    """Central differences of the oracle's per-particle loss (double inputs)
    against grad [6, n].  Particles whose pixel set changes between the two
    sides are left out.  Returns {field: (norm-wise relative error, number
    of particles compared)}."""
    d64 = {k: np.asarray(parts[k], dtype=np.float64) for k in FIELDS}
    if parts.get("sigmav") is not None:   # carried along, not differentiated
        d64["sigmav"] = np.asarray(parts["sigmav"], dtype=np.float64)
    out = {}
    for kk, k in enumerate(FIELDS):
        eps = rel_eps * (d64["h"] if k in ("x", "y", "z") else np.abs(d64[k]))
        eps = np.where(eps > 0, eps, rel_eps)
        pp, pm = dict(d64), dict(d64)
        pp[k] = d64[k] + eps
        pm[k] = d64[k] - eps
        Lp, sp = O.particle_losses(p, pp, G)
        Lm, sm = O.particle_losses(p, pm, G)
        ok = sp == sm
        fd = (Lp - Lm) / (2 * eps)
        num = np.linalg.norm((grad[kk] - fd)[ok])
        den = np.linalg.norm(fd[ok])
        out[k] = (num / den if den > 0 else num, int(ok.sum()))
    return out


def observer_fd(p, parts, G, step=1e-5):
    """Central differences of the summed oracle loss in the observer
    position, over the particles whose pixel sets stay fixed for all six
    displaced observers.  Returns (fd gradient [3], keep mask)."""
    d64 = {k: np.asarray(parts[k], dtype=np.float64) for k in FIELDS}
    o = np.array(p.obs_pos[:], dtype=np.float64)
    Ls, sigs = [], []
    for k in range(3):
        for s in (1.0, -1.0):
            q = o.copy()
            q[k] += s * step
            L, sg = O.particle_losses(O.with_observer(p, q), d64, G)
            Ls.append(L)
            sigs.append(sg)
    keep = np.ones(len(d64["x"]), dtype=bool)
    for sg in sigs[1:]:
        keep &= sg == sigs[0]
    fd = np.array([(Ls[2 * k][keep].sum() - Ls[2 * k + 1][keep].sum()) / (2 * step) for k in range(3)])
    return fd, keep
