"""CPU checks of the adjoint's references: the oracle's FP64 adjoint against
central finite differences of its own forward map (per particle and for the
observer position), and the library's forward-mode rotation Jacobian against
finite differences of the oracle's parameter set-up."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from adjoint_cases import FIELDS, fd_check, loss_grad, make_case, observer_fd


@pytest.fixture(scope="module")
def case():
    P, parts, p = make_case(3000, 128, single_frac=0.2, skipped=40)
    mp, st, _ = O.render(p, parts)
    assert st["single_small"] > 300 and st["disc"] > 1000 and st["skipped"] == 40
    target, _, _ = O.render(p, __import__("adjoint_cases").jittered(P))
    _, G = loss_grad(mp, target)
    grad, oacc = O.adjoint(p, parts, G)
    return P, parts, p, G, grad, oacc


def test_oracle_adjoint_matches_central_differences(case):
    P, parts, p, G, grad, oacc = case
    res = fd_check(p, parts, G, grad)
    for k in FIELDS:
        err, n_ok = res[k]
        assert n_ok > 2500, (k, n_ok)
        assert err < 1e-6, (k, err)


def test_oracle_adjoint_zero_for_skipped_particles(case):
    P, parts, p, G, grad, oacc = case
    skipped = (parts["rho"] < 0) | (parts["m"].astype(np.float64) >= p.hires_threshold)
    assert skipped.sum() == 40
    assert np.all(grad[:, skipped] == 0.0)
    assert np.all(np.isfinite(grad))


def test_oracle_observer_gradient_matches_central_differences(case):
    P, parts, p, G, grad, oacc = case
    fd, keep = observer_fd(p, parts, G)
    assert keep.sum() > 0.95 * len(keep)
    sub = {k: np.asarray(parts[k])[keep] for k in FIELDS}
    _, oa = O.adjoint(p, sub, G)
    go = O.observer_grad(p, oa)
    assert np.linalg.norm(go - fd) < 1e-6 * np.linalg.norm(fd)


def test_euler_identities_of_the_oracle_adjoint(case):
    """The map is linear in m and in rho, and scaling every offset from the
    observer and every h by s scales it by s^-2, so with L = sum G map:
    sum m dL/dm = sum rho dL/drho = L and sum (u . dL/du + h dL/dh) = -2 L."""
    P, parts, p, G, grad, oacc = case
    mp, _, _ = O.render(p, parts)
    L = float(np.dot(G, mp))
    o = np.array(p.obs_pos[:])
    u = np.stack([parts[k].astype(np.float64) - o[i] for i, k in enumerate(("x", "y", "z"))])
    m, rho, h = (parts[k].astype(np.float64) for k in ("m", "rho", "h"))
    assert np.sum(m * grad[3]) == pytest.approx(L, rel=1e-10)
    assert np.sum(rho * grad[4]) == pytest.approx(L, rel=1e-10)
    assert np.sum(u * grad[:3]) + np.sum(h * grad[5]) == pytest.approx(-2 * L, rel=1e-9)


def test_rotation_jacobian_matches_central_differences():
    from annmap import _lib
    L = _lib.load()
    # (points off the kinks of the roll angle |atan2(.)|, where only one-sided
    # derivatives exist)
    for opos, cpos, align in [((4.6, 4.6, 4.6), (0, 0, 0), (0, 0, 1)),
                              ((-3.0, 7.0, 1.5), (0.5, -0.2, 0.1), (0.3, 0.4, 0.866)),
                              ((8.0, 0.7, 0.1), (0, 0, 0), (0, 1, 0))]:
        p = O.make_params(nside=8, obs_pos=opos, centerpos=cpos, align_vec=align)
        jac = (C.c_double * 27)()
        d3 = lambda v: (C.c_double * 3)(*[float(a) for a in v])
        assert L.dmann_observer_rotation_jacobian(d3(opos), d3(cpos), d3(align), jac) == 0
        J = np.array(jac[:]).reshape(9, 3)
        Jfd = O.rotation_jacobian_fd(p)
        assert np.max(np.abs(J - Jfd)) < 1e-8 * max(1.0, np.max(np.abs(Jfd)))
        rot = (C.c_double * 9)()
        assert L.dmann_observer_rotation(d3(opos), d3(cpos), d3(align), rot, None) == 0
        assert np.array_equal(np.array(rot[:]).reshape(3, 3), O.rotmatrix(p))  # bit for bit
    jac = (C.c_double * 27)()
    z = (C.c_double * 3)(0, 0, 0)
    assert L.dmann_observer_rotation_jacobian(z, z, (C.c_double * 3)(0, 0, 1), jac) == 1


def test_sky_map_rejects_cpu_tensors():
    torch = pytest.importorskip("torch")
    from annmap.autograd import sky_map
    t = torch.zeros(4)
    with pytest.raises(ValueError):
        sky_map(t, t, t, t, t, t, torch.zeros(3, dtype=torch.float64), nside=4)


@pytest.fixture(scope="module")
def decay_case():
    """The decay law (src/flux/flux_decay.cpp): flux ~ m / d^2, no rho."""
    P, parts, p0 = make_case(2000, 128, seed=23, single_frac=0.2, skipped=20)
    p = O.make_params(nside=128, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                      particle_masses=(P.particle_mass,), flux_model=4)
    mp, _, _ = O.render(p, parts)
    target, _, _ = O.render(p, __import__("adjoint_cases").jittered(P))
    _, G = loss_grad(mp, target)
    grad, oacc = O.adjoint(p, parts, G)
    return P, parts, p, G, grad, mp


def test_oracle_adjoint_decay_law(decay_case):
    P, parts, p, G, grad, mp = decay_case
    assert np.all(grad[4] == 0.0)                      # no rho in the decay flux
    res = fd_check(p, parts, G, grad)
    for k in ("x", "y", "z", "m", "h"):
        err, n_ok = res[k]
        assert n_ok > 1600, (k, n_ok)
        assert err < 1e-6, (k, err)
    L = float(np.dot(G, mp))
    m = parts["m"].astype(np.float64)
    assert np.sum(m * grad[3]) == pytest.approx(L, rel=1e-10)


def core_halos(P, n=40, seed=9):
    """A halo-core table (x, y, z, radius in the table's units) whose cores
    hold some of P's particles: centres 1 kpc from particles (never on one:
    at r = 0 the reference's factor drops back to 1), core radii of a few kpc
    (the core radius is radius / (0.73 * 40000) box units)."""
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(P), n, replace=False)
    off = rng.standard_normal((n, 3))
    off /= np.linalg.norm(off, axis=1)[:, None]
    rad = rng.uniform(2.0, 8.0, n) * 0.73 * 40000.0
    return (P.x[idx] + off[:, 0], P.y[idx] + off[:, 1], P.z[idx] + off[:, 2], rad.astype(np.float32))


@pytest.mark.parametrize("law", [5, 6], ids=["adiabatic", "core"])
def test_oracle_adjoint_position_dependent_laws(law):
    """adiabatic (flux x f(r)^2, r from the halo centre) and ann_core_nosom
    (flux x the halo-core factor squared): the boost's own position gradient
    joins dL/dpos (the observer sums exclude it).  Central differences use
    the core factor on unrounded positions (exact_boost), the smooth
    function the adjoint differentiates."""
    P, parts, p0 = make_case(2000, 128, seed=50 + law, single_frac=0.2, skipped=20)
    halos = core_halos(P) if law == 6 else None
    kw = dict(nside=128, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
              particle_masses=(P.particle_mass,), flux_model=law, halos=halos)
    p = O.make_params(exact_boost=True, **kw)
    mp, _, _ = O.render(p, parts)
    target, _, _ = O.render(p, __import__("adjoint_cases").jittered(P))
    _, G = loss_grad(mp, target)
    grad, oacc = O.adjoint(p, parts, G)
    res = fd_check(p, parts, G, grad)
    for k in FIELDS:
        err, n_ok = res[k]
        assert n_ok > 1600, (k, n_ok)
        assert err < 1e-6, (k, err)
    L = float(np.dot(G, mp))
    m, rho = (parts[k].astype(np.float64) for k in ("m", "rho"))
    assert np.sum(m * grad[3]) == pytest.approx(L, rel=1e-10)
    assert np.sum(rho * grad[4]) == pytest.approx(L, rel=1e-10)
    # the boost term is present: without it the homogeneity identity
    # sum(u . dL/du) + sum(h dL/dh) = -2 L would hold; with it, it does not
    o = np.array(p.obs_pos[:])
    u = np.stack([parts[k].astype(np.float64) - o[i] for i, k in enumerate(("x", "y", "z"))])
    h = parts["h"].astype(np.float64)
    assert abs(np.sum(u * grad[:3]) + np.sum(h * grad[5]) + 2 * L) > 1e-6 * abs(L)
    # the observer gradient excludes the boost term (it moves with the
    # particle, not with the observer)
    fd, keep = observer_fd(p, parts, G)
    sub = {k: np.asarray(parts[k])[keep] for k in FIELDS}
    _, oa = O.adjoint(p, sub, G)
    go = O.observer_grad(p, oa)
    assert np.linalg.norm(go - fd) < 1e-6 * np.linalg.norm(fd)
    if law == 6:   # the parity (float-rounded) core factor moves the gradient by ~1e-7
        g_r, _ = O.adjoint(O.make_params(**kw), parts, G)
        assert np.linalg.norm(g_r - grad) < 1e-5 * np.linalg.norm(grad)


@pytest.mark.parametrize("law", [1, 2, 3], ids=["somv", "somv2", "pwave"])
def test_oracle_adjoint_sigma_v_laws(law):
    """somv, somv2, pwave: flux = rho m f(sigma v) / d^2 with sigma v held
    fixed (it is not differentiated); velocity dispersions straddle the
    somv / somv2 saturation speeds."""
    P, parts, p0 = make_case(2000, 128, seed=41 + law, single_frac=0.2, skipped=20)
    p = O.make_params(nside=128, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                      particle_masses=(P.particle_mass,), flux_model=law)
    rng = np.random.default_rng(law)
    kms = 1e5 / p.velocity_to_cgs                      # 1 km/s in code units
    parts = dict(parts, sigmav=(rng.uniform(0.2, 12.0, len(P)) * kms).astype(np.float32))
    mp, _, _ = O.render(p, parts)
    target, _, _ = O.render(p, dict(__import__("adjoint_cases").jittered(P), sigmav=parts["sigmav"]))
    _, G = loss_grad(mp, target)
    grad, oacc = O.adjoint(p, parts, G)
    res = fd_check(p, parts, G, grad)
    for k in FIELDS:
        err, n_ok = res[k]
        assert n_ok > 1600, (k, n_ok)
        assert err < 1e-6, (k, err)
    L = float(np.dot(G, mp))
    m, rho = (parts[k].astype(np.float64) for k in ("m", "rho"))
    assert np.sum(m * grad[3]) == pytest.approx(L, rel=1e-10)
    assert np.sum(rho * grad[4]) == pytest.approx(L, rel=1e-10)
    # without sigma v these laws' fluxes differ, and so does the gradient
    g0, _ = O.adjoint(p, {k: v for k, v in parts.items() if k != "sigmav"}, G)
    assert np.linalg.norm(g0[3] - grad[3]) > 0.1 * np.linalg.norm(grad[3]) > 0
