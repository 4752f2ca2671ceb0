"""The FP64 oracle against the reference's own CPU map path (golden
fixtures) and against HEALPix identities.  CPU only."""
import math

import numpy as np
import pytest

import golden_cases as G
import oracle as O


@pytest.mark.parametrize("name", G.names())
def test_oracle_matches_reference_build(name):
    case = G.load(name)
    p = G.oracle_params(case)
    mp, st, tot = O.render(p, case["parts"], nthreads=1)
    ref = case["map"]
    # Same float operations in the same order: bit for bit on this machine;
    # 1e-13 allows for libm last-bit differences on another architecture.
    assert mp.shape == ref.shape
    np.testing.assert_allclose(mp, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    # total flux: sum(map * dOmega) == sum of the kept particles' flux
    assert math.isclose(tot, ref.sum() * p.dOmega, rel_tol=1e-12)


@pytest.mark.parametrize("name", G.names())
def test_oracle_parameters_match_reference(name):
    case = G.load(name)
    p = G.oracle_params(case)
    par = case["par"]
    rot = O.rotmatrix(p)
    for i in range(3):
        np.testing.assert_allclose(rot[i], par[f"rotmatrix{i}"], rtol=0, atol=1e-15)
    assert p.otheta == pytest.approx(par["otheta"][0], rel=1e-15)
    assert p.ophi == pytest.approx(par["ophi"][0], rel=1e-15)
    assert p.annihilation_flux_to_cgs == pytest.approx(par["annihilation_flux_to_cgs"][0], rel=1e-15)
    assert p.mass_to_cgs == pytest.approx(par["mass_to_cgs"][0], rel=1e-15)
    assert p.dOmega == pytest.approx(par["dOmega"][0], rel=1e-15)


def test_oracle_threads_match_serial():
    case = G.load("nfw_sub_ns64")
    p = G.oracle_params(case)
    a, _, ta = O.render(p, case["parts"], nthreads=1)
    b, _, tb = O.render(p, case["parts"], nthreads=4)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14 * np.abs(a).max())
    assert math.isclose(ta, tb, rel_tol=1e-12)


# ------------------------------------------------------------------ HEALPix
@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16, 24, 32])
def test_ring_layout(nside):
    hp = O.Healpix(nside)
    total = 0
    for ring in range(1, 4 * nside):
        start, nr, shifted = hp.ring_info(ring)
        assert start == total
        expect = 4 * min(ring, nside, 4 * nside - ring)
        assert nr == expect
        total += nr
    assert total == 12 * nside * nside


@pytest.mark.parametrize("nside", [1, 4, 16, 24, 64])
def test_pix2vec_ang2pix_roundtrip(nside):
    hp = O.Healpix(nside)
    for pix in range(hp.npix):
        t, ph = hp.pix2ang(pix)
        assert hp.ang2pix(t, ph) == pix
        v = hp.pix2vec(pix)
        assert abs(np.linalg.norm(v) - 1) < 1e-15


def _angdist(v, w):
    return math.atan2(np.linalg.norm(np.cross(v, w)), float(np.dot(v, w)))


@pytest.mark.parametrize("nside", [4, 16, 24])
def test_query_disc_brute_force(nside):
    hp = O.Healpix(nside)
    vecs = np.array([hp.pix2vec(p) for p in range(hp.npix)])
    rng = np.random.Generator(np.random.PCG64(nside))
    for _ in range(60):
        th = math.acos(rng.uniform(-1, 1))
        ph = rng.uniform(0, 2 * math.pi)
        rad = rng.choice([0.02, 0.1, 0.5, 1.3, 2.5, 3.0])
        got = set(hp.query_disc(th, ph, rad).tolist())
        c = np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])
        dist = np.array([_angdist(v, c) for v in vecs])
        inside = set(np.nonzero(dist < rad - 1e-12)[0].tolist())
        maybe = set(np.nonzero(np.abs(dist - rad) <= 1e-12)[0].tolist())
        assert inside <= got
        assert got <= inside | maybe


def test_query_disc_allsky_and_poles():
    hp = O.Healpix(16)
    assert len(hp.query_disc(1.0, 2.0, math.pi)) == hp.npix
    # disc around the north pole: whole polar rings
    got = hp.query_disc(0.0, 0.0, 0.3)
    assert len(got) > 0 and got.min() == 0
    got = hp.query_disc(math.pi, 0.0, 0.3)
    assert got.max() == hp.npix - 1


def test_query_disc_area():
    nside = 64
    hp = O.Healpix(nside)
    dom = 4 * math.pi / hp.npix
    for rad in (0.1, 0.3, 1.0):
        n = len(hp.query_disc(1.1, 0.7, rad))
        area = 2 * math.pi * (1 - math.cos(rad))
        assert abs(n * dom - area) / area < 0.05


def test_single_pixel_particle_lands_at_ang2pix():
    case = G.load("nfw_ns16")
    p = G.oracle_params(case)
    # a distant tiny particle: all its flux in one pixel
    parts = {k: np.array([v], np.float32) for k, v in
             dict(x=300.0, y=-20.0, z=45.0, m=4100.0, rho=1e5, h=0.01).items()}
    mp, st, tot = O.render(p, parts)
    g = O.particle_geom(p, 4100.0, 1e5, 0.01, 300.0, -20.0, 45.0)
    assert st["single_small"] == 1
    nz = np.nonzero(mp)[0]
    assert nz.tolist() == [int(g["pix"])]
    assert mp[nz[0]] * p.dOmega == pytest.approx(g["flux"], rel=1e-15)
