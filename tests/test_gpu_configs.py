"""GPU parity at the sizes of the benchmark's configurations, against the FP64
oracle (the restated reference CPU map path, src/genmap.cpp:22-175) run on
every host thread.

  * 1,048,576-particle NFW halo at Nside 512 (the plain method's own size,
    rendered in full): the plain form and the compensated form;
  * the 16,777,216-particle NFW + 100 subhalo set at Nside 2048: a 2^16-
    particle prefix (the set is shuffled, so a prefix is an i.i.d. sample),
    both forms;
  * the batched set (8,388,608 particles, NFW + 50 subhalos): three observers
    on the 8 kpc sphere with Nside 256, 512 and 1024 rendered by one
    dmann_render_batch call, on a 2^17-particle prefix;
  * the large-map set (NFW + 500 subhalos, particles within 0.5 kpc of the
    observer) at Nside 4096: an i.i.d. sample of it, with one disc covering
    the whole sky;
  * the segmented render (FP32 deposits in segments of at most two octaves of
    the deposit scale, flushed into the FP64 plane) forced onto the samples
    above, which by default are small enough to deposit in FP64.

Tolerances: per-pixel relative error median <= 1e-5, max <= 1e-4 and total
flux <= 1e-9 relative for the compensated form; for the plain form the
per-pixel bound plain_tol(nside) and total flux <= 1e-11; the sets of
non-zero pixels equal.  Errors are taken over pixels above 1e-6 of the map
maximum.

The plain form repeats the CPU path's FP64 arithmetic, and its weights take
acos of the dot product of two unit vectors, as src/genmap.cpp:137-143
does.  Near 1 that acos is ill-conditioned: a one-ulp difference in the
particle's direction (CUDA's and the C library's sin and cos may round
differently) moves theta by about 1e-16 / theta, a relative weight error of
about 6e-16 / theta^2 at the disc edge.  The smallest discs have theta of a
few pixel widths, about 5e-4 * 2048 / nside radians, so the bound grows as
nside^2: 1e-9 * (nside / 1024)^2 (measured: 6e-10 at Nside 2048).
"""
import math
import os

import numpy as np
import pytest

import annmap
import oracle as O
from annmap import synth

pytestmark = pytest.mark.gpu

PLAIN, COMP = annmap.PLAIN_F64, annmap.COMP_F32
THREADS = os.cpu_count() or 1


def rel_errors(got, ref):
    mask = ref > 1e-6 * ref.max()
    rel = np.abs(got[mask] - ref[mask]) / ref[mask]
    return float(np.median(rel)), float(rel.max())


def plain_tol(nside):
    return max(1e-10, 1e-9 * (nside / 1024.0) ** 2)


def check(got, ref, total, dOmega, precision, what, nside):
    assert np.all(np.isfinite(got)), what
    assert np.array_equal(got != 0, ref != 0), f"{what}: non-zero pixel sets differ"
    med, mx = rel_errors(got, ref)
    tot_rel = abs(got.sum() * dOmega - total) / total
    print(f"{what}: median {med:.3e} max {mx:.3e} total flux {tot_rel:.3e}")
    if precision == PLAIN:
        assert mx <= plain_tol(nside), (what, med, mx)
        assert tot_rel <= 1e-11, (what, tot_rel)
    else:
        assert med <= 1e-5 and mx <= 1e-4, (what, med, mx)
        assert tot_rel <= 1e-9, (what, tot_rel)


def oracle_map(P, nside, obs_pos=None):
    o = O.make_params(nside=nside, obs_pos=obs_pos or P.obs_pos, centerpos=P.centerpos,
                      align_vec=P.align_vec, particle_masses=(P.particle_mass,))
    ref, st, tot = O.render(o, P.as_dict(), nthreads=THREADS)
    return o, ref, st, tot


@pytest.fixture(scope="module")
def rend():
    r = annmap.Renderer(0)
    yield r
    r.close()


def test_config_nfw1m_ns512_in_full(rend):
    """1,048,576 particles at Nside 512, the whole set: both forms against the
    oracle, and the deposit count equal to the oracle's."""
    P, nside = synth.workload("nfw1m_ns512")
    assert len(P) == 1 << 20
    o, ref, ost, tot = oracle_map(P, nside)
    rend.set_params(annmap.Parameters.for_synthetic(P, nside))
    for prec in (PLAIN, COMP):
        got = rend.render(P.as_dict(), nside, prec)
        check(got, ref, tot, o.dOmega, prec, f"nfw1m_ns512 precision {prec}", nside)
        assert rend.stats()["deposits"] == ost["deposits"]


def test_config_nfw16m_ns2048_prefix(rend):
    """The first 65,536 particles of the 16M-particle set at Nside 2048."""
    P, nside = synth.workload("nfw16m_sub100_ns2048")
    P = P.subset(slice(0, 1 << 16))
    o, ref, ost, tot = oracle_map(P, nside)
    rend.set_params(annmap.Parameters.for_synthetic(P, nside))
    for prec in (COMP, PLAIN):
        got = rend.render(P.as_dict(), nside, prec)
        check(got, ref, tot, o.dOmega, prec, f"nfw16m prefix precision {prec}", nside)
        assert rend.stats()["deposits"] == ost["deposits"]


def test_config_batched_three_observers(rend):
    """dmann_render_batch over three observers of the batched configuration
    (Nside 256, 512, 1024), each map against the oracle for its observer."""
    torch = pytest.importorskip("torch")
    P, _ = synth.workload("nfw8m_sub50_batched")
    P = P.subset(slice(0, 1 << 17))
    obs = synth.batched_observers(3)
    assert sorted(ns for _, ns in obs) == [256, 512, 1024]
    frames, nsides = [], []
    for opos, ns in obs:
        par = annmap.Parameters.for_synthetic(synth.Particles(
            P.x, P.y, P.z, P.m, P.rho, P.h, opos, P.centerpos, P.align_vec, P.particle_mass), ns)
        frames.append((par.rotmatrix, par.params.opos))
        nsides.append(ns)
    rend.set_params(annmap.Parameters.for_synthetic(P, 512))
    dev = {k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}
    outs = [torch.zeros(12 * ns * ns, dtype=torch.float64, device="cuda") for ns in nsides]
    rend.render_batch(dev, frames, nsides, COMP, outs=outs)
    torch.cuda.synchronize()
    for (opos, ns), out in zip(obs, outs):
        o, ref, _, tot = oracle_map(P, ns, obs_pos=opos)
        check(out.cpu().numpy(), ref, tot, o.dOmega, COMP, f"batched observer Nside {ns}", ns)


def large_map_sample():
    m = 4.1e3 * (1 << 24) / (1 << 27)
    P = synth.nfw_halo(1 << 16, seed=20240013, n_sub=500, particle_mass=m, near_observer=4,
                       n_total=1 << 27)
    # one near-observer particle moved to 0.02 kpc of the observer: its disc
    # (radius 2 h / d > pi) covers the whole sky
    obs = np.array(P.obs_pos)
    pos = np.stack([P.x, P.y, P.z], 1).astype(np.float64)
    d = np.linalg.norm(pos - obs, axis=1)
    near = np.flatnonzero(d < 0.5)
    assert len(near) >= 4
    k = near[0]
    P.x[k], P.y[k], P.z[k] = (obs + 0.02 / math.sqrt(3.0)).astype(np.float32)
    d[k] = np.linalg.norm(np.array([P.x[k], P.y[k], P.z[k]], np.float64) - obs)
    assert 2 * P.h[k] / d[k] > math.pi
    return P, 4096


def test_config_large_map_sample_ns4096(rend):
    """An i.i.d. sample of the large-map configuration: 65,536 particles of the
    134,217,728-particle NFW + 500 subhalo set (its particle mass and
    densities), 4 of them within 0.5 kpc of the observer, at Nside 4096
    (201,326,592 pixels), both forms."""
    P, nside = large_map_sample()
    o, ref, ost, tot = oracle_map(P, nside)
    rend.set_params(annmap.Parameters.for_synthetic(P, nside))
    for prec in (COMP, PLAIN):
        got = rend.render(P.as_dict(), nside, prec)
        check(got, ref, tot, o.dOmega, prec, f"large-map sample precision {prec}", nside)
        assert rend.stats()["deposits"] == ost["deposits"]
        assert np.all(got > 0)   # the all-sky disc reaches every pixel


@pytest.mark.parametrize("case", ["nfw1m_ns512", "nfw16m_prefix", "large_map_sample"])
@pytest.mark.parametrize("block_threads", [128, 256])
def test_segmented_render_forced(case, block_threads):
    """The segmented render taken on chunks of any size (its threshold at 2
    estimated deposits), both block shapes: the same bounds against the
    oracle, the same deposits, and the pass timings that only the segmented
    render records."""
    if case == "nfw1m_ns512":
        P, nside = synth.workload("nfw1m_ns512")
    elif case == "nfw16m_prefix":
        P, nside = synth.workload("nfw16m_sub100_ns2048")
        P = P.subset(slice(0, 1 << 16))
    else:
        P, nside = large_map_sample()
    o, ref, ost, tot = oracle_map(P, nside)
    r = annmap.Renderer(0)
    try:
        r.set_tuning(seg_min_deposits_log2=1, block_threads=block_threads)
        r.set_params(annmap.Parameters.for_synthetic(P, nside))
        got = r.render(P.as_dict(), nside, COMP)
        st = r.stats()
        check(got, ref, tot, o.dOmega, COMP, f"segmented {case} {block_threads} threads", nside)
        assert st["deposits"] == ost["deposits"]
        assert st["pass2_ms"] > 0.0
    finally:
        r.close()
