"""GPU parity: the CUDA projection (through the C ABI) against the reference.

  * golden fixtures -- maps made by the reference's own genmap.cpp build;
  * the FP64 oracle on larger seeded synthetic halos;
  * size-independent properties at full Nside: flux conservation
    (sum(map) * dOmega == sum of kept flux, the reference's "Total Conts"),
    linearity (chunked streaming == one call, accumulate doubles the map),
    host and device inputs agree.

Tolerances (stated per the contract of the two forms):
  plain FP64   per-pixel relative error <= 1e-10 (only the order of the FP64
               additions differs from the CPU path); total flux 1e-12
  compensated  per-pixel relative error: median <= 1e-5, max <= 1e-4; total
               flux <= 1e-9
  Relative errors are taken over pixels whose reference value exceeds
  1e-6 of the map maximum; the set of non-zero pixels must match exactly
  (disc membership is decided in FP64 by both forms).
"""
import math

import numpy as np
import pytest

import annmap
import golden_cases as G
import oracle as O
from annmap import synth

pytestmark = pytest.mark.gpu

PLAIN, COMP = annmap.PLAIN_F64, annmap.COMP_F32
FLOOR = 1e-6


def rel_errors(got, ref):
    mask = ref > FLOOR * ref.max()
    rel = np.abs(got[mask] - ref[mask]) / ref[mask]
    return float(np.median(rel)), float(rel.max())


def check(got, ref, precision, total=None, dOmega=None):
    assert np.all(np.isfinite(got))
    assert np.array_equal(got != 0, ref != 0), "non-zero pixel sets differ"
    med, mx = rel_errors(got, ref)
    if precision == PLAIN:
        assert mx <= 1e-10, (med, mx)
    else:
        assert med <= 1e-5 and mx <= 1e-4, (med, mx)
    if total is not None:
        tol = 1e-12 if precision == PLAIN else 1e-9
        assert math.isclose(got.sum() * dOmega, total, rel_tol=tol), (got.sum() * dOmega, total)
    return med, mx


@pytest.fixture(scope="module")
def rend():
    r = annmap.Renderer(0)
    yield r
    r.close()


@pytest.mark.parametrize("precision", [PLAIN, COMP])
@pytest.mark.parametrize("name", G.names())
def test_golden_maps(rend, name, precision):
    case = G.load(name)
    p = annmap.Parameters(text=case["info_text"].replace("@DIR@", "/x"))
    rend.set_params(p, flux_model=case["flux_law"])
    if len(case["halos"]):
        rend.set_halo_cores(*[case["halos"][:, k] for k in range(4)])
    got = rend.render(case["parts"], p.map.Nside, precision)
    ref = case["map"]
    st = rend.stats()
    check(got, ref, precision, total=ref.sum() * p.map.dOmega, dOmega=p.map.dOmega)
    assert math.isclose(st["total_flux"], ref.sum() * p.map.dOmega, rel_tol=1e-12)


@pytest.mark.parametrize("precision", [PLAIN, COMP])
def test_golden_via_mapgenerator(tmp_path, precision):
    """The reference's own flow: info file + native data file (+ mask, test
    limit, chunked buffer) through MapGenerator."""
    case = G.load("hires_mask_ns32")
    z = np.load(G.GOLDEN + "/hires_mask_ns32.npz")
    rec, mask = z["records"], z["mask"]
    data = tmp_path / "parts.bin"
    with open(data, "wb") as f:
        np.array([len(rec)], np.int32).tofile(f)
        rec.tofile(f)
    mpath = tmp_path / "mask.bin"
    with open(mpath, "wb") as f:
        np.array([len(rec)], np.int32).tofile(f)
        mask.tofile(f)
    text = case["info_text"].replace("@DIR@/parts.bin", str(data)).replace("@DIR@/mask.bin", str(mpath))
    par = annmap.Parameters(text=text.replace("mem_buffer = 1000", "mem_buffer = 333"))
    reader = annmap.DataReader(par.nativeDatafile, par.isMask, par.maskFileName)
    reader.setTest(par.testNum)
    reader.setBuf(par.memParts)
    reader.open()
    gen = annmap.MapGenerator(par, reader, precision=precision)
    gen.start()
    reader.close()
    assert gen.isFinished() and gen.getNside() == 32
    check(gen.getMap(), case["map"], precision)


@pytest.mark.parametrize("precision", [PLAIN, COMP])
def test_synthetic_vs_oracle(rend, precision):
    P = synth.nfw_halo(20000, seed=5150, n_sub=12)
    nside = 256
    par = annmap.Parameters.for_synthetic(P, nside)
    o = O.make_params(nside=nside, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                      particle_masses=(P.particle_mass,))
    ref, ost, tot = O.render(o, P.as_dict(), nthreads=8)
    rend.set_params(par)
    got = rend.render(P.as_dict(), nside, precision)
    st = rend.stats()
    med, mx = check(got, ref, precision, total=tot, dOmega=o.dOmega)
    assert st["deposits"] == ost["deposits"]
    assert st["n_single"] == ost["single_small"]
    print(f"precision={precision} median={med:.3e} max={mx:.3e}")


def test_comp_vs_plain_full_nside(rend):
    """Both forms at Nside 2048 on the first 4096 particles of a 2^16-particle
    version of the 16M-particle workload (fatter particles: about 3.6e6 disc
    pixels each): compensated against plain FP64 (the FP64 reference here)."""
    P, nside = synth.workload("nfw16m_sub100_ns2048", scale=1 / 256)
    P = P.subset(slice(0, 4096))
    par = annmap.Parameters.for_synthetic(P, nside)
    rend.set_params(par)
    plain = rend.render(P.as_dict(), nside, PLAIN)
    tp = rend.stats()
    comp = rend.render(P.as_dict(), nside, COMP)
    tc = rend.stats()
    assert np.array_equal(plain != 0, comp != 0)
    med, mx = rel_errors(comp, plain)
    assert med <= 1e-5 and mx <= 1e-4, (med, mx)
    dom = par.map.dOmega
    assert math.isclose(plain.sum() * dom, tp["total_flux"], rel_tol=1e-12)
    assert math.isclose(comp.sum() * dom, tc["total_flux"], rel_tol=1e-9)
    assert tp["deposits"] == tc["deposits"]
    print(f"nside 2048: median={med:.3e} max={mx:.3e} deposits={tc['deposits']} "
          f"plain {tp['kernel_ms']:.1f} ms comp {tc['kernel_ms']:.1f} ms")


@pytest.mark.parametrize("precision", [PLAIN, COMP])
def test_streaming_equals_single_call(rend, precision):
    P = synth.nfw_halo(6000, seed=77, n_sub=4)
    nside = 128
    par = annmap.Parameters.for_synthetic(P, nside)
    rend.set_params(par)
    one = rend.render(P.as_dict(), nside, precision)
    rend.begin(nside, precision)
    d = P.as_dict()
    for i0 in range(0, len(P), 1700):
        rend.add({k: v[i0:i0 + 1700] for k, v in d.items()})
    rend.add({k: v[:0] for k, v in d.items()})  # an empty chunk
    two = rend.end()
    # chunking changes only the order of the additions, which both forms make
    # in FP64 (rounding at ~1e-16 of a pixel).  In the compensated form the
    # order in which warps claim rings also moves a particle's normalisation
    # by ~1e-13, so a deposit lying that close to an FP32 rounding boundary
    # rounds the other way: at most 2^-24 of that deposit.
    tol = 1e-12 if precision == PLAIN else 1e-7
    np.testing.assert_allclose(two, one, rtol=tol, atol=0)
    acc = rend.render(P.as_dict(), nside, precision, out=one.copy(), accumulate=True)
    np.testing.assert_allclose(acc, 2 * one, rtol=tol)


def test_device_inputs_and_output(rend):
    torch = pytest.importorskip("torch")
    P = synth.nfw_halo(5000, seed=99)
    nside = 128
    par = annmap.Parameters.for_synthetic(P, nside)
    rend.set_params(par)
    host = rend.render(P.as_dict(), nside, COMP)
    dev = {k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}
    out = torch.zeros(12 * nside * nside, dtype=torch.float64, device="cuda")
    rend.render(dev, nside, COMP, out=out)
    torch.cuda.synchronize()
    # same arithmetic; the order of the FP64 reductions differs run to run,
    # and a deposit may round the other way in FP32 (see the chunking test)
    np.testing.assert_allclose(out.cpu().numpy(), host, rtol=1e-7)


def test_edge_cases(rend):
    nside = 64
    P = synth.nfw_halo(300, seed=3)
    par = annmap.Parameters.for_synthetic(P, nside)
    rend.set_params(par)
    d = P.as_dict()
    # empty input: an all-zero map
    empty = rend.render({k: v[:0] for k, v in d.items()}, nside, COMP)
    assert not empty.any() and rend.stats()["n_in"] == 0
    # all particles masked (rho < 0): nothing kept
    masked = dict(d, rho=-np.abs(d["rho"]))
    mp = rend.render(masked, nside, COMP)
    assert not mp.any() and rend.stats()["n_kept"] == 0
    # degenerate particles: at the observer, NaN / negative / infinite h
    o = np.array(P.obs_pos, np.float32)
    # an observer exactly representable in float32, so a particle can sit on it
    rend.set_frame(par.rotmatrix, o.astype(np.float64))
    bad = {k: v[:4].copy() for k, v in d.items()}
    bad["x"][0], bad["y"][0], bad["z"][0] = o
    bad["h"][1] = np.nan
    bad["h"][2] = -1.0
    bad["h"][3] = np.inf
    mp = rend.render(bad, nside, COMP)
    st = rend.stats()
    assert np.all(np.isfinite(mp)) and st["n_invalid"] == 4 and not mp.any()
    rend.set_params(par)
    # one all-sky particle (2 ar > pi): every pixel receives flux
    one = {k: v[:1].copy() for k, v in d.items()}
    one["x"][0], one["y"][0], one["z"][0] = o + np.float32(0.05)
    one["h"][0] = 2.0
    for prec in (PLAIN, COMP):
        mp = rend.render(one, nside, prec)
        assert np.all(mp > 0)
        assert math.isclose(mp.sum() * par.map.dOmega, rend.stats()["total_flux"], rel_tol=1e-9)


def test_invalid_arguments(rend):
    P = synth.nfw_halo(100, seed=4)
    par = annmap.Parameters.for_synthetic(P, 16)
    rend.set_params(par)
    with pytest.raises(annmap.DmannError):
        rend.render(P.as_dict(), 0, COMP)
    with pytest.raises(annmap.DmannError):
        rend.render(P.as_dict(), 16385, COMP)
    with pytest.raises(annmap.DmannError):
        rend.render(P.as_dict(), 16, 7)
    with pytest.raises(annmap.DmannError):
        rend.set_units(-1.0)
    with pytest.raises(annmap.DmannError):
        rend.set_observer((1, 1, 1), (1, 1, 1), (0, 0, 1))
    # the context stays usable after errors
    rend.set_params(par)
    assert rend.render(P.as_dict(), 16, COMP).sum() > 0


def test_open_map_refuses_other_calls(rend):
    """While a streamed map is open its buffers are in use: another begin, a
    render, a batch and an adjoint on the same context fail with
    DMANN_ERR_STATE and leave the open map intact; abort closes it."""
    P = synth.nfw_halo(3000, seed=44, n_sub=2)
    par = annmap.Parameters.for_synthetic(P, 32)
    rend.set_params(par)
    ref = rend.render(P.as_dict(), 32, COMP)
    half = {k: v[:1500] for k, v in P.as_dict().items()}
    rest = {k: v[1500:] for k, v in P.as_dict().items()}
    rend.begin(32, COMP)
    rend.add(half)
    for call in (lambda: rend.begin(32, COMP),
                 lambda: rend.render(P.as_dict(), 32, COMP),
                 lambda: rend.render_batch(P.as_dict(), [(par.rotmatrix, par.params.opos)], [32], COMP),
                 lambda: rend.adjoint(P.as_dict(), 32, np.ones(12 * 32 * 32))):
        with pytest.raises(annmap.DmannError) as e:
            call()
        assert e.value.status == annmap._lib.ERR_STATE
    rend.add(rest)
    got = rend.end()
    assert np.array_equal(got != 0, ref != 0)
    np.testing.assert_allclose(got, ref, rtol=1e-7, atol=0)
    # abort: the open map is dropped and the next render starts from zero
    rend.begin(32, COMP)
    rend.add(half)
    rend.abort()
    np.testing.assert_allclose(rend.render(P.as_dict(), 32, COMP), ref, rtol=1e-7, atol=0)


@pytest.mark.parametrize("device_maps", [False, True])
def test_render_batch_matches_single_renders(rend, device_maps):
    """Several observers on the 8 kpc sphere, Nside cycling 32/64/128, in one
    call: each map equals the map of a single render with that observer."""
    torch = pytest.importorskip("torch")
    P = synth.nfw_halo(8000, seed=808, n_sub=5)
    obs = synth.batched_observers(6, nsides=(32, 64, 128))
    frames, nsides = [], []
    for o, ns in obs:
        par = annmap.Parameters.for_synthetic(synth.Particles(
            P.x, P.y, P.z, P.m, P.rho, P.h, o, P.centerpos, P.align_vec, P.particle_mass), ns)
        frames.append((par.rotmatrix, par.params.opos))
        nsides.append(ns)
    par0 = annmap.Parameters.for_synthetic(P, 64)
    rend.set_params(par0)
    outs = None
    if device_maps:
        outs = [torch.zeros(12 * ns * ns, dtype=torch.float64, device="cuda") for ns in nsides]
    got = rend.render_batch(P.as_dict(), frames, nsides, COMP, outs=outs)
    if device_maps:
        got = [g.cpu().numpy() for g in got]
    for (rot, opos), ns, g in zip(frames, nsides, got):
        rend.set_frame(rot, opos)
        ref = rend.render(P.as_dict(), ns, COMP)
        assert np.array_equal(g != 0, ref != 0)
        # two independent compensated renders: the run-to-run bound (ring-claim
        # order can flip a deposit's one FP32 rounding; FP64 addition order)
        np.testing.assert_allclose(g, ref, rtol=1e-7, atol=0)
    rend.set_params(par0)


def test_flux_law_needs_velocity_dispersion(rend):
    case = G.load("flux_ann_somv_ns32")
    p = annmap.Parameters(text=case["info_text"].replace("@DIR@", "/x"))
    rend.set_params(p, flux_model="ann_somv")
    parts = {k: v for k, v in case["parts"].items() if k != "sigmav"}
    with pytest.raises(annmap.DmannError):
        rend.render(parts, p.map.Nside, COMP)
    rend.set_params(p)   # back to nosom: sigmav not needed
    rend.render(parts, p.map.Nside, COMP)


def test_torch_default_stream_orders_the_render():
    """On torch's default (legacy) stream the render is ordered before torch's
    next operation without any synchronisation by the caller."""
    torch = pytest.importorskip("torch")
    P = synth.nfw_halo(200000, seed=77, n_sub=3)
    par = annmap.Parameters.for_synthetic(P, 512)
    r = annmap.Renderer(0)
    r.set_params(par)
    d = {k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}
    ref = r.render(P.as_dict(), 512, COMP)          # host map: complete on return
    out = torch.zeros(12 * 512 * 512, dtype=torch.float64, device="cuda")
    assert torch.cuda.current_stream().cuda_stream == 0
    r.render(d, 512, COMP, out=out)                  # queued on torch's stream
    total = float(out.sum())                         # torch reads it at once
    assert math.isclose(total, float(ref.sum()), rel_tol=1e-9)
    maps = [torch.zeros(12 * 64 * 64, dtype=torch.float64, device="cuda") for _ in range(2)]
    frames = [(np.array(par.rot_flat()), P.obs_pos)] * 2
    r.render_batch(d, frames, [64, 64], COMP, outs=maps)
    assert float(maps[1].sum()) > 0 and math.isclose(float(maps[0].sum()), float(maps[1].sum()), rel_tol=1e-9)
    r.close()
