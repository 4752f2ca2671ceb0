"""Block shapes and footprint bins on the GPU: every tuning renders the same
map (to accumulation order), the per-Nside table is honoured by single and
batched renders, and the autotuner applies what it measured."""
import numpy as np
import pytest

import annmap
import oracle as O
from annmap import autotune, synth

pytestmark = pytest.mark.gpu

COMP, PLAIN = annmap.COMP_F32, annmap.PLAIN_F64


@pytest.fixture(scope="module")
def setup():
    P = synth.nfw_halo(60000, seed=31, n_sub=4, near_observer=30)
    par = annmap.Parameters.for_synthetic(P, 256)
    r = annmap.Renderer(0)
    r.set_params(par)
    yield P, par, r
    r.close()


def _rel(a, b):
    m = b > 1e-6 * b.max()
    return float(np.max(np.abs(a[m] - b[m]) / b[m]))


@pytest.mark.parametrize("bt", [128, 256, 512])
@pytest.mark.parametrize("wmp", [64, 1024, 1 << 20])
def test_every_tuning_gives_the_same_map(setup, bt, wmp):
    P, par, r = setup
    ref = r.render(P.as_dict(), 256, PLAIN)
    r.set_tuning(nside=256, block_threads=bt, warp_max_pixels=wmp)
    got = r.render(P.as_dict(), 256, COMP)
    st = r.stats()
    r.clear_tuning(256)
    assert np.array_equal(got != 0, ref != 0)
    assert _rel(got, ref) < 1e-4
    if wmp == 1 << 20:
        assert st["n_disc_block"] == 0 or st["n_disc_block"] < st["n_disc"]
    assert abs(got.sum() - ref.sum()) <= 1e-9 * ref.sum()


def test_tuning_table_validation(setup):
    P, par, r = setup
    with pytest.raises(annmap.DmannError):
        r.set_tuning(nside=256, block_threads=300)
    r.set_tuning(nside=512, block_threads=512, warp_max_pixels=128)
    t = r.get_tuning(512)
    assert t["block_threads"] == 512 and t["warp_max_pixels"] == 128 and t["ring_chunk"] == 640
    assert r.get_tuning(256)["block_threads"] == r.get_tuning()["block_threads"]
    r.clear_tuning(512)
    assert r.get_tuning(512) == r.get_tuning()


def test_batch_honours_per_nside_tuning(setup):
    torch = pytest.importorskip("torch")
    P, par, r = setup
    obs = synth.batched_observers(4, nsides=(64, 128))
    frames, nsides = [], []
    for opos, ns in obs:
        par.set_observer(opos)
        frames.append((np.array(par.rot_flat()), opos))
        nsides.append(ns)
    # the per-disc kernels' FP64 deposits (this halo's fat particles would
    # take the segmented render, whose FP32 partial sums depend on the order
    # of the deposits at their own ~1e-7 level)
    r.set_tuning(seg_min_deposits_log2=62)
    base = r.render_batch(P.as_dict(), frames, nsides, COMP)
    r.set_tuning(nside=64, block_threads=128, warp_max_pixels=64)
    r.set_tuning(nside=128, block_threads=512, warp_max_pixels=8192)
    outs = [torch.zeros(12 * ns * ns, dtype=torch.float64, device="cuda") for ns in nsides]
    r.render_batch({k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}, frames, nsides,
                   COMP, outs=outs)
    r.clear_tuning(64)
    r.clear_tuning(128)
    r.set_tuning(seg_min_deposits_log2=28)
    par.set_observer(P.obs_pos)
    for b, o in zip(base, outs):
        o = o.cpu().numpy()
        # other block shapes claim rings in another order: a deposit's one FP32
        # rounding may flip (at most 2^-24 of that deposit)
        assert np.array_equal(o != 0, b != 0) and _rel(o, b) < 1e-7


def test_autotune_applies_the_fastest(setup, tmp_path):
    torch = pytest.importorskip("torch")
    P, par, r = setup
    out = torch.zeros(12 * 256 * 256, dtype=torch.float64, device="cuda")
    dparts = {k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}
    res = autotune.tune(r, dparts, 256, COMP, sample=40000, reps=1, cache=str(tmp_path / "c.json"),
                        out=out)
    assert len(res["trials"]) == 9 and not res["cached"]
    best = min(res["trials"], key=lambda t: t["ms"])
    assert res["best"] == best["tuning"]
    t = r.get_tuning(256)
    assert all(t[k] == v for k, v in res["best"].items())
    r.clear_tuning(256)
