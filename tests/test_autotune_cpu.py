"""Autotuner search and cache logic against a stand-in renderer (no GPU)."""
import json

import numpy as np

from annmap import autotune


class FakeRenderer:
    """Duck-typed Renderer: kernel time is a fixed function of the tuning."""

    device = 0

    def __init__(self):
        self.tune = {}
        self.per_nside = {}
        self.renders = 0

    def set_tuning(self, nside=None, **kw):
        (self.per_nside.setdefault(nside, {}) if nside is not None else self.tune).update(kw)
        self._cur = dict(self.per_nside.get(nside, self.tune))

    def render(self, parts, nside, precision, out=None):
        self.renders += 1
        assert len(parts["x"]) <= 1000

    def stats(self):
        c = self._cur
        ms = abs(c.get("block_threads", 256) - 128) * 0.01 + abs(c.get("warp_max_pixels", 1024) - 4096) * 1e-3
        return {"kernel_ms": 10.0 + ms}


def _parts(n=5000):
    return {k: np.zeros(n, dtype=np.float32) for k in ("x", "y", "z", "m", "rho", "h")}


def test_tune_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "t.json")
    r = FakeRenderer()
    res = autotune.tune(r, _parts(), 256, sample=1000, reps=2, cache=path)
    assert res["best"] == {"block_threads": 128, "warp_max_pixels": 4096}
    assert not res["cached"] and len(res["trials"]) == 9 and r.renders == 18
    assert r.per_nside[256] == res["best"]
    table = json.load(open(path))
    assert res["key"] in table and "nside=256" in res["key"] and "n=2^10" in res["key"]
    r2 = FakeRenderer()
    res2 = autotune.tune(r2, _parts(), 256, sample=1000, cache=path)
    assert res2["cached"] and res2["best"] == res["best"] and r2.renders == 0
    assert r2.per_nside[256] == res["best"]


def test_tune_nsides_and_no_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("ANNMAP_TUNING_CACHE", str(tmp_path / "never.json"))
    r = FakeRenderer()
    out = autotune.tune_nsides(r, _parts(), [512, 256, 512], sample=500, reps=1, cache=False,
                               space={"block_threads": (256, 512)})
    assert sorted(out) == [256, 512]
    assert all(v["best"] == {"block_threads": 256} for v in out.values())
    assert not (tmp_path / "never.json").exists()


def test_tuning_key_buckets_sample_size():
    k1 = autotune.tuning_key("GB300", 2048, 1, 1 << 21)
    k2 = autotune.tuning_key("GB300", 2048, 1, (1 << 21) + 5)
    assert k1 == k2 and k1 != autotune.tuning_key("GB300", 1024, 1, 1 << 21)
