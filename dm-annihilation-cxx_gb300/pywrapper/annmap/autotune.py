"""Autotuner of the footprint-class work queue and the block kernel's shape.

The disc particles of a map are binned by estimated footprint (pixels of
the disc): discs up to ``warp_max_pixels`` are rendered one warp per
particle, larger ones one thread block per particle, with the block kernel
in one of three shapes (``block_threads`` 128 / 256 / 512 at the same 2048
resident threads per SM).  The best bin edge and shape depend on Nside and
on the particles' smoothing lengths, so they are measured: each candidate
renders a sample of the particles (a prefix of a shuffled set is an i.i.d.
sample) and the one with the least device time wins.  The winner becomes
the renderer's per-Nside tuning entry (dmann_set_tuning_nside), so later
renders -- including every observer of a batch with that Nside -- use it.

A prefix sample has the per-particle disc statistics of the whole set but
not its density: with fewer particles per sky region, fewer concurrently
rendered discs overlap, fewer reductions to one pixel queue up in L2, and a
shape that wins on the sample can lose on the whole set (16M particles at
Nside 2048: 256-thread blocks win on a 2M prefix, 128-thread blocks on the
whole set).  Tune with ``sample`` equal to the particle count when the
render is long enough to repay one trial render per candidate.
Results are cached in a JSON file keyed by device, Nside, precision form
and the sample size's power of two; ``ANNMAP_TUNING_CACHE`` names the file
(default ``~/.cache/annmap/tuning.json``), ``cache=False`` disables it.
"""
from __future__ import annotations

import json
import math
import os
import time

from ._lib import COMP_F32

SPACE = {"block_threads": (128, 256, 512), "warp_max_pixels": (256, 1024, 4096)}


def cache_path() -> str:
    return os.environ.get("ANNMAP_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "annmap", "tuning.json"))


def _device_name(renderer) -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(renderer.device)
    except Exception:
        pass
    return f"cuda:{renderer.device}"


def tuning_key(device_name: str, nside: int, precision: int, n: int) -> str:
    return f"{device_name}|nside={int(nside)}|precision={int(precision)}|n=2^{max(0, round(math.log2(max(n, 1))))}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _slice(parts: dict, k: int) -> dict:
    return {f: v[:k] for f, v in parts.items()}


def tune(renderer, parts: dict, nside: int, precision: int = COMP_F32, *, sample: int = 1 << 21,
         space: dict | None = None, reps: int = 2, cache=True, out=None) -> dict:
    """Measures every candidate of ``space`` (default ``SPACE``) on the first
    ``sample`` particles, applies the fastest as the renderer's tuning for
    ``nside`` and returns {"key", "best", "trials", "seconds", "cached"}.
    ``out`` is an optional output map of 12 nside^2 doubles; with CUDA
    tensor particles and no (or a wrongly sized) ``out`` a device map is
    made, so the maps stay on the device while tuning."""
    t0 = time.perf_counter()
    space = dict(space or SPACE)
    n = len(next(iter(parts.values())))
    k = min(n, int(sample))
    key = tuning_key(_device_name(renderer), nside, precision, k)
    path = cache_path() if cache is True else (cache or None)
    table = _load(path) if path else {}
    if key in table:
        best = table[key]["best"]
        renderer.set_tuning(nside=nside, **best)
        return {"key": key, "best": best, "trials": table[key].get("trials", []),
                "seconds": time.perf_counter() - t0, "cached": True}
    sub = _slice(parts, k)
    npix = 12 * int(nside) * int(nside)
    if out is None or len(out) != npix:
        out = None
        first = next(iter(sub.values()))
        if type(first).__module__.startswith("torch") and first.is_cuda:
            import torch
            out = torch.empty(npix, dtype=torch.float64, device=first.device)
    names = list(space)
    combos = [{}]
    for nm in names:
        combos = [dict(c, **{nm: v}) for c in combos for v in space[nm]]
    trials = []
    for c in combos:
        renderer.set_tuning(nside=nside, **c)
        times = []
        for _ in range(max(1, reps)):
            renderer.render(sub, nside, precision, out=out)
            times.append(float(renderer.stats()["kernel_ms"]))
        trials.append({"tuning": c, "ms": min(times)})
    best = min(trials, key=lambda t: t["ms"])["tuning"]
    renderer.set_tuning(nside=nside, **best)
    if path:
        table[key] = {"best": best, "trials": trials}
        _store(path, table)
    return {"key": key, "best": best, "trials": trials, "seconds": time.perf_counter() - t0,
            "cached": False}


def tune_nsides(renderer, parts: dict, nsides, precision: int = COMP_F32, **kw) -> dict:
    """tune() for every distinct Nside of a batch; returns {nside: result}."""
    return {int(ns): tune(renderer, parts, int(ns), precision, **kw) for ns in sorted(set(nsides))}
