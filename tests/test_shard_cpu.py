"""Sharding arithmetic of annmap.shard on two gloo ranks (CPU): the sum of
the ranks' partial maps equals the single-rank map, for a stand-in render
function that deposits each particle's value into its pixel (the real
kernels are tested for linearity over chunks on the GPU)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from annmap.shard import render_sharded, shard_bounds  # noqa: E402


def _stand_in_render(parts, nside):
    npix = 12 * nside * nside
    pix = (np.abs(parts["x"] * 1000.0 + parts["y"] * 37.0).astype(np.int64)) % npix
    m = np.zeros(npix)
    np.add.at(m, pix, parts["m"].astype(np.float64) * parts["rho"].astype(np.float64))
    return torch.from_numpy(m)


def _parts(n=10001):
    rng = np.random.default_rng(9)
    return {k: rng.uniform(0.5, 2.0, n).astype(np.float32) for k in ("x", "y", "z", "m", "rho", "h")}


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = render_sharded(_stand_in_render, _parts(), 16)
    np.save(os.path.join(out, f"r{rank}.npy"), m.numpy())
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_bounds_cover_every_particle():
    for n in (0, 1, 7, 10001):
        for w in (1, 2, 3, 8):
            b = [shard_bounds(n, r, w) for r in range(w)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] for i in range(w - 1))


def test_two_gloo_ranks_sum_to_the_single_map(tmp_path):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    full = _stand_in_render(_parts(), 16).numpy()
    for r in range(2):
        got = np.load(tmp_path / f"r{r}.npy")
        np.testing.assert_allclose(got, full, rtol=1e-14, atol=0)
