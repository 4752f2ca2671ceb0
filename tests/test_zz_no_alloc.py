"""dmann_render_noalloc: rendering with no device allocation at all.

Some callers cannot call cudaMalloc: a plug-in running inside a host program
whose own allocator has already reserved the GPU's memory, or a tight loop that
cannot afford cudaMalloc's implicit synchronisation.  For them the library
offers one entry point that works entirely in a fixed scratch array compiled
into it.  These tests call it through the C ABI on device buffers and check its
map against the ordinary compensated render (dmann_render through a context),
on two calls in a row.  The two are independent renders, so they differ by the
compensated form's run-to-run spread: the order in which warps claim rings
can move a particle's normalisation by ~1e-13 relative, which can flip the
one FP32 rounding of a deposit near a rounding boundary (at most 2^-24 of
that deposit), and the FP64 reductions add in a different order.  RTOL is the
bound the other run-to-run comparisons of the compensated form use.

This file is named to be collected last, so a run that stops at the first
failure has run everything else first; it also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

import annmap
from annmap import _lib, synth

pytestmark = pytest.mark.gpu

RTOL = 1e-7   # the compensated form's documented run-to-run bound per pixel


def _noalloc(L, parts, n, nside, par, out, accumulate=0, stream=None):
    d9 = (C.c_double * 9)(*[v for row in par.rotmatrix for v in row])
    d3 = (C.c_double * 3)(*par.params.opos)
    p = [C.c_void_p(parts[k].data_ptr()) for k in ("x", "y", "z", "m", "rho", "h")]
    return L.dmann_render_noalloc(*p, n, nside, d9, d3, par.unit_factor, par.hires_threshold,
                                  C.c_void_p(out.data_ptr()), accumulate,
                                  C.c_void_p(stream) if stream else None)


def test_noalloc_matches_render_on_two_calls():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    nside = 128
    stream = torch.cuda.current_stream().cuda_stream
    for call, seed in enumerate((2024, 2025)):
        P = synth.nfw_halo(20000, seed=seed, n_sub=6)
        par = annmap.Parameters.for_synthetic(P, nside)
        dev = {k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}
        with annmap.Renderer(0) as r:
            # the no-alloc entry point deposits in FP64 (the per-disc kernels);
            # so does the context's render below 2^62 estimated deposits
            # (this halo's fat particles would otherwise take the segmented
            # render, whose FP32 deposits differ by their own rounding)
            r.set_tuning(seg_min_deposits_log2=62)
            r.set_params(par)
            ref = r.render(P.as_dict(), nside, annmap.COMP_F32)
        out = torch.full((12 * nside * nside,), 7.0, dtype=torch.float64, device="cuda")
        st = _noalloc(L, dev, len(P), nside, par, out, stream=stream)
        assert st == _lib.OK, st
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got != 0, ref != 0), f"call {call}: pixel sets differ"
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)
        # accumulate into the same map: twice the map
        st = _noalloc(L, dev, len(P), nside, par, out, accumulate=1, stream=stream)
        assert st == _lib.OK
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), 2 * ref, rtol=RTOL, atol=0)


def test_noalloc_rejects_what_it_cannot_hold():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    P = synth.nfw_halo(100, seed=1)
    par = annmap.Parameters.for_synthetic(P, 4096)
    dev = {k: torch.from_numpy(v).cuda() for k, v in P.as_dict().items()}
    # Nside 4096 needs 1.6 GB of accumulation planes: beyond the fixed scratch
    big = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert _noalloc(L, dev, len(P), 4096, par, big) == _lib.ERR_TOO_LARGE
    # host buffers are refused: nothing is staged
    host = {k: torch.from_numpy(v) for k, v in P.as_dict().items()}
    out = torch.zeros(12 * 16 * 16, dtype=torch.float64, device="cuda")
    assert _noalloc(L, host, len(P), 16, par, out) == _lib.ERR_INVALID
