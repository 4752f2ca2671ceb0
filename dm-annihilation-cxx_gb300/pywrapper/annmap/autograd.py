"""Differentiable sky map: a torch.autograd.Function over the native render
(forward) and the native adjoint kernel (backward).

    maps = annmap.autograd.sky_map(x, y, z, m, rho, h, opos, nside=512,
                                   cpos=(0, 0, 0), align=(0, 0, 1),
                                   unit_factor=uf, hires_threshold=thr)
    loss = ((maps - target) ** 2 / (target + eps)).sum()
    loss.backward()      # x.grad ... h.grad and opos.grad are filled

The forward renders the FP64 map of the plain form (or, with
``precision=COMP_F32``, the compensated form, which agrees with it to about
1e-7 per pixel); the backward is the adjoint of the map with every
particle's disc pixel set held fixed, recomputing the kernel weights in the
same precision form (FP64, or FP32 weights with compensated sums).
The observer enters through the rotation set-up of the reference
(Parameters::setupRotation, src/parameters.cpp:183-289), differentiated with
respect to the observer position.  Inputs are CUDA tensors (float32
particles, float64 observer position); there is no CPU path.
"""
from __future__ import annotations

import numpy as np
import torch

from ._lib import FLUX_LAWS, PLAIN_F64
from .mapgen import Renderer

_RENDERERS: dict = {}


def _renderer(device: int) -> Renderer:
    r = _RENDERERS.get(device)
    if r is None:
        r = _RENDERERS[device] = Renderer(device)
    return r


class SkyMap(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, z, m, rho, h, opos, nside, cpos, align, unit_factor, hires_threshold,
                precision, flux_model, law_args):
        if not x.is_cuda:
            raise ValueError("sky_map needs CUDA tensors")
        dev = x.device.index if x.device.index is not None else torch.cuda.current_device()
        r = _renderer(dev)
        op = [float(v) for v in opos.detach().to("cpu", torch.float64)]
        sigmav, vel, halos = law_args
        _configure(r, op, cpos, align, unit_factor, hires_threshold, flux_model, vel, halos)
        out = torch.empty(12 * nside * nside, dtype=torch.float64, device=x.device)
        r.render(_parts(x, y, z, m, rho, h, sigmav), nside, precision, out=out)
        ctx.save_for_backward(x, y, z, m, rho, h)
        ctx.cfg = (dev, op, tuple(cpos), tuple(align), float(unit_factor), float(hires_threshold),
                   int(nside), int(precision), int(flux_model), law_args)
        return out

    @staticmethod
    def backward(ctx, grad_map):
        x, y, z, m, rho, h = ctx.saved_tensors
        dev, op, cpos, align, uf, thr, nside, precision, law, law_args = ctx.cfg
        r = _renderer(dev)
        sigmav, vel, halos = law_args
        _configure(r, op, cpos, align, uf, thr, law, vel, halos)
        g, gopos = r.adjoint(_parts(x, y, z, m, rho, h, sigmav), nside,
                             grad_map.detach().to(torch.float64).contiguous(), precision=precision)
        grads = [g[k].to(t.dtype) if t.requires_grad else None
                 for k, t in enumerate((x, y, z, m, rho, h))]
        gop = torch.as_tensor(np.asarray(gopos), dtype=torch.float64) if ctx.needs_input_grad[6] else None
        return (*grads, gop, None, None, None, None, None, None, None, None)


def _configure(r, op, cpos, align, unit_factor, hires_threshold, flux_model, vel, halos):
    r.set_observer(op, cpos, align)
    r.set_units(unit_factor, hires_threshold, flux_model)
    r.set_flux_params(vel, cpos)
    if halos is not None:
        r.set_halo_cores(*halos)


def _parts(x, y, z, m, rho, h, sigmav):
    parts = {"x": x.detach(), "y": y.detach(), "z": z.detach(), "m": m.detach(),
             "rho": rho.detach(), "h": h.detach()}
    if sigmav is not None:
        parts["sigmav"] = sigmav.detach()
    return parts


def sky_map(x, y, z, m, rho, h, opos, *, nside: int, cpos=(0.0, 0.0, 0.0), align=(0.0, 0.0, 1.0),
            unit_factor: float = 1.0, hires_threshold: float = float("inf"),
            precision: int = PLAIN_F64, flux_model=0, sigmav=None, velocity_to_cgs: float = 0.0,
            halo_cores=None):
    """The map (12 nside^2 float64, flux per steradian) as a differentiable
    function of the particle arrays and the observer position ``opos``
    (a length-3 float64 CPU tensor; its gradient is returned on the CPU).
    ``flux_model``: any flux law (number or name, e.g. "decay"; unit_factor
    is the law's own).  The somv, somv2 and pwave laws read ``sigmav`` (a
    CUDA float32 tensor, not differentiated) in code units times
    ``velocity_to_cgs``; the adiabatic law's halo centre is ``cpos``; the
    ann_core_nosom law reads ``halo_cores`` = (x, y, z, radius) arrays of
    its halo table (a particle's membership in a core is held fixed)."""
    if not torch.is_tensor(opos):
        opos = torch.as_tensor(opos, dtype=torch.float64)
    if isinstance(flux_model, str):
        flux_model = FLUX_LAWS[flux_model]
    law_args = (sigmav, float(velocity_to_cgs),
                None if halo_cores is None else tuple(np.asarray(a, dtype=np.float32) for a in halo_cores))
    return SkyMap.apply(x, y, z, m, rho, h, opos, int(nside), tuple(float(v) for v in cpos),
                        tuple(float(v) for v in align), unit_factor, hires_threshold, precision,
                        int(flux_model), law_args)
