"""Differentiable transport through per-voxel media.

``transport(mua, mus, g, engine, first, n)`` runs photons [first, first+n)
and returns, per launched photon,

* ``rd_r``: the weight detected at the detection plane binned by the distance
  from the z axis (``engine.set_radial_tally`` bins plus one overflow bin);
* ``absorbed``: the weight deposited in each voxel (NMC_TALLY_F3D, shaped
  like ``mua``); ``fluence(absorbed, mua, dV)`` turns it into fluence;

as torch tensors whose gradients with respect to the per-voxel absorption
``mua``, scattering ``mus`` and anisotropy ``g`` are the perturbation Monte
Carlo adjoint of the same photons (``nmc_adjoint_forward`` /
``nmc_adjoint_backward_ex`` in include/nmc_abi.h):

* d/dmua: pathwise, the weight carries exp(-sum mua * path);
* d/dmus, d/dg: likelihood ratio of the sampled scattering points and angles.

The reference has no gradient path (it tallies forward only, kernels.metal
:321-754); this is the inverse-problem entry point built on the same
transport.  Tensors may live on any device: properties go to the engine as
host arrays (the engine keeps its own device copy), results come back on the
device and dtype of ``mua``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import abi
from .engine import Engine


class _Transport(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mua, mus, g, engine: Engine, first: int, n: int, event_capacity: int | None,
                deposit_capacity: int):
        ctx.engine, ctx.first, ctx.n, ctx.cap, ctx.dcap = engine, int(first), int(n), event_capacity, deposit_capacity
        ctx.shape = tuple(mua.shape)
        ctx.save_for_backward(mua, mus, g)
        _forward(engine, mua, mus, g, first, n, event_capacity, deposit_capacity)
        ctx.token = engine._adj_token
        rd = engine.tally(abi.TALLY_RD_R) / float(n)
        ab = engine.tally(abi.TALLY_F3D) / float(n)
        kw = dict(dtype=mua.dtype, device=mua.device)
        return torch.as_tensor(rd, **kw), torch.as_tensor(ab.reshape(ctx.shape), **kw)

    @staticmethod
    def backward(ctx, grad_rd, grad_ab):
        e: Engine = ctx.engine
        if getattr(e, "_adj_token", None) != ctx.token:
            # the handle ran another forward since: record this one again
            # (same photon streams, so the same events)
            mua, mus, g = ctx.saved_tensors
            _forward(e, mua, mus, g, ctx.first, ctx.n, ctx.cap, ctx.dcap)
            ctx.token = e._adj_token

        def host(t):
            if t is None:
                return None
            a = t.detach().to("cpu", torch.float64).numpy().ravel() / float(ctx.n)
            return a.astype(np.float32) if np.any(a) else None

        G, GF = host(grad_rd), host(grad_ab)
        mua = ctx.saved_tensors[0]
        need = ctx.needs_input_grad
        if G is None and GF is None:
            z = torch.zeros_like(mua)
            return (z if need[0] else None, z if need[1] else None, z if need[2] else None,
                    None, None, None, None, None)
        ga, gs, gg = e.adjoint_backward(G, GF)

        def out(a, want):
            if not want:
                return None
            return torch.as_tensor(a.reshape(ctx.shape), dtype=mua.dtype, device=mua.device)

        return out(ga, need[0]), out(gs, need[1]), out(gg, need[2]), None, None, None, None, None


def _forward(e: Engine, mua, mus, g, first, n, cap, dcap):
    def host(t):
        return t.detach().to("cpu", torch.float32).contiguous().numpy().ravel()

    e.set_voxel_props(host(mua), host(mus), host(g))
    e.reset()
    e.adjoint_forward(first, n, cap, dcap)
    e._adj_token = getattr(e, "_adj_token", 0) + 1


def transport(mua: torch.Tensor, mus: torch.Tensor, g: torch.Tensor, engine: Engine, first: int = 0,
              n: int = 1_000_000, event_capacity: int | None = None, deposit_capacity: int | None = None):
    """(rd_r, absorbed) per launched photon for photons [first, first + n)
    through per-voxel media (arrays of Nz x Nx x Ny or flat, engine voxel
    order), differentiable in mua, mus and g.  `engine` is an NMC_SIM_MCXYZ
    Engine after prepare_data and set_radial_tally; its other tallies hold
    this forward's photons afterwards.  deposit_capacity (records of 8
    bytes; default 600 per photon) sizes the forward's deposit list, which
    spares a backward through `absorbed` its score replay; 0 keeps none."""
    if engine.sim_type != abi.SIM_MCXYZ:
        raise ValueError("transport needs an NMC_SIM_MCXYZ engine")
    dcap = 600 * int(n) if deposit_capacity is None else int(deposit_capacity)
    return _Transport.apply(mua, mus, g, engine, first, n, event_capacity, dcap)


def radial_reflectance(mua, mus, g, engine: Engine, first: int = 0, n: int = 1_000_000,
                       event_capacity: int | None = None) -> torch.Tensor:
    """Rd(r) per launched photon (bins + 1 values, last = overflow); no
    deposit list is kept (only detections score)."""
    return transport(mua, mus, g, engine, first, n, event_capacity, deposit_capacity=0)[0]


def fluence(absorbed: torch.Tensor, mua: torch.Tensor, voxel_volume: float) -> torch.Tensor:
    """Fluence per launched photon (1/cm^2) from the absorbed weight per
    voxel: absorbed / (mua * voxel volume), the normalisation the reference
    applies to F3D before writing _F.bin (main.m:271-281).  Voxels with
    mua = 0 give 0."""
    return torch.where(mua > 0, absorbed / (mua.clamp_min(1e-30) * voxel_volume), torch.zeros_like(absorbed))
