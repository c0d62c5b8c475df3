"""Differentiation of the data-consistency loss (the libtorch operator in
csrc/torch_ops.cpp) and a differentiable wave-CAIPI trajectory.

    ops = load_ops()
    k = wave_trajectory_torch(w, theta, lines)          # theta: float64 [6]
    loss = dc_loss(reco, x, k, y)                       # float64 scalar
    loss.backward()                                     # -> x.grad, theta.grad

dc_loss is a torch::autograd::Function over cgs_loss_grad_d: the FP32
gridding/FFT path of the library computes L = 1/2 sum D |E S x - y|^2,
dL/dx and dL/dk on the GPU; the wave trajectory's dependence on its six
parameters is plain PyTorch, so autograd chains dL/dk into dL/dtheta.

cg_unrolled runs the batched CG-SENSE solve (Reco.cpp:175-321) as PyTorch
operations over two libtorch operators, apply_a (E^H D E) and rhs
(E^H D y), whose backward passes give the trajectory vector-Jacobian
products; every iteration is checkpointed (recomputed in the backward
pass), so memory holds four vectors per iteration instead of its
intermediates.  CG scalars are FP64, vectors complex64.
"""
from __future__ import annotations

import importlib
import math
import os

import numpy as np
import torch

# the package's build() function shadows its build module as an attribute
_build = importlib.import_module(__package__ + ".build")

_LOADED = False


def load_ops():
    """Loads libcgsense_torch.so (torch.ops.cgsense); fails loudly when the
    library has not been built."""
    global _LOADED
    if not _LOADED:
        if not os.path.exists(_build.TORCH_LIB):
            raise RuntimeError("libcgsense_torch.so is missing: run 4d_lung_gb300.build.build()")
        torch.ops.load_library(_build.TORCH_LIB)
        _LOADED = True
    return torch.ops.cgsense


def dc_loss(reco, x, k, y, bin=0):
    """L = 1/2 sum_c sum_i D_i |(E_c S_c x)_i - y_ci|^2 of one bin of `reco`
    (coil maps, density weights and bins already set).  x: complex64 image,
    k: float64 [ns][3] (all samples of the context), y: complex64 [n_ch][ns]."""
    load_ops()
    return torch.ops.cgsense.dc_loss(reco.handle, int(bin), x, k, y)


def apply_a(reco, p, k, bin0=0):
    """q = A(k) p for bins [bin0, bin0 + len(p)): p complex64 [nb][voxels]."""
    load_ops()
    return torch.ops.cgsense.apply_a(reco.handle, int(bin0), int(p.shape[0]), p, k)


def rhs(reco, y, k, bin0=0, nb=None):
    """b = E^H D y of bins [bin0, bin0 + nb): complex64 [nb][voxels]."""
    load_ops()
    nb = reco.num_bins() - bin0 if nb is None else nb
    return torch.ops.cgsense.rhs(reco.handle, int(bin0), int(nb), y, k, int(reco.ni))


def _dot(a, b):
    """Per-bin sum of conj(a) b in FP64 (complex128 [nb])."""
    return torch.sum(a.conj().to(torch.complex128) * b.to(torch.complex128), dim=-1)


def cg_unrolled(reco, k, y, iters, checkpoint=True):
    """x after `iters` CG-SENSE iterations of every bin (complex64
    [nbins][voxels]), differentiable in k.  The reference's loop with complex
    alpha = rr / <p, q> and beta = rr_new / rr (Reco.cpp:232-309); no early
    stop (the iteration count is fixed for differentiation)."""
    from torch.utils.checkpoint import checkpoint as ckpt
    b = rhs(reco, y, k)
    x = torch.zeros_like(b)
    r = b
    p = b
    rr = _dot(r, r).real

    def step(x, r, p, rr, k):
        q = apply_a(reco, p.contiguous(), k)
        alpha = (rr / _dot(p, q)).to(torch.complex64)[:, None]
        x = x + alpha * p
        r = r - alpha * q
        rr_new = _dot(r, r).real
        beta = (rr_new / rr).to(torch.complex64)[:, None]
        p = r + beta * p
        return x, r, p, rr_new

    for _ in range(iters):
        if checkpoint:
            x, r, p, rr = ckpt(step, x, r, p, rr, k, use_reentrant=False)
        else:
            x, r, p, rr = step(x, r, p, rr, k)
    return x


def wave_trajectory_torch(w, theta, lines=None):
    """The parametric wave-CAIPI trajectory of synth.wave_trajectory in
    PyTorch (float64), differentiable in theta = (amp_y, amp_z, phase_y,
    phase_z, delay_y, delay_z).  Returns k [n_lines * n_read][3] on theta's
    device."""
    from . import synth
    if lines is None:
        lines = synth.readout_lines(w)
    dev = theta.device
    G = [float(g) for g in w.grid]
    sig = [G[a] / w.img[a] for a in range(3)]
    n = w.n_read
    t = torch.arange(n, dtype=torch.float64, device=dev) / n
    ux = G[0] / 2 + (torch.arange(n, dtype=torch.float64, device=dev) - n / 2) * sig[0] * w.img[0] / n
    om = 2 * math.pi * w.wave_cycles
    wy = theta[0] * torch.sin(om * (t - theta[4]) + theta[2])
    wz = theta[1] * torch.cos(om * (t - theta[5]) + theta[3])
    ln = torch.as_tensor(np.asarray(lines), dtype=torch.float64, device=dev)
    uy = G[1] / 2 + (ln[:, 0:1] - w.img[1] / 2) * sig[1] + wy[None, :]
    uz = G[2] / 2 + (ln[:, 1:2] - w.img[2] / 2) * sig[2] + wz[None, :]
    kx = (ux / (G[0] - 1))[None, :].expand(ln.shape[0], n)
    return torch.stack([kx, uy / (G[1] - 1), uz / (G[2] - 1)], dim=-1).reshape(-1, 3)
