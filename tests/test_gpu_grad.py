"""Differentiation on the GPU: the data-consistency loss
L = 1/2 sum_c sum_i D_i |(E_c S_c x)_i - y_ci|^2 and its gradients with
respect to the image and the sample coordinates (cgs_loss_grad_d, FP32
gridding and FFT), the FP64 reference (cgs_loss_grad_fp64_d), the libtorch
autograd operator, and the wave-trajectory parameters.

Tolerances:
  * FP32 path against the FP64 oracle: loss 1e-4, dL/dx 2e-4, dL/dk 1e-3
    (relative L2 over all samples).  The FP32 path keeps the reference's
    float distance arithmetic (float index times float dk, Reco.cpp:763-771),
    which moves a sample by up to ~6e-8 in k units (3e-6 cells on a 48-point
    axis) against the oracle's double distances: E x differs by ~1e-5;
  * FP64 GPU path against the FP64 oracle: 1e-6 (its coil maps and
    deapodisation factors are float, as in the reference);
  * dL/dtheta against central finite differences of the FP64 loss (step
    1e-3 in the parameters' natural units: cells, radians, wave periods):
    1e-3.
The tests use the reference's KB kernel (w = 4.25, b = 14.9086).  A KB kernel
jumps by I0(0)/I0(b) of its peak at the edge of its support (1e-3 for the
Beatty shape of w = 4, 3e-6 for the reference's), and with w = 4 the edge
falls exactly on the half-cell lattice of the readout samples: whether such a
tap is in the set then depends on the rounding of the distance, and finite
differences see the jumps of the samples whose tap set changes within the step.
"""
import importlib

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def wave_case(cgs, synth, oracle_mod, img, grid, nch, lines_every=1, seed=2):
    import torch
    w = synth.scaled(synth.WORKLOADS["cfg4"], img, grid, n_ch=nch, n_bins=1)
    lines = synth.readout_lines(w)[::lines_every]
    nom = synth.WaveParams(w.wave_cells, w.wave_cells)
    # the reference's own kernel (Reco.cpp:378-379): support +-2.125 cells,
    # off the half-cell lattice of the readout samples, and an edge jump of
    # I0(0)/I0(14.9) = 3e-6 of the peak
    kb_w, kb_b = 4.25, 14.9086
    r = cgs.Reco(img, grid, nch, kb_w=kb_w, kb_b=kb_b)
    k_true = synth.wave_trajectory(w, nom, lines=lines)
    r.set_trajectory(k_true)
    smaps = synth.coil_maps(img, nch)
    r.set_smaps(smaps)
    x = synth.phantom(img)
    dev = torch.device("cuda")
    y = torch.zeros((nch, k_true.shape[0]), dtype=torch.complex64, device=dev)
    r.nufft_fwd_tensor(torch.from_numpy(smaps * x[None]).to(dev).contiguous(), y)
    torch.cuda.synchronize()
    rms = float(torch.sqrt(torch.mean(torch.abs(y) ** 2)))
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    y += torch.complex(torch.randn(y.shape, generator=g, device=dev),
                       torch.randn(y.shape, generator=g, device=dev)) * (rms / 30 / np.sqrt(2))
    p = oracle_mod.make_params(img, grid, nch, kb_w=kb_w, kb_b=kb_b)
    return w, lines, r, smaps, x, y, p, kb_w, kb_b


def test_loss_grad_matches_oracle(gpu_lib, cgs, synth, oracle_mod, o64):
    import torch
    img, grid, nch = (24, 24, 16), (48, 48, 32), 3
    w, lines, r, smaps, x, y, p, _, _ = wave_case(cgs, synth, oracle_mod, img, grid, nch)
    th = synth.perturbed_wave(w)
    k = synth.wave_trajectory(w, th, lines=lines)
    r.set_trajectory(k)
    dcf = np.random.default_rng(4).uniform(0.5, 1.5, k.shape[0]).astype(np.float32)
    r.set_dcf(dcf)
    dev = torch.device("cuda")
    # a residual of the size of the data: with the measured samples of the
    # true trajectory the residual is small and the relative error of L and
    # of its gradients grows like |y| / |r| (FP32 rounding of E x)
    rng = np.random.default_rng(6)
    rms = float(torch.sqrt(torch.mean(torch.abs(y) ** 2)))
    y = torch.from_numpy(((rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)) * rms)
                         .astype(np.complex64)).to(dev)
    xt = torch.from_numpy(x).to(dev)
    gx = torch.zeros_like(xt)
    gk = torch.zeros((k.shape[0], 3), dtype=torch.float32, device=dev)
    L = r.loss_grad_tensor(xt, y, gx, gk)
    yh = y.cpu().numpy()
    Lo, gxo, gko = o64.loss_grad(p, k, o64.kernel_ft(p), smaps, dcf, x, yh)
    errs = (abs(L - Lo) / Lo, rel_l2(gx.cpu().numpy(), gxo), rel_l2(gk.cpu().numpy(), gko))
    print("FP32 vs FP64 oracle: loss %.3g  dL/dx %.3g  dL/dk %.3g" % errs)
    assert errs[0] < 1e-4 and errs[1] < 2e-4 and errs[2] < 1e-3, errs
    # the FP64 GPU reference
    x64 = xt.to(torch.complex128)
    gx64 = torch.zeros_like(x64)
    gk64 = torch.zeros((k.shape[0], 3), dtype=torch.float64, device=dev)
    L64 = r.loss_grad_fp64_tensor(x64, y, gx64, gk64)
    errs = (abs(L64 - Lo) / Lo, rel_l2(gx64.cpu().numpy(), gxo), rel_l2(gk64.cpu().numpy(), gko))
    print("FP64 GPU vs FP64 oracle: loss %.3g  dL/dx %.3g  dL/dk %.3g" % errs)
    assert max(errs) < 1e-6, errs
    # the loss alone (no gradient buffers) is the same number
    assert r.loss_grad_tensor(xt, y) == L


def test_autograd_operator(gpu_lib, cgs, synth, oracle_mod, o64):
    """torch.ops.cgsense.dc_loss: x.grad and k.grad equal the C-ABI
    gradients; x.grad follows PyTorch's convention for a real loss of a
    complex input (dL/dRe + i dL/dIm), checked against the oracle."""
    import torch
    ag = importlib.import_module("4d_lung_gb300.autograd")
    img, grid, nch = (24, 24, 16), (48, 48, 32), 3
    w, lines, r, smaps, x, y, p, _, _ = wave_case(cgs, synth, oracle_mod, img, grid, nch)
    th = synth.perturbed_wave(w)
    dev = torch.device("cuda")
    v = torch.tensor([th.amp_y, th.amp_z, th.phase_y, th.phase_z, th.delay_y, th.delay_z], dtype=torch.float64,
                     device=dev, requires_grad=True)
    xt = torch.from_numpy(x).to(dev).requires_grad_(True)
    k = ag.wave_trajectory_torch(w, v, lines)
    k.retain_grad()
    loss = ag.dc_loss(r, xt, k, y)
    loss.backward()
    kn = k.detach().cpu().numpy()
    Lo, gxo, gko = o64.loss_grad(p, kn, o64.kernel_ft(p), smaps, None, x, y.cpu().numpy())
    errs = (abs(loss.item() - Lo) / Lo, rel_l2(xt.grad.cpu().numpy(), gxo), rel_l2(k.grad.cpu().numpy(), gko))
    print("autograd vs FP64 oracle: loss %.3g  x.grad %.3g  k.grad %.3g" % errs)
    assert errs[0] < 1e-4 and errs[1] < 2e-4 and errs[2] < 1e-3, errs
    J = synth.wave_jacobian(w, th, lines=lines)
    g_theta = np.einsum("ia,iam->m", gko, J)
    assert np.allclose(v.grad.cpu().numpy(), g_theta, rtol=1e-3, atol=1e-3 * np.abs(g_theta).max())


def test_theta_gradient_vs_finite_differences(gpu_lib, cgs, synth, oracle_mod):
    """cfg4 differentiation form: 128x128x96 image, 12 coils, one bin of
    1.57 M wave-CAIPI samples, wave parameters perturbed by up to 5 %.
    dL/dtheta from the FP32 autograd operator and from the FP64 reference
    gradient against central finite differences of the FP64 loss."""
    import torch
    ag = importlib.import_module("4d_lung_gb300.autograd")
    w0 = synth.WORKLOADS["cfg4"]
    w, lines, r, smaps, x, y, p, _, _ = wave_case(cgs, synth, oracle_mod, w0.img, w0.grid, w0.n_ch)
    th = synth.perturbed_wave(w)
    dev = torch.device("cuda")
    v0 = np.array([th.amp_y, th.amp_z, th.phase_y, th.phase_z, th.delay_y, th.delay_z])
    xt = torch.from_numpy(x).to(dev)
    x64 = xt.to(torch.complex128)

    def loss64(vec, grad=False):
        k = ag.wave_trajectory_torch(w, torch.tensor(vec, dtype=torch.float64, device=dev), lines).contiguous()
        r.update_trajectory_tensor(k)
        gk = torch.zeros((k.shape[0], 3), dtype=torch.float64, device=dev) if grad else None
        return r.loss_grad_fp64_tensor(x64, y, None, gk), gk

    L0, gk64 = loss64(v0, grad=True)
    J = synth.wave_jacobian(w, th, lines=lines)
    g64 = np.einsum("ia,iam->m", gk64.cpu().numpy(), J)
    v = torch.tensor(v0, dtype=torch.float64, device=dev, requires_grad=True)
    loss = ag.dc_loss(r, xt, ag.wave_trajectory_torch(w, v, lines).contiguous(), y)
    loss.backward()
    g32 = v.grad.cpu().numpy()
    sc = synth.wave_param_scale(w)
    fd = np.zeros(6)
    for m in range(6):
        h = 1e-3 * sc[m]
        vp, vm = v0.copy(), v0.copy()
        vp[m] += h
        vm[m] -= h
        fd[m] = (loss64(vp)[0] - loss64(vm)[0]) / (2 * h)
    # compare in natural units (scale-free per parameter)
    err64 = np.abs(g64 - fd) / np.abs(fd)
    err32 = np.abs(g32 - g64) / np.abs(g64)
    print("dL/dtheta FP64", g64, "FD", fd, "FP32", g32, "err64", err64, "err32", err32)
    assert np.all(err64 < 1e-3), err64
    assert np.all(err32 < 1e-3), err32


def test_self_calibration_reduces_error(gpu_lib, cgs, synth, oracle_mod):
    """Trajectory self-calibration: Adam on the six wave parameters (in
    natural units) from a 5 % perturbation, image known: the loss and the
    trajectory error (RMS distance to the true coordinates, in cells) fall.
    Phase and delay of one axis enter only as phase - 2 pi cycles delay, so
    the parameters themselves are not all identifiable; the trajectory is."""
    import torch
    ag = importlib.import_module("4d_lung_gb300.autograd")
    img, grid, nch = (48, 48, 32), (96, 96, 64), 4
    w, lines, r, smaps, x, y, p, _, _ = wave_case(cgs, synth, oracle_mod, img, grid, nch)
    dev = torch.device("cuda")
    sc = torch.tensor(synth.wave_param_scale(w), dtype=torch.float64, device=dev)
    th = synth.perturbed_wave(w)
    v_true = torch.tensor([w.wave_cells, w.wave_cells, 0, 0, 0, 0], dtype=torch.float64, device=dev)
    u = (torch.tensor([th.amp_y, th.amp_z, th.phase_y, th.phase_z, th.delay_y, th.delay_z], dtype=torch.float64,
                      device=dev) / sc).requires_grad_(True)
    G = torch.tensor(w.grid, dtype=torch.float64, device=dev) - 1
    k_true = ag.wave_trajectory_torch(w, v_true, lines)

    def traj_err(uu):
        k = ag.wave_trajectory_torch(w, uu * sc, lines)
        return float(torch.sqrt(torch.mean(torch.sum(((k - k_true) * G) ** 2, dim=1))))

    xt = torch.from_numpy(x).to(dev)
    opt = torch.optim.Adam([u], lr=0.02)
    losses = []
    err0 = traj_err(u.detach())
    for _ in range(30):
        opt.zero_grad()
        loss = ag.dc_loss(r, xt, ag.wave_trajectory_torch(w, u * sc, lines).contiguous(), y)
        loss.backward()
        opt.step()
        losses.append(loss.item())
    err1 = traj_err(u.detach())
    assert losses[-1] < 0.5 * losses[0], losses
    assert err1 < 0.3 * err0, (err0, err1)


def test_unrolled_cg_gradient_vs_fp64_differences(gpu_lib, cgs, synth, oracle_mod):
    """Backpropagation through the unrolled, checkpointed CG (two bins, four
    iterations, FP32 operator, FP64 CG scalars): the forward pass equals the
    library's graph-captured batched solve, and dL/dtheta of
    L = 1/2 sum_b |x_b(theta) - x_true|^2 agrees with central differences
    of the same loss from the full-FP64 GPU solve (step 1e-3 in natural
    units) to 1e-2 (FP32 vectors through four CG iterations)."""
    import torch
    ag = importlib.import_module("4d_lung_gb300.autograd")
    img, grid, nch = (24, 24, 16), (48, 48, 32), 3
    w, lines, r, smaps, x, y, p, _, _ = wave_case(cgs, synth, oracle_mod, img, grid, nch)
    n_read = w.n_read
    half = len(lines) // 2
    r.set_bins(synth.bin_samples([np.arange(0, half), np.arange(half, len(lines))], n_read))
    dev = torch.device("cuda")
    iters = 4
    th = synth.perturbed_wave(w)
    v0 = np.array([th.amp_y, th.amp_z, th.phase_y, th.phase_z, th.delay_y, th.delay_z])
    xt = torch.from_numpy(x).to(dev).reshape(1, -1)
    # forward: the unrolled loop equals the graph-captured batched solve
    k0 = ag.wave_trajectory_torch(w, torch.tensor(v0, dtype=torch.float64, device=dev), lines).contiguous()
    x_unr = ag.cg_unrolled(r, k0, y, iters, checkpoint=False).detach()
    xb = torch.zeros((2,) + img, dtype=torch.complex64, device=dev)
    r.cg_sense_batched_tensor(y, xb, 0.0, iters)
    torch.cuda.synchronize()
    assert rel_l2(x_unr.cpu().numpy(), xb.reshape(2, -1).cpu().numpy()) < 1e-4
    # gradient through the checkpointed loop
    v = torch.tensor(v0, dtype=torch.float64, device=dev, requires_grad=True)
    k = ag.wave_trajectory_torch(w, v, lines).contiguous()
    xk = ag.cg_unrolled(r, k, y, iters, checkpoint=True)
    loss = 0.5 * torch.sum(torch.abs(xk.to(torch.complex128) - xt.to(torch.complex128)) ** 2)
    loss.backward()
    g = v.grad.cpu().numpy()

    def loss64(vec):
        kk = ag.wave_trajectory_torch(w, torch.tensor(vec, dtype=torch.float64, device=dev), lines).contiguous()
        r.update_trajectory_tensor(kk)
        x64 = torch.zeros((2,) + img, dtype=torch.complex128, device=dev)
        r.cg_sense_fp64_tensor(y, x64, 0.0, iters)
        torch.cuda.synchronize()
        return 0.5 * float(torch.sum(torch.abs(x64.reshape(2, -1) - xt.to(torch.complex128)) ** 2))

    sc = synth.wave_param_scale(w)
    fd = np.zeros(6)
    for m in range(6):
        h = 1e-3 * sc[m]
        vp, vm = v0.copy(), v0.copy()
        vp[m] += h
        vm[m] -= h
        fd[m] = (loss64(vp) - loss64(vm)) / (2 * h)
    err = np.abs(g - fd) / np.abs(fd)
    print("unrolled CG dL/dtheta", g, "FD (FP64 solve)", fd, "rel err", err)
    assert np.all(err < 1e-2), err
