"""Coil maps from low-resolution coil images (cgs_estimate_smaps_d), the
optional on-GPU companion of the root-sum-of-squares pre-step: against the
same algorithm on the FP64 oracle's adjoint NUFFT, and against the known
maps of a synthetic acquisition.

Tolerances: maps vs the FP64 restatement 1e-4 relative L2 over the voxels
clear of the mask threshold (the adjoint NUFFT's FP32 parity is 2e-5); the
estimate against the true maps normalised to unit root-sum-of-squares: per
voxel coherence |sum_c S_est conj(S_true)| >= 0.97 and magnitude error
<= 0.12 inside the object (a Hann window of 12 cells blurs the maps)."""
import importlib

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

IMG, GRID, NCH, RADIUS, EPS = (24, 20, 16), (48, 40, 32), 4, 12.0, 0.05


def lowpass(k, radius):
    d = np.sqrt(sum(((k[:, a] - 0.5) * (GRID[a] - 1)) ** 2 for a in range(3)))
    return np.where(d < radius, np.cos(np.pi * d / (2 * radius)) ** 2, 0.0).astype(np.float32)


@pytest.fixture(scope="module")
def acquisition(synth, oracle_mod, o64):
    w = synth.scaled(synth.WORKLOADS["cfg1"], IMG, GRID, n_ch=NCH, read_os=2)
    k = synth.wave_trajectory(w, synth.WaveParams(2.0, 2.0))
    kb_w = 4.0
    kb_b = float(np.pi * np.sqrt(kb_w ** 2 / 4 * 1.5 ** 2 - 0.8))
    p = oracle_mod.make_params(IMG, GRID, NCH, kb_w=kb_w, kb_b=kb_b)
    taps, kft = o64.taps(p, k), o64.kernel_ft(p)
    S, x = synth.coil_maps(IMG, NCH), synth.phantom(IMG)
    data = o64.nufft_fwd(p, taps, kft, S * x[None]).astype(np.complex64)
    return k, kb_w, kb_b, p, taps, kft, S, x, data


def estimate(cgs, k, kb_w, kb_b, data):
    import torch
    r = cgs.Reco(IMG, GRID, NCH, kb_w=kb_w, kb_b=kb_b)
    r.set_trajectory(k)
    maps = torch.zeros((NCH,) + IMG, dtype=torch.complex64, device="cuda")
    r.estimate_smaps_tensor(torch.from_numpy(data).cuda(), maps, RADIUS, EPS)
    torch.cuda.synchronize()
    return maps.cpu().numpy()


def test_smaps_match_fp64_restatement(gpu_lib, cgs, o64, acquisition):
    k, kb_w, kb_b, p, taps, kft, S, x, data = acquisition
    est = estimate(cgs, k, kb_w, kb_b, data)
    img = o64.nufft_adj(p, taps, kft, data.astype(np.complex128) * lowpass(k, RADIUS)[None])
    rss = np.sqrt((np.abs(img) ** 2).sum(0))
    lim = EPS * rss.max()
    ref = np.where((rss > lim)[None], img / np.where(rss > lim, rss, 1.0)[None], 0.0)
    clear = np.abs(rss - lim) > 0.01 * lim   # voxels away from the threshold
    assert np.array_equal((np.abs(est) > 0).any(0)[clear], (rss > lim)[clear])
    assert rel_l2(est[:, clear], ref[:, clear]) < 1e-4
    # unit root-sum-of-squares inside the mask
    m = rss > 1.01 * lim
    assert np.allclose((np.abs(est[:, m]) ** 2).sum(0), 1.0, atol=1e-5)


def test_smaps_recover_true_maps(gpu_lib, cgs, acquisition):
    k, kb_w, kb_b, p, taps, kft, S, x, data = acquisition
    est = estimate(cgs, k, kb_w, kb_b, data)
    St = S / np.sqrt((np.abs(S) ** 2).sum(0))[None]
    obj = np.abs(x) > 0.3 * np.abs(x).max()
    coh = np.abs((est * np.conj(St)).sum(0))[obj]
    assert coh.min() >= 0.97
    err = np.linalg.norm((np.abs(est) - np.abs(St))[:, obj]) / np.linalg.norm(np.abs(St)[:, obj])
    assert err <= 0.12


def test_smaps_argument_errors(gpu_lib, cgs, acquisition):
    import torch
    k, kb_w, kb_b, p, taps, kft, S, x, data = acquisition
    r = cgs.Reco(IMG, GRID, NCH, kb_w=kb_w, kb_b=kb_b)
    r.set_trajectory(k)
    maps = torch.zeros((NCH,) + IMG, dtype=torch.complex64, device="cuda")
    d = torch.from_numpy(data).cuda()
    for radius, eps in ((0.0, 0.05), (8.0, 1.0), (8.0, -0.1)):
        with pytest.raises(RuntimeError):
            r.estimate_smaps_tensor(d, maps, radius, eps)
    ns = k.shape[0]
    r.set_bins([np.arange(0, ns // 2), np.arange(ns // 2, ns)])
    with pytest.raises(RuntimeError):   # one bin (mask) only
        r.estimate_smaps_tensor(d, maps, RADIUS, EPS)
