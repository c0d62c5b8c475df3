"""GPU parity at realistic sizes, through the C ABI.

* The mid-size reference fixture (tests/golden/ref_cg_64x64x48_wave.npz):
  the reference's own calculateWeights / nufftFWD / nufftBWD /
  cgSenseDynamic (Reco.cpp:175-321,468-553,698-806) on a 64x64x48 grid ==
  image, 4 coils, 32 768 wave-CAIPI samples, KB w = 4.25 / b = 14.9086 --
  the reference's parameters, where its 11^3 tap neighbourhood and float
  distance arithmetic matter and readouts leave the grid.  Tolerances as for
  the small reference fixtures: forward / adjoint 2e-5 relative L2, CG
  image 2e-4, residual sequence 2e-4 element-wise, iteration count exact.
* The benchmark's CPU-path configuration at its full size: a 64^3 image on
  the 2x oversampled 128^3 grid, 8 coils, 1024 wave-CAIPI readouts of 256
  samples (262 144 samples, R = 2x2, +-4 cells, 7 cycles), Voronoi density
  weights, KB width 4, 10 CG iterations -- against the FP64 oracle:
  operator 2e-5, image after 5 and 10 iterations 1e-4, residual sequence
  1e-4 element-wise.
* A crop box off the grid centre (the offcenter of Reco.cpp:627-671)
  against the oracle with the same box.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel_l2

if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

pytestmark = pytest.mark.gpu


def beatty_beta(w, sigma=2.0):
    return float(np.pi * np.sqrt(w ** 2 / sigma ** 2 * (sigma - 0.5) ** 2 - 0.8))


@pytest.fixture(scope="module")
def wave_cg():
    import make_golden as mg
    z = golden(mg.WAVE_CG_NAME)
    w, k, smaps, x, dcf, y = mg.wave_cg_inputs()
    assert np.allclose(mg.input_fingerprint(k, y), z["fingerprint"], rtol=1e-6, atol=0), \
        "regenerated inputs drifted"
    return z, w, k, smaps, x, dcf, y


def test_wave_cg_fixture_vs_reference(gpu_lib, cgs, wave_cg):
    """The reference's own outputs at 64x64x48 / 4 coils / 32 768 samples."""
    z, w, k, smaps, x, dcf, y = wave_cg
    r = cgs.Reco(w.img, w.grid, w.n_ch)          # reference KB: w = 4.25, b = 14.9086
    r.set_trajectory(k)
    fwd = r.nufft_fwd(smaps * x[None])
    assert rel_l2(fwd[:, ::8], z["fwd_every8"]) < 2e-5
    # readouts that leave the grid keep only their in-grid taps, as in the
    # reference; samples whose every tap fell outside give exactly zero
    zero = z["tap_count"] == 0
    assert np.all(fwd[:, zero] == 0)
    bwd = r.nufft_adj(y * dcf[None])
    assert rel_l2(bwd[0][::2, ::2, ::2], z["bwd_coil0_sub2"]) < 2e-5
    r.set_dcf(dcf)
    r.set_smaps(smaps)
    xg, res, it = r.cg_sense(y, 0.0, 16)
    assert it == int(z["cg_iters"][0]) == 16
    assert np.allclose(res, z["cg_residuals"], rtol=2e-4, atol=0)
    assert rel_l2(xg[::2, ::2, ::2], z["cg_x_sub2"]) < 2e-4
    assert abs(np.linalg.norm(xg.astype(np.complex128)) / float(z["cg_x_norm"]) - 1) < 2e-4
    # the graph-captured batched solve of the same single bin
    xb, resb, itb = r.cg_sense_batched(y, 0.0, 16)
    assert itb[0] == 16
    assert np.allclose(resb[0], z["cg_residuals"], rtol=2e-4, atol=0)
    assert rel_l2(xb[0][::2, ::2, ::2], z["cg_x_sub2"]) < 2e-4


@pytest.fixture(scope="module")
def cfg1(cgs, synth, oracle_mod, o64):
    """Inputs of the 64^3 / 8-coil / 262 144-sample configuration and the
    FP64 oracle's taps and deapodisation for them."""
    w = synth.WORKLOADS["cfg1"]
    k = synth.wave_trajectory(w)
    assert k.shape[0] == 1024 * 256
    dcf = synth.cap_dcf(cgs.voronoi_dcf(k))
    smaps = synth.coil_maps(w.img, w.n_ch)
    x = synth.phantom(w.img)
    kb_w = 4.0
    kb_b = beatty_beta(kb_w)
    p = oracle_mod.make_params(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b)
    taps = o64.taps(p, k)
    kft = o64.kernel_ft(p)
    y = o64.nufft_fwd(p, taps, kft, smaps.astype(np.complex128) * x[None]).astype(np.complex64)
    y += synth.complex_noise(y.shape, 30.0, float(np.sqrt(np.mean(np.abs(y) ** 2))))
    return w, k, dcf, smaps, x, kb_w, kb_b, p, taps, kft, y


def test_cfg1_full_size_vs_fp64_oracle(gpu_lib, cgs, o64, cfg1):
    w, k, dcf, smaps, x, kb_w, kb_b, p, taps, kft, y = cfg1
    r = cgs.Reco(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b)
    r.set_trajectory(k)
    assert rel_l2(r.nufft_fwd(smaps * x[None]), o64.nufft_fwd(p, taps, kft, smaps * x[None])) < 2e-5
    assert rel_l2(r.nufft_adj(y), o64.nufft_adj(p, taps, kft, y)) < 2e-5
    r.set_dcf(dcf)
    r.set_smaps(smaps)
    assert rel_l2(r.apply_ehde(x), o64.apply_ehde(p, taps, kft, smaps, dcf, x)) < 2e-5
    for iters in (5, 10):
        xg, res, it = r.cg_sense(y, 0.0, iters)
        st, xo, reso, ito = o64.cg_sense(p, taps, kft, smaps, dcf, y, 0.0, iters)
        assert st == 0 and it == ito == iters
        assert np.allclose(res, reso, rtol=1e-4, atol=0), (res, reso)
        assert rel_l2(xg, xo) < 1e-4
    # the batched graph-captured form (the benchmark's path) on the same bin
    xb, resb, itb = r.cg_sense_batched(y, 0.0, 10)
    assert itb[0] == 10
    assert np.allclose(resb[0], reso, rtol=1e-4, atol=0)
    assert rel_l2(xb[0], xo) < 1e-4


@pytest.mark.parametrize("off", [(3, -2, 1), (-5, 0, 4)])
def test_offcenter_box_vs_oracle(gpu_lib, cgs, synth, oracle_mod, o64, off):
    """The image box shifted by offcenter voxels from the grid centre
    (Reco.cpp:627-671 keeps the box centre + offcenter): padding, crop,
    deapodisation and the solve use the shifted box."""
    img, grid, nch = (24, 20, 16), (48, 40, 32), 3
    rng = np.random.default_rng(17)
    n_lines, n_read = 40, 64
    t = np.linspace(0.02, 0.98, n_read)
    k = np.zeros((n_lines, n_read, 3))
    k[..., 0] = t
    k[..., 1] = rng.uniform(0.1, 0.9, n_lines)[:, None] + 0.03 * np.sin(2 * np.pi * 5 * t)
    k[..., 2] = rng.uniform(0.1, 0.9, n_lines)[:, None] + 0.03 * np.cos(2 * np.pi * 5 * t)
    k = k.reshape(-1, 3)
    kb_w = 4.0
    kb_b = beatty_beta(kb_w)
    p = oracle_mod.make_params(img, grid, nch, kb_w=kb_w, kb_b=kb_b, offcenter=off)
    taps = o64.taps(p, k)
    kft = o64.kernel_ft(p)
    smaps = synth.coil_maps(img, nch)
    x = synth.phantom(img)
    y = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    dcf = rng.uniform(0.5, 1.5, k.shape[0]).astype(np.float32)
    r = cgs.Reco(img, grid, nch, kb_w=kb_w, kb_b=kb_b, offcenter=off)
    r.set_trajectory(k)
    imgs = smaps * x[None]
    assert rel_l2(r.nufft_fwd(imgs), o64.nufft_fwd(p, taps, kft, imgs)) < 2e-5
    assert rel_l2(r.nufft_adj(y), o64.nufft_adj(p, taps, kft, y)) < 2e-5
    r.set_dcf(dcf)
    r.set_smaps(smaps)
    assert rel_l2(r.apply_ehde(x), o64.apply_ehde(p, taps, kft, smaps, dcf, x)) < 2e-5
    xg, res, it = r.cg_sense(y, 0.0, 6)
    st, xo, reso, ito = o64.cg_sense(p, taps, kft, smaps, dcf, y, 0.0, 6)
    assert it == ito == 6
    assert rel_l2(xg, xo) < 1e-4
    assert np.allclose(res, reso, rtol=1e-4, atol=0)
    # a shifted box differs from the centred one
    r0 = cgs.Reco(img, grid, nch, kb_w=kb_w, kb_b=kb_b)
    r0.set_trajectory(k)
    assert rel_l2(r0.nufft_fwd(imgs), r.nufft_fwd(imgs)) > 1e-2
