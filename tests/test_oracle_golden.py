"""Pins the CPU oracle to the reference: the golden vectors in tests/golden/
were produced by the reference's own Reco.cpp / Fourier.cpp /
Trajectory.cpp compiled unmodified (tests/golden/make_golden.py)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel_l2

if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

OPS = ["ref_ops_24x20x16.npz", "ref_ops_32x24x16_mask.npz", "ref_ops_40x20x16_stop.npz"]


def _setup(oracle_mod, o, z):
    grid = tuple(int(v) for v in z["grid"])
    nch = int(z["nch"])
    p = oracle_mod.make_params(grid, grid, nch)
    data = z["data"]
    mask = ~((data[0].real == 0) & (data[0].imag == 0))
    taps = o.taps(p, z["k"], mask.astype(np.uint8))
    return p, grid, nch, taps


@pytest.mark.parametrize("name", OPS)
def test_taps_bit_exact(oracle_mod, o64, name):
    """ConvKernel::calculateWeights + excludeMissingData: same taps, same
    float weights, same order (Reco.cpp:698-806)."""
    z = golden(name)
    p, grid, nch, taps = _setup(oracle_mod, o64, z)
    assert np.array_equal(np.diff(taps.ptr).astype(np.int32), z["tap_count"])
    assert np.array_equal(taps.idx, z["tap_idx"])
    assert np.array_equal(taps.w, z["tap_w"])


@pytest.mark.parametrize("name", OPS)
def test_kernel_ft(oracle_mod, o64, name):
    z = golden(name)
    p, grid, nch, taps = _setup(oracle_mod, o64, z)
    assert rel_l2(o64.kernel_ft(p), z["kernelft"]) < 1e-6


@pytest.mark.parametrize("name", OPS)
@pytest.mark.parametrize("prec", [64, 32])
def test_nufft_fwd_adj(oracle_mod, o64, o32, name, prec):
    """Reco::nufftFWD / nufftBWD: FP64 oracle and FP32 port within 1e-5."""
    o = o64 if prec == 64 else o32
    z = golden(name)
    p, grid, nch, taps = _setup(oracle_mod, o, z)
    kft = o.kernel_ft(p)
    assert rel_l2(o.nufft_fwd(p, taps, kft, z["img"]), z["fwd_data"]) < 1e-5
    assert rel_l2(o.nufft_adj(p, taps, kft, z["data"]), z["bwd_img"]) < 1e-5


@pytest.mark.parametrize("name", OPS)
@pytest.mark.parametrize("prec", [64, 32])
def test_cg_sense(oracle_mod, o64, o32, name, prec):
    """Reco::cgSenseDynamic: image within 1e-4, residual sequence within 1e-4,
    same number of iterations (incl. the threshold stop)."""
    o = o64 if prec == 64 else o32
    z = golden(name)
    p, grid, nch, taps = _setup(oracle_mod, o, z)
    kft = o.kernel_ft(p)
    st, x, res, it = o.cg_sense(p, taps, kft, z["smaps"], z["dcf"], z["data"],
                                float(z["cg_threshold"]), 16)
    assert st == 0
    assert it == int(z["cg_iters"][0])
    assert np.allclose(res, z["cg_residuals"], rtol=1e-4, atol=0)
    assert rel_l2(x, z["cg_x"]) < 1e-4


@pytest.mark.parametrize("name", ["ref_traj_wave.npz", "ref_traj_wave_b.npz"])
def test_wave_caipi(o64, name):
    """WaveCaipi::calculateTraj (Trajectory.cpp:18-184), double precision."""
    z = golden(name)
    wave = dict(z["wave"].tolist())
    g = [int(v) for v in z["grid"]]
    k = o64.wave_caipi(sx=int(z["sx"]), sy=int(z["sy"]), sz=int(z["sz"]), gx=g[0], gy=g[1], gz=g[2],
                       fov_y=float(z["fov_y"]), fov_z=float(z["fov_z"]), n_osc=int(wave["nosc"]),
                       grad_amp=wave["grad_amp"], amp_corr_y=wave["amp_corr_y"],
                       amp_corr_z=wave["amp_corr_z"], shift_y=wave["shift_y"],
                       shift_z=wave["shift_z"], dwell=wave["dwell"])
    assert np.max(np.abs(k - z["traj"])) < 1e-12


@pytest.fixture(scope="module")
def wave_cg():
    """The mid-size fixture (64x64x48 grid == image, 4 coils, 32 768
    wave-CAIPI samples, the reference's KB w = 4.25 / b = 14.9086) and its
    regenerated inputs (tests/golden/make_golden.py: wave_cg_inputs)."""
    import make_golden as mg
    z = golden(mg.WAVE_CG_NAME)
    w, k, smaps, x, dcf, y = mg.wave_cg_inputs()
    fp = mg.input_fingerprint(k, y)
    assert np.allclose(fp, z["fingerprint"], rtol=1e-6, atol=0), "regenerated inputs drifted"
    return z, w, k, smaps, x, dcf, y


def test_wave_cg_taps(oracle_mod, o64, wave_cg):
    """calculateWeights at a realistic size: the 11^3 neighbourhood, the
    float distance arithmetic and the grid faces (readouts leave the grid):
    per-sample tap counts exact, per-sample weight sums to float rounding."""
    z, w, k, smaps, x, dcf, y = wave_cg
    p = oracle_mod.make_params(w.img, w.grid, w.n_ch)
    taps = o64.taps(p, k)
    cnt = np.diff(taps.ptr)
    assert np.array_equal(cnt, z["tap_count"].astype(np.int64))
    ws = np.add.reduceat(taps.w.astype(np.float64), taps.ptr[:-1]) * (cnt > 0)
    assert np.allclose(ws, z["tap_wsum"], rtol=1e-6, atol=0)


@pytest.mark.parametrize("prec", [64, 32])
def test_wave_cg_operators_and_solve(oracle_mod, o64, o32, wave_cg, prec):
    """nufftFWD, nufftBWD and cgSenseDynamic of the mid-size fixture: the
    FP64 oracle and the FP32 port against the reference's own outputs."""
    o = o64 if prec == 64 else o32
    z, w, k, smaps, x, dcf, y = wave_cg
    p = oracle_mod.make_params(w.img, w.grid, w.n_ch)
    taps = o.taps(p, k)
    kft = o.kernel_ft(p)
    fwd = o.nufft_fwd(p, taps, kft, (smaps * x[None]).astype(np.complex64))
    assert rel_l2(fwd[:, ::8], z["fwd_every8"]) < 1e-5
    bwd = o.nufft_adj(p, taps, kft, y * dcf[None])
    assert rel_l2(bwd[0][::2, ::2, ::2], z["bwd_coil0_sub2"]) < 1e-5
    st, xo, res, it = o.cg_sense(p, taps, kft, smaps, dcf, y, 0.0, 16)
    assert st == 0 and it == int(z["cg_iters"][0]) == 16
    assert np.allclose(res, z["cg_residuals"], rtol=1e-4, atol=0)
    assert rel_l2(xo[::2, ::2, ::2], z["cg_x_sub2"]) < 1e-4
