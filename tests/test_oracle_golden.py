"""Pins the CPU oracle to the reference: the golden vectors in tests/golden/
were produced by the reference's own Reco.cpp / Fourier.cpp /
Trajectory.cpp compiled unmodified (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden, rel_l2

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
