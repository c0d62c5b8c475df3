"""GPU parity tests: the CUDA path (through the C ABI) against the
reference's golden vectors and the CPU oracle.

Tolerances (relative L2 unless stated):
  * centred FFT against the FP64 oracle: 2e-6;
  * deapodisation volume (kernelFT) against the reference: 1e-5;
  * NUFFT forward / adjoint against the reference: 2e-5 (FP32 gridding
    and FFT, different summation order);
  * CG-SENSE image against the reference after 16 iterations: 2e-4;
    residual sequence 2e-4 element-wise; iteration count exact;
  * oversampled operator (2x grid) against the FP64 oracle: 2e-5;
  * spreading is deterministic: two runs are bitwise equal.
"""
import numpy as np
import pytest

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu

OPS = ["ref_ops_24x20x16.npz", "ref_ops_32x24x16_mask.npz", "ref_ops_40x20x16_stop.npz"]


def make_reco(cgs, img, grid, nch, **kw):
    return cgs.Reco(img, grid, nch, **kw)


def golden_reco(cgs, z):
    grid = tuple(int(v) for v in z["grid"])
    nch = int(z["nch"])
    r = make_reco(cgs, grid, grid, nch)
    r.set_trajectory(z["k"])
    r.mask_from_data(z["data"])
    return r, grid, nch


@pytest.mark.parametrize("grid", [(24, 20, 16), (40, 20, 16), (64, 48, 32), (16, 512, 20)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft3_vs_oracle(gpu_lib, cgs, oracle_mod, o64, grid, sign):
    rng = np.random.default_rng(0)
    a = (rng.standard_normal(grid) + 1j * rng.standard_normal(grid)).astype(np.complex64)
    r = make_reco(cgs, grid, grid, 1)
    out = r.fft3(a, sign)
    ref = o64.centred_fft(oracle_mod.make_params(grid, grid, 1), a, sign, 0)
    assert rel_l2(out, ref) < 2e-6


@pytest.mark.parametrize("L", [16, 20, 24, 32, 40, 48, 64, 80, 96, 128, 160, 176, 192, 224, 256, 320,
                               352, 384, 448, 512])
def test_fft_every_line_length(gpu_lib, cgs, L):
    """Every supported line length, on each axis, against numpy."""
    rng = np.random.default_rng(L)
    for grid in [(L, 16, 16), (16, L, 16), (16, 16, L)]:
        a = (rng.standard_normal(grid) + 1j * rng.standard_normal(grid)).astype(np.complex64)
        r = make_reco(cgs, grid, grid, 1)
        out = r.fft3(a, -1)
        ref = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(a.astype(np.complex128))))
        ref *= (-1.0) ** sum(n // 2 for n in grid)
        assert rel_l2(out, ref) < 2e-6, grid
        r.close()


@pytest.mark.parametrize("name", OPS)
def test_kernel_ft_vs_reference(gpu_lib, cgs, name):
    z = golden(name)
    r, grid, nch = golden_reco(cgs, z)
    assert rel_l2(r.kernel_ft(), z["kernelft"]) < 1e-5


@pytest.mark.parametrize("name", OPS)
def test_nufft_fwd_vs_reference(gpu_lib, cgs, name):
    """Reco::nufftFWD (Reco.cpp:521-553), excluded samples included."""
    z = golden(name)
    r, grid, nch = golden_reco(cgs, z)
    out = r.nufft_fwd(z["img"])
    assert rel_l2(out, z["fwd_data"]) < 2e-5
    # samples excluded by excludeMissingData get no taps: exactly zero
    assert np.array_equal(out == 0, z["fwd_data"] == 0)


@pytest.mark.parametrize("name", OPS)
def test_nufft_adj_vs_reference(gpu_lib, cgs, name):
    """Reco::nufftBWD (Reco.cpp:468-519)."""
    z = golden(name)
    r, grid, nch = golden_reco(cgs, z)
    assert rel_l2(r.nufft_adj(z["data"]), z["bwd_img"]) < 2e-5


@pytest.mark.parametrize("name", OPS)
def test_cg_sense_vs_reference(gpu_lib, cgs, name):
    """Reco::cgSenseDynamic (Reco.cpp:175-321) with density weights, the
    16-iteration cap and the residual threshold."""
    z = golden(name)
    r, grid, nch = golden_reco(cgs, z)
    r.set_dcf(z["dcf"])
    r.set_smaps(z["smaps"])
    x, res, it = r.cg_sense(z["data"], float(z["cg_threshold"]), 16)
    assert it == int(z["cg_iters"][0])
    assert np.allclose(res, z["cg_residuals"], rtol=2e-4, atol=0)
    assert rel_l2(x, z["cg_x"]) < 2e-4


def oversampled_case(oracle_mod, o64, img, grid, nch, n_lines, n_read, seed=3, kb_w=4.0, kb_b=None):
    rng = np.random.default_rng(seed)
    t = np.linspace(0.02, 0.98, n_read)
    ky, kz = rng.uniform(0.1, 0.9, n_lines), rng.uniform(0.1, 0.9, n_lines)
    k = np.zeros((n_lines, n_read, 3))
    k[..., 0] = t
    k[..., 1] = ky[:, None] + 0.03 * np.sin(2 * np.pi * 5 * t)
    k[..., 2] = kz[:, None] + 0.03 * np.cos(2 * np.pi * 5 * t)
    k = k.reshape(-1, 3)
    if kb_b is None:
        kb_b = float(np.pi * np.sqrt(kb_w ** 2 / 4 * 1.5 ** 2 - 0.8))
    p = oracle_mod.make_params(img, grid, nch, kb_w=kb_w, kb_b=kb_b)
    taps = o64.taps(p, k)
    return k, p, taps, kb_w, kb_b


@pytest.mark.parametrize("img,grid", [((16, 16, 16), (32, 32, 32)), ((32, 24, 20), (64, 48, 40)),
                                      ((20, 16, 12), (32, 32, 24)),
                                      # Gx >= 128: wide pruned x passes
                                      ((64, 16, 16), (128, 32, 32)), ((100, 12, 10), (192, 24, 20))])
def test_oversampled_nufft_vs_oracle(gpu_lib, cgs, oracle_mod, o64, img, grid):
    """2x oversampled grid with zero-pad / crop (pruned FFT passes)."""
    nch = 3
    k, p, taps, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 40, 64)
    rng = np.random.default_rng(9)
    x = (rng.standard_normal((nch,) + img) + 1j * rng.standard_normal((nch,) + img)).astype(np.complex64)
    y = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    kft = o64.kernel_ft(p)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    assert rel_l2(r.nufft_fwd(x), o64.nufft_fwd(p, taps, kft, x)) < 2e-5
    assert rel_l2(r.nufft_adj(y), o64.nufft_adj(p, taps, kft, y)) < 2e-5


@pytest.mark.parametrize("img,grid", [((16, 16, 12), (32, 32, 24)), ((64, 16, 12), (128, 32, 24))])
def test_apply_ehde_vs_oracle_and_hermitian(gpu_lib, cgs, oracle_mod, o64, synth, img, grid):
    nch = 4
    k, p, taps, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 50, 64)
    smaps = synth.coil_maps(img, nch)
    dcf = np.random.default_rng(2).uniform(0.5, 1.5, k.shape[0]).astype(np.float32)
    rng = np.random.default_rng(4)
    x = (rng.standard_normal(img) + 1j * rng.standard_normal(img)).astype(np.complex64)
    v = (rng.standard_normal(img) + 1j * rng.standard_normal(img)).astype(np.complex64)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    r.set_dcf(dcf)
    r.set_smaps(smaps)
    q = r.apply_ehde(x)
    qo = o64.apply_ehde(p, taps, o64.kernel_ft(p), smaps, dcf, x)
    assert rel_l2(q, qo) < 2e-5
    qv = r.apply_ehde(v)
    lhs, rhs = np.vdot(v, q), np.vdot(qv, x)
    assert abs(lhs - rhs) < 1e-4 * abs(lhs)
    # determinism: spreading has no atomics
    assert np.array_equal(q, r.apply_ehde(x))


@pytest.mark.parametrize("img,grid", [((16, 16, 12), (32, 32, 24)), ((64, 16, 12), (128, 32, 24))])
def test_batched_bins_match_per_bin_oracle(gpu_lib, cgs, oracle_mod, o64, synth, img, grid):
    """All bins in one graph-captured solve equal independent solves."""
    nch = 3
    k, p, taps_all, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 60, 48)
    n_read = 48
    rb = [np.arange(0, 10), np.arange(10, 32), np.arange(32, 35), np.arange(35, 60)]
    bins = synth.bin_samples(rb, n_read)
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(6)
    data = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    dcf = rng.uniform(0.5, 1.5, k.shape[0]).astype(np.float32)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    r.set_dcf(dcf)
    r.set_bins(bins)
    r.set_smaps(smaps)
    x, res, it = r.cg_sense_batched(data, 0.0, 6)
    kft = o64.kernel_ft(p)
    for bi, s in enumerate(bins):
        mask = np.zeros(k.shape[0], np.uint8)
        mask[s] = 1
        tb = o64.taps(p, k, mask)
        st, xo, reso, ito = o64.cg_sense(p, tb, kft, smaps, dcf, data, 0.0, 6)
        assert it[bi] == ito == 6
        assert rel_l2(x[bi], xo) < 1e-4, bi
        assert np.allclose(res[bi, :6], reso, rtol=1e-4)


def test_autotune_keeps_results_bitwise(gpu_lib, cgs, oracle_mod, o64, synth):
    """The autotuner only changes launch shapes (coils per spreading block,
    coils per interpolation thread); every coil keeps its summation order,
    so the batched solve is bitwise unchanged."""
    img, grid, nch = (32, 24, 20), (64, 48, 40), 7
    k, p, taps_all, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 40, 48)
    bins = synth.bin_samples([np.arange(0, 15), np.arange(15, 40)], 48)
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(9)
    data = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    r.set_bins(bins)
    r.set_smaps(smaps)
    x0, res0, _ = r.cg_sense_batched(data, 0.0, 5)
    tune = r.autotune()
    assert tune["spread_variant"] in (1, 2, 4, 5, 6, 7, 8)
    if tune["spread_variant"] in (6, 7):   # the gather's parameter: coils per thread
        assert tune["spread_coils_per_block"] in (4, 6, 8)
    elif tune["spread_variant"] == 8:      # fused with the adjoint x pass: coils per block
        assert tune["spread_coils_per_block"] in (2, 4, 6)
    else:
        assert tune["spread_coils_per_block"] in range(1, nch + 1)
    assert tune["interp_coils_per_thread"] in (1, 2, 4, 6, 8)
    assert len(tune["candidates_ms"]) >= 6 and all(t > 0 for t in tune["candidates_ms"])
    x1, res1, _ = r.cg_sense_batched(data, 0.0, 5)
    assert np.array_equal(x0, x1)
    assert np.array_equal(res0, res1)


@pytest.mark.parametrize("img,grid,nch", [((32, 24, 20), (64, 48, 40), 7), ((48, 40, 24), (96, 80, 48), 12)])
def test_spreading_variants_bitwise(gpu_lib, cgs, oracle_mod, o64, synth, img, grid, nch):
    """The fixed-order spreading variants (one / two warps per x plane,
    plain or persistent and pipelined, the gather over the transposed tap
    matrix with and without its shared-memory staging, the gather fused with
    the adjoint x pass) and every coil chunk size give bitwise-identical
    solves: each grid value is summed in the same order, and the fused x
    transform does the unfused pass's operations."""
    k, p, taps_all, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 60, 48)
    bins = synth.bin_samples([np.arange(0, 7), np.arange(7, 41), np.arange(41, 60)], 48)
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(13)
    data = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    r.set_bins(bins)
    r.set_smaps(smaps)
    r.set_launch_shape(0, 1, 4)
    x0, res0, _ = r.cg_sense_batched(data, 0.0, 4)
    for cc in (0, 3, 5):
        for variant in (1, 2, 4, 5, 6, 7, 8):
            r.set_launch_shape(cc, variant, 2)
            x1, res1, _ = r.cg_sense_batched(data, 0.0, 4)
            assert np.array_equal(x1, x0), (cc, variant)
            assert np.array_equal(res1, res0), (cc, variant)
    # the fused kernel's coil chunks (with 7 coils none applies: variant 6 runs)
    for cc in (2, 4, 6):
        r.set_launch_shape(cc, 8, 2)
        x1, res1, _ = r.cg_sense_batched(data, 0.0, 4)
        assert np.array_equal(x1, x0) and np.array_equal(res1, res0), cc
        assert r.spread_fused() == (nch % cc == 0), cc
    # compensated sums: the tiled kernel and the transposed-matrix gather agree bitwise
    r.set_precision("compensated")
    r.set_launch_shape(0, 1, 2)
    xk, rk, _ = r.cg_sense_batched(data, 0.0, 4)
    r.set_launch_shape(0, 6, 2)
    xk6, rk6, _ = r.cg_sense_batched(data, 0.0, 4)
    assert np.array_equal(xk, xk6) and np.array_equal(rk, rk6)
    r.set_launch_shape(0, 7, 2)
    xk7, rk7, _ = r.cg_sense_batched(data, 0.0, 4)
    assert np.array_equal(xk, xk7) and np.array_equal(rk, rk7)
    r.set_launch_shape(0, 8, 2)
    xk8, rk8, _ = r.cg_sense_batched(data, 0.0, 4)
    assert np.array_equal(xk, xk8) and np.array_equal(rk, rk8)
    # every interpolation shape (coils per thread) sums each sample in the
    # same order
    r.set_precision(False)
    for icc in (1, 2, 4, 6, 8):
        r.set_launch_shape(0, 6, icc)
        x1, res1, _ = r.cg_sense_batched(data, 0.0, 4)
        assert np.array_equal(x1, x0), icc
        assert np.array_equal(res1, res0), icc


@pytest.mark.parametrize("img,grid,nch", [((32, 24, 20), (64, 48, 40), 5),
                                          # x passes with 8-column tiles (L = 320), Gz % 16 != 0
                                          ((160, 16, 12), (320, 32, 24), 3),
                                          ((48, 40, 24), (96, 80, 48), 4),
                                          # the forward y pass stores listed rows only
                                          ((32, 32, 16), (64, 64, 32), 3),
                                          # listed rows with 8-column x tiles inside 16-column y tiles
                                          ((32, 32, 20), (64, 64, 40), 3),
                                          # row masks read as 16-byte words (Gy / 32 a multiple of 4)
                                          ((32, 64, 16), (64, 128, 32), 4)])
def test_support_pruning_bitwise(gpu_lib, cgs, oracle_mod, o64, synth, img, grid, nch):
    """Sample-support pruning (x passes over the supported column tiles only,
    masked y passes, spreading tiles of supported columns only) leaves every
    result unchanged: the forward and adjoint NUFFT and the batched solve of
    sparse bins are bitwise equal with and without it."""
    k, p, taps_all, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 60, 48)
    bins = synth.bin_samples([np.arange(0, 3), np.arange(3, 11), np.arange(11, 60)], 48)
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(21)
    data = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    x = (rng.standard_normal((nch,) + img) + 1j * rng.standard_normal((nch,) + img)).astype(np.complex64)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    r.set_smaps(smaps)
    f0, a0 = r.nufft_fwd(x), r.nufft_adj(data)
    r.set_support_pruning(False)
    f1, a1 = r.nufft_fwd(x), r.nufft_adj(data)
    assert np.array_equal(f0, f1) and np.array_equal(a0, a1)
    r.set_bins(bins)
    out = {}
    for on in (True, False):
        r.set_support_pruning(on)
        for variant in (1, 2, 4, 6, 7, 8):
            r.set_launch_shape(0, variant, 2)
            out[on, variant] = r.cg_sense_batched(data, 0.0, 4)[:2]
    ref = out[False, 1]
    for key, (xv, res) in out.items():
        assert np.array_equal(xv, ref[0]), key
        assert np.array_equal(res, ref[1]), key
    # per-bin applications reuse workspace slot 0 for other bins between
    # replays of the batched solve's graph
    img1 = x[0]
    q_off = [r.apply_ehde(img1, bin=b) for b in range(3)]
    r.set_support_pruning(True)
    r.set_launch_shape(0, 1, 2)
    for b in (2, 0, 1, 2):
        assert np.array_equal(r.apply_ehde(img1, bin=b), q_off[b]), b
        xv, res = r.cg_sense_batched(data, 0.0, 4)[:2]
        assert np.array_equal(xv, ref[0]) and np.array_equal(res, ref[1]), b


def test_atomic_spreading_matches_fixed_order(gpu_lib, cgs, oracle_mod, o64, synth):
    """With determinism off the autotuner may pick shared-memory atomic
    spreading; forced here, the batched solve equals the fixed-order one to
    FP32 rounding."""
    img, grid, nch = (32, 24, 20), (64, 48, 40), 5
    k, p, taps_all, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 40, 48)
    bins = synth.bin_samples([np.arange(0, 15), np.arange(15, 40)], 48)
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(12)
    data = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    r.set_bins(bins)
    r.set_smaps(smaps)
    x0, res0, _ = r.cg_sense_batched(data, 0.0, 5)
    r.set_deterministic(False)
    tune = r.autotune()
    assert tune["spread_variant"] in (1, 2, 3, 4, 5, 6, 7, 8)
    x1, res1, _ = r.cg_sense_batched(data, 0.0, 5)
    assert rel_l2(x1, x0) < 1e-5
    assert np.allclose(res1, res0, rtol=1e-5)


def test_empty_bin_and_zero_data(gpu_lib, cgs, synth):
    """A bin without samples (or all-zero data) has a zero right-hand side:
    the solve returns x = 0 after 0 iterations."""
    img, grid, nch = (8, 8, 8), (16, 16, 16), 2
    rng = np.random.default_rng(0)
    k = rng.uniform(0.2, 0.8, (100, 3))
    r = make_reco(cgs, img, grid, nch)
    r.set_trajectory(k)
    r.set_bins([np.arange(100), np.array([], np.int64)])
    r.set_smaps(synth.coil_maps(img, nch))
    data = (rng.standard_normal((nch, 100)) + 1j * rng.standard_normal((nch, 100))).astype(np.complex64)
    x, res, it = r.cg_sense_batched(data, 0.0, 4)
    assert it[1] == 0 and np.all(x[1] == 0)
    assert it[0] == 4 and np.isfinite(x[0]).all() and np.abs(x[0]).max() > 0


def test_input_faults_are_reported(gpu_lib, cgs, synth):
    img, grid, nch = (8, 8, 8), (16, 16, 16), 2
    r = make_reco(cgs, img, grid, nch)
    with pytest.raises(cgs.CGSError) as e:
        r.nufft_fwd(np.zeros((nch,) + img, np.complex64))
    assert e.value.code == cgs.CGS_ERR_STATE
    k = np.random.default_rng(0).uniform(0.2, 0.8, (50, 3))
    r.set_trajectory(k)
    bad = synth.coil_maps(img, nch)
    bad[1, 2, 3, 4] = np.nan
    with pytest.raises(cgs.CGSError) as e:
        r.set_smaps(bad)
    assert e.value.code == cgs.CGS_ERR_NONFINITE
    with pytest.raises(ValueError):
        r.set_smaps(np.zeros((nch, 4, 4, 4), np.complex64))
    r.set_smaps(synth.coil_maps(img, nch))
    with pytest.raises(cgs.CGSError) as e:
        r.cg_sense(np.zeros((nch, 50), np.complex64), -1.0)
    assert e.value.code == cgs.CGS_ERR_NO_THRESHOLD
    kk = k.copy()
    kk[3, 1] = np.inf
    with pytest.raises(cgs.CGSError) as e:
        r.set_trajectory(kk)
    assert e.value.code == cgs.CGS_ERR_NONFINITE


@pytest.mark.parametrize("compensated", [False, True])
def test_precision_form_against_fp64(gpu_lib, cgs, oracle_mod, o64, synth, compensated):
    """The complex64 solve (FP32 gridding and FFT, FP64 CG scalars) against
    the full-FP64 GPU solve, iteration by iteration: relative L2 <= 1e-4.
    The FP64 GPU solve itself agrees with the FP64 CPU oracle to 1e-6 (its
    inputs -- coil maps, deapodisation, tap weights -- are float)."""
    import torch
    img, grid, nch = (32, 24, 20), (64, 48, 40), 4
    k, p, taps, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 60, 64)
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(8)
    x_true = synth.phantom(img)
    dcf = rng.uniform(0.5, 1.5, k.shape[0]).astype(np.float32)
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b)
    r.set_trajectory(k)
    data = r.nufft_fwd(smaps * x_true[None])
    data += synth.complex_noise(data.shape, 30.0, float(np.sqrt(np.mean(np.abs(data) ** 2))))
    r.set_dcf(dcf)
    r.set_smaps(smaps)
    r.set_precision(compensated)
    iters = 10
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        d = torch.from_numpy(data).cuda()
        x32 = torch.zeros((1,) + img, dtype=torch.complex64, device="cuda")
        x64 = torch.zeros((1,) + img, dtype=torch.complex128, device="cuda")
        t32 = torch.zeros((iters, 1) + img, dtype=torch.complex64, device="cuda")
        t64 = torch.zeros((iters, 1) + img, dtype=torch.complex128, device="cuda")
    stream.synchronize()
    res32, it32 = r.cg_sense_trace_tensor(d, x32, 0.0, iters, t32)
    res64, it64 = r.cg_sense_fp64_tensor(d, x64, 0.0, iters, t64)
    stream.synchronize()
    assert it32[0] == it64[0] == iters
    a32, a64 = t32.cpu().numpy(), t64.cpu().numpy()
    errs = [rel_l2(a32[i], a64[i]) for i in range(iters)]
    assert max(errs) < 1e-4, errs
    st, xo, reso, ito = o64.cg_sense(p, taps, o64.kernel_ft(p), smaps, dcf, data, 0.0, iters)
    assert rel_l2(x64.cpu().numpy()[0], xo) < 1e-6
    assert np.allclose(res64[0, :iters], reso, rtol=1e-6)


@pytest.mark.parametrize("groups,toeplitz", [(False, False), (True, False), (False, True)])
def test_fused_cg_updates_bitwise(gpu_lib, cgs, oracle_mod, o64, synth, groups, toeplitz):
    """The solve whose forward z pass applies the previous iteration's
    x += alpha p and p = r + beta p (Reco.cpp:285-290,306-307), with alpha
    folded into the residual update and beta into the loop test, gives the
    same bits as the solve with a kernel per update (the trace form): images,
    residuals and iteration counts -- with a bin that stops on the threshold
    before the others, an empty bin, several workspace groups and the
    Toeplitz operator."""
    import torch
    img, grid, nch = (16, 16, 12), (32, 32, 24), 3
    k, p, taps_all, w, b = oversampled_case(oracle_mod, o64, img, grid, nch, 60, 48)
    rb = [np.arange(0, 10), np.arange(10, 32), np.arange(32, 35), np.arange(35, 60)]
    bins = synth.bin_samples(rb, 48) + [np.array([], np.int64)]
    smaps = synth.coil_maps(img, nch)
    rng = np.random.default_rng(16)
    data = (rng.standard_normal((nch, k.shape[0])) + 1j * rng.standard_normal((nch, k.shape[0]))).astype(np.complex64)
    dcf = rng.uniform(0.5, 1.5, k.shape[0]).astype(np.float32)
    per_bin = nch * (img[0] * img[1] * grid[2] + 2 * img[0] * grid[1] * grid[2] + int(np.prod(grid))) * 8
    r = make_reco(cgs, img, grid, nch, kb_w=w, kb_b=b, workspace_bytes=2 * per_bin if groups else 0)
    r.set_trajectory(k)
    r.set_dcf(dcf)
    r.set_bins(bins)
    r.set_smaps(smaps)
    if toeplitz:
        r.set_toeplitz(1)
    iters, nb = 8, len(bins)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        d = torch.from_numpy(data).cuda()
        xf = torch.zeros((nb,) + img, dtype=torch.complex64, device="cuda")
        xs = torch.zeros_like(xf)
        tr = torch.zeros((iters, nb) + img, dtype=torch.complex64, device="cuda")
    stream.synchronize()
    res0, _ = r.cg_sense_trace_tensor(d, xs, 0.0, iters, tr)
    # a threshold between bin 1's residuals after its 3rd and 4th iterations
    # stops it early; the other bins may stop at other iterations
    thresh = float(0.5 * (res0[1, 2] + res0[1, 3]))
    for _ in range(2):   # the second call replays the captured graph
        resf, itf = r.cg_sense_batched_tensor(d, xf, thresh, iters)
        ress, its = r.cg_sense_trace_tensor(d, xs, thresh, iters, tr)
        stream.synchronize()
        assert np.array_equal(itf, its) and itf[1] == 4 and itf[nb - 1] == 0
        assert np.array_equal(resf, ress)
        assert torch.equal(xf, xs)
        assert torch.count_nonzero(xf[nb - 1]) == 0 and torch.count_nonzero(xf[0]) > 0
    r.close()
