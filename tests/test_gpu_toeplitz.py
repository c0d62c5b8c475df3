"""Toeplitz embedding of E^H D E (cgs_set_toeplitz): the library's operator
against the exact normal operator s sum_c conj(S_c) E^H D E S_c (FP64 numpy,
dense non-uniform DFT), the fused x stage against the unfused one, the
gridded operator against both, and CG solves with either operator.

Tolerances: Toeplitz vs the exact operator 2e-5 relative L2 (FP32 transforms
and spectrum); fused vs unfused x stage 1e-6 (summation order of the
transforms); gridded vs exact between 1e-5 and 5e-3 (the gridding error of
kernel width 4 at 2x oversampling); the Toeplitz CG against FP64 CG on the
exact operator 1e-4 after 10 iterations (FP32 vectors and operator)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

KB_W = 4.0
KB_B = float(np.pi * np.sqrt(KB_W ** 2 / 4 * 1.5 ** 2 - 0.8))


def random_case(img, nch, ns, nb, seed):
    rng = np.random.default_rng(seed)
    k = rng.uniform(0.1, 0.9, (ns, 3))
    dcf = rng.uniform(0.5, 1.5, ns).astype(np.float32)
    S = (rng.standard_normal((nch,) + img) + 1j * rng.standard_normal((nch,) + img)).astype(np.complex64)
    perm = rng.permutation(ns)
    bins = [np.sort(b) for b in np.array_split(perm, nb)]
    x = (rng.standard_normal((nb,) + img) + 1j * rng.standard_normal((nb,) + img)).astype(np.complex64)
    return k, dcf, S, bins, x


def make_reco(cgs, img, grid, nch, k, dcf, S, bins):
    r = cgs.Reco(img, grid, nch, kb_w=KB_W, kb_b=KB_B)
    r.set_trajectory(k)
    r.set_bins(bins)
    r.set_dcf(dcf)
    r.set_smaps(S)
    return r


def apply(r, x):
    import torch
    xt = torch.from_numpy(x).cuda()
    q = torch.zeros_like(xt)
    r.apply_ehde_tensor(xt, q, 0, x.shape[0])
    torch.cuda.synchronize()
    return q.cpu().numpy(), r.launch_count()


@pytest.mark.parametrize("img,grid,nch,ns", [
    ((16, 12, 8), (32, 24, 16), 2, 600),     # x lines of 32 (4 x 8)
    ((64, 12, 8), (128, 24, 16), 2, 500),    # 128 (8 x 16)
    ((128, 8, 8), (256, 16, 16), 3, 400),    # 256 (16 x 16), the benchmark's x length
])
def test_toeplitz_matches_exact_normal_operator(gpu_lib, cgs, oracle_mod, img, grid, nch, ns):
    k, dcf, S, bins, x = random_case(img, nch, ns, 2, seed=5)
    r = make_reco(cgs, img, grid, nch, k, dcf, S, bins)
    r.set_toeplitz(1)
    q1, n1 = apply(r, x)
    r.set_toeplitz(2)
    q2, n2 = apply(r, x)
    r.set_toeplitz(0)
    qg, _ = apply(r, x)
    assert n1 == 5 and n2 == 7   # fused x stage: one launch instead of three
    for b in range(2):
        ref = oracle_mod.exact_normal(k[bins[b]], img, grid, S.astype(np.complex128), dcf[bins[b]].astype(np.float64),
                                      x[b].astype(np.complex128))
        assert rel_l2(q1[b], ref) < 2e-5
        assert rel_l2(q2[b], ref) < 2e-5
        assert rel_l2(q1[b], q2[b]) < 1e-6
        assert 1e-5 < rel_l2(qg[b], ref) < 5e-3


def test_toeplitz_unfused_fallback_and_workspace_groups(gpu_lib, cgs, oracle_mod):
    """A grid oversampled by 2.5 along x (the fused x stage needs exactly 2x)
    falls back to the unfused x stage; a workspace of one bin runs the bins
    as separate groups, each with its own spectrum."""
    img, grid, nch = (16, 12, 8), (40, 24, 16), 2
    k, dcf, S, bins, x = random_case(img, nch, 600, 2, seed=13)
    r = make_reco(cgs, img, grid, nch, k, dcf, S, bins)
    r.set_toeplitz(1)
    q, n = apply(r, x)
    assert n == 7
    img2, grid2 = (16, 12, 8), (32, 24, 16)
    per_bin = nch * (img2[0] * img2[1] * grid2[2] + 2 * img2[0] * grid2[1] * grid2[2] + int(np.prod(grid2))) * 8
    r2 = cgs.Reco(img2, grid2, nch, kb_w=KB_W, kb_b=KB_B, workspace_bytes=per_bin)
    r2.set_trajectory(k)
    r2.set_bins(bins)
    r2.set_dcf(dcf)
    r2.set_smaps(S)
    r2.set_toeplitz(1)
    q2, n2 = apply(r2, x)
    assert n2 == 10   # two groups of five launches
    Sd = S.astype(np.complex128)
    for b in range(2):
        d = dcf[bins[b]].astype(np.float64)
        ref = oracle_mod.exact_normal(k[bins[b]], img, grid, Sd, d, x[b].astype(np.complex128))
        assert rel_l2(q[b], ref) < 2e-5
        ref2 = oracle_mod.exact_normal(k[bins[b]], img2, grid2, Sd, d, x[b].astype(np.complex128))
        assert rel_l2(q2[b], ref2) < 2e-5


def test_toeplitz_without_density_and_after_changes(gpu_lib, cgs, oracle_mod):
    """The spectra follow the density weights, the bins and the coordinates."""
    img, grid, nch = (16, 12, 8), (32, 24, 16), 2
    k, dcf, S, bins, x = random_case(img, nch, 500, 2, seed=9)
    r = make_reco(cgs, img, grid, nch, k, None, S, bins)
    r.set_toeplitz(1)
    ms, nbytes = r.toeplitz_stats()
    assert nbytes == 2 * int(np.prod(grid)) * 4 and ms > 0
    Sd = S.astype(np.complex128)

    def check(kk, d, bb):
        q, _ = apply(r, x)
        for b in range(2):
            ref = oracle_mod.exact_normal(kk[bb[b]], img, grid, Sd, None if d is None else d[bb[b]].astype(np.float64),
                                          x[b].astype(np.complex128))
            assert rel_l2(q[b], ref) < 2e-5

    check(k, None, bins)
    r.set_dcf(dcf)
    check(k, dcf, bins)
    bins2 = [bins[1], bins[0]]
    r.set_bins(bins2)
    check(k, dcf, bins2)
    # a new trajectory drops the density weights (they belong to the old samples)
    k2 = np.clip(k + 0.01, 0.05, 0.95)
    r.set_trajectory(k2)
    r.set_bins(bins2)
    check(k2, None, bins2)
    # coordinates updated on the device (the trajectory-optimisation path)
    import torch
    k3 = np.clip(k2 - 0.02, 0.05, 0.95)
    r.update_trajectory_tensor(torch.from_numpy(k3).cuda())
    check(k3, None, bins2)


def test_toeplitz_needs_room_for_the_embedding(gpu_lib, cgs):
    img, grid, nch = (16, 12, 8), (24, 24, 16), 1
    k, dcf, S, bins, x = random_case(img, nch, 200, 1, seed=3)
    r = make_reco(cgs, img, grid, nch, k, dcf, S[:1], bins)
    with pytest.raises(cgs.CGSError):
        r.set_toeplitz(1)
    with pytest.raises(cgs.CGSError):
        r.set_toeplitz(3)
    apply(r, x)   # the gridded operator still works


def test_toeplitz_refuses_the_gridded_trajectory_derivative(gpu_lib, cgs):
    """The operator's trajectory derivative belongs to the gridded operator:
    it is refused while the embedding is on, and works again once it is off."""
    import torch
    img, grid, nch = (16, 12, 8), (32, 24, 16), 2
    k, dcf, S, bins, x = random_case(img, nch, 300, 1, seed=17)
    r = make_reco(cgs, img, grid, nch, k, dcf, S, bins)
    p = torch.from_numpy(x).cuda()
    g = torch.zeros((300, 3), dtype=torch.float32, device="cuda")
    L = gpu_lib
    import ctypes as C
    r.set_toeplitz(1)
    st = L.cgs_apply_vjp_k_d(r.ctx, 0, 1, C.c_void_p(p.data_ptr()), C.c_void_p(p.data_ptr()), C.c_void_p(g.data_ptr()))
    assert st == cgs.CGS_ERR_STATE
    assert b"Toeplitz" in L.cgs_last_error(r.ctx)
    r.set_toeplitz(0)
    assert r.toeplitz_stats() == (0.0, 0)
    st = L.cgs_apply_vjp_k_d(r.ctx, 0, 1, C.c_void_p(p.data_ptr()), C.c_void_p(p.data_ptr()), C.c_void_p(g.data_ptr()))
    torch.cuda.synchronize()
    assert st == 0 and bool(torch.isfinite(g).all())


def test_toeplitz_cg_matches_exact_cg(gpu_lib, cgs, oracle_mod):
    """CG-SENSE from coil images with the Toeplitz operator against the same
    CG (Reco.cpp:175-321) in FP64 numpy on the exact normal operator."""
    img, grid, nch, iters = (16, 12, 8), (32, 24, 16), 3, 10
    k, dcf, S, bins, x = random_case(img, nch, 900, 1, seed=21)
    r = make_reco(cgs, img, grid, nch, k, dcf, S, bins)
    r.set_toeplitz(1)
    rng = np.random.default_rng(4)
    imgs = (rng.standard_normal((nch,) + img) + 1j * rng.standard_normal((nch,) + img)).astype(np.complex64)
    xg, res, it = r.cg_sense_images(imgs, 0.0, iters)
    assert it == iters
    Sd = S.astype(np.complex128)
    P = oracle_mod.toeplitz_spectrum(k, img, grid, dcf.astype(np.float64))
    b = (np.conj(Sd) * imgs).sum(0)
    xr = np.zeros(img, np.complex128)
    rv, pv = b.copy(), b.copy()
    rr = np.vdot(rv, rv)
    for _ in range(iters):
        q = oracle_mod.toeplitz_apply(P, img, grid, Sd, pv)
        a = rr / np.vdot(pv, q)
        xr += a * pv
        rv -= a * q
        rn = np.vdot(rv, rv)
        pv = rv + (rn / rr) * pv
        rr = rn
    assert rel_l2(xg, xr) < 1e-4
    assert abs(res[-1] / np.sqrt(rr.real) - 1) < 1e-3


def test_toeplitz_cg_solve(gpu_lib, cgs, synth):
    """Batched CG with the Toeplitz operator on a wave-CAIPI acquisition: the
    residual falls like the gridded solve's, and a graph replay repeats the
    solve bitwise.  (The images differ from the gridded solve's by the
    gridding error amplified by the solve's conditioning: reported by the
    benchmark, not bounded here.)"""
    import torch
    img, grid, nch = (32, 32, 24), (64, 64, 48), 4
    w = synth.scaled(synth.WORKLOADS["cfg1"], img, grid, n_ch=nch, read_os=2)
    k = synth.wave_trajectory(w, synth.WaveParams(2.0, 2.0))
    ns = k.shape[0]
    S = synth.coil_maps(img, nch)
    xt = synth.phantom(img)
    r = cgs.Reco(img, grid, nch, kb_w=KB_W, kb_b=KB_B)
    r.set_trajectory(k)
    rng = np.random.default_rng(2)
    perm = rng.permutation(ns)
    bins = [np.sort(b) for b in np.array_split(perm, 3)]
    r.set_bins(bins)
    r.set_smaps(S)
    # measured data: the library's gridded forward NUFFT of the coil images (all samples)
    one = cgs.Reco(img, grid, nch, kb_w=KB_W, kb_b=KB_B)
    one.set_trajectory(k)
    y = one.nufft_fwd((S * xt[None]).astype(np.complex64))
    yt = torch.from_numpy(y).cuda()
    out = {}
    for mode in (0, 1):
        r.set_toeplitz(mode)
        x = torch.zeros((3,) + img, dtype=torch.complex64, device="cuda")
        res, it = r.cg_sense_batched_tensor(yt, x, 0.0, 12)
        torch.cuda.synchronize()
        out[mode] = (x.cpu().numpy(), res, it)
        if mode == 1:
            x2 = torch.zeros_like(x)
            r.cg_sense_batched_tensor(yt, x2, 0.0, 12)
            torch.cuda.synchronize()
            assert np.array_equal(x2.cpu().numpy(), out[1][0])
    for b in range(3):
        rg, rt = out[0][1][b], out[1][1][b]
        assert rt[-1] < 0.2 * rt[0]
        assert abs(np.log(rt[-1] / rg[-1])) < np.log(3.0)


@pytest.mark.parametrize("img,grid,nch,ns", [
    ((16, 12, 8), (32, 24, 16), 2, 600),
    ((64, 12, 8), (128, 24, 16), 2, 500),
    ((20, 16, 12), (40, 32, 24), 2, 700),    # fine grid 80 x 64 x 48
    ((160, 8, 8), (320, 16, 16), 2, 300),    # 4 x 160 > 512: no fine-grid FFT, Dirichlet product
])
def test_toeplitz_spectrum_methods(gpu_lib, cgs, oracle_mod, img, grid, nch, ns):
    """Spectra through the point-spread function (adjoint NUFFT of D, the
    default) and by the Dirichlet product give the same operator to the
    window error (1e-5 here, FP32 transforms included); both match the exact
    normal operator to 2e-5.  Where the fine grid has no FFT kernels the
    default falls back to the Dirichlet product."""
    k, dcf, S, bins, x = random_case(img, nch, ns, 2, seed=21)
    r = make_reco(cgs, img, grid, nch, k, dcf, S, bins)
    r.set_toeplitz(1)
    psf = max(4 * i for i in img) <= 512
    assert r.toeplitz_spectrum_method() == (1 if psf else 2)
    q0, _ = apply(r, x)
    ms, nbytes = r.toeplitz_stats()
    assert ms > 0 and nbytes == 2 * int(np.prod(grid)) * 4
    r.set_toeplitz_spectrum(1)
    assert r.toeplitz_spectrum_method() == 2
    q1, _ = apply(r, x)
    r.set_toeplitz_spectrum(0)
    q2, _ = apply(r, x)
    # rebuilt the same way: FP64 atomic sums in another order, FP32 rounding apart
    assert rel_l2(q0, q2) < 1e-6
    for b in range(2):
        ref = oracle_mod.exact_normal(k[bins[b]], img, grid, S.astype(np.complex128), dcf[bins[b]].astype(np.float64),
                                      x[b].astype(np.complex128))
        assert rel_l2(q0[b], q1[b]) < 1e-5
        assert rel_l2(q0[b], ref) < 2e-5 and rel_l2(q1[b], ref) < 2e-5
    r.close()
