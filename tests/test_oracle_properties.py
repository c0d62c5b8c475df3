"""Known-answer checks of the oracle that do not depend on the reference:
Bessel I0, the centred FFT against numpy, adjointness of the NUFFT pair, and
the approximation of the exact non-uniform DFT."""
import numpy as np
import pytest

from conftest import rel_l2


def test_bessel_i0(o64):
    sp = pytest.importorskip("scipy.special")
    for x in [0.0, 0.5, 1.0, 3.7, 9.0, 14.9086, 20.0]:
        assert abs(o64.lib.cgso_bessel_i0(x) - sp.i0(x)) <= 1e-14 * sp.i0(x)


@pytest.mark.parametrize("grid", [(8, 6, 4), (24, 20, 16), (10, 14, 22)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_centred_fft_vs_numpy(oracle_mod, o64, grid, sign):
    """Fourier::transformFWD/BWD = (-1)^(sum N/2) fftshift(F(ifftshift(a))) for
    even sizes (the sign alternation before and after the transform equals
    the half-length shifts up to that global sign)."""
    rng = np.random.default_rng(1)
    a = rng.standard_normal(grid) + 1j * rng.standard_normal(grid)
    p = oracle_mod.make_params(grid, grid, 1)
    out = o64.centred_fft(p, a, sign, 0)
    if sign < 0:
        ref = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(a)))
    else:
        ref = np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(a))) * np.prod(grid)
    ref = ref * (-1.0) ** (sum(n // 2 for n in grid))
    assert rel_l2(out, ref) < 1e-13


def _case(oracle_mod, o, img, grid, nch=2, n=400, seed=5):
    rng = np.random.default_rng(seed)
    k = rng.uniform(0.05, 0.95, (n, 3))
    p = oracle_mod.make_params(img, grid, nch)
    taps = o.taps(p, k)
    return p, k, taps


@pytest.mark.parametrize("img,grid", [((16, 16, 16), (16, 16, 16)), ((12, 10, 8), (24, 20, 16))])
def test_adjointness(oracle_mod, o64, img, grid):
    """<E x, y> = <x, E^H y> / c with c = adj_scale / sqrt(N_grid)."""
    p, k, taps = _case(oracle_mod, o64, img, grid)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((2,) + img) + 1j * rng.standard_normal((2,) + img)
    y = rng.standard_normal((2, k.shape[0])) + 1j * rng.standard_normal((2, k.shape[0]))
    kft = o64.kernel_ft(p)
    ex = o64.nufft_fwd(p, taps, kft, x)
    ehy = o64.nufft_adj(p, taps, kft, y)
    c = 1e-3 / np.sqrt(np.prod(grid))
    lhs = np.vdot(ex, y)
    rhs = np.vdot(x, ehy) / c
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("kb_w,kb_b,tol", [
    (4.25, 14.9086, 5e-2),                                      # reference shape (Reco.cpp:378-379)
    (4.25, np.pi * np.sqrt(4.25 ** 2 / 4 * 1.5 ** 2 - 0.8), 2e-3),  # Beatty shape for 2x oversampling
    (4.0, np.pi * np.sqrt(4.0 ** 2 / 4 * 1.5 ** 2 - 0.8), 3e-3),
])
def test_nudft_known_answer(oracle_mod, o64, kb_w, kb_b, tol):
    """With a 2x oversampled grid the KB NUFFT approximates the exact NUDFT
    sum_r x[r] exp(-2 pi i (u - G/2) . (r + lo - G/2) / G), u = k (G - 1).
    The reference's shape parameter b = 14.9086 is tuned for a wider band than
    2x oversampling gives, so its error is about 3 %; the Beatty shape
    pi sqrt(w^2/s^2 (s - 1/2)^2 - 0.8) brings it near 1e-3.  The scale is 1."""
    img, grid = (16, 16, 16), (32, 32, 32)
    rng = np.random.default_rng(5)
    k = rng.uniform(0.1, 0.9, (300, 3))
    p = oracle_mod.make_params(img, grid, 1, kb_w=kb_w, kb_b=kb_b)
    taps = o64.taps(p, k)
    x = rng.standard_normal(img) + 1j * rng.standard_normal(img)
    e = o64.nufft_fwd(p, taps, o64.kernel_ft(p), x[None])[0]
    G = np.array(grid, float)
    lo = (G - np.array(img)) // 2
    u = k * (G - 1) - G / 2
    r = np.stack(np.meshgrid(*[np.arange(n) for n in img], indexing="ij"), -1).reshape(-1, 3) + lo - G / 2
    exact = np.exp(-2j * np.pi * (u / G) @ r.T) @ x.ravel()
    scale = np.vdot(exact, e) / np.vdot(exact, exact)
    assert abs(scale.imag) < 1e-3
    assert abs(scale.real - 1.0) < 5e-2
    assert rel_l2(e, scale.real * exact) < tol


@pytest.mark.parametrize("img,grid", [((16, 12, 8), (32, 24, 16)), ((10, 8, 6), (20, 16, 12))])
def test_toeplitz_embedding_is_exact(oracle_mod, img, grid):
    """The Toeplitz form crop F_c^H (P . F_c pad(.)) with the Dirichlet-kernel
    spectrum equals the exact normal operator s E^H D E (FP64 rounding)."""
    rng = np.random.default_rng(11)
    ns, nch = 300, 2
    k = rng.uniform(0.05, 0.95, (ns, 3))
    dcf = rng.uniform(0.5, 1.5, ns)
    smaps = rng.standard_normal((nch,) + img) + 1j * rng.standard_normal((nch,) + img)
    x = rng.standard_normal(img) + 1j * rng.standard_normal(img)
    P = oracle_mod.toeplitz_spectrum(k, img, grid, dcf)
    q_t = oracle_mod.toeplitz_apply(P, img, grid, smaps, x)
    q_e = oracle_mod.exact_normal(k, img, grid, smaps, dcf, x)
    assert rel_l2(q_t, q_e) < 1e-12


@pytest.mark.parametrize("img,grid", [((6, 5, 4), (12, 10, 8)), ((8, 6, 6), (16, 12, 14))])
def test_toeplitz_spectrum_by_psf_nufft(oracle_mod, img, grid):
    """The spectrum through the point-spread function (adjoint NUFFT of the
    density weights with a Kaiser-Bessel window on a 4x fine grid, the
    library's set-up algorithm) against the Dirichlet-kernel spectrum: the
    window error, below 1e-6 at width 7 and falling about tenfold per unit
    of width."""
    rng = np.random.default_rng(0)
    k = rng.uniform(0.02, 0.98, (200, 3))
    dcf = rng.uniform(0.5, 1.5, 200)
    P = oracle_mod.toeplitz_spectrum(k, img, grid, dcf)
    e6 = rel_l2(oracle_mod.toeplitz_spectrum_nufft(k, img, grid, dcf, W=6.0), P)
    e7 = rel_l2(oracle_mod.toeplitz_spectrum_nufft(k, img, grid, dcf, W=7.0), P)
    assert e7 < 1e-6 and e7 < 0.2 * e6


def test_gridded_normal_operator_vs_exact(oracle_mod, o64):
    """The gridded E^H D E (KB width 4, 2x oversampling, the Beatty shape)
    approximates the exact normal operator to its gridding error."""
    img, grid = (16, 12, 8), (32, 24, 16)
    rng = np.random.default_rng(5)
    ns, nch = 500, 2
    k = rng.uniform(0.1, 0.9, (ns, 3))
    w = 4.0
    p = oracle_mod.make_params(img, grid, nch, kb_w=w, kb_b=np.pi * np.sqrt(w ** 2 / 4 * 1.5 ** 2 - 0.8))
    taps = o64.taps(p, k)
    smaps = rng.standard_normal((nch,) + img) + 1j * rng.standard_normal((nch,) + img)
    dcf = rng.uniform(0.5, 1.5, ns).astype(np.float32)
    x = rng.standard_normal(img) + 1j * rng.standard_normal(img)
    q_g = o64.apply_ehde(p, taps, o64.kernel_ft(p), smaps, dcf, x)
    q_e = oracle_mod.exact_normal(k, img, grid, smaps, dcf.astype(np.float64), x)
    err = rel_l2(q_g, q_e)
    assert 1e-5 < err < 5e-3


def test_pipe_menon_restatement_known_answers(oracle_mod, o64):
    """The FP64 Pipe-Menon restatement: on a uniform lattice the interior
    weights are equal; a lattice twice as dense on one side gets half the
    weight there; w / (A A^T w) = 1 holds at the fixed point (interior)."""
    grid = (48, 24, 24)
    xs = np.concatenate([np.arange(6.0, 24.0, 1.0), np.arange(24.0, 42.0, 0.5)])
    X, Y, Z = np.meshgrid(xs, np.arange(6.0, 18.0), np.arange(6.0, 18.0), indexing="ij")
    k = np.stack([X, Y, Z], -1).reshape(-1, 3) / (np.array(grid) - 1)
    p = oracle_mod.make_params(grid, grid, 1)
    taps = o64.taps(p, k)
    w = oracle_mod.pipe_menon(taps, int(np.prod(grid)), 40).reshape(X.shape)
    assert abs(w.max() - 1.0) < 1e-12 and w.min() > 0
    inner = (np.abs(Y - 12) < 3) & (np.abs(Z - 12) < 3)
    sparse, dense = inner & (X > 10) & (X < 20), inner & (X > 28) & (X < 38)
    assert np.ptp(w[sparse]) / np.median(w[sparse]) < 3e-2
    assert abs(np.median(w[sparse]) / np.median(w[dense]) - 2.0) < 0.05
    # fixed point: one more iteration changes the interior weights little
    w2 = oracle_mod.pipe_menon(taps, int(np.prod(grid)), 41).reshape(X.shape)
    assert np.abs(w2[sparse] / w[sparse] - 1).max() < 1e-2
    # bins iterate independently
    half = np.arange(k.shape[0] // 2)
    wb = oracle_mod.pipe_menon(taps, int(np.prod(grid)), 10, bins=[half, np.arange(k.shape[0] // 2, k.shape[0])])
    wh = oracle_mod.pipe_menon(o64.taps(p, k[half]), int(np.prod(grid)), 10)
    assert np.allclose(wb[half], wh, rtol=1e-12, atol=0)
