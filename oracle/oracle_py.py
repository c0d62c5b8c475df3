"""ctypes bindings of the CPU oracle (cgs_oracle.c) and a runner for the
reference driver (ref_driver.cpp).

TEST INFRASTRUCTURE.  Imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker.  The product package never
imports this module.

``Oracle(precision=64)`` loads liboracle64.so (the FP64 oracle);
``Oracle(precision=32)`` loads liboracle32.so (the FP32 restatement of the
reference's arithmetic, used as the timed CPU port).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

KB_W = 4.25          # Reco.cpp:379
KB_B = 14.9086       # Reco.cpp:378
KB_ORDER = 5         # Reco.cpp:380
KB_THRESH = 1e-7     # Reco.cpp:717
ADJ_SCALE = 1e-3     # Reco.cpp:482


def build():
    """Compile liboracle{64,32}.so (and the reference driver when the
    reference sources are present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)   # skipped without the reference sources


class Params(C.Structure):
    _fields_ = [
        ("img", C.c_int32 * 3),
        ("grid", C.c_int32 * 3),
        ("n_ch", C.c_int32),
        ("kb_order", C.c_int32),
        ("kb_w", C.c_float),
        ("kb_b", C.c_float),
        ("kb_thresh", C.c_double),
        ("adj_scale", C.c_double),
        ("offcenter", C.c_int32 * 3),
    ]


class Wave(C.Structure):
    _fields_ = [
        ("sx", C.c_int32), ("sy", C.c_int32), ("sz", C.c_int32),
        ("gx", C.c_int32), ("gy", C.c_int32), ("gz", C.c_int32),
        ("fov_y", C.c_double), ("fov_z", C.c_double),
        ("n_osc", C.c_int32),
        ("grad_amp", C.c_double),
        ("amp_corr_y", C.c_double), ("amp_corr_z", C.c_double),
        ("shift_y", C.c_double), ("shift_z", C.c_double),
        ("dwell", C.c_double),
    ]


def make_params(img, grid, n_ch, kb_w=KB_W, kb_b=KB_B, kb_order=KB_ORDER,
                kb_thresh=KB_THRESH, adj_scale=ADJ_SCALE, offcenter=(0, 0, 0)):
    p = Params()
    p.img[:] = list(img)
    p.grid[:] = list(grid)
    p.n_ch = n_ch
    p.kb_order = kb_order
    p.kb_w = kb_w
    p.kb_b = kb_b
    p.kb_thresh = kb_thresh
    p.adj_scale = adj_scale
    p.offcenter[:] = list(offcenter)
    return p


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Taps:
    """CSR tap lists (ptr[ns+1], idx[T], w[T])."""

    def __init__(self, ptr, idx, w):
        self.ptr, self.idx, self.w = ptr, idx, w


class Oracle:
    def __init__(self, precision=64):
        path = os.path.join(BUILD, "liboracle%d.so" % precision)
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path)
        self.real = np.float64 if precision == 64 else np.float32
        self.cplx = np.complex128 if precision == 64 else np.complex64
        L = self.lib
        vp, i64 = C.c_void_p, C.c_int64
        L.cgso_bessel_i0.restype = C.c_double
        L.cgso_bessel_i0.argtypes = [C.c_double]
        L.cgso_conv_function.restype = C.c_float
        L.cgso_conv_function.argtypes = [vp, vp]
        L.cgso_tap_counts.restype = i64
        L.cgso_tap_counts.argtypes = [vp, vp, i64, vp, vp]
        L.cgso_taps_fill.restype = None
        L.cgso_taps_fill.argtypes = [vp, vp, i64, vp, vp, vp, vp]
        L.cgso_kernel_ft.argtypes = [vp, vp]
        L.cgso_centred_fft.argtypes = [vp, vp, C.c_int, C.c_int]
        L.cgso_nufft_fwd.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp]
        L.cgso_nufft_adj.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp]
        L.cgso_apply_ehde.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp, vp, vp]
        L.cgso_cg_sense.restype = C.c_int
        L.cgso_cg_sense.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp, vp, C.c_double, C.c_int,
                                    vp, vp, vp]
        L.cgso_wave_caipi.argtypes = [vp, vp]
        L.cgso_loss_grad.restype = C.c_double
        L.cgso_loss_grad.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp, vp, vp]
        L.cgso_bessel_i1.restype = C.c_double
        L.cgso_bessel_i1.argtypes = [C.c_double]

    # -- kernel ------------------------------------------------------------
    def taps(self, p, k, mask=None):
        k = np.ascontiguousarray(k, dtype=np.float64)
        ns = k.shape[0]
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        counts = np.zeros(ns, np.int32)
        self.lib.cgso_tap_counts(C.byref(p), _ptr(k), ns, _ptr(m), _ptr(counts))
        ptr = np.zeros(ns + 1, np.int64)
        np.cumsum(counts, out=ptr[1:])
        idx = np.zeros(int(ptr[-1]), np.int32)
        w = np.zeros(int(ptr[-1]), np.float32)
        self.lib.cgso_taps_fill(C.byref(p), _ptr(k), ns, _ptr(m), _ptr(ptr), _ptr(idx), _ptr(w))
        return Taps(ptr, idx, w)

    def kernel_ft(self, p):
        out = np.zeros(tuple(p.grid), self.cplx)
        self.lib.cgso_kernel_ft(C.byref(p), _ptr(out))
        return out

    def centred_fft(self, p, a, sign, rescale):
        a = np.ascontiguousarray(a, dtype=self.cplx).copy()
        self.lib.cgso_centred_fft(C.byref(p), _ptr(a), sign, int(rescale))
        return a

    # -- operators ---------------------------------------------------------
    def nufft_fwd(self, p, taps, kft, img):
        ns = taps.ptr.shape[0] - 1
        img = np.ascontiguousarray(img, dtype=self.cplx)
        kft = np.ascontiguousarray(kft, dtype=self.cplx)
        data = np.zeros((p.n_ch, ns), self.cplx)
        self.lib.cgso_nufft_fwd(C.byref(p), _ptr(taps.ptr), _ptr(taps.idx), _ptr(taps.w), ns,
                                _ptr(kft), _ptr(img), _ptr(data))
        return data

    def nufft_adj(self, p, taps, kft, data):
        ns = taps.ptr.shape[0] - 1
        data = np.ascontiguousarray(data, dtype=self.cplx)
        kft = np.ascontiguousarray(kft, dtype=self.cplx)
        img = np.zeros((p.n_ch,) + tuple(p.img), self.cplx)
        self.lib.cgso_nufft_adj(C.byref(p), _ptr(taps.ptr), _ptr(taps.idx), _ptr(taps.w), ns,
                                _ptr(kft), _ptr(data), _ptr(img))
        return img

    def apply_ehde(self, p, taps, kft, smaps, dcf, x):
        ns = taps.ptr.shape[0] - 1
        smaps = np.ascontiguousarray(smaps, dtype=self.cplx)
        kft = np.ascontiguousarray(kft, dtype=self.cplx)
        x = np.ascontiguousarray(x, dtype=self.cplx)
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float32)
        q = np.zeros(tuple(p.img), self.cplx)
        self.lib.cgso_apply_ehde(C.byref(p), _ptr(taps.ptr), _ptr(taps.idx), _ptr(taps.w), ns,
                                 _ptr(kft), _ptr(smaps), _ptr(d), _ptr(x), _ptr(q))
        return q

    def cg_sense(self, p, taps, kft, smaps, dcf, data, threshold, max_iter=16):
        ns = taps.ptr.shape[0] - 1
        smaps = np.ascontiguousarray(smaps, dtype=self.cplx)
        kft = np.ascontiguousarray(kft, dtype=self.cplx)
        data = np.ascontiguousarray(data, dtype=self.cplx)
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float32)
        x = np.zeros(tuple(p.img), self.cplx)
        res = np.zeros(max(max_iter, 1), np.float64)
        it = np.zeros(1, np.int32)
        st = self.lib.cgso_cg_sense(C.byref(p), _ptr(taps.ptr), _ptr(taps.idx), _ptr(taps.w), ns,
                                    _ptr(kft), _ptr(smaps), _ptr(d), _ptr(data), threshold,
                                    max_iter, _ptr(x), _ptr(res), _ptr(it))
        return st, x, res[: it[0]], int(it[0])

    def loss_grad(self, p, k, kft, smaps, dcf, x, y, want_x=True, want_k=True):
        """Data-consistency loss 1/2 sum D |E S x - y|^2 and its gradients
        (x: complex image, k: [ns][3]); returns (L, grad_x, grad_k)."""
        k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
        ns = k.shape[0]
        smaps = np.ascontiguousarray(smaps, dtype=self.cplx)
        kft = np.ascontiguousarray(kft, dtype=self.cplx)
        x = np.ascontiguousarray(x, dtype=self.cplx)
        y = np.ascontiguousarray(y, dtype=self.cplx)
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float32)
        gx = np.zeros(tuple(p.img), self.cplx) if want_x else None
        gk = np.zeros((ns, 3), np.float64) if want_k else None
        L = self.lib.cgso_loss_grad(C.byref(p), _ptr(k), ns, _ptr(kft), _ptr(smaps), _ptr(d), _ptr(x),
                                    _ptr(y), _ptr(gx), _ptr(gk))
        return L, gx, gk

    def wave_caipi(self, **kw):
        w = Wave()
        for name, _ in Wave._fields_:
            setattr(w, name, kw[name])
        n = w.sx * w.sy * w.sz
        out = np.zeros((n, 3), np.float64)
        self.lib.cgso_wave_caipi(C.byref(w), _ptr(out))
        return out


# ---------------------------------------------------------------------------
# Iterative density weights (Pipe and Menon, Magn. Reson. Med. 41:179-186,
# 1999), FP64: the documented alternative to the Voronoi volumes of
# estimateDensityV3D (functions.h:161-258).  With A the interpolation matrix
# of the taps (Reco.cpp:698-806; rows = samples), w <- w / (A A^T w): spread
# the weights onto the grid, interpolate back, divide.  Samples without taps
# get 0.  Each bin iterates on its own samples and is normalised by its
# maximum.
# ---------------------------------------------------------------------------

def pipe_menon(taps, n_grid, iters, bins=None):
    """taps: Taps of all samples (one grid, CSR); bins: list of sample index
    arrays (None: one bin of every sample).  Returns float64 [ns]."""
    ptr, idx, wt = taps.ptr, taps.idx.astype(np.int64), taps.w.astype(np.float64)
    ns = ptr.shape[0] - 1
    cnt = np.diff(ptr)
    out = np.zeros(ns, np.float64)
    for sel in ([np.arange(ns)] if bins is None else bins):
        sel = np.asarray(sel, np.int64)
        m = np.zeros(ns, bool)
        m[sel] = True
        tap_in = np.repeat(m, cnt)                      # taps of this bin's samples
        owner = np.repeat(np.arange(ns), cnt)[tap_in]
        ti, tw = idx[tap_in], wt[tap_in]
        w = np.where(m, 1.0, 0.0)
        for _ in range(iters):
            grid = np.bincount(ti, weights=tw * w[owner], minlength=n_grid)
            u = np.bincount(owner, weights=tw * grid[ti], minlength=ns)
            w = np.where(m & (u > 0), w / np.where(u > 0, u, 1.0), 0.0)
        mx = w[sel].max() if sel.size else 0.0
        out[sel] = w[sel] / mx if mx > 0 else 0.0
    return out


# ---------------------------------------------------------------------------
# Exact normal operator (numpy, FP64): the operator that the Toeplitz
# embedding computes and that the gridded operator approximates.  Small
# problems only (a dense samples x voxels matrix).
# ---------------------------------------------------------------------------

def sample_frequencies(k, grid):
    """nu = (k (G - 1) - G/2) / G per axis: the cycles per grid cell of each
    sample in the exact non-uniform DFT that the gridded forward operator
    approximates, exp(-2 pi i nu . (r + lo - G/2)) (k in [0, 1] maps to grid
    coordinate k (G - 1), Reco.cpp:698-806; the FFT centre is G/2,
    Fourier.cpp:19-42)."""
    G = np.asarray(grid, np.float64)
    return (np.asarray(k, np.float64) * (G - 1) - G / 2) / G


def exact_normal(k, img, grid, smaps, dcf, x, adj_scale=ADJ_SCALE):
    """q = s sum_c conj(S_c) E^H D E (S_c x) with E the exact non-uniform DFT
    and s = adj_scale / sqrt(N_grid), the adjoint scale of the gridded
    operator (Reco.cpp:482, Fourier.cpp:34)."""
    nu = sample_frequencies(k, grid)
    r = np.stack(np.meshgrid(*[np.arange(n) for n in img], indexing="ij"), -1).reshape(-1, 3)
    E = np.exp(-2j * np.pi * (nu @ r.T))
    d = np.ones(nu.shape[0]) if dcf is None else np.asarray(dcf, np.float64)
    s = adj_scale / np.sqrt(np.prod(grid))
    q = np.zeros(tuple(img), np.complex128)
    for c in range(smaps.shape[0]):
        v = (smaps[c] * x).ravel()
        q += np.conj(smaps[c]) * (s * (E.conj().T @ (d * (E @ v)))).reshape(img)
    return q


def toeplitz_spectrum(k, img, grid, dcf, adj_scale=ADJ_SCALE):
    """Real spectrum P on the grid such that crop F_c^H (P . F_c pad(.)) is
    s E^H D E, F_c the centred unscaled transform: per axis the Dirichlet
    kernel K(psi) = sum_{|d| < I} exp(2 pi i psi d) at psi = nu - k/G + 1/2,
    P = s / N_grid sum_i D_i Kx Ky Kz."""
    nu = sample_frequencies(k, grid)
    d = np.ones(nu.shape[0]) if dcf is None else np.asarray(dcf, np.float64)
    K = []
    for a in range(3):
        e = nu[:, a:a + 1] - np.arange(grid[a])[None, :] / grid[a] + 0.5
        e = e - np.floor(e + 0.5)
        m = 2 * img[a] - 1
        with np.errstate(invalid="ignore", divide="ignore"):
            v = np.sin(m * np.pi * e) / np.sin(np.pi * e)
        v[e == 0.0] = m
        K.append(v)
    s = adj_scale / np.sqrt(np.prod(grid))
    return np.einsum("i,ia,ib,ic->abc", d, K[0], K[1], K[2]) * (s / np.prod(grid))


def kb_window(x, W, beta):
    """Kaiser-Bessel window I0(beta sqrt(1 - (2x/W)^2)) on |x| <= W/2, 0 outside."""
    x = np.asarray(x, np.float64)
    t = 1.0 - (2.0 * x / W) ** 2
    return np.where(t >= 0.0, np.i0(beta * np.sqrt(np.clip(t, 0.0, None))), 0.0)


def kb_window_ft(xi, W, beta):
    """Continuous Fourier transform of kb_window at frequency xi (cycles per
    unit): W sinh(sqrt(beta^2 - (pi W xi)^2)) / sqrt(beta^2 - (pi W xi)^2)."""
    z = beta ** 2 - (np.pi * W * np.asarray(xi, np.float64)) ** 2
    r = np.sqrt(np.abs(z))
    with np.errstate(invalid="ignore", divide="ignore"):
        v = np.where(z > 0, np.sinh(r) / r, np.sin(r) / r)
    return W * np.where(r == 0.0, 1.0, v)


def toeplitz_spectrum_nufft(k, img, grid, dcf, adj_scale=ADJ_SCALE, W=7.0, fine=None):
    """The spectrum of toeplitz_spectrum through the point-spread function
    h(d) = sum_i D_i exp(2 pi i nu_i . d), |d_a| < I_a, computed by an adjoint
    (type-1) NUFFT, as the library's set-up does it: D spread with a
    Kaiser-Bessel window of width W onto a 2x oversampled fine grid of
    n_a = 4 I_a points (sample position n nu + n/2, periodic), the centred
    transform (sign +1) of the fine grid, division by the window's Fourier
    transform, then h placed at d + G/2 of the grid and the centred
    transform (sign -1): P = s/N_grid (-1)^(sum G/2) Re(...).  FP64, small
    problems only (a Python loop over samples)."""
    nu = sample_frequencies(k, grid)
    M = nu.shape[0]
    d = np.ones(M) if dcf is None else np.asarray(dcf, np.float64)
    n = [4 * i for i in img] if fine is None else list(fine)
    beta = np.pi * np.sqrt(W * W / 4.0 * 1.5 ** 2 - 0.8)
    b = np.zeros(n)
    for i in range(M):
        idx, wts = [], []
        for a in range(3):
            u = n[a] * nu[i, a] + n[a] / 2.0
            g = np.arange(int(np.ceil(u - W / 2.0)), int(np.floor(u + W / 2.0)) + 1)
            idx.append(np.mod(g, n[a]))
            wts.append(kb_window(g - u, W, beta))
        np.add.at(b, np.ix_(*idx), d[i] * np.einsum("a,b,c->abc", *wts))
    L = centred_fft_np(b, +1)
    box = []
    deap = []
    for a in range(3):
        dd = np.arange(-(img[a] - 1), img[a])
        box.append(dd + n[a] // 2)
        deap.append(kb_window_ft(dd / n[a], W, beta))
    h = L[np.ix_(*box)] / np.einsum("a,b,c->abc", *deap)
    h *= (-1.0) ** sum(v // 2 for v in n)
    buf = np.zeros(tuple(grid), np.complex128)
    buf[np.ix_(*[np.arange(-(img[a] - 1), img[a]) + grid[a] // 2 for a in range(3)])] = h
    L2 = centred_fft_np(buf, -1)
    s = adj_scale / np.sqrt(np.prod(grid))
    return (L2.real * ((-1.0) ** sum(g // 2 for g in grid))) * (s / np.prod(grid))


def centred_fft_np(a, sign):
    """Fourier::transformFWD (sign -1) / transformBWD (+1) without scaling:
    (-1)^n before and (-1)^k after an unnormalised transform on each axis."""
    out = np.asarray(a, np.complex128)
    for ax in range(out.ndim):
        n = out.shape[ax]
        shp = [1] * out.ndim
        shp[ax] = n
        sg = ((-1.0) ** np.arange(n)).reshape(shp)
        out = out * sg
        out = np.fft.fft(out, axis=ax) if sign < 0 else np.fft.ifft(out, axis=ax) * n
        out = out * sg
    return out


def toeplitz_apply(P, img, grid, smaps, x):
    """q = sum_c conj(S_c) crop F_c^H (P . F_c pad(S_c x)), the image centred
    in the grid at lo = (G - I) / 2."""
    lo = [(g - i) // 2 for g, i in zip(grid, img)]
    box = tuple(slice(l, l + i) for l, i in zip(lo, img))
    q = np.zeros(tuple(img), np.complex128)
    for c in range(smaps.shape[0]):
        pad = np.zeros(tuple(grid), np.complex128)
        pad[box] = smaps[c] * x
        q += np.conj(smaps[c]) * centred_fft_np(P * centred_fft_np(pad, -1), +1)[box]
    return q


# ---------------------------------------------------------------------------
# Reference driver runner (only where the reference sources were compiled)
# ---------------------------------------------------------------------------

def ref_available():
    return os.path.exists(REF_DRIVER)


def run_ref(mode, params, arrays, outputs, workdir=None):
    """Run oracle/_ref/ref_driver <mode> on a temp dir.

    params: dict written to params.txt; arrays: {name: ndarray} written as
    <name>.bin; outputs: {name: (dtype, count or None)} read back from
    <name>.bin.  Returns {name: ndarray}.
    """
    own = workdir is None
    d = tempfile.mkdtemp(prefix="cgsref_") if own else workdir
    with open(os.path.join(d, "params.txt"), "w") as f:
        for k, v in params.items():
            f.write("%s %s\n" % (k, repr(v) if isinstance(v, float) else v))
    for name, a in arrays.items():
        np.ascontiguousarray(a).tofile(os.path.join(d, name + ".bin"))
    subprocess.run([REF_DRIVER, mode, d], check=True, stdout=subprocess.DEVNULL)
    out = {}
    for name, (dt, cnt) in outputs.items():
        out[name] = np.fromfile(os.path.join(d, name + ".bin"), dtype=dt,
                                count=-1 if cnt is None else cnt)
    if own:
        import shutil
        shutil.rmtree(d, ignore_errors=True)
    return out
