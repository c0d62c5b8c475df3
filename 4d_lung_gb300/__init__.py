"""GB300-native CG-SENSE (expRad/4d_lung hot path): Python bindings.

The compute path is the in-tree CUDA library ``libcgsense.so`` (sm_103a
kernels behind the C ABI of ``include/cgsense_c.h``).  This module is a thin
ctypes layer over it; there is no CPU fallback: importing works anywhere, but
every compute call raises when the library or a GPU is missing.

The class :class:`Reco` mirrors the reference's ``Reco`` reconstruction
object (CGSense/Reco.h:13-214) for the operator and solver path:

    reco = Reco(img=(64,)*3, grid=(128,)*3, n_ch=8)
    reco.set_trajectory(k)             # Reco::setTrajectory + calculateWeights
    reco.set_dcf(d)                    # Reco::denCorr (Density::IMPORT)
    reco.set_smaps(maps)               # Reco::sMaps
    data = reco.nufft_fwd(coil_imgs)   # Reco::nufftFWD
    imgs = reco.nufft_adj(data)        # Reco::nufftBWD
    x, res, it = reco.cg_sense(data, threshold, max_iter=16)   # Reco::cgSenseDynamic
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcgsense.so")

CGS_OK = 0
CGS_ERR_ARG = 1
CGS_ERR_CUDA = 2
CGS_ERR_NONFINITE = 3
CGS_ERR_STATE = 4
CGS_ERR_NOMEM = 5
CGS_ERR_UNSUPPORTED = 6
CGS_ERR_NO_THRESHOLD = 7
CGS_ERR_TIMEOUT = 8

_ERR_NAMES = {
    1: "CGS_ERR_ARG", 2: "CGS_ERR_CUDA", 3: "CGS_ERR_NONFINITE", 4: "CGS_ERR_STATE",
    5: "CGS_ERR_NOMEM", 6: "CGS_ERR_UNSUPPORTED", 7: "CGS_ERR_NO_THRESHOLD", 8: "CGS_ERR_TIMEOUT",
}

# Every symbol declared in include/cgsense_c.h.
EXPORTS = [
    "cgs_default_params", "cgs_create", "cgs_destroy", "cgs_last_error", "cgs_set_stream",
    "cgs_sync", "cgs_wave_caipi", "cgs_set_trajectory", "cgs_set_mask", "cgs_mask_from_data",
    "cgs_set_bins", "cgs_num_bins", "cgs_set_dcf", "cgs_set_smaps", "cgs_set_smaps_d",
    "cgs_kernel_ft", "cgs_fft3", "cgs_fft3_d", "cgs_nufft_fwd", "cgs_nufft_fwd_d",
    "cgs_nufft_adj", "cgs_nufft_adj_d", "cgs_apply_ehde", "cgs_apply_ehde_d", "cgs_cg_solve",
    "cgs_cg_solve_batched", "cgs_cg_solve_batched_d", "cgs_last_launch_count",
    "cgs_profile_apply", "cgs_cg_solve_images", "cgs_alloc_host", "cgs_free_host",
    "cgs_fft3_noalloc", "cgs_cg_solve_plain_d", "cgs_voronoi_dcf", "cgs_cg_solve_trace_d",
    "cgs_cg_solve_fp64_d", "cgs_estimate_density_v3d", "cgs_loss_grad_d", "cgs_loss_grad_fp64_d",
    "cgs_update_trajectory_d", "cgs_set_precision", "cgs_autotune", "cgs_rhs_d", "cgs_apply_vjp_k_d",
    "cgs_rhs_vjp_k_d", "cgs_trajectory_serial", "cgs_get_stream", "cgs_import_data_bin", "cgs_permute_samples_d",
    "cgs_export_complex_bin", "cgs_export_float_bin", "cgs_import_smaps_bin", "cgs_import_density_bin", "cgs_rss_d",
    "cgs_reconstruct_states", "cgs_pipe_menon_dcf", "cgs_set_deterministic", "cgs_set_launch_shape",
    "cgs_set_support_pruning", "cgs_support_stats", "cgs_spread_matrix_stats", "cgs_spread_fused", "cgs_estimate_smaps_d",
    "cgs_forward_y_listed_rows", "cgs_set_toeplitz", "cgs_toeplitz_stats", "cgs_setup_stats", "cgs_e2e_stats", "cgs_set_toeplitz_spectrum", "cgs_toeplitz_spectrum_method",
]

# Stage names of cgs_profile_apply, in launch order (one group of bins).
STAGES = ["fwd_z", "fwd_y", "fwd_x", "interp", "spread", "adj_x", "adj_y", "adj_z"]


class CGSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERR_NAMES.get(code, "CGS_ERR"), code, msg))
        self.code = code


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
        ("device", C.c_int32),
        ("workspace_bytes", C.c_int64),
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


_lib = None


def build():
    """Compile libcgsense.so in place (nvcc, sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_cgs_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """Load libcgsense.so (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libcgsense.so is not built: run __graft_entry__.build() "
                           "or python 4d_lung_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "cgs_default_params": (None, [vp]),
        "cgs_create": (C.c_int, [vp, vp]),
        "cgs_destroy": (None, [vp]),
        "cgs_last_error": (C.c_char_p, [vp]),
        "cgs_set_stream": (C.c_int, [vp, vp]),
        "cgs_sync": (C.c_int, [vp]),
        "cgs_wave_caipi": (C.c_int, [vp, vp]),
        "cgs_set_trajectory": (C.c_int, [vp, vp, i64]),
        "cgs_set_mask": (C.c_int, [vp, vp]),
        "cgs_mask_from_data": (C.c_int, [vp, vp]),
        "cgs_set_bins": (C.c_int, [vp, i32, vp, vp]),
        "cgs_num_bins": (C.c_int, [vp]),
        "cgs_set_dcf": (C.c_int, [vp, vp]),
        "cgs_set_smaps": (C.c_int, [vp, vp]),
        "cgs_set_smaps_d": (C.c_int, [vp, vp]),
        "cgs_kernel_ft": (C.c_int, [vp, vp]),
        "cgs_fft3": (C.c_int, [vp, vp, i32, i32]),
        "cgs_fft3_d": (C.c_int, [vp, vp, i32, i32]),
        "cgs_nufft_fwd": (C.c_int, [vp, vp, vp]),
        "cgs_nufft_fwd_d": (C.c_int, [vp, vp, vp]),
        "cgs_nufft_adj": (C.c_int, [vp, vp, vp]),
        "cgs_nufft_adj_d": (C.c_int, [vp, vp, vp]),
        "cgs_apply_ehde": (C.c_int, [vp, i32, vp, vp]),
        "cgs_apply_ehde_d": (C.c_int, [vp, i32, i32, vp, vp]),
        "cgs_cg_solve": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp]),
        "cgs_cg_solve_batched": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp]),
        "cgs_cg_solve_batched_d": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp]),
        "cgs_last_launch_count": (i64, [vp]),
        "cgs_profile_apply": (C.c_int, [vp, i32, i32, vp, vp, vp, i32, vp]),
        "cgs_cg_solve_images": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp]),
        "cgs_alloc_host": (vp, [C.c_size_t]),
        "cgs_free_host": (None, [vp]),
        "cgs_fft3_noalloc": (C.c_int, [vp, vp, vp, i32, vp]),
        "cgs_cg_solve_plain_d": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp]),
        "cgs_voronoi_dcf": (C.c_int, [vp, i64, vp]),
        "cgs_estimate_density_v3d": (C.c_int, [vp, i64, C.c_int32, C.c_int32, C.c_double, vp]),
        "cgs_loss_grad_d": (C.c_int, [vp, C.c_int32, vp, vp, vp, vp, vp]),
        "cgs_loss_grad_fp64_d": (C.c_int, [vp, C.c_int32, vp, vp, vp, vp, vp]),
        "cgs_update_trajectory_d": (C.c_int, [vp, vp]),
        "cgs_set_precision": (C.c_int, [vp, C.c_int32]),
        "cgs_autotune": (C.c_int, [vp, vp, C.c_int32, vp, vp, vp, vp]),
        "cgs_rhs_d": (C.c_int, [vp, C.c_int32, C.c_int32, vp, vp]),
        "cgs_apply_vjp_k_d": (C.c_int, [vp, C.c_int32, C.c_int32, vp, vp, vp]),
        "cgs_rhs_vjp_k_d": (C.c_int, [vp, C.c_int32, C.c_int32, vp, vp, vp]),
        "cgs_trajectory_serial": (C.c_uint64, [vp]),
        "cgs_get_stream": (C.c_void_p, [vp]),
        "cgs_import_data_bin": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp, vp]),
        "cgs_permute_samples_d": (C.c_int, [vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp]),
        "cgs_export_complex_bin": (C.c_int, [C.c_char_p, vp, i64, C.c_int32, vp]),
        "cgs_export_float_bin": (C.c_int, [C.c_char_p, vp, i64, C.c_int32, vp]),
        "cgs_import_smaps_bin": (C.c_int, [C.c_char_p, i64, C.c_int32, vp]),
        "cgs_import_density_bin": (C.c_int, [C.c_char_p, i64, vp]),
        "cgs_rss_d": (C.c_int, [vp, C.c_int32, i64, vp, vp]),
        "cgs_pipe_menon_dcf": (C.c_int, [vp, C.c_int32, vp, C.c_int32]),
        "cgs_set_deterministic": (C.c_int, [vp, C.c_int32]),
        "cgs_set_launch_shape": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32]),
        "cgs_set_support_pruning": (C.c_int, [vp, C.c_int32]),
        "cgs_support_stats": (C.c_int, [vp, vp, vp]),
        "cgs_spread_matrix_stats": (C.c_int, [vp, vp, vp]),
        "cgs_spread_fused": (C.c_int, [vp, vp]),
        "cgs_forward_y_listed_rows": (C.c_int, [vp, vp]),
        "cgs_set_toeplitz": (C.c_int, [vp, C.c_int32]),
        "cgs_toeplitz_stats": (C.c_int, [vp, vp, vp]),
        "cgs_setup_stats": (C.c_int, [vp, vp, C.c_int32]),
        "cgs_e2e_stats": (C.c_int, [vp, vp, vp]),
        "cgs_set_toeplitz_spectrum": (C.c_int, [vp, C.c_int32]),
        "cgs_toeplitz_spectrum_method": (C.c_int, [vp]),
        "cgs_estimate_smaps_d": (C.c_int, [vp, vp, C.c_double, C.c_double, vp]),
        "cgs_reconstruct_states": (C.c_int, [vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_char_p,
                                             C.c_double, C.c_int32, C.c_int32, vp]),
        "cgs_cg_solve_trace_d": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp, vp]),
        "cgs_cg_solve_fp64_d": (C.c_int, [vp, vp, vp, dbl, i32, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def default_params():
    p = Params()
    lib().cgs_default_params(C.byref(p))
    return p


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.complex64)
    if shape is not None and a.size != int(np.prod(shape)):
        raise ValueError("expected %s complex values, got %d" % (shape, a.size))
    return a


def wave_caipi(sx, sy, sz, grid, fov_y, fov_z, n_osc=4, grad_amp=0.006, amp_corr_y=0.998,
               amp_corr_z=1.01, shift_y=5.6e-6, shift_z=6.5e-6, dwell=6.3e-6):
    """WaveCaipi::calculateTraj (Trajectory.cpp:18-184); defaults from CGSense.cpp:51-59."""
    w = Wave(sx, sy, sz, grid[0], grid[1], grid[2], fov_y, fov_z, n_osc, grad_amp, amp_corr_y,
             amp_corr_z, shift_y, shift_z, dwell)
    out = np.zeros((sx * sy * sz, 3), np.float64)
    st = lib().cgs_wave_caipi(C.byref(w), _p(out))
    if st != CGS_OK:
        raise CGSError(st, "invalid wave-CAIPI parameters")
    return out


def voronoi_dcf(k):
    """estimateDensityV3D (functions.h:161-258): normalised Voronoi volumes,
    0 on the convex hull."""
    k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(k.shape[0], np.float32)
    st = lib().cgs_voronoi_dcf(_p(k), k.shape[0], _p(out))
    if st != CGS_OK:
        raise CGSError(st, "cgs_voronoi_dcf failed")
    return out


def estimate_density_v3d(k, sX, average=False, cutoff=1.0):
    """estimateDensityV3D with its readout averaging (functions.h:212-232):
    k holds whole readouts of sX samples each (readout-major order)."""
    k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(k.shape[0], np.float32)
    st = lib().cgs_estimate_density_v3d(_p(k), k.shape[0], int(sX), int(bool(average)), float(cutoff), _p(out))
    if st != CGS_OK:
        raise CGSError(st, "cgs_estimate_density_v3d failed")
    return out


# -- file IO (IO.cpp) ---------------------------------------------------------

def _io_check(st, what):
    if st != CGS_OK:
        raise CGSError(st, what + " failed")


def import_smaps_bin(dirpath, n, nch):
    """IO::importSensitivityMaps: dirpath + "map<c>.bin" -> complex64 [nch][n]."""
    out = np.zeros((nch, n), np.complex64)
    d = dirpath if dirpath.endswith("/") else dirpath + "/"
    _io_check(lib().cgs_import_smaps_bin(d.encode(), n, nch, _p(out)), "cgs_import_smaps_bin")
    return out


def import_density_bin(path, n):
    """IO::importDensityCorr: n float32 weights."""
    out = np.zeros(n, np.float32)
    _io_check(lib().cgs_import_density_bin(path.encode(), n, _p(out)), "cgs_import_density_bin")
    return out


def export_complex_bin(path, a):
    """IO::exportFFTWComplexBin from a host array (complex64)."""
    a = np.ascontiguousarray(a, dtype=np.complex64)
    _io_check(lib().cgs_export_complex_bin(path.encode(), _p(a), a.size, 0, None), "cgs_export_complex_bin")


def export_float_bin(path, a):
    """IO::exportVectorBin from a host array (float32)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    _io_check(lib().cgs_export_float_bin(path.encode(), _p(a), a.size, 0, None), "cgs_export_float_bin")


def import_data_bin_tensor(path, sx, sy, sz, nch, out, stream=None):
    """IO::importDataBin onto the device (out: complex64 CUDA tensor [nch][sx*sy*sz])."""
    _io_check(lib().cgs_import_data_bin(path.encode(), sx, sy, sz, nch, C.c_void_p(out.data_ptr()),
                                        None if stream is None else C.c_void_p(stream)), "cgs_import_data_bin")


def rss_tensor(imgs, out, stream=None):
    """rssq2DVecImg on the device: imgs complex64 [nch][n] -> out float32 [n]."""
    _io_check(lib().cgs_rss_d(C.c_void_p(imgs.data_ptr()), imgs.shape[0], out.numel(), C.c_void_p(out.data_ptr()),
                              None if stream is None else C.c_void_p(stream)), "cgs_rss_d")


class Reco:
    """Reference-shaped reconstruction object over one CUDA context."""

    def __init__(self, img, grid, n_ch, kb_w=4.25, kb_b=14.9086, kb_order=5, kb_thresh=1e-7,
                 adj_scale=1e-3, offcenter=(0, 0, 0), device=0, workspace_bytes=0):
        L = lib()
        p = default_params()
        p.img[:] = list(img)
        p.grid[:] = list(grid)
        p.n_ch = n_ch
        p.kb_w, p.kb_b, p.kb_order = kb_w, kb_b, kb_order
        p.kb_thresh, p.adj_scale = kb_thresh, adj_scale
        p.offcenter[:] = list(offcenter)
        p.device = device
        p.workspace_bytes = workspace_bytes
        self.params = p
        self.img, self.grid, self.n_ch = tuple(img), tuple(grid), n_ch
        self.ni = int(np.prod(img))
        self.ng = int(np.prod(grid))
        self.ns = 0
        ctx = C.c_void_p()
        st = L.cgs_create(C.byref(p), C.byref(ctx))
        if st != CGS_OK:
            raise CGSError(st, "cgs_create failed (see stderr)")
        self._ctx = ctx
        self._L = L

    # -- plumbing -------------------------------------------------------
    def _check(self, st):
        if st != CGS_OK:
            raise CGSError(st, self._L.cgs_last_error(self._ctx).decode())

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.cgs_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def set_stream(self, stream_handle):
        self._check(self._L.cgs_set_stream(self._ctx, C.c_void_p(stream_handle)))

    def sync(self):
        self._check(self._L.cgs_sync(self._ctx))

    def launch_count(self):
        return int(self._L.cgs_last_launch_count(self._ctx))

    # -- set-up ---------------------------------------------------------
    def set_trajectory(self, k):
        k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
        self.ns = k.shape[0]
        self._check(self._L.cgs_set_trajectory(self._ctx, _p(k), self.ns))

    def set_mask(self, mask):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self._check(self._L.cgs_set_mask(self._ctx, _p(m)))

    def mask_from_data(self, data):
        d = _c64(data, (self.n_ch, self.ns))
        self._check(self._L.cgs_mask_from_data(self._ctx, _p(d)))

    def set_bins(self, bins):
        """bins: list of integer index arrays (one per respiratory bin)."""
        off = np.zeros(len(bins) + 1, np.int64)
        off[1:] = np.cumsum([len(b) for b in bins])
        idx = np.ascontiguousarray(np.concatenate([np.asarray(b, np.int32) for b in bins]), np.int32)
        self._check(self._L.cgs_set_bins(self._ctx, len(bins), _p(off), _p(idx)))

    def num_bins(self):
        return int(self._L.cgs_num_bins(self._ctx))

    def set_dcf(self, dcf):
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float32)
        self._check(self._L.cgs_set_dcf(self._ctx, _p(d)))

    def set_smaps(self, maps):
        m = _c64(maps, (self.n_ch,) + self.img)
        self._check(self._L.cgs_set_smaps(self._ctx, _p(m)))

    def set_smaps_tensor(self, maps):
        self._check(self._L.cgs_set_smaps_d(self._ctx, C.c_void_p(maps.data_ptr())))

    # -- operators (host arrays) -----------------------------------------
    def kernel_ft(self):
        out = np.zeros(self.grid, np.complex64)
        self._check(self._L.cgs_kernel_ft(self._ctx, _p(out)))
        return out

    def fft3(self, a, sign, rescale=False):
        a = _c64(a, self.grid).copy()
        self._check(self._L.cgs_fft3(self._ctx, _p(a), sign, int(rescale)))
        return a

    def nufft_fwd(self, imgs):
        imgs = _c64(imgs, (self.n_ch,) + self.img)
        out = np.zeros((self.n_ch, self.ns), np.complex64)
        self._check(self._L.cgs_nufft_fwd(self._ctx, _p(imgs), _p(out)))
        return out

    def nufft_adj(self, data):
        data = _c64(data, (self.n_ch, self.ns))
        out = np.zeros((self.n_ch,) + self.img, np.complex64)
        self._check(self._L.cgs_nufft_adj(self._ctx, _p(data), _p(out)))
        return out

    def apply_ehde(self, x, bin=0):
        x = _c64(x, self.img)
        q = np.zeros(self.img, np.complex64)
        self._check(self._L.cgs_apply_ehde(self._ctx, bin, _p(x), _p(q)))
        return q

    def cg_sense(self, data, threshold, max_iter=16):
        """Reco::cgSenseDynamic on bin 0: returns (x, residuals, iterations)."""
        data = _c64(data, (self.n_ch, self.ns))
        x = np.zeros(self.img, np.complex64)
        res = np.zeros(max(max_iter, 1), np.float64)
        it = np.zeros(1, np.int32)
        self._check(self._L.cgs_cg_solve(self._ctx, _p(data), _p(x), threshold, max_iter, _p(res), _p(it)))
        return x, res[: it[0]], int(it[0])

    def cg_sense_images(self, coil_imgs, threshold, max_iter=16):
        """Reco::cgSenseDynamic from coil images (the reference's own input)."""
        imgs = _c64(coil_imgs, (self.n_ch,) + self.img)
        x = np.zeros(self.img, np.complex64)
        res = np.zeros(max(max_iter, 1), np.float64)
        it = np.zeros(1, np.int32)
        self._check(self._L.cgs_cg_solve_images(self._ctx, _p(imgs), _p(x), threshold, max_iter,
                                                _p(res), _p(it)))
        return x, res[: it[0]], int(it[0])

    def cg_sense_batched(self, data, threshold, max_iter):
        """All bins: returns (x[nbins], residuals[nbins][max_iter], iters[nbins])."""
        nb = self.num_bins()
        data = _c64(data, (self.n_ch, self.ns))
        x = np.zeros((nb,) + self.img, np.complex64)
        res = np.zeros((nb, max(max_iter, 1)), np.float64)
        it = np.zeros(nb, np.int32)
        self._check(self._L.cgs_cg_solve_batched(self._ctx, _p(data), _p(x), threshold, max_iter,
                                                 _p(res), _p(it)))
        return x, res, it

    # -- device (torch) variants ------------------------------------------
    def nufft_fwd_tensor(self, imgs, out):
        self._check(self._L.cgs_nufft_fwd_d(self._ctx, C.c_void_p(imgs.data_ptr()), C.c_void_p(out.data_ptr())))

    def nufft_adj_tensor(self, data, out):
        self._check(self._L.cgs_nufft_adj_d(self._ctx, C.c_void_p(data.data_ptr()), C.c_void_p(out.data_ptr())))

    def apply_ehde_tensor(self, x, q, bin0=0, nb=1):
        self._check(self._L.cgs_apply_ehde_d(self._ctx, bin0, nb, C.c_void_p(x.data_ptr()),
                                             C.c_void_p(q.data_ptr())))

    def profile_apply_tensor(self, x, q, bin0=0, nb=1):
        """Per-stage kernel times (ms) of one E^H D E application."""
        out = np.zeros(256, np.float32)
        n = np.zeros(1, np.int32)
        self._check(self._L.cgs_profile_apply(self._ctx, bin0, nb, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(q.data_ptr()), _p(out), 256, _p(n)))
        return out[: n[0]].astype(np.float64)

    def fft3_tensor(self, a, sign):
        self._check(self._L.cgs_fft3_d(self._ctx, C.c_void_p(a.data_ptr()), sign, 0))

    def cg_sense_plain_tensor(self, data, x, threshold, max_iter):
        """The plain per-bin form (comparison point); returns (residuals, iters)."""
        nb = self.num_bins()
        res = np.zeros((nb, max(max_iter, 1)), np.float64)
        it = np.zeros(nb, np.int32)
        self._check(self._L.cgs_cg_solve_plain_d(self._ctx, C.c_void_p(data.data_ptr()), C.c_void_p(x.data_ptr()),
                                                 threshold, max_iter, _p(res), _p(it)))
        return res, it

    def cg_sense_trace_tensor(self, data, x, threshold, max_iter, x_trace):
        """Batched solve that also stores x after every iteration (x_trace:
        complex64 [max_iter][nbins][voxels] device tensor)."""
        nb = self.num_bins()
        res = np.zeros((nb, max(max_iter, 1)), np.float64)
        it = np.zeros(nb, np.int32)
        self._check(self._L.cgs_cg_solve_trace_d(self._ctx, C.c_void_p(data.data_ptr()), C.c_void_p(x.data_ptr()),
                                                 threshold, max_iter, _p(res), _p(it),
                                                 C.c_void_p(x_trace.data_ptr())))
        return res, it

    def cg_sense_fp64_tensor(self, data, x64, threshold, max_iter, x_trace=None):
        """Full-FP64 solve (x64: complex128 device tensor [nbins][voxels])."""
        nb = self.num_bins()
        res = np.zeros((nb, max(max_iter, 1)), np.float64)
        it = np.zeros(nb, np.int32)
        self._check(self._L.cgs_cg_solve_fp64_d(self._ctx, C.c_void_p(data.data_ptr()), C.c_void_p(x64.data_ptr()),
                                                threshold, max_iter, _p(res), _p(it),
                                                None if x_trace is None else C.c_void_p(x_trace.data_ptr())))
        return res, it

    def pipe_menon_dcf(self, iters=20):
        """GPU iterative density weights of every bin (host array [ns])."""
        out = np.zeros(self.ns, np.float32)
        self._check(self._L.cgs_pipe_menon_dcf(self._ctx, int(iters), _p(out), 0))
        return out

    def reconstruct_states(self, files, sx, sy, sz, out_dir, threshold, max_iter=16, write_rss=True):
        """The state loop of CGSense.cpp:200-282 (cgs_reconstruct_states);
        returns the iteration count of every state."""
        arr = (C.c_char_p * len(files))(*[f.encode() for f in files])
        it = np.zeros(len(files), np.int32)
        self._check(self._L.cgs_reconstruct_states(self._ctx, C.cast(arr, C.c_void_p), len(files), sx, sy, sz,
                                                   out_dir.encode(), threshold, max_iter, int(bool(write_rss)),
                                                   _p(it)))
        return it

    # -- differentiation --------------------------------------------------
    def loss_grad_tensor(self, x, y, grad_x=None, grad_k=None, bin=0):
        """Data-consistency loss 1/2 sum D |E S x - y|^2 of one bin and its
        gradients (device tensors: x complex64 image, y complex64 [n_ch][ns],
        grad_x complex64 image, grad_k float32 [ns][3]); returns the loss."""
        loss = C.c_double(0.0)
        self._check(self._L.cgs_loss_grad_d(
            self._ctx, int(bin), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.byref(loss),
            None if grad_x is None else C.c_void_p(grad_x.data_ptr()),
            None if grad_k is None else C.c_void_p(grad_k.data_ptr())))
        return loss.value

    def loss_grad_fp64_tensor(self, x64, y, grad_x=None, grad_k=None, bin=0):
        """The FP64 reference of loss_grad_tensor (x64, grad_x complex128,
        grad_k float64)."""
        loss = C.c_double(0.0)
        self._check(self._L.cgs_loss_grad_fp64_d(
            self._ctx, int(bin), C.c_void_p(x64.data_ptr()), C.c_void_p(y.data_ptr()), C.byref(loss),
            None if grad_x is None else C.c_void_p(grad_x.data_ptr()),
            None if grad_k is None else C.c_void_p(grad_k.data_ptr())))
        return loss.value

    def autotune(self):
        """Picks the fastest launch shapes for this context; returns
        {"spread_coils_per_block", "spread_variant" (see cgs_set_launch_shape;
         also under its older name "spread_warps_per_plane"),
         "interp_coils_per_thread", "candidates_ms"}."""
        t = np.zeros(32, np.float32)
        n = np.zeros(1, np.int32)
        sc = np.zeros(1, np.int32)
        sw = np.zeros(1, np.int32)
        ic = np.zeros(1, np.int32)
        self._check(self._L.cgs_autotune(self._ctx, _p(t), 32, _p(n), _p(sc), _p(sw), _p(ic)))
        return {"spread_coils_per_block": int(sc[0]), "spread_variant": int(sw[0]),
                "spread_warps_per_plane": int(sw[0]),
                "interp_coils_per_thread": int(ic[0]), "candidates_ms": [float(v) for v in t[: n[0]]]}

    def set_launch_shape(self, spread_cc=0, spread_variant=1, interp_cc=4):
        """Launch shape by hand (see cgs_set_launch_shape)."""
        self._check(self._L.cgs_set_launch_shape(self._ctx, spread_cc, spread_variant, interp_cc))

    def set_support_pruning(self, on):
        """Transform only the grid columns the samples' supports reach (default on;
        see cgs_set_support_pruning)."""
        self._check(self._L.cgs_set_support_pruning(self._ctx, 1 if on else 0))

    def support_stats(self):
        """Per bin: grid (y, z) columns the x passes transform and spreading
        tiles stored (see cgs_support_stats)."""
        nb = self.num_bins()
        cols = np.zeros(nb, np.int64)
        live = np.zeros(nb, np.int64)
        self._check(self._L.cgs_support_stats(self._ctx, _p(cols), _p(live)))
        return cols, live

    def estimate_smaps_tensor(self, data, maps, radius, eps=0.05):
        """Coil maps from low-resolution coil images (see cgs_estimate_smaps_d):
        data complex64 [n_ch][ns], maps complex64 [n_ch][img], device tensors."""
        self._check(self._L.cgs_estimate_smaps_d(self._ctx, C.c_void_p(data.data_ptr()), float(radius), float(eps),
                                                 C.c_void_p(maps.data_ptr())))

    def forward_y_listed_rows(self):
        """True when the forward y pass stores only the x pass's listed rows."""
        v = np.zeros(1, np.int32)
        self._check(self._L.cgs_forward_y_listed_rows(self._ctx, _p(v)))
        return bool(v[0])

    def set_toeplitz(self, mode):
        """Toeplitz embedding of E^H D E: 0 off (gridded operator), 1 on, 2 on
        with the unfused x stage (see cgs_set_toeplitz)."""
        self._check(self._L.cgs_set_toeplitz(self._ctx, int(mode)))

    def set_toeplitz_spectrum(self, method):
        """Spectrum build: 0 through the point-spread function (adjoint NUFFT)
        where the fine grid has FFT kernels, 1 the Dirichlet product (see
        cgs_set_toeplitz_spectrum)."""
        self._check(self._L.cgs_set_toeplitz_spectrum(self._ctx, int(method)))

    def toeplitz_spectrum_method(self):
        """1 point-spread function, 2 Dirichlet product, 0 not built."""
        return int(self._L.cgs_toeplitz_spectrum_method(self._ctx))

    def toeplitz_stats(self):
        """(build time of the spectra in ms, bytes they hold)."""
        ms = np.zeros(1, np.float64)
        b = np.zeros(1, np.int64)
        self._check(self._L.cgs_toeplitz_stats(self._ctx, _p(ms), _p(b)))
        return float(ms[0]), int(b[0])

    def setup_stats(self):
        """Set-up cost in ms (see cgs_setup_stats): {sort, tap_records, lists,
        transposed_matrix, workspace, graph_capture}."""
        v = np.zeros(6, np.float64)
        self._check(self._L.cgs_setup_stats(self._ctx, _p(v), 6))
        return dict(zip(("sort", "tap_records", "lists", "transposed_matrix", "workspace", "graph_capture"),
                        [float(x) for x in v]))

    def e2e_stats(self):
        """Device time (ms) of the parts of the last host-buffer batched
        solve and whether its buffers were page-locked (see cgs_e2e_stats):
        {upload, solve, download, pinned: [data, x]}."""
        v = np.zeros(3, np.float64)
        pin = np.zeros(2, np.int32)
        self._check(self._L.cgs_e2e_stats(self._ctx, _p(v), _p(pin)))
        out = dict(zip(("upload", "solve", "download"), [float(x) for x in v]))
        out["pinned"] = [int(pin[0]), int(pin[1])]
        return out

    def spread_matrix_stats(self):
        """(taps, grid points) of the transposed tap matrix (0, 0 when not built)."""
        t = np.zeros(1, np.int64)
        p = np.zeros(1, np.int64)
        self._check(self._L.cgs_spread_matrix_stats(self._ctx, _p(t), _p(p)))
        return int(t[0]), int(p[0])

    def spread_fused(self):
        """True when the last application ran the spreading fused with the
        adjoint x pass (see cgs_spread_fused)."""
        v = np.zeros(1, np.int32)
        self._check(self._L.cgs_spread_fused(self._ctx, _p(v)))
        return bool(v[0])

    def set_deterministic(self, on):
        """Fixed summation order (default); off lets the autotuner pick
        atomic spreading."""
        self._check(self._L.cgs_set_deterministic(self._ctx, 1 if on else 0))

    def set_precision(self, compensated):
        """Compensated (Kahan) spreading on or off."""
        self._check(self._L.cgs_set_precision(self._ctx, 1 if compensated else 0))

    def update_trajectory_tensor(self, k):
        """New coordinates (float64 device tensor [ns][3]) for the same samples."""
        self._check(self._L.cgs_update_trajectory_d(self._ctx, C.c_void_p(k.data_ptr())))

    @property
    def handle(self):
        """The C context pointer (for the libtorch operators)."""
        return int(C.cast(self._ctx, C.c_void_p).value or 0)

    def cg_sense_batched_tensor(self, data, x, threshold, max_iter, want_stats=True):
        nb = self.num_bins()
        res = np.zeros((nb, max(max_iter, 1)), np.float64) if want_stats else None
        it = np.zeros(nb, np.int32) if want_stats else None
        self._check(self._L.cgs_cg_solve_batched_d(self._ctx, C.c_void_p(data.data_ptr()),
                                                   C.c_void_p(x.data_ptr()), threshold, max_iter,
                                                   _p(res), _p(it)))
        return res, it
