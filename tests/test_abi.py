"""C ABI checks that need no GPU: the library builds, loads and exports every
symbol include/cgsense_c.h declares; host-only entry points agree with the
oracle; argument validation returns error codes before any CUDA call."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden

HEADER = os.path.join(ROOT, "include", "cgsense_c.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void\s*\*|void|const char\s*\*|int64_t|uint64_t)\s*(cgs_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib(cgs):
    if not os.path.exists(cgs.LIB_PATH):
        cgs.build()
    return cgs.lib()


def test_header_matches_binding_list(cgs):
    assert declared_symbols() == sorted(cgs.EXPORTS)


def test_library_exports_every_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_wave_caipi_host_entry_point(cgs, o64):
    """cgs_wave_caipi (host C++) against the reference's own trajectory."""
    for name in ["ref_traj_wave.npz", "ref_traj_wave_b.npz"]:
        z = golden(name)
        w = dict(z["wave"].tolist())
        k = cgs.wave_caipi(int(z["sx"]), int(z["sy"]), int(z["sz"]), [int(v) for v in z["grid"]],
                           float(z["fov_y"]), float(z["fov_z"]), n_osc=int(w["nosc"]),
                           grad_amp=w["grad_amp"], amp_corr_y=w["amp_corr_y"],
                           amp_corr_z=w["amp_corr_z"], shift_y=w["shift_y"], shift_z=w["shift_z"],
                           dwell=w["dwell"])
        assert np.max(np.abs(k - z["traj"])) < 1e-12


def test_wave_caipi_rejects_bad_args(cgs):
    with pytest.raises(cgs.CGSError):
        cgs.wave_caipi(1, 4, 4, (32, 32, 32), 0.5, 0.05)


@pytest.mark.parametrize("grid,img,code", [
    ((33, 32, 32), (33, 32, 32), 1),      # odd size (Fourier.cpp:54,64 reads k+1)
    ((36, 32, 32), (36, 32, 32), 6),      # no FFT kernel for 36
    ((32, 32, 32), (40, 32, 32), 1),      # image larger than grid
])
def test_create_validates_before_cuda(cgs, lib, grid, img, code):
    p = cgs.default_params()
    p.img[:] = list(img)
    p.grid[:] = list(grid)
    p.n_ch = 2
    ctx = C.c_void_p()
    assert lib.cgs_create(C.byref(p), C.byref(ctx)) == code
    assert not ctx.value


def test_default_params_are_reference_values(cgs):
    p = cgs.default_params()
    assert p.kb_w == 4.25 and abs(p.kb_b - 14.9086) < 1e-5 and p.kb_order == 5
    assert p.kb_thresh == 1e-7 and p.adj_scale == 1e-3
