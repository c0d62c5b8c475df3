"""cgs_fft3_noalloc: the centred 3-D FFT for callers that cannot let the
library allocate device memory (its scratch is a fixed device array inside
the library).  Checked through the C ABI against the existing context-based
transform cgs_fft3_d, on two calls in a row, and -- in a fresh process that
has created no library context -- against the FP64 oracle's centred FFT,
with the output written over the input, within the FFT tolerance used by
the other parity tests (relative L2 2e-6).

The file name sorts last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu


def _grid_arg(grid):
    return (C.c_int32 * 3)(*grid)


@pytest.mark.parametrize("grid", [(32, 24, 16), (64, 64, 128)])
def test_noalloc_fft_matches_context_fft(gpu_lib, cgs, grid):
    import torch
    L = gpu_lib
    reco = cgs.Reco(grid, grid, 1)
    stream = torch.cuda.Stream()
    reco.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(7)
    for call in range(2):                    # two calls in a row share the scratch
        for sign in (-1, 1):
            a = (rng.standard_normal(grid) + 1j * rng.standard_normal(grid)).astype(np.complex64)
            with torch.cuda.stream(stream):
                src = torch.from_numpy(a).cuda()
                ref = src.clone()
                out = torch.empty_like(src)
            stream.synchronize()
            assert L.cgs_fft3_d(reco.ctx, C.c_void_p(ref.data_ptr()), sign, 0) == 0
            st = L.cgs_fft3_noalloc(C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()),
                                    _grid_arg(grid), sign, C.c_void_p(stream.cuda_stream))
            assert st == 0
            stream.synchronize()
            assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 2e-6, (call, sign)
            assert torch.equal(src.cpu(), torch.from_numpy(a))     # input untouched
    reco.close()


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu_lib, cgs):
    import torch
    L = gpu_lib
    x = torch.zeros(8, dtype=torch.complex64, device="cuda")
    assert L.cgs_fft3_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                              _grid_arg((128, 128, 64)), -1, None) == cgs.CGS_ERR_ARG
    assert L.cgs_fft3_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                              _grid_arg((36, 32, 32)), -1, None) == cgs.CGS_ERR_UNSUPPORTED
    assert L.cgs_fft3_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                              _grid_arg((32, 32, 32)), 2, None) == cgs.CGS_ERR_ARG


def test_noalloc_rejects_misaligned_pointers(gpu_lib, cgs):
    """in / out are complex float arrays: a pointer off an 8-byte boundary is
    refused before anything is launched."""
    import torch
    L = gpu_lib
    x = torch.zeros(2 * 32 * 32 * 32 + 2, dtype=torch.float32, device="cuda")
    base = x.data_ptr()
    g = _grid_arg((32, 32, 32))
    assert L.cgs_fft3_noalloc(C.c_void_p(base + 4), C.c_void_p(base), g, -1, None) == cgs.CGS_ERR_ARG
    assert L.cgs_fft3_noalloc(C.c_void_p(base), C.c_void_p(base + 4), g, -1, None) == cgs.CGS_ERR_ARG
    torch.cuda.synchronize()


_FRESH = textwrap.dedent("""
    import ctypes as C, importlib, sys
    import numpy as np
    sys.path[:0] = [ROOT, ROOT + "/oracle"]
    cgs = importlib.import_module("4d_lung_gb300")
    import oracle_py
    import torch
    L = cgs.lib()
    o = oracle_py.Oracle(64)
    rng = np.random.default_rng(3)
    errs = []
    for grid in [(32, 24, 16), (48, 40, 64)]:
        p = oracle_py.make_params(grid, grid, 1)
        for call in range(2):
            for sign in (-1, 1):
                a = (rng.standard_normal(grid) + 1j * rng.standard_normal(grid)).astype(np.complex64)
                buf = torch.from_numpy(a).cuda()
                g = (C.c_int32 * 3)(*grid)
                # output written over the input (in == out)
                st = L.cgs_fft3_noalloc(C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), g, sign, None)
                assert st == 0, st
                torch.cuda.synchronize()
                ref = o.centred_fft(p, a, sign, 0)
                out = buf.cpu().numpy().astype(np.complex128)
                errs.append(float(np.linalg.norm(out - ref) / np.linalg.norm(ref)))
    print("ERRS", max(errs))
""")


def test_noalloc_first_call_in_fresh_process_vs_oracle(gpu_lib):
    """The case the entry point exists for: a process whose first library
    call is cgs_fft3_noalloc (no library context, no prior set-up), two calls
    in a row per size and sign, the output written over the input, against
    the FP64 oracle's centred FFT (Fourier.cpp:4-72)."""
    env = dict(os.environ)
    code = "ROOT = %r\n" % ROOT + _FRESH
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    err = float([ln for ln in r.stdout.splitlines() if ln.startswith("ERRS")][0].split()[1])
    assert err < 2e-6, err
