"""cgs_fft3_noalloc: the centred 3-D FFT for callers that cannot let the
library allocate device memory (its scratch is a fixed device array inside
the library).  Checked through the C ABI against the existing context-based
transform cgs_fft3_d, on two calls in a row, within the FFT tolerance used
by the other parity tests (relative L2 2e-6).

The file name sorts last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

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
