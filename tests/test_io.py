"""File IO of the reconstruction (IO.cpp): the reference's own import /
export run on seeded files (tests/golden/ref_io_12x5x4.npz) against the
library's IO entry points.  Host-side readers and writers run on the CPU;
the device import (permutation on the GPU), the coil-image root-sum-of-
squares and the state loop need a GPU."""
import os

import numpy as np
import pytest

from conftest import golden, rel_l2

IO = "ref_io_12x5x4.npz"


def test_permutation_restatement_matches_reference():
    """The oracle restatement of IO.cpp:55-98 (file index i1 + sx i2 + sx sy
    i3 -> memory index i3 + sz i2 + sy sz i1, per channel) reproduces the
    reference's importDataBin."""
    z = golden(IO)
    sx, sy, sz = int(z["sx"]), int(z["sy"]), int(z["sz"])
    raw = z["raw"]
    i3, i2, i1 = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    out = np.zeros_like(raw)
    out[:, (i3 + sz * i2 + sy * sz * i1).ravel()] = raw[:, (i1 + sx * i2 + sx * sy * i3).ravel()]
    assert np.array_equal(out, z["data_out"])


def test_smaps_import_and_export_match_reference(cgs, tmp_path):
    z = golden(IO)
    nch, ng = z["maps"].shape
    for c in range(nch):
        z["maps"][c].astype(np.complex64).tofile(str(tmp_path / ("map%d.bin" % c)))
    maps = cgs.import_smaps_bin(str(tmp_path), ng, nch)
    assert np.array_equal(maps, z["maps_out"])
    cgs.export_complex_bin(str(tmp_path / "exp.bin"), maps[0])
    assert (tmp_path / "exp.bin").read_bytes() == z["export"].astype(np.complex64).tobytes()


def test_host_io_errors_and_float_export(cgs, tmp_path):
    d = np.arange(7, dtype=np.float32)
    cgs.export_float_bin(str(tmp_path / "d.bin"), d)
    assert np.array_equal(cgs.import_density_bin(str(tmp_path / "d.bin"), 7), d)
    with pytest.raises(cgs.CGSError):
        cgs.import_density_bin(str(tmp_path / "d.bin"), 8)          # short file
    with pytest.raises(cgs.CGSError):
        cgs.import_smaps_bin(str(tmp_path / "missing"), 4, 1)      # missing map0.bin
    # an unopenable path is retried as path + "_1.bin" (IO.cpp:170-183)
    target = tmp_path / "no_dir" / "x.bin"
    with pytest.raises(cgs.CGSError):
        cgs.export_complex_bin(str(target), np.zeros(2, np.complex64))


@pytest.mark.gpu
def test_device_import_matches_reference(gpu_lib, cgs, tmp_path):
    import torch
    z = golden(IO)
    sx, sy, sz, nch = int(z["sx"]), int(z["sy"]), int(z["sz"]), int(z["nch"])
    path = str(tmp_path / "raw.bin")
    z["raw"].astype(np.complex64).tofile(path)
    out = torch.zeros((nch, sx * sy * sz), dtype=torch.complex64, device="cuda")
    cgs.import_data_bin_tensor(path, sx, sy, sz, nch, out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), z["data_out"])
    with pytest.raises(cgs.CGSError):
        cgs.import_data_bin_tensor(path, sx + 1, sy, sz, nch, out)   # file too short


@pytest.mark.gpu
def test_device_import_large_file_chunks(gpu_lib, cgs, tmp_path):
    """A file larger than one 32 MiB staging chunk (several double-buffered reads)."""
    import torch
    sx, sy, sz, nch = 512, 64, 40, 4
    rng = np.random.default_rng(3)
    raw = (rng.standard_normal((nch, sx * sy * sz)) + 1j * rng.standard_normal((nch, sx * sy * sz))).astype(np.complex64)
    path = str(tmp_path / "big.bin")
    raw.tofile(path)
    out = torch.zeros(raw.shape, dtype=torch.complex64, device="cuda")
    cgs.import_data_bin_tensor(path, sx, sy, sz, nch, out)
    torch.cuda.synchronize()
    i3, i2, i1 = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
    ref = np.zeros_like(raw)
    ref[:, (i3 + sz * i2 + sy * sz * i1).ravel()] = raw[:, (i1 + sx * i2 + sx * sy * i3).ravel()]
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.gpu
def test_rss_matches_reference_arithmetic(gpu_lib, cgs):
    """rssq2DVecImg (functions.h:290-316): float sums over coils in order."""
    import torch
    rng = np.random.default_rng(5)
    imgs = (rng.standard_normal((5, 1000)) + 1j * rng.standard_normal((5, 1000))).astype(np.complex64)
    acc = np.zeros(1000, np.float32)
    for c in range(5):
        acc = (acc + (imgs[c].real * imgs[c].real + imgs[c].imag * imgs[c].imag).astype(np.float32)).astype(np.float32)
    ref = np.sqrt(acc).astype(np.float32)
    out = torch.zeros(1000, dtype=torch.float32, device="cuda")
    cgs.rss_tensor(torch.from_numpy(imgs).cuda(), out)
    torch.cuda.synchronize()
    assert np.allclose(out.cpu().numpy(), ref, rtol=2e-7, atol=0)


@pytest.mark.gpu
def test_state_loop_matches_single_solves(gpu_lib, cgs, synth, tmp_path):
    """cgs_reconstruct_states over two state files (different missing
    samples) equals importing, masking and solving each file on its own; the
    exported root-sum-of-squares is that of the density-corrected coil
    images."""
    import torch
    img = grid = (16, 16, 16)
    nch = 3
    sx, sy, sz = 24, 8, 6
    rng = np.random.default_rng(11)
    # z-fastest memory order of the samples: index i3 + sz i2 + sy sz i1
    i1, i2, i3 = np.meshgrid(np.arange(sx), np.arange(sy), np.arange(sz), indexing="ij")
    k = np.stack([(i1 + 0.5) / sx, (i2 + 0.5) / sy, (i3 + 0.5) / sz], -1).reshape(-1, 3) * 0.9 + 0.05
    ns = k.shape[0]
    smaps = synth.coil_maps(img, nch)
    dcf = rng.uniform(0.5, 1.5, ns).astype(np.float32)
    files = []
    datas = []
    for s in range(2):
        data = (rng.standard_normal((nch, ns)) + 1j * rng.standard_normal((nch, ns))).astype(np.complex64)
        data[:, rng.random(ns) < 0.2 * (s + 1)] = 0      # missing samples (CAIPI / bin holes)
        datas.append(data)
        # file order: channel, then i1 + sx i2 + sx sy i3
        raw = np.zeros_like(data)
        j3, j2, j1 = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
        raw[:, (j1 + sx * j2 + sx * sy * j3).ravel()] = data[:, (j3 + sz * j2 + sy * sz * j1).ravel()]
        path = str(tmp_path / ("state%d.bin" % s))
        raw.tofile(path)
        files.append(path)
    r = cgs.Reco(img, grid, nch)
    r.set_trajectory(k)
    r.set_dcf(dcf)
    r.set_smaps(smaps)
    out = str(tmp_path / "out")
    its = r.reconstruct_states(files, sx, sy, sz, out, 0.0, 6)
    assert list(its) == [6, 6]
    r2 = cgs.Reco(img, grid, nch)
    r2.set_trajectory(k)
    r2.set_dcf(dcf)
    r2.set_smaps(smaps)
    for s in range(2):
        r2.mask_from_data(datas[s])
        x, _, it = r2.cg_sense(datas[s], 0.0, 6)
        got = np.fromfile(os.path.join(out, "results", "b_state%d.bin" % s), dtype=np.complex64).reshape(img)
        assert rel_l2(got, x) < 1e-5
    # RSS of the last state's density-corrected coil images
    coil = r2.nufft_adj(datas[1] * dcf[None])
    rss = np.sqrt(np.sum(np.abs(coil) ** 2, axis=0))
    got = np.fromfile(os.path.join(out, "resultRssq.bin"), dtype=np.float32).reshape(img)
    assert rel_l2(got, rss) < 1e-5
