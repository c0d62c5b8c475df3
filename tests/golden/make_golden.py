"""Generate the golden fixtures of tests/golden/ by running the reference's own
hot-path code (Reco.cpp, Fourier.cpp, Trajectory.cpp, IO.cpp of
expRad/4d_lung, compiled unmodified by oracle/Makefile into
oracle/_ref/ref_driver).

Run in a container that has the reference sources:

    make -C oracle ref && python tests/golden/make_golden.py

Each fixture is an .npz holding the seeded inputs and the reference outputs.
The reference FFTs run through oracle/fftw_adaptor (FFTW is not installed);
it computes in double precision and stores float, as FFTW's single-precision
plans store float.
"""
from __future__ import annotations

import os
import sys

import importlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)
import oracle_py as O  # noqa: E402


def crandn(rng, shape, scale=1.0):
    return ((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * scale).astype(np.complex64)


def readout_trajectory(rng, n_lines, n_read, jitter=0.02):
    """Readout lines along kx with random (ky, kz) offsets and a small wave,
    all inside [0.03, 0.97]^3 plus a few samples on the edges of [0, 1]."""
    t = np.linspace(0.03, 0.97, n_read)
    ky = rng.uniform(0.1, 0.9, n_lines)
    kz = rng.uniform(0.1, 0.9, n_lines)
    k = np.zeros((n_lines, n_read, 3))
    k[..., 0] = t[None, :]
    k[..., 1] = ky[:, None] + jitter * np.sin(2 * np.pi * 3 * t)[None, :]
    k[..., 2] = kz[:, None] + jitter * np.cos(2 * np.pi * 3 * t)[None, :]
    k = k.reshape(-1, 3)
    edge = np.array([[0.0, 0.5, 0.5], [1.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 1.0, 1.0],
                     [0.0, 0.0, 0.0], [1.0, 1.0, 1.0]])
    return np.concatenate([k, edge])


def ops_fixture(name, grid, nch, n_lines, n_read, seed, exclude_frac=0.0, cg_threshold=0.0):
    rng = np.random.default_rng(seed)
    k = readout_trajectory(rng, n_lines, n_read)
    ns = k.shape[0]
    data = crandn(rng, (nch, ns))
    if exclude_frac > 0:
        # excludeMissingData (Reco.cpp:681-696): coil-0 sample exactly zero
        drop = rng.random(ns) < exclude_frac
        data[0, drop] = 0
    img = crandn(rng, (nch,) + grid)
    smaps = crandn(rng, (nch,) + grid, 0.5)
    dcf = rng.uniform(0.5, 1.5, ns).astype(np.float32)
    params = dict(gx=grid[0], gy=grid[1], gz=grid[2], sx=ns, sy=1, sz=1, nch=nch, threads=4)
    out = {}
    r = O.run_ref("taps", params, {"traj": k, "data": data},
                  {"tap_count_out": (np.int32, None), "tap_idx_out": (np.int32, None),
                   "tap_w_out": (np.float32, None)})
    out.update(tap_count=r["tap_count_out"], tap_idx=r["tap_idx_out"], tap_w=r["tap_w_out"])
    r = O.run_ref("kernelft", params, {"traj": k}, {"kernelft_out": (np.complex64, None)})
    out["kernelft"] = r["kernelft_out"].reshape(grid)
    r = O.run_ref("fwd", params, {"traj": k, "img": img, "data": data},
                  {"data_out": (np.complex64, None)})
    out["fwd_data"] = r["data_out"].reshape(nch, ns)
    r = O.run_ref("bwd", params, {"traj": k, "data": data}, {"img_out": (np.complex64, None)})
    out["bwd_img"] = r["img_out"].reshape((nch,) + grid)
    r = O.run_ref("cg", dict(params, cg_threshold=cg_threshold),
                  {"traj": k, "data": data, "smaps": smaps, "dcf": dcf},
                  {"x_out": (np.complex64, None), "residuals_out": (np.float64, None),
                   "iters_out": (np.int32, None)})
    out.update(cg_x=r["x_out"].reshape(grid), cg_residuals=r["residuals_out"],
               cg_iters=r["iters_out"])
    np.savez_compressed(os.path.join(HERE, name), grid=np.array(grid), nch=nch, k=k, data=data,
                        img=img, smaps=smaps, dcf=dcf, cg_threshold=cg_threshold, **out)
    print("wrote", name, "samples", ns, "taps", int(out["tap_count"].sum()),
          "cg iters", int(out["cg_iters"][0]))


def traj_fixture(name, sx, sy, sz, grid, fov_y, fov_z, **wave):
    params = dict(gx=grid[0], gy=grid[1], gz=grid[2], sx=sx, sy=sy, sz=sz, nch=1,
                  fovy=fov_y, fovz=fov_z, **wave)
    r = O.run_ref("traj", params, {}, {"traj_out": (np.float64, None)})
    np.savez_compressed(os.path.join(HERE, name), sx=sx, sy=sy, sz=sz, grid=np.array(grid),
                        fov_y=fov_y, fov_z=fov_z, wave=np.array(list(wave.items()), dtype=object),
                        traj=r["traj_out"].reshape(-1, 3))
    print("wrote", name)


def io_fixture(name, sx, sy, sz, nch, grid, seed):
    """IO::importDataBin (readout-fastest file order -> z-fastest memory
    order, IO.cpp:55-98), IO::importSensitivityMaps (map<c>.bin, IO.cpp:25-51)
    and IO::exportFFTWComplexBin (IO.cpp:158-186) on seeded files."""
    rng = np.random.default_rng(seed)
    ns = sx * sy * sz
    raw = crandn(rng, (nch, ns))                 # file order: channel, then i1 + sx*i2 + sx*sy*i3
    ng = int(np.prod(grid))
    maps = crandn(rng, (nch, ng))
    params = dict(gx=grid[0], gy=grid[1], gz=grid[2], sx=sx, sy=sy, sz=sz, nch=nch, threads=2)
    arrays = {"raw_file": raw}
    arrays.update({"map%d" % c: maps[c] for c in range(nch)})
    r = O.run_ref("io", params, arrays, {"io_data_out": (np.complex64, None), "io_maps_out": (np.complex64, None),
                                         "io_export": (np.complex64, None)})
    np.savez_compressed(os.path.join(HERE, name), sx=sx, sy=sy, sz=sz, nch=nch, grid=np.array(grid), raw=raw,
                        maps=maps, data_out=r["io_data_out"].reshape(nch, ns),
                        maps_out=r["io_maps_out"].reshape(nch, ng), export=r["io_export"])
    print("wrote", name)


# The mid-size CG fixture: the reference's own parameters (grid == image,
# KB w = 4.25, b = 14.9086, the 11^3 tap neighbourhood, 16 CG iterations) on
# a 64x64x48 grid with 4 coils and a wave-CAIPI trajectory of 33 k samples.
# Its inputs are not stored: wave_cg_inputs() regenerates them from seeds
# (numpy's PCG64 streams and the FP64 oracle's forward operator), and the
# fixture keeps fingerprints of them so that a test can tell when the
# regenerated inputs drift.
WAVE_CG_NAME = "ref_cg_64x64x48_wave.npz"


def wave_cg_inputs():
    """(workload, k, smaps, x, dcf, data) of the mid-size CG fixture: a
    wave-CAIPI trajectory (R = 3x2, CAIPI shift 1, 64 samples per readout,
    +-3 cells over 5 cycles; readouts near the grid's faces leave it and lose
    taps there), Gaussian coil maps, the ellipsoid phantom, the radial
    density stand-in, and k-space = the FP64 oracle's nufftFWD of the coil
    images plus complex noise at SNR 30, rounded to complex64."""
    synth = importlib.import_module("4d_lung_gb300.synth")
    w = synth.Workload("ref_cg_64x64x48_wave", (64, 64, 48), (64, 64, 48), 4, (3, 2), 1, 1, 3.0, 5, 1, 16)
    k = synth.wave_trajectory(w)
    smaps = synth.coil_maps(w.img, w.n_ch)
    x = synth.phantom(w.img)
    dcf = synth.radial_dcf(k, w.grid)
    o = O.Oracle(64)
    p = O.make_params(w.img, w.grid, w.n_ch)
    taps = o.taps(p, k)
    y = o.nufft_fwd(p, taps, o.kernel_ft(p), smaps.astype(np.complex128) * x[None]).astype(np.complex64)
    y += synth.complex_noise(y.shape, 30.0, float(np.sqrt(np.mean(np.abs(y) ** 2))))
    return w, k, smaps, x, dcf, y


def input_fingerprint(k, data):
    """Sums that identify the regenerated inputs (FP64)."""
    d = data.astype(np.complex128)
    return np.array([k.sum(), (k * k).sum(), np.abs(d).sum(), (d.real * np.arange(d.size).reshape(d.shape)).sum()])


def wave_cg_fixture(threads=8):
    """Runs the reference's calculateWeights, nufftFWD, nufftBWD and
    cgSenseDynamic (Reco.cpp:175-321,468-553,698-806) on the mid-size inputs
    and stores subsampled outputs: per-sample tap counts and weight sums, the
    forward samples of every 8th sample, the adjoint image of coil 0 and the
    CG image on every second voxel per axis, the residual sequence and the
    iteration count."""
    w, k, smaps, x, dcf, y = wave_cg_inputs()
    grid, nch, ns = w.grid, w.n_ch, k.shape[0]
    params = dict(gx=grid[0], gy=grid[1], gz=grid[2], sx=ns, sy=1, sz=1, nch=nch, threads=threads)
    r = O.run_ref("taps", params, {"traj": k},
                  {"tap_count_out": (np.int32, None), "tap_idx_out": (np.int32, None),
                   "tap_w_out": (np.float32, None)})
    cnt = r["tap_count_out"]
    seg = np.repeat(np.arange(ns), cnt)
    wsum = np.bincount(seg, weights=r["tap_w_out"].astype(np.float64), minlength=ns)
    imgs = (smaps * x[None]).astype(np.complex64)
    r = O.run_ref("fwd", params, {"traj": k, "img": imgs}, {"data_out": (np.complex64, None)})
    fwd = r["data_out"].reshape(nch, ns)
    r = O.run_ref("bwd", params, {"traj": k, "data": y, "dcf": dcf}, {"img_out": (np.complex64, None)})
    bwd0 = r["img_out"].reshape((nch,) + grid)[0]
    r = O.run_ref("cg", dict(params, cg_threshold=0.0), {"traj": k, "data": y, "smaps": smaps, "dcf": dcf},
                  {"x_out": (np.complex64, None), "residuals_out": (np.float64, None),
                   "iters_out": (np.int32, None), "cg_seconds_out": (np.float64, None)})
    xr = r["x_out"].reshape(grid)
    np.savez_compressed(os.path.join(HERE, WAVE_CG_NAME), grid=np.array(grid), nch=nch, ns=ns,
                        fingerprint=input_fingerprint(k, y),
                        tap_count=cnt.astype(np.uint8), tap_wsum=wsum,
                        fwd_every8=fwd[:, ::8], bwd_coil0_sub2=bwd0[::2, ::2, ::2],
                        cg_x_sub2=xr[::2, ::2, ::2], cg_x_norm=np.linalg.norm(xr.astype(np.complex128)),
                        cg_residuals=r["residuals_out"], cg_iters=r["iters_out"],
                        ref_cg_seconds=r["cg_seconds_out"], ref_threads=threads)
    print("wrote", WAVE_CG_NAME, "samples", ns, "taps", int(cnt.sum()), "cg iters", int(r["iters_out"][0]),
          "ref cg %.1f s" % float(r["cg_seconds_out"][0]))


def main():
    if not O.ref_available():
        O.build()
    # operator + CG fixtures at the reference's own parameters (grid == image)
    ops_fixture("ref_ops_24x20x16.npz", (24, 20, 16), nch=2, n_lines=12, n_read=48, seed=11)
    ops_fixture("ref_ops_32x24x16_mask.npz", (32, 24, 16), nch=3, n_lines=20, n_read=64, seed=12,
                exclude_frac=0.3)
    ops_fixture("ref_ops_40x20x16_stop.npz", (40, 20, 16), nch=2, n_lines=30, n_read=80, seed=13,
                cg_threshold=8e-3)
    # wave-CAIPI trajectory: reference defaults of CGSense.cpp:47-59 on a
    # reduced sampling matrix
    traj_fixture("ref_traj_wave.npz", 112, 28, 14, (128, 128, 128), 0.5, 0.00223 * 14,
                 nosc=4, dwell=6.3e-6 * 4, grad_amp=0.006, amp_corr_y=0.998, amp_corr_z=1.01,
                 shift_y=5.6e-6, shift_z=6.5e-6)
    io_fixture("ref_io_12x5x4.npz", 12, 5, 4, 3, (8, 6, 4), seed=21)
    traj_fixture("ref_traj_wave_b.npz", 64, 16, 8, (96, 80, 64), 0.3, 0.05,
                 nosc=7, dwell=1e-5, grad_amp=0.01, amp_corr_y=1.0, amp_corr_z=0.97,
                 shift_y=0.0, shift_z=1e-5)
    wave_cg_fixture()


if __name__ == "__main__":
    if sys.argv[1:] == ["wave_cg"]:
        wave_cg_fixture()
    else:
        main()
