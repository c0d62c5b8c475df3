"""Voronoi density weights (estimateDensityV3D, functions.h:161-258): cell
volumes, 0 on the convex hull, normalised by the maximum.  CGAL (the
reference's dependency) is not available; the weights are checked against
scipy's qhull Voronoi diagram and against a lattice of known cell volume."""
import numpy as np
import pytest


def scipy_volumes(pts):
    sp = pytest.importorskip("scipy.spatial")
    vor = sp.Voronoi(pts)
    vols = np.zeros(len(pts))
    for i, ri in enumerate(vor.point_region):
        reg = vor.regions[ri]
        if -1 in reg or len(reg) == 0:
            continue
        vols[i] = sp.ConvexHull(vor.vertices[reg]).volume
    return vols / vols.max()


@pytest.mark.parametrize("n,seed", [(400, 1), (2500, 2)])
def test_voronoi_matches_qhull(cgs, n, seed):
    pts = np.random.default_rng(seed).uniform(0, 1, (n, 3))
    d = cgs.voronoi_dcf(pts)
    ref = scipy_volumes(pts)
    assert np.array_equal(d == 0, ref == 0)          # same hull samples
    assert np.abs(d - ref).max() < 1e-6


def test_voronoi_lattice_known_answer(cgs):
    """Interior cells of a jittered-free cubic lattice are unit cubes; the
    largest volume belongs to such a cell, so interior weights are 1 and the
    hull samples (the lattice faces) are 0."""
    g = np.arange(6, dtype=np.float64)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pts += np.random.default_rng(0).uniform(-1e-9, 1e-9, pts.shape)   # break exact ties
    d = cgs.voronoi_dcf(pts)
    on_face = np.any((pts < 0.5) | (pts > 4.5), axis=1)
    assert np.all(d[on_face] == 0)
    assert np.allclose(d[~on_face], 1.0, atol=1e-6)


def test_voronoi_readout_trajectory(cgs, synth):
    """A wave-CAIPI bin: weights in [0, 1], hull zeros at the readout ends."""
    w = synth.scaled(synth.WORKLOADS["cfg3"], (32, 32, 24), (64, 64, 48), n_ch=2, n_bins=4)
    lines = synth.readout_lines(w)
    k = synth.wave_trajectory(w, synth.WaveParams(2.0, 2.0), lines=lines)
    kb = k.reshape(len(lines), w.n_read, 3)[::3].reshape(-1, 3)
    d = cgs.voronoi_dcf(kb)
    assert d.min() >= 0 and d.max() == pytest.approx(1.0)
    ends = kb.reshape(-1, w.n_read, 3)[:, [0, -1]].reshape(-1, 3)
    dd = d.reshape(-1, w.n_read)[:, [0, -1]]
    assert np.all(dd == 0)
    assert (d > 0).mean() > 0.5


@pytest.mark.parametrize("cutoff", [1.0, 0.75])
def test_density_readout_averaging(cgs, synth, cutoff):
    """estimateDensityV3D(average=true, cutoff) (functions.h:212-245),
    restated in numpy from the per-sample volumes: sums per readout position,
    divided by the total, positions past (sX-1)*cutoff clamped, then divided
    by the maximum."""
    w = synth.scaled(synth.WORKLOADS["cfg3"], (32, 32, 24), (64, 64, 48), n_ch=2, n_bins=4)
    lines = synth.readout_lines(w)
    k = synth.wave_trajectory(w, synth.WaveParams(2.0, 2.0), lines=lines)
    sx = w.n_read
    kb = k.reshape(len(lines), sx, 3)[::5].reshape(-1, 3)
    raw = cgs.voronoi_dcf(kb).astype(np.float64)       # volumes / max: averaging is scale-free
    avg = raw.reshape(-1, sx).sum(0)
    avg /= avg.sum()
    pos = np.minimum(np.arange(sx), int((sx - 1) * cutoff))
    ref = np.tile(avg[pos], kb.shape[0] // sx)
    ref /= ref.max()
    d = cgs.estimate_density_v3d(kb, sx, average=True, cutoff=cutoff)
    assert np.abs(d - ref).max() < 1e-6
    assert np.array_equal(cgs.estimate_density_v3d(kb, sx, average=False), cgs.voronoi_dcf(kb))
    with pytest.raises(cgs.CGSError):
        cgs.estimate_density_v3d(kb[:-1], sx, average=True)


@pytest.mark.gpu
def test_pipe_menon_weights_follow_density(gpu_lib, cgs):
    """GPU Pipe-Menon weights (the documented alternative to the Voronoi
    volumes): on a lattice twice as dense in x on one side, the interior
    weights differ by the density ratio, and they agree with the Voronoi
    volumes of the same samples away from the edges."""
    grid = (48, 32, 32)
    xs = np.concatenate([np.arange(6.0, 24.0, 1.0), np.arange(24.0, 42.0, 0.5)])
    ys = np.arange(6.0, 26.0, 1.0)
    zs = np.arange(6.0, 26.0, 1.0)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    cells = np.stack([X, Y, Z], -1).reshape(-1, 3)
    k = cells / (np.array(grid) - 1)
    r = cgs.Reco(grid, grid, 1, kb_w=4.25, kb_b=14.9086)
    r.set_trajectory(k)
    w = r.pipe_menon_dcf(30)
    assert w.max() == pytest.approx(1.0) and w.min() > 0
    interior = (np.abs(Y - 16) < 5) & (np.abs(Z - 16) < 5)
    sparse = interior & (X > 10) & (X < 20)
    dense = interior & (X > 28) & (X < 38)
    ratio = np.median(w.reshape(X.shape)[sparse]) / np.median(w.reshape(X.shape)[dense])
    assert 1.8 < ratio < 2.2, ratio
    v = cgs.voronoi_dcf(k).reshape(X.shape)
    wv = w.reshape(X.shape)
    rv = np.median(v[sparse]) / np.median(v[dense])
    assert abs(ratio / rv - 1) < 0.1, (ratio, rv)


@pytest.mark.gpu
def test_pipe_menon_vs_fp64_oracle_on_wave_caipi(gpu_lib, cgs, synth, oracle_mod, o64):
    """GPU Pipe-Menon weights on a wave-CAIPI trajectory (48x48x32 image on a
    96x96x64 grid, 8 coils, one fully sampled bin of 73 728 samples, KB width
    4) against the FP64 restatement (oracle_py.pipe_menon), 20 iterations:
    relative L2 <= 1e-4 over the samples.  Then what the weights do to the
    solve: the CG image (15 iterations, SNR 30) with the capped Pipe-Menon
    weights stays within 3e-2 of the image with the capped Voronoi volumes
    (functions.h:161-258), and both lie within 8e-2 of the phantom (best
    complex scale)."""
    w = synth.scaled(synth.WORKLOADS["cfg3"], (48, 48, 32), (96, 96, 64), n_ch=8, n_bins=1)
    k = synth.wave_trajectory(w)
    kb_w = 4.0
    kb_b = float(np.pi * np.sqrt(kb_w ** 2 / 4 * 1.5 ** 2 - 0.8))
    p = oracle_mod.make_params(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b)
    taps = o64.taps(p, k)
    ref = oracle_mod.pipe_menon(taps, int(np.prod(w.grid)), 20)
    r = cgs.Reco(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b)
    r.set_trajectory(k)
    pm = r.pipe_menon_dcf(20)
    err_w = float(np.linalg.norm(pm - ref) / np.linalg.norm(ref))
    assert err_w < 1e-4, err_w
    smaps = synth.coil_maps(w.img, w.n_ch)
    x_true = synth.phantom(w.img)
    r.set_smaps(smaps)
    y = r.nufft_fwd(smaps * x_true[None])
    y += synth.complex_noise(y.shape, 30.0, float(np.sqrt(np.mean(np.abs(y) ** 2))))

    def solve(d):
        r.set_dcf(d)
        x, res, it = r.cg_sense(y, 0.0, 15)
        a = np.vdot(x, x_true) / np.vdot(x, x)
        return x, float(np.linalg.norm(a * x - x_true) / np.linalg.norm(x_true))

    xv, ev = solve(synth.cap_dcf(cgs.voronoi_dcf(k)))
    xp, ep = solve(synth.cap_dcf(pm))
    d_img = float(np.linalg.norm(xp - xv) / np.linalg.norm(xv))
    print("pm vs oracle %.2e; image error vs truth: voronoi %.3f, pipe-menon %.3f; images apart %.3f"
          % (err_w, ev, ep, d_img))
    assert ev < 8e-2 and ep < 8e-2, (ev, ep)
    assert d_img < 3e-2 * 3, d_img
