"""Seeded synthetic inputs for the CG-SENSE workloads (numpy, host side).

The reference's example dataset (a lung scan published on Zenodo) is not
available, so every workload is synthetic with the shapes of the benchmark
configurations:

* phantom: 10 random ellipsoids (seed 0), complex with a smooth random phase
  (low-order polynomial, seed 1);
* coils: Gaussian-profile sensitivities centred on a ring around the field of
  view, normalised so that sum_c |S_c|^2 = 1;
* trajectory: wave-CAIPI readouts on a ky/kz Cartesian base grid undersampled
  R_y x R_z with a CAIPI shift, sinusoidal y/z excursions (90 degrees apart)
  of +-A grid cells over n cycles, readouts oversampled along kx;
* respiratory bins: a breathing trace sin(2 pi t / 4 s) + 10 % Gaussian
  jitter (seed 3) sampled every TR = 5 ms, split into bins whose occupancies
  spread between 3 % and 12 % of the readouts.

Coordinates follow the reference: a sample at k in [0,1]^3 sits at grid
coordinate k*(N-1) (Reco.cpp:751-755); the k-space centre is the grid point
N/2 (Reco.cpp:568).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    img: tuple
    grid: tuple
    n_ch: int
    r: tuple              # (R_y, R_z)
    caipi: int
    read_os: int          # readout oversampling factor
    wave_cells: float
    wave_cycles: float
    n_bins: int
    cg_iters: int
    z_shift_max: float = 0.0   # phantom displacement per bin (voxels)
    notes: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n_read(self):
        return self.read_os * self.img[0]


# The five benchmark configurations (sizes only; see the module docstring).
WORKLOADS = {
    "cfg1": Workload("cfg1_64cube_8coil", (64, 64, 64), (128, 128, 128), 8, (2, 2), 1, 4, 4.0, 7, 1, 10),
    "cfg2": Workload("cfg2_160x160x112_16coil", (160, 160, 112), (320, 320, 224), 16, (3, 2), 1, 4, 6.0, 9, 1, 20),
    "cfg3": Workload("cfg3_128x128x96_12coil_16bin", (128, 128, 96), (256, 256, 192), 12, (2, 2), 1, 4, 5.0, 8,
                     16, 15, z_shift_max=8.0),
    "cfg4": Workload("cfg4_128x128x96_12coil_1bin", (128, 128, 96), (256, 256, 192), 12, (2, 2), 1, 4, 5.0, 8, 1, 15),
    "cfg5": Workload("cfg5_256x256x176_20coil_24bin", (256, 256, 176), (512, 512, 352), 20, (3, 2), 1, 4, 8.0, 11,
                     24, 10, z_shift_max=8.0),
}


def scaled(w: Workload, img, grid, n_ch=None, n_bins=None, read_os=None):
    """A smaller copy of a workload (tests)."""
    return Workload(w.name + "_small", tuple(img), tuple(grid), n_ch or w.n_ch, w.r, w.caipi,
                    read_os or w.read_os, w.wave_cells, w.wave_cycles, n_bins or w.n_bins, w.cg_iters,
                    w.z_shift_max)


# ---------------------------------------------------------------------------
# phantom and coils
# ---------------------------------------------------------------------------

def phantom(img, n_ellipsoids=10, seed=0, phase_seed=1, z_shift=0.0):
    rng = np.random.default_rng(seed)
    axes = [np.linspace(-1, 1, n, endpoint=False) + 1.0 / n for n in img]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    Z = Z - 2.0 * z_shift / img[2]
    mag = np.zeros(img, np.float32)
    for _ in range(n_ellipsoids):
        c = rng.uniform(-0.4, 0.4, 3)
        r = rng.uniform(0.1, 0.45, 3)
        a = rng.uniform(0.2, 1.0)
        inside = ((X - c[0]) / r[0]) ** 2 + ((Y - c[1]) / r[1]) ** 2 + ((Z - c[2]) / r[2]) ** 2 <= 1.0
        mag[inside] += a
    prng = np.random.default_rng(phase_seed)
    co = prng.uniform(-1.0, 1.0, 10)
    ph = (co[0] + co[1] * X + co[2] * Y + co[3] * Z + co[4] * X * Y + co[5] * Y * Z + co[6] * X * Z
          + co[7] * X ** 2 + co[8] * Y ** 2 + co[9] * Z ** 2)
    return (mag * np.exp(1j * np.pi * 0.5 * ph)).astype(np.complex64)


def coil_maps(img, n_ch, seed=4):
    rng = np.random.default_rng(seed)
    axes = [np.linspace(-1, 1, n, endpoint=False) + 1.0 / n for n in img]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    maps = np.zeros((n_ch,) + tuple(img), np.complex64)
    for c in range(n_ch):
        ang = 2 * np.pi * c / n_ch
        cz = 0.5 * ((c % 2) * 2 - 1) if n_ch > 4 else 0.0
        cx, cy = 1.3 * np.cos(ang), 1.3 * np.sin(ang)
        g = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) / (2 * 0.8 ** 2))
        ph = rng.uniform(-np.pi, np.pi) + 0.5 * (X * np.cos(ang) + Y * np.sin(ang))
        maps[c] = (g * np.exp(1j * ph)).astype(np.complex64)
    rss = np.sqrt(np.sum(np.abs(maps) ** 2, axis=0))
    maps /= rss[None]
    return maps.astype(np.complex64)


# ---------------------------------------------------------------------------
# trajectory
# ---------------------------------------------------------------------------

@dataclass
class WaveParams:
    """Six wave parameters (per axis amplitude in grid cells, phase in
    radians, gradient delay as a fraction of the readout)."""
    amp_y: float
    amp_z: float
    phase_y: float = 0.0
    phase_z: float = 0.0
    delay_y: float = 0.0
    delay_z: float = 0.0

    def vector(self):
        return np.array([self.amp_y, self.amp_z, self.phase_y, self.phase_z, self.delay_y, self.delay_z])


def readout_lines(w: Workload):
    """(ky, kz) base-line indices of the undersampled CAIPI pattern, in
    acquisition order (kz outer, ky inner)."""
    ry, rz = w.r
    ny, nz = w.img[1], w.img[2]
    lines = []
    for b, iz in enumerate(range(0, nz, rz)):
        shift = (b * w.caipi) % ry
        for iy in range(shift, ny, ry):
            lines.append((iy, iz))
    return np.array(lines, np.int64)


def wave_trajectory(w: Workload, wave: WaveParams | None = None, lines=None):
    """k[n_lines * n_read][3] in [0,1]^3, readout-major order."""
    wave = wave or WaveParams(w.wave_cells, w.wave_cells)
    if lines is None:
        lines = readout_lines(w)
    G = np.array(w.grid, np.float64)
    sig = G / np.array(w.img, np.float64)          # grid cells per Nyquist step
    n = w.n_read
    t = np.arange(n) / n
    ux = G[0] / 2 + (np.arange(n) - n / 2) * sig[0] * w.img[0] / n
    cyc = w.wave_cycles
    wy = wave.amp_y * np.sin(2 * np.pi * cyc * (t - wave.delay_y) + wave.phase_y)
    wz = wave.amp_z * np.cos(2 * np.pi * cyc * (t - wave.delay_z) + wave.phase_z)
    uy = G[1] / 2 + (lines[:, 0:1] - w.img[1] / 2) * sig[1] + wy[None, :]
    uz = G[2] / 2 + (lines[:, 1:2] - w.img[2] / 2) * sig[2] + wz[None, :]
    k = np.zeros((lines.shape[0], n, 3))
    k[..., 0] = ux[None, :] / (G[0] - 1)
    k[..., 1] = uy / (G[1] - 1)
    k[..., 2] = uz / (G[2] - 1)
    return k.reshape(-1, 3)


WAVE_PARAM_NAMES = ("amp_y", "amp_z", "phase_y", "phase_z", "delay_y", "delay_z")


def wave_jacobian(w: Workload, wave: WaveParams | None = None, lines=None):
    """dk/dtheta of wave_trajectory: [n_lines * n_read][3][6] for theta =
    (amp_y, amp_z, phase_y, phase_z, delay_y, delay_z); kx does not depend
    on theta."""
    wave = wave or WaveParams(w.wave_cells, w.wave_cells)
    if lines is None:
        lines = readout_lines(w)
    G = np.array(w.grid, np.float64)
    n = w.n_read
    t = np.arange(n) / n
    om = 2 * np.pi * w.wave_cycles
    py = om * (t - wave.delay_y) + wave.phase_y
    pz = om * (t - wave.delay_z) + wave.phase_z
    J = np.zeros((n, 3, 6))
    J[:, 1, 0] = np.sin(py) / (G[1] - 1)
    J[:, 1, 2] = wave.amp_y * np.cos(py) / (G[1] - 1)
    J[:, 1, 4] = -wave.amp_y * np.cos(py) * om / (G[1] - 1)
    J[:, 2, 1] = np.cos(pz) / (G[2] - 1)
    J[:, 2, 3] = -wave.amp_z * np.sin(pz) / (G[2] - 1)
    J[:, 2, 5] = wave.amp_z * np.sin(pz) * om / (G[2] - 1)
    return np.broadcast_to(J[None], (lines.shape[0], n, 3, 6)).reshape(-1, 3, 6)


def wave_from_vector(v):
    return WaveParams(*[float(a) for a in v])


def perturbed_wave(w: Workload, frac=0.05, seed=5):
    """Nominal wave parameters perturbed by up to `frac`: amplitudes by a
    relative frac, phases by frac radians, delays by frac of a wave period."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, 6) * frac
    nom = WaveParams(w.wave_cells, w.wave_cells)
    return WaveParams(nom.amp_y * (1 + u[0]), nom.amp_z * (1 + u[1]), u[2], u[3],
                      u[4] / w.wave_cycles, u[5] / w.wave_cycles)


def wave_param_scale(w: Workload):
    """Natural unit of each wave parameter (cells, cells, rad, rad, period,
    period): finite-difference steps are taken in these units."""
    return np.array([1.0, 1.0, 1.0, 1.0, 1.0 / w.wave_cycles, 1.0 / w.wave_cycles])


# ---------------------------------------------------------------------------
# respiratory bins
# ---------------------------------------------------------------------------

def breathing_bins(n_readouts, n_bins, tr=5e-3, period=4.0, jitter=0.1, seed=3, occ=(0.03, 0.12)):
    """Readout indices per bin.  Readouts are sorted by breathing amplitude
    and cut into consecutive chunks whose sizes ramp from occ[0] to occ[1]
    of all readouts (quantile bins with uneven occupancy)."""
    if n_bins == 1:
        return [np.arange(n_readouts)]
    rng = np.random.default_rng(seed)
    t = np.arange(n_readouts) * tr
    amp = np.sin(2 * np.pi * t / period) + jitter * rng.standard_normal(n_readouts)
    order = np.argsort(amp, kind="stable")
    lo, hi = occ
    # occupancies lo + (hi - lo) * s^p with p chosen so they sum to 1
    s = np.linspace(0.0, 1.0, n_bins)
    target = 1.0
    if lo * n_bins > target or hi * n_bins < target:
        frac = np.full(n_bins, 1.0 / n_bins)
    else:
        a, b = 1e-3, 1e3
        for _ in range(200):
            p = np.sqrt(a * b)
            tot = np.sum(lo + (hi - lo) * s ** p)
            if tot > target:
                a = p
            else:
                b = p
        frac = lo + (hi - lo) * s ** p
        frac /= frac.sum()
    # interleave sizes so neighbouring amplitudes do not all get small bins
    perm = np.random.default_rng(seed + 1).permutation(n_bins)
    frac = frac[perm]
    counts = np.floor(frac * n_readouts).astype(np.int64)
    counts[np.argmax(counts)] += n_readouts - counts.sum()
    edges = np.concatenate([[0], np.cumsum(counts)])
    return [np.sort(order[edges[b]:edges[b + 1]]) for b in range(n_bins)]


def bin_samples(readout_bins, n_read):
    """Sample indices (readout-major order) of each readout bin."""
    return [(r[:, None] * n_read + np.arange(n_read)[None, :]).reshape(-1) for r in readout_bins]


# ---------------------------------------------------------------------------
# density compensation
# ---------------------------------------------------------------------------

def radial_dcf(k, grid):
    """A smooth stand-in density weight: distance from the k-space centre in
    grid cells (used only where the Voronoi weights are not computed)."""
    G = np.asarray(grid, np.float64)
    u = k * (G - 1) - G / 2
    r = np.sqrt(np.sum(u ** 2, axis=1))
    d = (r + 1.0) / (r.max() + 1.0)
    return d.astype(np.float32)


def cap_dcf(d, q=99.0):
    """Caps Voronoi weights at the q-th percentile of the positive ones and
    renormalises to max 1.  The raw weights (estimateDensityV3D's definition)
    of one respiratory bin span five orders of magnitude (cfg3 bins: median
    ~2e-5 of the largest, 99th percentile ~2e-3): the few bounded cells next
    to the convex hull are huge.  With them the weighted normal equations are
    so ill-conditioned that 15 complex64 CG iterations end 8e-2 away from the
    FP64 solve (cap at the 99.9th percentile); capped at the 99th percentile
    the difference is 1.5e-6 (the reference's readout averaging: 2.5e-6)."""
    d = np.asarray(d, np.float32)
    pos = d[d > 0]
    if pos.size == 0:
        return d
    cap = np.percentile(pos, q)
    out = np.minimum(d, cap)
    return (out / out.max()).astype(np.float32)


def complex_noise(shape, snr, signal_rms, seed=2):
    rng = np.random.default_rng(seed)
    sigma = signal_rms / snr / np.sqrt(2.0)
    return ((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * sigma).astype(np.complex64)
