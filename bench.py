"""Benchmark of the GB300 CG-SENSE path (E^H D E applies/s; s per 16-bin 4D
reconstruction).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (default): the batched 4D reconstruction of 128x128x96 images on a
2x oversampled 256x256x192 grid, 12 coils, wave-CAIPI R=2x2 (+-5 cells,
8 cycles), 512 samples per readout, 16 respiratory bins of uneven occupancy,
15 CG iterations per bin, all bins in one graph-captured solve.  Synthetic,
seeded inputs (4d_lung_gb300/synth.py).

One step = one full 16-bin reconstruction; value = E^H D E applies per
second (bins x iterations per step / time per step).  With torchrun
(N > 1) the scan's bins are partitioned over the ranks (greedy by sample
count, 4d_lung_gb300/dist.py): every rank solves its bins, with no
collective on the data path, and the step time is the slowest rank's
(strong scaling: the total work is one scan whatever N).

Beside the headline the line carries the plain per-bin GPU form, the
per-iteration precision against the FP64 form, the differentiation form,
and the same solve with the Toeplitz-embedded operator ("toeplitz": the
exact normal operator, not the reference's gridded one; skip with
--no-toeplitz).

--impl reference times the reference's CPU implementation of the same
operator on the host cores: the oracle port (oracle/cgs_oracle.c, FP32,
OpenMP over coils like Reco.cpp:470,523), one E^H D E application of bin 0
per step.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "E^H D E applies/s; s per 16-bin 4D recon; chosen vs plain at <=1e-4 rel err"
UNIT = "applies/s"
STAGES = ["fwd_z", "fwd_y", "fwd_x", "interp", "spread", "adj_x", "adj_y", "adj_z"]
# the stages when the spreading runs fused with the adjoint x pass (variant 8)
STAGES_FUSED = ["fwd_z", "fwd_y", "fwd_x", "interp", "spread_adjx", "adj_y", "adj_z"]


def beatty_beta(w, sigma=2.0):
    return float(np.pi * np.sqrt(w ** 2 / sigma ** 2 * (sigma - 0.5) ** 2 - 0.8))


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# stage -> kernel family (the roofline's "kernel")
FAMILY = {"fwd_z": "k_fwd_z_pipe+k_adj_z_pipe", "adj_z": "k_fwd_z_pipe+k_adj_z_pipe",
          "fwd_y": "k_fft_strided_tma", "fwd_x": "k_fft_strided_tma", "adj_x": "k_fft_strided_tma",
          "adj_y": "k_fft_strided_tma", "interp": "k_interp", "spread": "k_spread",
          "spread_adjx": "k_spread_adjx"}


def traffic_record():
    """DRAM bytes (read + write) against algorithmic bytes of each kernel
    family in one application of the first two cfg3 bins, from an ncu capture
    small enough for a shared GPU (profiles/traffic.json); a run's traffic is
    its own algorithmic bytes times that ratio."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


class MemSampler:
    """Device memory in use (nvidia-smi memory.used, MiB) sampled every
    100 ms in the background; stop() returns the maximum in GiB."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="mem_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=memory.used", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        vals = []
        with open(self.path) as f:
            for line in f:
                try:
                    vals.append(float(line.strip()))
                except ValueError:
                    pass
        os.unlink(self.path)
        return max(vals) / 1024.0 if vals else None


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def scan_bins(synth, name, max_bins=0):
    """Sample indices of the workload's respiratory bins (the first max_bins)."""
    w = synth.WORKLOADS[name]
    lines = synth.readout_lines(w)
    sbins = synth.bin_samples(synth.breathing_bins(len(lines), w.n_bins), w.n_read)
    return sbins[:max_bins] if max_bins > 0 else sbins


def torch_copy_ms(torch, dev, stream, data, x, h_data, h_x):
    """Device times (ms) of PyTorch's upload of h_data and download into h_x
    (the end-to-end call's buffers), medians of three."""
    out = {}
    d_tmp = torch.empty_like(data)
    for name, f in (("upload", lambda: d_tmp.copy_(h_data, non_blocking=True)),
                    ("download", lambda: h_x.copy_(x, non_blocking=True))):
        t = []
        for _ in range(3):
            r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            r0.record(stream)
            f()
            r1.record(stream)
            torch.cuda.synchronize(dev)
            t.append(r0.elapsed_time(r1))
        out[name] = round(statistics.median(t), 3)
    del d_tmp
    return out


_HOST_BUFS = []


def host_buffer(cgs, torch, shape):
    """A complex64 host tensor in page-locked memory from the library's own
    allocator (cgs_alloc_host), the buffer a C-ABI caller hands to the
    host-buffer calls; kept until the process exits."""
    import ctypes as C
    n = int(np.prod(shape))
    p = cgs.lib().cgs_alloc_host(n * 8)
    if not p:
        raise MemoryError("cgs_alloc_host failed")
    _HOST_BUFS.append(p)
    a = np.ctypeslib.as_array((C.c_float * (2 * n)).from_address(p)).view(np.complex64).reshape(shape)
    a[...] = 0
    return torch.from_numpy(a)


def make_workload(cgs, synth, torch, name, device, stream_handle, dcf_kind="voronoi", max_bins=0, bin_subset=None):
    """The workload's context, data and weights.  bin_subset: the indices of
    the bins this process reconstructs (the multi-GPU bin partition), None
    for all."""
    w = synth.WORKLOADS[name]
    kb_w = 4.0
    kb_b = beatty_beta(kb_w)
    lines = synth.readout_lines(w)
    k = synth.wave_trajectory(w, lines=lines)
    sbins = scan_bins(synth, name, max_bins)
    if bin_subset is not None:
        sbins = [sbins[b] for b in bin_subset]
    smaps = synth.coil_maps(w.img, w.n_ch)
    # per-bin Voronoi weights (estimateDensityV3D, host C++), or the radial stand-in
    t0 = time.perf_counter()
    if dcf_kind == "voronoi":
        dcf = np.zeros(k.shape[0], np.float32)
        for idx in sbins:
            dcf[idx] = synth.cap_dcf(cgs.voronoi_dcf(k[idx]))
    elif dcf_kind == "radial":
        dcf = synth.radial_dcf(k, w.grid)
    else:
        dcf = None   # Pipe-Menon weights on the GPU once the bins are set
    dcf_s = time.perf_counter() - t0
    reco = cgs.Reco(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b, device=device)
    reco.set_stream(stream_handle)
    reco.set_trajectory(k)
    ns = k.shape[0]
    dev = torch.device("cuda", device)
    smaps_t = torch.from_numpy(smaps).to(dev)
    data = torch.zeros((w.n_ch, ns), dtype=torch.complex64, device=dev)
    full = torch.zeros((w.n_ch, ns), dtype=torch.complex64, device=dev)
    # k-space of each bin from its own (z-displaced) phantom: y = E(S x_b)
    for j, idx in enumerate(sbins):
        b = j if bin_subset is None else bin_subset[j]
        shift = w.z_shift_max * (b / max(w.n_bins - 1, 1))
        x_b = torch.from_numpy(synth.phantom(w.img, z_shift=shift)).to(dev)
        imgs = (smaps_t * x_b[None]).contiguous()
        reco.nufft_fwd_tensor(imgs, full)
        it = torch.from_numpy(np.asarray(idx, np.int64)).to(dev)
        data[:, it] = full[:, it]
    torch.cuda.synchronize(dev)
    rms = float(torch.sqrt(torch.mean(torch.abs(data) ** 2)).item())
    g = torch.Generator(device=dev)
    g.manual_seed(2)
    sigma = rms / 30.0 / np.sqrt(2.0)
    noise = torch.complex(torch.randn(data.shape, generator=g, device=dev),
                          torch.randn(data.shape, generator=g, device=dev)) * sigma
    data += noise
    reco.set_bins(sbins)
    if dcf is None:
        t0 = time.perf_counter()
        dcf = reco.pipe_menon_dcf(20)
        dcf_s = time.perf_counter() - t0
        for idx in sbins:   # the same per-bin cap as the Voronoi weights
            dcf[idx] = synth.cap_dcf(dcf[idx])
    reco.set_dcf(dcf)
    reco.set_smaps_tensor(smaps_t)
    return w, reco, data, sbins, smaps, dcf, k, kb_w, kb_b, dcf_s


def stage_bytes(w, sizes, support=None, matrix=None, y_listed=False, fused=False):
    """Algorithmic bytes of each stage of one E^H D E application over all
    bins: every stage reads its input and writes its output once.
    support = (listed columns, stored spreading tiles) per bin, from
    Reco.support_stats(): with sample-support pruning the x passes move only
    the listed (y, z) columns, the interpolation reads within them and the
    spreading stores only the listed tiles.  None: the full grid.
    matrix = (taps, points) of the transposed tap matrix when the spreading
    is its gather: it stores every point of its listed columns (its rows) and
    reads the row offsets (4 bytes per point), the taps (8 bytes each) and
    the coil values of the samples.  y_listed: the forward y pass stores only the
    listed columns' rows (8 bytes x Ix per listed column).  fused: the
    gather runs fused with the adjoint x pass (stage "spread_adjx"): the
    matrix and the samples are read, the x pass's Ix output rows written,
    the grid never stored or reloaded."""
    Ix, Iy, Iz = w.img
    Gx, Gy, Gz = w.grid
    Ni, Ng, Nl = Ix * Iy * Iz, Gx * Gy * Gz, Ix * Iy
    C8 = 8 * w.n_ch
    nb = len(sizes)
    M = int(sum(sizes))
    if support is None:
        cols = [Gy * Gz] * nb
        tiles = [Ng // 512] * nb
    else:
        cols, tiles = [int(v) for v in support[0]], [int(v) for v in support[1]]
    scol, stile = sum(cols), sum(tiles)
    if fused and matrix:
        sb = stage_bytes(w, sizes, support, matrix, y_listed)
        sb["spread_adjx"] = 4 * matrix[1] + 8 * matrix[0] + M * C8 + C8 * scol * Ix
        return {k: sb[k] for k in STAGES_FUSED}
    return {
        # the coil maps once per application: the z passes run the bins of a
        # line block side by side, so the other bins read the maps from L2
        "fwd_z": nb * (8 * Ni + C8 * Nl * Gz) + C8 * Ni,
        "fwd_y": C8 * (nb * Nl * Gz + Ix * scol) if y_listed else nb * C8 * (Nl * Gz + Ix * Gy * Gz),
        "fwd_x": C8 * scol * (Ix + Gx),
        "interp": C8 * scol * Gx + M * (64 + 4 + C8),
        "spread": (C8 * matrix[1] + 4 * matrix[1] + 8 * matrix[0] + M * C8) if matrix
        else C8 * stile * 512 + M * (64 + C8),   # tiled kernels: 4 x 8 x 16 points per tile
        "adj_x": C8 * scol * (Gx + Ix),
        "adj_y": nb * C8 * (Ix * Gy * Gz + Nl * Gz),
        "adj_z": nb * (C8 * Nl * Gz + 8 * Ni) + C8 * Ni,
    }


def apply_bytes(w, sizes, support=None, matrix=None, y_listed=False, fused=False):
    """Algorithmic bytes of one application of the operator (its eight
    stages, seven fused; the CG vector updates of a solve, 64 bytes per voxel
    and bin and iteration, are not part of it)."""
    return sum(stage_bytes(w, sizes, support, matrix, y_listed, fused).values())


# ---------------------------------------------------------------------------
# CPU baseline (oracle port)
# ---------------------------------------------------------------------------

def cpu_apply_sample(synth, name, budget_s=12.0, max_reps=3, warmup=0, all_bins=False):
    """The FP32 oracle port (the reference's arithmetic, OpenMP over coils)
    on the host cores.  all_bins: a step is one E^H D E application of every
    bin of the scan (the unit the GPU arm's value counts), else one
    application of the bin whose size is the median of the scan's.  At most
    max_reps timed steps, fewer when budget_s runs out."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    o = oracle_py.Oracle(32)
    w = synth.WORKLOADS[name]
    kb_w = 4.0
    lines = synth.readout_lines(w)
    k = synth.wave_trajectory(w, lines=lines)
    rbins = synth.breathing_bins(len(lines), w.n_bins)
    sbins = synth.bin_samples(rbins, w.n_read)
    sizes = [len(b) for b in sbins]
    order = np.argsort(sizes, kind="stable")
    chosen = list(range(len(sbins))) if all_bins else [int(order[len(order) // 2])]
    p = oracle_py.make_params(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=beatty_beta(kb_w))
    kft = o.kernel_ft(p)                     # ConvKernel::calculateKernelFT (set-up)
    prep = []
    for b in chosen:
        kb = k[sbins[b]]
        prep.append((o.taps(p, kb), synth.radial_dcf(kb, w.grid)))   # calculateWeights (set-up)
    smaps = synth.coil_maps(w.img, w.n_ch)
    x = synth.phantom(w.img)

    def step():
        for taps, dcf in prep:
            o.apply_ehde(p, taps, kft, smaps, dcf, x)

    for _ in range(warmup):
        step()
    times = []
    t_all = time.perf_counter()
    while len(times) < max_reps:
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget_s:
            break
    what = ("one E^H D E application of each of the %d bins (%d samples in all)" % (len(chosen), sum(sizes))
            if all_bins else "E^H D E applications of the median-size bin %d (%d samples)" % (chosen[0], sizes[chosen[0]]))
    return {
        "times": times, "threads": threads, "applies_per_step": len(chosen),
        "samples_in_bin": int(sizes[chosen[0]]),
        "sample": "%s, %d coils, %s grid, %d timed" % (what, w.n_ch, "x".join(map(str, w.grid)), len(times)),
    }


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    synth = importlib.import_module("4d_lung_gb300.synth")
    w = synth.WORKLOADS[args.workload]
    res = cpu_apply_sample(synth, args.workload, budget_s=1e9, max_reps=args.steps, warmup=args.warmup,
                           all_bins=True)
    t = res["times"]
    value = res["applies_per_step"] * len(t) / sum(t)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(t), "warmup": args.warmup, "ms_per_step": 1e3 * sum(t) / len(t),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "c64/f32",
        "data": "synthetic", "config": {"workload": w.name, "bins": w.n_bins, "cg_iters": w.cg_iters,
                                        "step": "one E^H D E application of every bin of the scan on the "
                                                "host cores (the GPU arm's unit: bin-applies)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["threads"], "kind": "port",
                         "sample": res["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "s_per_4d_recon_extrapolated": w.cg_iters * sum(t) / len(t),
    }
    print(json.dumps(line), flush=True)
    return 0


def precision_report(reco, data, x, iters, torch, dev):
    """Relative L2 error of x after every CG iteration against the FP64 GPU
    form (max over bins), for plain and compensated FP32 spreading."""
    nb = x.shape[0]
    t64 = torch.zeros((iters,) + tuple(x.shape), dtype=torch.complex128, device=dev)
    x64 = torch.zeros(x.shape, dtype=torch.complex128, device=dev)
    t0 = time.perf_counter()
    reco.cg_sense_fp64_tensor(data, x64, 0.0, iters, t64)
    torch.cuda.synchronize(dev)
    t_fp64 = time.perf_counter() - t0
    out = {"reference": "full-FP64 GPU form (cuFFT Z2Z, FP64 gridding, vectors and scalars)",
           "fp64_s_per_recon": t_fp64}
    for name, comp in (("fp32", False), ("compensated", True)):
        reco.set_precision(comp)
        tr = torch.zeros((iters,) + tuple(x.shape), dtype=torch.complex64, device=dev)
        xx = torch.zeros_like(x)
        reco.cg_sense_trace_tensor(data, xx, 0.0, iters, tr)
        torch.cuda.synchronize(dev)
        errs = []
        for it in range(iters):
            d = (tr[it].to(torch.complex128) - t64[it]).reshape(nb, -1)
            e = torch.linalg.vector_norm(d, dim=1) / torch.linalg.vector_norm(t64[it].reshape(nb, -1), dim=1)
            errs.append(float(e.max()))
        out["rel_l2_per_iter_" + name] = errs
        del tr
        if comp:
            # the compensated form's own speed: its graph-captured batched
            # solve, timed like the headline (warm-up replays, then events)
            stream = torch.cuda.current_stream(dev)
            xx.zero_()
            for _ in range(3):
                reco.cg_sense_batched_tensor(data, xx, 0.0, iters, want_stats=False)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            reps = 5
            torch.cuda.synchronize(dev)
            e0.record(stream)
            for _ in range(reps):
                reco.cg_sense_batched_tensor(data, xx, 0.0, iters, want_stats=False)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) / reps
            out["compensated_s_per_recon"] = ms / 1e3
            out["compensated_applies_per_s"] = nb * iters / (ms / 1e3)
        del xx
    reco.set_precision(False)
    out["max_rel_l2_fp32"] = max(out["rel_l2_per_iter_fp32"])
    out["max_rel_l2_compensated"] = max(out["rel_l2_per_iter_compensated"])
    del t64
    return out


def differentiation_report(cgs, synth, torch, dev, stream_handle, steps=50):
    """cfg4 differentiation form: 128x128x96 image, 12 coils, one bin of
    1.57 M wave-CAIPI samples, the reference's KB kernel (w = 4.25,
    b = 14.9086); wave parameters perturbed by up to 5 % from nominal.
    dL/dtheta of L = 1/2 |E(theta) x - y|^2 from the FP32 libtorch operator,
    the FP64 reference gradient and central finite differences of the FP64
    loss (step 1e-3 in the parameters' natural units); the time of one loss
    + gradient evaluation; `steps` Adam steps of trajectory self-calibration."""
    ag = importlib.import_module("4d_lung_gb300.autograd")
    w = synth.WORKLOADS["cfg4"]
    lines = synth.readout_lines(w)
    kb_w, kb_b = 4.25, 14.9086
    reco = cgs.Reco(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b, device=dev.index or 0)
    reco.set_stream(stream_handle)
    v_true = torch.tensor([w.wave_cells, w.wave_cells, 0, 0, 0, 0], dtype=torch.float64, device=dev)
    k_true = ag.wave_trajectory_torch(w, v_true, lines).contiguous()
    reco.set_trajectory(k_true.cpu().numpy())
    smaps = torch.from_numpy(synth.coil_maps(w.img, w.n_ch)).to(dev)
    reco.set_smaps_tensor(smaps)
    x = torch.from_numpy(synth.phantom(w.img)).to(dev)
    y = torch.zeros((w.n_ch, k_true.shape[0]), dtype=torch.complex64, device=dev)
    reco.nufft_fwd_tensor((smaps * x[None]).contiguous(), y)
    torch.cuda.synchronize(dev)
    rms = float(torch.sqrt(torch.mean(torch.abs(y) ** 2)))
    g = torch.Generator(device=dev)
    g.manual_seed(2)
    y += torch.complex(torch.randn(y.shape, generator=g, device=dev),
                       torch.randn(y.shape, generator=g, device=dev)) * (rms / 30 / np.sqrt(2))
    th = synth.perturbed_wave(w)
    v0 = np.array([th.amp_y, th.amp_z, th.phase_y, th.phase_z, th.delay_y, th.delay_z])
    sc = synth.wave_param_scale(w)
    x64 = x.to(torch.complex128)

    def loss64(vec, grad=False):
        k = ag.wave_trajectory_torch(w, torch.tensor(vec, dtype=torch.float64, device=dev), lines).contiguous()
        reco.update_trajectory_tensor(k)
        gk = torch.zeros((k.shape[0], 3), dtype=torch.float64, device=dev) if grad else None
        return reco.loss_grad_fp64_tensor(x64, y, None, gk), gk

    L64, gk64 = loss64(v0, grad=True)
    g64 = np.einsum("ia,iam->m", gk64.cpu().numpy(), synth.wave_jacobian(w, th, lines=lines))
    fd = np.zeros(6)
    for m in range(6):
        h = 1e-3 * sc[m]
        vp, vm = v0.copy(), v0.copy()
        vp[m] += h
        vm[m] -= h
        fd[m] = (loss64(vp)[0] - loss64(vm)[0]) / (2 * h)
    # FP32 operator: loss, dL/dx and dL/dtheta through autograd; timed
    times = []
    for rep in range(6):
        v = torch.tensor(v0, dtype=torch.float64, device=dev, requires_grad=True)
        xr = x.clone().requires_grad_(True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        loss = ag.dc_loss(reco, xr, ag.wave_trajectory_torch(w, v, lines).contiguous(), y)
        loss.backward()
        e1.record()
        torch.cuda.synchronize(dev)
        if rep > 0:
            times.append(e0.elapsed_time(e1))
    g32 = v.grad.cpu().numpy()
    # self-calibration (image known): Adam on theta / scale
    scale = torch.tensor(sc, dtype=torch.float64, device=dev)
    u = (torch.tensor(v0, dtype=torch.float64, device=dev) / scale).requires_grad_(True)
    opt = torch.optim.Adam([u], lr=0.01)
    G = torch.tensor(w.grid, dtype=torch.float64, device=dev) - 1

    def traj_err(uu):
        k = ag.wave_trajectory_torch(w, uu * scale, lines)
        return float(torch.sqrt(torch.mean(torch.sum(((k - k_true) * G) ** 2, dim=1))))

    hist_loss, hist_err = [], [traj_err(u.detach())]
    t0 = time.perf_counter()
    for _ in range(steps):
        opt.zero_grad()
        loss = ag.dc_loss(reco, x, ag.wave_trajectory_torch(w, u * scale, lines).contiguous(), y)
        loss.backward()
        opt.step()
        hist_loss.append(loss.item())
        hist_err.append(traj_err(u.detach()))
    t_cal = time.perf_counter() - t0
    del reco
    return {
        "workload": w.name, "samples": int(k_true.shape[0]), "coils": w.n_ch, "kb_w": kb_w, "kb_b": kb_b,
        "theta0": v0.tolist(), "params": list(synth.WAVE_PARAM_NAMES),
        "dL_dtheta_fp32": g32.tolist(), "dL_dtheta_fp64": g64.tolist(), "dL_dtheta_fd_fp64": fd.tolist(),
        "fd_step": "1e-3 in natural units (cells, rad, wave periods)",
        "rel_err_fp64_vs_fd": (np.abs(g64 - fd) / np.abs(fd)).tolist(),
        "rel_err_fp32_vs_fp64": (np.abs(g32 - g64) / np.abs(g64)).tolist(),
        "rel_err_fp32_vs_fd": (np.abs(g32 - fd) / np.abs(fd)).tolist(),
        "ms_loss_grad_x_theta": float(np.median(times)),
        "calibration": {"steps": steps, "optimizer": "Adam lr 0.01 on theta / natural unit", "s_total": t_cal,
                        "loss_first_last": [hist_loss[0], hist_loss[-1]],
                        "traj_rms_err_cells_first_last": [hist_err[0], hist_err[-1]],
                        "traj_rms_err_cells": hist_err[:: max(1, steps // 10)]},
    }


def toeplitz_report(reco, synth, data, x, iters, torch, dev, stream, steps, w, sizes):
    """The same batched solve with the Toeplitz embedding of E^H D E
    (cgs_set_toeplitz): the spectra's build time, the timed reconstruction,
    the per-stage times of one application and its images against the
    gridded solve's (the operators differ by the gridding error).  The
    library is left on the gridded operator."""
    nb = len(sizes)
    reco.set_toeplitz(1)
    try:
        build_ms, pbytes = reco.toeplitz_stats()
        xt = torch.zeros_like(x)
        for _ in range(3):
            reco.cg_sense_batched_tensor(data, xt, 0.0, iters, want_stats=False)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            reco.cg_sense_batched_tensor(data, xt, 0.0, iters, want_stats=False)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        res, its = reco.cg_sense_batched_tensor(data, xt, 0.0, iters, want_stats=True)
        launches = reco.launch_count()
        rel = float(torch.linalg.vector_norm(xt - x) / torch.linalg.vector_norm(x))
        xa = torch.from_numpy(np.stack([synth.phantom(w.img)] * nb)).to(dev)
        qa = torch.empty_like(xa)
        reps = [reco.profile_apply_tensor(xa, qa, 0, nb) for _ in range(5)]
        st = np.median(np.stack(reps), axis=0)
        names = ["fwd_z", "fwd_y", "toep_x", "adj_y", "adj_z"]
        groups = len(st) // len(names)
        stage_ms = {s: float(sum(st[g * len(names) + i] for g in range(groups))) for i, s in enumerate(names)}
        sb = stage_bytes(w, sizes)
        Ix, Gy, Gz = w.img[0], w.grid[1], w.grid[2]
        ng = int(np.prod(w.grid))
        tb = {"fwd_z": sb["fwd_z"], "fwd_y": sb["fwd_y"], "adj_y": sb["adj_y"], "adj_z": sb["adj_z"],
              "toep_x": nb * (2 * 8 * w.n_ch * Ix * Gy * Gz + 4 * ng)}
        peak, _ = measured_peaks()
        apply_ms = float(sum(stage_ms.values()))
        return {
            "operator": "Toeplitz embedding: crop F_c^H (P_b . F_c pad(S_c x)), P_b the real spectrum of bin b's "
                        "point-spread function (exact normal operator; no gridding inside CG)",
            "spectra_build_s": build_ms / 1e3, "spectra_bytes": pbytes,
            "s_per_4d_recon": ms / 1e3, "applies_per_s": nb * iters / (ms / 1e3),
            "launches_per_recon": launches,
            "iters": [int(v) for v in its],
            # None for a bin whose initial residual is zero (an empty bin), so
            # that it cannot pass for a solve that converged
            "final_residual_rel": [float(r[-1] / r[0]) if r[0] > 0 else None for r in res],
            "rel_l2_vs_gridded_solve": rel,
            "apply_ms": apply_ms, "stage_ms": stage_ms,
            "stage_frac_of_peak": {s: tb[s] / (stage_ms[s] / 1e3) / 1e9 / peak for s in stage_ms},
            "apply_achieved_gbs": sum(tb.values()) / (apply_ms / 1e3) / 1e9,
        }
    finally:
        reco.set_toeplitz(0)


def pipe_menon_report(reco, synth, data, x, iters, sbins, dcf_voronoi, torch, dev, stream, steps):
    """The headline solve with GPU Pipe-Menon density weights (20 iterations
    per bin on the library's own gridding kernels, capped at each bin's 99th
    percentile like the Voronoi volumes) in place of the host Voronoi
    volumes: their set-up time, the timed reconstruction and the images'
    distance from the Voronoi solve's.  The Voronoi weights are restored."""
    t0 = time.perf_counter()
    pm = reco.pipe_menon_dcf(20)
    for idx in sbins:
        pm[idx] = synth.cap_dcf(pm[idx])
    pm_s = time.perf_counter() - t0
    try:
        reco.set_dcf(pm)
        xp = torch.zeros_like(x)
        for _ in range(2):
            reco.cg_sense_batched_tensor(data, xp, 0.0, iters, want_stats=False)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            reco.cg_sense_batched_tensor(data, xp, 0.0, iters, want_stats=False)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        d = (xp - x).reshape(len(sbins), -1)
        per_bin = (torch.linalg.vector_norm(d, dim=1) / torch.linalg.vector_norm(x.reshape(len(sbins), -1), dim=1))
        # each solve against its bin's phantom (best complex scale): how far
        # either weighting's 15-iteration image is from the truth
        w = synth.WORKLOADS["cfg3"]
        err_v, err_p = [], []
        for b in range(len(sbins)):
            xt = torch.from_numpy(synth.phantom(w.img, z_shift=w.z_shift_max * b / max(w.n_bins - 1, 1))).to(dev)
            for img, out in ((x[b], err_v), (xp[b], err_p)):
                a = torch.vdot(img.reshape(-1), xt.reshape(-1)) / torch.vdot(img.reshape(-1), img.reshape(-1))
                out.append(float(torch.linalg.vector_norm(a * img - xt) / torch.linalg.vector_norm(xt)))
        return {"dcf": "Pipe-Menon, 20 iterations per bin on the GPU, capped at the 99th percentile",
                "dcf_s": pm_s, "s_per_4d_recon": ms / 1e3,
                "rel_l2_vs_voronoi_solve": float(torch.linalg.vector_norm(xp - x) / torch.linalg.vector_norm(x)),
                "rel_l2_vs_voronoi_solve_per_bin_max": float(per_bin.max()),
                "rel_l2_vs_phantom_median": {"voronoi": float(np.median(err_v)), "pipe_menon": float(np.median(err_p))},
                "rel_l2_vs_phantom_per_bin": {"voronoi": [round(v, 4) for v in err_v],
                                              "pipe_menon": [round(v, 4) for v in err_p]}}
    finally:
        reco.set_dcf(dcf_voronoi)


def cfg1_report(cgs, synth, torch, dev, stream, steps=5, with_cpu=True):
    """The reference's CPU-path configuration at its full size: a 64^3 image on
    the 2x oversampled 128^3 grid, 8 coils, 1024 wave-CAIPI readouts of 256
    samples (262 144 samples, R = 2x2, +-4 cells, 7 cycles), Voronoi density
    weights (capped at their 99th percentile), KB width 4, 10 CG iterations.
    GPU: the graph-captured solve (device-timed) and its host-buffer C-ABI
    call.  CPU: the FP32 oracle port (the reference's arithmetic, OpenMP over
    coils as Reco.cpp:470,523) on all host cores -- one E^H D E application
    and the full 10-iteration solve, with its residual sequence -- and the
    relative L2 distance between the two images."""
    import ctypes as C
    w = synth.WORKLOADS["cfg1"]
    kb_w = 4.0
    kb_b = beatty_beta(kb_w)
    k = synth.wave_trajectory(w)
    t0 = time.perf_counter()
    dcf = synth.cap_dcf(cgs.voronoi_dcf(k))
    dcf_s = time.perf_counter() - t0
    smaps = synth.coil_maps(w.img, w.n_ch)
    x_true = synth.phantom(w.img)
    reco = cgs.Reco(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b, device=dev.index or 0)
    reco.set_stream(stream.cuda_stream)
    reco.set_trajectory(k)
    smaps_t = torch.from_numpy(smaps).to(dev)
    y = torch.zeros((w.n_ch, k.shape[0]), dtype=torch.complex64, device=dev)
    reco.nufft_fwd_tensor((smaps_t * torch.from_numpy(x_true).to(dev)[None]).contiguous(), y)
    torch.cuda.synchronize(dev)
    rms = float(torch.sqrt(torch.mean(torch.abs(y) ** 2)))
    g = torch.Generator(device=dev)
    g.manual_seed(2)
    y += torch.complex(torch.randn(y.shape, generator=g, device=dev),
                       torch.randn(y.shape, generator=g, device=dev)) * (rms / 30 / np.sqrt(2))
    reco.set_dcf(dcf)
    reco.set_smaps_tensor(smaps_t)
    iters = w.cg_iters
    x = torch.zeros((1,) + w.img, dtype=torch.complex64, device=dev)
    for _ in range(3):
        res, its = reco.cg_sense_batched_tensor(y, x, 0.0, iters, want_stats=True)
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        reco.cg_sense_batched_tensor(y, x, 0.0, iters, want_stats=False)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    gpu_s = e0.elapsed_time(e1) / 1e3 / steps
    # host buffers through the C ABI (copies and the result read back included)
    h_y = torch.empty(y.shape, dtype=torch.complex64, pin_memory=True)
    h_y.copy_(y.cpu())
    h_x = torch.zeros(x.shape, dtype=torch.complex64, pin_memory=True)
    h_res = np.zeros((1, iters), np.float64)
    h_it = np.zeros(1, np.int32)
    L = cgs.lib()

    def host_call():
        st = L.cgs_cg_solve_batched(reco.ctx, C.c_void_p(h_y.data_ptr()), C.c_void_p(h_x.data_ptr()), 0.0, iters,
                                    h_res.ctypes.data_as(C.c_void_p), h_it.ctypes.data_as(C.c_void_p))
        if st != 0:
            raise RuntimeError(L.cgs_last_error(reco.ctx).decode())

    host_call()
    t0 = time.perf_counter()
    for _ in range(steps):
        host_call()
    e2e_s = (time.perf_counter() - t0) / steps
    out = {"workload": w.name, "img": list(w.img), "grid": list(w.grid), "coils": w.n_ch,
           "samples": int(k.shape[0]), "cg_iters": iters, "kb_w": kb_w, "kb_b": round(kb_b, 4),
           "dcf": "Voronoi volumes capped at the 99th percentile (host, %.1f s)" % dcf_s,
           "gpu_s_per_solve": gpu_s, "gpu_applies_per_s": iters / gpu_s,
           "gpu_e2e_s_per_solve": e2e_s, "gpu_residuals": [float(v) for v in res[0, :iters]],
           "setup_ms": reco.setup_stats()}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py
        o = oracle_py.Oracle(32)
        p = oracle_py.make_params(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b)
        yh = y.cpu().numpy()
        t0 = time.perf_counter()
        taps = o.taps(p, k)                 # ConvKernel::calculateWeights
        kft = o.kernel_ft(p)                # ConvKernel::calculateKernelFT
        t_setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        o.apply_ehde(p, taps, kft, smaps, dcf, x_true)
        t_apply = time.perf_counter() - t0
        t0 = time.perf_counter()
        st, xc, resc, itc = o.cg_sense(p, taps, kft, smaps, dcf, yh, 0.0, iters)
        t_solve = time.perf_counter() - t0
        xg = x.cpu().numpy()[0].astype(np.complex128)
        out["cpu"] = {"kind": "port", "cores": os.cpu_count() or 1,
                      "what": "FP32 oracle port of Reco.cpp (taps, kernelFT, nufftFWD/BWD, cgSenseDynamic), "
                              "OpenMP over coils, the project's mixed-radix FFT",
                      "s_setup_taps_kernelft": t_setup, "s_per_apply": t_apply, "s_per_solve": t_solve,
                      "iters": int(itc), "residuals": [float(v) for v in resc],
                      "rel_l2_gpu_vs_cpu": float(np.linalg.norm(xg - xc) / np.linalg.norm(xc)),
                      "gpu_speedup_per_solve": t_solve / gpu_s}
    del reco
    return out


def cfg2_precision_report(cgs, synth, torch, dev, stream):
    """The precision configuration (160x160x112 image, 320x320x224 grid, 16
    coils, R = 3x2 wave-CAIPI, 640 samples per readout, 20 CG iterations):
    per-iteration relative L2 error of the FP32 and the compensated solves
    against the FP64 GPU solve.  D: Pipe-Menon weights on the GPU (the host
    Voronoi volumes of these 1.9 M samples take minutes), capped at their
    99th percentile."""
    w, reco, data, sbins, smaps, dcf, k, kb_w, kb_b, dcf_s = make_workload(
        cgs, synth, torch, "cfg2", dev.index or 0, stream.cuda_stream, "pipe-menon")
    x = torch.zeros((len(sbins),) + w.img, dtype=torch.complex64, device=dev)
    rep = precision_report(reco, data, x, w.cg_iters, torch, dev)
    rep.update({"workload": w.name, "img": list(w.img), "grid": list(w.grid), "coils": w.n_ch,
                "samples": int(sum(len(s) for s in sbins)), "cg_iters": w.cg_iters, "kb_w": kb_w,
                "kb_b": round(kb_b, 4), "dcf": "Pipe-Menon (GPU, %.2f s), capped at the 99th percentile" % dcf_s})
    del reco, data, x
    return rep


def run_diff_only(args):
    """The differentiation form alone (cfg4), one JSON line."""
    import torch
    cgs = importlib.import_module("4d_lung_gb300")
    synth = importlib.import_module("4d_lung_gb300.synth")
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    rep = differentiation_report(cgs, synth, torch, dev, stream.cuda_stream)
    print(json.dumps({"metric": "dL/dtheta vs FD and FP64; self-calibration", "differentiation": rep}), flush=True)
    return 0


def run_cg_grad_only(args):
    """Combined large workload (cfg5: 256x256x176 image, 512x512x352 grid, 20
    coils, R = 3x2 wave-CAIPI +-8 cells / 11 cycles, 1024 samples per
    readout, 24 breathing bins): a 10-iteration CG of all bins unrolled in
    PyTorch over the library's operators, every iteration checkpointed, and
    the gradient of L = 1/2 sum_b |x_b(theta) - x_true,b|^2 with respect to
    the six wave parameters.  D is the radial stand-in (per-bin Voronoi
    weights of 7.7 M samples take minutes on the host).  One JSON line:
    forward / backward seconds, device memory, the gradient."""
    import torch
    cgs = importlib.import_module("4d_lung_gb300")
    synth = importlib.import_module("4d_lung_gb300.synth")
    ag = importlib.import_module("4d_lung_gb300.autograd")
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    name = args.workload if args.workload != "cfg3" else "cfg5"
    w = synth.WORKLOADS[name]
    kb_w, kb_b = 4.0, beatty_beta(4.0)
    lines = synth.readout_lines(w)
    sbins = synth.bin_samples(synth.breathing_bins(len(lines), w.n_bins), w.n_read)
    budget = int(args.workspace_gb * (1 << 30))
    reco = cgs.Reco(w.img, w.grid, w.n_ch, kb_w=kb_w, kb_b=kb_b, workspace_bytes=budget)
    reco.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    v_nom = torch.tensor([w.wave_cells, w.wave_cells, 0, 0, 0, 0], dtype=torch.float64, device=dev)
    k_nom = ag.wave_trajectory_torch(w, v_nom, lines).contiguous()
    k_np = k_nom.cpu().numpy()
    reco.set_trajectory(k_np)
    reco.set_dcf(synth.radial_dcf(k_np, w.grid))
    smaps = torch.from_numpy(synth.coil_maps(w.img, w.n_ch)).to(dev)
    reco.set_smaps_tensor(smaps)
    ns = k_np.shape[0]
    y = torch.zeros((w.n_ch, ns), dtype=torch.complex64, device=dev)
    full = torch.zeros_like(y)
    xs = []
    for b, idx in enumerate(sbins):
        x_b = torch.from_numpy(synth.phantom(w.img, z_shift=w.z_shift_max * b / max(w.n_bins - 1, 1))).to(dev)
        xs.append(x_b.reshape(-1))
        reco.nufft_fwd_tensor((smaps * x_b[None]).contiguous(), full)
        it = torch.from_numpy(np.asarray(idx, np.int64)).to(dev)
        y[:, it] = full[:, it]
    del full
    reco.set_bins(sbins)
    x_true = torch.stack(xs)
    torch.cuda.synchronize(dev)
    t_setup = time.perf_counter() - t0
    th = synth.perturbed_wave(w)
    v = torch.tensor([th.amp_y, th.amp_z, th.phase_y, th.phase_z, th.delay_y, th.delay_z], dtype=torch.float64,
                     device=dev, requires_grad=True)
    torch.cuda.reset_peak_memory_stats(dev)
    mem = MemSampler(0)
    mem.start()
    t0 = time.perf_counter()
    k = ag.wave_trajectory_torch(w, v, lines).contiguous()
    xk = ag.cg_unrolled(reco, k, y, w.cg_iters, checkpoint=True)
    loss = 0.5 * torch.sum(torch.abs(xk.to(torch.complex128) - x_true.to(torch.complex128)) ** 2)
    torch.cuda.synchronize(dev)
    t_fwd = time.perf_counter() - t0
    free_fwd, total = torch.cuda.mem_get_info(dev)
    t0 = time.perf_counter()
    loss.backward()
    torch.cuda.synchronize(dev)
    t_bwd = time.perf_counter() - t0
    free, total = torch.cuda.mem_get_info(dev)
    peak_smi = mem.stop()
    line = {"metric": "unrolled CG trajectory gradient (checkpointed backward)", "workload": w.name,
            "config": {"img": list(w.img), "grid": list(w.grid), "coils": w.n_ch, "bins": len(sbins),
                       "samples": int(ns), "cg_iters": w.cg_iters, "kb_w": kb_w, "kb_b": round(kb_b, 4),
                       "dcf": "radial stand-in", "workspace_gb": args.workspace_gb,
                       "checkpoint": "every CG iteration (x, r, p, rr saved; the rest recomputed)"},
            "s_setup": t_setup, "s_forward": t_fwd, "s_backward": t_bwd, "loss": float(loss.item()),
            "dL_dtheta": v.grad.cpu().numpy().tolist(), "params": list(synth.WAVE_PARAM_NAMES),
            "device_gb_in_use_after_forward": (total - free_fwd) / 2 ** 30,
            "device_gb_in_use_end": (total - free) / 2 ** 30,
            "device_gb_peak_sampled": peak_smi,
            "torch_peak_gb": torch.cuda.max_memory_allocated(dev) / 2 ** 30,
            "budget_gb": 180.0}
    line["fits_in_budget"] = all(v is None or v <= 180.0 for v in
                                 (line["device_gb_peak_sampled"], line["device_gb_in_use_after_forward"],
                                  line["device_gb_in_use_end"]))
    print(json.dumps(line), flush=True)
    return 0


def run_precision_only(args):
    """Precision form of a workload (cfg2: 160x160x112, 16 coils, 20 CG
    iterations): per-iteration relative L2 error of the FP32 and the
    compensated-spreading solves against the FP64 GPU solve; one JSON line."""
    import torch
    cgs = importlib.import_module("4d_lung_gb300")
    synth = importlib.import_module("4d_lung_gb300.synth")
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    w, reco, data, sbins, smaps, dcf, k, kb_w, kb_b, dcf_s = make_workload(
        cgs, synth, torch, args.workload, 0, stream.cuda_stream, args.dcf)
    x = torch.zeros((len(sbins),) + w.img, dtype=torch.complex64, device=dev)
    rep = precision_report(reco, data, x, w.cg_iters, torch, dev)
    line = {"metric": "rel L2 vs FP64 per CG iteration (max over bins)", "workload": w.name,
            "config": {"img": list(w.img), "grid": list(w.grid), "coils": w.n_ch, "bins": len(sbins),
                       "samples": int(sum(len(s) for s in sbins)), "cg_iters": w.cg_iters, "kb_w": kb_w,
                       "kb_b": round(kb_b, 4), "dcf": args.dcf}, "precision": rep}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    import torch.distributed as dist

    cgs = importlib.import_module("4d_lung_gb300")
    synth = importlib.import_module("4d_lung_gb300.synth")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if not os.path.exists(cgs.LIB_PATH):
        raise RuntimeError("libcgsense.so missing: run __graft_entry__.build() first")

    # all library work and the timing events on one dedicated stream
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    # pinned host buffers of the end-to-end call, allocated and touched before
    # the host-side set-up (the Voronoi weights allocate and free gigabytes on
    # all cores); allocated after it, the end-to-end step measured 5 ms slower
    w0 = synth.WORKLOADS[args.workload]
    ns0 = len(synth.readout_lines(w0)) * w0.n_read
    # N GPUs: the scan's bins are partitioned over the ranks (greedy by sample
    # count); every rank solves its own bins, no collective on the data path
    all_sizes = [len(b) for b in scan_bins(synth, args.workload, args.max_bins)]
    mine = None
    if world > 1:
        mine = importlib.import_module("4d_lung_gb300.dist").partition_bins(all_sizes, world)[rank]
    nb0 = len(all_sizes) if mine is None else len(mine)
    h_data = host_buffer(cgs, torch, (w0.n_ch, ns0))
    h_x = host_buffer(cgs, torch, (max(nb0, 1),) + tuple(w0.img))
    w, reco, data, sbins, smaps, dcf, k, kb_w, kb_b, dcf_s = make_workload(
        cgs, synth, torch, args.workload, local, stream.cuda_stream, args.dcf, args.max_bins, mine)
    assert tuple(h_data.shape) == tuple(data.shape) and (h_x.shape[0] == len(sbins) or not sbins)
    torch.cuda.synchronize(dev)
    nb = len(sbins)
    sizes = [len(s) for s in sbins]
    x = torch.zeros((nb,) + w.img, dtype=torch.complex64, device=dev)
    iters = w.cg_iters
    # launch shapes picked by the library's autotuner (timed batched applies)
    if args.nondeterministic:
        reco.set_deterministic(False)
    t0 = time.perf_counter()
    tune = None
    if args.spread_variant:   # launch shape by hand (profiling a variant), no autotuning
        reco.set_launch_shape(args.spread_cc, args.spread_variant, args.interp_cc)
        tune = {"spread_coils_per_block": args.spread_cc, "spread_variant": args.spread_variant,
                "interp_coils_per_thread": args.interp_cc, "candidates_ms": [], "by_hand": True}
    elif not args.no_autotune:
        tune = reco.autotune()
    autotune_s = time.perf_counter() - t0

    if args.applies_only:
        # profiling mode: the operator alone, args.applies_only applications of
        # all bins (8 launches each: fwd z / y / x, interp, spread, adj x / y / z
        # when one workspace group holds the bins; 7 with the spreading fused
        # with the adjoint x pass), then the algorithmic bytes
        xa = torch.from_numpy(np.stack([synth.phantom(w.img)] * nb)).to(dev)
        qa = torch.empty_like(xa)
        for _ in range(args.applies_only):
            reco.apply_ehde_tensor(xa, qa, 0, nb)
        torch.cuda.synchronize(dev)
        support = reco.support_stats()
        taps, points = reco.spread_matrix_stats()
        fused = reco.spread_fused()
        print(json.dumps({"applies": args.applies_only, "bins": nb, "spread_fused_with_adjoint_x": fused,
                          "algorithmic_bytes": stage_bytes(w, sizes, support, (taps, points) if taps > 0 else None,
                                                           reco.forward_y_listed_rows(), fused)}))
        return 0

    t0 = time.perf_counter()
    for i in range(args.warmup):
        res, its = reco.cg_sense_batched_tensor(data, x, 0.0, iters, want_stats=True)
        if i == 0:
            first_solve_s = time.perf_counter() - t0
    launches_per_step = reco.launch_count()
    setup = {"density_weights_s": dcf_s, "autotune_s": autotune_s,
             "first_solve_s": first_solve_s if args.warmup > 0 else None,
             "library_ms": reco.setup_stats(),
             "what": "density weights (host Voronoi or GPU Pipe-Menon); the library's rebuild of the bins "
                     "(sort, tap records, tile and support lists, transposed tap matrix, workspaces) and the "
                     "capture of the solve's CUDA graph; the autotuner's timed candidate applications; the "
                     "first solve (capture included).  Not part of the timed steps."}

    # end to end through the host-buffer C ABI call (pinned host memory),
    # before the device-timed solves and before the clock sampler polls the
    # GPU
    applies_per_step = nb * iters                       # this rank's bins
    total_applies_per_step = len(all_sizes) * iters     # the whole scan, all ranks
    h_data.copy_(data.cpu())
    h_res = np.zeros((nb, iters), np.float64)
    h_it = np.zeros(nb, np.int32)
    import ctypes as C
    L = cgs.lib()

    def host_call():
        st = L.cgs_cg_solve_batched(reco.ctx, C.c_void_p(h_data.data_ptr()), C.c_void_p(h_x.data_ptr()),
                                    0.0, iters, h_res.ctypes.data_as(C.c_void_p),
                                    h_it.ctypes.data_as(C.c_void_p))
        if st != 0:
            raise RuntimeError(L.cgs_last_error(reco.ctx).decode())

    for _ in range(max(1, args.warmup)):
        host_call()
    raw_before = torch_copy_ms(torch, dev, stream, data, x, h_data, h_x)
    if world > 1:
        dist.barrier()
    # per call: host wall time, and the device time between events recorded on
    # the library's stream just before and just after the call (the copies,
    # the graph and the state read-back; host work between them is not in it)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    host_ms = []
    parts = []
    t0 = time.perf_counter()
    for i in range(args.steps):
        t1 = time.perf_counter()
        ev[i][0].record(stream)
        host_call()
        ev[i][1].record(stream)
        host_ms.append(1e3 * (time.perf_counter() - t1))
        parts.append(reco.e2e_stats())
    e2e_s = time.perf_counter() - t0
    # the same copies by PyTorch from / to the same page-locked buffers
    raw = torch_copy_ms(torch, dev, stream, data, x, h_data, h_x)
    torch.cuda.synchronize(dev)
    e2e_diag = {"host_ms_per_call": statistics.median(host_ms),
                "device_ms_per_call": statistics.median([a.elapsed_time(b) for a, b in ev]),
                "parts_ms": {k: statistics.median([p[k] for p in parts]) for k in ("upload", "solve", "download")},
                "parts_ms_per_call": [[round(p[k], 3) for k in ("upload", "solve", "download")] for p in parts],
                "host_buffers_pinned": parts[-1]["pinned"],
                "torch_copies_ms_before": raw_before, "torch_copies_ms_after": raw}
    te = torch.tensor([e2e_s], device=dev)
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = total_applies_per_step * args.steps / float(te.item())
    h2d = data.numel() * 8
    d2h = x.numel() * 8 + h_res.nbytes + h_it.nbytes

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        reco.cg_sense_batched_tensor(data, x, 0.0, iters, want_stats=False)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    value = total_applies_per_step * args.steps / (ms / 1e3)
    ms_step = ms / args.steps

    # residual check of the last solve
    res, its = reco.cg_sense_batched_tensor(data, x, 0.0, iters, want_stats=True)
    assert np.all(its == iters) and np.all(np.isfinite(res))
    e2e_diag["device_timed_ms_per_step"] = ms_step

    # the plain per-bin GPU form (frozen comparison point): same solve
    plain = None
    extras = world == 1   # the comparison forms and reports: single-GPU runs only
    if extras and not args.no_plain:
        xp = torch.zeros_like(x)
        reco.cg_sense_plain_tensor(data, xp, 0.0, 1)          # warm-up (cuFFT plan, first touch)
        torch.cuda.synchronize(dev)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        pres, pits = reco.cg_sense_plain_tensor(data, xp, 0.0, iters)
        p1.record(stream)
        torch.cuda.synchronize(dev)
        t_plain = p0.elapsed_time(p1) / 1e3
        err = float(torch.linalg.vector_norm(x - xp) / torch.linalg.vector_norm(xp))
        plain = {"s_per_4d_recon": t_plain, "applies_per_s": applies_per_step / t_plain,
                 "speedup_chosen_vs_plain": t_plain / (ms_step / 1e3),
                 "rel_l2_chosen_vs_plain": err, "iters": [int(v) for v in pits],
                 "launches": reco.launch_count(),
                 "form": "per-bin, per-coil launches, unfused, cuFFT full-grid c2c, global-atomic spreading, "
                         "host loop test per iteration"}

    # precision: the chosen form (and its compensated-spreading variant)
    # against the full-FP64 GPU form, iteration by iteration
    precision = None
    if extras and not args.no_precision:
        precision = precision_report(reco, data, x, iters, torch, dev)

    # differentiation form (cfg4): trajectory gradients and self-calibration
    diff = None
    if extras and not args.no_diff:
        diff = differentiation_report(cgs, synth, torch, dev, stream.cuda_stream)


    # the Toeplitz-embedded operator on the same solve (an alternative
    # operator for fixed trajectories; not the headline form)
    toep = None
    if extras and not args.no_toeplitz:
        try:
            toep = toeplitz_report(reco, synth, data, x, iters, torch, dev, stream, max(1, args.steps), w, sizes)
        except cgs.CGSError as e:   # e.g. no cuBLAS on the host: the headline stands without it
            toep = {"unavailable": str(e)}

    # the same solve with GPU Pipe-Menon weights in place of the host Voronoi volumes
    pmr = None
    if extras and args.dcf == "voronoi" and not args.no_pipe_menon:
        pmr = pipe_menon_report(reco, synth, data, x, iters, sbins, dcf, torch, dev, stream, max(1, args.steps))

    # the reference's CPU-path configuration at full size, GPU and CPU
    cfg1 = None
    if extras and not args.no_cfg1:
        cfg1 = cfg1_report(cgs, synth, torch, dev, stream, with_cpu=(rank == 0 and not args.no_cpu))

    # per-stage kernel times of one batched application (roofline)
    xa = torch.from_numpy(np.stack([synth.phantom(w.img)] * nb)).to(dev)
    qa = torch.empty_like(xa)
    reps = []
    for _ in range(5):
        reps.append(reco.profile_apply_tensor(xa, qa, 0, nb))
    st = np.median(np.stack(reps), axis=0)
    fused = reco.spread_fused()
    names = STAGES_FUSED if fused else STAGES
    groups = len(st) // len(names)
    stage_ms = {s: float(sum(st[g * len(names) + i] for g in range(groups))) for i, s in enumerate(names)}
    # the right-hand side alone (sample gather + adjoint chain of all bins),
    # to split the step into applications, right-hand side and CG updates
    import ctypes as C
    b_rhs = torch.empty_like(xa)
    rhs_t = []
    for _ in range(4):
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        st_rhs = cgs.lib().cgs_rhs_d(reco.ctx, 0, nb, C.c_void_p(data.data_ptr()), C.c_void_p(b_rhs.data_ptr()))
        r1.record(stream)
        torch.cuda.synchronize(dev)
        if st_rhs != 0:
            raise RuntimeError(cgs.lib().cgs_last_error(reco.ctx).decode())
        rhs_t.append(r0.elapsed_time(r1))
    rhs_ms = float(np.median(rhs_t[1:]))
    del b_rhs
    support = reco.support_stats()
    taps, points = reco.spread_matrix_stats()
    variant = tune.get("spread_variant") if tune else 8   # the library's default is the fused gather
    gather = variant in (6, 7, 8) and taps > 0
    matrix = (taps, points) if gather else None
    y_listed = reco.forward_y_listed_rows()
    sb = stage_bytes(w, sizes, support, matrix, y_listed, fused)
    apply_ms = float(sum(stage_ms.values()))
    # kernel families: the x/y passes are one kernel template
    family = dict(FAMILY, spread="k_spread_csr" if gather else "k_spread")
    fam = {k: [s for s in names if family[s] == k] for k in dict.fromkeys(family[s] for s in names)}
    fam_ms = {k: sum(stage_ms[s] for s in v) for k, v in fam.items()}
    dom = max(fam_ms, key=fam_ms.get)
    dom_bytes = sum(sb[s] for s in fam[dom])
    peak, peak_kind = measured_peaks()
    achieved = dom_bytes / (fam_ms[dom] / 1e3) / 1e9
    rec = traffic_record()
    tr = rec.get("families", {}).get(dom) if args.workload == "cfg3" else None
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"
        if peak_kind == "measured" else "fallback 6800 GB/s",
        "traffic": None if tr is None else tr["ratio"] * dom_bytes,
        "traffic_source": None if tr is None else (
            "DRAM read + write bytes / algorithmic bytes = %.3f for this kernel family in one application of the "
            "first two cfg3 bins (ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/traffic.json, "
            "profiles/traffic_cfg3_2bin.md), times this run's algorithmic bytes" % tr["ratio"]),
        "traffic_ratio_by_family": {k: v["ratio"] for k, v in rec.get("families", {}).items()},
        "launches_per_apply": len(fam[dom]),
        "algorithmic_bytes_per_apply": dom_bytes,
        "kernel_ms": fam_ms,
        "stage_ms": stage_ms,
        "stage_frac_of_peak": {s: sb[s] / (stage_ms[s] / 1e3) / 1e9 / peak for s in stage_ms},
        "apply_ms": apply_ms,
        "rhs_ms": rhs_ms,
        "cg_update_ms_per_iter": (ms_step - iters * apply_ms - rhs_ms) / max(iters, 1),
        "apply_achieved_gbs": apply_bytes(w, sizes, support, matrix, y_listed, fused) / (apply_ms / 1e3) / 1e9,
        "apply_bytes": apply_bytes(w, sizes, support, matrix, y_listed, fused),
        "spread_fused_with_adjoint_x": fused,
        "support": {"listed_column_fraction": float(sum(support[0])) / (nb * w.grid[1] * w.grid[2]),
                    "stored_tile_fraction": float(sum(support[1])) / (nb * int(np.prod(w.grid)) // 512)},
    }

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "c64/f32 (fp64 CG scalars)", "data": "synthetic",
        "config": {"workload": w.name, "img": list(w.img), "grid": list(w.grid), "coils": w.n_ch,
                   "bins": nb, "samples_per_bin": [min(sizes), max(sizes)], "samples_total": int(sum(sizes)),
                   "cg_iters": iters, "kb_w": kb_w, "kb_b": round(kb_b, 4),
                   "dcf": ("per-bin Voronoi volumes capped at the 99th percentile (host, %.1f s set-up)" % dcf_s)
                   if args.dcf == "voronoi" else
                   ("per-bin Pipe-Menon weights, 20 iterations (GPU, %.2f s set-up), capped at the 99th percentile" % dcf_s)
                   if args.dcf == "pipe-menon"
                   else "radial stand-in",
                   "step": "one 16-bin 4D CG-SENSE reconstruction (graph replay)",
                   "l2": "inputs larger than L2 (data %d MB, workspace > 30 GB)" % (h2d // 2 ** 20),
                   "parallelism": ("bin partition over %d GPUs (greedy by samples; no data-path collective)" % world)
                   if world > 1 else "single GPU"},
        "s_per_4d_recon": ms_step / 1e3,
        "gpu_launches": int(launches_per_step) * args.steps,
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "s_per_4d_recon": float(te.item()) / args.steps, "breakdown": e2e_diag},
        "roofline": roofline,
        "precision": precision,
        "autotune": tune,
        "differentiation": diff,
        "plain": plain,
        "toeplitz": toep,
        "setup": setup,
        "pipe_menon": pmr,
        "cfg1": cfg1,
    }
    if rank == 0 and extras and not args.no_cpu:
        cb = cpu_apply_sample(synth, args.workload)
        v = len(cb["times"]) / sum(cb["times"])
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cb["threads"], "kind": "port",
                                "sample": cb["sample"]}
        if cfg1 and "cpu" in cfg1:
            line["cpu_baseline"]["cfg1"] = cfg1["cpu"]
    # the precision configuration (its own context; the headline's is freed first)
    if extras and not args.no_precision and not args.no_cfg2:
        del reco, xa, qa
        torch.cuda.synchronize(dev)
        torch.cuda.empty_cache()
        line["precision_cfg2"] = cfg2_precision_report(cgs, synth, torch, dev, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg3")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-bin GPU form")
    ap.add_argument("--no-precision", action="store_true", help="skip the per-iteration FP64 comparison")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--spread-variant", type=int, default=0,
                    help="launch shape by hand instead of the autotuner: spreading variant (cgs_set_launch_shape)")
    ap.add_argument("--spread-cc", type=int, default=6, help="with --spread-variant: its coils per block / thread")
    ap.add_argument("--interp-cc", type=int, default=2, help="with --spread-variant: coils per interpolation thread")
    ap.add_argument("--nondeterministic", action="store_true",
                    help="let the autotuner pick atomic spreading (results not bitwise reproducible)")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiation form (cfg4)")
    ap.add_argument("--no-toeplitz", action="store_true", help="skip the Toeplitz-embedded solve")
    ap.add_argument("--no-cfg1", action="store_true",
                    help="skip the 64^3 / 8-coil / 262 144-sample configuration (GPU and CPU port)")
    ap.add_argument("--no-cfg2", action="store_true", help="skip the cfg2 precision report")
    ap.add_argument("--no-pipe-menon", action="store_true",
                    help="skip the solve with GPU Pipe-Menon weights in place of the Voronoi volumes")
    ap.add_argument("--diff-only", action="store_true", help="only the differentiation form (one JSON line)")
    ap.add_argument("--cg-grad-only", action="store_true",
                    help="only the unrolled-CG trajectory gradient of the combined workload (cfg5)")
    ap.add_argument("--workspace-gb", type=float, default=56.0, help="grid workspace budget (--cg-grad-only)")
    ap.add_argument("--applies-only", type=int, default=0,
                    help="profiling mode: only this many operator applications of all bins, then exit")
    ap.add_argument("--max-bins", type=int, default=0,
                    help="keep only the first N respiratory bins (small cases for profiling)")
    ap.add_argument("--precision-only", action="store_true",
                    help="only the precision form of --workload (one JSON line of per-iteration errors)")
    ap.add_argument("--dcf", default="voronoi", choices=["voronoi", "radial", "pipe-menon"],
                    help="density weights: per-bin Voronoi volumes or a radial stand-in")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.precision_only:
        return run_precision_only(args)
    if args.diff_only:
        return run_diff_only(args)
    if args.cg_grad_only:
        return run_cg_grad_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
