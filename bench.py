"""Benchmark of the GB300 scalar-propagation hot path.

Workload (default): the 2048 x 2048 multi-wavelength, multi-mode batch -- 48
fields (3 wavelengths 0.640 / 0.538 / 0.455 um x 16 Hermite-Gauss modes, waist
80 um, ds = 0.5 um), cascade Phase -> ASProp(5000 um) -> Phase -> ASProp ->
Phase -> ASProp, SquaredIntensityDifference against a per-wavelength target,
gradient with respect to the three masks and one Fista + ClampProx step,
captured as one CUDA graph.  One step = one optimisation iteration =
3 forward + 3 adjoint propagations of 48 fields = 288 propagations.

Inputs are synthetic and seeded (the reference publishes no dataset for this
path).  All fields live in HBM (1.5 GiB per field batch, > L2), so no L2 flush
is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the FP64 CPU restatement of the reference path (the
oracle; the Julia reference cannot run here) on the host cores.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# Streams share the device's hardware work queues (8 by default). The e2e loop's copy
# stream and compute stream must not share one, or the input copy of step k+1
# waits behind the compute of step k. 32 queues for this process.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

N = 2048
DS = (0.5, 0.5)
LAMBDAS = (0.640, 0.538, 0.455)
N_MODES = 16
W0 = 80.0
Z = 5000.0
N_MASKS = 3
ETA = 2e-4
SEED = 1234
METRIC = "fwd+adjoint propagations/s"
UNIT = "propagations/s"
WORKLOAD = "2048x2048 x {fields} fields (3 lambdas x HG modes), 3 trainable phase masks, ASProp z=5000um, " \
           "SquaredIntensityDifference, fwd+adjoint+Fista/ClampProx step in one CUDA graph"


def hg_orders():
    # hermite_gaussian_groups(w0, 5) gives the 15 modes with m+n <= 4; the 16th is HG(5,0)
    orders = [(m, n) for m in range(5) for n in range(5 - m)]
    return orders + [(5, 0)]


def make_inputs(n=N):
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(SEED)
    x = (np.arange(n) - (n - 1) / 2) * DS[0]
    y = (np.arange(n) - (n - 1) / 2) * DS[1]

    def hg(m, k):
        def one(q, s):
            c = (2 / math.pi) ** 0.25 / math.sqrt(W0) / math.sqrt(2.0 ** q * math.factorial(q))
            h0 = np.ones_like(s)
            if q > 0:
                h1 = 2 * np.sqrt(2) * s / W0
                hp = h0
                for j in range(1, q):
                    hp, h1 = h1, 2 * np.sqrt(2) * s / W0 * h1 - 2 * j * hp
                h0 = h1
            return c * h0 * np.exp(-(s / W0) ** 2)
        return (one(k, y)[:, None] * one(m, x)[None, :]).astype(np.complex64)

    modes = np.stack([hg(m, k) for (m, k) in hg_orders()[:N_MODES]])  # (modes, n, n)
    fields = np.broadcast_to(modes[:, None], (N_MODES, len(LAMBDAS), n, n)).copy()  # Julia (n, n, 3, 16)
    masks = []
    for _ in range(N_MASKS):
        w = gaussian_filter(rng.standard_normal((n, n)), 8.0)
        masks.append((np.pi * w / np.max(np.abs(w))).astype(np.float32))
    targets = []
    for _ in LAMBDAS:
        t = gaussian_filter(rng.standard_normal((n, n)), 32.0) ** 2
        t *= N_MODES / (t.sum() * DS[0] * DS[1])
        targets.append(t.astype(np.float32))
    return fields, masks, np.stack(targets)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# GB300 path
# ---------------------------------------------------------------------------
def build_system(fo, fields_np, masks_np, targets_np):
    import torch
    u0 = fo.ScalarField(torch.from_numpy(fields_np).cuda(), DS, np.array(LAMBDAS))
    phases = [fo.Phase(u0, m, trainable=True, buffered=True) for m in masks_np]
    prop = fo.ASProp(u0, Z)
    comps = []
    for ph in phases:
        comps += [ph, prop]
    system = fo.OpticalSystem(fo.ScalarSource(u0), comps)
    metric = fo.SquaredIntensityDifference((u0, targets_np))
    rule = fo.ProxRule(fo.Fista(ETA), fo.ClampProx(-np.pi, np.pi))
    opt = fo.setup(rule, system)
    return u0, system, metric, opt, prop


def iteration(fo, system, metric, opt, x, du, src):
    """One optimisation step: forward, SquaredIntensityDifference and the seeded adjoint
    sweep in one library call (the chain's last forward row pass and the adjoint's first
    row pass share one pass; the output field is not written), then the optimiser."""
    grads = system.forward_backward_sid(du, src, metric)
    if grads is None:  # a system the fused call does not cover
        tape = []
        system.forward(x, tape, src=src, metric=metric)  # the metric runs inside the last forward pass
        grads = system.backward(du, tape, seed=(metric, x))
    loss = metric.loss
    fo.update_(opt, system, grads)
    return loss


def algorithmic_bytes_per_step(n=N, batch=None):
    batch = batch or N_MODES * len(LAMBDAS)
    n2 = n * n
    props = 2 * N_MASKS * batch * 16 * n2                 # read + write one c32 field per propagation
    fwd_phase = N_MASKS * (4 * n2 + 8 * n2 * batch)       # mask read + saved input written
    adj_phase = N_MASKS * (8 * n2 * batch + 4 * n2)       # saved input read + gradient written
    h = 2 * N_MASKS * len(LAMBDAS) * 8 * n2               # one transfer function per wavelength per pass
    fista = N_MASKS * 6 * 4 * n2                          # x, xk, dx read; x, xk, newdx written
    return props + fwd_phase + adj_phase + h + fista


def pass_bytes_per_step(n=N, batch=None):
    """DRAM bytes the iteration's passes must move: each of the 4K+1 passes (the
    forward sweep's last row pass and the adjoint's first share one pass) reads and
    writes every field once, plus saves, saved reads, masks, gradients, transfer
    functions, the metric's target and residual, and Fista.  The first mask's adjoint
    reads the source field (no save); the shared pass writes no output field, and its
    second reading of the spectrum is not counted (it comes partly from L2)."""
    batch = batch or N_MODES * len(LAMBDAS)
    n2 = n * n
    fld = 8 * n2 * batch                                    # one c32 copy of the batch
    col = 2 * fld + len(LAMBDAS) * 8 * n2                   # column pass: field in and out, one H per wavelength
    fwd_rows = (2 * fld + 4 * n2) + (N_MASKS - 1) * (3 * fld + 4 * n2)  # source pass, mask passes with saves
    shared = 2 * fld + 2 * len(LAMBDAS) * 4 * n2            # metric + seed: spectrum in, adjoint spectrum out
    adj_rows = (N_MASKS - 1) * (3 * fld + 8 * n2) + (2 * fld + 8 * n2)  # gradient passes, last gradient pass
    fista = N_MASKS * 6 * 4 * n2
    return 2 * N_MASKS * col + fwd_rows + shared + adj_rows + fista


def col_pass_bytes(n=N, batch=None):
    batch = batch or N_MODES * len(LAMBDAS)
    # one column pass over the batch: every field read and written once, one
    # transfer-function table per wavelength
    return batch * 16 * n * n + len(LAMBDAS) * 8 * n * n


def numa_pages(addr, nbytes):
    """Pages per NUMA node of the host mappings that overlap [addr, addr + nbytes)
    ({"N0": pages, ...}), from /proc/self/numa_maps; empty where it does not exist."""
    try:
        with open("/proc/self/maps") as f:
            spans = {}
            for ln in f:
                a, b = (int(v, 16) for v in ln.split()[0].split("-"))
                spans[a] = b
        with open("/proc/self/numa_maps") as f:
            lines = f.readlines()
    except OSError:
        return {}
    out = {}
    for ln in lines:
        parts = ln.split()
        start = int(parts[0], 16)
        end = spans.get(start)
        if end is None or end <= addr or start >= addr + nbytes:
            continue
        for kv in parts[1:]:
            k, _, v = kv.partition("=")
            if k.startswith("N") and k[1:].isdigit() and v.isdigit():
                out[k] = out.get(k, 0) + int(v)
    return out


def max_over_ranks(ms, device="cuda"):
    """The slowest rank's step time: every replica processed its own share, so the
    job took as long as the slowest one (barrier on both sides)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_rate(props_per_rank_step, world, ms):
    """Whole-job propagations/s of `world` replicas that each ran one step in ms."""
    return props_per_rank_step * world / (ms * 1e-3)


def run_gb300(args, rank, world):
    import torch
    from __graft_entry__ import build, load_package

    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    build()
    fo = load_package()
    lib = fo.load_library()
    fields_np, masks_np, targets_np = make_inputs()
    u0, system, metric, opt, prop = build_system(fo, fields_np, masks_np, targets_np)
    batch = u0.batch
    props_per_step = 2 * N_MASKS * batch
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        src = system.source.u0
        x = src.similar()
        du = src.similar()
        iteration(fo, system, metric, opt, x, du, src)   # creates every plan before the capture
        torch.cuda.synchronize()
        sp = C.c_void_p(stream.cuda_stream)
        g = C.c_void_p()
        fo._capi.check(lib.fo_graph_begin(sp))
        loss_t = iteration(fo, system, metric, opt, x, du, src)
        fo._capi.check(lib.fo_graph_end(sp, C.byref(g)))
        nk = C.c_int()
        fo._capi.check(lib.fo_graph_info(g, C.byref(nk)))
        for _ in range(args.warmup):
            fo._capi.check(lib.fo_graph_launch(g, sp))
        stream.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(torch.cuda.current_device()) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                fo._capi.check(lib.fo_graph_launch(g, sp))
            e1.record(stream)
            stream.synchronize()
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
        final_loss = float(loss_t.sum())

        # per-pass device times of the same iteration, eager, events around every pass
        fo._capi.check(lib.fo_profile_begin())
        for _ in range(2):
            iteration(fo, system, metric, opt, x, du, src)
        arr_ms = (C.c_double * 3)()
        arr_n = (C.c_int * 3)()
        fo._capi.check(lib.fo_profile_end(arr_ms, arr_n))
        col_ms = arr_ms[2] / max(1, arr_n[2])
        pass_ms = {"row_single": arr_ms[0] / max(1, arr_n[0]), "row_fused": arr_ms[1] / max(1, arr_n[1]),
                   "col": col_ms}
        pass_share = {k: arr_ms[i] / max(1e-9, sum(arr_ms)) for i, k in enumerate(pass_ms)}

        # End to end through the public C ABI with host buffers: every step uploads its
        # 48 input fields from pinned host memory (fo_copy) and reads the loss back.
        # Each step is one graph: the iteration on one input buffer and, on a parallel
        # branch, the upload of the next step's input into the other buffer, so the
        # graph itself states that the two are independent.  The first step's input is
        # uploaded before it, inside the timed region.
        host_in = torch.from_numpy(fields_np).pin_memory()
        in_bytes = host_in.numel() * host_in.element_size()
        host_numa = numa_pages(host_in.data_ptr(), in_bytes)
        host_loss = torch.empty((len(LAMBDAS),), dtype=torch.float32).pin_memory()
        bufs = (src, src.similar())
        copy_stream = torch.cuda.Stream()
        cp = C.c_void_p(copy_stream.cuda_stream)

        def dptr(t):
            return C.c_void_p(t.data_ptr())

        def capture_step(cur, nxt):
            gg = C.c_void_p()
            fo._capi.check(lib.fo_graph_begin(sp))
            fork, join = torch.cuda.Event(), torch.cuda.Event()
            fork.record(stream)
            copy_stream.wait_event(fork)
            fo._capi.check(lib.fo_copy(dptr(bufs[nxt].electric), dptr(host_in), in_bytes, cp))
            join.record(copy_stream)
            iteration(fo, system, metric, opt, x, du, bufs[cur])
            fo._capi.check(lib.fo_copy(dptr(host_loss), dptr(metric.loss), host_loss.numel() * 4, sp))
            stream.wait_event(join)
            fo._capi.check(lib.fo_graph_end(sp, C.byref(gg)))
            return gg

        step_graphs = (capture_step(0, 1), capture_step(1, 0))
        # host->device bandwidth of this machine for the step's input, alone (the e2e
        # rate is bounded by it when the copy takes longer than the compute)
        # (the fastest of three copies: a single one can stall on the host side)
        copy_times = []
        for _ in range(3):
            torch.cuda.synchronize()
            h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            h0.record(copy_stream)
            fo._capi.check(lib.fo_copy(dptr(bufs[1].electric), dptr(host_in), in_bytes, cp))
            h1.record(copy_stream)
            torch.cuda.synchronize()
            copy_times.append(h0.elapsed_time(h1))
        copy_alone_ms = min(copy_times)
        h2d_gbs = in_bytes / (copy_alone_ms * 1e-3) / 1e9
        # as many e2e steps as timed device steps: the first step's input upload (not
        # overlapped with any compute) is part of the measurement, spread over the same count
        e2_steps = max(1, args.steps)
        ev_step = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(e2_steps)]
        e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e2.record(stream)
        fo._capi.check(lib.fo_copy(dptr(bufs[0].electric), dptr(host_in), in_bytes, sp))
        for k in range(e2_steps):
            ev_step[k][0].record(stream)
            fo._capi.check(lib.fo_graph_launch(step_graphs[k % 2], sp))
            ev_step[k][1].record(stream)
        e3.record(stream)
        stream.synchronize()
        # the slowest rank's time, as for the device-timed value (whole-job rate below)
        e2e_ms = max_over_ranks(e2.elapsed_time(e3) / e2_steps)
        e2e_step_ms = statistics.median(a.elapsed_time(b) for a, b in ev_step)
        # start / end (ms from the start of the e2e region) of the first steps, and every
        # step's duration (a step that waited for its input upload shows up here)
        e2e_timeline = [[round(e2.elapsed_time(ev), 2) for ev in ev_step[k]] for k in range(min(4, e2_steps))]
        e2e_steps_ms = [round(a.elapsed_time(b), 3) for a, b in ev_step]
        for gg in step_graphs:
            fo._capi.check(lib.fo_graph_destroy(gg))
        fo._capi.check(lib.fo_graph_destroy(g))

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = col_pass_bytes(batch=batch) / (col_ms * 1e-3) / 1e9
    # the committed DRAM-traffic capture is of the full 48-field launch
    traffic = read_traffic() if batch == 48 else None
    row_name, col_name = C.create_string_buffer(160), C.create_string_buffer(160)
    fo._capi.check(lib.fo_prop_variants(prop.plan_for(u0), None, None, row_name, col_name, 160))
    value = job_rate(props_per_step, world, ms)
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c32 (fp32 complex; fp64 transfer-function phase)",
        "data": "synthetic, seeded (HG modes, Gaussian-filtered random masks and targets)",
        "config": headline_config(batch, world),
        "algorithmic_gb_per_step": round(algorithmic_bytes_per_step() / 1e9, 3),
        "algorithmic_gbs": round(algorithmic_bytes_per_step() / (ms * 1e-3) / 1e9, 1),
        "pass_gb_per_step": round(pass_bytes_per_step() / 1e9, 3),
        "pass_gbs": round(pass_bytes_per_step() / (ms * 1e-3) / 1e9, 1),
        "roofline": {"bound": "hbm",
                     "kernel": f"column pass {col_name.value.decode()} (FFT_y * H * IFFT_y over {batch} fields)",
                     "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(achieved / hbm_peak, 4), "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": traffic, "algorithmic_bytes_per_launch": col_pass_bytes(batch=batch)},
        "row_kernel": row_name.value.decode(),
        "pass_ms": {k: round(v, 4) for k, v in pass_ms.items()},
        "pass_share": {k: round(v, 3) for k, v in pass_share.items()},
        "gpu_launches": int(nk.value) * args.steps,
        "gpu_launches_per_step": int(nk.value),
        "e2e": {"value": round(job_rate(props_per_step, world, e2e_ms), 1), "unit": UNIT, "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": int(fields_np.nbytes), "d2h_bytes_per_step": int(len(LAMBDAS) * 4),
                "overlap": "each step is one graph: the iteration, and on a parallel branch the "
                           "upload of the next step's input (fo_copy from pinned memory)",
                "step_ms": round(e2e_step_ms, 4), "copy_alone_ms": round(copy_alone_ms, 4),
                # the rate of the median step, for runs where a few uploads stalled on the host side
                "median_step_value": round(job_rate(props_per_step, world, e2e_step_ms), 1),
                "timeline_ms": {"steps": "[step start, step end]", "first_steps": e2e_timeline,
                                "every_step": e2e_steps_ms},
                "h2d_gbs_measured": round(h2d_gbs, 1),
                "host_buffer_numa": host_numa},
        "clocks": clk.summary(),
        "final_loss": final_loss,
    }
    return line


def read_traffic():
    """DRAM bytes per column-pass launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "col_tma_2048x48_traffic.txt")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_launch"):
                return int(float(ln.split("=")[1]))
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# plain cuFFT + elementwise path (the reference's CUDA.jl launch sequence in torch)
# ---------------------------------------------------------------------------
def run_plain(steps=3, warmup=1):
    import torch
    fields_np, masks_np, targets_np = make_inputs()
    dev = "cuda"
    u0 = torch.from_numpy(fields_np).to(dev).reshape(-1, N, N)
    B = u0.shape[0]
    lam_f = np.tile(np.array(LAMBDAS), N_MODES)
    fx = torch.fft.fftfreq(N, DS[0], dtype=torch.float64, device=dev)
    fy = torch.fft.fftfreq(N, DS[1], dtype=torch.float64, device=dev)
    H = {}
    for lam in LAMBDAS:
        arg = (1 / lam ** 2 - fx[None, :] ** 2 - fy[:, None] ** 2).to(torch.complex128)
        H[lam] = torch.exp(1j * 2 * np.pi * Z * torch.sqrt(arg)).to(torch.complex64)
    phis = [torch.from_numpy(m).to(dev) for m in masks_np]
    xks = [p.clone() for p in phis]
    ts = [1.0] * N_MASKS
    target = torch.from_numpy(targets_np).to(dev)

    def prop(u, conj):
        u = torch.fft.fft2(u)
        for b in range(B):                       # one multiply launch per trailing slice
            h = H[lam_f[b]]
            u[b] *= h.conj() if conj else h
        return torch.fft.ifft2(u)

    def step():
        u = u0.clone()
        saves = []
        for k in range(N_MASKS):
            saves.append(u.clone())
            u = u * torch.exp(1j * phis[k])
            u = prop(u, False)
        inten = (u.abs() ** 2).reshape(N_MODES, len(LAMBDAS), N, N).sum(0)
        r = inten - target
        loss = (r ** 2).sum()
        du = 4 * r.repeat(N_MODES, 1, 1) * u
        for k in reversed(range(N_MASKS)):
            du = prop(du, True)
            du = du * torch.exp(-1j * phis[k])
            g = torch.imag(du * saves[k].conj()).sum(0)
            tn = (1 + np.sqrt(1 + 4 * ts[k] ** 2)) / 2
            beta = (ts[k] - 1) / tn
            newdx = ETA ** 2 * g - beta * (phis[k] - xks[k])
            xks[k] = phis[k].clone()
            phis[k] -= newdx
            phis[k].clamp_(-np.pi, np.pi)
            ts[k] = tn
        return loss

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"value": round(2 * N_MASKS * B / (ms * 1e-3), 1), "unit": UNIT, "ms_per_step": round(ms, 3),
            "impl": "torch.fft (cuFFT) + per-slice elementwise launches, the reference's CUDA.jl sequence"}


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 oracle (restatement of the reference path)
# ---------------------------------------------------------------------------
def headline_config(batch, world):
    """The `config` object of the headline workload, shared by both bench arms."""
    return {"workload": WORKLOAD.format(fields=batch), "grid": N, "fields": batch, "masks": N_MASKS,
            "props_per_step": 2 * N_MASKS * batch, "parallelism": f"replicas x{world}",
            "l2": f"inputs larger than L2 ({batch * N * N * 8 / 2**30:.1f} GiB field batch), no flush"}


def run_cpu_sample(budget_s=12.0, threads=None, inputs=None):
    """The FP64 oracle on the host cores: repetitions of one field of the batch through
    the chain, forward + adjoint, until budget_s has passed (at least one)."""
    from oracle import fluxoptics_oracle as orc
    threads = threads or os.cpu_count() or 1
    orc.set_workers(threads)
    fields_np, masks_np, targets_np = inputs if inputs is not None else make_inputs()
    u0 = fields_np[0, 0].astype(np.complex128)      # HG00 at lambda = 0.640 um
    lam = LAMBDAS[0]
    phis = [m.astype(np.float64) for m in masks_np]
    t0 = time.perf_counter()
    reps = 0
    while True:
        v = u0
        saves = []
        for k in range(N_MASKS):
            saves.append(v)
            v = orc.asprop(orc.phase_forward(v, phis[k]), DS[0], DS[1], lam, Z)
        dv = orc.sid_backward(v, targets_np[0])
        for k in reversed(range(N_MASKS)):
            dv = orc.asprop(dv, DS[0], DS[1], lam, Z, orc.BACKWARD)
            dv, _ = orc.phase_backward(dv, phis[k], saves[k])
        reps += 1
        el = time.perf_counter() - t0
        if el > budget_s or reps >= 50:
            break
    return {"value": round(2 * N_MASKS * reps / el, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "seconds_per_rep": el / reps,
            "sample": f"{reps} x (1 of 48 fields, HG00 at 0.640 um, 2048^2) through the 3-mask chain, "
                      f"forward + adjoint, FP64 numpy/scipy.fft with {threads} workers, {el:.1f} s"}


# ---------------------------------------------------------------------------
# Other configurations (reported with --config 2 / 4 / 5)
# ---------------------------------------------------------------------------
def _graph_time(fo, lib, step_fn, steps, warmup):
    """Capture step_fn once on a side stream, replay it; returns (ms/step, kernel nodes)."""
    import torch
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        step_fn()
        torch.cuda.synchronize()
        sp = C.c_void_p(stream.cuda_stream)
        g = C.c_void_p()
        fo._capi.check(lib.fo_graph_begin(sp))
        step_fn()
        fo._capi.check(lib.fo_graph_end(sp, C.byref(g)))
        nk = C.c_int()
        fo._capi.check(lib.fo_graph_info(g, C.byref(nk)))
        for _ in range(warmup):
            fo._capi.check(lib.fo_graph_launch(g, sp))
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fo._capi.check(lib.fo_graph_launch(g, sp))
        e1.record(stream)
        stream.synchronize()
        fo._capi.check(lib.fo_graph_destroy(g))
    return e0.elapsed_time(e1) / steps, nk.value


def run_config2(args):
    """Two-DOE RSProp chain, 512^2 padded to 1024^2, forward + gradient + Fista."""
    import torch
    from __graft_entry__ import build, load_package
    build()
    fo = load_package()
    lib = fo.load_library()
    n, ds, lam = 512, (1.0, 1.0), 1.064
    rng = np.random.default_rng(SEED + 2)
    x, y = fo.spatial_vectors((n, n), ds)
    u = fo.ScalarField(fo.gaussian(30.0, x, y).astype(np.complex64), ds, lam)
    fo.normalize_power_(u)
    t = fo.gaussian(30.0, x - 60.0, y) + fo.gaussian(30.0, x + 60.0, y)
    t = np.abs(t) ** 2
    t /= t.sum() * ds[0] * ds[1]
    m1 = fo.Phase(u, rng.uniform(0, 2 * np.pi, (n, n)), trainable=True, buffered=True)
    m2 = fo.Phase(u, rng.uniform(0, 2 * np.pi, (n, n)), trainable=True, buffered=True)
    system = fo.ScalarSource(u) | fo.RSProp(u, 1500.0) | m1 | fo.RSProp(u, 2000.0) | m2 | fo.RSProp(u, 1500.0)
    metric = fo.SquaredIntensityDifference((u, t))
    opt = fo.setup(fo.Fista(1.0), system)
    src = system.source.u0
    x_, du = src.similar(), src.similar()
    ms, nk = _graph_time(fo, lib, lambda: iteration(fo, system, metric, opt, x_, du, src), args.steps, args.warmup)
    return {"config": "two-DOE RSProp chain 512^2 (pad 1024^2), fwd + adjoint + Fista, CUDA graph",
            "props_per_step": 6, "ms_per_step": round(ms, 4), "value": round(6 / (ms * 1e-3), 1),
            "unit": UNIT, "gpu_launches_per_step": nk}


CONFIG4 = {"n": 1024, "ds": (0.25, 0.25), "lam": 1.064, "n0": 1.45, "slices": 256}


def config4_inputs(n=CONFIG4["n"], ns=CONFIG4["slices"]):
    """AS_BPM workload inputs: dn (ns, n, n) float32 of seeded white noise filtered with
    sigma = 8 slices axially and 4 px transversally, scaled to max |dn| = 5e-3; a plane
    wave tilted by a seeded angle within 2 degrees (baked into the data) under a
    Gaussian envelope of waist 150 um, unit power (complex64); an intensity target."""
    from scipy.ndimage import gaussian_filter
    ds, lam, n0 = CONFIG4["ds"], CONFIG4["lam"], CONFIG4["n0"]
    rng = np.random.default_rng(SEED + 4)
    dn = gaussian_filter(rng.standard_normal((ns, n, n)).astype(np.float32), (8.0, 4.0, 4.0))
    dn *= 5e-3 / np.max(np.abs(dn))
    x = (np.arange(n) - (n - 1) / 2) * ds[0]
    y = (np.arange(n) - (n - 1) / 2) * ds[1]
    th = np.deg2rad(rng.uniform(-2, 2))
    env = np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 150.0 ** 2)
    u0 = env * np.exp(1j * 2 * np.pi * n0 / lam * np.sin(th) * x[None, :])
    u0 = (u0 / np.sqrt(np.sum(np.abs(u0) ** 2) * ds[0] * ds[1])).astype(np.complex64)
    target = (np.abs(gaussian_filter(rng.standard_normal((n, n)), 16.0)) ** 2).astype(np.float32)
    return u0, dn.astype(np.float32), target


def run_config4(args):
    """AS_BPM 1024^2 x 256 slices, gradient w.r.t. dn with sqrt(N) checkpoints."""
    import torch
    from __graft_entry__ import build, load_package
    build()
    fo = load_package()
    lib = fo.load_library()
    n, ds, lam, n0, ns = CONFIG4["n"], CONFIG4["ds"], CONFIG4["lam"], CONFIG4["n0"], CONFIG4["slices"]
    u0, dn, target = config4_inputs()
    u = fo.ScalarField(u0, ds, lam)
    bpm = fo.AS_BPM(u, float(ns), n0, dn, trainable=True, buffered=True)
    system = fo.ScalarSource(u) | bpm
    metric = fo.SquaredIntensityDifference((u, target))
    opt = fo.setup(fo.Fista(1e-3), system)
    src = system.source.u0
    x_, du = src.similar(), src.similar()
    ms, nk = _graph_time(fo, lib, lambda: iteration(fo, system, metric, opt, x_, du, src), max(3, args.steps // 2),
                         args.warmup)
    props = 2 * (ns + 1)
    return {"config": "AS_BPM 1024^2 x 256 slices (dz=1um, n0=1.45), d(dn) with sqrt(N)=16 checkpoints "
                      "+ recompute, Fista on dn, CUDA graph",
            "props_per_step": props, "recompute_props_per_step": ns - 16, "ms_per_step": round(ms, 3),
            "value": round(props / (ms * 1e-3), 1), "unit": UNIT, "gpu_launches_per_step": nk}


def ragged_problems(seed=SEED + 5, count=64, sizes=(256, 512, 1024, 2048, 4096)):
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        probs.append({"n": n, "lam": float(rng.uniform(0.4, 1.6)), "z": float(np.exp(rng.uniform(np.log(100), np.log(2e4)))),
                      "w0": float(rng.uniform(10, 200)), "off": tuple(rng.uniform(-0.1, 0.1, 2) * n),
                      "seed": int(rng.integers(1 << 30))})
    return probs


def build_ragged(fo, probs):
    systems = []
    for pr in probs:
        n = pr["n"]
        rng = np.random.default_rng(pr["seed"])
        x, y = fo.spatial_vectors((n, n), (1.0, 1.0))
        u = fo.ScalarField(fo.gaussian(pr["w0"], x - pr["off"][0], y - pr["off"][1]).astype(np.complex64),
                           (1.0, 1.0), pr["lam"])
        fo.normalize_power_(u)
        ph = fo.Phase(u, rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32), trainable=True, buffered=True)
        system = fo.ScalarSource(u) | ph | fo.ASProp(u, pr["z"])
        t = np.abs(fo.gaussian(pr["w0"], x, y)) ** 2
        metric = fo.SquaredIntensityDifference((u, t))
        src = system.source.u0
        systems.append((system, metric, ph, src, src.similar(), src.similar()))
    return systems


def ragged_specs(fo, probs):
    """Inputs of the ragged problems for fo.RaggedBatch: Gaussian beams (waist and
    offset per problem, power 1), a uniform random phase mask, the centred beam's
    intensity as the target."""
    specs = []
    for pr in probs:
        n = pr["n"]
        rng = np.random.default_rng(pr["seed"])
        x, y = fo.spatial_vectors((n, n), (1.0, 1.0))
        u = fo.ScalarField(fo.gaussian(pr["w0"], x - pr["off"][0], y - pr["off"][1]).astype(np.complex64),
                           (1.0, 1.0), pr["lam"])
        fo.normalize_power_(u)
        phi = rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32)
        t = (np.abs(fo.gaussian(pr["w0"], x, y)) ** 2).astype(np.float32)
        specs.append({"u": u, "phase": phi, "target": t, "z": pr["z"]})
    return specs


def run_config5(args):
    """Ragged batch of 64 ASProp forward + adjoint problems (256^2 .. 4096^2), each
    Phase -> ASProp -> SquaredIntensityDifference with its phase gradient, all in ONE
    persistent cooperative launch per step (fo_ragged_batch)."""
    import torch
    from __graft_entry__ import build, load_package
    build()
    fo = load_package()
    lib = fo.load_library()
    probs = ragged_problems(count=args.problems)
    rb = fo.RaggedBatch(ragged_specs(fo, probs))
    for _ in range(max(3, args.warmup)):
        rb.run()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(3, args.steps)
    e0.record(stream)
    for _ in range(steps):
        rb.run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    fo._capi.check(lib.fo_device_status(C.c_void_p(stream.cuda_stream)))
    pix = sum(p["n"] ** 2 for p in probs)
    info = rb.info()
    pass_ms = rb.pass_ms()
    return {"config": f"ragged batch: {len(probs)} ASProp problems, N in {{256..4096}}^2 (seeded), random lambda/z/waist/"
                      "offset/phase mask, intensity loss, fwd + adjoint + phase gradient, one persistent "
                      f"cooperative launch per step ({info['grid_ctas']} CTAs, one per SM)",
            "props_per_step": 2 * len(probs), "ms_per_step": round(ms, 3),
            "value": round(2 * len(probs) / (ms * 1e-3), 1), "unit": UNIT, "gpu_launches_per_step": 1,
            "pixels_per_step": pix, "algorithmic_gbs": round(2 * 16 * pix / (ms * 1e-3) / 1e9, 1),
            "pass_ms": dict(zip(["row_fwd", "col_fwd", "row_mid_loss_seed", "col_adj", "row_grad_loss"],
                                [round(v, 3) for v in pass_ms]))}


def config_bytes(cfg, result):
    """Algorithmic HBM bytes of one step of the other configurations: every propagation
    reads and writes its unpadded field once (16 n^2), every modulation reads its
    parameter once (4 n^2), saves and reads back its input (8 n^2 each way) and writes
    its gradient (4 n^2); the optimiser step reads x, xk, dx and writes x, xk, newdx."""
    if cfg == 2:          # 512^2 two-DOE RSProp chain: 3 + 3 propagations, 2 phase masks, Fista
        n2 = 512 * 512
        return 6 * 16 * n2 + 2 * (4 + 8 + 8 + 4) * n2 + 2 * 24 * n2
    if cfg == 4:          # AS_BPM 1024^2 x 256 slices: 257 + 257 propagations, dn read twice,
        n2, ns = CONFIG4["n"] ** 2, CONFIG4["slices"]   # slice inputs saved and read, d(dn) written, Fista on dn
        return 2 * (ns + 1) * 16 * n2 + ns * (4 + 8 + 4 + 8 + 4) * n2 + 24 * ns * n2
    if cfg == 5:          # ragged: one forward + one adjoint propagation per problem, the mask read in
        pix = result["pixels_per_step"]   # both, the input read again by the gradient, target, gradient written
        return pix * (2 * 16 + 2 * 4 + 8 + 4 + 4)
    raise ValueError(cfg)


def run_other_configs(args):
    """Bounded runs of configurations 2, 4 and 5 (a few steps each) for the JSON line:
    value, time per step and the whole step's algorithmic bandwidth against the
    measured HBM peak."""
    import torch
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    sub = argparse.Namespace(steps=max(3, min(args.steps, 6)), warmup=max(3, min(args.warmup, 3)),
                             problems=args.problems)
    out = {}
    for cfg, fn in ((2, run_config2), (4, run_config4), (5, run_config5)):
        r = fn(sub)
        torch.cuda.synchronize()
        b = config_bytes(cfg, r)
        gbs = b / (r["ms_per_step"] * 1e-3) / 1e9
        out[str(cfg)] = {"config": r["config"], "value": r["value"], "unit": r["unit"],
                         "ms_per_step": r["ms_per_step"], "props_per_step": r["props_per_step"],
                         "steps": sub.steps, "gpu_launches_per_step": r.get("gpu_launches_per_step"),
                         "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s",
                                      "frac": round(gbs / hbm, 4), "scope": "whole step, algorithmic bytes",
                                      "algorithmic_bytes_per_step": int(b)}}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 30 steps: the e2e region's first input upload, which nothing can overlap, is spread
    # over a run of steady-state steps (about 0.3 s of device time)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain cuFFT comparison")
    ap.add_argument("--no-configs", action="store_true", help="skip the bounded runs of configurations 2, 4 and 5")
    ap.add_argument("--config", type=int, default=3, choices=[2, 3, 4, 5],
                    help="3: the 2048^2 x 48 headline (default); 2 / 4 / 5: the other configurations")
    ap.add_argument("--modes", type=int, default=16,
                    help="modes per wavelength (default 16; smaller values only for profiler captures)")
    ap.add_argument("--wavelengths", type=int, default=3, choices=[1, 2, 3],
                    help="wavelengths of the batch (default 3; fewer only for profiler captures)")
    ap.add_argument("--problems", type=int, default=64,
                    help="problems of the ragged batch (--config 5; default 64, smaller only for profiler captures)")
    args = ap.parse_args()
    global N_MODES, LAMBDAS
    N_MODES = args.modes
    LAMBDAS = LAMBDAS[:args.wavelengths]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        # One step = one sample: 1 of the 48 fields through the 3-mask chain, forward +
        # adjoint (6 propagations).  Every propagation of the workload costs the same, so
        # the per-propagation rate of the sample is the workload's rate.  `steps` counts
        # the samples actually timed and `ms_per_step` is the median time of one sample.
        inputs = make_inputs()
        for _ in range(max(1, args.warmup)):
            run_cpu_sample(budget_s=0.0, inputs=inputs)
        samples, secs = [], []
        for _ in range(args.steps):
            smp = run_cpu_sample(budget_s=0.0, inputs=inputs)
            secs.append(smp.pop("seconds_per_rep"))  # the sample's own timed repetition
            samples.append(smp)
        props_per_sample = 2 * N_MASKS
        sec = statistics.median(secs)
        v = round(props_per_sample / sec, 3)
        cpu = dict(samples[0])
        cpu["value"] = v
        cpu["sample"] = (f"per step: 1 of 48 fields (HG00 at 0.640 um, 2048^2) through the 3-mask chain, forward + "
                         f"adjoint = {props_per_sample} propagations, FP64 numpy/scipy.fft with {cpu['cores']} workers")
        config = headline_config(48, world)
        config["sample"] = "1 of 48 fields per step (6 of the 288 propagations of the workload)"
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": round(sec * 1e3, 1),
                "props_per_sample": props_per_sample, "total_timed_s": round(sum(secs), 2),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (fp64)",
                "data": "synthetic, seeded", "config": config,
                "cpu_baseline": cpu,
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "Julia is absent on this box: the reference arm is the FP64 oracle restatement of the "
                        "reference's CPU path (FFTW replaced by pocketfft), one field of the batch per step"}
        print(json.dumps(line))
        return

    if args.config != 3:
        if rank == 0:
            fn = {2: run_config2, 4: run_config4, 5: run_config5}[args.config]
            print(json.dumps(fn(args)))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    line = run_gb300(args, rank, world)
    if rank == 0:
        if not args.no_plain:
            line["plain_cufft"] = run_plain()
            line["speedup_vs_plain_cufft"] = round(line["value"] / line["plain_cufft"]["value"] / world, 2)
        if not args.no_cpu and world == 1:
            line["cpu_baseline"] = run_cpu_sample()
            line["cpu_baseline"].pop("seconds_per_rep", None)
            one = run_cpu_sample(budget_s=6.0, threads=1)
            line["cpu_baseline"]["single_thread"] = {"value": one["value"], "unit": one["unit"], "cores": 1,
                                                     "sample": one["sample"]}
        if not args.no_configs and world == 1:
            line["configs"] = run_other_configs(args)
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
