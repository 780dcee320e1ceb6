#!/usr/bin/env python3
"""Benchmark of the GB300 BLINK dirty-imaging path; prints one JSON line on rank 0.

Workload (one step): a block of 256 antennas (32,896 baselines incl. autos), 64 channels over
150-180 MHz x 10 intervals of 1 s with Earth-rotated zenith UVW, 4-pol visibilities, imaged to
640 dirty images of 512x512 (pol XX, oversampling 2, natural weighting): geometric + cable
corrections, nearest-neighbour gridding, inverse 2D FFT, fftshift and normalisation.  Inputs are
seeded synthetic data with that shape (no public data set exists for this path).

The timed step images the block from its stored form (--storage): by default 16-bit block
floating point (int16 pol planes with one FP32 scale per 128 baselines, encoded once before
timing, as stored data), checked against the FP64 oracle of the original complex64
visibilities; complex64 storage, bf16/fp16 storage, the deterministic gridder, the full-plane
path and the reference's plain FP32 call sequence are timed beside it as variants.  The other
workloads run as sections of the same line: `serving` (Poisson and closed-loop requests from
three arrays), `batched_uneven` (four image sizes as direct calls and as one CUDA graph) and
`precision_form` (768 channels x 20 intervals at 1024^2 in every storage format, errors
against the FP64 oracle).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference] [--storage s16|c64|bf16|fp16]

`--impl reference` times the reference's CPU imaging path (the C restatement in oracle/, run
with every host thread) on bounded samples of the same workload.  Under torchrun each rank
images its own block (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
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

METRIC = "images/s & vis/s: mixed-precision batched vs plain FP32 GPU at ≤1e-4 rel err"
WORKLOAD = ("256 antennas in a 35 m disk (32896 baselines incl. autos), 64 channels 150-180 MHz x "
            "10 intervals (1 s, Earth-rotated zenith UVW), complex64 4-pol visibilities -> 640 dirty "
            "images 512x512, pol XX, osf 2, natural weighting: geometric+cable corrections, "
            "nearest-neighbour gridding, inverse 2D FFT, fftshift + 1/sum(w)")
HBM_PEAK_FALLBACK = 6800.0


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return HBM_PEAK_FALLBACK, "fallback"


# ------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples every 100 ms; lines are kept for the GPU whose UUID matches."""
    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, uuid: str):
        self.samples = []
        self.proc = None
        self.uuid = uuid.lower().replace("gpu-", "") if uuid else ""

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            uid = parts[0].lower().replace("gpu-", "")
            if self.uuid and uid != self.uuid:
                continue
            if not self.uuid:
                self.uuid = uid
            try:
                self.samples.append((time.monotonic(), float(parts[1]), float(parts[2]), parts[4:8]))
            except ValueError:
                pass

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        inside = [s for s in self.samples if t0 <= s[0] <= t1]
        basis = "timed region"
        if len(inside) < 3:
            inside = self.samples
            basis = "whole run (timed region shorter than the sampling period)"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "basis": "nvidia-smi unavailable"}
        reasons = sorted({self.NAMES[i] for s in inside for i, r in enumerate(s[3]) if r.lower() == "active"})
        return {"sm_mhz": statistics.median(s[1] for s in inside), "sm_max_mhz": max(s[2] for s in inside),
                "reasons": reasons, "samples": len(inside), "basis": basis}


# ------------------------------------------------------------------------------------------
# CPU baseline: the reference CPU path restated in oracle/ (OpenMP, every host thread)
# ------------------------------------------------------------------------------------------
def cpu_sample_rate(obs, n_channels_sample: int, seconds: float, steps: int = 0):
    """Images/s of the CPU path on interval 0 x the first n channels: corrections, gridding,
    FFT (FP32), normalise, shift.  Repeats until `seconds` or for `steps` repetitions."""
    from oracle import oracle as O
    O.build()
    vis0 = np.ascontiguousarray(obs.vis_f32()[:1, :n_channels_sample])
    u, v, w = obs.u[:1], obs.v[:1], obs.w[:1]
    freqs = obs.freqs[:n_channels_sample]
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, obs.n_pixels), O.delta_uv(2.0, vmax, obs.n_pixels)
    times = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        vis = vis0.copy()
        O.apply_geometric(vis, w, freqs)
        O.apply_cable(vis, obs.cable, freqs)
        O.run_f32(vis, u, v, obs.flags, freqs, du, dv, obs.n_pixels, -1000.0, "XX")
        times.append(time.perf_counter() - t0)
        if steps and len(times) >= steps:
            break
        if not steps and time.perf_counter() - t_start >= seconds:
            break
    return n_channels_sample / statistics.median(times), times, O.library().bgo_max_threads()


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from imager_gb300 import synth
    obs = synth.config2(device="cpu", n_intervals=1)
    n_sample = 16
    from oracle import oracle as O
    O.build()
    # warm-up steps, then K timed steps (each a bounded 16-image sample of the workload)
    cpu_sample_rate(obs, n_sample, 0.0, steps=max(1, args.warmup))
    rate, times, threads = cpu_sample_rate(obs, n_sample, 0.0, steps=args.steps)
    ms = 1000.0 * statistics.mean(times)
    out = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "images/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded; shapes of the workload)",
           "config": {"workload": WORKLOAD, "images_per_step": n_sample},
           "cpu_baseline": {"value": rate, "unit": "images/s", "cores": threads, "kind": "port",
                            "sample": f"{n_sample} images (interval 0, channels 0-{n_sample - 1}) per step: "
                                      "corrections, gridding, FP32 FFT, normalise, shift"},
           "e2e": {"value": rate, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference CPU path restated in C (oracle/); the reference's own build needs astroio, "
                   "FFTW, cfitsio and msfitslib, absent on this box"}
    print(json.dumps(out), flush=True)
    return 0


# ------------------------------------------------------------------------------------------
# our arm
# ------------------------------------------------------------------------------------------
SAMPLES = ((0, 0), (-1, 63), (4, 31))  # (interval, channel) of the images checked each run


def sample_references(obs, du, dv, T):
    """FP64 oracle images of the sample images from the original complex64 visibilities."""
    from oracle import oracle as O
    O.build()
    vis_np = obs.vis_f32()
    refs = {}
    for t, c in SAMPLES:
        t = t % T
        corr = np.ascontiguousarray(vis_np[t:t + 1, c:c + 1])
        O.apply_geometric(corr, np.ascontiguousarray(obs.w[t:t + 1]), obs.freqs[c:c + 1])
        O.apply_cable(corr, obs.cable, obs.freqs[c:c + 1])
        g, cnt, _ = O.gridding(corr, obs.u[t:t + 1], obs.v[t:t + 1], obs.flags, obs.freqs[c:c + 1], du, dv,
                               obs.n_pixels)
        refs[(t, c)] = O.image_f64(g, cnt)[0, 0]
    return refs


def image_errors(out, refs):
    """Per sample image: relative L2, max |err| / max |ref| and RMS err / RMS ref; the worst of each."""
    worst = {"rel_l2": 0.0, "max_err_rel": 0.0, "rms_err_rel": 0.0}
    for (t, c), ref in refs.items():
        got = out[t, c].cpu().numpy().astype(np.complex128)
        d = np.abs(got - ref)
        worst["rel_l2"] = max(worst["rel_l2"], float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
        worst["max_err_rel"] = max(worst["max_err_rel"], float(d.max() / np.abs(ref).max()))
        worst["rms_err_rel"] = max(worst["rms_err_rel"], float(np.sqrt((d ** 2).mean() / (np.abs(ref) ** 2).mean())))
    return worst


L2_FLUSH_BYTES = 512 << 20  # written between timed steps: four times the 129 MB L2


class L2Flush:
    def __init__(self):
        import torch
        self.buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.zero_()


def timed_steps(step, k, stream, flush, pre=None):
    """Total ms of k steps, each bracketed by its own CUDA events on `stream` with the L2 flushed
    before it (outside the events); `pre()`, when given, runs before the flush (outside too)."""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    for e0, e1 in evs:
        if pre:
            pre()
        flush()
        e0.record(stream)
        step()
        e1.record(stream)
    torch.cuda.synchronize()
    return sum(e0.elapsed_time(e1) for e0, e1 in evs)


def time_steps(step, k, stream, flush, pre=None):
    """ms per step of `step()` over k steps after two untimed ones."""
    import torch
    for _ in range(2):
        if pre:
            pre()
        step()
    torch.cuda.synchronize()
    return timed_steps(step, k, stream, flush, pre) / k


def plain_dropin_step(obs, vis, du, dv, out, cufft=False):
    """The reference GPU imager's call sequence (src/gpu/pacer_imager_hip.cpp:36-146) through
    the free functions: corrections in place, grids and counters zeroed, atomic gridding with
    per-channel counters, unfused inverse FFT into the images, counter sums, fftshift and
    normalisation -- FP32 and complex64 throughout, full plane, no fusion.  cufft: the FFT stage
    is cuFFT (torch.fft.ifft2, unnormalised), as the reference's gpufftExecC2C call -- a timing
    arm only; the product's FFT is its own."""
    import torch
    from imager_gb300 import capi
    from imager_gb300 import imager as IM
    T, Cn, B = vis.shape[:3]
    N = obs.n_pixels
    work = torch.empty_like(vis)
    w, cable, freqs = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (obs.w, obs.cable, obs.freqs))
    u, v, flags = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (obs.u, obs.v, obs.flags))
    grids = torch.empty((T, Cn, N, N), dtype=torch.complex64, device="cuda")
    counters = torch.empty((Cn, N, N), dtype=torch.float32, device="cuda")
    fnorm = torch.empty(Cn, dtype=torch.float32, device="cuda")

    def step():
        IM.apply_geometric_corrections(work, w, freqs, n_uvw_sets=T)
        IM.apply_cable_corrections(work, cable, freqs)
        grids.zero_()
        counters.zero_()
        IM.gridding(work, u, v, flags, freqs, du, dv, N, -1000.0, "XX", grids, counters,
                    counter_mode=capi.COUNTERS_FIRST_INTERVAL, n_uvw_sets=T)
        if cufft:
            torch.fft.ifft2(grids, norm="forward", out=out)
        else:
            IM.fft_inverse(grids, out)
        IM.vector_sum(counters, N * N, Cn, fnorm)
        IM.fft_shift_and_norm(out, fnorm)

    def fresh():  # the reference corrects each block's visibilities in place once
        work.copy_(vis)

    return step, fresh


def serving_measure(args):
    """The serving workload through bgi_server: blocks of 32 channels x 1 interval from a mix of
    128/256/512-antenna arrays (images 256/512/1024^2), stored as s16, complex images back to
    pinned host buffers.  Phase 1: Poisson arrivals (mean args.serve_interarrival_ms) -> latency
    p50/p99.  Phase 2: closed loop with args.serve_outstanding requests outstanding -> sustained
    images/s.  Errors: channel 0 of one request per array against the FP64 oracle."""
    import collections
    import torch
    from imager_gb300 import imager as IM
    from imager_gb300 import server as SV
    from imager_gb300 import synth
    from oracle import oracle as O
    arrays = synth.serving_arrays(device="cuda")
    rng = np.random.default_rng(1239)
    K = args.serve_outstanding
    res = {"workload": "arrays of 128 (35 m disk, 256^2), 256 (35 m disk, 512^2) and 512 antennas (16 sub-stations "
                       "over 3 km, 1024^2); blocks of 32 channels x 1 interval, s16 stored, pol XX, corrections "
                       "fused, complex images to pinned host memory; array of each request drawn uniformly",
           "slots": args.serve_slots}
    with SV.Server(max_slots=args.serve_slots) as sv:
        ids = [sv.add_array(o.n_pixels, o.u, o.v, o.w, o.flags, o.cable, o.freqs) for o in arrays]
        stored = []
        for o in arrays:
            d, sc = IM.compress_visibilities(torch.from_numpy(o.vis_f32()).cuda(), "s16")
            stored.append((d.cpu().pin_memory(), sc.cpu().pin_memory()))
        bufs = [collections.deque(torch.empty((1, o.n_channels, o.n_pixels, o.n_pixels), dtype=torch.complex64,
                                              pin_memory=True) for _ in range(K)) for o in arrays]
        busy = collections.deque()  # (ticket, array index, buffer, submit time), in submission order
        lat = [[] for _ in arrays]   # client-side submit-to-collected ms per array

        def collect():
            t, kk, b, ts = busy.popleft()
            sv.wait(t)
            lat[kk].append((time.perf_counter() - ts) * 1000.0)
            bufs[kk].append(b)

        def collect_finished():  # without blocking: the oldest requests that are done
            while busy:
                t, kk, b, ts = busy[0]
                if sv.poll(t) is None:
                    return
                busy.popleft()
                lat[kk].append((time.perf_counter() - ts) * 1000.0)
                bufs[kk].append(b)

        def submit(k):
            while not bufs[k]:  # reuse a buffer only after its request is collected
                collect()
            b = bufs[k].popleft()
            ts = time.perf_counter()
            t = sv.submit(ids[k], data=stored[k][0], scales=stored[k][1], fmt="s16", out=b)
            busy.append((t, k, b, ts))

        def drain():
            while busy:
                collect()

        def per_array():
            out = {f"{o.n_pixels}px_{o.n_ant}ant": {"requests": len(x), "p50_ms": float(np.percentile(x, 50)),
                                                    "max_ms": float(np.max(x))}
                   for o, x in zip(arrays, lat) if x}
            for x in lat:
                x.clear()
            return out

        for k in range(len(arrays)):  # warm every slot's handle for every array
            for _ in range(args.serve_slots):
                submit(k)
            drain()
        # errors of one request per array, channel 0
        errs = []
        for k, o in enumerate(arrays):
            submit(k)
            t, kk, b, _ = busy.pop()
            out = sv.wait(t)[0, 0].numpy().astype(np.complex128)
            bufs[kk].append(b)
            corr = np.ascontiguousarray(o.vis_f32()[:, :1])
            O.apply_geometric(corr, o.w, o.freqs[:1])
            O.apply_cable(corr, o.cable, o.freqs[:1])
            umax, vmax = O.uv_max(o.u, o.v, o.flags)
            du, dv = O.delta_uv(2.0, umax, o.n_pixels), O.delta_uv(2.0, vmax, o.n_pixels)
            g, cnt, _ = O.gridding(corr, o.u, o.v, o.flags, o.freqs[:1], du, dv, o.n_pixels)
            ref = O.image_f64(g, cnt)[0, 0]
            errs.append(float(np.linalg.norm(out - ref) / np.linalg.norm(ref)))
        res["errors_vs_fp64_rel_l2"] = max(errs)
        # phase 1: Poisson arrivals
        per_array()
        sv.reset_stats()
        t0 = time.perf_counter()
        arrival = 0.0
        for _ in range(args.serve_requests):
            arrival += rng.exponential(args.serve_interarrival_ms / 1000.0)
            while time.perf_counter() - t0 < arrival:
                collect_finished()
                time.sleep(0.0002)
            submit(int(rng.integers(len(arrays))))
        drain()
        st = sv.stats()
        res["poisson"] = {"mean_interarrival_ms": args.serve_interarrival_ms, "requests": st["completed"],
                          "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                          "p99_note": "p99 over >= 1000 requests" if st["completed"] >= 1000 else
                                      f"only {st['completed']} requests: p99 is close to the maximum",
                          "images_per_s": st["images_per_s"], "failed": st["failed"],
                          "client_latency_by_array": per_array()}
        # phase 2: closed loop, K outstanding per array
        sv.reset_stats()
        for _ in range(args.serve_requests * 3):
            submit(int(rng.integers(len(arrays))))
        drain()
        st = sv.stats()
        res["saturated"] = {"outstanding_per_array": K, "requests": st["completed"], "p50_ms": st["p50_ms"],
                            "p99_ms": st["p99_ms"], "images_per_s": st["images_per_s"],
                            "admission_waits": st["admission_waits"], "failed": st["failed"],
                            "client_latency_by_array": per_array()}
    return res


def host_link_rates(host_out, h2d_bytes, reps=3):
    """Plain copies over the host link with the step's byte counts: the pinned image buffer
    from a device buffer of its size (device to host) and h2d_bytes from pinned memory (host to
    device), each timed with CUDA events on the current stream, best of `reps`.  The end-to-end
    step cannot beat max(d2h / d2h_gbs, h2d / h2d_gbs), the two directions running at once."""
    import torch
    s = torch.cuda.current_stream()
    dev = torch.empty(host_out.numel(), dtype=host_out.dtype, device="cuda")
    src_h = torch.empty(max(h2d_bytes // 4, 1), dtype=torch.float32).pin_memory()
    dst_d = torch.empty_like(src_h, device="cuda")
    host_flat = host_out.view(-1)

    def rate(fn, nbytes):
        best = float("inf")
        for _ in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(s)
            fn()
            e1.record(s)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return nbytes / (best / 1000.0) / 1e9

    d2h = rate(lambda: host_flat.copy_(dev, non_blocking=True), host_out.numel() * host_out.element_size())
    h2d = rate(lambda: dst_d.copy_(src_h, non_blocking=True), src_h.numel() * 4)
    del dev, dst_d, src_h
    return {"d2h_gbs": d2h, "h2d_gbs": h2d,
            "what": "plain pinned copies of the step's bytes over the host link (cudaMemcpyAsync through "
                    "torch), each direction alone, best of 3"}


def batched_measure(args, stream, flush):
    """The uneven batch workload: 512 antennas in 16 sub-stations, 256 channels in four bands of 64
    imaged at 256/512/1024/2048 pixels, 5 intervals, s16 stored, complex images on the device.
    Times the four bgi_image_compressed calls issued directly, the same batch replayed as one CUDA
    graph (bgi_batch_*), and the graph with the ordered gridder; checks one image per band against
    the FP64 oracle."""
    import torch
    from imager_gb300 import imager as IM
    from imager_gb300 import synth
    from oracle import oracle as O
    bands = synth.batched_bands(device="cuda")
    flags = IM.APPLY_GEOMETRIC | IM.APPLY_CABLE
    items, schedules = [], []
    for o in bands:
        h = IM.Imager(o.n_pixels, 2.0, "XX", -1000.0)
        h.set_array(o.u, o.v, o.w, o.flags, o.cable)
        h.set_frequencies(o.freqs)
        vis = torch.from_numpy(o.vis_f32()).cuda()
        d, sc = IM.compress_visibilities(vis, "s16")
        del vis
        out = torch.empty((o.n_intervals, o.n_channels, o.n_pixels, o.n_pixels), dtype=torch.complex64, device="cuda")
        schedules.append(h.autotune(d, sc, "s16", flags=flags, out=out)[:2])
        items.append(dict(imager=h, data=d, scales=sc, fmt="s16", flags=flags, out=out))
    n_images = sum(o.n_intervals * o.n_channels for o in bands)
    aggs = {f"{o.n_pixels}": it["imager"].gridding_aggregation for o, it in zip(bands, items)}  # autotuned
    k = max(3, min(args.steps, 10))

    def direct():
        for it in items:
            it["imager"].image_compressed(it["data"], it["scales"], "s16", flags=flags, out=it["out"])

    ms_direct = time_steps(direct, k, stream, flush)
    ms_band = {}
    for o, it in zip(bands, items):
        ms_band[f"{o.n_pixels}"] = time_steps(
            lambda it=it: it["imager"].image_compressed(it["data"], it["scales"], "s16", flags=flags, out=it["out"]),
            k, stream, flush)
    batch = IM.Batch(items)
    ms_graph = time_steps(batch.launch, k, stream, flush)
    torch.cuda.synchronize()
    errs = []
    for o, it in zip(bands, items):
        corr = np.ascontiguousarray(o.vis_f32()[:1, :1])
        O.apply_geometric(corr, np.ascontiguousarray(o.w[:1]), o.freqs[:1])
        O.apply_cable(corr, o.cable, o.freqs[:1])
        du, dv, _, _ = it["imager"].uv_cell
        g, cnt, _ = O.gridding(corr, o.u[:1], o.v[:1], o.flags, o.freqs[:1], du, dv, o.n_pixels)
        ref = O.image_f64(g, cnt)[0, 0]
        got = it["out"][0, 0].cpu().numpy().astype(np.complex128)
        errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    batch.close()
    for it in items:
        it["imager"].set_deterministic(True)
    batch = IM.Batch(items)
    ms_det = time_steps(batch.launch, k, stream, flush)
    batch.close()
    for it in items:
        it["imager"].close()
    return {"workload": "512 antennas in 16 sub-stations over 3 km (131,328 baselines), 256 channels 100-200 MHz in "
                        "four bands of 64 imaged at 256/512/1024/2048 pixels, 5 intervals (1,280 images per step), "
                        "400 point sources + diffuse power-law background, s16 stored, pol XX, corrections fused",
            "images_per_step": n_images, "steps": k,
            "schedules": {f"{o.n_pixels}": {"images_per_wave": w or "auto", "lanes": l}
                          for o, (w, l) in zip(bands, schedules)},
            "direct_calls": {"ms_per_step": ms_direct, "images_per_s": n_images / (ms_direct / 1000.0),
                             "ms_per_band": ms_band},
            "gridding_aggregation": aggs,
            "cuda_graph": {"ms_per_step": ms_graph, "images_per_s": n_images / (ms_graph / 1000.0)},
            "cuda_graph_deterministic": {"ms_per_step": ms_det, "images_per_s": n_images / (ms_det / 1000.0)},
            "errors_vs_fp64_rel_l2": {f"{o.n_pixels}": e for o, e in zip(bands, errs)}}


def precision_measure(args, stream, flush):
    """The precision form: 128 antennas in a 3 km disk with log-radial density, 768 channels of
    10 kHz from 150 MHz x 20 intervals, 1024x1024 images (15,360 per step, complex64 on the
    device: 129 GB), from complex64 records and from 16-bit storage with one FP32 scale per 128
    baselines (256 components): s16, bf16 and fp16.  Per format: images/s over the whole block
    and, for three sampled images, the error against the FP64 oracle (relative L2 and the
    largest absolute error relative to the image peak)."""
    import torch
    from imager_gb300 import imager as IM
    from imager_gb300 import synth
    from oracle import oracle as O
    obs = synth.precision_form(device="cuda")
    T, Cn, n = obs.n_intervals, obs.n_channels, obs.n_pixels
    vis = obs.vis_f32()  # float32 [T][C][B][4][2] on the device
    flags = IM.APPLY_GEOMETRIC | IM.APPLY_CABLE
    h = IM.Imager(n, 2.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    du, dv, _, _ = h.uv_cell
    # schedule tuned on the first interval (a one-set imager with the block's uv cell)
    t1 = IM.Imager(n, 2.0, "XX", -1000.0)
    t1.set_array(obs.u[:1], obs.v[:1], obs.w[:1], obs.flags, obs.cable)
    t1.set_frequencies(obs.freqs)
    t1.set_uv_cell(du, dv)
    d1, s1 = IM.compress_visibilities(vis[:1], "s16")
    wave, lanes, _ = t1.autotune(d1, s1, "s16", flags=flags)
    t1.close()
    del d1, s1
    h.set_schedule(wave, lanes)
    # complex images of the whole block (129 GB); real images (half) when the device has less free
    free, _ = torch.cuda.mem_get_info()
    need_complex = T * Cn * n * n * 8 + 4 * vis.numel() + (4 << 30)  # images, stored forms, margin
    real_out = free < need_complex
    flags = flags | (IM.OUTPUT_REAL if real_out else 0)
    out = torch.empty((T, Cn, n, n), dtype=torch.float32 if real_out else torch.complex64, device="cuda")
    samples = ((0, 0), (T // 2, Cn // 2), (T - 1, Cn - 1))
    refs = {}
    for t, c in samples:
        corr = np.ascontiguousarray(vis[t:t + 1, c:c + 1].cpu().numpy())
        O.apply_geometric(corr, np.ascontiguousarray(obs.w[t:t + 1]), obs.freqs[c:c + 1])
        O.apply_cable(corr, obs.cable, obs.freqs[c:c + 1])
        g, cnt, _ = O.gridding(corr, obs.u[t:t + 1], obs.v[t:t + 1], obs.flags, obs.freqs[c:c + 1], du, dv, n)
        refs[(t, c)] = O.image_f64(g, cnt)[0, 0]
    k = max(3, min(args.steps, 5))
    n_images = T * Cn
    gridded = int((obs.flags == 0).sum())
    formats = {}
    for fmt in ("s16", "bf16", "fp16", "c64"):
        if fmt == "c64":
            step = lambda: h.image(vis, flags=flags, out=out)  # noqa: E731
        else:
            data, scales = IM.compress_visibilities(vis, fmt)
            step = lambda: h.image_compressed(data, scales, fmt, flags=flags, out=out)  # noqa: E731
        ms = time_steps(step, k, stream, flush)
        torch.cuda.synchronize()
        errs = []
        for t, c in samples:
            got = out[t, c].cpu().numpy().astype(np.complex128)
            ref = refs[(t, c)]
            errs.append((float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                         float(np.abs(got - ref).max() / np.abs(ref).max())))
        formats[fmt] = {"ms_per_step": ms, "images_per_s": n_images / (ms / 1000.0),
                        "vis_per_s": n_images * gridded / (ms / 1000.0),
                        "rel_l2_max": max(e[0] for e in errs), "max_abs_err_rel_peak": max(e[1] for e in errs),
                        "rel_l2_per_image": [e[0] for e in errs]}
        if fmt != "c64":
            del data, scales
    h.close()
    del out, vis, obs
    torch.cuda.empty_cache()
    return {"workload": "128 antennas in a 3 km disk with log-radial density (8,256 baselines), 768 channels of "
                        "10 kHz from 150 MHz x 20 intervals (1 s, Earth-rotated zenith UVW) -> 15,360 dirty images "
                        "1024x1024 per step (complex64, 129 GB on the device), pol XX, corrections fused (delay "
                        "phase reduced in double-float), 16-bit formats with one FP32 scale per 128 baselines",
            "images_per_step": n_images, "steps": k,
            "schedule": {"images_per_wave": wave or "auto", "lanes": lanes, "chosen_by": "bgi_autotune on interval 0"},
            "images": "real (float32): the device had less free memory than the complex block needs" if real_out
            else "complex64",
            "sampled_images": [f"interval {t}, channel {c}" for t, c in samples],
            "oracle": "FP64 oracle of the original complex64 visibilities",
            "fft": "FP32 Stockham passes of our own (the tensor-core row pass is built for 512^2 only)",
            "formats": formats}


def run_ours(args, rank, world, local_rank):
    import torch
    from imager_gb300 import capi, synth
    from imager_gb300 import imager as IM
    from imager_gb300.imager import APPLY_CABLE, APPLY_GEOMETRIC, Imager

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    capi.lib(build_if_missing=True)
    whole_cell = None
    if world == 1:
        obs = synth.config2(device="cuda", n_intervals=args.intervals)
    else:
        # N GPUs: one observation of N blocks' intervals, split by the library's shard plan (each
        # rank images its own intervals with the whole observation's uv cell; no collective on
        # the data path) -- weak scaling, the same 64 x args.intervals images per GPU
        from imager_gb300 import shard as SH
        whole = synth.config2(device="cuda", n_intervals=args.intervals * world)
        probe = Imager(whole.n_pixels, 2.0, "XX", -1000.0)
        probe.set_array(whole.u, whole.v, whole.w, whole.flags, whole.cable)
        whole_cell = probe.uv_cell[:2]
        probe.close()
        _, obs = SH.shard_observation(whole, world, rank)
        del whole
    T, Cn, B = obs.vis.shape[:3]
    N = obs.n_pixels
    n_images = T * Cn
    vis_np = obs.vis_f32()
    vis = torch.from_numpy(vis_np).cuda()
    out = torch.empty((T, Cn, N, N), dtype=torch.complex64, device="cuda")
    fmt = args.storage
    # stored visibilities: the block arrives in the storage format (encoded once, untimed)
    stored = {f: IM.compress_visibilities(vis, f) for f in ("s16", "bf16", "fp16")}
    torch.cuda.synchronize()
    im = Imager(N, 2.0, "XX", -1000.0, max_images_per_wave=args.wave)
    im.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    im.set_frequencies(obs.freqs)
    if whole_cell:
        im.set_uv_cell(*whole_cell)
    flags = APPLY_GEOMETRIC | APPLY_CABLE
    stream = torch.cuda.current_stream()

    def step_for(h, f):
        if f == "c64":
            return lambda: h.image(vis, flags=flags, out=out)
        d, sc = stored[f]
        return lambda: h.image_compressed(d, sc, f, flags=flags, out=out)

    step = step_for(im, fmt)
    tuned = None
    if args.autotune:  # wave size and lane count timed on this block (bgi_autotune), untimed here
        if fmt == "c64":
            tuned = im.autotune(vis, None, "c64", flags=flags, out=out)
        else:
            tuned = im.autotune(stored[fmt][0], stored[fmt][1], fmt, flags=flags, out=out)
    if args.fft_mode:
        im.set_fft_mode(args.fft_mode)
    if args.gridding_images_per_thread:
        im.set_gridding_images_per_thread(args.gridding_images_per_thread)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sums = im.weight_sums(n_images)
    gridded_vis = int(sums.sum()) // 2  # each gridded visibility lands at two cells

    props = torch.cuda.get_device_properties(local_rank)
    uuid = str(getattr(props, "uuid", "") or "")
    clocks = ClockSampler(uuid if len(uuid.replace("GPU-", "")) == 36 else "")
    clocks.start()
    time.sleep(0.3)
    flush = L2Flush()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.monotonic()
    ms = timed_steps(step, args.steps, stream, flush)
    t1 = time.monotonic()
    if dist:
        dist.barrier()
    # per-stage device times from a separate pass (the stage events cost a few percent, so the
    # timed steps above run without them)
    stage_steps = max(3, min(args.steps, 20))
    im.set_stage_timing(True)
    timed_steps(step, stage_steps, stream, flush)
    stages = im.stage_times()
    im.set_stage_timing(False)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    du, dv, _, _ = im.uv_cell
    refs = sample_references(obs, du, dv, T) if rank == 0 else {}
    errs = image_errors(out, refs) if rank == 0 else {}

    # variants of the same step, timed the same way over fewer steps, with their sample errors
    variants = {}
    if args.variants:
        k = max(3, min(args.steps, 20))
        for f in ("c64", "s16", "bf16", "fp16"):
            if f == fmt:
                continue
            v_ms = time_steps(step_for(im, f), k, stream, flush)
            variants[f"storage_{f}"] = {"images_per_s": world * n_images / (v_ms / 1000.0), "ms_per_step": v_ms,
                                        "steps": k, **({"errors_vs_fp64": image_errors(out, refs)} if rank == 0 else {})}
        # the complex-to-real pass on the tensor cores (split-FP16 DFT products), same step
        step_mode = im.fft_mode
        im.set_fft_mode("tensor_split16")
        v_ms = time_steps(step, k, stream, flush)
        tc_errs = image_errors(out, refs) if rank == 0 else {}
        im.set_stage_timing(True)
        timed_steps(step, stage_steps, stream, flush)
        tc_stages = im.stage_times()
        im.set_stage_timing(False)
        im.set_fft_mode(step_mode)
        tc_pass2 = tc_stages.get("fft_pass2", (0.0, 0))
        variants["fft_tensor_split16"] = {
            "images_per_s": world * n_images / (v_ms / 1000.0), "ms_per_step": v_ms, "steps": k, "storage": fmt,
            "fft_pass2_ms_per_launch": tc_pass2[0] / tc_pass2[1] if tc_pass2[1] else None,
            "what": "complex-to-real row pass with its length-256 transforms as two 16-point DFT products on "
                    "the tensor cores (mma.sync m16n8k16, FP16 hi+lo operand splits, three products, FP32 "
                    "accumulation)",
            **({"errors_vs_fp64": tc_errs} if rank == 0 else {})}
        im.set_deterministic(True)
        v_ms = time_steps(step, k, stream, flush)
        im.set_deterministic(False)
        variants["deterministic_sorted_gridding"] = {"images_per_s": world * n_images / (v_ms / 1000.0),
                                                     "ms_per_step": v_ms, "steps": k, "plane": "full",
                                                     "storage": fmt}
        full = Imager(N, 2.0, "XX", -1000.0, max_images_per_wave=args.wave, full_plane=True)
        full.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
        full.set_frequencies(obs.freqs)
        if whole_cell:
            full.set_uv_cell(*whole_cell)
        v_ms = time_steps(step_for(full, fmt), k, stream, flush)
        full.close()
        variants["full_plane_atomic_gridding"] = {"images_per_s": world * n_images / (v_ms / 1000.0),
                                                  "ms_per_step": v_ms, "steps": k, "plane": "full", "storage": fmt}
        out_r = torch.empty((T, Cn, N, N), dtype=torch.float32, device="cuda")
        d, sc = stored[fmt] if fmt != "c64" else (None, None)
        real_step = (lambda: im.image(vis, flags=flags | IM.OUTPUT_REAL, out=out_r)) if fmt == "c64" else \
            (lambda: im.image_compressed(d, sc, fmt, flags=flags | IM.OUTPUT_REAL, out=out_r))
        v_ms = time_steps(real_step, k, stream, flush)
        variants["real_output"] = {"images_per_s": world * n_images / (v_ms / 1000.0), "ms_per_step": v_ms,
                                   "steps": k, "storage": fmt,
                                   "what": "BGI_OUTPUT_REAL: float images (the real part) from the last FFT pass",
                                   **({"errors_vs_fp64": image_errors(out_r.to(torch.complex64), refs)}
                                      if rank == 0 else {})}
        del out_r
        plain_step, plain_fresh = plain_dropin_step(obs, vis, du, dv, out)
        v_ms = time_steps(plain_step, k, stream, flush, pre=plain_fresh)
        refs0 = {key: r for key, r in refs.items() if key[0] == 0}  # per-channel norm equals per-image at t=0
        variants["plain_fp32_dropin"] = {
            "images_per_s": world * n_images / (v_ms / 1000.0), "ms_per_step": v_ms, "steps": k,
            "what": "reference GPU call order through the free functions: corrections in place, gridding "
                    "with counters, unfused FFT, vector sum, fftshift+norm; complex64/FP32, full plane",
            **({"errors_vs_fp64_interval0": image_errors(out, refs0)} if rank == 0 else {})}
        plain_step, plain_fresh = plain_dropin_step(obs, vis, du, dv, out, cufft=True)
        v_ms = time_steps(plain_step, k, stream, flush, pre=plain_fresh)
        variants["plain_fp32_dropin_cufft"] = {
            "images_per_s": world * n_images / (v_ms / 1000.0), "ms_per_step": v_ms, "steps": k,
            "what": "the same call order with the FFT stage done by cuFFT (torch.fft.ifft2, unnormalised) as "
                    "the reference's gpufftExecC2C -- timing arm only, never in the product",
            **({"errors_vs_fp64_interval0": image_errors(out, refs0)} if rank == 0 else {})}

        # the reference's gridding call alone (bgi_gridding_gpu, gridding_gpu.cpp:130): complex64
        # records, full-plane grids [T][C][N][N], per-channel counters of the first interval;
        # grids and counters zeroed before each step outside its events
        cnt = torch.empty((Cn, N, N), dtype=torch.float32, device="cuda")
        u_d, v_d, fl_d, fr_d = (torch.from_numpy(np.ascontiguousarray(a)).cuda()
                                for a in (obs.u, obs.v, obs.flags, obs.freqs))

        def zero_grids():
            out.zero_()
            cnt.zero_()

        grid_step = lambda: IM.gridding(vis, u_d, v_d, fl_d, fr_d, du, dv, N, -1000.0, "XX", out, cnt,  # noqa: E731
                                        counter_mode=capi.COUNTERS_FIRST_INTERVAL, n_uvw_sets=T)
        g_ms = time_steps(grid_step, k, stream, flush, pre=zero_grids)
        g_alg = B * 32 + 8 * N * N + 4 * N * N / T  # per image: records, grid, counters (per channel)
        g_gbs = n_images * g_alg / (g_ms / 1000.0) / 1e9
        g_peak, _ = measured_peaks()
        # The atomics touch only the cells that visibilities land in.  Each touched 32-byte sector
        # of the zeroed (and flushed) grids and counters is read from DRAM once and written back
        # once; with the records that is the traffic the kernel cannot avoid.
        zero_grids()
        grid_step()
        grid_sectors = int((out.view(torch.float32).reshape(n_images, -1, 8) != 0).any(-1).sum())
        cnt_sectors = int((cnt.reshape(Cn, -1, 8) != 0).any(-1).sum())
        g_min = B * 32 + 64 * (grid_sectors + cnt_sectors / T) / n_images
        g_min_gbs = n_images * g_min / (g_ms / 1000.0) / 1e9
        variants["gridding_free_function"] = {
            "ms_per_step": g_ms, "images_per_s": world * n_images / (g_ms / 1000.0), "steps": k,
            "algorithmic_bytes_per_image": g_alg, "achieved_gbs": g_gbs, "frac_of_hbm": g_gbs / g_peak,
            "touched_sector_bytes_per_image": g_min, "touched_sector_gbs": g_min_gbs,
            "touched_sector_frac_of_hbm": g_min_gbs / g_peak,
            "what": "gridding_gpu's call alone: complex64 records in, full-plane complex64 grids and per-channel "
                    "counters out (atomics), all the step's images in one call; algorithmic bytes B*32 + 8*N^2 + 4*N^2/T per image; "
                    "touched-sector bytes B*32 + 64 per grid or counter sector the atomics touch (read and "
                    "written back)"}
        del cnt

    # end to end through the host-buffer entry points: pinned input, pinned output, the uploads
    # and downloads inside the timed region.  The headline uploads the stored block (for the
    # 16-bit formats only the XX plane and its scales) and downloads real images: XX images are
    # real (BGI_OUTPUT_REAL stores the real part; the half-plane path makes no imaginary part).
    # Beside it: complex images back (the reference's Images type), and the reference caller's
    # own input -- complex64 records -- with real and with complex images back.
    e2e_steps = max(3, min(args.steps, 20))

    def e2e_time(fn):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(e2e_steps):
            fn()
        return (time.perf_counter() - t) / e2e_steps

    out_hr = torch.empty((T, Cn, N, N), dtype=torch.float32).pin_memory()
    vis_h = torch.from_numpy(vis_np).pin_memory()
    h2d_c64 = vis_np.nbytes
    if fmt == "c64":
        e2e_step = lambda: im.image_host(vis_h, flags=flags | IM.OUTPUT_REAL, out=out_hr)  # noqa: E731
        h2d = h2d_c64
    else:
        d_h = stored[fmt][0].cpu().pin_memory()
        s_h = stored[fmt][1].cpu().pin_memory()
        e2e_step = lambda: im.image_compressed_host(d_h, s_h, fmt, flags=flags | IM.OUTPUT_REAL, out=out_hr)  # noqa: E731
        n_planes = 1  # pol XX reads one plane
        h2d = n_images * n_planes * (B * 4 + int(s_h.shape[-1]) * 4)
    e2e_s = e2e_time(e2e_step)
    d2h_real, d2h_complex = n_images * N * N * 4, n_images * N * N * 8
    link = host_link_rates(out_hr, h2d)
    e2e_variants = {}
    if args.variants:
        out_h = torch.empty((T, Cn, N, N), dtype=torch.complex64).pin_memory()
        cplx = (lambda: im.image_host(vis_h, flags=flags, out=out_h)) if fmt == "c64" else \
            (lambda: im.image_compressed_host(d_h, s_h, fmt, flags=flags, out=out_h))
        e2e_variants[f"{fmt}_input_complex_output"] = {
            "images_per_s": world * n_images / e2e_time(cplx), "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h_complex}
        if fmt != "c64":
            e2e_variants["c64_input_real_output"] = {
                "images_per_s": world * n_images / e2e_time(lambda: im.image_host(vis_h, flags=flags | IM.OUTPUT_REAL,
                                                                                  out=out_hr)),
                "h2d_bytes_per_step": h2d_c64, "d2h_bytes_per_step": d2h_real,
                "what": "the reference caller's complex64 records uploaded whole (4 pols, 32 B per baseline)"}
            e2e_variants["c64_input_complex_output"] = {
                "images_per_s": world * n_images / e2e_time(lambda: im.image_host(vis_h, flags=flags, out=out_h)),
                "h2d_bytes_per_step": h2d_c64, "d2h_bytes_per_step": d2h_complex,
                "what": "the reference caller's input and output types end to end"}
        # correlator output: the XX correlation matrices (element (i, j), j <= i, is baseline
        # i(i+1)/2 + j) uploaded, converted to s16 visibilities on the device and imaged
        n_ant = obs.n_ant
        ii, jj = np.tril_indices(n_ant)
        xx = np.zeros((T, Cn, n_ant, n_ant), np.complex64)
        xx[:, :, ii, jj] = np.asarray(obs.vis)[:, :, :, 0]
        re_h = torch.from_numpy(np.ascontiguousarray(xx.real)).pin_memory()
        im_h = torch.from_numpy(np.ascontiguousarray(xx.imag)).pin_memory()
        del xx
        e2e_variants["correlation_matrices_input_real_output"] = {
            "images_per_s": world * n_images / e2e_time(lambda: im.image_matrices_host(
                re_h, im_h, fmt="s16", flags=flags | IM.OUTPUT_REAL, out=out_hr)),
            "h2d_bytes_per_step": 2 * n_images * n_ant * n_ant * 4, "d2h_bytes_per_step": d2h_real,
            "what": "bgi_image_correlation_matrices_host: XX correlation matrices (float32 re, im) in, "
                    "ingested to s16 on the device, real images back"}
        del re_h, im_h
        del out_h
    t3 = time.monotonic()
    clocks.stop()
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    if rank != 0:
        dist.destroy_process_group()
        return 0
    def section(enabled, fn, *a):
        """A workload section of the line; its failure is reported in the line instead of ending
        the run (the headline above stands on its own)."""
        if not (enabled and world == 1):
            return None
        try:
            return fn(*a)
        except Exception as e:  # noqa: BLE001
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            return {"error": f"{type(e).__name__}: {e}"[:400]}

    serving = section(args.serving, serving_measure, args)
    batched = section(args.batched, batched_measure, args, stream, flush)
    precision = section(args.precision, precision_measure, args, stream, flush)

    images_per_s = world * n_images * args.steps / (ms / 1000.0)
    hbm_peak, peak_kind = measured_peaks()
    # algorithmic bytes per image of each stage, for the path the handle took
    # stored visibility bytes per image that the gridding must read: the complex64 record, or
    # for the 16-bit formats the one pol plane XX needs and its block scales
    vis_bytes = B * 32 if fmt == "c64" else B * 4 + int(stored[fmt][1].shape[-1]) * 4
    half = im.half_plane
    ext_u, ext_v = im.uv_extent
    if half:
        # the half-plane passes are pruned to the uv coverage: columns 0..ext_u, rows within
        # ext_v of row 0; gridding writes that region, the column pass reads its rows and writes
        # every row of its columns, the complex-to-real pass reads those columns of every row
        cols, rows_in = ext_u + 1, min(N, 2 * ext_v + 1)
        alg = {"gridding": vis_bytes + 8 * cols * rows_in, "fft_pass1": 8 * cols * (rows_in + N),
               "fft_pass2": 8 * cols * N + 8 * N * N}
        kernel_names = {"gridding": "grid_kernel", "fft_pass1": "fft_cols_half_kernel", "fft_pass2": "c2r_rows_kernel"}
    else:
        alg = {"gridding": vis_bytes + 8 * N * N, "fft_pass1": 16 * N * N, "fft_pass2": 16 * N * N}
        kernel_names = {"gridding": "grid_kernel", "fft_pass1": "fft_rows_kernel", "fft_pass2": "fft_cols_kernel"}
    stage_info = {}
    for k, (tot_ms, launches) in stages.items():
        if launches:
            per_launch_ms = tot_ms / launches
            imgs_per_launch = n_images * stage_steps / launches
            gbs = alg[k] * imgs_per_launch / (per_launch_ms / 1000.0) / 1e9
            stage_info[k] = {"ms_per_launch": per_launch_ms, "launches": launches,
                             "images_per_launch": imgs_per_launch, "achieved_gbs": gbs,
                             "share": tot_ms / max(sum(v[0] for v in stages.values()), 1e-12)}
    if "gridding" in stage_info:
        # the fixed per-image count for gridding (stored visibilities read, the whole N x N grid
        # written, the counters per channel) beside the pruned one above
        g = stage_info["gridding"]
        fixed = vis_bytes + 8 * N * N + 4 * N * N / T
        g["fixed_count_bytes_per_image"] = fixed
        g["fixed_count_gbs"] = fixed * g["images_per_launch"] / (g["ms_per_launch"] / 1000.0) / 1e9
        g["fixed_count_frac"] = g["fixed_count_gbs"] / hbm_peak
    dom = max(stage_info, key=lambda k: stage_info[k]["share"])
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            tr = json.load(f)
        per_image = tr.get("bytes_per_image", {}).get(fmt, {})
        if dom in per_image:
            traffic = per_image[dom] * stage_info[dom]["images_per_launch"]
    except Exception:
        traffic = None
    # whole step: compulsory DRAM bytes (stored visibilities in, images out) and the passes'
    # algorithmic bytes (the grid scratch traffic of which stays in L2), over the step time
    step_s = ms / args.steps / 1000.0
    compulsory = n_images * (vis_bytes + 8 * N * N)
    passes = n_images * sum(alg.values())
    step_roof = {"compulsory_bytes_per_step": compulsory, "compulsory_gbs": compulsory / step_s / 1e9,
                 "compulsory_frac": compulsory / step_s / 1e9 / hbm_peak,
                 "all_passes_bytes_per_step": passes, "all_passes_gbs": passes / step_s / 1e9,
                 "note": "lanes run concurrently, so per-launch stage times overlap; these use the step time"}
    roof = {"kernel": kernel_names[dom], "stage": dom, "bound": "hbm", "achieved": stage_info[dom]["achieved_gbs"],
            "peak": hbm_peak,
            "unit": "GB/s", "frac": stage_info[dom]["achieved_gbs"] / hbm_peak,
            "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "traffic": traffic,
            "algorithmic_bytes_per_image": alg[dom],
            "path": "half plane (complex-to-real)" if half else "full plane",
            "uv_extent_pixels": [ext_u, ext_v], "step": step_roof}

    cpu_rate, cpu_times, cpu_threads = cpu_sample_rate(obs, 16, args.cpu_seconds)
    d2h = n_images * N * N * 8
    plain = variants.get("plain_fp32_dropin", {}).get("images_per_s")
    plain_cufft = variants.get("plain_fp32_dropin_cufft", {}).get("images_per_s")
    line = {
        "metric": METRIC, "value": images_per_s, "unit": "images/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 arithmetic" + ("" if fmt == "c64" else f", {fmt} storage"),
        "storage": {"c64": "complex64 (the reference's layout)",
                    "s16": "16-bit block floating point: int16 pol planes, one FP32 scale per 128 baselines",
                    "bf16": "bfloat16 pol planes, one FP32 scale per 128 baselines",
                    "fp16": "binary16 pol planes, one FP32 scale per 128 baselines"}[fmt],
        "vs_plain_fp32_dropin": images_per_s / plain if plain else None,
        "vs_plain_fp32_dropin_cufft": images_per_s / plain_cufft if plain_cufft else None,
        "data": "synthetic (seeded; shapes and distributions of the workload)",
        "config": {"workload": WORKLOAD if T == 10 else WORKLOAD.replace("10 intervals", f"{T} intervals"),
                   "images_per_step": n_images, "n_pixels": N, "baselines": B,
                   "schedule": {"images_per_wave": im.schedule[0] or "auto", "lanes": im.schedule[1],
                                "gridding_images_per_thread": im.gridding_images_per_thread or "auto",
                                "fft_mode": im.fft_mode, "column_radix": im.column_radix,
                                "chosen_by": "bgi_autotune on this block" if tuned else "default"},
                   "l2": "flushed before every timed step (512 MB written outside the step's events)",
                   "storage": fmt,
                   "bytes_per_step": {"stored_visibilities_read": n_images * vis_bytes, "images_written": d2h},
                   "parallelism": (f"one observation of {world} blocks sharded by interval "
                                   "(imager_gb300.shard.plan_shard, whole-observation uv cell), no collective")
                                  if world > 1 else "single GPU"},
        "vis_per_s": world * gridded_vis * args.steps / (ms / 1000.0),
        "e2e": {"value": world * n_images / e2e_s, "unit": "images/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h_real,
                "link": dict(link, bound_images_per_s=world * n_images / max(d2h_real / link["d2h_gbs"] / 1e9,
                                                                             h2d / link["h2d_gbs"] / 1e9),
                             frac=(n_images / e2e_s) / (n_images / max(d2h_real / link["d2h_gbs"] / 1e9,
                                                                       h2d / link["h2d_gbs"] / 1e9))),
                "api": ("bgi_image_host" if fmt == "c64" else "bgi_image_compressed_host") +
                       " with BGI_OUTPUT_REAL (pinned host buffers; XX images are real)",
                "variants": e2e_variants},
        "roofline": roof,
        "stages": stage_info,
        "cpu_baseline": {"value": cpu_rate, "unit": "images/s", "cores": cpu_threads, "kind": "port",
                         "sample": f"16 images (interval 0, channels 0-15) per repetition, "
                                   f"{len(cpu_times)} repetitions: corrections, gridding, FP32 FFT, "
                                   "normalise, shift (oracle/ restatement, OpenMP)"},
        "clocks": clocks.summary(t0, t3),
        "gpu_launches": sum(v[1] for v in stages.values()) * args.steps // stage_steps,
        "variants": variants,
        "serving": serving,
        "batched_uneven": batched,
        "precision_form": precision,
        "parity_sample_rel_l2": errs["rel_l2"],
        "errors_vs_fp64": {**errs, "images": [f"interval {t % T}, channel {c}" for t, c in SAMPLES],
                           "oracle": "FP64 oracle of the original complex64 visibilities"},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--wave", type=int, default=0, help="images per launch wave (0 = auto)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--storage", choices=["s16", "bf16", "fp16", "c64"], default="s16",
                    help="visibility storage of the timed step (s16: 16-bit block floating point)")
    ap.add_argument("--gridding-images-per-thread", type=int, choices=[2, 4, 8], default=None,
                    help="force the gridding's images per thread of the timed step (default: the autotuner's)")
    ap.add_argument("--fft-mode", choices=["simt", "tensor_split16"], default=None,
                    help="force the FFT arithmetic of the timed step (default: the autotuner's choice)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default schedule (auto wave, two lanes) instead of bgi_autotune's")
    ap.add_argument("--no-serving", dest="serving", action="store_false", help="skip the serving measurement")
    ap.add_argument("--no-batched", dest="batched", action="store_false", help="skip the uneven-batch measurement")
    ap.add_argument("--no-precision", dest="precision", action="store_false",
                    help="skip the precision-form measurement (768 channels x 20 intervals at 1024^2)")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="Poisson-phase requests (p99 needs >= 1000; the closed loop runs 3x as many)")
    ap.add_argument("--serve-interarrival-ms", type=float, default=100.0)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-outstanding", type=int, default=3)
    ap.add_argument("--no-variants", dest="variants", action="store_false",
                    help="skip timing the deterministic and full-plane variants")
    ap.add_argument("--intervals", type=int, default=10,
                    help="intervals per block (10 = the measured workload; fewer only for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
