#!/usr/bin/env python3
"""Benchmark: frame-pairs/s for SSIMULACRA2 at 1080p (headline) and Butteraugli at 4K, plus the
batched multi-resolution form and the serving loop.

Workloads (seeded synthetic frames, vship_gb300.synth; no dataset is available offline):
  * ssimu2_1080p : 240 pairs of 1920x1080 YUV420P10 (BT.709, limited range; 8x8 block-DCT
                   distortion, step U[4, 32], chroma x2).
  * butter_4k    : 60 pairs of 3840x2160 YUV420P10, Gaussian blur sigma U[0.5, 2] + noise sigma
                   U[1, 6], intensity 203, Qnorm 2.
  Each is scored from three input forms: RGB48 (16-bit R'G'B' planes: what the reference's own
  front-end converts every frame to before its Uint16 compute calls) -- the headline -- and,
  beside it, float32 R'G'B' planes and the 10-bit 4:2:0 planes themselves (converted on the GPU).
  * batched_multi: 64 sources at 360p/720p/1080p/2160p (26/19/13/6) x 8 block-DCT candidates,
                   both metrics, one call per step (Vship_MultiComputeDeviceAsync).
  * serving      : Poisson request arrivals at 50..2000 req/s against the serving runtime.

A step scores every pair of the workload once.
  value : inputs resident in HBM, batched device entry points (Vship_*ComputeDeviceAsync) in
          launches of --chunk SSIMU2 / --butter-chunk Butteraugli pairs (120 / 15), CUDA
          events on the launching stream around the K timed steps. Inputs (6-12 GB per workload)
          are far larger than L2, so no flush is needed between steps.
  e2e   : the reference-facing C ABI (Vship_ComputeSSIMU2Uint16 / Vship_ComputeButteraugliUint16v3)
          from pinned host buffers, one handler per host thread; every call copies its planes
          host->device and reads its score back.

  reference_cuda: the reference's own CUDA build (oracle/_ref/libvship_ref.so, built from
          pkp24/Vship's sources by oracle/ref_build.py) through its stock C ABI calls on the same
          pinned RGB48 host planes, 3 and 8 handler threads; its frame-pairs/s, this library's e2e
          and device rates over it, and the score / norm differences on every pair.
  error_vs_fp64: each reported form's error against the FP64 oracle on the first pairs.

--impl reference runs the reference's math on the host cores instead (the reference has no CPU
implementation, so this is the FP32 CPU restatement in oracle/, threaded over all host cores),
one bounded sample per step.

Multi-GPU: every rank runs the full workload on its own GPU (frame pairs are independent,
replicas only); value = pairs over all ranks / max over ranks of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W1080, H1080 = 1920, 1080
W4K, H4K = 3840, 2160


def total_scale_pixels(w: int, h: int) -> int:
    t = 0
    for _ in range(6):
        t += w * h
        w, h = (w - 1) // 2 + 1, (h - 1) // 2 + 1
    return t


# Algorithmic bytes of the dominant kernels, per frame pair (FP32 planes):
#   ssimu2_stats reads both XYB pyramids once: 2 images x 3 channels x 4 B x T pixels.
#   butter_diff reads the 20 band planes (LF vals, MF, HF, UHF of both images) once and writes
#   2 planes (AC sum, DC sum) at each of the two scales.
def ssimu2_stats_bytes(w, h):
    return 2 * 3 * 4 * total_scale_pixels(w, h)


def ssimu2_stats_flops(w, h):
    """Algorithmic FP32 work of the stats kernel per pair: per channel and pyramid pixel, the
    17-tap horizontal and vertical passes over four moments (136 FMA = 272 FLOP); the maps and
    pooling (a few tens of FLOP) and the vertical halo of the horizontal pass are not counted."""
    return 272 * 3 * total_scale_pixels(w, h)


def fp32_peak_tflops(clock_mhz):
    """Dense FP32 FMA peak at the sampled SM clock: 128 FMA lanes per SM per cycle, 2 FLOP each."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return sms * 128 * 2 * clock_mhz * 1e6 / 1e12


def butter_diff_bytes(w, h):
    n = w * h
    nh = ((w - 1) // 2 + 1) * ((h - 1) // 2 + 1)
    return 22 * 4 * (n + nh)


def kernel_bytes_per_pair(kind, w, h, in_bytes):
    """Algorithmic DRAM bytes each kernel moves per frame pair with FP32 planes: every plane it
    must read or write, once (halos and re-reads not counted); in_bytes = input bytes per pixel
    of one frame (6 for RGB48)."""
    if kind == "ssimu2":
        t = total_scale_pixels(w, h)
        return {"ssimu2_pyramid": 2 * in_bytes * w * h + 2 * 12 * t, "ssimu2_stats": 2 * 12 * t}
    n = w * h
    nh = ((w - 1) // 2 + 1) * ((h - 1) // 2 + 1)
    ns = n + nh
    return {"butter_decode": 2 * in_bytes * n + 2 * 12 * ns,  # linear RGB at both scales
            "butter_opsin": 2 * 24 * ns,      # linear RGB in, XYB out
            "butter_hblur_lf": 2 * 24 * ns,   # 3 planes in, 3 out
            "butter_lf_v": 2 * 48 * ns,       # 3 blurred + 3 XYB in, D and LF vals out
            "butter_mf": 2 * 32 * ns,         # 3 D in, 2 HF_pre + 3 MF out (both passes in one)
            "butter_hf": 2 * 28 * ns,         # 2 HF_pre in, HF, UHF and the mask precompute out
            "butter_diff": 88 * ns,           # 20 band planes in, 2 pair planes out
            "butter_mask_blur": 20 * ns,      # 2 mask precomputes + AC in, blurred mask + AC out
            "butter_diffmap": 16 * ns + 4 * nh}


# Whole-pipeline algorithmic bytes per pair (b_in = 3 B/px for 16-bit 4:2:0 input; FP32 planes).
def ssimu2_pair_bytes(w, h):
    return 2 * 3 * w * h + 2 * 12 * total_scale_pixels(w, h) * 2


def butter_pair_bytes(w, h):
    n = w * h
    nh = ((w - 1) // 2 + 1) * ((h - 1) // 2 + 1)
    return 2 * 3 * n + 272 * (n + nh) + 8 * n + 4 * nh


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes per frame pair (read + write, both scales for Butteraugli) measured by ncu
# (profiles/dram_traffic_bench_config.md): ssimu2_stats reads each pyramid once (66.38 MB per
# 1080p pair, equal to its algorithmic bytes); butter_diff reads its band planes about 1.18x
# (tile halos, epilogue re-reads) once a batch's planes exceed L2, as every batch of 4 or more
# 3840x2160 pairs does.
NCU_DRAM_BYTES_PER_PAIR = {
    "ssimu2_stats": (7962.84e6 + 7.55e6) / 120,
    "butter_diff": (2488.55e6 + 250.61e6 + 9955.46e6 + 1017.72e6) / 15,
}


def ncu_traffic(kernel: str):
    """DRAM bytes per pair for `kernel` from the committed ncu measurement, if one exists."""
    return NCU_DRAM_BYTES_PER_PAIR.get(kernel)


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for ln in f:
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# distributed helpers (replicas only)

def dist_setup(args):
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    from vship_gb300.dist import max_over_ranks as _m
    return _m(x, ws)


# ------------------------------------------------------------------------------------------
# workloads

def parse_size(txt: str):
    w, h = txt.lower().split("x")
    return int(w), int(h)


def make_inputs(kind: str, npairs: int, device, size):
    """Device-resident float32 R'G'B' planes: (npairs, 3, H, W) for reference and distorted."""
    import torch
    from vship_gb300 import synth
    w, h = size
    dist = "dct" if kind == "ssimu2" else "blur_noise"
    ref = torch.empty((npairs, 3, h, w), dtype=torch.float32, device=device)
    dst = torch.empty_like(ref)
    cw, ch = (w + 1) // 2, (h + 1) // 2
    # the same frames as 10-bit 4:2:0 planes (uint16 containers): [pair][image] -> (Y, Cb, Cr)
    yuv = torch.empty((npairs, 2, h * w + 2 * ch * cw), dtype=torch.int16, device=device)
    for t in range(npairs):
        r, d = synth.yuv420p10_frames(h, w, t, seed=7 if kind == "ssimu2" else 11, distortion=dist, device=device)
        ref[t] = synth.yuv420p10_to_rgb(r)
        dst[t] = synth.yuv420p10_to_rgb(d)
        for m, f in enumerate((r, d)):
            yuv[t, m] = torch.cat([p.reshape(-1) for p in f]).to(torch.int16)
    return ref, dst, yuv


def frames_table(v, ref, dst, start, count):
    frames = []
    for t in range(start, start + count):
        for x in (ref, dst):
            frames.append(([x[t, c].data_ptr() for c in range(3)], x.stride(2) * x.element_size()))
    return v.device_frames_table(frames)


def yuv_table(v, yuv, start, count):
    yuvt, (w, h) = yuv
    cw, ch = (w + 1) // 2, (h + 1) // 2
    frames = []
    for t in range(start, start + count):
        for m in range(2):
            base = yuvt[t, m].data_ptr()
            frames.append(([base, base + 2 * h * w, base + 2 * (h * w + ch * cw)], 2 * w, 2 * cw))
    return v.device_frames_table(frames)


def run_device(v, kind, ref, dst, steps, warmup, ws, chunk, yuv=None, half_bands=False, fp16_deltas=False):
    """Batched device-resident throughput; returns (seconds for `steps` steps, profile dict, launches,
    results). half_bands: Butteraugli with its UHF bands stored as FP16."""
    import torch
    if yuv is not None:
        yuvt, (w, h) = yuv
        npairs = yuvt.shape[0]
    else:
        npairs, _, h, w = ref.shape
    if kind == "ssimu2":
        eng = v.SSIMU2Batch(w, h, chunk, fp16_deltas=fp16_deltas)
        out = torch.zeros(npairs, dtype=torch.float64, device="cuda")
    else:
        eng = v.ButteraugliBatch(w, h, chunk, 2, 203.0, half_bands=half_bands)
        out = torch.zeros(npairs * 3, dtype=torch.float64, device="cuda")
    tables = []
    for s in range(0, npairs, chunk):
        c = min(chunk, npairs - s)
        tables.append((s, c, frames_table(v, ref, dst, s, c) if yuv is None else yuv_table(v, yuv, s, c)))
    stream = torch.cuda.current_stream()
    itype = v.IN_YUV420P10 if yuv is not None else (v.IN_UINT16 if ref.dtype == torch.int16 else v.IN_FLOAT)

    def step():
        for s, c, tb in tables:
            if kind == "ssimu2":
                eng.compute_async(tb.data_ptr(), c, itype, out[s:].data_ptr(), stream.cuda_stream)
            else:
                eng.compute_async(tb.data_ptr(), c, itype, out[3 * s:].data_ptr(), 0, stream.cuda_stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    sec = e0.elapsed_time(e1) / 1e3
    # per-kernel breakdown: the same steps again with every launch bracketed by CUDA events (kept
    # out of the timed region above: the events cost about 1 % there)
    v.profile_report()  # clear
    v.profile_enable(True)
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    v.profile_enable(False)
    prof = v.profile_report()
    launches = sum(n for n, _ in prof.values())
    result = out.cpu()
    eng.free()
    return sec, prof, launches, result


E2E_TRIALS = 5


def run_e2e(v, kind, ref, dst, steps, warmup, nthreads, yuv=None, half_bands=False):
    """Through the C ABI from pinned host memory, one handler per thread: the reference-facing
    float-RGB calls, or (yuv=...) the 4:2:0 extension calls."""
    import ctypes
    import numpy as np
    import torch
    L = v.lib()
    plane_ptrs = []
    if yuv is None:
        npairs, _, h, w = ref.shape
        href = ref.cpu().pin_memory()
        hdst = dst.cpu().pin_memory()
        for t in range(npairs):
            a = (ctypes.c_void_p * 3)(*[href[t, c].data_ptr() for c in range(3)])
            b = (ctypes.c_void_p * 3)(*[hdst[t, c].data_ptr() for c in range(3)])
            plane_ptrs.append((a, b))
    else:
        yuvt, (w, h) = yuv
        npairs = yuvt.shape[0]
        cw, ch = (w + 1) // 2, (h + 1) // 2
        hy = yuvt.cpu().pin_memory()
        ystr = (ctypes.c_int64 * 3)(2 * w, 2 * cw, 2 * cw)
        for t in range(npairs):
            pp = []
            for m in range(2):
                base = hy[t, m].data_ptr()
                pp.append((ctypes.c_void_p * 3)(base, base + 2 * h * w, base + 2 * (h * w + ch * cw)))
            plane_ptrs.append(tuple(pp))
    u16 = yuv is None and ref.dtype == torch.int16
    stride = w * (2 if u16 else 4)
    handlers = []
    for _ in range(nthreads):
        hd = v.Handler()
        if kind == "ssimu2":
            rc = L.Vship_SSIMU2Init(ctypes.byref(hd), w, h)
        else:
            rc = L.Vship_ButteraugliInitEx(ctypes.byref(hd), w, h, 2, ctypes.c_float(203.0),
                                           v.BUTTER_HALF_BANDS if half_bands else 0)
        if rc:
            raise v.VshipError(rc, "init")
        handlers.append(hd)
    scores = [None] * npairs
    errors = []

    def worker(k):
        hd = handlers[k]
        sc = ctypes.c_double()
        norms = (ctypes.c_double * 3)()
        for i in range(k, npairs, nthreads):
            a, b = plane_ptrs[i]
            if yuv is not None and kind == "ssimu2":
                rc = L.Vship_ComputeSSIMU2Yuv420p10(hd, ctypes.byref(sc), ctypes.cast(a, v._PP), ystr,
                                                    ctypes.cast(b, v._PP), ystr)
                scores[i] = sc.value
            elif yuv is not None:
                rc = L.Vship_ComputeButteraugliYuv420p10(hd, norms, None, 0, ctypes.cast(a, v._PP), ystr,
                                                         ctypes.cast(b, v._PP), ystr)
                scores[i] = norms[0]
            elif kind == "ssimu2" and u16:
                rc = L.Vship_ComputeSSIMU2Uint16(hd, ctypes.byref(sc), ctypes.cast(a, v._PP), ctypes.cast(b, v._PP),
                                                 stride)
                scores[i] = sc.value
            elif kind == "ssimu2":
                rc = L.Vship_ComputeSSIMU2Float(hd, ctypes.byref(sc), ctypes.cast(a, v._PP), ctypes.cast(b, v._PP),
                                                stride)
                scores[i] = sc.value
            elif u16:
                rc = L.Vship_ComputeButteraugliUint16v3(hd, norms, None, 0, ctypes.cast(a, v._PP),
                                                        ctypes.cast(b, v._PP), stride, stride)
                scores[i] = norms[0]
            else:
                rc = L.Vship_ComputeButteraugliFloatv3(hd, norms, None, 0, ctypes.cast(a, v._PP),
                                                       ctypes.cast(b, v._PP), stride, stride)
                scores[i] = norms[0]
            if rc:
                errors.append(rc)

    def step():
        th = [threading.Thread(target=worker, args=(k,)) for k in range(nthreads)]
        [t.start() for t in th]
        [t.join() for t in th]

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    # the host link and host memory are shared with other work on the machine: time E2E_TRIALS
    # trials of `steps` steps and report the median (each trial's rate is kept beside it)
    trials = []
    for _ in range(E2E_TRIALS):
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        torch.cuda.synchronize()
        trials.append(time.perf_counter() - t0)
    sec = sorted(trials)[len(trials) // 2]
    for hd in handlers:
        if kind == "ssimu2":
            L.Vship_SSIMU2Free(hd)
        else:
            L.Vship_ButteraugliFree(hd)
    if errors:
        raise v.VshipError(errors[0], "e2e compute")
    h2d = npairs * 2 * 3 * w * h * (2 if u16 else 4) if yuv is None else npairs * 2 * 2 * (h * w + 2 * ((w + 1) // 2) * ((h + 1) // 2))
    d2h = npairs * (8 if kind == "ssimu2" else 24)
    return sec, h2d, d2h, np.array(scores), [npairs * steps / t for t in trials]


REF_THREADS = (3, 8)


def run_reference_cuda(kind, ref, dst, steps, warmup):
    """The reference's own CUDA build (oracle/_ref/libvship_ref.so, pkp24/Vship src/VshipLib.cpp
    compiled for sm_103a) through its stock C ABI calls -- Vship_ComputeSSIMU2Uint16 /
    Vship_ComputeButteraugliUint16 -- from the same pinned RGB48 host planes as this library's e2e,
    one handler per host thread, at the 3 threads its documentation recommends and at 8 (the
    e2e setting of this library); the better rate is the baseline. Every call copies its planes
    host->device, computes and returns its result, as the reference always does. Returns None when
    the library is not built on this machine.

    The reference's ABI truncates Butteraugli norms to ints, so after the timed trials one untimed
    pass scores every pair through VshipRef_ComputeButteraugli (the same computing implementation,
    float norms) for the parity figures."""
    import ctypes
    import numpy as np
    import torch
    from oracle import reference_cuda as R
    if not R.available():
        return None
    L = R.lib()
    npairs, _, h, w = ref.shape
    if kind != "ssimu2" and not R.butteraugli_size_safe(w, h):
        return None
    href = ref.cpu().pin_memory()
    hdst = dst.cpu().pin_memory()
    ptrs = []
    for t in range(npairs):
        a = (ctypes.c_void_p * 3)(*[href[t, c].data_ptr() for c in range(3)])
        b = (ctypes.c_void_p * 3)(*[hdst[t, c].data_ptr() for c in range(3)])
        ptrs.append((a, b))
    stride = w * 2
    out = {"calls": "Vship_ComputeSSIMU2Uint16" if kind == "ssimu2" else "Vship_ComputeButteraugliUint16",
           "input": "RGB48 planes, pinned host memory (the same buffers as e2e)", "by_threads": {}}
    scores = [None] * npairs
    best = 0.0
    for nthreads in REF_THREADS:
        handlers = []
        for _ in range(nthreads):
            hd = R._Handler()
            rc = (L.Vship_SSIMU2Init(ctypes.byref(hd), w, h) if kind == "ssimu2"
                  else L.Vship_ButteraugliInitv2(ctypes.byref(hd), w, h, 2, ctypes.c_float(203.0)))
            R._check(rc, "reference init")
            handlers.append(hd)
        errors = []

        def worker(k):
            hd = handlers[k]
            sc = ctypes.c_double()
            bs = R._ButterScore()
            for i in range(k, npairs, nthreads):
                a, b = ptrs[i]
                if kind == "ssimu2":
                    rc = L.Vship_ComputeSSIMU2Uint16(hd, ctypes.byref(sc), ctypes.cast(a, R._PP),
                                                     ctypes.cast(b, R._PP), stride)
                    scores[i] = sc.value
                else:
                    rc = L.Vship_ComputeButteraugliUint16(hd, ctypes.byref(bs), None, 0, ctypes.cast(a, R._PP),
                                                          ctypes.cast(b, R._PP), stride)
                if rc:
                    errors.append(rc)

        def step():
            th = [threading.Thread(target=worker, args=(k,)) for k in range(nthreads)]
            [t.start() for t in th]
            [t.join() for t in th]

        for _ in range(warmup):
            step()
        trials = []
        for _ in range(E2E_TRIALS):
            t0 = time.perf_counter()
            for _ in range(steps):
                step()
            trials.append(time.perf_counter() - t0)
        if errors:
            R._check(errors[0], "reference compute")
        if kind != "ssimu2":
            norms = (ctypes.c_float * 3)()
            hd = handlers[0]
            for i in range(npairs):
                a, b = ptrs[i]
                R._check(L.VshipRef_ComputeButteraugli(hd, norms, 1, None, 0, ctypes.cast(a, R._PP),
                                                       ctypes.cast(b, R._PP), stride, stride), "reference norms")
                scores[i] = (float(norms[0]), float(norms[1]), float(norms[2]))
        for hd in handlers:
            (L.Vship_SSIMU2Free if kind == "ssimu2" else L.Vship_ButteraugliFree)(hd)
        sec = sorted(trials)[len(trials) // 2]
        v = npairs * steps / sec
        out["by_threads"][str(nthreads)] = {"value": v, "trials": [round(npairs * steps / t, 1) for t in trials]}
        best = max(best, v)
    torch.cuda.synchronize()
    out.update({"value": best, "unit": "frame-pairs/s", "steps": steps, "warmup": warmup, "of_trials": "median",
                "h2d_bytes_per_step": npairs * 2 * 3 * w * h * 2,
                "d2h_bytes_per_step": npairs * (8 if kind == "ssimu2" else 12)})
    return out, np.array(scores, dtype=np.float64)


def error_vs_fp64(kind, ref, dst, forms, npairs, nthreads):
    """For each form (name -> per-pair results), the max over the first npairs of |got - FP64
    oracle| (SSIMU2, absolute) or of the relative error of each of {Qnorm, 3-norm, inf-norm}
    (Butteraugli). ref/dst: (pairs, 3, H, W) float32, or uint16 bits held in int16."""
    import numpy as np
    import oracle
    u16 = str(ref.dtype) == "torch.int16"
    conv = (lambda x: np.ascontiguousarray(x.cpu().numpy().view(np.uint16))) if u16 else \
        (lambda x: np.ascontiguousarray(x.cpu().numpy()))
    worst = {k: None for k in forms}
    for t in range(npairs):
        a = [conv(ref[t, c]) for c in range(3)]
        b = [conv(dst[t, c]) for c in range(3)]
        if kind == "ssimu2":
            want = oracle.ssimu2(a, b, precision=64, nthreads=nthreads)
        else:
            want = oracle.butteraugli(a, b, precision=64, nthreads=nthreads)
        for k, got in forms.items():
            e = abs(float(got[t]) - want) if kind == "ssimu2" else rel_err(got[t], want)
            w = worst[k]
            worst[k] = e if w is None else (max(w, e) if kind == "ssimu2" else [max(x, y) for x, y in zip(w, e)])
    return worst


def cpu_baseline(kind, ref, dst, sample_pairs, nthreads, fp64_pairs=0):
    """The reference's math (FP32 restatement in oracle/) on the host cores for a bounded sample.
    With fp64_pairs > 0 the FP64 instantiation also scores the first pairs (untimed), the
    reference against which the GPU results' error is stated."""
    import numpy as np
    import oracle
    t_total = 0.0
    exact = []
    for t in range(max(sample_pairs, fp64_pairs)):
        a = [np.ascontiguousarray(ref[t, c].cpu().numpy()) for c in range(3)]
        b = [np.ascontiguousarray(dst[t, c].cpu().numpy()) for c in range(3)]
        if t < sample_pairs:
            t0 = time.perf_counter()
            if kind == "ssimu2":
                oracle.ssimu2(a, b, precision=32, nthreads=nthreads)
            else:
                oracle.butteraugli(a, b, precision=32, nthreads=nthreads)
            t_total += time.perf_counter() - t0
        if t < fp64_pairs:
            if kind == "ssimu2":
                exact.append(oracle.ssimu2(a, b, precision=64, nthreads=nthreads))
            else:
                exact.append(oracle.butteraugli(a, b, precision=64, nthreads=nthreads))
    return sample_pairs / t_total, t_total, exact


def host_link_gbs():
    """Pinned host -> device copy bandwidth (256 MiB, best of 3, CUDA events): the ceiling of
    every e2e number, whose inputs cross this link each step."""
    import torch
    n = 256 << 20
    src = torch.empty(n, dtype=torch.uint8).pin_memory()
    dst = torch.empty(n, dtype=torch.uint8, device="cuda")
    best = 0.0
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, n / (e0.elapsed_time(e1) / 1e3) / 1e9)
    del src, dst
    return best


def link_frac(link, e2e, npairs):
    """An e2e run's host->device bytes per second as a fraction of the measured link bandwidth."""
    return round(e2e["h2d_bytes_per_step"] / npairs * e2e["value"] / 1e9 / link, 3)


def rel_err(got, want):
    return [abs(g - w) / max(abs(w), 1e-12) for g, w in zip(got, want)]


def to_rgb48(x):
    """float32 R'G'B' in [0, 1] -> 16-bit code values (uint16 bits held in int16), the RGB48
    planes the reference's own front-end hands to its compute calls."""
    import torch
    return torch.round(x.clamp(0.0, 1.0) * 65535.0).to(torch.int32).to(torch.int16)


def bench_workload(v, kind, args, ws, rank):
    """The headline form is the reference front-end's own input: 16-bit R'G'B' planes (FFVship
    converts every frame to RGB48 and calls the Uint16 entry points). Float32 R'G'B' and
    10-bit 4:2:0 (converted on the GPU) are measured beside it."""
    import numpy as np
    import torch
    npairs = args.pairs if kind == "ssimu2" else args.butter_pairs
    chunk = args.chunk if kind == "ssimu2" else args.butter_chunk
    size = parse_size(args.ssimu2_size if kind == "ssimu2" else args.butter_size)
    ref, dst, yuv = make_inputs(kind, npairs, "cuda", size)
    torch.cuda.synchronize()
    w, h = size
    # float32 R'G'B' planes
    fsec, _, _, fres = run_device(v, kind, ref, dst, args.steps, args.warmup, ws, chunk)
    fsec = max_over_ranks(fsec, ws)
    fe2e_sec, fh2d, d2h, _, ftrials = run_e2e(v, kind, ref, dst, args.e2e_steps, args.e2e_warmup, args.e2e_threads)
    fe2e_sec = max_over_ranks(fe2e_sec, ws)
    # the CPU leg runs after every GPU measurement (an all-core run before them measurably slowed
    # the host side of the e2e calls); keep the frames it needs on the host
    ns = nx = 0
    if rank == 0 and args.cpu_sample > 0:
        ns = args.cpu_sample if kind == "ssimu2" else max(1, args.cpu_sample // 4)
        nx = args.error_pairs if kind == "ssimu2" else args.butter_error_pairs
    ref_cpu, dst_cpu = ref[:ns].cpu(), dst[:ns].cpu()
    # 16-bit R'G'B' (headline)
    ref16, dst16 = to_rgb48(ref), to_rgb48(dst)
    ref16_cpu, dst16_cpu = ref16[:nx].cpu(), dst16[:nx].cpu()
    del ref, dst
    torch.cuda.empty_cache()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    sec, prof, launches, dev_scores = run_device(v, kind, ref16, dst16, args.steps, args.warmup, ws, chunk)
    clocks = sampler.stop()
    sec = max_over_ranks(sec, ws)
    value = npairs * ws * args.steps / sec
    e2e_sec, h2d, d2h, host_scores, trials = run_e2e(v, kind, ref16, dst16, args.e2e_steps, args.e2e_warmup, args.e2e_threads)
    e2e_sec = max_over_ranks(e2e_sec, ws)
    e2e_value = npairs * ws * args.e2e_steps / e2e_sec
    refc = None
    if rank == 0 and not args.skip_reference_cuda:
        # the reference's own CUDA build on the same pinned RGB48 frames, through its own C ABI
        refc = run_reference_cuda(kind, ref16, dst16, args.ref_steps, args.ref_warmup)
    worst_frames = None
    if refc is not None and kind == "ssimu2":
        # host copies of the pairs where the two builds differ most, for the FP64 check below
        d_ = np.abs(dev_scores.numpy() - refc[1])
        sub = torch.tensor([int(i) for i in np.argsort(-d_)[:args.ref_worst_pairs]], dtype=torch.long)
        worst_frames = (ref16[sub.cuda()].cpu(), dst16[sub.cuda()].cpu())
    barrier(ws)
    kname = "ssimu2_stats" if kind == "ssimu2" else "butter_diff"
    per_pair = ssimu2_stats_bytes(w, h) if kind == "ssimu2" else butter_diff_bytes(w, h)
    peak, peak_kind = measured_peaks()
    # every kernel's algorithmic bytes over its summed CUDA-event time, against the HBM peak
    kroof = {}
    for k, kb in kernel_bytes_per_pair(kind, w, h, 6).items():
        if k in prof and prof[k][1] > 0:
            gbs = kb * npairs * args.steps / (prof[k][1] / 1e3) / 1e9
            kroof[k] = {"gbs": round(gbs, 1), "frac": round(gbs / peak, 3)}
    n_launch, tot_ms = prof.get(kname, (0, 0.0))
    # algorithmic bytes moved by this kernel over the timed region / its summed launch time
    # (for Butteraugli the per-pair figure covers both scales, i.e. two launches per batch)
    total_alg = per_pair * npairs * args.steps
    alg = total_alg / max(n_launch, 1)
    avg_s = (tot_ms / 1e3) / max(n_launch, 1)
    achieved = total_alg / (tot_ms / 1e3) / 1e9 if tot_ms > 0 else 0.0
    pairs_per_launch = npairs * args.steps / max(n_launch, 1)
    traffic = ncu_traffic(kname)
    total_kernel_ms = sum(t for _, t in prof.values())
    fp32_roof = None
    if kind == "ssimu2" and tot_ms > 0:
        # the stats kernel is bound by the FP32 pipe, not by HBM: its arithmetic against the FP32 peak
        mhz = clocks.get("sm_mhz") or 2070.0
        tf = ssimu2_stats_flops(w, h) * npairs * args.steps / (tot_ms / 1e3) / 1e12
        pk = fp32_peak_tflops(mhz)
        fp32_roof = {"kernel": kname, "achieved": tf, "peak": pk, "unit": "TFLOP/s", "frac": tf / pk,
                     "flops_per_pair": ssimu2_stats_flops(w, h),
                     "peak_source": f"128 FP32 FMA lanes x SMs x {mhz:.0f} MHz (sampled clock)"}
    half = None
    dres = None
    if kind == "ssimu2" and not args.skip_half_bands:
        # the distorted pyramids stored as FP16 deltas from the references' (Vship_SSIMU2Fp16Deltas)
        dsec, dprof, _, dres = run_device(v, kind, ref16, dst16, args.steps, args.warmup, ws, chunk, fp16_deltas=True)
        dsec = max_over_ranks(dsec, ws)
        L = v.lib()
        res_fp16 = {"value": npairs * ws * args.steps / dsec, "unit": "frame-pairs/s",
                    "device_bytes_per_pair": int(L.Vship_SSIMU2DeviceBytesEx(w, h, 1, v.SSIMU2_FP16_DELTAS)),
                    "device_bytes_per_pair_fp32": int(L.Vship_SSIMU2DeviceBytes(w, h, 1)),
                    "kernel_ms": {k: round(t, 3) for k, (n, t) in sorted(dprof.items(), key=lambda x: -x[1][1])},
                    "note": "distorted XYB pyramid as FP16 deltas from the reference's, all arithmetic FP32; "
                            "error in error_vs_fp64"}
    hres = None
    if kind != "ssimu2" and not args.skip_half_bands:
        hsec, hprof, _, hres = run_device(v, kind, ref16, dst16, args.steps, args.warmup, ws, chunk, half_bands=True)
        hsec = max_over_ranks(hsec, ws)
        he2e_sec, _, _, _, htrials = run_e2e(v, kind, ref16, dst16, args.e2e_steps, args.e2e_warmup, args.e2e_threads, half_bands=True)
        he2e_sec = max_over_ranks(he2e_sec, ws)
        L = v.lib()
        half = {"value": npairs * ws * args.steps / hsec,
                "e2e": {"value": npairs * ws * args.e2e_steps / he2e_sec, "unit": "frame-pairs/s",
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "trials": [round(x, 1) for x in htrials],
                        "call": "Vship_ComputeButteraugliUint16v3 (Vship_ButteraugliInitEx, Vship_ButterHalfBands)"},
                "device_bytes_per_pair": int(L.Vship_ButteraugliDeviceBytesEx(w, h, 1, v.BUTTER_HALF_BANDS)),
                "device_bytes_per_pair_fp32": int(L.Vship_ButteraugliDeviceBytes(w, h, 1)),
                "kernel_ms": {k: round(t, 3) for k, (n, t) in sorted(hprof.items(), key=lambda x: -x[1][1])},
                "note": "UHF bands stored as FP16, all arithmetic FP32; error in error_vs_fp64"}
    del ref16, dst16
    torch.cuda.empty_cache()
    # 10-bit 4:2:0 planes converted on the GPU (a quarter of the bytes of float RGB)
    ysec, _, _, _ = run_device(v, kind, None, None, args.steps, args.warmup, ws, chunk, yuv=(yuv, size))
    ysec = max_over_ranks(ysec, ws)
    ye2e_sec, yh2d, _, _, ytrials = run_e2e(v, kind, None, None, args.e2e_steps, args.e2e_warmup, args.e2e_threads, yuv=(yuv, size))
    ye2e_sec = max_over_ranks(ye2e_sec, ws)
    res = {
        "value": value, "unit": "frame-pairs/s", "ms_per_step": sec / args.steps * 1e3,
        "input": "RGB48 (16-bit R'G'B' planes)",
        "float32_rgb": {"value": npairs * ws * args.steps / fsec,
                        "e2e": {"value": npairs * ws * args.e2e_steps / fe2e_sec, "unit": "frame-pairs/s",
                                "h2d_bytes_per_step": fh2d, "d2h_bytes_per_step": d2h,
                                "trials": [round(x, 1) for x in ftrials]}},
        "yuv420p10": {"value": npairs * ws * args.steps / ysec,
                      "e2e": {"value": npairs * ws * args.e2e_steps / ye2e_sec, "unit": "frame-pairs/s",
                              "h2d_bytes_per_step": yh2d, "d2h_bytes_per_step": d2h,
                              "trials": [round(x, 1) for x in ytrials]}},
        "pairs_per_step": npairs,
        "launch_chunk_pairs": chunk,
        "e2e": {"value": e2e_value, "unit": "frame-pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "threads": args.e2e_threads, "steps": args.e2e_steps, "warmup": args.e2e_warmup,
                "trials": [round(x, 1) for x in trials], "of_trials": "median",
                "call": "Vship_ComputeSSIMU2Uint16" if kind == "ssimu2" else "Vship_ComputeButteraugliUint16v3"},
        "fp32_roofline": fp32_roof,
        "kernel_roofline": kroof,
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic * pairs_per_launch if traffic is not None else None,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_s * 1e3},
        "pipeline_bytes_per_pair": ssimu2_pair_bytes(w, h) if kind == "ssimu2" else butter_pair_bytes(w, h),
        "kernel_share": {k: {"launches": n, "ms": round(t, 3), "share": round(t / total_kernel_ms, 4)}
                         for k, (n, t) in sorted(prof.items(), key=lambda x: -x[1][1])} if total_kernel_ms > 0 else {},
        "gpu_launches": launches,
        "clocks": clocks,
        "score_check": {"device_vs_e2e_max_abs": float(abs(
            (dev_scores.numpy() if kind == "ssimu2" else dev_scores.numpy()[0::3]) - host_scores).max()),
                        **({"note": "SSIMU2 launches of 16 or more pairs tile the stats kernel's pooled sums "
                                    "in taller segments than single-pair calls: the two agree to FP32 rounding "
                                    "of those sums, not bit for bit"} if kind == "ssimu2" else {})},
    }
    if half:
        res["fp16_bands"] = half
    if dres is not None:
        res["fp16_deltas"] = res_fp16
    if refc is not None:
        rinfo, rscores = refc
        mine = dev_scores.numpy() if kind == "ssimu2" else dev_scores.numpy().reshape(-1, 3)
        if kind == "ssimu2":
            diff = np.abs(mine - rscores)
            rinfo["score_diff_max_abs"] = float(diff.max())
            rinfo["score_diff_p99_abs"] = float(np.percentile(diff, 99))
            rinfo["pairs_over_1e-3"] = int((diff > 1e-3).sum())
            rinfo["tolerance"] = "1e-3 absolute"
            if rank == 0 and args.cpu_sample > 0:
                # the pairs where the two builds differ most, against the FP64 oracle: which of the
                # two is off (the reference pools its per-block sums in FP32 on the host)
                worst = [int(i) for i in np.argsort(-diff)[:args.ref_worst_pairs]]
                if worst:
                    wr, wd = worst_frames
                    e = error_vs_fp64(kind, wr, wd, {"ours": mine[worst], "reference": rscores[worst]}, len(worst),
                                      os.cpu_count() or 1)
                    rinfo["largest_differences_vs_fp64"] = {
                        "pairs": worst, "diff": [float(diff[i]) for i in worst],
                        "ours_max_abs_err": e["ours"], "reference_max_abs_err": e["reference"]}
        else:
            rinfo["norm_diff_max_rel"] = [float(x) for x in (np.abs(mine - rscores) / np.abs(rscores)).max(axis=0)]
            rinfo["tolerance"] = "1e-4 relative"
        rinfo["pairs_compared"] = int(len(rscores))
        rinfo["e2e_ratio"] = e2e_value / rinfo["value"]
        rinfo["device_ratio"] = value / rinfo["value"]
        rinfo["target"] = ">= 2x the reference CUDA build's frame-pairs/s"
        res["reference_cuda"] = rinfo
    if nx > 0:
        nt = os.cpu_count() or 1
        err = {"pairs": nx, "input": "RGB48 planes (the headline input)", "oracle": "FP64 oracle (oracle/)"}
        if kind == "ssimu2":
            forms = {"score_max_abs": dev_scores.numpy()}
            if dres is not None:
                forms["fp16_deltas_score_max_abs"] = dres.numpy()
        else:
            forms = {"fp32_planes_max_rel": dev_scores.numpy().reshape(-1, 3)}
            if hres is not None:
                forms["fp16_bands_max_rel"] = hres.numpy().reshape(-1, 3)
            err["norms"] = "Qnorm (2), 3-norm, inf-norm"
        if refc is not None:
            forms["reference_cuda_" + ("score_max_abs" if kind == "ssimu2" else "max_rel")] = refc[1]
        err.update(error_vs_fp64(kind, ref16_cpu, dst16_cpu, forms, nx, nt))
        res["error_vs_fp64"] = err
    if ns > 0:
        cv, csec, _ = cpu_baseline(kind, ref_cpu, dst_cpu, ns, os.cpu_count() or 1)
        res["cpu_baseline"] = {"value": cv, "unit": "frame-pairs/s", "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"{ns} pairs of the same workload ({csec:.1f} s)"}
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------------------------------------------
# batched multi-resolution workload: 64 sources x 8 candidates = 512 pairs, both metrics

MULTI_RES = [(640, 360), (1280, 720), (1920, 1080), (3840, 2160)]
MULTI_SOURCES = [26, 19, 13, 6]  # 4:3:2:1 over 64 sources (25.6 : 19.2 : 12.8 : 6.4, rounded)
MULTI_DCT_STEPS = [4, 6, 8, 12, 16, 20, 26, 32]


def ssimu2_stats_bytes_fp16(w, h):
    """Fused stats kernel over FP32 source + FP16-delta candidate pyramids: 3 x (4 + 2) B/sample."""
    return 3 * (4 + 2) * total_scale_pixels(w, h)


def make_multi_inputs(device, sources):
    """One flat int16 buffer holding every frame as Y, Cb, Cr planes back to back; returns the
    buffer, per-frame (offset, w, h), source resolutions, candidate -> source map, frame index of
    each source and candidate."""
    import torch
    from vship_gb300 import synth
    metas, chunks = [], []
    src_res, cand_src, src_frame, cand_frame = [], [], [], []
    off = 0

    def add(planes, w, h):
        nonlocal off
        flat = torch.cat([p.reshape(-1) for p in planes]).to(torch.int16)
        chunks.append(flat)
        metas.append((off, w, h))
        off += flat.numel()
        return len(metas) - 1

    for r, (w, h) in enumerate(MULTI_RES):
        for k in range(sources[r]):
            src = synth.yuv420p10_source(h, w, k, seed=100 + r, device=device)
            si = len(src_res)
            src_res.append(r)
            src_frame.append(add(src, w, h))
            for st in MULTI_DCT_STEPS:
                cand = (synth.block_dct_quantise(src[0], st, 64, 940),
                        synth.block_dct_quantise(src[1], 2 * st, 64, 960),
                        synth.block_dct_quantise(src[2], 2 * st, 64, 960))
                cand_src.append(si)
                cand_frame.append(add(cand, w, h))
    buf = torch.cat(chunks)
    return buf, metas, src_res, cand_src, src_frame, cand_frame


def multi_descs(buf, metas, idx):
    base = buf.data_ptr()
    out = []
    for i in idx:
        off, w, h = metas[i]
        cw, ch = (w + 1) // 2, (h + 1) // 2
        a = base + 2 * off
        out.append(([a, a + 2 * w * h, a + 2 * (w * h + cw * ch)], 2 * w, 2 * cw))
    return out


def bench_multi(v, args, ws, rank):
    import ctypes
    import torch
    sources = [max(1, int(round(n * args.multi_scale))) for n in MULTI_SOURCES]
    buf, metas, src_res, cand_src, src_frame, cand_frame = make_multi_inputs("cuda", sources)
    npairs, nsrc = len(cand_src), len(src_res)
    ms = [src_res.count(r) for r in range(len(MULTI_RES))]
    mp = [8 * n for n in ms]
    flags = v.MULTI_SSIMU2 | v.MULTI_BUTTERAUGLI | v.MULTI_FP16 | v.MULTI_AUTOTUNE
    # the autotuner's cache file: $VSHIP_MULTI_TUNE_CACHE, else one of this run and rank in the
    # system temp folder (never shared with other jobs, nor with this job's other ranks)
    tune = os.environ.get("VSHIP_MULTI_TUNE_CACHE") or os.path.join(
        tempfile.gettempdir(), f"vship_multi_tune.{os.getpid()}.{rank}.json")
    sc = v.MultiScorer(MULTI_RES, ms, mp, flags, 2, 203.0, tune)
    srcs = multi_descs(buf, metas, src_frame)
    cands = multi_descs(buf, metas, cand_frame)
    s2 = torch.zeros(npairs, dtype=torch.float64, device="cuda")
    bn = torch.zeros(3 * npairs, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def step(b=buf):
        sc.compute_async(srcs, src_res, cands, cand_src, v.IN_YUV420P10, s2.data_ptr(), bn.data_ptr(),
                         stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    barrier(ws)
    sec = max_over_ranks(e0.elapsed_time(e1) / 1e3, ws)
    scores = s2.cpu()
    # kernel breakdown: one more step with every launch bracketed by events (no graph)
    v.profile_report()
    v.profile_enable(True)
    step()
    torch.cuda.synchronize()
    v.profile_enable(False)
    prof = v.profile_report()
    launches = sum(n for n, _ in prof.values())
    total_ms = sum(t for _, t in prof.values())
    s2_ms = sum(t for k, (_, t) in prof.items() if k.startswith("ssimu2"))
    # stats kernel roofline (FP32 source + FP16-delta candidate pyramids)
    stats_n, stats_ms = prof.get("ssimu2_multi_stats", (0, 0.0))
    alg = sum(ssimu2_stats_bytes_fp16(*MULTI_RES[src_res[s]]) for s in cand_src)
    peak, peak_kind = measured_peaks()
    achieved = alg / (stats_ms / 1e3) / 1e9 if stats_ms > 0 else 0.0
    knobs = sc.knobs()

    # end to end: every step copies all frames (64 sources once, 512 candidates) from pinned host
    # memory and reads both score arrays back
    hbuf = buf.cpu().pin_memory()
    dbuf = torch.empty_like(buf)
    srcs_e = multi_descs(dbuf, metas, src_frame)
    cands_e = multi_descs(dbuf, metas, cand_frame)
    hs2 = torch.empty(npairs, dtype=torch.float64).pin_memory()
    hbn = torch.empty(3 * npairs, dtype=torch.float64).pin_memory()

    def e2e_step():
        dbuf.copy_(hbuf, non_blocking=True)
        sc.compute_async(srcs_e, src_res, cands_e, cand_src, v.IN_YUV420P10, s2.data_ptr(), bn.data_ptr(),
                         stream.cuda_stream)
        hs2.copy_(s2, non_blocking=True)
        hbn.copy_(bn, non_blocking=True)
        stream.synchronize()

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_sec = max_over_ranks(time.perf_counter() - t0, ws)
    e2e_ok = bool(torch.equal(hs2, scores))
    sc.free()

    # the plain per-pair path on the same pairs: one-resolution batch handlers, FP32, no reuse
    plain_ms = 0.0
    for r, (w, h) in enumerate(MULTI_RES):
        js = [j for j in range(npairs) if src_res[cand_src[j]] == r]
        if not js:
            continue
        fr = []
        for j in js:
            fr += multi_descs(buf, metas, [src_frame[cand_src[j]], cand_frame[j]])
        table = v.device_frames_table(fr)
        bchunk = max(1, min(len(js), int(6e9 // v.lib().Vship_ButteraugliDeviceBytes(w, h, 1))))
        e_s = v.SSIMU2Batch(w, h, len(js))
        e_b = v.ButteraugliBatch(w, h, bchunk, 2, 203.0)
        o_s = torch.zeros(len(js), dtype=torch.float64, device="cuda")
        o_b = torch.zeros(3 * len(js), dtype=torch.float64, device="cuda")
        fsz = ctypes.sizeof(v.DeviceFrame)

        def pstep():
            e_s.compute_async(table.data_ptr(), len(js), v.IN_YUV420P10, o_s.data_ptr(), stream.cuda_stream)
            for c0 in range(0, len(js), bchunk):
                n = min(bchunk, len(js) - c0)
                e_b.compute_async(table.data_ptr() + 2 * c0 * fsz, n, v.IN_YUV420P10, o_b[3 * c0:].data_ptr(), 0,
                                  stream.cuda_stream)

        pstep()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            pstep()
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms += e0.elapsed_time(e1) / args.steps
        e_s.free()
        e_b.free()
    plain_ms = max_over_ranks(plain_ms / 1e3, ws) * 1e3
    res = {
        "value": npairs * ws * args.steps / sec, "unit": "frame-pairs/s (SSIMU2 + Butteraugli)",
        "ms_per_step": sec / args.steps * 1e3, "pairs_per_step": npairs, "sources_per_step": nsrc,
        "config": {"workload": "batched_multi: " + " + ".join(f"{n}x{w}x{h}" for n, (w, h) in zip(ms, MULTI_RES))
                               + " YUV420P10 sources x 8 block-DCT candidates (steps 4..32), both metrics",
                   "flags": "ssimu2+butteraugli+fp16_delta+autotune, CUDA graph replay",
                   "l2": "inputs 1.3 GB and pyramids > L2, no flush"},
        "e2e": {"value": npairs * ws * args.steps / e2e_sec, "unit": "frame-pairs/s",
                "h2d_bytes_per_step": int(buf.numel() * 2), "d2h_bytes_per_step": npairs * 32,
                "scores_match_device": e2e_ok},
        "plain_per_pair_path": {"value": npairs * ws / (plain_ms / 1e3), "ms_per_step": plain_ms,
                                "what": "per-resolution batch handlers, FP32 pyramids, every pair decodes its source"},
        "ssimu2_share": s2_ms / total_ms if total_ms > 0 else None,
        "roofline": {"bound": "hbm", "kernel": "ssimu2_multi_stats", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": stats_ms / max(stats_n, 1)},
        "knobs": knobs,
        "kernel_share": {k: {"launches": n, "ms": round(t, 3), "share": round(t / total_ms, 4)}
                         for k, (n, t) in sorted(prof.items(), key=lambda x: -x[1][1])} if total_ms > 0 else {},
        "kernel_share_how": ("one more step with every launch on one stream, each bracketed by CUDA events (the "
                             "timed steps overlap the resolutions' chains on side streams; serialised, an event pair "
                             "times its own kernel only)"),
        "serialised_step_ms": total_ms,
        "gpu_launches": launches * args.steps,
        "clocks": clocks,
    }
    del buf, dbuf
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------------------------------------------
# serving loop: Poisson arrivals, 70 % SSIMU2 / 30 % Butteraugli, 1..16 pairs per request,
# source reuse probability 0.8, 64 GB admission budget

SERVE_RATES = [50, 100, 200, 500, 1000, 2000]


def wait_until(t0, ta):
    """Sleep, then spin the last millisecond, until ta seconds after t0 (the spin is short, so
    worker threads keep getting the interpreter)."""
    while True:
        dt = ta - (time.perf_counter() - t0)
        if dt <= 0:
            return
        if dt > 0.002:
            time.sleep(dt - 0.001)


def serve_stream(rate, nreq, nsrc_pool, seed):
    """Seeded request stream: (arrival_s, metric, npairs, source_key, pool_source, candidate idx)."""
    import numpy as np
    rs = np.random.default_rng(seed)
    t = np.cumsum(rs.exponential(1.0 / rate, nreq))
    out, used, next_key = [], [], 1
    for i in range(nreq):
        metric = 0 if rs.random() < 0.7 else 1
        npairs = int(rs.integers(1, 17))
        if used and rs.random() < 0.8:
            key, ps = used[int(rs.integers(0, len(used)))]
        else:
            key, ps = next_key, int(rs.integers(0, nsrc_pool))
            next_key += 1
            used.append((key, ps))
        cand = [int(x) for x in rs.integers(0, len(MULTI_DCT_STEPS), npairs)]
        out.append((float(t[i]), metric, npairs, key, ps, cand))
    return out


def run_serving(v, stream, pool_frames, res_index, admission, cache):
    """Drive the serving runtime with the stream; returns (latencies s, wall s, stats)."""
    import numpy as np
    srv = v.Server([pool_frames["size"]], v.IN_YUV420P10, admission_bytes=admission, cache_bytes=cache,
                   max_batch_pairs=32)
    done = {}
    stop = threading.Event()

    def poller():
        while not stop.is_set() or len(done) < len(stream):
            for rid, status, lat in srv.poll(256, 0.05):
                done[rid] = (status, lat)
            if stop.is_set() and len(done) >= len(stream):
                break

    th = threading.Thread(target=poller)
    th.start()
    outs = []
    t0 = time.perf_counter()
    for i, (ta, metric, npairs, key, ps, cand) in enumerate(stream):
        wait_until(t0, ta)
        src, cands = pool_frames["src"][ps], pool_frames["cands"][ps]
        out = np.zeros(npairs * (1 if metric == 0 else 3))
        outs.append(out)
        srv.submit(i, metric, res_index, key, src, [cands[c] for c in cand], out)
    srv.drain()
    wall = time.perf_counter() - t0
    stop.set()
    th.join()
    stats = srv.stats()
    srv.free()
    bad = [r for r, (s, _) in done.items() if s != 0]
    if bad:
        raise RuntimeError(f"serving: {len(bad)} requests failed")
    return np.array([done[i][1] for i in range(len(stream))]), wall, stats


def run_plain_serving(v, stream, pool_frames):
    """The same stream through the plain per-pair path: one batch handler per metric, requests in
    arrival order, one call each (no cache, no cross-request batching)."""
    import numpy as np
    import queue as _q
    import torch
    w, h = pool_frames["size"]
    e_s = v.SSIMU2Batch(w, h, 16)
    e_b = v.ButteraugliBatch(w, h, 16, 2, 203.0)
    o_s = torch.zeros(16, dtype=torch.float64, device="cuda")
    o_b = torch.zeros(48, dtype=torch.float64, device="cuda")
    tables = {}
    q = _q.Queue()
    lat = np.zeros(len(stream))
    stream_ = torch.cuda.current_stream()

    def worker():
        while True:
            item = q.get()
            if item is None:
                return
            i, t_sub = item
            _, metric, npairs, key, ps, cand = stream[i]
            fr = []
            for c in cand:
                fr += [pool_frames["src"][ps], pool_frames["cands"][ps][c]]
            tb = v.device_frames_table(fr)
            if metric == 0:
                e_s.compute_async(tb.data_ptr(), npairs, v.IN_YUV420P10, o_s.data_ptr(), stream_.cuda_stream)
                o_s[:npairs].cpu()
            else:
                e_b.compute_async(tb.data_ptr(), npairs, v.IN_YUV420P10, o_b.data_ptr(), 0, stream_.cuda_stream)
                o_b[:3 * npairs].cpu()
            lat[i] = time.perf_counter() - t_sub

    th = threading.Thread(target=worker)
    th.start()
    t0 = time.perf_counter()
    for i, (ta, *_rest) in enumerate(stream):
        wait_until(t0, ta)
        q.put((i, time.perf_counter()))
    q.put(None)
    th.join()
    wall = time.perf_counter() - t0
    e_s.free()
    e_b.free()
    return lat, wall


def bench_serving(v, args, ws, rank):
    import numpy as np
    import torch
    w, h = parse_size(args.serve_size)
    nsrc_pool = 8
    buf, metas, src_res, cand_src, src_frame, cand_frame = make_multi_inputs_one(w, h, nsrc_pool)
    pool_frames = {"size": (w, h), "src": multi_descs(buf, metas, src_frame),
                   "cands": [multi_descs(buf, metas, cand_frame[8 * s: 8 * s + 8]) for s in range(nsrc_pool)]}
    admission, cache = 64 << 30, 16 << 30
    sys.setswitchinterval(1e-4)
    # warm-up: builds the pool's blocks, loads kernels
    run_serving(v, serve_stream(50, 20, nsrc_pool, 99), pool_frames, 0, admission, cache)
    rows = []
    for rate in SERVE_RATES:
        nreq = int(min(max(rate * args.serve_seconds, 40), args.serve_max_requests))
        stream = serve_stream(rate, nreq, nsrc_pool, 1000 + rate)
        lat, wall, stats = run_serving(v, stream, pool_frames, 0, admission, cache)
        pairs = sum(x[2] for x in stream)
        row = {"offered_req_s": rate, "requests": nreq, "pairs": pairs,
               "throughput_req_s": nreq / wall, "throughput_pairs_s": pairs / wall,
               "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
               "cache_hit_rate": stats["cache_hits"] / max(1, stats["cache_hits"] + stats["cache_misses"]),
               "batches": stats["batches"], "mean_batch_pairs": pairs / max(1, stats["batches"]),
               "admission_peak_gb": stats["admission_peak_bytes"] / 1e9}
        if rate <= args.serve_plain_max_rate:
            plat, pwall = run_plain_serving(v, stream, pool_frames)
            row["plain"] = {"throughput_req_s": nreq / pwall, "throughput_pairs_s": pairs / pwall,
                            "p50_ms": float(np.percentile(plat, 50) * 1e3),
                            "p99_ms": float(np.percentile(plat, 99) * 1e3)}
        rows.append(row)
    del buf
    torch.cuda.empty_cache()
    return {"workload": f"serving: {w}x{h} YUV420P10, Poisson arrivals, 70% SSIMU2 / 30% Butteraugli, "
                        f"1-16 pairs per request, source reuse p=0.8 over a pool of {nsrc_pool} sources x 8 "
                        f"DCT candidates, admission 64 GB (48N / 124N B per pair), source cache 16 GB",
            "latency": "host submit -> results in the request's host buffer",
            "plain": "same stream, one request at a time through the per-resolution batch handlers "
                     "(no cache, no cross-request batching)",
            "rates": rows}


def make_multi_inputs_one(w, h, nsrc):
    """nsrc sources of one resolution, each with the 8 DCT candidates (make_multi_inputs layout)."""
    global MULTI_RES
    saved = MULTI_RES
    try:
        MULTI_RES = [(w, h)]
        return make_multi_inputs("cuda", [nsrc])
    finally:
        MULTI_RES = saved


def main_ours(args):
    import torch
    ws, rank, local = dist_setup(args)
    import vship_gb300 as v
    if not os.path.exists(v.LIB_PATH):
        from vship_gb300 import build
        build.build()
    v.lib()
    link = host_link_gbs()
    out = {"metric": "frame-pairs/s (1080p SSIMU2)", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "gpu_launches": 0}
    s2 = {}
    if not args.skip_ssimu2:
        s2 = bench_workload(v, "ssimu2", args, ws, rank)
        out.update({
        "value": s2["value"], "unit": "frame-pairs/s", "ms_per_step": s2["ms_per_step"],
        "dtype": "f32", "data": "synthetic (seeded gratings + noise, block-DCT distortion)",
        "config": {"workload": f"ssimu2_1080p: {args.pairs} pairs 1920x1080 YUV420P10 -> RGB48 planes (the "
                               "reference front-end's conversion), 8x8 block-DCT distortion",
                   "pairs_per_step": args.pairs,
                   "parallelism": f"replicas x{ws}", "l2": "inputs 12 GB > L2, no flush",
                   "launch_chunk_pairs": args.chunk},
        "e2e": s2["e2e"], "roofline": s2["roofline"], "fp32_roofline": s2["fp32_roofline"],
        "gpu_launches": s2["gpu_launches"], "clocks": s2["clocks"],
        "kernel_share": s2["kernel_share"], "pipeline_bytes_per_pair": s2["pipeline_bytes_per_pair"],
        "kernel_roofline": s2["kernel_roofline"],
        "yuv420p10": s2["yuv420p10"], "float32_rgb": s2["float32_rgb"], "input": s2["input"],
        "score_check": s2["score_check"],
        })
    for k in ("reference_cuda", "error_vs_fp64", "cpu_baseline", "fp16_deltas"):
        if k in s2:
            out[k] = s2[k]
    out["host_link"] = {"h2d_gbs": round(link, 1),
                        "note": "pinned host -> device copy, 256 MiB; e2e frac = its h2d bytes/s over this"}
    if s2:
        n = s2["pairs_per_step"]
        out["host_link"]["ssimu2_e2e_frac"] = {"rgb48": link_frac(link, s2["e2e"], n),
                                              "float32_rgb": link_frac(link, s2["float32_rgb"]["e2e"], n),
                                              "yuv420p10": link_frac(link, s2["yuv420p10"]["e2e"], n)}
    if not args.skip_butter:
        b = bench_workload(v, "butter", args, ws, rank)
        out["butteraugli_4k"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "pairs_per_step", "launch_chunk_pairs",
                                                   "e2e", "yuv420p10",
                                                   "float32_rgb", "input",
                                                   "roofline", "gpu_launches", "clocks", "kernel_share",
                                                   "pipeline_bytes_per_pair", "score_check", "fp16_bands",
                                                   "kernel_roofline", "reference_cuda", "error_vs_fp64")
                                 if k in b}
        if "cpu_baseline" in b:
            out["butteraugli_4k"]["cpu_baseline"] = b["cpu_baseline"]
        out["gpu_launches"] += b["gpu_launches"]
    if not args.skip_multi:
        m = bench_multi(v, args, ws, rank)
        out["batched_multi"] = m
        out["gpu_launches"] += m["gpu_launches"]
    if not args.skip_serving:
        out["serving"] = bench_serving(v, args, ws, rank)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main_reference(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    import numpy as np
    import oracle
    from vship_gb300 import synth
    oracle.lib()
    nt = os.cpu_count() or 1
    # each step: one 1080p pair of the same workload through the reference's math on all cores
    frames = []
    for t in range(args.warmup + args.steps):
        r, d = synth.yuv420p10_frames(H1080, W1080, t, seed=7, distortion="dct", device="cpu")
        # RGB48 planes, the input form of the measured workload
        a = to_rgb48(synth.yuv420p10_to_rgb(r)).numpy().view(np.uint16)
        b = to_rgb48(synth.yuv420p10_to_rgb(d)).numpy().view(np.uint16)
        frames.append(([np.ascontiguousarray(a[c]) for c in range(3)], [np.ascontiguousarray(b[c]) for c in range(3)]))
    for t in range(args.warmup):
        oracle.ssimu2(*frames[t], precision=32, nthreads=nt)
    t0 = time.perf_counter()
    for t in range(args.warmup, args.warmup + args.steps):
        oracle.ssimu2(*frames[t], precision=32, nthreads=nt)
    sec = time.perf_counter() - t0
    value = args.steps / sec
    out = {
        "impl": "reference", "metric": "frame-pairs/s (1080p SSIMU2)", "value": value, "unit": "frame-pairs/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded gratings + noise, block-DCT distortion)",
        "config": {"workload": "ssimu2_1080p: 1 pair per step of the 1920x1080 YUV420P10 block-DCT workload, "
                               "RGB48 planes", "pairs_per_step": 1},
        "cpu_baseline": {"value": value, "unit": "frame-pairs/s", "cores": nt, "kind": "port",
                         "sample": f"{args.steps} pairs, 1 per step"},
        "e2e": {"value": value, "unit": "frame-pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU implementation (its math exists only as CUDA kernels); this is that math "
                "restated in C++ (oracle/, FP32 instantiation), threaded over all host cores. The reference's own "
                "CUDA build on the GPU is measured in the main run's reference_cuda block",
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--pairs", type=int, default=240)
    ap.add_argument("--chunk", type=int, default=120, help="SSIMU2 pairs per batched launch")
    ap.add_argument("--butter-pairs", type=int, default=60)
    ap.add_argument("--butter-chunk", type=int, default=15, help="Butteraugli pairs per batched launch")
    ap.add_argument("--e2e-threads", type=int, default=8)
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--e2e-warmup", type=int, default=4,
                    help="untimed e2e steps first (host threads, pinned pages and copy engines settle)")
    ap.add_argument("--cpu-sample", type=int, default=4)
    ap.add_argument("--skip-butter", action="store_true")
    ap.add_argument("--skip-ssimu2", action="store_true")
    ap.add_argument("--skip-multi", action="store_true")
    ap.add_argument("--skip-serving", action="store_true")
    ap.add_argument("--skip-half-bands", action="store_true",
                    help="skip the FP16 storage forms (Butteraugli FP16 bands, SSIMU2 FP16 deltas)")
    ap.add_argument("--error-pairs", type=int, default=8,
                    help="SSIMU2 pairs scored by the FP64 oracle for the headline's error")
    ap.add_argument("--butter-error-pairs", type=int, default=4,
                    help="Butteraugli pairs scored by the FP64 oracle for the error of each storage form")
    ap.add_argument("--skip-reference-cuda", action="store_true",
                    help="skip the reference CUDA build's leg (reference_cuda)")
    ap.add_argument("--ref-steps", type=int, default=2, help="timed steps per trial of the reference CUDA leg")
    ap.add_argument("--ref-warmup", type=int, default=1)
    ap.add_argument("--ref-worst-pairs", type=int, default=4,
                    help="SSIMU2 pairs where the builds differ most, scored by the FP64 oracle")
    ap.add_argument("--serve-size", default=f"{W4K}x{H4K}")
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--serve-max-requests", type=int, default=400)
    ap.add_argument("--serve-plain-max-rate", type=float, default=2000)
    ap.add_argument("--multi-scale", type=float, default=1.0, help="fraction of the 64 sources (small runs)")
    ap.add_argument("--ssimu2-size", default=f"{W1080}x{H1080}")
    ap.add_argument("--butter-size", default=f"{W4K}x{H4K}")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        main_reference(args)
    else:
        main_ours(args)


if __name__ == "__main__":
    main()
