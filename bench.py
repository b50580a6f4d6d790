#!/usr/bin/env python3
"""Transform-PAL 3D throughput on GB300 (fields/s), one JSON line.

Workload (one "step"): decode every frame of a 500-field synthetic PAL
capture (1135x313 uint16 fields, seeded encoder, panning 1.5 px/field and
0.5 line/field plus a static bar region, AWGN 0.5%) with Transform-PAL 3D,
threshold 0.4, to yuv444p16 (or yuv444ps with --format ps).

  value  -- inputs already resident in HBM; device-timed (CUDA events on the
            launching stream) over exactly --steps steps.
  e2e    -- the same decode through the reference-facing chd_* ABI: the
            capture is a .tbc + JSON sidecar in host memory, decoded with
            chd_decode_frames_async; field windows are uploaded and frames
            downloaded inside the timed region (overlapped with the kernels).
  --impl reference -- the reference's algorithm on the host cores (the CPU
            restatement in oracle/, all threads), on a bounded sample per step.

Multi-GPU: the path does not shard beyond independent replicas; under
torchrun each rank decodes its own copy of the workload on its own GPU and
value = fields processed by all ranks / max over ranks of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Transform-PAL 3D fields/s on 1 GB300: plain vs TC+NN form at matched chroma PSNR"
FIELD_BYTES_IN = 1135 * 313 * 2                  # 710,510 B per input field
OUT_BYTES = {"p16": 948 * 288 * 3 * 2, "ps": 948 * 288 * 3 * 4}   # per output field
# Algorithmic work per output field (fixed convention of the roofline
# accounting: 2.5 N log2 N per real FFT each way, window, threshold, OLA,
# demod+pack), in FLOP; bytes = input field + its output planes.
FLOP_PER_FIELD_3D = 692_311_680
# the transform's share of it (2,220 tiles x 259,584 FLOP), for the
# transform kernel's FP32 roofline
FLOP_PER_FIELD_3D_TRANSFORM = 576_276_480
# Transform-PAL 2D by the same convention: 2,257 tiles of 16 x 32 per field,
# 2 (2.5 x 512 x 9) + 512 + 10 x 80 + 2 x 512 = 25,376 FLOP each
FLOP_PER_FIELD_2D_TRANSFORM = 57_273_632


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fields", type=int, default=500)
    ap.add_argument("--format", default="p16", choices=["p16", "ps"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the tensor-core forms and chroma PSNR report")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-captures measurement")
    ap.add_argument("--kind", default="3d", choices=["3d", "2d"],
                    help="Transform-PAL 3D (the metric) or 2D (for profiling the 2D kernel)")
    ap.add_argument("--form", default="plain", choices=["plain", "tc_3xtf32", "tc_bf16x3", "learned"],
                    help="transform form of the timed decode (the tensor-core and learned forms for profiling them)")
    ap.add_argument("--workload", default="stream", choices=["stream", "batched"],
                    help="stream: the 500-field 3D capture (the headline line); batched: 48 captures of "
                         "6-300 fields, 40%% 2D / 60%% 3D, one threshold each, through chdg_batch_*")
    return ap.parse_args()


def workload_desc(a):
    two = getattr(a, "kind", "3d") == "2d"
    return (f"Transform-PAL {'2D' if two else '3D'}, {a.fields} PAL fields 1135x313 uint16 (seed {a.seed}, "
            f"pan 1.5 px/field + 0.5 line/field, static 75% bars, AWGN 0.5%), "
            f"{'16x32' if two else '8x32x16'} tiles, threshold 0.4, "
            f"yuv444{'p16' if a.format == 'p16' else 'ps'} out")


def make_capture(a):
    import numpy as np
    from libchromadec_gb300 import synth
    cache = f"/tmp/chdg_bench_{a.fields}_{a.seed}.npy"
    if os.path.exists(cache):
        try:
            return np.load(cache)
        except Exception:
            pass
    cap = synth.make_capture(a.fields, synth.SynthConfig(seed=a.seed, pan_x=1.5, pan_y=0.5))
    try:
        np.save(cache, cap.fields)
    except Exception:
        pass
    return cap.fields


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp32_sgemm_peak(device: int):
    """FP32 CUDA-core throughput as cuBLAS reaches it on this GPU: an 8192^3
    SGEMM with TF32 off, best of 5 (CUDA events), in TFLOP/s -- the FP32
    counterpart of the driver's measured bf16 peak. None if it cannot run."""
    try:
        import torch
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        try:
            n = 8192
            x = torch.randn(n, n, device=f"cuda:{device}", dtype=torch.float32)
            y = torch.randn(n, n, device=f"cuda:{device}", dtype=torch.float32)
            for _ in range(2):
                torch.matmul(x, y)
            best = None
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(x, y)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            del x, y
            return 2.0 * n ** 3 / (best / 1000.0) / 1e12
        finally:
            torch.backends.cuda.matmul.allow_tf32 = prev
    except Exception:
        return None


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_cpu(a, fields, nframes_sample, threads, kind=3, first=0):
    """Oracle (the reference's algorithm restated in C) on the host cores."""
    from oracle import oracle as O
    p = O.params(kind=kind, fmt=O.FMT_P16 if a.format == "p16" else O.FMT_PS)
    t0 = time.perf_counter()
    O.decode_frames(p, fields, first, nframes_sample, threads=threads)
    return time.perf_counter() - t0


def _median_rate(a, fields, nframes, threads, reps=3, kind=3):
    times = [run_cpu(a, fields, nframes, threads, kind=kind) for _ in range(reps)]
    return 2 * nframes / statistics.median(times), times


def cpu_baseline(a, fields, budget_s=6.0):
    """The CPU path on the host cores, a reported baseline: the median of 3
    repetitions on all host threads and on one thread, for the 3D workload
    (a bounded sample of the same capture) and for the 16-field Transform-PAL
    2D capture (whole)."""
    import numpy as np
    from libchromadec_gb300 import synth
    threads = cpu_threads()
    nfr = fields.shape[0] // 2
    # calibrate on a few frames, then size the sample to the budget
    t1 = run_cpu(a, fields, max(1, min(threads, 4)), threads)
    per_frame = t1 / max(1, min(threads, 4)) * min(threads, 4) / threads
    n = int(max(threads, min(nfr, budget_s / max(per_frame, 1e-6))))
    n = min(n, nfr)
    v_all, t_all = _median_rate(a, fields, n, threads)
    n1 = 2
    v_one, t_one = _median_rate(a, fields, n1, 1)
    cap2 = synth.make_capture(16, synth.SynthConfig(seed=a.seed, pan_x=0.0, pan_y=0.0)).fields
    v2_all, _ = _median_rate(a, cap2, 8, threads, kind=2)
    v2_one, _ = _median_rate(a, cap2, 8, 1, kind=2)
    return {"value": v_all, "unit": "fields/s", "cores": threads, "kind": "port",
            "sample": f"frames 0..{n - 1} ({2 * n} fields) of the same capture, all {threads} host threads, one "
                      f"decoder instance per thread (chd_decode_frames_async's model), FP64 CPU oracle (radix-2 "
                      f"FP64 FFT; FFTW is not installed on these hosts); median of 3 repetitions "
                      f"({', '.join(f'{t:.2f}' for t in t_all)} s)",
            "one_thread": {"value": v_one, "unit": "fields/s", "cores": 1,
                           "sample": f"frames 0..{n1 - 1} ({2 * n1} fields), median of 3 "
                                     f"({', '.join(f'{t:.2f}' for t in t_one)} s)"},
            "transform_2d_16_fields": {
                "all_threads": v2_all, "one_thread": v2_one, "unit": "fields/s",
                "sample": "the whole 16-field capture (seeded, static content), Transform-PAL 2D 16x32 tiles, "
                          "threshold 0.4, median of 3"}}


def reference_arm(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    fields = make_capture(a)
    threads = cpu_threads()
    # each step: a bounded sample of frames on all host threads, sized so
    # the timed steps take about 90 s in all (at most 10 s each)
    budget = max(1.0, min(10.0, 90.0 / max(1, a.steps)))
    t1 = run_cpu(a, fields, max(1, threads), threads)
    per_frame = t1 / max(1, threads)
    n = int(max(threads, min(fields.shape[0] // 2, budget / max(per_frame, 1e-6))))
    n = min(n, fields.shape[0] // 2)
    for _ in range(a.warmup):
        run_cpu(a, fields, min(n, threads), threads)
    times = [run_cpu(a, fields, n, threads) for _ in range(a.steps)]
    total = sum(times)
    value = 2 * n * a.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "fields/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000 * total / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(a), "sample_frames_per_step": n},
        "cpu_baseline": {"value": value, "unit": "fields/s", "cores": threads, "kind": "port",
                         "sample": f"{n} frames per step of the same capture, all {threads} host threads; the "
                                   f"reference's Transform-PAL/PALcolour/OutputWriter restated in C (oracle/), "
                                   f"FP64 FFT (FFTW is not installed on this host)"},
        "e2e": {"value": value, "unit": "fields/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def pipeline_batches(a: int, b: int, batch: int, edge: int):
    """The batch boundaries FramePipeline::decode uses for frames [a, b)."""
    out, c = [], a
    edge = min(edge, batch)
    if b - a <= batch:
        return [(a, b)] if b > a else []
    out.append((c, c + edge))
    c += edge
    while b - c > batch + edge:
        out.append((c, c + batch))
        c += batch
    if b - c > edge:
        out.append((c, b - edge))
        c = b - edge
    out.append((c, b))
    return out


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """The slowest rank's time: replicas are timed together and the job takes
    as long as its slowest GPU."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(fields_per_rank_step: int, steps: int, seconds_local: float, dist, device: str = "cuda"):
    """Whole-job fields/s of N independent replicas: all ranks' fields over
    the max over ranks of the timed region."""
    world = dist.get_world_size() if dist is not None else 1
    slowest = max_over_ranks(seconds_local, dist, device)
    return fields_per_rank_step * steps * world / slowest, slowest


def e2e_abi(a, fields_np, rank, barrier, dist):
    """Fields/s through chd_video_open_composite + chd_decode_frames_async."""
    import ctypes as C
    from libchromadec_gb300 import abi, synth
    nfields = fields_np.shape[0]
    nframes = nfields // 2
    path = f"/tmp/chdg_bench_{a.fields}_{a.seed}_r{rank}.tbc"
    if not (os.path.exists(path) and os.path.getsize(path) == fields_np.nbytes):
        synth.write_tbc(path, synth.SynthCapture(fields=fields_np, dropouts=[[] for _ in range(nfields)]))
    # Write back the page cache's dirty data first (this capture, and whatever
    # an earlier job on the host wrote): the kernel's background writeback
    # would otherwise compete with the timed steps for the host's memory.
    os.sync()
    L = abi.lib()
    v = abi.Video(path)
    d = abi.Decoder(v, abi.DEC_TRANSFORM_3D)
    d.set("output_format", "yuv444p16" if a.format == "p16" else "yuv444ps")
    d.commit()
    oi = d.output_info()
    got = [0]
    free = L.chd_frame_free

    def on_frame(user, status, idx, frame):
        if frame:
            free(frame)
        if status == 0:
            got[0] += 1

    cb = abi.FRAME_DONE_CB(on_frame)
    idx = (C.c_int64 * nframes)(*range(nframes))

    def step():
        if L.chd_decode_frames_async(d._h, idx, nframes, cb, None, None) != 0:
            raise RuntimeError("chd_decode_frames_async failed")

    for _ in range(max(1, a.warmup)):
        step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        step()
    dt = time.perf_counter() - t0
    if got[0] != nframes * (a.steps + max(1, a.warmup)):
        raise RuntimeError(f"chd_decode_frames_async delivered {got[0]} frames")
    value, dt = replica_throughput(nfields, a.steps, dt, dist)
    # uploaded per step: the pipeline's batches (16 frames first and last,
    # 64 in between), each with its 2 + 4 frame window halo
    h2d = 0
    for b, be in pipeline_batches(0, nframes, 64, 16):
        h2d += (min(nframes, be + 4) - max(0, b - 2)) * 2 * FIELD_BYTES_IN
    frame_bytes = oi.width * oi.height * 3 * (2 if a.format == "p16" else 4)
    d.close()
    v.close()
    return {"value": value, "unit": "fields/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": nframes * frame_bytes, "timer": "host wall clock around the blocking call",
            "path": "chd_video_open_composite(.tbc + .tbc.json) -> chd_decode_frames_async(all frames) -> "
                    "per-frame callback frees the chd_frame_t"}


BATCH_CAPTURES = 48


def batched_specs(seed: int):
    """The batched workload: 48 captures of uniform 6-300 fields, 40 % Transform
    2D / 60 % 3D, threshold U[0.3, 0.6], horizontal pan U[0, 3] px/field and
    vertical U[0, 1] line/field, each its own seeded content, 1 % of lines
    with dropouts (runs of 20-400 samples at the sync tip, with sidecar spans)."""
    import numpy as np
    rng = np.random.default_rng(seed + 100)
    specs = []
    for i in range(BATCH_CAPTURES):
        n = int(rng.integers(6, 301))
        kind = 7 if rng.random() < 0.4 else 8
        specs.append(dict(nfields=n, kind=kind, threshold=float(rng.uniform(0.3, 0.6)),
                          pan_x=float(rng.uniform(0.0, 3.0)), pan_y=float(rng.uniform(0.0, 1.0)),
                          seed=seed * 1000 + 17 * i + 5))
    return specs


def _gen_capture(args):
    """Worker: encode one capture into its slice of the shared field file."""
    import numpy as np
    from libchromadec_gb300 import synth
    path, offset, spec = args
    cap = synth.make_capture(spec["nfields"], synth.SynthConfig(seed=spec["seed"], pan_x=spec["pan_x"],
                                                                pan_y=spec["pan_y"], dropout_line_fraction=0.01))
    mm = np.memmap(path, dtype=np.uint16, mode="r+", offset=offset * 2, shape=cap.fields.shape)
    mm[:] = cap.fields
    mm.flush()
    del mm
    return [(f, s[0], s[1], s[2]) for f, spans in enumerate(cap.dropouts) for s in spans]


def batched_workload(a):
    """Every capture's fields in one file (generated once per host in
    parallel worker processes, started with spawn) and their dropouts."""
    import multiprocessing as mp
    import pickle
    import numpy as np
    from libchromadec_gb300 import synth
    specs = batched_specs(a.seed)
    flen = synth.FIELD_WIDTH * synth.FIELD_HEIGHT
    total = sum(s["nfields"] for s in specs)
    path = f"/tmp/chdg_batch_{a.seed}_{total}.u16"
    dpath = path + ".drop.pkl"
    offsets, o = [], 0
    for sp in specs:
        offsets.append(o)
        o += sp["nfields"] * flen
    if not (os.path.exists(path) and os.path.exists(dpath) and os.path.getsize(path) == 2 * total * flen):
        np.memmap(path, dtype=np.uint16, mode="w+", shape=(total * flen,)).flush()
        with mp.get_context("spawn").Pool(max(1, min(cpu_threads(), 32))) as pool:
            drops = pool.map(_gen_capture, [(path, offsets[i], sp) for i, sp in enumerate(specs)])
        with open(dpath, "wb") as fp:
            pickle.dump(drops, fp)
    with open(dpath, "rb") as fp:
        drops = pickle.load(fp)
    fields = np.memmap(path, dtype=np.uint16, mode="r", shape=(total, synth.FIELD_HEIGHT, synth.FIELD_WIDTH))
    return fields, specs, offsets, drops


def batched_measure(a):
    """Device-resident fields/s of the batched workload through chdg_batch_*:
    concealment, masks and both Transform modes of all 48 captures per step,
    replayed from one CUDA graph after autotuning."""
    import numpy as np
    import torch
    from libchromadec_gb300 import device as D, synth
    fields, specs, offsets, drops = batched_workload(a)
    fmt = D.FMT_P16 if a.format == "p16" else D.FMT_PS
    dtype = torch.int16 if fmt == D.FMT_P16 else torch.float32
    flen = synth.FIELD_WIDTH * synth.FIELD_HEIGHT
    dfields = torch.from_numpy(np.ascontiguousarray(fields).reshape(-1, flen).view(np.int16)).cuda()
    items, total_fields = [], 0
    for sp, off, dr in zip(specs, offsets, drops):
        n = sp["nfields"]
        f0 = off // flen
        out = torch.empty((n // 2, 3, 576, 948), dtype=dtype, device="cuda")
        mask = torch.empty((n // 2, 576, 948), dtype=torch.int16, device="cuda")
        items.append((dfields[f0:f0 + n], sp["kind"], sp["threshold"], out, dr, D.CONCEAL, mask))
        total_fields += 2 * (n // 2)
    s = torch.cuda.Stream()
    b = D.Batch(D.default_geometry(), D.default_config(kind=8, fmt=fmt))
    arr = D.Batch.captures(items)
    tuning = b.autotune(arr, s)
    warm = max(3, a.warmup)
    for _ in range(warm):
        b.decode(arr, s)
    s.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(3, a.steps // 4)
    with torch.cuda.stream(s):
        e0.record(s)
        for _ in range(steps):
            b.decode(arr, s)
        e1.record(s)
    s.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.close()
    n2d = sum(1 for sp in specs if sp["kind"] == 7)
    return {"metric": "Transform-PAL batched captures fields/s on 1 GB300", "value": total_fields / (ms / 1000.0),
            "unit": "fields/s", "ms_per_step": ms, "steps": steps, "warmup": warm,
            "workload": f"{len(specs)} captures of 6-300 fields ({total_fields} fields decoded), {n2d} Transform 2D / "
                        f"{len(specs) - n2d} 3D, thresholds U[0.3, 0.6], pans U[0, 3] px/field + U[0, 1] line/field, "
                        f"each its own seeded content, 1 % of lines with dropouts ({sum(len(d) for d in drops)} "
                        f"spans) concealed and masked inside the batch, yuv444{a.format}, device-resident, one "
                        f"CUDA graph per step",
            "dropout_spans": sum(len(d) for d in drops),
            "tuning": {"chunk_frames": tuning.chunk_frames, "max_blocks": tuning.max_blocks, "ms": tuning.ms}}


def run_batched(a):
    r = batched_measure(a)
    line = {"metric": r["metric"], "value": r["value"], "unit": "fields/s", "n_gpus": 1, "steps": r["steps"],
            "warmup": r["warmup"], "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": r["workload"], "tuning": r["tuning"]}}
    print(json.dumps(line), flush=True)


def learned_report(a, dfields, nfields, stream):
    """The learned form on the same workload: device-resident fields/s of the
    whole decode (feature pass, mask network, apply pass, demodulator), and
    chroma PSNR, cross-colour and cross-luma energy of the learned and the
    plain form against the encoder's ground truth over all the held-out
    fields (the network was trained on other seeds)."""
    import torch
    from libchromadec_gb300 import device as D, masknet_train as MT
    from tests import learned_eval as E
    try:
        w = MT.load_weights()
    except (OSError, ValueError) as exc:
        return f"no trained weights: {exc}"
    g = D.default_geometry()
    nframes = nfields // 2
    net = D.MaskNet(w)
    eng = D.Engine(g, D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_P16))
    eng.set_masknet(net)
    dout = torch.empty((nframes, 3, eng.out_height, eng.out_width), dtype=torch.int16, device="cuda")
    for _ in range(max(3, a.warmup)):
        eng.decode(dfields, 0, nframes, dout, stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(3, a.steps // 4)
    e0.record(stream)
    for _ in range(steps):
        eng.decode(dfields, 0, nframes, dout, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    tiles, fb_tiles = eng.learned_stats()
    del dout, eng
    ev = E.evaluate(w, nfields=nfields, seed=a.seed)
    net.close()
    return {"fields_per_s": nfields / (ms / 1000.0), "ms_per_step": ms, "evaluation": ev,
            "fallback_fraction": fb_tiles / tiles if tiles else None,
            "form": "FP32 walk DFTs; per-bin fractions from the 3-layer 16-channel 3x3x3 mask network "
                    "(BF16 weights and activations, FP32 accumulation) in place of the 0.4 threshold; tiles "
                    "with mean |p - 1/2| < 0.1 keep the threshold"}


def forms_report(a, dfields, nfields, plain_value, stream):
    """The metric's comparison of forms, outside the timed region: the plain
    form and the tensor-core forms (3xTF32, BF16x3 split products on tcgen05)
    on the same 500-field workload -- device-resident fields/s of each, chroma
    PSNR against the encoder's true chroma on the first 48 fields (same seed
    and content), each tensor-core form's yuv444ps planes against the plain
    form's (which the parity tests hold within 1e-4 of the FP64 oracle), and
    its spectra against numpy's FP64 FFT of the same tiles with the share of
    threshold decisions that flip."""
    import numpy as np
    import torch
    from libchromadec_gb300 import device as D, synth
    from tests import tc_study as T

    g = D.default_geometry()
    nframes = nfields // 2
    forms = {-1: "plain", D.TC_3XTF32: "tc_3xtf32", D.TC_BF16X3: "tc_bf16x3"}
    out = {name: {} for name in forms.values()}
    out["plain"]["fields_per_s"] = plain_value
    # throughput of the tensor-core forms on the bench workload
    for form in (D.TC_3XTF32, D.TC_BF16X3):
        eng = D.Engine(g, D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_P16))
        eng.set_tc_form(form)
        dout = torch.empty((nframes, 3, eng.out_height, eng.out_width), dtype=torch.int16, device="cuda")
        for _ in range(max(3, a.warmup)):
            eng.decode(dfields, 0, nframes, dout, stream)
        D.tc3d_sync(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps = max(3, a.steps // 4)
        e0.record(stream)
        for _ in range(steps):
            eng.decode(dfields, 0, nframes, dout, stream)
        e1.record(stream)
        D.tc3d_sync(stream)
        ms = e0.elapsed_time(e1) / steps
        out[forms[form]].update({"fields_per_s": nfields / (ms / 1000.0), "ms_per_step": ms})
        del dout, eng
    # chroma PSNR against the true chroma, and planes against the plain form
    cap = synth.make_capture(48, synth.SynthConfig(seed=a.seed, pan_x=1.5, pan_y=0.5), truth=True)
    tf = torch.from_numpy(cap.fields.reshape(48, -1).view(np.int16)).cuda()
    truth = cap.chroma[8:40, 22:310, 177:1125].astype(np.float64)
    peak = float(g.white - g.black)
    frames = {}
    for form, name in forms.items():
        eng = D.Engine(g, D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
        eng.set_tc_form(form)
        ch = torch.empty((32, 288, 948), dtype=torch.float32, device="cuda")
        eng.chroma(tf, 4, 20, ch, stream)
        fr = torch.empty((16, 3, eng.out_height, eng.out_width), dtype=torch.float32, device="cuda")
        eng.decode(tf, 4, 20, fr, stream)
        D.tc3d_sync(stream)
        mse = float(np.mean((ch.cpu().numpy().astype(np.float64) - truth) ** 2))
        out[name]["chroma_psnr_db"] = 10.0 * np.log10(peak * peak / mse)
        frames[form] = fr.cpu().numpy()
    for form in (D.TC_3XTF32, D.TC_BF16X3):
        d = np.abs(frames[form].astype(np.float64) - frames[-1])
        out[forms[form]]["planes_vs_plain_ps"] = {
            pl: {"max": float(d[:, i].max()), "rms": float(np.sqrt(np.mean(d[:, i] ** 2)))}
            for i, pl in enumerate(("Y", "Cb", "Cr"))}
    # spectra against FP64 on a sample of tiles of 4 Z tiles mid-capture
    tx0, ty0, ntx, nty = T.tile_grid(g)
    ntiles = ntx * nty
    fields_np = dfields.cpu().numpy().view(np.uint16).reshape(nfields, g.field_height, g.field_width)
    m0 = min(100, max(0, nframes // 2))
    tiles = np.random.default_rng(a.seed).choice(ntiles, 300, replace=False)
    spec = torch.empty((4, ntiles, 8, 5, 32), dtype=torch.complex64, device="cuda")
    refs = [T.fp64_spectra(fields_np, m0 + i, tiles, g) for i in range(4)]
    for form in (D.TC_3XTF32, D.TC_BF16X3):
        D.tc3d_spectra(dfields, m0, m0 + 4, spec, form, stream=stream)
        D.tc3d_sync(stream)
        S = spec.cpu().numpy()
        rs = [T.report(S[i][tiles], refs[i], 0.4) for i in range(4)]
        out[forms[form]]["spectra_vs_fp64"] = {
            "rms_rel_err": max(r["rms_rel_err"] for r in rs), "max_rel_err": max(r["max_rel_err"] for r in rs),
            "flip_fraction": sum(r["flips"] for r in rs) / sum(r["bins"] for r in rs),
            "bins": sum(r["bins"] for r in rs)}
    out["learned_nn"] = learned_report(a, dfields, nfields, stream)
    out["note"] = ("plain: FP32 CUDA cores with every threshold decision taken exactly (the value above); "
                   "tc_*: tcgen05 split-precision DFT stages (3 MMAs per contraction, FP32 accumulation in "
                   "tensor memory) with FP32 decisions on their spectra; chroma PSNR over fields 8-39 of the "
                   "same seeded content against the encoder's chroma, peak = white - black; learned_nn: the "
                   "per-bin chroma fraction of the trained mask network in place of the threshold, evaluated "
                   "on the whole held-out workload")
    return out


def main():
    a = parse()
    if a.impl == "reference":
        reference_arm(a)
        return
    if a.workload == "batched":
        run_batched(a)
        return
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from libchromadec_gb300 import device as D

    fields_np = make_capture(a)
    nfields = fields_np.shape[0]
    nframes = nfields // 2
    fmt = D.FMT_P16 if a.format == "p16" else D.FMT_PS
    two = a.kind == "2d"
    if two:   # the end-to-end, CPU, forms and batched legs are the 3D metric's
        a.no_e2e = a.no_cpu = a.no_forms = a.no_batched = True
    eng = D.Engine(D.default_geometry(),
                   D.default_config(kind=D.KIND_TRANSFORM_2D if two else D.KIND_TRANSFORM_3D, fmt=fmt))
    tc_form = {"plain": -1, "tc_3xtf32": D.TC_3XTF32, "tc_bf16x3": D.TC_BF16X3, "learned": -1}[a.form]
    if two and (tc_form >= 0 or a.form == "learned"):
        raise SystemExit("the tensor-core and learned forms are Transform 3D only")
    eng.set_tc_form(tc_form)
    if a.form == "learned":
        from libchromadec_gb300 import masknet_train as MT
        learned_net = D.MaskNet(MT.load_weights())
        eng.set_masknet(learned_net)
        a.no_forms = True
    lib = D.lib()
    dfields = torch.from_numpy(fields_np.reshape(nfields, -1).view(np.int16)).cuda()
    out_dtype = torch.int16 if fmt == D.FMT_P16 else torch.float32
    dout = torch.empty((nframes, 3, eng.out_height, eng.out_width), dtype=out_dtype, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- device-resident value
    for _ in range(a.warmup):
        eng.decode(dfields, 0, nframes, dout, stream)
    torch.cuda.synchronize()
    lib.chdg_engine_set_profiling(eng._h, 1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            eng.decode(dfields, 0, nframes, dout, stream)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    import ctypes as C
    mt, md, nl = C.c_double(), C.c_double(), C.c_int64()
    lib.chdg_engine_kernel_times(eng._h, C.byref(mt), C.byref(md), C.byref(nl))
    lib.chdg_engine_set_profiling(eng._h, 0)
    value, s_max = replica_throughput(nfields, a.steps, ms / 1000.0, dist)
    ms_max = 1000.0 * s_max

    # roofline of the dominant kernel (the transform): launches per step
    # one engine batch = 4 launches: the transform walk, the resolve pass,
    # the exact re-walk of the items it lists, the demodulator
    launches_transform = (nl.value // 2 if two else nl.value // (5 if a.form == "learned" else 4)) if tc_form < 0 \
        else a.steps * ((nframes + 255) // 256)
    per_launch_ms = mt.value / max(1, launches_transform)
    fields_per_launch = nfields * a.steps / max(1, launches_transform)
    bytes_per_field = FIELD_BYTES_IN + OUT_BYTES[a.format]
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fp:
            peaks = json.load(fp)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved_gbs = fields_per_launch * bytes_per_field / (per_launch_ms / 1000.0) / 1e9
    # DRAM bytes per field of the transform from the committed ncu summary
    # (a smaller capture of the same kernel; traffic grows with the fields)
    traffic = None
    try:
        if tc_form >= 0 or two:
            raise FileNotFoundError("the committed traffic figure is the plain 3D form's")
        with open(os.path.join(ROOT, "profiles", "tpal3d_traffic_200fields.md")) as fp:
            for ln in fp:
                if ln.startswith("traffic_bytes_per_field:"):
                    traffic = int(ln.split(":")[1]) * fields_per_launch
    except Exception:
        pass
    clocks = clk.summary()
    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    fp32_nominal = sms * 128 * 2 * (clocks["sm_mhz"] or 2070.0) * 1e6 / 1e12
    fp32_meas = fp32_sgemm_peak(local)
    fp32_peak = fp32_meas if fp32_meas else fp32_nominal
    flop_field = FLOP_PER_FIELD_2D_TRANSFORM if two else FLOP_PER_FIELD_3D_TRANSFORM
    tr_tflops = fields_per_launch * flop_field / (per_launch_ms / 1000.0) / 1e12

    line = {
        "metric": METRIC, "value": value, "unit": "fields/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": workload_desc(a), "form": a.form, "fields_per_step": nfields, "frames_per_step": nframes,
                   "format": "yuv444" + a.format, "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "l2": f"inputs {nfields * FIELD_BYTES_IN / 1e6:.0f} MB > 129 MB L2 (no flush)"},
        "roofline": {
            "bound": "fp32", "kernel": ("tpal2d_kernel" if two else "tpal3d transform stage (walk, resolve, exact re-walk)")
            if tc_form < 0 else "tensor-core transform stage (tc3_xy, tc3_zd, tc3_yx)",
            "achieved": tr_tflops, "peak": fp32_peak, "unit": "TFLOP/s", "frac": tr_tflops / fp32_peak,
            "traffic": traffic,
            "peak_source": (f"measured: cuBLAS SGEMM 8192^3 with TF32 off, best of 5 on this GPU ({fp32_meas:.1f}; "
                            f"nominal {sms} SMs x 128 lanes x 2 FLOP x {clocks['sm_mhz'] or 2070.0:.0f} MHz = "
                            f"{fp32_nominal:.1f})") if fp32_meas else
                           f"nominal: {sms} SMs x 128 FP32 lanes x 2 FLOP x the sampled SM clock",
            "algorithmic_flop_per_field": flop_field,
            "per_launch_ms": per_launch_ms, "fields_per_launch": fields_per_launch,
            "demod_ms_per_launch": md.value / max(1, launches_transform),
            "note": ("the transform's convention FLOP count (2.5 N log2 N per real FFT each way, window, "
                     "threshold, overlap-add; 2,257 16x32 tiles per field)") if two else
                    ("the transform's convention FLOP count (2.5 N log2 N per real FFT each way, window, "
                     "threshold, overlap-add; 2,220 distinct tiles per field); the kernel shares the X/Y "
                     "stages across Z tiles, so it executes fewer FLOPs than counted"),
            "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                    "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks
                    else "fallback 6.8 TB/s",
                    "algorithmic_bytes_per_field": bytes_per_field, "traffic": traffic},
        },
        "clocks": clocks,
        "gpu_launches": int(nl.value),
    }

    # ---- end to end through the reference-facing chd_* ABI: the capture is a
    # .tbc + JSON sidecar on the host (page cache), decoded with
    # chd_decode_frames_async; field windows are uploaded and frames
    # downloaded inside the timed region, frames are handed to a callback.
    if not a.no_e2e:
        line["e2e"] = e2e_abi(a, fields_np, rank, barrier, dist)
        # the device-level host entry point (pinned host buffers), for reference
        hfields = torch.from_numpy(fields_np.reshape(nfields, -1).view(np.int16)).pin_memory()
        hout = torch.empty((nframes, 3, eng.out_height, eng.out_width), dtype=out_dtype).pin_memory()
        for _ in range(max(1, a.warmup)):
            rc = lib.chdg_decode_host(eng._h, C.c_void_p(hfields.data_ptr()), hfields[0].numel(), nfields, 0,
                                      nframes, C.c_void_p(hout.data_ptr()), C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError("chdg_decode_host failed")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            lib.chdg_decode_host(eng._h, C.c_void_p(hfields.data_ptr()), hfields[0].numel(), nfields, 0, nframes,
                                 C.c_void_p(hout.data_ptr()), C.c_void_p(stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        line["e2e"]["pinned_buffer_entry_point"] = {
            "value": nfields * a.steps / (e0.elapsed_time(e1) / 1000.0), "unit": "fields/s",
            "path": "chdg_decode_host: pinned host fields -> pinned host frames, one call per step"}

    if rank == 0 and not a.no_forms and a.format == "p16" and tc_form < 0 and not two:
        line["forms"] = forms_report(a, dfields, nfields, value, stream)
    if rank == 0 and not a.no_batched and not two and a.form == "plain":
        line["batched"] = batched_measure(a)
    if rank == 0 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(a, fields_np)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
