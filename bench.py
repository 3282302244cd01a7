"""Benchmark of the multi-tau path: frames/s on the 1024x1024, 10,000-frame
sparse series (Poisson speckle, mean 0.005 photons/pixel/frame, tau_c
log-uniform [5,500] per ring, 36/18 rings, 8 delays per level).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--width W --frames F]   (reduced series, for profiling)

One JSON line on rank 0.  `value`: frames/s of one step with the raw frames
resident in HBM (filter/transpose + multi-tau + normalisation, CUDA events on
the library's stream).  `e2e`: the same step through the C ABI from pinned
host frames, host-to-device copies and the g2/stderr readback inside the
timed region (wall clock).  Every step reads/writes > 1 GB, far above L2.
`--impl reference` times the CPU restatement of the reference's path (the
oracle port; the reference's own sources are not present where the GPU runs)
on the same whole series, every step.

Multi-GPU: each rank runs an independent replica of the series (the path has
no cross-series exchange); value = frames of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import collections
import json
import os
import shutil
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT / "xpcs-eigen_gb300")]

import xpcs_synth as xs  # noqa: E402

WORKLOAD = "c1"
WORKLOAD_DESC = ("1024x1024 detector, 10000 sparse IMM frames (uint16 counts), Poisson speckle "
                 "mean 0.005 photons/pixel/frame, tau_c log-uniform [5,500] per dynamic ring, "
                 "36 static / 18 dynamic rings, 5% masked pixels, 8 delays per level")


def workload_desc(acq) -> str:
    if (acq.width, acq.height, acq.frames, acq.mean) == (1024, 1024, 10000, 0.005):
        return WORKLOAD_DESC
    return (f"{acq.width}x{acq.height} detector, {acq.frames} sparse IMM frames, mean "
            f"{acq.mean:g} photons/pixel/frame, otherwise as the 1024x1024 10000-frame series "
            "(a reduced case for profiling)")


def bench_config(acq, delays: int, qbins: int, raw_events: int, world: int) -> dict:
    """The `config` object of both arms: the workload and what the timed step
    reads, identical for the GPU arm and the reference arm."""
    return {"workload": workload_desc(acq), "detector": f"{acq.width}x{acq.height}",
            "frames": acq.frames, "delays": delays, "qbins": qbins, "raw_events": raw_events,
            "mode": "reference",
            "l2": (f"no flush: every step reads {raw_events * 6 >> 20} MB of raw events, "
                   "above the 126 MB L2"),
            "parallelism": f"replicas x{world}"}


def rank_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Dist:
    """Barrier and max-over-ranks for replica runs (gloo on the host)."""

    def __init__(self):
        self.rank, self.world, self.local = rank_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        smi = shutil.which("nvidia-smi")
        if not smi:
            return
        self.proc = subprocess.Popen(
            [smi, "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
             "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        t0 = time.perf_counter()  # nvidia-smi takes a moment to print its first sample
        while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_series_data(name=WORKLOAD, width=None, frames=None, mean=None):
    over = {}
    if width:
        over.update(width=width, height=width)
    if frames:
        over["frames"] = frames
    if mean:
        over["mean"] = mean
    acq = xs.preset(name, **over)
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    return acq, dq, sq, nnz, idx, val


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------- CPU (oracle)

def cpu_pipeline(acq, dq, sq, nnz, idx, val, frames, threads=0):
    """The reference's path restated in C (oracle): SparseFilter (serial),
    multiTau2 (OpenMP over pixels), normalizeG2s (serial) on the first
    `frames` frames.  Returns wall seconds."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    off = int(np.sum(nnz[:frames], dtype=np.int64))
    qm = oracle.QMap(dq, sq)
    t0 = time.perf_counter()
    rows, _ = oracle.sparse_filter(qm, nnz[:frames], idx[:off], val[:off], frames)
    G2, IP, IF = oracle.multitau2(rows, frames, acq.dpl, 0, threads)
    oracle.normalize_f32(qm, G2, IP, IF)
    return time.perf_counter() - t0


def cpu_cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def run_reference_arm(args, dist):
    """The reference's CPU path (the oracle restatement of SparseFilter::Apply,
    Corr::multiTau2 and Corr::normalizeG2s) on the whole series the GPU arm
    runs: every step is the full --frames series, filter and normalisation
    serial as in the reference, multi-tau OpenMP over every host thread."""
    if dist.rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    acq, dq, sq, nnz, idx, val = make_series_data(width=args.width, frames=args.frames, mean=args.mean)
    qm = oracle.QMap(dq, sq)
    lv, _ = oracle.delays(acq.frames, acq.dpl)
    for _ in range(args.warmup):
        cpu_pipeline(acq, dq, sq, nnz, idx, val, acq.frames)
    times = [cpu_pipeline(acq, dq, sq, nnz, idx, val, acq.frames) for _ in range(args.steps)]
    t = sum(times) / len(times)
    v = acq.frames / t
    sample = (f"the whole {acq.frames}-frame {acq.width}x{acq.height} series every step "
              "(no sampling); sparse filter and normalisation serial, multi-tau OpenMP over "
              "all host threads")
    print(json.dumps({
        "impl": "reference", "metric": "multitau_frames_per_s", "value": v, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": bench_config(acq, int(lv.size), int(qm.nq), int(idx.size), dist.world),
        "cpu_baseline": {"value": v, "unit": "frames/s", "cores": cpu_cores(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ------------------------------------------------------------------- GPU

def algorithmic_bytes(P, D, Q, npix, raw_events, events):
    """Compulsory bytes per launch of each stage: K-a reads 6 B per raw event and writes
    8 B per event + 12 B per pixel of offsets; K-c reads the lists and writes 12 B per
    (pixel, delay); K-d reads 12 B per (mapped pixel, delay) and writes 24 B per (q, delay)."""
    ka = 6 * raw_events + 8 * events + 12 * P          # read idx+val, write lists + offsets
    kc = 8 * events + 12 * P + 12 * D * P              # read lists + offsets, write G2/IP/IF
    kd = 12 * D * npix + 24 * D * Q                    # read G2/IP/IF of mapped pixels, write g2/se
    return ka, kc, kd


BATCH_DESC = ("64 independent sparse series: square detector side log-uniform [256, 1024], "
              "frames log-uniform [500, 20000], mean photons/pixel/frame log-uniform "
              "[0.1 %, 5 %], tau_c log-uniform [2, 2000] per ring, 4 or 8 delays per level, "
              "9-36 dynamic rings (2 static per dynamic), seed 2026")


def batch_mix(n=64, seed=2026):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(np.exp(rng.uniform(np.log(256), np.log(1024))))
        frames = int(np.exp(rng.uniform(np.log(500), np.log(20000))))
        mean = float(np.exp(rng.uniform(np.log(0.001), np.log(0.05))))
        dpl = int(rng.choice([4, 8]))
        q = int(rng.integers(9, 37))
        out.append(xs.Acquisition(width=side, height=side, frames=frames, n_static=2 * q,
                                  n_dynamic=q, mean=mean, tau_min=2.0, tau_max=2000.0,
                                  seed=seed + 1 + i, dpl=dpl))
    return out


def run_batch(args, dev):
    """Batched vs plain per-series throughput on the 64-series mix: the same
    series, resident in HBM, run one after another through the per-series
    calls (xpcs_multitau + xpcs_normalize, each waited for) and as one batch
    graph (xpcs_batch_run, autotuned: members' knobs, the graph's form -- work
    queue or chains -- and its chain count).  Every series is autotuned first
    (xpcs_autotune), and both paths run once untimed to size their buffers.
    The batch form the autotuner did not keep is timed too."""
    import xpcs_gpu as xg

    mix = batch_mix(args.batch_series)
    series, events = [], 0
    for acq in mix:
        dq, sq, _, _ = xs.maps(acq)
        d = xs.DeviceFrames(acq)
        s = xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, device=dev)
        s.ingest_sparse_device(d.nnz, d.idx, d.val)
        s.synchronize()
        d.close()
        events += d.events
        series.append(s)
    outs = [(np.empty((s.D, s.nq)), np.empty((s.D, s.nq)), None, None) for s in series]
    caps = [s.autotune(xg.MODE_REFERENCE) for s in series]  # both forms use the tuned kernels

    def plain():
        for s, o in zip(series, outs):
            s.multitau(xg.MODE_REFERENCE)
            s.normalize(out=o)

    plain()
    t0 = time.perf_counter()
    for _ in range(args.batch_reps):
        plain()
    t_plain = (time.perf_counter() - t0) / args.batch_reps
    # per-series device time of the plain path (one more pass, each series waited for)
    per = []
    for a, s_ in zip(mix, series):
        s_.multitau(xg.MODE_REFERENCE)
        s_.normalize(out=(np.empty((s_.D, s_.nq)), np.empty((s_.D, s_.nq)), None, None))
        st = s_.stage_times()
        per.append({"side": a.width, "frames": a.frames, "events": int(s_.info().raw_events),
                    "filter_ms": st["filter_ms"], "multitau_ms": st["multitau_ms"],
                    "normalize_ms": st["normalize_ms"], "step_ms": st["step_ms"]})
    b = xg.Batch(series)
    b.run(xg.MODE_REFERENCE, f64=True, autotune=True)  # tunes the chain count, captures
    t0 = time.perf_counter()
    dev_ms = []
    for _ in range(args.batch_reps):
        b.run(xg.MODE_REFERENCE, f64=True, autotune=True)
        dev_ms.append(b.stats()[0])
    t_batch = (time.perf_counter() - t0) / args.batch_reps
    _, kernels, lanes = b.stats()
    start, end = b.timeline()
    queue, _ = b.form()
    # the other form, its chain count tuned, for comparison
    b.set_form(not queue)
    b.run(xg.MODE_REFERENCE, f64=True, autotune=True)
    other_ms = []
    for _ in range(args.batch_reps):
        b.run(xg.MODE_REFERENCE, f64=True, autotune=True)
        other_ms.append(b.stats()[0])
    other_chains = b.form()[1]
    forms = {("work_queue" if queue else "chains"):
             {"device_ms": statistics.median(dev_ms), "chains": int(lanes)},
             ("chains" if queue else "work_queue"):
             {"device_ms": statistics.median(other_ms), "chains": int(other_chains)}}
    # the batch's results are those of the plain run
    same = all(np.array_equal(s.normalized(f64=True)[0], o[0], equal_nan=True)
               for s, o in zip(series, outs))
    b.close()
    for s in series:
        s.close()
    n = len(mix)
    busy = float(np.sum(end - start))
    makespan = float(np.max(end)) if n else 0.0
    order = np.argsort([-p["step_ms"] for p in per])
    plain_dev = float(sum(p["step_ms"] for p in per))
    top4 = float(sum(per[i]["step_ms"] for i in order[:4]))
    timeline = [{"series": int(i), "side": per[i]["side"], "frames": per[i]["frames"],
                 "events": per[i]["events"], "plain_step_ms": per[i]["step_ms"],
                 "batch_start_ms": float(start[i]), "batch_end_ms": float(end[i])}
                for i in range(n)]
    return {"workload": BATCH_DESC, "series": n, "raw_events": int(events),
            "pixel_frames": int(sum(a.width * a.height * a.frames for a in mix)),
            "plain_ms": t_plain * 1e3, "batched_ms": t_batch * 1e3,
            "batched_device_ms": statistics.median(dev_ms),
            "plain_series_per_s": n / t_plain, "batched_series_per_s": n / t_batch,
            "batched_over_plain": t_plain / t_batch, "kernels_in_graph": int(kernels),
            "concurrent_chains": int(lanes),
            "form": "work_queue" if queue else "chains", "forms": forms,
            "thread_caps": {str(c): caps.count(c) for c in sorted(set(caps))},
            "identical_results": bool(same), "reps": args.batch_reps,
            "plain_device_ms_sum": plain_dev,
            "plain_device_ms_largest_4": top4,
            "plain_stage_ms_sum": {k: float(sum(p[k] for p in per))
                                   for k in ("filter_ms", "multitau_ms", "normalize_ms")},
            "batch_timeline": {"makespan_ms": makespan, "series_busy_ms_sum": busy,
                               "mean_series_in_flight": busy / makespan if makespan else None,
                               "per_series": timeline}}


def run_serving(args, dev):
    """Streaming: 16 concurrent 1024x1024 sparse acquisitions at 200 Hz each
    with staggered starts, pushed frame by frame into one xpcs_server as the
    frames fall due (one feeder thread replays the merged arrival schedule).
    The server transposes every acquisition's frames in blocks of 512 as they
    arrive into pixel-major rows resident in HBM; each acquisition is finished
    after its last frame and its g2 read back.  Reports frames/s, the
    per-frame ingest latency and the time to final g2 (last frame's arrival
    to the end of its normalisation)."""
    import xpcs_gpu as xg

    rng = np.random.default_rng(4242)
    n = args.serve_streams
    lengths = [int(round(L * args.serve_length_scale))
               for L in rng.choice([2000, 5000, 20000], size=n)]
    acqs, data = [], []
    for i, F in enumerate(lengths):
        acq = xs.Acquisition(width=1024, height=1024, frames=F, n_static=36, n_dynamic=18,
                             mean=0.01, tau_min=5.0, tau_max=1000.0, seed=5000 + i, dpl=8)
        dq, sq, _, _ = xs.maps(acq)
        d = xs.DeviceFrames(acq)
        nnz, idx, val = d.to_host()
        d.close()
        off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
        acqs.append((acq, dq, sq))
        data.append((nnz, idx, val, off))
    starts = [i * args.serve_stagger for i in range(n)]
    sched = sorted((starts[i] + k / args.serve_hz, i, k)
                   for i in range(n) for k in range(lengths[i]))
    budget = int(args.serve_budget_gb * (1 << 30))
    with xg.Server(memory_budget=budget, device=dev) as srv:
        ids = []
        for (acq, dq, sq), (nnz, idx, _, _) in zip(acqs, data):
            ids.append(srv.submit(acq.width, acq.height, acq.frames, acq.dpl, dq, sq,
                                  expected_events=idx.size))
        t0 = time.perf_counter()
        for t, i, k in sched:
            dt = t0 + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            nnz, idx, val, off = data[i]
            srv.push(ids[i], nnz[k:k + 1], idx[off[k]:off[k + 1]], val[off[k]:off[k + 1]])
            if k == lengths[i] - 1:
                srv.finish(ids[i])
        for i in ids:
            srv.result(i)
        wall = time.perf_counter() - t0
        st = srv.stats()
        for i in ids:
            srv.release(i)
    frames = int(sum(lengths))
    return {"workload": (f"{n} concurrent 1024x1024 sparse acquisitions at {args.serve_hz:g} Hz "
                         f"each, mean 0.01 photons/pixel/frame, tau_c log-uniform [5, 1000], "
                         f"lengths drawn from 2000/5000/20000 frames x {args.serve_length_scale:g}, "
                         f"starts {args.serve_stagger:g} s apart, seed 4242; frames transposed "
                         "into resident pixel-major rows in blocks of 512 as they arrive"),
            "lengths": lengths, "length_scale": args.serve_length_scale,
            "streams": n, "frames": frames, "events": int(sum(d[1].size for d in data)),
            "wall_s": wall, "frames_per_s": frames / wall,
            "ingest_p50_ms": st["ingest_p50_ms"], "ingest_p99_ms": st["ingest_p99_ms"],
            "ingest_max_ms": st["ingest_max_ms"],
            "time_to_final_g2_p50_ms": st["final_p50_ms"],
            "time_to_final_g2_p99_ms": st["final_p99_ms"],
            "peak_active": st["peak_active"], "memory_budget_gb": args.serve_budget_gb,
            "peak_footprint_gb": st["peak_used_bytes"] / (1 << 30)}


def run_twotime_bench(args, dev):
    """Two-time on 8 series of 512x512 x 4096 sparse frames (the batch mix's
    two-time option): the EXACT mode (integer Gram of the counts on the tensor
    cores, float64 smoothing) on every series, and the REFERENCE mode (float32
    in the reference's order on CUDA cores) on the first, with the largest
    relative difference between the two.  Symmetric smoothing, all 9 q rings.
    Times are of the computation (xpcs_twotime, results left on the device);
    the 9 x 4096^2 float32 matrices are read back separately for the check."""
    import xpcs_gpu as xg

    rng = np.random.default_rng(777)
    n = args.twotime_series
    exact_ms, gram_ms, gram_flop, gram_alg, ref_ms, dev_rel = [], 0.0, 0.0, 0.0, None, None
    for i in range(n):
        mean = float(np.exp(rng.uniform(np.log(0.001), np.log(0.05))))
        acq = xs.Acquisition(width=512, height=512, frames=args.twotime_frames, n_static=18,
                             n_dynamic=9, mean=mean, tau_min=2.0, tau_max=2000.0,
                             seed=9000 + i, dpl=4)
        dq, sq, _, _ = xs.maps(acq)
        d = xs.DeviceFrames(acq)
        with xg.Series(acq.width, acq.height, acq.frames, 4, dq, sq, device=dev) as s:
            s.ingest_sparse_device(d.nnz, d.idx, d.val)
            s.synchronize()
            d.close()
            qs = list(range(1, 10))
            s.twotime(qs, mode=xg.MODE_EXACT, window=8, fetch=False)  # sizes buffers
            t0 = time.perf_counter()
            r = s.twotime(qs, mode=xg.MODE_EXACT, window=8, fetch=False)
            exact_ms.append((time.perf_counter() - t0) * 1e3)
            gram_ms += r["gram_ms"]
            gram_flop += r["gram_flop"]
            gram_alg += r["gram_flop_algorithmic"]
            if i == 0:
                r = s.twotime(qs, mode=xg.MODE_EXACT, window=8)
                t0 = time.perf_counter()
                ref = s.twotime(qs, mode=xg.MODE_REFERENCE, window=8, fetch=False)
                ref_ms = (time.perf_counter() - t0) * 1e3
                ref = s.twotime(qs, mode=xg.MODE_REFERENCE, window=8)
                dev_rel = max(float(np.max(np.abs(r["c2t"][q].astype(np.float64) - ref["c2t"][q]))
                                    / max(float(np.max(np.abs(ref["c2t"][q]))), 1e-30))
                              for q in ref["c2t"])
    peak = 1916.2
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peak = float(json.loads(pk.read_text()).get("bf16_tflops", peak))
    # the roofline counts the Gram's own work (the upper triangle, no tile or K
    # padding); the rate of every multiply-add the tensor cores ran is beside it
    achieved = gram_alg / (gram_ms * 1e-3) / 1e12 if gram_ms > 0 else None
    computed = gram_flop / (gram_ms * 1e-3) / 1e12 if gram_ms > 0 else None
    return {"workload": (f"{n} sparse series, 512x512 x {args.twotime_frames} frames, mean "
                         "photons/pixel/frame log-uniform [0.1 %, 5 %], tau_c log-uniform "
                         "[2, 2000], 18 static / 9 dynamic rings, all 9 q rings, symmetric "
                         "smoothing, window 8, seed 777"),
            "series": n, "exact_ms_per_series": statistics.median(exact_ms),
            "reference_order_ms_one_series": ref_ms,
            "exact_vs_reference_order_max_rel": dev_rel,
            "gram_roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                              "peak_kind": "measured bf16 dense (fp16 runs at the same rate)",
                              "unit": "TFLOP/s",
                              "frac": achieved / peak if achieved else None,
                              "flop": gram_alg,
                              "flop_note": "2 x rows x F(F+1)/2 per smoothing group: the "
                                           "upper triangle, diagonal included",
                              "computed_tile_flop": gram_flop,
                              "computed_tile_tflops": computed,
                              "kernel_ms": gram_ms}}


def run_corr(args, acq, dq, sq, nnz, idx, val):
    """The drop-in `corr` driver on the same series: the IMM file and the
    analysis container are written to a scratch directory, and `corr` reads
    them, runs the GPU path and writes its datasets back (wall time of the
    process, including CUDA start-up and file I/O)."""
    import tempfile
    sys.path.insert(0, str(ROOT / "tests"))
    import refio  # the IMM / XH5C writers of the driver's tests
    from build import build_corr

    corr = build_corr()
    with tempfile.TemporaryDirectory() as wd:
        wd = Path(wd)
        imm = wd / "series.imm"
        refio.write_imm_sparse(imm, acq.height, acq.width, nnz, idx, val)
        cfg = refio.config_entries(acq.width, acq.height, dq, sq, imm, first=1, last=acq.frames,
                                   dpl=acq.dpl)
        path = wd / "analysis.h5"
        walls, log = [], ""
        for _ in range(2):
            refio.write_xh5c(path, cfg)
            t0 = time.perf_counter()
            r = subprocess.run([str(corr), str(path)], capture_output=True, text=True, cwd=wd)
            walls.append(time.perf_counter() - t0)
            if r.returncode != 0:
                return {"error": r.stderr.strip()[-300:]}
            log = r.stdout
    stages = {}
    for ln in log.splitlines():
        for key, label in (("load_ms", "Loading data took"), ("multitau_ms", "Computing G2 MultiTau took"),
                           ("normalize_ms", "Normalizing Data took"), ("total_ms", "Total took")):
            if label in ln:
                stages[key] = float(ln.split(label)[1].split()[0])
    return {"workload": "the same series through the corr driver: IMM file + analysis container "
                        "in, norm-0-g2 / norm-0-stderr (float32, bit-identical) and the side "
                        "datasets written back",
            "wall_s": min(walls), "stages_ms": stages}


def run_normalize(args, dev):
    """The headline series' normalisation on its own: the float64 result the
    bench step reports, and the float32 replay of the reference's own
    arithmetic that `corr` writes (norm-0-g2 / norm-0-stderr, bit-identical),
    each the median of 4 timed runs after one untimed."""
    import xpcs_gpu as xg

    acq, dq, sq, nnz, idx, val = make_series_data(width=args.width, frames=args.frames,
                                                  mean=args.mean)
    s = xg.Series(acq.width, acq.height, acq.frames, acq.dpl, dq, sq, device=dev)
    s.ingest_sparse(nnz, idx, val)
    s.multitau(xg.MODE_REFERENCE)
    res = {"workload": f"{acq.width}x{acq.height} x {acq.frames} frames, D = {s.D}, "
                       f"{s.nq} q rings"}
    for key, f64, f32 in (("f64_ms", True, False), ("f32_replay_ms", False, True)):
        ts = []
        for _ in range(5):
            s.normalize(f64=f64, f32=f32)
            s.synchronize()
            ts.append(s.stage_times()["normalize_ms"])
        res[key] = statistics.median(ts[1:])
    s.close()
    return res


def run_dense(args, dev):
    """Dense CCD series: 960x960 x 20,000 int16 frames after 100 dark frames
    (dark ~ N(100, 8^2), read noise 4 ADU, 35 ADU/photon on the speckle
    process at 0.02 photons/pixel/frame, gain U[0.9, 1.1], 3-sigma threshold),
    frames resident in HBM.  A step = dark-subtract/threshold/flatfield and
    compaction of every frame (K-b), transpose, multi-tau, FP64 normalisation."""
    import xpcs_gpu as xg

    acq = xs.preset("c2", frames=args.dense_frames)
    dq, sq, flat, _ = xs.maps(acq)
    F, P, nd = acq.frames, acq.width * acq.height, acq.dark_frames
    frames = xs.DeviceDenseFrames(acq)
    darks = frames.to_host(0, nd)
    s = xg.Series(acq.width, acq.height, F, acq.dpl, dq, sq, flatfield=flat, device=dev,
                  dense=True, lld=acq.lld, sigma=acq.sigma)
    s.set_dark(darks)
    D, Q = s.D, s.nq
    out = (np.empty((D, Q), np.float64), np.empty((D, Q), np.float64), None, None)

    def step():
        s.reset()
        s.ingest_dense_device(frames.frame_ptr(nd), F)
        s.multitau(xg.MODE_REFERENCE)
        s.normalize(out=out)
        s.synchronize()

    for _ in range(2):
        step()
    walls, stages = [], []
    for _ in range(args.dense_steps):
        t0 = time.perf_counter()
        step()
        walls.append((time.perf_counter() - t0) * 1e3)
        stages.append(s.stage_times())
    info = s.info()
    frames.close()
    s.close()
    med = {k: statistics.median(st[k] for st in stages)
           for k in ("h2d_ms", "filter_ms", "multitau_int_ms", "multitau_float_ms",
                     "normalize_ms")}
    wall = statistics.median(walls)
    raw_bytes = 2 * P * F
    peak, peak_kind = peaks()
    kb_gbs = raw_bytes / (med["h2d_ms"] * 1e-3) / 1e9 if med["h2d_ms"] > 0 else None
    return {"workload": (f"{acq.width}x{acq.height} x {F} dense int16 frames after {nd} darks, "
                         "dark N(100, 8^2), read noise 4 ADU, 35 ADU/photon at 0.02 "
                         "photons/pixel/frame, gain U[0.9, 1.1], lld 0, 3 sigma, 36/18 rings, "
                         "dpl 8, frames resident in HBM"),
            "frames_per_s": F / (wall * 1e-3), "ms_per_step": wall,
            "stages_ms": {"dense_filter": med["h2d_ms"], "filter_transpose": med["filter_ms"],
                          "multitau_int": med["multitau_int_ms"],
                          "multitau_float": med["multitau_float_ms"],
                          "normalize": med["normalize_ms"]},
            "events": int(info.events), "float_path_pixels": int(info.float_path_pixels),
            "delays": D,
            "dense_filter_roofline": {"bound": "hbm", "achieved": kb_gbs, "peak": peak,
                                      "peak_kind": peak_kind, "unit": "GB/s",
                                      "frac": kb_gbs / peak if kb_gbs else None,
                                      "algorithmic_bytes": raw_bytes,
                                      "note": "2 B/pixel/frame read; event writes not counted"}}


def run_gpu_arm(args, dist):
    import xpcs_gpu as xg

    dev = dist.local
    acq, dq, sq, nnz, idx, val = make_series_data(width=args.width, frames=args.frames, mean=args.mean)
    F, P = acq.frames, acq.width * acq.height
    xg.pin(idx)
    xg.pin(val)
    s = xg.Series(acq.width, acq.height, F, acq.dpl, dq, sq, device=dev)
    info0 = s.info()
    D, Q = s.D, s.nq
    shp = (D, Q)
    # the reported result: float64 g2 and stderr; the float32 replay of the
    # reference's own arithmetic is timed separately below
    out = (np.empty(shp, np.float64), np.empty(shp, np.float64), None, None)

    def e2e_step():
        s.reset()
        s.ingest_sparse(nnz, idx, val)
        s.multitau(xg.MODE_REFERENCE)
        s.normalize(out=out)

    # end to end, H series handles in turn: the frame copy of step k (copy
    # engine, NVLink-C2C) runs while steps k-H+1 .. k-1 compute; every step
    # still copies its frames in, computes and reads its g2/stderr back
    H = max(2, args.e2e_handles)
    hs = [(s, out)] + [(xg.Series(acq.width, acq.height, F, acq.dpl, dq, sq, device=dev),
                        (np.empty(shp, np.float64), np.empty(shp, np.float64), None, None))
                       for _ in range(H - 1)]

    def e2e_run(steps):
        pend = collections.deque()
        for k in range(steps):
            cur, o = hs[k % H]
            cur.reset()
            cur.ingest_sparse(nnz, idx, val)
            cur.multitau(xg.MODE_REFERENCE)
            pend.append((cur, o))
            if len(pend) == H:  # step k-H+1: its handle is reused next
                h, ho = pend.popleft()
                h.normalize(out=ho)
        while pend:
            h, ho = pend.popleft()
            h.normalize(out=ho)

    # warm-up: full end-to-end steps
    for _ in range(args.warmup):
        e2e_step()
    e2e_run(2)
    info = s.info()

    clocks = ClockSampler(dev)
    clocks.start()
    # value: raw frames resident in HBM; each step = filter/transpose + multitau + normalize
    dist.barrier()
    s.synchronize()
    dev_ms, stages, launches = [], [], 0
    for _ in range(args.steps):
        s.multitau(xg.MODE_REFERENCE)
        s.normalize(out=out)
        st = s.stage_times()
        dev_ms.append(st["step_ms"])
        stages.append(st)
        launches += st["launches"]
    s.synchronize()
    dist.barrier()
    t_dev = dist.max(sum(dev_ms) / 1e3)
    # e2e: pinned host frames -> device, compute, g2/stderr back
    dist.barrier()
    t0 = time.perf_counter()
    e2e_run(args.steps)
    for h, _ in hs:
        h.synchronize()
    t_e2e = dist.max(time.perf_counter() - t0)
    dist.barrier()
    clk = clocks.stop()

    world = dist.world
    value = world * F * args.steps / t_dev
    e2e_value = world * F * args.steps / t_e2e
    med = {k: statistics.median(st[k] for st in stages)
           for k in ("filter_ms", "multitau_int_ms", "multitau_float_ms", "multitau_ms",
                     "normalize_ms", "step_ms")}
    npix = int(np.count_nonzero((dq.ravel() >= 1) & (sq.ravel() >= 1)))
    ka, kc, kd = algorithmic_bytes(P, D, Q, npix, int(info.raw_events), int(info.events))
    peak, peak_kind = peaks()
    cand = {"multitau": (kc, med["multitau_int_ms"]), "filter_transpose": (ka, med["filter_ms"]),
            "normalize": (kd, med["normalize_ms"])}
    top = max(cand, key=lambda k: cand[k][1])
    gbs = {k: b / (ms * 1e-3) / 1e9 if ms > 0 else None for k, (b, ms) in cand.items()}
    achieved = gbs[top]
    traffic = None
    tp = ROOT / "profiles" / "traffic.txt"  # ncu DRAM bytes per launch at the 1024x1024 series
    if tp.exists() and (acq.width, acq.height, F) == (1024, 1024, 10000):
        for ln in tp.read_text().splitlines():
            parts = ln.split()
            if len(parts) == 2 and not ln.startswith("#") and parts[0] == top:
                traffic = int(parts[1])

    # the instruction-issue roofline of the same kernel: warp instructions of one launch (ncu,
    # committed) over its CUDA-event time, against 4 issue slots per SM per cycle
    issue = None
    ip = ROOT / "profiles" / "instructions.txt"
    if ip.exists() and (acq.width, acq.height, F, acq.mean) == (1024, 1024, 10000, 0.005):
        for ln in ip.read_text().splitlines():
            parts = ln.split()
            if len(parts) == 2 and not ln.startswith("#") and parts[0] == top:
                n_inst = int(parts[1])
                mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
                sms = xg.device_sm_count(dev)
                if mhz and sms and cand[top][1] > 0:
                    ach = n_inst / (cand[top][1] * 1e-3)
                    pk = sms * 4 * mhz * 1e6
                    issue = {"warp_instructions": n_inst,
                             "warp_instructions_per_event": n_inst / max(int(info.events), 1),
                             "achieved": ach, "peak": pk, "unit": "warp instructions/s",
                             "frac": ach / pk,
                             "peak_note": f"{sms} SMs x 4 schedulers x {mhz:g} MHz (median "
                                          "SM clock during the timed region)"}
    h2d = int(idx.nbytes + val.nbytes + 8 * (F + 1))
    d2h = int(sum(a.nbytes for a in out if a is not None))
    s.multitau(xg.MODE_REFERENCE)
    s.normalize(f64=False, f32=True)
    f32_ms = s.stage_times()["normalize_ms"]
    result = {
        "metric": "multitau_frames_per_s", "value": value, "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/f32 (bit-exact multi-tau), f64 normalisation",
        "data": "synthetic",
        "config": bench_config(acq, D, Q, int(info.raw_events), world),
        "series": {"events": int(info.events), "float_path_pixels": int(info.float_path_pixels),
                   "g2ipif_written": True},
        "pixel_frames_per_s": value * P,
        "stages_ms": med,
        "normalize_f32_replay_ms": f32_ms,
        "stage_gbs": gbs,
        "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e / args.steps * 1e3,
                "pipelining": f"{H} series handles in turn: the H2D copy of step k overlaps "
                              "the compute of the steps before it (H2D is ~180 GB/s over "
                              "NVLink-C2C)"},
        "roofline": {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None,
                     "algorithmic_bytes": cand[top][0], "traffic": traffic,
                     "issue": issue},
        "clocks": clk,
        "gpu_launches": launches,
    }
    if not args.no_batch:
        result["batch"] = run_batch(args, dev)
    if not args.no_serving:
        result["serving"] = run_serving(args, dev)
    if not args.no_twotime:
        result["twotime"] = run_twotime_bench(args, dev)
    if not args.no_dense:
        result["dense"] = run_dense(args, dev)
    if not args.no_corr and dist.rank == 0:
        result["corr"] = run_corr(args, acq, dq, sq, nnz, idx, val)
    if dist.rank == 0 and world == 1 and not args.no_cpu_baseline:
        t_cpu = cpu_pipeline(acq, dq, sq, nnz, idx, val, F)
        result["cpu_baseline"] = {
            "value": F / t_cpu, "unit": "frames/s", "cores": cpu_cores(), "kind": "port",
            "sample": f"the whole {F}-frame {acq.width}x{acq.height} series, once (oracle "
                      "restatement of SparseFilter + multiTau2 + normalizeG2s)"}
    for h, _ in hs:
        h.close()
    xg.unpin(idx)
    xg.unpin(val)
    if dist.rank == 0:
        print(json.dumps(result))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-series batch measure")
    ap.add_argument("--no-serving", action="store_true", help="skip the streaming measure")
    ap.add_argument("--no-twotime", action="store_true", help="skip the two-time measure")
    ap.add_argument("--twotime-series", type=int, default=8)
    ap.add_argument("--twotime-frames", type=int, default=4096)
    ap.add_argument("--no-dense", action="store_true", help="skip the dense-frame measure")
    ap.add_argument("--no-corr", action="store_true", help="skip the corr driver measure")
    ap.add_argument("--dense-frames", type=int, default=20000)
    ap.add_argument("--dense-steps", type=int, default=3)
    ap.add_argument("--dense-only", action="store_true",
                    help="run only the dense-frame measure and print its object (profiling)")
    ap.add_argument("--only", choices=["batch", "serving", "twotime", "dense", "normalize"],
                    default=None,
                    help="run only this measure and print its object (profiling)")
    ap.add_argument("--e2e-handles", type=int, default=2,
                    help="series handles in flight in the end-to-end measure (at least 2)")
    ap.add_argument("--serve-streams", type=int, default=16)
    ap.add_argument("--serve-hz", type=float, default=200.0)
    ap.add_argument("--serve-stagger", type=float, default=0.2, help="seconds between starts")
    ap.add_argument("--serve-length-scale", type=float, default=1.0,
                    help="scale of the 2000/5000/20000-frame lengths (1.0: the full lengths, "
                         "about 100 s of streaming)")
    ap.add_argument("--serve-budget-gb", type=float, default=128.0)
    ap.add_argument("--batch-series", type=int, default=64)
    ap.add_argument("--batch-reps", type=int, default=3)
    ap.add_argument("--width", type=int, default=None,
                    help="square detector side (reduced case for profiling; default 1024)")
    ap.add_argument("--frames", type=int, default=None,
                    help="frames in the series (reduced case for profiling; default 10000)")
    ap.add_argument("--mean", type=float, default=None,
                    help="photons per pixel per frame (profiling case; default 0.005)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference_arm(args, dist)
        elif args.dense_only or args.only:
            fn = {"batch": run_batch, "serving": run_serving, "twotime": run_twotime_bench,
                  "dense": run_dense, "normalize": run_normalize}[args.only or "dense"]
            r = fn(args, dist.local)
            if dist.rank == 0:
                print(json.dumps(r))
        else:
            run_gpu_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
