"""Benchmark: EM session-iterations/s of DBN on 20M synthetic sessions.

Workload (one "step" = one EM iteration over all training sessions):
  20,000,000 sessions over 1,000,000 queries (Zipf s = 1.0), 50-doc pools,
  top-10 shown, clicks from a ground-truth CCM (tau = 0.6, 0.3, 0.2,
  relevance ~ Beta(1, 3)); test share 0.2 -> 16,000,000 training sessions;
  a DBN is fitted.  Inputs are seeded synthetic sessions of that shape (the
  reference measured on the Yandex click log, which is not available here).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl ours` (default) prints one JSON line with the fused GPU throughput
(`value`), the kernel's HBM roofline, the plain two-kernel GPU EM and the CPU
baseline beside it, and an end-to-end number through the C-ABI with host
buffers.  `--impl reference` times the reference's CPU training path (its
restatement in oracle/, FP32, all host threads) on a bounded sample of the
same workload.  Under torchrun (N > 1) every rank fits its own replica of the
workload (weak scaling, no collective on the data path); rank 0 prints.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "EM session-iterations/s (20M sessions, DBN)"
MODELS = {"pbm": 0, "ccm": 1, "dbn": 2, "ubm": 3}


def metric_for(model: str) -> str:
    """The headline metric for DBN; the same measurement for the other models."""
    return METRIC if model == "dbn" else METRIC.replace("DBN", model.upper())
UNIT = "session-iterations/s"
def _count(n: int) -> str:
    return f"{n / 1e6:g}M" if n >= 1_000_000 else f"{n:,}"


def data_text(args) -> str:
    return (f"synthetic: {_count(args.sessions)} sessions, {_count(args.queries)} queries Zipf(1.0), 50-doc pools, "
            "top-10 shown, ground-truth CCM clicks (tau 0.6/0.3/0.2, relevance Beta(1,3)), seeded; test share 0.2")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--sessions", type=int, default=20_000_000)
    ap.add_argument("--queries", type=int, default=1_000_000)
    ap.add_argument("--cpu-sample", type=int, default=1_000_000,
                    help="training sessions in the CPU baseline's bounded sample")
    ap.add_argument("--e2e-iters", type=int, default=50)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-models", action="store_true",
                    help="skip timing the other three models on the same sessions")
    ap.add_argument("--no-train", action="store_true",
                    help="adjoint workload: skip EM's curve and Adam (EM and adjoint timing, gradient error only)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg (profiling runs)")
    ap.add_argument("--parity-iters", type=int, default=50,
                    help="iterations of the fused GPU fit and the FP64 oracle on the CPU leg's sample "
                         "(the bench line's error against the oracle; 0 skips)")
    ap.add_argument("--workload", choices=["dbn20m", "batched", "adjoint"], default="dbn20m",
                    help="dbn20m: the headline DBN fit; batched: 256 mixed fits in one launch; "
                         "adjoint: EM against the gradient trainer")
    ap.add_argument("--batch-fits", type=int, default=256)
    ap.add_argument("--model", choices=sorted(MODELS), default="dbn",
                    help="click model of the 20M-session workload (dbn is the headline)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing
# ---------------------------------------------------------------------------
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_dataset(args, rank: int):
    from massiveclicks_gb300 import api
    cfg = api.synth_config(2, n_sessions=args.sessions, n_queries=args.queries)
    cfg.seed = cfg.seed + 1000 * rank
    t0 = time.perf_counter()
    q, d, m = api.synth_sessions(cfg)
    t1 = time.perf_counter()
    ds = api.Dataset.from_sessions(q, d, m, 0.2)
    t2 = time.perf_counter()
    del q, d, m
    return ds, {"generate_s": round(t1 - t0, 3), "ingest_s": round(t2 - t1, 3)}


def cpu_sample(ds, n_sample: int) -> np.ndarray:
    """Indices of a bounded sample of the sorted training set: whole queries,
    visited in a seeded random order (so head and tail queries both appear)
    and taken while they fit in what is left of the budget, then put back in
    sorted order."""
    q = ds.train.query
    if len(q) == 0:
        return np.zeros(0, np.int64)
    starts = np.flatnonzero(np.r_[True, q[1:] != q[:-1]])
    ends = np.r_[starts[1:], len(q)]
    chosen, left = [], n_sample
    for g in np.random.default_rng(0).permutation(len(starts)).tolist():
        size = int(ends[g] - starts[g])
        if size <= left:
            chosen.append(g)
            left -= size
            if left == 0:
                break
    chosen.sort()
    return np.concatenate([np.arange(starts[g], ends[g]) for g in chosen]) if chosen else np.zeros(0, np.int64)


def time_cpu_oracle(ds, idx: np.ndarray, iters: int, warmup: int, threads: int, model: int = 2):
    """The reference's CPU path (FP32 restatement, reference threading) on the
    training sessions idx (whole queries): seconds per iteration, one entry
    per step."""
    from oracle import bindings
    sub = ds.train
    p = sub.pidx[idx]
    nq = int(p.max()) + 1 if len(idx) else 0
    fit = bindings.OracleFit("f32", model, 0, sub.query[idx], p, sub.click[idx], nq)
    fit.run(warmup, threads)
    times = []
    for _ in range(iters):
        t0 = time.perf_counter()
        fit.run(1, threads)
        times.append(time.perf_counter() - t0)
    return times


def sample_sets(ds, idx: np.ndarray):
    """The training sessions idx (whole queries) with their qd indices
    renumbered densely in order, and the test sessions of the same queries with
    the same renumbering (a test doc unseen in training stays -1)."""
    from massiveclicks_gb300 import api
    tr = ds.train
    p = tr.pidx[idx]
    used = np.unique(p)
    remap = np.full(ds.n_qd + 1, -1, np.int64)        # slot n_qd maps -1 to -1
    remap[used] = np.arange(len(used))
    train = api.SessionSet(tr.query[idx], tr.docs[idx], remap[p].astype(np.int32), tr.click[idx])
    te = ds.test
    keep = np.isin(te.query, np.unique(tr.query[idx]))
    tp = te.pidx[keep]
    test = api.SessionSet(te.query[keep], te.docs[keep], remap[np.where(tp < 0, ds.n_qd, tp)].astype(np.int32),
                          te.click[keep])
    return train, test, int(len(used))


def parity_vs_oracle(ds, idx: np.ndarray, model: int, iters: int, threads: int, stream, device: int) -> dict:
    """The fused GPU fit and the FP64 oracle (the reference's CPU path in
    double precision) on the same bounded sample, from the prior, for `iters`
    iterations: parameter and test-set errors of the GPU against the oracle."""
    from massiveclicks_gb300 import api
    from massiveclicks_gb300._capi import IMPL_FUSED
    from oracle import bindings
    train, test, n_qd = sample_sets(ds, idx)
    cm = api.ClickModel.create(model, device=device)
    cm.upload(train, n_qd, stream)
    cm.upload_test(test, stream)
    cm.em(iters, IMPL_FUSED, stream)
    ev = cm.evaluate(1, stream)
    got = cm.get_parameters()
    cm.destroy_parameters()
    f = bindings.OracleFit("f64", model, 0, train.query, train.pidx, train.click, n_qd)
    f.run(iters, threads=threads, copy_sessions=False)
    ref = f.values()
    ref_ev = f.evaluate(test.pidx, test.click)
    worst_rel, worst_abs, worst_bar = 0.0, 0.0, 0.0
    for k, r in ref.items():
        err = np.abs(got[k].astype(np.float64) - r)
        worst_abs = max(worst_abs, float(err.max()))
        worst_rel = max(worst_rel, float((err / np.maximum(np.abs(r), 1e-30)).max()))
        worst_bar = max(worst_bar, float((err / (1e-5 * np.abs(r) + 1e-6)).max()))
    return {"against": "FP64 oracle (the reference's CPU path in double precision)", "iterations": iters,
            "train_sessions": len(train), "test_sessions": len(test), "n_qd": n_qd,
            "max_param_abs_err": worst_abs, "max_param_rel_err": worst_rel,
            "max_param_err_over_bar": worst_bar, "param_bar": "1e-5 * |f64| + 1e-6",
            "test_llh": ev.llh, "oracle_test_llh": ref_ev["llh"],
            "test_llh_rel_err": abs(ev.llh - ref_ev["llh"]) / abs(ref_ev["llh"]),
            "perplexity": ev.perplexity, "oracle_perplexity": ref_ev["ppl"],
            "perplexity_rel_err": abs(ev.perplexity - ref_ev["ppl"]) / ref_ev["ppl"]}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in self.rows:
            try:
                sm.append(float(row[1]))
                mx.append(float(row[2]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, row[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def profile_traffic() -> dict | None:
    """DRAM bytes per launch of the fused kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "em_fused_dbn_traffic.json"
    if p.exists():
        return json.loads(p.read_text())
    return None


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ds, prep = make_dataset(args, 0)
    # The per-step sample shrinks with --steps so that the arm stays near a
    # minute of CPU work (at most 250M session-iterations, at least 50,000
    # sessions per step).
    idx = cpu_sample(ds, min(args.cpu_sample, max(50_000, 250_000_000 // max(1, args.steps))))
    n = len(idx)
    times = time_cpu_oracle(ds, idx, args.steps, max(1, min(args.warmup, 2)), threads, MODELS[args.model])
    total = sum(times)
    value = n * len(times) / total
    line = {
        "impl": "reference", "metric": metric_for(args.model), "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": data_text(args),
        "config": {"workload": f"{args.model.upper()} EM, {_count(args.sessions)} sessions ({_count(len(ds.train))} train), "
                               "one EM iteration per step; "
                               f"each step times a bounded sample of {n} training sessions",
                   "sessions": args.sessions, "train_sessions": len(ds.train), "sample_sessions": n,
                   "parallelism": f"{threads} host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} training sessions (whole queries) of the 16M, {len(times)} iterations"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank: int, world: int, local: int):
    import torch
    from massiveclicks_gb300 import api
    from massiveclicks_gb300._capi import IMPL_FUSED, IMPL_PLAIN

    torch.cuda.set_device(local)
    dist = Dist(world, "nccl")
    ds, prep = make_dataset(args, rank)
    n_train, n_qd = len(ds.train), ds.n_qd
    stream = torch.cuda.Stream()

    cm = api.ClickModel.create(MODELS[args.model], device=local)
    t0 = time.perf_counter()
    cm.upload(ds.train, n_qd, stream)
    cm.upload_test(ds.test, stream)
    prep["upload_s"] = round(time.perf_counter() - t0, 3)
    if not args.no_autotune:
        t0 = time.perf_counter()
        cm.autotune(stream)
        prep["autotune_s"] = round(time.perf_counter() - t0, 3)
    spt, wqd, block = cm.get_config()

    # ---- fused: warm-up, then exactly K timed iterations -------------------
    cm.em(args.warmup, IMPL_FUSED, stream)
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    cm.em(args.steps, IMPL_FUSED, stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms_max = dist.max(ms)
    value = world * n_train / (ms_max / 1000.0)

    # ---- roofline of the fused kernel (one launch = one iteration) ----------
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    # Algorithmic bytes per launch, the per-unit model of the reference's data
    # path: per session int32 pidx x10 + uint16 click mask (42 B); per qd and private
    # parameter a 4 B value read, a 16 B FP64 statistic write and read and a
    # 4 B value write (40 B; DBN has two private parameters, 80 B).
    per_qd = 80 if args.model == "dbn" else 40
    algo_bytes = 42 * n_train + per_qd * n_qd
    achieved = algo_bytes / (ms / 1000.0) / 1e9
    # This design's own bytes: packed sessions that carry variable statistics
    # (22 B: uint16 window indices x10 + clicks) and per qd 24 B (atr, sat,
    # counts read; atr, sat written).
    path, n_entries = cm.fused_path()
    if path == "dense":
        # PBM dense kernel: 20 B of uint16 counts by rank per qd; 8 B occurrence/click
        # counts, 4 B value read and 4 B value written.
        design_bytes = 36 * n_qd
        design_model = "dense count path: 36 B/qd (uint16 counts x10, occurrences/clicks, value read and write)"
    elif path == "counts":
        # PBM/UBM count kernel: 4 B per count entry; per qd 4 B offset, 8 B
        # occurrence/click counts, 4 B value read and 4 B value written.
        design_bytes = 4 * n_entries + 20 * n_qd
        design_model = f"count path: 4 B x {n_entries} entries + 20 B/qd"
    else:
        n_packed = int(np.count_nonzero(ds.train.click)) if args.model in ("dbn", "ccm") else n_train
        design_bytes = 22 * n_packed + (24 if args.model == "dbn" else 16) * n_qd
        design_model = f"tile path: 22 B x {n_packed} packed sessions + {24 if args.model == 'dbn' else 16} B/qd"
    tr = profile_traffic()
    traffic = None
    traffic_source = None
    if args.model == "dbn" and tr and tr.get("bytes_per_launch") and tr.get("n_train") and tr.get("n_qd"):
        if tr["n_train"] == n_train and tr["n_qd"] == n_qd:
            traffic = tr["bytes_per_launch"]
            traffic_source = "ncu dram__bytes_read.sum + dram__bytes_write.sum, this workload"
        else:
            # scaled from the profiled case by the bytes model 42 B/session + 24 B/qd
            scale = (42 * n_train + 24 * n_qd) / (42 * tr["n_train"] + 24 * tr["n_qd"])
            traffic = tr["bytes_per_launch"] * scale
            traffic_source = f"ncu capture of {tr['n_train']} training sessions, scaled"
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic, "traffic_source": traffic_source,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks.get("hbm_gbs") else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": algo_bytes,
                "bytes_model": f"42 B/session (int32 pidx x10 + uint16 clicks) + {per_qd} B/qd (per private parameter: 4 B value read + 16 B FP64 statistic write + read + 4 B value write)",
                "design_bytes_per_launch": design_bytes,
                "design_bytes_model": design_model,
                "dram_gbs_measured": (traffic / (ms / 1000.0) / 1e9) if traffic else None,
                "dram_frac_measured": (traffic / (ms / 1000.0) / 1e9 / hbm) if traffic else None}

    out = {}
    if rank == 0:
        # ---- equal test LL: fused vs plain from the prior, same iterations --
        ll_iters = 10
        cm.reset_to_prior(stream)
        cm.em(ll_iters, IMPL_FUSED, stream)
        torch.cuda.synchronize()
        ev_f = cm.evaluate(1, stream)
        if not args.no_plain:
            cm.reset_to_prior(stream)
            cm.em(1, IMPL_PLAIN, stream)   # allocates the plain buffers; warm-up
            torch.cuda.synchronize()
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            plain_steps = 3
            p0.record(stream)
            cm.em(plain_steps, IMPL_PLAIN, stream)
            p1.record(stream)
            torch.cuda.synchronize()
            plain_ms = p0.elapsed_time(p1) / plain_steps
            cm.reset_to_prior(stream)
            cm.em(ll_iters, IMPL_PLAIN, stream)
            torch.cuda.synchronize()
            ev_p = cm.evaluate(1, stream)
            out["plain_gpu"] = {"value": n_train / (plain_ms / 1000.0), "unit": UNIT, "ms_per_step": plain_ms,
                                "steps": plain_steps, "fused_speedup": plain_ms / ms}
            out["test_llh"] = {"iterations": ll_iters, "fused": ev_f.llh, "plain": ev_p.llh,
                               "rel_diff": abs(ev_f.llh - ev_p.llh) / abs(ev_p.llh),
                               "fused_perplexity": ev_f.perplexity, "plain_perplexity": ev_p.perplexity}
        else:
            out["test_llh"] = {"iterations": ll_iters, "fused": ev_f.llh, "fused_perplexity": ev_f.perplexity}

    # ---- end to end through the C-ABI with pinned host buffers --------------
    e2e = None
    if not args.no_e2e:
        pq = torch.from_numpy(ds.train.query).pin_memory()
        pp = torch.from_numpy(ds.train.pidx.reshape(-1)).pin_memory()
        pm = torch.from_numpy(ds.train.click.view(np.int16)).pin_memory()
        sizes = [(name, size) for name, size, _ in cm.parameter_information()]
        host_out = {name: torch.empty(size, dtype=torch.float32).pin_memory() for name, size in sizes}
        lib = api._capi.load()
        h2d = pq.numel() * 4 + pp.numel() * 4 + pm.numel() * 2
        d2h = sum(size * 4 for _, size in sizes)
        import ctypes as C

        def e2e_step():
            """One end-to-end step; returns its phase times (host clock, each
            phase synchronised on the stream)."""
            t = [time.perf_counter()]
            m2 = C.c_void_p()
            api.check(lib.mc_model_create(MODELS[args.model], 0, local, C.byref(m2)))
            api.check(lib.mc_model_upload(m2, n_train, C.c_void_p(pq.data_ptr()), C.c_void_p(pp.data_ptr()),
                                          C.c_void_p(pm.data_ptr()), n_qd, C.c_void_p(stream.cuda_stream)))
            api.check(lib.mc_model_configure(m2, spt, wqd, block))
            stream.synchronize()
            t.append(time.perf_counter())
            api.check(lib.mc_model_em(m2, args.e2e_iters, IMPL_FUSED, C.c_void_p(stream.cuda_stream)))
            stream.synchronize()
            t.append(time.perf_counter())
            for i, (name, _) in enumerate(sizes):
                api.check(lib.mc_model_get_param(m2, i, C.c_void_p(host_out[name].data_ptr()),
                                                 C.c_void_p(stream.cuda_stream)))
            lib.mc_model_destroy(m2)
            t.append(time.perf_counter())
            return {"create_upload_ms": 1e3 * (t[1] - t[0]), "iterations_ms": 1e3 * (t[2] - t[1]),
                    "download_destroy_ms": 1e3 * (t[3] - t[2])}

        e2e_step()  # warm-up (the first upload of a process also allocates the library's caches)
        torch.cuda.synchronize()
        dist.barrier()
        # Python's collector stays off in the timed loop (a full pass can take
        # tens of milliseconds; a C++ caller of the C-ABI has none); the mean
        # over the steps is the figure, the median is reported beside it.
        import gc
        gc.collect()
        gc.disable()
        e2e_steps = 20
        step_s, phases = [], []
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            t1 = time.perf_counter()
            phases.append(e2e_step())
            step_s.append(time.perf_counter() - t1)
        torch.cuda.synchronize()
        e2e_s = dist.max((time.perf_counter() - t0) / e2e_steps)
        gc.enable()
        slowest = max(range(e2e_steps), key=lambda i: step_s[i])
        e2e = {"value": world * n_train * args.e2e_iters / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s,
               "seconds_per_step_median": statistics.median(step_s), "steps": e2e_steps,
               "phases_median_ms": {k: round(statistics.median(p[k] for p in phases), 3) for k in phases[0]},
               "slowest_step_phases_ms": {k: round(v, 3) for k, v in phases[slowest].items()},
               "slowest_step_index": slowest,
               "step": f"mc_model_create + mc_model_upload (pinned host sessions) + {args.e2e_iters} fused "
                       "iterations + mc_model_get_param of every array + destroy"}

    # ---- the other models on the same sessions: fused EM, default tile shape,
    # 200 iterations timed with CUDA events after 10 ---------------------------
    if not args.no_models:
        others = {}
        for name in [k for k in ("pbm", "ubm", "ccm", "dbn") if k != args.model]:
            om = api.ClickModel.create(MODELS[name], device=local)
            om.upload(ds.train, n_qd, stream)
            om.em(10, IMPL_FUSED, stream)
            stream.synchronize()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            om.em(200, IMPL_FUSED, stream)
            ev1.record(stream)
            ev1.synchronize()
            ms = ev0.elapsed_time(ev1) / 200
            survey_bytes = 42 * n_train + (80 if name == "dbn" else 40) * n_qd
            path, _ = om.fused_path()
            others[name] = {"ms_per_iteration": ms, "session_iterations_per_s": world * n_train / (ms / 1e3),
                            "roofline_frac_survey_bytes": survey_bytes / (ms / 1e3) / 1e9 / hbm,
                            "path": path}
            om.destroy_parameters()
        out["other_models"] = others

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        idx = cpu_sample(ds, args.cpu_sample)
        n = len(idx)
        times = time_cpu_oracle(ds, idx, 2, 1, threads, MODELS[args.model])
        cpu = {"value": n * len(times) / sum(times), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} training sessions (whole queries), {len(times)} iterations after 1 warm-up; "
                         "FP32 restatement of the reference's CPU path with its threading"}
        if args.parity_iters > 0:
            out["parity"] = parity_vs_oracle(ds, idx, MODELS[args.model], args.parity_iters, threads, stream, local)

    if rank == 0:
        line = {
            "metric": metric_for(args.model), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": data_text(args),
            "config": {"workload": f"{args.model.upper()} EM over {_count(n_train)} training sessions "
                                   f"({_count(args.sessions)} sessions, test share 0.2); "
                                   "one fused kernel launch per iteration, replayed from a CUDA graph",
                       "sessions": args.sessions, "train_sessions": n_train, "n_qd": n_qd,
                       "model": args.model.upper(), "mode": "parity", "tile": {"sessions_per_tile": spt, "window_qd": wqd,
                                                                   "block": block},
                       "l2": "inputs larger than L2 (sessions 672 MB + parameters), no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU", "prep": prep},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": args.steps,
            "clocks": clk,
        }
        line.update(out)
        print(json.dumps(line), flush=True)
    dist.close()


def run_batched(args, rank: int, world: int, local: int):
    """256 independent fits (PBM/UBM/DBN in turn) on disjoint query partitions
    of log-uniform size 1k..500k sessions (about 30M in total), generated like
    the 40k-session PBM workload (1k queries Zipf 1.1 per partition, 20-doc
    pools, PBM clicks).  One step = one EM iteration of every fit.  Compared:
    one persistent launch for all fits (mc_batch_em) against each fit's own
    fused launch and each fit's plain two-kernel EM, run one after another."""
    import torch
    from massiveclicks_gb300 import api
    from massiveclicks_gb300._capi import IMPL_FUSED, IMPL_PLAIN

    torch.cuda.set_device(local)
    rng = np.random.default_rng(4242 + rank)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(500000), args.batch_fits)).astype(np.int64)
    types = [0, 3, 2]
    models, n_train = [], 0
    t0 = time.perf_counter()
    for i, n in enumerate(sizes):
        cfg = api.synth_config(0, n_sessions=int(n), n_queries=1000, seed=9000 + 7919 * i + rank)
        q, d, m = api.synth_sessions(cfg)
        ds = api.Dataset.from_sessions(q, d, m, 0.2)
        cm = api.ClickModel.create(types[i % 3])
        cm.upload(ds.train, ds.n_qd)
        models.append(cm)
        n_train += len(ds.train)
    prep_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    batch = api.Batch(models)
    n_fits, n_tiles, _ = batch.info()
    n_count_fits = sum(1 for cm in models if cm.fused_path()[0] in ("counts", "dense"))
    # per iteration: the tile launch (DBN/CCM fits) and the batched count launch (PBM/UBM fits)
    launches_per_iteration = batch.launches_per_iteration()

    def timed(fn, steps):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    batch.em(args.warmup, stream)
    clocks = ClockSampler(local)
    clocks.start()
    ms_batch = timed(lambda k: batch.em(k, stream), args.steps)
    clk = clocks.stop()
    # the same iterations with the count chunks taken by the tile launch itself
    batch.configure(True)
    batch.em(args.warmup, stream)
    ms_single = timed(lambda k: batch.em(k, stream), max(1, args.steps // 4))
    batch.configure(False)
    for cm in models:
        cm.em(1, IMPL_FUSED, stream)
    ms_sep = timed(lambda k: [cm.em(k, IMPL_FUSED, stream) for cm in models], max(1, args.steps // 4))
    plain_steps = 2
    for cm in models:
        cm.em(1, IMPL_PLAIN, stream)
    ms_plain = timed(lambda k: [cm.em(k, IMPL_PLAIN, stream) for cm in models], plain_steps)
    value = n_train / (ms_batch / 1000.0)
    if rank == 0:
        line = {
            "metric": "EM session-iterations/s, 256 batched fits (mixed PBM/UBM/DBN)", "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batch,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: per fit 1k queries Zipf(1.1), 20-doc pools, PBM clicks; sizes log-uniform 1k..500k",
            "config": {"workload": f"{n_fits} fits, {int(sizes.sum())} sessions ({n_train} training), per iteration "
                                   "one tile launch for the DBN fits and one count launch for the PBM/UBM fits",
                       "tiles": n_tiles, "count_path_fits": n_count_fits, "prep_s": round(prep_s, 2)},
            "single_launch": {"value": n_train / (ms_single / 1000.0), "ms_per_step": ms_single,
                              "note": "count chunks taken by the persistent tile launch after its tiles"},
            "separate_fused": {"value": n_train / (ms_sep / 1000.0), "ms_per_step": ms_sep},
            "separate_plain": {"value": n_train / (ms_plain / 1000.0), "ms_per_step": ms_plain,
                               "batched_speedup": ms_plain / ms_batch},
            "gpu_launches": args.steps * launches_per_iteration, "clocks": clk,
        }
        print(json.dumps(line), flush=True)


def run_adjoint(args, rank: int, world: int, local: int):
    """DBN on 5M sessions (DBN-generated, 250k queries, 30-doc pools): EM
    (fused, 50 iterations from the prior) against Adam on the logits (lr 0.05,
    batches of 262,144 sessions, the adjoint kernel for gradients), compared on
    wall time to reach EM's best test log-likelihood, and the adjoint's own
    throughput."""
    import torch
    from massiveclicks_gb300 import api, gradient
    from massiveclicks_gb300._capi import IMPL_FUSED

    torch.cuda.set_device(local)
    cfg = api.synth_config(1, n_sessions=5_000_000, n_queries=250_000, seed=55_000 + rank)
    q, d, m = api.synth_sessions(cfg)
    ds = api.Dataset.from_sessions(q, d, m, 0.2)
    n_train, n_qd = len(ds.train), ds.n_qd
    em = api.DBNModel(device=local)
    em.init_parameters(ds)
    em_curve = []
    t_em = 0.0
    for it in range(0 if args.no_train else 50):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        em.em(1, IMPL_FUSED)
        torch.cuda.synchronize()
        t_em += time.perf_counter() - t0
        em_curve.append((t_em, em.evaluate(1).llh))
    target = max(ll for _, ll in em_curve) if em_curve else None  # EM's best test LL within 50 iterations
    t_em_target = next(t for t, ll in em_curve if ll >= target - 1e-4 * abs(target)) if em_curve else None
    # EM's own device time per iteration on these sessions (CUDA events, the
    # fit's graph replay), for the per-session cost of the adjoint
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    em.em(64, IMPL_FUSED)
    ev1.record()
    torch.cuda.synchronize()
    em_ms = ev0.elapsed_time(ev1) / 64

    # Adam's minibatches: consecutive ranges of a random order of whole
    # queries (unbiased, and the adjoint's tile path applies).
    t_sessions, t_nqd, to_orig = gradient.query_order(ds.train, seed=rank)
    assert t_nqd == n_qd
    trainer_model = api.DBNModel(device=local)
    trainer_model.upload(t_sessions, n_qd)
    # Test-set evaluation from the logits on the device (mc_evaluate_static),
    # outside the trainer's clock.
    lib = api._capi.load()
    dev = torch.device("cuda", local)
    to_orig_t = torch.from_numpy(to_orig).to(dev)
    test_pidx = torch.from_numpy(np.ascontiguousarray(ds.test.pidx, np.int32).reshape(-1)).to(dev)
    test_click = torch.from_numpy(np.ascontiguousarray(ds.test.click, np.uint16).view(np.int16)).to(dev)
    n_test = len(ds.test)
    curve = []
    import ctypes as C

    def test_llh(a, b, g):
        atr = torch.empty(n_qd, dtype=torch.float32, device=dev)
        sat = torch.empty(n_qd, dtype=torch.float32, device=dev)
        atr[to_orig_t] = torch.sigmoid(a.detach())
        sat[to_orig_t] = torch.sigmoid(b.detach())
        pub = torch.sigmoid(g.detach()).contiguous()
        torch.cuda.synchronize()
        ll = C.c_double()
        l2 = np.zeros(10)
        api.check(lib.mc_evaluate_static(2, n_test, C.c_void_p(test_pidx.data_ptr()), C.c_void_p(test_click.data_ptr()),
                                         n_qd, C.c_void_p(atr.data_ptr()), C.c_void_p(sat.data_ptr()),
                                         C.c_void_p(pub.data_ptr()), C.byref(ll), l2.ctypes.data_as(C.c_void_p), None))
        return ll.value / n_test

    def cb(step, seconds, a, b, g):
        curve.append((step, seconds, test_llh(a, b, g)))

    batch = 262_144
    steps_per_epoch = (n_train + batch - 1) // batch
    if not args.no_train:
        # Warm-up outside the clock: the first use of torch's fused Adam kernels
        # (module loading, which measured seconds on a fresh GB300) and the
        # adjoint's one-time per-tile counts.
        gradient.train_adam(trainer_model, n_qd, steps=2, batch=batch, lr=0.05, device=local)
        torch.cuda.synchronize()
        gradient.train_adam(trainer_model, n_qd, steps=20 * steps_per_epoch, batch=batch, lr=0.05, callback=cb,
                            callback_every=steps_per_epoch, device=local)
    reach = next(((s, t, ll) for s, t, ll in curve if ll >= target - 1e-4 * abs(target)), None)
    t_steps = curve[-1][1] if curve else None

    # adjoint throughput: one log-likelihood + gradient pass over all training
    # sessions through the C-ABI (mc_dbn_loglik_grad: gradient clear, the tile
    # kernel, FP32 conversion), and the same pass through the autograd wrapper
    # (forward + backward), whose Python and autograd dispatch the GPU waits for
    a = torch.zeros(n_qd, device=dev, requires_grad=True)
    b = torch.zeros(n_qd, device=dev, requires_grad=True)
    g = torch.zeros(1, device=dev, requires_grad=True)
    da_, db_, dg_ = torch.empty_like(a), torch.empty_like(b), torch.empty_like(g)
    ll_ = torch.empty((), dtype=torch.float64, device=dev)
    stream_ = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def c_pass():
        api.check(lib.mc_dbn_loglik_grad(trainer_model._h, 0, n_train, C.c_void_p(a.data_ptr()),
                                         C.c_void_p(b.data_ptr()), C.c_void_p(g.data_ptr()), 0,
                                         C.c_void_p(da_.data_ptr()), C.c_void_p(db_.data_ptr()),
                                         C.c_void_p(dg_.data_ptr()), C.c_void_p(ll_.data_ptr()), stream_))

    def autograd_pass():
        gradient.dbn_loglik(a, b, g, trainer_model).backward()

    def timed_ms(fn, k=10):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    ms_grad = timed_ms(c_pass)
    ms_autograd = timed_ms(autograd_pass)
    # the FP32 gradient against the FP64 one at logits drawn N(-1, 1)
    gen = torch.Generator(device="cpu").manual_seed(7)
    a_init = (torch.randn(n_qd, generator=gen) - 1).to(dev)
    b_init = (torch.randn(n_qd, generator=gen) - 1).to(dev)
    grads = {}
    for fp64 in (False, True):
        a2 = a_init.clone().requires_grad_(True)
        b2 = b_init.clone().requires_grad_(True)
        g2 = torch.full((1,), 1.5, device=dev, requires_grad=True)
        gradient.dbn_loglik(a2, b2, g2, trainer_model, fp64=fp64).backward()
        grads[fp64] = (a2.grad.double(), b2.grad.double(), float(g2.grad))
    grad_err = {}
    for k_, i_ in (("alpha", 0), ("beta", 1)):
        d_ = (grads[False][i_] - grads[True][i_]).abs()
        grad_err[k_] = {"max_abs": float(d_.max()),
                        "max_rel_floor1": float((d_ / grads[True][i_].abs().clamp_min(1.0)).max())}
    grad_err["gamma_rel"] = abs(grads[False][2] - grads[True][2]) / abs(grads[True][2])
    if rank == 0:
        line = {
            "metric": "seconds for Adam to reach EM's best 50-iteration test LL (DBN, 5M sessions)",
            "value": reach[1] if reach else None, "unit": "s", "higher_is_better": False, "n_gpus": world,
            "dtype": "f32", "data": "synthetic: 5M sessions, 250k queries Zipf(1.0), 30-doc pools, DBN clicks",
            "config": {"workload": "DBN EM (fused, from the prior) vs Adam lr 0.05, batch 262,144 sessions",
                       "train_sessions": n_train, "n_qd": n_qd},
            "em": {"target_test_llh": target, "seconds_to_target": t_em_target, "seconds_50_iterations": t_em,
                   "final_test_llh": em_curve[-1][1] if em_curve else None},
            "adam": {"reached": reach is not None, "steps": reach[0] if reach else None,
                     "seconds": reach[1] if reach else None, "final_test_llh": curve[-1][2] if curve else None,
                     "best_test_llh": max(ll for _, _, ll in curve) if curve else None},
            "adam_ms_per_step": 1000.0 * t_steps / (20 * steps_per_epoch) if t_steps else None,
            "adjoint": {"ms_per_forward_backward": ms_grad,
                        "autograd_ms_per_forward_backward": ms_autograd,
                        "session_gradients_per_s": n_train / (ms_grad / 1000.0),
                        "em_ms_per_iteration": em_ms,
                        "forward_backward_over_em_iteration": ms_grad / em_ms,
                        "fp32_gradient_vs_fp64": grad_err,
                        "em_session_iterations_per_s": n_train * 50 / t_em if t_em else None,
                        "path": "tiles (sessions grouped by query, gradient summed per tile in shared memory)"},
        }
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "ours" and args.workload == "adjoint":
        run_adjoint(args, rank, world, local)
        return
    if args.impl == "ours" and args.workload == "batched":
        run_batched(args, rank, world, local)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
