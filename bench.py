"""Benchmark: suffix-array construction throughput (Msuffixes/s) on GB300.

Workload (default): the DNA-like text with planted repeats — n = 2^28 u8
symbols over {0,1,2,3}, 30% of positions covered by copies of log-uniform
length 100..10,000 taken from earlier offsets with 1% substitutions — built
with build_in_memory (PlainText, u32 index).  Synthetic and seeded (no public
dataset backs this workload).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       one JSON line; `value` = suffixes/s with the text resident in HBM
            (device pointers through the C ABI), `e2e` = the same call with
            pinned host text and host output (copies inside the timed region).
reference:  the reference's CPU algorithm (the C restatement in oracle/, the
            Rust crate cannot be built here) on the host cores, each step a
            bounded prefix of the same text.
N > 1:      independent replicas, one per GPU (the path has no exchange step);
            value = all ranks' suffixes / max-over-ranks time.
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
sys.path.insert(0, os.path.join(ROOT, "caps-sa_gb300"))

import numpy as np  # noqa: E402

CPU_SAMPLE_LOG2 = 24  # bounded CPU sample: the first 2^24 symbols of the text


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--log2n", type=int, default=28)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the secondary forms (sample sort with splitter / learned "
                         "partition, batched texts, segmented filtered subset)")
    ap.add_argument("--form", choices=FORMS,
                    help="run this secondary form alone (no bench step) and print its "
                         "JSON; for profiling one workload")
    return ap.parse_args()


def workload(log2n, seed=2):
    from capssa import workloads
    return workloads.dna_with_repeats(1 << log2n, seed=seed)


def config(log2n, n):
    # working set: two 8-byte record buffers per suffix, plus the text
    ws_bytes = 16 * n + n
    l2 = ("no flush: inputs (%d MiB text, ~%.1f GiB working set) exceed the 129 MB L2"
          % (n >> 20, ws_bytes / 2**30) if ws_bytes > 129e6 else
          "no flush; a small case whose working set (%.1f MiB) fits the 129 MB L2"
          % (ws_bytes / 2**20))
    return {"workload": "dna-repeats: n=2^%d u8 over {0,1,2,3}, 30%% planted repeats "
                        "(log-uniform 100..10000, 1%% substitutions), build_in_memory "
                        "PlainText, u32 index" % log2n,
            "n": n, "symbol": "u8", "index": "u32", "limits": "PlainText",
            "l2": l2,
            "parallelism": "replicas (one independent text per GPU)"}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    return rank, ws, local, dist


def max_over_ranks(x, dist, device):
    """The largest value of x over all ranks (x itself without a process
    group): the job's time is its slowest replica's."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(n_per_rank, world, steps, elapsed_s):
    """Whole-job Msuffixes/s: every rank's suffixes over the max-over-ranks time."""
    return n_per_rank * world * steps / elapsed_s / 1e6


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------------ peaks / profile

def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(n, item_bytes):
    """DRAM bytes per radix-pass launch from the committed ncu summary for
    this record width (captured at 2^26 records, input 4x L2), scaled by
    records per launch (traffic grows linearly with the records)."""
    p = os.path.join(ROOT, "profiles", "radix_onesweep_pass_%dB.txt" % item_bytes)
    try:
        vals = {}
        for ln in open(p):
            if ":" in ln:
                k, v = ln.split(":", 1)
                vals[k.strip()] = v.strip().split()[0]
        per_rec = float(vals["dram_bytes_per_record"])
        return per_rec * n
    except Exception:
        return None


# ------------------------------------------------------------------ CPU baseline

def cpu_baseline(text, repeats=3):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    sample = np.ascontiguousarray(text[: 1 << CPU_SAMPLE_LOG2])
    cores = oracle.max_threads()
    oracle.build_in_memory(sample[: 1 << 20])  # warm-up
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        oracle.build_in_memory(sample)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return {"value": len(sample) / t / 1e6, "unit": "Msuffixes/s", "cores": cores,
            "kind": "port",
            "sample": "build_in_memory restated in C (merge sort + LCP merge, OpenMP tasks) on "
                      "the first 2^%d symbols of the workload text; median of %d"
                      % (CPU_SAMPLE_LOG2, repeats)}


REF_BUDGET_S = 150.0  # wall time the reference arm's timed steps may take in all


def run_reference(args):
    """The reference's CPU algorithm (the C restatement in oracle/) on the
    host cores.  Each timed step sorts the longest prefix of the workload
    text (a power of two, up to the whole text) whose estimated time keeps
    all K steps within REF_BUDGET_S; `config.n` is that prefix.  Warm-up
    steps sort a 2^20-symbol prefix."""
    rank, ws, local, dist = dist_init()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    log2n = args.log2n
    text = workload(log2n)
    cores = oracle.max_threads()
    for _ in range(args.warmup):
        oracle.build_in_memory(np.ascontiguousarray(text[: 1 << 20]))
    # rate probe on a 2^22 prefix, then the largest prefix that fits the budget
    probe = np.ascontiguousarray(text[: 1 << min(22, log2n)])
    t0 = time.perf_counter()
    oracle.build_in_memory(probe)
    rate = len(probe) / (time.perf_counter() - t0)
    lg = min(22, log2n)
    lg0 = lg

    def est(lg_):  # seconds for all steps: n log n from the probe, with margin
        return (1 << lg_) * lg_ / (rate * lg0) * 1.3 * args.steps

    while lg < log2n and est(lg + 1) <= REF_BUDGET_S:
        lg += 1
    sample = np.ascontiguousarray(text[: 1 << lg])
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.build_in_memory(sample)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = len(sample) * args.steps / total / 1e6
    cfg = config(log2n, 1 << lg)  # the workload's text; n = the symbols each step sorts
    if lg < log2n:
        cfg["sample"] = ("the first 2^%d symbols of the 2^%d-symbol workload text per step "
                         "(all %d steps within %.0f s of host time)"
                         % (lg, log2n, args.steps, REF_BUDGET_S))
    line = {"impl": "reference", "metric": "Msuffixes/s", "value": value, "unit": "Msuffixes/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": "Msuffixes/s", "cores": cores,
                             "kind": "port",
                             "sample": "the first 2^%d symbols of the workload text per step; "
                                       "the Rust crate cannot be built here, so its algorithm "
                                       "restated in C (oracle/, OpenMP tasks for rayon::join) "
                                       "runs on all %d host threads" % (lg, cores)},
            "e2e": {"value": value, "unit": "Msuffixes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm

def _timed(fn, reps):
    """Median wall time (ms) of fn() over reps calls (each call synchronises)."""
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(ts)


FORMS = ("sample_sort", "batched", "segmented_filtered")


def run_forms(ctx, t_dev, n, only=FORMS):
    """The secondary forms of the metric, each on its own workload:
    sample sort of the bench text with p = 4096 partitions found by splitter
    search (indexed by the pivots' leading key bits, or a plain bisection over
    all pivots) vs the learned CDF model (16,384 training samples); 8,192
    independent texts sorted in one batched call vs a per-text loop; the
    segmented, filtered subset build (n = 2^29, u64 index).  `only` picks
    some of them (bench.py --form)."""
    out = {}
    if "sample_sort" in only:
        out["sample_sort_p4096"] = form_sample_sort(ctx, t_dev, n)
    if "batched" in only:
        out["batched_8192_texts"] = form_batched(ctx)
    if "segmented_filtered" in only:
        out["segmented_filtered_2p29"] = form_segmented_filtered(ctx)
    return out


def form_sample_sort(ctx, t_dev, n):
    import capssa

    # ---- sample sort: splitter vs learned partition (plan = SA + partition),
    # bucketed before the sort; and the reference's sampling rule, whose
    # chunk order comes from a full sort first
    ss = {}
    for name, part, smp in (("splitters", capssa.Partition.SPLITTERS, capssa.Sampling.AUTO),
                            ("bisection", capssa.Partition.BISECT, capssa.Sampling.AUTO),
                            ("learned", capssa.Partition.LEARNED, capssa.Sampling.AUTO),
                            ("reference_rule_sort_first", capssa.Partition.SPLITTERS,
                             capssa.Sampling.REFERENCE)):
        opts = capssa.ExtMemOpts(subproblem_count=4096, partition=part, sampling=smp)
        ctx.sample_sort_plan(t_dev, opts)  # warm
        ms = _timed(lambda: ctx.sample_sort_plan(t_dev, opts), 3)
        k, pv, sz = ctx.sample_sort_plan(t_dev, opts)
        st = ctx.stats()
        ss[name] = {"value": n / (ms / 1e3) / 1e6, "unit": "Msuffixes/s", "ms": ms,
                    "partition_ms": st["partition_ms"],
                    "partition_gbs": (n * 8.25 / (st["partition_ms"] / 1e3) / 1e9
                                      if st["partition_ms"] > 0 else None),
                    "probes_per_suffix": st["partition_probes"] / n,
                    "mispredicted_rate": st["mispredicted"] / n,
                    "imbalance_max_over_mean": float(sz.max()) / (n / k),
                    "train_ms": st["train_ms"], "train_samples": st["train_samples"],
                    "model_loss": st["model_loss"], "p": k,
                    "keys_ms": st["keys_ms"], "sort_ms": st["sort_ms"],
                    "refine_ms": st["refine_ms"], "sort_passes": st["sort_passes"],
                    "sizes_sha": hash(sz.tobytes()) & 0xFFFFFFFF}
    ss["same_partition"] = ss["splitters"]["sizes_sha"] == ss["learned"]["sizes_sha"]
    return ss


def form_batched(ctx):
    import torch

    from capssa import workloads

    # ---- batched: 8,192 texts, log-uniform 2^10..2^20, 10% repeats
    cat, offs = workloads.batched_texts()
    c_dev = torch.from_numpy(cat).to("cuda")
    total = int(offs[-1])
    o_dev = torch.empty(total, dtype=torch.int32, device="cuda")  # results stay in HBM
    ctx.build_batched(c_dev, offs, out=o_dev)  # warm
    b_ms = _timed(lambda: ctx.build_batched(c_dev, offs, out=o_dev), 2)
    # per-text loop of plain builds on every 16th text (bounded sample)
    idx = list(range(0, len(offs) - 1, 16))
    sample_syms = sum(int(offs[i + 1] - offs[i]) for i in idx)

    def loop():
        for i in idx:
            a, b = int(offs[i]), int(offs[i + 1])
            ctx.build_in_memory(c_dev[a:b], out=o_dev[a:b])

    loop()
    l_ms = _timed(loop, 1)
    res = {
        "value": total / (b_ms / 1e3) / 1e6, "unit": "Msuffixes/s", "ms": b_ms,
        "symbols": total,
        "per_text_loop": {"value": sample_syms / (l_ms / 1e3) / 1e6, "unit": "Msuffixes/s",
                          "sample": "every 16th text (%d texts, %d symbols)"
                                    % (len(idx), sample_syms)}}
    del c_dev, o_dev
    return res


def form_segmented_filtered(ctx):
    import torch

    import capssa
    from capssa import workloads

    # ---- segmented, filtered subset: n = 2^29, lognormal segments, symbol < 4 kept
    text3, ends3, pos3 = workloads.segmented_filtered(1 << 29)
    t3 = torch.from_numpy(text3).to("cuda")
    p3 = torch.from_numpy(pos3.view(np.int64)).to("cuda")
    o3 = torch.empty(len(pos3), dtype=torch.int64, device="cuda")
    lp3 = capssa.SegmentedText(len(text3), ends3)
    ctx.build_in_memory_for_positions(t3, p3, lp3, out=o3)  # warm
    s_ms = _timed(lambda: ctx.build_in_memory_for_positions(t3, p3, lp3, out=o3), 2)
    # the same with every tie class in the reference's merge order
    ref_ties = capssa.Opts(tie_order=capssa.TieOrder.REFERENCE)
    ctx.build_in_memory_for_positions(t3, p3, lp3, ref_ties, out=o3)  # warm
    r_ms = _timed(lambda: ctx.build_in_memory_for_positions(t3, p3, lp3, ref_ties, out=o3), 2)
    r_st = ctx.stats()
    # the same through the GPU filter source (positions selected on the device)
    ctx.build_in_memory_for_filter(t3, 0, 4, lp3, out=o3)
    f_ms = _timed(lambda: ctx.build_in_memory_for_filter(t3, 0, 4, lp3, out=o3), 2)
    # build_ext_mem_for_filter: host text in, suffix order streamed to a host
    # callback in 32 MiB batches (host clock around the whole call)
    sent = [0]

    def sink(batch):
        sent[0] += len(batch)

    ctx.try_build_ext_mem(text3, None, sink, lp3, keep=(0, 4))  # warm
    sent[0] = 0
    t0 = time.perf_counter()
    ctx.try_build_ext_mem(text3, None, sink, lp3, keep=(0, 4))
    e_ms = (time.perf_counter() - t0) * 1e3
    assert sent[0] == len(pos3)
    res = {"value": len(pos3) / (s_ms / 1e3) / 1e6,
                                      "unit": "Msuffixes/s", "ms": s_ms,
                                      "positions": int(len(pos3)), "segments": int(len(ends3)),
                                      "reference_tie_order": {
                                          "value": len(pos3) / (r_ms / 1e3) / 1e6,
                                          "unit": "Msuffixes/s", "ms": r_ms,
                                          "tie_order_ms": r_st["tie_order_ms"],
                                          "tie_classes": int(r_st["tie_classes"])},
                                      "filter_source": {"value": len(pos3) / (f_ms / 1e3) / 1e6,
                                                        "unit": "Msuffixes/s", "ms": f_ms},
                                      "ext_mem_for_filter": {
                                          "value": len(pos3) / (e_ms / 1e3) / 1e6,
                                          "unit": "Msuffixes/s", "ms": e_ms,
                                          "h2d_bytes": int(text3.nbytes),
                                          "d2h_bytes": int(8 * len(pos3)),
                                          "clock": "host, whole call (text upload, build, "
                                                   "streamed emit)"}}
    del t3, p3, o3
    torch.cuda.synchronize()
    return res


def run_ours(args):
    import torch

    import capssa

    rank, ws, local, dist = dist_init()
    torch.cuda.set_device(local)
    if dist is not None:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    log2n = args.log2n
    n = 1 << log2n
    text = workload(log2n, seed=2 + rank)
    ctx = capssa.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    t_dev = torch.from_numpy(text).to("cuda")
    sa_dev = torch.empty(n, dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        ctx.build_in_memory(t_dev, out=sa_dev)
    torch.cuda.synchronize()

    # correctness guard on the timed configuration: a permutation check on
    # the device (every position appears once)
    seen = torch.zeros(n, dtype=torch.int32, device="cuda")
    seen.index_add_(0, sa_dev.long(), torch.ones(n, dtype=torch.int32, device="cuda"))
    if not bool((seen == 1).all()):
        raise SystemExit("suffix array is not a permutation")
    del seen

    clocks = ClockSampler(local)
    clocks.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    pass_ms, passes, phase = [], [], {"keys_ms": 0, "sort_ms": 0, "refine_ms": 0, "finish_ms": 0}
    item_bytes = 12
    rounds = 0
    ev0.record(stream)
    for _ in range(args.steps):
        ctx.build_in_memory(t_dev, out=sa_dev)
        st = ctx.stats()
        launches += st["kernel_launches"]
        pass_ms.append(st["sort_pass_ms"])
        passes.append(st["sort_passes"])
        item_bytes = st["sort_item_bytes"] or 12
        rounds = st["refine_rounds"]
        for k in phase:
            phase[k] += st[k] / args.steps
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    elapsed_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    elapsed_ms = max_over_ranks(elapsed_ms, dist, "cuda")
    ms_per_step = elapsed_ms / args.steps
    value = job_throughput(n, ws, args.steps, elapsed_ms / 1e3)

    # roofline of the dominant kernel: one onesweep radix pass over the n
    # suffix records reads and writes each record once (8 B when the
    # position is packed below the key, else a u64 key + a u32 position)
    peak, peak_kind = hbm_peak()
    avg_pass_ms = sum(pass_ms) / max(1, sum(passes))
    alg_bytes = 2.0 * item_bytes * n
    achieved = alg_bytes / (avg_pass_ms / 1e3) / 1e9
    traffic = profiled_traffic(n, item_bytes)
    roofline = {"kernel": "radix onesweep pass (initial sort of the %d-byte suffix records)"
                % item_bytes, "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_pass_ms,
                "launches_per_step": sum(passes) / len(passes),
                "phase_ms": phase, "refine_rounds": rounds}

    e2e = None
    if not args.no_e2e:
        h_text = torch.from_numpy(text).pin_memory()
        h_out = torch.empty(n, dtype=torch.int32).pin_memory()
        for _ in range(max(1, args.warmup)):
            ctx.build_in_memory(h_text.numpy(), out=h_out.numpy().view(np.uint32))
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.build_in_memory(h_text.numpy(), out=h_out.numpy().view(np.uint32))
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        el = max_over_ranks(el, dist, "cuda")
        st = ctx.stats()  # the last step's host-side copy times
        e2e = {"value": job_throughput(n, ws, args.steps, el), "unit": "Msuffixes/s",
               "h2d_bytes_per_step": int(n), "d2h_bytes_per_step": int(4 * n),
               "ms_per_step": el / args.steps * 1e3,
               "h2d_ms": round(st["h2d_ms"], 3), "d2h_ms": round(st["d2h_ms"], 3)}
        if not np.array_equal(h_out.numpy().view(np.uint32), sa_dev.cpu().numpy().view(np.uint32)):
            raise SystemExit("host-path suffix array differs from the device-path one")

    forms = None
    if rank == 0 and ws == 1 and not args.no_forms:
        forms = run_forms(ctx, t_dev, n)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(text)

    if rank == 0:
        line = {"metric": "Msuffixes/s", "value": value, "unit": "Msuffixes/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
                "data": "synthetic (seeded generator, caps-sa_gb300/capssa/workloads.py)",
                "config": config(log2n, n), "roofline": roofline, "cpu_baseline": cpu,
                "e2e": e2e, "clocks": clk, "gpu_launches": launches, "forms": forms}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_form(args):
    """One secondary form alone on cuda:0 (no bench step, no contract line)."""
    import torch

    import capssa

    torch.cuda.set_device(0)
    ctx = capssa.Context(0)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    t_dev, n = None, 0
    if args.form == "sample_sort":
        n = 1 << args.log2n
        t_dev = torch.from_numpy(workload(args.log2n)).to("cuda")
    print(json.dumps({"form": args.form, **run_forms(ctx, t_dev, n, only=(args.form,))}))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.form:
        return run_form(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
