"""bench.py — k-mers/s of the GB300 graph build on the 5 Mbp paired-end workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one complete graph build (parse, k-mer extraction, canonicalisation,
aggregation, serialization of every (VKmer, Node) record) of the workload:
5 Mbp genome at GC 50% with 10 x 1 kbp segments repeated 10 times, 833,333 pairs of
2 x 150 bp (50x), insert N(500, 50), 1% substitutions, 0.01% N, k = 31 (seeded synthetic
reads, see genomix_gb300/synth.py).

  value      k-mers/s with the readid text already in HBM (CUDA events on the library's
             stream over K steps; the text (258 MB) and the table (6.3 GB) exceed L2, so no
             flush is needed between steps)
  e2e        the same metric through the C ABI with host buffers: pinned readid text in,
             H2D copy, build, D2H copy of every record into pinned memory, per step; steps
             are pipelined (gx_job_emit_async): step i's copy out overlaps step i+1's build
  roofline   the largest kernel of the build, the per-bucket aggregation (k_aggregate): its
             algorithmic bytes per launch (every occurrence's key and edge bits read, each
             node's key, count/meta word and record offset written, each read head's entries)
             over its CUDA-event duration, against the measured HBM copy bandwidth;
             `roofline_writer` does the same for the record writer pair, and `random_access`
             gives k-mers/s against the hash-table random-access bound (64 B per occurrence)
  cpu_baseline  the oracle (C++ restatement of the reference's sort + group graph build) on
             the first pairs of the same workload, all host threads
  batched    the 64-sample workload (genomes log-uniform 20 kbp - 2 Mbp, 10-60x single-end
             150 bp, k = 31) built one gx_job_run per sample and as one gx_batch_run pass
  long_k     the 50 Mbp workload (2 x 250 bp pairs at 20x, k = 55, 128-bit keys), plain build
  autotune   the autotuner's choice (algorithm x table fill) on a prefix of the workload,
             used by the timed builds; every candidate's time
  serving    a Poisson stream of jobs (genomes log-uniform 10 kbp - 5 Mbp, 30x, 2 x 150 bp
             pairs, k in {21, 31, 55}) through gx_serve_*, offered rate swept: p50/p99
             latency from arrival to completion and k-mers/s per rate

With --impl reference the oracle itself is the measured implementation (the reference is
Java 7 on Hyracks and cannot run on the box).  With N > 1 (torchrun) every rank builds its
own replica of the workload (the build does not shard across GPUs; replicas only).
"""
import argparse
import json
import os
import statistics
import subprocess
import threading
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-mers/s, bit-exact graph build, batched vs per-job, 1 GB300; p99 job latency"
UNIT = "k-mers/s"
CPU_SAMPLE_PAIRS = 120_000   # cpu_baseline sample (one run)
REF_STEP_PAIRS = 60_000      # --impl reference: sample per step
TUNE_PAIRS = 200_000         # autotuner sample: the first pairs of the workload
LAYOUT_PARTS = 16            # parts of the reference part layout measurement
# DRAM bytes per algorithmic byte of each roofline kernel, from its committed ncu capture
TRAFFIC_RATIOS = os.path.join(ROOT, "profiles", "traffic_ratios.json")
AGG_HEAD_BYTES = 112         # per read head in k_aggregate: Head read and written, HeadOut, its read's line
HEADOUT_BYTES = 48           # one HeadOut entry (uuid, two text offsets, position, counts)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(alg_bytes, kernel):
    """DRAM bytes of one launch of `kernel` (a key of profiles/traffic_ratios.json): its ncu
    capture ran a smaller case of the same workload, whose DRAM bytes per algorithmic byte scale
    to the full launch (the traffic grows in proportion to the occurrences and records)."""
    if not os.path.exists(TRAFFIC_RATIOS):
        return None
    with open(TRAFFIC_RATIOS) as f:
        ratio = json.load(f).get(kernel, {}).get("dram_bytes_per_algorithmic_byte")
    return None if ratio is None else ratio * alg_bytes


def aggregate_alg_bytes(st, k):
    """Bytes k_aggregate must move per launch: every occurrence's key and edge bits read once,
    each node's key, count/meta word and record offset written once, and per read head its
    Head entry (read and updated), its HeadOut entry and its read's line record."""
    kb = 8 if k <= 32 else 16
    return st["kmers"] * (kb + 2) + st["nodes"] * (kb + 12) + st["read_heads"] * AGG_HEAD_BYTES


def writer_alg_bytes(st, k, read_len, paired):
    """Bytes the record writer must move per launch: the records it writes, the compacted node
    arrays it reads (key, count/meta word, node offset) and, per read head, its HeadOut entry
    and the letters of the read and its mate."""
    kb = 8 if k <= 32 else 16
    letters = read_len * (2 if paired else 1)
    return st["record_bytes"] + st["nodes"] * (kb + 8 + 4) + st["read_heads"] * (HEADOUT_BYTES + letters)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        self.lines = []
        self.first = threading.Event()
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        if self.proc:
            def reader():
                for line in self.proc.stdout:
                    self.lines.append(line)
                    self.first.set()
            self.thread = threading.Thread(target=reader, daemon=True)
            self.thread.start()
            # nvidia-smi's start-up queries the GPU through the NVIDIA kernel module: let it finish first
            self.first.wait(timeout=10)
            time.sleep(0.25)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)
            self.out = "".join(self.lines)

    def summary(self):
        sm, mx, reasons = [], None, set()
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(text_sample, k, pairs, warm=False):
    from oracle import gx_oracle as go
    threads = os.cpu_count() or 1
    if warm:
        go.build_graph(text_sample[: len(text_sample) // 20], k, threads=threads, parts=threads)
    t0 = time.perf_counter()
    r = go.build_graph(text_sample, k, threads=threads, parts=threads)
    dt = time.perf_counter() - t0
    assert r.status == 0
    return {"value": r.kmers / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {pairs} pairs of the workload ({r.kmers} k-mer occurrences, a prefix whose "
                      f"tables are smaller than the whole run's, so the per-k-mer cost measured is a lower "
                      f"bound), oracle sort+group build, {threads} threads, {dt:.2f} s"}, r


def workload(max_pairs=None):
    from genomix_gb300 import synth
    return synth.pe_5mbp(max_pairs=max_pairs)


def batched_workload(n_samples=64):
    """The 64-sample batch, generated in a spawn pool (before any CUDA call)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    from genomix_gb300 import synth
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        return synth.batched_64(n_samples=n_samples, pool=ex)


def serving_workload(n_pool=48):
    """A pool of distinct serving jobs, generated in a spawn pool (before any CUDA call)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    from genomix_gb300 import synth
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        return [w for _, w in synth.serving_jobs(n_pool, 1.0, pool=ex)]


SERVE_RATES = (25, 50, 100, 200, 400, 800)  # offered jobs/s
SERVE_REQUESTS = 192                        # requests per rate, cycling through the job pool
SERVE_CLIENTS = 4                           # client threads submitting the arrivals


def pct(v, q):
    """The q-quantile of the values (nearest rank); None for none."""
    if not v:
        return None
    v = sorted(v)
    return v[min(len(v) - 1, int(q * len(v)))]


def bench_serving(ctx, works, rates=SERVE_RATES, n_req=SERVE_REQUESTS):
    """Poisson arrivals of graph-build jobs at each offered rate: client threads create each
    job at its arrival time (input copied from pinned host memory) and hand it to the server;
    the results stay on the device.  Latency runs from arrival to completion."""
    import threading
    import genomix_gb300 as gx
    from genomix_gb300 import synth
    pins = []
    for w in works:
        p = gx.PinnedBuffer(len(w.text))
        p.array()[:] = memoryview(w.text)
        pins.append(p)
    # jobs at or below the pool's median input size are "small", the rest "large"
    median_bytes = sorted(len(w.text) for w in works)[len(works) // 2]
    out = []
    with gx.Server(ctx) as srv:
        # warm the lanes (first passes grow the memory pool), untimed
        warm = []
        for q in range(min(8, len(works))):
            j = gx.GraphBuildJob(ctx, works[q].k)
            j.add_input(pins[q])
            warm.append((j, srv.submit(j)))
        for j, t in warm:
            assert srv.poll(t)[0] == 0
            j.close()
        for rate in rates:
            arr = synth.poisson_arrivals(n_req, rate, seed_sample=1)
            tickets, jobs, t_sub = [None] * n_req, [None] * n_req, [0.0] * n_req
            ready = [threading.Event() for _ in range(n_req)]
            t0 = time.perf_counter() + 0.01

            def submitter(first):
                for i in range(first, n_req, SERVE_CLIENTS):
                    dt = t0 + arr[i] - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                    q = i % len(works)
                    j = gx.GraphBuildJob(ctx, works[q].k)
                    j.add_input(pins[q])
                    jobs[i] = j
                    tickets[i] = srv.submit(j)
                    t_sub[i] = time.perf_counter()
                    ready[i].set()

            ths = [threading.Thread(target=submitter, args=(c,)) for c in range(SERVE_CLIENTS)]
            for th in ths:
                th.start()
            lat, kmers, t_end = [], 0, t0
            lat_small, lat_large, srv_small, cli_small = [], [], [], []
            for i in range(n_req):
                ready[i].wait()
                st, srv_ms = srv.poll(tickets[i])
                assert st == 0, st
                cli_ms = (t_sub[i] - (t0 + arr[i])) * 1e3  # arrival -> submitted (job made, input copied)
                lt = cli_ms + srv_ms  # arrival -> done
                lat.append(lt)
                if len(works[i % len(works)].text) <= median_bytes:
                    lat_small.append(lt)
                    srv_small.append(srv_ms)
                    cli_small.append(cli_ms)
                else:
                    lat_large.append(lt)
                t_end = max(t_end, t0 + arr[i] + lt / 1e3)
                kmers += jobs[i].stats()["kmers"]
                jobs[i].close()
            for th in ths:
                th.join()
            span = t_end - t0
            out.append({"offered_jobs_per_s": rate, "jobs": n_req, "achieved_jobs_per_s": n_req / span,
                        "kmers_per_s": kmers / span, "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                        "p50_small_ms": pct(lat_small, 0.5), "p99_small_ms": pct(lat_small, 0.99),
                        "p50_large_ms": pct(lat_large, 0.5), "p99_large_ms": pct(lat_large, 0.99),
                        "p99_small_server_ms": pct(srv_small, 0.99), "p99_small_client_ms": pct(cli_small, 0.99)})
        st = srv.stats()
    for p in pins:
        p.close()
    sustained = [r for r in out if r["achieved_jobs_per_s"] >= 0.9 * r["offered_jobs_per_s"]]
    top = max(sustained, key=lambda r: r["offered_jobs_per_s"]) if sustained else None
    return {"workload": "serving_pe150_30x_k21_31_55", "job_pool": len(works), "median_job_bytes": median_bytes,
            "mean_job_bytes": sum(len(w.text) for w in works) / len(works), "rates": out,
            "highest_sustained": top, "passes": st["batches"], "max_jobs_per_pass": st["max_batch_jobs"]}


def long_k_workload():
    """The 50 Mbp, 2 x 250 bp, k = 55 workload, generated in a spawn pool (before any CUDA call)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    from genomix_gb300 import synth
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        return synth.pe_50mbp(pool=ex)


def bench_long_k(ctx, w, steps, warmup, local, autotune=True):
    """The plain build of the long-k workload (128-bit keys), text resident in HBM."""
    import torch
    import genomix_gb300 as gx
    tune = ctx.autotune(sample_prefix(w.text, 50_000), w.k) if autotune else None
    d = torch.frombuffer(bytearray(w.text), dtype=torch.uint8).to(f"cuda:{local}")
    torch.cuda.synchronize()

    def step():
        job = gx.GraphBuildJob(ctx, w.k)
        job.add_input_device(d.data_ptr(), d.numel())
        job.run()
        st = job.stats()
        job.close()
        return st

    for _ in range(warmup):
        step()
    ctx.mark(8)
    sts = [step() for _ in range(steps)]
    ctx.mark(9)
    ms = ctx.elapsed_ms(8, 9) / steps
    st = sts[0]
    del d
    return {"workload": w.name, "genome_bp": w.genome_len, "pairs": w.reads, "k": w.k, "key_bits": st["key_bits"],
            "kmers": st["kmers"], "nodes": st["nodes"], "record_bytes": st["record_bytes"],
            "kmers_per_s": st["kmers"] / (ms / 1e3), "ms_per_build": ms,
            "phases_ms": {"parse": st["ms_parse"], "partition": st["ms_insert"], "aggregate": st["ms_aggregate"],
                          "write": st["ms_write"]},
            "autotune": tune}


def bench_batched(ctx, samples, steps, warmup, local):
    """The 64 samples built one job per launch sequence (gx_job_run each) and as one batch
    (gx_batch_run), text resident in HBM; k-mers/s of each over `steps` repetitions."""
    import torch
    import genomix_gb300 as gx
    dev = [torch.frombuffer(bytearray(w.text), dtype=torch.uint8).to(f"cuda:{local}") for w in samples]
    torch.cuda.synchronize()
    k = samples[0].k

    def make_jobs():
        jobs = []
        for d in dev:
            j = gx.GraphBuildJob(ctx, k)
            j.add_input_device(d.data_ptr(), d.numel())
            jobs.append(j)
        return jobs

    def plain():
        out = []
        for j in make_jobs():
            j.run()
            out.append(j.stats())
            j.close()
        return out

    def batched():
        jobs = make_jobs()
        sts = gx.batch_run(ctx, jobs)
        assert all(st == 0 for st in sts), sts
        out = [j.stats() for j in jobs]
        for j in jobs:
            j.close()
        return out

    for _ in range(warmup):
        ref = plain()
        got = batched()
    # every sample's graph is the same size both ways (the tests check the records themselves)
    for a, b in zip(ref, got):
        assert (a["nodes"], a["kmers"], a["read_heads"], a["record_bytes"]) == \
               (b["nodes"], b["kmers"], b["read_heads"], b["record_bytes"])
    torch.cuda.synchronize()
    ctx.mark(4)
    for _ in range(steps):
        plain()
    ctx.mark(5)
    ms_plain = ctx.elapsed_ms(4, 5) / steps
    ctx.mark(6)
    for _ in range(steps):
        got = batched()
    ctx.mark(7)
    ms_batched = ctx.elapsed_ms(6, 7) / steps
    kmers = sum(st["kmers"] for st in ref)
    del dev
    return {"workload": "batched_64_se150_k31", "samples": len(samples), "kmers": kmers,
            "input_bytes": sum(len(w.text) for w in samples),
            "nodes": sum(st["nodes"] for st in ref),
            "plain_kmers_per_s": kmers / (ms_plain / 1e3), "batched_kmers_per_s": kmers / (ms_batched / 1e3),
            "speedup": ms_plain / ms_batched, "ms_plain": ms_plain, "ms_batched": ms_batched,
            "buckets": sum(st["table_partitions"] for st in got), "passes": int(got[0]["attempts"]),
            "gpu_launches_plain": int(sum(st["kernel_launches"] for st in ref)),
            "gpu_launches_batched": int(got[0]["kernel_launches"]),
            "batched_phases_ms": {"parse": got[0]["ms_parse"], "partition": got[0]["ms_insert"],
                                  "aggregate": got[0]["ms_aggregate"], "write": got[0]["ms_write"]}}


def host_link(local, h2d_bytes, d2h_bytes, reps=3):
    """The host link's copy rates, measured with plain copies of the e2e step's sizes between
    pinned host memory and HBM (the best of `reps`)."""
    import torch

    dev = torch.empty(max(h2d_bytes, d2h_bytes), dtype=torch.uint8, device=f"cuda:{local}")
    host = torch.empty(max(h2d_bytes, d2h_bytes), dtype=torch.uint8, pin_memory=True)
    s = torch.cuda.current_stream()
    out = {}
    for name, n, dst, src in (("d2h_gbs", d2h_bytes, host, dev), ("h2d_gbs", h2d_bytes, dev, host)):
        best = None
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            dst[:n].copy_(src[:n], non_blocking=True)
            b.record(s)
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = n / (best / 1e3) / 1e9
    del dev, host
    return out


def bench_layout(ctx, w, d_text, warmup, pin, parts=LAYOUT_PARTS, reps=3):
    """The same build written into the reference's part layout (records regrouped by the
    reference's Kmer partitioner, one extra pass on the device): its cost beside the job's."""
    import genomix_gb300 as gx

    sts = []
    for i in range(max(1, warmup // 2) + reps):
        job = gx.GraphBuildJob(ctx, w.k, out_parts=parts, layout="reference", **pin)
        job.add_input_device(d_text.data_ptr(), d_text.numel())
        job.run()
        if i >= max(1, warmup // 2):
            sts.append(job.stats())
        job.close()
    ms = statistics.mean(s["ms_layout"] for s in sts)
    rb = sts[0]["record_bytes"]
    # records read once while indexed and once while copied, written once; 24 B of index per record
    alg = 3 * rb + 40 * sts[0]["nodes"]
    return {"parts": parts, "ms_regroup": ms, "ms_build": statistics.mean(s["ms_total"] for s in sts),
            "record_bytes": rb, "alg_gbs": alg / (ms / 1e3) / 1e9}


def compact_tune(t):
    """The autotuner's choice without its per-candidate list (that goes to --details)."""
    if not t:
        return t
    out = {k: t[k] for k in ("algorithm", "load_factor", "threads_per_read", "ms") if k in t}
    # the fastest of each tiling, so the line shows what the tiling dimension is worth
    best = {}
    for c in t.get("candidates", []):
        if c["algorithm"] == "partitioned" and c["ms"] >= 0:
            tp = c["threads_per_read"]
            best[tp] = min(best.get(tp, c["ms"]), c["ms"])
    return out | {"tried": len(t.get("candidates", [])), "best_ms_by_threads_per_read": best}


def compact_serving(srv):
    """Serving summary for the bench line: per offered rate [offered, achieved jobs/s, p50 ms,
    p99 ms], the highest sustained rate in full; the full per-rate records go to --details."""
    if not srv:
        return srv
    out = {k: v for k, v in srv.items() if k != "rates"}
    cols = ["offered_jobs_per_s", "achieved_jobs_per_s", "p50_ms", "p99_ms", "p99_small_ms", "p99_large_ms",
            "p99_small_server_ms", "p99_small_client_ms"]
    out["rates"] = [[None if r[c] is None else round(r[c], 2) for c in cols] for r in srv["rates"]]
    out["rates_columns"] = cols
    return out


def config_of(w, n):
    return {"workload": w.name, "genome_bp": w.genome_len, "pairs": w.reads, "read_len": 150, "k": w.k,
            "input_bytes": len(w.text), "parallelism": f"replicas{n}" if n > 1 else "single",
            "l2": "inputs and table larger than L2 (129 MB); no flush"}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    w = workload(args.max_pairs)
    sample = sample_prefix(w.text, REF_STEP_PAIRS)
    vals = []
    for i in range(args.warmup + args.steps):
        cb, r = cpu_baseline(sample, w.k, REF_STEP_PAIRS)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r.kmers / v * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/int64", "data": "synthetic (seeded)", "config": config_of(w, 1),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def sample_prefix(text, pairs):
    idx = -1
    for _ in range(pairs):
        idx = text.find(b"\n", idx + 1)
        if idx < 0:
            return text
    return text[: idx + 1]


def run_gb300(args, ws, rank, local):
    import torch
    import genomix_gb300 as gx

    w = workload(args.max_pairs)
    samples = None if args.no_batched else batched_workload()
    serve_pool = None if args.no_serving else serving_workload()
    w50 = None if args.no_long_k else long_k_workload()
    ctx = gx.Context(local)
    torch.cuda.set_device(local)
    # the autotuner picks algorithm and fill on a prefix of the workload (untimed)
    tune = None if (args.no_autotune or args.fill) else ctx.autotune(sample_prefix(w.text, TUNE_PAIRS), w.k)
    d_text = torch.frombuffer(bytearray(w.text), dtype=torch.uint8).to(f"cuda:{local}")
    torch.cuda.synchronize()

    pin = {"algorithm": "partitioned", "load_factor": args.fill} if args.fill else {}

    def step_device():
        job = gx.GraphBuildJob(ctx, w.k, **pin)
        job.add_input_device(d_text.data_ptr(), d_text.numel())
        job.run()
        st = job.stats()
        job.close()
        return st

    for _ in range(args.warmup):
        st0 = step_device()
    barrier(ws)
    torch.cuda.synchronize()
    stats = []
    with ClockSampler(local) as clk:
        ctx.mark(0)
        for _ in range(args.steps):
            stats.append(step_device())
        ctx.mark(1)
        ms = ctx.elapsed_ms(0, 1)
    torch.cuda.synchronize()
    barrier(ws)
    ms_max = max_over_ranks(ws, ms)
    kmers = stats[0]["kmers"]
    value = ws * args.steps * kmers / (ms_max / 1e3)

    # ---- e2e: host buffers through the C ABI ----
    pin_in = gx.PinnedBuffer(len(w.text))
    pin_in.array()[:] = memoryview(w.text)
    out_bytes = stats[0]["record_bytes"]
    outs = [gx.PinnedBuffer(out_bytes + 16), gx.PinnedBuffer(out_bytes + 16)]

    def run_e2e(n, stamps=None):
        """n jobs back to back, each: pinned text in, build, every record out into pinned memory.
        Job i's copy out (asynchronous emit) overlaps job i + 1's copy in and build; the two
        output buffers alternate.  `stamps` collects, per job, the host time of each call and
        the build's device time."""
        prev = None
        for i in range(n):
            t0 = time.perf_counter()
            job = gx.GraphBuildJob(ctx, w.k, **pin)
            job.add_input(pin_in)
            t1 = time.perf_counter()
            job.run()
            t2 = time.perf_counter()
            wr, more = job.emit_async(0, outs[i % 2].ptr, outs[i % 2].nbytes)
            assert not more and wr == out_bytes
            t3 = time.perf_counter()
            if prev is not None:
                prev.emit_wait()
                t4 = time.perf_counter()
                prev.close()
            else:
                t4 = t3
            t5 = time.perf_counter()
            if stamps is not None:
                stamps.append((t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4, job.stats()["ms_total"]))
            prev = job
        prev.emit_wait()
        prev.close()

    run_e2e(max(2, args.warmup // 2))
    barrier(ws)
    stamps = []
    ctx.mark(2)
    run_e2e(args.steps, stamps)
    ctx.mark(3)
    ms_e2e = max_over_ranks(ws, ctx.elapsed_ms(2, 3))
    e2e_steps_ms = {name: 1e3 * statistics.mean(s[q] for s in stamps) if q < 5 else statistics.mean(s[q] for s in stamps)
                    for q, name in enumerate(("input_copy", "build", "emit_queue", "wait_prev_copy", "close_prev",
                                              "build_device"))}
    e2e_value = ws * args.steps * kmers / (ms_e2e / 1e3)
    link = host_link(local, len(w.text), out_bytes)

    lay = None
    if not args.no_layout:
        lay = bench_layout(ctx, w, d_text, args.warmup, pin)
    bat = srv = None
    if samples is not None:
        bat = bench_batched(ctx, samples, args.steps, args.warmup, local)
        del samples
    if serve_pool is not None:
        srv = bench_serving(ctx, serve_pool)
    lk = None
    if w50 is not None:
        lk = bench_long_k(ctx, w50, args.steps, args.warmup, local, autotune=not args.no_autotune)
        del w50

    if rank != 0:
        return
    peak, peak_kind = peaks()
    ins_ms = statistics.mean(s["ms_insert"] for s in stats)
    wr_ms = statistics.mean(s["ms_write"] for s in stats)
    wr_bytes = writer_alg_bytes(stats[0], w.k, 150, True)
    achieved = wr_bytes / (wr_ms / 1e3) / 1e9
    traffic = profiled_traffic(wr_bytes, "k_emit_write_part+k_write_heads_part")
    agg_ms = statistics.mean(s["ms_aggregate"] for s in stats)
    agg_bytes = aggregate_alg_bytes(stats[0], w.k)
    agg_achieved = agg_bytes / (agg_ms / 1e3) / 1e9
    b_alg = len(w.text) + 64.0 * kmers + out_bytes
    job_ms = ms / args.steps
    cb = None
    if not args.no_cpu_baseline:
        cb, _ = cpu_baseline(sample_prefix(w.text, CPU_SAMPLE_PAIRS), w.k, CPU_SAMPLE_PAIRS)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8/int64", "data": "synthetic (seeded reads of the named shapes)",
        "config": config_of(w, ws),
        "reads_per_s": value / kmers * stats[0]["reads"],
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": len(w.text),
                "d2h_bytes_per_step": out_bytes, "ms_per_step": ms_e2e / args.steps,
                "pipelined": "job i's record copy to the host overlaps job i+1's input copy and build",
                "host_link": link,
                "link_bound_ms_per_step": (out_bytes / link["d2h_gbs"] + len(w.text) / link["h2d_gbs"]) / 1e6,
                "host_ms_per_step": e2e_steps_ms,
                "link_bound_note": "both copies through the host link one after the other: the bound if "
                                   "the link does not carry both directions at full rate at once"},
        "roofline": {"bound": "hbm", "kernel": "k_aggregate", "achieved": agg_achieved, "peak": peak,
                     "unit": "GB/s", "frac": agg_achieved / peak, "peak_kind": f"{peak_kind} copy bandwidth",
                     "traffic": profiled_traffic(agg_bytes, "k_aggregate"), "alg_bytes_per_launch": agg_bytes,
                     "ms_per_launch": agg_ms,
                     "unit_of_work": "k-mer occurrence aggregated (10 B read; 20 B per node and 112 B per read "
                                     "head written)"},
        "roofline_writer": {"bound": "hbm", "kernel": "k_emit_write_part + k_write_heads_part", "achieved": achieved,
                            "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                            "peak_kind": f"{peak_kind} copy bandwidth", "traffic": traffic,
                            "alg_bytes_per_launch": wr_bytes, "ms_per_launch": wr_ms,
                            "unit_of_work": "record byte written (plus its node and read-head inputs)"},
        "random_access": {"bound_kmers_per_s": peak * 1e9 / 64.0, "frac": value / ws / (peak * 1e9 / 64.0),
                          "note": "64 B per k-mer occurrence (one 32 B sector read + one written)"},
        "job_roofline": {"alg_bytes": b_alg, "achieved_gbs": b_alg / (job_ms / 1e3) / 1e9,
                         "frac": b_alg / (job_ms / 1e3) / 1e9 / peak},
        "phases_ms": {"parse": statistics.mean(s["ms_parse"] for s in stats), "partition": ins_ms,
                      "aggregate": agg_ms, "write": wr_ms,
                      "job": job_ms},
        "graph": {"kmers": kmers, "reads": stats[0]["reads"], "nodes": stats[0]["nodes"],
                  "read_heads": stats[0]["read_heads"], "record_bytes": out_bytes,
                  "table_slots": stats[0]["table_slots"], "max_probe": stats[0]["max_probe"]},
        "clocks": clk.summary(),
        "autotune": compact_tune(tune),
        "batched": bat,
        "serving": compact_serving(srv),
        "long_k": dict(lk, autotune=compact_tune(lk["autotune"])) if lk else None,
        "reference_layout": lay,
        "cpu_baseline": cb,
    }
    if args.details:
        with open(args.details, "w") as f:
            json.dump({"autotune": tune, "serving": srv, "long_k_autotune": lk["autotune"] if lk else None}, f)
    print(json.dumps(line), flush=True)
    pin_in.close()
    for b in outs:
        b.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-sample batched vs per-job measurement")
    ap.add_argument("--no-serving", action="store_true", help="skip the served-stream measurement")
    ap.add_argument("--no-autotune", action="store_true", help="run with the built-in settings")
    ap.add_argument("--no-long-k", action="store_true", help="skip the 50 Mbp k = 55 measurement")
    ap.add_argument("--no-layout", action="store_true", help="skip the reference part layout measurement")
    ap.add_argument("--fill", type=float, default=0.0,
                    help="partitioned build at this bucket fill instead of the autotuner's choice (profiling runs)")
    ap.add_argument("--details", default=None,
                    help="write the per-candidate and per-rate records to this JSON file")
    ap.add_argument("--max-pairs", type=int, default=None,
                    help="use only the first pairs of the workload (profiling captures)")
    args = ap.parse_args()
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gb300(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
