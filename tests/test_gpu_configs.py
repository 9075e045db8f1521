"""The five benchmark workloads on the GPU.

Bit-exact against the oracle where the oracle finishes in seconds: all of the plain CPU-sized
workload (10,000 single-end reads, k = 21), prefixes of the 5 Mbp paired-end (k = 31) and
50 Mbp long-k (k = 55) workloads, shrunken samples of the 64-sample batch and of the served
stream, and at full size the 5 Mbp workload in all its records and the 50 Mbp workload in a
seeded 5 % of them (one part of the reference part layout at a time).  At full size, also
through size-independent properties: the partitioned build, the
global-table build and the batched build of the same reads give the same order-independent
digest of their normalised records, the coverage of all nodes sums to the k-mer occurrences,
the read heads to the valid mates (no read id repeats in these workloads), and the digest
counts agree with the build's own statistics.
"""
import multiprocessing as mp
import os
import random
from concurrent.futures import ProcessPoolExecutor

import pytest

import genomix_gb300 as gx
from genomix_gb300 import synth
from oracle import gx_oracle as go

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = gx.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def pool():
    with ProcessPoolExecutor(max_workers=8, mp_context=mp.get_context("spawn")) as ex:
        yield ex


def build(ctx, text, k, algorithm="partitioned", out_parts=1):
    job = gx.GraphBuildJob(ctx, k, algorithm=algorithm, out_parts=out_parts)
    job.add_input(text)
    job.run()
    return job


def job_digest(job, chunk=1 << 30):
    """Digest of a job's records, streamed through a pinned buffer one chunk at a time (each
    chunk ends on a record boundary, and digests of disjoint record sets add up)."""
    tot = {"records": 0, "edges": 0, "heads": 0, "coverage": 0, "sum": 0, "xor_": 0}
    offs = job.part_offsets()
    cap = max(1, min(chunk, max(offs[q + 1] - offs[q] for q in range(job.out_parts))))
    buf = gx.PinnedBuffer(cap)
    job.rewind()
    for q in range(job.out_parts):
        while True:
            w, more = job.emit_into(q, buf.ptr, cap)
            if w:
                d = gx.records_digest(buf.ptr, w)
                for f in ("records", "edges", "heads", "coverage"):
                    tot[f] += d[f]
                tot["sum"] = (tot["sum"] + d["sum"]) & ((1 << 64) - 1)
                tot["xor_"] ^= d["xor_"]
            if not more:
                break
    buf.close()
    return tot


def check_vs_oracle(ctx, text, k, algorithms=("partitioned", "table")):
    ref = go.build_graph(text, k, threads=8, parts=4)
    assert ref.status == 0
    dref = gx.records_digest(ref.records)
    for algo in algorithms:
        job = build(ctx, text, k, algorithm=algo)
        st, rec = job.stats(), job.records()
        job.close()
        assert (st["nodes"], st["kmers"], st["reads"], st["read_heads"]) == \
               (ref.nodes, ref.kmers, ref.reads, ref.read_heads), algo
        assert go.normalize(rec) == go.normalize(ref.records), algo
        assert gx.records_digest(rec) == dref, algo


def check_full_size(ctx, w, parts):
    digests = []
    stats = None
    for algo in ("partitioned", "table"):
        job = build(ctx, w.text, w.k, algorithm=algo, out_parts=parts)
        st = job.stats()
        digests.append(job_digest(job))
        job.close()
        if stats is None:
            stats = st
        else:
            assert (st["nodes"], st["kmers"], st["read_heads"], st["record_bytes"]) == \
                   (stats["nodes"], stats["kmers"], stats["read_heads"], stats["record_bytes"])
    # the batched build of the same reads (a batch of one sample)
    job = gx.GraphBuildJob(ctx, w.k, out_parts=parts)
    job.add_input(w.text)
    assert gx.batch_run(ctx, [job]) == [0]
    digests.append(job_digest(job))
    job.close()
    assert digests[0] == digests[1] == digests[2]
    d = digests[0]
    assert d["records"] == stats["nodes"]
    assert d["coverage"] == stats["kmers"]
    assert d["heads"] == stats["read_heads"] == stats["reads"]
    return stats, d


def part_digest(job, q, buf, cap):
    """Digest of output part q of a job, streamed through a pinned buffer."""
    tot = {"records": 0, "edges": 0, "heads": 0, "coverage": 0, "sum": 0, "xor_": 0}
    job.rewind(q)
    while True:
        w, more = job.emit_into(q, buf.ptr, cap)
        if w:
            d = gx.records_digest(buf.ptr, w)
            for f in ("records", "edges", "heads", "coverage"):
                tot[f] += d[f]
            tot["sum"] = (tot["sum"] + d["sum"]) & ((1 << 64) - 1)
            tot["xor_"] ^= d["xor_"]
        if not more:
            return tot


def check_parts_vs_oracle(ctx, w, parts, which, full_bytes_part=None):
    """The whole-size build against the oracle, one part at a time: the GPU build writes its
    records in the reference's part layout (the reference's Kmer partitioner), and the oracle
    builds only the records of one part per run, so host memory holds one part.  Every part in
    `which` must carry the same digest (records, edges, heads, coverage and the record-hash sum
    and xor) as the oracle's part of the same number; part `full_bytes_part` is also compared
    byte for byte in normal form."""
    threads = os.cpu_count() or 8
    job = gx.GraphBuildJob(ctx, w.k, out_parts=parts, layout="reference")
    job.add_input(w.text)
    job.run()
    st = job.stats()
    offs = job.part_offsets()
    cap = max(offs[q + 1] - offs[q] for q in range(parts)) + 16
    buf = gx.PinnedBuffer(cap)
    nodes = 0
    try:
        for q in which:
            ref = go.build_graph(w.text, w.k, threads=threads, parts=parts, only_part=q)
            assert ref.status == 0
            assert (ref.kmers, ref.reads) == (st["kmers"], st["reads"])
            got = part_digest(job, q, buf, cap)
            assert got == gx.records_digest(ref.records), f"part {q} of {parts}"
            if q == full_bytes_part:
                job.rewind(q)
                w_, more = job.emit_into(q, buf.ptr, cap)
                assert not more
                mine = bytes(buf.array()[:w_])
                assert go.normalize(mine) == go.normalize(ref.records), f"part {q} bytes"
            nodes += ref.nodes
            del ref
    finally:
        buf.close()
        job.close()
    return st, nodes


# ---- configuration 1: 50 kbp genome, 10,000 x 100 bp single-end, k = 21 --------------------
def test_plain_cpu_workload_vs_oracle(ctx):
    w = synth.plain_cpu()
    assert w.reads == 10_000
    check_vs_oracle(ctx, w.text, 21)


# ---- configuration 2: 5 Mbp, 2 x 150 bp pairs, k = 31 ---------------------------------------
def test_pe_5mbp_prefix_vs_oracle(ctx):
    check_vs_oracle(ctx, synth.pe_5mbp(max_pairs=15_000).text, 31)


def test_pe_5mbp_full_size_properties(ctx):
    w = synth.pe_5mbp()
    stats, d = check_full_size(ctx, w, parts=8)
    assert stats["kmers"] == 197_007_720 and stats["reads"] == 1_641_731


def test_pe_5mbp_full_size_vs_oracle(ctx):
    """Every record of the benchmarked build (197,007,720 occurrences) against the oracle: all
    four parts of the reference part layout, part 0 byte for byte in normal form."""
    w = synth.pe_5mbp()
    st, nodes = check_parts_vs_oracle(ctx, w, 4, range(4), full_bytes_part=0)
    assert st["kmers"] == 197_007_720
    assert nodes == st["nodes"]


# ---- configuration 3: 50 Mbp, 2 x 250 bp pairs, k = 55 (128-bit keys) ------------------------
def test_pe_50mbp_prefix_vs_oracle(ctx, pool):
    check_vs_oracle(ctx, synth.pe_50mbp(max_pairs=5_000, pool=pool).text, 55)


def test_pe_50mbp_full_size_properties(ctx, pool):
    w = synth.pe_50mbp(pool=pool)
    assert w.reads == 2_000_000
    stats, d = check_full_size(ctx, w, parts=16)
    assert stats["key_bits"] == 128


def test_pe_50mbp_full_size_sampled_parts_vs_oracle(ctx, pool):
    """The 784 M-occurrence long-k build against the oracle on a seeded 5 % of its records: one
    part of 20 of the reference part layout (the oracle over every part would take minutes)."""
    w = synth.pe_50mbp(pool=pool)
    q = random.Random(20261204).randrange(20)
    check_parts_vs_oracle(ctx, w, 20, [q], full_bytes_part=q)


# ---- configuration 4: the 64-sample batch ---------------------------------------------------
def test_batched_samples_vs_oracle(ctx):
    samples = synth.batched_64(n_samples=64, scale=0.01)
    jobs = []
    for w in samples:
        j = gx.GraphBuildJob(ctx, 31)
        j.add_input(w.text)
        jobs.append(j)
    assert gx.batch_run(ctx, jobs) == [0] * 64
    for w, j in zip(samples, jobs):
        ref = go.build_graph(w.text, 31, threads=4, parts=2)
        assert gx.records_digest(j.records()) == gx.records_digest(ref.records), w.name
        j.close()


def test_batched_full_size_matches_plain(ctx, pool):
    samples = synth.batched_64(pool=pool)
    jobs = []
    for w in samples:
        j = gx.GraphBuildJob(ctx, 31)
        j.add_input(w.text)
        jobs.append(j)
    assert gx.batch_run(ctx, jobs) == [0] * 64
    for w, j in zip(samples, jobs):
        solo = build(ctx, w.text, 31)
        ds, dj = job_digest(solo), job_digest(j)
        assert ds == dj, w.name
        assert dj["coverage"] == j.stats()["kmers"]
        solo.close()
        j.close()


# ---- configuration 5: the served stream -----------------------------------------------------
def test_served_jobs_vs_oracle(ctx):
    works = [w for _, w in synth.serving_jobs(10, 100.0, scale=0.003, seed_sample=3)]
    jobs = []
    for w in works:
        j = gx.GraphBuildJob(ctx, w.k)
        j.add_input(w.text)
        jobs.append(j)
    with gx.Server(ctx, lanes=2) as srv:
        tickets = [srv.submit(j) for j in jobs]
        assert [srv.poll(t)[0] for t in tickets] == [0] * len(jobs)
    for w, j in zip(works, jobs):
        ref = go.build_graph(w.text, w.k, threads=4, parts=2)
        assert gx.records_digest(j.records()) == gx.records_digest(ref.records), w.name
        j.close()
