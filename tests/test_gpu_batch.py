"""Batched graph build (gx_batch_run) on the GPU: every job of a batch gets exactly the Node set
of its own plain build, checked against the oracle on small samples and against the plain GPU
build (itself parity-tested) on the 64-sample workload's shapes.
"""
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


def solo(ctx, text, k, **kw):
    job = gx.GraphBuildJob(ctx, k, **kw)
    job.add_input(text)
    job.run()
    rec, st = job.records(), job.stats()
    job.close()
    return rec, st


def batch(ctx, items, **kw):
    """items: (text, k[, job kwargs]) -> [(status, records, stats)]"""
    jobs = []
    for it in items:
        text, k = it[0], it[1]
        extra = dict(kw, **(it[2] if len(it) > 2 else {}))
        j = gx.GraphBuildJob(ctx, k, **extra)
        if isinstance(text, tuple) and text[0] == "device":
            j.add_input_device(text[1].data_ptr(), text[1].numel(), keepalive=text[1])
        elif text:
            j.add_input(text)
        jobs.append(j)
    sts = gx.batch_run(ctx, jobs)
    out = []
    for j, st in zip(jobs, sts):
        if st == 0:
            out.append((st, j.records(), j.stats()))
        else:
            out.append((st, None, j.stats()))
        j.close()
    return out


def same_graph(a_rec, b_rec):
    assert go.normalize(a_rec) == go.normalize(b_rec)


def test_batch_matches_oracle_per_sample(ctx):
    texts = [synth.small_random(100 + i, n, 100, 21, paired=(i % 2 == 1), genome_len=3000 + 700 * i,
                                n_rate=0.002 * (i % 3))
             for i, n in enumerate([300, 5, 1200, 80, 2500, 40, 700])]
    res = batch(ctx, [(t, 21) for t in texts])
    for t, (st, rec, s) in zip(texts, res):
        assert st == 0
        ref = go.build_graph(t, 21, threads=2, parts=2)
        assert s["nodes"] == ref.nodes and s["kmers"] == ref.kmers and s["reads"] == ref.reads
        assert s["read_heads"] == ref.read_heads
        same_graph(rec, ref.records)


@pytest.mark.parametrize("k", [31, 55])
def test_batch_matches_plain_builds(ctx, k):
    samples = synth.batched_64(n_samples=12, scale=0.05)
    res = batch(ctx, [(w.text, k) for w in samples])
    for w, (st, rec, s) in zip(samples, res):
        assert st == 0
        r2, s2 = solo(ctx, w.text, k)
        for f in ("lines", "reads", "kmers", "nodes", "read_heads", "record_bytes"):
            assert s[f] == s2[f], f
        same_graph(rec, r2)


def test_batch_empty_and_unterminated_inputs(ctx):
    torch = pytest.importorskip("torch")
    a = synth.small_random(7, 200, 90, 25)
    b = synth.small_random(8, 150, 90, 25)
    assert a.endswith(b"\n")
    dev = torch.frombuffer(bytearray(a[:-1]), dtype=torch.uint8).cuda()  # no final newline
    res = batch(ctx, [(b"", 25), (("device", dev), 25), (b, 25), (b"", 25)])
    assert [r[0] for r in res] == [0, 0, 0, 0]
    assert res[0][2]["nodes"] == 0 and res[3][2]["nodes"] == 0
    same_graph(res[1][1], go.build_graph(a, 25).records)
    same_graph(res[2][1], go.build_graph(b, 25).records)


def test_batch_mixed_k_and_algorithms(ctx):
    t1 = synth.small_random(11, 400, 120, 31)
    t2 = synth.small_random(12, 300, 120, 55, paired=True)
    t3 = synth.small_random(13, 500, 120, 31)
    res = batch(ctx, [(t1, 31), (t2, 55), (t3, 31, {"algorithm": "table"}), (t1, 21)])
    for (st, rec, _), (t, k) in zip(res, [(t1, 31), (t2, 55), (t3, 31), (t1, 21)]):
        assert st == 0
        same_graph(rec, go.build_graph(t, k).records)


def test_batch_parse_error_is_per_job(ctx):
    good = synth.small_random(21, 300, 100, 21)
    cut = good.index(b"\n", 500) + 1
    bad = good[:cut] + b"not-a-number\tACGTACGTACGTACGTACGTACGT\n" + good[cut:]
    res = batch(ctx, [(good, 21), (bad, 21), (good, 21)])
    assert res[0][0] == 0 and res[2][0] == 0
    assert res[1][0] == 3  # GX_EINVAL_NUMBER
    ref = go.build_graph(bad, 21)
    assert ref.status == 3 and res[1][2]["error_line"] == ref.error_line
    same_graph(res[0][1], res[2][1])


def test_batch_output_parts_and_chunked_emit(ctx):
    texts = [synth.small_random(31 + i, 800, 100, 31) for i in range(3)]
    jobs = []
    for t in texts:
        j = gx.GraphBuildJob(ctx, 31, out_parts=3)
        j.add_input(t)
        jobs.append(j)
    assert gx.batch_run(ctx, jobs) == [0, 0, 0]
    for t, j in zip(texts, jobs):
        whole = j.records()
        parts = b"".join(j.records(part=q, chunk=4096) for q in range(3))
        assert parts == whole
        same_graph(whole, go.build_graph(t, 31).records)
    for j in jobs:
        j.close()


def test_batch_jobs_outlive_each_other(ctx):
    texts = [synth.small_random(41 + i, 600, 100, 21) for i in range(4)]
    jobs = []
    for t in texts:
        j = gx.GraphBuildJob(ctx, 21)
        j.add_input(t)
        jobs.append(j)
    assert gx.batch_run(ctx, jobs) == [0, 0, 0, 0]
    # destroying jobs in any order keeps the shared record buffer alive for the others
    jobs[1].close()
    jobs[3].close()
    same_graph(jobs[2].records(), go.build_graph(texts[2], 21).records)
    jobs[0].close()
    same_graph(jobs[2].records(), go.build_graph(texts[2], 21).records)
    jobs[2].close()


def test_batch_hot_bucket_falls_back_to_counting(ctx):
    """A batch scatters without counting first; a sample made of 100,000 copies of one read
    crowds a few super buckets past their room, so the batch counts its samples and scatters
    again into exact offsets.  Every sample still equals its plain build and the oracle."""
    import random
    rnd = random.Random(5)
    read = "".join(rnd.choice("ACGT") for _ in range(100))
    hot = "".join(f"{i}\t{read}\n" for i in range(100_000)).encode()
    items = [(synth.small_random(600 + i, 800, 100, 31, genome_len=4000, err=0.01), 31) for i in range(3)]
    items.insert(1, (hot, 31))
    out = batch(ctx, items)
    assert out[1][2]["super_counted"] == 1
    for (text, k), (st, rec, _) in zip(items, out):
        assert st == 0
        want, _ = solo(ctx, text, k)
        assert go.normalize(rec) == go.normalize(want)
    ref = go.build_graph(hot, 31, threads=8, parts=1)
    assert go.normalize(out[1][1]) == go.normalize(ref.records)


@pytest.mark.parametrize("tpr", [1, 4])
def test_batch_split_read_walk(ctx, tpr):
    items = [(synth.small_random(700 + i, 600 + 200 * i, 150, 31, genome_len=3000 + 1000 * i, err=0.01), 31)
             for i in range(5)]
    for (text, k), (st, rec, stats) in zip(items, batch(ctx, items, threads_per_read=tpr)):
        assert st == 0 and stats["super_counted"] == 0  # no counting pass
        ref = go.build_graph(text, k, threads=4, parts=2)
        assert go.normalize(rec) == go.normalize(ref.records)
