"""Served graph builds (gx_serve_*): continuous batching over concurrent lanes.  Every result is
the same alone and in the mix: each served job's records equal its plain build's, exactly (as a
sorted set of records with sorted edge lists), whatever it was batched with.
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


def mix(n, seed=0):
    """Small jobs of the serving workload's shape (2x150 pairs, k in {21, 31, 55})."""
    return [w for _, w in synth.serving_jobs(n, rate_per_s=100.0, scale=0.004, seed_sample=seed)]


def alone(ctx, w):
    j = gx.GraphBuildJob(ctx, w.k)
    j.add_input(w.text)
    j.run()
    rec = j.records()
    j.close()
    return rec


def serve_all(ctx, works, **opts):
    jobs = []
    for w in works:
        j = gx.GraphBuildJob(ctx, w.k)
        j.add_input(w.text)
        jobs.append(j)
    with gx.Server(ctx, **opts) as srv:
        tickets = [srv.submit(j) for j in jobs]
        done = [srv.poll(t) for t in tickets]
        stats = srv.stats()
    recs = [j.records() if st == 0 else None for j, (st, _) in zip(jobs, done)]
    for j in jobs:
        j.close()
    return done, recs, stats


@pytest.mark.parametrize("lanes", [1, 2, 3])
def test_served_results_equal_alone(ctx, lanes):
    works = mix(14, seed=lanes)
    done, recs, stats = serve_all(ctx, works, lanes=lanes)
    assert [st for st, _ in done] == [0] * len(works)
    assert all(lat > 0 for _, lat in done)
    assert stats["jobs_done"] == len(works) and stats["jobs_waiting"] == 0
    for w, rec in zip(works, recs):
        assert go.normalize(rec) == go.normalize(alone(ctx, w)), w.name


def test_jobs_arriving_during_a_pass_are_batched(ctx):
    works = mix(12, seed=7)
    done, recs, stats = serve_all(ctx, works, lanes=1)
    assert [st for st, _ in done] == [0] * len(works)
    # one lane: the first pass starts with the first arrival, the rest queue up behind it
    assert stats["batches"] < len(works) and stats["max_batch_jobs"] > 1


def test_memory_budget_admits_one_job_at_a_time(ctx):
    works = mix(6, seed=11)
    done, recs, stats = serve_all(ctx, works, lanes=2, mem_budget=1)
    assert [st for st, _ in done] == [0] * len(works)
    assert stats["batches"] == len(works) and stats["max_batch_jobs"] == 1
    for w, rec in zip(works[:3], recs[:3]):
        assert go.normalize(rec) == go.normalize(alone(ctx, w))


def test_failing_job_in_the_mix(ctx):
    works = mix(5, seed=13)
    bad = b"12\tACGT\tAC\tGT\n"  # four fields
    jobs = []
    for w in works[:2]:
        j = gx.GraphBuildJob(ctx, w.k)
        j.add_input(w.text)
        jobs.append(j)
    jb = gx.GraphBuildJob(ctx, works[0].k)
    jb.add_input(bad)
    jobs.insert(1, jb)
    with gx.Server(ctx, lanes=1) as srv:
        tickets = [srv.submit(j) for j in jobs]
        done = [srv.poll(t) for t in tickets]
    assert [st for st, _ in done] == [0, 2, 0]  # GX_EINVAL_LINE for the bad one
    assert jb.stats()["error_line"] == 1
    assert go.normalize(jobs[2].records()) == go.normalize(alone(ctx, works[1]))
    for j in jobs:
        j.close()


def test_destroy_runs_queued_jobs_and_oracle_parity(ctx):
    works = mix(4, seed=17)
    jobs = []
    for w in works:
        j = gx.GraphBuildJob(ctx, w.k)
        j.add_input(w.text)
        jobs.append(j)
    srv = gx.Server(ctx, lanes=1)
    tickets = [srv.submit(j) for j in jobs]
    srv.close()  # waits for every queued job
    for w, j in zip(works, jobs):
        ref = go.build_graph(w.text, w.k, threads=2, parts=2)
        assert go.normalize(j.records()) == go.normalize(ref.records)
        j.close()
    assert len(tickets) == 4


def test_cancel_a_queued_job(ctx):
    """One lane busy with a large job; three small ones queue behind it and the middle one is
    withdrawn: its poll reports GX_ECANCELLED, the job is unrun, and the others' records equal
    their plain builds."""
    big = synth.pe_5mbp(max_pairs=300_000)
    works = mix(3, seed=19)
    jbig = gx.GraphBuildJob(ctx, big.k)
    jbig.add_input(big.text)
    jobs = []
    for w in works:
        j = gx.GraphBuildJob(ctx, w.k)
        j.add_input(w.text)
        jobs.append(j)
    with gx.Server(ctx, lanes=1) as srv:
        tb = srv.submit(jbig)
        tickets = [srv.submit(j) for j in jobs]
        assert srv.cancel(tickets[1])
        assert not srv.cancel(tickets[1])  # already withdrawn (done)
        done = [srv.poll(t) for t in tickets]
        assert srv.poll(tb)[0] == 0
        st = srv.stats()
        with pytest.raises(gx.GraphBuildError):
            srv.cancel(123456789)  # unknown ticket
    assert [s for s, _ in done] == [0, 11, 0]  # GX_ECANCELLED
    assert st["jobs_cancelled"] == 1 and st["jobs_done"] == 3
    for q in (0, 2):
        assert go.normalize(jobs[q].records()) == go.normalize(alone(ctx, works[q]))
    # the withdrawn job is the caller's again, unrun: it can still be built
    jobs[1].run()
    assert go.normalize(jobs[1].records()) == go.normalize(alone(ctx, works[1]))
    for j in jobs + [jbig]:
        j.close()


def test_pass_cap_keeps_small_jobs_out_of_a_large_pass(ctx):
    """A pass admits jobs up to pass_bytes of estimated device memory (its first job always):
    with a cap below two jobs' estimate every pass holds one job."""
    works = mix(6, seed=23)
    done, recs, stats = serve_all(ctx, works, lanes=1, pass_bytes=1)
    assert [st for st, _ in done] == [0] * len(works)
    assert stats["batches"] == len(works) and stats["max_batch_jobs"] == 1
    for w, rec in zip(works[:2], recs[:2]):
        assert go.normalize(rec) == go.normalize(alone(ctx, w))


def test_out_of_memory_batch_splits_in_halves():
    """A context whose run allocations above a limit fail as out of memory (the testing option):
    a batch whose buffers exceed it is split in halves until the pieces fit, and every job's
    records still equal its plain build's."""
    works = [synth.small_random(200 + i, 3000, 150, 31, paired=False, genome_len=40_000, err=0.005)
             for i in range(8)]
    limit = 12 * max(len(t) for t in works)  # one job's buffers fit, the whole batch's do not
    refs = []
    with gx.Context(0) as plain_ctx:
        for t in works:
            j = gx.GraphBuildJob(plain_ctx, 31)
            j.add_input(t)
            j.run()
            refs.append(j.records())
            j.close()
    with gx.Context(0, test_alloc_fail_above=limit) as c:
        jobs = []
        for t in works:
            j = gx.GraphBuildJob(c, 31)
            j.add_input(t)
            jobs.append(j)
        assert gx.batch_run(c, jobs) == [0] * len(works)
        passes = {j.stats()["ms_total"] for j in jobs}
        assert len(passes) > 1  # not one pass
        for j, ref in zip(jobs, refs):
            assert go.normalize(j.records()) == go.normalize(ref)
            j.close()
