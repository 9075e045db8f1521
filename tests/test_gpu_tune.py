"""The autotuner (gx_autotune): every candidate is timed, the fastest is kept for jobs at the
default settings, and whatever it picks, the records stay the oracle's."""
import pytest

import genomix_gb300 as gx
from genomix_gb300 import synth
from oracle import gx_oracle as go

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_results_stay_exact():
    sample = synth.pe_5mbp(max_pairs=20_000).text
    text = synth.small_random(91, 1500, 150, 31, paired=True)
    ref = go.build_graph(text, 31, threads=4, parts=2)
    with gx.Context(0) as ctx:
        r = ctx.autotune(sample, 31, repeats=2)
        assert len(r["candidates"]) == 15
        # both tilings of the k-mer walk are among the candidates
        assert {c["threads_per_read"] for c in r["candidates"] if c["algorithm"] == "partitioned"} == {1, 2, 4}
        assert r["algorithm"] in ("partitioned", "table") and r["ms"] > 0
        assert r["threads_per_read"] in (1, 2, 4)
        assert r["ms"] == min(c["ms"] for c in r["candidates"] if c["ms"] >= 0)
        # a job at the defaults runs with the choice; explicit settings are left alone
        for kw in ({}, {"algorithm": "partitioned", "load_factor": 0.3}, {"algorithm": "table"},
                   {"threads_per_read": 4}):
            job = gx.GraphBuildJob(ctx, 31, **kw)
            job.add_input(text)
            job.run()
            assert go.normalize(job.records()) == go.normalize(ref.records), kw
            job.close()
        # batched jobs at the defaults too
        jobs = []
        for _ in range(3):
            j = gx.GraphBuildJob(ctx, 31)
            j.add_input(text)
            jobs.append(j)
        assert gx.batch_run(ctx, jobs) == [0, 0, 0]
        for j in jobs:
            assert gx.records_digest(j.records()) == gx.records_digest(ref.records)
            j.close()
        ctx.autotune_clear()


def test_autotune_per_key_width():
    with gx.Context(0) as ctx:
        r55 = ctx.autotune(synth.pe_50mbp(max_pairs=3000).text, 55, repeats=1)
        assert r55["ms"] > 0
        assert {c["threads_per_read"] for c in r55["candidates"]} >= {1, 2, 4}
        text = synth.small_random(92, 400, 120, 55)
        job = gx.GraphBuildJob(ctx, 55)
        job.add_input(text)
        job.run()
        assert go.normalize(job.records()) == go.normalize(go.build_graph(text, 55).records)
        job.close()
