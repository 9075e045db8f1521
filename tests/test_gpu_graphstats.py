"""Graph statistics on the GPU (gx_job_graph_stats) against GraphStatistics restated in Python
over the same records (oracle/graph_stats.py)."""
import pytest

from conftest import golden_cases, golden_input
import genomix_gb300 as gx
from genomix_gb300 import synth
from oracle import graph_stats as ogs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = gx.Context(0)
    yield c
    c.close()


def compare(g, ref):
    t, m, b = ref["totals"], ref["maximum"], ref["bins"]
    assert g["nodes"] == t.get("nodes", 0)
    assert g["path_nodes"] == t.get("pathNode", 0)
    assert g["tips_reverse"] == t.get("tips-REVERSE", 0) and g["tips_forward"] == t.get("tips-FORWARD", 0)
    assert g["tips_both"] == t.get("tips-BOTH", 0) and g["tips_one"] == t.get("tips-ONE", 0)
    assert g["self_edges"] == [t.get("selfEdge-" + e, 0) for e in ("FF", "FR", "RF", "RR")]
    names = {f: f for f in ogs.STATS}
    for d, i in (("REVERSE", 0), ("FORWARD", 1)):
        names[f"kmer_length-with-{d}"] = ("kmer_length_with", i)
        names[f"coverage-with-{d}"] = ("coverage_with", i)
        names[f"seed_score-with-{d}"] = ("seed_score_with", i)
    for name, f in names.items():
        h = g[f] if isinstance(f, str) else g[f[0]][f[1]]
        assert h["total"] == t.get(name, 0), name
        assert h["maximum"] == m.get(name, 0), name
        want = {v: c for v, c in b.get(name, {}).items() if v < gx._lib.STAT_BINS}
        assert h["bins"] == want, name
        assert h["above"] == sum(c for v, c in b.get(name, {}).items() if v >= gx._lib.STAT_BINS), name


def job_for(ctx, text, k, **kw):
    j = gx.GraphBuildJob(ctx, k, **kw)
    j.add_input(text)
    j.run()
    return j


@pytest.mark.parametrize("case", golden_cases(), ids=[c["name"] for c in golden_cases()])
def test_graph_stats_golden(ctx, case):
    j = job_for(ctx, golden_input(case["name"]), case["k"])
    compare(j.graph_stats(), ogs.graph_stats(j.records()))
    j.close()


@pytest.mark.parametrize("k,paired,algo", [(21, True, "partitioned"), (31, False, "table"), (55, True, "default")])
def test_graph_stats_random(ctx, k, paired, algo):
    text = synth.small_random(300 + k, 2500, 150, k, paired=paired, genome_len=4000, n_rate=0.001)
    j = job_for(ctx, text, k, algorithm=algo)
    compare(j.graph_stats(), ogs.graph_stats(j.records()))
    j.close()


def test_graph_stats_high_coverage_and_batched(ctx):
    # a short genome read many times: coverages past the histogram's dense range
    text = synth.small_random(404, 40000, 60, 15, genome_len=200)
    j = job_for(ctx, text, 15)
    g, ref = j.graph_stats(), ogs.graph_stats(j.records())
    assert g["coverage"]["maximum"] >= gx._lib.STAT_BINS
    compare(g, ref)
    j.close()
    jobs = []
    for s in range(3):
        jb = gx.GraphBuildJob(ctx, 21)
        jb.add_input(synth.small_random(500 + s, 800, 100, 21))
        jobs.append(jb)
    assert gx.batch_run(ctx, jobs) == [0, 0, 0]
    for jb in jobs:
        compare(jb.graph_stats(), ogs.graph_stats(jb.records()))
        jb.close()
