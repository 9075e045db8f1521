"""The BUILD_READ_PARSER plan on the GPU: one (Kmer, Node) record per k-mer occurrence in read
order, byte-identical to the oracle's parser tuples (oracle.gx_oracle.read_parser)."""
import pytest

from conftest import golden_cases, golden_input
import genomix_gb300 as gx
from genomix_gb300 import synth
from oracle import gx_oracle as go

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = gx.Context(0)
    yield c
    c.close()


def dump(ctx, text, k, **kw):
    j = gx.GraphBuildJob(ctx, k, plan="BUILD_READ_PARSER", **kw)
    j.add_input(text)
    j.run()
    rec, st = j.records(), j.stats()
    j.close()
    return rec, st


@pytest.mark.parametrize("case", golden_cases(), ids=[c["name"] for c in golden_cases()])
def test_parser_golden_inputs(ctx, case):
    text = golden_input(case["name"])
    st, _, occ, ref = go.read_parser(text, case["k"])
    assert st == 0
    rec, s = dump(ctx, text, case["k"])
    assert rec == ref
    assert s["nodes"] == occ == s["kmers"]


@pytest.mark.parametrize("k", [3, 5, 21, 31, 32, 33, 55, 64])
def test_parser_random(ctx, k):
    text = synth.small_random(600 + k, 300, 100, k, paired=True, n_rate=0.002)
    st, _, occ, ref = go.read_parser(text, k)
    assert st == 0
    rec, s = dump(ctx, text, k, out_parts=3)
    assert rec == ref


def test_parser_chunked_emit_and_errors(ctx):
    text = synth.small_random(700, 2000, 120, 25)
    _, _, _, ref = go.read_parser(text, 25)
    j = gx.GraphBuildJob(ctx, 25, plan="BUILD_READ_PARSER", out_parts=4)
    j.add_input(text)
    j.run()
    assert b"".join(j.records(part=q, chunk=1000) for q in range(4)) == ref
    j.close()
    bad = b"1\tACGTACGTAC\n2\tACG\n"
    st, line, _, _ = go.read_parser(bad, 5)
    j = gx.GraphBuildJob(ctx, 5, plan="BUILD_READ_PARSER")
    j.add_input(bad)
    with pytest.raises(gx.GraphBuildError):
        j.run()
    assert j.stats()["error_line"] == line == 2
    j.close()


def test_parser_driver_writes_kmer_keyed_files(ctx, tmp_path):
    text = synth.small_random(701, 200, 80, 21)
    (tmp_path / "in").mkdir()
    (tmp_path / "in" / "reads.readids").write_bytes(text)
    drv = gx.GenomixGpuDriver(0)
    drv.run_job({gx.graph.KMER_LENGTH: "21", gx.graph.INPUT_DIR: str(tmp_path / "in"),
                 gx.graph.OUTPUT_DIR: str(tmp_path / "out"), gx.graph.THREADS_PER_MACHINE: "2"},
                plan="BUILD_READ_PARSER")
    data = b"".join(gx.seqfile_read((tmp_path / "out" / f"part-{q}").read_bytes()) for q in range(2))
    assert data == go.read_parser(text, 21)[3]
    assert b"edu.uci.ics.genomix.data.types.Kmer" in (tmp_path / "out" / "part-0").read_bytes()[:100]
