"""The reference's part layout (gx_job_opts.layout = GX_LAYOUT_REFERENCE_PARTS) on the GPU.

KmerNodePairSequenceWriterFactory writes each record into the part that the M:N
hash-partitioning connector picked for its key (KmerPartitionComputerFactory.java:28-52).  With
this layout part q of a GPU job holds exactly the records of the oracle's part q (the oracle
routes groups with the same partitioner), for both aggregation algorithms, with one and two
counting-sort passes (up to 256 parts and above), and at full size every record sits in the part
its key hashes to while the whole record set stays that of the bucket layout.
"""
import os

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


def java_part(kmer_bytes, nparts):
    """KmerPartitionComputerFactory.hashBytes + partition, in Python integers."""
    h = 1
    for b in kmer_bytes:
        h = (31 * h + (b - 256 if b > 127 else b)) & 0xFFFFFFFF
    if h >= 1 << 31:
        h -= 1 << 32
    if h < 0:
        h = -(h + 1)
    return h % nparts


def build(ctx, text, k, parts, layout="reference", algorithm="partitioned"):
    job = gx.GraphBuildJob(ctx, k, out_parts=parts, layout=layout, algorithm=algorithm)
    job.add_input(text)
    job.run()
    return job


def check_parts_vs_oracle(ctx, text, k, parts, algorithms=("partitioned", "table")):
    ref = go.build_graph(text, k, threads=4, parts=parts)
    assert ref.status == 0
    po = ref.part_offsets
    for algo in algorithms:
        job = build(ctx, text, k, parts, algorithm=algo)
        assert job.stats()["nodes"] == ref.nodes
        for q in range(parts):
            mine = job.records(q)
            theirs = ref.records[po[q]:po[q + 1]]
            assert go.normalize(mine) == go.normalize(theirs), (algo, q)
        offs = job.part_offsets()
        assert offs[0] == 0 and offs[-1] == job.stats()["record_bytes"]
        job.close()


@pytest.mark.parametrize("parts", [2, 7, 300])
def test_plain_workload_parts_vs_oracle(ctx, parts):
    check_parts_vs_oracle(ctx, synth.plain_cpu().text, 21, parts)


def test_pe_5mbp_prefix_parts_vs_oracle(ctx):
    check_parts_vs_oracle(ctx, synth.pe_5mbp(max_pairs=15_000).text, 31, 8)


def test_long_k_prefix_parts_vs_oracle(ctx):
    check_parts_vs_oracle(ctx, synth.pe_50mbp(max_pairs=2_000).text, 55, 5)


def test_more_parts_than_records(ctx):
    text = b"1\tACGTACGTTGCAAGT\n"
    check_parts_vs_oracle(ctx, text, 5, 64)


def test_giant_record_reference_layout(ctx):
    """A node whose read heads make its record larger than one round's shared-memory stage."""
    import random
    rnd = random.Random(7)
    head = "".join(rnd.choice("ACGT") for _ in range(25))
    lines = []
    for i in range(6000):
        tail = "".join(rnd.choice("ACGT") for _ in range(75))
        lines.append(f"{i}\t{head}{tail}")
    text = ("\n".join(lines) + "\n").encode()
    check_parts_vs_oracle(ctx, text, 21, 5)


def test_empty_input_reference_layout(ctx):
    job = build(ctx, b"", 21, 4)
    assert job.part_offsets() == [0] * 5
    assert all(job.records(q) == b"" for q in range(4))
    job.close()


def test_full_size_reference_layout(ctx):
    w = synth.pe_5mbp()
    parts = 16
    base = build(ctx, w.text, w.k, parts, layout="buckets")
    job = build(ctx, w.text, w.k, parts)
    sb, sj = base.stats(), job.stats()
    assert (sj["nodes"], sj["read_heads"], sj["record_bytes"]) == (sb["nodes"], sb["read_heads"], sb["record_bytes"])
    # the same record set (digests add up over parts), emitted in small chunks
    from test_gpu_configs import job_digest
    assert job_digest(job, chunk=1 << 20) == job_digest(base)
    # every record in the part its key hashes to: the first and last records of each part
    offs = job.part_offsets()
    for q in range(parts):
        rec = job.records(q)
        assert len(rec) == offs[q + 1] - offs[q]
        keys = [key for key, _ in gx.iter_records(rec)]
        assert keys, q
        for key in keys[:2000] + keys[-200:]:
            assert java_part(key[4:], parts) == q
    # the graph statistics walk the regrouped records the same way
    gb, gj = base.graph_stats(), job.graph_stats()
    assert gj == gb
    base.close()
    job.close()


def test_batch_runs_reference_layout_jobs_solo(ctx):
    text = synth.plain_cpu().text
    ref = go.build_graph(text, 21, threads=4, parts=3)
    jobs = []
    for layout in ("reference", "buckets", "reference"):
        j = gx.GraphBuildJob(ctx, 21, out_parts=3, layout=layout)
        j.add_input(text)
        jobs.append(j)
    assert gx.batch_run(ctx, jobs) == [0, 0, 0]
    for j in (jobs[0], jobs[2]):
        for q in range(3):
            theirs = ref.records[ref.part_offsets[q]:ref.part_offsets[q + 1]]
            assert go.normalize(j.records(q)) == go.normalize(theirs)
    assert go.normalize(jobs[1].records()) == go.normalize(ref.records)
    for j in jobs:
        j.close()


def test_invalid_layout_options(ctx):
    with pytest.raises(gx.GraphBuildError) as e:
        gx.GraphBuildJob(ctx, 21, out_parts=2, layout="reference", plan="BUILD_READ_PARSER")
    assert e.value.name == "GX_EINVAL"
    with pytest.raises(gx.GraphBuildError) as e:
        gx.GraphBuildJob(ctx, 21, out_parts=65537, layout="reference")
    assert e.value.name == "GX_EINVAL"


def test_driver_part_files_match_reference_parts(ctx, tmp_path):
    text = synth.plain_cpu().text
    os.makedirs(tmp_path / "in")
    (tmp_path / "in" / "reads.txt").write_bytes(text)
    drv = gx.GenomixGpuDriver(0)
    drv.run_job({gx.graph.KMER_LENGTH: "21", gx.graph.INPUT_DIR: str(tmp_path / "in"),
                 gx.graph.OUTPUT_DIR: str(tmp_path / "out"), gx.graph.THREADS_PER_MACHINE: "3"})
    ref = go.build_graph(text, 21, threads=3, parts=3)
    for q in range(3):
        mine = gx.seqfile_read((tmp_path / "out" / f"part-{q}").read_bytes())
        theirs = ref.records[ref.part_offsets[q]:ref.part_offsets[q + 1]]
        assert go.normalize(mine) == go.normalize(theirs), q


def test_bulk_copy_wait_times_out_cleanly():
    """The regrouping's source bytes arrive by bulk copy with a bounded wait.  A context with the
    testing flag that withholds those copies makes every wait run out: the job returns
    GX_ETIMEOUT after about a second, and the device stays usable (a normal context then builds
    the same input in the same layout, equal to the oracle's parts)."""
    from genomix_gb300 import _lib
    text = synth.plain_cpu(max_reads=3000).text
    with gx.Context(0, test_flags=_lib.CTX_TEST_WITHHOLD_COPIES) as bad:
        job = gx.GraphBuildJob(bad, 21, out_parts=8, layout="reference")
        job.add_input(text)
        with pytest.raises(gx.GraphBuildError) as ei:
            job.run()
        assert ei.value.status == _lib.GX_ETIMEOUT
        job.close()
    with gx.Context(0) as good:
        job = gx.GraphBuildJob(good, 21, out_parts=8, layout="reference")
        job.add_input(text)
        job.run()
        ref = go.build_graph(text, 21, threads=4, parts=8)
        for q in range(8):
            got = job.records(part=q)
            want = ref.records[ref.part_offsets[q]:ref.part_offsets[q + 1]]
            assert go.normalize(got) == go.normalize(want), q
        job.close()
