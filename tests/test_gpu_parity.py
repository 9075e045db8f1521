"""GPU graph build vs the oracle and the reference's golden fixtures, through the C ABI.

Bit-exact: the comparison form is the sorted set of records with every edge list sorted
(the reference's own test treats the edge lists as unordered, BatchTestFilesTest.java:171);
record bytes, read-head order and coverage are compared exactly.
"""
import numpy as np
import pytest

from conftest import golden_cases, golden_expected, golden_input
import genomix_gb300 as gx
from genomix_gb300 import synth
from oracle import gx_oracle as go
import refcompare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = gx.Context(0)
    yield c
    c.close()


def gpu_build(ctx, text, k, **kw):
    job = gx.GraphBuildJob(ctx, k, **kw)
    job.add_input(text)
    job.run()
    rec = job.records()
    st = job.stats()
    job.close()
    return rec, st


def assert_same(ctx, text, k, threads=2, parts=3, **kw):
    rec, st = gpu_build(ctx, text, k, **kw)
    ref = go.build_graph(text, k, threads=threads, parts=parts)
    assert ref.status == 0
    assert st["nodes"] == ref.nodes
    assert st["kmers"] == ref.kmers
    assert st["reads"] == ref.reads
    assert st["read_heads"] == ref.read_heads
    assert go.normalize(rec) == go.normalize(ref.records)
    return rec, st


ALGOS = ["partitioned", "table"]


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("case", golden_cases(), ids=[c["name"] for c in golden_cases()])
def test_golden_fixtures(ctx, case, algo):
    rec, _ = gpu_build(ctx, golden_input(case["name"]), case["k"], algorithm=algo)
    text = gx.records_to_text(rec)
    exp = golden_expected(case["name"])
    refcompare.compare_unordered(exp, text)
    assert refcompare.strict_normal_form(text) == refcompare.strict_normal_form(exp)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("k", [3, 4, 5, 8, 15, 16, 21, 31, 32, 33, 36, 47, 55, 63, 64])
def test_random_single_end_all_k(ctx, k, algo):
    text = synth.small_random(100 + k, 300, max(k + 20, 70), k, genome_len=1500, err=0.02)
    assert_same(ctx, text, k, algorithm=algo)


@pytest.mark.parametrize("tpr", [2, 4, 32])
@pytest.mark.parametrize("k", [3, 4, 5, 8, 15, 16, 21, 31, 32, 33, 36, 47, 55, 63, 64])
def test_split_read_walk_all_k(ctx, k, tpr):
    """The partitioned build with each read's k-mer walk split over tpr threads (segments of
    its occurrences, edge bits carried across the cuts): the oracle's records for every k,
    including reads shorter than the number of segments."""
    text = synth.small_random(300 + k, 300, max(k + 20, 70), k, genome_len=1500, err=0.02)
    assert_same(ctx, text, k, algorithm="partitioned", threads_per_read=tpr)


@pytest.mark.parametrize("tpr", [2, 4, 8])
@pytest.mark.parametrize("k", [21, 31, 55])
def test_split_read_walk_paired(ctx, k, tpr):
    text = synth.small_random(400 + k, 400, 150, k, paired=True, genome_len=5000, err=0.01, n_rate=0.003)
    assert_same(ctx, text, k, algorithm="partitioned", threads_per_read=tpr)


def test_threads_per_read_must_be_a_power_of_two(ctx):
    for bad in (3, 6, 64, -1):
        with pytest.raises(gx.GraphBuildError):
            gx.GraphBuildJob(ctx, 31, threads_per_read=bad)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("k", [21, 31, 55])
def test_random_paired_with_n(ctx, k, algo):
    text = synth.small_random(200 + k, 400, 150, k, paired=True, genome_len=5000, err=0.01, n_rate=0.003)
    assert_same(ctx, text, k, algorithm=algo)


def test_palindromes_even_k(ctx):
    # tandem palindromic sequence: every k-mer for even k is close to its own reverse complement
    unit = b"ACGT" * 10 + b"AATT" * 10 + b"GGCC" * 5
    lines = [b"%d\t%s" % (4 * i + 2, unit[i % 7:] + unit[: i % 5]) for i in range(50)]
    text = b"\n".join(lines) + b"\n"
    for k in (4, 6, 8, 10):
        assert_same(ctx, text, k)


def test_high_multiplicity_repeats(ctx):
    # one 40-base unit repeated: few nodes with very high coverage and many read heads
    rng = np.random.default_rng(5)
    unit = "".join(rng.choice(list("ACGT"), 40))
    genome = unit * 60
    lines = []
    for i in range(3000):
        s = int(rng.integers(0, len(genome) - 120))
        lines.append(f"{4 * i + 2}\t{genome[s:s + 100]}\t{genome[s + 10:s + 110]}")
    text = ("\n".join(lines) + "\n").encode()
    for algo in ALGOS:
        rec, st = assert_same(ctx, text, 21, algorithm=algo)
        assert st["read_heads"] <= 6000  # heads merge into few nodes


def test_many_heads_one_partition(ctx):
    # every read starts with the same k-mer: one node carries > 1024 read heads
    rng = np.random.default_rng(9)
    prefix = "ACGTTGCAAGGCTTCA"
    lines = []
    for i in range(2500):
        tail = "".join(rng.choice(list("ACGT"), 30))
        lines.append(f"{i}\t{prefix}{tail}")
    text = ("\n".join(lines) + "\n").encode()
    for algo in ALGOS:
        assert_same(ctx, text, 11, algorithm=algo)


def test_duplicate_read_ids(ctx):
    text = b"5\tACGTACGTAC\n5\tACGTACGTAC\n5\tACGTACGGGC\n7\tACGTACGTAC\n"
    assert_same(ctx, text, 5)


def test_lowercase_crlf_and_missing_final_newline(ctx):
    text = b"1\tacgtacGGTA\r\n2\tGGCATTaCCA\t\tx\r3\tTTGACCAGTA\tACGNNAC\n4\tCCCCGGGGAA"
    ref = go.build_graph(text, 5)
    assert ref.status == 2  # line 2 has 4 fields
    with pytest.raises(gx.GraphBuildError):
        gpu_build(ctx, text, 5)
    text = b"1\tacgtacGGTA\r\n2\tGGCATTaCCA\t\t\r3\tTTGACCAGTA\tACGNNAC\n4\tCCCCGGGGAA"
    assert_same(ctx, text, 5)


@pytest.mark.parametrize("text,status,line", [
    (b"1\tACGTACG\n2\n", "GX_EINVAL_LINE", 2),
    (b"1\tACGTA\tCC\tGG\n", "GX_EINVAL_LINE", 1),
    (b"x\tACGTA\n", "GX_EINVAL_NUMBER", 1),
    (b"1\tACGTA\n+\tAC\n", "GX_EINVAL_NUMBER", 2),
    (b"99999999999999999999\tACGTA\n", "GX_EINVAL_NUMBER", 1),
    (b"-1\tACGTA\n", "GX_EREADID_RANGE", 1),
    (b"34359738368\tACGTA\n", "GX_EREADID_RANGE", 1),
    (b"1\tACGTAC\n2\tACG\n", "GX_EREAD_TOO_SHORT", 2),
    (b"1\tACGTAC\n2\tACGTAC\tACG\n", "GX_EREAD_TOO_SHORT", 2),
    (b"1\tACGTAC\n\n3\tACGTAC\n", "GX_EINVAL_LINE", 2),
    (b"1\tACGTAC\n2\tAC\n3\t\n", "GX_EREAD_TOO_SHORT", 2),
])
def test_parse_errors(ctx, text, status, line):
    ref = go.build_graph(text, 3)
    assert gx._lib.STATUS_NAMES[ref.status] == status and ref.error_line == line
    with pytest.raises(gx.GraphBuildError) as e:
        gpu_build(ctx, text, 3)
    assert e.value.name == status
    assert e.value.line == line


def test_invalid_mates_and_unchecked_read_id(ctx):
    # no valid mate: the read id is never range-checked; N drops the whole mate
    text = b"34359738368\tNNNN\n2\tACGNT\tACGTTA\n3\t\tACGTTGCA\n"
    assert_same(ctx, text, 3)


def test_empty_input(ctx):
    job = gx.GraphBuildJob(ctx, 21)
    job.run()
    assert job.records() == b""
    assert job.stats()["nodes"] == 0
    job.close()
    rec, st = gpu_build(ctx, b"1\tNNNNNNNNNNNNNNNNNNNNNN\n", 5)
    assert rec == b"" and st["nodes"] == 0


def test_multiple_inputs_and_parts(ctx):
    a = synth.small_random(11, 200, 80, 21)
    b = synth.small_random(12, 200, 80, 21)
    job = gx.GraphBuildJob(ctx, 21, out_parts=4)
    job.add_input(a[:-1])  # a file without its final newline
    job.add_input(b)
    job.run()
    parts = [job.records(q) for q in range(4)]
    whole = job.records()
    assert b"".join(parts) == whole
    chunked = job.records(2, chunk=500)
    assert chunked == parts[2]
    job.close()
    ref = go.build_graph(a + b, 21)
    assert go.normalize(whole) == go.normalize(ref.records)


def test_device_input(ctx):
    torch = pytest.importorskip("torch")
    text = synth.small_random(21, 500, 120, 31, paired=True, genome_len=4000)
    t = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()
    job = gx.GraphBuildJob(ctx, 31)
    job.add_input_device(t.data_ptr(), t.numel(), keepalive=t)
    job.run()
    rec = job.records()
    job.close()
    ref = go.build_graph(text, 31)
    assert go.normalize(rec) == go.normalize(ref.records)


def test_fastq_input(ctx):
    rng = np.random.default_rng(4)
    n, L = 300, 90
    g = "".join(rng.choice(list("ACGT"), 3000))
    fq1, fq2 = [], []
    for i in range(n):
        s = int(rng.integers(0, 2800))
        fq1.append(f"@r{i}\n{g[s:s + L]}\n+\n{'?' * L}\n")
        fq2.append(f"@r{i}\n{g[s + 50:s + 50 + L]}\n+\n{'?' * L}\n")
    f1, f2 = "".join(fq1).encode(), "".join(fq2).encode()
    job = gx.GraphBuildJob(ctx, 21, input_kind="fastq", paired=True)
    job.add_input(f1, 0)
    job.add_input(f2, 1)
    job.run()
    rec = job.records()
    job.close()
    ref = go.build_graph(go.fastq_to_readid(f1, f2)[1], 21)
    assert go.normalize(rec) == go.normalize(ref.records)


def test_deterministic_output(ctx):
    text = synth.small_random(31, 2000, 150, 31, paired=True, genome_len=20000)
    a, _ = gpu_build(ctx, text, 31)
    b, _ = gpu_build(ctx, text, 31)
    assert a == b


@pytest.mark.parametrize("algo", ALGOS)
def test_high_load_factor_and_retry(ctx, algo):
    # partitioned: buckets aimed at 95% fill overflow their shared tables and are retried
    text = synth.small_random(41, 3000, 100, 21, genome_len=100000, err=0.05)
    assert_same(ctx, text, 21, load_factor=0.95, algorithm=algo)


def test_algorithms_agree_after_normalizing(ctx):
    text = synth.small_random(61, 4000, 150, 55, paired=True, genome_len=30000, err=0.01)
    a, _ = gpu_build(ctx, text, 55, algorithm="partitioned")
    b, _ = gpu_build(ctx, text, 55, algorithm="table")
    assert go.normalize(a) == go.normalize(b)


@pytest.mark.parametrize("algo", ALGOS)
def test_medium_case_against_oracle(ctx, algo):
    w = synth.pe_5mbp(max_pairs=20000, genome_len=200_000)
    assert_same(ctx, w.text, 31, threads=4, parts=4, algorithm=algo)


def test_seqfile_of_gpu_records(ctx):
    text = synth.small_random(51, 300, 100, 21, paired=True)
    rec, _ = gpu_build(ctx, text, 21)
    assert gx.seqfile_read(gx.seqfile_write(rec, seed=1)) == rec


def test_job_outlives_its_context():
    text = synth.small_random(77, 200, 80, 21)
    c = gx.Context(0)
    job = gx.GraphBuildJob(c, 21)
    job.add_input(text)
    c.close()  # the job keeps the context alive
    job.run()
    rec = job.records()
    job.close()
    assert go.normalize(rec) == go.normalize(go.build_graph(text, 21).records)


def test_async_emit_pipeline(ctx):
    texts = [synth.small_random(80 + i, 1500, 120, 31, paired=True) for i in range(4)]
    want = [gpu_build(ctx, t, 31)[0] for t in texts]
    bufs = [gx.PinnedBuffer(max(len(r) for r in want) + 16) for _ in range(2)]
    prev = None
    got = [None] * 4
    for i, t in enumerate(texts):
        job = gx.GraphBuildJob(ctx, 31)
        job.add_input(t)
        job.run()
        w, more = job.emit_async(0, bufs[i % 2].ptr, bufs[i % 2].nbytes)
        assert not more and w == len(want[i])
        if prev is not None:
            pj, pi, pw = prev
            pj.emit_wait()
            got[pi] = bytes(bufs[pi % 2].array()[:pw])
            pj.close()
        prev = (job, i, w)
    pj, pi, pw = prev
    pj.close()  # destroy waits for the copy
    got[pi] = bytes(bufs[pi % 2].array()[:pw])
    assert got == want
    for b in bufs:
        b.close()


def test_super_bucket_overflow_falls_back_to_counting(ctx):
    """100,000 copies of one read: 70 distinct k-mers of 100,000 occurrences each crowd a few
    super buckets past the room the uncounted first scatter gives them, so the build counts its
    super buckets and scatters again; the result still equals the oracle's."""
    import random
    rnd = random.Random(11)
    read = "".join(rnd.choice("ACGT") for _ in range(100))
    text = "".join(f"{i}\t{read}\n" for i in range(100_000)).encode()
    ref = go.build_graph(text, 31, threads=8, parts=1)
    for algo in ("partitioned",):
        job = gx.GraphBuildJob(ctx, 31, algorithm=algo)
        job.add_input(text)
        job.run()
        st, rec = job.stats(), job.records()
        job.close()
        assert st["super_counted"] == 1
        assert (st["nodes"], st["kmers"], st["read_heads"]) == (ref.nodes, ref.kmers, ref.read_heads)
        assert go.normalize(rec) == go.normalize(ref.records)


def test_memory_limit_between_counted_and_uncounted_scatter():
    """A context whose memory limit holds the exact-count build but not the uncounted scatter's
    room per bucket (about 1.3 x the occurrences): the build counts first instead of failing,
    and its records are the oracle's."""
    text = synth.pe_5mbp(max_pairs=20_000).text
    ref = go.build_graph(text, 31, threads=8, parts=2)
    with gx.Context(0) as c:
        _, base = gpu_build(c, text, 31, algorithm="partitioned")
    n_occ = base["kmers"]
    # the uncounted pass asks for about 23 B per occurrence, the counted one for about 14
    with gx.Context(0, mem_limit=int(19 * n_occ)) as c:
        rec, st = gpu_build(c, text, 31, algorithm="partitioned")
    assert base["super_counted"] == 0 and st["super_counted"] == 1  # the counting pass ran
    assert (st["nodes"], st["kmers"], st["read_heads"]) == (ref.nodes, ref.kmers, ref.read_heads)
    assert go.normalize(rec) == go.normalize(ref.records)


@pytest.mark.parametrize("algo", ALGOS)
def test_long_reads_read_heads_from_global_memory(ctx, algo):
    """600 bp pairs: the read heads' sequences are longer than the head writer stages in shared
    memory, so every head reads its letters from global memory."""
    rng = np.random.Generator(np.random.PCG64(91))
    g = synth.random_genome(rng, 30_000)
    mates = synth.simulate_chunk(rng, g, 120, 600, True, 1400, 50, 0.01, 0.002)
    text = synth.readid_lines(0, mates).tobytes()
    assert_same(ctx, text, 31, algorithm=algo)


def test_mixed_read_lengths_in_one_job(ctx):
    """150 bp single reads and 300 bp pairs in one job (the head writer's slots follow the
    longest sequence; the 150 bp heads use part of theirs), and a text that starts and ends
    inside a staged chunk."""
    rng = np.random.Generator(np.random.PCG64(92))
    g = synth.random_genome(rng, 20_000)
    short = synth.simulate_chunk(rng, g, 400, 150, False, None, None, 0.01, 0.0)
    long_ = synth.simulate_chunk(rng, g, 200, 300, True, 700, 30, 0.01, 0.002)
    text = synth.readid_lines(0, short).tobytes() + synth.readid_lines(1000, long_).tobytes()
    assert_same(ctx, text, 25)
    # no trailing newline, and the last read's letters run to the end of the text
    assert_same(ctx, text[:-1], 25)
