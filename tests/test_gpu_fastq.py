"""FASTQ to readid on the GPU (gx_fastq_to_readid_gpu, and jobs with FASTQ input): byte for byte
the oracle's restatement of GenomixDriver.convertAndUploadFastqToHDFS (GenomixDriver.java:665-714)."""
import numpy as np
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


CASES = {
    "simple": (b"@a\nACGTACGTAC\n+\n??????????\n@b\nGGGTTTAAAC\n+\n??????????\n", None),
    "paired": (b"@a\nACGTACGTAC\n+\nIIIIIIIIII\n", b"@a\nTTTTGGGGCC\n+\nIIIIIIIIII\n"),
    "crlf_and_cr": (b"@a\r\nACGTAC \t\r\n+\r\nIIIIII\r@b\rgtgcaNN\r+\r??\r", None),
    "trim_both_ends": (b"@r\n  \tACGT ACGT\t \n+\nq\n", b"@r\n\x01\x1fTTTT\x7f \n+\nq\n"),
    "no_final_newline": (b"@a\nACGTACGT\n+\n????????\n@b\nCCCCAAAA", None),
    "partial_records": (b"l0\nl1\nl2\nl3\nl4\nl5", None),
    "two_lines": (b"@x\nACGT", None),
    "empty_lines": (b"\n\n\n\n\n\n\n\n\n", b"\n\n\n\n\n\n\n\n\n"),
    "non_ascii": (b"@a\n\xc3\xa9ACGT\xff\n+\n??\n", None),
    "empty": (b"", None),
}


@pytest.mark.parametrize("name", list(CASES))
def test_conversion_matches_oracle(ctx, name):
    m1, m2 = CASES[name]
    st, ref = go.fastq_to_readid(m1, m2)
    assert st == 0
    assert gx.fastq_to_readid_gpu(ctx, m1, m2) == ref
    assert gx.fastq_to_readid(m1, m2) == ref  # the host helper too


def test_pairing_error(ctx):
    with pytest.raises(gx.GraphBuildError) as e:
        gx.fastq_to_readid_gpu(ctx, b"@a\nAC\n+\n??\n", b"@a\nAC\n+\n")
    assert e.value.status == 12  # GX_EFASTQ_PAIRING


def test_large_paired_conversion(ctx):
    rng = synth.rng_for(2, 99)
    g = synth.random_genome(rng, 200_000)
    m1, m2 = synth.simulate_chunk(rng, g, 20_000, 150, True, 400, 40, 0.01, 0.001)
    f1, f2 = synth.fastq_records(0, m1), synth.fastq_records(0, m2)
    st, ref = go.fastq_to_readid(f1, f2)
    assert st == 0 and gx.fastq_to_readid_gpu(ctx, f1, f2) == ref


def test_job_with_several_fastq_files(ctx):
    rng = np.random.default_rng(5)
    files = []
    for f in range(3):
        g = "".join(rng.choice(list("ACGT"), 2000))
        a, b = [], []
        for i in range(120 + 40 * f):
            s = int(rng.integers(0, 1800))
            a.append(f"@r{i}\n{g[s:s + 80]}\n+\n{'?' * 80}\n")
            b.append(f"@r{i}\r\n{g[s + 40:s + 120]}  \r\n+\r\n{'?' * 80}\r\n")
        files.append(("".join(a).encode(), "".join(b).encode()))
    job = gx.GraphBuildJob(ctx, 25, input_kind="fastq", paired=True)
    for a, b in files:
        job.add_input(a, 0)
        job.add_input(b, 1)
    job.run()
    rec = job.records()
    job.close()
    text = b"".join(go.fastq_to_readid(a, b)[1] for a, b in files)  # read ids restart per file
    assert go.normalize(rec) == go.normalize(go.build_graph(text, 25).records)
