"""Seeded synthetic sequencing workloads for the graph build.

Five workload shapes (the reference publishes no benchmark data set, so these stand alone):

  plain_cpu    50 kbp uniform genome, 10,000 x 100 bp single-end reads (20x), 0.5% errors, k=21
  pe_5mbp      5 Mbp genome at GC 50% with 10 distinct 1 kbp segments x 10 copies, 2x150 bp pairs,
               insert N(500, 50), 833,333 pairs (50x), 1% errors, 0.01% N bases, k=31
  pe_50mbp     50 Mbp genome at GC 41% with 2.5 Mbp of 300 bp units x 20 copies, 2x250 bp pairs,
               insert N(600, 60), 2,000,000 pairs (20x), error rising 0.2% -> 1.5% along the read, k=55
  batched_64   64 samples: genome log-uniform 20 kbp - 2 Mbp, GC U[0.35, 0.60], coverage U[10, 60],
               150 bp single-end, 0.5% errors, k=31
  serving      jobs: genome log-uniform 10 kbp - 5 Mbp, 30x, 2x150 pairs, insert N(400, 40),
               0.8% errors, k drawn from {21, 31, 55}, Poisson arrivals

Generator: numpy Generator(PCG64(seed)), seed = 20261203 + 1000 * config + sample.  Reads are
taken from the forward strand or reverse-complemented with p = 0.5; a substitution goes to
one of the three other bases uniformly; FASTQ qualities are a constant Phred 30 ('?');
record i carries readId 4*i + 2, the id the reference driver gives FASTQ record i.
"""
import numpy as np

SEED_BASE = 20261203
LUT = np.frombuffer(b"ACGT", dtype=np.uint8)
CHUNK = 65536  # reads per generation chunk


def rng_for(config, sample=0):
    return np.random.Generator(np.random.PCG64(SEED_BASE + 1000 * config + sample))


def random_genome(rng, length, gc=0.5):
    p = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
    return rng.choice(4, size=int(length), p=p).astype(np.uint8)


def plant_repeats(rng, genome, unit_len, copies, total_len):
    """Writes copies of random units over block-aligned, non-overlapping positions."""
    units = max(1, int(round(total_len / (unit_len * copies))))
    blocks = len(genome) // unit_len
    slots = rng.choice(blocks, size=min(blocks, units * copies), replace=False)
    for u in range(units):
        seg = rng.integers(0, 4, size=unit_len, dtype=np.uint8)
        for c in range(copies):
            i = u * copies + c
            if i >= len(slots):
                break
            s = int(slots[i]) * unit_len
            genome[s:s + unit_len] = seg
    return genome


def revcomp(codes):
    return (3 - codes[..., ::-1]).astype(np.uint8)


def _errors(rng, codes, rate):
    """Substitutions: rate is a scalar or a per-position vector."""
    n, L = codes.shape
    r = np.asarray(rate, dtype=np.float32)
    hit = rng.random((n, L), dtype=np.float32) < r
    shift = rng.integers(1, 4, size=(n, L), dtype=np.uint8)
    codes = np.where(hit, (codes + shift) & 3, codes).astype(np.uint8)
    return codes


def simulate_chunk(rng, genome, n, read_len, paired, frag_mu=None, frag_sd=None, err=0.0, n_rate=0.0):
    """n reads (or pairs) as ASCII uint8 arrays (n, L): mate1[, mate2]."""
    G = len(genome)
    L = read_len
    if paired:
        f = np.rint(rng.normal(frag_mu, frag_sd, size=n)).astype(np.int64)
        f = np.clip(f, L, G)
    else:
        f = np.full(n, L, dtype=np.int64)
    start = (rng.random(n) * (G - f + 1)).astype(np.int64)
    flip = rng.random(n) < 0.5
    ar = np.arange(L, dtype=np.int64)
    # mate 1: first L bases of the fragment on its strand; mate 2: rc of its last L bases
    fwd1 = genome[start[:, None] + ar]
    rev1 = revcomp(genome[(start + f - L)[:, None] + ar])  # first L of rc(fragment)
    m1 = np.where(flip[:, None], rev1, fwd1)
    out = [m1]
    if paired:
        # fragment strand forward: mate2 = rc(last L); reversed: mate2 = rc(last L of rc(frag)) = first L
        m2 = np.where(flip[:, None], genome[start[:, None] + ar], rev1)
        out.append(m2)
    res = []
    for m in out:
        m = _errors(rng, m, err)
        ch = LUT[m]
        if n_rate > 0:
            ch = np.where(rng.random(m.shape, dtype=np.float32) < n_rate, np.uint8(ord("N")), ch)
        res.append(ch.astype(np.uint8))
    return res


def _digits(ids):
    """ASCII digit matrix (right-aligned in width w) and lengths of non-negative ints."""
    ids = np.asarray(ids, dtype=np.int64)
    nd = np.maximum(1, np.floor(np.log10(np.maximum(ids, 1))).astype(np.int64) + 1)
    w = int(nd.max()) if len(ids) else 1
    mat = np.zeros((len(ids), w), dtype=np.uint8)
    v = ids.copy()
    for c in range(w - 1, -1, -1):
        mat[:, c] = 48 + (v % 10)
        v //= 10
    return mat, nd, w


def readid_lines(first_id_index, mates):
    """readid text "id \\t seq [\\t mate]" for reads numbered from first_id_index (readId 4i+2)."""
    n, L = mates[0].shape
    ids = 4 * (first_id_index + np.arange(n, dtype=np.int64)) + 2
    mat, nd, w = _digits(ids)
    seq_bytes = sum(m.shape[1] + 1 for m in mates)
    line_len = nd + seq_bytes + 1  # + "\n"
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(line_len, out=off[1:])
    buf = np.empty(int(off[-1]), dtype=np.uint8)
    # id digits (right-aligned in the matrix, left-aligned in the line)
    cols = np.arange(w)
    take = cols[None, :] >= (w - nd)[:, None]
    dst = off[:-1, None] + (cols[None, :] - (w - nd)[:, None])
    buf[dst[take]] = mat[take]
    pos = off[:-1] + nd
    for m in mates:
        Lm = m.shape[1]
        buf[pos] = 9  # '\t'
        buf[(pos + 1)[:, None] + np.arange(Lm)] = m
        pos = pos + 1 + Lm
    buf[off[1:] - 1] = 10  # '\n'
    return buf


def fastq_records(first_id_index, mates_one_side):
    """FASTQ text of one mate file: @r{i} / seq / + / constant Phred 30."""
    n, L = mates_one_side.shape
    out = []
    q = b"?" * L
    for i in range(n):
        out.append(b"@r%d\n%s\n+\n%s\n" % (first_id_index + i, mates_one_side[i].tobytes(), q))
    return b"".join(out)


class Workload:
    def __init__(self, name, k, text, reads, pairs, genome_len, meta=None):
        self.name = name
        self.k = k
        self.text = text              # readid text (bytes)
        self.reads = reads            # single-end reads or pairs
        self.pairs = pairs
        self.genome_len = genome_len
        self.meta = meta or {}

    def __repr__(self):
        return f"Workload({self.name}, k={self.k}, {len(self.text)} bytes)"


def _build(rng, genome, n, read_len, paired, frag_mu, frag_sd, err, n_rate, max_reads=None):
    n = int(n if max_reads is None else min(n, max_reads))
    chunks = []
    for c0 in range(0, n, CHUNK):
        c = min(CHUNK, n - c0)
        mates = simulate_chunk(rng, genome, c, read_len, paired, frag_mu, frag_sd, err, n_rate)
        chunks.append(readid_lines(c0, mates).tobytes())
    return b"".join(chunks), n


def plain_cpu(max_reads=None):
    rng = rng_for(1)
    g = random_genome(rng, 50_000, 0.5)
    text, n = _build(rng, g, 10_000, 100, False, None, None, 0.005, 0.0, max_reads)
    return Workload("plain_cpu_50kbp_se100_k21", 21, text, n, False, len(g))


def pe_5mbp(max_pairs=None, genome_len=5_000_000):
    rng = rng_for(2)
    g = random_genome(rng, genome_len, 0.5)
    plant_repeats(rng, g, 1000, 10, 0.02 * genome_len)
    pairs = int(round(50 * genome_len / 300))
    text, n = _build(rng, g, pairs, 150, True, 500, 50, 0.01, 1e-4, max_pairs)
    return Workload("pe_5mbp_2x150_k31", 31, text, n, True, len(g))


def _err_ramp(L=250):
    pos = np.arange(1, L + 1, dtype=np.float64)
    return 0.002 + 0.013 * (pos - 1) / (L - 1)


_GENOMES = {}


def _pe50_genome(genome_len):
    """The 50 Mbp genome at GC 41% with 5% of its length in 300 bp units repeated 20 times."""
    if genome_len not in _GENOMES:
        rng = rng_for(3)
        g = random_genome(rng, genome_len, 0.41)
        plant_repeats(rng, g, 300, 20, 0.05 * genome_len)
        _GENOMES[genome_len] = g
    return _GENOMES[genome_len]


def _pe50_chunk(c, n, genome_len):
    """Pairs [c * CHUNK, c * CHUNK + n) of the long-k workload, from their own seed."""
    g = _pe50_genome(genome_len)
    rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([SEED_BASE + 3000, c])))
    mates = simulate_chunk(rng, g, n, 250, True, 600, 60, _err_ramp(250), 0.0)
    return readid_lines(c * CHUNK, mates).tobytes()


def pe_50mbp(max_pairs=None, genome_len=50_000_000, pool=None):
    """2 x 250 bp pairs at 20x, insert N(600, 60), substitutions rising from 0.2% to 1.5% along
    the read, k = 55.  Every CHUNK of pairs has its own seed, so `pool` (an executor) can
    generate the chunks in parallel with the same result."""
    pairs = int(round(20 * genome_len / 500))
    n = pairs if max_pairs is None else min(pairs, int(max_pairs))
    nch = (n + CHUNK - 1) // CHUNK
    cs = list(range(nch))
    ns = [min(CHUNK, n - c * CHUNK) for c in cs]
    if pool is None:
        parts = [_pe50_chunk(c, m, genome_len) for c, m in zip(cs, ns)]
    else:
        parts = list(pool.map(_pe50_chunk, cs, ns, [genome_len] * nch))
    return Workload("pe_50mbp_2x250_k55", 55, b"".join(parts), n, True, genome_len)


def batched_sample(s, scale=1.0):
    """Sample s of the 64-sample batch: genome log-uniform 20 kbp - 2 Mbp, GC U[0.35, 0.60],
    coverage U[10, 60], single-end 150 bp, 0.5% substitutions, k = 31."""
    rng = rng_for(4, s)
    G = int(np.exp(rng.uniform(np.log(20_000), np.log(2_000_000))) * scale)
    G = max(G, 2000)
    gc = rng.uniform(0.35, 0.60)
    cov = rng.uniform(10, 60)
    g = random_genome(rng, G, gc)
    n = int(round(cov * G / 150))
    text, n = _build(rng, g, n, 150, False, None, None, 0.005, 0.0)
    return Workload(f"batched_s{s}", 31, text, n, False, G, {"gc": gc, "coverage": cov})


def batched_64(n_samples=64, scale=1.0, pool=None):
    """64 independent single-end samples (scale < 1 shrinks every genome for tests); `pool`
    (an executor) generates them in parallel, with the same result."""
    if pool is None:
        return [batched_sample(s, scale) for s in range(n_samples)]
    return list(pool.map(batched_sample, range(n_samples), [scale] * n_samples))


def serving_job(i, scale=1.0, seed_sample=0):
    """Job i of the serving stream: genome log-uniform 10 kbp - 5 Mbp at 30x, 2 x 150 bp pairs,
    insert N(400, 40), 0.8% substitutions, k drawn from {21, 31, 55}."""
    r = rng_for(5, seed_sample * 100_000 + i)
    G = max(2000, int(np.exp(r.uniform(np.log(10_000), np.log(5_000_000))) * scale))
    k = int(r.choice([21, 31, 55]))
    g = random_genome(r, G, 0.5)
    pairs = int(round(30 * G / 300))
    text, n = _build(r, g, pairs, 150, True, 400, 40, 0.008, 0.0)
    return Workload(f"serve_{i}", k, text, n, True, G)


def poisson_arrivals(n_jobs, rate_per_s, seed_sample=0):
    """Arrival times (s) of a Poisson stream at rate_per_s."""
    rng = rng_for(5, 10_000 + seed_sample)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=n_jobs))


def serving_jobs(n_jobs, rate_per_s, scale=1.0, seed_sample=0, pool=None):
    """(arrival_s, Workload) for a Poisson stream of graph-build jobs; `pool` (an executor)
    generates the jobs in parallel, with the same result."""
    t = poisson_arrivals(n_jobs, rate_per_s, seed_sample)
    idx = list(range(n_jobs))
    if pool is None:
        works = [serving_job(i, scale, seed_sample) for i in idx]
    else:
        works = list(pool.map(serving_job, idx, [scale] * n_jobs, [seed_sample] * n_jobs))
    return [(float(t[i]), works[i]) for i in idx]


def small_random(seed, n_reads, read_len, k, paired=False, genome_len=2000, err=0.01, n_rate=0.0, gc=0.5):
    """Small seeded case for parity tests."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = random_genome(rng, genome_len, gc)
    mates = simulate_chunk(rng, g, n_reads, read_len, paired, read_len * 2 + 50, 20, err, n_rate)
    return readid_lines(0, mates).tobytes()
