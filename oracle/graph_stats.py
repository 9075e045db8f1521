"""Oracle (test infrastructure): GraphStatistics.map restated over a graph-build record stream.

Follows genomix-hadoop/src/main/java/edu/uci/ics/genomix/hadoop/utils/GraphStatistics.java:78-131
(updateStats :133-141) with Node.inDegree/outDegree/degree (genomix-data/.../types/Node.java:
820-836, DIR.edgeTypesInDir: REVERSE = {RF, RR}, FORWARD = {FF, FR}), isPathNode (:846-848) and
calculateSeedScore (:859-862) for nodes of a graph build (no internal k-mer: kmer length = k).
Pure Python over the record bytes: for small cases only.
"""
import math
import struct
from collections import Counter, defaultdict

STATS = ("degree", "kmer_length", "coverage", "unflipped_read_ids", "flipped_read_ids", "seed_score")


def _records(rec):
    p, n = 0, len(rec)
    while p < n:
        rl, kl = struct.unpack_from(">ii", rec, p)
        yield rec[p + 8:p + 8 + kl], rec[p + 8 + kl:p + 8 + rl]
        p += 8 + rl


def _node(key, val):
    k = struct.unpack_from(">i", key, 0)[0]
    nb = (k + 3) // 4
    kbytes = key[4:4 + nb]
    q = 0
    active = val[q]
    q += 1
    edges = [[], [], [], []]
    for t in range(4):
        if active & (1 << t):
            (cnt,) = struct.unpack_from(">i", val, q)
            q += 4
            for _ in range(cnt):
                (kk,) = struct.unpack_from(">i", val, q)
                eb = (kk + 3) // 4
                edges[t].append(val[q + 4:q + 4 + eb])
                q += 4 + eb
    heads = [0, 0]
    for s in range(2):
        if active & (0x10 << s):
            assert val[q] == 1
            (cnt,) = struct.unpack_from(">i", val, q + 1)
            q += 5
            heads[s] = cnt
            for _ in range(cnt):
                flags = val[q]
                q += 9
                for _m in range(2 if flags & 1 else 1):
                    (L,) = struct.unpack_from(">i", val, q)
                    q += 4 + (L + 3) // 4
    (cov,) = struct.unpack(">f", val[q:q + 4])
    assert q + 4 == len(val)
    return k, kbytes, edges, heads, cov


def graph_stats(records):
    """{"totals": {...}, "maximum": {...}, "<name>-bins": Counter} as GraphStatistics' counters."""
    totals, maximum, bins = defaultdict(int), defaultdict(int), defaultdict(Counter)

    def update(name, v):
        bins[name][v] += 1
        totals[name] += v
        maximum[name] = max(maximum[name], v)

    for key, val in _records(records):
        k, kbytes, edges, heads, cov = _node(key, val)
        totals["nodes"] += 1
        out_deg = len(edges[0]) + len(edges[1])
        in_deg = len(edges[2]) + len(edges[3])
        covr = int(math.floor(cov + 0.5))  # Math.round(float)
        seed = k * (heads[0] + heads[1])
        seeded = -1000.0 <= cov <= 1000.0
        update("degree", in_deg + out_deg)
        update("kmer_length", k)
        update("coverage", covr)
        update("unflipped_read_ids", heads[0])
        update("flipped_read_ids", heads[1])
        if seeded:
            update("seed_score", seed)
        for t, name in enumerate(("FF", "FR", "RF", "RR")):
            totals["selfEdge-" + name] += sum(1 for e in edges[t] if e == kbytes)
        if in_deg == 1 and out_deg == 1:
            totals["pathNode"] += 1
        for d, deg in (("REVERSE", in_deg), ("FORWARD", out_deg)):
            if deg == 0:
                totals["tips-" + d] += 1
            else:
                update("kmer_length-with-" + d, k)
                update("coverage-with-" + d, covr)
                if seeded:
                    update("seed_score-with-" + d, seed)
        if in_deg == 0 and out_deg == 0:
            totals["tips-BOTH"] += 1
        if (in_deg == 0) != (out_deg == 0):
            totals["tips-ONE"] += 1
    return {"totals": dict(totals), "maximum": dict(maximum), "bins": {k: dict(v) for k, v in bins.items()}}
