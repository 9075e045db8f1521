// gx_device.cuh — device-side building blocks of the graph build (sm_103a).
//
// K-mer values.  A k-mer is held as the integer V = sum_i code(base_i) * 4^i with the
// FIRST base least significant (A=0, C=1, G=2, T=3).  Writing V big-endian over
// nb = ceil(k/4) bytes gives exactly the reference's packed Kmer bytes (base i at bits
// 2*(i%4) of byte nb-1-i/4, Kmer.java:225-242), so Hadoop's unsigned lexicographic byte
// compare (BinaryComparable.compareTo) is the integer compare of V, and the canonical
// orientation test `fwd.compareTo(rc) <= 0` (ReadsKeyValueParserFactory.java:163,181) is
// `Vf <= Vr`.  k <= 32 uses a 64-bit word, 33 <= k <= 64 a 128-bit word.
//
// Edges.  Every edge the reference records (setEdgesForCurAndNext,
// ReadsKeyValueParserFactory.java:209-233) goes from a node X to a neighbour Y that
// differs from X by one base on one side.  With t = (a, b) the EDGETYPE (FF=0, FR=1,
// RF=2, RR=3; a = X's side, b = Y's) and e the extension base:
//     a = F:  S = X[1..k-1] + e,  Y = (b == F) ? S : revcomp(S)
//     a = R:  S = e + X[0..k-2],  Y = (b == R) ? S : revcomp(S)
// so (t, e) names Y uniquely and each node's four edge sets are exactly a 16-bit mask,
// bit 4*t + e.  This holds for palindromes (even k) too, where FF and FR of one base
// can both occur.  An occurrence j of a read contributes at most two bits:
//     to the next k-mer:  t = (d_j, d_{j+1}),            e = d_j == F ? x : 3 - x
//     from the previous:  t = (!d_j, !d_{j-1}),          e = d_j == R ? 3 - y : y
// with x = base j+k, y = base j-1 and d the orientation (F iff V_fwd <= V_rc).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gx {

typedef unsigned __int128 u128;

// ---- status words ---------------------------------------------------------------------
struct DevStatus {
    unsigned long long parse_err;  // min over (line << 8 | gx_status) of failing lines
    unsigned long long n_reads;    // valid mates
    unsigned long long n_occ;      // k-mer occurrences
    unsigned int table_full;       // inserts that found no slot within the probe limit
    unsigned int max_probe;        // longest probe sequence
    unsigned int big_head_parts;   // partitions whose read heads exceeded the in-CTA sort
    unsigned int cov_inexact;      // nodes with count >= 2^24
    unsigned int internal_err;     // emission size check failed (never expected)
    unsigned int max_seq;          // longest read or mate sequence of a kept read head (letters)
};

// ---- bases ------------------------------------------------------------------------------
// GeneCode.getCodeFromSymbol (GeneCode.java:29-50): A/a=0 C/c=1 G/g=2 T/t=3, other = 0.
__device__ __forceinline__ uint32_t base_code(uint32_t ch) {
    // (ch >> 1) & 3 maps A->0 C->1 G->3 T->2 for both cases; fix G/T with an xor.
    uint32_t c = (ch >> 1) & 3u;
    return c ^ (c >> 1);
}
__device__ __forceinline__ uint32_t base_code_checked(uint32_t ch) {
    uint32_t u = ch & 0xDFu;  // upper-case
    return (u == 'A' || u == 'C' || u == 'G' || u == 'T') ? base_code(ch) : 0u;
}
__device__ __forceinline__ bool is_acgt(uint32_t ch) {
    uint32_t u = ch & 0xDFu;
    return (u == 'A' || u == 'C' || u == 'G' || u == 'T') && (ch == u || ch == (u | 0x20u));
}

// ---- key traits -------------------------------------------------------------------------
template <class K> struct KeyOps;

template <> struct KeyOps<uint64_t> {
    static constexpr int BITS = 64;
    __device__ __forceinline__ static uint64_t mask(int k) { return k >= 32 ? ~0ULL : ((1ULL << (2 * k)) - 1); }
    __device__ __forceinline__ static uint64_t swap_pairs(uint64_t x) {
        return ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
    }
    // reverse complement of a k-mer value
    __device__ __forceinline__ static uint64_t revcomp(uint64_t v, int k) {
        uint64_t c = v ^ mask(k);
        return swap_pairs(__brevll(c)) >> (64 - 2 * k);
    }
    __device__ __forceinline__ static uint64_t hash(uint64_t v) {
        // MurmurHash3 64-bit finaliser
        v ^= v >> 33;
        v *= 0xff51afd7ed558ccdULL;
        v ^= v >> 33;
        v *= 0xc4ceb9fe1a85ec53ULL;
        v ^= v >> 33;
        return v;
    }
    __device__ __forceinline__ static uint32_t byte_at(uint64_t v, int i) { return (uint32_t)(v >> (8 * i)) & 0xffu; }
};

template <> struct KeyOps<u128> {
    static constexpr int BITS = 128;
    __device__ __forceinline__ static u128 mask(int k) {
        return k >= 64 ? ~(u128)0 : (((u128)1 << (2 * k)) - 1);
    }
    __device__ __forceinline__ static u128 revcomp(u128 v, int k) {
        u128 c = v ^ mask(k);
        uint64_t lo = (uint64_t)c, hi = (uint64_t)(c >> 64);
        uint64_t rlo = KeyOps<uint64_t>::swap_pairs(__brevll(hi));
        uint64_t rhi = KeyOps<uint64_t>::swap_pairs(__brevll(lo));
        u128 r = ((u128)rhi << 64) | rlo;
        return r >> (128 - 2 * k);
    }
    __device__ __forceinline__ static uint64_t hash(u128 v) {
        uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
        return KeyOps<uint64_t>::hash(lo ^ KeyOps<uint64_t>::hash(hi ^ 0x9e3779b97f4a7c15ULL));
    }
    __device__ __forceinline__ static uint32_t byte_at(u128 v, int i) { return (uint32_t)(v >> (8 * i)) & 0xffu; }
};

// Neighbour Y of node X for edge bit (t, e), see the file header.
template <class K>
__device__ __forceinline__ K edge_neighbor(K x, int t, int e, int k) {
    const int a = t >> 1, b = t & 1;
    K s;
    if (a == 0)
        s = (x >> 2) | ((K)e << (2 * (k - 1)));
    else
        s = ((x << 2) | (K)e) & KeyOps<K>::mask(k);
    const bool keep = (a == 0) ? (b == 0) : (b == 1);
    return keep ? s : KeyOps<K>::revcomp(s, k);
}

// ---- hash-table slots -------------------------------------------------------------------
// The stored key is V + 1 so that an all-zero slot is empty (the all-T k-mer, whose V + 1
// would overflow for k = 32 / 64, is never canonical).  meta: bits 0-15 edge mask,
// bit 16 an unflipped read head, bit 17 a flipped read head.
enum : uint32_t { META_UNFLIPPED = 1u << 16, META_FLIPPED = 1u << 17 };

struct __align__(16) Slot64 {
    unsigned long long key1;
    unsigned int count;
    unsigned int meta;
};
struct __align__(32) Slot128 {
    unsigned long long lo1, hi1;
    unsigned int count;
    unsigned int meta;
    unsigned long long pad;
};

template <class K> struct SlotOf;
template <> struct SlotOf<uint64_t> { typedef Slot64 T; };
template <> struct SlotOf<u128> { typedef Slot128 T; };

__device__ __forceinline__ ulonglong2 ld_cg16(const void *p) {
    ulonglong2 v;
    asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ void cas128(unsigned long long *p, unsigned long long clo, unsigned long long chi,
                                       unsigned long long vlo, unsigned long long vhi, unsigned long long &olo,
                                       unsigned long long &ohi) {
    asm volatile(
        "{\n\t.reg .b128 d, b, c;\n\t"
        "mov.b128 b, {%2, %3};\n\t"
        "mov.b128 c, {%4, %5};\n\t"
        "atom.relaxed.gpu.global.cas.b128 d, [%6], b, c;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(olo), "=l"(ohi)
        : "l"(clo), "l"(chi), "l"(vlo), "l"(vhi), "l"(p)
        : "memory");
}

// ---- bulk copies into shared memory (TMA, one thread issues) ---------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// an mbarrier that completes when `count` threads have arrived and the bytes they announced landed
__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier shared-memory accesses before its next bulk copy's writes
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// arrive on the barrier and announce `bytes` of bulk-copy data for its current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// 1-D bulk copy global -> shared: both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the barrier's phase `parity` to complete, for at most `limit` clock cycles; false if
// it did not.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

__device__ __forceinline__ void cas128_shared(void *p, unsigned long long clo, unsigned long long chi,
                                              unsigned long long vlo, unsigned long long vhi, unsigned long long &olo,
                                              unsigned long long &ohi) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile(
        "{\n\t.reg .b128 d, b, c;\n\t"
        "mov.b128 b, {%2, %3};\n\t"
        "mov.b128 c, {%4, %5};\n\t"
        "atom.shared.cas.b128 d, [%6], b, c;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(olo), "=l"(ohi)
        : "l"(clo), "l"(chi), "l"(vlo), "l"(vhi), "r"(a)
        : "memory");
}

// Insert one occurrence: count += 1, meta |= bits.  Linear probing inside the key's
// partition, at most `smask + 1` probes.  Returns the slot index or -1 (partition full).
__device__ __forceinline__ int table_insert(Slot64 *part, uint32_t smask, uint64_t key, uint32_t h, uint32_t bits,
                                            uint32_t &probes) {
    const unsigned long long want = (unsigned long long)key + 1ULL;
    uint32_t i = h & smask;
    for (uint32_t n = 0; n <= smask; ++n) {
        Slot64 *s = part + i;
        ulonglong2 v = ld_cg16(s);
        unsigned long long cur = v.x;
        uint32_t meta = (uint32_t)(v.y >> 32);
        if (cur == 0ULL) {
            cur = atomicCAS(&s->key1, 0ULL, want);
            if (cur == 0ULL) cur = want;
            meta = 0;
        }
        if (cur == want) {
            atomicAdd(&s->count, 1u);
            if ((meta & bits) != bits) atomicOr(&s->meta, bits);
            probes = n + 1;
            return (int)i;
        }
        i = (i + 1) & smask;
    }
    probes = smask + 1;
    return -1;
}

__device__ __forceinline__ int table_insert(Slot128 *part, uint32_t smask, u128 key, uint32_t h, uint32_t bits,
                                            uint32_t &probes) {
    const u128 want = key + 1;
    const unsigned long long wlo = (unsigned long long)want, whi = (unsigned long long)(want >> 64);
    uint32_t i = h & smask;
    for (uint32_t n = 0; n <= smask; ++n) {
        Slot128 *s = part + i;
        ulonglong2 kv = ld_cg16(&s->lo1);
        ulonglong2 cm = ld_cg16(&s->count);
        unsigned long long clo = kv.x, chi = kv.y;
        uint32_t meta = (uint32_t)(cm.x >> 32);
        if (clo != wlo || chi != whi) {
            // a 16-byte load is not guaranteed to be single-copy atomic: decide claim / hit /
            // occupied from the value the CAS returns, which is
            cas128(&s->lo1, 0ULL, 0ULL, wlo, whi, clo, chi);
            if (clo == 0ULL && chi == 0ULL) {
                clo = wlo;
                chi = whi;
            }
            meta = 0;
        }
        if (clo == wlo && chi == whi) {
            atomicAdd(&s->count, 1u);
            if ((meta & bits) != bits) atomicOr(&s->meta, bits);
            probes = n + 1;
            return (int)i;
        }
        i = (i + 1) & smask;
    }
    probes = smask + 1;
    return -1;
}

__device__ __forceinline__ uint64_t slot_key1(const Slot64 &s) { return s.key1; }

// partition of a key hash: the high 32 bits scaled to [0, P)
__device__ __forceinline__ uint32_t hash_partition(uint64_t h, uint32_t nparts) {
    return __umulhi((uint32_t)(h >> 32), nparts);
}

// ---- read heads ---------------------------------------------------------------------------
// One per valid mate, for its first k-mer.  uuid as ReadHeadInfo.makeUUID builds it
// (ReadHeadInfo.java:100-127): offset << 40 | library << 36 | mate << 35 | readId, with
// offset 0 (unflipped) or k-1 (flipped, ReadsKeyValueParserFactory.java:165-170) and
// library 0 (:98-106).
struct Head {
    uint32_t part;  // table partition of the first k-mer
    uint32_t slot;  // slot in the partition; after compaction, the node's rank
    unsigned long long uuid;
    unsigned long long klo, khi;  // canonical first k-mer (the partitioned build looks it up)
};

// A read head gathered into its bucket's order for the partitioned build's aggregation: the
// first k-mer, the uuid, and the read's text (offsets and lengths of the read and its mate),
// so one load brings the aggregation everything it needs.
struct __align__(16) HeadIn {
    unsigned long long uuid;
    unsigned long long klo, khi;      // canonical first k-mer
    unsigned long long s_off, m_off;  // text offsets of the read and of its mate
    uint32_t L, Lm;                   // read and mate lengths (Lm = 0: no mate sequence)
    uint32_t r;                       // read ordinal (orders read heads with equal uuids)
    uint32_t pad0;
    unsigned long long pad1;
};

// A read head as the record writer needs it, in the partition's output order (partitioned
// build): the head's byte position in its partition's records and, on the first head of a
// set, the set's size.
struct HeadOut {
    unsigned long long uuid;
    unsigned long long s_off, m_off;  // text offsets of the read and of its mate
    uint32_t pos;                     // partition-local byte position of the ReadHeadInfo
    uint32_t set_count;               // > 0 on the first head of a set: heads in the set
    uint32_t L, Lm;                   // read and mate lengths (Lm = 0: no mate sequence)
    uint32_t part;                    // the partition (fine bucket); HEAD_DROPPED for a duplicate
};
constexpr uint32_t HEAD_DROPPED = 0xffffffffu;

// ---- per-line parse output ---------------------------------------------------------------
struct LineRec {
    long long read_id;
    unsigned long long s0, s1;  // byte offsets of mate 0 / mate 1 sequences
    uint32_t l0, l1;            // their lengths
};
enum : uint8_t { LF_M0_VALID = 1, LF_HAS_M1 = 2, LF_M1_VALID = 4 };

}  // namespace gx
