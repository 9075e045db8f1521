// gx_kernels.cu — the graph-build kernels (sm_103a).
//
//   K1  line split + per-line parse    ReadsKeyValueParserFactory.parse (:95-148)
//   K2  k-mer roll + canonical + edges SplitReads / setEdgesForCurAndNext (:150-233)
//   K3  table insert                   ExternalSort + PreclusteredGroup +
//                                      AggregateKmerAggregateFactory (:93-175)
//   K4  read-head bucketing + sort     ReadHeadSet / ExternalableTreeSet.union (:138-145)
//   K5  compaction + serialization     outputFinalResult (:185-214), Node.write,
//                                      KmerNodePairSequenceWriterFactory.write (:79-94)
#include <algorithm>
#include <cstring>
#include <vector>
#include <cmath>
#include <cstdio>

#include "gx_kernels.cuh"

namespace gx {

thread_local uint64_t t_launches = 0;  // kernels this host thread launched
uint64_t launches_this_thread() { return t_launches; }

// ---- device -> host reads through mapped pinned memory -----------------------------------------
__global__ void k_readback(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

namespace {
struct Stage {
    uint8_t *p = nullptr;  // pinned, mapped (unified addressing: the same pointer on the device)
    size_t cap = 0, used = 0;
    cudaStream_t s = nullptr;
    struct Pending {
        void *dst;
        size_t off, n;
    };
    std::vector<Pending> pend;
};
thread_local Stage t_stage;

cudaError_t deliver(Stage &b) {
    for (const Stage::Pending &q : b.pend) memcpy(q.dst, b.p + q.off, q.n);
    b.pend.clear();
    b.used = 0;
    return cudaSuccess;
}
}  // namespace

cudaError_t sync_stream(cudaStream_t s) {
    const cudaError_t e = cudaStreamSynchronize(s);
    Stage &b = t_stage;
    if (e == cudaSuccess && !b.pend.empty() && b.s == s) deliver(b);
    return e;
}

cudaError_t d2h_async(void *dst, const void *src, size_t n, cudaStream_t s) {
    if (!n) return cudaSuccess;
    Stage &b = t_stage;
    if (!b.pend.empty() && b.s != s) {  // reads of another stream first
        const cudaError_t e = cudaStreamSynchronize(b.s);
        if (e != cudaSuccess) return e;
        deliver(b);
    }
    const size_t sz = (n + 15) & ~(size_t)15;
    if (b.used + sz > b.cap) {
        if (!b.pend.empty()) {
            const cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return e;
            deliver(b);
        }
        if (sz > b.cap) {
            if (b.p) cudaFreeHost(b.p);
            b.p = nullptr;
            b.cap = 0;
            const size_t cap = std::max<size_t>(sz, 16u << 20);
            const cudaError_t e = cudaMallocHost((void **)&b.p, cap);
            if (e != cudaSuccess) return e;
            b.cap = cap;
        }
    }
    const unsigned blocks = (unsigned)std::min<size_t>((n + 4095) / 4096, 64);
    t_launches++;
    k_readback<<<blocks, 256, 0, s>>>((const uint8_t *)src, b.p + b.used, n);
    b.pend.push_back(Stage::Pending{dst, b.used, n});
    b.used += sz;
    b.s = s;
    return cudaGetLastError();
}

// =========================================================================================
// scans
// =========================================================================================
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr uint64_t SCAN_TILE = (uint64_t)SCAN_THREADS * SCAN_ITEMS;

template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// a 64-bit value from lane src (all lanes call)
__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
    const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src), hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
    return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ unsigned long long shfl64_up(unsigned long long v, int d) {
    const uint32_t lo = __shfl_up_sync(0xffffffffu, (uint32_t)v, d), hi = __shfl_up_sync(0xffffffffu, (uint32_t)(v >> 32), d);
    return ((unsigned long long)hi << 32) | lo;
}

// Block-wide exclusive scan of one value per thread; ws must hold 33 T.  All threads call.
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *ws, T &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? ws[lane] : (T)0;
        T wi = warp_inclusive_scan(w);
        if (lane < nw) ws[lane] = wi - w;
        if (lane == 31) ws[32] = wi;
    }
    __syncthreads();
    T r = ws[warp] + inc - v;
    total = ws[32];
    __syncthreads();
    return r;
}

template <class T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile(const T *in, T *out, uint64_t n, T *tile_sums) {
    __shared__ T ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    T v[SCAN_ITEMS];
    T sum = 0;
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
        v[q] = base + q < n ? in[base + q] : (T)0;
        sum += v[q];
    }
    T total;
    T ex = block_exclusive_scan(sum, ws, total);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
        if (base + q < n) out[base + q] = ex;
        ex += v[q];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

template <class T>
__global__ void k_scan_add(T *out, uint64_t n, const T *tile_offs) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_offs[i / SCAN_TILE];
}

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

size_t scan_scratch_bytes(uint64_t n, size_t elem) {
    size_t total = 0;
    while (true) {
        uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
        if (tiles == 0) tiles = 1;
        total += align_up(tiles * elem, 256);
        if (tiles <= 1) break;
        n = tiles;
    }
    return total;
}

template <class T>
static void scan_impl(const T *in, T *out, uint64_t n, T *total, char *scratch, cudaStream_t s) {
    if (n == 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(T), s);
        return;
    }
    const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    T *sums = (T *)scratch;
    char *next = scratch + align_up(tiles * sizeof(T), 256);
    t_launches++;
    k_scan_tile<T><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, sums);
    if (tiles == 1) {
        if (total) cudaMemcpyAsync(total, sums, sizeof(T), cudaMemcpyDeviceToDevice, s);
        return;
    }
    scan_impl<T>(sums, sums, tiles, total, next, s);
    t_launches++;
    k_scan_add<T><<<(unsigned)((n + 1023) / 1024), 1024, 0, s>>>(out, n, sums);
}

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total, void *scratch,
                        cudaStream_t s) {
    scan_impl<uint32_t>(in, out, n, total, (char *)scratch, s);
}
void exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, uint64_t n,
                        unsigned long long *total, void *scratch, cudaStream_t s) {
    scan_impl<unsigned long long>(in, out, n, total, (char *)scratch, s);
}

// =========================================================================================
// K1a: line terminators.  Hadoop's LineReader ends a line at '\n', at '\r' and at "\r\n"
// (one terminator); a last line without a terminator is still a line.
// =========================================================================================
__device__ __forceinline__ void load16(const uint8_t *text, uint64_t n, uint64_t p0, uint32_t w[4]) {
    if (p0 + 16 <= n) {
        uint4 v = *reinterpret_cast<const uint4 *>(text + p0);
        w[0] = v.x;
        w[1] = v.y;
        w[2] = v.z;
        w[3] = v.w;
    } else {
        w[0] = w[1] = w[2] = w[3] = 0;
        for (int b = 0; b < 16 && p0 + b < n; b++) w[b >> 2] |= (uint32_t)text[p0 + b] << (8 * (b & 3));
    }
}

// per-byte mask of '\n' or '\r' in a word (bit 7 of each byte)
__device__ __forceinline__ uint32_t nl_or_cr_mask(uint32_t x) {
    // bytes equal to 0x0A or 0x0D: classic zero-byte detection on x ^ 0x0A0A0A0A etc.
    uint32_t a = x ^ 0x0A0A0A0Au, c = x ^ 0x0D0D0D0Du;
    uint32_t za = (a - 0x01010101u) & ~a & 0x80808080u;
    uint32_t zc = (c - 0x01010101u) & ~c & 0x80808080u;
    return za | zc;
}

// Number of line ends owned by this thread's 64 bytes (and writes them if out != null).
__device__ __forceinline__ uint32_t scan_terms(const uint8_t *text, uint64_t n, uint64_t base,
                                               unsigned long long *out) {
    uint32_t cnt = 0;
    for (int v = 0; v < LINE_TILE_VECS; v++) {
        const uint64_t p0 = base + 16 * v;
        if (p0 >= n) break;
        uint32_t w[4];
        load16(text, n, p0, w);
        for (int q = 0; q < 4; q++) {
            uint32_t m = nl_or_cr_mask(w[q]);
            // zero-byte detection can flag a byte after a true zero; recheck each flagged byte
            while (m) {
                const int bit = __ffs(m) - 1;
                m &= m - 1;
                const int b = bit >> 3;
                const uint64_t p = p0 + 4 * q + b;
                if (p >= n) continue;
                const uint32_t c = (w[q] >> (8 * b)) & 0xffu;
                bool term = false;
                if (c == '\n')
                    term = true;
                else if (c == '\r')
                    term = (p + 1 >= n) || text[p + 1] != '\n';
                if (term) {
                    if (out) out[cnt] = p;
                    cnt++;
                }
            }
        }
    }
    // a final line without a terminator ends at n
    if (n > 0 && base <= n - 1 && n - 1 < base + 16 * LINE_TILE_VECS) {
        const uint32_t c = text[n - 1];
        if (c != '\n' && c != '\r') {
            if (out) out[cnt] = n;
            cnt++;
        }
    }
    return cnt;
}

__global__ void __launch_bounds__(LINE_TILE_THREADS) k_count_lines(const uint8_t *text, uint64_t n,
                                                                   uint32_t *tile_cnt) {
    __shared__ uint32_t ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * LINE_TILE_BYTES + (uint64_t)threadIdx.x * 16 * LINE_TILE_VECS;
    uint32_t c = scan_terms(text, n, base, nullptr);
    uint32_t total;
    block_exclusive_scan(c, ws, total);
    if (threadIdx.x == 0) tile_cnt[blockIdx.x] = total;
}

__global__ void __launch_bounds__(LINE_TILE_THREADS) k_write_lines(const uint8_t *text, uint64_t n,
                                                                   const uint32_t *tile_off,
                                                                   unsigned long long *line_end) {
    __shared__ uint32_t ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * LINE_TILE_BYTES + (uint64_t)threadIdx.x * 16 * LINE_TILE_VECS;
    uint32_t c = scan_terms(text, n, base, nullptr);
    uint32_t total;
    uint32_t ex = block_exclusive_scan(c, ws, total);
    if (c) scan_terms(text, n, base, line_end + tile_off[blockIdx.x] + ex);
}

uint64_t line_tiles(uint64_t n_text) { return (n_text + LINE_TILE_BYTES - 1) / LINE_TILE_BYTES; }

void launch_count_lines(const uint8_t *text, uint64_t n, uint32_t *tile_cnt, cudaStream_t s) {
    const uint64_t t = line_tiles(n);
    t_launches++;
    if (t) k_count_lines<<<(unsigned)t, LINE_TILE_THREADS, 0, s>>>(text, n, tile_cnt);
}
void launch_write_lines(const uint8_t *text, uint64_t n, const uint32_t *tile_off, unsigned long long *line_end,
                        cudaStream_t s) {
    const uint64_t t = line_tiles(n);
    t_launches++;
    if (t) k_write_lines<<<(unsigned)t, LINE_TILE_THREADS, 0, s>>>(text, n, tile_off, line_end);
}

// =========================================================================================
// K1b: per-line parse, one thread per line.  Reproduces, in order, the checks of
// ReadsKeyValueParserFactory.parse (:95-148) and SplitReads (:152-155):
//   value.toString().split("\\t") must give 2 or 3 fields   -> GX_EINVAL_LINE
//   Long.parseLong(field 0)                                 -> GX_EINVAL_NUMBER
//   for each mate matching [ACGTacgt]+ :  readId in [0, 2^35) -> GX_EREADID_RANGE
//                                         k < length         -> GX_EREAD_TOO_SHORT
// =========================================================================================
__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v) { return __reduce_add_sync(0xffffffffu, v); }

// Java Long.parseLong, ASCII digits, optional sign; false where Java throws.
__device__ bool java_parse_long(const uint8_t *s, uint32_t n, long long &out) {
    if (n == 0) return false;
    uint32_t i = 0;
    bool neg = false;
    if (s[0] == '-' || s[0] == '+') {
        if (n == 1) return false;
        neg = s[0] == '-';
        i = 1;
    }
    const unsigned long long limit = neg ? (1ULL << 63) : ((1ULL << 63) - 1);
    unsigned long long v = 0;
    for (; i < n; i++) {
        const uint32_t c = s[i];
        if (c < '0' || c > '9') return false;
        const unsigned long long d = c - '0';
        if (v > (limit - d) / 10) return false;
        v = v * 10 + d;
    }
    out = neg ? (long long)(0ULL - v) : (long long)v;
    return true;
}

// SWAR byte classes of one 32-bit word of text (4 bytes, first in the low byte): bit q of the
// result is byte q's flag.
__device__ __forceinline__ uint32_t zero_bytes(uint32_t t) {  // high bit of every zero byte, exact
    return ~(((t & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | t) & 0x80808080u;
}
__device__ __forceinline__ uint32_t high_bits_to_mask4(uint32_t z) {
    return (((z >> 7) & 0x01010101u) * 0x01020408u) >> 24;
}
// tab bytes, and bytes outside [ACGTacgt]
__device__ __forceinline__ void classify_word(uint32_t w, uint32_t &tab4, uint32_t &bad4) {
    tab4 = high_bits_to_mask4(zero_bytes(w ^ 0x09090909u));
    const uint32_t u = w & 0xDFDFDFDFu;
    const uint32_t ok = zero_bytes(u ^ 0x41414141u) | zero_bytes(u ^ 0x43434343u) | zero_bytes(u ^ 0x47474747u) |
                        zero_bytes(u ^ 0x54545454u);
    bad4 = high_bits_to_mask4(~ok & 0x80808080u);
}
// bits [lo, hi) of a 32-bit mask (lo, hi clamped to [0, 32])
__device__ __forceinline__ uint32_t bit_range(long long lo, long long hi) {
    lo = lo < 0 ? 0 : (lo > 32 ? 32 : lo);
    hi = hi < 0 ? 0 : (hi > 32 ? 32 : hi);
    if (hi <= lo) return 0u;
    const uint32_t top = hi >= 32 ? 0xffffffffu : ((1u << (uint32_t)hi) - 1u);
    return top & ~((1u << (uint32_t)lo) - 1u);
}

// One thread per line.  The thread reads its line in 16-byte loads (two in flight) and
// classifies four bytes per word operation: tab bytes, bytes outside [ACGTacgt], the last
// non-tab byte.  Words without a tab (all but two or three per line) cost a few operations;
// a word holding a tab is walked byte by byte to place the tab and split the field marks.
__global__ void __launch_bounds__(256) k_parse_lines(const uint8_t *text, uint64_t n_text,
                                                     const unsigned long long *line_end, uint32_t n_lines, int k,
                                                     LineRec *lines, uint8_t *lflags, uint32_t *nvalid,
                                                     DevStatus *st) {
    const uint64_t line = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= n_lines) return;
    const uint64_t b = line == 0 ? 0 : line_end[line - 1] + 1;
    uint64_t e = line_end[line];
    if (e < n_text && e > b && text[e] == '\n' && text[e - 1] == '\r') e--;
    const uint32_t len = (uint32_t)(e - b);

    // tabs: where the first three are and how many; the last non-tab byte; which of fields 1
    // and 2 hold a byte outside [ACGTacgt] (bit f of badf)
    uint32_t tabs = 0, t0 = len, t1 = len, t2 = len, field = 0, badf = 0;
    long long last_nt = -1;
    for (uint64_t c = b & ~15ULL; c < e; c += 32) {
        uint32_t wd[8];
        load16(text, n_text, c, wd);
        if (c + 16 < e)
            load16(text, n_text, c + 16, wd + 4);
        else
            wd[4] = wd[5] = wd[6] = wd[7] = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const uint64_t p = c + 4 * q;
            const uint32_t vm = bit_range((long long)b - (long long)p, (long long)e - (long long)p) & 15u;
            if (!vm) continue;
            uint32_t t4, b4;
            classify_word(wd[q], t4, b4);
            t4 &= vm;
            b4 &= vm;
            const uint32_t nt4 = vm & ~t4;
            if (nt4) last_nt = (long long)(p - b) + 31 - __clz(nt4);
            if (!t4) {
                if (b4) badf |= 1u << min(field, 3u);
                continue;
            }
            for (uint32_t j = 0; j < 4; j++) {
                if (!((vm >> j) & 1u)) continue;
                if ((t4 >> j) & 1u) {
                    const uint32_t at = (uint32_t)(p + j - b);
                    if (tabs == 0)
                        t0 = at;
                    else if (tabs == 1)
                        t1 = at;
                    else if (tabs == 2)
                        t2 = at;
                    tabs++;
                    field++;
                } else if ((b4 >> j) & 1u) {
                    badf |= 1u << min(field, 3u);
                }
            }
        }
    }
    // String.split: trailing empty fields removed; no tab at all gives one field
    int nf;
    if (tabs == 0)
        nf = 1;
    else if (last_nt < 0)
        nf = 0;
    else
        nf = 1 + (int)tabs - (int)(len - 1 - (uint32_t)last_nt);
    // field ranges (relative to b)
    const uint32_t f1b = t0 + 1, f1e = tabs >= 2 ? t1 : len;
    const uint32_t f2b = t1 + 1, f2e = tabs >= 3 ? t2 : len;
    const bool bad1 = (badf >> 1) & 1u, bad2 = (badf >> 2) & 1u;
    uint32_t code = 0;
    long long rid = 0;
    LineRec lr;
    lr.read_id = 0;
    lr.s0 = b + f1b;
    lr.l0 = 0;
    lr.s1 = b + f2b;
    lr.l1 = 0;
    uint8_t fl = 0;
    if (nf != 2 && nf != 3) {
        code = 2;  // GX_EINVAL_LINE
    } else if (!java_parse_long(text + b, t0, rid)) {
        code = 3;  // GX_EINVAL_NUMBER
    } else {
        lr.read_id = rid;
        lr.l0 = f1e - f1b;
        if (nf == 3) {
            lr.l1 = f2e - f2b;
            fl |= LF_HAS_M1;
        }
        const bool id_ok = rid >= 0 && rid < (1LL << 35);
        const bool m0v = lr.l0 > 0 && !bad1;
        const bool m1v = nf == 3 && lr.l1 > 0 && !bad2;
        if (m0v) {
            fl |= LF_M0_VALID;
            if (!id_ok)
                code = 4;  // GX_EREADID_RANGE
            else if ((uint32_t)k >= lr.l0)
                code = 5;  // GX_EREAD_TOO_SHORT
        }
        if (code == 0 && m1v) {
            fl |= LF_M1_VALID;
            if (!id_ok)
                code = 4;
            else if ((uint32_t)k >= lr.l1)
                code = 5;
        }
    }
    if (code) {
        atomicMin(&st->parse_err, (line << 8) | code);
        fl = 0;
    }
    lines[line] = lr;
    lflags[line] = fl;
    nvalid[line] = (fl & LF_M0_VALID ? 1u : 0u) + (fl & LF_M1_VALID ? 1u : 0u);
}

void launch_parse_lines(const uint8_t *text, uint64_t n_text, const unsigned long long *line_end, uint32_t n_lines,
                        int k, LineRec *lines, uint8_t *lflags, uint32_t *nvalid, DevStatus *st, cudaStream_t s) {
    if (!n_lines) return;
    t_launches++;
    k_parse_lines<<<(n_lines + 255) / 256, 256, 0, s>>>(text, n_text, line_end, n_lines, k, lines, lflags, nvalid,
                                                        st);
}

// list of valid reads (line << 1 | mate) and the occurrence count
__global__ void __launch_bounds__(256) k_read_list(const uint8_t *lflags, const uint32_t *read_off,
                                                   const LineRec *lines, uint32_t n_lines, int k, uint32_t *reads,
                                                   DevStatus *st) {
    __shared__ unsigned long long ws[33];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long occ = 0;
    if (i < n_lines) {
        const uint8_t f = lflags[i];
        uint32_t o = read_off[i];
        if (f & LF_M0_VALID) {
            reads[o++] = i << 1;
            occ += lines[i].l0 - k + 1;
        }
        if (f & LF_M1_VALID) {
            reads[o] = (i << 1) | 1u;
            occ += lines[i].l1 - k + 1;
        }
    }
    unsigned long long total;
    block_exclusive_scan(occ, ws, total);
    if (threadIdx.x == 0 && total) atomicAdd(&st->n_occ, total);
}

void launch_read_list(const uint8_t *lflags, const uint32_t *read_off, const LineRec *lines, uint32_t n_lines, int k,
                      uint32_t *reads, DevStatus *st, cudaStream_t s) {
    if (!n_lines) return;
    t_launches++;
    k_read_list<<<(n_lines + 255) / 256, 256, 0, s>>>(lflags, read_off, lines, n_lines, k, reads, st);
}

// =========================================================================================
// K2 + K3: one thread per read.  Rolling forward / reverse-complement windows (the
// reference re-packs the reverse complement from the text at every base, :180), the
// canonical orientation, the <= 2 edge bits of each occurrence, one table insert per
// occurrence, and the read head of occurrence 0.
// =========================================================================================
template <class K>
__global__ void __launch_bounds__(256) k_insert(typename SlotOf<K>::T *table, uint32_t nparts, const uint8_t *text,
                                                const LineRec *lines, const uint32_t *reads, uint32_t n_reads, int k,
                                                Head *heads, uint32_t *head_cnt, DevStatus *st) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t maxp = 0;
    if (r < n_reads) {
        const uint32_t rl = reads[r];
        const uint32_t line = rl >> 1, mate = rl & 1u;
        const LineRec lr = lines[line];
        const uint8_t *s = text + (mate ? lr.s1 : lr.s0);
        const uint32_t L = mate ? lr.l1 : lr.l0;
        const K mask = KeyOps<K>::mask(k);
        const int sh = 2 * (k - 1);
        K fwd = 0, rc = 0;
        for (int i = 0; i < k; i++) {
            const uint32_t c = base_code(s[i]);
            fwd = (fwd >> 2) | ((K)c << sh);
            rc = ((rc << 2) | (K)(3u - c)) & mask;
        }
        const uint32_t nk = L - (uint32_t)k + 1;
        uint32_t d = fwd <= rc ? 0u : 1u;  // 0 = FORWARD
        uint32_t pd = 0;
        uint64_t h = KeyOps<K>::hash(d == 0 ? fwd : rc);
        for (uint32_t j = 0; j < nk; j++) {
            const bool hn = j + 1 < nk;
            K nf = fwd, nr = rc;
            uint32_t nd = 0, x = 0;
            uint64_t hnext = 0;
            if (hn) {
                x = base_code(s[j + k]);
                nf = (fwd >> 2) | ((K)x << sh);
                nr = ((rc << 2) | (K)(3u - x)) & mask;
                nd = nf <= nr ? 0u : 1u;
                hnext = KeyOps<K>::hash(nd == 0 ? nf : nr);
            }
            uint32_t bits = 0;
            if (hn) bits |= 1u << (4 * (2 * d + nd) + (d == 0 ? x : 3u - x));
            if (j > 0) {
                const uint32_t y = base_code(s[j - 1]);
                bits |= 1u << (4 * (2 * (d ^ 1u) + (pd ^ 1u)) + (d == 1 ? 3u - y : y));
            }
            if (j == 0) bits |= d == 0 ? META_UNFLIPPED : META_FLIPPED;
            const K canon = d == 0 ? fwd : rc;
            const uint32_t p = hash_partition(h, nparts);
            uint32_t probes;
            const int si = table_insert(table + (size_t)p * PART_SLOTS, PART_SLOTS - 1, canon, (uint32_t)h, bits,
                                        probes);
            maxp = max(maxp, probes);
            if (si < 0) atomicAdd(&st->table_full, 1u);
            if (j == 0) {
                Head hd;
                hd.part = si < 0 ? 0xffffffffu : p;
                hd.slot = (uint32_t)si;
                hd.uuid = ((unsigned long long)(d == 0 ? 0 : k - 1) << 40) | ((unsigned long long)mate << 35) |
                          (unsigned long long)lr.read_id;
                hd.klo = (unsigned long long)canon;
                hd.khi = (unsigned long long)((u128)canon >> 64);
                heads[r] = hd;
                if (si >= 0) atomicAdd(&head_cnt[p], 1u);
            }
            pd = d;
            d = nd;
            fwd = nf;
            rc = nr;
            h = hnext;
        }
    }
    maxp = __reduce_max_sync(0xffffffffu, maxp);
    if ((threadIdx.x & 31) == 0 && maxp) atomicMax(&st->max_probe, maxp);
}

void launch_insert(const TableGeom &g, const uint8_t *text, const LineRec *lines, const uint32_t *reads,
                   uint32_t n_reads, int k, Head *heads, uint32_t *head_cnt, DevStatus *st, cudaStream_t s) {
    if (!n_reads) return;
    const unsigned blocks = (n_reads + 255) / 256;
    t_launches++;
    if (g.wide)
        k_insert<u128><<<blocks, 256, 0, s>>>((Slot128 *)g.table, g.nparts, text, lines, reads, n_reads, k, heads,
                                              head_cnt, st);
    else
        k_insert<uint64_t><<<blocks, 256, 0, s>>>((Slot64 *)g.table, g.nparts, text, lines, reads, n_reads, k, heads,
                                                  head_cnt, st);
}

__global__ void k_head_scatter(const Head *heads, uint32_t n_reads, const uint32_t *head_off, uint32_t *head_cur,
                               uint32_t *head_idx) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_reads) return;
    const uint32_t p = heads[r].part;
    if (p == 0xffffffffu) return;
    head_idx[head_off[p] + atomicAdd(&head_cur[p], 1u)] = r;
}

void launch_head_scatter(const Head *heads, uint32_t n_reads, const uint32_t *head_off, uint32_t *head_cur,
                         uint32_t *head_idx, uint32_t nparts, cudaStream_t s) {
    (void)nparts;
    if (!n_reads) return;
    t_launches++;
    k_head_scatter<<<(n_reads + 255) / 256, 256, 0, s>>>(heads, n_reads, head_off, head_cur, head_idx);
}

__global__ void k_head_scatter_part(const Head *heads, const uint32_t *reads, const LineRec *lines,
                                    uint32_t n_reads, const uint32_t *head_off, uint32_t *head_cur,
                                    uint32_t *head_idx, HeadIn *hsorted) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_reads) return;
    const Head h = heads[r];
    if (h.part == 0xffffffffu) return;
    const uint32_t rl = reads[r], mate = rl & 1u;
    const LineRec lr = lines[rl >> 1];
    const uint32_t pos = head_off[h.part] + atomicAdd(&head_cur[h.part], 1u);
    head_idx[pos] = r;
    HeadIn hi;
    hi.uuid = h.uuid;
    hi.klo = h.klo;
    hi.khi = h.khi;
    hi.s_off = mate ? lr.s1 : lr.s0;
    hi.m_off = mate ? lr.s0 : lr.s1;
    hi.L = mate ? lr.l1 : lr.l0;
    hi.Lm = mate ? lr.l0 : lr.l1;
    hi.r = r;
    hi.pad0 = 0;
    hi.pad1 = 0;
    hsorted[pos] = hi;
}

void launch_head_scatter_part(const Head *heads, const uint32_t *reads, const LineRec *lines, uint32_t n_reads,
                              const uint32_t *head_off, uint32_t *head_cur, uint32_t *head_idx, HeadIn *hsorted,
                              cudaStream_t s) {
    if (!n_reads) return;
    t_launches++;
    k_head_scatter_part<<<(n_reads + 255) / 256, 256, 0, s>>>(heads, reads, lines, n_reads, head_off, head_cur,
                                                              head_idx, hsorted);
}

// =========================================================================================
// K4 + K5: emission, one CTA per table partition.
//   prepare: compact occupied slots, sort them by canonical key, write them back to the
//            front of the partition; sort + de-duplicate the partition's read heads by
//            (node, TreeSet order); total the record bytes.
//   write:   serialize every record at its final offset through a shared-memory window,
//            stored to HBM with aligned 16-byte stores.
// Record order: by table partition, then by canonical key.  Deterministic for a given
// table geometry.
// =========================================================================================

// Ascending-only bitonic network over (key, val) pairs with virtual +inf past n.
template <class KT, class VT>
__device__ void bitonic_sort_pairs(KT *key, VT *val, uint32_t n) {
    uint32_t N = 1, logN = 0;
    while (N < n) {
        N <<= 1;
        logN++;
    }
    for (uint32_t ls = 1; ls <= logN; ls++) {
        const uint32_t size = 1u << ls;
        for (uint32_t lt = ls; lt-- > 0;) {
            const uint32_t stride = 1u << lt;
            for (uint32_t i = threadIdx.x; i < N / 2; i += blockDim.x) {
                const uint32_t blk = i >> lt, off = i & (stride - 1);
                uint32_t lo, hi;
                if (lt == ls - 1) {
                    lo = (blk << ls) + off;
                    hi = (blk << ls) + size - 1 - off;
                } else {
                    lo = (blk << (lt + 1)) + off;
                    hi = lo + stride;
                }
                if (hi < n) {
                    const KT a = key[lo], b = key[hi];
                    const VT va = val[lo], vb = val[hi];
                    if (b < a || (b == a && vb < va)) {
                        key[lo] = b;
                        key[hi] = a;
                        val[lo] = vb;
                        val[hi] = va;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ uint32_t packed_len(uint32_t L) { return (L + 3) >> 2; }

// serialized size of one ReadHeadInfo (ReadHeadInfo.write, :205-212)
__device__ __forceinline__ uint32_t head_bytes(const LineRec &lr, uint32_t mate) {
    const uint32_t L = mate ? lr.l1 : lr.l0;
    const uint32_t Lm = mate ? lr.l0 : lr.l1;
    return 1 + 8 + 4 + packed_len(L) + (Lm > 0 ? 4 + packed_len(Lm) : 0);
}

// record bytes of a node without its read heads: frame (8) + key + Node fields
__device__ __forceinline__ uint32_t node_base_bytes(uint32_t meta, int nb) {
    uint32_t sz = 8 + (4 + nb) + 1 + 4;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const uint32_t m = (meta >> (4 * t)) & 15u;
        if (m) sz += 4 + __popc(m) * (4 + nb);
    }
    if (meta & META_UNFLIPPED) sz += 5;
    if (meta & META_FLIPPED) sz += 5;
    return sz;
}

template <class K> struct EmitSmem;
template <> struct EmitSmem<uint64_t> {
    __device__ static uint64_t load_key1(const Slot64 *s, bool &occ) {
        const uint64_t k1 = s->key1;
        occ = k1 != 0;
        return k1 - 1;
    }
    __device__ static void store(Slot64 *s, uint64_t key, uint32_t cnt, uint32_t meta) {
        s->key1 = key + 1;
        s->count = cnt;
        s->meta = meta;
    }
};
template <> struct EmitSmem<u128> {
    __device__ static u128 load_key1(const Slot128 *s, bool &occ) {
        const u128 k1 = ((u128)s->hi1 << 64) | s->lo1;
        occ = k1 != 0;
        return k1 - 1;
    }
    __device__ static void store(Slot128 *s, u128 key, uint32_t cnt, uint32_t meta) {
        const u128 k1 = key + 1;
        s->lo1 = (unsigned long long)k1;
        s->hi1 = (unsigned long long)(k1 >> 64);
        s->count = cnt;
        s->meta = meta;
        s->pad = 0;
    }
};

template <class K> struct SlotLoad;
template <> struct SlotLoad<uint64_t> {
    // whole slot in one 16-byte load
    __device__ __forceinline__ static void get(const Slot64 *s, uint64_t &key, uint32_t &cnt, uint32_t &meta,
                                               bool &occ) {
        const ulonglong2 v = ld_cg16(s);
        occ = v.x != 0;
        key = v.x - 1;
        cnt = (uint32_t)v.y;
        meta = (uint32_t)(v.y >> 32);
    }
};
template <> struct SlotLoad<u128> {
    __device__ __forceinline__ static void get(const Slot128 *s, u128 &key, uint32_t &cnt, uint32_t &meta,
                                               bool &occ) {
        const ulonglong2 a = ld_cg16(&s->lo1), b = ld_cg16(&s->count);
        const u128 k1 = ((u128)a.y << 64) | a.x;
        occ = k1 != 0;
        key = k1 - 1;
        cnt = (uint32_t)b.x;
        meta = (uint32_t)(b.x >> 32);
    }
};

template <class K>
struct PrepSmem {
    K key[PART_SLOTS];
    uint32_t cnt[PART_SLOTS];
    uint32_t meta[PART_SLOTS];
    uint16_t slot[PART_SLOTS];
    uint16_t ord[PART_SLOTS];
    uint16_t rank_of_slot[PART_SLOTS];
    unsigned long long hk[HEAD_CAP];
    uint32_t hv[HEAD_CAP];
    unsigned long long ws[33];
    uint32_t n;
};

// sort key of a read head inside its partition: node rank, then the TreeSet order of
// ReadHeadInfo.compareTo (:247-264) = (offset, library, mate, readId); offset is 0 or k-1
// and the library is 0, so (flipped, mate, readId) orders it.
__device__ __forceinline__ unsigned long long head_sort_key(uint32_t rank, unsigned long long uuid) {
    const unsigned long long flipped = (uuid >> 40) != 0 ? 1ULL : 0ULL;
    return ((unsigned long long)rank << 37) | (flipped << 36) | (uuid & ((1ULL << 36) - 1));
}

template <class K>
__global__ void __launch_bounds__(EMIT_THREADS) k_emit_prepare(EmitArgs a) {
    typedef typename SlotOf<K>::T Slot;
    extern __shared__ __align__(16) uint8_t smem_raw[];
    PrepSmem<K> &sm = *reinterpret_cast<PrepSmem<K> *>(smem_raw);
    const uint32_t p = blockIdx.x;
    Slot *part = (Slot *)a.g.table + (size_t)p * PART_SLOTS;
    const int nb = (a.k + 3) / 4;
    if (threadIdx.x == 0) sm.n = 0;
    __syncthreads();
    // 1. compact occupied slots (all of a thread's slots are loaded before any is used)
    {
        constexpr int PER = PART_SLOTS / EMIT_THREADS;
        K kk[PER];
        uint32_t cc[PER], mm[PER];
        bool oo[PER];
#pragma unroll
        for (int q = 0; q < PER; q++) SlotLoad<K>::get(part + threadIdx.x + q * EMIT_THREADS, kk[q], cc[q], mm[q], oo[q]);
#pragma unroll
        for (int q = 0; q < PER; q++) {
            if (!oo[q]) continue;
            const uint32_t j = atomicAdd(&sm.n, 1u);
            sm.key[j] = kk[q];
            sm.cnt[j] = cc[q];
            sm.meta[j] = mm[q];
            sm.slot[j] = (uint16_t)(threadIdx.x + q * EMIT_THREADS);
            sm.ord[j] = (uint16_t)j;
        }
    }
    __syncthreads();
    const uint32_t n = sm.n;
    // 2. sort by canonical key (unique)
    bitonic_sort_pairs<K, uint16_t>(sm.key, sm.ord, n);
    // 3. write back the sorted nodes; remember each original slot's rank
    unsigned long long bytes = 0;
    uint32_t inexact = 0;
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
        const uint32_t o = sm.ord[j];
        EmitSmem<K>::store(part + j, sm.key[j], sm.cnt[o], sm.meta[o]);
        sm.rank_of_slot[sm.slot[o]] = (uint16_t)j;
        bytes += node_base_bytes(sm.meta[o], nb);
        if (sm.cnt[o] >= (1u << 24)) inexact++;
    }
    if (inexact) atomicAdd(&a.st->cov_inexact, inexact);
    __syncthreads();
    // 4. read heads: sort by (node, TreeSet order), drop duplicates, total their bytes
    const uint32_t hb = a.head_off[p], hc = a.head_cnt[p];
    const bool big = hc > HEAD_CAP;
    unsigned long long *hk = big ? a.head_sk + hb : sm.hk;
    uint32_t *hv = big ? a.head_idx + hb : sm.hv;
    if (big && threadIdx.x == 0) atomicAdd(&a.st->big_head_parts, 1u);
    for (uint32_t i = threadIdx.x; i < hc; i += blockDim.x) {
        const uint32_t r = a.head_idx[hb + i];
        const Head h = a.heads[r];
        hk[i] = head_sort_key(sm.rank_of_slot[h.slot], h.uuid);
        hv[i] = r;
    }
    __syncthreads();
    bitonic_sort_pairs<unsigned long long, uint32_t>(hk, hv, hc);
    // de-duplicate equal (node, uuid): TreeSet.add keeps the element already present
    uint32_t kept_total = 0;
    for (uint32_t c0 = 0; c0 < hc; c0 += blockDim.x) {
        const uint32_t i = c0 + threadIdx.x;
        uint32_t keep = 0, r = 0;
        if (i < hc) {
            keep = (i == 0 || hk[i] != hk[i - 1]) ? 1u : 0u;
            r = hv[i];
        }
        unsigned long long tot;
        const unsigned long long ex = block_exclusive_scan((unsigned long long)keep, sm.ws, tot);
        if (keep) {
            a.head_idx[hb + kept_total + (uint32_t)ex] = r;
            const uint32_t rl = a.reads[r];
            const LineRec lr = a.lines[rl >> 1];
            bytes += head_bytes(lr, rl & 1u);
            Head h = a.heads[r];
            h.slot = (uint32_t)(hk[i] >> 37);  // node rank
            a.heads[r] = h;
        }
        kept_total += (uint32_t)tot;
    }
    unsigned long long tot_bytes;
    block_exclusive_scan(bytes, sm.ws, tot_bytes);
    if (threadIdx.x == 0) {
        a.part_nodes[p] = n;
        a.part_bytes[p] = tot_bytes;
        a.head_cnt2[p] = kept_total;
    }
}

template <class K>
static size_t prep_smem_bytes() {
    return sizeof(PrepSmem<K>);
}

void launch_emit_prepare(const EmitArgs &a, cudaStream_t s) {
    if (!a.g.nparts) return;
    if (a.g.wide) {
        const size_t sm = prep_smem_bytes<u128>();
        cudaFuncSetAttribute(k_emit_prepare<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        t_launches++;
        k_emit_prepare<u128><<<a.g.nparts, EMIT_THREADS, sm, s>>>(a);
    } else {
        const size_t sm = prep_smem_bytes<uint64_t>();
        cudaFuncSetAttribute(k_emit_prepare<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        t_launches++;
        k_emit_prepare<uint64_t><<<a.g.nparts, EMIT_THREADS, sm, s>>>(a);
    }
}

// ---- record serialization ---------------------------------------------------------------
// Writes bytes at partition-local positions; only positions inside [lo, hi) reach the
// staging window.
struct Sink {
    uint8_t *st;
    long long lo, hi;
    bool all_in;  // the whole record lies inside the window: no per-byte check
    __device__ __forceinline__ void b(long long pos, uint32_t v) const {
        if (all_in || (pos >= lo && pos < hi)) st[pos - lo] = (uint8_t)v;
    }
    __device__ __forceinline__ void u32(long long pos, uint32_t v) const {
        b(pos, v >> 24);
        b(pos + 1, v >> 16);
        b(pos + 2, v >> 8);
        b(pos + 3, v);
    }
    __device__ __forceinline__ bool touches(long long pos, long long n) const {
        return all_in || (pos < hi && pos + n > lo);
    }
};

// VKmer bytes of a k-mer value: int32 BE k, then nb bytes of V big-endian (VKmer.write)
template <class K>
__device__ __forceinline__ long long put_vkmer(const Sink &o, long long pos, K v, int k, int nb) {
    o.u32(pos, (uint32_t)k);
    pos += 4;
    if (o.touches(pos, nb))
        for (int i = 0; i < nb; i++) o.b(pos + i, KeyOps<K>::byte_at(v, nb - 1 - i));
    return pos + nb;
}

// VKmer of a read sequence (VKmer.setAsCopy(String), VKmer.java:450-479): L letters packed
// 4 per byte, first letter in the low bits of the last byte; non-ACGT letters pack as A.
__device__ __forceinline__ long long put_seq(const Sink &o, long long pos, const uint8_t *s, uint32_t L) {
    o.u32(pos, L);
    pos += 4;
    const uint32_t nbr = packed_len(L);
    if (o.touches(pos, nbr)) {
        for (uint32_t j = 0; j < nbr; j++) {
            const uint32_t i0 = 4 * (nbr - 1 - j);
            uint32_t v = 0;
            for (uint32_t q = 0; q < 4 && i0 + q < L; q++) v |= base_code_checked(s[i0 + q]) << (2 * q);
            o.b(pos + j, v);
        }
    }
    return pos + nbr;
}

// packs L letters of s (4 per byte, as put_seq) with one warp: lane l writes bytes l, l+32, ...
__device__ __forceinline__ void pack_seq_warp(const Sink &o, long long pos, const uint8_t *s, uint32_t L, int lane) {
    const uint32_t nbr = packed_len(L);
    for (uint32_t j = lane; j < nbr; j += 32) {
        if (!o.touches(pos + j, 1)) continue;
        const uint32_t i0 = 4 * (nbr - 1 - j);
        uint32_t c[4];
#pragma unroll
        for (int q = 0; q < 4; q++) c[q] = i0 + q < L ? (uint32_t)s[i0 + q] : (uint32_t)'A';
        uint32_t v = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) v |= base_code_checked(c[q]) << (2 * q);
        o.b(pos + j, v);
    }
}

template <class K>
struct WriteSmem {
    K key[PART_SLOTS];
    uint32_t cnt[PART_SLOTS];
    uint32_t meta[PART_SLOTS];
    uint32_t off[PART_SLOTS];
    // read heads of the partition (when at most HEAD_CAP): node rank | flipped << 15, read
    // ordinal, sequence lengths and the partition-local position of the head's bytes
    uint16_t hrank[HEAD_CAP];
    uint32_t hread[HEAD_CAP];
    uint32_t hL[HEAD_CAP];
    uint32_t hLm[HEAD_CAP];
    uint32_t hpos[HEAD_CAP];
    __align__(16) uint8_t stage[EMIT_STAGE_BYTES + 32];
    unsigned long long ws[33];
};

template <class K>
__global__ void __launch_bounds__(EMIT_THREADS) k_emit_write(EmitArgs a) {
    typedef typename SlotOf<K>::T Slot;
    extern __shared__ __align__(16) uint8_t smem_raw[];
    WriteSmem<K> &sm = *reinterpret_cast<WriteSmem<K> *>(smem_raw);
    const uint32_t p = blockIdx.x;
    const Slot *part = (const Slot *)a.g.table + (size_t)p * PART_SLOTS;
    const int k = a.k, nb = (k + 3) / 4;
    const uint32_t n = a.part_nodes[p];
    const unsigned long long pbytes = a.part_bytes[p];
    const unsigned long long base = a.part_off[p];
    const uint32_t hb = a.head_off[p], hc = a.head_cnt2[p];
    const bool hsm = hc <= HEAD_CAP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    // nodes: up to PART_SLOTS / EMIT_THREADS independent loads per thread
    constexpr int PER = PART_SLOTS / EMIT_THREADS;
    if (a.nkey) {
        // partitioned build: compacted nodes in (key, count | meta << 32) arrays
        const K *nk = (const K *)a.nkey + a.node_base[p];
        const unsigned long long *ncm = a.ncm + a.node_base[p];
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            sm.key[j] = nk[j];
            const unsigned long long cm = ncm[j];
            sm.cnt[j] = (uint32_t)cm;
            sm.meta[j] = (uint32_t)(cm >> 32);
        }
    } else {
        K kk[PER];
        uint32_t cc[PER], mm[PER];
        bool oo[PER];
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const uint32_t j = threadIdx.x + q * EMIT_THREADS;
            oo[q] = false;
            if (j < n) SlotLoad<K>::get(part + j, kk[q], cc[q], mm[q], oo[q]);
        }
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const uint32_t j = threadIdx.x + q * EMIT_THREADS;
            if (j < n) {
                sm.key[j] = kk[q];
                sm.cnt[j] = cc[q];
                sm.meta[j] = mm[q];
            }
        }
    }
    if (hsm) {
        for (uint32_t i = threadIdx.x; i < hc; i += blockDim.x) {
            const uint32_t r = a.head_idx[hb + i];
            const Head h = a.heads[r];
            const uint32_t rl = a.reads[r];
            const LineRec lr = a.lines[rl >> 1];
            const uint32_t mate = rl & 1u;
            sm.hread[i] = r;
            sm.hrank[i] = (uint16_t)(h.slot | ((h.uuid >> 40) != 0 ? 0x8000u : 0u));
            sm.hL[i] = mate ? lr.l1 : lr.l0;
            sm.hLm[i] = mate ? lr.l0 : lr.l1;
        }
    }
    __syncthreads();
    auto hrank = [&](uint32_t i) -> uint32_t {
        return hsm ? (uint32_t)(sm.hrank[i] & 0x7fffu) : a.heads[a.head_idx[hb + i]].slot;
    };
    auto hflip = [&](uint32_t i) -> uint32_t {
        return hsm ? (uint32_t)(sm.hrank[i] >> 15) : ((a.heads[a.head_idx[hb + i]].uuid >> 40) != 0 ? 1u : 0u);
    };
    auto hsize = [&](uint32_t i) -> uint32_t {
        uint32_t L, Lm;
        if (hsm) {
            L = sm.hL[i];
            Lm = sm.hLm[i];
        } else {
            const uint32_t rl = a.reads[a.head_idx[hb + i]];
            const LineRec lr = a.lines[rl >> 1];
            L = (rl & 1u) ? lr.l1 : lr.l0;
            Lm = (rl & 1u) ? lr.l0 : lr.l1;
        }
        return 1 + 8 + 4 + packed_len(L) + (Lm > 0 ? 4 + packed_len(Lm) : 0);
    };
    // first head index of node j (heads are sorted by node rank)
    auto head_lb = [&](uint32_t j) -> uint32_t {
        uint32_t lo = 0, hi = hc;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (hrank(mid) < j)
                lo = mid + 1;
            else
                hi = mid;
        }
        return lo;
    };
    auto edge_bytes = [&](uint32_t meta) -> uint32_t {
        uint32_t b = 0;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const uint32_t m = (meta >> (4 * t)) & 15u;
            if (m) b += 4 + __popc(m) * (4 + nb);
        }
        return b;
    };
    // record sizes and offsets: thread t owns a contiguous node range
    const uint32_t npt = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t j0 = min(n, threadIdx.x * npt), j1 = min(n, j0 + npt);
    unsigned long long mine = 0;
    for (uint32_t j = j0; j < j1; j++) {
        uint32_t sz = node_base_bytes(sm.meta[j], nb);
        if (sm.meta[j] & (META_UNFLIPPED | META_FLIPPED))
            for (uint32_t h = head_lb(j); h < hc && hrank(h) == j; h++) sz += hsize(h);
        sm.off[j] = sz;  // size for now
        mine += sz;
    }
    unsigned long long tot;
    unsigned long long run = block_exclusive_scan(mine, sm.ws, tot);
    for (uint32_t j = j0; j < j1; j++) {
        const uint32_t sz = sm.off[j];
        sm.off[j] = (uint32_t)run;
        if (hsm && (sm.meta[j] & (META_UNFLIPPED | META_FLIPPED))) {
            // positions of the node's read heads: after frame, key, active byte and edges
            long long pos = (long long)run + 8 + (4 + nb) + 1 + edge_bytes(sm.meta[j]);
            const uint32_t h0 = head_lb(j);
            for (uint32_t fl = 0; fl < 2; fl++) {
                if (!(sm.meta[j] & (fl == 0 ? META_UNFLIPPED : META_FLIPPED))) continue;
                pos += 5;
                for (uint32_t h = h0; h < hc && hrank(h) == j; h++) {
                    if (hflip(h) != fl) continue;
                    sm.hpos[h] = (uint32_t)pos;
                    pos += hsize(h);
                }
            }
        }
        run += sz;
    }
    if (threadIdx.x == 0 && tot != pbytes) atomicAdd(&a.st->internal_err, 1u);
    __syncthreads();
    const long long my_lo = j0 < j1 ? (long long)sm.off[j0] : 0;
    const long long my_hi = j0 < j1 ? (long long)(j1 == n ? tot : sm.off[j1]) : 0;
    for (unsigned long long W = 0; W < tot; W += EMIT_STAGE_BYTES) {
        const unsigned long long wlen = min((unsigned long long)EMIT_STAGE_BYTES, tot - W);
        const Sink ow{sm.stage, (long long)W, (long long)(W + wlen), false};
        if (j0 < j1 && my_lo < ow.hi && my_hi > ow.lo) {
            for (uint32_t j = j0; j < j1; j++) {
                const long long st = sm.off[j];
                const long long en = j + 1 < n ? (long long)sm.off[j + 1] : (long long)tot;
                if (!ow.touches(st, en - st)) continue;
                Sink o = ow;
                o.all_in = st >= ow.lo && en <= ow.hi;
                const K key = sm.key[j];
                const uint32_t meta = sm.meta[j];
                const uint32_t key_len = 4 + nb;
                o.u32(st, (uint32_t)(en - st - 8));
                o.u32(st + 4, key_len);
                long long pos = put_vkmer<K>(o, st + 8, key, k, nb);
                uint32_t active = 0x80u;
                for (int t = 0; t < 4; t++)
                    if ((meta >> (4 * t)) & 15u) active |= 1u << t;
                if (meta & META_UNFLIPPED) active |= 0x10u;
                if (meta & META_FLIPPED) active |= 0x20u;
                o.b(pos++, active);
                for (int t = 0; t < 4; t++) {
                    const uint32_t m = (meta >> (4 * t)) & 15u;
                    if (!m) continue;
                    const int c = __popc(m);
                    o.u32(pos, (uint32_t)c);
                    pos += 4;
                    if (!o.touches(pos, (long long)c * (4 + nb))) {
                        pos += (long long)c * (4 + nb);
                        continue;
                    }
                    K y[4];
                    int ny = 0;
                    for (int e = 0; e < 4; e++)
                        if (m & (1u << e)) y[ny++] = edge_neighbor<K>(key, t, e, k);
                    for (int u = 1; u < ny; u++)  // insertion sort, <= 4 items
                        for (int v = u; v > 0 && y[v] < y[v - 1]; v--) {
                            const K tmp = y[v];
                            y[v] = y[v - 1];
                            y[v - 1] = tmp;
                        }
                    for (int u = 0; u < ny; u++) pos = put_vkmer<K>(o, pos, y[u], k, nb);
                }
                if (meta & (META_UNFLIPPED | META_FLIPPED)) {
                    const uint32_t h0 = head_lb(j);
                    uint32_t h1 = h0;
                    while (h1 < hc && hrank(h1) == j) h1++;
                    // unflipped set, then flipped set (uuid offset 0 sorts first)
                    for (uint32_t fl = 0; fl < 2; fl++) {
                        const uint32_t flag = fl == 0 ? META_UNFLIPPED : META_FLIPPED;
                        if (!(meta & flag)) continue;
                        uint32_t cnt = 0;
                        for (uint32_t h = h0; h < h1; h++) cnt += hflip(h) == fl ? 1u : 0u;
                        o.b(pos++, 1);  // ExternalableTreeSet: whole body in stream
                        o.u32(pos, cnt);
                        pos += 4;
                        for (uint32_t h = h0; h < h1; h++) {
                            if (hflip(h) != fl) continue;
                            const uint32_t hsz = hsize(h);
                            if (!o.touches(pos, hsz)) {
                                pos += hsz;
                                continue;
                            }
                            const uint32_t r = a.head_idx[hb + h];
                            const unsigned long long uuid = a.heads[r].uuid;
                            const uint32_t rl = a.reads[r];
                            const LineRec lr = a.lines[rl >> 1];
                            const uint32_t mate = rl & 1u;
                            const uint32_t L = mate ? lr.l1 : lr.l0, Lm = mate ? lr.l0 : lr.l1;
                            o.b(pos, Lm > 0 ? 1u : 0u);
                            o.u32(pos + 1, (uint32_t)(uuid >> 32));
                            o.u32(pos + 5, (uint32_t)uuid);
                            o.u32(pos + 9, L);
                            if (Lm > 0) o.u32(pos + 13 + packed_len(L), Lm);
                            if (!hsm) {  // large head sets: this thread packs the letters too
                                put_seq(o, pos + 9, a.text + (mate ? lr.s1 : lr.s0), L);
                                if (Lm > 0) put_seq(o, pos + 13 + packed_len(L), a.text + (mate ? lr.s0 : lr.s1), Lm);
                            }
                            pos += hsz;
                        }
                    }
                }
                const float cov = (float)sm.cnt[j];
                o.u32(pos, __float_as_uint(cov));
            }
        }
        if (hsm) {
            const Sink o = ow;
            // read and mate letters of the partition's heads: one warp per head
            for (uint32_t h = warp; h < hc; h += nwarp) {
                const uint32_t L = sm.hL[h], Lm = sm.hLm[h];
                const long long hp = sm.hpos[h];
                const uint32_t hsz = 13 + packed_len(L) + (Lm > 0 ? 4 + packed_len(Lm) : 0);
                if (!o.touches(hp, hsz)) continue;
                const uint32_t rl = a.reads[sm.hread[h]];
                const LineRec lr = a.lines[rl >> 1];
                const uint32_t mate = rl & 1u;
                pack_seq_warp(o, hp + 13, a.text + (mate ? lr.s1 : lr.s0), L, lane);
                if (Lm > 0) pack_seq_warp(o, hp + 17 + packed_len(L), a.text + (mate ? lr.s0 : lr.s1), Lm, lane);
            }
        }
        __syncthreads();
        // copy the window out with aligned 16-byte stores
        const unsigned long long g0 = base + W, g1 = g0 + wlen;
        const unsigned long long c_first = g0 & ~15ULL;
        const uint32_t *st32 = reinterpret_cast<const uint32_t *>(sm.stage);
        for (unsigned long long c = c_first + 16ULL * threadIdx.x; c < g1; c += 16ULL * blockDim.x) {
            if (c >= g0 && c + 16 <= g1) {
                const uint32_t ofs = (uint32_t)(c - g0);
                const uint32_t w0 = ofs >> 2, sh = (ofs & 3u) * 8u;
                uint32_t w[5];
#pragma unroll
                for (int q = 0; q < 5; q++) w[q] = st32[w0 + q];
                uint4 v;
                v.x = __funnelshift_r(w[0], w[1], sh);
                v.y = __funnelshift_r(w[1], w[2], sh);
                v.z = __funnelshift_r(w[2], w[3], sh);
                v.w = __funnelshift_r(w[3], w[4], sh);
                *reinterpret_cast<uint4 *>(a.out + c) = v;
            } else {
                for (int q = 0; q < 16; q++) {
                    const unsigned long long g = c + q;
                    if (g >= g0 && g < g1) a.out[g] = sm.stage[g - g0];
                }
            }
        }
        __syncthreads();
    }
}

void launch_emit_write(const EmitArgs &a, cudaStream_t s) {
    if (!a.g.nparts) return;
    if (a.g.wide) {
        const size_t sm = sizeof(WriteSmem<u128>);
        cudaFuncSetAttribute(k_emit_write<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        t_launches++;
        k_emit_write<u128><<<a.g.nparts, EMIT_THREADS, sm, s>>>(a);
    } else {
        const size_t sm = sizeof(WriteSmem<uint64_t>);
        cudaFuncSetAttribute(k_emit_write<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        t_launches++;
        k_emit_write<uint64_t><<<a.g.nparts, EMIT_THREADS, sm, s>>>(a);
    }
}


// =========================================================================================
// Partitioned build.  Every occurrence is streamed twice through shared-memory counting
// sorts (super bucket, then fine bucket), then each fine bucket is aggregated by one CTA in
// a shared-memory hash table: no random DRAM access, no global table.
//   A1  occurrence counts per super bucket + HyperLogLog of the canonical k-mers
//   A2  occurrences -> super buckets              (key, 16 edge bits)
//   B1  counts per fine bucket
//   B2  super buckets -> fine buckets
//   C   per fine bucket: shared-memory aggregation, read heads, key sort, record sizes
// then the record writer (k_emit_write) as in the table build.
// =========================================================================================

// Rolling walk over the k-mer occurrences of one read (the same arithmetic as k_insert).
// Letters are read 8 at a time with aligned loads; the letter leaving the window (base j-1
// for occurrence j) is the low two bits of the previous forward value.
template <class K>
struct Walker {
    const uint8_t *text;
    unsigned long long n_text, xo;  // next unread letter offset
    unsigned long long xbuf;
    uint32_t xn;
    uint32_t nk, j, jend, yb;  // occurrences of the read; the walk's next and end
    int k, sh;
    K mask, fwd, rc;
    uint32_t d, pd;
    __device__ __forceinline__ uint32_t letter() {
        if (xn == 0) {
            const unsigned long long al = xo & ~7ULL;
            if (al + 8 <= n_text) {
                xbuf = *reinterpret_cast<const unsigned long long *>(text + al) >> (8 * (xo - al));
                xn = 8 - (uint32_t)(xo - al);
            } else {
                xbuf = 0;
                xn = 0;
                for (unsigned long long q = xo; q < n_text && xn < 8; q++, xn++) xbuf |= (unsigned long long)text[q] << (8 * xn);
            }
        }
        const uint32_t c = base_code((uint32_t)xbuf & 0xffu);
        xbuf >>= 8;
        xn--;
        xo++;
        return c;
    }
    __device__ __forceinline__ void init(const uint8_t *text_, unsigned long long n_text_, unsigned long long s_off,
                                         uint32_t L, int k_) {
        init_range(text_, n_text_, s_off, L, k_, 0, L - (uint32_t)k_ + 1);
    }
    // Occurrences [jb, je) of a read only (one segment of a read split over several threads).
    // A segment after the first starts one k-mer early and steps over it, so its first
    // occurrence gets the edge bits from its predecessor exactly as a whole-read walk does;
    // whether an occurrence has a successor is judged by the read's own length.
    __device__ __forceinline__ void init_range(const uint8_t *text_, unsigned long long n_text_,
                                               unsigned long long s_off, uint32_t L, int k_, uint32_t jb, uint32_t je) {
        text = text_;
        n_text = n_text_;
        k = k_;
        nk = L - (uint32_t)k + 1;
        if (je > nk) je = nk;
        if (jb >= je) {
            j = jend = 0;
            return;
        }
        const uint32_t j0 = jb ? jb - 1 : 0;
        xo = s_off + j0;
        xn = 0;
        xbuf = 0;
        // the segment's sectors requested up front: the walk then consumes them from L1 instead
        // of waiting on one 8-byte load after another
        const unsigned long long seg_end = s_off + je + (uint32_t)k - 1;
        for (unsigned long long a = xo & ~31ULL; a < seg_end && a < n_text; a += 32)
            asm volatile("prefetch.global.L1 [%0];" ::"l"(text + a));
        sh = 2 * (k - 1);
        mask = KeyOps<K>::mask(k);
        fwd = 0;
        rc = 0;
        for (int i = 0; i < k; i++) {
            const uint32_t c = letter();
            fwd = (fwd >> 2) | ((K)c << sh);
            rc = ((rc << 2) | (K)(3u - c)) & mask;
        }
        j = j0;
        jend = je;
        d = fwd <= rc ? 0u : 1u;
        pd = 0;
        yb = 0;
        if (jb) {  // occurrence jb - 1: its direction and first letter carry over
            K c;
            uint32_t b, dd;
            next(c, b, dd);
        }
    }
    __device__ __forceinline__ void empty() {
        nk = 0;
        j = jend = 0;
    }
    __device__ __forceinline__ bool done() const { return j >= jend; }
    // the current occurrence: canonical value, its <= 2 edge bits, orientation; then advance
    __device__ __forceinline__ void next(K &canon, uint32_t &bits, uint32_t &dir) {
        const bool hn = j + 1 < nk;
        K nf = fwd, nr = rc;
        uint32_t nd = 0, x = 0;
        if (hn) {
            x = letter();
            nf = (fwd >> 2) | ((K)x << sh);
            nr = ((rc << 2) | (K)(3u - x)) & mask;
            nd = nf <= nr ? 0u : 1u;
        }
        bits = 0;
        if (hn) bits |= 1u << (4 * (2 * d + nd) + (d == 0 ? x : 3u - x));
        if (j > 0) bits |= 1u << (4 * (2 * (d ^ 1u) + (pd ^ 1u)) + (d == 1 ? 3u - yb : yb));
        canon = d == 0 ? fwd : rc;
        dir = d;
        yb = (uint32_t)(fwd & (K)3);
        pd = d;
        d = nd;
        fwd = nf;
        rc = nr;
        j++;
    }
};

template <class K>
__device__ __forceinline__ void walker_for(Walker<K> &w, const uint8_t *text, unsigned long long n_text,
                                           const LineRec *lines, const uint32_t *reads, uint32_t r, int k) {
    const uint32_t rl = reads[r];
    const LineRec lr = lines[rl >> 1];
    const uint32_t mate = rl & 1u;
    w.init(text, n_text, mate ? lr.s1 : lr.s0, mate ? lr.l1 : lr.l0, k);
}

// Segment `seg` of `tpr` near-equal segments of read r's occurrences.
template <class K>
__device__ __forceinline__ void walker_for_seg(Walker<K> &w, const uint8_t *text, unsigned long long n_text,
                                               const LineRec *lines, const uint32_t *reads, uint32_t r, int k,
                                               uint32_t seg, uint32_t tpr) {
    const uint32_t rl = reads[r];
    const LineRec lr = lines[rl >> 1];
    const uint32_t mate = rl & 1u;
    const uint32_t L = mate ? lr.l1 : lr.l0, nk = L - (uint32_t)k + 1;
    const uint32_t per = (nk + tpr - 1) / tpr;
    w.init_range(text, n_text, mate ? lr.s1 : lr.s0, L, k, seg * per, seg * per + per);
}

__device__ __forceinline__ uint32_t super_of(uint64_t h, uint32_t log_s) { return (uint32_t)(h >> (64 - log_s)); }

// super bucket inside a sample (log_s may be 0) and fine bucket inside a super bucket: the
// 32 hash bits below the super bits pick the fine bucket; the low bits are left for the
// shared-memory table slot
__device__ __forceinline__ uint32_t super_local(uint64_t h, uint32_t log_s) {
    return log_s ? (uint32_t)(h >> (64 - log_s)) : 0u;
}
__device__ __forceinline__ uint32_t fine_in_super(uint64_t h, uint32_t log_s, uint32_t F) {
    return __umulhi((uint32_t)(h >> (32 - log_s)), F);
}
// sample owning read r: the last s with read_base[s] <= r (empty samples are skipped)
__device__ __forceinline__ uint32_t sample_of_read(const SampleMap &m, uint32_t r) {
    if (m.n <= 1) return 0;
    uint32_t lo = 0, hi = m.n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&m.read_base[mid]) <= r)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Exclusive scan, in place, of a shared array of n <= blockDim * 32 entries; returns the total.
__device__ uint32_t block_scan_array(uint32_t *a, uint32_t n, uint32_t *ws) {
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t t0 = min(n, threadIdx.x * per), t1 = min(n, t0 + per);
    uint32_t sum = 0;
    for (uint32_t i = t0; i < t1; i++) sum += a[i];
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(sum, ws, tot);
    for (uint32_t i = t0; i < t1; i++) {
        const uint32_t v = a[i];
        a[i] = ex;
        ex += v;
    }
    __syncthreads();
    return tot;
}

// ---- A1 -------------------------------------------------------------------------------------
template <class K>
__global__ void __launch_bounds__(256) k_count_occ(const uint8_t *text, unsigned long long n_text,
                                                   const LineRec *lines, const uint32_t *reads,
                                                   const uint32_t *n_reads_dev, int k, uint32_t log_s,
                                                   uint32_t *s_cnt, uint32_t *hll) {
    __shared__ uint32_t hist[MAX_SUPERS];
    __shared__ uint32_t reg[HLL_REGS];
    const uint32_t S = 1u << log_s;
    for (uint32_t i = threadIdx.x; i < S; i += blockDim.x) hist[i] = 0;
    for (uint32_t i = threadIdx.x; i < HLL_REGS; i += blockDim.x) reg[i] = 0;
    __syncthreads();
    const uint32_t n_reads = *n_reads_dev;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += gridDim.x * blockDim.x) {
        Walker<K> w;
        walker_for(w, text, n_text, lines, reads, r, k);
        while (!w.done()) {
            K c;
            uint32_t b, d;
            w.next(c, b, d);
            const uint64_t h = KeyOps<K>::hash(c);
            atomicAdd(&hist[super_of(h, log_s)], 1u);
            const uint64_t w2 = h >> 11;  // HyperLogLog: register = low 11 bits, rank of the rest
            const uint32_t rho = w2 ? (uint32_t)(__clzll(w2) - 10) : 54u;
            atomicMax(&reg[h & (HLL_REGS - 1)], rho);
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < S; i += blockDim.x)
        if (hist[i]) atomicAdd(&s_cnt[i], hist[i]);
    for (uint32_t i = threadIdx.x; i < HLL_REGS; i += blockDim.x)
        if (reg[i]) atomicMax(&hll[i], reg[i]);
}

// HyperLogLog (Flajolet, Fusy, Gandouet, Meunier 2007) with the small-range correction
double hll_estimate(const uint32_t *regs, int n_regs) {
    const double m = n_regs;
    double z = 0;
    int zeros = 0;
    for (int i = 0; i < n_regs; i++) {
        z += ldexp(1.0, -(int)regs[i]);
        if (regs[i] == 0) zeros++;
    }
    const double alpha = 0.7213 / (1.0 + 1.079 / m);
    double e = alpha * m * m / z;
    if (e <= 2.5 * m && zeros > 0) e = m * log(m / zeros);
    return e;
}

PartPlan plan_partitions(double distinct_est, double safety, double target) {
    double want = distinct_est * safety / target;
    if (want < 1) want = 1;
    uint64_t P = (uint64_t)ceil(want);
    uint32_t log_s = 0;
    while ((1ull << (2 * log_s)) < P && log_s < 11) log_s++;  // S ~ sqrt(P)
    // then half of that while the fine buckets per super bucket stay within MAX_FINE: fewer bins
    // per super-scatter round, still long runs in the fine pass (measured: 3 % off the partition)
    if (log_s > 6 && ((P + (1ull << (log_s - 1)) - 1) >> (log_s - 1)) <= MAX_FINE) log_s--;
    if (log_s < 6) log_s = 6;
    const uint64_t S = 1ull << log_s;
    uint64_t F = (P + S - 1) / S;
    if (F < 1) F = 1;
    if (F > MAX_FINE) F = MAX_FINE;
    PartPlan pp;
    pp.log_s = log_s;
    pp.F = (uint32_t)F;
    pp.P = (uint32_t)(S * F);
    return pp;
}

void launch_count_occ(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines, const uint32_t *reads,
                      const uint32_t *n_reads_dev, uint32_t n_reads_max, int k, uint32_t log_s, uint32_t *s_cnt,
                      uint32_t *hll, cudaStream_t s) {
    if (!n_reads_max) return;
    const unsigned blocks = (unsigned)std::min<uint64_t>((n_reads_max + 255) / 256, 152ull * 8);
    t_launches++;
    if (wide)
        k_count_occ<u128><<<blocks, 256, 0, s>>>(text, n_text, lines, reads, n_reads_dev, k, log_s, s_cnt, hll);
    else
        k_count_occ<uint64_t><<<blocks, 256, 0, s>>>(text, n_text, lines, reads, n_reads_dev, k, log_s, s_cnt,
                                                     hll);
}

// Batched A1.  Each CTA takes a contiguous range of reads and walks it one sample segment at a
// time, with the segment's super histogram and HyperLogLog registers in shared memory.
template <class K>
__global__ void __launch_bounds__(256) k_count_occ_batch(const uint8_t *text, unsigned long long n_text,
                                                         const LineRec *lines, const uint32_t *reads,
                                                         const uint32_t *read_base, uint32_t n_samples, int k,
                                                         uint32_t *s_cnt, uint32_t *hll) {
    __shared__ uint32_t hist[MAX_SUPERS];
    __shared__ uint32_t reg[HLL_REGS];
    const uint32_t n_reads = read_base[n_samples];
    uint32_t r0 = (uint32_t)((unsigned long long)blockIdx.x * n_reads / gridDim.x);
    const uint32_t r1 = (uint32_t)((unsigned long long)(blockIdx.x + 1) * n_reads / gridDim.x);
    SampleMap m{read_base, nullptr, n_samples};
    uint32_t smp = r0 < r1 ? sample_of_read(m, r0) : n_samples;
    while (r0 < r1) {
        const uint32_t seg_end = min(r1, read_base[smp + 1]);
        for (uint32_t i = threadIdx.x; i < MAX_SUPERS; i += blockDim.x) hist[i] = 0;
        for (uint32_t i = threadIdx.x; i < HLL_REGS; i += blockDim.x) reg[i] = 0;
        __syncthreads();
        for (uint32_t r = r0 + threadIdx.x; r < seg_end; r += blockDim.x) {
            Walker<K> w;
            walker_for(w, text, n_text, lines, reads, r, k);
            while (!w.done()) {
                K c;
                uint32_t b, d;
                w.next(c, b, d);
                const uint64_t h = KeyOps<K>::hash(c);
                atomicAdd(&hist[(uint32_t)(h >> 53)], 1u);
                const uint64_t w2 = h >> 11;
                const uint32_t rho = w2 ? (uint32_t)(__clzll(w2) - 10) : 54u;
                atomicMax(&reg[h & (HLL_REGS - 1)], rho);
            }
        }
        __syncthreads();
        uint32_t *gc = s_cnt + (size_t)smp * MAX_SUPERS, *gh = hll + (size_t)smp * HLL_REGS;
        for (uint32_t i = threadIdx.x; i < MAX_SUPERS; i += blockDim.x)
            if (hist[i]) atomicAdd(&gc[i], hist[i]);
        for (uint32_t i = threadIdx.x; i < HLL_REGS; i += blockDim.x)
            if (reg[i]) atomicMax(&gh[i], reg[i]);
        __syncthreads();
        r0 = seg_end;
        smp++;
        while (smp < n_samples && read_base[smp + 1] <= r0) smp++;  // skip empty samples
    }
}

void launch_count_occ_batch(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines,
                            const uint32_t *reads, const uint32_t *read_base, uint32_t n_samples,
                            uint32_t n_reads_max, int k, uint32_t *s_cnt, uint32_t *hll, cudaStream_t s) {
    if (!n_reads_max || !n_samples) return;
    const unsigned blocks = (unsigned)std::min<uint64_t>((n_reads_max + 255) / 256, 152ull * 8);
    t_launches++;
    if (wide)
        k_count_occ_batch<u128><<<blocks, 256, 0, s>>>(text, n_text, lines, reads, read_base, n_samples, k, s_cnt,
                                                       hll);
    else
        k_count_occ_batch<uint64_t><<<blocks, 256, 0, s>>>(text, n_text, lines, reads, read_base, n_samples, k,
                                                           s_cnt, hll);
}

__global__ void k_sample_bounds(const unsigned long long *text_base, uint32_t n_samples,
                                const unsigned long long *line_end, uint32_t n_lines, const uint32_t *nvalid,
                                const uint32_t *nvalid_total, uint32_t *line_base, uint32_t *read_base) {
    const uint32_t smp = blockIdx.x * blockDim.x + threadIdx.x;
    if (smp > n_samples) return;
    uint32_t lb = n_lines;
    if (smp < n_samples) {
        // first line whose terminator lies at or after the sample's first byte
        const unsigned long long tb = text_base[smp];
        uint32_t lo = 0, hi = n_lines;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (line_end[mid] < tb)
                lo = mid + 1;
            else
                hi = mid;
        }
        lb = lo;
    }
    line_base[smp] = lb;
    read_base[smp] = lb < n_lines ? nvalid[lb] : *nvalid_total;
}

void launch_sample_bounds(const unsigned long long *text_base, uint32_t n_samples,
                          const unsigned long long *line_end, uint32_t n_lines, const uint32_t *nvalid,
                          const uint32_t *nvalid_total, uint32_t *line_base, uint32_t *read_base, cudaStream_t s) {
    t_launches++;
    k_sample_bounds<<<(n_samples + 1 + 127) / 128, 128, 0, s>>>(text_base, n_samples, line_end, n_lines, nvalid,
                                                                nvalid_total, line_base, read_base);
}

// Occurrences of every sample: each thread its read's L - k + 1, summed over the runs of one
// sample inside the warp (reads are in sample order), one atomic per run.
__global__ void k_sample_occ(const LineRec *lines, const uint32_t *reads, int k, SampleMap m,
                             unsigned long long *occ) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n_reads = m.read_base[m.n];  // the grid covers an upper bound
    unsigned long long v = 0;
    uint32_t smp = 0xffffffffu;
    if (r < n_reads) {
        const uint32_t rl = reads[r];
        const LineRec lr = lines[rl >> 1];
        v = (rl & 1u ? lr.l1 : lr.l0) - (uint32_t)k + 1;
        smp = sample_of_read(m, r);
    }
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = shfl64_up(inc, o);
        if (lane >= o) inc += y;
    }
    const uint32_t s_next = __shfl_down_sync(full, smp, 1);
    const bool end = lane == 31 || s_next != smp;
    const uint32_t ends = __ballot_sync(full, end);
    const uint32_t below = ends & ((1u << lane) - 1u);
    const int pe = below ? 31 - __clz(below) : 0;
    const unsigned long long before = shfl64(inc, pe);
    if (end && smp != 0xffffffffu) atomicAdd(&occ[smp], inc - (below ? before : 0ull));
}

void launch_sample_occ(const LineRec *lines, const uint32_t *reads, uint32_t n_reads_max, int k, SampleMap m,
                       unsigned long long *occ, cudaStream_t s) {
    if (!n_reads_max) return;
    t_launches++;
    k_sample_occ<<<(n_reads_max + 255) / 256, 256, 0, s>>>(lines, reads, k, m, occ);
}

// ---- A2 -------------------------------------------------------------------------------------
// A round's k-mers stay in registers between counting and placing them (ten per thread with
// 64-bit keys, where more spill; twelve with 128-bit keys, whose walk, done twice, cost more
// than the registers of its cache).
template <class K> struct SuperRound {
    static constexpr bool CACHE = true;
    static constexpr int N = sizeof(K) == 8 ? 10 : 12;  // k-mers per thread per round
};

// shared layout of k_scatter_super: staging for one round, then four S-entry arrays
template <class K>
struct SuperSmem {
    K key[SC_THREADS * SuperRound<K>::N];
    uint16_t bits[SC_THREADS * SuperRound<K>::N];
    uint16_t sup[SC_THREADS * SuperRound<K>::N];
    uint32_t ws[33];
    uint32_t rounds, total;
    uint32_t hll[SC_HLL_REGS];  // this block's HyperLogLog registers (when the build asks for them)
    uint32_t arrays[1];  // loff[S], gbase[S], cur[S], glo[S]
    static size_t bytes(uint32_t S) { return sizeof(SuperSmem) + 4ull * S * sizeof(uint32_t); }
};


template <class K>
__global__ void __launch_bounds__(SC_THREADS, sizeof(K) == 8 ? 4 : 2) k_scatter_super(const uint8_t *text, unsigned long long n_text,
                                                              const LineRec *lines,
                                                              const uint32_t *reads, uint32_t n_reads, int k,
                                                              SampleMap m, uint32_t S,
                                                              const unsigned long long *s_off,
                                                              uint32_t *s_cur, K *okey, uint16_t *obits,
                                                              uint32_t cap, uint32_t *hll, uint32_t *ovf,
                                                              uint32_t tpr) {
    constexpr bool CACHE = SuperRound<K>::CACHE;
    constexpr int RN = SuperRound<K>::N;
    extern __shared__ __align__(16) uint8_t smem_raw[];
    SuperSmem<K> &sm = *reinterpret_cast<SuperSmem<K> *>(smem_raw);
    uint32_t *const sm_loff = sm.arrays, *const sm_gbase = sm.arrays + S, *const sm_cur = sm.arrays + 2 * S;
    uint32_t *const sm_glo = sm.arrays + 3 * S;
    // tpr threads per read (a power of two up to 32): thread t walks segment t % tpr of read
    // t / tpr, so a read's occurrences are spread over tpr threads of one warp
    const uint32_t lg_tpr = 31 - __clz(tpr), per_cta = SC_THREADS >> lg_tpr;
    const uint32_t r = blockIdx.x * per_cta + (threadIdx.x >> lg_tpr);
    Walker<K> w;
    uint32_t sbase = 0, log_s = 0;
    if (r < n_reads) {
        if (tpr == 1)
            walker_for(w, text, n_text, lines, reads, r, k);
        else
            walker_for_seg(w, text, n_text, lines, reads, r, k, threadIdx.x & (tpr - 1), tpr);
        const SamplePlan pl = m.plan[sample_of_read(m, r)];
        sbase = pl.super_base;
        log_s = pl.log_s;
    } else {
        w.empty();
    }
    // The super buckets this CTA can reach: its reads lie in a run of consecutive samples, which
    // own a contiguous range of buckets (a plain job: all of them).  The per-round loops below
    // cover that range only, so a batch of many samples pays for its own samples' buckets.
    uint32_t lo = 0, hi = S, sa = 0, sb = 0;
    if (m.n > 1) {
        const uint32_t ra = blockIdx.x * per_cta, rb = min(n_reads, ra + per_cta) - 1;
        sa = sample_of_read(m, ra);
        sb = sample_of_read(m, rb);
        const SamplePlan pa = m.plan[sa], pb = m.plan[sb];
        lo = pa.super_base;
        hi = pb.super_base + (1u << pb.log_s);
    }
    // HyperLogLog registers: SC_HLL_REGS per sample at hll + sample * SC_HLL_REGS, gathered in
    // shared memory when the CTA's reads are of one sample (nearly always), else directly
    const uint32_t my_s = (m.n > 1 && r < n_reads) ? sample_of_read(m, r) : 0u;
    const bool hll_smem = sa == sb;
    if (threadIdx.x == 0) sm.rounds = 0;
    if (hll)
        for (uint32_t i = threadIdx.x; i < SC_HLL_REGS; i += blockDim.x) sm.hll[i] = 0;
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) sm_cur[i] = 0;  // then by each round's write-out
    __syncthreads();
    atomicMax(&sm.rounds, (w.jend - w.j + RN - 1) / RN);
    __syncthreads();
    const uint32_t rounds = sm.rounds;
    K ck[CACHE ? RN : 1];
    uint32_t cb[CACHE ? RN : 1];  // edge bits | super << 16
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t round = 0; round < rounds; round++) {
        const Walker<K> w0 = w;
        const uint32_t nq = w.j < w.jend ? min((uint32_t)RN, w.jend - w.j) : 0u;
        // count this round's occurrences per super bucket
#pragma unroll
        for (int q = 0; q < RN; q++) {
            if ((uint32_t)q >= nq) break;
            K c;
            uint32_t b, d;
            w.next(c, b, d);
            const uint64_t h = KeyOps<K>::hash(c);
            const uint32_t sp = sbase + super_local(h, log_s);
            atomicAdd(&sm_cur[sp], 1u);
            if (hll) {
                const uint64_t w2 = h >> 9;  // HyperLogLog: register = low 9 bits, rank of the rest
                const uint32_t rho = w2 ? (uint32_t)(__clzll(w2) - 8) : 56u;
                if (hll_smem)
                    atomicMax(&sm.hll[h & (SC_HLL_REGS - 1)], rho);
                else
                    atomicMax(&hll[(size_t)my_s * SC_HLL_REGS + (h & (SC_HLL_REGS - 1))], rho);
            }
            if (CACHE) {
                ck[q] = c;
                cb[q] = b | (sp << 16);
            }
        }
        __syncthreads();
        // Each bucket claims its run in global memory (s_cur) and gets its offset in the round's
        // staging (loff, exclusive).  Element i of bucket sp then goes to s_off[sp] + claim +
        // (i - loff[sp]): that base is kept as gbase (high word, ~0 for a bucket out of room)
        // and glo (low word).
        uint32_t tot;
        if (hi - lo <= SC_THREADS) {
            // one bucket per thread: its claim is in flight while the block scans the counts
            const uint32_t i = lo + threadIdx.x;
            const bool mine = i < hi;
            const uint32_t c = mine ? sm_cur[i] : 0u;
            const uint32_t g = c ? atomicAdd(&s_cur[i], c) : 0u;
            const uint32_t inc = warp_inclusive_scan(c);
            if (lane == 31) sm.ws[warp] = inc;
            __syncthreads();
            uint32_t before = 0;
            tot = 0;
#pragma unroll
            for (int q = 0; q < SC_THREADS / 32; q++) {
                const uint32_t x = sm.ws[q];
                if (q < warp) before += x;
                tot += x;
            }
            if (mine) {
                const uint32_t ex = before + inc - c;
                sm_loff[i] = ex;
                const unsigned long long room = cap ? (unsigned long long)cap : s_off[i + 1] - s_off[i];
                if (c && (unsigned long long)g + c > room) {  // the bucket's room is used up: nothing of it is written
                    atomicOr(ovf, 1u);
                    sm_gbase[i] = 0xffffffffu;
                } else {
                    const unsigned long long b = s_off[i] + g - ex;
                    sm_glo[i] = (uint32_t)b;
                    sm_gbase[i] = (uint32_t)(b >> 32);
                }
            }
        } else {
            for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
                const uint32_t c = sm_cur[i];
                sm_loff[i] = c;
                uint32_t g = c ? atomicAdd(&s_cur[i], c) : 0u;
                const unsigned long long room = cap ? (unsigned long long)cap : s_off[i + 1] - s_off[i];
                if (c && (unsigned long long)g + c > room) {
                    atomicOr(ovf, 1u);
                    g = 0xffffffffu;
                }
                sm_gbase[i] = g;
            }
            __syncthreads();
            tot = block_scan_array(sm_loff + lo, hi - lo, sm.ws);
            for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
                const uint32_t g = sm_gbase[i];
                if (g != 0xffffffffu) {
                    const unsigned long long b = s_off[i] + g - sm_loff[i];
                    sm_glo[i] = (uint32_t)b;
                    sm_gbase[i] = (uint32_t)(b >> 32);
                }
            }
        }
        __syncthreads();
        // place them in shared memory grouped by super bucket
        if (!CACHE) w = w0;
#pragma unroll
        for (int q = 0; q < RN; q++) {
            if ((uint32_t)q >= nq) break;
            K c;
            uint32_t b, sp;
            if (CACHE) {
                c = ck[q];
                b = cb[q] & 0xffffu;
                sp = cb[q] >> 16;
            } else {
                uint32_t d;
                w.next(c, b, d);
                sp = sbase + super_local(KeyOps<K>::hash(c), log_s);
            }
            const uint32_t pos = atomicAdd(&sm_loff[sp], 1u);  // loff runs through the bucket's staging
            sm.key[pos] = c;
            sm.bits[pos] = (uint16_t)b;
            sm.sup[pos] = (uint16_t)sp;
        }
        __syncthreads();
        // write the runs out; the counts start from zero for the next round
        for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) sm_cur[i] = 0;
        for (uint32_t i = threadIdx.x; i < tot; i += blockDim.x) {
            const uint32_t sp = sm.sup[i], hi = sm_gbase[sp];
            if (hi == 0xffffffffu) continue;
            const unsigned long long g = (((unsigned long long)hi << 32) | sm_glo[sp]) + i;
            okey[g] = sm.key[i];
            obits[g] = sm.bits[i];
        }
        __syncthreads();
    }
    if (hll && hll_smem)
        for (uint32_t i = threadIdx.x; i < SC_HLL_REGS; i += blockDim.x)
            if (sm.hll[i]) atomicMax(&hll[(size_t)sa * SC_HLL_REGS + i], sm.hll[i]);
}

void launch_scatter_super(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines,
                          const uint32_t *reads, uint32_t n_reads, int k, SampleMap m, uint32_t n_super,
                          const unsigned long long *s_off, uint32_t *s_cur, void *okey, uint16_t *obits,
                          uint32_t cap, uint32_t *hll, uint32_t *ovf, cudaStream_t s, uint32_t tpr) {
    if (!n_reads) return;
    if (tpr < 1 || tpr > 32 || (tpr & (tpr - 1))) tpr = 1;
    const unsigned blocks = (unsigned)(((uint64_t)n_reads * tpr + SC_THREADS - 1) / SC_THREADS);
    t_launches++;
    if (wide) {
        const size_t sm = SuperSmem<u128>::bytes(n_super);
        cudaFuncSetAttribute(k_scatter_super<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_scatter_super<u128><<<blocks, SC_THREADS, sm, s>>>(text, n_text, lines, reads, n_reads, k, m, n_super,
                                                             s_off, s_cur, (u128 *)okey, obits, cap, hll, ovf, tpr);
    } else {
        const size_t sm = SuperSmem<uint64_t>::bytes(n_super);
        cudaFuncSetAttribute(k_scatter_super<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_scatter_super<uint64_t><<<blocks, SC_THREADS, sm, s>>>(text, n_text, lines, reads, n_reads, k, m,
                                                                 n_super, s_off, s_cur, (uint64_t *)okey, obits, cap,
                                                                 hll, ovf, tpr);
    }
}

// the CHUNK-sized pieces of each super bucket, (start, super << 32 | length), super by super:
// bucket q's pieces are chunks[cbase[q] .. cbase[q + 1])
__global__ void k_make_chunks(const unsigned long long *soff, const uint32_t *scount, const uint32_t *cbase,
                              uint32_t S, ulonglong2 *chunks) {
    for (uint32_t q = blockIdx.x; q < S; q += gridDim.x) {
        const uint32_t c0 = cbase[q], nc = cbase[q + 1] - c0, cnt = scount[q];
        const unsigned long long base = soff[q];
        for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) {
            const uint32_t st = c * CHUNK;
            const uint32_t len = min(CHUNK, cnt - st);
            chunks[c0 + c] = make_ulonglong2(base + st, ((unsigned long long)q << 32) | len);
        }
    }
}

void launch_make_chunks(const unsigned long long *soff, const uint32_t *scount, const uint32_t *cbase, uint32_t S,
                        ulonglong2 *chunks, cudaStream_t s) {
    if (!S) return;
    t_launches++;
    k_make_chunks<<<S, 256, 0, s>>>(soff, scount, cbase, S, chunks);
}

// ---- B1 -------------------------------------------------------------------------------------
constexpr int FINE_PER_THREAD = CHUNK / 256;  // occurrences of a chunk per thread

template <class K>
__global__ void __launch_bounds__(256) k_fine_count(const K *okey, const ulonglong2 *chunks, const SuperInfo *sinfo,
                                                    unsigned long long *fine_cnt) {
    __shared__ uint32_t bins[MAX_FINE];
    const ulonglong2 ch = chunks[blockIdx.x];
    const uint32_t sp = (uint32_t)(ch.y >> 32), len = (uint32_t)ch.y;
    const SuperInfo si = sinfo[sp];
    for (uint32_t i = threadIdx.x; i < si.F; i += blockDim.x) bins[i] = 0;
    // all of the thread's loads first, then the bins
    K kk[FINE_PER_THREAD];
#pragma unroll
    for (int q = 0; q < FINE_PER_THREAD; q++) {
        const uint32_t i = q * 256 + threadIdx.x;
        kk[q] = i < len ? okey[ch.x + i] : (K)0;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < FINE_PER_THREAD; q++)
        if (q * 256 + threadIdx.x < len)
            atomicAdd(&bins[fine_in_super(KeyOps<K>::hash(kk[q]), si.log_s, si.F)], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < si.F; i += blockDim.x)
        if (bins[i]) atomicAdd(&fine_cnt[si.fine_first + i], (unsigned long long)bins[i]);
}

void launch_fine_count(int wide, const void *okey, const ulonglong2 *chunks, uint32_t n_chunks,
                       const SuperInfo *sinfo, unsigned long long *fine_cnt, cudaStream_t s) {
    if (!n_chunks) return;
    t_launches++;
    if (wide)
        k_fine_count<u128><<<n_chunks, 256, 0, s>>>((const u128 *)okey, chunks, sinfo, fine_cnt);
    else
        k_fine_count<uint64_t><<<n_chunks, 256, 0, s>>>((const uint64_t *)okey, chunks, sinfo, fine_cnt);
}

// ---- B2 -------------------------------------------------------------------------------------
constexpr int FINE_BOOK = 2;  // fine buckets per thread in the scatter's fast bookkeeping (F <= 512)
template <class K>
struct FineSmem {
    K key[CHUNK];
    uint16_t bits[CHUNK];
    uint16_t bkt[CHUNK];
    uint32_t loff[MAX_FINE];
    uint32_t gbase[MAX_FINE];
    uint32_t cur[MAX_FINE];
    uint32_t ws[33];
};

template <class K>
__global__ void __launch_bounds__(256, sizeof(K) == 8 ? 3 : 2) k_scatter_fine(const K *okey, const uint16_t *obits, const ulonglong2 *chunks,
                                                      const SuperInfo *sinfo, const unsigned long long *fine_off,
                                                      uint32_t *fine_cur, K *okey2, uint16_t *obits2) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    FineSmem<K> &sm = *reinterpret_cast<FineSmem<K> *>(smem_raw);
    const ulonglong2 ch = chunks[blockIdx.x];
    const uint32_t sp = (uint32_t)(ch.y >> 32), len = (uint32_t)ch.y;
    const SuperInfo si = sinfo[sp];
    const uint32_t f0 = si.fine_first, F = si.F, log_s = si.log_s;
    for (uint32_t i = threadIdx.x; i < F; i += blockDim.x) sm.cur[i] = 0;
    // the thread's occurrences stay in registers between the count and the placement
    K kk[FINE_PER_THREAD];
    uint32_t bk[FINE_PER_THREAD / 2];  // two fine-bucket indexes per word
    uint32_t bb[FINE_PER_THREAD / 2];  // two edge-bit words per word
#pragma unroll
    for (int q = 0; q < FINE_PER_THREAD; q++) {
        const uint32_t i = q * 256 + threadIdx.x;
        kk[q] = i < len ? okey[ch.x + i] : (K)0;
        const uint32_t bits = i < len ? (uint32_t)obits[ch.x + i] : 0u;
        if (q & 1)
            bb[q >> 1] |= bits << 16;
        else
            bb[q >> 1] = bits;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < FINE_PER_THREAD; q++) {
        const uint32_t bkt = fine_in_super(KeyOps<K>::hash(kk[q]), log_s, F);
        if (q & 1)
            bk[q >> 1] |= bkt << 16;
        else
            bk[q >> 1] = bkt;
        if (q * 256 + threadIdx.x < len) atomicAdd(&sm.cur[bkt], 1u);
    }
    __syncthreads();
    // Each bucket claims its run of the fine bucket (fine_cur) and gets its offset in the
    // chunk's staging (loff, exclusive).  Element i of bucket b (staged at loff[b] + its rank)
    // goes to fine_off[f0 + b] + claim + rank = base0 + gbase'[b] + i, with gbase'[b] =
    // fine_off[f0 + b] - base0 + claim - loff[b]: never negative (loff[b] counts this chunk's
    // part of the buckets before b) and below the super bucket's 32-bit size, so the write-out
    // needs no global load per element.
    const unsigned long long base0 = fine_off[f0];
    const uint32_t per = (F + blockDim.x - 1) / blockDim.x;
    if (per <= FINE_BOOK) {
        // a thread's (at most FINE_BOOK) consecutive buckets: their claims are in flight while the
        // block scans the counts
        const uint32_t b0 = threadIdx.x * per;
        uint32_t c[FINE_BOOK], g[FINE_BOOK], sum = 0;
#pragma unroll
        for (int q = 0; q < FINE_BOOK; q++) {
            const uint32_t i = b0 + q;
            c[q] = ((uint32_t)q < per && i < F) ? sm.cur[i] : 0u;
            g[q] = c[q] ? atomicAdd(&fine_cur[f0 + i], c[q]) : 0u;
            sum += c[q];
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const uint32_t inc = warp_inclusive_scan(sum);
        if (lane == 31) sm.ws[warp] = inc;
        __syncthreads();
        uint32_t ex = inc - sum;
#pragma unroll
        for (int q = 0; q < 8; q++)
            if (q < warp) ex += sm.ws[q];
#pragma unroll
        for (int q = 0; q < FINE_BOOK; q++) {
            const uint32_t i = b0 + q;
            if ((uint32_t)q < per && i < F) {
                sm.loff[i] = ex;
                sm.gbase[i] = (uint32_t)(fine_off[f0 + i] - base0) + g[q] - ex;
                ex += c[q];
            }
        }
    } else {
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x) {
            sm.loff[i] = sm.cur[i];
            sm.gbase[i] = sm.cur[i] ? atomicAdd(&fine_cur[f0 + i], sm.cur[i]) : 0u;
        }
        __syncthreads();
        block_scan_array(sm.loff, F, sm.ws);
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x)
            sm.gbase[i] = (uint32_t)(fine_off[f0 + i] - base0) + sm.gbase[i] - sm.loff[i];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < FINE_PER_THREAD; q++) {
        if (q * 256 + threadIdx.x >= len) continue;
        const uint32_t bkt = (bk[q >> 1] >> (16 * (q & 1))) & 0xffffu;
        const uint32_t pos = atomicAdd(&sm.loff[bkt], 1u);  // loff runs through the bucket's staging
        sm.key[pos] = kk[q];
        sm.bits[pos] = (uint16_t)(bb[q >> 1] >> (16 * (q & 1)));
        sm.bkt[pos] = (uint16_t)bkt;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) {
        const unsigned long long g = base0 + sm.gbase[sm.bkt[i]] + i;
        okey2[g] = sm.key[i];
        obits2[g] = sm.bits[i];
    }
}

void launch_scatter_fine(int wide, const void *okey, const uint16_t *obits, const ulonglong2 *chunks,
                         uint32_t n_chunks, const SuperInfo *sinfo, const unsigned long long *fine_off,
                         uint32_t *fine_cur, void *okey2, uint16_t *obits2, cudaStream_t s) {
    if (!n_chunks) return;
    t_launches++;
    if (wide) {
        const size_t sm = sizeof(FineSmem<u128>);
        cudaFuncSetAttribute(k_scatter_fine<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_scatter_fine<u128><<<n_chunks, 256, sm, s>>>((const u128 *)okey, obits, chunks, sinfo, fine_off, fine_cur,
                                                      (u128 *)okey2, obits2);
    } else {
        const size_t sm = sizeof(FineSmem<uint64_t>);
        cudaFuncSetAttribute(k_scatter_fine<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_scatter_fine<uint64_t><<<n_chunks, 256, sm, s>>>((const uint64_t *)okey, obits, chunks, sinfo, fine_off,
                                                          fine_cur, (uint64_t *)okey2, obits2);
    }
}

// ---- read heads (partitioned build) ----------------------------------------------------------
template <class K>
__global__ void k_heads_part(const uint8_t *text, unsigned long long n_text, const LineRec *lines,
                             const uint32_t *reads, uint32_t n_reads,
                             int k, SampleMap m, Head *heads, uint32_t *head_cnt) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_reads) return;
    Walker<K> w;
    walker_for(w, text, n_text, lines, reads, r, k);
    K c;
    uint32_t b, d;
    w.next(c, b, d);
    const uint32_t mate = reads[r] & 1u;
    const long long rid = lines[reads[r] >> 1].read_id;
    const SamplePlan pl = m.plan[sample_of_read(m, r)];
    const uint64_t h = KeyOps<K>::hash(c);
    const uint32_t f = pl.fine_base + super_local(h, pl.log_s) * pl.F + fine_in_super(h, pl.log_s, pl.F);
    Head hd;
    hd.part = f;
    hd.slot = 0;
    hd.uuid = ((unsigned long long)(d == 0 ? 0 : k - 1) << 40) | ((unsigned long long)mate << 35) |
              (unsigned long long)rid;
    hd.klo = (unsigned long long)c;
    hd.khi = (unsigned long long)((u128)c >> 64);
    heads[r] = hd;
    atomicAdd(&head_cnt[f], 1u);
}

void launch_heads_part(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines, const uint32_t *reads,
                       uint32_t n_reads, int k, SampleMap m, Head *heads, uint32_t *head_cnt, cudaStream_t s) {
    if (!n_reads) return;
    t_launches++;
    if (wide)
        k_heads_part<u128><<<(n_reads + 255) / 256, 256, 0, s>>>(text, n_text, lines, reads, n_reads, k, m, heads,
                                                                head_cnt);
    else
        k_heads_part<uint64_t><<<(n_reads + 255) / 256, 256, 0, s>>>(text, n_text, lines, reads, n_reads, k, m,
                                                                    heads, head_cnt);
}

// ---- C --------------------------------------------------------------------------------------
template <class K> struct AggTable;
template <> struct AggTable<uint64_t> {
    // stored key = V + 1, 0 = empty; every probe is a CAS so a racing claim is never missed
    __device__ __forceinline__ static int insert(uint64_t *key1, uint64_t key, uint32_t h, uint32_t &claimed) {
        const unsigned long long want = (unsigned long long)key + 1ULL;
        uint32_t i = h & (AGG_SLOTS - 1);
        for (uint32_t n = 0; n < AGG_SLOTS; n++) {
            unsigned long long cur = ((volatile unsigned long long *)key1)[i];
            if (cur != want) cur = atomicCAS((unsigned long long *)&key1[i], 0ULL, want);
            if (cur == 0ULL) claimed = 1;
            if (cur == 0ULL || cur == want) return (int)i;
            i = (i + 1) & (AGG_SLOTS - 1);
        }
        return -1;
    }
    __device__ __forceinline__ static int find(const uint64_t *key1, uint64_t key, uint32_t h) {
        const uint64_t want = key + 1;
        uint32_t i = h & (AGG_SLOTS - 1);
        for (uint32_t n = 0; n < AGG_SLOTS; n++) {
            const uint64_t cur = key1[i];
            if (cur == want) return (int)i;
            if (cur == 0) return -1;
            i = (i + 1) & (AGG_SLOTS - 1);
        }
        return -1;
    }
};
template <> struct AggTable<u128> {
    __device__ __forceinline__ static int insert(u128 *key1, u128 key, uint32_t h, uint32_t &claimed) {
        const u128 want = key + 1;
        const unsigned long long wlo = (unsigned long long)want, whi = (unsigned long long)(want >> 64);
        uint32_t i = h & (AGG_SLOTS - 1);
        for (uint32_t n = 0; n < AGG_SLOTS; n++) {
            unsigned long long clo, chi;
            cas128_shared(&key1[i], 0ULL, 0ULL, wlo, whi, clo, chi);
            if (clo == 0ULL && chi == 0ULL) claimed = 1;
            if ((clo == 0ULL && chi == 0ULL) || (clo == wlo && chi == whi)) return (int)i;
            i = (i + 1) & (AGG_SLOTS - 1);
        }
        return -1;
    }
    __device__ __forceinline__ static int find(const u128 *key1, u128 key, uint32_t h) {
        const u128 want = key + 1;
        uint32_t i = h & (AGG_SLOTS - 1);
        for (uint32_t n = 0; n < AGG_SLOTS; n++) {
            const u128 cur = key1[i];
            if (cur == want) return (int)i;
            if (cur == 0) return -1;
            i = (i + 1) & (AGG_SLOTS - 1);
        }
        return -1;
    }
};

// Home slot of a key in a bucket's shared table: the top 11 bits of a multiplicative hash (the
// bucket itself was picked by other bits of the MurmurHash3 finaliser).
__device__ __forceinline__ uint32_t agg_home(uint64_t v) {
    return (uint32_t)((v * 0x9E3779B97F4A7C15ULL) >> (64 - 11));
}
__device__ __forceinline__ uint32_t agg_home(u128 v) {
    const uint64_t x = (uint64_t)v ^ ((uint64_t)(v >> 64) * 0xC2B2AE3D27D4EB4FULL);
    return (uint32_t)((x * 0x9E3779B97F4A7C15ULL) >> (64 - 11));
}
static_assert(AGG_SLOTS == 1u << 11, "agg_home gives 11-bit slots");

// One fine bucket per CTA.  The bucket's distinct k-mers are counted in a shared-memory
// open-addressing table (linear probing), then put in a deterministic order without sorting:
// with linear probing the set of occupied slots, and the set of keys in each cluster (maximal
// run of occupied slots), depend only on the keys, not on the order of the inserts.  So nodes
// are numbered cluster by cluster, starting after the first empty slot, and by key inside a
// cluster (a cluster that wraps past the last slot is numbered last).  Five phases with a
// barrier between them:
//   1. read heads (which claim or find their k-mer's slot and mark the set they belong to)
//      and occurrences inserted: count += 1, edge bits OR-ed in;
//   2. occupancy bitmap (warp ballots) and per-warp counts;
//   3. every node's rank: its cluster's start, the occupied slots before it, its place by key
//      in the cluster; key, count/meta word and base record size out;
//   4. warp 0 sorts, de-duplicates and sizes the read heads (at most 32: registers and
//      shuffles) while warps 1-7 scan the base record sizes;
//   5. record offsets (base offset + bytes of the kept heads of earlier nodes) and the read
//      heads' output entries.
// A bucket with more than 32 read heads sorts them with the whole block after phase 3 and
// scans sizes that include them (the general path, rare).
template <class K>
struct AggSmem {
    K key1[AGG_SLOTS];                 // key + 1; 0 = empty
    uint32_t cnt[AGG_SLOTS];           // occurrences
    uint32_t meta[AGG_SLOTS];          // edge bits, read-head set flags
    uint32_t nbytes[AGG_SLOTS];        // record bytes per node in rank order, then offsets
    uint16_t ord[AGG_SLOTS];           // slot of the node of each rank
    uint16_t rank_of_slot[AGG_SLOTS];
    uint32_t occ[AGG_SLOTS / 32];      // occupancy bitmap
    uint32_t wtot[8];                  // occupied slots in each warp's 256 slots
    uint32_t ws7[8];                   // warps 1-7's scan
    unsigned long long ws[33];
    unsigned long long wsk[32];        // warp 0's head sort
    uint32_t wsv[32];
    uint32_t hrank[32];                // kept read heads in order: their node's rank ...
    uint32_t hcum[33];                 // ... and the bytes of the kept heads before each
    unsigned long long carry;
    uint32_t n, fail, kept, base_total;
};

constexpr int AGG_BATCH = 8;  // occurrence loads in flight per thread
static_assert(AGG_SLOTS == 2048, "k_aggregate maps 8 warps x 8 ballots onto the table");

// first of the kept head keys (sorted) that is >= x
__device__ __forceinline__ uint32_t kept_lower_bound(const unsigned long long *hk, uint32_t kept,
                                                     unsigned long long x) {
    uint32_t lo = 0, hi = kept;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (hk[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void bar_named(int id, int threads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// Exclusive scan of v[0..n) in place by the 224 threads of warps 1-7 (named barrier 1);
// returns the total.
__device__ __forceinline__ uint32_t scan_warps_1_7(uint32_t *v, uint32_t n, uint32_t *ws7) {
    const uint32_t t = threadIdx.x - 32;
    const uint32_t per = (n + 223) / 224;
    const uint32_t t0 = min(n, t * per), t1 = min(n, t0 + per);
    uint32_t s = 0;
    for (uint32_t j = t0; j < t1; j++) s += v[j];
    const uint32_t inc = warp_inclusive_scan(s);
    const int lane = threadIdx.x & 31, w = (int)(threadIdx.x >> 5) - 1;
    if (lane == 31) ws7[w] = inc;
    bar_named(1, 224);
    uint32_t base = 0, total = 0;
#pragma unroll
    for (int i = 0; i < 7; i++) {
        const uint32_t x = ws7[i];
        if (i < w) base += x;
        total += x;
    }
    uint32_t run = base + inc - s;
    for (uint32_t j = t0; j < t1; j++) {
        const uint32_t b = v[j];
        v[j] = run;
        run += b;
    }
    return total;
}

// the slot after the last empty slot before `slot` (cyclically); the table has an empty slot
__device__ __forceinline__ uint32_t cluster_start(const uint32_t *occ, uint32_t slot) {
    uint32_t wi = slot >> 5;
    uint32_t m = ~occ[wi] & ((1u << (slot & 31)) - 1u);
    while (!m) {
        wi = (wi - 1) & (AGG_SLOTS / 32 - 1);
        m = ~occ[wi];
    }
    return ((wi << 5) + (31 - __clz(m)) + 1) & (AGG_SLOTS - 1);
}

// bytes of a node's edge lists
__device__ __forceinline__ uint32_t edge_bytes(uint32_t meta, int nb) {
    uint32_t edges = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const uint32_t m = (meta >> (4 * t)) & 15u;
        if (m) edges += 4 + __popc(m) * (4 + nb);
    }
    return edges;
}

template <class K>
__global__ void __launch_bounds__(256, sizeof(K) == 8 ? 4 : 3) k_aggregate(AggArgs a) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    AggSmem<K> &sm = *reinterpret_cast<AggSmem<K> *>(smem_raw);
    const unsigned full = 0xffffffffu;
    constexpr int BATCH = sizeof(K) == 8 ? AGG_BATCH : AGG_BATCH / 2;  // occurrence loads in flight per thread
    const uint32_t f = blockIdx.x;
    const int nb = (a.k + 3) / 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long o0 = a.fine_off[f], o1 = a.fine_off[f + 1];
    const K *okey = (const K *)a.okey2 + o0;
    const uint16_t *obits = a.obits2 + o0;
    const uint32_t M = (uint32_t)(o1 - o0);
    // A bucket with at most 32 read heads (the usual case) leaves them to warp 0: lane i loads
    // head i's entry, its read and the read's line now, so the loads land while the table clears.
    const uint32_t hb = a.head_off[f], hc = a.head_cnt[f];
    const bool warp_heads = hc <= 32;
    HeadIn p_h{};
    uint32_t p_slot = 0;
    if (warp_heads && threadIdx.x < hc) p_h = a.hsorted[hb + threadIdx.x];
    K kk[BATCH];
    uint32_t bb[BATCH];
#pragma unroll
    for (int q = 0; q < BATCH; q++) {
        const uint32_t i = q * blockDim.x + threadIdx.x;
        kk[q] = i < M ? okey[i] : (K)0;
        bb[q] = i < M ? (uint32_t)obits[i] : 0u;
    }
    {
        const uint4 z = make_uint4(0, 0, 0, 0);
        uint4 *k4 = reinterpret_cast<uint4 *>(sm.key1);
        for (uint32_t i = threadIdx.x; i < AGG_SLOTS * sizeof(K) / 16; i += blockDim.x) k4[i] = z;
        for (uint32_t i = threadIdx.x; i < AGG_SLOTS / 4; i += blockDim.x) {
            reinterpret_cast<uint4 *>(sm.cnt)[i] = z;
            reinterpret_cast<uint4 *>(sm.meta)[i] = z;
        }
    }
    if (threadIdx.x == 0) {
        sm.n = 0;
        sm.fail = 0;
    }
    __syncthreads();
    // ---- 1. read heads, then occurrences ----
    // A head claims (or finds) its first k-mer's slot and marks the set it belongs to; that
    // k-mer is one of the bucket's occurrences, which give the count.
    if (warp_heads) {
        if (threadIdx.x < hc) {
            const K key = (K)(((u128)p_h.khi << 64) | p_h.klo);
            uint32_t claimed = 0;
            const int sl = AggTable<K>::insert(sm.key1, key, agg_home(key), claimed);
            if (sl < 0) {
                sm.fail = 1;
            } else {
                if (claimed) atomicAdd(&sm.n, 1u);
                atomicOr(&sm.meta[sl], (p_h.uuid >> 40) != 0 ? META_FLIPPED : META_UNFLIPPED);
                p_slot = (uint32_t)sl;
            }
        }
    } else {
        for (uint32_t i = threadIdx.x; i < hc; i += blockDim.x) {
            const uint32_t r = a.head_idx[hb + i];
            const Head h = a.heads[r];
            const K key = (K)(((u128)h.khi << 64) | h.klo);
            uint32_t claimed = 0;
            const int sl = AggTable<K>::insert(sm.key1, key, agg_home(key), claimed);
            if (sl < 0) {
                sm.fail = 1;
                continue;
            }
            if (claimed) atomicAdd(&sm.n, 1u);
            atomicOr(&sm.meta[sl], (h.uuid >> 40) != 0 ? META_FLIPPED : META_UNFLIPPED);
            a.heads[r].slot = (uint32_t)sl;
        }
    }
    // In groups of four: the home slots are read first, all four loads in flight (a key never
    // leaves the slot it was put in, so a plain read that shows it is final); an occurrence
    // whose key is not in its home slot takes the probe with compare-and-swap.  The thread's
    // occurrences are i = q * blockDim.x + threadIdx.x; with 64-bit keys two groups are held
    // in registers, and the loads of the group after next go out as soon as a group is
    // inserted, so they land while the next one is.
    if constexpr (BATCH == 8) {
        auto insert4 = [&](const K *kq, const uint32_t *bq, uint32_t q0) {
            uint32_t hm[4];
            K cur[4];
    #pragma unroll
            for (int u = 0; u < 4; u++) {
                hm[u] = agg_home(kq[u]);
                cur[u] = sm.key1[hm[u]];
            }
    #pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t i = (q0 + u) * blockDim.x + threadIdx.x;
                if (i >= M) continue;
                int sl = (int)hm[u];
                if (cur[u] != kq[u] + 1) {
                    uint32_t claimed = 0;
                    sl = AggTable<K>::insert(sm.key1, kq[u], hm[u], claimed);
                    if (sl < 0) {
                        sm.fail = 1;
                        continue;
                    }
                    if (claimed) atomicAdd(&sm.n, 1u);
                }
                atomicAdd(&sm.cnt[sl], 1u);  // no result used: both are fire-and-forget reductions
                if (bq[u]) atomicOr(&sm.meta[sl], bq[u]);
            }
        };
        auto load4 = [&](K *kq, uint32_t *bq, uint32_t q0) {
    #pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t i = (q0 + u) * blockDim.x + threadIdx.x;
                kq[u] = i < M ? okey[i] : (K)0;
                bq[u] = i < M ? (uint32_t)obits[i] : 0u;
            }
        };
        for (uint32_t q0 = 0; q0 * blockDim.x < M; q0 += 8) {
            insert4(kk, bb, q0);
            load4(kk, bb, q0 + 8);
            if ((q0 + 4) * blockDim.x < M) {
                insert4(kk + 4, bb + 4, q0 + 4);
                load4(kk + 4, bb + 4, q0 + 12);
            }
        }
    } else {
        for (uint32_t c0 = 0; c0 < M; c0 += BATCH * blockDim.x) {
            if (c0) {
#pragma unroll
                for (int q = 0; q < BATCH; q++) {
                    const uint32_t i = c0 + q * blockDim.x + threadIdx.x;
                    kk[q] = i < M ? okey[i] : (K)0;
                    bb[q] = i < M ? (uint32_t)obits[i] : 0u;
                }
            }
#pragma unroll
            for (int g = 0; g < BATCH; g += 4) {
                uint32_t hm[4];
                K cur[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    hm[u] = agg_home(kk[g + u]);
                    cur[u] = sm.key1[hm[u]];
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int q = g + u;
                    const uint32_t i = c0 + q * blockDim.x + threadIdx.x;
                    if (i >= M) continue;
                    int sl = (int)hm[u];
                    if (cur[u] != kk[q] + 1) {
                        uint32_t claimed = 0;
                        sl = AggTable<K>::insert(sm.key1, kk[q], hm[u], claimed);
                        if (sl < 0) {
                            sm.fail = 1;
                            continue;
                        }
                        if (claimed) atomicAdd(&sm.n, 1u);
                    }
                    atomicAdd(&sm.cnt[sl], 1u);
                    if (bb[q]) atomicOr(&sm.meta[sl], bb[q]);
                }
            }
        }
    }
    __syncthreads();
    const uint32_t n = sm.n;
    if (sm.fail || n >= AGG_SLOTS) {  // the ordering below needs an empty slot
        if (threadIdx.x == 0) atomicAdd(&a.st->table_full, 1u);
        return;
    }
    // ---- 2. occupancy: warp w owns slots [256 w, 256 w + 256), lane q keeps word 8 w + q ----
    uint32_t myocc = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const uint32_t b = __ballot_sync(full, sm.key1[warp * 256 + q * 32 + lane] != (K)0);
        if (lane == q) myocc = b;
    }
    const uint32_t pc = lane < 8 ? __popc(myocc) : 0u;
    const uint32_t pc_incl = warp_inclusive_scan(pc);
    if (lane < 8) sm.occ[warp * 8 + lane] = myocc;
    if (lane == 7) sm.wtot[warp] = pc_incl;
    __syncthreads();
    // ---- 3. ranks ----
    // When a cluster wraps from the last slot to the first, its part at the front (the slots
    // before the first empty one, z) is numbered last: ranks start z slots in.
    uint32_t z = 0;
    if (sm.occ[AGG_SLOTS / 32 - 1] >> 31) {
        const uint32_t w0 = sm.occ[lane], w1 = sm.occ[lane + 32];
        const uint32_t nf0 = __ballot_sync(full, w0 != full), nf1 = __ballot_sync(full, w1 != full);
        const uint32_t zw = nf0 ? (uint32_t)__ffs(nf0) - 1 : 32u + (uint32_t)__ffs(nf1) - 1;
        const uint32_t zword = __shfl_sync(full, zw < 32 ? w0 : w1, (int)(zw & 31));
        z = zw * 32 + (uint32_t)__ffs(~zword) - 1;
    }
    const uint32_t wbase = __reduce_add_sync(full, lane < warp ? sm.wtot[lane] : 0u);
    K *nkey = (K *)a.nkey + o0;
    unsigned long long *ncm = a.ncm + o0;
    uint32_t inexact = 0, phantom = 0;
    // the warp's occupied slots, 32 at a time: lane i takes the i-th (its word by the words'
    // running counts, its bit by a popcount search)
    uint32_t winc[8];
#pragma unroll
    for (int q = 0; q < 8; q++) winc[q] = __shfl_sync(full, pc_incl, q);
    const uint32_t wocc = winc[7];
    for (uint32_t idx = lane; idx < wocc + ((32 - (wocc & 31)) & 31); idx += 32) {
        uint32_t q = 0;
#pragma unroll
        for (int j = 0; j < 7; j++) q += winc[j] <= idx ? 1u : 0u;
        const uint32_t word = __shfl_sync(full, myocc, (int)q);
        const uint32_t wexcl = __shfl_sync(full, pc_incl - pc, (int)q);
        if (idx >= wocc) continue;
        uint32_t m = idx - wexcl, w = word, bit = 0;
#pragma unroll
        for (uint32_t sh = 16; sh; sh >>= 1) {
            const uint32_t lo = __popc(w & ((1u << sh) - 1u));
            if (m >= lo) {
                m -= lo;
                w >>= sh;
                bit += sh;
            }
        }
        const uint32_t slot = warp * 256 + q * 32 + bit;
        const uint32_t before = wbase + idx;  // occupied slots before this one
        const K mine = sm.key1[slot];
        const uint32_t sl_prev = (slot - 1) & (AGG_SLOTS - 1), sl_next = (slot + 1) & (AGG_SLOTS - 1);
        uint32_t pre_c0, within = 0;
        if (!((sm.occ[sl_prev >> 5] >> (sl_prev & 31)) & 1u) && !((sm.occ[sl_next >> 5] >> (sl_next & 31)) & 1u)) {
            pre_c0 = before;  // a cluster of one
        } else {
            const uint32_t c0 = cluster_start(sm.occ, slot);
            // occupied slots before the cluster: the run from c0 to this slot is all occupied; a
            // cluster that wraps past the last slot occupies everything from c0 to the end
            pre_c0 = c0 <= slot ? before - (slot - c0) : n - (AGG_SLOTS - c0);
            for (uint32_t j = c0;; j = (j + 1) & (AGG_SLOTS - 1)) {
                if (!((sm.occ[j >> 5] >> (j & 31)) & 1u)) break;
                within += sm.key1[j] < mine ? 1u : 0u;
            }
        }
        const uint32_t rank = pre_c0 - z + within;
        if (rank >= n) {  // never expected: the ranks are a permutation of [0, n)
            phantom++;
            continue;
        }
        sm.rank_of_slot[slot] = (uint16_t)rank;
        sm.ord[rank] = (uint16_t)slot;
        const uint32_t cnt = sm.cnt[slot], meta = sm.meta[slot];
        nkey[rank] = mine - 1;
        ncm[rank] = (unsigned long long)cnt | ((unsigned long long)meta << 32);
        if (cnt >= (1u << 24)) inexact++;
        if (cnt == 0) phantom++;  // a read head whose k-mer has no occurrence here
        sm.nbytes[rank] = node_base_bytes(meta, nb);
    }
    if (inexact) atomicAdd(&a.st->cov_inexact, inexact);
    if (phantom) atomicAdd(&a.st->internal_err, phantom);
    __syncthreads();
    HeadOut *hout = a.hout + hb;
    const uint32_t keylen = 4 + nb;
    uint32_t *noff = a.noff + o0;
    if (warp_heads) {
        // ---- 4. warp 0: read heads sorted by (node, TreeSet order), duplicates dropped;
        //         warps 1-7: exclusive scan of the base record sizes ----
        unsigned long long wk = 0;
        uint32_t wkeep = 0, wkept_idx = 0, wkeep_mask = 0, hsz = 0, w_slot = 0;
        unsigned long long w_uuid = 0, w_soff = 0, w_moff = 0;
        uint32_t w_L = 0, w_Lm = 0;
        if (warp == 0) {
            unsigned long long mk = ~0ULL;
            uint32_t mv = 0xffffffffu;
            if (lane < (int)hc) {
                mv = p_h.r;
                mk = head_sort_key(sm.rank_of_slot[p_slot], p_h.uuid);
            }
            uint32_t rank = 0;
#pragma unroll 4
            for (int j = 0; j < (int)hc; j++) {
                const unsigned long long kj = shfl64(mk, j);
                const uint32_t vj = __shfl_sync(full, mv, j);
                rank += (kj < mk || (kj == mk && vj < mv)) ? 1u : 0u;
            }
            if (lane < (int)hc) {
                sm.wsk[rank] = mk;
                sm.wsv[rank] = (uint32_t)lane;
            }
            __syncwarp();
            uint32_t src = (uint32_t)lane;
            if (lane < (int)hc) {
                wk = sm.wsk[lane];
                src = sm.wsv[lane];
            }
            w_uuid = shfl64(p_h.uuid, (int)src);
            w_soff = shfl64(p_h.s_off, (int)src);
            w_moff = shfl64(p_h.m_off, (int)src);
            w_L = __shfl_sync(full, p_h.L, (int)src);
            w_Lm = __shfl_sync(full, p_h.Lm, (int)src);
            w_slot = __shfl_sync(full, p_slot, (int)src);
            const unsigned long long prev = shfl64(wk, lane > 0 ? lane - 1 : 0);
            wkeep = (lane < (int)hc && (lane == 0 || wk != prev)) ? 1u : 0u;
            wkeep_mask = __ballot_sync(full, wkeep);
            wkept_idx = __popc(wkeep_mask & ((1u << lane) - 1u));
            hsz = wkeep ? 1 + 8 + 4 + packed_len(w_L) + (w_Lm > 0 ? 4 + packed_len(w_Lm) : 0) : 0u;
            const uint32_t longest = __reduce_max_sync(full, wkeep ? max(w_L, w_Lm) : 0u);
            if (lane == 0 && longest) atomicMax(&a.st->max_seq, longest);
            const uint32_t incl = warp_inclusive_scan(hsz);
            const uint32_t kept_w = __popc(wkeep_mask);
            // kept heads in order: node rank and the bytes of the kept heads before
            if (wkeep) {
                sm.hrank[wkept_idx] = (uint32_t)(wk >> 37);
                sm.hcum[wkept_idx] = incl - hsz;
            }
            if (lane == 31) sm.hcum[kept_w] = incl;
            if ((uint32_t)lane >= kept_w) sm.hrank[lane] = 0xffffffffu;  // padding for the search
            if (lane == 0) sm.kept = kept_w;
        } else {
            const uint32_t t = scan_warps_1_7(sm.nbytes, n, sm.ws7);
            if (threadIdx.x == 32) sm.base_total = t;
        }
        __syncthreads();
        // ---- 5. record offsets; read-head entries ----
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            // kept heads of nodes before j: hrank is sorted, padded with ~0 to 32 entries
            uint32_t pos = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1)
                if (sm.hrank[pos + step - 1] < j) pos += step;
            if (sm.hrank[pos] < j) pos++;  // all 32 before j
            noff[j] = sm.nbytes[j] + sm.hcum[pos];
        }
        if (warp == 0) {
            const uint32_t kept_w = __popc(wkeep_mask);
            const uint32_t rank = (uint32_t)(wk >> 37);
            const bool flipped = (wk >> 36) & 1ULL;
            // the node's kept lanes, its flipped ones, its first lane
            const uint32_t node_mask = __match_any_sync(full, wkeep ? rank : 0xffffffffu) & wkeep_mask;
            const uint32_t flip_mask = __ballot_sync(full, wkeep && flipped);
            if (wkeep) {
                const int first = __ffs(node_mask) - 1;
                const uint32_t cu = __popc(node_mask & ~flip_mask), cf = __popc(node_mask & flip_mask);
                const uint32_t meta = sm.meta[w_slot];
                const uint32_t st = __popc(wkeep_mask & ((1u << first) - 1u));  // kept index of the node's first
                HeadOut ho;
                ho.uuid = w_uuid;
                ho.s_off = w_soff;
                ho.m_off = w_moff;
                ho.L = w_L;
                ho.Lm = w_Lm;
                ho.pos = sm.nbytes[rank] + sm.hcum[wkept_idx] + 8 + keylen + 1 + edge_bytes(meta, nb) + 5 +
                         ((flipped && cu > 0) ? 5 : 0);
                ho.set_count = (wkept_idx == st && !flipped) ? cu : ((flipped && wkept_idx == st + cu) ? cf : 0u);
                ho.part = f;
                hout[wkept_idx] = ho;
            }
            // the slots past the kept heads: duplicates, skipped by the head writer
            if ((uint32_t)lane >= kept_w && (uint32_t)lane < hc) hout[lane].part = HEAD_DROPPED;
        }
        if (threadIdx.x == 0) {
            a.part_nodes[f] = n;
            a.part_bytes[f] = (unsigned long long)sm.base_total + sm.hcum[sm.kept];
            a.head_cnt2[f] = sm.kept;
        }
        return;
    }
    // ---- the general path: more than 32 read heads ----
    unsigned long long *hk = a.head_sk + hb;
    uint32_t *hv = a.head_idx + hb;
    if (hc > HEAD_CAP && threadIdx.x == 0) atomicAdd(&a.st->big_head_parts, 1u);
    for (uint32_t i = threadIdx.x; i < hc; i += blockDim.x) {
        const uint32_t r = hv[i];
        const Head h = a.heads[r];
        hk[i] = head_sort_key(sm.rank_of_slot[h.slot], h.uuid);
    }
    __syncthreads();
    if (hc <= blockDim.x) {
        // each thread places its own head by counting the smaller (key, read) pairs; read
        // ordinals are distinct, so the ranks are too
        unsigned long long mk = 0;
        uint32_t mv = 0, rank = 0;
        if (threadIdx.x < hc) {
            mk = hk[threadIdx.x];
            mv = hv[threadIdx.x];
            for (uint32_t j = 0; j < hc; j++) {
                const unsigned long long kj = hk[j];
                const uint32_t vj = hv[j];
                rank += (kj < mk || (kj == mk && vj < mv)) ? 1u : 0u;
            }
        }
        __syncthreads();
        if (threadIdx.x < hc) {
            hk[rank] = mk;
            hv[rank] = mv;
        }
        __syncthreads();
    } else {
        bitonic_sort_pairs<unsigned long long, uint32_t>(hk, hv, hc);
    }
    if (threadIdx.x == 0) {
        sm.kept = 0;
        sm.carry = 0;
    }
    __syncthreads();
    // keep the first of equal keys; add the kept heads' bytes to their node's size
    for (uint32_t c0 = 0; c0 < hc; c0 += blockDim.x) {
        const uint32_t i = c0 + threadIdx.x;
        unsigned long long key = 0;
        uint32_t keep = 0, r = 0;
        if (i < hc) {
            key = hk[i];
            const unsigned long long prev = i == 0 ? ~0ULL : (i == c0 ? sm.carry : hk[i - 1]);
            keep = key != prev ? 1u : 0u;
            r = hv[i];
        }
        const unsigned long long last = hk[min(hc, c0 + blockDim.x) - 1];
        unsigned long long tot;
        const unsigned long long ex = block_exclusive_scan((unsigned long long)keep, sm.ws, tot);
        if (keep) {
            const uint32_t w = sm.kept + (uint32_t)ex;
            hk[w] = key;
            hv[w] = r;
            const uint32_t rank = (uint32_t)(key >> 37);
            const uint32_t rl = a.reads[r];
            atomicAdd(&sm.nbytes[rank], head_bytes(a.lines[rl >> 1], rl & 1u));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            sm.kept += (uint32_t)tot;
            sm.carry = last;
        }
        __syncthreads();
    }
    const uint32_t kept = sm.kept;
    // record offsets of the nodes, read heads included
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t t0 = min(n, threadIdx.x * per), t1 = min(n, t0 + per);
    unsigned long long mine = 0;
    for (uint32_t j = t0; j < t1; j++) mine += sm.nbytes[j];
    unsigned long long tot_bytes;
    unsigned long long run = block_exclusive_scan(mine, sm.ws, tot_bytes);
    for (uint32_t j = t0; j < t1; j++) {
        const uint32_t b = sm.nbytes[j];
        sm.nbytes[j] = (uint32_t)run;
        noff[j] = (uint32_t)run;
        run += b;
    }
    __syncthreads();
    // byte position of every kept head: node offset, frame + key + active + edges, the set
    // headers, the heads of the node before it
    unsigned long long hrun = 0;
    for (uint32_t c0 = 0; c0 < kept; c0 += blockDim.x) {
        const uint32_t i = c0 + threadIdx.x;
        uint32_t hsz = 0;
        if (i < kept) {
            const uint32_t rl = a.reads[hv[i]];
            hsz = head_bytes(a.lines[rl >> 1], rl & 1u);
        }
        unsigned long long tot;
        const unsigned long long ex = block_exclusive_scan((unsigned long long)hsz, sm.ws, tot);
        // the running byte count of kept heads: stash each head's prefix in hk's low bits
        if (i < kept) {
            const unsigned long long pre = hrun + ex;
            const unsigned long long key = hk[i];
            hk[i] = (key & ~((1ULL << 36) - 1)) | pre;  // rank << 37 | flipped << 36 | prefix
        }
        hrun += tot;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kept; i += blockDim.x) {
        const unsigned long long key = hk[i];
        const uint32_t rank = (uint32_t)(key >> 37);
        const bool flipped = (key >> 36) & 1ULL;
        // the node's kept heads: [st, st + cu) unflipped, then cf flipped (hk is sorted by
        // rank, flipped, position)
        const unsigned long long rbase = (unsigned long long)rank << 37;
        const uint32_t st = kept_lower_bound(hk, kept, rbase);
        const uint32_t fl = kept_lower_bound(hk, kept, rbase | (1ULL << 36));
        const uint32_t cu = fl - st, cf = kept_lower_bound(hk, kept, rbase + (1ULL << 37)) - fl;
        const unsigned long long pre = key & ((1ULL << 36) - 1);
        const unsigned long long pre0 = hk[st] & ((1ULL << 36) - 1);
        const uint32_t meta = sm.meta[sm.ord[rank]];
        const uint32_t pos = sm.nbytes[rank] + 8 + keylen + 1 + edge_bytes(meta, nb) + 5 +
                             ((flipped && cu > 0) ? 5 : 0) + (uint32_t)(pre - pre0);
        const uint32_t r = hv[i];
        const uint32_t rl = a.reads[r];
        const LineRec lr = a.lines[rl >> 1];
        const uint32_t mate = rl & 1u;
        HeadOut ho;
        ho.uuid = a.heads[r].uuid;
        ho.s_off = mate ? lr.s1 : lr.s0;
        ho.m_off = mate ? lr.s0 : lr.s1;
        ho.L = mate ? lr.l1 : lr.l0;
        ho.Lm = mate ? lr.l0 : lr.l1;
        atomicMax(&a.st->max_seq, max(ho.L, ho.Lm));
        ho.pos = pos;
        ho.set_count = (i == st && !flipped) ? cu : ((flipped && i == st + cu) ? cf : 0u);
        ho.part = f;
        hout[i] = ho;
    }
    for (uint32_t i = kept + threadIdx.x; i < hc; i += blockDim.x) hout[i].part = HEAD_DROPPED;
    if (threadIdx.x == 0) {
        a.part_nodes[f] = n;
        a.part_bytes[f] = tot_bytes;
        a.head_cnt2[f] = kept;
    }
}

void launch_aggregate(const AggArgs &a, cudaStream_t s) {
    if (!a.pp.P) return;
    t_launches++;
    if (a.wide) {
        const size_t sm = sizeof(AggSmem<u128>);
        cudaFuncSetAttribute(k_aggregate<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_aggregate<u128><<<a.pp.P, 256, sm, s>>>(a);
    } else {
        const size_t sm = sizeof(AggSmem<uint64_t>);
        cudaFuncSetAttribute(k_aggregate<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_aggregate<uint64_t><<<a.pp.P, 256, sm, s>>>(a);
    }
}

// ---- D: record writer of the partitioned build ------------------------------------------------
// Each warp writes the records of a contiguous node range.  It cuts the range into windows
// that end on record boundaries and hold at most WARP_STAGE bytes, assembles each window in
// a private piece of shared memory and copies it out with aligned 16-byte stores.  Inside a
// window, lane i of an iteration writes record j0 + i: every word that lies wholly inside its
// record is stored as soon as it fills, and the word two neighbouring records share (the
// previous record's tail and this one's head) is put together with a warp shuffle and
// stored once, so no word is written by two lanes and nothing has to be cleared first.  The
// read-head sets are written warp-cooperatively afterwards, byte by byte, into the gaps
// the records leave for them.  A record larger than a window (a node with very many read
// heads) is written alone, byte by byte, over as many windows as it needs.
constexpr uint32_t WARP_STAGE = 6144;
constexpr int WRITER_WARPS = 8;

// Bytes appended in memory order through a 32-bit accumulator.  The record's first word,
// when the record starts mid-word, is kept in `first` instead of being stored (it holds the
// predecessor's tail too); the trailing partial word stays in `cur`.
struct RecAcc {
    uint32_t *w;
    uint32_t wi;    // word being filled
    uint32_t fill;  // bytes of that word already in cur (0..3)
    uint32_t cur;
    uint32_t fw;    // the record's first word
    uint32_t first;
    bool hold_first;
    __device__ __forceinline__ void init(uint32_t *w_, uint32_t pos) {
        w = w_;
        wi = fw = pos >> 2;
        fill = pos & 3;
        cur = first = 0;
        hold_first = fill != 0;
    }
    // n (1..4) bytes, the first in the low byte of le, the bytes above n zero
    __device__ __forceinline__ void put(uint32_t le, uint32_t n) {
        const uint32_t sh = fill * 8;
        const uint32_t lo = cur | (le << sh);
        fill += n;
        if (fill >= 4) {
            if (hold_first && wi == fw)
                first = lo;
            else
                w[wi] = lo;
            wi++;
            fill -= 4;
            cur = __funnelshift_rc(le, 0u, 32 - sh);  // the bytes that spill into the next word
        } else {
            cur = lo;
        }
    }
    __device__ __forceinline__ void be32(uint32_t v) { put(__byte_perm(v, 0, 0x0123), 4); }
};

// the nb big-endian bytes of a k-mer value, as little-endian words in memory order
__device__ __forceinline__ void key_words(uint64_t v, int nb, uint32_t w[4]) {
    const uint64_t u = v << (64 - 8 * nb);
    w[0] = __byte_perm((uint32_t)(u >> 32), 0, 0x0123);
    w[1] = __byte_perm((uint32_t)u, 0, 0x0123);
    w[2] = w[3] = 0;
}
__device__ __forceinline__ void key_words(u128 v, int nb, uint32_t w[4]) {
    const u128 u = v << (128 - 8 * nb);
    const uint64_t hi = (uint64_t)(u >> 64), lo = (uint64_t)u;
    w[0] = __byte_perm((uint32_t)(hi >> 32), 0, 0x0123);
    w[1] = __byte_perm((uint32_t)hi, 0, 0x0123);
    w[2] = __byte_perm((uint32_t)(lo >> 32), 0, 0x0123);
    w[3] = __byte_perm((uint32_t)lo, 0, 0x0123);
}

template <class K>
__device__ __forceinline__ void put_key(RecAcc &o, K v, int nb) {
    uint32_t w[4];
    key_words(v, nb, w);
#pragma unroll
    for (int q = 0; q < (sizeof(K) == 8 ? 2 : 4); q++) {
        const int rem = nb - 4 * q;
        if (rem > 0) o.put(w[q], rem < 4 ? (uint32_t)rem : 4u);
    }
}

// a record larger than a window: byte by byte, only the bytes inside the window
template <class K>
__device__ __noinline__ void write_record_bytes(const Sink &o, long long st, long long en, K key, uint32_t meta,
                                                uint32_t active, uint32_t cov, int k, int nb) {
    o.u32(st, (uint32_t)(en - st - 8));
    o.u32(st + 4, (uint32_t)(4 + nb));
    o.u32(st + 8, (uint32_t)k);
    long long pos = st + 12;
    for (int i = 0; i < nb; i++) o.b(pos + i, KeyOps<K>::byte_at(key, nb - 1 - i));
    pos += nb;
    o.b(pos++, active);
    for (int t = 0; t < 4; t++) {
        uint32_t m = (meta >> (4 * t)) & 15u;
        if (!m) continue;
        o.u32(pos, (uint32_t)__popc(m));
        pos += 4;
        while (m) {
            const int e = __ffs(m) - 1;
            m &= m - 1;
            const K y = edge_neighbor<K>(key, t, e, k);
            o.u32(pos, (uint32_t)k);
            pos += 4;
            for (int i = 0; i < nb; i++) o.b(pos + i, KeyOps<K>::byte_at(y, nb - 1 - i));
            pos += nb;
        }
    }
    o.u32(en - 4, cov);
}

// Four letters (the first in the low byte) packed into one VKmer byte, first letter in the low
// bits: A/a=0 C/c=1 G/g=2 T/t=3, any other byte 0 (GeneCode.getCodeFromSymbol), four at a time.
__device__ __forceinline__ uint32_t pack4_letters(uint32_t w) {
    const uint32_t u = w & 0xDFDFDFDFu;
    const uint32_t ok = zero_bytes(u ^ 0x41414141u) | zero_bytes(u ^ 0x43434343u) | zero_bytes(u ^ 0x47474747u) |
                        zero_bytes(u ^ 0x54545454u);
    uint32_t c = (w >> 1) & 0x03030303u;  // A 0, C 1, G 3, T 2 in each byte
    c ^= (c >> 1) & 0x01010101u;          // G 2, T 3
    c &= (ok >> 7) * 3u;                  // other bytes 0
    const uint32_t y = c | (c >> 6);
    return (y | (y >> 12)) & 0xFFu;
}

// Bytes appended to global memory in address order: whole aligned 32-bit words inside the run,
// single bytes in its first and last word, which it may share with its neighbours' bytes.
struct ByteRun {
    uint8_t *out;
    unsigned long long wa;  // address of the word being filled (a multiple of 4)
    uint32_t lo;            // first byte of that word inside the run (nonzero only in the first word)
    uint32_t fill;          // bytes of that word filled so far (lo <= fill < 4)
    uint32_t cur;           // their values: byte b of the word in bits 8b .. 8b + 7
    __device__ __forceinline__ void init(uint8_t *o, unsigned long long pos) {
        out = o;
        wa = pos & ~3ULL;
        lo = fill = (uint32_t)(pos & 3);
        cur = 0;
    }
    __device__ __forceinline__ void word_out(uint32_t v) {
        if (lo == 0) {
            *reinterpret_cast<uint32_t *>(out + wa) = v;
        } else {
            for (uint32_t b = lo; b < 4; b++) out[wa + b] = (uint8_t)(v >> (8 * b));
            lo = 0;
        }
    }
    // n (1..4) bytes, the first in the low byte of le, the bytes above n zero
    __device__ __forceinline__ void put(uint32_t le, uint32_t n) {
        const uint32_t sh = fill * 8;
        const uint32_t v = cur | (le << sh);
        fill += n;
        if (fill >= 4) {
            word_out(v);
            wa += 4;
            fill -= 4;
            cur = __funnelshift_rc(le, 0u, 32 - sh);  // the bytes that spill into the next word
        } else {
            cur = v;
        }
    }
    __device__ __forceinline__ void finish() {
        for (uint32_t b = lo; b < fill; b++) out[wa + b] = (uint8_t)(cur >> (8 * b));
    }
};

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

// The aligned 16 bytes at address c as four little-endian words; bytes outside the text
// [text, text + n_text) read as 0 (only the text's first and last 16 bytes take the byte loop).
__device__ __forceinline__ uint4 text_chunk(const uint8_t *text, unsigned long long n_text, uintptr_t c) {
    const uintptr_t tb = (uintptr_t)text, te = tb + n_text;
    if (c >= tb && c + 16 <= te) return *reinterpret_cast<const uint4 *>(c);
    uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int b = 0; b < 16; b++)
        if (c + b >= tb && c + b < te) w[b >> 2] |= (uint32_t)*reinterpret_cast<const uint8_t *>(c + b) << (8 * (b & 3));
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// the 16 bytes starting o (0..15) bytes into the 32 bytes lo, hi, as four little-endian words
__device__ __forceinline__ void realign16(const uint4 &lo, const uint4 &hi, uint32_t o, uint32_t v[4]) {
    const uint32_t q = o >> 2, sh = (o & 3u) * 8u;
    const uint32_t e0 = q == 0 ? lo.x : q == 1 ? lo.y : q == 2 ? lo.z : lo.w;
    const uint32_t e1 = q == 0 ? lo.y : q == 1 ? lo.z : q == 2 ? lo.w : hi.x;
    const uint32_t e2 = q == 0 ? lo.z : q == 1 ? lo.w : q == 2 ? hi.x : hi.y;
    const uint32_t e3 = q == 0 ? lo.w : q == 1 ? hi.x : q == 2 ? hi.y : hi.z;
    const uint32_t e4 = q == 0 ? hi.x : q == 1 ? hi.y : q == 2 ? hi.z : hi.w;
    v[0] = __funnelshift_r(e0, e1, sh);
    v[1] = __funnelshift_r(e1, e2, sh);
    v[2] = __funnelshift_r(e2, e3, sh);
    v[3] = __funnelshift_r(e3, e4, sh);
}

// 16-byte chunks of the text read straight from global memory (bytes outside the text as 0)
struct TextChunks {
    const uint8_t *text;
    unsigned long long n_text;
    __device__ __forceinline__ uint4 get(uintptr_t c) const { return text_chunk(text, n_text, c); }
};
// the same chunks from a copy in shared memory of the chunks [c0, c0 + 16 n)
struct StagedChunks {
    const uint4 *s;
    uintptr_t c0;
    __device__ __forceinline__ uint4 get(uintptr_t c) const { return s[(c - c0) >> 4]; }
};

// The packed letters of a sequence of L letters at address a (VKmer.setAsCopy(String),
// VKmer.java:450-479): nb = ceil(L / 4) bytes, byte j holding letters 4 (nb - 1 - j) .. + 3, the
// first in the low bits, letters past L as 0.  Four bytes per step, from the 16 letters at
// a + 4 nb - 16 - 16 s: the sequence is read backwards, one aligned 16-byte chunk per step.  The
// windows start at most 12 bytes before the sequence (letters of groups before its first,
// never written); the chunks they touch are [floor16(a - 12), floor16(a + 4 nb) + 16).
// Four letters known to be in [ACGTacgt] (or 0 bytes past the sequence's end) packed the same
// way: (b >> 1) & 3 gives A 0, C 1, G 3, T 2 in both cases, bit 2 of the letter swaps G and T.
__device__ __forceinline__ uint32_t pack4_acgt(uint32_t w) {
    const uint32_t c = ((w >> 1) & 0x03030303u) ^ ((w >> 2) & 0x01010101u);
    const uint32_t y = c | (c >> 6);
    return (y | (y >> 12)) & 0xFFu;
}
template <bool ACGT>
__device__ __forceinline__ uint32_t pack4(uint32_t w) {
    return ACGT ? pack4_acgt(w) : pack4_letters(w);
}

template <bool ACGT, class Run, class Src>
__device__ __forceinline__ void put_packed_seq(Run &o, const Src &src, uintptr_t a, uint32_t L) {
    const uint32_t nb = packed_len(L);
    if (!nb) return;
    const uintptr_t a0 = a + 4ull * nb - 16ull;
    const uint32_t off = (uint32_t)(a0 & 15u);
    uintptr_t c = a0 & ~(uintptr_t)15;
    uint4 hi = src.get(c + 16), lo = src.get(c);
    const uint32_t tail = L - 4 * (nb - 1);  // letters of the last group (1..4)
    const uint32_t tail_mask = tail >= 4 ? 0xffffffffu : (1u << (8 * tail)) - 1u;
    for (uint32_t j0 = 0; j0 < nb; j0 += 4) {
        uint32_t v[4];
        realign16(lo, hi, off, v);
        if (j0 == 0) v[3] &= tail_mask;
        const uint32_t n = min(4u, nb - j0);
        uint32_t w = pack4<ACGT>(v[3]);
        if (n > 1) w |= pack4<ACGT>(v[2]) << 8;
        if (n > 2) w |= pack4<ACGT>(v[1]) << 16;
        if (n > 3) w |= pack4<ACGT>(v[0]) << 24;
        o.put(w, n);
        if (j0 + 4 < nb) {
            c -= 16;
            hi = lo;
            lo = src.get(c);
        }
    }
}

// bytes of one read head, with the set header ahead of a set's first head
__device__ __forceinline__ uint32_t head_out_bytes(const HeadOut &h) {
    return (h.set_count ? 5u : 0u) + 1u + 8u + 4u + packed_len(h.L) + (h.Lm ? 4u + packed_len(h.Lm) : 0u);
}

__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst_smem)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// The chunks a sequence's packing reads: [floor16(a - 12), floor16(a + 4 nb) + 16).
__device__ __forceinline__ uintptr_t seq_chunk0(uintptr_t a) { return (a - 12) & ~(uintptr_t)15; }
__device__ __forceinline__ uint32_t seq_chunks(uintptr_t a, uint32_t L) {
    return L ? (uint32_t)(((((a + 4ull * packed_len(L)) & ~(uintptr_t)15) + 16) - seq_chunk0(a)) >> 4) : 0u;
}

// Warp-collective: each lane's sequence (where `want`) into the lane's slot of `slots` (seqc
// chunks per lane) by asynchronous copies (the text's first and last chunk, which may reach past
// it, by plain loads).  The warp's chunks are numbered through a prefix over the lanes' counts
// and taken 32 at a time, a chunk per lane; a chunk's lane is found by a 5-step search over
// that prefix.
__device__ __forceinline__ void stage_seqs(uint4 *slots, uint32_t seqc, bool want, uintptr_t a, uint32_t L,
                                           const uint8_t *text, unsigned long long n_text, int lane) {
    const unsigned full = 0xffffffffu;
    const uintptr_t tb = (uintptr_t)text, te = tb + n_text;
    const uint32_t cnt = want ? seq_chunks(a, L) : 0u;  // at most seqc <= 31: `want` is only set when it fits
    const unsigned long long c0 = (unsigned long long)seq_chunk0(a);
    const uint32_t incl = warp_inclusive_scan(cnt), excl = incl - cnt;
    const uint32_t total = __shfl_sync(full, incl, 31);
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t idx = base + (uint32_t)lane;
        // the last lane whose chunks start at or before idx owns it
        uint32_t q = 0;
#pragma unroll
        for (uint32_t s = 16; s; s >>= 1) {
            const uint32_t e = __shfl_sync(full, excl, (int)(q + s));
            if (e <= idx) q += s;
        }
        const uint32_t j = idx - __shfl_sync(full, excl, (int)q);
        const uintptr_t c = (uintptr_t)shfl64(c0, (int)q) + 16ull * j;
        if (idx < total) {
            uint4 *dst = slots + (size_t)q * seqc + j;
            if (c >= tb && c + 16 <= te)
                cp_async16(dst, reinterpret_cast<const void *>(c));
            else
                *dst = text_chunk(text, n_text, c);
        }
    }
    cp_async_wait_all();
    __syncwarp();
}

// The read-head sets of the partitioned build, straight into the record stream after the record
// writer: the writer leaves those byte ranges to this kernel (it copies whatever its window held
// there).  A warp takes 32 head slots at a time, one per lane (slots of dropped duplicates are
// skipped); each lane writes its head in order: on a set's first head the set header
// (ExternalableTreeSet.write: [1, set count]), then ReadHeadInfo.write: a mate flag, the uuid,
// the read's length and letters, the mate's length and letters when it has one.  The letters
// come through shared memory: the warp copies the 16-byte chunks of its 32 reads, one read after
// another and a chunk per lane, so the loads are coalesced and in flight together; the lanes
// pack their reads from there; then the same for the mates.  seqc (odd, so the lanes' slots
// start in different bank groups) is the chunks of the longest sequence; a sequence that needs
// more (or every one, when seqc is 0) is read straight from global memory.  A head's own read
// matched [ACGTacgt]+ in the parse, so it packs with the shorter letter code; the mate may hold
// any letter.
constexpr int HEAD_WARPS = 4;
constexpr uint32_t HEAD_MAX_SEQ_CHUNKS = 31;

__global__ void __launch_bounds__(HEAD_WARPS * 32) k_write_heads_part(const HeadOut *hout, uint64_t n,
                                                                      const unsigned long long *part_off,
                                                                      const uint8_t *text, unsigned long long n_text,
                                                                      uint8_t *out, uint32_t seqc) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint4 *slots = reinterpret_cast<uint4 *>(smem_raw) + (size_t)warp * 32 * seqc;
    const uint4 *mine = slots + (size_t)lane * seqc;
    const uintptr_t tb = (uintptr_t)text;
    const TextChunks gsrc{text, n_text};
    const uint64_t step = (uint64_t)gridDim.x * HEAD_WARPS * 32;
    for (uint64_t h0 = ((uint64_t)blockIdx.x * HEAD_WARPS + warp) * 32; h0 < n; h0 += step) {
        const uint64_t i = h0 + lane;
        HeadOut h{};
        h.part = HEAD_DROPPED;
        if (i < n) h = hout[i];
        const bool live = h.part != HEAD_DROPPED;
        const uintptr_t ar = tb + h.s_off, am = tb + h.m_off;
        ByteRun o;
        if (live) {
            const unsigned long long hp = part_off[h.part] + h.pos;
            o.init(out, h.set_count ? hp - 5 : hp);
            if (h.set_count) {
                o.put(1u, 1);
                o.put(bswap32(h.set_count), 4);
            }
            o.put(h.Lm ? 1u : 0u, 1);
            o.put(bswap32((uint32_t)(h.uuid >> 32)), 4);
            o.put(bswap32((uint32_t)h.uuid), 4);
            o.put(bswap32(h.L), 4);
        }
        const bool sr = live && seq_chunks(ar, h.L) <= seqc;
        stage_seqs(slots, seqc, sr, ar, h.L, text, n_text, lane);
        if (live) {
            if (sr)
                put_packed_seq<true>(o, StagedChunks{mine, seq_chunk0(ar)}, ar, h.L);
            else
                put_packed_seq<true>(o, gsrc, ar, h.L);
            if (h.Lm) o.put(bswap32(h.Lm), 4);
        }
        __syncwarp();  // the slots are read before the mates go in
        const bool sm = live && h.Lm && seq_chunks(am, h.Lm) <= seqc;
        stage_seqs(slots, seqc, sm, am, h.Lm, text, n_text, lane);
        if (live) {
            if (sm)
                put_packed_seq<false>(o, StagedChunks{mine, seq_chunk0(am)}, am, h.Lm);
            else if (h.Lm)
                put_packed_seq<false>(o, gsrc, am, h.Lm);
            o.finish();
        }
        __syncwarp();
    }
}

// window [W, wend) of the partition out to global memory with aligned 16-byte stores
__device__ __forceinline__ void window_out(uint8_t *out, const uint8_t *stage, unsigned long long g0,
                                           unsigned long long g1, int lane) {
    const uint32_t *stage32 = reinterpret_cast<const uint32_t *>(stage);
    for (unsigned long long c = (g0 & ~15ULL) + 16ULL * lane; c < g1; c += 16ULL * 32) {
        if (c >= g0 && c + 16 <= g1) {
            const uint32_t ofs = (uint32_t)(c - g0);
            const uint32_t w0 = ofs >> 2, sh = (ofs & 3u) * 8u;
            uint32_t w[5];
#pragma unroll
            for (int q = 0; q < 5; q++) w[q] = stage32[w0 + q];
            uint4 v;
            v.x = __funnelshift_r(w[0], w[1], sh);
            v.y = __funnelshift_r(w[1], w[2], sh);
            v.z = __funnelshift_r(w[2], w[3], sh);
            v.w = __funnelshift_r(w[3], w[4], sh);
            *reinterpret_cast<uint4 *>(out + c) = v;
        } else {
            for (int q = 0; q < 16; q++) {
                const unsigned long long g = c + q;
                if (g >= g0 && g < g1) out[g] = stage[g - g0];
            }
        }
    }
}

template <class K>
__global__ void __launch_bounds__(WRITER_WARPS * 32, sizeof(K) == 8 ? 4 : 3) k_emit_write_part(EmitArgs a) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint8_t *stage = smem_raw + (size_t)warp * (WARP_STAGE + 32);
    uint32_t *stage32 = reinterpret_cast<uint32_t *>(stage);
    const uint32_t p = blockIdx.x;
    const int k = a.k, nb = (k + 3) / 4;
    const uint32_t n = a.part_nodes[p];
    const unsigned long long pbytes = a.part_bytes[p];
    const unsigned long long base = a.part_off[p];
    const unsigned long long nbase = a.node_base[p];
    const K *nkey = (const K *)a.nkey + nbase;
    const unsigned long long *ncm = a.ncm + nbase;
    const uint32_t *noff = a.noff + nbase;
    const uint32_t npw = (n + WRITER_WARPS - 1) / WRITER_WARPS;
    const uint32_t j0 = min(n, warp * npw), j1 = min(n, j0 + npw);
    // record j starts at off_at(j); off_at(n) is the partition's end
    auto off_at = [&](uint32_t j) -> unsigned long long {
        return j < n ? (unsigned long long)noff[j] : pbytes;
    };
    const unsigned full = 0xffffffffu;
    uint32_t ja = j0;
    while (ja < j1) {
        const unsigned long long W = off_at(ja);
        if (off_at(ja + 1) - W > WARP_STAGE) {
            // ---- one record larger than a window ----
            const unsigned long long en = off_at(ja + 1);
            const unsigned long long cm = ncm[ja];
            const uint32_t meta = (uint32_t)(cm >> 32);
            uint32_t active = 0x80u;
            for (int t = 0; t < 4; t++)
                if ((meta >> (4 * t)) & 15u) active |= 1u << t;
            if (meta & META_UNFLIPPED) active |= 0x10u;
            if (meta & META_FLIPPED) active |= 0x20u;
            const uint32_t cov = __float_as_uint((float)(uint32_t)cm);
            const K key = nkey[ja];
            for (unsigned long long Wg = W; Wg < en; Wg += WARP_STAGE) {
                const unsigned long long we = min(en, Wg + WARP_STAGE);
                const Sink o{stage, (long long)Wg, (long long)we, false};
                if (lane == 0) write_record_bytes<K>(o, (long long)W, (long long)en, key, meta, active, cov, k, nb);
                __syncwarp();
                window_out(a.out, stage, base + Wg, base + we, lane);
                __syncwarp();
            }
            ja++;
            continue;
        }
        // ---- records [ja, jb): the most that fit in one window (usually all the warp's) ----
        uint32_t lo = ja + 1, hi = j1;
        if (off_at(j1) - W <= WARP_STAGE) lo = j1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (off_at(mid) - W <= WARP_STAGE)
                lo = mid;
            else
                hi = mid - 1;
        }
        const uint32_t jb = lo;
        const unsigned long long wend = off_at(jb);
        const uint32_t iters = (jb - ja + 31) / 32;
        uint32_t carry = 0;  // tail bytes of the previous iteration's last record
        for (uint32_t it = 0; it < iters; it++) {
            const uint32_t j = ja + 32 * it + lane;
            const bool live = j < jb;
            uint32_t st = 0, en = 0, lv = 0, first = 0;
            if (live) {
                st = (uint32_t)(noff[j] - W);
                en = (uint32_t)(off_at(j + 1) - W);
                const K key = nkey[j];
                const unsigned long long cm = ncm[j];
                const uint32_t meta = (uint32_t)(cm >> 32);
                uint32_t active = 0x80u;
#pragma unroll
                for (int t = 0; t < 4; t++)
                    if ((meta >> (4 * t)) & 15u) active |= 1u << t;
                const bool heads = (meta & (META_UNFLIPPED | META_FLIPPED)) != 0;
                if (meta & META_UNFLIPPED) active |= 0x10u;
                if (meta & META_FLIPPED) active |= 0x20u;
                const uint32_t cov_le = __byte_perm(__float_as_uint((float)(uint32_t)cm), 0, 0x0123);
                RecAcc o;
                o.init(stage32, st);
                o.be32(en - st - 8);
                o.be32((uint32_t)(4 + nb));
                o.be32((uint32_t)k);
                put_key<K>(o, key, nb);
                o.put(active, 1);
                // the edge lists in FF, FR, RF, RR order; a list's neighbours in the order of
                // their extension base (the reference's lists are unordered sets)
                uint32_t lists = active & 15u;
                while (lists) {
                    const int t = __ffs(lists) - 1;
                    lists &= lists - 1;
                    uint32_t m = (meta >> (4 * t)) & 15u;
                    o.be32((uint32_t)__popc(m));
                    while (m) {
                        const int e = __ffs(m) - 1;
                        m &= m - 1;
                        o.be32((uint32_t)k);
                        put_key<K>(o, edge_neighbor<K>(key, t, e, k), nb);
                    }
                }
                if (!heads) {
                    o.put(cov_le, 4);
                    lv = o.fill ? o.cur : 0u;
                } else {
                    // the head sets fill [lists end, en - 4): store the partial word that
                    // ends the lists (its other bytes come with the heads), then the coverage
                    // bytes; the coverage's tail word is shared with the next record
                    if (o.fill) stage32[o.wi] = o.cur;
#pragma unroll
                    for (int q = 0; q < 4; q++) stage[en - 4 + q] = (uint8_t)(cov_le >> (8 * q));
                    lv = (en & 3) ? cov_le >> (8 * (4 - (en & 3))) : 0u;
                }
                first = o.first;
            }
            // the word shared with the previous record: its tail bytes | this record's head
            uint32_t prev = __shfl_up_sync(full, lv, 1);
            if (lane == 0) prev = carry;
            if (live && (st & 3)) stage32[st >> 2] = first | prev;
            // the window's last record keeps its own tail word
            if (live && j == jb - 1 && (en & 3)) stage32[en >> 2] = lv;
            carry = __shfl_sync(full, lv, 31);
        }
        __syncwarp();
        window_out(a.out, stage, base + W, base + wend, lane);
        __syncwarp();
        ja = jb;
    }
}

void launch_emit_write_part(const EmitArgs &a, cudaStream_t s) {
    if (!a.g.nparts) return;
    const size_t sm = (size_t)WRITER_WARPS * (WARP_STAGE + 32);
    t_launches++;
    if (a.g.wide) {
        cudaFuncSetAttribute(k_emit_write_part<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_emit_write_part<u128><<<a.g.nparts, WRITER_WARPS * 32, sm, s>>>(a);
    } else {
        cudaFuncSetAttribute(k_emit_write_part<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_emit_write_part<uint64_t><<<a.g.nparts, WRITER_WARPS * 32, sm, s>>>(a);
    }
    if (a.n_head_slots) {
        t_launches++;
        // slots of the longest read-head sequence's chunks (odd), when they fit
        uint32_t seqc = a.max_seq ? ((4u * ((a.max_seq + 3) / 4) + 27) >> 4) + 1 : 13u;
        seqc |= 1u;
        if (seqc > HEAD_MAX_SEQ_CHUNKS) seqc = 0;
        const size_t smem = (size_t)HEAD_WARPS * 32 * seqc * 16;
        const unsigned blocks = (unsigned)std::min<uint64_t>((a.n_head_slots + HEAD_WARPS * 32 - 1) / (HEAD_WARPS * 32), 152ull * 16);
        cudaFuncSetAttribute(k_write_heads_part, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_write_heads_part<<<blocks, HEAD_WARPS * 32, smem, s>>>(a.hout, a.n_head_slots, a.part_off, a.text, a.n_text, a.out, seqc);
    }
}

// ---- the BUILD_READ_PARSER plan ----------------------------------------------------------------
//
// JobGenReadLetterParser (genomix-hyracks/.../graph/job/JobGenReadLetterParser.java:60-147)
// writes the parser's tuples unaggregated: one (Kmer, Node) SequenceFile record per k-mer
// occurrence, in read order.  Per occurrence j of a read (ReadsKeyValueParserFactory.SplitReads,
// :150-196, setEdgesForCurAndNext :209-233):
//   key    the canonical k-mer, Kmer.write: its nb packed bytes (Kmer.java:344-346)
//   value  a Node with coverage 1, one edge to the previous occurrence (type by the two
//          orientations: FF->RR, FR->FR, RF->RF, RR->FF) and one to the next (FF, FR, RF, RR),
//          and on the first occurrence the read head (unflipped at offset 0 or flipped at k-1).
// Record sizes follow from the read lengths alone, so one scan places every record; one
// thread per read walks its k-mers and writes them.
// bytes of one read's records: n occurrences, n - 1 edges on each side, the head
__device__ __forceinline__ unsigned long long rp_read_bytes(const LineRec &lr, uint32_t mate, int k) {
    const uint32_t L = mate ? lr.l1 : lr.l0;
    const unsigned long long n = L - (uint32_t)k + 1, nb = (uint32_t)(k + 3) / 4;
    return n * (8 + nb + 1 + 4) + 2 * (n - 1) * (8 + nb) + 5 + head_bytes(lr, mate);
}

__global__ void k_rp_sizes(const LineRec *lines, const uint32_t *reads, uint32_t n_reads, int k,
                           unsigned long long *rbytes) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_reads) return;
    const uint32_t rl = reads[r];
    rbytes[r] = rp_read_bytes(lines[rl >> 1], rl & 1u, k);
}

template <class K>
__device__ __forceinline__ long long rp_key(const Sink &o, long long pos, K v, int nb) {
    for (int i = 0; i < nb; i++) o.b(pos + i, KeyOps<K>::byte_at(v, nb - 1 - i));
    return pos + nb;
}

template <class K>
__global__ void k_rp_write(const uint8_t *text, unsigned long long n_text, const LineRec *lines,
                           const uint32_t *reads, uint32_t n_reads, int k, const unsigned long long *roff,
                           uint8_t *out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_reads) return;
    const Sink o{out, 0, 0, true};
    const int nb = (k + 3) / 4;
    const uint32_t rl = reads[r], mate = rl & 1u;
    const LineRec lr = lines[rl >> 1];
    Walker<K> w;
    walker_for(w, text, n_text, lines, reads, r, k);
    const uint32_t n = w.nk;
    long long pos = (long long)roff[r];
    K c, pc = 0, nc = 0;
    uint32_t bits, d, pd = 0, nd = 0;
    w.next(c, bits, d);
    const uint32_t d0 = d;
    for (uint32_t j = 0; j < n; j++) {
        const bool has_next = j + 1 < n, has_prev = j > 0;
        if (has_next) w.next(nc, bits, nd);
        // edge types: from the previous occurrence, and to the next
        const uint32_t tp = has_prev ? (pd == 0 ? (d == 0 ? 3u : 1u) : (d == 0 ? 2u : 0u)) : 4u;
        const uint32_t tn = has_next ? 2u * d + nd : 4u;
        uint32_t active = 0x80u;
        if (has_prev) active |= 1u << tp;
        if (has_next) active |= 1u << tn;
        if (j == 0) active |= d0 == 0 ? 0x10u : 0x20u;
        const long long st = pos;
        pos += 8;
        pos = rp_key<K>(o, pos, c, nb);
        o.b(pos++, active);
        for (uint32_t t = 0; t < 4; t++) {
            if (t != tp && t != tn) continue;
            o.u32(pos, 1);
            o.u32(pos + 4, (uint32_t)k);
            pos = rp_key<K>(o, pos + 8, t == tp ? pc : nc, nb);
        }
        if (j == 0) {
            // the read head: ReadHeadSet with one ReadHeadInfo (ReadHeadInfo.write, :205-212)
            const uint32_t L = mate ? lr.l1 : lr.l0, Lm = mate ? lr.l0 : lr.l1;
            const unsigned long long uuid = ((unsigned long long)(d0 == 0 ? 0 : k - 1) << 40) |
                                            ((unsigned long long)mate << 35) | (unsigned long long)lr.read_id;
            o.b(pos, 1);
            o.u32(pos + 1, 1);
            o.b(pos + 5, Lm > 0 ? 1u : 0u);
            o.u32(pos + 6, (uint32_t)(uuid >> 32));
            o.u32(pos + 10, (uint32_t)uuid);
            pos = put_seq(o, pos + 14, text + (mate ? lr.s1 : lr.s0), L);
            if (Lm > 0) pos = put_seq(o, pos, text + (mate ? lr.s0 : lr.s1), Lm);
        }
        o.u32(pos, 0x3f800000u);  // coverage 1.0f
        pos += 4;
        o.u32(st, (uint32_t)(pos - st - 8));
        o.u32(st + 4, (uint32_t)nb);
        pc = c;
        pd = d;
        c = nc;
        d = nd;
    }
}

void launch_rp_sizes(const LineRec *lines, const uint32_t *reads, uint32_t n_reads, int k,
                     unsigned long long *rbytes, cudaStream_t s) {
    if (!n_reads) return;
    t_launches++;
    k_rp_sizes<<<(n_reads + 255) / 256, 256, 0, s>>>(lines, reads, n_reads, k, rbytes);
}

void launch_rp_write(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines, const uint32_t *reads,
                     uint32_t n_reads, int k, const unsigned long long *roff, uint8_t *out, cudaStream_t s) {
    if (!n_reads) return;
    t_launches++;
    if (wide)
        k_rp_write<u128><<<(n_reads + 127) / 128, 128, 0, s>>>(text, n_text, lines, reads, n_reads, k, roff, out);
    else
        k_rp_write<uint64_t><<<(n_reads + 127) / 128, 128, 0, s>>>(text, n_text, lines, reads, n_reads, k, roff,
                                                                    out);
}


// ---- the reference's part layout ----------------------------------------------------------------
// KmerNodePairSequenceWriterFactory writes each record into the part the Hyracks partitioner
// picked for its key: KmerPartitionComputerFactory.java:28-52, hash = 31 * hash + (signed)
// byte over the Kmer's packed bytes, sign-folded, modulo the part count.  Regrouping a finished
// record stream that way: each record's part, a stable counting sort of the record indexes by
// part (8-bit digits, one or two passes), a scan of the lengths in the new order, and a copy.
__device__ __forceinline__ uint32_t java_kmer_part(const uint8_t *b, int len, uint32_t nparts) {
    int32_t h = 1;
    for (int i = 0; i < len; i++) h = (int32_t)(31u * (uint32_t)h + (uint32_t)(int32_t)(int8_t)b[i]);
    if (h < 0) h = -(h + 1);
    return (uint32_t)h % nparts;
}

__device__ __forceinline__ uint32_t rd_be32_dev(const uint8_t *p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

// one thread per table partition walks its records: part, offset and length of each
__global__ void k_rl_index(const uint8_t *rec, const unsigned long long *seg, const uint32_t *node_base,
                           uint32_t n_seg, uint32_t nparts, uint32_t *rpart, unsigned long long *roff,
                           uint32_t *rlen) {
    const uint32_t sg = blockIdx.x * blockDim.x + threadIdx.x;
    if (sg >= n_seg) return;
    unsigned long long p = seg[sg];
    uint32_t idx = node_base[sg];
    const unsigned long long e = seg[sg + 1];
    while (p < e) {
        const uint8_t *r = rec + p;
        const uint32_t rl = rd_be32_dev(r), kl = rd_be32_dev(r + 4);
        rpart[idx] = java_kmer_part(r + 12, (int)kl - 4, nparts);  // the VKmer's packed bytes
        roff[idx] = p;
        rlen[idx] = 8 + rl;
        idx++;
        p += 8ull + rl;
    }
}

// partitioned build: the nodes of bucket p sit at node_base[p] .. + part_nodes[p] in nkey (their
// keys) and noff (their record offsets within the bucket): the part from the key's packed bytes,
// most significant first as the record holds them; one block per bucket, one thread per record
template <class K>
__global__ void k_rl_index_nodes(const K *nkey, const unsigned long long *part_off, const unsigned long long *node_base,
                                 const uint32_t *noff, const uint32_t *dense_base, const uint32_t *part_nodes,
                                 uint32_t n_buckets, uint32_t nparts, int nb, uint32_t *rpart,
                                 unsigned long long *roff, uint32_t *rlen) {
    for (uint32_t p = blockIdx.x; p < n_buckets; p += gridDim.x) {
        const uint32_t n = part_nodes[p], db = dense_base[p];
        const unsigned long long base = part_off[p], end = part_off[p + 1];
        const uint32_t *no = noff + node_base[p];
        const K *nk = nkey + node_base[p];
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            const unsigned long long o = base + no[j];
            const unsigned long long e = j + 1 < n ? base + no[j + 1] : end;
            const K v = nk[j];
            int32_t h = 1;
            for (int i = nb - 1; i >= 0; i--)
                h = (int32_t)(31u * (uint32_t)h + (uint32_t)(int32_t)(int8_t)KeyOps<K>::byte_at(v, i));
            if (h < 0) h = -(h + 1);
            rpart[db + j] = (uint32_t)h % nparts;
            roff[db + j] = o;
            rlen[db + j] = (uint32_t)(e - o);
        }
    }
}

constexpr int RL_TILE = 4096;  // records per block in the counting passes

// Up to 256 parts: one stable pass that moves bytes, not indexes.  The records are cut into
// tiles of consecutive records (a source range without gaps): per tile and part, the part's bytes
// in the tile ([part][tile]); their exclusive scan is where each tile's run of each part lands,
// and every entry of it is a record boundary of the new layout.  Two record sources: arrays of
// (part, length, offset) per record in tiles of RL_TILE, or the partitioned build's buckets as
// tiles, read straight from its node keys and record offsets.
struct RecArrays {
    const uint32_t *rpart, *rlen;
    const unsigned long long *roff;
    uint64_t n;
    __device__ uint32_t tile_size(uint32_t t) const {
        const uint64_t rem = n - (uint64_t)t * RL_TILE;
        return rem < (uint64_t)RL_TILE ? (uint32_t)rem : (uint32_t)RL_TILE;
    }
    __device__ void get(uint32_t t, uint32_t j, uint32_t, uint32_t &d, uint32_t &len,
                        unsigned long long &off) const {
        const uint64_t i = (uint64_t)t * RL_TILE + j;
        d = rpart[i];
        len = rlen[i];
        off = roff[i];
    }
};

template <class K>
struct RecNodes {
    const K *nkey;
    const uint32_t *noff;
    const unsigned long long *node_base, *part_off;
    const uint32_t *part_nodes;
    int nb;
    uint32_t nparts;
    __device__ uint32_t tile_size(uint32_t t) const { return part_nodes[t]; }
    __device__ void get(uint32_t t, uint32_t j, uint32_t n, uint32_t &d, uint32_t &len,
                        unsigned long long &off) const {
        const unsigned long long nbase = node_base[t], base = part_off[t];
        off = base + noff[nbase + j];
        const unsigned long long e = j + 1 < n ? base + noff[nbase + j + 1] : part_off[t + 1];
        len = (uint32_t)(e - off);
        const K v = nkey[nbase + j];
        int32_t h = 1;
        for (int i = nb - 1; i >= 0; i--)
            h = (int32_t)(31u * (uint32_t)h + (uint32_t)(int32_t)(int8_t)KeyOps<K>::byte_at(v, i));
        if (h < 0) h = -(h + 1);
        d = (uint32_t)h % nparts;
    }
};

// per tile, each part's bytes; lanes of one part in a warp add up before one shared atomic
template <class Src>
__global__ void __launch_bounds__(256) k_rl_tile_bytes(Src src, uint32_t n_tiles, uint32_t nparts,
                                                       unsigned long long *cnt) {
    __shared__ unsigned long long bins[256];
    __shared__ uint32_t slen[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        bins[threadIdx.x] = 0;
        __syncthreads();
        const uint32_t n = src.tile_size(t);
        for (uint32_t j0 = 0; j0 < n; j0 += 256) {
            const uint32_t j = j0 + threadIdx.x;
            uint32_t d = 256u + lane, len = 0;
            unsigned long long off;
            if (j < n) src.get(t, j, n, d, len, off);
            slen[threadIdx.x] = len;
            const uint32_t same = __match_any_sync(0xffffffffu, d);
            __syncwarp();
            if (j < n && (same & ((1u << lane) - 1u)) == 0) {
                unsigned long long sum = 0;
                for (uint32_t m = same; m; m &= m - 1) sum += slen[warp * 32 + __ffs(m) - 1];
                atomicAdd(&bins[d], sum);
            }
            __syncwarp();
        }
        __syncthreads();
        if (threadIdx.x < nparts) cnt[(uint64_t)threadIdx.x * n_tiles + t] = bins[threadIdx.x];
        __syncthreads();
    }
}

constexpr int RL_STAGE = 36 * 1024;              // source bytes of one round, staged in shared memory
constexpr int RL_OUT = RL_STAGE + 256 * 16;        // the round's output runs, each at its destination's alignment
constexpr int RL_SMEM = RL_STAGE + 16 + RL_OUT;    // dynamic shared memory of k_rl_move

// copies n bytes between shared-memory addresses of any alignment: bytes up to the destination's
// word boundary, then whole destination words assembled from two source words, then the rest
__device__ __forceinline__ void smem_copy_bytes(uint8_t *d, const uint8_t *s, uint32_t n) {
    uint32_t i = min(n, (4u - ((uint32_t)(uintptr_t)d & 3u)) & 3u);
    for (uint32_t x = 0; x < i; x++) d[x] = s[x];
    const uint32_t nw = (n - i) >> 2;
    if (nw) {
        const uint8_t *sp = s + i;
        const uint32_t sh = ((uint32_t)(uintptr_t)sp & 3u) * 8u;
        const uint32_t *sw = reinterpret_cast<const uint32_t *>((uintptr_t)sp & ~(uintptr_t)3);
        uint32_t *dw = reinterpret_cast<uint32_t *>(d + i);
        uint32_t lo = sw[0];
        for (uint32_t w = 0; w < nw; w++) {
            const uint32_t hi = sw[w + 1];
            dw[w] = __funnelshift_r(lo, hi, sh);
            lo = hi;
        }
        i += nw * 4;
    }
    for (; i < n; i++) d[i] = s[i];
}

constexpr long long RL_WAIT_CYCLES = 2000000000LL;  // about a second: a bulk copy takes microseconds

// The tile's records in source order, 256 at a time.  A record lands after the earlier records
// of its part (earlier rounds, earlier warps of this round, earlier lanes of its warp), so this
// round's records of part d form one run of the output, starting where the part's previous run
// ended.  The round's source bytes (one range, its ends rounded to 16 bytes) come in with one
// bulk copy (TMA) issued by thread 0 and completed on an mbarrier, while the threads rank the
// round's records; the waits are bounded: a copy that has not landed after about a second
// (never expected; `withhold` makes it happen, for testing) sets *err, waits once more for the
// copy and ends the CTA.  Each thread copies
// its record into that run's image in shared memory, the image placed at the run's own 16-byte
// alignment; each warp then writes whole runs out with aligned 16-byte stores (the ragged ends
// byte by byte, one lane per byte).  A round whose range does not fit (a giant record) copies
// each record from global memory with a warp instead.  The next round's record descriptors and
// the next tile's part offsets are loaded while the current round works.
template <class Src>
__global__ void __launch_bounds__(256) k_rl_move(const uint8_t *sbytes, Src src, uint32_t n_tiles, uint32_t nparts,
                                                 const unsigned long long *off, uint8_t *dst, uint32_t *err,
                                                 int withhold) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint8_t *stage = smem;                 // RL_STAGE + 16 (word reads may run 3 bytes past a record)
    uint8_t *img = smem + RL_STAGE + 16;   // RL_OUT
    __shared__ unsigned long long bar;     // completion of the round's bulk copy
    __shared__ unsigned long long run[256];
    __shared__ unsigned long long wb[8][256];
    __shared__ unsigned long long sdst[256], ssrc[256];
    __shared__ uint32_t slen[256], obase[256], wsum[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t tid = threadIdx.x;
    uint32_t t = blockIdx.x;
    if (t >= n_tiles) return;
    uint32_t n = src.tile_size(t), j0 = 0;
    // this round's descriptor (d, len, so) and the tile's offsets, loaded one round ahead
    uint32_t d = 256u + lane, len = 0;
    unsigned long long so = 0;
    if (tid < n) src.get(t, tid, n, d, len, so);
    run[tid] = tid < nparts ? off[(uint64_t)tid * n_tiles + t] : 0ull;
    if (tid == 0) mbar_init(&bar, 1);
    __syncthreads();
    uint32_t parity = 0;
    for (;;) {
        const bool live = j0 + tid < n;
        for (int w = 0; w < 8; w++) wb[w][tid] = 0;
        slen[tid] = len;
        ssrc[tid] = so;
        __syncthreads();
        // the next round: the rest of this tile, else the next tile
        uint32_t nt = t, nj0 = j0 + 256, nn = n;
        if (nj0 >= n) {
            nt = t + gridDim.x;
            nj0 = 0;
            nn = nt < n_tiles ? src.tile_size(nt) : 0u;
        }
        // the round's source range, brought in by one bulk copy while the records are ranked
        // records this round; an empty bucket (no nodes) still takes one round, with nothing to move
        const uint32_t cnt = n > j0 ? min(256u, n - j0) : 0u;
        const unsigned long long lo = cnt ? ssrc[0] & ~15ull : 0ull;
        const unsigned long long hi = cnt ? (ssrc[cnt - 1] + slen[cnt - 1] + 15) & ~15ull : 0ull;
        const bool fits = hi - lo <= (unsigned long long)RL_STAGE;
        const bool bulk = fits && hi > lo;
        if (bulk && tid == 0 && !withhold) {
            fence_proxy_async_smem();  // the last round's reads of the stage come first
            mbar_arrive_expect_tx(&bar, (uint32_t)(hi - lo));
            bulk_g2s(stage, sbytes + lo, (uint32_t)(hi - lo), &bar);
        }
        uint32_t d2 = 256u + lane, len2 = 0;
        unsigned long long so2 = 0, run2 = 0;
        if (nt < n_tiles && nj0 + tid < nn) src.get(nt, nj0 + tid, nn, d2, len2, so2);
        if (nt != t && nt < n_tiles && tid < nparts) run2 = off[(uint64_t)tid * n_tiles + nt];
        // ranks within the warp
        const uint32_t same = __match_any_sync(0xffffffffu, d);
        uint32_t pre = 0;
        for (uint32_t m = same & ((1u << lane) - 1u); m; m &= m - 1) pre += slen[warp * 32 + __ffs(m) - 1];
        if (live && (same >> lane) == 1u) wb[warp][d] = (unsigned long long)pre + len;  // the group's last lane
        if (bulk) {
            const bool late = !mbar_wait_bounded(&bar, parity, RL_WAIT_CYCLES);
            if (__syncthreads_or(late)) {
                if (tid == 0) atomicOr(err, 1u);
                if (!withhold) mbar_wait_bounded(&bar, parity, 4 * RL_WAIT_CYCLES);  // the copy in flight
                return;
            }
            parity ^= 1u;
        }
        __syncthreads();
        // this thread's part (tid): its run this round and the run's image slot
        unsigned long long bytes = 0;
        for (int w = 0; w < 8; w++) bytes += wb[w][tid];
        const uint32_t g15 = (uint32_t)run[tid] & 15u;
        const uint32_t res = bytes ? (uint32_t)min((g15 + bytes + 15ull) & ~15ull, (unsigned long long)RL_OUT + 16) : 0u;
        uint32_t inc = res;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int w = 0; w < 8; w++) {
            const uint32_t v = wsum[w];
            before += w < warp ? v : 0u;
            total += v;
        }
        obase[tid] = before + inc - res;
        const bool staged = fits && total <= (uint32_t)RL_OUT;
        __syncthreads();
        if (live) {
            unsigned long long rank = pre;  // bytes of the part before this record, this round
            for (int w = 0; w < warp; w++) rank += wb[w][d];
            if (staged)
                smem_copy_bytes(img + obase[d] + ((uint32_t)run[d] & 15u) + (uint32_t)rank,
                                stage + (uint32_t)(so - lo), len);
            else
                sdst[tid] = run[d] + rank;
        }
        __syncthreads();
        if (staged) {
            for (uint32_t q = warp; q < nparts; q += 8) {
                unsigned long long b = 0;
                for (int w = 0; w < 8; w++) b += wb[w][q];
                if (!b) continue;
                const unsigned long long s0 = run[q];
                const uint32_t h = (uint32_t)s0 & 15u;                    // image offset of the run's first byte
                const uint32_t e = h + (uint32_t)b;                        // image offset of its end
                uint8_t *dq = dst + (s0 & ~15ull);
                const uint8_t *im = img + obase[q];
                const uint32_t fe = e & ~15u;                              // whole 16-byte units: [fb, fe)
                const uint32_t fb = (h + 15u) & ~15u;
                for (uint32_t u = fb + 16u * lane; u < fe; u += 16u * 32u)
                    *reinterpret_cast<uint4 *>(dq + u) = *reinterpret_cast<const uint4 *>(im + u);
                // ragged ends: the head [h, min(fb, e)) and the tail [max(fe, fb), e), one lane per byte
                const uint32_t hx = h + lane;
                if (hx < fb && hx < e) dq[hx] = im[hx];
                const uint32_t tx = max(fe, fb) + lane;
                if (lane < 16 && tx < e) dq[tx] = im[tx];
            }
        } else {
            for (uint32_t q = 0; q < 32; q++) {
                const uint32_t r = warp * 32 + q;
                if (r >= cnt) break;
                const uint32_t L = slen[r];
                const uint8_t *sp = sbytes + ssrc[r];
                uint8_t *dp = dst + sdst[r];
                for (uint32_t x = lane; x < L; x += 32) dp[x] = sp[x];
            }
        }
        __syncthreads();
        if (nt >= n_tiles) break;
        if (nt != t) {
            run[tid] = run2;
        } else {
            run[tid] += bytes;
        }
        t = nt;
        j0 = nj0;
        n = nn;
        d = d2;
        len = len2;
        so = so2;
    }
}

__global__ void k_rl_part_starts(const unsigned long long *off, uint32_t n_tiles, uint32_t nparts,
                                 unsigned long long total, unsigned long long *bounds) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nparts) bounds[q] = off[(uint64_t)q * n_tiles];
    if (q == nparts) bounds[q] = total;
}

// per tile, how many of its records fall in each digit (column-major: [digit][tile])
__global__ void __launch_bounds__(256) k_rl_count(const uint32_t *key, const uint32_t *val, uint64_t n, int shift,
                                                  uint32_t n_tiles, uint32_t *cnt) {
    __shared__ uint32_t bins[256];
    bins[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t t0 = (uint64_t)blockIdx.x * RL_TILE;
    for (uint64_t i = t0 + threadIdx.x; i < min(n, t0 + RL_TILE); i += 256)
        atomicAdd(&bins[(key[val ? val[i] : i] >> shift) & 255u], 1u);
    __syncthreads();
    cnt[(uint64_t)threadIdx.x * n_tiles + blockIdx.x] = bins[threadIdx.x];
}

// stable scatter: the tile's records in order, 256 at a time; a record's rank among the same
// digit = earlier rounds + earlier warps of this round + earlier lanes of its warp
__global__ void __launch_bounds__(256) k_rl_scatter(const uint32_t *key, const uint32_t *val, uint64_t n, int shift,
                                                    uint32_t n_tiles, const uint32_t *off, uint32_t *out_val) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wcnt[8][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    run[threadIdx.x] = off[(uint64_t)threadIdx.x * n_tiles + blockIdx.x];
    const uint64_t t0 = (uint64_t)blockIdx.x * RL_TILE;
    for (int r = 0; r < RL_TILE / 256; r++) {
        for (int w = 0; w < 8; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const uint64_t i = t0 + (uint64_t)r * 256 + threadIdx.x;
        const bool live = i < n;
        const uint32_t v = live ? (val ? val[i] : (uint32_t)i) : 0u;
        const uint32_t d = live ? (key[v] >> shift) & 255u : 256u + lane;  // idle lanes never match
        const uint32_t same = __match_any_sync(0xffffffffu, d);
        const uint32_t wr = __popc(same & ((1u << lane) - 1u));
        if (live && wr == 0) wcnt[warp][d] = __popc(same);
        __syncthreads();
        if (live) {
            uint32_t before = run[d] + wr;
            for (int w = 0; w < warp; w++) before += wcnt[w][d];
            out_val[before] = v;
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < 8; w++) add += wcnt[w][threadIdx.x];
        run[threadIdx.x] += add;
        __syncthreads();
    }
}

__global__ void k_rl_gather_len(const uint32_t *perm, const uint32_t *rlen, uint64_t n, unsigned long long *len2) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) len2[i] = rlen[perm[i]];
}

// one warp per record: its bytes to their new place
__global__ void k_rl_copy(const uint8_t *src, const uint32_t *perm, const unsigned long long *roff,
                          const unsigned long long *noff, const uint32_t *rlen, uint64_t n, uint8_t *dst) {
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint32_t o = perm[i], len = rlen[o];
    const uint8_t *s = src + roff[o];
    uint8_t *d = dst + noff[i];
    for (uint32_t x = lane; x < len; x += 32) d[x] = s[x];
}

// the first sorted record of each part (empty parts start where the next one does) and the
// byte offset it lands at; then every stride-th record's offset (emit split points)
__global__ void k_rl_bounds(const uint32_t *rpart, const uint32_t *perm, uint64_t n, uint32_t nparts,
                            const unsigned long long *noff, unsigned long long *bounds) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = rpart[perm[i]];
    const uint32_t q0 = i == 0 ? 0u : rpart[perm[i - 1]] + 1u;
    for (uint32_t q = q0; q <= p; q++) bounds[q] = noff[i];
    if (i == n - 1)
        for (uint32_t q = p + 1; q <= nparts; q++) bounds[q] = noff[n];
}

__global__ void k_rl_sample(const unsigned long long *noff, uint64_t n, uint32_t stride, uint64_t m,
                            unsigned long long *out) {
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < m) out[g] = noff[min(n, g * stride)];
}

void launch_rl_bounds(const uint32_t *rpart, const uint32_t *perm, uint64_t n, uint32_t nparts,
                      const unsigned long long *noff, unsigned long long *bounds, cudaStream_t s) {
    if (!n) return;
    t_launches++;
    k_rl_bounds<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rpart, perm, n, nparts, noff, bounds);
}

void launch_rl_sample(const unsigned long long *noff, uint64_t n, uint32_t stride, uint64_t m,
                      unsigned long long *out, cudaStream_t s) {
    if (!m) return;
    t_launches++;
    k_rl_sample<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(noff, n, stride, m, out);
}

void launch_rl_index(const uint8_t *rec, const unsigned long long *seg, const uint32_t *node_base,
                     uint32_t n_seg, uint32_t nparts, uint32_t *rpart, unsigned long long *roff, uint32_t *rlen,
                     cudaStream_t s) {
    if (!n_seg) return;
    t_launches++;
    k_rl_index<<<(n_seg + 127) / 128, 128, 0, s>>>(rec, seg, node_base, n_seg, nparts, rpart, roff, rlen);
}

uint32_t rl_tiles(uint64_t n) { return (uint32_t)((n + RL_TILE - 1) / RL_TILE); }

void launch_rl_index_nodes(const void *nkey, int wide, int k, const unsigned long long *part_off,
                           const unsigned long long *node_base, const uint32_t *noff, const uint32_t *dense_base,
                           const uint32_t *part_nodes, uint32_t n_buckets, uint32_t nparts, uint32_t *rpart,
                           unsigned long long *roff, uint32_t *rlen, cudaStream_t s) {
    if (!n_buckets) return;
    t_launches++;
    const unsigned blocks = std::min<uint32_t>(n_buckets, 152u * 8u);
    const int nb = (k + 3) / 4;
    if (wide)
        k_rl_index_nodes<u128><<<blocks, 256, 0, s>>>((const u128 *)nkey, part_off, node_base, noff, dense_base,
                                                      part_nodes, n_buckets, nparts, nb, rpart, roff, rlen);
    else
        k_rl_index_nodes<uint64_t><<<blocks, 256, 0, s>>>((const uint64_t *)nkey, part_off, node_base, noff,
                                                          dense_base, part_nodes, n_buckets, nparts, nb, rpart, roff,
                                                          rlen);
}

template <class Src>
static void rl_regroup(const uint8_t *sbytes, Src src, uint32_t n_tiles, uint32_t nparts, unsigned long long *cnt,
                       void *scratch, uint8_t *dst, uint32_t *err, int withhold, cudaStream_t s) {
    const uint64_t ncnt = (uint64_t)nparts * n_tiles;
    const unsigned blocks = std::min<uint32_t>(n_tiles, 152u * 16u);
    t_launches += 2;
    k_rl_tile_bytes<Src><<<blocks, 256, 0, s>>>(src, n_tiles, nparts, cnt);
    exclusive_scan_u64(cnt, cnt, ncnt, cnt + ncnt, scratch, s);
    cudaFuncSetAttribute(k_rl_move<Src>, cudaFuncAttributeMaxDynamicSharedMemorySize, RL_SMEM);
    k_rl_move<Src><<<blocks, 256, RL_SMEM, s>>>(sbytes, src, n_tiles, nparts, cnt, dst, err, withhold);
}

void launch_rl_regroup_arrays(const uint8_t *sbytes, const uint32_t *rpart, const uint32_t *rlen,
                              const unsigned long long *roff, uint64_t n, uint32_t nparts, unsigned long long *cnt,
                              void *scratch, uint8_t *dst, uint32_t *err, int withhold, cudaStream_t s) {
    if (!n) return;
    RecArrays src{rpart, rlen, roff, n};
    rl_regroup(sbytes, src, rl_tiles(n), nparts, cnt, scratch, dst, err, withhold, s);
}

void launch_rl_regroup_nodes(const uint8_t *sbytes, const void *nkey, int wide, int k, const uint32_t *noff,
                             const unsigned long long *node_base, const unsigned long long *part_off,
                             const uint32_t *part_nodes, uint32_t n_buckets, uint32_t nparts, unsigned long long *cnt,
                             void *scratch, uint8_t *dst, uint32_t *err, int withhold, cudaStream_t s) {
    if (!n_buckets) return;
    const int nb = (k + 3) / 4;
    if (wide) {
        RecNodes<u128> src{(const u128 *)nkey, noff, node_base, part_off, part_nodes, nb, nparts};
        rl_regroup(sbytes, src, n_buckets, nparts, cnt, scratch, dst, err, withhold, s);
    } else {
        RecNodes<uint64_t> src{(const uint64_t *)nkey, noff, node_base, part_off, part_nodes, nb, nparts};
        rl_regroup(sbytes, src, n_buckets, nparts, cnt, scratch, dst, err, withhold, s);
    }
}

void launch_rl_part_starts(const unsigned long long *off, uint32_t n_tiles, uint32_t nparts, unsigned long long total,
                           unsigned long long *bounds, cudaStream_t s) {
    t_launches++;
    k_rl_part_starts<<<(nparts + 256) / 256, 256, 0, s>>>(off, n_tiles, nparts, total, bounds);
}

void launch_rl_count(const uint32_t *key, const uint32_t *val, uint64_t n, int shift, uint32_t *cnt, cudaStream_t s) {
    const uint32_t t = rl_tiles(n);
    if (!t) return;
    t_launches++;
    k_rl_count<<<t, 256, 0, s>>>(key, val, n, shift, t, cnt);
}

void launch_rl_scatter(const uint32_t *key, const uint32_t *val, uint64_t n, int shift, const uint32_t *off,
                       uint32_t *out_val, cudaStream_t s) {
    const uint32_t t = rl_tiles(n);
    if (!t) return;
    t_launches++;
    k_rl_scatter<<<t, 256, 0, s>>>(key, val, n, shift, t, off, out_val);
}

void launch_rl_gather_len(const uint32_t *perm, const uint32_t *rlen, uint64_t n, unsigned long long *len2,
                          cudaStream_t s) {
    if (!n) return;
    t_launches++;
    k_rl_gather_len<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(perm, rlen, n, len2);
}

void launch_rl_copy(const uint8_t *src, const uint32_t *perm, const unsigned long long *roff,
                    const unsigned long long *noff, const uint32_t *rlen, uint64_t n, uint8_t *dst, cudaStream_t s) {
    if (!n) return;
    t_launches++;
    k_rl_copy<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(src, perm, roff, noff, rlen, n, dst);
}

}  // namespace gx
