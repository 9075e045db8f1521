// gx_kernels.cu — the graph-build kernels (sm_103a).
//
//   K1  line split + per-line parse    ReadsKeyValueParserFactory.parse (:95-148)
//   K2  k-mer roll + canonical + edges SplitReads / setEdgesForCurAndNext (:150-233)
//   K3  table insert                   ExternalSort + PreclusteredGroup +
//                                      AggregateKmerAggregateFactory (:93-175)
//   K4  read-head bucketing + sort     ReadHeadSet / ExternalableTreeSet.union (:138-145)
//   K5  compaction + serialization     outputFinalResult (:185-214), Node.write,
//                                      KmerNodePairSequenceWriterFactory.write (:79-94)
#include <cstdio>

#include "gx_kernels.cuh"

namespace gx {

static thread_local uint64_t t_launches = 0;
uint64_t launches_this_thread() { return t_launches; }

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
// K1b: per-line parse, one warp per line.  Reproduces, in order, the checks of
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

__global__ void __launch_bounds__(256) k_parse_lines(const uint8_t *text, uint64_t n_text,
                                                     const unsigned long long *line_end, uint32_t n_lines, int k,
                                                     LineRec *lines, uint8_t *lflags, uint32_t *nvalid,
                                                     DevStatus *st) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t line = warp0; line < n_lines; line += nwarps) {
        const uint64_t b = line == 0 ? 0 : line_end[line - 1] + 1;
        uint64_t e = line_end[line];
        if (e < n_text && e > b && text[e] == '\n' && text[e - 1] == '\r') e--;
        const uint32_t len = (uint32_t)(e - b);

        // pass 1: tabs (first three positions, total) and the last non-tab byte
        uint32_t tab[3] = {len, len, len};
        uint32_t found = 0, tabs = 0;
        int last_nt = -1;
        const uint64_t c0 = b & ~15ULL;
        for (uint64_t w = c0; w < e; w += 512) {
            const uint64_t chunk = w + 16 * (uint64_t)lane;
            uint32_t tm = 0;
            int lnt = -1;
            if (chunk < e) {
                uint32_t wd[4];
                load16(text, n_text, chunk, wd);
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const uint64_t p = chunk + q;
                    if (p < b || p >= e) continue;
                    const uint32_t c = (wd[q >> 2] >> (8 * (q & 3))) & 0xffu;
                    if (c == '\t')
                        tm |= 1u << q;
                    else
                        lnt = (int)(p - b);
                }
            }
            const uint32_t cl = __popc(tm);
            const uint32_t incl = warp_inclusive_scan(cl);
            const uint32_t pre = incl - cl;
            const uint32_t wt = __shfl_sync(0xffffffffu, incl, 31);
            for (uint32_t r = found; r < 3 && r < found + wt; r++) {
                const uint32_t rr = r - found;
                const bool own = rr >= pre && rr < incl;
                const uint32_t om = __ballot_sync(0xffffffffu, own);
                uint32_t pos = 0;
                if (own) {
                    uint32_t m = tm;
                    for (uint32_t i = 0; i < rr - pre; i++) m &= m - 1;
                    pos = (uint32_t)(chunk + (__ffs(m) - 1) - b);
                }
                tab[r] = __shfl_sync(0xffffffffu, pos, __ffs(om) - 1);
            }
            found = min(3u, found + wt);
            tabs += wt;
            last_nt = max(last_nt, __reduce_max_sync(0xffffffffu, lnt));
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
        const uint32_t f1b = tab[0] + 1, f1e = tabs >= 2 ? tab[1] : len;
        const uint32_t f2b = tab[1] + 1, f2e = tabs >= 3 ? tab[2] : len;
        bool bad1 = false, bad2 = false;
        if (nf == 2 || nf == 3) {
            // pass 2: [ACGTacgt]+ over fields 1 and 2
            const uint32_t vb = f1b, ve = nf == 3 ? f2e : f1e;
            uint32_t lb1 = 0, lb2 = 0;
            for (uint64_t w = (b + vb) & ~15ULL; w < b + ve; w += 512) {
                const uint64_t chunk = w + 16 * (uint64_t)lane;
                if (chunk < b + ve) {
                    uint32_t wd[4];
                    load16(text, n_text, chunk, wd);
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const uint64_t p = chunk + q;
                        if (p < b + vb || p >= b + ve) continue;
                        const uint32_t rel = (uint32_t)(p - b);
                        const uint32_t c = (wd[q >> 2] >> (8 * (q & 3))) & 0xffu;
                        const bool ok = is_acgt(c);
                        if (rel >= f1b && rel < f1e && !ok) lb1 = 1;
                        if (nf == 3 && rel >= f2b && rel < f2e && !ok) lb2 = 1;
                    }
                }
            }
            bad1 = __any_sync(0xffffffffu, lb1);
            bad2 = __any_sync(0xffffffffu, lb2);
        }
        if (lane == 0) {
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
            } else if (!java_parse_long(text + b, tab[0], rid)) {
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
                atomicMin(&st->parse_err, ((unsigned long long)line << 8) | code);
                fl = 0;
            }
            lines[line] = lr;
            lflags[line] = fl;
            nvalid[line] = (fl & LF_M0_VALID ? 1u : 0u) + (fl & LF_M1_VALID ? 1u : 0u);
        }
    }
}

void launch_parse_lines(const uint8_t *text, uint64_t n_text, const unsigned long long *line_end, uint32_t n_lines,
                        int k, LineRec *lines, uint8_t *lflags, uint32_t *nvalid, DevStatus *st, cudaStream_t s) {
    if (!n_lines) return;
    const uint64_t warps = n_lines;
    uint64_t blocks = (warps * 32 + 255) / 256;
    if (blocks > 152ull * 64) blocks = 152ull * 64;
    t_launches++;
    k_parse_lines<<<(unsigned)blocks, 256, 0, s>>>(text, n_text, line_end, n_lines, k, lines, lflags, nvalid, st);
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
    uint32_t N = 1;
    while (N < n) N <<= 1;
    for (uint32_t size = 2; size <= N; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < N / 2; i += blockDim.x) {
                const uint32_t blk = i / stride, off = i % stride;
                uint32_t lo, hi;
                if (stride == (size >> 1)) {
                    lo = blk * size + off;
                    hi = blk * size + size - 1 - off;
                } else {
                    lo = blk * 2 * stride + off;
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
    {
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

}  // namespace gx
