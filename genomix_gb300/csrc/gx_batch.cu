// gx_batch.cu — many graph builds in one pass over the device (gx_batch_run).
//
// The jobs of a batch (same k) are laid end to end in one text buffer and go through the
// partitioned build together: one parse, one occurrence count that keeps a super-bucket
// histogram and HyperLogLog registers per sample, then one bucket space in which every
// sample owns its own contiguous range of super and fine buckets (sized from its own
// distinct-k-mer estimate).  Buckets never mix samples, so each sample's records come out
// as one contiguous run of the shared record buffer, and its Node set is the one its plain
// gx_job_run produces.  Small samples stop costing a full launch sequence each: the whole
// batch takes the same ~40 launches and 3 host round trips as one job.
//
// A batch falls back to running its jobs one by one when any input has a parse error (so
// every job reports its own status and line), when a bucket overflows three times, or when
// the batch does not fit in device memory (it is split in halves first).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/gxgpu.h"
#include "gx_job_internal.h"
#include "gx_kernels.cuh"

using namespace gx;
using namespace gxi;

namespace {

constexpr uint32_t MAX_BATCH = 1024;  // samples per pass: each needs at least one super bucket
constexpr gx_status BATCH_FALLBACK = (gx_status)-1;

// Bucket plan of a batch.  Sample s wants P_s fine buckets (distinct estimate x safety /
// target per bucket); its super buckets S_s = 2^log_s start near sqrt(P_s) / 2 and are halved,
// largest first, until the batch fits MAX_SUPERS; F_s = ceil(P_s / S_s) <= MAX_FINE.
bool plan_batch(const std::vector<double> &d_est, double safety, double target, std::vector<SamplePlan> &plans,
                uint32_t &n_super, uint32_t &n_fine) {
    const size_t n = d_est.size();
    std::vector<uint64_t> P(n);
    std::vector<uint32_t> lg(n), lmin(n);
    uint64_t sum = 0;
    for (size_t i = 0; i < n; i++) {
        double want = d_est[i] * safety / target;
        P[i] = (uint64_t)std::max(1.0, std::ceil(want));
        uint32_t lo = 0;  // F <= MAX_FINE needs S >= P / MAX_FINE
        while ((uint64_t)MAX_FINE << lo < P[i]) lo++;
        if (lo > 11) return false;
        uint32_t l = 0;
        while ((1ull << (2 * l)) < P[i] && l < 11) l++;
        if (l > 6) l--;  // half of sqrt(P), as a single job's plan (lo keeps F within MAX_FINE)
        lmin[i] = lo;
        lg[i] = std::max(l, lo);
        sum += 1ull << lg[i];
    }
    while (sum > MAX_SUPERS) {
        size_t best = n;
        for (size_t i = 0; i < n; i++)
            if (lg[i] > lmin[i] && (best == n || lg[i] > lg[best])) best = i;
        if (best == n) return false;
        sum -= 1ull << (lg[best] - 1);
        lg[best]--;
    }
    plans.resize(n);
    uint64_t sb = 0, fb = 0;
    for (size_t i = 0; i < n; i++) {
        const uint64_t S = 1ull << lg[i];
        const uint64_t F = std::max<uint64_t>(1, (P[i] + S - 1) / S);
        if (F > MAX_FINE) return false;
        plans[i] = SamplePlan{(uint32_t)sb, lg[i], (uint32_t)F, (uint32_t)fb};
        sb += S;
        fb += S * F;
        if (fb > 0x7fffffffULL) return false;
    }
    n_super = (uint32_t)sb;
    n_fine = (uint32_t)fb;
    return true;
}

// One pass over a group of jobs with the same k, all with readid text on the device.
gx_status run_group_impl(gx_ctx *c, const std::vector<gx_job *> &jobs);

gx_status run_group(gx_ctx *c, const std::vector<gx_job *> &jobs) {
    return guarded("gx_batch_run", [&] { return run_group_impl(c, jobs); });
}

gx_status run_group_impl(gx_ctx *c, const std::vector<gx_job *> &jobs) {
    cudaStream_t s = c->stream;
    const uint32_t n = (uint32_t)jobs.size();
    const int k = jobs[0]->k, wide = jobs[0]->wide;
    const size_t kb = wide ? 16 : 8;
    const uint64_t l0 = launches_this_thread();
    Timers tm;
    tm.init();
    struct TimersGuard {
        Timers &t;
        ~TimersGuard() { t.destroy(); }
    } tg{tm};
    gx_status e;

    // a borrowed device input may lack its final terminator: add one so that lines never
    // join across samples
    std::vector<uint8_t> lastb(n, '\n');
    bool any_borrowed = false;
    for (uint32_t i = 0; i < n; i++)
        if (jobs[i]->text_borrowed && jobs[i]->text_len) {
            CK(d2h_async(&lastb[i], jobs[i]->d_text + jobs[i]->text_len - 1, 1, s));
            any_borrowed = true;
        }
    if (any_borrowed) CK(sync_stream(s));
    std::vector<unsigned long long> tb(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) tb[i + 1] = tb[i] + jobs[i]->text_len + (lastb[i] != '\n' ? 1 : 0);
    const uint64_t n_text = tb[n];
    for (gx_job *j : jobs) {
        memset(&j->st, 0, sizeof j->st);
        j->st.key_bits = wide ? 128 : 64;
        j->part_bounds.assign(j->o.out_parts + 1, 0);
        j->cursor.assign(j->o.out_parts, 0);
    }
    if (n_text == 0) return GX_OK;

    RunArena ar(s);
    uint8_t *text;
    DevStatus *d_st;
    if ((e = ar.alloc(text, n_text + 16)) != GX_OK) return e;
    if ((e = ar.alloc(d_st, 1)) != GX_OK) return e;
    CK(cudaEventRecord(tm.ev[0], s));
    for (uint32_t i = 0; i < n; i++) {
        if (jobs[i]->text_len)
            CK(cudaMemcpyAsync(text + tb[i], jobs[i]->d_text, jobs[i]->text_len, cudaMemcpyDeviceToDevice, s));
        if (lastb[i] != '\n') CK(cudaMemsetAsync(text + tb[i] + jobs[i]->text_len, '\n', 1, s));
    }
    {
        DevStatus init{};
        init.parse_err = ~0ULL;
        CK(cudaMemcpyAsync(d_st, &init, sizeof init, cudaMemcpyHostToDevice, s));
    }

    // ---- parse the whole batch, then find each sample's lines and reads ----
    const uint64_t tiles = line_tiles(n_text);
    uint32_t *tile_cnt, *d_nlines, *line_base, *read_base;
    unsigned long long *d_tb;
    void *scratch;
    const size_t scratch_bytes = std::max(scan_scratch_bytes(std::max<uint64_t>(tiles, 1), 8),
                                          scan_scratch_bytes(n_text + 16, 8));
    if ((e = ar.alloc(tile_cnt, tiles + 1)) != GX_OK) return e;
    if ((e = ar.alloc(d_nlines, 4)) != GX_OK) return e;
    if ((e = ar.alloc(scratch, scratch_bytes)) != GX_OK) return e;
    unsigned long long *d_occ;
    if ((e = ar.alloc(d_occ, n)) != GX_OK) return e;
    if ((e = ar.alloc(line_base, n + 1)) != GX_OK) return e;
    if ((e = ar.alloc(read_base, n + 1)) != GX_OK) return e;
    if ((e = ar.alloc(d_tb, n + 1)) != GX_OK) return e;
    CK(cudaMemsetAsync(d_occ, 0, (size_t)n * 8, s));
    CK(cudaMemcpyAsync(d_tb, tb.data(), (n + 1) * 8ull, cudaMemcpyHostToDevice, s));
    launch_count_lines(text, n_text, tile_cnt, s);
    exclusive_scan_u32(tile_cnt, tile_cnt, tiles, d_nlines, scratch, s);
    uint32_t n_lines = 0;
    CK(d2h_async(&n_lines, d_nlines, 4, s));
    CK(sync_stream(s));
    unsigned long long *line_end;
    LineRec *lines;
    uint8_t *lflags;
    uint32_t *nvalid, *reads;
    if ((e = ar.alloc(line_end, n_lines)) != GX_OK) return e;
    if ((e = ar.alloc(lines, n_lines)) != GX_OK) return e;
    if ((e = ar.alloc(lflags, n_lines)) != GX_OK) return e;
    if ((e = ar.alloc(nvalid, n_lines)) != GX_OK) return e;
    if ((e = ar.alloc(reads, 2ull * n_lines)) != GX_OK) return e;
    launch_write_lines(text, n_text, tile_cnt, line_end, s);
    launch_parse_lines(text, n_text, line_end, n_lines, k, lines, lflags, nvalid, d_st, s);
    exclusive_scan_u32(nvalid, nvalid, n_lines, d_nlines + 1, scratch, s);
    launch_read_list(lflags, nvalid, lines, n_lines, k, reads, d_st, s);
    launch_sample_bounds(d_tb, n, line_end, n_lines, nvalid, d_nlines + 1, line_base, read_base, s);
    launch_sample_occ(lines, reads, 2 * n_lines, k, SampleMap{read_base, nullptr, n}, d_occ, s);
    CK(cudaEventRecord(tm.ev[1], s));
    DevStatus hs;
    std::vector<uint32_t> h_lb(n + 1), h_rb(n + 1);
    std::vector<unsigned long long> occ(n, 0);
    CK(d2h_async(&hs, d_st, sizeof hs, s));
    CK(d2h_async(h_lb.data(), line_base, (n + 1) * 4ull, s));
    CK(d2h_async(h_rb.data(), read_base, (n + 1) * 4ull, s));
    CK(d2h_async(occ.data(), d_occ, (size_t)n * 8, s));
    CK(sync_stream(s));
    CK(cudaGetLastError());
    if (hs.parse_err != ~0ULL) return BATCH_FALLBACK;  // every job reruns alone for its own status

    const uint32_t n_reads = h_rb[n];
    // before any count: the occurrences bound each sample's distinct k-mers (they set its super
    // buckets); the super scatter's HyperLogLog registers then set its fine buckets
    std::vector<double> d_est(n);
    for (uint32_t i = 0; i < n; i++) {
        d_est[i] = (double)occ[i];
        gx_stats &st = jobs[i]->st;
        st.lines = h_lb[i + 1] - h_lb[i];
        st.reads = h_rb[i + 1] - h_rb[i];
        st.kmers = occ[i];
    }
    unsigned long long n_occ = 0;
    for (uint32_t i = 0; i < n; i++) n_occ += occ[i];
    if (n_occ != hs.n_occ) return GX_ECUDA;
    const float ms_parse = tm.ms(0, 1);
    if (n_reads == 0) {
        for (gx_job *j : jobs) j->st.ms_parse = j->st.ms_total = ms_parse;
        return GX_OK;
    }

    double safety = 1.15;
    const double target = bucket_target(jobs[0]->eff_load_factor);  // one fill for the pass
    const uint32_t tpr = (uint32_t)jobs[0]->eff_threads_per_read;
    // The first pass scatters without a counting pass, as a single job does: every super bucket
    // gets room for 1.3 x its sample's mean plus SC_SLACK, and the scatter gathers each sample's
    // HyperLogLog registers, which then size its fine buckets.  A bucket that runs out of room
    // (a k-mer repeated very many times) makes the batch count its samples exactly and go on with
    // exact offsets.
    bool counted = false;
    std::vector<uint32_t> h_scnt, h_hll;  // the counting pass's, when it ran
    for (int attempt = 0;; attempt++) {
        std::vector<SamplePlan> plans;
        uint32_t S = 0, P = 0;
        if (!plan_batch(d_est, safety, target, plans, S, P)) return BATCH_FALLBACK;
        // super offsets: exact counts, or room per bucket
        std::vector<unsigned long long> soff(S + 1, 0);
        std::vector<uint32_t> scount(S, 0);
        std::vector<SuperInfo> sinfo(S);
        for (uint32_t i = 0; i < n; i++) {
            const SamplePlan &pl = plans[i];
            const uint32_t Si = 1u << pl.log_s, fold = MAX_SUPERS >> pl.log_s;
            const unsigned long long room =
                std::min<unsigned long long>(0xfffffff0ULL, (unsigned long long)((double)occ[i] / Si * SC_ROOM) + SC_SLACK);
            for (uint32_t q = 0; q < Si; q++) {
                unsigned long long cnt = room;
                if (counted) {
                    cnt = 0;
                    for (uint32_t t = 0; t < fold; t++) cnt += h_scnt[(size_t)i * MAX_SUPERS + q * fold + t];
                    scount[pl.super_base + q] = (uint32_t)cnt;
                }
                soff[pl.super_base + q + 1] = cnt;
            }
        }
        for (uint32_t g = 0; g < S; g++) soff[g + 1] += soff[g];
        const unsigned long long occ_room = counted ? n_occ : soff[S];

        RunArena tar(s);
        uint8_t *okey_b, *okey2_b;
        uint16_t *obits, *obits2;
        unsigned long long *d_soff, *fine_cnt, *fine_off, *head_sk, *part_bytes;
        ulonglong2 *d_chunks;
        uint32_t *s_cur, *fine_cur, *head_cnt, *head_off, *head_cur, *head_idx, *head_cnt2, *part_nodes, *noff;
        Head *heads;
        HeadOut *hout;
        SamplePlan *d_plan;
        SuperInfo *d_sinfo;
        void *pscratch;
        if ((e = tar.alloc(okey_b, occ_room * kb)) != GX_OK) return e;
        if ((e = tar.alloc(obits, occ_room)) != GX_OK) return e;
        if ((e = tar.alloc(d_soff, S + 1)) != GX_OK) return e;
        if ((e = tar.alloc(s_cur, S)) != GX_OK) return e;
        if ((e = tar.alloc(d_plan, n)) != GX_OK) return e;
        void *okey = okey_b;
        CK(cudaMemcpyAsync(d_soff, soff.data(), (S + 1) * 8ull, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(s_cur, 0, S * 4ull, s));
        const SampleMap smap{read_base, d_plan, n};
        CK(cudaEventRecord(tm.ev[2], s));
        if (!counted) {
            uint32_t *d_shll, *d_ovf;
            if ((e = tar.alloc(d_shll, (size_t)n * SC_HLL_REGS)) != GX_OK) return e;
            if ((e = tar.alloc(d_ovf, 1)) != GX_OK) return e;
            CK(cudaMemsetAsync(d_shll, 0, (size_t)n * SC_HLL_REGS * 4, s));
            CK(cudaMemsetAsync(d_ovf, 0, 4, s));
            CK(cudaMemcpyAsync(d_plan, plans.data(), n * sizeof(SamplePlan), cudaMemcpyHostToDevice, s));
            launch_scatter_super(wide, text, n_text, lines, reads, n_reads, k, smap, S, d_soff, s_cur, okey, obits,
                                 0u, d_shll, d_ovf, s, tpr);
            std::vector<uint32_t> hh((size_t)n * SC_HLL_REGS);
            uint32_t ovf = 0;
            CK(d2h_async(scount.data(), s_cur, S * 4ull, s));
            CK(d2h_async(hh.data(), d_shll, hh.size() * 4, s));
            CK(d2h_async(&ovf, d_ovf, 4, s));
            CK(sync_stream(s));
            CK(cudaGetLastError());
            if (ovf) {
                // count every sample exactly, then scatter again into exact offsets (not an attempt)
                tar.release();
                uint32_t *d_scnt, *d_hll;
                if ((e = ar.alloc(d_scnt, (size_t)n * MAX_SUPERS)) != GX_OK) return e;
                if ((e = ar.alloc(d_hll, (size_t)n * HLL_REGS)) != GX_OK) return e;
                CK(cudaMemsetAsync(d_scnt, 0, (size_t)n * MAX_SUPERS * 4, s));
                CK(cudaMemsetAsync(d_hll, 0, (size_t)n * HLL_REGS * 4, s));
                launch_count_occ_batch(wide, text, n_text, lines, reads, read_base, n, n_reads, k, d_scnt, d_hll, s);
                h_scnt.resize((size_t)n * MAX_SUPERS);
                h_hll.resize((size_t)n * HLL_REGS);
                CK(d2h_async(h_scnt.data(), d_scnt, h_scnt.size() * 4, s));
                CK(d2h_async(h_hll.data(), d_hll, h_hll.size() * 4, s));
                CK(sync_stream(s));
                CK(cudaGetLastError());
                for (uint32_t i = 0; i < n; i++)
                    d_est[i] = h_rb[i + 1] > h_rb[i] ? hll_estimate(&h_hll[(size_t)i * HLL_REGS]) : 0.0;
                counted = true;
                attempt--;
                continue;
            }
            // each sample's fine buckets from its HyperLogLog estimate (its super buckets stay)
            uint64_t fb = 0;
            for (uint32_t i = 0; i < n; i++) {
                SamplePlan &pl = plans[i];
                const double dist = h_rb[i + 1] > h_rb[i] ? hll_estimate(&hh[(size_t)i * SC_HLL_REGS], SC_HLL_REGS) : 0.0;
                const uint64_t Pi = (uint64_t)std::max(1.0, std::ceil(dist * safety / target));
                const uint64_t Si = 1ull << pl.log_s;
                pl.F = (uint32_t)std::min<uint64_t>(MAX_FINE, std::max<uint64_t>(1, (Pi + Si - 1) / Si));
                pl.fine_base = (uint32_t)fb;
                fb += Si * pl.F;
                if (fb > 0x7fffffffULL) return BATCH_FALLBACK;
            }
            P = (uint32_t)fb;
        } else {
            for (uint32_t g = 0; g < S; g++) scount[g] = (uint32_t)(soff[g + 1] - soff[g]);
        }
        for (uint32_t i = 0; i < n; i++) {
            const SamplePlan &pl = plans[i];
            for (uint32_t q = 0; q < (1u << pl.log_s); q++)
                sinfo[pl.super_base + q] = SuperInfo{pl.fine_base + q * pl.F, pl.F, pl.log_s, 0};
        }
        // CHUNK-sized pieces of every super bucket's occurrences
        std::vector<ulonglong2> chunks;
        chunks.reserve(n_occ / CHUNK + S + 1);
        unsigned long long placed = 0;
        for (uint32_t g = 0; g < S; g++) {
            placed += scount[g];
            for (unsigned long long st = 0; st < scount[g]; st += CHUNK) {
                const unsigned long long len = std::min<unsigned long long>(CHUNK, scount[g] - st);
                chunks.push_back(make_ulonglong2(soff[g] + st, ((unsigned long long)g << 32) | len));
            }
        }
        if (placed != n_occ) return GX_ECUDA;
        const uint32_t n_chunks = (uint32_t)chunks.size();
        if ((e = tar.alloc(okey2_b, n_occ * kb)) != GX_OK) return e;
        if ((e = tar.alloc(obits2, n_occ)) != GX_OK) return e;
        if ((e = tar.alloc(d_chunks, std::max<uint32_t>(n_chunks, 1))) != GX_OK) return e;
        if ((e = tar.alloc(fine_cnt, P)) != GX_OK) return e;
        if ((e = tar.alloc(fine_off, P + 1)) != GX_OK) return e;
        if ((e = tar.alloc(fine_cur, P)) != GX_OK) return e;
        if ((e = tar.alloc(heads, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(hout, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(noff, n_occ)) != GX_OK) return e;
        if ((e = tar.alloc(head_cnt, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_off, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_cur, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_idx, n_reads)) != GX_OK) return e;
        HeadIn *hsorted;
        if ((e = tar.alloc(hsorted, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(head_cnt2, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_sk, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(part_nodes, P)) != GX_OK) return e;
        if ((e = tar.alloc(part_bytes, P)) != GX_OK) return e;
        if ((e = tar.alloc(pscratch, scan_scratch_bytes(P + 1, 8))) != GX_OK) return e;
        if ((e = tar.alloc(d_sinfo, S)) != GX_OK) return e;
        unsigned long long *part_off = nullptr;
        if ((e = tar.alloc(part_off, P + 1)) != GX_OK) return e;
        void *okey2 = okey2_b;
        CK(cudaMemcpyAsync(d_plan, plans.data(), n * sizeof(SamplePlan), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_sinfo, sinfo.data(), S * sizeof(SuperInfo), cudaMemcpyHostToDevice, s));
        if (n_chunks)
            CK(cudaMemcpyAsync(d_chunks, chunks.data(), n_chunks * sizeof(ulonglong2), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(fine_cnt, 0, P * 8ull, s));
        CK(cudaMemsetAsync(fine_cur, 0, P * 4ull, s));
        CK(cudaMemsetAsync(head_cnt, 0, P * 4ull, s));
        CK(cudaMemsetAsync(head_cur, 0, P * 4ull, s));
        if (counted)
            launch_scatter_super(wide, text, n_text, lines, reads, n_reads, k, smap, S, d_soff, s_cur, okey, obits,
                                 0xffffffffu, nullptr, nullptr, s, tpr);
        launch_heads_part(wide, text, n_text, lines, reads, n_reads, k, smap, heads, head_cnt, s);
        exclusive_scan_u32(head_cnt, head_off, P, nullptr, pscratch, s);
        launch_head_scatter_part(heads, reads, lines, n_reads, head_off, head_cur, head_idx, hsorted, s);
        launch_fine_count(wide, okey, d_chunks, n_chunks, d_sinfo, fine_cnt, s);
        exclusive_scan_u64(fine_cnt, fine_off, P, fine_off + P, pscratch, s);
        launch_scatter_fine(wide, okey, obits, d_chunks, n_chunks, d_sinfo, fine_off, fine_cur, okey2, obits2, s);
        CK(cudaEventRecord(tm.ev[3], s));
        AggArgs g{};
        g.wide = wide;
        g.k = k;
        g.pp = PartPlan{0, 0, P};
        g.okey2 = okey2;
        g.obits2 = obits2;
        g.fine_off = fine_off;
        g.lines = lines;
        g.reads = reads;
        g.heads = heads;
        g.head_idx = head_idx;
        g.hsorted = hsorted;
        g.head_sk = head_sk;
        g.head_off = head_off;
        g.head_cnt = head_cnt;
        g.head_cnt2 = head_cnt2;
        g.nkey = okey2;
        g.ncm = (unsigned long long *)okey;
        g.noff = noff;
        g.hout = hout;
        g.part_nodes = part_nodes;
        g.part_bytes = part_bytes;
        g.st = d_st;
        launch_aggregate(g, s);
        exclusive_scan_u64(part_bytes, part_off, P, part_off + P, pscratch, s);
        CK(cudaEventRecord(tm.ev[4], s));
        unsigned long long total = 0;
        CK(d2h_async(&hs, d_st, sizeof hs, s));
        CK(d2h_async(&total, part_off + P, 8, s));
        CK(sync_stream(s));
        CK(cudaGetLastError());
        if (hs.internal_err) {
            fprintf(stderr, "gxgpu: internal error: a read head's k-mer was not aggregated\n");
            return GX_ECUDA;
        }
        if (hs.table_full) {
            DevStatus zero{};
            zero.parse_err = ~0ULL;
            CK(cudaMemcpyAsync(d_st, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
            if (attempt >= 3) return BATCH_FALLBACK;
            safety *= 2;
            continue;
        }
        // ---- records of every sample into one buffer ----
        void *outp = nullptr;
        CK(cudaMallocAsync(&outp, total + 16, s));
        // freed with the last job that refers to it, by then all its uses on the device are done
        // (every pass and every emit synchronizes), so any stream may order the free
        std::shared_ptr<void> owner(outp, [](void *p) { cudaFreeAsync(p, 0); });
        if (((uintptr_t)outp & 15) != 0) return GX_ECUDA;
        EmitArgs a{};
        a.g = TableGeom{nullptr, P, wide};
        a.k = k;
        a.text = text;
        a.n_text = n_text;
        a.lines = lines;
        a.reads = reads;
        a.heads = heads;
        a.head_idx = head_idx;
        a.head_sk = head_sk;
        a.head_off = head_off;
        a.head_cnt = head_cnt;
        a.head_cnt2 = head_cnt2;
        a.part_nodes = part_nodes;
        a.part_bytes = part_bytes;
        a.part_off = part_off;
        a.out = (uint8_t *)outp;
        a.st = d_st;
        a.nkey = okey2;
        a.ncm = (const unsigned long long *)okey;
        a.node_base = fine_off;
        a.noff = noff;
        a.hout = hout;
        a.n_head_slots = n_reads;
        a.max_seq = hs.max_seq;
        CK(cudaEventRecord(tm.ev[5], s));
        launch_emit_write_part(a, s);
        CK(cudaEventRecord(tm.ev[6], s));
        std::vector<unsigned long long> h_po(P + 1);
        std::vector<uint32_t> h_pn(P), h_hc(P);
        CK(d2h_async(&hs, d_st, sizeof hs, s));
        CK(d2h_async(h_po.data(), part_off, (P + 1) * 8ull, s));
        CK(d2h_async(h_pn.data(), part_nodes, P * 4ull, s));
        CK(d2h_async(h_hc.data(), head_cnt2, P * 4ull, s));
        CK(sync_stream(s));
        CK(cudaGetLastError());
        if (hs.internal_err) {
            fprintf(stderr, "gxgpu: internal error: record sizes disagree between emission passes\n");
            return GX_ECUDA;
        }
        const uint64_t launches = launches_this_thread() - l0;
        for (uint32_t i = 0; i < n; i++) {
            gx_job *j = jobs[i];
            const SamplePlan &pl = plans[i];
            const uint32_t Pi = (1u << pl.log_s) * pl.F, fb = pl.fine_base;
            const unsigned long long base = h_po[fb];
            j->out_owner = owner;
            j->d_out = (uint8_t *)outp + base;
            j->out_bytes = h_po[fb + Pi] - base;
            j->d_part_off = nullptr;
            j->nparts = Pi;
            j->h_part_off.resize(Pi + 1);
            for (uint32_t t = 0; t <= Pi; t++) j->h_part_off[t] = h_po[fb + t] - base;
            const int OP = j->o.out_parts;
            for (int q = 0; q < OP; q++) j->part_bounds[q] = j->h_part_off[(uint64_t)Pi * q / OP];
            j->part_bounds[OP] = j->out_bytes;
            for (int q = 0; q < OP; q++) j->cursor[q] = j->part_bounds[q];
            uint64_t nn = 0, nh = 0;
            for (uint32_t t = 0; t < Pi; t++) {
                nn += h_pn[fb + t];
                nh += h_hc[fb + t];
            }
            gx_stats &st = j->st;
            st.nodes = nn;
            st.read_heads = nh;
            st.record_bytes = j->out_bytes;
            st.table_partitions = Pi;
            st.attempts = (uint64_t)attempt + 1;
            st.table_slots = (uint64_t)Pi * AGG_SLOTS;
            st.super_counted = counted ? 1 : 0;  // batch-wide
            st.cov_inexact_nodes = hs.cov_inexact;  // batch-wide
            st.kernel_launches = launches;         // the whole batch's launches
            st.ms_parse = ms_parse;
            st.ms_insert = tm.ms(2, 3);
            st.ms_emit = tm.ms(3, 4) + tm.ms(5, 6);
            st.ms_aggregate = tm.ms(3, 4);
            st.ms_write = tm.ms(5, 6);
            st.ms_total = tm.ms(0, 6);
        }
        return GX_OK;
    }
}

// Runs a group; splits it when it does not fit, and falls back to single jobs when the
// batch cannot report per-job results.
void run_group_or_split(gx_ctx *c, const std::vector<gx_job *> &jobs, std::map<gx_job *, gx_status> &result) {
    gx_status st = run_group(c, jobs);
    if (st == GX_OK) {
        for (gx_job *j : jobs) result[j] = GX_OK;
        return;
    }
    cudaGetLastError();
    if (st == GX_ENOMEM && jobs.size() > 1) {
        const size_t h = jobs.size() / 2;
        run_group_or_split(c, std::vector<gx_job *>(jobs.begin(), jobs.begin() + h), result);
        run_group_or_split(c, std::vector<gx_job *>(jobs.begin() + h, jobs.end()), result);
        return;
    }
    for (gx_job *j : jobs) {
        j->out_owner.reset();
        j->d_out = nullptr;
        result[j] = run_job_locked(j);
    }
}

}  // namespace

static gx_status batch_run(gx_ctx *c, gx_job **jobs, int n, gx_status *statuses);

extern "C" gx_status gx_batch_run(gx_ctx *c, gx_job **jobs, int n, gx_status *statuses) {
    return guarded("gx_batch_run", [&] { return batch_run(c, jobs, n, statuses); });
}

static gx_status batch_run(gx_ctx *c, gx_job **jobs, int n, gx_status *statuses) {
    if (!c || (!jobs && n) || n < 0) return GX_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    cudaSetDevice(c->device);
    const AllocLimitScope als(c->test_alloc_fail_above);
    std::map<gx_job *, gx_status> result;
    std::map<long long, std::vector<gx_job *>> by_k;
    for (int i = 0; i < n; i++) {
        gx_job *j = jobs[i];
        if (!j || j->ctx != c) continue;
        if (j->state != JS_INPUT || result.count(j)) {
            result[j] = GX_ESTATE;
            continue;
        }
        resolve_options(j);
        if (j->eff_algorithm == GX_ALGO_TABLE || j->o.plan != GX_PLAN_BUILD_DEBRUIJN_GRAPH ||
            j->o.layout != GX_LAYOUT_BUCKETS) {
            result[j] = run_job_locked(j);
            continue;
        }
        const gx_status pe = prepare_text(j);
        if (pe != GX_OK) {
            j->state = JS_FAILED;
            result[j] = pe;
            continue;
        }
        // one pass per k, fill and tiling
        by_k[((long long)j->k * 4096 + (int)(j->eff_load_factor * 1000)) * 64 + j->eff_threads_per_read].push_back(j);
        result[j] = GX_OK;  // placeholder until its group runs
    }
    for (auto &kv : by_k) {
        const std::vector<gx_job *> &g = kv.second;
        for (size_t a = 0; a < g.size(); a += MAX_BATCH) {
            std::vector<gx_job *> part(g.begin() + a, g.begin() + std::min(g.size(), a + MAX_BATCH));
            run_group_or_split(c, part, result);
            for (gx_job *j : part) {
                if (j->state == JS_INPUT) j->state = result[j] == GX_OK ? JS_RAN : JS_FAILED;
                if (j->text_borrowed) {
                    j->d_text = nullptr;
                    j->text_borrowed = false;
                }
            }
        }
    }
    gx_status first = GX_OK;
    for (int i = 0; i < n; i++) {
        gx_status st = GX_EINVAL;
        if (jobs[i] && jobs[i]->ctx == c) st = result.count(jobs[i]) ? result[jobs[i]] : GX_EINVAL;
        if (statuses) statuses[i] = st;
        if (st != GX_OK && first == GX_OK) first = st;
    }
    return first;
}
