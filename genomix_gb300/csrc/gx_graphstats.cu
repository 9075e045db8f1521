// gx_graphstats.cu — graph statistics over a job's device-resident records
// (gx_job_graph_stats).
//
// The counters GraphStatistics.map (genomix-hadoop/.../utils/GraphStatistics.java:78-131)
// collects per node, for the nodes of a graph build (kmer length k, no internal k-mer):
//   degree = inDegree + outDegree (REVERSE = RF + RR edges, FORWARD = FF + FR), kmerLength,
//   coverage = Math.round(averageCoverage), unflipped / flipped read-id counts, and the
//   scaffold seed score k * (unflipped + flipped) for coverage within 0 +- 1000; per direction
//   with edges, the same three again; tips per direction, tips-BOTH / tips-ONE, path nodes,
//   self edges per edge type.  Every statistic keeps its total, maximum and a histogram
//   ("<name>-bins"), the coverage histogram being what the coverage-cutoff fit reads
//   (GraphStatistics.getCoverageStats, :168-185).
//
// One thread walks one table partition's records (each partition starts on a record
// boundary); histograms of small values live in shared memory per block.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gxgpu.h"
#include "gx_job_internal.h"

using namespace gx;
using namespace gxi;

namespace {

enum {
    S_DEGREE, S_KLEN, S_COVERAGE, S_UNFLIPPED, S_FLIPPED, S_SEED,
    S_KLEN_R, S_COV_R, S_SEED_R, S_KLEN_F, S_COV_F, S_SEED_F, N_STATS
};
enum { C_NODES, C_PATH, C_TIPS_R, C_TIPS_F, C_TIPS_BOTH, C_TIPS_ONE, C_SELF0, N_COUNTERS = C_SELF0 + 4 };
constexpr int SMEM_BINS = 256;  // values below this are binned in shared memory first

struct DevGraphStats {
    unsigned long long counters[N_COUNTERS];
    unsigned long long total[N_STATS], maximum[N_STATS], above[N_STATS];
    unsigned long long bins[N_STATS][GX_STAT_BINS];
};

__device__ __forceinline__ uint32_t rd_be32(const uint8_t *p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

struct StatAcc {
    uint32_t *sbins;  // [N_STATS][SMEM_BINS] in shared memory
    DevGraphStats *g;
    unsigned long long total[N_STATS];
    unsigned long long maximum[N_STATS];
    __device__ void add(int s, unsigned long long v) {
        total[s] += v;
        maximum[s] = v > maximum[s] ? v : maximum[s];
        if (v < SMEM_BINS)
            atomicAdd(&sbins[s * SMEM_BINS + (uint32_t)v], 1u);
        else if (v < GX_STAT_BINS)
            atomicAdd(&g->bins[s][v], 1ULL);
        else
            atomicAdd(&g->above[s], 1ULL);
    }
};

__global__ void __launch_bounds__(256) k_graph_stats(const uint8_t *rec, const unsigned long long *seg,
                                                     uint32_t n_seg, int k, DevGraphStats *g) {
    __shared__ uint32_t sbins[N_STATS * SMEM_BINS];
    __shared__ unsigned long long scnt[N_COUNTERS];
    for (uint32_t i = threadIdx.x; i < N_STATS * SMEM_BINS; i += blockDim.x) sbins[i] = 0;
    if (threadIdx.x < N_COUNTERS) scnt[threadIdx.x] = 0;
    __syncthreads();
    StatAcc acc;
    acc.sbins = sbins;
    acc.g = g;
    for (int s = 0; s < N_STATS; s++) acc.total[s] = acc.maximum[s] = 0;
    unsigned long long cnt[N_COUNTERS];
    for (int c = 0; c < N_COUNTERS; c++) cnt[c] = 0;
    const int nb = (k + 3) / 4;
    for (uint32_t sg = blockIdx.x * blockDim.x + threadIdx.x; sg < n_seg; sg += gridDim.x * blockDim.x) {
        unsigned long long p = seg[sg];
        const unsigned long long e = seg[sg + 1];
        while (p < e) {
            const uint8_t *r = rec + p;
            const uint32_t rl = rd_be32(r), kl = rd_be32(r + 4);
            const uint8_t *key = r + 12;  // after the VKmer's own k
            const uint8_t *q = r + 8 + kl;
            const uint32_t active = *q++;
            uint32_t deg[4] = {0, 0, 0, 0};
            for (int t = 0; t < 4; t++) {
                if (!(active & (1u << t))) continue;
                const uint32_t n = rd_be32(q);
                q += 4;
                deg[t] = n;
                for (uint32_t i = 0; i < n; i++) {
                    bool same = true;
                    for (int b = 0; b < nb; b++) same &= q[4 + b] == key[b];
                    if (same) cnt[C_SELF0 + t]++;
                    q += 4 + nb;
                }
            }
            uint32_t heads[2] = {0, 0};
            for (int set = 0; set < 2; set++) {
                if (!(active & (0x10u << set))) continue;
                q++;  // ExternalableTreeSet: whole body in stream
                const uint32_t n = rd_be32(q);
                q += 4;
                heads[set] = n;
                for (uint32_t i = 0; i < n; i++) {
                    const uint32_t flags = *q;
                    q += 9;  // flags + uuid
                    for (int m = 0; m < ((flags & 1u) ? 2 : 1); m++) {
                        const uint32_t L = rd_be32(q);
                        q += 4 + (L + 3) / 4;
                    }
                }
            }
            const float cov = __uint_as_float(rd_be32(r + 8 + rl - 4));
            const unsigned long long covr = (unsigned long long)floorf(cov + 0.5f);  // Math.round(float)
            const uint32_t out_deg = deg[0] + deg[1], in_deg = deg[2] + deg[3];
            const unsigned long long seed = (unsigned long long)k * (heads[0] + heads[1]);
            const bool seeded = cov >= -1000.0f && cov <= 1000.0f;
            cnt[C_NODES]++;
            acc.add(S_DEGREE, in_deg + out_deg);
            acc.add(S_KLEN, (unsigned long long)k);
            acc.add(S_COVERAGE, covr);
            acc.add(S_UNFLIPPED, heads[0]);
            acc.add(S_FLIPPED, heads[1]);
            if (seeded) acc.add(S_SEED, seed);
            if (in_deg == 1 && out_deg == 1) cnt[C_PATH]++;
            // DIR.values(): REVERSE, then FORWARD
            if (in_deg == 0) {
                cnt[C_TIPS_R]++;
            } else {
                acc.add(S_KLEN_R, (unsigned long long)k);
                acc.add(S_COV_R, covr);
                if (seeded) acc.add(S_SEED_R, seed);
            }
            if (out_deg == 0) {
                cnt[C_TIPS_F]++;
            } else {
                acc.add(S_KLEN_F, (unsigned long long)k);
                acc.add(S_COV_F, covr);
                if (seeded) acc.add(S_SEED_F, seed);
            }
            if (in_deg == 0 && out_deg == 0) cnt[C_TIPS_BOTH]++;
            if ((in_deg == 0) != (out_deg == 0)) cnt[C_TIPS_ONE]++;
            p += 8ULL + rl;
        }
    }
    for (int c = 0; c < N_COUNTERS; c++)
        if (cnt[c]) atomicAdd(&scnt[c], cnt[c]);
    for (int s = 0; s < N_STATS; s++) {
        if (acc.total[s]) atomicAdd(&g->total[s], acc.total[s]);
        if (acc.maximum[s]) atomicMax(&g->maximum[s], acc.maximum[s]);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < N_STATS * SMEM_BINS; i += blockDim.x)
        if (sbins[i]) atomicAdd(&g->bins[i / SMEM_BINS][i % SMEM_BINS], (unsigned long long)sbins[i]);
    if (threadIdx.x < N_COUNTERS && scnt[threadIdx.x]) atomicAdd(&g->counters[threadIdx.x], scnt[threadIdx.x]);
}

void copy_hist(gx_stat_hist &h, const DevGraphStats &d, int s) {
    h.total = d.total[s];
    h.maximum = d.maximum[s];
    h.above = d.above[s];
    memcpy(h.bins, d.bins[s], sizeof h.bins);
}

gx_status graph_stats(gx_job *j, gx_graph_stats *out) {
    if (!j || !out || out->struct_size < sizeof(gx_graph_stats)) return GX_EINVAL;
    if (j->state != JS_RAN) return GX_ESTATE;
    if (j->o.plan != GX_PLAN_BUILD_DEBRUIJN_GRAPH) return GX_EINVAL;  // per-occurrence records are no graph
    std::lock_guard<std::mutex> lk(j->ctx->mu);
    cudaSetDevice(j->ctx->device);
    cudaStream_t s = j->ctx->stream;
    const size_t ss = out->struct_size;
    memset(out, 0, sizeof *out);
    out->struct_size = ss;
    if (!j->out_bytes) return GX_OK;
    // record segments: the table partitions (each starts on a record boundary)
    std::vector<unsigned long long> segs;
    if (!j->h_part_off.empty()) {
        segs.assign(j->h_part_off.begin(), j->h_part_off.end());
    } else {
        segs.resize(j->nparts + 1);
        CK(cudaMemcpyAsync(segs.data(), j->d_part_off, (j->nparts + 1) * 8ull, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    RunArena ar(s);
    unsigned long long *d_seg;
    DevGraphStats *d_gs;
    gx_status e;
    if ((e = ar.alloc(d_seg, segs.size())) != GX_OK) return e;
    if ((e = ar.alloc(d_gs, 1)) != GX_OK) return e;
    CK(cudaMemcpyAsync(d_seg, segs.data(), segs.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d_gs, 0, sizeof(DevGraphStats), s));
    const uint32_t n_seg = (uint32_t)(segs.size() - 1);
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n_seg + 255) / 256, 152ull * 8));
    k_graph_stats<<<blocks, 256, 0, s>>>(j->d_out, d_seg, n_seg, j->k, d_gs);
    std::vector<DevGraphStats> h(1);
    CK(cudaMemcpyAsync(h.data(), d_gs, sizeof(DevGraphStats), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    const DevGraphStats &d = h[0];
    out->nodes = d.counters[C_NODES];
    out->path_nodes = d.counters[C_PATH];
    out->tips_reverse = d.counters[C_TIPS_R];
    out->tips_forward = d.counters[C_TIPS_F];
    out->tips_both = d.counters[C_TIPS_BOTH];
    out->tips_one = d.counters[C_TIPS_ONE];
    for (int t = 0; t < 4; t++) out->self_edges[t] = d.counters[C_SELF0 + t];
    copy_hist(out->degree, d, S_DEGREE);
    copy_hist(out->kmer_length, d, S_KLEN);
    copy_hist(out->coverage, d, S_COVERAGE);
    copy_hist(out->unflipped_read_ids, d, S_UNFLIPPED);
    copy_hist(out->flipped_read_ids, d, S_FLIPPED);
    copy_hist(out->seed_score, d, S_SEED);
    copy_hist(out->kmer_length_with[0], d, S_KLEN_R);
    copy_hist(out->coverage_with[0], d, S_COV_R);
    copy_hist(out->seed_score_with[0], d, S_SEED_R);
    copy_hist(out->kmer_length_with[1], d, S_KLEN_F);
    copy_hist(out->coverage_with[1], d, S_COV_F);
    copy_hist(out->seed_score_with[1], d, S_SEED_F);
    return GX_OK;
}

}  // namespace

extern "C" gx_status gx_job_graph_stats(gx_job *j, gx_graph_stats *out) {
    return guarded("gx_job_graph_stats", [&] { return graph_stats(j, out); });
}
