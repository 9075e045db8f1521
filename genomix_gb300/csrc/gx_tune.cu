// gx_tune.cu — the autotuner (gx_autotune).
//
// Times each candidate (aggregation algorithm x table fill x threads per read) on a sample of
// the caller's reads and keeps the fastest in the context, per key width: jobs created with
// the default algorithm, load factor and tiling then run with it (plain, batched and served
// alike).  The best fill (the partitioned build's bucket width: distinct k-mers per bucket
// table) depends on the data: more per bucket means fewer buckets and less per-bucket work, up
// to the point where probing and overflow retries cost more.  The tiling splits each read's
// k-mer walk over 1, 2 or 4 threads: shorter walks per thread and a smaller text footprint per
// CTA, against one extra k-mer window per segment.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/gxgpu.h"
#include "gx_job_internal.h"

using namespace gxi;

namespace {

struct Candidate {
    int algorithm;
    double load_factor;
    int threads_per_read;
};

const Candidate kCandidates[] = {
    {GX_ALGO_PARTITIONED, 0.35, 1},   {GX_ALGO_PARTITIONED, 0.4375, 1}, {GX_ALGO_PARTITIONED, 0.50, 1},
    {GX_ALGO_PARTITIONED, 0.60, 1},   {GX_ALGO_PARTITIONED, 0.35, 2},   {GX_ALGO_PARTITIONED, 0.4375, 2},
    {GX_ALGO_PARTITIONED, 0.50, 2},   {GX_ALGO_PARTITIONED, 0.60, 2},   {GX_ALGO_PARTITIONED, 0.35, 4},
    {GX_ALGO_PARTITIONED, 0.4375, 4}, {GX_ALGO_PARTITIONED, 0.50, 4},   {GX_ALGO_PARTITIONED, 0.60, 4},
    {GX_ALGO_TABLE, 0.35, 1},         {GX_ALGO_TABLE, 0.50, 1},         {GX_ALGO_TABLE, 0.70, 1},
};
static_assert(sizeof kCandidates / sizeof kCandidates[0] <= GX_TUNE_MAX, "gx_tune_result holds every candidate");

// device time of one build of the sample with the given settings (< 0: the build failed)
double time_one(gx_ctx *c, const void *d_text, size_t bytes, int k, const Candidate &cd, gx_status &st) {
    gx_job_opts o{};
    o.struct_size = sizeof o;
    o.kmer_length = k;
    o.input_kind = GX_INPUT_READID;
    o.out_parts = 1;
    o.algorithm = cd.algorithm;
    o.load_factor = cd.load_factor;
    o.threads_per_read = cd.threads_per_read;
    gx_job *j = nullptr;
    if ((st = gx_job_create(c, &o, &j)) != GX_OK) return -1;
    double ms = -1;
    if ((st = gx_job_add_input_device(j, d_text, bytes, 0)) == GX_OK && (st = gx_job_run(j)) == GX_OK) {
        gx_stats s;
        gx_job_stats(j, &s);
        ms = s.ms_total;
    }
    gx_job_destroy(j);
    return ms;
}

}  // namespace

extern "C" gx_status gx_autotune(gx_ctx *c, const void *sample, size_t bytes, int k, int repeats,
                                 gx_tune_result *out) {
    return guarded("gx_autotune", [&]() -> gx_status {
        if (!c || !sample || !bytes || !out || k < 3 || k > 64) return GX_EINVAL;
        if (out->struct_size < sizeof(gx_tune_result)) return GX_EINVAL;
        const size_t ss = out->struct_size;
        *out = gx_tune_result{};
        out->struct_size = ss;
        if (repeats < 1) repeats = 2;
        void *d_text = nullptr;
        {
            std::lock_guard<std::mutex> lk(c->mu);
            cudaSetDevice(c->device);
            if (cudaMallocAsync(&d_text, bytes, c->stream) != cudaSuccess) {
                cudaGetLastError();
                return GX_ENOMEM;
            }
            if (cudaMemcpyAsync(d_text, sample, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess) {
                cudaFreeAsync(d_text, c->stream);
                return GX_ECUDA;
            }
        }
        const int n = (int)(sizeof kCandidates / sizeof kCandidates[0]);
        int best = -1;
        gx_status first_err = GX_OK;
        for (int i = 0; i < n && i < GX_TUNE_MAX; i++) {
            double t = -1;
            for (int r = 0; r < repeats; r++) {
                gx_status st = GX_OK;
                const double ms = time_one(c, d_text, bytes, k, kCandidates[i], st);
                if (ms < 0) {
                    if (first_err == GX_OK) first_err = st;
                    t = -1;
                    break;
                }
                t = t < 0 ? ms : std::min(t, ms);
            }
            out->cand[i].algorithm = kCandidates[i].algorithm;
            out->cand[i].load_factor = kCandidates[i].load_factor;
            out->cand[i].threads_per_read = kCandidates[i].threads_per_read;
            out->cand[i].ms = t;
            out->tried++;
            if (t >= 0 && (best < 0 || t < out->cand[best].ms)) best = i;
        }
        {
            std::lock_guard<std::mutex> lk(c->mu);
            cudaSetDevice(c->device);
            cudaFreeAsync(d_text, c->stream);
            cudaStreamSynchronize(c->stream);
        }
        if (best < 0) return first_err != GX_OK ? first_err : GX_ECUDA;
        out->algorithm = kCandidates[best].algorithm;
        out->load_factor = kCandidates[best].load_factor;
        out->threads_per_read = kCandidates[best].threads_per_read;
        out->ms = out->cand[best].ms;
        std::lock_guard<std::mutex> lk(c->mu);
        gx_ctx::Tuned &tu = c->tuned[k > 32 ? 1 : 0];
        tu.valid = true;
        tu.algorithm = out->algorithm;
        tu.load_factor = out->load_factor;
        tu.threads_per_read = out->threads_per_read;
        return GX_OK;
    });
}

extern "C" gx_status gx_autotune_clear(gx_ctx *c) {
    if (!c) return GX_EINVAL;
    std::lock_guard<std::mutex> lk(c->mu);
    c->tuned[0] = gx_ctx::Tuned{};
    c->tuned[1] = gx_ctx::Tuned{};
    return GX_OK;
}
