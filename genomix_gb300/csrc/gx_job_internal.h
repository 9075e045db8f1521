// gx_job_internal.h — contexts, jobs and run-scoped device memory, shared by the plain build
// (gx_job.cu) and the batched and served builds (gx_batch.cu, gx_serve.cu).
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <exception>
#include <functional>
#include <memory>
#include <new>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gxgpu.h"
#include "gx_kernels.cuh"

namespace gxi {

enum JobState { JS_INPUT = 0, JS_RAN = 1, JS_FAILED = 2 };

struct Timers {
    cudaEvent_t ev[10] = {};
    bool ok = false;
    void init() {
        for (auto &e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) return;
        ok = true;
    }
    void destroy() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
    float ms(int a, int b) const {
        float t = 0;
        if (ok) cudaEventElapsedTime(&t, ev[a], ev[b]);
        return t;
    }
};

}  // namespace gxi

struct gx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // gx_job_emit_async copies: they overlap the next build
    std::mutex mu;
    size_t mem_limit = 0;
    size_t test_alloc_fail_above = 0;  // testing: run allocations above this fail as out of memory
    int test_flags = 0;                // testing: GX_CTX_TEST_* (gx_ctx_opts.flags)
    cudaEvent_t marks[16] = {};
    // the handle holds one reference and every job one more: a context destroyed while jobs
    // still live is freed with the last of them
    std::atomic<int> refs{1};
    // gx_autotune's choice per key width (64- / 128-bit), used by jobs left at the defaults
    struct Tuned {
        bool valid = false;
        int algorithm = GX_ALGO_PARTITIONED;
        double load_factor = 0;
        int threads_per_read = 1;
    } tuned[2];
};

struct gx_job {
    gx_ctx *ctx = nullptr;
    gx_job_opts o{};
    int k = 0;
    int wide = 0;
    gxi::JobState state = gxi::JS_INPUT;
    // readid input on the device
    uint8_t *d_text = nullptr;
    size_t text_len = 0, text_cap = 0;
    bool text_borrowed = false;
    int n_device_inputs = 0;
    // FASTQ inputs kept on the host until run (mate stream 0 / 1, one entry per file)
    std::vector<std::string> fastq[2];
    // results
    uint8_t *d_out = nullptr;
    size_t out_bytes = 0;
    uint32_t nparts = 0;
    unsigned long long *d_part_off = nullptr;  // table-partition byte offsets (nparts + 1)
    std::vector<uint64_t> part_bounds;         // output-part byte offsets (out_parts + 1)
    std::vector<uint64_t> cursor;              // emit cursor per output part
    std::vector<unsigned long long> h_part_off;  // lazily fetched copy of d_part_off
    gx_stats st{};
    gxi::Timers tm;
    cudaEvent_t ev_copy = nullptr;  // the last asynchronous emit's copy
    bool copy_pending = false;
    // the algorithm and fill this run uses: the job's options, or the context's tuned choice
    int eff_algorithm = GX_ALGO_PARTITIONED;
    double eff_load_factor = 0;
    int eff_threads_per_read = 1;
    // a batched run writes every sample's records into one buffer: the jobs share ownership
    std::shared_ptr<void> out_owner;
};

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            fprintf(stderr, "gxgpu: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                                      \
            return e_ == cudaErrorMemoryAllocation ? GX_ENOMEM : GX_ECUDA;                          \
        }                                                                                           \
    } while (0)

namespace gxi {

// Set while a run executes on a context with gx_ctx_opts.test_alloc_fail_above (testing): run
// allocations above it fail as if the device were out of memory.
extern thread_local size_t t_alloc_fail_above;
struct AllocLimitScope {
    size_t saved;
    explicit AllocLimitScope(size_t v) : saved(t_alloc_fail_above) { t_alloc_fail_above = v; }
    ~AllocLimitScope() { t_alloc_fail_above = saved; }
};

// Allocations of one run, released together (stream ordered).
struct RunArena {
    cudaStream_t s;
    std::vector<void *> ptrs;
    explicit RunArena(cudaStream_t st) : s(st) {}
    template <class T>
    gx_status alloc(T *&p, size_t count) {
        void *q = nullptr;
        const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
        if (t_alloc_fail_above && bytes > t_alloc_fail_above) return GX_ENOMEM;
        cudaError_t e = cudaMallocAsync(&q, bytes, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return GX_ENOMEM;
        }
        ptrs.push_back(q);
        p = (T *)q;
        return GX_OK;
    }
    void release() {
        for (void *p : ptrs) cudaFreeAsync(p, s);
        ptrs.clear();
    }
    ~RunArena() { release(); }
};

// No C++ exception may cross the C ABI: a host allocation failure becomes GX_ENOMEM,
// anything else GX_ECUDA, with the reason on stderr.
template <class F>
gx_status guarded(const char *where, F &&f) {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        fprintf(stderr, "gxgpu: %s: out of host memory\n", where);
        return GX_ENOMEM;
    } catch (const std::exception &e) {
        fprintf(stderr, "gxgpu: %s: %s\n", where, e.what());
        return GX_ECUDA;
    } catch (...) {
        fprintf(stderr, "gxgpu: %s: unexpected exception\n", where);
        return GX_ECUDA;
    }
}

// The algorithm, fill and threads per read a job runs with: its own options where set, else the
// context's tuned choice for its key width, else the built-in defaults.
void resolve_options(gx_job *j);
// Fine-bucket fill aimed for by the partitioned build (distinct k-mers per 2048-slot table).
double bucket_target(double load_factor);

// Drops one reference to a context; the last one frees it.
void ctx_release(gx_ctx *c);

// Runs one job; the caller holds the context's lock and has made its device current.
gx_status run_job_locked(gx_job *j);
// FASTQ inputs converted to readid text on the device (the reference driver's pre-pass).
gx_status prepare_text(gx_job *j);
// One FASTQ file (pair) to readid text on the device: `dest(total)` gives the device buffer
// for the total bytes (null: out of memory).
gx_status fastq_to_readid_device(cudaStream_t s, const uint8_t *h1, size_t n1, const uint8_t *h2, size_t n2,
                                 const std::function<uint8_t *(uint64_t)> &dest, uint64_t &written);

}  // namespace gxi
