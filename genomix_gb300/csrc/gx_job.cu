// gx_job.cu — contexts, jobs and the plain (one job per launch sequence) graph build.
//
// Run sequence of gx_job_run, all on the context's stream:
//   K1   count + write line ends, parse lines, list valid mates     (host sync: line count,
//        then errors + occurrence count, which sizes the table)
//   K2/3 k-mer extraction and table inserts, one thread per read
//   K4   read heads bucketed per table partition
//   K5a  per-partition compaction, sort and sizing                  (host sync: output bytes)
//   K5b  per-partition serialization
// Device memory comes from the device's stream-ordered pool, kept warm between jobs.
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/gxgpu.h"
#include "gx_host.h"
#include "gx_job_internal.h"
#include "gx_kernels.cuh"

using namespace gx;

using namespace gxi;

static gx_status ensure_text_cap(gx_job *j, size_t need) {
    if (j->text_borrowed) {
        // switch a borrowed single input to an owned buffer before appending
        uint8_t *old = j->d_text;
        size_t cap = std::max<size_t>(need + 64, j->text_len * 2);
        void *q = nullptr;
        CK(cudaMallocAsync(&q, cap, j->ctx->stream));
        CK(cudaMemcpyAsync(q, old, j->text_len, cudaMemcpyDeviceToDevice, j->ctx->stream));
        j->d_text = (uint8_t *)q;
        j->text_cap = cap;
        j->text_borrowed = false;
        return GX_OK;
    }
    if (need <= j->text_cap) return GX_OK;
    size_t cap = std::max<size_t>(need + 64, j->text_cap * 2);
    if (j->o.est_input_bytes > cap) cap = j->o.est_input_bytes + 64;
    void *q = nullptr;
    CK(cudaMallocAsync(&q, cap, j->ctx->stream));
    if (j->d_text) {
        CK(cudaMemcpyAsync(q, j->d_text, j->text_len, cudaMemcpyDeviceToDevice, j->ctx->stream));
        cudaFreeAsync(j->d_text, j->ctx->stream);
    }
    j->d_text = (uint8_t *)q;
    j->text_cap = cap;
    return GX_OK;
}

// Appends one readid "file"; a file that does not end in '\n' gets one, so lines never
// join across files ("...\r" + "\n" is a single CRLF terminator).
static gx_status append_text(gx_job *j, const void *src, size_t bytes, cudaMemcpyKind kind, bool src_ends_nl) {
    if (!bytes) return GX_OK;
    const size_t add = bytes + (src_ends_nl ? 0 : 1);
    gx_status st = ensure_text_cap(j, j->text_len + add);
    if (st != GX_OK) return st;
    CK(cudaMemcpyAsync(j->d_text + j->text_len, src, bytes, kind, j->ctx->stream));
    if (!src_ends_nl) CK(cudaMemsetAsync(j->d_text + j->text_len + bytes, '\n', 1, j->ctx->stream));
    j->text_len += add;
    return GX_OK;
}

extern "C" {

gx_status gx_fastq_to_readid_gpu(gx_ctx *c, const void *mate1, size_t bytes1, const void *mate2, size_t bytes2,
                                 char **out, size_t *out_bytes) {
    return guarded("gx_fastq_to_readid_gpu", [&]() -> gx_status {
        if (!c || !out || !out_bytes || (!mate1 && bytes1)) return GX_EINVAL;
        *out = nullptr;
        *out_bytes = 0;
        std::lock_guard<std::mutex> lk(c->mu);
        cudaSetDevice(c->device);
        cudaStream_t s = c->stream;
        void *dev = nullptr;
        uint64_t w = 0;
        gx_status st = fastq_to_readid_device(
            s, (const uint8_t *)mate1, bytes1, (const uint8_t *)mate2, bytes2,
            [&](uint64_t total) -> uint8_t * {
                if (cudaMallocAsync(&dev, total + 1, s) != cudaSuccess) {
                    cudaGetLastError();
                    dev = nullptr;
                }
                return (uint8_t *)dev;
            },
            w);
        if (st == GX_OK) {
            *out = (char *)malloc(w + 1);
            if (!*out) {
                st = GX_ENOMEM;
            } else if (w) {
                CK(cudaMemcpyAsync(*out, dev, w, cudaMemcpyDeviceToHost, s));
                CK(sync_stream(s));
            }
            *out_bytes = w;
        }
        if (dev) cudaFreeAsync(dev, s);
        return st;
    });
}

gx_status gx_pinned_alloc(size_t bytes, void **out) {
    if (!out) return GX_EINVAL;
    *out = nullptr;
    if (cudaMallocHost(out, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return GX_ENOMEM;
    }
    return GX_OK;
}

void gx_pinned_free(void *ptr) {
    if (ptr) cudaFreeHost(ptr);
}

gx_status gx_ctx_create(int device, const gx_ctx_opts *opts, gx_ctx **out) {
    if (!out) return GX_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        fprintf(stderr, "gxgpu: no CUDA device available\n");
        return GX_ECUDA;
    }
    if (device < 0 || device >= n) return GX_EINVAL;
    gx_ctx *c = new (std::nothrow) gx_ctx();
    if (!c) return GX_ENOMEM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) !=
                                                    cudaSuccess) {
        delete c;
        return GX_ECUDA;
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    c->mem_limit = (opts && opts->device_mem_limit) ? opts->device_mem_limit : (size_t)(0.9 * (double)fr);
    if (opts && opts->struct_size >= offsetof(gx_ctx_opts, test_alloc_fail_above) + sizeof(size_t))
        c->test_alloc_fail_above = opts->test_alloc_fail_above;
    if (opts) c->test_flags = opts->flags;
    for (auto &e : c->marks) cudaEventCreate(&e);
    if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return GX_ECUDA;
    }
    *out = c;
    return GX_OK;
}

void gx_ctx_destroy(gx_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    sync_stream(c->stream);
    ctx_release(c);
}

gx_status gx_ctx_mark(gx_ctx *c, int slot) {
    if (!c || slot < 0 || slot >= 16) return GX_EINVAL;
    cudaSetDevice(c->device);
    CK(cudaEventRecord(c->marks[slot], c->stream));
    return GX_OK;
}

gx_status gx_ctx_elapsed_ms(gx_ctx *c, int a, int b, double *ms) {
    if (!c || !ms || a < 0 || b < 0 || a >= 16 || b >= 16) return GX_EINVAL;
    cudaSetDevice(c->device);
    CK(cudaEventSynchronize(c->marks[b]));
    float t = 0;
    CK(cudaEventElapsedTime(&t, c->marks[a], c->marks[b]));
    *ms = t;
    return GX_OK;
}

gx_status gx_ctx_synchronize(gx_ctx *c) {
    if (!c) return GX_EINVAL;
    cudaSetDevice(c->device);
    CK(sync_stream(c->stream));
    return GX_OK;
}

static gx_status job_create_impl(gx_ctx *c, const gx_job_opts *opts, gx_job **out);

gx_status gx_job_create(gx_ctx *c, const gx_job_opts *opts, gx_job **out) {
    return guarded("gx_job_create", [&] { return job_create_impl(c, opts, out); });
}

static gx_status job_create_impl(gx_ctx *c, const gx_job_opts *opts, gx_job **out) {
    if (!c || !opts || !out) return GX_EINVAL;
    *out = nullptr;
    if (opts->kmer_length < 3 || opts->kmer_length > 64) return GX_EINVAL;
    if (opts->input_kind != GX_INPUT_READID && opts->input_kind != GX_INPUT_FASTQ) return GX_EINVAL;
    if (opts->out_parts < 0 || opts->load_factor < 0 || opts->load_factor > 0.95) return GX_EINVAL;
    if (opts->max_readids_per_edge < 0) return GX_EINVAL;  // GenomixJobConf.validateConf :456-457
    {
        const int t = opts->threads_per_read;
        if (t < 0 || t > 32 || (t & (t - 1))) return GX_EINVAL;  // 0 or a power of two up to 32
    }
    const bool has_plan = opts->struct_size >= offsetof(gx_job_opts, plan) + sizeof(int);
    if (has_plan && opts->plan != GX_PLAN_BUILD_DEBRUIJN_GRAPH && opts->plan != GX_PLAN_BUILD_READ_PARSER)
        return GX_EINVAL;
    const bool has_layout = opts->struct_size >= offsetof(gx_job_opts, layout) + sizeof(int);
    if (has_layout) {
        if (opts->layout != GX_LAYOUT_BUCKETS && opts->layout != GX_LAYOUT_REFERENCE_PARTS) return GX_EINVAL;
        // the read parser's parts follow its input splits, not a key partitioner
        if (opts->layout == GX_LAYOUT_REFERENCE_PARTS &&
            ((has_plan && opts->plan != GX_PLAN_BUILD_DEBRUIJN_GRAPH) || opts->out_parts > 65536))
            return GX_EINVAL;
    }
    gx_job *j = new (std::nothrow) gx_job();
    if (!j) return GX_ENOMEM;
    j->ctx = c;
    c->refs.fetch_add(1);
    memcpy(&j->o, opts, std::min(sizeof j->o, opts->struct_size));
    if (!has_plan) j->o.plan = GX_PLAN_BUILD_DEBRUIJN_GRAPH;
    if (!has_layout) j->o.layout = GX_LAYOUT_BUCKETS;
    if (j->o.out_parts == 0) j->o.out_parts = 1;
    j->k = opts->kmer_length;
    j->wide = j->k > 32 ? 1 : 0;
    cudaSetDevice(c->device);
    j->tm.init();
    *out = j;
    return GX_OK;
}

static gx_status job_add_input_impl(gx_job *j, const void *host, size_t bytes, int mate_stream);

gx_status gx_job_add_input(gx_job *j, const void *host, size_t bytes, int mate_stream) {
    return guarded("gx_job_add_input", [&] { return job_add_input_impl(j, host, bytes, mate_stream); });
}

static gx_status job_add_input_impl(gx_job *j, const void *host, size_t bytes, int mate_stream) {
    if (!j || (!host && bytes)) return GX_EINVAL;
    if (j->state != JS_INPUT) return GX_ESTATE;
    std::lock_guard<std::mutex> lk(j->ctx->mu);
    cudaSetDevice(j->ctx->device);
    if (j->o.input_kind == GX_INPUT_FASTQ) {
        if (mate_stream < 0 || mate_stream > (j->o.paired ? 1 : 0)) return GX_EINVAL;
        j->fastq[mate_stream].emplace_back((const char *)host, bytes);
        return GX_OK;
    }
    if (mate_stream != 0) return GX_EINVAL;
    const bool nl = bytes > 0 && ((const uint8_t *)host)[bytes - 1] == '\n';
    gx_status st = append_text(j, host, bytes, cudaMemcpyHostToDevice, nl);
    if (st != GX_OK) return st;
    CK(sync_stream(j->ctx->stream));  // the host buffer is only borrowed for this call
    return GX_OK;
}

gx_status gx_job_add_input_device(gx_job *j, const void *dev, size_t bytes, int mate_stream) {
    if (!j || (!dev && bytes) || mate_stream != 0) return GX_EINVAL;
    if (j->o.input_kind != GX_INPUT_READID) return GX_EINVAL;
    if (((uintptr_t)dev & 15) != 0) return GX_EINVAL;
    if (j->state != JS_INPUT) return GX_ESTATE;
    if (!bytes) return GX_OK;
    std::lock_guard<std::mutex> lk(j->ctx->mu);
    cudaSetDevice(j->ctx->device);
    if (j->text_len == 0 && j->n_device_inputs == 0) {
        // a single device input is used in place; a missing final terminator is handled
        // by the line kernels (a last line ends at the buffer end)
        j->d_text = (uint8_t *)dev;
        j->text_len = bytes;
        j->text_cap = bytes;
        j->text_borrowed = true;
        j->n_device_inputs = 1;
        return GX_OK;
    }
    uint8_t last = 0;
    CK(d2h_async(&last, (const uint8_t *)dev + bytes - 1, 1, j->ctx->stream));
    CK(sync_stream(j->ctx->stream));
    if (j->text_borrowed && j->text_len) {
        // make the borrowed first input end with a terminator before appending
        uint8_t l0 = 0;
        CK(d2h_async(&l0, j->d_text + j->text_len - 1, 1, j->ctx->stream));
        CK(sync_stream(j->ctx->stream));
        gx_status st = ensure_text_cap(j, j->text_len + bytes + 2);
        if (st != GX_OK) return st;
        if (l0 != '\n') {
            CK(cudaMemsetAsync(j->d_text + j->text_len, '\n', 1, j->ctx->stream));
            j->text_len++;
        }
    }
    j->n_device_inputs++;
    return append_text(j, dev, bytes, cudaMemcpyDeviceToDevice, last == '\n');
}

gx_status gx_job_run(gx_job *j) {
    if (!j) return GX_EINVAL;
    if (j->state != JS_INPUT) return GX_ESTATE;
    std::lock_guard<std::mutex> lk(j->ctx->mu);
    cudaSetDevice(j->ctx->device);
    return run_job_locked(j);  // exception-safe
}

gx_status gx_job_stats(const gx_job *j, gx_stats *out) {
    if (!j || !out) return GX_EINVAL;
    *out = j->st;
    return GX_OK;
}

gx_status gx_job_records_device(gx_job *j, const void **dev, size_t *bytes, const uint64_t **part_offsets) {
    if (!j || !dev || !bytes) return GX_EINVAL;
    if (j->state != JS_RAN) return GX_ESTATE;
    *dev = j->d_out;
    *bytes = j->out_bytes;
    if (part_offsets) *part_offsets = j->part_bounds.data();
    return GX_OK;
}

static gx_status job_emit(gx_job *j, int part, void *host_out, size_t cap, size_t *written, int *more,
                          bool async);

gx_status gx_job_emit(gx_job *j, int part, void *host_out, size_t cap, size_t *written, int *more) {
    return guarded("gx_job_emit", [&] { return job_emit(j, part, host_out, cap, written, more, false); });
}

gx_status gx_job_emit_async(gx_job *j, int part, void *host_out, size_t cap, size_t *written, int *more) {
    return guarded("gx_job_emit_async", [&] { return job_emit(j, part, host_out, cap, written, more, true); });
}

static gx_status wait_copy(gx_job *j) {
    if (!j->copy_pending) return GX_OK;
    j->copy_pending = false;
    CK(cudaEventSynchronize(j->ev_copy));
    return GX_OK;
}

gx_status gx_job_emit_wait(gx_job *j) {
    if (!j) return GX_EINVAL;
    cudaSetDevice(j->ctx->device);
    return wait_copy(j);
}

static gx_status job_emit(gx_job *j, int part, void *host_out, size_t cap, size_t *written, int *more,
                          bool async) {
    if (!j || !written || !more || (!host_out && cap)) return GX_EINVAL;
    if (j->state != JS_RAN) return GX_ESTATE;
    if (part < 0 || part >= j->o.out_parts) return GX_EINVAL;
    std::lock_guard<std::mutex> lk(j->ctx->mu);
    cudaSetDevice(j->ctx->device);
    if (!async) {
        gx_status we = wait_copy(j);
        if (we != GX_OK) return we;
    }
    const uint64_t end = j->part_bounds[part + 1];
    uint64_t cur = j->cursor[part];
    *written = 0;
    *more = cur < end ? 1 : 0;
    if (cur >= end || cap == 0) return GX_OK;
    uint64_t stop = end;
    if (end - cur > cap) {
        // end on a record boundary: the last table-partition boundary that fits, else walk
        // the records of the partition that straddles the limit
        if (j->h_part_off.empty()) {
            j->h_part_off.resize(j->nparts + 1);
            CK(cudaMemcpy(j->h_part_off.data(), j->d_part_off, (j->nparts + 1) * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost));
        }
        const uint64_t lim = cur + cap;
        auto it = std::upper_bound(j->h_part_off.begin(), j->h_part_off.end(), (unsigned long long)lim);
        uint64_t b = (it == j->h_part_off.begin()) ? 0 : *(it - 1);
        if (b > cur) {
            stop = b;
        } else {
            CK(cudaMemcpy(host_out, j->d_out + cur, std::min<uint64_t>(cap, end - cur), cudaMemcpyDeviceToHost));
            const uint8_t *h = (const uint8_t *)host_out;
            uint64_t p = 0;
            while (p + 8 <= cap) {
                const uint32_t rl = ((uint32_t)h[p] << 24) | ((uint32_t)h[p + 1] << 16) | ((uint32_t)h[p + 2] << 8) |
                                    h[p + 3];
                if (p + 8 + rl > cap) break;
                p += 8 + rl;
            }
            if (p == 0) return GX_EINVAL;  // one record is larger than the buffer
            j->cursor[part] = cur + p;
            *written = p;
            *more = cur + p < end ? 1 : 0;
            return GX_OK;
        }
    }
    if (async) {
        // the build is complete (runs end synchronized): the copy needs no other dependency.  It
        // runs on the copy stream, alongside whatever the context's stream does next, in pieces:
        // copies in one direction share a copy engine, and the small status reads of a build
        // running meanwhile then wait for one piece, not for the whole copy
        if (!j->ev_copy) CK(cudaEventCreateWithFlags(&j->ev_copy, cudaEventDisableTiming));
        const uint64_t piece = 32ull << 20;
        for (uint64_t o = cur; o < stop; o += piece)
            CK(cudaMemcpyAsync((uint8_t *)host_out + (o - cur), j->d_out + o, std::min<uint64_t>(piece, stop - o),
                               cudaMemcpyDeviceToHost, j->ctx->copy_stream));
        CK(cudaEventRecord(j->ev_copy, j->ctx->copy_stream));
        j->copy_pending = true;
    } else {
        CK(cudaMemcpyAsync(host_out, j->d_out + cur, stop - cur, cudaMemcpyDeviceToHost, j->ctx->stream));
        CK(sync_stream(j->ctx->stream));
    }
    j->cursor[part] = stop;
    *written = stop - cur;
    *more = stop < end ? 1 : 0;
    return GX_OK;
}

gx_status gx_job_emit_rewind(gx_job *j, int part) {
    if (!j) return GX_EINVAL;
    cudaSetDevice(j->ctx->device);
    if (wait_copy(j) != GX_OK) return GX_ECUDA;
    if (j->state != JS_RAN) return GX_ESTATE;
    if (part < -1 || part >= j->o.out_parts) return GX_EINVAL;
    for (int q = 0; q < j->o.out_parts; q++)
        if (part == -1 || part == q) j->cursor[q] = j->part_bounds[q];
    return GX_OK;
}

void gx_job_destroy(gx_job *j) {
    if (!j) return;
    {
        std::lock_guard<std::mutex> lk(j->ctx->mu);
        cudaSetDevice(j->ctx->device);
        wait_copy(j);  // an asynchronous emit still reading the records
        if (j->ev_copy) cudaEventDestroy(j->ev_copy);
        cudaStream_t s = j->ctx->stream;
        if (j->d_text && !j->text_borrowed) cudaFreeAsync(j->d_text, s);
        if (j->out_owner)
            j->out_owner.reset();  // the last job of a batch frees the shared record buffer
        else if (j->d_out)
            cudaFreeAsync(j->d_out, s);
        if (j->d_part_off) cudaFreeAsync(j->d_part_off, s);
        sync_stream(s);
        j->tm.destroy();
    }
    gx_ctx *c = j->ctx;
    delete j;
    ctx_release(c);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// the run
// ---------------------------------------------------------------------------------------
// state shared by the phases of one run
struct RunCtx {
    gx_job *j;
    cudaStream_t s;
    RunArena &ar;
    DevStatus *d_st;
    void *scratch;
    const uint8_t *text;
    uint64_t n_text;
    LineRec *lines;
    uint32_t *reads;
    uint32_t n_lines, n_reads;
    unsigned long long n_occ;
    // partitioned build: exact super counts (2048) and HyperLogLog registers, when it counted
    uint32_t *d_scnt, *d_hll;
    std::vector<uint32_t> scnt, hll;
};

// Where the partitioned build keeps its records: node j of bucket p starts noff[node_base[p] + j]
// bytes into the bucket's records (no walk needed to index them).
struct NodeRecords {
    const void *nkey = nullptr;  // node keys, same indexing
    const uint32_t *noff = nullptr;
    const unsigned long long *node_base = nullptr;
};

// Regroups a finished record stream into the reference's parts (GX_LAYOUT_REFERENCE_PARTS):
// each record's part from its key (KmerPartitionComputerFactory.java:28-52), then a stable
// regrouping by part into a new buffer.  Up to 256 parts: one pass that moves the records
// straight to their places (per tile and part, byte counts; their scan; a staged copy), the
// tiles being the partitioned build's buckets (read from its node keys and offsets) or runs of
// records indexed by a walk.  More parts: a stable counting sort of record indexes (two 8-bit
// passes), the lengths scanned in the new order, a gather copy.  On success `outp` and
// `part_off` are replaced (the old ones freed) by the new records and a sorted list of record
// boundaries (for chunked emits), and part_bounds are set.
static gx_status relayout_reference_parts(RunCtx &rc, uint32_t &nparts, unsigned long long total,
                                          const std::vector<uint32_t> &pn, const uint32_t *d_part_nodes, uint64_t nn,
                                          const NodeRecords *nr, unsigned long long *&part_off, void *&outp) {
    gx_job *j = rc.j;
    cudaStream_t s = rc.s;
    const uint32_t P = (uint32_t)j->o.out_parts;
    if (nn > 0xffffffffULL) return GX_ENOMEM;  // record indexes are 32-bit
    const uint32_t N = (uint32_t)nn;
    const bool one_pass = P <= 256;
    const bool by_bucket = one_pass && nr;  // no per-record arrays
    RunArena ar(s);
    gx_status e;
    uint32_t *rpart = nullptr, *rlen = nullptr;
    unsigned long long *roff = nullptr, *bounds;
    if ((e = ar.alloc(bounds, P + 1)) != GX_OK) return e;
    if (!by_bucket) {
        std::vector<uint32_t> nbase(nparts);
        uint32_t acc = 0;
        for (uint32_t q = 0; q < nparts; q++) {
            nbase[q] = acc;
            acc += pn[q];
        }
        uint32_t *d_nbase;
        if ((e = ar.alloc(d_nbase, nparts)) != GX_OK) return e;
        if ((e = ar.alloc(rpart, N)) != GX_OK) return e;
        if ((e = ar.alloc(rlen, N)) != GX_OK) return e;
        if ((e = ar.alloc(roff, N)) != GX_OK) return e;
        CK(cudaMemcpyAsync(d_nbase, nbase.data(), nparts * 4ull, cudaMemcpyHostToDevice, s));
        CK(sync_stream(s));  // nbase is read by the copy
        CK(cudaEventRecord(j->tm.ev[7], s));
        if (nr)
            launch_rl_index_nodes(nr->nkey, j->wide, j->k, part_off, nr->node_base, nr->noff, d_nbase, d_part_nodes,
                                  nparts, P, rpart, roff, rlen, s);
        else
            launch_rl_index((const uint8_t *)outp, part_off, d_nbase, nparts, P, rpart, roff, rlen, s);
    } else {
        CK(cudaEventRecord(j->tm.ev[7], s));
    }
    void *nout = nullptr;
    if (cudaMallocAsync(&nout, total + 16, s) != cudaSuccess) {
        cudaGetLastError();
        return GX_ENOMEM;
    }
    struct OutGuard {
        void *&p;
        cudaStream_t s;
        ~OutGuard() {
            if (p) cudaFreeAsync(p, s);
        }
    } guard{nout, s};
    // the record boundaries of the new layout: every entry of the scanned tile counts, or every
    // 1024th record; at most ~64K of them are kept
    const unsigned long long *bnd;
    uint64_t n_bnd;  // entries of bnd, the last one the total
    unsigned long long moved = 0;
    uint32_t late = 0;  // a bulk copy of the regrouping that did not land in time
    if (one_pass) {
        const uint32_t tiles = by_bucket ? nparts : rl_tiles(N);
        const uint64_t ncnt = (uint64_t)P * tiles;
        unsigned long long *cnt;
        uint32_t *d_late;
        void *scratch;
        if ((e = ar.alloc(cnt, ncnt + 1)) != GX_OK) return e;
        if ((e = ar.alloc(scratch, scan_scratch_bytes(ncnt, 8))) != GX_OK) return e;
        if ((e = ar.alloc(d_late, 1)) != GX_OK) return e;
        CK(cudaMemsetAsync(d_late, 0, 4, s));
        const int withhold = (j->ctx->test_flags & GX_CTX_TEST_WITHHOLD_COPIES) ? 1 : 0;
        if (by_bucket)
            launch_rl_regroup_nodes((const uint8_t *)outp, nr->nkey, j->wide, j->k, nr->noff, nr->node_base, part_off,
                                    d_part_nodes, nparts, P, cnt, scratch, (uint8_t *)nout, d_late, withhold, s);
        else
            launch_rl_regroup_arrays((const uint8_t *)outp, rpart, rlen, roff, N, P, cnt, scratch, (uint8_t *)nout,
                                     d_late, withhold, s);
        launch_rl_part_starts(cnt, tiles, P, total, bounds, s);
        CK(d2h_async(&moved, cnt + ncnt, 8, s));
        CK(d2h_async(&late, d_late, 4, s));
        bnd = cnt;
        n_bnd = ncnt + 1;
    } else {
        uint32_t *perm, *perm2, *cnt;
        unsigned long long *len2, *noff;
        void *scratch;
        const uint64_t ncnt = 256ull * rl_tiles(N);
        if ((e = ar.alloc(perm, N)) != GX_OK) return e;
        if ((e = ar.alloc(perm2, N)) != GX_OK) return e;
        if ((e = ar.alloc(cnt, ncnt)) != GX_OK) return e;
        if ((e = ar.alloc(len2, N)) != GX_OK) return e;
        if ((e = ar.alloc(noff, (uint64_t)N + 1)) != GX_OK) return e;
        if ((e = ar.alloc(scratch, std::max(scan_scratch_bytes(ncnt, 8), scan_scratch_bytes((uint64_t)N + 1, 8)))) !=
            GX_OK)
            return e;
        const uint32_t *order = nullptr;
        uint32_t *dst = perm;
        for (int shift = 0; shift < 16; shift += 8) {
            launch_rl_count(rpart, order, N, shift, cnt, s);
            exclusive_scan_u32(cnt, cnt, ncnt, nullptr, scratch, s);
            launch_rl_scatter(rpart, order, N, shift, cnt, dst, s);
            order = dst;
            dst = dst == perm ? perm2 : perm;
        }
        launch_rl_gather_len(order, rlen, N, len2, s);
        exclusive_scan_u64(len2, noff, N, noff + N, scratch, s);
        launch_rl_copy((const uint8_t *)outp, order, roff, noff, rlen, N, (uint8_t *)nout, s);
        launch_rl_bounds(rpart, order, N, P, noff, bounds, s);
        CK(d2h_async(&moved, noff + N, 8, s));
        bnd = noff;
        n_bnd = (uint64_t)N + 1;
    }
    const uint64_t stride = std::max<uint64_t>(1, (n_bnd + 65535) / 65536);
    const uint64_t n_groups = (n_bnd - 1 + stride - 1) / stride;  // the total comes last
    unsigned long long *groups = nullptr;
    if (cudaMallocAsync(&groups, (n_groups + 1) * sizeof(unsigned long long), s) != cudaSuccess) {
        cudaGetLastError();
        return GX_ENOMEM;
    }
    launch_rl_sample(bnd, n_bnd - 1, (uint32_t)stride, n_groups + 1, groups, s);
    CK(cudaEventRecord(j->tm.ev[8], s));
    std::vector<unsigned long long> hb(P + 1);
    CK(d2h_async(hb.data(), bounds, (P + 1) * 8ull, s));
    CK(sync_stream(s));
    CK(cudaGetLastError());
    if (late) {
        cudaFreeAsync(groups, s);
        fprintf(stderr, "gxgpu: the regrouping into the reference's parts timed out waiting for a bulk copy\n");
        return GX_ETIMEOUT;
    }
    if (moved != total || hb[0] != 0 || hb[P] != total) {
        cudaFreeAsync(groups, s);
        fprintf(stderr, "gxgpu: internal error: the regrouped records do not add up\n");
        return GX_ECUDA;
    }
    for (uint32_t q = 0; q <= P; q++) j->part_bounds[q] = hb[q];
    j->st.ms_layout = j->tm.ms(7, 8);
    cudaFreeAsync(outp, s);
    cudaFreeAsync(part_off, s);
    outp = nout;
    nout = nullptr;  // the job owns it now: the guard lets go
    part_off = groups;
    nparts = (uint32_t)n_groups;
    return GX_OK;
}

// After the record writer: its status (into hs), the node and head counts per partition and the
// output parts' bounds, all read back in one round trip.
static gx_status finish_outputs(RunCtx &rc, uint32_t nparts, unsigned long long total, unsigned long long *part_off,
                                const uint32_t *part_nodes, const uint32_t *head_cnt2, void *outp, DevStatus &hs,
                                const NodeRecords *nr = nullptr) {
    gx_job *j = rc.j;
    const int P = j->o.out_parts;
    const bool regroup = j->o.layout == GX_LAYOUT_REFERENCE_PARTS && P > 1;
    std::vector<uint32_t> pn(nparts), hc(nparts);
    std::vector<unsigned long long> bounds(P + 1, 0);
    CK(d2h_async(&hs, rc.d_st, sizeof hs, rc.s));
    CK(d2h_async(pn.data(), part_nodes, nparts * 4ull, rc.s));
    CK(d2h_async(hc.data(), head_cnt2, nparts * 4ull, rc.s));
    if (!regroup)
        for (int q = 1; q < P; q++) {
            const uint64_t tp = (uint64_t)nparts * q / P;
            if (tp > 0) CK(d2h_async(&bounds[q], part_off + tp, 8, rc.s));
        }
    CK(sync_stream(rc.s));
    CK(cudaGetLastError());
    if (hs.internal_err) {
        cudaFreeAsync(outp, rc.s);
        cudaFreeAsync(part_off, rc.s);
        fprintf(stderr, "gxgpu: internal error: record sizes disagree between emission passes\n");
        return GX_ECUDA;
    }
    uint64_t nn = 0, nh = 0;
    for (uint32_t q = 0; q < nparts; q++) {
        nn += pn[q];
        nh += hc[q];
    }
    if (regroup && nn > 0) {
        const gx_status e = relayout_reference_parts(rc, nparts, total, pn, part_nodes, nn, nr, part_off, outp);
        if (e != GX_OK) {
            cudaFreeAsync(outp, rc.s);
            cudaFreeAsync(part_off, rc.s);
            return e;
        }
    } else {
        bounds[P] = total;
        for (int q = 0; q <= P; q++) j->part_bounds[q] = bounds[q];
    }
    for (int q = 0; q < P; q++) j->cursor[q] = j->part_bounds[q];
    j->st.nodes = nn;
    j->st.read_heads = nh;
    j->d_out = (uint8_t *)outp;
    j->out_bytes = total;
    j->d_part_off = part_off;
    j->nparts = nparts;
    j->st.record_bytes = total;
    return GX_OK;
}

// ---- the global-table build ------------------------------------------------------------
static gx_status build_table(RunCtx &rc) {
    gx_job *j = rc.j;
    cudaStream_t s = rc.s;
    Timers &tm = j->tm;
    gx_status e;
    const int k = j->k;
    const uint32_t n_reads = rc.n_reads;
    const size_t slot_bytes = j->wide ? sizeof(Slot128) : sizeof(Slot64);
    double lf = j->eff_load_factor > 0 ? j->eff_load_factor : 0.5;
    DevStatus hs;
    for (int attempt = 0;; attempt++) {
        const uint64_t want = (uint64_t)((double)rc.n_occ / lf) + 1;
        const uint64_t nparts64 = std::max<uint64_t>(1, (want + PART_SLOTS - 1) / PART_SLOTS);
        if (nparts64 > 0x7fffffffULL) return GX_ENOMEM;
        const uint32_t nparts = (uint32_t)nparts64;
        const size_t table_bytes = (size_t)nparts * PART_SLOTS * slot_bytes;
        if (table_bytes > j->ctx->mem_limit) return GX_ENOMEM;
        RunArena tar(s);
        void *table;
        Head *heads;
        uint32_t *head_cnt, *head_off, *head_cur, *head_idx, *head_cnt2, *part_nodes;
        unsigned long long *head_sk, *part_bytes, *part_off;
        if ((e = tar.alloc(table, table_bytes / 16 * 16 + 16)) != GX_OK) return e;
        if ((e = tar.alloc(heads, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(head_cnt, nparts)) != GX_OK) return e;
        if ((e = tar.alloc(head_off, nparts)) != GX_OK) return e;
        if ((e = tar.alloc(head_cur, nparts)) != GX_OK) return e;
        if ((e = tar.alloc(head_idx, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(head_cnt2, nparts)) != GX_OK) return e;
        if ((e = tar.alloc(head_sk, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(part_nodes, nparts)) != GX_OK) return e;
        if ((e = tar.alloc(part_bytes, nparts)) != GX_OK) return e;
        void *pscratch;
        if ((e = tar.alloc(pscratch, scan_scratch_bytes(nparts, 8))) != GX_OK) return e;
        void *part_off_v = nullptr;
        CK(cudaMallocAsync(&part_off_v, (nparts + 1) * sizeof(unsigned long long), s));
        part_off = (unsigned long long *)part_off_v;

        TableGeom g{table, nparts, j->wide};
        CK(cudaMemsetAsync(table, 0, table_bytes, s));
        CK(cudaMemsetAsync(head_cnt, 0, nparts * 4ull, s));
        CK(cudaMemsetAsync(head_cur, 0, nparts * 4ull, s));
        CK(cudaEventRecord(tm.ev[2], s));
        launch_insert(g, rc.text, rc.lines, rc.reads, n_reads, k, heads, head_cnt, rc.d_st, s);
        CK(cudaEventRecord(tm.ev[3], s));
        exclusive_scan_u32(head_cnt, head_off, nparts, nullptr, pscratch, s);
        launch_head_scatter(heads, n_reads, head_off, head_cur, head_idx, nparts, s);
        EmitArgs a{};
        a.g = g;
        a.k = k;
        a.text = rc.text;
        a.n_text = rc.n_text;
        a.lines = rc.lines;
        a.reads = rc.reads;
        a.heads = heads;
        a.head_idx = head_idx;
        a.head_sk = head_sk;
        a.head_off = head_off;
        a.head_cnt = head_cnt;
        a.head_cnt2 = head_cnt2;
        a.part_nodes = part_nodes;
        a.part_bytes = part_bytes;
        a.part_off = part_off;
        a.st = rc.d_st;
        launch_emit_prepare(a, s);
        exclusive_scan_u64(part_bytes, part_off, nparts, part_off + nparts, pscratch, s);
        CK(cudaEventRecord(tm.ev[4], s));
        unsigned long long total = 0;
        CK(d2h_async(&hs, rc.d_st, sizeof hs, s));
        CK(d2h_async(&total, part_off + nparts, 8, s));
        CK(sync_stream(s));
        CK(cudaGetLastError());
        if (hs.table_full) {
            cudaFreeAsync(part_off, s);
            DevStatus zero{};
            zero.parse_err = ~0ULL;
            CK(cudaMemcpyAsync(rc.d_st, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
            if (attempt >= 2) return GX_ETABLE_FULL;
            lf *= 0.5;
            continue;
        }
        void *outp = nullptr;
        CK(cudaMallocAsync(&outp, total + 16, s));
        if (((uintptr_t)outp & 15) != 0) {  // the record writer stores aligned 16-byte vectors
            cudaFreeAsync(outp, s);
            cudaFreeAsync(part_off, s);
            return GX_ECUDA;
        }
        a.out = (uint8_t *)outp;
        CK(cudaEventRecord(tm.ev[5], s));
        launch_emit_write(a, s);
        CK(cudaEventRecord(tm.ev[6], s));
        if ((e = finish_outputs(rc, nparts, total, part_off, part_nodes, head_cnt2, outp, hs)) != GX_OK) return e;
        j->st.table_slots = (uint64_t)nparts * PART_SLOTS;
        j->st.table_partitions = nparts;
        j->st.attempts = (uint64_t)attempt + 1;
        j->st.max_probe = hs.max_probe;
        j->st.cov_inexact_nodes = hs.cov_inexact;
        j->st.ms_insert = tm.ms(2, 3);
        j->st.ms_emit = tm.ms(3, 4) + tm.ms(5, 6);
        j->st.ms_aggregate = tm.ms(3, 4);
        j->st.ms_write = tm.ms(5, 6);
        j->st.ms_total = tm.ms(0, 6);
        return GX_OK;
    }
}

// ---- the read-parser plan: every occurrence's (Kmer, Node) record, in read order -----------
static gx_status build_read_parser(RunCtx &rc) {
    gx_job *j = rc.j;
    cudaStream_t s = rc.s;
    Timers &tm = j->tm;
    const uint32_t n = rc.n_reads;
    RunArena tar(s);
    unsigned long long *rbytes;
    void *pscratch;
    gx_status e;
    if ((e = tar.alloc(rbytes, n)) != GX_OK) return e;
    if ((e = tar.alloc(pscratch, scan_scratch_bytes((uint64_t)n + 1, 8))) != GX_OK) return e;
    void *roff_v = nullptr, *outp = nullptr;
    CK(cudaMallocAsync(&roff_v, (n + 1ull) * 8, s));
    unsigned long long *roff = (unsigned long long *)roff_v;
    CK(cudaEventRecord(tm.ev[2], s));
    launch_rp_sizes(rc.lines, rc.reads, n, j->k, rbytes, s);
    exclusive_scan_u64(rbytes, roff, n, roff + n, pscratch, s);
    unsigned long long total = 0;
    CK(d2h_async(&total, roff + n, 8, s));
    CK(sync_stream(s));
    if (cudaMallocAsync(&outp, total + 16, s) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(roff, s);
        return GX_ENOMEM;
    }
    CK(cudaEventRecord(tm.ev[5], s));
    launch_rp_write(j->wide, rc.text, rc.n_text, rc.lines, rc.reads, n, j->k, roff, (uint8_t *)outp, s);
    CK(cudaEventRecord(tm.ev[6], s));
    CK(sync_stream(s));
    CK(cudaGetLastError());
    // output parts split between reads
    const int P = j->o.out_parts;
    for (int q = 0; q <= P; q++) {
        unsigned long long v = total;
        const uint64_t r = (uint64_t)n * q / P;
        if (q < P && r > 0) {
            CK(d2h_async(&v, roff + r, 8, s));
            CK(sync_stream(s));
        }
        if (q < P && r == 0) v = 0;
        j->part_bounds[q] = v;
    }
    for (int q = 0; q < P; q++) j->cursor[q] = j->part_bounds[q];
    j->d_out = (uint8_t *)outp;
    j->out_bytes = total;
    j->d_part_off = roff;  // record groups for chunked emits: one per read
    j->nparts = n;
    j->st.nodes = rc.n_occ;  // one record per occurrence
    j->st.read_heads = n;
    j->st.record_bytes = total;
    j->st.table_partitions = n;
    j->st.attempts = 1;
    j->st.ms_write = tm.ms(5, 6);
    j->st.ms_emit = tm.ms(2, 6);
    j->st.ms_total = tm.ms(0, 6);
    return GX_OK;
}

// the exact super counts and HyperLogLog registers of the whole input (a counting pass)
static gx_status count_supers(RunCtx &rc) {
    cudaStream_t s = rc.s;
    gx_status e;
    if (!rc.d_scnt) {
        if ((e = rc.ar.alloc(rc.d_scnt, MAX_SUPERS)) != GX_OK) return e;
        if ((e = rc.ar.alloc(rc.d_hll, HLL_REGS)) != GX_OK) return e;
    }
    CK(cudaMemsetAsync(rc.d_scnt, 0, MAX_SUPERS * 4, s));
    CK(cudaMemsetAsync(rc.d_hll, 0, HLL_REGS * 4, s));
    uint32_t *d_n;
    if ((e = rc.ar.alloc(d_n, 1)) != GX_OK) return e;
    CK(cudaMemcpyAsync(d_n, &rc.n_reads, 4, cudaMemcpyHostToDevice, s));
    launch_count_occ(rc.j->wide, rc.text, rc.n_text, rc.lines, rc.reads, d_n, rc.n_reads, rc.j->k, 11, rc.d_scnt,
                     rc.d_hll, s);
    rc.scnt.resize(MAX_SUPERS);
    rc.hll.resize(HLL_REGS);
    CK(d2h_async(rc.scnt.data(), rc.d_scnt, MAX_SUPERS * 4, s));
    CK(d2h_async(rc.hll.data(), rc.d_hll, HLL_REGS * 4, s));
    CK(sync_stream(s));
    CK(cudaGetLastError());
    return GX_OK;
}

// ---- the partitioned build ---------------------------------------------------------------
// A job's first pass needs no counting pass: the super scatter writes into buckets with room
// for SC_ROOM x the mean (the hash spreads k-mers evenly; only a k-mer repeated very many times
// can fill one) and gathers the HyperLogLog registers on the way, which size the fine buckets.
// If a bucket runs out of room, the job counts its super buckets exactly and scatters again.
static gx_status build_partitioned(RunCtx &rc) {
    gx_job *j = rc.j;
    cudaStream_t s = rc.s;
    Timers &tm = j->tm;
    gx_status e;
    const int k = j->k, wide = j->wide;
    const uint32_t n_reads = rc.n_reads;
    const uint64_t n_occ = rc.n_occ;
    const size_t kb = wide ? 16 : 8;
    double safety = 1.15;
    DevStatus hs;
    bool counted = !rc.scnt.empty();
    if (!counted && n_occ / 2 > 0xfffffff0ULL - SC_SLACK) {  // bucket cursors are 32-bit
        if ((e = count_supers(rc)) != GX_OK) return e;
        counted = true;
    }
    double d_est = counted ? hll_estimate(rc.hll.data()) : 0.0;
    for (int attempt = 0;; attempt++) {
        const double target = bucket_target(j->eff_load_factor);
        // super buckets: from the distinct estimate, or (before any count) from the occurrences,
        // which bound the distinct k-mers
        PartPlan pp = plan_partitions(counted ? d_est : (double)n_occ, safety, target);
        const uint32_t S = 1u << pp.log_s;
        const uint64_t cap = counted ? 0 : std::min<uint64_t>(0xfffffff0ULL, (uint64_t)((double)n_occ / S * SC_ROOM) + SC_SLACK);
        const uint64_t occ_room = counted ? n_occ : std::max<uint64_t>(n_occ, (uint64_t)S * cap);
        RunArena tar(s);
        void *okey, *okey2;
        uint16_t *obits, *obits2;
        unsigned long long *d_soff, *fine_cnt, *fine_off, *head_sk, *part_bytes, *part_off;
        ulonglong2 *d_chunks;
        uint32_t *s_cur, *fine_cur, *head_cnt, *head_off, *head_cur, *head_idx, *head_cnt2, *part_nodes;
        Head *heads;
        HeadOut *hout;
        uint32_t *noff;
        uint8_t *okey_b, *okey2_b;
        // The room per bucket of the uncounted scatter costs (occ_room - n_occ) x (kb + 2) bytes
        // more than the exact counts: when that does not fit (the context's limit, or a failed
        // allocation), count first and scatter into the exact offsets instead.
        if (!counted) {
            const double need = (double)(occ_room + n_occ) * (double)(kb + 2) + (double)n_occ * 4.0 +
                                (double)n_reads * (sizeof(Head) + sizeof(HeadOut) + 12.0);
            bool fits = need <= (double)j->ctx->mem_limit;
            if (fits) fits = tar.alloc(okey_b, occ_room * kb) == GX_OK && tar.alloc(obits, occ_room) == GX_OK;
            if (!fits) {
                tar.release();
                if ((e = count_supers(rc)) != GX_OK) return e;
                counted = true;
                d_est = hll_estimate(rc.hll.data());
                attempt--;
                continue;
            }
        } else {
            if ((e = tar.alloc(okey_b, occ_room * kb)) != GX_OK) return e;
            if ((e = tar.alloc(obits, occ_room)) != GX_OK) return e;
        }
        if ((e = tar.alloc(okey2_b, n_occ * kb)) != GX_OK) return e;
        okey = okey_b;
        okey2 = okey2_b;
        if ((e = tar.alloc(obits2, n_occ)) != GX_OK) return e;
        if ((e = tar.alloc(d_soff, S + 1)) != GX_OK) return e;
        if ((e = tar.alloc(s_cur, S)) != GX_OK) return e;
        if ((e = tar.alloc(heads, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(hout, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(noff, n_occ)) != GX_OK) return e;
        if ((e = tar.alloc(head_idx, n_reads)) != GX_OK) return e;
        HeadIn *hsorted;
        if ((e = tar.alloc(hsorted, n_reads)) != GX_OK) return e;
        if ((e = tar.alloc(head_sk, n_reads)) != GX_OK) return e;
        // the job is a batch of one sample
        SamplePlan *d_plan;
        SuperInfo *d_sinfo;
        uint32_t *d_rbase;
        if ((e = tar.alloc(d_plan, 1)) != GX_OK) return e;
        if ((e = tar.alloc(d_sinfo, S)) != GX_OK) return e;
        if ((e = tar.alloc(d_rbase, 2)) != GX_OK) return e;
        const SampleMap smap{d_rbase, d_plan, 1};
        {
            const uint32_t hrb[2] = {0, n_reads};
            CK(cudaMemcpyAsync(d_rbase, hrb, sizeof hrb, cudaMemcpyHostToDevice, s));
        }
        std::vector<unsigned long long> soff(S + 1, 0);
        std::vector<uint32_t> scount(S, 0);
        CK(cudaMemsetAsync(s_cur, 0, S * 4ull, s));
        CK(cudaEventRecord(tm.ev[2], s));
        if (!counted) {
            // A2 first, with room per bucket; the HyperLogLog registers come back with the counts
            uint32_t *d_hll, *d_ovf;
            if ((e = tar.alloc(d_hll, SC_HLL_REGS)) != GX_OK) return e;
            if ((e = tar.alloc(d_ovf, 1)) != GX_OK) return e;
            CK(cudaMemsetAsync(d_hll, 0, SC_HLL_REGS * 4, s));
            CK(cudaMemsetAsync(d_ovf, 0, 4, s));
            for (uint32_t q = 0; q <= S; q++) soff[q] = (unsigned long long)q * cap;
            const SamplePlan hp{0, pp.log_s, 1, 0};
            CK(cudaMemcpyAsync(d_plan, &hp, sizeof hp, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(d_soff, soff.data(), (S + 1) * 8ull, cudaMemcpyHostToDevice, s));
            launch_scatter_super(wide, rc.text, rc.n_text, rc.lines, rc.reads, n_reads, k, smap, S, d_soff, s_cur,
                                 okey, obits, (uint32_t)cap, d_hll, d_ovf, s, (uint32_t)j->eff_threads_per_read);
            std::vector<uint32_t> hh(SC_HLL_REGS);
            uint32_t ovf = 0;
            CK(d2h_async(scount.data(), s_cur, S * 4ull, s));
            CK(d2h_async(hh.data(), d_hll, SC_HLL_REGS * 4, s));
            CK(d2h_async(&ovf, d_ovf, 4, s));
            CK(sync_stream(s));
            CK(cudaGetLastError());
            if (ovf) {
                // a bucket needed more room: count exactly, then scatter again (not an attempt)
                tar.release();
                if ((e = count_supers(rc)) != GX_OK) return e;
                counted = true;
                d_est = hll_estimate(rc.hll.data());
                attempt--;
                continue;
            }
            if (attempt == 0) d_est = hll_estimate(hh.data(), SC_HLL_REGS);
            // fine buckets for this S
            double want = d_est * safety / target;
            const uint64_t P64 = (uint64_t)std::max(1.0, std::ceil(want));
            pp.F = (uint32_t)std::min<uint64_t>(MAX_FINE, std::max<uint64_t>(1, (P64 + S - 1) / S));
            pp.P = S * pp.F;
        } else {
            // super counts at this resolution, offsets
            const uint32_t fold = MAX_SUPERS >> pp.log_s;
            for (uint32_t q = 0; q < S; q++) {
                unsigned long long c = 0;
                for (uint32_t t = 0; t < fold; t++) c += rc.scnt[q * fold + t];
                scount[q] = (uint32_t)c;
                soff[q + 1] = soff[q] + c;
            }
            if (soff[S] != n_occ) return GX_ECUDA;
        }
        const uint32_t P = pp.P;
        // CHUNK-sized pieces of every super bucket: counted here, written on the device
        std::vector<uint32_t> cbase(S + 1, 0);
        uint64_t placed = 0, nc64 = 0;
        for (uint32_t q = 0; q < S; q++) {
            placed += scount[q];
            cbase[q] = (uint32_t)nc64;
            nc64 += (scount[q] + CHUNK - 1) / CHUNK;
        }
        if (placed != n_occ || nc64 > 0x7fffffffULL) return GX_ECUDA;
        cbase[S] = (uint32_t)nc64;
        const uint32_t n_chunks = (uint32_t)nc64;
        uint32_t *d_scount, *d_cbase;
        if ((e = tar.alloc(d_chunks, std::max<uint32_t>(n_chunks, 1))) != GX_OK) return e;
        if ((e = tar.alloc(d_scount, S)) != GX_OK) return e;
        if ((e = tar.alloc(d_cbase, S + 1)) != GX_OK) return e;
        if ((e = tar.alloc(fine_cnt, P)) != GX_OK) return e;
        if ((e = tar.alloc(fine_off, P + 1)) != GX_OK) return e;
        if ((e = tar.alloc(fine_cur, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_cnt, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_off, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_cur, P)) != GX_OK) return e;
        if ((e = tar.alloc(head_cnt2, P)) != GX_OK) return e;
        if ((e = tar.alloc(part_nodes, P)) != GX_OK) return e;
        if ((e = tar.alloc(part_bytes, P)) != GX_OK) return e;
        void *pscratch;
        if ((e = tar.alloc(pscratch, scan_scratch_bytes(P + 1, 8))) != GX_OK) return e;
        {
            const SamplePlan hp{0, pp.log_s, pp.F, 0};
            std::vector<SuperInfo> hsi(S);
            for (uint32_t q = 0; q < S; q++) hsi[q] = SuperInfo{q * pp.F, pp.F, pp.log_s, 0};
            CK(cudaMemcpyAsync(d_plan, &hp, sizeof hp, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(d_sinfo, hsi.data(), S * sizeof(SuperInfo), cudaMemcpyHostToDevice, s));
        }
        void *part_off_v = nullptr;
        CK(cudaMallocAsync(&part_off_v, (P + 1) * sizeof(unsigned long long), s));
        part_off = (unsigned long long *)part_off_v;
        if (counted) CK(cudaMemcpyAsync(d_soff, soff.data(), (S + 1) * 8ull, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_scount, scount.data(), S * 4ull, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_cbase, cbase.data(), (S + 1) * 4ull, cudaMemcpyHostToDevice, s));
        launch_make_chunks(d_soff, d_scount, d_cbase, S, d_chunks, s);
        CK(cudaMemsetAsync(fine_cnt, 0, P * 8ull, s));
        CK(cudaMemsetAsync(fine_cur, 0, P * 4ull, s));
        CK(cudaMemsetAsync(head_cnt, 0, P * 4ull, s));
        CK(cudaMemsetAsync(head_cur, 0, P * 4ull, s));
        if (counted) {
            // A2 into the counted offsets
            launch_scatter_super(wide, rc.text, rc.n_text, rc.lines, rc.reads, n_reads, k, smap, S, d_soff, s_cur,
                                 okey, obits, 0xffffffffu, nullptr, nullptr, s, (uint32_t)j->eff_threads_per_read);
        }
        // read heads
        launch_heads_part(wide, rc.text, rc.n_text, rc.lines, rc.reads, n_reads, k, smap, heads, head_cnt, s);
        exclusive_scan_u32(head_cnt, head_off, P, nullptr, pscratch, s);
        launch_head_scatter_part(heads, rc.reads, rc.lines, n_reads, head_off, head_cur, head_idx, hsorted, s);
        // B1, B2
        launch_fine_count(wide, okey, d_chunks, n_chunks, d_sinfo, fine_cnt, s);
        exclusive_scan_u64(fine_cnt, fine_off, P, fine_off + P, pscratch, s);
        launch_scatter_fine(wide, okey, obits, d_chunks, n_chunks, d_sinfo, fine_off, fine_cur, okey2, obits2, s);
        CK(cudaEventRecord(tm.ev[3], s));
        // C
        AggArgs g{};
        g.wide = wide;
        g.k = k;
        g.pp = pp;
        g.okey2 = okey2;
        g.obits2 = obits2;
        g.fine_off = fine_off;
        g.lines = rc.lines;
        g.reads = rc.reads;
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
        g.st = rc.d_st;
        launch_aggregate(g, s);
        exclusive_scan_u64(part_bytes, part_off, P, part_off + P, pscratch, s);
        CK(cudaEventRecord(tm.ev[4], s));
        unsigned long long total = 0;
        CK(d2h_async(&hs, rc.d_st, sizeof hs, s));
        CK(d2h_async(&total, part_off + P, 8, s));
        CK(sync_stream(s));
        CK(cudaGetLastError());
        if (hs.internal_err) {
            cudaFreeAsync(part_off, s);
            fprintf(stderr, "gxgpu: internal error: a read head's k-mer was not aggregated\n");
            return GX_ECUDA;
        }
        if (hs.table_full) {
            // more distinct k-mers in a bucket than its shared table holds: more buckets
            cudaFreeAsync(part_off, s);
            DevStatus zero{};
            zero.parse_err = ~0ULL;
            CK(cudaMemcpyAsync(rc.d_st, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
            if (attempt >= 3 || pp.F >= MAX_FINE) return GX_ETABLE_FULL;
            safety *= 2;
            continue;
        }
        // D: records
        void *outp = nullptr;
        CK(cudaMallocAsync(&outp, total + 16, s));
        if (((uintptr_t)outp & 15) != 0) {
            cudaFreeAsync(outp, s);
            cudaFreeAsync(part_off, s);
            return GX_ECUDA;
        }
        EmitArgs a{};
        a.g = TableGeom{nullptr, P, wide};
        a.k = k;
        a.text = rc.text;
        a.n_text = rc.n_text;
        a.lines = rc.lines;
        a.reads = rc.reads;
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
        a.st = rc.d_st;
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
        NodeRecords nr;
        nr.nkey = okey2;
        nr.noff = noff;
        nr.node_base = fine_off;
        if ((e = finish_outputs(rc, P, total, part_off, part_nodes, head_cnt2, outp, hs, &nr)) != GX_OK) return e;
        j->st.table_slots = (uint64_t)P * AGG_SLOTS;
        j->st.table_partitions = P;
        j->st.super_counted = counted ? 1 : 0;
        j->st.attempts = (uint64_t)attempt + 1;
        j->st.max_probe = 0;
        j->st.cov_inexact_nodes = hs.cov_inexact;
        j->st.ms_insert = tm.ms(2, 3);
        j->st.ms_emit = tm.ms(3, 4) + tm.ms(5, 6);
        j->st.ms_aggregate = tm.ms(3, 4);
        j->st.ms_write = tm.ms(5, 6);
        j->st.ms_total = tm.ms(0, 6);
        return GX_OK;
    }
}

namespace gxi {

// line ends of one FASTQ file on the device; returns the line count
static gx_status fastq_lines(cudaStream_t s, RunArena &ar, const uint8_t *d, uint64_t n, unsigned long long *&le,
                             uint32_t &n_lines) {
    const uint64_t tiles = line_tiles(n);
    uint32_t *tile_cnt, *d_n;
    void *scratch;
    gx_status e;
    if ((e = ar.alloc(tile_cnt, tiles + 1)) != GX_OK) return e;
    if ((e = ar.alloc(d_n, 1)) != GX_OK) return e;
    if ((e = ar.alloc(scratch, scan_scratch_bytes(std::max<uint64_t>(tiles, 1), 8))) != GX_OK) return e;
    launch_count_lines(d, n, tile_cnt, s);
    exclusive_scan_u32(tile_cnt, tile_cnt, tiles, d_n, scratch, s);
    CK(d2h_async(&n_lines, d_n, 4, s));
    CK(sync_stream(s));
    if ((e = ar.alloc(le, n_lines)) != GX_OK) return e;
    launch_write_lines(d, n, tile_cnt, le, s);
    return GX_OK;
}

gx_status fastq_to_readid_device(cudaStream_t s, const uint8_t *h1, size_t n1, const uint8_t *h2, size_t n2,
                                 const std::function<uint8_t *(uint64_t)> &dest, uint64_t &written) {
    written = 0;
    RunArena ar(s);
    uint8_t *d1, *d2 = nullptr;
    gx_status e;
    if ((e = ar.alloc(d1, n1 + 16)) != GX_OK) return e;
    if (n1) CK(cudaMemcpyAsync(d1, h1, n1, cudaMemcpyHostToDevice, s));
    if (h2) {
        if ((e = ar.alloc(d2, n2 + 16)) != GX_OK) return e;
        if (n2) CK(cudaMemcpyAsync(d2, h2, n2, cudaMemcpyHostToDevice, s));
    }
    unsigned long long *le1, *le2 = nullptr;
    uint32_t nl1 = 0, nl2 = 0;
    if ((e = fastq_lines(s, ar, d1, n1, le1, nl1)) != GX_OK) return e;
    if (h2) {
        if ((e = fastq_lines(s, ar, d2, n2, le2, nl2)) != GX_OK) return e;
        if (nl1 != nl2) return GX_EFASTQ_PAIRING;  // GenomixDriver.java:682-686
    }
    const uint64_t n_rec = ((uint64_t)nl1 + 2) / 4;  // lines 1, 5, 9, ...
    if (!n_rec) return GX_OK;
    FqRec *rec;
    unsigned long long *len, *off;
    void *scratch;
    if ((e = ar.alloc(rec, n_rec)) != GX_OK) return e;
    if ((e = ar.alloc(len, n_rec)) != GX_OK) return e;
    if ((e = ar.alloc(off, n_rec + 1)) != GX_OK) return e;
    if ((e = ar.alloc(scratch, scan_scratch_bytes(n_rec + 1, 8))) != GX_OK) return e;
    launch_fq_lines(d1, n1, le1, d2, n2, le2, n_rec, rec, len, s);
    exclusive_scan_u64(len, off, n_rec, off + n_rec, scratch, s);
    unsigned long long total = 0;
    CK(d2h_async(&total, off + n_rec, 8, s));
    CK(sync_stream(s));
    uint8_t *out = dest(total);
    if (!out) return GX_ENOMEM;
    launch_fq_write(d1, d2, n_rec, rec, off, out, s);
    CK(sync_stream(s));
    CK(cudaGetLastError());
    written = total;
    return GX_OK;
}

gx_status prepare_text(gx_job *j) {
    // FASTQ: the reference driver's conversion (on the device), then the readid path
    if (j->o.input_kind == GX_INPUT_FASTQ) {
        const size_t nf = j->fastq[0].size();
        if (j->o.paired && j->fastq[1].size() != nf) return GX_EFASTQ_PAIRING;
        for (size_t f = 0; f < nf; f++) {
            const std::string &a = j->fastq[0][f];
            const std::string *b = j->o.paired ? &j->fastq[1][f] : nullptr;
            gx_status grow = GX_OK;
            uint64_t w = 0;
            const gx_status st = fastq_to_readid_device(
                j->ctx->stream, (const uint8_t *)a.data(), a.size(), b ? (const uint8_t *)b->data() : nullptr,
                b ? b->size() : 0,
                [&](uint64_t total) -> uint8_t * {
                    grow = ensure_text_cap(j, j->text_len + total);
                    return grow == GX_OK ? j->d_text + j->text_len : nullptr;
                },
                w);
            if (st != GX_OK) return grow != GX_OK ? grow : st;
            j->text_len += w;
        }
        j->fastq[0].clear();
        j->fastq[1].clear();
    }
    return GX_OK;
}

}  // namespace gxi

static gx_status run_job(gx_job *j) {
    cudaStream_t s = j->ctx->stream;
    Timers &tm = j->tm;
    memset(&j->st, 0, sizeof j->st);
    j->st.key_bits = j->wide ? 128 : 64;
    const int k = j->k;
    resolve_options(j);
    const bool partitioned = j->eff_algorithm != GX_ALGO_TABLE && j->o.plan == GX_PLAN_BUILD_DEBRUIJN_GRAPH;
    {
        const gx_status pe = prepare_text(j);
        if (pe != GX_OK) return pe;
    }

    const uint64_t n_text = j->text_len;
    const uint8_t *text = j->d_text;
    j->part_bounds.assign(j->o.out_parts + 1, 0);
    j->cursor.assign(j->o.out_parts, 0);
    if (n_text == 0) return GX_OK;

    RunArena ar(s);
    DevStatus *d_st;
    gx_status e;
    if ((e = ar.alloc(d_st, 1)) != GX_OK) return e;
    {
        DevStatus init{};
        init.parse_err = ~0ULL;
        CK(cudaMemcpyAsync(d_st, &init, sizeof init, cudaMemcpyHostToDevice, s));
    }
    const uint64_t tiles = line_tiles(n_text);
    uint32_t *tile_cnt, *d_nlines, *d_scnt = nullptr, *d_hll = nullptr;
    void *scratch;
    const size_t scratch_bytes = std::max(scan_scratch_bytes(std::max<uint64_t>(tiles, 1), 8),
                                          scan_scratch_bytes(n_text + 16, 8));
    if ((e = ar.alloc(tile_cnt, tiles + 1)) != GX_OK) return e;
    if ((e = ar.alloc(d_nlines, 4)) != GX_OK) return e;
    if ((e = ar.alloc(scratch, scratch_bytes)) != GX_OK) return e;

    // ---- K1 ----
    CK(cudaEventRecord(tm.ev[0], s));
    launch_count_lines(text, n_text, tile_cnt, s);
    exclusive_scan_u32(tile_cnt, tile_cnt, tiles, d_nlines, scratch, s);
    uint32_t n_lines = 0;
    CK(d2h_async(&n_lines, d_nlines, 4, s));
    CK(sync_stream(s));
    j->st.lines = n_lines;
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
    CK(cudaEventRecord(tm.ev[1], s));
    DevStatus hs;
    uint32_t n_reads = 0;
    RunCtx rc{j, s, ar, d_st, scratch, text, n_text, lines, reads, n_lines, 0, 0, d_scnt, d_hll, {}, {}};
    CK(d2h_async(&hs, d_st, sizeof hs, s));
    CK(d2h_async(&n_reads, d_nlines + 1, 4, s));
    CK(sync_stream(s));
    CK(cudaGetLastError());
    if (hs.parse_err != ~0ULL) {
        j->st.error_line = (hs.parse_err >> 8) + 1;
        return (gx_status)(hs.parse_err & 0xff);
    }
    j->st.reads = n_reads;
    j->st.kmers = hs.n_occ;
    j->st.ms_parse = tm.ms(0, 1);
    if (n_reads == 0) {
        j->st.ms_total = tm.ms(0, 1);
        return GX_OK;
    }
    rc.n_reads = n_reads;
    rc.n_occ = hs.n_occ;
    if (j->o.plan == GX_PLAN_BUILD_READ_PARSER) return build_read_parser(rc);
    return partitioned ? build_partitioned(rc) : build_table(rc);
}

void gxi::resolve_options(gx_job *j) {
    j->eff_algorithm = j->o.algorithm == GX_ALGO_TABLE ? GX_ALGO_TABLE : GX_ALGO_PARTITIONED;
    j->eff_load_factor = j->o.load_factor;
    j->eff_threads_per_read = j->o.threads_per_read > 0 ? j->o.threads_per_read : 1;
    const gx_ctx::Tuned &t = j->ctx->tuned[j->wide];
    if (j->o.algorithm == GX_ALGO_DEFAULT && j->o.load_factor == 0 && t.valid) {
        j->eff_algorithm = t.algorithm;
        j->eff_load_factor = t.load_factor;
    }
    if (j->o.threads_per_read == 0 && t.valid) j->eff_threads_per_read = t.threads_per_read;
}

double gxi::bucket_target(double load_factor) {
    return load_factor > 0 ? load_factor * AGG_SLOTS : (double)AGG_TARGET;
}

void gxi::ctx_release(gx_ctx *c) {
    if (c->refs.fetch_sub(1) != 1) return;
    cudaSetDevice(c->device);
    sync_stream(c->stream);
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
    for (auto &e : c->marks)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(c->stream);
    delete c;
}

thread_local size_t gxi::t_alloc_fail_above = 0;

gx_status gxi::run_job_locked(gx_job *j) {
    const AllocLimitScope als(j->ctx->test_alloc_fail_above);
    const uint64_t l0 = launches_this_thread();
    gx_status st = guarded("gx_job_run", [&] { return run_job(j); });
    j->st.kernel_launches = launches_this_thread() - l0;
    j->state = st == GX_OK ? JS_RAN : JS_FAILED;
    if (j->text_borrowed) {
        j->d_text = nullptr;  // the caller's buffer is no longer referenced
        j->text_borrowed = false;
    }
    return st;
}
