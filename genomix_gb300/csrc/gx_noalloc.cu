// gx_noalloc.cu — the graph build for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a JVM or service that hands the
// library a slice of device memory it manages itself and forbids allocation behind its
// back, code running while the device allocator is locked or exhausted, and hosts that
// budget device memory up front.  gx_build_noalloc serves them: it runs the table build
// (GX_ALGO_TABLE) of one small readid input entirely inside a fixed scratch array that the
// library holds in device memory, writing the records into a buffer the caller owns.
//
// The scratch is a file-scope __device__ array of GX_NOALLOC_SCRATCH_BYTES; every GPU that
// loads the library holds it until the process exits.  Its device address is looked up once
// per device, on the first call made with that device current (cudaGetSymbolAddress); make
// that first call before any stream capture begins.  Each call clears, on the device, the
// pieces of the array that must start at zero (the status block, the hash table, the
// per-partition head counters), so one call's leftovers never reach the next.  There is a
// single array per device: calls that overlap (two host threads at once) race on it and
// must not be made.  Inputs whose working set does not fit are refused with GX_ENOMEM and a
// message on stderr, before any kernel touches the array past its end.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gxgpu.h"
#include "gx_kernels.cuh"

using namespace gx;

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[GX_NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void *g_scratch_ptr[MAX_DEVICES] = {};

// Bump allocation inside the scratch array (256-byte aligned pieces).
struct ScratchArena {
    unsigned char *base;
    size_t used = 0, cap;
    template <class T>
    bool take(T *&p, size_t count) {
        const size_t bytes = (std::max<size_t>(count * sizeof(T), 16) + 255) & ~(size_t)255;
        if (used + bytes > cap) return false;
        p = (T *)(base + used);
        used += bytes;
        return true;
    }
};

gx_status too_big(const char *what) {
    fprintf(stderr,
            "gxgpu: gx_build_noalloc: the input needs more scratch than the %d MiB array holds (%s); "
            "use gx_job_run for inputs of this size\n",
            (int)(GX_NOALLOC_SCRATCH_BYTES >> 20), what);
    return GX_ENOMEM;
}

#define NA_CK(call)                                                                                  \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            fprintf(stderr, "gxgpu: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                                       \
            return GX_ECUDA;                                                                         \
        }                                                                                            \
    } while (0)

}  // namespace

// The build proper; the caller has made `device` current.
static gx_status build_noalloc(int device, const void *text_dev, size_t n_text, int k, void *out_dev, size_t out_cap,
                               size_t *out_bytes);

extern "C" gx_status gx_build_noalloc(int device, const void *text_dev, size_t n_text, int k, void *out_dev,
                                      size_t out_cap, size_t *out_bytes) {
    if (!out_bytes || (!text_dev && n_text) || k < 3 || k > 64 || device < 0 || device >= MAX_DEVICES)
        return GX_EINVAL;
    if (((uintptr_t)text_dev & 15) != 0 || (out_dev && ((uintptr_t)out_dev & 15) != 0)) return GX_EINVAL;
    *out_bytes = 0;
    // the caller's current device is put back on every return: a JVM thread, for one, keeps
    // using the device it had chosen
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        prev = -1;
    }
    if (cudaSetDevice(device) != cudaSuccess) return GX_ECUDA;
    const gx_status st = build_noalloc(device, text_dev, n_text, k, out_dev, out_cap, out_bytes);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return st;
}

static gx_status build_noalloc(int device, const void *text_dev, size_t n_text, int k, void *out_dev, size_t out_cap,
                               size_t *out_bytes) {
    void *scratch_base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_ptr[device]) {
            void *p = nullptr;
            NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_scratch_ptr[device] = p;
        }
        scratch_base = g_scratch_ptr[device];
    }
    if (n_text == 0) return GX_OK;
    const int wide = k > 32 ? 1 : 0;
    const cudaStream_t s = 0;  // the legacy default stream of `device`
    const uint8_t *text = (const uint8_t *)text_dev;
    ScratchArena ar{(unsigned char *)scratch_base, 0, (size_t)GX_NOALLOC_SCRATCH_BYTES};

    // ---- parse (the kernels of gx_job_run) ----
    const uint64_t tiles = line_tiles(n_text);
    DevStatus *d_st;
    uint32_t *tile_cnt, *d_nlines;
    void *scratch;
    if (!ar.take(d_st, 1) || !ar.take(tile_cnt, tiles + 1) || !ar.take(d_nlines, 4)) return too_big("line tiles");
    const size_t scan_bytes = scan_scratch_bytes(n_text + 16, 8);
    if (!ar.take(scratch, scan_bytes)) return too_big("scan");
    {
        DevStatus init{};
        init.parse_err = ~0ULL;  // the array keeps the last call's contents: start from a clean status
        NA_CK(cudaMemcpyAsync(d_st, &init, sizeof init, cudaMemcpyHostToDevice, s));
    }
    launch_count_lines(text, n_text, tile_cnt, s);
    exclusive_scan_u32(tile_cnt, tile_cnt, tiles, d_nlines, scratch, s);
    uint32_t n_lines = 0;
    NA_CK(cudaMemcpyAsync(&n_lines, d_nlines, 4, cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    unsigned long long *line_end;
    LineRec *lines;
    uint8_t *lflags;
    uint32_t *nvalid, *reads;
    if (!ar.take(line_end, n_lines) || !ar.take(lines, n_lines) || !ar.take(lflags, n_lines) ||
        !ar.take(nvalid, n_lines) || !ar.take(reads, 2ull * n_lines))
        return too_big("lines");
    launch_write_lines(text, n_text, tile_cnt, line_end, s);
    launch_parse_lines(text, n_text, line_end, n_lines, k, lines, lflags, nvalid, d_st, s);
    exclusive_scan_u32(nvalid, nvalid, n_lines, d_nlines + 1, scratch, s);
    launch_read_list(lflags, nvalid, lines, n_lines, k, reads, d_st, s);
    DevStatus hs;
    uint32_t n_reads = 0;
    NA_CK(cudaMemcpyAsync(&hs, d_st, sizeof hs, cudaMemcpyDeviceToHost, s));
    NA_CK(cudaMemcpyAsync(&n_reads, d_nlines + 1, 4, cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    NA_CK(cudaGetLastError());
    if (hs.parse_err != ~0ULL) return (gx_status)(hs.parse_err & 0xff);
    if (n_reads == 0) return GX_OK;

    // ---- table build: the geometry gx_job_run uses at the default fill (0.5); a partition
    //      that overflows retries at half the fill, up to three attempts, as gx_job_run does
    const size_t mark = ar.used;
    double lf = 0.5;
    for (int attempt = 0;; attempt++, lf *= 0.5) {
        ar.used = mark;
        const uint64_t want = (uint64_t)((double)hs.n_occ / lf) + 1;
        const uint32_t nparts = (uint32_t)std::max<uint64_t>(1, (want + PART_SLOTS - 1) / PART_SLOTS);
        const size_t slot_bytes = wide ? sizeof(Slot128) : sizeof(Slot64);
        const size_t table_bytes = (size_t)nparts * PART_SLOTS * slot_bytes;
        unsigned char *table;
        Head *heads;
        uint32_t *head_cnt, *head_off, *head_cur, *head_idx, *head_cnt2, *part_nodes;
        unsigned long long *head_sk, *part_bytes, *part_off;
        void *pscratch;
        if (!ar.take(table, table_bytes) || !ar.take(heads, n_reads) || !ar.take(head_cnt, nparts) ||
            !ar.take(head_off, nparts) || !ar.take(head_cur, nparts) || !ar.take(head_idx, n_reads) ||
            !ar.take(head_cnt2, nparts) || !ar.take(head_sk, n_reads) || !ar.take(part_nodes, nparts) ||
            !ar.take(part_bytes, nparts) || !ar.take(part_off, nparts + 1) ||
            !ar.take(pscratch, scan_scratch_bytes(nparts, 8)))
            return too_big("hash table");
        // everything that must start at zero
        NA_CK(cudaMemsetAsync(table, 0, table_bytes, s));
        NA_CK(cudaMemsetAsync(head_cnt, 0, nparts * 4ull, s));
        NA_CK(cudaMemsetAsync(head_cur, 0, nparts * 4ull, s));
        TableGeom g{table, nparts, wide};
        launch_insert(g, text, lines, reads, n_reads, k, heads, head_cnt, d_st, s);
        exclusive_scan_u32(head_cnt, head_off, nparts, nullptr, pscratch, s);
        launch_head_scatter(heads, n_reads, head_off, head_cur, head_idx, nparts, s);
        EmitArgs a{};
        a.g = g;
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
        a.st = d_st;
        launch_emit_prepare(a, s);
        exclusive_scan_u64(part_bytes, part_off, nparts, part_off + nparts, pscratch, s);
        unsigned long long total = 0;
        NA_CK(cudaMemcpyAsync(&hs, d_st, sizeof hs, cudaMemcpyDeviceToHost, s));
        NA_CK(cudaMemcpyAsync(&total, part_off + nparts, 8, cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        NA_CK(cudaGetLastError());
        if (hs.table_full) {
            if (attempt >= 2) return GX_ETABLE_FULL;
            DevStatus again{};
            again.parse_err = ~0ULL;
            again.n_occ = hs.n_occ;
            NA_CK(cudaMemcpyAsync(d_st, &again, sizeof again, cudaMemcpyHostToDevice, s));
            continue;
        }
        *out_bytes = total;
        if (!out_dev || total > out_cap) return GX_EINVAL;  // *out_bytes tells the size needed
        a.out = (uint8_t *)out_dev;
        launch_emit_write(a, s);
        NA_CK(cudaMemcpyAsync(&hs, d_st, sizeof hs, cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        NA_CK(cudaGetLastError());
        if (hs.internal_err) return GX_ECUDA;
        return GX_OK;
    }
}
