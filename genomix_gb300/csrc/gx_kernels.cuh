// gx_kernels.cuh — declarations of the graph-build kernels and their host launchers.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "gx_device.cuh"

namespace gx {

// ---- geometry ---------------------------------------------------------------------------
constexpr int LINE_TILE_THREADS = 256;
constexpr int LINE_TILE_VECS = 4;  // uint4 per thread
constexpr uint64_t LINE_TILE_BYTES = (uint64_t)LINE_TILE_THREADS * LINE_TILE_VECS * 16;

constexpr int PART_SLOTS_LOG2 = 11;  // slots per table partition (both key widths)
constexpr uint32_t PART_SLOTS = 1u << PART_SLOTS_LOG2;
constexpr int EMIT_THREADS = 256;
constexpr uint32_t HEAD_CAP = 1024;         // read heads per partition sorted in shared memory
constexpr uint32_t EMIT_STAGE_BYTES = 16384;  // output staging window per partition CTA

// Kernel launches made by the calling host thread (read before and after a run).
uint64_t launches_this_thread();

// Device -> host reads of a build (counts, status, offsets).  A small kernel copies the bytes
// into this thread's mapped pinned staging buffer, so no copy engine is involved: a large
// record copy running on a copy engine meanwhile (gx_job_emit_async) cannot delay them.
// d2h_async queues one read on stream s; sync_stream synchronizes s and delivers the queued
// reads to their host destinations.
cudaError_t d2h_async(void *dst, const void *src, size_t bytes, cudaStream_t s);
cudaError_t sync_stream(cudaStream_t s);
extern thread_local uint64_t t_launches;  // incremented by every launcher

// ---- scans (device-wide, exclusive) -----------------------------------------------------
// Scratch needed by exclusive_scan for n items of T.
size_t scan_scratch_bytes(uint64_t n, size_t elem);
// out[i] = sum(in[0..i)); total (device pointer, may be null) = sum(in[0..n)).  in == out allowed.
void exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total, void *scratch,
                        cudaStream_t s);
void exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, uint64_t n,
                        unsigned long long *total, void *scratch, cudaStream_t s);

// ---- parse ------------------------------------------------------------------------------
uint64_t line_tiles(uint64_t n_text);
void launch_count_lines(const uint8_t *text, uint64_t n, uint32_t *tile_cnt, cudaStream_t s);
void launch_write_lines(const uint8_t *text, uint64_t n, const uint32_t *tile_off, unsigned long long *line_end,
                        cudaStream_t s);
void launch_parse_lines(const uint8_t *text, uint64_t n_text, const unsigned long long *line_end, uint32_t n_lines,
                        int k, LineRec *lines, uint8_t *lflags, uint32_t *nvalid, DevStatus *st, cudaStream_t s);
void launch_read_list(const uint8_t *lflags, const uint32_t *read_off, const LineRec *lines, uint32_t n_lines, int k,
                      uint32_t *reads, DevStatus *st, cudaStream_t s);

// ---- build ------------------------------------------------------------------------------
struct TableGeom {
    void *table;        // Slot64[] or Slot128[]
    uint32_t nparts;    // partitions
    int wide;           // 0: 64-bit keys, 1: 128-bit keys
};
void launch_insert(const TableGeom &g, const uint8_t *text, const LineRec *lines, const uint32_t *reads,
                   uint32_t n_reads, int k, Head *heads, uint32_t *head_cnt, DevStatus *st, cudaStream_t s);
void launch_head_scatter(const Head *heads, uint32_t n_reads, const uint32_t *head_off, uint32_t *head_cur,
                         uint32_t *head_idx, uint32_t nparts, cudaStream_t s);
// The same scatter for the partitioned build, which also gathers each head's HeadIn record
// into hsorted (same positions as head_idx).
void launch_head_scatter_part(const Head *heads, const uint32_t *reads, const LineRec *lines, uint32_t n_reads,
                              const uint32_t *head_off, uint32_t *head_cur, uint32_t *head_idx, HeadIn *hsorted,
                              cudaStream_t s);

// ---- emission ---------------------------------------------------------------------------
struct EmitArgs {
    TableGeom g;
    int k;
    const uint8_t *text;
    uint64_t n_text;             // bytes of text (the head writer reads no byte past them)
    const LineRec *lines;
    const uint32_t *reads;
    Head *heads;
    uint32_t *head_idx;          // read ordinals bucketed by partition, sorted in place
    unsigned long long *head_sk; // scratch sort keys for partitions above HEAD_CAP
    const uint32_t *head_off;
    const uint32_t *head_cnt;
    uint32_t *head_cnt2;         // heads kept after de-duplication
    uint32_t *part_nodes;
    unsigned long long *part_bytes;
    const unsigned long long *part_off;
    uint8_t *out;
    DevStatus *st;
    // partitioned build: compacted nodes of partition p at node_base[p] in nkey / ncm
    const void *nkey = nullptr;
    const unsigned long long *ncm = nullptr;
    const unsigned long long *node_base = nullptr;
    const uint32_t *noff = nullptr;
    const HeadOut *hout = nullptr;
    uint64_t n_head_slots = 0;   // entries of hout: kept heads and dropped duplicates
    uint32_t max_seq = 0;        // longest sequence of a kept read head (0: not known)
};
void launch_emit_prepare(const EmitArgs &a, cudaStream_t s);
void launch_emit_write(const EmitArgs &a, cudaStream_t s);

// ---- partitioned build --------------------------------------------------------------------
// Occurrences are streamed into S super buckets (top hash bits), each super bucket into F
// fine buckets; a fine bucket's distinct k-mers are aggregated in a shared-memory table.
constexpr int HLL_REGS = 2048;               // HyperLogLog registers for the distinct estimate
constexpr uint32_t AGG_SLOTS = 2048;         // shared-memory table of one fine bucket
constexpr uint32_t AGG_TARGET = 896;         // distinct k-mers per fine bucket aimed for
constexpr uint32_t CHUNK = 4096;             // occurrences per CTA in the fine passes
constexpr int SC_THREADS = 256;              // super scatter: one read per thread
constexpr int SC_HLL_REGS = 512;             // HyperLogLog registers kept by the super scatter
// A super scatter without a counting pass first: every super bucket gets room for this share of
// the mean bucket plus SC_SLACK; a bucket that needs more sets the overflow flag.
constexpr double SC_ROOM = 1.3;
constexpr uint32_t SC_SLACK = 8192;
constexpr uint32_t MAX_SUPERS = 2048, MAX_FINE = 2048;

struct PartPlan {
    uint32_t log_s;  // S = 1 << log_s super buckets
    uint32_t F;      // fine buckets per super bucket
    uint32_t P;      // S * F
};
// distinct k-mer estimate from the HyperLogLog registers
double hll_estimate(const uint32_t *regs, int n_regs = HLL_REGS);
PartPlan plan_partitions(double distinct_est, double safety, double target);

// Bucket plan of one sample.  A batch of samples shares one bucket space: sample s owns the
// super buckets [super_base, super_base + 2^log_s) and the fine buckets
// [fine_base, fine_base + 2^log_s * F), so its records come out as one contiguous run.  A
// plain job is a batch of one sample with super_base = fine_base = 0.
struct SamplePlan {
    uint32_t super_base;
    uint32_t log_s;  // 0 allowed: one super bucket
    uint32_t F;      // fine buckets per super bucket
    uint32_t fine_base;
};
// Per global super bucket: its first global fine bucket, its fine-bucket count and the
// owning sample's log_s (the hash bits below the super bits pick the fine bucket).
struct SuperInfo {
    uint32_t fine_first, F, log_s, pad;
};
// Reads of sample s are [read_base[s], read_base[s + 1]).
struct SampleMap {
    const uint32_t *read_base;  // n + 1 entries
    const SamplePlan *plan;     // n entries
    uint32_t n;
};

void launch_count_occ(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines, const uint32_t *reads,
                      const uint32_t *n_reads_dev, uint32_t n_reads_max, int k, uint32_t log_s, uint32_t *s_cnt,
                      uint32_t *hll, cudaStream_t s);
// Batched A1: per sample, MAX_SUPERS super counts (top 11 hash bits) and HLL_REGS
// HyperLogLog registers, at s_cnt + s * MAX_SUPERS and hll + s * HLL_REGS.
void launch_count_occ_batch(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines,
                            const uint32_t *reads, const uint32_t *read_base, uint32_t n_samples,
                            uint32_t n_reads_max, int k, uint32_t *s_cnt, uint32_t *hll, cudaStream_t s);
// read_base[s] for each sample from the text offset where the sample starts: the first line
// that starts at or after text_base[s] (line_end: exclusive line ends; nvalid: exclusive
// scan of valid mates per line, total at nvalid_total).
void launch_sample_bounds(const unsigned long long *text_base, uint32_t n_samples,
                          const unsigned long long *line_end, uint32_t n_lines, const uint32_t *nvalid,
                          const uint32_t *nvalid_total, uint32_t *line_base, uint32_t *read_base, cudaStream_t s);
// Occurrences (L - k + 1 summed over its reads) of every sample, added into occ[sample]; the
// reads are m.read_base[m.n] (on the device), at most n_reads_max.
void launch_sample_occ(const LineRec *lines, const uint32_t *reads, uint32_t n_reads_max, int k, SampleMap m,
                       unsigned long long *occ, cudaStream_t s);
// The super scatter.  cap: room per super bucket (0: s_off[i + 1] - s_off[i]); a bucket out of
// room sets *ovf and is not written.  hll (may be null): SC_HLL_REGS registers per sample.
void launch_scatter_super(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines,
                          const uint32_t *reads, uint32_t n_reads, int k, SampleMap m, uint32_t n_super,
                          const unsigned long long *s_off, uint32_t *s_cur, void *okey, uint16_t *obits,
                          uint32_t cap, uint32_t *hll, uint32_t *ovf, cudaStream_t s, uint32_t tpr = 1);
// chunks: (start, super << 32 | length) of CHUNK-sized pieces of each super bucket
void launch_make_chunks(const unsigned long long *soff, const uint32_t *scount, const uint32_t *cbase, uint32_t S,
                        ulonglong2 *chunks, cudaStream_t s);
void launch_fine_count(int wide, const void *okey, const ulonglong2 *chunks, uint32_t n_chunks,
                       const SuperInfo *sinfo, unsigned long long *fine_cnt, cudaStream_t s);
void launch_scatter_fine(int wide, const void *okey, const uint16_t *obits, const ulonglong2 *chunks,
                         uint32_t n_chunks, const SuperInfo *sinfo, const unsigned long long *fine_off,
                         uint32_t *fine_cur, void *okey2, uint16_t *obits2, cudaStream_t s);
void launch_heads_part(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines, const uint32_t *reads,
                       uint32_t n_reads, int k, SampleMap m, Head *heads, uint32_t *head_cnt, cudaStream_t s);
struct AggArgs {
    int wide;
    int k;
    PartPlan pp;
    const void *okey2;
    const uint16_t *obits2;
    const unsigned long long *fine_off;
    const LineRec *lines;
    const uint32_t *reads;
    Head *heads;
    uint32_t *head_idx;
    const HeadIn *hsorted;      // the heads in bucket order (positions of head_idx)
    unsigned long long *head_sk;
    const uint32_t *head_off;
    const uint32_t *head_cnt;
    uint32_t *head_cnt2;
    void *nkey;                 // node keys (written over okey2)
    unsigned long long *ncm;    // count | meta << 32
    uint32_t *noff;             // partition-local byte offset of each node's record
    HeadOut *hout;              // read heads in output order (indexed like head_idx)
    uint32_t *part_nodes;
    unsigned long long *part_bytes;
    DevStatus *st;
};
void launch_aggregate(const AggArgs &a, cudaStream_t s);

// the reference's part layout: each record's part (Java 31-hash of its key, modulo nparts),
// a stable counting sort of record indexes by part (8-bit digits at `shift`; val NULL means
// the identity), lengths in the new order, and the copy
void launch_rl_index(const uint8_t *rec, const unsigned long long *seg, const uint32_t *node_base,
                     uint32_t n_seg, uint32_t nparts, uint32_t *rpart, unsigned long long *roff, uint32_t *rlen,
                     cudaStream_t s);
uint32_t rl_tiles(uint64_t n);
void launch_rl_count(const uint32_t *key, const uint32_t *val, uint64_t n, int shift, uint32_t *cnt, cudaStream_t s);
void launch_rl_scatter(const uint32_t *key, const uint32_t *val, uint64_t n, int shift, const uint32_t *off,
                       uint32_t *out_val, cudaStream_t s);
void launch_rl_gather_len(const uint32_t *perm, const uint32_t *rlen, uint64_t n, unsigned long long *len2,
                          cudaStream_t s);
void launch_rl_copy(const uint8_t *src, const uint32_t *perm, const unsigned long long *roff,
                    const unsigned long long *noff, const uint32_t *rlen, uint64_t n, uint8_t *dst, cudaStream_t s);
void launch_rl_index_nodes(const void *nkey, int wide, int k, const unsigned long long *part_off,
                           const unsigned long long *node_base, const uint32_t *noff, const uint32_t *dense_base,
                           const uint32_t *part_nodes, uint32_t n_buckets, uint32_t nparts, uint32_t *rpart,
                           unsigned long long *roff, uint32_t *rlen, cudaStream_t s);
// Up to 256 parts: per tile and part byte counts into cnt ([part][tile], parts x tiles + 1 entries,
// scanned in place, the total last), then the records moved to their places in dst.  Tiles are
// RL_TILE records of the arrays, or the buckets of the partitioned build.
// The source bytes of each round arrive by bulk copy; *err is set when a copy did not land
// within about a second (withhold != 0: the copies are not issued, for testing that path).
void launch_rl_regroup_arrays(const uint8_t *sbytes, const uint32_t *rpart, const uint32_t *rlen,
                              const unsigned long long *roff, uint64_t n, uint32_t nparts, unsigned long long *cnt,
                              void *scratch, uint8_t *dst, uint32_t *err, int withhold, cudaStream_t s);
void launch_rl_regroup_nodes(const uint8_t *sbytes, const void *nkey, int wide, int k, const uint32_t *noff,
                             const unsigned long long *node_base, const unsigned long long *part_off,
                             const uint32_t *part_nodes, uint32_t n_buckets, uint32_t nparts, unsigned long long *cnt,
                             void *scratch, uint8_t *dst, uint32_t *err, int withhold, cudaStream_t s);
void launch_rl_part_starts(const unsigned long long *off, uint32_t n_tiles, uint32_t nparts, unsigned long long total,
                           unsigned long long *bounds, cudaStream_t s);
void launch_rl_bounds(const uint32_t *rpart, const uint32_t *perm, uint64_t n, uint32_t nparts,
                      const unsigned long long *noff, unsigned long long *bounds, cudaStream_t s);
void launch_rl_sample(const unsigned long long *noff, uint64_t n, uint32_t stride, uint64_t m,
                      unsigned long long *out, cudaStream_t s);

// FASTQ -> readid on the device: each record's trimmed sequence line(s) and output length,
// then the readid lines at their scanned offsets
struct FqRec {
    unsigned long long b1, e1, b2, e2;
};
void launch_fq_lines(const uint8_t *t1, uint64_t n1, const unsigned long long *le1, const uint8_t *t2, uint64_t n2,
                     const unsigned long long *le2, uint64_t n_rec, FqRec *rec, unsigned long long *len,
                     cudaStream_t s);
void launch_fq_write(const uint8_t *t1, const uint8_t *t2, uint64_t n_rec, const FqRec *rec,
                     const unsigned long long *off, uint8_t *out, cudaStream_t s);

// the BUILD_READ_PARSER plan: bytes of each read's per-occurrence records, then the records
void launch_rp_sizes(const LineRec *lines, const uint32_t *reads, uint32_t n_reads, int k,
                     unsigned long long *rbytes, cudaStream_t s);
void launch_rp_write(int wide, const uint8_t *text, uint64_t n_text, const LineRec *lines, const uint32_t *reads,
                     uint32_t n_reads, int k, const unsigned long long *roff, uint8_t *out, cudaStream_t s);
// record writer of the partitioned build (node offsets and head positions precomputed)
void launch_emit_write_part(const EmitArgs &a, cudaStream_t s);

}  // namespace gx
