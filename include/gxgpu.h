/*
 * gxgpu.h — C ABI of libgxgpu.so, the GB300 (sm_103a) graph-build step of Genomix.
 *
 * The graph-build step reads sequencing reads, extracts every k-mer, canonicalises it
 * against its reverse complement and aggregates the occurrences into de Bruijn Node
 * records.  The records are byte-compatible with genomix-data's Writables, so a
 * SequenceFile<VKmer, Node> written from them is read unchanged by the genomix-pregelix
 * cleaning jobs (genomix-pregelix/.../base/BinaryVertexInputFormat.java:25).
 *
 * Reference interfaces this ABI replaces (paths inside the genomix project):
 *   - GenomixHyracksDriver.runJob(conf, Plan.BUILD_DEBRUIJN_GRAPH, profile)
 *       genomix-hyracks/.../graph/driver/GenomixHyracksDriver.java:84-135
 *   - the three operator plug-ins wired by JobGenBuildBrujinGraph.assignJob (:79-154):
 *       IKeyValueParserFactory  ReadsKeyValueParserFactory.java:95-254
 *       IAggregatorDescriptorFactory  AggregateKmerAggregateFactory.java:93-214
 *       ITupleWriterFactory  KmerNodePairSequenceWriterFactory.java:66-94
 *   - the FASTQ -> readid conversion GenomixDriver.convertAndUploadFastqToHDFS
 *       genomix-driver/.../driver/GenomixDriver.java:665-714
 *
 * Conventions
 *   - Every call returns a gx_status; no C++ exception crosses the ABI.
 *   - Host buffers passed in are borrowed for the duration of the call only.
 *   - Device buffers passed in (the *_device calls) are borrowed until gx_job_run returns.
 *   - The library owns all device tables; they live until gx_job_destroy.
 *   - k is a per-job value: there is no process-wide k (the reference keeps it in a
 *     JVM-wide static, Kmer.java:41-54).
 *   - A gx_ctx owns one CUDA stream.  Distinct gx_job objects may be driven from
 *     different host threads; submissions on one context are serialised by a lock.
 */
#ifndef GXGPU_H
#define GXGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The parse errors reproduce the exceptions that abort the reference job. */
typedef enum gx_status {
    GX_OK = 0,
    GX_EINVAL = 1,            /* bad argument: null pointer, k outside 3..64, bad option */
    GX_EINVAL_LINE = 2,       /* a readid line does not split into 2 or 3 tab fields:
                                 IllegalStateException, ReadsKeyValueParserFactory.java:118-122 */
    GX_EINVAL_NUMBER = 3,     /* readId field is not a Java long: NumberFormatException from
                                 Long.parseLong, ReadsKeyValueParserFactory.java:112,115 */
    GX_EREADID_RANGE = 4,     /* readId outside [0, 2^35): IllegalArgumentException,
                                 ReadHeadInfo.makeUUID, ReadHeadInfo.java:110-113 */
    GX_EREAD_TOO_SHORT = 5,   /* k >= read length: IllegalArgumentException,
                                 ReadsKeyValueParserFactory.java:152-155 */
    GX_ENOMEM = 6,            /* device or pinned allocation failed */
    GX_ETABLE_FULL = 7,       /* a hash-table partition overflowed its probe limit */
    GX_ETIMEOUT = 8,          /* a bounded device wait ran out (a bulk copy that did not land) */
    GX_ECUDA = 9,             /* a CUDA runtime call failed */
    GX_ESTATE = 10,           /* call out of order (e.g. emit before run) */
    GX_ECANCELLED = 11,       /* job cancelled (serving) */
    GX_EFASTQ_PAIRING = 12,   /* paired FASTQ streams differ in line count: IOException,
                                 GenomixDriver.java:682-686 */
    GX_EBUSY = 13,            /* serving: no admission slot or memory right now */
    GX_EAGAIN = 14            /* serving: result not ready yet */
} gx_status;

/* Text of a status code (static storage). */
const char *gx_status_str(gx_status s);

/* Input kinds (gx_job_opts.input_kind). */
enum {
    GX_INPUT_READID = 0,      /* "readId \t seq [\t mateSeq]" lines, as the graph build reads */
    GX_INPUT_FASTQ = 1        /* FASTQ; converted with the reference's readId = 4*i+2 rule */
};

typedef struct gx_ctx gx_ctx;
typedef struct gx_job gx_job;

/* gx_ctx_opts.flags (testing only): the bulk copies of the regrouping into the reference's
   parts are not issued, so its bounded waits run out (after about a second) and the job
   returns GX_ETIMEOUT; lets tests reach the timeout path without a fault. */
#define GX_CTX_TEST_WITHHOLD_COPIES 1

typedef struct gx_ctx_opts {
    size_t struct_size;       /* sizeof(gx_ctx_opts) */
    size_t device_mem_limit;  /* bytes the context may hold on the device; 0 = 90% of free */
    int flags;                /* 0, or GX_CTX_TEST_* flags (testing only) */
    size_t test_alloc_fail_above; /* testing only: any working-buffer allocation of a run on this
                                     context larger than this many bytes fails as if the device
                                     were out of memory (0 = off); lets tests reach the
                                     out-of-memory paths without exhausting the GPU */
} gx_ctx_opts;

typedef struct gx_job_opts {
    size_t struct_size;       /* sizeof(gx_job_opts) */
    int kmer_length;          /* GenomixJobConf.KMER_LENGTH; 3..64 (64-bit keys k<=32, 128-bit k<=64) */
    int input_kind;           /* GX_INPUT_READID or GX_INPUT_FASTQ */
    int paired;               /* FASTQ only: 1 = mate streams 0 and 1 are paired files */
    int out_parts;            /* output parts (SequenceFile part files); 0 means 1 */
    double load_factor;       /* fill of the hash tables aimed for; 0 = the context's autotuned choice,
                                 else the built-in default (table build: slots = occurrences / 0.5;
                                 partitioned build: 896 of 2048 per bucket) */
    int max_readids_per_edge; /* accepted and ignored, as in the reference (GenomixJobConf.java:718) */
    int threads_per_read;     /* threads that walk one read in the partitioned build's occurrence scatter,
                                 each a contiguous segment of its k-mers: 1, 2, 4, 8, 16 or 32;
                                 0 = the context's autotuned choice, else 1 */
    size_t est_input_bytes;   /* capacity hint for the device input buffer; 0 = grow on demand */
    int algorithm;            /* GX_ALGO_*: how occurrences are aggregated */
    int plan;                 /* GX_PLAN_*: what the job writes */
    int layout;               /* GX_LAYOUT_*: which records go to which output part */
} gx_job_opts;

/* Output part layouts (gx_job_opts.layout); the records are the same in both, only their
   grouping into parts differs. */
enum {
    GX_LAYOUT_BUCKETS = 0,         /* part q = a contiguous range of the build's hash buckets
                                      (no extra pass) */
    GX_LAYOUT_REFERENCE_PARTS = 1  /* part q = the records whose key the reference's partitioner
                                      sends to part q (KmerPartitionComputerFactory.java:28-52:
                                      31-hash of the packed k-mer bytes, sign-folded, mod parts),
                                      so part files hold the same record sets as the reference's
                                      part-NNNNN files; within a part the order is the build's.
                                      Graph plan only; out_parts <= 65536.  Costs a regrouping
                                      pass over the records and a second record buffer. */
};

/* Plans (gx_job_opts.plan), GenomixHyracksDriver.Plan (GenomixHyracksDriver.java:55-60). */
enum {
    GX_PLAN_BUILD_DEBRUIJN_GRAPH = 0,  /* one (VKmer, Node) record per distinct canonical k-mer */
    GX_PLAN_BUILD_READ_PARSER = 1      /* one (Kmer, Node) record per k-mer occurrence, in read order,
                                          unaggregated (JobGenReadLetterParser.java:60-147) */
};

/* Aggregation algorithms (gx_job_opts.algorithm); both give identical records. */
enum {
    GX_ALGO_DEFAULT = 0,      /* the partitioned build */
    GX_ALGO_PARTITIONED = 1,  /* stream occurrences into hash buckets, aggregate each bucket in
                                 shared memory (no random DRAM access) */
    GX_ALGO_TABLE = 2         /* one open-addressing table in HBM, CAS inserts per occurrence */
};

typedef struct gx_stats {
    uint64_t lines;           /* input lines (readid) or records (FASTQ) */
    uint64_t reads;           /* mates that passed the [ACGTacgt]+ filter */
    uint64_t kmers;           /* k-mer occurrences: sum over valid mates of (L - k + 1) */
    uint64_t nodes;           /* distinct canonical k-mers = output records */
    uint64_t read_heads;      /* read heads attached to nodes */
    uint64_t record_bytes;    /* bytes of the serialized record stream */
    uint64_t table_slots;     /* hash-table slots allocated */
    uint64_t table_partitions;
    uint64_t error_line;      /* 1-based line (or FASTQ record) that failed; 0 if none */
    uint64_t cov_inexact_nodes; /* nodes with count >= 2^24 (float coverage no longer exact) */
    uint32_t max_probe;       /* longest probe sequence seen during inserts */
    uint32_t key_bits;        /* 64 or 128 */
    uint64_t kernel_launches; /* kernels launched by gx_job_run */
    double ms_parse;          /* device time of the parse kernels */
    double ms_insert;         /* device time of k-mer extraction + table inserts */
    double ms_emit;           /* device time of compaction + record serialization */
    double ms_total;          /* device time of gx_job_run */
    double ms_aggregate;      /* device time of the per-bucket aggregation (part of ms_emit) */
    double ms_write;          /* device time of the record-writer kernel (part of ms_emit) */
    uint64_t attempts;        /* passes run: 1, plus one per table/bucket overflow retried */
    double ms_layout;         /* device time of the regrouping into the reference's parts
                                 (GX_LAYOUT_REFERENCE_PARTS; 0 otherwise) */
    uint64_t super_counted;   /* partitioned build: 1 when it counted its super buckets before
                                 scattering (a hot bucket, or room per bucket beyond the memory
                                 limit), 0 when it scattered straight away */
} gx_stats;

/* ---- context ------------------------------------------------------------------------- */

/* Create a context on CUDA device `device`.  opts may be NULL.  Replaces the connection to
 * the Hyracks cluster controller made in GenomixHyracksDriver.java:70-78. */
gx_status gx_ctx_create(int device, const gx_ctx_opts *opts, gx_ctx **out);
/* Jobs created on a context keep it alive: after gx_ctx_destroy they can still run, emit and
 * be destroyed, and the context goes with the last of them. */
void gx_ctx_destroy(gx_ctx *ctx);

/* Device-side timing on the context's stream: gx_ctx_mark records event `slot` (0..15),
 * gx_ctx_elapsed_ms waits for event b and returns the time from a to b. */
gx_status gx_ctx_mark(gx_ctx *ctx, int slot);
gx_status gx_ctx_elapsed_ms(gx_ctx *ctx, int a, int b, double *ms);
/* Wait until all work submitted on the context has finished. */
gx_status gx_ctx_synchronize(gx_ctx *ctx);

/* ---- plain (one job per launch sequence) ---------------------------------------------- */

/* Create a graph-build job.  Replaces JobGenBuildBrujinGraph's construction from a
 * GenomixJobConf (JobGenBuildBrujinGraph.java:79-90, JobGen.java:61-111). */
gx_status gx_job_create(gx_ctx *ctx, const gx_job_opts *opts, gx_job **out);

/* Append input bytes from host memory (any host memory; pinned is fastest).  Each call is
 * one input file: a final line without a terminator is still a line, as Hadoop's
 * LineRecordReader reads it.  For readid input mate_stream must be 0; for paired FASTQ,
 * 0 and 1 are the two mate files.  Replaces the HDFS read of the input splits
 * (HDFSReadOperatorDescriptor.java:98-143). */
gx_status gx_job_add_input(gx_job *job, const void *host, size_t bytes, int mate_stream);

/* Same, from device memory.  The pointer must be 16-byte aligned and stay valid until
 * gx_job_run returns.  No copy is made for a single readid input. */
gx_status gx_job_add_input_device(gx_job *job, const void *dev, size_t bytes, int mate_stream);

/* Build the graph on the device: parse, k-mer extraction, canonicalisation, aggregation
 * and serialization of every (VKmer, Node) record.  Replaces the parse -> sort -> group ->
 * merge -> group pipeline of JobGenBuildBrujinGraph.generateGroupbyKmerJob (:92-117).
 * Returns the first parse error by line order, with gx_stats.error_line set. */
gx_status gx_job_run(gx_job *job);

/* Copy the serialized records of output part `part` to host memory.  The stream is a
 * concatenation of SequenceFile record bodies: int32 BE record length, int32 BE key length,
 * VKmer key, Node value (the bytes SequenceFile.Writer.append writes for one record,
 * KmerNodePairSequenceWriterFactory.java:79-94).  Repeated calls continue where the last
 * stopped; *more is 1 while bytes remain.  Each call ends on a record boundary. */
gx_status gx_job_emit(gx_job *job, int part, void *host_out, size_t cap, size_t *written, int *more);

/* gx_job_emit, but the copy is only queued (on the context's copy stream, which runs beside its
 * build stream): it overlaps whatever the context does next, e.g. the next job's build.  The
 * host buffer must not be read or reused until gx_job_emit_wait(job) returns; any other call
 * on the job waits for the copy first.  *written and *more are final when the call returns.
 * No counterpart in the reference (its writer streams to HDFS synchronously). */
gx_status gx_job_emit_async(gx_job *job, int part, void *host_out, size_t cap, size_t *written, int *more);
gx_status gx_job_emit_wait(gx_job *job);

/* Restart gx_job_emit of output part `part` (-1: every part) from its first record. */
gx_status gx_job_emit_rewind(gx_job *job, int part);

/* Device view of the whole record stream (all parts in order) and the per-part byte
 * offsets (out_parts + 1 entries, host memory, owned by the job). */
gx_status gx_job_records_device(gx_job *job, const void **dev, size_t *bytes,
                                const uint64_t **part_offsets);

/* Statistics of the last gx_job_run. */
gx_status gx_job_stats(const gx_job *job, gx_stats *out);

void gx_job_destroy(gx_job *job);

/* ---- batched: many jobs in one pass over the device ---------------------------------- */

/* Run n jobs of one context together.  Every job must have its inputs added and not yet
 * have run.  Jobs with the same k go through one partitioned build: one parse of all their
 * text, then one bucket space in which every job owns its own contiguous range of buckets
 * sized from its own distinct-k-mer estimate, so each job's Node set is exactly its
 * gx_job_run result (records may come in a different order).  Per-job results are read as
 * usual (gx_job_emit, gx_job_stats); the ms_* and kernel_launches fields describe the whole
 * pass.  Jobs with GX_ALGO_TABLE, and every job of a pass in which some input fails to parse
 * (so that each reports its own status and line), run one by one.  Per-job status codes go
 * to statuses[i] (may be NULL); the call returns the first non-OK status.  Replaces running
 * one Hyracks job per read set (GenomixHyracksDriver.java:84-135 per sample). */
gx_status gx_batch_run(gx_ctx *ctx, gx_job **jobs, int n, gx_status *statuses);

/* ---- graph statistics on the device-resident graph ------------------------------------- */

#define GX_STAT_BINS 4096

/* One statistic: its total over the nodes, its maximum, and how many nodes had each value
 * (values >= GX_STAT_BINS are counted in `above`). */
typedef struct gx_stat_hist {
    uint64_t total, maximum, above;
    uint64_t bins[GX_STAT_BINS];
} gx_stat_hist;

/* The counters GraphStatistics.map collects (genomix-hadoop/.../utils/GraphStatistics.java:
 * 78-131) over a job's nodes: "totals", "maximum" and "<name>-bins" of each statistic. */
typedef struct gx_graph_stats {
    size_t struct_size;   /* sizeof(gx_graph_stats), set by the caller */
    uint64_t nodes, path_nodes;
    uint64_t tips_reverse, tips_forward, tips_both, tips_one;
    uint64_t self_edges[4];                      /* selfEdge-FF, -FR, -RF, -RR */
    gx_stat_hist degree, kmer_length, coverage;  /* coverage = Math.round(averageCoverage) */
    gx_stat_hist unflipped_read_ids, flipped_read_ids;
    gx_stat_hist seed_score;                     /* k * read heads, for coverage in 0 +- 1000 */
    gx_stat_hist kmer_length_with[2], coverage_with[2], seed_score_with[2];  /* [0] REVERSE, [1] FORWARD */
} gx_graph_stats;

/* Statistics of a job's graph, computed on the GPU from its device-resident records (the
 * graph never leaves the device).  Replaces the GraphStatistics MapReduce job run over the
 * graph-build output (GraphStatistics.run, :136-152; GenomixDriver.java:120-137 for the
 * coverage cutoff). */
gx_status gx_job_graph_stats(gx_job *job, gx_graph_stats *out);

/* ---- autotuning ------------------------------------------------------------------------ */

#define GX_TUNE_MAX 16

typedef struct gx_tune_result {
    size_t struct_size;  /* sizeof(gx_tune_result), set by the caller */
    int algorithm;       /* the fastest: GX_ALGO_PARTITIONED or GX_ALGO_TABLE */
    double load_factor;  /* and its fill: the bucket width of the partitioned build (distinct
                            k-mers per 2048-slot bucket table), the table build's load factor */
    double ms;           /* its device time on the sample */
    int tried;
    int threads_per_read;  /* and its tiling of the k-mer walk (partitioned build) */
    struct {
        int algorithm;
        double load_factor;
        double ms;       /* best of the repeats; < 0 if the candidate failed */
        int threads_per_read;
    } cand[GX_TUNE_MAX];
} gx_tune_result;

/* Time every candidate (algorithm x fill x threads per read) on `sample` (readid text in host memory, e.g. the
 * first tens of MB of a run's input) `repeats` times (0 = 2) and keep the fastest in the
 * context for k-mers of k's key width (64-bit for k <= 32, 128-bit above): jobs created with
 * GX_ALGO_DEFAULT, load_factor 0 and threads_per_read 0 then use it, in gx_job_run,
 * gx_batch_run and serving.
 * The reference has no counterpart (its sort-based aggregation has no such parameters). */
gx_status gx_autotune(gx_ctx *ctx, const void *sample, size_t bytes, int k, int repeats, gx_tune_result *out);
/* Forget the tuned choices: jobs at the defaults use the built-in settings again. */
gx_status gx_autotune_clear(gx_ctx *ctx);

/* ---- serving: graph builds admitted as they arrive ------------------------------------ */

typedef struct gx_server gx_server;

typedef struct gx_serve_opts {
    size_t struct_size;  /* sizeof(gx_serve_opts) */
    size_t mem_budget;   /* device bytes the admitted jobs may use together; 0 = the context's limit */
    int lanes;           /* passes in flight at once, each on its own stream; 0 = 4 */
    int max_batch;       /* jobs admitted into one pass; 0 = 64 */
    size_t pass_bytes;   /* estimated device bytes one pass admits; its first job always goes in, so a
                            job above this runs in a pass of its own and small jobs never wait for a
                            large one's pass; 0 = 2 GiB */
} gx_serve_opts;

typedef struct gx_serve_stats {
    uint64_t jobs_submitted, jobs_done;
    uint64_t batches;         /* passes run */
    uint64_t max_batch_jobs;  /* most jobs admitted into one pass */
    uint64_t jobs_waiting, jobs_running;
    uint64_t bytes_in_use;    /* estimated device bytes of the running jobs */
    uint64_t jobs_cancelled;  /* withdrawn by gx_serve_cancel before they started */
} gx_serve_stats;

/* Start a server on ctx's device.  Each lane is a context of its own with one worker thread.
 * An idle lane admits, in arrival order, every waiting job whose estimated device memory
 * (from its input size) fits the budget next to the jobs already running and the pass's
 * pass_bytes, up to max_batch, and runs them as one gx_batch_run pass; jobs that arrive
 * meanwhile wait for the next free lane, so batches form continuously and the lanes' passes
 * overlap on the device.  The oldest waiting job is always admitted when nothing runs, and
 * always opens the pass it is admitted to.  Large jobs (estimated above a quarter of
 * pass_bytes) hold at most lanes - 1 lanes at a time, so small jobs always find a lane; while
 * they do, an idle lane passes over the large jobs waiting.  Replaces submitting one
 * GenomixHyracksDriver.runJob (GenomixHyracksDriver.java:84-135) per request; the
 * reference has no serving mode. */
gx_status gx_serve_create(gx_ctx *ctx, const gx_serve_opts *opts, gx_server **out);
/* Hand a job with its inputs added (not yet run) to the server.  The job belongs to the
 * server until gx_serve_poll reports it done: make no call on it before that.  Its results
 * then stay device-resident in the job (gx_job_emit, gx_job_records_device) until
 * gx_job_destroy.  GX_EBUSY once the server is being destroyed. */
gx_status gx_serve_submit(gx_server *srv, gx_job *job, uint64_t *ticket);
/* Wait up to timeout_ms (0: do not wait, < 0: wait until done) for a ticket.  GX_EAGAIN if
 * it is not done yet; GX_OK once done, with the job's own status and its latency from
 * submission to completion (the ticket is then released). */
gx_status gx_serve_poll(gx_server *srv, uint64_t ticket, int timeout_ms, gx_status *job_status,
                        double *latency_ms);
/* Withdraw a job that has not started yet: GX_OK, and the ticket's gx_serve_poll then reports
 * GX_ECANCELLED; the job is the caller's again, unrun (destroy it, or submit it anew).
 * GX_EBUSY when the job is already running (it completes as usual), GX_ESTATE when it is done,
 * GX_EINVAL for an unknown ticket.  The reference has no counterpart: a Hyracks job is
 * aborted as a whole (GenomixHyracksDriver.java:132-134). */
gx_status gx_serve_cancel(gx_server *srv, uint64_t ticket);
gx_status gx_serve_stats_get(gx_server *srv, gx_serve_stats *out);
/* Runs every job still queued, then stops the lanes. */
void gx_serve_destroy(gx_server *srv);

/* ---- graph build without device allocation ------------------------------------------- */

/* Bytes of the device scratch array behind gx_build_noalloc. */
#define GX_NOALLOC_SCRATCH_BYTES (32u << 20)

/* Graph build of one small readid input, for callers that cannot allocate device memory:
 * a JVM or service that manages its own slice of device memory and forbids allocations
 * behind its back, or a process whose device allocator is exhausted or locked.  The call
 * makes no cudaMalloc, cudaFree or other allocating call; all working memory comes from a
 * file-scope device array of GX_NOALLOC_SCRATCH_BYTES, which every GPU that loads this
 * library holds until the process exits.  The caller passes the readid text (device memory,
 * 16-byte aligned) and a device output buffer (16-byte aligned, out_cap bytes) that
 * receives the same record stream gx_job_run writes with algorithm GX_ALGO_TABLE.
 *  - The first call on a device looks up the array's device address with that device
 *    current; make that first call before any stream capture.  The address is kept for the
 *    life of the process: after a cudaDeviceReset of that device this call must not be used
 *    on it again.
 *  - Work runs on the legacy default stream of `device`; the call returns when it is done,
 *    with the caller's current device as it was before the call.
 *  - A hash-table partition that overflows is retried at half the fill, up to three
 *    attempts, as gx_job_run's table build does; GX_ETABLE_FULL after the third.
 *  - Calls share the one array (each starts by clearing what must start at zero): calls
 *    that overlap on the GPU, from different host threads, race and must not be made.
 *  - An input whose working set does not fit the array returns GX_ENOMEM with a message
 *    on stderr (about 800,000 k-mer occurrences fit for k <= 32, half that above).
 *    An output buffer that is too small (or NULL) returns GX_EINVAL with *out_bytes set
 *    to the size needed; the next call with a larger buffer repeats the whole build.
 * No counterpart in the reference: its graph build always runs on the JVM heap. */
gx_status gx_build_noalloc(int device, const void *text_dev, size_t n_text, int k, void *out_dev, size_t out_cap,
                           size_t *out_bytes);

/* ---- host helpers -------------------------------------------------------------------- */

/* Page-locked host memory, suitable for direct ByteBuffers / FFM MemorySegments. */
gx_status gx_pinned_alloc(size_t bytes, void **out);
void gx_pinned_free(void *ptr);

/* Convert FASTQ to readid text exactly as GenomixDriver.convertAndUploadFastqToHDFS does
 * (GenomixDriver.java:665-714): record i gets readId 4*i+2; sequence lines are trimmed;
 * paired input writes "id \t mate1 \t mate2".  mate2 may be NULL for single-end input.
 * *out is allocated with malloc; free it with gx_host_free. */
gx_status gx_fastq_to_readid(const void *mate1, size_t bytes1, const void *mate2, size_t bytes2,
                             char **out, size_t *out_bytes);
/* The same conversion run on the GPU of `ctx` (what jobs with GX_INPUT_FASTQ do): byte for
 * byte gx_fastq_to_readid's output.  *out is malloc'ed (gx_host_free). */
gx_status gx_fastq_to_readid_gpu(gx_ctx *ctx, const void *mate1, size_t bytes1, const void *mate2, size_t bytes2,
                                 char **out, size_t *out_bytes);
void gx_host_free(void *ptr);

/* Write one Hadoop SequenceFile (version 6, uncompressed, key class
 * edu.uci.ics.genomix.data.types.VKmer, value class edu.uci.ics.genomix.data.types.Node)
 * from a record stream as returned by gx_job_emit.  sync (16 bytes) is the file's sync
 * marker; NULL derives a deterministic marker from `seed`.  Replaces the SequenceFile.Writer
 * opened in KmerNodePairSequenceWriterFactory.java:66-73.  *out is malloc'ed. */
gx_status gx_seqfile_write(const void *records, size_t bytes, const uint8_t *sync, uint64_t seed,
                           uint8_t **out, size_t *out_bytes);

/* The same container with key class edu.uci.ics.genomix.data.types.Kmer: the part files of
 * the read-parser plan (JobGenReadLetterParser.java:100-103). */
gx_status gx_seqfile_write_kmer_keys(const void *records, size_t bytes, const uint8_t *sync, uint64_t seed,
                                     uint8_t **out, size_t *out_bytes);

/* Extract the record stream from a SequenceFile written by gx_seqfile_write or by Hadoop
 * (uncompressed).  *out is malloc'ed. */
gx_status gx_seqfile_read(const void *file, size_t bytes, uint8_t **out, size_t *out_bytes);

/* Order-independent digest of a record stream: every record hashed in its normal form
 * (each edge list's elements in byte order, read-head sets in their TreeSet order), the
 * hashes combined by sum and by xor; with counts of records, edges, read heads and the
 * coverage total.  Two streams hold the same Node set exactly when their digests agree
 * (up to hash collisions).  A verification helper with no counterpart in the reference (its
 * tests compare sorted text dumps, TestUtils.java:67-181). */
typedef struct gx_digest {
    uint64_t records, edges, heads, coverage;
    uint64_t sum, xor_;
} gx_digest;
gx_status gx_records_digest(const void *records, size_t bytes, gx_digest *out);

/* Text dump of a record stream, one line per record in the form
 * key.toString() + "\t" + value.toString() that GenomixClusterManager.copyBinAndTextToLocal
 * writes (GenomixClusterManager.java:371; Node.toString Node.java:524-537).  *out is malloc'ed. */
gx_status gx_records_to_text(const void *records, size_t bytes, char **out, size_t *out_bytes);

#ifdef __cplusplus
}
#endif

#endif /* GXGPU_H */
