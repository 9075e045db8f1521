"""ctypes binding of libgxgpu.so (include/gxgpu.h).

The library is built in-tree by genomix_gb300.build; importing this module fails loudly
when it is missing — there is no CPU fallback.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgxgpu.so")

GX_OK = 0
GX_EAGAIN = 14
GX_ESTATE = 10
GX_ECANCELLED = 11
GX_EBUSY = 13
GX_ETIMEOUT = 8
CTX_TEST_WITHHOLD_COPIES = 1
STATUS_NAMES = {
    0: "GX_OK", 1: "GX_EINVAL", 2: "GX_EINVAL_LINE", 3: "GX_EINVAL_NUMBER", 4: "GX_EREADID_RANGE",
    5: "GX_EREAD_TOO_SHORT", 6: "GX_ENOMEM", 7: "GX_ETABLE_FULL", 8: "GX_ETIMEOUT", 9: "GX_ECUDA",
    10: "GX_ESTATE", 11: "GX_ECANCELLED", 12: "GX_EFASTQ_PAIRING", 13: "GX_EBUSY", 14: "GX_EAGAIN",
}
INPUT_READID, INPUT_FASTQ = 0, 1
ALGO_DEFAULT, ALGO_PARTITIONED, ALGO_TABLE = 0, 1, 2
PLAN_BUILD_DEBRUIJN_GRAPH, PLAN_BUILD_READ_PARSER = 0, 1
LAYOUT_BUCKETS, LAYOUT_REFERENCE_PARTS = 0, 1

# every symbol include/gxgpu.h declares
EXPORTS = [
    "gx_status_str", "gx_ctx_create", "gx_ctx_destroy", "gx_ctx_mark", "gx_ctx_elapsed_ms", "gx_ctx_synchronize",
    "gx_job_create", "gx_job_add_input", "gx_job_add_input_device", "gx_job_run", "gx_job_emit",
    "gx_job_emit_rewind", "gx_job_records_device", "gx_job_stats", "gx_job_destroy", "gx_batch_run", "gx_pinned_alloc",
    "gx_pinned_free", "gx_fastq_to_readid", "gx_host_free", "gx_seqfile_write", "gx_seqfile_read",
    "gx_records_to_text", "gx_build_noalloc",
    "gx_serve_create", "gx_serve_submit", "gx_serve_poll", "gx_serve_stats_get", "gx_serve_destroy",
    "gx_serve_cancel",
    "gx_records_digest", "gx_autotune", "gx_autotune_clear", "gx_job_graph_stats", "gx_seqfile_write_kmer_keys",
    "gx_fastq_to_readid_gpu", "gx_job_emit_async", "gx_job_emit_wait",
]


class CtxOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("device_mem_limit", ctypes.c_size_t), ("flags", ctypes.c_int),
                ("test_alloc_fail_above", ctypes.c_size_t)]


class JobOpts(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_size_t),
        ("kmer_length", ctypes.c_int),
        ("input_kind", ctypes.c_int),
        ("paired", ctypes.c_int),
        ("out_parts", ctypes.c_int),
        ("load_factor", ctypes.c_double),
        ("max_readids_per_edge", ctypes.c_int),
        ("threads_per_read", ctypes.c_int),
        ("est_input_bytes", ctypes.c_size_t),
        ("algorithm", ctypes.c_int),
        ("plan", ctypes.c_int),
        ("layout", ctypes.c_int),
    ]


class ServeOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("mem_budget", ctypes.c_size_t), ("lanes", ctypes.c_int),
                ("max_batch", ctypes.c_int), ("pass_bytes", ctypes.c_size_t)]


class ServeStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("jobs_submitted", "jobs_done", "batches", "max_batch_jobs",
                                                "jobs_waiting", "jobs_running", "bytes_in_use", "jobs_cancelled")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


STAT_BINS = 4096


class StatHist(ctypes.Structure):
    _fields_ = [("total", ctypes.c_uint64), ("maximum", ctypes.c_uint64), ("above", ctypes.c_uint64),
                ("bins", ctypes.c_uint64 * STAT_BINS)]

    def as_dict(self):
        nz = {i: self.bins[i] for i in range(STAT_BINS) if self.bins[i]}
        return {"total": self.total, "maximum": self.maximum, "above": self.above, "bins": nz}


class GraphStats(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t),
                ("nodes", ctypes.c_uint64), ("path_nodes", ctypes.c_uint64),
                ("tips_reverse", ctypes.c_uint64), ("tips_forward", ctypes.c_uint64),
                ("tips_both", ctypes.c_uint64), ("tips_one", ctypes.c_uint64),
                ("self_edges", ctypes.c_uint64 * 4),
                ("degree", StatHist), ("kmer_length", StatHist), ("coverage", StatHist),
                ("unflipped_read_ids", StatHist), ("flipped_read_ids", StatHist), ("seed_score", StatHist),
                ("kmer_length_with", StatHist * 2), ("coverage_with", StatHist * 2),
                ("seed_score_with", StatHist * 2)]

    def as_dict(self):
        d = {f: getattr(self, f) for f in ("nodes", "path_nodes", "tips_reverse", "tips_forward", "tips_both",
                                           "tips_one")}
        d["self_edges"] = list(self.self_edges)
        for f in ("degree", "kmer_length", "coverage", "unflipped_read_ids", "flipped_read_ids", "seed_score"):
            d[f] = getattr(self, f).as_dict()
        for f in ("kmer_length_with", "coverage_with", "seed_score_with"):
            d[f] = [getattr(self, f)[i].as_dict() for i in range(2)]
        return d


class TuneCand(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int), ("load_factor", ctypes.c_double), ("ms", ctypes.c_double),
                ("threads_per_read", ctypes.c_int)]


class TuneResult(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("algorithm", ctypes.c_int), ("load_factor", ctypes.c_double),
                ("ms", ctypes.c_double), ("tried", ctypes.c_int), ("threads_per_read", ctypes.c_int),
                ("cand", TuneCand * 16)]


class Digest(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("records", "edges", "heads", "coverage", "sum", "xor_")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [
        ("lines", ctypes.c_uint64), ("reads", ctypes.c_uint64), ("kmers", ctypes.c_uint64),
        ("nodes", ctypes.c_uint64), ("read_heads", ctypes.c_uint64), ("record_bytes", ctypes.c_uint64),
        ("table_slots", ctypes.c_uint64), ("table_partitions", ctypes.c_uint64), ("error_line", ctypes.c_uint64),
        ("cov_inexact_nodes", ctypes.c_uint64), ("max_probe", ctypes.c_uint32), ("key_bits", ctypes.c_uint32),
        ("kernel_launches", ctypes.c_uint64),
        ("ms_parse", ctypes.c_double), ("ms_insert", ctypes.c_double), ("ms_emit", ctypes.c_double),
        ("ms_total", ctypes.c_double), ("ms_aggregate", ctypes.c_double), ("ms_write", ctypes.c_double),
        ("attempts", ctypes.c_uint64), ("ms_layout", ctypes.c_double), ("super_counted", ctypes.c_uint64),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def load():
    """Loads libgxgpu.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m genomix_gb300.build` "
                          "(the graph build has no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, i, P = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER
    sig = {
        "gx_status_str": ([i], ctypes.c_char_p),
        "gx_ctx_create": ([i, P(CtxOpts), P(vp)], i),
        "gx_ctx_destroy": ([vp], None),
        "gx_ctx_mark": ([vp, i], i),
        "gx_ctx_elapsed_ms": ([vp, i, i, P(ctypes.c_double)], i),
        "gx_ctx_synchronize": ([vp], i),
        "gx_job_create": ([vp, P(JobOpts), P(vp)], i),
        "gx_job_add_input": ([vp, vp, sz, i], i),
        "gx_job_add_input_device": ([vp, vp, sz, i], i),
        "gx_job_run": ([vp], i),
        "gx_job_emit": ([vp, i, vp, sz, P(sz), P(i)], i),
        "gx_job_emit_rewind": ([vp, i], i),
        "gx_job_records_device": ([vp, P(vp), P(sz), P(P(ctypes.c_uint64))], i),
        "gx_job_stats": ([vp, P(Stats)], i),
        "gx_job_destroy": ([vp], None),
        "gx_batch_run": ([vp, P(vp), i, P(i)], i),
        "gx_pinned_alloc": ([sz, P(vp)], i),
        "gx_pinned_free": ([vp], None),
        "gx_fastq_to_readid": ([vp, sz, vp, sz, P(vp), P(sz)], i),
        "gx_host_free": ([vp], None),
        "gx_seqfile_write": ([vp, sz, vp, ctypes.c_uint64, P(vp), P(sz)], i),
        "gx_seqfile_read": ([vp, sz, P(vp), P(sz)], i),
        "gx_records_to_text": ([vp, sz, P(vp), P(sz)], i),
        "gx_build_noalloc": ([i, vp, sz, i, vp, sz, P(sz)], i),
        "gx_serve_create": ([vp, P(ServeOpts), P(vp)], i),
        "gx_serve_submit": ([vp, vp, P(ctypes.c_uint64)], i),
        "gx_serve_poll": ([vp, ctypes.c_uint64, i, P(i), P(ctypes.c_double)], i),
        "gx_serve_stats_get": ([vp, P(ServeStats)], i),
        "gx_serve_cancel": ([vp, ctypes.c_uint64], i),
        "gx_serve_destroy": ([vp], None),
        "gx_records_digest": ([vp, sz, P(Digest)], i),
        "gx_autotune": ([vp, vp, sz, i, i, P(TuneResult)], i),
        "gx_autotune_clear": ([vp], i),
        "gx_job_graph_stats": ([vp, P(GraphStats)], i),
        "gx_seqfile_write_kmer_keys": ([vp, sz, vp, ctypes.c_uint64, P(vp), P(sz)], i),
        "gx_fastq_to_readid_gpu": ([vp, vp, sz, vp, sz, P(vp), P(sz)], i),
        "gx_job_emit_async": ([vp, i, vp, sz, P(sz), P(i)], i),
        "gx_job_emit_wait": ([vp], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def status_str(st):
    return load().gx_status_str(st).decode()
