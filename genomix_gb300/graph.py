"""Host-side mirror of the Genomix graph-build interface over libgxgpu.so.

    GenomixGpuDriver.run_job(conf, plan)  ~ GenomixHyracksDriver.runJob
        (genomix-hyracks/.../graph/driver/GenomixHyracksDriver.java:84-135)
    GraphBuildJob                          ~ one BUILD_DEBRUIJN_GRAPH job: the parser,
        aggregator and writer plug-ins of JobGenBuildBrujinGraph (:79-154) in one object
    GenomixJobConf keys                    ~ GenomixJobConf.java:303-370

Failures raise GraphBuildError carrying the library status; parse failures carry the
1-based input line, like the exceptions that abort the reference job.
"""
import ctypes
import os

import numpy as np

from . import _lib

# GenomixJobConf keys read by the graph build (GenomixJobConf.java:303-370) and the Hadoop
# keys FileInputFormat / FileOutputFormat store the paths under.
KMER_LENGTH = "genomix.conf.kmerLength"
SINGLE_END_FASTQ_INPUTS = "genomix.conf.singleEndFastqInputs"
PAIRED_END_FASTQ_INPUTS = "genomix.conf.pairedEndFastqInputs"
MAX_READIDS_PER_EDGE = "genomix.maxReadidsPerEdge"
INPUT_DIR = "mapred.input.dir"
OUTPUT_DIR = "mapred.output.dir"
THREADS_PER_MACHINE = "genomix.threadsPerMachine"


class GraphBuildError(RuntimeError):
    def __init__(self, status, where="", line=0):
        self.status = status
        self.name = _lib.STATUS_NAMES.get(status, str(status))
        self.line = line
        msg = f"{where}: {self.name} ({_lib.status_str(status)})"
        if line:
            msg += f" at input line {line}"
        super().__init__(msg)


def _check(st, where, line=0):
    if st != _lib.GX_OK:
        raise GraphBuildError(st, where, line)


def _host_ptr(data):
    """(pointer, nbytes, keepalive) of a host buffer: bytes, bytearray, numpy, memoryview,
    PinnedBuffer or a CPU torch tensor."""
    if isinstance(data, PinnedBuffer):
        return data.ptr, data.nbytes, data
    if isinstance(data, bytes):
        buf = ctypes.c_char_p(data)
        return ctypes.cast(buf, ctypes.c_void_p).value, len(data), (data, buf)
    if hasattr(data, "data_ptr") and hasattr(data, "is_cuda"):
        if data.is_cuda:
            raise ValueError("device tensor: use add_input_device")
        t = data.contiguous()
        return t.data_ptr(), t.numel() * t.element_size(), t
    arr = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if not isinstance(data, np.ndarray) else data)
    return arr.ctypes.data, arr.nbytes, arr


class PinnedBuffer:
    """Page-locked host memory from gx_pinned_alloc (a direct ByteBuffer in the Java shim)."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        _check(_lib.load().gx_pinned_alloc(self.nbytes, ctypes.byref(p)), "gx_pinned_alloc")
        self.ptr = p.value

    def array(self):
        if not self.nbytes:
            return np.zeros(0, np.uint8)
        return np.ctypeslib.as_array((ctypes.c_uint8 * self.nbytes).from_address(self.ptr))

    def close(self):
        if self.ptr:
            _lib.load().gx_pinned_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A device and its stream (replaces the Hyracks cluster-controller connection)."""

    def __init__(self, device=0, mem_limit=0, test_alloc_fail_above=0, test_flags=0):
        L = _lib.load()
        self._L = L
        opts = _lib.CtxOpts(ctypes.sizeof(_lib.CtxOpts), mem_limit, int(test_flags), int(test_alloc_fail_above))
        h = ctypes.c_void_p()
        _check(L.gx_ctx_create(device, ctypes.byref(opts), ctypes.byref(h)), "gx_ctx_create")
        self.h = h.value
        self.device = device

    def mark(self, slot):
        _check(self._L.gx_ctx_mark(self.h, slot), "gx_ctx_mark")

    def elapsed_ms(self, a, b):
        ms = ctypes.c_double()
        _check(self._L.gx_ctx_elapsed_ms(self.h, a, b, ctypes.byref(ms)), "gx_ctx_elapsed_ms")
        return ms.value

    def autotune(self, sample, k, repeats=2):
        """gx_autotune: times every algorithm x fill x threads-per-read on `sample` (readid text)
        and keeps the fastest for jobs at the defaults; returns the choice and every candidate's
        time."""
        r = _lib.TuneResult()
        r.struct_size = ctypes.sizeof(_lib.TuneResult)
        p, n, keep = _host_ptr(sample)
        _check(self._L.gx_autotune(self.h, p, n, int(k), int(repeats), ctypes.byref(r)), "gx_autotune")
        del keep
        names = {_lib.ALGO_PARTITIONED: "partitioned", _lib.ALGO_TABLE: "table"}
        return {"algorithm": names[r.algorithm], "load_factor": r.load_factor, "ms": r.ms,
                "threads_per_read": r.threads_per_read,
                "candidates": [{"algorithm": names[r.cand[i].algorithm], "load_factor": r.cand[i].load_factor,
                                "threads_per_read": r.cand[i].threads_per_read, "ms": r.cand[i].ms}
                               for i in range(r.tried)]}

    def autotune_clear(self):
        _check(self._L.gx_autotune_clear(self.h), "gx_autotune_clear")

    def synchronize(self):
        _check(self._L.gx_ctx_synchronize(self.h), "gx_ctx_synchronize")

    def close(self):
        if self.h:
            self._L.gx_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GraphBuildJob:
    """One graph build: inputs -> run() -> (VKmer, Node) records.

    layout="buckets" splits the records into out_parts contiguous ranges of hash buckets;
    layout="reference" puts each record in the part the reference's Kmer partitioner picks
    (KmerPartitionComputerFactory.java:28-52), so part q holds the record set of the
    reference's part q (the order within a part is the build's own)."""

    def __init__(self, ctx, kmer_length, input_kind="readid", paired=False, out_parts=1, load_factor=0.0,
                 max_readids_per_edge=250, threads_per_read=0, est_input_bytes=0, algorithm="default",
                 plan="BUILD_DEBRUIJN_GRAPH", layout="buckets"):
        self.ctx = ctx
        self._L = ctx._L
        kind = {"readid": _lib.INPUT_READID, "fastq": _lib.INPUT_FASTQ}[input_kind]
        algo = {"default": _lib.ALGO_DEFAULT, "partitioned": _lib.ALGO_PARTITIONED, "table": _lib.ALGO_TABLE}[algorithm]
        pl = {"BUILD_DEBRUIJN_GRAPH": _lib.PLAN_BUILD_DEBRUIJN_GRAPH, "BUILD_READ_PARSER": _lib.PLAN_BUILD_READ_PARSER}[plan]
        o = _lib.JobOpts(ctypes.sizeof(_lib.JobOpts), int(kmer_length), kind, 1 if paired else 0, int(out_parts),
                         float(load_factor), int(max_readids_per_edge), int(threads_per_read), int(est_input_bytes),
                         algo, pl, {"buckets": _lib.LAYOUT_BUCKETS, "reference": _lib.LAYOUT_REFERENCE_PARTS}[layout])
        self.plan = plan
        self.layout = layout
        h = ctypes.c_void_p()
        _check(self._L.gx_job_create(ctx.h, ctypes.byref(o), ctypes.byref(h)), "gx_job_create")
        self.h = h.value
        self.k = int(kmer_length)
        self.out_parts = max(1, int(out_parts))
        self._keep = []

    def add_input(self, data, mate_stream=0):
        """Appends one input file from host memory (copied during the call)."""
        p, n, keep = _host_ptr(data)
        _check(self._L.gx_job_add_input(self.h, p, n, mate_stream), "gx_job_add_input")
        del keep

    def add_input_device(self, ptr, nbytes, keepalive=None):
        """Appends readid text already in device memory (borrowed until run() returns)."""
        _check(self._L.gx_job_add_input_device(self.h, ptr, nbytes, 0), "gx_job_add_input_device")
        if keepalive is not None:
            self._keep.append(keepalive)

    def run(self):
        st = self._L.gx_job_run(self.h)
        self._keep.clear()
        if st != _lib.GX_OK:
            raise GraphBuildError(st, "gx_job_run", self.stats()["error_line"])
        return self

    def stats(self):
        s = _lib.Stats()
        _check(self._L.gx_job_stats(self.h, ctypes.byref(s)), "gx_job_stats")
        return s.as_dict()

    def part_offsets(self):
        d, n, po = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.POINTER(ctypes.c_uint64)()
        _check(self._L.gx_job_records_device(self.h, ctypes.byref(d), ctypes.byref(n), ctypes.byref(po)),
               "gx_job_records_device")
        return [po[i] for i in range(self.out_parts + 1)]

    def records_device(self):
        """(device pointer, bytes) of the whole record stream."""
        d, n = ctypes.c_void_p(), ctypes.c_size_t()
        _check(self._L.gx_job_records_device(self.h, ctypes.byref(d), ctypes.byref(n), None),
               "gx_job_records_device")
        return d.value, n.value

    def emit_into(self, part, buf_ptr, cap):
        """One gx_job_emit call: (written, more)."""
        w, m = ctypes.c_size_t(), ctypes.c_int()
        _check(self._L.gx_job_emit(self.h, part, buf_ptr, cap, ctypes.byref(w), ctypes.byref(m)), "gx_job_emit")
        return w.value, bool(m.value)

    def graph_stats(self):
        """GraphStatistics counters of the job's graph, computed on the GPU (gx_job_graph_stats):
        totals, maxima and value histograms (non-zero bins) of each statistic."""
        g = _lib.GraphStats()
        g.struct_size = ctypes.sizeof(_lib.GraphStats)
        _check(self._L.gx_job_graph_stats(self.h, ctypes.byref(g)), "gx_job_graph_stats")
        return g.as_dict()

    def rewind(self, part=None):
        """Restarts gx_job_emit at the beginning of one part (or of every part)."""
        _check(self._L.gx_job_emit_rewind(self.h, -1 if part is None else part), "gx_job_emit_rewind")

    def emit_async(self, part, buf_ptr, cap):
        """gx_job_emit_async: queues the copy of (the next piece of) a part; (written, more).
        The buffer is ready after emit_wait()."""
        w, m = ctypes.c_size_t(), ctypes.c_int()
        _check(self._L.gx_job_emit_async(self.h, part, buf_ptr, cap, ctypes.byref(w), ctypes.byref(m)),
               "gx_job_emit_async")
        return w.value, bool(m.value)

    def emit_wait(self):
        _check(self._L.gx_job_emit_wait(self.h), "gx_job_emit_wait")

    def records(self, part=None, chunk=None):
        """Serialized record stream of one part (or all parts in order) as bytes."""
        parts = range(self.out_parts) if part is None else [part]
        offs = self.part_offsets()
        _check(self._L.gx_job_emit_rewind(self.h, -1 if part is None else part), "gx_job_emit_rewind")
        out = []
        for q in parts:
            total = offs[q + 1] - offs[q]
            cap = total if chunk is None else int(chunk)
            buf = PinnedBuffer(max(cap, 1))
            pieces = []
            while True:
                w, more = self.emit_into(q, buf.ptr, cap)
                pieces.append(bytes(buf.array()[:w]))
                if not more:
                    break
            buf.close()
            out.append(b"".join(pieces))
        return b"".join(out)

    def close(self):
        if self.h:
            self._L.gx_job_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_run(ctx, jobs):
    """Runs several prepared jobs in one call (gx_batch_run); returns per-job statuses."""
    L = ctx._L
    arr = (ctypes.c_void_p * len(jobs))(*[j.h for j in jobs])
    sts = (ctypes.c_int * len(jobs))()
    L.gx_batch_run(ctx.h, arr, len(jobs), sts)
    for j in jobs:
        j._keep.clear()
    return list(sts)


class Server:
    """Graph builds served as they arrive (gx_serve_*): continuous batching by estimated device
    memory over `lanes` concurrent passes.  submit() hands a job over; poll() returns
    (status, latency_ms) once it is done, or None while it is not."""

    def __init__(self, ctx, mem_budget=0, lanes=0, max_batch=0, pass_bytes=0):
        self.ctx = ctx
        self._L = ctx._L
        o = _lib.ServeOpts(ctypes.sizeof(_lib.ServeOpts), int(mem_budget), int(lanes), int(max_batch),
                           int(pass_bytes))
        h = ctypes.c_void_p()
        _check(self._L.gx_serve_create(ctx.h, ctypes.byref(o), ctypes.byref(h)), "gx_serve_create")
        self.h = h.value
        self._jobs = {}

    def submit(self, job):
        t = ctypes.c_uint64()
        _check(self._L.gx_serve_submit(self.h, job.h, ctypes.byref(t)), "gx_serve_submit")
        self._jobs[t.value] = job
        return t.value

    def poll(self, ticket, timeout_ms=-1):
        st, lat = ctypes.c_int(), ctypes.c_double()
        r = self._L.gx_serve_poll(self.h, ticket, int(timeout_ms), ctypes.byref(st), ctypes.byref(lat))
        if r == _lib.GX_EAGAIN:
            return None
        _check(r, "gx_serve_poll")
        job = self._jobs.pop(ticket, None)
        if job is not None:
            job._keep.clear()
        return st.value, lat.value

    def cancel(self, ticket):
        """Withdraws a job that has not started (gx_serve_cancel): True when cancelled (its
        poll() then reports GX_ECANCELLED), False when it is already running or done."""
        r = self._L.gx_serve_cancel(self.h, ticket)
        if r in (_lib.GX_EBUSY, _lib.GX_ESTATE):
            return False
        _check(r, "gx_serve_cancel")
        return True

    def stats(self):
        s = _lib.ServeStats()
        _check(self._L.gx_serve_stats_get(self.h, ctypes.byref(s)), "gx_serve_stats_get")
        return s.as_dict()

    def close(self):
        if self.h:
            self._L.gx_serve_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _buf_out(fn, *args):
    L = _lib.load()
    out, n = ctypes.c_void_p(), ctypes.c_size_t()
    st = fn(*args, ctypes.byref(out), ctypes.byref(n))
    data = ctypes.string_at(out, n.value) if out.value and n.value else b""
    if out.value:
        L.gx_host_free(out)
    return st, data


def fastq_to_readid(mate1: bytes, mate2: bytes = None) -> bytes:
    """GenomixDriver.convertAndUploadFastqToHDFS (GenomixDriver.java:665-714)."""
    L = _lib.load()
    st, data = _buf_out(L.gx_fastq_to_readid, mate1, len(mate1), mate2, len(mate2) if mate2 else 0)
    _check(st, "gx_fastq_to_readid")
    return data


def fastq_to_readid_gpu(ctx, mate1: bytes, mate2: bytes = None) -> bytes:
    """The same conversion on the GPU (gx_fastq_to_readid_gpu), as jobs with FASTQ input run it."""
    L = ctx._L
    out, n = ctypes.c_void_p(), ctypes.c_size_t()
    p1, n1, k1 = _host_ptr(mate1)
    p2, n2, k2 = _host_ptr(mate2) if mate2 is not None else (None, 0, None)
    _check(L.gx_fastq_to_readid_gpu(ctx.h, p1, n1, p2, n2, ctypes.byref(out), ctypes.byref(n)),
           "gx_fastq_to_readid_gpu")
    data = ctypes.string_at(out, n.value) if n.value else b""
    L.gx_host_free(out)
    del k1, k2
    return data


def seqfile_write(records: bytes, sync: bytes = None, seed: int = 0, key_class="VKmer") -> bytes:
    """A Hadoop SequenceFile<VKmer, Node> (or <Kmer, Node>, the read-parser plan's files)
    holding the record stream."""
    L = _lib.load()
    fn = {"VKmer": L.gx_seqfile_write, "Kmer": L.gx_seqfile_write_kmer_keys}[key_class]
    st, data = _buf_out(fn, records, len(records), sync, seed)
    _check(st, "gx_seqfile_write")
    return data


def seqfile_read(data: bytes) -> bytes:
    L = _lib.load()
    st, out = _buf_out(L.gx_seqfile_read, data, len(data))
    _check(st, "gx_seqfile_read")
    return out


def records_to_text(records: bytes) -> str:
    """key.toString() + '\\t' + value.toString() per record (GenomixClusterManager.java:371)."""
    L = _lib.load()
    st, out = _buf_out(L.gx_records_to_text, records, len(records))
    _check(st, "gx_records_to_text")
    return out.decode()


def records_digest(records, nbytes=None):
    """Order-independent digest of a record stream (host bytes, or a host pointer + size)."""
    L = _lib.load()
    d = _lib.Digest()
    if isinstance(records, int):
        p, n = records, nbytes
        _check(L.gx_records_digest(p, n, ctypes.byref(d)), "gx_records_digest")
    else:
        p, n, keep = _host_ptr(records)
        _check(L.gx_records_digest(p, n, ctypes.byref(d)), "gx_records_digest")
        del keep
    return d.as_dict()


def iter_records(records: bytes):
    """Yields (key_bytes, value_bytes) of a record stream."""
    p, n = 0, len(records)
    while p < n:
        rl = int.from_bytes(records[p:p + 4], "big")
        kl = int.from_bytes(records[p + 4:p + 8], "big")
        yield records[p + 8:p + 8 + kl], records[p + 8 + kl:p + 8 + rl]
        p += 8 + rl


def _input_files(paths):
    out = []
    for p in paths:
        if os.path.isdir(p):
            out.extend(sorted(os.path.join(p, f) for f in os.listdir(p)
                              if not f.startswith((".", "_")) and os.path.isfile(os.path.join(p, f))))
        else:
            out.append(p)
    return out


class GenomixGpuDriver:
    """Drop-in for GenomixHyracksDriver for Plan.BUILD_DEBRUIJN_GRAPH and Plan.BUILD_READ_PARSER."""

    BUILD_DEBRUIJN_GRAPH = "BUILD_DEBRUIJN_GRAPH"
    BUILD_READ_PARSER = "BUILD_READ_PARSER"

    def __init__(self, device=0, threads_per_machine=1, layout="reference"):
        """layout="reference" (the default) writes the graph plan's part files with the record
        sets of the reference's part files; "buckets" skips that regrouping pass."""
        self.ctx = Context(device)
        self.threads_per_machine = threads_per_machine
        self.layout = layout

    def run_job(self, conf, plan=BUILD_DEBRUIJN_GRAPH, profile=False):
        """Reads the readid (or FASTQ) inputs named in conf, writes part-N SequenceFiles under
        the output directory, returns the job statistics."""
        if plan not in (self.BUILD_DEBRUIJN_GRAPH, self.BUILD_READ_PARSER):
            raise ValueError(f"unsupported plan {plan}: the GPU runs the graph build and the read parser")
        k = int(conf[KMER_LENGTH])
        out_dir = conf[OUTPUT_DIR]
        parts = int(conf.get(THREADS_PER_MACHINE, self.threads_per_machine))
        fastq_pe = conf.get(PAIRED_END_FASTQ_INPUTS)
        fastq_se = conf.get(SINGLE_END_FASTQ_INPUTS)
        lay = dict(plan=plan, layout=self.layout if plan == self.BUILD_DEBRUIJN_GRAPH else "buckets")
        jobs = []
        if fastq_pe or fastq_se:
            if fastq_pe:
                fs = fastq_pe.split(",")
                job = GraphBuildJob(self.ctx, k, "fastq", paired=True, out_parts=parts, **lay)
                for a, b in zip(fs[0::2], fs[1::2]):
                    job.add_input(open(a, "rb").read(), 0)
                    job.add_input(open(b, "rb").read(), 1)
                jobs.append(job)
            if fastq_se:
                job = GraphBuildJob(self.ctx, k, "fastq", paired=False, out_parts=parts, **lay)
                for a in fastq_se.split(","):
                    job.add_input(open(a, "rb").read(), 0)
                jobs.append(job)
            if len(jobs) > 1:
                # one job over both libraries: convert on the host, then one readid job
                text = b""
                for a, b in zip(fastq_pe.split(",")[0::2], fastq_pe.split(",")[1::2]):
                    text += fastq_to_readid(open(a, "rb").read(), open(b, "rb").read())
                for a in fastq_se.split(","):
                    text += fastq_to_readid(open(a, "rb").read())
                for j in jobs:
                    j.close()
                job = GraphBuildJob(self.ctx, k, "readid", out_parts=parts, **lay)
                job.add_input(text)
                jobs = [job]
        else:
            job = GraphBuildJob(self.ctx, k, "readid", out_parts=parts, **lay)
            for f in _input_files(conf[INPUT_DIR].split(",")):
                with open(f, "rb") as fh:
                    job.add_input(fh.read())
            jobs = [job]
        job = jobs[0]
        job.run()
        os.makedirs(out_dir, exist_ok=True)
        for q in range(job.out_parts):
            with open(os.path.join(out_dir, f"part-{q}"), "wb") as fh:
                fh.write(seqfile_write(job.records(q), seed=q,
                                       key_class="Kmer" if plan == self.BUILD_READ_PARSER else "VKmer"))
        st = job.stats()
        job.close()
        return st
