"""ctypes binding of the oracle (liboracle: gx_oracle.cpp).

Test infrastructure only.  Used by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker; the product library never imports it.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgxoracle.so")
SRC = os.path.join(HERE, "gx_oracle.cpp")

_lib = None


def build(force=False):
    """Compiles the oracle shared library with g++ (a few seconds)."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-ffp-contract=off",
           SRC, "-o", LIB_PATH + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.gxo_build.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_void_p)]
        L.gxo_build.restype = ctypes.c_int
        L.gxo_build_part.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.gxo_build_part.restype = ctypes.c_int
        L.gxo_result_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.gxo_result_records.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]
        L.gxo_result_records.restype = ctypes.c_void_p
        L.gxo_result_part_offsets.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]
        L.gxo_result_part_offsets.restype = ctypes.POINTER(ctypes.c_uint64)
        L.gxo_result_free.argtypes = [ctypes.c_void_p]
        for name in ("gxo_normalize", "gxo_dump_text"):
            f = getattr(L, name)
            f.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p),
                          ctypes.POINTER(ctypes.c_size_t)]
            f.restype = ctypes.c_int
        L.gxo_fastq_to_readid.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t)]
        L.gxo_fastq_to_readid.restype = ctypes.c_int
        L.gxo_free.argtypes = [ctypes.c_void_p]
        L.gxo_read_parser.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t),
                                      ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        L.gxo_read_parser.restype = ctypes.c_int
        L.gxo_kat_kmer.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_char_p]
        L.gxo_kat_kmer_shift.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_char,
                                         ctypes.c_char_p]
        L.gxo_kat_uuid.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int]
        L.gxo_kat_uuid.restype = ctypes.c_int64
        L.gxo_kat_uuid_offset.argtypes = [ctypes.c_int64]
        L.gxo_kat_uuid_offset.restype = ctypes.c_int
        L.gxo_kat_float_to_string.argtypes = [ctypes.c_float, ctypes.c_char_p]
        _lib = L
    return _lib


class OracleResult:
    def __init__(self, status, stats, records, part_offsets):
        self.status = status
        self.lines, self.reads, self.kmers, self.read_heads, self.nodes, self.error_line = stats
        self.records = records
        self.part_offsets = part_offsets


def build_graph(text: bytes, k: int, threads: int = 1, parts: int = 1, only_part: int = -1) -> OracleResult:
    """Runs the oracle graph build over readid text; returns status, stats and records.
    only_part >= 0 keeps only the records of that part of `parts` (the reference's Kmer
    partitioner): the parts built one at a time add up to the whole build, in the memory of one."""
    L = lib()
    h = ctypes.c_void_p()
    st = L.gxo_build_part(text, len(text), k, threads, parts, only_part, ctypes.byref(h))
    stats = (ctypes.c_uint64 * 6)()
    L.gxo_result_stats(h, stats)
    n = ctypes.c_size_t()
    p = L.gxo_result_records(h, ctypes.byref(n))
    records = ctypes.string_at(p, n.value) if n.value else b""
    np_ = ctypes.c_size_t()
    po = L.gxo_result_part_offsets(h, ctypes.byref(np_))
    offs = [po[i] for i in range(np_.value + 1)]
    L.gxo_result_free(h)
    return OracleResult(st, tuple(stats), records, offs)


def _buf_call(fn, *args):
    L = lib()
    out = ctypes.c_void_p()
    n = ctypes.c_size_t()
    st = fn(*args, ctypes.byref(out), ctypes.byref(n))
    data = ctypes.string_at(out, n.value) if n.value else b""
    if out:
        L.gxo_free(out)
    return st, data


def normalize(records: bytes) -> bytes:
    """Comparison form: records sorted by key, edge lists sorted."""
    st, data = _buf_call(lib().gxo_normalize, records, len(records))
    if st != 0:
        raise ValueError("malformed record stream")
    return data


def dump_text(records: bytes) -> str:
    """Text form of the records as the reference's copyBinAndTextToLocal writes it."""
    st, data = _buf_call(lib().gxo_dump_text, records, len(records))
    if st != 0:
        raise ValueError("malformed record stream")
    return data.decode()


def fastq_to_readid(mate1: bytes, mate2: bytes = None):
    st, data = _buf_call(lib().gxo_fastq_to_readid, mate1, len(mate1), mate2, len(mate2) if mate2 else 0)
    return st, data


def kat_kmer(s: str, k: int, start: int = 0, reverse: bool = False) -> str:
    b = s.encode()
    out = ctypes.create_string_buffer(k + 1)
    lib().gxo_kat_kmer(b, len(b), k, start, 1 if reverse else 0, out)
    return out.value.decode()


def kat_kmer_shift(s: str, k: int, nxt: str) -> str:
    b = s.encode()
    out = ctypes.create_string_buffer(k + 1)
    lib().gxo_kat_kmer_shift(b, len(b), k, nxt.encode(), out)
    return out.value.decode()


def kat_uuid(mate, lib_id, read_id, offset):
    return lib().gxo_kat_uuid(mate, lib_id, read_id, offset)


def kat_uuid_offset(uuid):
    return lib().gxo_kat_uuid_offset(uuid)


def java_float_to_string(f: float) -> str:
    out = ctypes.create_string_buffer(64)
    lib().gxo_kat_float_to_string(f, out)
    return out.value.decode()


def read_parser(text: bytes, k: int):
    """(status, error_line, occurrences, records) of the BUILD_READ_PARSER plan: one
    (Kmer, Node) record per k-mer occurrence, in read order."""
    L = lib()
    p, n, el, occ = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_uint64(), ctypes.c_uint64()
    st = L.gxo_read_parser(text, len(text), k, ctypes.byref(p), ctypes.byref(n), ctypes.byref(el), ctypes.byref(occ))
    rec = ctypes.string_at(p, n.value)
    L.gxo_free(p)
    return st, el.value, occ.value, rec
