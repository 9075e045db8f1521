"""The C ABI library on the CPU: it loads, exports every declared symbol, and its host-side
formats agree with the oracle.  No kernel runs here."""
import os
import re

import pytest

from conftest import ROOT, golden_cases, golden_expected, golden_input
from genomix_gb300 import _lib, build as gbuild
import genomix_gb300 as gx
from oracle import gx_oracle as go


@pytest.fixture(scope="module", autouse=True)
def built():
    gbuild.build()
    return _lib.load()


def declared_symbols():
    with open(os.path.join(ROOT, "include", "gxgpu.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gx_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(built):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(built, n), n
    assert sorted(_lib.EXPORTS) == names


def test_status_strings(built):
    for code, name in _lib.STATUS_NAMES.items():
        assert _lib.status_str(code)
    assert "kmersize" in _lib.status_str(5)


def test_context_fails_loudly_without_gpu():
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("GPU present")
    with pytest.raises(gx.GraphBuildError) as e:
        gx.Context(0)
    assert e.value.name == "GX_ECUDA"


def test_fastq_conversion_matches_oracle():
    fq1 = b"@a\nACGTAC\n+\nIIIIII\n@b\n\tGGCATT \r\n+\nIIIIII\n@c\nAC\n+\nII"
    fq2 = b"@a\nTTTGCA\n+\nIIIIII\n@b\nCCCGGA\n+\nIIIIII\n@c\nGG\n+\nII"
    assert gx.fastq_to_readid(fq1, fq2) == go.fastq_to_readid(fq1, fq2)[1]
    assert gx.fastq_to_readid(fq1) == go.fastq_to_readid(fq1)[1]
    with pytest.raises(gx.GraphBuildError) as e:
        gx.fastq_to_readid(fq1, fq2 + b"\n@d\n")
    assert e.value.name == "GX_EFASTQ_PAIRING"


@pytest.mark.parametrize("case", golden_cases(), ids=[c["name"] for c in golden_cases()])
def test_product_text_dump_matches_golden(case):
    """The library's text dump of oracle records equals the reference's dump form."""
    res = go.build_graph(golden_input(case["name"]), case["k"], threads=2, parts=4)
    assert gx.records_to_text(res.records) == go.dump_text(res.records)


def test_seqfile_round_trip_and_header():
    from genomix_gb300 import synth
    text = synth.small_random(3, 300, 80, 21, paired=True)
    res = go.build_graph(text, 21)
    f = gx.seqfile_write(res.records, seed=5)
    assert f[:4] == b"SEQ\x06"
    assert b"edu.uci.ics.genomix.data.types.VKmer" in f[:100]
    assert b"edu.uci.ics.genomix.data.types.Node" in f[:100]
    assert gx.seqfile_read(f) == res.records
    # sync escapes appear roughly every 2000 bytes
    assert f.count(b"\xff\xff\xff\xff" + f[f.index(b"Node") + 4 + 6:f.index(b"Node") + 4 + 6 + 16]) >= len(
        res.records) // 2200
    assert gx.seqfile_write(res.records, seed=5) == f  # deterministic sync marker
    assert gx.seqfile_write(res.records, seed=6) != f


def test_records_digest_is_order_independent_and_counts():
    from conftest import golden_input
    text = golden_input("Random100_k3")
    ref = go.build_graph(text, 3, threads=2, parts=3)
    d = gx.records_digest(ref.records)
    assert d["records"] == ref.nodes and d["heads"] == ref.read_heads and d["coverage"] == ref.kmers
    recs = [(len(k) + len(v)).to_bytes(4, "big") + len(k).to_bytes(4, "big") + k + v
            for k, v in gx.iter_records(ref.records)]
    assert b"".join(recs) == ref.records
    assert gx.records_digest(b"".join(reversed(recs))) == d
    # another thread/part split of the oracle orders records differently: same digest
    assert gx.records_digest(go.build_graph(text, 3, threads=1, parts=1).records) == d
    # one changed byte (the last coverage byte of the first record) changes the digest
    bad = bytearray(ref.records)
    first_len = int.from_bytes(bad[0:4], "big") + 8
    bad[first_len - 1] ^= 1
    d2 = gx.records_digest(bytes(bad))
    assert (d2["sum"], d2["xor_"]) != (d["sum"], d["xor_"])


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors have the C structs' sizes and field offsets (a C program compiled
    against include/gxgpu.h prints them)."""
    import ctypes
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {
        "gx_job_opts": _lib.JobOpts, "gx_stats": _lib.Stats, "gx_serve_opts": _lib.ServeOpts,
        "gx_serve_stats": _lib.ServeStats, "gx_digest": _lib.Digest, "gx_graph_stats": _lib.GraphStats,
        "gx_ctx_opts": _lib.CtxOpts, "gx_stat_hist": _lib.StatHist, "gx_tune_result": _lib.TuneResult,
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gxgpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def java_part(kmer_bytes, nparts):
    """KmerPartitionComputerFactory.hashBytes + partition (KmerPartitionComputerFactory.java:28-52),
    in Python integers: h = 1, then 31 h + (signed) byte, as a Java int; sign-folded; mod parts."""
    h = 1
    for b in kmer_bytes:
        h = (31 * h + (b - 256 if b > 127 else b)) & 0xFFFFFFFF
    if h >= 1 << 31:
        h -= 1 << 32
    if h < 0:
        h = -(h + 1)
    return h % nparts


@pytest.mark.parametrize("parts", [3, 7, 300])
def test_oracle_parts_follow_the_reference_partitioner(parts):
    """Every record of the oracle's part q has a key the restated partitioner sends to q: the
    oracle's part layout, which the GPU's reference part layout is checked against, is pinned to
    the reference's hash."""
    from genomix_gb300 import synth
    text = synth.plain_cpu().text
    ref = go.build_graph(text, 21, threads=4, parts=parts)
    assert ref.status == 0
    po = ref.part_offsets
    seen = 0
    for q in range(parts):
        for key, _ in gx.iter_records(ref.records[po[q]:po[q + 1]]):
            assert java_part(key[4:], parts) == q
            seen += 1
    assert seen == ref.nodes


def test_jni_shim_compiles_against_the_header(tmp_path):
    """The JNI side of the Java binding (genomix_gb300/jni/gxgpu_jni.c) compiles against
    include/gxgpu.h.  No JDK is installed here, so a minimal jni.h with the types and the
    JNIEnv functions the shim calls stands in for the real one."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    (tmp_path / "jni.h").write_text("""
#include <stdint.h>
typedef int32_t jint; typedef int64_t jlong; typedef void *jobject; typedef jobject jclass;
typedef jobject jstring; typedef jobject jintArray; typedef int64_t jsize;
struct JNINativeInterface_;
typedef const struct JNINativeInterface_ *JNIEnv;
struct JNINativeInterface_ {
    void *(*GetDirectBufferAddress)(JNIEnv *, jobject);
    void (*SetIntArrayRegion)(JNIEnv *, jintArray, jsize, jsize, const jint *);
    jstring (*NewStringUTF)(JNIEnv *, const char *);
    jobject (*NewDirectByteBuffer)(JNIEnv *, void *, jlong);
};
#define JNIEXPORT __attribute__((visibility("default")))
#define JNICALL
""")
    src = os.path.join(ROOT, "genomix_gb300", "jni", "gxgpu_jni.c")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", str(tmp_path), "-I",
                    os.path.join(ROOT, "include"), src], check=True)
