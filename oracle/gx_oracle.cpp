// gx_oracle.cpp — THE ORACLE.  Test infrastructure only: the checker for the GPU graph
// build and the timed CPU baseline.  Nothing in the product library links or calls it.
//
// A CPU restatement, in C++17, of the Genomix graph-build step as the genomix-hyracks job
// runs it (paths are inside the genomix project of uci-cbcl/genomix):
//
//   parse     ReadsKeyValueParserFactory.parse / SplitReads / setEdgesForCurAndNext
//             (genomix-hyracks/.../graph/dataflow/ReadsKeyValueParserFactory.java:95-254)
//             emits one (Kmer, marshalled Node) tuple per k-mer occurrence;
//   sort      ExternalSortOperatorDescriptor on KmerPointable order (KmerPointable.java:94-107);
//   group     PreclusteredGroup with AggregateKmerAggregateFactory.init/aggregate
//             (AggregateKmerAggregateFactory.java:93-175), locally per input split;
//   exchange  MToNPartitioningMergingConnector by KmerPartitionComputerFactory
//             (KmerPartitionComputerFactory.java:28-52), merge-sorted at the receiver;
//   group     the same aggregator again, globally (JobGenBuildBrujinGraph.java:92-117);
//   write     (VKmer, Node) records as SequenceFile.Writer.append frames them
//             (KmerNodePairSequenceWriterFactory.java:79-94), one part per partition.
//
// The k-mers are handled as the reference handles them: as packed byte arrays, re-packed
// from the read text per window (Kmer.java:225-303), compared as Hadoop's BinaryComparable
// compares them (unsigned lexicographic bytes).  The parity of this restatement is pinned
// by the reference's own golden fixtures (tests/golden/, copied from
// genomix-hyracks/src/test/resources/data) and its Kmer / ReadHeadInfo unit tests.
//
// Edge lists: the reference keeps each VKmerList as the iteration order of a Java HashSet
// (VKmerList.java:117-133), which its own test compares as unordered fields
// (BatchTestFilesTest.java:171-172).  This restatement keeps each list sorted by VKmer
// bytes; that is one of the orders the reference can produce and the order the GPU build
// writes.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../include/gxgpu.h"

namespace gxo {

// ---------------------------------------------------------------------------------------
// GeneCode (genomix-data/.../utils/GeneCode.java:29-61) and KmerUtil (KmerUtil.java:21-48)
// ---------------------------------------------------------------------------------------
static inline uint8_t code_from_symbol(uint8_t ch) {
    switch (ch) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': return 3;
    }
    return 0;  // any other symbol encodes as A (GeneCode.java:30, r = 0 by default)
}
static inline uint8_t paired_code_from_symbol(uint8_t ch) { return 3 - code_from_symbol(ch); }
static inline int byte_num_from_k(int k) { return k / 4 + (k % 4 != 0 ? 1 : 0); }
static const char GENE_SYMBOL[4] = {'A', 'C', 'G', 'T'};

// KmerUtil.recoverKmerFrom (KmerUtil.java:34-48)
static std::string recover_kmer(int k, const uint8_t *bytes, int nb) {
    std::string s;
    if (nb <= 0 || k < 1) return s;
    int byte_id = nb - 1;
    uint8_t cur = bytes[byte_id];
    s.reserve(k);
    for (int g = 0; g < k; g++) {
        if (g % 4 == 0 && g > 0) cur = bytes[--byte_id];
        s.push_back(GENE_SYMBOL[(cur >> ((g % 4) * 2)) & 3]);
    }
    return s;
}

// Big-endian marshalling (Marshal.java:20-63; java.io.DataOutput)
static inline void put_i32(std::string &o, int32_t v) {
    uint32_t u = (uint32_t)v;
    char b[4] = {(char)(u >> 24), (char)(u >> 16), (char)(u >> 8), (char)u};
    o.append(b, 4);
}
static inline void put_i64(std::string &o, int64_t v) {
    uint64_t u = (uint64_t)v;
    char b[8];
    for (int i = 0; i < 8; i++) b[i] = (char)(u >> (56 - 8 * i));
    o.append(b, 8);
}
static inline void put_f32(std::string &o, float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put_i32(o, (int32_t)u);
}
static inline int32_t get_i32(const uint8_t *p) {
    return (int32_t)(((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]);
}
static inline int64_t get_i64(const uint8_t *p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    return (int64_t)v;
}
static inline float get_f32(const uint8_t *p) {
    uint32_t u = (uint32_t)get_i32(p);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// ---------------------------------------------------------------------------------------
// Kmer: fixed-length packed k-mer (genomix-data/.../types/Kmer.java)
// ---------------------------------------------------------------------------------------
struct KmerOps {
    int k;
    int nb;
    // Kmer.setFromStringBytes (Kmer.java:225-242)
    void set_from_string(uint8_t *b, const uint8_t *s, int start, int len) const {
        uint8_t l = 0;
        int bytecount = 0, bcount = nb - 1;
        for (int i = start; i < start + k && i < len; i++) {
            uint8_t code = code_from_symbol(s[i]);
            l |= (uint8_t)(code << bytecount);
            bytecount += 2;
            if (bytecount == 8) {
                b[bcount--] = l;
                l = 0;
                bytecount = 0;
            }
        }
        if (bcount >= 0) b[0] = l;
    }
    // Kmer.setReversedFromStringBytes (Kmer.java:253-272)
    void set_reversed_from_string(uint8_t *b, const uint8_t *s, int start, int len) const {
        uint8_t l = 0;
        int bytecount = 0, bcount = nb - 1;
        for (int i = start + k - 1; i >= start && i < len; i--) {
            uint8_t code = paired_code_from_symbol(s[i]);
            l |= (uint8_t)(code << bytecount);
            bytecount += 2;
            if (bytecount == 8) {
                b[bcount--] = l;
                l = 0;
                bytecount = 0;
            }
        }
        if (bcount >= 0) b[0] = l;
    }
    // Kmer.clearLeadBit (Kmer.java:332-336)
    void clear_lead_bit(uint8_t *b) const {
        if (k % 4 != 0) b[0] &= (uint8_t)((1 << ((k % 4) << 1)) - 1);
    }
    // Kmer.shiftKmerWithNextCode (Kmer.java:292-303)
    void shift_with_next_char(uint8_t *b, uint8_t ch) const {
        uint8_t c = code_from_symbol(ch);
        for (int i = nb - 1; i > 0; i--) {
            uint8_t in = b[i - 1] & 0x03;
            b[i] = (uint8_t)(((b[i] >> 2) & 0x3f) | (in << 6));
        }
        int pos = ((k - 1) % 4) << 1;
        b[0] = (uint8_t)(((b[0] >> 2) & 0x3f) | (uint8_t)(c << pos));
        clear_lead_bit(b);
    }
};

// Hadoop BinaryComparable.compareTo -> WritableComparator.compareBytes: unsigned
// lexicographic order over the packed bytes (call sites ReadsKeyValueParserFactory.java:163,181).
static inline int compare_bytes(const uint8_t *a, int la, const uint8_t *b, int lb) {
    int n = la < lb ? la : lb;
    for (int i = 0; i < n; i++) {
        int x = a[i], y = b[i];
        if (x != y) return x - y;
    }
    return la - lb;
}

// KmerPointable.compareTo (genomix-hyracks/.../data/primitive/KmerPointable.java:94-107):
// length first, then bytes from the last to the first, unsigned.
static inline int kmer_pointable_compare(const uint8_t *a, int la, const uint8_t *b, int lb) {
    if (la != lb) return la - lb;
    for (int i = la - 1; i >= 0; i--) {
        int c = (int)a[i] - (int)b[i];
        if (c != 0) return c;
    }
    return 0;
}

// KmerPartitionComputerFactory.hashBytes + partition (KmerPartitionComputerFactory.java:28-52)
static inline int kmer_partition(const uint8_t *b, int len, int nparts) {
    int32_t hash = 1;
    for (int i = 0; i < len; i++) hash = (int32_t)((uint32_t)(31 * (uint32_t)hash) + (uint32_t)(int32_t)(int8_t)b[i]);
    if (hash < 0) hash = -(hash + 1);
    return hash % nparts;
}

// ---------------------------------------------------------------------------------------
// VKmer bytes = int32 BE letter count + packed bytes (VKmer.java:366-391)
// ---------------------------------------------------------------------------------------
static std::string vkmer_from_kmer(int k, const uint8_t *b, int nb) {
    std::string o;
    put_i32(o, k);
    o.append((const char *)b, nb);
    return o;
}
// VKmer.setAsCopy(String) -> setFromStringBytes(len, bytes, 0) (VKmer.java:140-142,450-479)
static std::string vkmer_from_string(const uint8_t *s, int len) {
    int nb = byte_num_from_k(len);
    std::string o;
    put_i32(o, len);
    std::string packed(nb, '\0');
    uint8_t *b = (uint8_t *)&packed[0];
    uint8_t l = 0;
    int bytecount = 0, bcount = nb - 1;
    for (int i = 0; i < len; i++) {
        l |= (uint8_t)(code_from_symbol(s[i]) << bytecount);
        bytecount += 2;
        if (bytecount == 8) {
            b[bcount--] = l;
            l = 0;
            bytecount = 0;
        }
    }
    if (bcount >= 0) b[0] = l;
    o += packed;
    return o;
}

// ---------------------------------------------------------------------------------------
// ReadHeadInfo (genomix-data/.../types/ReadHeadInfo.java)
// ---------------------------------------------------------------------------------------
static const int RH_BITS_READID = 35, RH_MATE_SHIFT = 35, RH_LIB_SHIFT = 36, RH_OFFSET_SHIFT = 40;
static const int RH_MAX_OFFSET = (1 << 23) - 1;

// ReadHeadInfo.makeUUID (ReadHeadInfo.java:100-127); the range checks are done by the caller.
static inline int64_t make_uuid(int mate, int lib, int64_t read_id, int offset) {
    if (offset < 0) offset = -offset | (RH_MAX_OFFSET + 1);
    return (int64_t)(((uint64_t)(int64_t)offset << RH_OFFSET_SHIFT) + ((uint64_t)lib << RH_LIB_SHIFT) +
                     ((uint64_t)mate << RH_MATE_SHIFT) + (uint64_t)read_id);
}
static inline int uuid_mate(int64_t v) { return (int)(((uint64_t)v >> RH_MATE_SHIFT) & 1); }
static inline int uuid_lib(int64_t v) { return (int)(((uint64_t)v >> RH_LIB_SHIFT) & 0xf); }
static inline int64_t uuid_read_id(int64_t v) { return (int64_t)((uint64_t)v & ((1ULL << RH_BITS_READID) - 1)); }
// ReadHeadInfo.getOffset (ReadHeadInfo.java:168-176)
static inline int uuid_offset(int64_t v) {
    int off = (int)((uint64_t)v >> RH_OFFSET_SHIFT);
    if ((off & (RH_MAX_OFFSET + 1)) != 0) off = -(off & RH_MAX_OFFSET);
    return off;
}

struct ReadHead {
    int64_t uuid = 0;
    std::string read;  // VKmer bytes (header + packed)
    std::string mate;  // VKmer bytes; empty string = no mate sequence
};
// ReadHeadInfo.compareTo order (ReadHeadInfo.java:247-264): offset, library, mate, readId
struct RHKey {
    int offset;
    int lib;
    int mate;
    int64_t read_id;
    bool operator<(const RHKey &o) const {
        return std::tie(offset, lib, mate, read_id) < std::tie(o.offset, o.lib, o.mate, o.read_id);
    }
};
static inline RHKey rh_key(int64_t uuid) {
    return RHKey{uuid_offset(uuid), uuid_lib(uuid), uuid_mate(uuid), uuid_read_id(uuid)};
}
using ReadHeadSet = std::map<RHKey, ReadHead>;  // TreeSet<ReadHeadInfo>

// ReadHeadInfo.write (ReadHeadInfo.java:205-212)
static void write_read_head(std::string &o, const ReadHead &h) {
    bool has_mate = h.mate.size() > 4 && get_i32((const uint8_t *)h.mate.data()) > 0;
    o.push_back(has_mate ? 1 : 0);
    put_i64(o, h.uuid);
    o += h.read;
    if (has_mate) o += h.mate;
}

// ---------------------------------------------------------------------------------------
// Node (genomix-data/.../types/Node.java:408-487)
// ---------------------------------------------------------------------------------------
struct Node {
    bool has_edges[4] = {false, false, false, false};
    std::vector<std::string> edges[4];  // VKmer bytes per EDGETYPE FF, FR, RF, RR
    bool has_unflipped = false, has_flipped = false;
    ReadHeadSet unflipped, flipped;
    bool has_cov = false;
    float cov = 0.0f;
};
enum { NODE_UNFLIPPED = 1 << 4, NODE_FLIPPED = 1 << 5, NODE_INTERNAL_KMER = 1 << 6, NODE_COVERAGE = 1 << 7 };

// ExternalableTreeSet.write with writeEntireBody forced (ExternalableTreeSet.java:235-267,
// ReadsKeyValueParserFactory.java:78): boolean true, int32 size, elements in TreeSet order.
static void write_read_head_set(std::string &o, const ReadHeadSet &s) {
    o.push_back(1);
    put_i32(o, (int32_t)s.size());
    for (auto &kv : s) write_read_head(o, kv.second);
}

// Node.write (Node.java:408-427) with getActiveFields (:466-487)
static void write_node(std::string &o, const Node &n) {
    uint8_t active = 0;
    for (int e = 0; e < 4; e++)
        if (n.has_edges[e] && !n.edges[e].empty()) active |= (uint8_t)(1 << e);
    if (n.has_unflipped && !n.unflipped.empty()) active |= NODE_UNFLIPPED;
    if (n.has_flipped && !n.flipped.empty()) active |= NODE_FLIPPED;
    if (n.has_cov) active |= NODE_COVERAGE;
    o.push_back((char)active);
    for (int e = 0; e < 4; e++) {
        if (!(active & (1 << e))) continue;
        // VKmerList.write (VKmerList.java:313-316): int32 count, then the VKmers
        put_i32(o, (int32_t)n.edges[e].size());
        for (auto &v : n.edges[e]) o += v;
    }
    if (active & NODE_UNFLIPPED) write_read_head_set(o, n.unflipped);
    if (active & NODE_FLIPPED) write_read_head_set(o, n.flipped);
    if (active & NODE_COVERAGE) put_f32(o, n.cov);
}

struct Reader {
    const uint8_t *p;
    const uint8_t *end;
    bool ok = true;
    bool need(size_t n) {
        if ((size_t)(end - p) < n) ok = false;
        return ok;
    }
    uint8_t u8() { return need(1) ? *p++ : 0; }
    int32_t i32() {
        if (!need(4)) return 0;
        int32_t v = get_i32(p);
        p += 4;
        return v;
    }
    int64_t i64() {
        if (!need(8)) return 0;
        int64_t v = get_i64(p);
        p += 8;
        return v;
    }
    float f32() {
        if (!need(4)) return 0;
        float v = get_f32(p);
        p += 4;
        return v;
    }
    // VKmer.readFields (VKmer.java:371-383)
    std::string vkmer() {
        int32_t k = i32();
        if (!ok || k < 0) {
            ok = false;
            return std::string();
        }
        int nb = byte_num_from_k(k);
        if (!need(nb)) return std::string();
        std::string o;
        put_i32(o, k);
        o.append((const char *)p, nb);
        p += nb;
        return o;
    }
};

// ExternalableTreeSet.readFields (ExternalableTreeSet.java:217-233) + ReadHeadInfo.readFields
static void read_read_head_set(Reader &r, ReadHeadSet &s) {
    s.clear();
    uint8_t whole = r.u8();
    if (!whole) {  // a spilled set names a local file; the graph build always writes whole bodies
        r.ok = false;
        return;
    }
    int32_t n = r.i32();
    for (int32_t i = 0; i < n && r.ok; i++) {
        ReadHead h;
        uint8_t flags = r.u8();
        h.uuid = r.i64();
        h.read = r.vkmer();
        if (flags & 1) h.mate = r.vkmer();
        s.emplace(rh_key(h.uuid), std::move(h));  // TreeSet.add keeps the first equal element
    }
}

// Node.readFields (Node.java:435-456)
static bool read_node(Reader &r, Node &n) {
    n = Node();
    uint8_t active = r.u8();
    for (int e = 0; e < 4; e++) {
        if (active & (1 << e)) {
            n.has_edges[e] = true;
            int32_t cnt = r.i32();
            for (int32_t i = 0; i < cnt && r.ok; i++) n.edges[e].push_back(r.vkmer());
        }
    }
    if (active & NODE_UNFLIPPED) {
        n.has_unflipped = true;
        read_read_head_set(r, n.unflipped);
    }
    if (active & NODE_FLIPPED) {
        n.has_flipped = true;
        read_read_head_set(r, n.flipped);
    }
    if (active & NODE_INTERNAL_KMER) r.vkmer();  // never set by the graph build
    if (active & NODE_COVERAGE) {
        n.has_cov = true;
        n.cov = r.f32();
    }
    return r.ok;
}

// VKmerList.unionUpdate (VKmerList.java:117-133): set union keyed by the VKmer bytes.
// The result is kept sorted by bytes (see the file header).
static void union_edges(std::vector<std::string> &mine, const std::vector<std::string> &other) {
    mine.insert(mine.end(), other.begin(), other.end());
    std::sort(mine.begin(), mine.end());
    mine.erase(std::unique(mine.begin(), mine.end()), mine.end());
}

// AggregateKmerAggregateFactory.init (:93-125) and aggregate (:128-175)
static void aggregate_into(Node &acc, const Node &rd, bool first) {
    for (int e = 0; e < 4; e++) {
        acc.has_edges[e] = true;  // getEdges(e) creates the list
        union_edges(acc.edges[e], rd.edges[e]);
    }
    acc.has_unflipped = acc.has_flipped = true;
    for (auto &kv : rd.unflipped) acc.unflipped.emplace(kv.first, kv.second);  // TreeSet.addAll
    for (auto &kv : rd.flipped) acc.flipped.emplace(kv.first, kv.second);
    acc.has_cov = true;
    if (first) {
        acc.cov = rd.cov;
    } else {
        volatile float s = acc.cov + rd.cov;  // Java float addition, no contraction
        acc.cov = s;
    }
}

// ---------------------------------------------------------------------------------------
// Tuples: (Kmer bytes, Node bytes), stored in one arena per producer
// ---------------------------------------------------------------------------------------
struct TupleStore {
    std::string arena;
    struct T {
        uint64_t off;
        uint32_t klen, vlen;
    };
    std::vector<T> t;
    void add(const uint8_t *key, int klen, const std::string &val) {
        T x{arena.size(), (uint32_t)klen, (uint32_t)val.size()};
        arena.append((const char *)key, klen);
        arena += val;
        t.push_back(x);
    }
    const uint8_t *key(size_t i) const { return (const uint8_t *)arena.data() + t[i].off; }
    const uint8_t *val(size_t i) const { return (const uint8_t *)arena.data() + t[i].off + t[i].klen; }
};

// ---------------------------------------------------------------------------------------
// Line handling
// ---------------------------------------------------------------------------------------
struct Line {
    uint64_t begin, end;  // content bytes [begin, end) within the input
};

// Hadoop's LineReader: '\n', '\r' and "\r\n" end a line; the last line needs no terminator.
static void split_lines(const uint8_t *s, size_t n, std::vector<Line> &out) {
    size_t start = 0;
    for (size_t i = 0; i < n; i++) {
        if (s[i] == '\n') {
            out.push_back(Line{start, i});
            start = i + 1;
        } else if (s[i] == '\r') {
            out.push_back(Line{start, i});
            if (i + 1 < n && s[i + 1] == '\n') i++;
            start = i + 1;
        }
    }
    if (start < n) out.push_back(Line{start, n});
}

// Long.parseLong with radix 10 (ASCII digits), returns false where Java throws.
static bool java_parse_long(const uint8_t *s, size_t n, int64_t &out) {
    if (n == 0) return false;
    size_t i = 0;
    bool neg = false;
    if (s[0] == '-' || s[0] == '+') {
        if (n == 1) return false;
        neg = s[0] == '-';
        i = 1;
    }
    uint64_t limit = neg ? (1ULL << 63) : ((1ULL << 63) - 1);
    uint64_t v = 0;
    for (; i < n; i++) {
        if (s[i] < '0' || s[i] > '9') return false;
        uint64_t d = s[i] - '0';
        if (v > (limit - d) / 10) return false;
        v = v * 10 + d;
    }
    out = neg ? (int64_t)(0 - v) : (int64_t)v;
    return true;
}

static inline bool matches_acgt(const uint8_t *s, size_t n) {
    if (n == 0) return false;
    for (size_t i = 0; i < n; i++) {
        switch (s[i]) {
            case 'A': case 'C': case 'G': case 'T': case 'a': case 'c': case 'g': case 't': break;
            default: return false;
        }
    }
    return true;
}

struct Field {
    const uint8_t *p;
    size_t n;
};

// value.toString().split("\\t"): every tab splits, trailing empty strings are removed; a
// line without a tab is one field (possibly empty).  Returns the field count; fills the
// first `cap` fields.
static int java_split_tab(const uint8_t *s, size_t n, Field *f, int cap) {
    std::vector<Field> all;
    size_t st = 0;
    bool any_tab = false;
    for (size_t i = 0; i < n; i++) {
        if (s[i] == '\t') {
            all.push_back(Field{s + st, i - st});
            st = i + 1;
            any_tab = true;
        }
    }
    all.push_back(Field{s + st, n - st});
    if (!any_tab) {
        f[0] = all[0];
        return 1;
    }
    while (!all.empty() && all.back().n == 0) all.pop_back();
    for (int i = 0; i < (int)all.size() && i < cap; i++) f[i] = all[i];
    return (int)all.size();
}

// ---------------------------------------------------------------------------------------
// The parser: ReadsKeyValueParserFactory.parse / SplitReads
// ---------------------------------------------------------------------------------------
struct ParseStats {
    uint64_t reads = 0, kmers = 0, heads = 0;
};

enum DIR { FORWARD = 0, REVERSE = 1 };
enum EDGETYPE { FF = 0, FR = 1, RF = 2, RR = 3 };

struct Parser {
    KmerOps ko;
    TupleStore &out;
    ParseStats st;
    // Only the tuples whose key the reference's partitioner sends to part keep_part of keep_of
    // are stored (keep_part < 0: all).  Every occurrence of a key goes to the same part, so the
    // parts built one at a time hold exactly the records of the whole build, with the memory of
    // one part: this is how whole benchmark-size inputs are checked.
    int keep_part = -1, keep_of = 1;
    bool kept(const uint8_t *key) const { return keep_part < 0 || kmer_partition(key, ko.nb, keep_of) == keep_part; }

    Parser(int k, TupleStore &o) : out(o) {
        ko.k = k;
        ko.nb = byte_num_from_k(k);
    }

    // SplitReads (ReadsKeyValueParserFactory.java:150-196)
    int split_reads(const ReadHead &rh_in, const uint8_t *s, int len) {
        const int k = ko.k, nb = ko.nb;
        if (k >= len) return GX_EREAD_TOO_SHORT;
        st.reads++;
        st.kmers += (uint64_t)(len - k + 1);
        std::vector<uint8_t> curF(nb), curR(nb), nextF(nb), nextR(nb);
        ReadHead rh = rh_in;
        Node cur;
        cur.has_cov = true;
        cur.cov = 1.0f;
        ko.set_from_string(curF.data(), s, 0, len);
        ko.set_reversed_from_string(curR.data(), s, 0, len);
        DIR curDir = compare_bytes(curF.data(), nb, curR.data(), nb) <= 0 ? FORWARD : REVERSE;
        if (curDir == FORWARD) {
            cur.has_unflipped = true;
            cur.unflipped.emplace(rh_key(rh.uuid), rh);
        } else {
            // readHeadInfo.resetOffset(k - 1)
            rh.uuid = make_uuid(uuid_mate(rh.uuid), uuid_lib(rh.uuid), uuid_read_id(rh.uuid), k - 1);
            cur.has_flipped = true;
            cur.flipped.emplace(rh_key(rh.uuid), rh);
        }
        st.heads++;
        Node next;
        next.has_cov = true;
        next.cov = 1.0f;
        nextF = curF;
        for (int i = k; i < len; i++) {
            ko.shift_with_next_char(nextF.data(), s[i]);
            ko.set_reversed_from_string(nextR.data(), s, i - k + 1, len);
            DIR nextDir = compare_bytes(nextF.data(), nb, nextR.data(), nb) <= 0 ? FORWARD : REVERSE;
            set_edges(curDir, cur, nextDir, next, curF, curR, nextF, nextR);
            write_to_frame(curF, curR, curDir, cur);
            curF = nextF;
            curR = nextR;
            cur = std::move(next);
            curDir = nextDir;
            next = Node();
            next.has_cov = true;
            next.cov = 1.0f;
        }
        write_to_frame(curF, curR, curDir, cur);
        return GX_OK;
    }

    // setEdgesForCurAndNext (ReadsKeyValueParserFactory.java:209-233)
    void set_edges(DIR cd, Node &cur, DIR nd, Node &next, const std::vector<uint8_t> &curF,
                   const std::vector<uint8_t> &curR, const std::vector<uint8_t> &nextF,
                   const std::vector<uint8_t> &nextR) {
        const int k = ko.k, nb = ko.nb;
        // an edge of a node that is not stored changes no output (the skip only saves time)
        const bool keep_cur = keep_part < 0 || kept(cd == FORWARD ? curF.data() : curR.data());
        const bool keep_next = keep_part < 0 || kept(nd == FORWARD ? nextF.data() : nextR.data());
        auto app = [&](Node &n, int e, const std::vector<uint8_t> &km) {
            if (&n == &cur ? !keep_cur : !keep_next) return;
            n.has_edges[e] = true;
            n.edges[e].push_back(vkmer_from_kmer(k, km.data(), nb));
        };
        if (cd == FORWARD && nd == FORWARD) {
            app(cur, FF, nextF);
            app(next, RR, curF);
        } else if (cd == FORWARD && nd == REVERSE) {
            app(cur, FR, nextR);
            app(next, FR, curF);
        } else if (cd == REVERSE && nd == FORWARD) {
            app(cur, RF, nextF);
            app(next, RF, curR);
        } else {
            app(cur, RR, nextR);
            app(next, FF, curR);
        }
    }

    // writeToFrame / InsertToFrame (ReadsKeyValueParserFactory.java:198-254)
    void write_to_frame(const std::vector<uint8_t> &f, const std::vector<uint8_t> &r, DIR d, const Node &n) {
        if (!kept(d == FORWARD ? f.data() : r.data())) return;
        std::string v;
        write_node(v, n);
        out.add(d == FORWARD ? f.data() : r.data(), ko.nb, v);
    }

    // parse (ReadsKeyValueParserFactory.java:95-148); library id is always 0 (:98-106)
    int parse(const uint8_t *s, size_t n) {
        Field f[3];
        int nf = java_split_tab(s, n, f, 3);
        if (nf != 2 && nf != 3) return GX_EINVAL_LINE;
        int64_t read_id;
        if (!java_parse_long(f[0].p, f[0].n, read_id)) return GX_EINVAL_NUMBER;
        const Field m0 = f[1];
        const bool has_m1 = nf == 3;
        const Field m1 = has_m1 ? f[2] : Field{nullptr, 0};
        const bool id_ok = read_id >= 0 && read_id < (1LL << RH_BITS_READID);
        if (matches_acgt(m0.p, m0.n)) {
            if (!id_ok) return GX_EREADID_RANGE;
            ReadHead rh;
            rh.uuid = make_uuid(0, 0, read_id, 0);
            rh.read = vkmer_from_string(m0.p, (int)m0.n);
            if (has_m1) rh.mate = vkmer_from_string(m1.p, (int)m1.n);
            int e = split_reads(rh, m0.p, (int)m0.n);
            if (e != GX_OK) return e;
        }
        if (has_m1 && matches_acgt(m1.p, m1.n)) {
            if (!id_ok) return GX_EREADID_RANGE;
            ReadHead rh;
            rh.uuid = make_uuid(1, 0, read_id, 0);
            rh.read = vkmer_from_string(m1.p, (int)m1.n);
            rh.mate = vkmer_from_string(m0.p, (int)m0.n);
            int e = split_reads(rh, m1.p, (int)m1.n);
            if (e != GX_OK) return e;
        }
        return GX_OK;
    }
};

// ---------------------------------------------------------------------------------------
// Sort + group (Hyracks ExternalSort + PreclusteredGroup with the Genomix aggregator)
// ---------------------------------------------------------------------------------------
struct Grouped {
    std::string key;  // Kmer bytes
    std::string val;  // Node bytes after aggregation
};

static void sort_tuples(const TupleStore &ts, std::vector<uint32_t> &idx) {
    idx.resize(ts.t.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (uint32_t)i;
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
        return kmer_pointable_compare(ts.key(a), ts.t[a].klen, ts.key(b), ts.t[b].klen) < 0;
    });
}

// Groups a key-sorted sequence of (key, node bytes) items; calls emit per group.
template <class KeyAt, class ValAt, class Emit>
static void group_sorted(size_t n, KeyAt key_at, ValAt val_at, Emit emit) {
    size_t i = 0;
    while (i < n) {
        const uint8_t *kp;
        int kl;
        key_at(i, kp, kl);
        Node acc;
        bool first = true;
        size_t j = i;
        for (; j < n; j++) {
            const uint8_t *kq;
            int kql;
            key_at(j, kq, kql);
            if (kmer_pointable_compare(kp, kl, kq, kql) != 0) break;
            const uint8_t *vp;
            size_t vl;
            val_at(j, vp, vl);
            Reader r{vp, vp + vl};
            Node rd;
            read_node(r, rd);
            aggregate_into(acc, rd, first);
            first = false;
        }
        std::string v;
        write_node(v, acc);
        emit(std::string((const char *)kp, kl), std::move(v), acc);
        i = j;
    }
}

struct Result {
    int status = GX_OK;
    uint64_t error_line = 0;
    uint64_t lines = 0, reads = 0, kmers = 0, heads = 0, nodes = 0;
    std::vector<std::string> parts;  // serialized SequenceFile record bodies per partition
};

// KmerNodePairSequenceWriterFactory.write (:79-94) framed as SequenceFile.Writer.append:
// int32 record length, int32 key length, key (VKmer), value (Node).
static void append_record(std::string &o, int k, const std::string &kmer, const std::string &node) {
    std::string key = vkmer_from_kmer(k, (const uint8_t *)kmer.data(), (int)kmer.size());
    put_i32(o, (int32_t)(key.size() + node.size()));
    put_i32(o, (int32_t)key.size());
    o += key;
    o += node;
}

// The whole job.  threads = input splits = partitions (one NC partition per thread).
// only_part >= 0: build only the records of that part (the others stay empty).
static Result build(const uint8_t *text, size_t n, int k, int threads, int parts, int only_part = -1) {
    Result res;
    if (k < 3 || threads < 1 || parts < 1 || only_part >= parts) {
        res.status = GX_EINVAL;
        return res;
    }
    std::vector<Line> lines;
    split_lines(text, n, lines);
    res.lines = lines.size();
    const int T = threads, P = parts;
    // local stage: parse -> sort -> group, then route groups to partitions
    std::vector<std::vector<std::vector<Grouped>>> routed(T, std::vector<std::vector<Grouped>>(P));
    std::vector<int> t_status(T, GX_OK);
    std::vector<uint64_t> t_err(T, 0);
    std::vector<ParseStats> t_stats(T);
    auto local = [&](int t) {
        size_t a = lines.size() * (size_t)t / T, b = lines.size() * (size_t)(t + 1) / T;
        TupleStore ts;
        Parser ps(k, ts);
        ps.keep_part = only_part;
        ps.keep_of = P;
        for (size_t i = a; i < b; i++) {
            int e = ps.parse(text + lines[i].begin, lines[i].end - lines[i].begin);
            if (e != GX_OK) {
                t_status[t] = e;
                t_err[t] = i + 1;
                return;
            }
        }
        t_stats[t] = ps.st;
        std::vector<uint32_t> idx;
        sort_tuples(ts, idx);
        group_sorted(
            idx.size(),
            [&](size_t i, const uint8_t *&p, int &l) {
                p = ts.key(idx[i]);
                l = (int)ts.t[idx[i]].klen;
            },
            [&](size_t i, const uint8_t *&p, size_t &l) {
                p = ts.val(idx[i]);
                l = ts.t[idx[i]].vlen;
            },
            [&](std::string &&key, std::string &&val, const Node &) {
                int p = kmer_partition((const uint8_t *)key.data(), (int)key.size(), P);
                routed[t][p].push_back(Grouped{std::move(key), std::move(val)});
            });
    };
    {
        std::vector<std::thread> th;
        for (int t = 1; t < T; t++) th.emplace_back(local, t);
        local(0);
        for (auto &x : th) x.join();
    }
    // the first error by line order aborts the job
    for (int t = 0; t < T; t++) {
        if (t_status[t] != GX_OK) {
            res.status = t_status[t];
            res.error_line = t_err[t];
            return res;
        }
    }
    for (auto &s : t_stats) {
        res.reads += s.reads;
        res.kmers += s.kmers;
        res.heads += s.heads;
    }
    // global stage: merge the sorted runs of each partition (M:N partitioning-merging
    // connector), group again, write the part
    res.parts.assign(P, std::string());
    std::vector<uint64_t> p_nodes(P, 0), p_heads(P, 0);
    auto global = [&](int p) {
        std::vector<const Grouped *> items;
        for (int t = 0; t < T; t++)
            for (auto &g : routed[t][p]) items.push_back(&g);
        std::stable_sort(items.begin(), items.end(), [](const Grouped *a, const Grouped *b) {
            return kmer_pointable_compare((const uint8_t *)a->key.data(), (int)a->key.size(),
                                          (const uint8_t *)b->key.data(), (int)b->key.size()) < 0;
        });
        std::string &o = res.parts[p];
        group_sorted(
            items.size(),
            [&](size_t i, const uint8_t *&kp, int &l) {
                kp = (const uint8_t *)items[i]->key.data();
                l = (int)items[i]->key.size();
            },
            [&](size_t i, const uint8_t *&vp, size_t &l) {
                vp = (const uint8_t *)items[i]->val.data();
                l = items[i]->val.size();
            },
            [&](std::string &&key, std::string &&val, const Node &acc) {
                append_record(o, k, key, val);
                p_nodes[p]++;
                p_heads[p] += acc.unflipped.size() + acc.flipped.size();
            });
    };
    {
        std::vector<std::thread> th;
        for (int p = 1; p < P; p++) th.emplace_back(global, p);
        global(0);
        for (auto &x : th) x.join();
    }
    for (auto v : p_nodes) res.nodes += v;
    res.heads = 0;  // read heads in the output (TreeSet de-duplicates equal uuids)
    for (auto v : p_heads) res.heads += v;
    return res;
}

// The BUILD_READ_PARSER plan (JobGenReadLetterParser.java:60-147): the parser's tuples as
// they come, one (Kmer, Node) SequenceFile record per k-mer occurrence in read order.  The
// key is Kmer.write: the nb packed bytes alone (Kmer.java:344-346).
static int read_parser(const uint8_t *text, size_t n, int k, std::string &out, uint64_t &error_line,
                       uint64_t &occurrences) {
    std::vector<Line> lines;
    split_lines(text, n, lines);
    TupleStore ts;
    Parser ps(k, ts);
    for (size_t i = 0; i < lines.size(); i++) {
        const int e = ps.parse(text + lines[i].begin, lines[i].end - lines[i].begin);
        if (e != GX_OK) {
            error_line = i + 1;
            return e;
        }
    }
    occurrences = ts.t.size();
    for (size_t i = 0; i < ts.t.size(); i++) {
        put_i32(out, (int32_t)(ts.t[i].klen + ts.t[i].vlen));
        put_i32(out, (int32_t)ts.t[i].klen);
        out.append((const char *)ts.key(i), ts.t[i].klen + ts.t[i].vlen);
    }
    return GX_OK;
}

// ---------------------------------------------------------------------------------------
// Record streams: parse, normalise (the comparison form), text dump
// ---------------------------------------------------------------------------------------
struct Rec {
    std::string key;  // VKmer bytes
    Node node;
};

static bool parse_records(const uint8_t *s, size_t n, std::vector<Rec> &out) {
    Reader r{s, s + n};
    while (r.p < r.end) {
        int32_t rec_len = r.i32();
        int32_t key_len = r.i32();
        if (!r.ok || rec_len < key_len || key_len < 4 || !r.need((size_t)rec_len)) return false;
        const uint8_t *rec_end = r.p + rec_len;
        Rec x;
        x.key = std::string((const char *)r.p, key_len);
        Reader rv{r.p + key_len, rec_end};
        if (!read_node(rv, x.node) || rv.p != rec_end) return false;
        r.p = rec_end;
        out.push_back(std::move(x));
    }
    return r.ok;
}

// Comparison form: records sorted by VKmer order (VKmer.Comparator, VKmer.java:418-433),
// every edge list sorted by bytes.
static std::string normalize(const uint8_t *s, size_t n, bool &ok) {
    std::vector<Rec> recs;
    ok = parse_records(s, n, recs);
    std::string o;
    if (!ok) return o;
    for (auto &r : recs)
        for (int e = 0; e < 4; e++) std::sort(r.node.edges[e].begin(), r.node.edges[e].end());
    std::sort(recs.begin(), recs.end(), [](const Rec &a, const Rec &b) {
        const uint8_t *x = (const uint8_t *)a.key.data(), *y = (const uint8_t *)b.key.data();
        int ka = get_i32(x), kb = get_i32(y);
        if (ka != kb) return ka < kb;
        return compare_bytes(x + 4, (int)a.key.size() - 4, y + 4, (int)b.key.size() - 4) < 0;
    });
    for (auto &r : recs) {
        std::string v;
        write_node(v, r.node);
        put_i32(o, (int32_t)(r.key.size() + v.size()));
        put_i32(o, (int32_t)r.key.size());
        o += r.key;
        o += v;
    }
    return o;
}

static std::string vkmer_to_string(const std::string &v) {
    const uint8_t *p = (const uint8_t *)v.data();
    int k = get_i32(p);
    return recover_kmer(k, p + 4, (int)v.size() - 4);
}

// Java Float.toString: the shortest decimal that reads back as the same float; plain
// notation for 1e-3 <= |f| < 1e7, computerized scientific notation otherwise.
static std::string java_float_to_string(float f) {
    if (std::isnan(f)) return "NaN";
    if (std::isinf(f)) return f > 0 ? "Infinity" : "-Infinity";
    if (f == 0.0f) return std::signbit(f) ? "-0.0" : "0.0";
    char buf[64];
    int prec = 1;
    for (; prec <= 9; prec++) {
        snprintf(buf, sizeof buf, "%.*e", prec - 1, (double)f);
        if (strtof(buf, nullptr) == f) break;
    }
    // buf = [-]d.ddde[+-]XX ; pull the digits and exponent
    std::string m(buf);
    bool neg = m[0] == '-';
    if (neg) m = m.substr(1);
    size_t epos = m.find('e');
    int exp10 = atoi(m.c_str() + epos + 1);
    std::string digits;
    for (size_t i = 0; i < epos; i++)
        if (m[i] != '.') digits.push_back(m[i]);
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    std::string o = neg ? "-" : "";
    double a = std::fabs((double)f);
    if (a >= 1e-3 && a < 1e7) {
        if (exp10 >= 0) {
            std::string ip = digits.substr(0, std::min((size_t)exp10 + 1, digits.size()));
            while ((int)ip.size() < exp10 + 1) ip.push_back('0');
            std::string fp = (size_t)exp10 + 1 < digits.size() ? digits.substr(exp10 + 1) : "0";
            o += ip + "." + fp;
        } else {
            o += "0.";
            for (int i = 0; i < -exp10 - 1; i++) o.push_back('0');
            o += digits;
        }
    } else {
        o += digits.substr(0, 1) + "." + (digits.size() > 1 ? digits.substr(1) : "0") + "E" +
             std::to_string(exp10);
    }
    return o;
}

// ReadHeadInfo.toString (ReadHeadInfo.java:235-240) after a readFields round trip
static std::string read_head_to_string(const ReadHead &h) {
    std::string o = std::to_string(uuid_read_id(h.uuid)) + "-" + std::to_string(uuid_offset(h.uuid)) + "_" +
                    std::to_string(uuid_mate(h.uuid)) + "-" + std::to_string(uuid_lib(h.uuid)) + " readSeq: " +
                    vkmer_to_string(h.read) + " mateReadSeq: " + (h.mate.empty() ? "null" : vkmer_to_string(h.mate));
    return o;
}
static std::string read_head_set_to_string(const ReadHeadSet &s) {
    std::string o = "[";
    const char *delim = "";
    for (auto &kv : s) {
        o += delim + read_head_to_string(kv.second);
        delim = ",";
    }
    return o + "]";
}

// GenomixClusterManager.java:371 line: key.toString() + "\t" + Node.toString() (Node.java:524-537)
static std::string dump_text(const uint8_t *s, size_t n, bool &ok) {
    std::vector<Rec> recs;
    ok = parse_records(s, n, recs);
    std::string o;
    static const char *ET[4] = {"FF", "FR", "RF", "RR"};
    for (auto &r : recs) {
        o += vkmer_to_string(r.key);
        o += "\t{";
        for (int e = 0; e < 4; e++) {
            o += ET[e];
            o += ":";
            if (!r.node.has_edges[e]) {
                o += "null";
            } else {
                o += "[";
                for (size_t i = 0; i < r.node.edges[e].size(); i++) {
                    if (i) o += ",";
                    o += vkmer_to_string(r.node.edges[e][i]);
                }
                o += "]";
            }
            o += "\t";
        }
        o += "5':" + (r.node.has_unflipped ? read_head_set_to_string(r.node.unflipped) : std::string("null"));
        o += ", ~5':" + (r.node.has_flipped ? read_head_set_to_string(r.node.flipped) : std::string("null"));
        o += "\tkmer:null\tcov:" + (r.node.has_cov ? java_float_to_string(r.node.cov) + "x" : std::string("null")) + "}\n";
    }
    return o;
}

// ---------------------------------------------------------------------------------------
// GenomixDriver.convertAndUploadFastqToHDFS (GenomixDriver.java:665-714)
// ---------------------------------------------------------------------------------------
// BufferedReader.readLine: '\n', '\r', "\r\n" terminate; a last unterminated line counts.
static void reader_lines(const uint8_t *s, size_t n, std::vector<Line> &out) { split_lines(s, n, out); }

// String.trim: strips leading and trailing chars <= ' '
static inline void java_trim(const uint8_t *s, uint64_t &b, uint64_t &e) {
    while (b < e && s[b] <= ' ') b++;
    while (e > b && s[e - 1] <= ' ') e--;
}

static int fastq_to_readid(const uint8_t *m1, size_t n1, const uint8_t *m2, size_t n2, bool paired,
                           std::string &out) {
    std::vector<Line> l1, l2;
    reader_lines(m1, n1, l1);
    if (paired) {
        reader_lines(m2, n2, l2);
        if (l1.size() != l2.size()) return GX_EFASTQ_PAIRING;
    }
    for (size_t i = 0; i < l1.size(); i++) {
        if (i % 4 != 1) continue;
        out += std::to_string(i + 1);
        out.push_back('\t');
        uint64_t b = l1[i].begin, e = l1[i].end;
        java_trim(m1, b, e);
        out.append((const char *)m1 + b, e - b);
        if (paired) {
            out.push_back('\t');
            uint64_t b2 = l2[i].begin, e2 = l2[i].end;
            java_trim(m2, b2, e2);
            out.append((const char *)m2 + b2, e2 - b2);
        }
        out.push_back('\n');
    }
    return GX_OK;
}

}  // namespace gxo

// =======================================================================================
// C API for the tests and the CPU-baseline leg of the bench (ctypes)
// =======================================================================================
extern "C" {

struct gxo_result;
int gxo_build_part(const char *text, size_t n, int k, int threads, int parts, int part, gxo_result **out);

struct gxo_result {
    gxo::Result r;
    std::string all;  // parts concatenated in partition order
    std::vector<uint64_t> part_off;
};

// Builds the graph of readid text `text` with k, `threads` input splits and `parts`
// output partitions.  Returns the status; *out always receives a handle (free with
// gxo_result_free).
int gxo_build(const char *text, size_t n, int k, int threads, int parts, gxo_result **out) {
    return gxo_build_part(text, n, k, threads, parts, -1, out);
}

// The same build keeping only the records of part `part` of `parts` (the reference's
// partitioner, KmerPartitionComputerFactory.java:28-52); part -1 keeps every part.  The
// statistics other than nodes and heads are those of the whole input.
int gxo_build_part(const char *text, size_t n, int k, int threads, int parts, int part, gxo_result **out) {
    gxo_result *h = new gxo_result();
    h->r = gxo::build((const uint8_t *)text, n, k, threads, parts, part);
    h->part_off.push_back(0);
    for (auto &p : h->r.parts) {
        h->all += p;
        h->part_off.push_back(h->all.size());
    }
    h->r.parts.clear();
    h->r.parts.shrink_to_fit();
    *out = h;
    return h->r.status;
}

// stats: lines, reads, kmers, heads, nodes, error_line
void gxo_result_stats(const gxo_result *h, uint64_t *st6) {
    st6[0] = h->r.lines;
    st6[1] = h->r.reads;
    st6[2] = h->r.kmers;
    st6[3] = h->r.heads;
    st6[4] = h->r.nodes;
    st6[5] = h->r.error_line;
}
const char *gxo_result_records(const gxo_result *h, size_t *n) {
    *n = h->all.size();
    return h->all.data();
}
const uint64_t *gxo_result_part_offsets(const gxo_result *h, size_t *nparts) {
    *nparts = h->part_off.size() - 1;
    return h->part_off.data();
}
void gxo_result_free(gxo_result *h) { delete h; }

// Per-occurrence (Kmer, Node) records of the read-parser plan; *out is malloc'ed (gxo_free).
int gxo_read_parser(const char *text, size_t n, int k, char **out, size_t *out_n, uint64_t *error_line,
                    uint64_t *occurrences) {
    std::string o;
    *error_line = 0;
    *occurrences = 0;
    const int st = gxo::read_parser((const uint8_t *)text, n, k, o, *error_line, *occurrences);
    *out = (char *)malloc(o.size() ? o.size() : 1);
    memcpy(*out, o.data(), o.size());
    *out_n = o.size();
    return st;
}

static char *dup_out(const std::string &s, size_t *n) {
    char *p = (char *)malloc(s.size() + 1);
    if (!p) return nullptr;
    memcpy(p, s.data(), s.size());
    p[s.size()] = 0;
    *n = s.size();
    return p;
}

// Comparison form of a record stream (see gxo::normalize).  Returns 0 on success.
int gxo_normalize(const char *s, size_t n, char **out, size_t *out_n) {
    bool ok;
    std::string o = gxo::normalize((const uint8_t *)s, n, ok);
    *out = dup_out(o, out_n);
    return ok ? 0 : 1;
}
int gxo_dump_text(const char *s, size_t n, char **out, size_t *out_n) {
    bool ok;
    std::string o = gxo::dump_text((const uint8_t *)s, n, ok);
    *out = dup_out(o, out_n);
    return ok ? 0 : 1;
}
int gxo_fastq_to_readid(const char *m1, size_t n1, const char *m2, size_t n2, char **out, size_t *out_n) {
    std::string o;
    int st = gxo::fastq_to_readid((const uint8_t *)m1, n1, (const uint8_t *)m2, n2, m2 != nullptr, o);
    *out = dup_out(o, out_n);
    return st;
}
void gxo_free(void *p) { free(p); }

// Known-answer hooks for the unit tests (Kmer / ReadHeadInfo fixtures).
// Packs s[start..start+k) as Kmer.setFromStringBytes (reverse=0) or
// setReversedFromStringBytes (reverse=1) and returns it as a string.
int gxo_kat_kmer(const char *s, int len, int k, int start, int reverse, char *out_str) {
    gxo::KmerOps ko{k, gxo::byte_num_from_k(k)};
    std::vector<uint8_t> b(ko.nb);
    if (reverse)
        ko.set_reversed_from_string(b.data(), (const uint8_t *)s, start, len);
    else
        ko.set_from_string(b.data(), (const uint8_t *)s, start, len);
    std::string r = gxo::recover_kmer(k, b.data(), ko.nb);
    memcpy(out_str, r.data(), r.size());
    out_str[r.size()] = 0;
    return 0;
}
// Kmer.shiftKmerWithNextChar after setFromStringBytes(s, 0)
int gxo_kat_kmer_shift(const char *s, int len, int k, char next, char *out_str) {
    gxo::KmerOps ko{k, gxo::byte_num_from_k(k)};
    std::vector<uint8_t> b(ko.nb);
    ko.set_from_string(b.data(), (const uint8_t *)s, 0, len);
    ko.shift_with_next_char(b.data(), (uint8_t)next);
    std::string r = gxo::recover_kmer(k, b.data(), ko.nb);
    memcpy(out_str, r.data(), r.size());
    out_str[r.size()] = 0;
    return 0;
}
int64_t gxo_kat_uuid(int mate, int lib, int64_t read_id, int offset) { return gxo::make_uuid(mate, lib, read_id, offset); }
int gxo_kat_uuid_offset(int64_t uuid) { return gxo::uuid_offset(uuid); }
int gxo_kat_float_to_string(float f, char *out_str) {
    std::string r = gxo::java_float_to_string(f);
    memcpy(out_str, r.data(), r.size());
    out_str[r.size()] = 0;
    return 0;
}
}
