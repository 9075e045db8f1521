// gx_formats.cpp — host-side formats of the graph-build boundary:
//   - status strings
//   - FASTQ -> readid conversion (GenomixDriver.convertAndUploadFastqToHDFS, :665-714)
//   - Hadoop 0.20.2 SequenceFile container (KmerNodePairSequenceWriterFactory.java:66-73)
//   - text dump of records (GenomixClusterManager.copyBinAndTextToLocal, :371)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gxgpu.h"
#include "gx_host.h"

namespace gxh {

// ---- lines as java.io.BufferedReader.readLine / Hadoop LineReader split them --------------
void split_lines(const uint8_t *s, size_t n, std::vector<std::pair<size_t, size_t>> &out) {
    size_t st = 0;
    for (size_t i = 0; i < n; i++) {
        const uint8_t c = s[i];
        if (c == '\n' || c == '\r') {
            out.emplace_back(st, i);
            if (c == '\r' && i + 1 < n && s[i + 1] == '\n') i++;
            st = i + 1;
        }
    }
    if (st < n) out.emplace_back(st, n);
}

// String.trim(): drop leading and trailing chars <= ' '
static inline void trim(const uint8_t *s, size_t &b, size_t &e) {
    while (b < e && s[b] <= ' ') b++;
    while (e > b && s[e - 1] <= ' ') e--;
}

static void append_u64(std::string &o, uint64_t v) {
    char buf[24];
    int n = snprintf(buf, sizeof buf, "%llu", (unsigned long long)v);
    o.append(buf, (size_t)n);
}

// The i-th line (0-based) with i % 4 == 1 is a sequence line; its readId is i + 1, the
// 1-based line number, i.e. 4 * record + 2.
gx_status fastq_to_readid(const uint8_t *m1, size_t n1, const uint8_t *m2, size_t n2, std::string &out) {
    std::vector<std::pair<size_t, size_t>> l1, l2;
    split_lines(m1, n1, l1);
    if (m2) {
        split_lines(m2, n2, l2);
        if (l1.size() != l2.size()) return GX_EFASTQ_PAIRING;
    }
    out.reserve(out.size() + n1 + n2);
    for (size_t i = 1; i < l1.size(); i += 4) {
        append_u64(out, i + 1);
        out.push_back('\t');
        size_t b = l1[i].first, e = l1[i].second;
        trim(m1, b, e);
        out.append((const char *)m1 + b, e - b);
        if (m2) {
            out.push_back('\t');
            size_t b2 = l2[i].first, e2 = l2[i].second;
            trim(m2, b2, e2);
            out.append((const char *)m2 + b2, e2 - b2);
        }
        out.push_back('\n');
    }
    return GX_OK;
}

// ---- big-endian helpers -------------------------------------------------------------------
static inline uint32_t rd32(const uint8_t *p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static inline void wr32(std::string &o, uint32_t v) {
    const char b[4] = {(char)(v >> 24), (char)(v >> 16), (char)(v >> 8), (char)v};
    o.append(b, 4);
}

// ---- SequenceFile --------------------------------------------------------------------------
static const char KEY_CLASS[] = "edu.uci.ics.genomix.data.types.VKmer";
static const char VAL_CLASS[] = "edu.uci.ics.genomix.data.types.Node";
static const uint32_t SYNC_INTERVAL = 100 * (4 + 16);  // SequenceFile.SYNC_INTERVAL

// Text.writeString: WritableUtils vint length + UTF-8 bytes
static void write_text(std::string &o, const char *s) {
    const size_t n = strlen(s);
    o.push_back((char)n);  // class names are shorter than 128 bytes: a one-byte vint
    o.append(s, n);
}

gx_status seqfile_write(const uint8_t *rec, size_t n, const uint8_t *sync_in, uint64_t seed, std::string &out,
                        const char *key_class) {
    uint8_t sync[16];
    if (sync_in) {
        memcpy(sync, sync_in, 16);
    } else {
        uint64_t x = seed;
        for (int i = 0; i < 2; i++) {  // SplitMix64
            x += 0x9e3779b97f4a7c15ULL;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            z ^= z >> 31;
            for (int b = 0; b < 8; b++) sync[8 * i + b] = (uint8_t)(z >> (56 - 8 * b));
        }
    }
    out.clear();
    out.reserve(n + n / SYNC_INTERVAL * 20 + 256);
    // writeFileHeader: "SEQ" version 6, key/value class, compress flags, metadata, sync
    out.append("SEQ\x06", 4);
    write_text(out, key_class ? key_class : KEY_CLASS);
    write_text(out, VAL_CLASS);
    out.push_back(0);  // compressed
    out.push_back(0);  // block compressed
    wr32(out, 0);      // empty Metadata
    out.append((const char *)sync, 16);
    uint64_t last_sync = 0;
    size_t p = 0;
    while (p < n) {
        if (n - p < 8) return GX_EINVAL;
        const uint32_t rl = rd32(rec + p);
        if ((uint64_t)rl + 8 > n - p) return GX_EINVAL;
        // Writer.append -> checkAndWriteSync: escape + sync once 2000 bytes have passed
        if (out.size() >= last_sync + SYNC_INTERVAL && last_sync != out.size()) {
            wr32(out, 0xffffffffu);
            out.append((const char *)sync, 16);
            last_sync = out.size();
        }
        out.append((const char *)rec + p, (size_t)rl + 8);
        p += (size_t)rl + 8;
    }
    return GX_OK;
}

gx_status seqfile_read(const uint8_t *f, size_t n, std::string &out) {
    size_t p = 0;
    auto need = [&](size_t k) { return n - p >= k; };
    if (!need(4) || memcmp(f, "SEQ", 3) != 0 || f[3] != 6) return GX_EINVAL;
    p = 4;
    for (int i = 0; i < 2; i++) {  // class names (one-byte vint lengths)
        if (!need(1)) return GX_EINVAL;
        const int8_t l = (int8_t)f[p++];
        if (l < 0 || !need((size_t)l)) return GX_EINVAL;
        p += (size_t)l;
    }
    if (!need(2)) return GX_EINVAL;
    if (f[p] != 0 || f[p + 1] != 0) return GX_EINVAL;  // compressed files are not supported
    p += 2;
    if (!need(4)) return GX_EINVAL;
    const uint32_t nmeta = rd32(f + p);
    p += 4;
    for (uint32_t i = 0; i < 2 * nmeta; i++) {
        if (!need(1)) return GX_EINVAL;
        const int8_t l = (int8_t)f[p++];
        if (l < 0 || !need((size_t)l)) return GX_EINVAL;
        p += (size_t)l;
    }
    if (!need(16)) return GX_EINVAL;
    const uint8_t *sync = f + p;
    p += 16;
    out.clear();
    while (p < n) {
        if (!need(4)) return GX_EINVAL;
        const uint32_t rl = rd32(f + p);
        if (rl == 0xffffffffu) {
            if (!need(20) || memcmp(f + p + 4, sync, 16) != 0) return GX_EINVAL;
            p += 20;
            continue;
        }
        if (!need((size_t)rl + 8)) return GX_EINVAL;
        out.append((const char *)f + p, (size_t)rl + 8);
        p += (size_t)rl + 8;
    }
    return GX_OK;
}

// ---- text dump -----------------------------------------------------------------------------
static const char SYM[4] = {'A', 'C', 'G', 'T'};

// KmerUtil.recoverKmerFrom: letter i from bits 2*(i%4) of byte nb-1-i/4
static void put_kmer_text(std::string &o, uint32_t k, const uint8_t *b, size_t nb) {
    for (uint32_t i = 0; i < k; i++) o.push_back(SYM[(b[nb - 1 - i / 4] >> (2 * (i % 4))) & 3]);
}

// Float.toString: shortest digits that read back as the same float
static void put_java_float(std::string &o, float f) {
    if (std::isnan(f)) {
        o += "NaN";
        return;
    }
    if (std::isinf(f)) {
        o += f > 0 ? "Infinity" : "-Infinity";
        return;
    }
    if (f == 0.0f) {
        o += std::signbit(f) ? "-0.0" : "0.0";
        return;
    }
    char buf[48];
    for (int prec = 1; prec <= 9; prec++) {
        snprintf(buf, sizeof buf, "%.*e", prec - 1, (double)f);
        if (strtof(buf, nullptr) == f) break;
    }
    const char *q = buf;
    if (*q == '-') {
        o.push_back('-');
        q++;
    }
    std::string digits;
    while (*q && *q != 'e') {
        if (*q != '.') digits.push_back(*q);
        q++;
    }
    const int e10 = atoi(q + 1);
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    const double a = std::fabs((double)f);
    if (a >= 1e-3 && a < 1e7) {
        if (e10 >= 0) {
            std::string ip = digits.substr(0, std::min(digits.size(), (size_t)e10 + 1));
            while ((int)ip.size() < e10 + 1) ip.push_back('0');
            const std::string fp = (size_t)e10 + 1 < digits.size() ? digits.substr((size_t)e10 + 1) : "0";
            o += ip + "." + fp;
        } else {
            o += "0.";
            for (int i = 0; i < -e10 - 1; i++) o.push_back('0');
            o += digits;
        }
    } else {
        o += digits.substr(0, 1) + "." + (digits.size() > 1 ? digits.substr(1) : std::string("0")) + "E" +
             std::to_string(e10);
    }
}

struct Cur {
    const uint8_t *p, *e;
    bool ok = true;
    bool need(size_t n) {
        if ((size_t)(e - p) < n) ok = false;
        return ok;
    }
    uint8_t u8() { return need(1) ? *p++ : 0; }
    uint32_t u32() {
        if (!need(4)) return 0;
        const uint32_t v = rd32(p);
        p += 4;
        return v;
    }
    // a VKmer as text
    void vkmer(std::string &o) {
        const uint32_t k = u32();
        const size_t nb = (k + 3) / 4;
        if (!ok || k > (1u << 30) || !need(nb)) {
            ok = false;
            return;
        }
        put_kmer_text(o, k, p, nb);
        p += nb;
    }
};

static void read_head_set_text(Cur &c, std::string &o) {
    if (c.u8() != 1) {  // spilled sets are never written by the graph build
        c.ok = false;
        return;
    }
    const uint32_t n = c.u32();
    o.push_back('[');
    for (uint32_t i = 0; i < n && c.ok; i++) {
        if (i) o.push_back(',');
        const uint8_t flags = c.u8();
        if (!c.need(8)) return;
        uint64_t u = 0;
        for (int b = 0; b < 8; b++) u = (u << 8) | c.p[b];
        c.p += 8;
        // ReadHeadInfo.toString: readId-offset_mate-library readSeq: .. mateReadSeq: ..
        int off = (int)(u >> 40);
        if (off & (1 << 23)) off = -(off & ((1 << 23) - 1));
        append_u64(o, u & ((1ULL << 35) - 1));
        o += "-" + std::to_string(off) + "_" + std::to_string((u >> 35) & 1) + "-" + std::to_string((u >> 36) & 15) +
             " readSeq: ";
        c.vkmer(o);
        o += " mateReadSeq: ";
        if (flags & 1)
            c.vkmer(o);
        else
            o += "null";
    }
    o.push_back(']');
}

// ---- order-independent digest of a record stream ----------------------------------------
static inline uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline uint64_t hash_bytes(uint64_t h, const uint8_t *s, size_t n) {  // FNV-1a, 64-bit
    for (size_t i = 0; i < n; i++) h = (h ^ s[i]) * 0x100000001B3ULL;
    return h;
}

static gx_status digest_range(const uint8_t *rec, size_t n, gx_digest &d);

// Every record hashed in its normal form (each edge list's elements in byte order; read-head
// sets as written, since their order is the TreeSet's), the hashes combined by sum and xor.
// Large streams are cut at record boundaries and digested on all host threads.
gx_status records_digest(const uint8_t *rec, size_t n, gx_digest &d) {
    memset(&d, 0, sizeof d);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    if (n < (64u << 20) || hw == 1) return digest_range(rec, n, d);
    std::vector<size_t> cut{0};
    const size_t step = n / hw;
    size_t p = 0, next = step;
    while (p < n) {
        if (n - p < 8) return GX_EINVAL;
        const uint64_t rl = rd32(rec + p);
        if (rl + 8 > n - p) return GX_EINVAL;
        p += 8 + rl;
        if (p >= next && p < n) {
            cut.push_back(p);
            next = p + step;
        }
    }
    cut.push_back(n);
    const size_t T = cut.size() - 1;
    std::vector<gx_digest> part(T);
    std::vector<gx_status> st(T, GX_OK);
    std::vector<std::thread> th;
    for (size_t t = 0; t < T; t++)
        th.emplace_back([&, t] { st[t] = digest_range(rec + cut[t], cut[t + 1] - cut[t], part[t]); });
    for (auto &x : th) x.join();
    for (size_t t = 0; t < T; t++) {
        if (st[t] != GX_OK) return st[t];
        d.records += part[t].records;
        d.edges += part[t].edges;
        d.heads += part[t].heads;
        d.coverage += part[t].coverage;
        d.sum += part[t].sum;
        d.xor_ ^= part[t].xor_;
    }
    return GX_OK;
}

static gx_status digest_range(const uint8_t *rec, size_t n, gx_digest &d) {
    memset(&d, 0, sizeof d);
    size_t p = 0;
    std::vector<const uint8_t *> el;
    while (p < n) {
        if (n - p < 8) return GX_EINVAL;
        const uint32_t rl = rd32(rec + p), kl = rd32(rec + p + 4);
        if ((uint64_t)rl + 8 > n - p || kl > rl || kl < 4) return GX_EINVAL;
        const uint8_t *r = rec + p + 8, *re = r + rl;
        uint64_t h = hash_bytes(0xCBF29CE484222325ULL, r, kl);  // the key
        Cur c{r + kl, re};
        const uint8_t active = c.u8();
        h = hash_bytes(h, &active, 1);
        for (int t = 0; t < 4; t++) {
            if (!(active & (1 << t))) continue;
            const uint32_t cnt = c.u32();
            el.clear();
            size_t esz = 0;
            for (uint32_t i = 0; i < cnt && c.ok; i++) {
                if (!c.need(4)) break;
                const uint32_t kk = rd32(c.p);
                esz = 4 + (kk + 3) / 4;
                if (!c.need(esz)) break;
                el.push_back(c.p);
                c.p += esz;
            }
            if (!c.ok) return GX_EINVAL;
            std::sort(el.begin(), el.end(),
                      [esz](const uint8_t *a, const uint8_t *b) { return memcmp(a, b, esz) < 0; });
            const uint8_t tb = (uint8_t)t;
            h = hash_bytes(h, &tb, 1);
            for (const uint8_t *e : el) h = hash_bytes(h, e, esz);
            d.edges += cnt;
        }
        for (int set = 0; set < 2; set++) {
            if (!(active & (0x10 << set))) continue;
            const uint8_t *s0 = c.p;
            if (c.u8() != 1) return GX_EINVAL;
            const uint32_t cnt = c.u32();
            for (uint32_t i = 0; i < cnt && c.ok; i++) {
                const uint8_t flags = c.u8();
                if (!c.need(8)) return GX_EINVAL;
                c.p += 8;
                for (int m = 0; m < ((flags & 1) ? 2 : 1) && c.ok; m++) {
                    const uint32_t L = c.u32();
                    if (c.need((L + 3) / 4)) c.p += (L + 3) / 4;
                }
            }
            if (!c.ok) return GX_EINVAL;
            h = hash_bytes(h, s0, (size_t)(c.p - s0));
            d.heads += cnt;
        }
        if (!(active & 0x80) || !c.need(4) || c.p + 4 != re) return GX_EINVAL;
        const uint32_t cb = rd32(c.p);
        float cov;
        memcpy(&cov, &cb, 4);
        d.coverage += (uint64_t)cov;
        h = hash_bytes(h, c.p, 4);
        h = mix64(h);
        d.records++;
        d.sum += h;
        d.xor_ ^= h;
        p += 8 + rl;
    }
    return GX_OK;
}

gx_status records_to_text(const uint8_t *rec, size_t n, std::string &o) {
    static const char *ET[4] = {"FF", "FR", "RF", "RR"};
    size_t p = 0;
    while (p < n) {
        if (n - p < 8) return GX_EINVAL;
        const uint32_t rl = rd32(rec + p), kl = rd32(rec + p + 4);
        if ((uint64_t)rl + 8 > n - p || kl > rl) return GX_EINVAL;
        Cur key{rec + p + 8, rec + p + 8 + kl};
        key.vkmer(o);
        o.push_back('\t');
        Cur c{rec + p + 8 + kl, rec + p + 8 + rl};
        const uint8_t active = c.u8();
        o.push_back('{');
        for (int t = 0; t < 4; t++) {
            o += ET[t];
            o.push_back(':');
            if (active & (1 << t)) {
                const uint32_t cnt = c.u32();
                o.push_back('[');
                for (uint32_t i = 0; i < cnt && c.ok; i++) {
                    if (i) o.push_back(',');
                    c.vkmer(o);
                }
                o.push_back(']');
            } else {
                o += "null";
            }
            o.push_back('\t');
        }
        o += "5':";
        if (active & 0x10)
            read_head_set_text(c, o);
        else
            o += "null";
        o += ", ~5':";
        if (active & 0x20)
            read_head_set_text(c, o);
        else
            o += "null";
        o += "\tkmer:";
        if (active & 0x40)
            c.vkmer(o);
        else
            o += "null";
        o += "\tcov:";
        if (active & 0x80) {
            if (!c.need(4)) return GX_EINVAL;
            const uint32_t u = rd32(c.p);
            c.p += 4;
            float f;
            memcpy(&f, &u, 4);
            put_java_float(o, f);
            o.push_back('x');
        } else {
            o += "null";
        }
        o += "}\n";
        if (!key.ok || !c.ok || c.p != c.e) return GX_EINVAL;
        p += (size_t)rl + 8;
    }
    return GX_OK;
}

}  // namespace gxh

// ---- C ABI --------------------------------------------------------------------------------
extern "C" {

const char *gx_status_str(gx_status s) {
    switch (s) {
        case GX_OK: return "ok";
        case GX_EINVAL: return "invalid argument";
        case GX_EINVAL_LINE:
            return "input format is not correct! only support id'\\t'readSeq'\\t'mateReadSeq or id'\\t'readSeq";
        case GX_EINVAL_NUMBER: return "readId is not a number (NumberFormatException)";
        case GX_EREADID_RANGE: return "readId will lose some of its bits when saved (must be in [0, 2^35))";
        case GX_EREAD_TOO_SHORT: return "kmersize is larger than the read length";
        case GX_ENOMEM: return "out of memory";
        case GX_ETABLE_FULL: return "hash table partition full";
        case GX_ETIMEOUT: return "bounded device wait timed out";
        case GX_ECUDA: return "CUDA error";
        case GX_ESTATE: return "call out of order";
        case GX_ECANCELLED: return "job cancelled";
        case GX_EFASTQ_PAIRING: return "paired FASTQ files didn't have the same number of lines";
        case GX_EBUSY: return "busy: no admission slot or device memory";
        case GX_EAGAIN: return "not ready";
    }
    return "unknown status";
}

static gx_status give(const std::string &s, void **out, size_t *n) {
    char *p = (char *)malloc(s.size() + 1);
    if (!p) return GX_ENOMEM;
    memcpy(p, s.data(), s.size());
    p[s.size()] = 0;
    *out = p;
    *n = s.size();
    return GX_OK;
}

gx_status gx_fastq_to_readid(const void *mate1, size_t bytes1, const void *mate2, size_t bytes2, char **out,
                             size_t *out_bytes) {
    if ((!mate1 && bytes1) || !out || !out_bytes) return GX_EINVAL;
    std::string o;
    gx_status st = gxh::fastq_to_readid((const uint8_t *)mate1, bytes1, (const uint8_t *)mate2, bytes2, o);
    if (st != GX_OK) return st;
    return give(o, (void **)out, out_bytes);
}

void gx_host_free(void *ptr) { free(ptr); }

gx_status gx_seqfile_write(const void *records, size_t bytes, const uint8_t *sync, uint64_t seed, uint8_t **out,
                           size_t *out_bytes) {
    if ((!records && bytes) || !out || !out_bytes) return GX_EINVAL;
    std::string o;
    gx_status st = gxh::seqfile_write((const uint8_t *)records, bytes, sync, seed, o, nullptr);
    if (st != GX_OK) return st;
    return give(o, (void **)out, out_bytes);
}

gx_status gx_seqfile_write_kmer_keys(const void *records, size_t bytes, const uint8_t *sync, uint64_t seed,
                                     uint8_t **out, size_t *out_bytes) {
    if ((!records && bytes) || !out || !out_bytes) return GX_EINVAL;
    std::string o;
    gx_status st = gxh::seqfile_write((const uint8_t *)records, bytes, sync, seed, o,
                                      "edu.uci.ics.genomix.data.types.Kmer");
    if (st != GX_OK) return st;
    return give(o, (void **)out, out_bytes);
}

gx_status gx_seqfile_read(const void *file, size_t bytes, uint8_t **out, size_t *out_bytes) {
    if (!file || !out || !out_bytes) return GX_EINVAL;
    std::string o;
    gx_status st = gxh::seqfile_read((const uint8_t *)file, bytes, o);
    if (st != GX_OK) return st;
    return give(o, (void **)out, out_bytes);
}

gx_status gx_records_digest(const void *records, size_t bytes, gx_digest *out) {
    if ((!records && bytes) || !out) return GX_EINVAL;
    try {
        return gxh::records_digest((const uint8_t *)records, bytes, *out);
    } catch (...) {
        return GX_ENOMEM;
    }
}

gx_status gx_records_to_text(const void *records, size_t bytes, char **out, size_t *out_bytes) {
    if ((!records && bytes) || !out || !out_bytes) return GX_EINVAL;
    std::string o;
    gx_status st = gxh::records_to_text((const uint8_t *)records, bytes, o);
    if (st != GX_OK) return st;
    return give(o, (void **)out, out_bytes);
}
}
