// gx_fastq.cu — FASTQ to readid text on the GPU.
//
// The reference driver converts FASTQ before the graph build (GenomixDriver.
// convertAndUploadFastqToHDFS, genomix-driver/.../driver/GenomixDriver.java:665-714): lines
// are split as BufferedReader.readLine splits them (\n, \r, \r\n), and every line i
// (0-based) with i % 4 == 1 becomes the readid line "{i + 1}\t{seq.trim()}[\t{mate.trim()}]";
// paired files must have the same number of lines.  Here the line ends come from the same
// kernels as the readid parse, one thread per record finds and trims its sequence lines, a
// scan places the output lines, and one warp per record writes its line into the job's
// device text.  The result is byte for byte the host conversion's.
#include "gx_kernels.cuh"

namespace gx {

// the content [b, e) of line i: CR of a CRLF terminator excluded, then String.trim()
__device__ __forceinline__ void fq_line(const uint8_t *t, uint64_t n, const unsigned long long *le, uint64_t i,
                                        unsigned long long &b, unsigned long long &e) {
    b = i == 0 ? 0 : le[i - 1] + 1;
    e = le[i];
    if (e < n && e > b && t[e] == '\n' && t[e - 1] == '\r') e--;
    while (b < e && t[b] <= ' ') b++;
    while (e > b && t[e - 1] <= ' ') e--;
}

__device__ __forceinline__ uint32_t dec_digits(unsigned long long v) {
    uint32_t d = 1;
    while (v >= 10) {
        v /= 10;
        d++;
    }
    return d;
}

__global__ void k_fq_lines(const uint8_t *t1, uint64_t n1, const unsigned long long *le1, const uint8_t *t2,
                           uint64_t n2, const unsigned long long *le2, uint64_t n_rec, FqRec *rec,
                           unsigned long long *len) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rec) return;
    const uint64_t i = 4 * r + 1;
    FqRec q;
    fq_line(t1, n1, le1, i, q.b1, q.e1);
    q.b2 = q.e2 = 0;
    unsigned long long l = dec_digits(i + 1) + 1 + (q.e1 - q.b1) + 1;
    if (t2) {
        fq_line(t2, n2, le2, i, q.b2, q.e2);
        l += 1 + (q.e2 - q.b2);
    }
    rec[r] = q;
    len[r] = l;
}

__global__ void k_fq_write(const uint8_t *t1, const uint8_t *t2, uint64_t n_rec, const FqRec *rec,
                           const unsigned long long *off, uint8_t *out) {
    const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n_rec) return;
    const FqRec q = rec[r];
    uint8_t *o = out + off[r];
    const unsigned long long id = 4 * r + 2;
    const uint32_t nd = dec_digits(id);
    if (lane == 0) {
        unsigned long long v = id;
        for (int d = (int)nd - 1; d >= 0; d--) {
            o[d] = (uint8_t)('0' + v % 10);
            v /= 10;
        }
        o[nd] = '\t';
    }
    o += nd + 1;
    const unsigned long long l1 = q.e1 - q.b1;
    for (unsigned long long x = lane; x < l1; x += 32) o[x] = t1[q.b1 + x];
    o += l1;
    if (t2) {
        const unsigned long long l2 = q.e2 - q.b2;
        if (lane == 0) o[0] = '\t';
        for (unsigned long long x = lane; x < l2; x += 32) o[1 + x] = t2[q.b2 + x];
        o += 1 + l2;
    }
    if (lane == 0) o[0] = '\n';
}

void launch_fq_lines(const uint8_t *t1, uint64_t n1, const unsigned long long *le1, const uint8_t *t2, uint64_t n2,
                     const unsigned long long *le2, uint64_t n_rec, FqRec *rec, unsigned long long *len,
                     cudaStream_t s) {
    if (!n_rec) return;
    t_launches++;
    k_fq_lines<<<(unsigned)((n_rec + 255) / 256), 256, 0, s>>>(t1, n1, le1, t2, n2, le2, n_rec, rec, len);
}

void launch_fq_write(const uint8_t *t1, const uint8_t *t2, uint64_t n_rec, const FqRec *rec,
                     const unsigned long long *off, uint8_t *out, cudaStream_t s) {
    if (!n_rec) return;
    t_launches++;
    k_fq_write<<<(unsigned)((n_rec * 32 + 255) / 256), 256, 0, s>>>(t1, t2, n_rec, rec, off, out);
}

}  // namespace gx
