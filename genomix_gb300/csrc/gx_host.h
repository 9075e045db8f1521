// gx_host.h — host-side helpers shared by the job runner and the format code.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gxgpu.h"

namespace gxh {
void split_lines(const uint8_t *s, size_t n, std::vector<std::pair<size_t, size_t>> &out);
gx_status fastq_to_readid(const uint8_t *m1, size_t n1, const uint8_t *m2, size_t n2, std::string &out);
gx_status seqfile_write(const uint8_t *rec, size_t n, const uint8_t *sync, uint64_t seed, std::string &out,
                        const char *key_class);
gx_status seqfile_read(const uint8_t *f, size_t n, std::string &out);
gx_status records_to_text(const uint8_t *rec, size_t n, std::string &out);
gx_status records_digest(const uint8_t *rec, size_t n, gx_digest &d);
}  // namespace gxh
