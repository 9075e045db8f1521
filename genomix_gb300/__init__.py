"""genomix_gb300 — the Genomix graph-build step on one GB300 (CUDA sm_103a).

The compute path is libgxgpu.so (genomix_gb300/csrc, C ABI in include/gxgpu.h); this
package is its host-side mirror of the reference's driver and operator interface.
"""
from . import _lib
from .graph import (
    Context,
    GenomixGpuDriver,
    GraphBuildError,
    GraphBuildJob,
    PinnedBuffer,
    Server,
    batch_run,
    fastq_to_readid,
    fastq_to_readid_gpu,
    iter_records,
    records_digest,
    records_to_text,
    seqfile_read,
    seqfile_write,
)

__all__ = [
    "Context", "GenomixGpuDriver", "GraphBuildError", "GraphBuildJob", "PinnedBuffer", "Server", "batch_run",
    "fastq_to_readid", "fastq_to_readid_gpu", "iter_records", "records_digest", "records_to_text", "seqfile_read", "seqfile_write",
]
