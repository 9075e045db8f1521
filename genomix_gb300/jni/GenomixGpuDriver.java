/*
 * GenomixGpuDriver — the graph-build step of Genomix run on the GPU through libgxgpu.so.
 *
 * Drop-in beside GenomixHyracksDriver (genomix-hyracks/.../graph/driver/GenomixHyracksDriver.java:
 * 84-135): same runJob(conf, plan, profile) signature, same input (the readid files under
 * FileInputFormat's input paths) and the same output (SequenceFile<VKmer, Node> part files under
 * FileOutputFormat's output path, read unchanged by BinaryVertexInputFormat).  Selected from
 * GenomixDriver.addStep (GenomixDriver.java:188-197), e.g. for a BUILD_GPU pattern:
 *
 *     case BUILD_GPU:
 *         new GenomixGpuDriver(0).runJob(conf, Plan.BUILD_DEBRUIJN_GRAPH, runLocal);
 *         break;
 *
 * The native side is gxgpu_jni.c (built into libgxgpu_jni.so, linked against libgxgpu.so).
 * Every native call returns the library's status code; check() maps non-zero codes onto the
 * exceptions the reference job dies with.
 */
package edu.uci.ics.genomix.hyracks.graph.driver;

import java.io.DataOutputStream;
import java.io.IOException;
import java.io.InputStream;
import java.nio.ByteBuffer;

import org.apache.hadoop.fs.FileStatus;
import org.apache.hadoop.fs.FileSystem;
import org.apache.hadoop.fs.Path;
import org.apache.hadoop.io.SequenceFile;
import org.apache.hadoop.io.SequenceFile.CompressionType;
import org.apache.hadoop.mapred.FileInputFormat;
import org.apache.hadoop.mapred.FileOutputFormat;

import edu.uci.ics.genomix.config.GenomixJobConf;
import edu.uci.ics.genomix.data.types.Node;
import edu.uci.ics.genomix.data.types.VKmer;
import edu.uci.ics.genomix.hyracks.graph.driver.GenomixHyracksDriver.Plan;
import edu.uci.ics.hyracks.api.exceptions.HyracksException;

public class GenomixGpuDriver {
    static {
        System.loadLibrary("gxgpu_jni");
    }

    // status codes of include/gxgpu.h
    private static final int GX_OK = 0, GX_EINVAL_LINE = 2, GX_EINVAL_NUMBER = 3, GX_EREADID_RANGE = 4,
            GX_EREAD_TOO_SHORT = 5, GX_EFASTQ_PAIRING = 12;
    private static final int GX_INPUT_READID = 0;
    private static final int EMIT_BUFFER = 64 << 20;

    // ---- the C ABI, one native method per entry point used (gxgpu_jni.c) ----
    private static native long ctxCreate(int device);                       // gx_ctx_create; 0 on failure
    private static native void ctxDestroy(long ctx);                        // gx_ctx_destroy
    private static native long jobCreate(long ctx, int k, int inputKind, int paired, int outParts,
            int referenceLayout);                                            // gx_job_create; 0 on failure
    private static native int jobAddInput(long job, ByteBuffer direct, long bytes, int mate);  // gx_job_add_input
    private static native int jobRun(long job);                             // gx_job_run
    private static native long jobErrorLine(long job);                      // gx_job_stats().error_line
    private static native long jobEmit(long job, int part, ByteBuffer direct, long cap, int[] more);  // gx_job_emit
    private static native void jobDestroy(long job);                        // gx_job_destroy
    private static native String statusStr(int status);                     // gx_status_str
    private static native ByteBuffer pinnedAlloc(long bytes);               // gx_pinned_alloc, as a direct buffer
    private static native void pinnedFree(ByteBuffer direct);               // gx_pinned_free

    private final long ctx;

    public GenomixGpuDriver(int device) throws HyracksException {
        ctx = ctxCreate(device);
        if (ctx == 0)
            throw new HyracksException("no GB300 context on device " + device);
    }

    public void close() {
        ctxDestroy(ctx);
    }

    public void runJob(GenomixJobConf conf, Plan plan, boolean profile) throws Exception {
        if (plan != Plan.BUILD_DEBRUIJN_GRAPH)
            throw new IllegalArgumentException("the GPU driver runs the graph build (BUILD_DEBRUIJN_GRAPH) only");
        int k = Integer.parseInt(conf.get(GenomixJobConf.KMER_LENGTH));
        int parts = Math.max(1, conf.getInt(GenomixJobConf.THREADS_PER_MACHINE, 1));
        // part-q holds the records the reference's partitioner sends to part q
        long job = jobCreate(ctx, k, GX_INPUT_READID, 0, parts, 1);
        if (job == 0)
            throw new HyracksException("gx_job_create failed (k = " + k + ")");
        ByteBuffer emit = null;
        try {
            FileSystem fs = FileSystem.get(conf);
            for (Path in : FileInputFormat.getInputPaths(conf))
                for (FileStatus f : fs.listStatus(in)) {
                    if (f.isDir())
                        continue;
                    ByteBuffer b = readWhole(fs, f);
                    try {
                        check(jobAddInput(job, b, f.getLen(), 0), job);  // the bytes are copied to the GPU here
                    } finally {
                        pinnedFree(b);
                    }
                }
            long t0 = System.currentTimeMillis();
            check(jobRun(job), job);
            if (profile)
                System.out.println("GPU graph build: " + (System.currentTimeMillis() - t0) + " ms");
            Path out = FileOutputFormat.getOutputPath(conf);
            emit = pinnedAlloc(EMIT_BUFFER);
            byte[] heap = new byte[EMIT_BUFFER];
            int[] more = new int[1];
            for (int q = 0; q < parts; q++) {
                SequenceFile.Writer w = SequenceFile.createWriter(fs, conf, new Path(out, String.format("part-%05d", q)),
                        VKmer.class, Node.class, CompressionType.NONE);
                try {
                    do {
                        long n = jobEmit(job, q, emit, EMIT_BUFFER, more);
                        if (n < 0)
                            throw new HyracksException("gx_job_emit failed on part " + q);
                        emit.clear();
                        emit.get(heap, 0, (int) n);
                        appendRawRecords(w, heap, (int) n);
                    } while (more[0] != 0);
                } finally {
                    w.close();
                }
            }
        } finally {
            if (emit != null)
                pinnedFree(emit);
            jobDestroy(job);
        }
    }

    /** One input file into pinned host memory (the library copies it to the GPU from there). */
    private static ByteBuffer readWhole(FileSystem fs, FileStatus f) throws IOException {
        ByteBuffer b = pinnedAlloc(f.getLen());
        if (b == null)
            throw new IOException("gx_pinned_alloc of " + f.getLen() + " bytes failed");
        byte[] chunk = new byte[1 << 20];
        InputStream in = fs.open(f.getPath());
        try {
            int r;
            while ((r = in.read(chunk)) > 0)
                b.put(chunk, 0, r);
        } finally {
            in.close();
        }
        return b;
    }

    /**
     * The emitted bytes are SequenceFile record bodies (int32 record length, int32 key length, key,
     * value: what SequenceFile.Writer.append writes); each goes to the writer unchanged with
     * appendRaw, so the part files are byte for byte what KmerNodePairSequenceWriterFactory writes
     * (KmerNodePairSequenceWriterFactory.java:79-94), sync markers aside.
     */
    static void appendRawRecords(SequenceFile.Writer w, byte[] buf, int n) throws IOException {
        RawValue v = new RawValue();
        int p = 0;
        while (p + 8 <= n) {
            int recLen = readInt(buf, p), keyLen = readInt(buf, p + 4);
            if (keyLen < 0 || recLen < keyLen || p + 8 + recLen > n)
                throw new IOException("malformed record at byte " + p);
            v.data = buf;
            v.off = p + 8 + keyLen;
            v.len = recLen - keyLen;
            w.appendRaw(buf, p + 8, keyLen, v);
            p += 8 + recLen;
        }
        if (p != n)
            throw new IOException("record stream ends inside a record");
    }

    private static int readInt(byte[] b, int p) {
        return ((b[p] & 0xff) << 24) | ((b[p + 1] & 0xff) << 16) | ((b[p + 2] & 0xff) << 8) | (b[p + 3] & 0xff);
    }

    /** A Node's serialized bytes as SequenceFile's raw value (uncompressed files only). */
    private static final class RawValue implements SequenceFile.ValueBytes {
        byte[] data;
        int off, len;

        public void writeUncompressedBytes(DataOutputStream out) throws IOException {
            out.write(data, off, len);
        }

        public void writeCompressedBytes(DataOutputStream out) throws IOException {
            throw new IllegalArgumentException("the graph build writes uncompressed SequenceFiles");
        }

        public int getSize() {
            return len;
        }
    }

    /** Non-zero statuses as the exceptions that abort the reference job. */
    private static void check(int st, long job) throws HyracksException {
        if (st == GX_OK)
            return;
        long line = jobErrorLine(job);
        String msg = statusStr(st) + (line > 0 ? " at input line " + line : "");
        switch (st) {
            case GX_EINVAL_LINE:          // ReadsKeyValueParserFactory.java:118-122
                throw new IllegalStateException("input format is not correct! " + msg);
            case GX_EINVAL_NUMBER:        // Long.parseLong, ReadsKeyValueParserFactory.java:112,115
                throw new NumberFormatException(msg);
            case GX_EREADID_RANGE:        // ReadHeadInfo.java:110-113
            case GX_EREAD_TOO_SHORT:      // ReadsKeyValueParserFactory.java:152-155
                throw new IllegalArgumentException(msg);
            default:                      // GenomixHyracksDriver.java:132-134
                throw new HyracksException(msg);
        }
    }
}
