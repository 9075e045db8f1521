/*
 * gxgpu_jni.c — the JNI side of GenomixGpuDriver: each native method forwards to one entry
 * point of the C ABI (include/gxgpu.h).  Build (JDK headers required):
 *
 *   cc -O2 -shared -fPIC -I$JAVA_HOME/include -I$JAVA_HOME/include/linux -I<repo>/include \
 *      gxgpu_jni.c -L<repo>/genomix_gb300 -lgxgpu -o libgxgpu_jni.so
 *
 * Handles (gx_ctx *, gx_job *) travel to Java as jlong; 0 means "no object".
 */
#include <jni.h>
#include <stdint.h>

#include "gxgpu.h"

#define JNI_FN(name) Java_edu_uci_ics_genomix_hyracks_graph_driver_GenomixGpuDriver_##name

JNIEXPORT jlong JNICALL JNI_FN(ctxCreate)(JNIEnv *env, jclass cls, jint device) {
    gx_ctx *c = NULL;
    (void)env;
    (void)cls;
    return gx_ctx_create(device, NULL, &c) == GX_OK ? (jlong)(intptr_t)c : 0;
}

JNIEXPORT void JNICALL JNI_FN(ctxDestroy)(JNIEnv *env, jclass cls, jlong ctx) {
    (void)env;
    (void)cls;
    gx_ctx_destroy((gx_ctx *)(intptr_t)ctx);
}

JNIEXPORT jlong JNICALL JNI_FN(jobCreate)(JNIEnv *env, jclass cls, jlong ctx, jint k, jint kind, jint paired,
                                          jint parts, jint reference_layout) {
    gx_job_opts o = {0};
    gx_job *j = NULL;
    (void)env;
    (void)cls;
    o.struct_size = sizeof o;
    o.kmer_length = k;
    o.input_kind = kind;
    o.paired = paired;
    o.out_parts = parts;
    o.layout = reference_layout ? GX_LAYOUT_REFERENCE_PARTS : GX_LAYOUT_BUCKETS;
    return gx_job_create((gx_ctx *)(intptr_t)ctx, &o, &j) == GX_OK ? (jlong)(intptr_t)j : 0;
}

JNIEXPORT jint JNICALL JNI_FN(jobAddInput)(JNIEnv *env, jclass cls, jlong job, jobject buf, jlong bytes,
                                           jint mate) {
    void *p = (*env)->GetDirectBufferAddress(env, buf);
    (void)cls;
    if (!p && bytes) return GX_EINVAL;
    return gx_job_add_input((gx_job *)(intptr_t)job, p, (size_t)bytes, mate);
}

JNIEXPORT jint JNICALL JNI_FN(jobRun)(JNIEnv *env, jclass cls, jlong job) {
    (void)env;
    (void)cls;
    return gx_job_run((gx_job *)(intptr_t)job);
}

JNIEXPORT jlong JNICALL JNI_FN(jobErrorLine)(JNIEnv *env, jclass cls, jlong job) {
    gx_stats s;
    (void)env;
    (void)cls;
    if (gx_job_stats((gx_job *)(intptr_t)job, &s) != GX_OK) return 0;
    return (jlong)s.error_line;
}

/* bytes written, or -1 on failure; more[0] = 1 while the part has records left */
JNIEXPORT jlong JNICALL JNI_FN(jobEmit)(JNIEnv *env, jclass cls, jlong job, jint part, jobject buf, jlong cap,
                                        jintArray more) {
    size_t w = 0;
    int m = 0;
    jint jm;
    void *p = (*env)->GetDirectBufferAddress(env, buf);
    (void)cls;
    if (!p || gx_job_emit((gx_job *)(intptr_t)job, part, p, (size_t)cap, &w, &m) != GX_OK) return -1;
    jm = m;
    (*env)->SetIntArrayRegion(env, more, 0, 1, &jm);
    return (jlong)w;
}

JNIEXPORT void JNICALL JNI_FN(jobDestroy)(JNIEnv *env, jclass cls, jlong job) {
    (void)env;
    (void)cls;
    gx_job_destroy((gx_job *)(intptr_t)job);
}

JNIEXPORT jstring JNICALL JNI_FN(statusStr)(JNIEnv *env, jclass cls, jint st) {
    (void)cls;
    return (*env)->NewStringUTF(env, gx_status_str((gx_status)st));
}

/* page-locked host memory as a direct ByteBuffer (null when the allocation fails) */
JNIEXPORT jobject JNICALL JNI_FN(pinnedAlloc)(JNIEnv *env, jclass cls, jlong bytes) {
    void *p = NULL;
    (void)cls;
    if (bytes < 0 || gx_pinned_alloc((size_t)bytes, &p) != GX_OK) return NULL;
    return (*env)->NewDirectByteBuffer(env, p, bytes);
}

JNIEXPORT void JNICALL JNI_FN(pinnedFree)(JNIEnv *env, jclass cls, jobject buf) {
    (void)cls;
    if (buf) gx_pinned_free((*env)->GetDirectBufferAddress(env, buf));
}
