// Context, memory, stream, event and graph entry points of the C ABI.
// These replace the ctypes wrappers of the CUDA driver that the reference
// backend binds (pyfr/backends/cuda/driver.py) for the operations the
// right-hand-side path needs.
#include <stdarg.h>
#include <string.h>

#include "common.cuh"
#include "../../include/pyfrb200.h"

namespace b200 {

static thread_local char g_errbuf[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_errbuf, sizeof(g_errbuf), fmt, ap);
    va_end(ap);
    return code;
}

int check_cuda(cudaError_t err, const char *what) {
    if (err == cudaSuccess) return B200_OK;
    return set_error(B200_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(err),
                     cudaGetErrorString(err));
}

}  // namespace b200

using b200::check_cuda;
using b200::set_error;

namespace {

// Eight independent FMA chains per thread: enough instruction-level
// parallelism to keep the FP64 pipe issuing every cycle.  x -> a x + b with
// 0 < a < 1 converges to b/(1 - a), so the values stay bounded.
constexpr int PROBE_CHAINS = 8;

__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(double *out, int iters, double a,
                                                             double b) {
    double x[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) x[k] = 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < PROBE_CHAINS; k++) x[k] = fma(x[k], a, b);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) s += x[k];
    // Never true for these inputs; keeps the chains live
    if (s < -1.0) out[0] = s;
}

}  // namespace

extern "C" {

const char *b200_version(void) { return "pyfrb200 0.1 sm_103a"; }

int b200_get_last_error(char *buf, size_t len) {
    if (!buf || !len) return B200_ERR_ARG;
    strncpy(buf, b200::g_errbuf, len - 1);
    buf[len - 1] = '\0';
    return B200_OK;
}

int b200_init(int device) {
    int n = 0;
    int rc = check_cuda(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (rc) return rc;
    if (device < 0 || device >= n)
        return set_error(B200_ERR_ARG, "device %d out of range (%d devices)", device, n);
    rc = check_cuda(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    return check_cuda(cudaFree(0), "context creation");
}

int b200_device_info(int *sm_count, int *cc_major, int *cc_minor, size_t *free_b,
                     size_t *total_b, char *name, size_t namelen) {
    int dev;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    cudaDeviceProp p;
    rc = check_cuda(cudaGetDeviceProperties(&p, dev), "cudaGetDeviceProperties");
    if (rc) return rc;
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    if (free_b || total_b) {
        size_t f, t;
        rc = check_cuda(cudaMemGetInfo(&f, &t), "cudaMemGetInfo");
        if (rc) return rc;
        if (free_b) *free_b = f;
        if (total_b) *total_b = t;
    }
    if (name && namelen) {
        strncpy(name, p.name, namelen - 1);
        name[namelen - 1] = '\0';
    }
    return B200_OK;
}

int b200_malloc(void **ptr, size_t nbytes) {
    if (!ptr) return set_error(B200_ERR_ARG, "null pointer");
    *ptr = nullptr;
    int rc = check_cuda(cudaMalloc(ptr, nbytes ? nbytes : 1), "cudaMalloc");
    if (rc) return rc;
    return check_cuda(cudaMemset(*ptr, 0, nbytes), "cudaMemset");
}

int b200_free(void *ptr) { return check_cuda(cudaFree(ptr), "cudaFree"); }

int b200_host_alloc(void **ptr, size_t nbytes) {
    if (!ptr) return set_error(B200_ERR_ARG, "null pointer");
    return check_cuda(cudaMallocHost(ptr, nbytes ? nbytes : 1), "cudaMallocHost");
}

int b200_host_free(void *ptr) { return check_cuda(cudaFreeHost(ptr), "cudaFreeHost"); }

int b200_memset(void *ptr, int value, size_t nbytes, void *stream) {
    return check_cuda(cudaMemsetAsync(ptr, value, nbytes, (cudaStream_t)stream),
                      "cudaMemsetAsync");
}

int b200_memcpy_htod(void *dst, const void *src, size_t nbytes, void *stream) {
    return check_cuda(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyHostToDevice,
                                      (cudaStream_t)stream), "memcpy HtoD");
}

int b200_memcpy_dtoh(void *dst, const void *src, size_t nbytes, void *stream) {
    return check_cuda(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDeviceToHost,
                                      (cudaStream_t)stream), "memcpy DtoH");
}

int b200_memcpy_dtod(void *dst, const void *src, size_t nbytes, void *stream) {
    return check_cuda(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDeviceToDevice,
                                      (cudaStream_t)stream), "memcpy DtoD");
}

int b200_stream_create(void **stream) {
    if (!stream) return set_error(B200_ERR_ARG, "null pointer");
    return check_cuda(cudaStreamCreateWithFlags((cudaStream_t *)stream, cudaStreamNonBlocking),
                      "cudaStreamCreate");
}

int b200_stream_destroy(void *stream) {
    return check_cuda(cudaStreamDestroy((cudaStream_t)stream), "cudaStreamDestroy");
}

int b200_stream_sync(void *stream) {
    return check_cuda(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
}

int b200_device_sync(void) { return check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); }

int b200_event_create(void **evt) {
    if (!evt) return set_error(B200_ERR_ARG, "null pointer");
    return check_cuda(cudaEventCreate((cudaEvent_t *)evt), "cudaEventCreate");
}

int b200_event_destroy(void *evt) {
    return check_cuda(cudaEventDestroy((cudaEvent_t)evt), "cudaEventDestroy");
}

int b200_event_record(void *evt, void *stream) {
    return check_cuda(cudaEventRecord((cudaEvent_t)evt, (cudaStream_t)stream), "cudaEventRecord");
}

int b200_event_sync(void *evt) {
    return check_cuda(cudaEventSynchronize((cudaEvent_t)evt), "cudaEventSynchronize");
}

int b200_event_elapsed(float *ms, void *start, void *stop) {
    if (!ms) return set_error(B200_ERR_ARG, "null pointer");
    return check_cuda(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop),
                      "cudaEventElapsedTime");
}

int b200_graph_begin_capture(void *stream) {
    return check_cuda(cudaStreamBeginCapture((cudaStream_t)stream,
                                             cudaStreamCaptureModeThreadLocal),
                      "cudaStreamBeginCapture");
}

int b200_graph_end_capture(void *stream, void **gexec) {
    if (!gexec) return set_error(B200_ERR_ARG, "null pointer");
    cudaGraph_t g;
    int rc = check_cuda(cudaStreamEndCapture((cudaStream_t)stream, &g), "cudaStreamEndCapture");
    if (rc) return rc;
    rc = check_cuda(cudaGraphInstantiate((cudaGraphExec_t *)gexec, g, 0), "cudaGraphInstantiate");
    cudaGraphDestroy(g);
    return rc;
}

int b200_graph_launch(void *gexec, void *stream) {
    return check_cuda(cudaGraphLaunch((cudaGraphExec_t)gexec, (cudaStream_t)stream),
                      "cudaGraphLaunch");
}

int b200_probe_fp64_fma(int iters, double *flops_per_s, void *stream) {
    if (!flops_per_s || iters <= 0) return set_error(B200_ERR_ARG, "probe: bad arguments");
    int dev, nsm;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    rc = check_cuda(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev),
                    "cudaDeviceGetAttribute");
    if (rc) return rc;
    const cudaStream_t st = (cudaStream_t)stream;
    const int blocks = 8 * nsm, threads = 256;
    cudaEvent_t e0, e1;
    if ((rc = check_cuda(cudaEventCreate(&e0), "cudaEventCreate"))) return rc;
    if ((rc = check_cuda(cudaEventCreate(&e1), "cudaEventCreate"))) {
        cudaEventDestroy(e0);
        return rc;
    }
    // One untimed launch, then the timed one
    fp64_fma_probe_kernel<<<blocks, threads, 0, st>>>(nullptr, iters, 0.999999, 1e-6);
    cudaEventRecord(e0, st);
    fp64_fma_probe_kernel<<<blocks, threads, 0, st>>>(nullptr, iters, 0.999999, 1e-6);
    cudaEventRecord(e1, st);
    rc = check_cuda(cudaGetLastError(), "fp64 probe launch");
    if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
    float ms = 0;
    if (!rc) rc = check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *flops_per_s = 2.0 * PROBE_CHAINS * (double)iters * blocks * threads / (ms * 1e-3);
    return B200_OK;
}

int b200_graph_destroy(void *gexec) {
    return check_cuda(cudaGraphExecDestroy((cudaGraphExec_t)gexec), "cudaGraphExecDestroy");
}

}  // extern "C"
