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
    // Mapped, so that kernels may also reach it (b200_memcpy_roundtrip)
    return check_cuda(cudaHostAlloc(ptr, nbytes ? nbytes : 1, cudaHostAllocMapped),
                      "cudaHostAlloc");
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

// Copy streams and events of the pipelined round trip, made on first use
namespace {
constexpr int RT_MAX_CHUNKS = 64;
struct RoundTrip {
    cudaStream_t down[2] = {nullptr, nullptr}, up[2] = {nullptr, nullptr};
    cudaEvent_t ready = nullptr, done[2] = {nullptr, nullptr};
    cudaEvent_t chunk[RT_MAX_CHUNKS] = {};
    bool made = false;
};
RoundTrip g_rt;

int roundtrip_make() {
    if (g_rt.made) return 0;
    for (int i = 0; i < 2; i++) {
        if (int rc = check_cuda(cudaStreamCreateWithFlags(&g_rt.down[i], cudaStreamNonBlocking),
                                "cudaStreamCreate")) return rc;
        if (int rc = check_cuda(cudaStreamCreateWithFlags(&g_rt.up[i], cudaStreamNonBlocking),
                                "cudaStreamCreate")) return rc;
        if (int rc = check_cuda(cudaEventCreateWithFlags(&g_rt.done[i], cudaEventDisableTiming),
                                "cudaEventCreate")) return rc;
    }
    if (int rc = check_cuda(cudaEventCreateWithFlags(&g_rt.ready, cudaEventDisableTiming),
                            "cudaEventCreate")) return rc;
    for (int k = 0; k < RT_MAX_CHUNKS; k++)
        if (int rc = check_cuda(cudaEventCreateWithFlags(&g_rt.chunk[k], cudaEventDisableTiming),
                                "cudaEventCreate")) return rc;
    g_rt.made = true;
    return 0;
}
}  // namespace

namespace {

// Copy by the SMs: 16-byte loads and stores over a grid-stride loop (the
// tail, under 16 bytes, byte by byte); src or dst may be page-locked host
// memory mapped into the device's address space
__global__ void sm_copy_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n16,
                               const unsigned char *__restrict__ src_tail,
                               unsigned char *__restrict__ dst_tail, int ntail) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride)
        dst[i] = src[i];
    if (blockIdx.x == 0 && (int)threadIdx.x < ntail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

int sm_copy(const void *src, void *dst, size_t len, cudaStream_t st) {
    if (((uintptr_t)src | (uintptr_t)dst) & 15)
        return set_error(B200_ERR_ARG, "memcpy_roundtrip: kernel copies need 16-byte alignment");
    const size_t n16 = len / 16;
    const int ntail = (int)(len - 16 * n16);
    int nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    size_t blocks = (n16 + 255) / 256;
    const size_t cap = (size_t)(nsm > 0 ? nsm : 1) * 4;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    sm_copy_kernel<<<(unsigned)blocks, 256, 0, st>>>(
        (const uint4 *)src, (uint4 *)dst, n16, (const unsigned char *)src + 16 * n16,
        (unsigned char *)dst + 16 * n16, ntail);
    return check_cuda(cudaGetLastError(), "sm_copy");
}

}  // namespace

int b200_memcpy_roundtrip(void *host, const void *dsrc, void *ddst, size_t nbytes,
                          int nchunks, int nstreams, void *stream) {
    if (!host || !dsrc) return set_error(B200_ERR_ARG, "null pointer");
    // nstreams < 0: the copies run as kernels on |nstreams| streams per
    // direction, reading and writing the host buffer through its device
    // mapping (which must exist: page-locked memory of this context)
    const bool by_sm = nstreams < 0;
    if (by_sm) nstreams = -nstreams;
    if (nchunks < 1 || nchunks > RT_MAX_CHUNKS || nstreams < 1 || nstreams > 2)
        return set_error(B200_ERR_ARG, "memcpy_roundtrip: 1-%d chunks on 1-2 streams",
                         RT_MAX_CHUNKS);
    if (int rc = roundtrip_make()) return rc;
    void *hdev = host;
    if (by_sm &&
        check_cuda(cudaHostGetDevicePointer(&hdev, host, 0), "cudaHostGetDevicePointer"))
        return set_error(B200_ERR_ARG, "memcpy_roundtrip: host buffer not mapped for the device");
    cudaStream_t st = (cudaStream_t)stream;
    // Both directions start after the work queued on `stream` (which
    // produced dsrc and may still read ddst)
    if (int rc = check_cuda(cudaEventRecord(g_rt.ready, st), "cudaEventRecord")) return rc;
    for (int i = 0; i < nstreams; i++) {
        if (int rc = check_cuda(cudaStreamWaitEvent(g_rt.down[i], g_rt.ready, 0), "wait")) return rc;
        if (int rc = check_cuda(cudaStreamWaitEvent(g_rt.up[i], g_rt.ready, 0), "wait")) return rc;
    }
    // Chunk k goes down on stream k % nstreams and, once it has landed,
    // back up on the matching up stream
    const size_t per = ((nbytes + nchunks - 1) / nchunks + 255) / 256 * 256;
    int k = 0;
    for (size_t off = 0; off < nbytes; off += per, k++) {
        const size_t len = nbytes - off < per ? nbytes - off : per;
        const int i = k % nstreams;
        char *h = (char *)host + off;
        char *hd = (char *)hdev + off;
        if (by_sm) {
            if (int rc = sm_copy((const char *)dsrc + off, hd, len, g_rt.down[i])) return rc;
        } else if (int rc = check_cuda(cudaMemcpyAsync(h, (const char *)dsrc + off, len,
                                                       cudaMemcpyDeviceToHost, g_rt.down[i]),
                                       "memcpy DtoH")) return rc;
        if (!ddst) continue;
        if (int rc = check_cuda(cudaEventRecord(g_rt.chunk[k], g_rt.down[i]), "cudaEventRecord"))
            return rc;
        if (int rc = check_cuda(cudaStreamWaitEvent(g_rt.up[i], g_rt.chunk[k], 0), "wait"))
            return rc;
        if (by_sm) {
            if (int rc = sm_copy(hd, (char *)ddst + off, len, g_rt.up[i])) return rc;
        } else if (int rc = check_cuda(cudaMemcpyAsync((char *)ddst + off, h, len,
                                                       cudaMemcpyHostToDevice, g_rt.up[i]),
                                       "memcpy HtoD")) return rc;
    }
    // `stream` continues once every chunk is back (or, without ddst, down)
    for (int i = 0; i < nstreams; i++) {
        cudaStream_t last = ddst ? g_rt.up[i] : g_rt.down[i];
        if (int rc = check_cuda(cudaEventRecord(g_rt.done[i], last), "cudaEventRecord")) return rc;
        if (int rc = check_cuda(cudaStreamWaitEvent(st, g_rt.done[i], 0), "wait")) return rc;
    }
    return 0;
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
