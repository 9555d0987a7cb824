// Operator apply on the 5th-generation tensor cores, split-BF16 form:
//     out = alpha * A @ B + beta * out        (FP32 in, FP32 out)
// with A = Ahi + Alo and B = Bhi + Blo split into BF16 halves and the
// product formed as Ahi*Bhi + Ahi*Blo + Alo*Bhi (three tcgen05.mma per K
// step, FP32 accumulation in tensor memory).  This is the chosen-precision
// replacement of the reference's `mul` providers
// (pyfr/backends/cuda/gimmik.py:23-121, pyfr/backends/cuda/cublaslt.py:169-280).
//
// One persistent CTA per SM walks 64- (or, for long operators, 32-)
// column tiles of B/out:
//   warp 4 lane 0   bulk-copies (TMA engine, cp.async.bulk) each FP32 B
//                   tile row by row into one of two staging buffers;
//   warps 5-8       split the staged tile into BF16 hi/lo in the
//                   canonical K-major no-swizzle UMMA layout (two stages);
//   warp 9 lane 0   issues the MMAs into one of two TMEM accumulators;
//   warps 0-3       read the accumulator (tcgen05.ld, one row per thread)
//                   and write alpha*D + beta*out.
// The operator halves are laid out on the host in the same canonical
// layout and bulk-copied into shared memory once per CTA.  All hand-offs
// are mbarriers; every wait is bounded and records an error code instead
// of hanging.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "../../include/pyfrb200.h"

namespace {

constexpr int MTILE = 128;        // UMMA M
constexpr int NTHREADS = 320;     // 10 warps
constexpr int NCONV = 128;        // converter threads (warps 5-8)
constexpr int NEPI = 128;         // epilogue threads (warps 0-3)
constexpr int MAX_MT = 4;         // up to 512 operator rows (TMEM: 2*4*64 cols)
constexpr long long WAIT_LIMIT = 1LL << 22;

constexpr int MAX_S32 = 4;        // FP32 staging stages (bytes in flight)

struct UmmaHandle {
    int m, k, mpad, kpad, mt, nt, s32;
    unsigned char *aimg;   // device: [hi | lo], each mpad x kpad bf16 canonical
    size_t aimg_bytes;
    size_t smem_bytes;
};

// Shared-memory plan; stage buffers are addressed arithmetically (a
// runtime-indexed array here would live in local memory)
struct Layout {
    uint32_t a_hi, a_lo;
    uint32_t b32, b32_stride;     // FP32 staging stage s at b32 + s*b32_stride
    uint32_t b16, b16_stride;     // BF16 stage s: hi at b16 + s*b16_stride, lo after hi
    uint32_t b16_half;            // bytes of one (hi or lo) BF16 tile
    uint32_t epi;                 // 4 warps x (32 rows x 128 B), 1024-aligned, swizzled
    uint32_t bar, tslot, abort_flag, total;
};

constexpr uint32_t EPI_WARP_BYTES = 32 * 128;

__host__ __device__ inline Layout make_layout(int mpad, int kpad, int k, int nt, int s32) {
    Layout L;
    uint32_t off = 0;
    const uint32_t abytes = (uint32_t)mpad * kpad * 2;
    const uint32_t b32bytes = ((uint32_t)k * nt * 4 + 127) & ~127u;
    const uint32_t b16bytes = (uint32_t)nt * kpad * 2;
    L.a_hi = off; off += abytes;
    L.a_lo = off; off += abytes;
    L.b32 = off; L.b32_stride = b32bytes; off += s32 * b32bytes;
    L.b16 = off; L.b16_stride = 2 * b16bytes; L.b16_half = b16bytes; off += 2 * 2 * b16bytes;
    off = (off + 1023) & ~1023u;
    L.epi = off; off += 4 * EPI_WARP_BYTES;
    L.bar = off; off += 24 * 8;
    L.tslot = off; off += 8;
    L.abort_flag = off; off += 8;
    L.total = off;
    return L;
}

// Barrier indices within the barrier block
enum { BAR_A = 0, BAR_FULL32 = 1, BAR_EMPTY32 = 1 + MAX_S32, BAR_FULL16 = 1 + 2 * MAX_S32,
       BAR_EMPTY16 = 3 + 2 * MAX_S32, BAR_ACCFULL = 5 + 2 * MAX_S32,
       BAR_ACCEMPTY = 7 + 2 * MAX_S32, BAR_DRAIN = 9 + 2 * MAX_S32 };

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count));
}

__device__ __forceinline__ void bar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void bar_arrive_tx(uint32_t bar, uint32_t tx) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;"
                 :: "r"(bar), "r"(tx) : "memory");
}

__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n.reg .pred P1;\nmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
                 "selp.b32 %0, 1, 0, P1;\n}\n"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

// Bounded wait: false (and the CTA's abort flag set, error recorded) if the
// phase does not complete within the limit or another role aborted.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                         int *err, int code) {
    for (long long it = 0; it < WAIT_LIMIT; it++) {
        if (bar_try(bar, parity)) return true;
        if (*abort_flag) return false;
        if (it > 32) __nanosleep(64);
    }
    *abort_flag = 1;
    atomicCAS(err, 0, code);
    return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;                 // descriptor version for tcgen05
    return d;                               // no swizzle, base offset 0
}

// kind::f16 instruction descriptor: BF16 A/B, FP32 D, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc,
                                     uint32_t acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(dtmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(bar) : "memory");
}

// One 2-D TMA load of a k-row x NT-column box of B into the dense FP32
// staging buffer (columns past ncol are zero-filled by the hardware)
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];"
                 :: "r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar) : "memory");
}

// Store (or add, for beta = 1) a 32x32 FP32 tile from 128-byte-swizzled
// shared memory into out through the tensor map of out
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int x, int y,
                                             int add) {
    if (add)
        asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group"
                     " [%0, {%1, %2}], [%3];"
                     :: "l"((uint64_t)map), "r"(x), "r"(y), "r"(src) : "memory");
    else
        asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group"
                     " [%0, {%1, %2}], [%3];"
                     :: "l"((uint64_t)map), "r"(x), "r"(y), "r"(src) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

struct UmmaArgs {
    CUtensorMap tmap;           // B as a (k x ncol) FP32 tensor, box NT x k
    CUtensorMap cmap;           // out as a (m x ncol) FP32 tensor, box 32 x 32, 128B swizzle
    const unsigned char *aimg;
    const float *b;
    float *c;
    int64_t ldb, ldc, ncol;
    int m, k, kpad, mt, s32;
    float alpha, beta;
    int epi;            // 0: alpha*D, 1: alpha*D + beta*C
    int *err;
};

template <int NT>
__global__ void __launch_bounds__(NTHREADS, 1) mul_umma_kernel(const __grid_constant__ UmmaArgs p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const Layout L = make_layout(p.mt * MTILE, p.kpad, p.k, NT, p.s32);
    const int S32 = p.s32;
    const uint32_t sbase = smem_addr(smem);
    const uint32_t bar0 = sbase + L.bar;
    auto bar = [&](int i) { return bar0 + 8u * i; };
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + L.abort_flag);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + L.tslot);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (p.ncol + NT - 1) / NT;
    const int mt = p.mt;
    const uint32_t tcols = 2 * mt * NT <= 32 ? 32 : (2 * mt * NT <= 64 ? 64 :
                          (2 * mt * NT <= 128 ? 128 : (2 * mt * NT <= 256 ? 256 : 512)));

    if (tid == 0) {
        *abort_flag = 0;
        bar_init(bar(BAR_A), 1);
        for (int s = 0; s < S32; s++) {
            bar_init(bar(BAR_FULL32 + s), 1);
            bar_init(bar(BAR_EMPTY32 + s), NCONV);
        }
        for (int s = 0; s < 2; s++) {
            bar_init(bar(BAR_FULL16 + s), NCONV);
            bar_init(bar(BAR_EMPTY16 + s), 1);
            bar_init(bar(BAR_ACCFULL + s), 1);
            bar_init(bar(BAR_ACCEMPTY + s), NEPI);
        }
        bar_init(bar(BAR_DRAIN), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tslot)), "r"(tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tslot;

    const uint32_t abytes = (uint32_t)(mt * MTILE) * p.kpad * 2;
    const uint32_t SBO = (uint32_t)p.kpad * 16, LBO = 128;

    if (warp == 4) {
        // ---- producer: operator image once, then the FP32 B tiles ----
        // (every lane issues a share of the row copies of a tile)
        if (lane == 0) bar_arrive_tx(bar(BAR_A), 2 * abytes);
        __syncwarp();
        {
            const uint32_t chunk = ((2 * abytes / 32) + 15) & ~15u;
            const uint32_t a0 = lane * chunk;
            if (a0 < 2 * abytes) {
                const uint32_t nb = 2 * abytes - a0 < chunk ? 2 * abytes - a0 : chunk;
                bulk_g2s(sbase + L.a_hi + a0, p.aimg + a0, nb, bar(BAR_A));
            }
        }
        int i = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int s = i % S32, ph = (i / S32) & 1;
            if (i >= S32 && !bar_wait(bar(BAR_EMPTY32 + s), ph ^ 1, abort_flag, p.err, 1))
                break;
            const uint32_t dst = sbase + L.b32 + (uint32_t)s * L.b32_stride;
            if (lane == 0) {
                bar_arrive_tx(bar(BAR_FULL32 + s), (uint32_t)p.k * NT * 4);
                tma_load_2d(dst, &p.tmap, (int)(t * NT), 0, bar(BAR_FULL32 + s));
            }
            __syncwarp();
        }
    } else if (warp >= 5 && warp <= 8) {
        // ---- converters: FP32 stage -> BF16 hi/lo canonical K-major ----
        const int ct = tid - 5 * 32;
        const int n = ct % NT;
        int i = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int s = i % S32, s2 = i & 1;
            if (!bar_wait(bar(BAR_FULL32 + s), (i / S32) & 1, abort_flag, p.err, 2)) break;
            if (i >= 2 && !bar_wait(bar(BAR_EMPTY16 + s2), ((i >> 1) + 1) & 1, abort_flag, p.err, 3))
                break;
            const float *b32 = reinterpret_cast<const float *>(smem + L.b32 + s * L.b32_stride);
            unsigned char *bhi = smem + L.b16 + s2 * L.b16_stride;
            unsigned char *blo = bhi + L.b16_half;
            for (int k8 = ct / NT; k8 < p.kpad / 8; k8 += NCONV / NT) {
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                    const int r0 = k8 * 8 + j;
                    const float x0 = r0 < p.k ? b32[r0 * NT + n] : 0.f;
                    const float x1 = r0 + 1 < p.k ? b32[(r0 + 1) * NT + n] : 0.f;
                    const __nv_bfloat16 h0 = __float2bfloat16_rn(x0);
                    const __nv_bfloat16 h1 = __float2bfloat16_rn(x1);
                    const __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
                    const __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
                    hw[j / 2] = (uint32_t)__bfloat16_as_ushort(h0) |
                                ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                    lw[j / 2] = (uint32_t)__bfloat16_as_ushort(l0) |
                                ((uint32_t)__bfloat16_as_ushort(l1) << 16);
                }
                const uint32_t off = (uint32_t)(n / 8) * SBO + (uint32_t)k8 * LBO + (n % 8) * 16;
                *reinterpret_cast<uint4 *>(bhi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(blo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bar_arrive(bar(BAR_EMPTY32 + s));
            bar_arrive(bar(BAR_FULL16 + s2));
        }
    } else if (warp == 9) {
        // ---- MMA issuer ----
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(MTILE, NT);
            bool ok = bar_wait(bar(BAR_A), 0, abort_flag, p.err, 4);
            int i = 0;
            for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x, i++) {
                const int s = i & 1, bsel = i & 1;
                if (!bar_wait(bar(BAR_FULL16 + s), (i >> 1) & 1, abort_flag, p.err, 5)) break;
                if (i >= 2 &&
                    !bar_wait(bar(BAR_ACCEMPTY + bsel), ((i >> 1) + 1) & 1, abort_flag, p.err, 6))
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                for (int q = 0; q < mt; q++) {
                    const uint32_t d = tmem + (uint32_t)(bsel * mt + q) * NT;
                    const uint32_t ahi = sbase + L.a_hi + (uint32_t)q * MTILE * p.kpad * 2;
                    const uint32_t alo = sbase + L.a_lo + (uint32_t)q * MTILE * p.kpad * 2;
                    for (int ks = 0; ks < p.kpad / 16; ks++) {
                        const uint32_t ko = (uint32_t)ks * 2 * LBO;
                        const uint64_t dah = sdesc(ahi + ko, LBO, SBO);
                        const uint64_t dal = sdesc(alo + ko, LBO, SBO);
                        const uint32_t bst = sbase + L.b16 + s * L.b16_stride;
                        const uint64_t dbh = sdesc(bst + ko, LBO, SBO);
                        const uint64_t dbl = sdesc(bst + L.b16_half + ko, LBO, SBO);
                        umma(d, dah, dbh, idesc, ks > 0);
                        umma(d, dah, dbl, idesc, 1);
                        umma(d, dal, dbh, idesc, 1);
                    }
                }
                umma_commit(bar(BAR_EMPTY16 + s));
                umma_commit(bar(BAR_ACCFULL + bsel));
            }
            // Drain: every MMA issued so far has completed once this arrives
            umma_commit(bar(BAR_DRAIN));
            bar_wait(bar(BAR_DRAIN), 0, abort_flag, p.err, 7);
        }
        __syncwarp();
    } else {
        // ---- epilogue: TMEM -> registers -> shared memory -> TMA store ----
        int i = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int bsel = i & 1;
            if (!bar_wait(bar(BAR_ACCFULL + bsel), (i >> 1) & 1, abort_flag, p.err, 8)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const int64_t col0 = t * NT;
            for (int q = 0; q < mt; q++) {
                // 32x32 sub-tiles: TMEM -> registers -> swizzled shared
                // memory -> one TMA store (or reduce-add) per warp; rows
                // beyond m and columns beyond ncol are clipped by the TMA
                for (int cc = 0; cc < NT; cc += 32) {
                    if (col0 + cc >= p.ncol) break;
                    uint32_t v[32];
                    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) +
                                           (uint32_t)(bsel * mt + q) * NT + cc;
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                          "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                          "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
                          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                          "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]),
                          "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                        : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");

                    // The previous store from this warp's buffer must have
                    // finished reading it
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    __syncwarp();
                    unsigned char *buf = smem + L.epi + warp * EPI_WARP_BYTES;
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const float4 o = make_float4(p.alpha * __uint_as_float(v[4 * j]),
                                                     p.alpha * __uint_as_float(v[4 * j + 1]),
                                                     p.alpha * __uint_as_float(v[4 * j + 2]),
                                                     p.alpha * __uint_as_float(v[4 * j + 3]));
                        *reinterpret_cast<float4 *>(buf + lane * 128 + ((j ^ (lane & 7)) * 16)) = o;
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0 && q * MTILE + warp * 32 < p.m)
                        tma_store_2d(&p.cmap, sbase + L.epi + warp * EPI_WARP_BYTES,
                                     (int)(col0 + cc), q * MTILE + warp * 32, p.epi);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            bar_arrive(bar(BAR_ACCEMPTY + bsel));
        }
        // Every store issued by this warp has completed before exit
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        __syncwarp();
    }

    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"(tcols));
}

// Host: split A into BF16 hi/lo and lay both out in the canonical K-major
// no-swizzle layout ((r/8)*SBO + (k/8)*128 + (r%8)*16 + (k%8)*2 bytes).
void build_image(const double *a, int m, int k, int mpad, int kpad, std::vector<uint16_t> &img) {
    const size_t n = (size_t)mpad * kpad;
    img.assign(2 * n, 0);
    const size_t SBO = (size_t)kpad * 16;
    for (int r = 0; r < m; r++)
        for (int c = 0; c < k; c++) {
            const float x = (float)a[(size_t)r * k + c];
            const __nv_bfloat16 h = __float2bfloat16_rn(x);
            const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
            const size_t off = (r / 8) * SBO + (c / 8) * 128 + (r % 8) * 16 + (c % 8) * 2;
            img[off / 2] = __bfloat16_as_ushort(h);
            img[n + off / 2] = __bfloat16_as_ushort(l);
        }
}

int g_sm_count = 0;
PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;

// Tensor map of B: rank 2, dims (ncol, k) innermost first, row stride
// ldb*4 bytes, box (nt, k), no swizzle, out-of-range elements read as 0
int encode_b_map(CUtensorMap *map, const float *b, int64_t ldb, int64_t ncol, int k, int nt) {
    cuuint64_t gdim[2] = {(cuuint64_t)ncol, (cuuint64_t)k};
    cuuint64_t gstride[1] = {(cuuint64_t)ldb * 4};
    cuuint32_t box[2] = {(cuuint32_t)nt, (cuuint32_t)k};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = g_encode_tiled(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)b, gdim, gstride,
                                box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return b200::set_error(B200_ERR_CUDA, "mul_bf16x3: cuTensorMapEncodeTiled failed (%d)",
                               (int)r);
    return B200_OK;
}

// Tensor map of out: dims (ncol, m), row stride ldc*4 bytes, box 32 x 32
// with the 128-byte swizzle the epilogue writes its staging tiles in
int encode_c_map(CUtensorMap *map, float *c, int64_t ldc, int64_t ncol, int m) {
    cuuint64_t gdim[2] = {(cuuint64_t)ncol, (cuuint64_t)m};
    cuuint64_t gstride[1] = {(cuuint64_t)ldc * 4};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = g_encode_tiled(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)c, gdim, gstride,
                                box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return b200::set_error(B200_ERR_CUDA, "mul_bf16x3: cuTensorMapEncodeTiled (out) failed (%d)",
                               (int)r);
    return B200_OK;
}

}  // namespace

extern "C" {

int b200_mul_bf16x3_create(const double *a, int m, int k, void **handle, size_t *smem_bytes) {
    if (!a || !handle || m <= 0 || k <= 0)
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3_create: bad arguments");
    const int mpad = (m + MTILE - 1) / MTILE * MTILE, kpad = (k + 15) / 16 * 16;
    const int mt = mpad / MTILE;
    // Widest column tile, then the deepest FP32 staging (bytes in flight
    // per SM), whose pipeline fits in shared memory
    int nt = 0, s32 = 0;
    Layout L = make_layout(mpad, kpad, k, 32, 2);
    for (int cand_nt : {64, 32}) {
        for (int cand_s = MAX_S32; cand_s >= 2 && !nt; cand_s--) {
            Layout c = make_layout(mpad, kpad, k, cand_nt, cand_s);
            if (c.total <= 227 * 1024) {
                nt = cand_nt;
                s32 = cand_s;
                L = c;
            }
        }
        if (nt) break;
    }
    if (smem_bytes) *smem_bytes = L.total;
    // (a TMA box spans at most 256 rows of B)
    if (mt > MAX_MT || !nt || L.total > 227 * 1024 || k > 256 || kpad / 16 * 3 * mt > 1024)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "mul_bf16x3: operator %dx%d needs %u bytes of shared memory", m,
                               k, L.total);

    // One-time device set-up here rather than at launch: changing a
    // function attribute while a stream capture is open invalidates it
    if (!g_sm_count) {
        int dev, sms = 0;
        int rc0 = b200::check_cuda(cudaGetDevice(&dev), "mul_bf16x3_create");
        if (!rc0)
            rc0 = b200::check_cuda(
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                "mul_bf16x3_create");
        if (!rc0)
            rc0 = b200::check_cuda(cudaFuncSetAttribute(mul_umma_kernel<64>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        227 * 1024),
                                   "mul_bf16x3: smem attribute");
        if (!rc0)
            rc0 = b200::check_cuda(cudaFuncSetAttribute(mul_umma_kernel<32>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        227 * 1024),
                                   "mul_bf16x3: smem attribute");
        if (!rc0) {
            void *fn = nullptr;
            cudaDriverEntryPointQueryResult q;
            rc0 = b200::check_cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn,
                                                                    12000, cudaEnableDefault, &q),
                                   "mul_bf16x3: driver entry point");
            if (!rc0 && (q != cudaDriverEntryPointSuccess || !fn))
                rc0 = b200::set_error(B200_ERR_CUDA, "mul_bf16x3: cuTensorMapEncodeTiled missing");
            g_encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        }
        if (rc0) return rc0;
        g_sm_count = sms;
    }

    std::vector<uint16_t> img;
    build_image(a, m, k, mpad, kpad, img);

    UmmaHandle *h = (UmmaHandle *)calloc(1, sizeof(UmmaHandle));
    if (!h) return b200::set_error(B200_ERR_STATE, "mul_bf16x3_create: out of host memory");
    h->m = m; h->k = k; h->mpad = mpad; h->kpad = kpad; h->mt = mt; h->nt = nt; h->s32 = s32;
    h->aimg_bytes = img.size() * 2;
    h->smem_bytes = L.total;
    int rc = b200::check_cuda(cudaMalloc(&h->aimg, h->aimg_bytes), "mul_bf16x3_create");
    if (!rc)
        rc = b200::check_cuda(cudaMemcpy(h->aimg, img.data(), h->aimg_bytes,
                                         cudaMemcpyHostToDevice), "mul_bf16x3_create");
    if (rc) {
        cudaFree(h->aimg);
        free(h);
        return rc;
    }
    *handle = h;
    return B200_OK;
}

int b200_mul_bf16x3_destroy(void *handle) {
    if (!handle) return B200_OK;
    UmmaHandle *h = (UmmaHandle *)handle;
    cudaFree(h->aimg);
    free(h);
    return B200_OK;
}

int b200_mul_bf16x3(void *handle, const float *b, int64_t ldb, float *c, int64_t ldc,
                    int64_t ncol, float alpha, float beta, int *err, void *stream) {
    UmmaHandle *h = (UmmaHandle *)handle;
    if (!h || !err) return b200::set_error(B200_ERR_ARG, "mul_bf16x3: null handle/status");
    if (ncol <= 0) return B200_OK;
    if (ldb < ncol || ldc < ncol)
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: leading dimension smaller than ncol");
    // Bulk copies need 16-byte aligned rows and 16-byte multiples
    if ((((uintptr_t)b) & 15) || (((uintptr_t)c) & 15) || (ldb % 4) || (ldc % 4) || (ncol % 4))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: operands must be 16-byte aligned");

    if (!g_sm_count)
        return b200::set_error(B200_ERR_STATE, "mul_bf16x3: no handle created on this device");

    // The epilogue stores (beta = 0) or adds (beta = 1) through the TMA
    if (beta != 0.0f && beta != 1.0f)
        return b200::set_error(B200_ERR_UNSUPPORTED, "mul_bf16x3: beta must be 0 or 1");
    UmmaArgs p;
    int rc = encode_b_map(&p.tmap, b, ldb, ncol, h->k, h->nt);
    if (!rc) rc = encode_c_map(&p.cmap, c, ldc, ncol, h->m);
    if (rc) return rc;
    p.aimg = h->aimg; p.b = b; p.c = c; p.ldb = ldb; p.ldc = ldc; p.ncol = ncol;
    p.m = h->m; p.k = h->k; p.kpad = h->kpad; p.mt = h->mt; p.s32 = h->s32;
    p.alpha = alpha; p.beta = beta; p.epi = beta != 0.0f; p.err = err;

    const int64_t ntiles = (ncol + h->nt - 1) / h->nt;
    const unsigned grid = (unsigned)(ntiles < g_sm_count ? ntiles : g_sm_count);
    if (h->nt == 64)
        mul_umma_kernel<64><<<grid, NTHREADS, h->smem_bytes, (cudaStream_t)stream>>>(p);
    else
        mul_umma_kernel<32><<<grid, NTHREADS, h->smem_bytes, (cudaStream_t)stream>>>(p);
    B200_CHECK_LAUNCH("mul_umma_kernel");
    return B200_OK;
}

}  // extern "C"
