// Operator apply on the 5th-generation tensor cores, split-BF16 form:
//     out = alpha * A @ B + beta * out        (FP32 in, FP32 out, beta 0 or 1)
// with A = Ahi + Alo and B = Bhi + Blo split into BF16 halves and the
// product formed as Ahi*Bhi + Ahi*Blo + Alo*Bhi (three tcgen05.mma per K
// step, FP32 accumulation in tensor memory), or with Alo*Blo as a fourth
// product (the exact product of the split operands).  A handle may also hold
// the operator in three BF16 terms (24 significant bits, as FP32): the fifth
// product Ax3*Bhi then removes the operator's representation error, which
// is systematic (the same in every apply) and against data with a large
// mean it dominates that of the data's split.  This is the chosen-precision
// replacement of the reference's `mul` providers
// (pyfr/backends/cuda/gimmik.py:23-121, pyfr/backends/cuda/cublaslt.py:169-280).
//
// A TF32 variant (b200_mul_tf32_create*) runs the same pipeline with one
// tcgen05.mma.kind::tf32 product per K step: the converters round the
// staged FP32 chunk to TF32 in place and the operator image is TF32.
//
// The general form (b200_mul_bf16x3_apply) fuses what the reference runs
// as separate kernels:
//     out_z = alpha * S (.) (A1 @ B1_z + A2 @ B2_z) + beta * out_z
// with a second operator block A2 on a second input B2 (concatenated along
// K), z over nbatch equally strided slices of B and out, and S an optional
// per-(row, element) scale read in the epilogue.
//
// Orientation: the streamed data is the M side of the MMA.  One
// tcgen05.mma forms D[128 x N] += B^T[128 x 16] A^T[16 x N] for 128 columns
// of B/out at once, N being the operator's rows rounded up to 32 (at most
// 256).  Every operator row is then applied to a data tile with one read
// of that tile from shared memory, and the accumulator holds one column of
// out per TMEM lane with the operator rows along its columns.
//
// One persistent CTA per SM walks 128-column tiles of B/out, each in
// chunks of 32 rows of B (K), through one ring of 16 KB stages:
//   warp 16 lane 0  loads each 32 x 128 FP32 chunk with one 2-D tensor TMA
//                   into a free stage;
//   warps 8-15      split a staged chunk into BF16 hi/lo in place, in two
//                   groups of four warps that take alternate chunks: every
//                   thread reads its column of the chunk (32 values), the
//                   group meets at a named barrier, then writes the halves
//                   in the canonical K-major no-swizzle UMMA layout over the
//                   same 16 KB;
//   warp 17 lane 0  issues the MMAs into one of two TMEM accumulators; the
//                   completion of a chunk's MMAs frees its stage;
//   warps 0-7       read the accumulator (tcgen05.ld, one column of out per
//                   thread, 32 operator rows per load) in two sets of four,
//                   one warp per TMEM lane quadrant, the sets taking
//                   alternate 32-row groups; a set scales its group by
//                   alpha into one 128 x 32 staging tile (two per set) and
//                   writes it with a TMA tensor store (beta = 0) or
//                   reduce-add (beta = 1) of 512-byte rows.
// The operator halves are laid out on the host in the canonical layout
// and bulk-copied into shared memory once per CTA.  All hand-offs are
// mbarriers; every wait is bounded and records an error code instead of
// hanging.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "../../include/pyfrb200.h"

namespace {

constexpr int TCOLS = 128;        // columns of B/out per tile (UMMA M)
constexpr int KC = 32;            // rows of B per pipeline chunk
constexpr int NTHREADS = 576;     // 18 warps
constexpr int NEPI = 256;         // epilogue threads (warps 0-7)
constexpr int NCONV = 256;        // converter threads (warps 8-15)
constexpr int WARP_CONV = 8, WARP_PROD = 16, WARP_MMA = 17;
constexpr int CONV_BARRIER = 1;   // named barriers 1, 4: the two converter groups
constexpr int CONV_BARRIER2 = 4;
constexpr int EPI_BARRIER = 2;    // named barriers 2, 3: the epilogue sets
constexpr int MAX_N = 256;        // UMMA N limit (operator rows, padded)
constexpr int MAX_S = 10;         // ring stages (bytes in flight)
constexpr int MAX_EB = 2;         // staging tiles per epilogue set (1 when short of room)
constexpr long long WAIT_LIMIT = 1LL << 22;

constexpr uint32_t CHUNK32 = KC * TCOLS * 4;       // 16 KB FP32 chunk (one stage)
constexpr uint32_t CHUNK16 = KC * TCOLS * 2;       // 8 KB per BF16 half of a stage
constexpr uint32_t SBO_CHUNK = KC * 16;            // 8-row group stride of a chunk
constexpr uint32_t EPI_BUF = 32 * TCOLS * 4;       // one 32-row x 128-column staging tile

struct UmmaHandle {
    int m, k1, k2, nch1, npad, kfull, ns, eb;
    int tf32;              // operator image and MMAs in TF32 (one product)
    int nterms;            // BF16 terms of the operator split (2 or 3)
    unsigned char *aimg;   // device: [hi | lo (| third)], each npad x kfull
                           // bf16 canonical
    size_t aimg_bytes;
    size_t smem_bytes;
};

// Shared-memory plan; stage buffers are addressed arithmetically (a
// runtime-indexed array here would live in local memory)
struct Layout {
    uint32_t a_hi, a_lo, a_x3;    // operator terms (a_x3: third, if any)
    uint32_t ring;                // stage s at ring + s*CHUNK32: FP32 chunk, then
                                  // BF16 hi (first 8 KB) and lo (second 8 KB)
    uint32_t epi;                 // staging tile b of set h at epi + (h*eb + b)*EPI_BUF
    uint32_t bar, tslot, abort_flag, total;
};

__host__ __device__ inline Layout make_layout(int npad, int kfull, int ns, int eb,
                                              int nterms) {
    Layout L;
    uint32_t off = 0;
    const uint32_t abytes = (uint32_t)npad * kfull * 2;
    L.a_hi = off; off += abytes;
    L.a_lo = off; off += abytes;
    L.a_x3 = off; off += nterms == 3 ? abytes : 0;
    off = (off + 1023) & ~1023u;
    L.ring = off; off += ns * CHUNK32;
    L.epi = off; off += 2 * eb * EPI_BUF;
    L.bar = off; off += 40 * 8;
    L.tslot = off; off += 8;
    L.abort_flag = off; off += 8;
    L.total = off;
    return L;
}

// Barrier indices within the barrier block: per stage, loaded (TMA),
// converted (converter warps) and free (MMA completion)
enum { BAR_A = 0, BAR_LOADED = 1, BAR_CONVERTED = 1 + MAX_S, BAR_FREE = 1 + 2 * MAX_S,
       BAR_ACCFULL = 1 + 3 * MAX_S, BAR_ACCEMPTY = 3 + 3 * MAX_S, BAR_DRAIN = 5 + 3 * MAX_S };
static_assert(BAR_DRAIN < 40, "barrier block holds 40 slots");

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory accesses by 32-bit shared address, so that they are
// shared-window loads and stores whatever the compiler infers about a
// pointer's address space
__device__ __forceinline__ float lds_f32(uint32_t a) {
    float x;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(x) : "r"(a) : "memory");
    return x;
}

__device__ __forceinline__ void sts_f32(uint32_t a, float x) {
    asm volatile("st.shared.f32 [%0], %1;" :: "r"(a), "f"(x) : "memory");
}

__device__ __forceinline__ void sts_v4(uint32_t a, uint32_t x, uint32_t y, uint32_t z,
                                       uint32_t w) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};"
                 :: "r"(a), "r"(x), "r"(y), "r"(z), "r"(w) : "memory");
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
        if (it > 4096) __nanosleep(64);
    }
    *abort_flag = 1;
    atomicCAS(err, 0, code);
    return false;
}

// Bounded wait that ignores the abort flag: for copies in flight that must
// land before the CTA exits
__device__ __forceinline__ void bar_drain(uint32_t bar, uint32_t parity) {
    for (long long it = 0; it < WAIT_LIMIT && !bar_try(bar, parity); it++)
        if (it > 4096) __nanosleep(64);
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

// kind::tf32 instruction descriptor: TF32 A/B (format 2), FP32 D, K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t ad, uint64_t bd,
                                          uint32_t idesc, uint32_t acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(dtmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

// FP32 -> TF32 (round to nearest, ties away from zero), as FP32 bits
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
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

// One 3-D TMA load of a KC-row x TCOLS-column box of slice z of B into a
// dense FP32 staging buffer (rows past k and columns past ncol are
// zero-filled)
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            int z, uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];"
                 :: "r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(bar) : "memory");
}

// Store (or add, for beta = 1) a 32-row x 128-column FP32 tile from dense
// row-major shared memory into slice z of out through the tensor map of out
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, uint32_t src, int x, int y,
                                             int z, int add) {
    if (add)
        asm volatile("cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
                     " [%0, {%1, %2, %3}], [%4];"
                     :: "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(src) : "memory");
    else
        asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group"
                     " [%0, {%1, %2, %3}], [%4];"
                     :: "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(src) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

struct UmmaArgs {
    CUtensorMap tmap[2];        // B1, B2 as (nbatch x k_i x ncol) FP32 tensors, box TCOLS x KC x 1
    CUtensorMap cmap;           // out as a (nbatch x m x ncol) FP32 tensor, box TCOLS x 32 x 1
    const unsigned char *aimg;
    const float *rs;            // row scale S (null: none), S[row*ldr + element]
    int64_t ncol, ntc, ldr;     // ntc: column tiles per slice
    int64_t ldc;                // leading dimension of out (and of the RK registers)
    int m, npad, kfull, nch1, ns, eb, nbatch, nvars, products;
    int nterms;                 // operator terms in the image (2 or 3)
    // Stacked issue: the operator's terms lie one after the other along N
    // in the image, so one MMA applies all of them to a data half; the
    // products land in npart partial accumulators of npad columns (hh;
    // hl + lh; x3h + ll) that the epilogue sums.  accols: TMEM columns of
    // one accumulator (npad, or npart*npad stacked)
    int stack, npart, accols;
    float alpha;
    int epi;            // 0: store, 1: add to out
    int *err;
    // RK stage in the epilogue (rk 1: a stage, 2: the last stage; 0: off)
    double *rk_acc;
    float *rk_u;
    const double *rk_dtp;
    double rk_dt, rk_a, rk_b;
    int rk;
};

// 32 columns of one TMEM lane quadrant (32x32b shape, 32 repetitions):
// v[r] is column r of this thread's lane; completes at tcgen05.wait::ld
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t *v) {
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
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t *v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                   "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr));
}

template <bool TF32, bool RK>
__global__ void __launch_bounds__(NTHREADS, 1) mul_umma_kernel(const __grid_constant__ UmmaArgs p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const Layout L = make_layout(p.npad, p.kfull, p.ns, p.eb, p.nterms);
    const int eb = p.eb;
    const int NS = p.ns;
    // (the host plans a ring of at least four stages; see create)
    if (NS < 4 || NS > MAX_S) {
        if (threadIdx.x == 0) atomicCAS(p.err, 0, 9);
        return;
    }
    const uint32_t sbase = smem_addr(smem);
    const uint32_t bar0 = sbase + L.bar;
    auto bar = [&](int i) { return bar0 + 8u * i; };
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + L.abort_flag);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + L.tslot);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // tile T covers columns (T % ntc)*TCOLS.. of slice T / ntc
    const int64_t ntiles = p.ntc * p.nbatch;
    const int npad = p.npad, nch = p.kfull / KC;
    const int acc2 = 2 * p.accols;
    const uint32_t tcols = acc2 <= 32 ? 32 : (acc2 <= 64 ? 64 :
                          (acc2 <= 128 ? 128 : (acc2 <= 256 ? 256 : 512)));

    if (tid == 0) {
        *abort_flag = 0;
        bar_init(bar(BAR_A), 1);
        for (int s = 0; s < NS; s++) {
            bar_init(bar(BAR_LOADED + s), 1);
            bar_init(bar(BAR_CONVERTED + s), NCONV / 2);
            bar_init(bar(BAR_FREE + s), 1);
        }
        for (int s = 0; s < 2; s++) {
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

    const uint32_t abytes = (uint32_t)npad * p.kfull * 2;
    const uint32_t imgbytes = (uint32_t)p.nterms * abytes;
    // 8-row group strides of the operator image and of a converted chunk:
    // (K extent / elements per 16-byte core-matrix row) x 128 bytes
    const uint32_t SBO_OP = (uint32_t)p.kfull * (TF32 ? 32 : 16), LBO = 128;
    const uint32_t SBO_D = TF32 ? KC * 32 : SBO_CHUNK;

    if (warp == WARP_PROD) {
        // ---- producer: operator image once, then the FP32 chunks of B ----
        if (lane == 0) bar_arrive_tx(bar(BAR_A), imgbytes);
        __syncwarp();
        {
            const uint32_t chunk = ((imgbytes / 32) + 15) & ~15u;
            const uint32_t a0 = lane * chunk;
            if (a0 < imgbytes) {
                const uint32_t nb = imgbytes - a0 < chunk ? imgbytes - a0 : chunk;
                bulk_g2s(sbase + L.a_hi + a0, p.aimg + a0, nb, bar(BAR_A));
            }
        }
        if (lane == 0) {
            // (ring stage s and phase ph of chunk j, advanced per chunk: no
            // 64-bit divisions on the hand-off path)
            int64_t j = 0;
            int s = 0;
            uint32_t ph = 0;
            for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
                bool ok = true;
                const int tx = (int)((t % p.ntc) * TCOLS), tz = (int)(t / p.ntc);
                for (int c = 0; c < nch; c++, j++) {
                    if (j >= NS &&
                        !bar_wait(bar(BAR_FREE + s), ph ^ 1, abort_flag, p.err, 1)) {
                        ok = false;
                        break;
                    }
                    // chunks of the first block, then of the second
                    const int src = c < p.nch1 ? 0 : 1;
                    bar_arrive_tx(bar(BAR_LOADED + s), CHUNK32);
                    tma_load_3d(sbase + L.ring + (uint32_t)s * CHUNK32, &p.tmap[src], tx,
                                (src ? c - p.nch1 : c) * KC, tz, bar(BAR_LOADED + s));
                    if (++s == NS) {
                        s = 0;
                        ph ^= 1;
                    }
                }
                if (!ok) break;
            }
            // Every copy into shared memory has landed before the CTA may
            // exit (after an abort nobody else waits for them)
            bar_drain(bar(BAR_A), 0);
            for (int64_t q = j > NS ? j - NS : 0; q < j; q++)
                bar_drain(bar(BAR_LOADED + (int)(q % NS)), (uint32_t)((q / NS) & 1));
        }
        __syncwarp();
    } else if (warp >= WARP_CONV && warp < WARP_CONV + NCONV / 32) {
        // ---- converters: FP32 chunk -> BF16 hi/lo (or TF32) canonical
        // K-major, in place.  Two groups of four warps take the chunks of
        // alternate ring stages (even stages, odd stages), so that two
        // chunks are converted at once and every stage has one group,
        // which meets its phases in order whatever the ring's length;
        // thread ct of a group owns column cc of its chunks.
        const int ct = tid - WARP_CONV * 32, cc = ct % TCOLS, grp = ct / TCOLS;
        const uint32_t gbar = grp ? CONV_BARRIER2 : CONV_BARRIER;
        const uint32_t coff = (uint32_t)(cc / 8) * SBO_D + (uint32_t)(cc % 8) * 16;
        int64_t j = 0;
        int sn = 0;
        uint32_t phn = 0;
        bool ok = true;
        for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
            for (int c = 0; c < nch; c++, j++) {
                const int s = sn;
                const uint32_t ph = phn;
                if (++sn == NS) {
                    sn = 0;
                    phn ^= 1;
                }
                if ((s & 1) != grp) continue;
                // (a converter that gives up still meets the others of its
                // group at the named barrier below, so none of them waits
                // there forever)
                ok = bar_wait(bar(BAR_LOADED + s), ph, abort_flag, p.err, 2);
                const uint32_t stage = sbase + L.ring + (uint32_t)s * CHUNK32;
                float x[KC];
                if (ok) {
#pragma unroll
                    for (int r = 0; r < KC; r++)
                        x[r] = lds_f32(stage + (uint32_t)(r * TCOLS + cc) * 4);
                }
                asm volatile("bar.sync %0, %1;" :: "r"(gbar), "n"(NCONV / 2) : "memory");
                if (!ok || *abort_flag) {
                    ok = false;
                    break;
                }
                if (TF32) {
                    // eight 16-byte core-matrix rows of 4 TF32 values each
#pragma unroll
                    for (int q = 0; q < KC / 4; q++) {
                        const uint32_t off = coff + (uint32_t)q * LBO;
                        sts_v4(stage + off, to_tf32(x[4 * q]), to_tf32(x[4 * q + 1]),
                               to_tf32(x[4 * q + 2]), to_tf32(x[4 * q + 3]));
                    }
                }
#pragma unroll
                for (int q = 0; q < KC / 8 && !TF32; q++) {
                    uint32_t hw[4], lw[4];
#pragma unroll
                    for (int jj = 0; jj < 8; jj += 2) {
                        const float x0 = x[8 * q + jj], x1 = x[8 * q + jj + 1];
                        // (the low half of a bfloat162 is its first value)
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(x0, x1);
                        const float2 hf = __bfloat1622float2(h2);
                        const __nv_bfloat162 l2 = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
                        hw[jj / 2] = *reinterpret_cast<const uint32_t *>(&h2);
                        lw[jj / 2] = *reinterpret_cast<const uint32_t *>(&l2);
                    }
                    const uint32_t off = coff + (uint32_t)q * LBO;
                    sts_v4(stage + off, hw[0], hw[1], hw[2], hw[3]);
                    sts_v4(stage + CHUNK16 + off, lw[0], lw[1], lw[2], lw[3]);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                bar_arrive(bar(BAR_CONVERTED + s));
            }
        }
    } else if (warp == WARP_MMA) {
        // ---- MMA issuer ----
        if (lane == 0) {
            const uint32_t idesc = TF32 ? idesc_tf32(TCOLS, npad) : idesc_bf16(TCOLS, npad);
            // Stacked: the data's hi half against hi | lo (| x3) and its lo
            // half against hi | lo (five products: hh, hl, hx3 and lh, ll
            // into partials hh, hl + lh, hx3 + ll), or hi | lo and hi
            // (three products); four products add ll as a third MMA
            const int n1 = p.products == 5 ? 3 * npad : 2 * npad;
            const int n2 = p.products == 5 ? 2 * npad : npad;
            const uint32_t idesc1 = idesc_bf16(TCOLS, n1), idesc2 = idesc_bf16(TCOLS, n2);
            bool ok = bar_wait(bar(BAR_A), 0, abort_flag, p.err, 4);
            int64_t j = 0;
            int i = 0, sn = 0;
            uint32_t phn = 0;
            for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x, i++) {
                const int bsel = i & 1;
                if (i >= 2 &&
                    !bar_wait(bar(BAR_ACCEMPTY + bsel), ((i >> 1) & 1) ^ 1, abort_flag, p.err, 6))
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t d = tmem + (uint32_t)(bsel * p.accols);
                for (int c = 0; c < nch; c++, j++) {
                    const int s2 = sn;
                    const uint32_t ph = phn;
                    if (++sn == NS) {
                        sn = 0;
                        phn ^= 1;
                    }
                    if (!bar_wait(bar(BAR_CONVERTED + s2), ph, abort_flag, p.err, 5)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t bhi = sbase + L.ring + (uint32_t)s2 * CHUNK32;
                    if (TF32) {
                        // K steps of 8 (32 bytes: two core matrices)
#pragma unroll
                        for (int ks = 0; ks < KC / 8; ks++) {
                            const uint32_t ko = (uint32_t)ks * 2 * LBO;
                            const uint32_t kg = (uint32_t)(c * (KC / 8) + ks) * 2 * LBO;
                            umma_tf32(d, sdesc(bhi + ko, LBO, SBO_D),
                                      sdesc(sbase + L.a_hi + kg, LBO, SBO_OP), idesc, (c | ks) != 0);
                        }
                    }
#pragma unroll
                    for (int ks = 0; ks < KC / 16 && !TF32 && p.stack; ks++) {
                        const uint32_t ko = (uint32_t)ks * 2 * LBO;
                        const uint32_t kg = (uint32_t)(c * (KC / 16) + ks) * 2 * LBO;
                        const uint64_t dh = sdesc(bhi + ko, LBO, SBO_CHUNK);
                        const uint64_t dl = sdesc(bhi + CHUNK16 + ko, LBO, SBO_CHUNK);
                        const uint64_t oh = sdesc(sbase + L.a_hi + kg, LBO, SBO_OP);
                        umma(d, dh, oh, idesc1, (c | ks) != 0);
                        umma(d + (uint32_t)npad, dl, oh, idesc2, 1);
                        if (p.products == 4)
                            umma(d + (uint32_t)(2 * npad), dl,
                                 sdesc(sbase + L.a_lo + kg, LBO, SBO_OP), idesc, (c | ks) != 0);
                    }
#pragma unroll
                    for (int ks = 0; ks < KC / 16 && !TF32 && !p.stack; ks++) {
                        const uint32_t ko = (uint32_t)ks * 2 * LBO;
                        const uint32_t kg = (uint32_t)(c * (KC / 16) + ks) * 2 * LBO;
                        const uint64_t dh = sdesc(bhi + ko, LBO, SBO_CHUNK);
                        const uint64_t dl = sdesc(bhi + CHUNK16 + ko, LBO, SBO_CHUNK);
                        const uint64_t oh = sdesc(sbase + L.a_hi + kg, LBO, SBO_OP);
                        const uint64_t ol = sdesc(sbase + L.a_lo + kg, LBO, SBO_OP);
                        umma(d, dh, oh, idesc, (c | ks) != 0);
                        umma(d, dl, oh, idesc, 1);
                        umma(d, dh, ol, idesc, 1);
                        if (p.products >= 4) umma(d, dl, ol, idesc, 1);
                        if (p.products == 5)
                            umma(d, dh, sdesc(sbase + L.a_x3 + kg, LBO, SBO_OP), idesc, 1);
                    }
                    umma_commit(bar(BAR_FREE + s2));
                }
                if (!ok) break;
                umma_commit(bar(BAR_ACCFULL + bsel));
            }
            // Drain: every MMA issued so far has completed once this arrives
            // (waited for even after an abort: tensor memory is released
            // when the CTA ends)
            umma_commit(bar(BAR_DRAIN));
            bar_drain(bar(BAR_DRAIN), 0);
        }
        __syncwarp();
    } else {
        // ---- epilogue: TMEM -> registers -> shared memory -> TMA store ----
        // warp w reads TMEM lane quadrant w%4 (columns 32(w%4)..+31 of the
        // tile); set h = w/4 takes the row groups g with g%2 == h.  The
        // set's waits are collective (named barrier, then the abort flag)
        // so that no warp of a set is left at a barrier the others skip.
        const int quad = warp % 4, half = warp / 4;
        const bool issuer = quad == 0 && lane == 0;
        int i = 0, sb = 0;
        // RK stage products, as the stage kernel forms them: dt*a rounded
        // to FP32, dt*b in FP64
        double rk_dtb = 0;
        float rk_dta = 0;
        if (RK) {
            const double h = p.rk_dtp ? *p.rk_dtp : p.rk_dt;
            rk_dtb = h * p.rk_b;
            rk_dta = (float)(h * p.rk_a);
        }
        // Row-scale factors alpha*S[row, element] of row group g for this
        // thread's column (alpha alone without a scale)
        auto load_scale = [&](float *f, int g, int64_t col, int64_t ele) {
            if (p.rs && p.ldr == 0) {
                // One scale for every row (affine elements: 1/|J| is the
                // same at every solution point)
                const float fu = col < p.ncol ? p.alpha * __ldg(p.rs + ele) : 0.f;
#pragma unroll
                for (int r = 0; r < 32; r++) f[r] = g * 32 + r < p.m ? fu : 0.f;
            } else if (p.rs) {
#pragma unroll
                for (int r = 0; r < 32; r++)
                    f[r] = col < p.ncol && g * 32 + r < p.m
                               ? p.alpha * __ldg(p.rs + (int64_t)(g * 32 + r) * p.ldr + ele)
                               : 0.f;
            } else {
#pragma unroll
                for (int r = 0; r < 32; r++) f[r] = p.alpha;
            }
        };
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int bsel = i & 1;
            const int64_t x0 = (t % p.ntc) * TCOLS;
            const int z = (int)(t / p.ntc);
            // Element of this thread's column (AoSoA: blocks of 32 elements
            // with the variables of a block contiguous), for the row scale
            const int64_t col = x0 + quad * 32 + lane;
            const int64_t ele = (col / (32 * p.nvars)) * 32 + col % 32;
            // The first group's scale loads are in flight during the wait
            float f[32];
            load_scale(f, half, col, ele);
            // RK stage: the tile's FP64 solution rows are brought into L2
            // while its MMAs run, so that the epilogue's loads of them do
            // not wait on HBM (one bulk prefetch of up to 1 KB per row, by
            // the first warp of each set)
            if (RK && quad == 0) {
                const int64_t nc = p.ncol - x0 < TCOLS ? p.ncol - x0 : TCOLS;
                const uint32_t bytes = (uint32_t)(nc * 8) & ~15u;
                for (int g = half; g < npad / 32; g += 2) {
                    const int row = g * 32 + lane;
                    if (row < p.m && bytes)
                        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;"
                                     :: "l"(p.rk_acc + (int64_t)row * p.ldc + x0), "r"(bytes)
                                     : "memory");
                }
            }
            const bool ok = bar_wait(bar(BAR_ACCFULL + bsel), (i >> 1) & 1, abort_flag, p.err, 8);
            asm volatile("bar.sync %0, %1;" :: "r"(EPI_BARRIER + half), "n"(128) : "memory");
            if (!ok || *abort_flag) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            for (int g = half; g < npad / 32; g += 2) {
                if (g != half) load_scale(f, g, col, ele);
                uint32_t v[32];
                const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) +
                                       (uint32_t)(bsel * p.accols + g * 32);
                if (!TF32 && p.stack) {
                    // The partials, eight columns at a time: the small ones
                    // first (hl + lh, plus x3h + ll when there are three),
                    // then hh onto their sum
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        uint32_t u[8], w[8];
                        tmem_ld8(taddr + (uint32_t)(npad + 8 * q), u);
                        if (p.npart == 3) tmem_ld8(taddr + (uint32_t)(2 * npad + 8 * q), w);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int r = 0; r < 8; r++)
                            v[8 * q + r] = p.npart == 3 ? __float_as_uint(__uint_as_float(u[r]) +
                                                                          __uint_as_float(w[r]))
                                                        : u[r];
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        uint32_t u[8];
                        tmem_ld8(taddr + (uint32_t)(8 * q), u);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int r = 0; r < 8; r++)
                            v[8 * q + r] = __float_as_uint(__uint_as_float(u[r]) +
                                                           __uint_as_float(v[8 * q + r]));
                    }
                } else {
                    tmem_ld32(taddr, v);
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");

                if (RK) {
                    // R never goes to memory: the stage update of this
                    // thread's column in place, RKB rows at a time (one warp
                    // reads 32 consecutive FP64 values per row).  Each
                    // value is read and then written by this thread only,
                    // so the reads take the non-coherent path, and the next
                    // rows are in flight while the current ones are
                    // updated.
#pragma unroll
                    for (int r = 0; r < 32; r++) f[r] *= __uint_as_float(v[r]);
                    if (col < p.ncol) {
                        const double *acc = p.rk_acc + col;
                        constexpr int RKB = 4;
                        auto loadb = [&](double *t, int h2) {
#pragma unroll
                            for (int r = 0; r < RKB; r++) {
                                const int row = g * 32 + h2 * RKB + r;
                                t[r] = row < p.m ? __ldg(acc + (int64_t)row * p.ldc) : 0.0;
                            }
                        };
                        double t[RKB], tn[RKB];
                        loadb(t, 0);
#pragma unroll
                        for (int h2 = 0; h2 < 32 / RKB; h2++) {
                            if (h2 < 32 / RKB - 1) loadb(tn, h2 + 1);
#pragma unroll
                            for (int r = 0; r < RKB; r++) {
                                const int row = g * 32 + h2 * RKB + r;
                                if (row < p.m) {
                                    const float rf = f[h2 * RKB + r];
                                    const float t32 = b200::narrow_f64(t[r]);
                                    const double tw = fma(rk_dtb, b200::widen_f32(rf), t[r]);
                                    const int64_t ix = (int64_t)row * p.ldc + col;
                                    p.rk_acc[ix] = tw;
                                    p.rk_u[ix] = p.rk == 2 ? b200::narrow_f64(tw)
                                                           : fmaf(rk_dta, rf, t32);
                                }
                            }
#pragma unroll
                            for (int r = 0; r < RKB; r++) t[r] = tn[r];
                        }
                    }
                    continue;
                }

                // The store issued eb stores ago from this staging tile
                // must have finished reading it
                if (issuer) {
                    if (eb == 2)
                        asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                    else
                        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                }
                asm volatile("bar.sync %0, %1;" :: "r"(EPI_BARRIER + half), "n"(128) : "memory");
                const uint32_t boff = L.epi + (uint32_t)(half * eb + sb) * EPI_BUF;
                const uint32_t buf = sbase + boff + (uint32_t)(quad * 32 + lane) * 4;
#pragma unroll
                for (int r = 0; r < 32; r++)
                    sts_f32(buf + (uint32_t)(r * TCOLS) * 4, f[r] * __uint_as_float(v[r]));
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("bar.sync %0, %1;" :: "r"(EPI_BARRIER + half), "n"(128) : "memory");
                // (columns past ncol are clipped by the TMA)
                if (issuer) tma_store_3d(&p.cmap, sbase + boff, (int)x0, g * 32, z, p.epi);
                sb = sb + 1 == eb ? 0 : sb + 1;
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            bar_arrive(bar(BAR_ACCEMPTY + bsel));
        }
        // Every store issued by this set has completed before exit
        if (issuer) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        __syncwarp();
    }

    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"(tcols));
}

// Host: split [A1 | A2] into BF16 terms (hi, lo and, with three terms, the
// rounded remainder: 8, 16 or 24 leading significant bits of each entry) and
// lay each out in the canonical K-major no-swizzle layout ((r/8)*SBO +
// (k/8)*128 + (r%8)*16 + (k%8)*2 bytes, SBO = kfull*16), A2's columns
// starting at column k2off (a chunk boundary); rows past m and the padding
// columns are zero.  Remainders are formed in FP64 from the FP64 operator.
void build_block(const double *a, int m, int k, int koff, int kfull, size_t n, int nterms,
                 std::vector<uint16_t> &img) {
    const size_t SBO = (size_t)kfull * 16;
    for (int r = 0; r < m; r++)
        for (int c0 = 0; c0 < k; c0++) {
            const int c = koff + c0;
            const size_t off = (r / 8) * SBO + (c / 8) * 128 + (r % 8) * 16 + (c % 8) * 2;
            double rem = a[(size_t)r * k + c0];
            for (int t = 0; t < nterms; t++) {
                const __nv_bfloat16 h = __float2bfloat16_rn((float)rem);
                img[t * n + off / 2] = __bfloat16_as_ushort(h);
                rem -= (double)__bfloat162float(h);
            }
        }
}

// Host: round [A1 | A2] to TF32 (nearest, ties to even, on the binary32
// encoding: 10 stored mantissa bits) and lay it out in the canonical K-major
// no-swizzle layout for 4-byte elements ((r/8)*SBO + (k/4)*128 + (r%8)*16 +
// (k%4)*4 bytes, SBO = kfull*32).
void build_block_tf32(const double *a, int m, int k, int koff, int kfull,
                      std::vector<uint16_t> &img) {
    const size_t SBO = (size_t)kfull * 32;
    uint32_t *w = reinterpret_cast<uint32_t *>(img.data());
    for (int r = 0; r < m; r++)
        for (int c0 = 0; c0 < k; c0++) {
            const int c = koff + c0;
            const float x = (float)a[(size_t)r * k + c0];
            uint32_t u;
            memcpy(&u, &x, 4);
            if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0xfffu + ((u >> 13) & 1u)) & ~0x1fffu;
            w[((r / 8) * SBO + (c / 4) * 128 + (r % 8) * 16 + (c % 4) * 4) / 4] = u;
        }
}

int g_sm_count = 0;
PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;

// Tensor map of B: rank 3, dims (ncol, k, nbatch) innermost first, row
// stride ldb*4 bytes, slice stride bs*4 bytes, box (TCOLS, KC, 1), no
// swizzle, out-of-range elements read as 0
int encode_b_map(CUtensorMap *map, const float *b, int64_t ldb, int64_t ncol, int k, int nbatch,
                 int64_t bs) {
    cuuint64_t gdim[3] = {(cuuint64_t)ncol, (cuuint64_t)k, (cuuint64_t)nbatch};
    cuuint64_t gstride[2] = {(cuuint64_t)ldb * 4, (cuuint64_t)bs * 4};
    cuuint32_t box[3] = {(cuuint32_t)TCOLS, (cuuint32_t)KC, 1};
    cuuint32_t estride[3] = {1, 1, 1};
    CUresult r = g_encode_tiled(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)b, gdim, gstride,
                                box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return b200::set_error(B200_ERR_CUDA, "mul_bf16x3: cuTensorMapEncodeTiled failed (%d)",
                               (int)r);
    return B200_OK;
}

// Tensor map of out: dims (ncol, m, nbatch), row stride ldc*4 bytes, slice
// stride cs*4 bytes, box (TCOLS, 32, 1), dense row-major staging tiles
int encode_c_map(CUtensorMap *map, float *c, int64_t ldc, int64_t ncol, int m, int nbatch,
                 int64_t cs) {
    cuuint64_t gdim[3] = {(cuuint64_t)ncol, (cuuint64_t)m, (cuuint64_t)nbatch};
    cuuint64_t gstride[2] = {(cuuint64_t)ldc * 4, (cuuint64_t)cs * 4};
    cuuint32_t box[3] = {(cuuint32_t)TCOLS, 32, 1};
    cuuint32_t estride[3] = {1, 1, 1};
    CUresult r = g_encode_tiled(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)c, gdim, gstride,
                                box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return b200::set_error(B200_ERR_CUDA, "mul_bf16x3: cuTensorMapEncodeTiled (out) failed (%d)",
                               (int)r);
    return B200_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

int create_impl(const double *a1, int k1, const double *a2, int k2, int m, int tf32,
                int nterms, int want_ns, int want_eb, void **handle, size_t *smem_bytes) {
    if (!a1 || !handle || m <= 0 || k1 <= 0 || k2 < 0 || (k2 > 0 && !a2))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3_create: bad arguments");
    if (nterms != 2 && !(nterms == 3 && !tf32))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3_create: %d operator terms", nterms);
    const int nch1 = (k1 + KC - 1) / KC, nch2 = (k2 + KC - 1) / KC;
    const int npad = (m + 31) / 32 * 32, kfull = (nch1 + nch2) * KC;
    // The deepest ring (bytes in flight per SM) that fits in shared memory
    // with two staging tiles per epilogue set, or failing four stages that
    // way, with one (each converter group owns the even or the odd stages,
    // so the ring may have any length).  An operator of at most 64 rows
    // gives each set one store per tile, which a second staging tile would
    // not overlap with anything: it takes one and the ring the room.  A
    // caller (the autotuner) may ask for a given plan instead (want_ns
    // 4..MAX_S; want_eb 1 or 2).
    int ns = 0, eb = npad <= 64 ? 1 : MAX_EB;
    Layout L = make_layout(npad, kfull, 2, eb, nterms);
    if (want_ns || want_eb) {
        if (want_ns < 4 || want_ns > MAX_S || want_eb < 1 || want_eb > MAX_EB)
            return b200::set_error(B200_ERR_ARG, "mul_bf16x3: plan (%d stages, %d tiles) invalid",
                                   want_ns, want_eb);
        ns = want_ns;
        eb = want_eb;
        L = make_layout(npad, kfull, ns, eb, nterms);
    } else {
        for (; eb >= 1 && ns < 4; eb--) {
            ns = 0;
            for (int cand = MAX_S; cand >= 4 && !ns; cand--) {
                Layout c = make_layout(npad, kfull, cand, eb, nterms);
                if (c.total <= 227 * 1024) {
                    ns = cand;
                    L = c;
                }
            }
            if (ns >= 4) break;
        }
        if (eb < 1) eb = 1;
    }
    if (smem_bytes) *smem_bytes = L.total;
    if (npad > MAX_N || !ns || L.total > 227 * 1024)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "mul_bf16x3: operator %dx(%d+%d) needs %u bytes of shared memory "
                               "(or more than %d rows)", m, k1, k2, L.total, MAX_N);

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
            rc0 = b200::check_cuda(cudaFuncSetAttribute(mul_umma_kernel<false, false>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        227 * 1024),
                                   "mul_bf16x3: smem attribute");
        if (!rc0)
            rc0 = b200::check_cuda(cudaFuncSetAttribute(mul_umma_kernel<true, false>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        227 * 1024),
                                   "mul_tf32: smem attribute");
        if (!rc0)
            rc0 = b200::check_cuda(cudaFuncSetAttribute(mul_umma_kernel<false, true>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        227 * 1024),
                                   "mul_bf16x3 (RK stage): smem attribute");
        if (!rc0)
            rc0 = b200::check_cuda(cudaFuncSetAttribute(mul_umma_kernel<true, true>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        227 * 1024),
                                   "mul_tf32 (RK stage): smem attribute");
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

    const size_t n = (size_t)npad * kfull;
    std::vector<uint16_t> img((size_t)nterms * n, 0);
    if (tf32) {
        build_block_tf32(a1, m, k1, 0, kfull, img);
        if (k2) build_block_tf32(a2, m, k2, nch1 * KC, kfull, img);
    } else {
        build_block(a1, m, k1, 0, kfull, n, nterms, img);
        if (k2) build_block(a2, m, k2, nch1 * KC, kfull, n, nterms, img);
    }

    UmmaHandle *h = (UmmaHandle *)calloc(1, sizeof(UmmaHandle));
    if (!h) return b200::set_error(B200_ERR_STATE, "mul_bf16x3_create: out of host memory");
    h->m = m; h->k1 = k1; h->k2 = k2; h->nch1 = nch1; h->npad = npad; h->kfull = kfull;
    h->ns = ns; h->eb = eb; h->tf32 = tf32; h->nterms = nterms;
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

}  // namespace

extern "C" {

int b200_mul_bf16x3_create_cat(const double *a1, int k1, const double *a2, int k2, int m,
                                void **handle, size_t *smem_bytes) {
    return create_impl(a1, k1, a2, k2, m, 0, 2, 0, 0, handle, smem_bytes);
}

int b200_mul_bf16x3_create(const double *a, int m, int k, void **handle, size_t *smem_bytes) {
    return create_impl(a, k, nullptr, 0, m, 0, 2, 0, 0, handle, smem_bytes);
}

int b200_mul_tf32_create_cat(const double *a1, int k1, const double *a2, int k2, int m,
                             void **handle, size_t *smem_bytes) {
    return create_impl(a1, k1, a2, k2, m, 1, 2, 0, 0, handle, smem_bytes);
}

int b200_mul_tf32_create(const double *a, int m, int k, void **handle, size_t *smem_bytes) {
    return create_impl(a, k, nullptr, 0, m, 1, 2, 0, 0, handle, smem_bytes);
}

int b200_mul_tc_create_plan(const double *a1, int k1, const double *a2, int k2, int m, int tf32,
                            int nstages, int ntiles, void **handle, size_t *smem_bytes) {
    return create_impl(a1, k1, a2, k2, m, tf32 ? 1 : 0, 2, nstages, ntiles, handle, smem_bytes);
}

int b200_mul_tc_create_terms(const double *a1, int k1, const double *a2, int k2, int m,
                             int tf32, int nterms, int nstages, int ntiles, void **handle,
                             size_t *smem_bytes) {
    return create_impl(a1, k1, a2, k2, m, tf32 ? 1 : 0, nterms, nstages, ntiles, handle,
                       smem_bytes);
}

int b200_mul_tc_terms(void *handle, int *nterms) {
    UmmaHandle *h = (UmmaHandle *)handle;
    if (!h || !nterms) return b200::set_error(B200_ERR_ARG, "mul_tc_terms: null argument");
    *nterms = h->nterms;
    return B200_OK;
}

int b200_mul_tc_plan(void *handle, int *nstages, int *ntiles) {
    UmmaHandle *h = (UmmaHandle *)handle;
    if (!h) return b200::set_error(B200_ERR_ARG, "mul_tc_plan: null handle");
    if (nstages) *nstages = h->ns;
    if (ntiles) *ntiles = h->eb;
    return B200_OK;
}

int b200_mul_bf16x3_destroy(void *handle) {
    if (!handle) return B200_OK;
    UmmaHandle *h = (UmmaHandle *)handle;
    cudaFree(h->aimg);
    free(h);
    return B200_OK;
}

int b200_mul_bf16x3_apply(void *handle, const b200_mul_bf16x3_args_t *a, void *stream) {
    UmmaHandle *h = (UmmaHandle *)handle;
    if (!h || !a || !a->err) return b200::set_error(B200_ERR_ARG, "mul_bf16x3: null handle/args");
    if (a->ncol <= 0 || a->nbatch == 0) return B200_OK;
    if (a->nbatch < 0 || !a->b1 || !a->c || (h->k2 && !a->b2))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: bad arguments");
    if (a->ldb1 < a->ncol || a->ldc < a->ncol || (h->k2 && a->ldb2 < a->ncol))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: leading dimension smaller than ncol");
    // Tensor maps need 16-byte aligned bases and strides; tiles start at
    // multiples of 32 columns (128 bytes)
    const uintptr_t ptrs = (uintptr_t)a->b1 | (uintptr_t)a->b2 | (uintptr_t)a->c;
    if ((ptrs & 15) || (a->ldb1 % 4) || (a->ldc % 4) || (a->ncol % 4) ||
        (h->k2 && a->ldb2 % 4) ||
        (a->nbatch > 1 && ((a->bstride1 % 4) || (a->cstride % 4) || (h->k2 && a->bstride2 % 4))))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: operands must be 16-byte aligned");
    if (a->products != 0 && a->products != 3 && a->products != 4 && a->products != 5)
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: products must be 3, 4 or 5");
    if (a->products == 5 && (h->nterms != 3 || h->tf32))
        return b200::set_error(B200_ERR_ARG,
                               "mul_bf16x3: five products need a three-term operator");
    if (a->rowscale && (a->nvars <= 0 || a->ldr < 0 || a->nbatch != 1))
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: row scale needs nvars, ldr, one slice");

    if (!g_sm_count)
        return b200::set_error(B200_ERR_STATE, "mul_bf16x3: no handle created on this device");

    // The epilogue stores (beta = 0) or adds (beta = 1) through the TMA
    if (a->beta != 0.0f && a->beta != 1.0f)
        return b200::set_error(B200_ERR_UNSUPPORTED, "mul_bf16x3: beta must be 0 or 1");
    if (a->rk_stage < 0 || a->rk_stage > 2)
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: rk_stage must be 0, 1 or 2");
    if (a->rk_stage && (!a->rk_acc || !a->rk_u || a->nbatch != 1 || a->beta != 0.0f ||
                        (((uintptr_t)a->rk_acc) & 7) || (((uintptr_t)a->rk_u) & 3)))
        return b200::set_error(B200_ERR_ARG,
                               "mul_bf16x3: the RK stage needs acc and u, one slice, beta = 0");
    UmmaArgs p;
    const int one = a->nbatch == 1;
    int rc = encode_b_map(&p.tmap[0], a->b1, a->ldb1, a->ncol, h->k1, a->nbatch,
                          one ? a->ldb1 * h->k1 : a->bstride1);
    if (!rc && h->k2)
        rc = encode_b_map(&p.tmap[1], a->b2, a->ldb2, a->ncol, h->k2, a->nbatch,
                          one ? a->ldb2 * h->k2 : a->bstride2);
    else
        p.tmap[1] = p.tmap[0];
    if (!rc)
        rc = encode_c_map(&p.cmap, a->c, a->ldc, a->ncol, h->m, a->nbatch,
                          one ? a->ldc * h->m : a->cstride);
    if (rc) return rc;
    p.aimg = h->aimg; p.rs = a->rowscale; p.ldr = a->ldr; p.nvars = a->nvars;
    p.ncol = a->ncol; p.ntc = (a->ncol + TCOLS - 1) / TCOLS;
    p.m = h->m; p.npad = h->npad; p.kfull = h->kfull; p.nch1 = h->nch1; p.ns = h->ns;
    p.eb = h->eb;
    p.nbatch = a->nbatch;
    p.alpha = a->alpha; p.epi = a->beta != 0.0f; p.err = a->err;
    p.products = a->products == 0 ? 3 : a->products;
    p.nterms = h->nterms;
    // Stacked issue where the stacked operand (N <= 256) and two
    // accumulators of the partials fit tensor memory (512 columns)
    p.npart = p.products == 3 ? 2 : 3;
    p.stack = !h->tf32 && (p.products == 5 ? 3 : 2) * h->npad <= 256 &&
              2 * p.npart * h->npad <= 512;
    p.accols = p.stack ? p.npart * h->npad : h->npad;
    p.rk = a->rk_stage; p.rk_acc = a->rk_acc; p.rk_u = a->rk_u; p.rk_dtp = a->rk_dt_dev;
    p.rk_dt = a->rk_dt; p.rk_a = a->rk_a; p.rk_b = a->rk_b;
    p.ldc = a->ldc;

    const int64_t ntiles = p.ntc * p.nbatch;
    const unsigned grid = (unsigned)(ntiles < g_sm_count ? ntiles : g_sm_count);
    const cudaStream_t st = (cudaStream_t)stream;
    if (h->tf32 && p.rk)
        mul_umma_kernel<true, true><<<grid, NTHREADS, h->smem_bytes, st>>>(p);
    else if (h->tf32)
        mul_umma_kernel<true, false><<<grid, NTHREADS, h->smem_bytes, st>>>(p);
    else if (p.rk)
        mul_umma_kernel<false, true><<<grid, NTHREADS, h->smem_bytes, st>>>(p);
    else
        mul_umma_kernel<false, false><<<grid, NTHREADS, h->smem_bytes, st>>>(p);
    B200_CHECK_LAUNCH("mul_umma_kernel");
    return B200_OK;
}

int b200_mul_bf16x3(void *handle, const float *b, int64_t ldb, float *c, int64_t ldc,
                    int64_t ncol, float alpha, float beta, int *err, void *stream) {
    b200_mul_bf16x3_args_t a = {};
    a.b1 = b; a.ldb1 = ldb; a.c = c; a.ldc = ldc; a.ncol = ncol; a.nbatch = 1;
    a.alpha = alpha; a.beta = beta; a.err = err;
    if (!handle || !err) return b200::set_error(B200_ERR_ARG, "mul_bf16x3: null handle/status");
    if (((UmmaHandle *)handle)->k2)
        return b200::set_error(B200_ERR_ARG, "mul_bf16x3: two-block operator needs _apply");
    return b200_mul_bf16x3_apply(handle, &a, stream);
}

}  // extern "C"
