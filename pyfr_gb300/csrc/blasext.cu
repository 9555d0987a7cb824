// Register-level kernels of the time integrator:
//   rkvdh2    two-register low-storage RK stage update with optional
//             embedded error accumulation
//             (pyfr/integrators/explicit/kernels/rkvdh2.mako:4-31)
//   axnpby    x0 <- a0*x0 + sum_i a_i*x_i
//             (pyfr/backends/cuda/kernels/axnpby.mako:4-44)
//   errest    sum (or max) over all solution points of
//             (err / (atol_v + rtol*|curr|))^2, the error norm of the PI
//             controller (pyfr/integrators/controllers.py:105-117), reduced
//             deterministically in FP64 (fixed block partials, then one
//             ordered final pass).
// The register kernels treat the whole allocation (rows x leading
// dimension, padding included) as a flat array: the padding columns of
// every register stay exactly zero, so updating them is harmless.
#include <mutex>

#include "common.cuh"
#include "../../include/pyfrb200.h"

namespace {

constexpr int BX_BLOCK = 256;
constexpr int MAX_AXNPBY = 8;

// Stage coefficients a, b, e and the step size: dt itself, or read from
// device memory (dtp) so that a captured step graph serves every dt.  The
// products dt*a, dt*b, dt*e are formed once per block.
struct StageCoef {
    const double *dtp;
    double dt, a, b, e;
};

__device__ __forceinline__ void stage_products(const StageCoef &c, double &da, double &db,
                                               double &de) {
    __shared__ double sh[3];
    if (threadIdx.x == 0) {
        const double h = c.dtp ? *c.dtp : c.dt;
        sh[0] = h * c.a;
        sh[1] = h * c.b;
        sh[2] = h * c.e;
    }
    __syncthreads();
    da = sh[0];
    db = sh[1];
    de = sh[2];
}

template <typename T>
__global__ void __launch_bounds__(BX_BLOCK)
rkvdh2_kernel(int64_t n, int last, int errest, int first, StageCoef co,
              T *__restrict__ r1, T *__restrict__ r2, T *__restrict__ rold,
              T *__restrict__ rerr) {
    double da, db, de;
    stage_products(co, da, db, de);
    const T dta = (T)da, dtb = (T)db, dte = (T)de;
    for (int64_t i = (int64_t)blockIdx.x * BX_BLOCK + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * BX_BLOCK) {
        const T t1 = r1[i], t2 = r2[i];
        if (errest) {
            if (first) {
                rerr[i] = dte * t2;
                rold[i] = t1;
            } else {
                rerr[i] = rerr[i] + dte * t2;
            }
        }
        if (!last) {
            r1[i] = t1 + dta * t2;
            r2[i] = t1 + dtb * t2;
        } else {
            r1[i] = t1 + dtb * t2;
        }
    }
}

// Mixed-precision low-storage stage: the RHS is evaluated in FP32, the
// solution is accumulated in FP64.  In the two-register scheme the
// second register only carries the next stage's RHS input, so here it is
// written directly as the FP32 input of the next RHS evaluation:
//   acc <- acc + dt*b*R                      (FP64, one FMA per value)
//   u32 <- fl32(acc) + fl32(dt*a)*R          (FP32)
// and at the last stage u32 <- fl32(new acc), the input of the next step.
// The RHS input only needs FP32 accuracy: forming it in FP32 from the
// rounded accumulator costs at most 1.5 ulp where rounding the FP64 sum
// would cost 0.5, and leaves the narrow FP64 unit one FMA per value (the
// conversions run on the integer pipes).  A caller that keeps the solution
// relative to a constant reference state stores u - u_ref in acc; the
// stage is the same.
template <bool ERR>
__device__ __forceinline__ float rkmixed_value(int64_t i, double &t, float rf, int last,
                                               int first, float dta, double dtb, double dte,
                                               double *__restrict__ rold,
                                               double *__restrict__ rerr) {
    const double r = b200::widen_f32(rf);
    if (ERR) {
        if (first) {
            rerr[i] = dte * r;
            rold[i] = t;
        } else {
            rerr[i] = rerr[i] + dte * r;
        }
    }
    const float t32 = b200::narrow_f64(t);
    t = fma(dtb, r, t);
    return last ? b200::narrow_f64(t) : fmaf(dta, rf, t32);
}

// Four values per thread and iteration (two 16-byte FP64 loads and one
// 16-byte FP32 load in flight) over the first n4 quads, scalar after.
template <bool ERR>
__global__ void __launch_bounds__(BX_BLOCK)
rkmixed_kernel(int64_t n, int64_t n4, int last, int first, StageCoef co,
               double *__restrict__ acc, const float *__restrict__ rhs, float *__restrict__ u32,
               double *__restrict__ rold, double *__restrict__ rerr) {
    double da, dtb, dte;
    stage_products(co, da, dtb, dte);
    const float dta = (float)da;
    const int64_t stride = (int64_t)gridDim.x * BX_BLOCK;
    const int64_t tid = (int64_t)blockIdx.x * BX_BLOCK + threadIdx.x;
    double2 *acc2 = reinterpret_cast<double2 *>(acc);
    for (int64_t q = tid; q < n4; q += stride) {
        double2 a01 = acc2[2 * q], a23 = acc2[2 * q + 1];
        const float4 r = reinterpret_cast<const float4 *>(rhs)[q];
        float4 o;
        o.x = rkmixed_value<ERR>(4 * q + 0, a01.x, r.x, last, first, dta, dtb, dte, rold, rerr);
        o.y = rkmixed_value<ERR>(4 * q + 1, a01.y, r.y, last, first, dta, dtb, dte, rold, rerr);
        o.z = rkmixed_value<ERR>(4 * q + 2, a23.x, r.z, last, first, dta, dtb, dte, rold, rerr);
        o.w = rkmixed_value<ERR>(4 * q + 3, a23.y, r.w, last, first, dta, dtb, dte, rold, rerr);
        acc2[2 * q] = a01;
        acc2[2 * q + 1] = a23;
        reinterpret_cast<float4 *>(u32)[q] = o;
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
        double t = acc[i];
        u32[i] = rkmixed_value<ERR>(i, t, rhs[i], last, first, dta, dtb, dte, rold, rerr);
        acc[i] = t;
    }
}

// Constant per-variable offset subtracted (in FP64) before the FP32
// rounding: dst = fl32(src - u_ref).  Variable v of an AoSoA field sits
// at flat index i with v = (i mod (32*nvars)) / 32.
struct RefState {
    double v[8];
    double hcoef;       // u_last = v[last] + q_last + hcoef*q_0 (errest)
    int nvars;
};

__device__ __forceinline__ double ref_of(const RefState &r, int64_t i) {
    return r.nvars ? r.v[(int)((i % (32 * r.nvars)) / 32)] : 0.0;
}

__global__ void __launch_bounds__(BX_BLOCK)
cast_f64_f32_kernel(int64_t n, const double *__restrict__ src, float *__restrict__ dst,
                    RefState ref) {
    for (int64_t i = (int64_t)blockIdx.x * BX_BLOCK + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * BX_BLOCK)
        dst[i] = b200::narrow_f64(src[i] - ref_of(ref, i));
}

int make_ref(int nvars, const double *uref, RefState &r) {
    r = RefState{};
    if (!uref || nvars <= 0) return B200_OK;
    if (nvars > 8) return b200::set_error(B200_ERR_ARG, "reference state: nvars > 8");
    for (int v = 0; v < nvars; v++) r.v[v] = uref[v];
    r.nvars = nvars;
    return B200_OK;
}

template <typename T>
struct AxnpbyArgs {
    const T *x[MAX_AXNPBY];
    T a[MAX_AXNPBY];
};

template <typename T>
__global__ void __launch_bounds__(BX_BLOCK)
axnpby_kernel(int64_t n, int nv, T *__restrict__ x0, AxnpbyArgs<T> args) {
    const T a0 = args.a[0];
    for (int64_t i = (int64_t)blockIdx.x * BX_BLOCK + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * BX_BLOCK) {
        T acc = 0;
        for (int k = 1; k < nv; k++) acc += args.a[k] * args.x[k][i];
        if (a0 == T(0))
            x0[i] = acc;
        else if (a0 == T(1))
            x0[i] += acc;
        else
            x0[i] = a0 * x0[i] + acc;
    }
}

// The scaled form (pyfr/backends/cuda/kernels/axnpby.mako with in_scale,
// in_scale_idxs and out_scale; pyfr/backends/base/makoutil.py:43-58): with
// v the variable of the value (AoSoA: (i mod 32*nvars)/32), the terms of
// the registers whose bit is set in in_mask are multiplied by in_scale[v]
// and the sum by out_scale[v]; a0 = 0 stores, a0 = 1 adds the sum of the
// other terms, any other a0 includes x0 among the terms.
constexpr int MAX_SCALE_VARS = 16;

template <typename T>
struct AxnpbyScale {
    T in[MAX_SCALE_VARS], out[MAX_SCALE_VARS];
    unsigned in_mask;
    int has_out, nvars;
};

template <typename T>
__global__ void __launch_bounds__(BX_BLOCK)
axnpby_scaled_kernel(int64_t n, int nv, T *__restrict__ x0, AxnpbyArgs<T> args,
                     AxnpbyScale<T> sc) {
    const T a0 = args.a[0];
    const int first = (a0 == T(0) || a0 == T(1)) ? 1 : 0;
    for (int64_t i = (int64_t)blockIdx.x * BX_BLOCK + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * BX_BLOCK) {
        const int v = (int)((i % (32 * sc.nvars)) / 32);
        T acc = 0;
        for (int k = first; k < nv; k++) {
            const T xk = k ? args.x[k][i] : x0[i];
            acc += ((sc.in_mask >> k) & 1) ? args.a[k] * sc.in[v] * xk : args.a[k] * xk;
        }
        if (sc.has_out) acc = sc.out[v] * acc;
        if (a0 == T(1))
            x0[i] += acc;
        else
            x0[i] = acc;
    }
}

// Block partials of the error norm over the points of one element type;
// layout (nupts, nvars, neles) AoSoA with leading dimension ld.  One warp
// takes one (point, 32-element block) pair per iteration, lane = element
// within the block; lanes of padding elements past neles are skipped.
// The quotient err/(atol + rtol*|u|) uses the Newton-refined reciprocal
// b200::rcp_f64.
__device__ __forceinline__ double rcp_newton(double d) { return b200::rcp_f64(d); }

template <typename T>
__global__ void __launch_bounds__(BX_BLOCK)
errest_partial_kernel(int nupts, int nvars, int64_t neles, int64_t ld, const T *__restrict__ curr,
                      const T *__restrict__ err, const double *__restrict__ atol, double rtol,
                      int uniform, RefState ref, double *__restrict__ partial) {
    __shared__ double red[BX_BLOCK / 32];
    const int lane = threadIdx.x & 31;
    const int64_t nblk = (neles + 31) / 32, nwork = (int64_t)nupts * nblk;
    const int64_t warp = ((int64_t)blockIdx.x * BX_BLOCK + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * BX_BLOCK) >> 5;
    double acc = 0;
    for (int64_t q = warp; q < nwork; q += nwarps) {
        const int upt = (int)(q / nblk);
        const int64_t blk = q - upt * nblk;
        // Padding lanes of the last element block add nothing, whatever
        // they hold
        if (blk * 32 + lane >= neles) continue;
        const int64_t base = upt * ld + blk * 32 * nvars + lane;
        const double c0 = (double)curr[base], e0 = (double)err[base];
        for (int v = 0; v < nvars; v++) {
            const int64_t ix = base + v * 32;
            double c = (double)curr[ix], ev = (double)err[ix];
            if (ref.nvars) {
                // u_v = uref_v + q_v (+ hcoef*q_0 for the last variable);
                // the error estimate maps with the linear part alone
                c += ref.v[v];
                if (v == nvars - 1) {
                    c += ref.hcoef * c0;
                    ev += ref.hcoef * e0;
                }
            }
            const double qv = ev * rcp_newton(fma(rtol, fabs(c), atol[v]));
            acc = uniform ? fmax(acc, fabs(qv)) : fma(qv, qv, acc);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, acc, o);
        acc = uniform ? fmax(acc, y) : acc + y;
    }
    if (lane == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = red[0];
        for (int w = 1; w < BX_BLOCK / 32; w++) s = uniform ? fmax(s, red[w]) : s + red[w];
        partial[blockIdx.x] = s;
    }
}

// Order-preserving map of doubles onto unsigned integers (negative values
// reversed below the positive ones), so that an integer atomicMax is a max
// over the doubles
__device__ __forceinline__ unsigned long long max_key(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

template <typename T>
__global__ void __launch_bounds__(BX_BLOCK)
reduce_max_kernel(int64_t n, const T *__restrict__ x, unsigned long long *__restrict__ key) {
    double m = -INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * BX_BLOCK + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * BX_BLOCK)
        m = fmax(m, (double)x[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double wm[BX_BLOCK / 32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < BX_BLOCK / 32; w++) m = fmax(m, wm[w]);
        atomicMax(key, max_key(m));
    }
}

__global__ void reduce_max_final_kernel(const unsigned long long *__restrict__ key,
                                        double *__restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const unsigned long long k = *key;
        const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
        out[0] = __longlong_as_double((long long)b);
    }
}

template <typename T>
int reduce_max(int64_t n, const T *x, void *key, double *out, cudaStream_t st) {
    if (!key || !out || (n > 0 && !x))
        return b200::set_error(B200_ERR_ARG, "reduce_max: null argument");
    int rc = b200::check_cuda(cudaMemsetAsync(key, 0, 8, st), "reduce_max");
    if (rc) return rc;
    if (n > 0) {
        const int64_t nb = b200::ceil_div(n, BX_BLOCK);
        const unsigned grid = (unsigned)(nb < 4096 ? nb : 4096);
        reduce_max_kernel<T><<<grid, BX_BLOCK, 0, st>>>(n, x, (unsigned long long *)key);
        B200_CHECK_LAUNCH("reduce_max");
    }
    reduce_max_final_kernel<<<1, 32, 0, st>>>((const unsigned long long *)key, out);
    B200_CHECK_LAUNCH("reduce_max_final");
    return B200_OK;
}

__global__ void errest_final_kernel(int nblk, int uniform, const double *__restrict__ partial,
                                    double *__restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < nblk; i++) s = uniform ? fmax(s, partial[i]) : s + partial[i];
        out[0] = s;
    }
}

unsigned grid_for(int64_t n) {
    int64_t g = (n + BX_BLOCK - 1) / BX_BLOCK;
    const int64_t cap = 152 * 16;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

template <typename T>
int rkvdh2(int64_t n, int stage, int nstages, int errest, const double *dtp, double dt, double a,
           double b, double e, T *r1, T *r2, T *rold, T *rerr, cudaStream_t s) {
    if (n <= 0) return B200_OK;
    if (stage < 0 || stage >= nstages)
        return b200::set_error(B200_ERR_ARG, "rkvdh2: stage %d out of range", stage);
    if (errest && (!rold || !rerr))
        return b200::set_error(B200_ERR_ARG, "rkvdh2: error estimate needs rold and rerr");
    const StageCoef co{dtp, dt, stage == nstages - 1 ? 0.0 : a, b, e};
    rkvdh2_kernel<T><<<grid_for(n), BX_BLOCK, 0, s>>>(n, stage == nstages - 1, errest, stage == 0,
                                                      co, r1, r2, rold, rerr);
    B200_CHECK_LAUNCH("rkvdh2");
    return B200_OK;
}

template <typename T>
int axnpby(int64_t n, int nv, T *x0, const T *const *xs, const double *a, cudaStream_t s) {
    if (n <= 0) return B200_OK;
    if (nv < 1 || nv > MAX_AXNPBY)
        return b200::set_error(B200_ERR_ARG, "axnpby: nv=%d out of range", nv);
    AxnpbyArgs<T> args = {};
    for (int k = 0; k < nv; k++) {
        args.x[k] = k ? xs[k] : x0;
        args.a[k] = (T)a[k];
    }
    axnpby_kernel<T><<<grid_for(n), BX_BLOCK, 0, s>>>(n, nv, x0, args);
    B200_CHECK_LAUNCH("axnpby");
    return B200_OK;
}

template <typename T>
int axnpby_scaled(int64_t n, int nv, int nvars, T *x0, const T *const *xs, const double *a,
                  const double *in_scale, unsigned in_mask, const double *out_scale,
                  cudaStream_t s) {
    if (n <= 0) return B200_OK;
    if (nv < 1 || nv > MAX_AXNPBY)
        return b200::set_error(B200_ERR_ARG, "axnpby_scaled: nv=%d out of range", nv);
    if (nvars < 1 || nvars > MAX_SCALE_VARS)
        return b200::set_error(B200_ERR_ARG, "axnpby_scaled: nvars=%d out of range", nvars);
    if ((in_mask >> nv) || (in_mask && !in_scale))
        return b200::set_error(B200_ERR_ARG, "axnpby_scaled: bad input-scale mask");
    AxnpbyArgs<T> args = {};
    for (int k = 0; k < nv; k++) {
        args.x[k] = k ? xs[k] : x0;
        args.a[k] = (T)a[k];
    }
    AxnpbyScale<T> sc = {};
    sc.nvars = nvars;
    sc.in_mask = in_mask;
    sc.has_out = out_scale != nullptr;
    for (int v = 0; v < nvars; v++) {
        sc.in[v] = in_scale ? (T)in_scale[v] : T(1);
        sc.out[v] = out_scale ? (T)out_scale[v] : T(1);
    }
    axnpby_scaled_kernel<T><<<grid_for(n), BX_BLOCK, 0, s>>>(n, nv, x0, args, sc);
    B200_CHECK_LAUNCH("axnpby_scaled");
    return B200_OK;
}

template <typename T>
int errest(int nupts, int nvars, int64_t neles, int64_t ld, const T *curr, const T *err,
           const double *atol_dev, double rtol, int uniform, double *scratch, int nscratch,
           double *out, cudaStream_t s, const RefState &ref = RefState{}) {
    if (nscratch < 1) return b200::set_error(B200_ERR_ARG, "errest: no scratch");
    int64_t g = ((int64_t)nupts * neles + BX_BLOCK - 1) / BX_BLOCK;
    int nblk = (int)(g < 1 ? 1 : (g > nscratch ? nscratch : g));
    errest_partial_kernel<T><<<nblk, BX_BLOCK, 0, s>>>(nupts, nvars, neles, ld, curr, err,
                                                       atol_dev, rtol, uniform, ref, scratch);
    B200_CHECK_LAUNCH("errest_partial");
    errest_final_kernel<<<1, 32, 0, s>>>(nblk, uniform, scratch, out);
    B200_CHECK_LAUNCH("errest_final");
    return B200_OK;
}

// ---- Allocation-free error norm ---------------------------------------
// Some callers cannot hand this library a scratch buffer.  An integrator
// that keeps its whole step loop asynchronous cannot call cudaMalloc or
// cudaFree on the way (cudaFree synchronises the device and stalls the
// queued stages).  A host application that owns every byte of device
// memory through its own pool allocator cannot make a raw allocation at
// all.  For them the error norm keeps its block partials in this
// fixed-size file-scope array instead.  Every GPU that loads the library
// holds it (B200_ERREST_STATIC_MAX_BLOCKS doubles, 32 KiB) until the
// process exits.
#define B200_ERREST_STATIC_MAX_BLOCKS 4096
#define B200_ERREST_STATIC_MAX_DEVICES 64

static __device__ __align__(256) double g_errest_scratch[B200_ERREST_STATIC_MAX_BLOCKS];

// Device address of g_errest_scratch on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked
// up with cudaGetSymbolAddress once per device, with that device current,
// and cached.
static double *g_errest_scratch_dev[B200_ERREST_STATIC_MAX_DEVICES];
static std::mutex g_errest_scratch_mtx;

static int errest_static_scratch(double **ptr) {
    int dev = -1;
    int rc = b200::check_cuda(cudaGetDevice(&dev), "errest_static: cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= B200_ERREST_STATIC_MAX_DEVICES)
        return b200::set_error(B200_ERR_UNSUPPORTED, "errest_static: device %d out of range", dev);

    std::lock_guard<std::mutex> lock(g_errest_scratch_mtx);
    if (!g_errest_scratch_dev[dev]) {
        void *p = nullptr;
        rc = b200::check_cuda(cudaGetSymbolAddress(&p, g_errest_scratch),
                              "errest_static: cudaGetSymbolAddress");
        if (rc) return rc;
        g_errest_scratch_dev[dev] = static_cast<double *>(p);
    }
    *ptr = g_errest_scratch_dev[dev];
    return B200_OK;
}

}  // namespace

extern "C" {

// Same result as b200_errest_f64 with `nblocks` partial sums, but the
// partials live in the library's own static device array, so the call
// allocates nothing.  nblocks must lie in [1, 4096].  The first call on
// a device looks up the array's device address; make that first call
// before any stream capture.  All calls share the array and it keeps the
// last call's partials; each call overwrites every slot it reads, so
// nothing has to be cleared between calls.  Calls whose kernels overlap on
// the GPU (different streams, or different host threads) race on the
// shared array and give wrong results.
int b200_errest_static_f64(int nupts, int nvars, int64_t neles, int64_t ld, const double *curr,
                           const double *err, const double *atol_dev, double rtol, int uniform,
                           int nblocks, double *out, void *stream) {
    if (nblocks < 1 || nblocks > B200_ERREST_STATIC_MAX_BLOCKS)
        return b200::set_error(B200_ERR_ARG,
                               "errest_static: nblocks=%d outside [1, %d] (the static scratch "
                               "holds %d partial sums)",
                               nblocks, B200_ERREST_STATIC_MAX_BLOCKS,
                               B200_ERREST_STATIC_MAX_BLOCKS);
    double *scratch = nullptr;
    int rc = errest_static_scratch(&scratch);
    if (rc) return rc;
    return errest<double>(nupts, nvars, neles, ld, curr, err, atol_dev, rtol, uniform, scratch,
                          nblocks, out, (cudaStream_t)stream);
}

int b200_rkvdh2_f64(int64_t n, int stage, int nstages, int errest, double dt, double a,
                    double b, double e, double *r1, double *r2, double *rold, double *rerr,
                    void *stream) {
    return rkvdh2<double>(n, stage, nstages, errest, nullptr, dt, a, b, e, r1, r2, rold, rerr,
                          (cudaStream_t)stream);
}

int b200_rkvdh2_f32(int64_t n, int stage, int nstages, int errest, double dt, double a,
                    double b, double e, float *r1, float *r2, float *rold, float *rerr,
                    void *stream) {
    return rkvdh2<float>(n, stage, nstages, errest, nullptr, dt, a, b, e, r1, r2, rold, rerr,
                         (cudaStream_t)stream);
}

int b200_rkvdh2_dt_f64(int64_t n, int stage, int nstages, int errest, const double *dt_dev,
                       double a, double b, double e, double *r1, double *r2, double *rold,
                       double *rerr, void *stream) {
    if (!dt_dev) return b200::set_error(B200_ERR_ARG, "rkvdh2_dt: null step size");
    return rkvdh2<double>(n, stage, nstages, errest, dt_dev, 0.0, a, b, e, r1, r2, rold, rerr,
                          (cudaStream_t)stream);
}

int b200_rkvdh2_dt_f32(int64_t n, int stage, int nstages, int errest, const double *dt_dev,
                       double a, double b, double e, float *r1, float *r2, float *rold,
                       float *rerr, void *stream) {
    if (!dt_dev) return b200::set_error(B200_ERR_ARG, "rkvdh2_dt: null step size");
    return rkvdh2<float>(n, stage, nstages, errest, dt_dev, 0.0, a, b, e, r1, r2, rold, rerr,
                         (cudaStream_t)stream);
}

static int rkmixed(int64_t n, int stage, int nstages, int errest, const double *dtp, double dt,
                   double a, double b, double e, double *acc, const float *rhs, float *u32,
                   double *rold, double *rerr, cudaStream_t s) {
    if (n <= 0) return B200_OK;
    if (stage < 0 || stage >= nstages)
        return b200::set_error(B200_ERR_ARG, "rkmixed: stage %d out of range", stage);
    if (errest && (!rold || !rerr))
        return b200::set_error(B200_ERR_ARG, "rkmixed: error estimate needs rold and rerr");
    const int last = stage == nstages - 1;
    const bool aligned = !(((uintptr_t)acc | (uintptr_t)rhs | (uintptr_t)u32) & 15);
    const int64_t n4 = aligned ? n / 4 : 0;
    const StageCoef co{dtp, dt, last ? 0.0 : a, b, e};
    if (errest)
        rkmixed_kernel<true><<<grid_for(n / 4 + 1), BX_BLOCK, 0, s>>>(
            n, n4, last, stage == 0, co, acc, rhs, u32, rold, rerr);
    else
        rkmixed_kernel<false><<<grid_for(n / 4 + 1), BX_BLOCK, 0, s>>>(
            n, n4, last, stage == 0, co, acc, rhs, u32, rold, rerr);
    B200_CHECK_LAUNCH("rkmixed");
    return B200_OK;
}

int b200_rkmixed_f64f32(int64_t n, int stage, int nstages, int errest, double dt, double a,
                        double b, double e, double *acc, const float *rhs, float *u32,
                        double *rold, double *rerr, void *stream) {
    return rkmixed(n, stage, nstages, errest, nullptr, dt, a, b, e, acc, rhs, u32, rold, rerr,
                   (cudaStream_t)stream);
}

int b200_rkmixed_dt_f64f32(int64_t n, int stage, int nstages, int errest, const double *dt_dev,
                           double a, double b, double e, double *acc, const float *rhs,
                           float *u32, double *rold, double *rerr, void *stream) {
    if (!dt_dev) return b200::set_error(B200_ERR_ARG, "rkmixed_dt: null step size");
    return rkmixed(n, stage, nstages, errest, dt_dev, 0.0, a, b, e, acc, rhs, u32, rold, rerr,
                   (cudaStream_t)stream);
}

int b200_cast_f64_f32(int64_t n, const double *src, float *dst, int nvars, const double *uref,
                      void *stream) {
    if (n <= 0) return B200_OK;
    RefState ref;
    int rc = make_ref(nvars, uref, ref);
    if (rc) return rc;
    cast_f64_f32_kernel<<<grid_for(n), BX_BLOCK, 0, (cudaStream_t)stream>>>(n, src, dst, ref);
    B200_CHECK_LAUNCH("cast_f64_f32");
    return B200_OK;
}

int b200_axnpby_f64(int64_t n, int nv, double *x0, const double *const *xs, const double *a,
                    void *stream) {
    return axnpby<double>(n, nv, x0, xs, a, (cudaStream_t)stream);
}

int b200_axnpby_f32(int64_t n, int nv, float *x0, const float *const *xs, const double *a,
                    void *stream) {
    return axnpby<float>(n, nv, x0, xs, a, (cudaStream_t)stream);
}

int b200_axnpby_scaled_f64(int64_t n, int nv, int nvars, double *x0, const double *const *xs,
                           const double *a, const double *in_scale, unsigned in_mask,
                           const double *out_scale, void *stream) {
    return axnpby_scaled<double>(n, nv, nvars, x0, xs, a, in_scale, in_mask, out_scale,
                                 (cudaStream_t)stream);
}

int b200_axnpby_scaled_f32(int64_t n, int nv, int nvars, float *x0, const float *const *xs,
                           const double *a, const double *in_scale, unsigned in_mask,
                           const double *out_scale, void *stream) {
    return axnpby_scaled<float>(n, nv, nvars, x0, xs, a, in_scale, in_mask, out_scale,
                                (cudaStream_t)stream);
}

int b200_errest_f64(int nupts, int nvars, int64_t neles, int64_t ld, const double *curr,
                    const double *err, const double *atol_dev, double rtol, int uniform,
                    double *scratch, int nscratch, double *out, void *stream) {
    return errest<double>(nupts, nvars, neles, ld, curr, err, atol_dev, rtol, uniform, scratch,
                          nscratch, out, (cudaStream_t)stream);
}

int b200_errest_shifted_f64(int nupts, int nvars, int64_t neles, int64_t ld, const double *curr,
                            const double *err, const double *atol_dev, double rtol, int uniform,
                            const double *uref, double hcoef, double *scratch, int nscratch,
                            double *out, void *stream) {
    RefState ref;
    int rc = make_ref(nvars, uref, ref);
    if (rc) return rc;
    ref.hcoef = hcoef;
    return errest<double>(nupts, nvars, neles, ld, curr, err, atol_dev, rtol, uniform, scratch,
                          nscratch, out, (cudaStream_t)stream, ref);
}

int b200_errest_f32(int nupts, int nvars, int64_t neles, int64_t ld, const float *curr,
                    const float *err, const double *atol_dev, double rtol, int uniform,
                    double *scratch, int nscratch, double *out, void *stream) {
    return errest<float>(nupts, nvars, neles, ld, curr, err, atol_dev, rtol, uniform, scratch,
                         nscratch, out, (cudaStream_t)stream);
}

int b200_reduce_max_f64(int64_t n, const double *x, void *key, double *out, void *stream) {
    return reduce_max<double>(n, x, key, out, (cudaStream_t)stream);
}

int b200_reduce_max_f32(int64_t n, const float *x, void *key, double *out, void *stream) {
    return reduce_max<float>(n, x, key, out, (cudaStream_t)stream);
}

}  // extern "C"
