/*
 * pyfrb200 -- C ABI of the GB300-native flux-reconstruction right-hand
 * side and Runge-Kutta stage update (the `b200` backend).
 *
 * Every entry point returns an int status: 0 on success, nonzero on error,
 * with a message available from b200_get_last_error().  Pointers are raw
 * device pointers unless stated otherwise; `stream` is a cudaStream_t
 * passed as void*.  Fields use the reference CUDA backend's AoSoA layout
 * with a SoA block of 32: a field of io-shape (nrow, nvars, neles) with
 * leading dimension `ld` stores variable v of element e on row r at
 *     r*ld + (e/32)*32*nvars + v*32 + e%32.
 * Interface views are (base pointer, gather map) pairs: the map holds
 * element offsets from the base (int32 or int64, selected by `ix64`), the
 * variables of a point are 32 elements apart, and vector views add a
 * per-point row stride for the spatial index.
 *
 * Each declaration cites the reference interface it replaces (paths within
 * the PyFR source tree).
 */
#ifndef PYFRB200_H
#define PYFRB200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gas and viscosity constants of the flux kernels ([constants] gamma, mu,
 * Pr, cpTref, cpTs; viscosity-correction = sutherland when sutherland != 0);
 * pyfr/solvers/navstokes/kernels/flux.mako:48-105.
 * shifted != 0 (Navier-Stokes kernels and the *_shift Euler kernels,
 * Rusanov only): the solution inputs are q = T(u - u_ref), the
 * perturbation from the constant state (rho_ref, rho_ref*v_ref,
 * E_ref = p_ref/(gamma - 1) + rho_ref |v_ref|^2/2) with its energy
 * component replaced by dE - h_t*drho (h_t = (E_ref + p_ref)/rho_ref); the
 * kernels compute the right-hand side of q, i.e. T times that of u (energy
 * row minus h_t times the mass row), with the reference state's constant
 * flux left out and the rest formed from the perturbation.  Exact in exact
 * arithmetic; the low-precision rounding no longer scales with the mean
 * pressure, enthalpy or flow.
 * p_min: the floor that the exact Riemann solver's Newton iterations put on
 * the star pressure (pyfr/solvers/euler/inters.py:12-25). */
typedef struct {
    double gamma, mu, pr, cpTref, cpTs;
    int sutherland;
    int shifted;
    double rho_ref, p_ref;
    double p_min;   /* floor of the exact Riemann solver's star pressure */
    double v_ref[3];    /* reference velocity (zeros: the fluid at rest) */
} b200_gas_t;

/* Boundary conditions: the types of pyfr/solvers/euler/inters.py:83-112
 * and pyfr/solvers/navstokes/inters.py:101-150 with uniform constants
 * (free-stream or inflow state rho, p, u; wall velocity u and cpTw for the
 * isothermal wall). */
enum {
    B200_BC_SUP_IN_FA = 1,        /* supersonic inflow: the given state */
    B200_BC_SUP_OUT_FN = 2,       /* supersonic outflow: the interior state */
    B200_BC_SLP_ADIA_WALL = 3,    /* slip adiabatic wall */
    B200_BC_CHAR_RIEM_INV = 4,    /* characteristic Riemann invariants */
    B200_BC_NO_SLP_ADIA_WALL = 5, /* no-slip adiabatic wall (NS) */
    B200_BC_NO_SLP_ISOT_WALL = 6, /* no-slip isothermal wall (NS) */
    B200_BC_SUB_IN_FRV = 7,       /* subsonic inflow, given rho and velocity (NS) */
    B200_BC_SUB_IN_FTPTTANG = 8,  /* subsonic inflow, given total state and direction (NS) */
    B200_BC_SUB_OUT_FP = 9,       /* subsonic outflow, given pressure (NS) */
    B200_BC_CHAR_RIEM_INV_CTRL = 10 /* characteristic Riemann invariants with a controlled
                                     * pressure p = ic + im*t (char-riem-inv-mass-flow and
                                     * char-riem-inv-pressure; Euler and NS) */
};
/* One instruction of a boundary-value or source-term program: postfix
 * code evaluated per point on a stack of at most 16 values.  Opcodes:
 * 0 push val, 1-3 push x, y, z of the point, 4 push t, 5-9 + - * / pow,
 * 10 negate, 11-23 sin cos tan exp log sqrt tanh fabs asin acos atan sinh
 * cosh, 24-26 atan2 fmin fmax, 27-28 floor ceil, 29 push solution
 * variable pad (source terms only). */
typedef struct {
    int op, pad;
    double val;
} b200_bcop_t;
typedef struct {
    int type;
    double rho, p, u[3];
    double cpTw;
    /* sub-in-ftpttang: total cp*T, total pressure, flow direction */
    double cpTt, pt, vc[3];
    /* Values given as expressions of position and time
     * (pyfr/solvers/baseadvec/inters.py:95-116): for rho, p, u, v, w and
     * cpTw the start and length of its program in prog (length 0: the
     * constant above); the point coordinates ploc (ndims x n, leading
     * dimension ldp, in the boundary's point order and the kernels'
     * precision); the time at t_dev[0] (device memory). */
    const b200_bcop_t *prog;
    int expr_start[6], expr_len[6];
    const void *ploc;
    int64_t ldp;
    const double *t_dev;
    /* The time when t_dev is NULL (a value bound on the host) */
    double t;
    /* B200_BC_CHAR_RIEM_INV_CTRL: the controller's pressure interpolation
     * p(t) = ic + im*t (pyfr/solvers/euler/kernels/bcs/
     * char-riem-inv-controlled.mako), from ctrl[0], ctrl[1] (device
     * memory) when ctrl is not NULL, else from ic and im */
    double ic, im;
    const double *ctrl;
} b200_bc_t;
/* t[1] = t[0] + c*dt (dt from dt_dev when it is not NULL): the time of an
 * RK stage for the boundary values, enqueued before each stage so that a
 * captured step graph serves every step. */
int b200_stage_time(double *t, const double *dt_dev, double dt, double c, void *stream);

/* Riemann solver ids: [solver-interfaces] riemann-solver */
#define B200_RSOLVER_RUSANOV 0
#define B200_RSOLVER_HLLC 1
#define B200_RSOLVER_HLL 2
#define B200_RSOLVER_ROE 3
#define B200_RSOLVER_ROEM 4
#define B200_RSOLVER_EXACT 5

/* ---- context, memory, streams, events, graphs ------------------------ */
/* Replace the driver wrappers of pyfr/backends/cuda/driver.py (context,
 * mem_alloc/memset/memcpy, streams, events, graphs) used by
 * pyfr/backends/cuda/base.py:9-144 and pyfr/backends/cuda/types.py. */
const char *b200_version(void);
int b200_get_last_error(char *buf, size_t len);
int b200_init(int device);
int b200_device_info(int *sm_count, int *cc_major, int *cc_minor, size_t *free_bytes,
                     size_t *total_bytes, char *name, size_t namelen);
int b200_malloc(void **ptr, size_t nbytes);          /* zero-filled, as base.py:137-144 */
int b200_free(void *ptr);
int b200_host_alloc(void **ptr, size_t nbytes);      /* page-locked, device-mapped host memory */
int b200_host_free(void *ptr);
int b200_memset(void *ptr, int value, size_t nbytes, void *stream);
int b200_memcpy_htod(void *dst, const void *src, size_t nbytes, void *stream);
int b200_memcpy_dtoh(void *dst, const void *src, size_t nbytes, void *stream);
int b200_memcpy_dtod(void *dst, const void *src, size_t nbytes, void *stream);
/* Host round trip of a device array, pipelined: after the work queued on
 * `stream`, `dsrc` goes down to page-locked `host` and back up into `ddst`
 * in `nchunks` pieces (1-64) on `nstreams` copy streams per direction
 * (1-2), each piece going up as soon as it has come down, so that the two
 * directions overlap; `stream` then waits for the last piece.  `ddst` null:
 * down only.  `ddst` may equal `dsrc`.  nstreams -1 or -2: the pieces are
 * copied by kernels through the host buffer's device mapping (memory from
 * b200_host_alloc) instead of the copy engines.  No counterpart in the reference
 * (its MPI exchanges stage through host memory, pyfr/backends/cuda/
 * packing.py:8-112, without this overlap). */
int b200_memcpy_roundtrip(void *host, const void *dsrc, void *ddst, size_t nbytes,
                          int nchunks, int nstreams, void *stream);
int b200_stream_create(void **stream);
int b200_stream_destroy(void *stream);
int b200_stream_sync(void *stream);
int b200_device_sync(void);
int b200_event_create(void **evt);
int b200_event_destroy(void *evt);
int b200_event_record(void *evt, void *stream);
int b200_event_sync(void *evt);
int b200_event_elapsed(float *ms, void *start, void *stop);

/* Measured FP64 FMA throughput of this device (flops per second): eight
 * independent FMA chains per thread over 8 blocks of 256 threads per SM,
 * timed with events on `stream`.  The roofline denominator of the plain
 * FP64 form's kernels, which the FP64 pipe bounds on this GPU.  No
 * counterpart in the reference (a measurement utility). */
int b200_probe_fp64_fma(int iters, double *flops_per_s, void *stream);
/* Graph capture of a kernel sequence; replaces CUDAGraph
 * (pyfr/backends/cuda/types.py:79-116). */
int b200_graph_begin_capture(void *stream);
int b200_graph_end_capture(void *stream, void **gexec);
int b200_graph_launch(void *gexec, void *stream);
int b200_graph_destroy(void *gexec);

/* ---- operator apply: out = alpha*A@B + beta*out ----------------------- */
/* Replaces the `mul` providers CUDAGiMMiKKernels.mul
 * (pyfr/backends/cuda/gimmik.py:23-121) and CUDACUBLASLtKernels.mul
 * (pyfr/backends/cuda/cublaslt.py:169-280).  `a` is the dense m x k
 * operator on the host (row-major); the handle keeps its nonzeros on the
 * device.  B and out are row-major with leading dimensions ldb/ldc. */
int b200_mul_create(const double *a, int m, int k, void **handle);
int b200_mul_nnz(void *handle, int *nnz);
int b200_mul_destroy(void *handle);
int b200_mul_f64(void *handle, const double *b, int64_t ldb, double *c, int64_t ldc,
                 int64_t ncol, double alpha, double beta, void *stream);
int b200_mul_f32(void *handle, const float *b, int64_t ldb, float *c, int64_t ldc,
                 int64_t ncol, float alpha, float beta, void *stream);

/* Tensor-core operator apply for FP32 data (the chosen precision form):
 * A and B are split into BF16 hi/lo halves and out = alpha*(Ahi*Bhi +
 * Ahi*Blo + Alo*Bhi) + beta*out is formed with tcgen05.mma (FP32
 * accumulation in tensor memory).  Same contract as b200_mul_f32 plus:
 * operands 16-byte aligned, ldb/ldc/ncol multiples of 4.  _create fails
 * with B200_ERR_UNSUPPORTED (and reports the shared memory it would need)
 * when the operator does not fit the kernel's shared-memory budget.
 * `err` is a device int that records a pipeline timeout (0 = none). */
int b200_mul_bf16x3_create(const double *a, int m, int k, void **handle, size_t *smem_bytes);
int b200_mul_bf16x3_destroy(void *handle);
int b200_mul_bf16x3(void *handle, const float *b, int64_t ldb, float *c, int64_t ldc,
                    int64_t ncol, float alpha, float beta, int *err, void *stream);

/* Fused operator applies of the chosen form.  A handle made by _create_cat
 * holds two operator blocks, m x k1 and m x k2 (both host, row-major), that
 * act on two inputs, as one operator [A1 | A2] on B1 stacked over B2:
 *     out_z = alpha * S (.) (A1 @ B1_z + A2 @ B2_z) + beta * out_z
 * for the nbatch slices z (slice z of B1 starts bstride1 elements after
 * slice z-1, likewise B2 and out).  S is an optional row scale read in the
 * epilogue: S[r*ldr + e] for row r and element e of the column, the
 * columns being an AoSoA field with nvars variables (slices: one).  This
 * fuses, on the reference's NS graph: tgradpcoru_upts + tgradcoru_upts
 * (pyfr/solvers/baseadvecdiff/elements.py:48-55, blocks M4-M6*M0 and M6),
 * tdivtpcorf + tdivtconf + negdivconf (pyfr/solvers/baseadvec/elements.py:
 * 91-120: blocks M1-M3*M2 and M3, alpha = -1, S = 1/|J|), and the ndims
 * gradcoru_fpts products (pyfr/solvers/baseadvecdiff/elements.py:87-101,
 * one handle, nbatch = ndims).  k2 = 0 makes a one-block handle. */
typedef struct {
    const float *b1, *b2;       /* b2 null for a one-block handle */
    int64_t ldb1, ldb2;
    float *c;
    int64_t ldc, ncol;
    int nbatch;                 /* >= 1 */
    int64_t bstride1, bstride2, cstride;
    float alpha, beta;          /* beta 0 or 1 */
    const float *rowscale;      /* null: none */
    int64_t ldr;                /* 0: one row of scales for every output
                                   row (S[row, e] = rowscale[e]) */
    int nvars;
    int products;               /* 3 (or 0): Ahi*Bhi + Ahi*Blo + Alo*Bhi;
                                   4: plus Alo*Blo; 5: plus Ax3*Bhi (a
                                   handle with a three-term operator) */
    int *err;                   /* device int: pipeline timeout code */
    /* Low-storage RK stage in the epilogue (pyfr/integrators/explicit/
     * kernels/rkvdh2.mako:4-31 in the mixed form of b200_rkmixed_f64f32):
     * with rk_stage != 0 the output R = alpha*S(.)(...) is not stored;
     * instead, for every output value, the FP64 solution acc (leading
     * dimension ldc, the output's layout) becomes acc + dt*b*R and the FP32
     * next-stage input u becomes fl32(acc_old) + fl32(dt*a)*R (rk_stage 1)
     * or fl32(acc_new) (rk_stage 2, the last stage).  dt is read from
     * rk_dt_dev when it is not null, else rk_dt.  One slice, beta = 0, no
     * error estimate.  Replaces the separate stage kernel after the
     * divergence apply of the chosen form. */
    double *rk_acc;
    float *rk_u;
    const double *rk_dt_dev;
    double rk_dt, rk_a, rk_b;
    int rk_stage;
} b200_mul_bf16x3_args_t;
int b200_mul_bf16x3_create_cat(const double *a1, int k1, const double *a2, int k2, int m,
                                void **handle, size_t *smem_bytes);
int b200_mul_bf16x3_apply(void *handle, const b200_mul_bf16x3_args_t *args, void *stream);
/* TF32 variant (the second reduced contraction precision): operator
 * and data rounded to TF32, one tcgen05.mma.kind::tf32 product per K step,
 * FP32 accumulation.  The handles are applied and destroyed with the
 * _bf16x3 entry points (b200_mul_bf16x3, _apply, _destroy); `products` is
 * ignored. */
int b200_mul_tf32_create(const double *a, int m, int k, void **handle, size_t *smem_bytes);
int b200_mul_tf32_create_cat(const double *a1, int k1, const double *a2, int k2, int m,
                             void **handle, size_t *smem_bytes);
/* The kernel's pipeline plan, for an autotuner: a handle with a given
 * number of 16 KB ring stages (even, 4..10) and of epilogue staging tiles
 * per set (1 or 2), split-BF16 (tf32 = 0) or TF32; fails with
 * B200_ERR_UNSUPPORTED when the plan does not fit shared memory.  _plan
 * reports a handle's plan (the _create entry points pick the deepest ring
 * that fits). */
int b200_mul_tc_create_plan(const double *a1, int k1, const double *a2, int k2, int m, int tf32,
                            int nstages, int ntiles, void **handle, size_t *smem_bytes);
int b200_mul_tc_plan(void *handle, int *nstages, int *ntiles);
/* As _create_plan with the operator split into nterms BF16 terms: 2 (hi,
 * lo) or 3 (hi, lo and the rounded remainder, 24 significant bits; split-
 * BF16 only, applied with products = 5).  nstages = ntiles = 0 picks the
 * deepest ring that fits; B200_ERR_UNSUPPORTED when no plan fits shared
 * memory.  _terms reports a handle's operator terms. */
int b200_mul_tc_create_terms(const double *a1, int k1, const double *a2, int k2, int m,
                             int tf32, int nterms, int nstages, int ntiles, void **handle,
                             size_t *smem_bytes);
int b200_mul_tc_terms(void *handle, int *nterms);

/* ---- element pointwise kernels over [nupts, neles] ------------------- */
/* Geometry mode `linear`: 1 computes the metric terms from the element
 * vertices `verts` (nverts, ndims, neles) at the reference solution points
 * `upts` (nupts x ndims, row-major with leading dimension ldup); 0 reads
 * stored metric terms `smats` (ndims, nupts, ndims, neles) and `rcpdjac`
 * (nupts x neles, leading dimension ldr); 2 reads one stored set per
 * element, smats (ndims, 1, ndims, neles) and rcpdjac (1 x neles), for
 * affine elements whose Jacobian is the same at every point. */

/* Euler transformed flux; pyfr/solvers/euler/kernels/tflux.mako:8-30,
 * provider call pyfr/solvers/euler/elements.py:149-206. */
int b200_tflux_euler_f64(int ndims, int nupts, int64_t neles, int linear, double gamma,
                         const double *u, int64_t ldu, double *f, int64_t ldf,
                         const double *smats, int64_t lds, const double *verts, int64_t ldv,
                         const double *upts, int64_t ldup, void *stream);
int b200_tflux_euler_f32(int ndims, int nupts, int64_t neles, int linear, double gamma,
                         const float *u, int64_t ldu, float *f, int64_t ldf,
                         const float *smats, int64_t lds, const float *verts, int64_t ldv,
                         const float *upts, int64_t ldup, void *stream);
/* The Euler flux on shifted inputs q = T(u - u_ref) (b200_gas_t with
 * `shifted`): the flux less the reference state's, formed from the
 * perturbation.  No counterpart in the reference. */
int b200_tflux_euler_shift_f64(int ndims, int nupts, int64_t neles, int linear,
                               const b200_gas_t *gas, const double *u, int64_t ldu, double *f,
                               int64_t ldf, const double *smats, int64_t lds,
                               const double *verts, int64_t ldv, const double *upts,
                               int64_t ldup, void *stream);
int b200_tflux_euler_shift_f32(int ndims, int nupts, int64_t neles, int linear,
                               const b200_gas_t *gas, const float *u, int64_t ldu, float *f,
                               int64_t ldf, const float *smats, int64_t lds, const float *verts,
                               int64_t ldv, const float *upts, int64_t ldup, void *stream);

/* Navier-Stokes fused gradient transform + transformed flux;
 * pyfr/solvers/navstokes/kernels/tflux.mako:13-50, provider call
 * pyfr/solvers/navstokes/elements.py:64-128.  gradu is updated in place.
 * With gradu NULL (the unfused kernel of flux anti-aliasing) f holds the
 * physical gradient at the points on entry, and rcpdjac is not read. */
int b200_tflux_ns_f64(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                      const double *u, int64_t ldu, double *f, int64_t ldf, double *gradu,
                      int64_t ldg, const double *smats, int64_t lds, const double *rcpdjac,
                      int64_t ldr, const double *verts, int64_t ldv, const double *upts,
                      int64_t ldup, void *stream);
int b200_tflux_ns_f32(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                      const float *u, int64_t ldu, float *f, int64_t ldf, float *gradu,
                      int64_t ldg, const float *smats, int64_t lds, const float *rcpdjac,
                      int64_t ldr, const float *verts, int64_t ldv, const float *upts,
                      int64_t ldup, void *stream);
/* The same, leaving gradu in reference space (the transformed gradient is
 * used at the points and not stored): for affine elements whose interface
 * kernels transform the face gradients themselves
 * (b200_intcflux_ns_refgrad_*).  No counterpart in the reference, which
 * always stores the transformed gradient. */
int b200_tflux_ns_refgrad_f64(int ndims, int nupts, int64_t neles, int linear,
                              const b200_gas_t *gas, const double *u, int64_t ldu, double *f,
                              int64_t ldf, double *gradu, int64_t ldg, const double *smats,
                              int64_t lds, const double *rcpdjac, int64_t ldr,
                              const double *verts, int64_t ldv, const double *upts,
                              int64_t ldup, void *stream);
int b200_tflux_ns_refgrad_f32(int ndims, int nupts, int64_t neles, int linear,
                              const b200_gas_t *gas, const float *u, int64_t ldu, float *f,
                              int64_t ldf, float *gradu, int64_t ldg, const float *smats,
                              int64_t lds, const float *rcpdjac, int64_t ldr, const float *verts,
                              int64_t ldv, const float *upts, int64_t ldup, void *stream);

/* Common normal flux at boundary flux points, written over the interior
 * state in the flux-point field (view ul, n points; nl: scaled normals,
 * ndims x n with leading dimension ldn); Euler types 1-4;
 * pyfr/solvers/euler/kernels/bccflux.mako:7-26. */
int b200_bccflux_euler_f64(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                           const b200_bc_t *bc,
                           double *ul_base, const void *ul_map, int ix64, const double *nl,
                           int64_t ldn, void *stream);
int b200_bccflux_euler_f32(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                           const b200_bc_t *bc,
                           float *ul_base, const void *ul_map, int ix64, const float *nl,
                           int64_t ldn, void *stream);
/* LDG common solution at boundary flux points (view ulin -> view ulout);
 * pyfr/solvers/navstokes/kernels/bcconu.mako:6-14. */
int b200_bcconu_f64(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const double *ulin_base, const void *ulin_map, double *ulout_base,
                    const void *ulout_map, int ix64, const double *nl, int64_t ldn,
                    void *stream);
int b200_bcconu_f32(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const float *ulin_base, const void *ulin_map, float *ulout_base,
                    const void *ulout_map, int ix64, const float *nl, int64_t ldn,
                    void *stream);
/* Navier-Stokes common flux (inviscid + LDG viscous) at boundary flux
 * points from the interior state and gradient (vector view gl); the gas
 * must not be shifted; pyfr/solvers/navstokes/kernels/bccflux.mako:10-20
 * with the ghost, ghost-imperm and slip-wall flux states. */
int b200_bccflux_ns_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double tau,
                        const b200_bc_t *bc, double *ul_base, const void *ul_map,
                        const double *gl_base, const void *gl_map, const void *gl_rstr,
                        int ix64, const double *nl, int64_t ldn, void *stream);
int b200_bccflux_ns_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double tau,
                        const b200_bc_t *bc, float *ul_base, const void *ul_map,
                        const float *gl_base, const void *gl_map, const void *gl_rstr,
                        int ix64, const float *nl, int64_t ldn, void *stream);

/* ---- entropy filter -------------------------------------------------- */
/* Shock capturing by the bounds-preserving entropy filter
 * (pyfr/solvers/baseadvec/entfilter.py:5-213).  Elements of one type:
 * ndims, nupts solution points (quads of order 1-5, hexes of order 1-4),
 * nfpts flux points on nfaces faces, nefpts = nupts (+ nfpts when the flux
 * points are not solution points); bounds d_min, p_min, entropy tolerance
 * e_tol; bisection tolerance f_tol and at most niters steps. */
typedef struct {
    int ndims, nupts, nfpts, nefpts, nfaces, order;
    int fpts_in_upts, linearise, niters;
    double gamma, d_min, p_min, e_tol, f_tol;
} b200_ef_t;
/* Filter the solution u (nupts x nvars x neles AoSoA) in place against
 * the smallest entropy of each element's faces entmin (nfaces x neles),
 * then store the element's new minimum in entmin and its filter strength
 * in ef_filter; vdm (nefpts x nupts) modal->nodal, invvdm (nupts x nupts)
 * nodal->modal, m0 (nfpts x nupts), mean_wts (nupts x neles), each with its
 * leading dimension, degs (nupts device ints, the degree of each mode);
 * pyfr/solvers/euler/kernels/entropyfilter.mako:153-221. */
int b200_entropyfilter_f64(const b200_ef_t *p, int64_t neles, double *u, int64_t ldu,
                           double *entmin, int64_t lde, double *ef_filter, const double *vdm,
                           int64_t ldv, const double *invvdm, int64_t ldi, const double *m0,
                           int64_t ldm, const double *mean_wts, int64_t ldw, const int *degs,
                           void *stream);
int b200_entropyfilter_f32(const b200_ef_t *p, int64_t neles, float *u, int64_t ldu,
                           float *entmin, int64_t lde, float *ef_filter, const float *vdm,
                           int64_t ldv, const float *invvdm, int64_t ldi, const float *m0,
                           int64_t ldm, const float *mean_wts, int64_t ldw, const int *degs,
                           void *stream);
/* Artificial viscosity (pyfr/solvers/baseadvecdiff/artvisc.py:24-200):
 * the sensor's sizes and constants.  kwh selects the Klockner-Warburton-
 * Hesthaven decay fit (orders >= 2) over the Persson-Peraire modal ratio;
 * s_weights and baseline hold the fit weights and baseline decay of
 * degrees 1..ndeg-1, se0 = log10(s0 / order^4). */
typedef struct {
    int nupts, nvars, svar, nverts, nmodes, ndeg, kwh;
    double kappa, max_av, se0;
    double s_weights[16], baseline[16];
} b200_av_t;
/* Shock sensor of the variable svar of u (nupts x nvars x neles AoSoA):
 * per element the viscosity of its modal content (invvdm: nmodes x nupts
 * nodal->modal, degs: the degree of each mode, ind: 1 for the modes of
 * the highest degree), maximised into vtx at the element's vertices
 * (vnodes: nverts x neles node numbers, leading dimension ldn); vtx must be
 * zeroed first; pyfr/solvers/baseadvecdiff/kernels/shocksensor.mako. */
int b200_shocksensor_f64(const b200_av_t *p, int64_t neles, const double *u, int64_t ldu,
                         const double *invvdm, int64_t ldi, const int *degs, const int *ind,
                         const int *vnodes, int64_t ldn, double *vtx, void *stream);
int b200_shocksensor_f32(const b200_av_t *p, int64_t neles, const float *u, int64_t ldu,
                         const float *invvdm, int64_t ldi, const int *degs, const int *ind,
                         const int *vnodes, int64_t ldn, float *vtx, void *stream);
/* Viscosity at npts points of each element, linear in its vertex values:
 * out (npts x neles) = op (npts x nverts) . vtx[vnodes];
 * pyfr/solvers/baseadvecdiff/kernels/avfill.mako (and the interpolation
 * at the solution points of pyfr/solvers/navstokes/kernels/tflux.mako). */
int b200_avfill_f64(int nverts, int npts, int64_t neles, const double *vtx, const int *vnodes,
                    int64_t ldn, const double *op, int64_t ldo, double *out, int64_t ldout,
                    void *stream);
int b200_avfill_f32(int nverts, int npts, int64_t neles, const float *vtx, const int *vnodes,
                    int64_t ldn, const float *op, int64_t ldo, float *out, int64_t ldout,
                    void *stream);
/* The Navier-Stokes flux, interface flux and boundary flux with artificial
 * viscosity: as b200_tflux_ns_*, b200_intcflux_ns_* and b200_bccflux_ns_*,
 * with -mu grad u added to the viscous flux (mu at the solution points,
 * av (nupts x neles, leading dimension lda); at the interface and
 * boundary points through the scalar view av_base/av_map of the left
 * side); pyfr/solvers/baseadvecdiff/kernels/artvisc.mako. */
int b200_tflux_ns_av_f64(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                         const double *u, int64_t ldu, double *f, int64_t ldf, double *gradu,
                         int64_t ldg, const double *smats, int64_t lds, const double *rcpdjac,
                         int64_t ldr, const double *verts, int64_t ldv, const double *upts,
                         int64_t ldup, const double *av, int64_t lda, void *stream);
int b200_tflux_ns_av_f32(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                         const float *u, int64_t ldu, float *f, int64_t ldf, float *gradu,
                         int64_t ldg, const float *smats, int64_t lds, const float *rcpdjac,
                         int64_t ldr, const float *verts, int64_t ldv, const float *upts,
                         int64_t ldup, const float *av, int64_t lda, void *stream);
int b200_intcflux_ns_av_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                            double beta, double tau, double *ul_base, const void *ul_map,
                            double *ur_base, const void *ur_map, const double *gl_base,
                            const void *gl_map, const void *gl_rstr, const double *gr_base,
                            const void *gr_map, const void *gr_rstr, int ix64, const double *nl,
                            int64_t ldn, int nl_unit, const double *av_base, const void *av_map, void *stream);
int b200_intcflux_ns_av_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                            double beta, double tau, float *ul_base, const void *ul_map,
                            float *ur_base, const void *ur_map, const float *gl_base,
                            const void *gl_map, const void *gl_rstr, const float *gr_base,
                            const void *gr_map, const void *gr_rstr, int ix64, const float *nl,
                            int64_t ldn, int nl_unit, const float *av_base, const void *av_map, void *stream);
int b200_bccflux_ns_av_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                           double tau, const b200_bc_t *bc, double *ul_base, const void *ul_map,
                           const double *gl_base, const void *gl_map, const void *gl_rstr,
                           int ix64, const double *nl, int64_t ldn, const double *av_base,
                           const void *av_map, void *stream);
int b200_bccflux_ns_av_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                           double tau, const b200_bc_t *bc, float *ul_base, const void *ul_map,
                           const float *gl_base, const void *gl_map, const void *gl_rstr,
                           int ix64, const float *nl, int64_t ldn, const float *av_base,
                           const void *av_map, void *stream);
/* The chosen form's FP64 solution acc takes the FP32 values u32 of the
 * elements whose filter strength is below 1 (both nupts x nvars x neles
 * AoSoA, leading dimensions ldu and lda). */
int b200_ef_merge_f64f32(int nupts, int nvars, int64_t neles, const float *ef_filter,
                         const float *u32, int64_t ldu, double *acc, int64_t lda,
                         void *stream);
/* Minimum entropy of each element on all its faces;
 * pyfr/solvers/euler/kernels/entropylocal.mako:5-40. */
int b200_entropylocal_f64(const b200_ef_t *p, int64_t neles, const double *u, int64_t ldu,
                          double *entmin, int64_t lde, const double *m0, int64_t ldm,
                          void *stream);
int b200_entropylocal_f32(const b200_ef_t *p, int64_t neles, const float *u, int64_t ldu,
                          float *entmin, int64_t lde, const float *m0, int64_t ldm,
                          void *stream);
/* Both faces of each interface take the smaller entropy (views of one
 * value per face); pyfr/solvers/baseadvec/kernels/intcent.mako:4-8. */
int b200_intcent_f64(int64_t n, double *lbase, const void *lmap, double *rbase,
                     const void *rmap, int ix64, void *stream);
int b200_intcent_f32(int64_t n, float *lbase, const void *lmap, float *rbase, const void *rmap,
                     int ix64, void *stream);
/* Boundary faces take the smaller of their value and the entropy of the
 * boundary ghost state at each of their flux points (ent: a view mapping
 * every flux point of a face to the face's value);
 * pyfr/solvers/euler/kernels/bccent.mako:7-25. */
int b200_bccent_f64(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const double *ul_base, const void *ul_map, double *ent_base,
                    const void *ent_map, int ix64, const double *nl, int64_t ldn, void *stream);
int b200_bccent_f32(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const float *ul_base, const void *ul_map, float *ent_base,
                    const void *ent_map, int ix64, const float *nl, int64_t ldn, void *stream);

/* Largest reference-space wave speed of each element for the CFL
 * controller: wspd[e] = max over the solution points of
 * sum_i |sum_j (S_ij/|J|) v_j| + c*sqrt(sum_j (S_ij/|J|)^2);
 * pyfr/solvers/euler/kernels/wavespeed.mako:9-44, provider call
 * pyfr/solvers/euler/elements.py:38-66.  With gas->shifted the input is the
 * reference-state perturbation q (see b200_gas_t). */
int b200_wavespeed_f64(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                       const double *u, int64_t ldu, const double *smats, int64_t lds,
                       const double *rcpdjac, int64_t ldr, const double *verts, int64_t ldv,
                       const double *upts, int64_t ldup, double *wspd, void *stream);
int b200_wavespeed_f32(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                       const float *u, int64_t ldu, const float *smats, int64_t lds,
                       const float *rcpdjac, int64_t ldr, const float *verts, int64_t ldv,
                       const float *upts, int64_t ldup, float *wspd, void *stream);

/* Physical gradient; pyfr/solvers/baseadvecdiff/kernels/gradcoru.mako:10-24. */
int b200_gradcoru_f64(int ndims, int nupts, int64_t neles, int linear, double *gradu,
                      int64_t ldg, const double *smats, int64_t lds, const double *rcpdjac,
                      int64_t ldr, const double *verts, int64_t ldv, const double *upts,
                      int64_t ldup, void *stream);
int b200_gradcoru_f32(int ndims, int nupts, int64_t neles, int linear, float *gradu,
                      int64_t ldg, const float *smats, int64_t lds, const float *rcpdjac,
                      int64_t ldr, const float *verts, int64_t ldv, const float *upts,
                      int64_t ldup, void *stream);

/* R <- -R/|J|; pyfr/solvers/baseadvec/kernels/negdivconf.mako:7-22 (no
 * source terms). */
int b200_negdivconf_f64(int nvars, int nupts, int64_t neles, double *r, int64_t ldr,
                        const double *rcpdjac, int64_t ldj, void *stream);
int b200_negdivconf_f32(int nvars, int nupts, int64_t neles, float *r, int64_t ldr,
                        const float *rcpdjac, int64_t ldj, void *stream);

/* Pack the n points of a view (base, map and, for nrow > 1, the row
 * strides rstr; int64 maps when ix64) into the exchange buffer out of
 * leading dimension ldo: out[r*ldo + (i/32)*32*ncol + c*32 + i%32] = the
 * view's value (r, c) of point i -- the layout of a matrix of io-shape
 * (nrow, ncol, n), which a view of identity map reads back.  Replaces the
 * pack kernel of pyfr/backends/cuda/packing.py:8-60 (and
 * pyfr/backends/base/kernels/packing.mako) for the faces shared with
 * another partition; the unpack is a host-to-device copy of the peer's
 * buffer. */
int b200_pack_view_f64(int64_t n, int nrow, int ncol, const double *base, const void *map,
                       const void *rstr, int ix64, double *out, int64_t ldo, void *stream);
int b200_pack_view_f32(int64_t n, int nrow, int ncol, const float *base, const void *map,
                       const void *rstr, int ix64, float *out, int64_t ldo, void *stream);

/* Source terms: the [solver-plugin-source] expressions of each variable
 * (pyfr/plugins/source.py:15-31, pyfr/plugins/kernels/source.mako) as
 * programs of the point's coordinates ploc, the time and the solution u,
 * evaluated at every solution point by
 *   mode B200_SRC_NEGDIVCONF: R <- -R/|J| + src (negdivconf with its source
 *     macros, pyfr/solvers/baseadvec/kernels/negdivconf.mako:7-22);
 *   mode B200_SRC_ADD: R <- R + src (after an operator apply that already
 *     formed -R/|J|; rcpdjac unused);
 *   mode B200_SRC_EVAL: R <- src (evalsrcmacros,
 *     pyfr/solvers/baseadvec/kernels/evalsrcmacros.mako:7-22; u may be R).
 * prog holds the programs, expr_start/expr_len each variable's (length 0:
 * no source for it); ploc is (nupts x ndims x neles) with leading
 * dimension ldp and u (nupts x nvars x neles) with ldu, both in the
 * kernels' precision and AoSoA layout, u NULL when no program reads it;
 * the time is t_dev[0] (device memory) when t_dev is not NULL, else t.
 * nvars <= 8. */
#define B200_SRC_NEGDIVCONF 0
#define B200_SRC_ADD 1
#define B200_SRC_EVAL 2
typedef struct {
    const b200_bcop_t *prog;
    int expr_start[8], expr_len[8];
    const void *ploc;
    int64_t ldp;
    const void *u;
    int64_t ldu;
    double t;
    const double *t_dev;
} b200_src_t;
int b200_srcterms_f64(int mode, int ndims, int nvars, int nupts, int64_t neles, double *r,
                      int64_t ldr, const double *rcpdjac, int64_t ldj, const b200_src_t *src,
                      void *stream);
int b200_srcterms_f32(int mode, int ndims, int nvars, int nupts, int64_t neles, float *r,
                      int64_t ldr, const float *rcpdjac, int64_t ldj, const b200_src_t *src,
                      void *stream);

/* ---- interface kernels over the interior flux-point pairs ------------ */
/* Euler common normal flux, written +/- to both sides;
 * pyfr/solvers/euler/kernels/intcflux.mako:6-22.  rsolver selects the
 * Riemann solver of pyfr/solvers/euler/kernels/rsolvers/: 0 rusanov,
 * 1 hllc, 2 hll, 3 roe, 4 roem, 5 exact (B200_RSOLVER_*); p_min is the
 * exact solver's star-pressure floor.  nl is the (ndims x n) matrix of
 * scaled left normals, leading dimension ldn; with nl_unit != 0 it is the
 * (ndims + 1) x n matrix of the unit normals (rows 0..ndims-1) and their
 * magnitudes (row ndims), formed once instead of per call (the NS
 * interface kernels below take the same). */
int b200_intcflux_euler_f64(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                            double *ul_base, const void *ul_map, double *ur_base,
                            const void *ur_map, int ix64, const double *nl, int64_t ldn, int nl_unit,
                            void *stream);
int b200_intcflux_euler_f32(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                            float *ul_base,
                            const void *ul_map, float *ur_base, const void *ur_map, int ix64,
                            const float *nl, int64_t ldn, int nl_unit, void *stream);
/* The Rusanov common flux on shifted inputs (b200_gas_t with `shifted`).
 * No counterpart in the reference. */
int b200_intcflux_euler_shift_f64(int ndims, int64_t n, const b200_gas_t *gas, double *ul_base,
                                  const void *ul_map, double *ur_base, const void *ur_map,
                                  int ix64, const double *nl, int64_t ldn, int nl_unit,
                                  void *stream);
int b200_intcflux_euler_shift_f32(int ndims, int64_t n, const b200_gas_t *gas, float *ul_base,
                                  const void *ul_map, float *ur_base, const void *ur_map,
                                  int ix64, const float *nl, int64_t ldn, int nl_unit,
                                  void *stream);

/* Navier-Stokes common flux (Riemann + LDG viscous with beta, tau);
 * pyfr/solvers/navstokes/kernels/intcflux.mako:10-54. */
int b200_intcflux_ns_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double beta,
                         double tau, double *ul_base, const void *ul_map, double *ur_base,
                         const void *ur_map, const double *gl_base, const void *gl_map,
                         const void *gl_rstr, const double *gr_base, const void *gr_map,
                         const void *gr_rstr, int ix64, const double *nl, int64_t ldn, int nl_unit,
                         void *stream);
int b200_intcflux_ns_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double beta,
                         double tau, float *ul_base, const void *ul_map, float *ur_base,
                         const void *ur_map, const float *gl_base, const void *gl_map,
                         const void *gl_rstr, const float *gr_base, const void *gr_map,
                         const void *gr_rstr, int ix64, const float *nl, int64_t ldn, int nl_unit,
                         void *stream);
/* The same with face gradients in reference space, transformed here with
 * the metric terms of affine elements: emet holds (ndims*ndims + 1) rows of
 * one column per element (S[i][j] in row i*ndims + j, 1/|J| in the last
 * row; leading dimension ldm), eidx_l/eidx_r the column of each pair's left
 * and right element (the side that beta = +-1/2 does not read may be
 * NULL).  Pairs with b200_tflux_ns_refgrad_*. */
int b200_intcflux_ns_refgrad_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                                 double beta, double tau, double *ul_base, const void *ul_map,
                                 double *ur_base, const void *ur_map, const double *gl_base,
                                 const void *gl_map, const void *gl_rstr, const double *gr_base,
                                 const void *gr_map, const void *gr_rstr, int ix64,
                                 const double *nl, int64_t ldn, int nl_unit, const double *emet,
                                 int64_t ldm, const int *eidx_l, const int *eidx_r, void *stream);
int b200_intcflux_ns_refgrad_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                                 double beta, double tau, float *ul_base, const void *ul_map,
                                 float *ur_base, const void *ur_map, const float *gl_base,
                                 const void *gl_map, const void *gl_rstr, const float *gr_base,
                                 const void *gr_map, const void *gr_rstr, int ix64,
                                 const float *nl, int64_t ldn, int nl_unit, const float *emet,
                                 int64_t ldm, const int *eidx_l, const int *eidx_r, void *stream);

/* LDG common solution; pyfr/solvers/navstokes/kernels/intconu.mako:4-19. */
int b200_intconu_f64(int nvars, int64_t n, double beta, const double *lin_base,
                     const void *lin_map, const double *rin_base, const void *rin_map,
                     double *lout_base, const void *lout_map, double *rout_base,
                     const void *rout_map, int ix64, void *stream);
int b200_intconu_f32(int nvars, int64_t n, double beta, const float *lin_base,
                     const void *lin_map, const float *rin_base, const void *rin_map,
                     float *lout_base, const void *lout_map, float *rout_base,
                     const void *rout_map, int ix64, void *stream);
/* Same, writing the common solution to both sides for every beta (for
 * beta = +-1/2 the reference writes one side and relies on a prior copy of
 * the solution into the output for the other; when every flux point lies
 * on an interior interface this writes both and the copy is not needed). */
int b200_intconu_both_f64(int nvars, int64_t n, double beta, const double *lin_base,
                          const void *lin_map, const double *rin_base, const void *rin_map,
                          double *lout_base, const void *lout_map, double *rout_base,
                          const void *rout_map, int ix64, void *stream);
int b200_intconu_both_f32(int nvars, int64_t n, double beta, const float *lin_base,
                          const void *lin_map, const float *rin_base, const void *rin_map,
                          float *lout_base, const void *lout_map, float *rout_base,
                          const void *rout_map, int ix64, void *stream);

/* ---- integrator register kernels (flat over n scalars) --------------- */
/* RK stage of the two-register low-storage schemes;
 * pyfr/integrators/explicit/kernels/rkvdh2.mako:4-31 and
 * pyfr/integrators/explicit/steppers.py:165-190. */
int b200_rkvdh2_f64(int64_t n, int stage, int nstages, int errest, double dt, double a,
                    double b, double e, double *r1, double *r2, double *rold, double *rerr,
                    void *stream);
int b200_rkvdh2_f32(int64_t n, int stage, int nstages, int errest, double dt, double a,
                    double b, double e, float *r1, float *r2, float *rold, float *rerr,
                    void *stream);

/* Same with the step size read from device memory at run time (dt_dev: one
 * double), so that one captured step graph serves every dt an adaptive
 * controller picks (the reference rebinds the kernel argument instead,
 * pyfr/backends/cuda/provider.py:15-125). */
int b200_rkvdh2_dt_f64(int64_t n, int stage, int nstages, int errest, const double *dt_dev,
                       double a, double b, double e, double *r1, double *r2, double *rold,
                       double *rerr, void *stream);
int b200_rkvdh2_dt_f32(int64_t n, int stage, int nstages, int errest, const double *dt_dev,
                       double a, double b, double e, float *r1, float *r2, float *rold,
                       float *rerr, void *stream);

/* Mixed-precision form of the rkvdh2 stage (FP32 right-hand side, FP64
 * solution accumulator): acc <- acc + dt*b*rhs in FP64 and u32 <- the next
 * stage's FP32 input, fl32(acc) + fl32(dt*a)*rhs formed in FP32 (the new
 * fl32(acc) at the last stage); the embedded error registers as in rkvdh2.
 * A solution kept relative to a constant reference state (u - u_ref) is
 * stored as that difference in acc.  Replaces the rkvdh2 kernel
 * (pyfr/integrators/explicit/kernels/rkvdh2.mako:4-31) for the chosen
 * precision form, whose second register is only ever an RHS input. */
int b200_rkmixed_f64f32(int64_t n, int stage, int nstages, int errest, double dt, double a,
                        double b, double e, double *acc, const float *rhs, float *u32,
                        double *rold, double *rerr, void *stream);
/* Same with the step size read from device memory (dt_dev: one double). */
int b200_rkmixed_dt_f64f32(int64_t n, int stage, int nstages, int errest, const double *dt_dev,
                           double a, double b, double e, double *acc, const float *rhs,
                           float *u32, double *rold, double *rerr, void *stream);
/* dst <- (float)(src - uref[v]) over n scalars of an AoSoA field with
 * nvars variables (uref null: no shift). */
int b200_cast_f64_f32(int64_t n, const double *src, float *dst, int nvars, const double *uref,
                      void *stream);

/* x0 <- a[0]*x0 + sum_{k>=1} a[k]*xs[k]; xs is a host array of nv device
 * pointers (xs[0] ignored), nv <= 8; pyfr/backends/cuda/kernels/axnpby.mako. */
int b200_axnpby_f64(int64_t n, int nv, double *x0, const double *const *xs, const double *a,
                    void *stream);
int b200_axnpby_f32(int64_t n, int nv, float *x0, const float *const *xs, const double *a,
                    void *stream);

/* Scaled linear combination, per variable v of each value (AoSoA with
 * nvars variables): the terms a[k]*x_k of the registers k whose bit is set
 * in in_mask are multiplied by in_scale[v], the sum by out_scale[v] (null:
 * no scaling); a[0] = 0 stores the sum of the terms k >= 1, a[0] = 1 adds
 * it to x0, any other a[0] stores the sum over all terms including x0.
 * in_scale and out_scale are host arrays of nvars (<= 16) doubles;
 * pyfr/backends/base/blasext.py:9-19 with in_scale, in_scale_idxs and
 * out_scale (pyfr/backends/cuda/kernels/axnpby.mako). */
int b200_axnpby_scaled_f64(int64_t n, int nv, int nvars, double *x0, const double *const *xs,
                           const double *a, const double *in_scale, unsigned in_mask,
                           const double *out_scale, void *stream);
int b200_axnpby_scaled_f32(int64_t n, int nv, int nvars, float *x0, const float *const *xs,
                           const double *a, const double *in_scale, unsigned in_mask,
                           const double *out_scale, void *stream);

/* PI-controller error norm: out[0] = sum (or max when uniform != 0) over
 * the valid points of (err/(atol[v] + rtol*|curr|))^2 (|.| when uniform);
 * atol_dev holds nvars device doubles, scratch at least one double per
 * block (nscratch).  Replaces the reduction kernel of
 * pyfr/backends/cuda/kernels/reduction.mako:4-95 as called from
 * pyfr/integrators/controllers.py:105-117. */
int b200_errest_f64(int nupts, int nvars, int64_t neles, int64_t ld, const double *curr,
                    const double *err, const double *atol_dev, double rtol, int uniform,
                    double *scratch, int nscratch, double *out, void *stream);
/* Same for a solution stored relative to a reference state: curr holds q
 * with u_v = uref[v] + q_v, plus hcoef*q_0 for the last variable (uref:
 * nvars host doubles); err holds the error estimate of q, mapped the same
 * way without the offset; the norm is that of the error of u scaled by |u|. */
int b200_errest_shifted_f64(int nupts, int nvars, int64_t neles, int64_t ld, const double *curr,
                            const double *err, const double *atol_dev, double rtol, int uniform,
                            const double *uref, double hcoef, double *scratch, int nscratch,
                            double *out, void *stream);
int b200_errest_f32(int nupts, int nvars, int64_t neles, int64_t ld, const float *curr,
                    const float *err, const double *atol_dev, double rtol, int uniform,
                    double *scratch, int nscratch, double *out, void *stream);

/* out[0] (a device double) = max of the n values of x; key is 8 bytes of
 * device scratch.  The 'max' reduction of pyfr/backends/base/blasext.py:21-46
 * (pyfr/backends/cuda/kernels/reduction.mako) over one variable, as the
 * CFL controller uses it (pyfr/solvers/baseadvec/system.py:48-52). */
int b200_reduce_max_f64(int64_t n, const double *x, void *key, double *out, void *stream);
int b200_reduce_max_f32(int64_t n, const float *x, void *key, double *out, void *stream);

/* Allocation-free variant of b200_errest_f64; it has no counterpart in the
 * reference.  It is for callers that cannot give the library scratch memory:
 * an asynchronous step loop cannot pay the device synchronisation of
 * cudaFree, and an application whose own pool allocator owns all device
 * memory cannot make a raw allocation.  The partial sums live in a static
 * device array of 4096 doubles that the library holds on every GPU it is
 * loaded on; nblocks (the number of partial sums, as nscratch above) must
 * be in [1, 4096] or the call fails with B200_ERR_ARG.  The first call on
 * a device looks up the array's device address (make it before any stream
 * capture); calls that overlap on the GPU race on the shared array. */
int b200_errest_static_f64(int nupts, int nvars, int64_t neles, int64_t ld, const double *curr,
                           const double *err, const double *atol_dev, double rtol, int uniform,
                           int nblocks, double *out, void *stream);

/* ---- field integrals (kinetic energy, enstrophy, volume) ------------- */
/* out[0] = sum w*rho*|u|^2, out[1] = sum w*rho*|curl u|^2, out[2] = sum w
 * over all solution points, w = quadrature weight * |J| held in `wts`
 * (nupts x neles, leading dimension ldw, FP64); u is the conserved
 * solution, gradu its physical gradient (ndims, nupts, nvars, neles).
 * Accumulated in FP64; scratch holds 3 doubles per block (nscratch
 * blocks).  Replaces the fieldeval reduction of the integrate plugin
 * (pyfr/plugins/fieldeval.py:25-248, pyfr/plugins/kernels/fieldeval.mako)
 * for its documented Taylor-Green integrands. */
int b200_integrals_f64(int ndims, int nupts, int64_t neles, const double *u, int64_t ldu,
                       const double *gradu, int64_t ldg, const double *wts, int64_t ldw,
                       double *scratch, int nscratch, double *out, void *stream);
/* Same with FP32 gradients (the chosen precision form); density and
 * momentum are u_v + uref[v] (uref: ndims + 2 host doubles, or null) for a
 * solution kept relative to a reference state (the energy is not used). */
int b200_integrals_f64f32(int ndims, int nupts, int64_t neles, const double *u, int64_t ldu,
                          const float *gradu, int64_t ldg, const double *wts, int64_t ldw,
                          const double *uref, double *scratch, int nscratch, double *out,
                          void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYFRB200_H */
