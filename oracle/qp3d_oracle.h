/*
 * qp3d_oracle.h -- CPU oracle for the 3D pure-qP VTI time-stepping loop.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only tests/, the smoke check and the CPU baseline leg of
 * bench.py use it, and only as the checker.
 *
 * Three variants of the same per-shot loop (reference: modeling3D.c:49-125,
 * 3dPureqPModeling_single_shot.cu:277-411):
 *
 *   ORACLE_REF32   FP32, restating the reference CPU operators of
 *                  CPU_function.c:301-480 expression by expression, including
 *                  the C++ promotions the reference gets from g++
 *                  (pow(float,int) -> double, sqrt(float) -> float,
 *                  1.0e-02 * uxyzMax -> double).  The copy rotation of
 *                  GPU_kernel.cu:733-812 is used (CPU_function.c:497 never
 *                  sets its index, so the shipped CPU exchange is a no-op on
 *                  garbage); buffers are zeroed and sized as the GPU driver
 *                  sizes them (3dPureqPModeling_single_shot.cu:100-186).
 *   ORACLE_F64     the same discrete scheme evaluated entirely in double
 *                  (inputs promoted from float); used to state the FP32
 *                  rounding error of every result.
 *   ORACLE_MIRROR  FP32, the arithmetic the CUDA kernels perform in their
 *                  fast mode (folded 1/dx coefficients, second differences
 *                  in the reference's (u[+m] - 2u) + u[-m] form, fused
 *                  multiply-adds, a Newton-Raphson reciprocal in the scalar
 *                  operator, IEEE square root), written out operation by
 *                  operation so that a correct kernel matches it bit for bit.
 *                  The kernels' other mode reproduces ORACLE_REF32 itself.
 *
 * Parity pin: ORACLE_REF32 is checked bit-exact against the reference's own
 * CPU_function.c compiled from source (oracle/build.py); with that build
 * absent, the committed golden vectors under tests/golden/ pin it.
 *
 * Data layout: volumes are [nz][nx][ny] float, y fastest (array_new.c:2).
 * PML state, when exchanged with callers, uses the reference face layouts
 * (GPU_kernel.cu:568-628): faces L,R,F,Bk,T,Bo in that order, each holding
 * ten arrays w11,w12,w13,w21,w31,w32,w33,p1,p2,p3 of face size
 *   L,R : pml*ny*nz  index z*ny*pml + xi*ny + y
 *   F,Bk: pml*nx*nz  index z*nx*pml + x*pml + yi
 *   T,Bo: pml*nx*ny  index zi*nx*ny + x*ny + y
 */
#ifndef QP3D_ORACLE_H
#define QP3D_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_REF32 = 0, ORACLE_F64 = 1, ORACLE_MIRROR = 2 };

typedef struct {
    int nx, ny, nz;          /* padded grid */
    int pml;                 /* PML thickness (cells) */
    int sz;                  /* receiver depth (padded z index) */
    float dx, dy, dz, dt;
    const float *vp, *epsilon, *delta;   /* padded volumes [nz][nx][ny] */
    const float *source;                 /* padded volume, or NULL */
    const float *wavelet;                /* per step amplitude */
    const float *dlr, *ddlr, *dtb, *ddtb, *dfb, *ddfb;  /* pml each */
    const float *c, *c2;                 /* 36-entry FD tables (fdcoff1/2) */
    int nthreads;                        /* OpenMP threads, <=0: default */
} oracle_args;

/* Total floats of the canonical PML state buffer. */
size_t oracle_pml_state_size(int nx, int ny, int nz, int pml);

/* Run nsteps steps starting at step index k0 (wavelet[k0..k0+nsteps) used).
 *   u1, u2    : in/out wavefield volumes (previous, current), N floats
 *   u3        : in/out "new" volume, N floats (the reference keeps it between
 *               steps; cells never updated accumulate the source there)
 *   pml_state : in/out canonical PML state, or NULL to start from zero and
 *               discard it
 *   record    : out, nsteps * (nx-2pml) * (ny-2pml) floats, or NULL
 *   uxyzmax   : out, nsteps floats, or NULL
 * For ORACLE_F64 the volume/state/record buffers are double.
 * Returns 0, or a negative value on invalid arguments / allocation failure. */
int oracle_run(int variant, const oracle_args *a, int k0, int nsteps,
               void *u1, void *u2, void *u3, void *pml_state,
               void *record, void *uxyzmax);

/* Mirror-variant helpers, exported so tests can check the product's host-side
 * derivation of the same quantities. */
float oracle_threshold_f(float uxyzmax);        /* largest float <= 0.01*max */
float oracle_threshold_m2(float uxyzmax);       /* largest m2 with sqrtf(m2) <= T */

/* Host utilities restated from CPU_function.c (for parity of derived inputs). */
void oracle_fdcoff1(float *c);                   /* CPU_function.c:111-128 */
void oracle_fdcoff2(float *c);                   /* CPU_function.c:131-148 */
void oracle_pmlcoff(int pml, float vpmax, float dx, float dy, float dz,
                    float *dlr, float *ddlr, float *dtb, float *ddtb,
                    float *dfb, float *ddfb);    /* CPU_function.c:150-169 */
void oracle_source(int sx, int sy, int sz, float fm, float amp, float alpha,
                   float dt, float dx, float dy, float dz, float t0, int nt,
                   int nx, int ny, int nz, float *source, float *wavelet);
                                                 /* CPU_function.c:37-64 */
void oracle_extend_model(const float *in, float *out, int nx, int ny, int nz,
                         int pml);               /* CPU_function.c:67-108 */
float oracle_absmax(const float *a, size_t n);   /* CPU_function.c:10-22 */

/* ---- FP64 adjoint (qp3d_adjoint.c) --------------------------------------
 * The step with the scalar operator frozen per step and cell by the factors
 * a = nx^2+ny^2, b = nz^2 of a base run (0 where it was below the
 * threshold); model in double so that finite differences can perturb it.
 * Volumes are padded [nz][nx][ny] doubles; per-step arrays nt * N. */
typedef struct {
    int nx, ny, nz, pml, sz, nt;
    double dx, dy, dz, dt;
    const double *vp, *eps, *del;        /* N each */
    const float *source;                 /* N, or NULL */
    const float *wavelet;                /* nt */
    const float *dlr, *ddlr, *dtb, *ddtb, *dfb, *ddfb;
    const float *c, *c2;
    int nthreads;
    int live;      /* backward: 1 = also the terms of S's dependence on grad u
                      (the gradient of the live operator), 0 = S frozen */
} oracle_adj_args;

/* Base run with the live scalar operator: the frozen factors of every step. */
int oracle_adj_freeze(const oracle_adj_args *a, double *fa, double *fb);
/* Frozen-operator run: records (nt * hx * hy), and u^k before each step
 * (nt * N) when u_hist is given; extra = nt * N additive sources or NULL. */
int oracle_adj_forward(const oracle_adj_args *a, const double *fa, const double *fb,
                       const double *extra, double *record, double *u_hist);
/* Adjoint run for record residuals resid (nt * hx * hy): gradient of
 * 1/2 |resid|^2 with respect to vp, eps, delta on the cells outside the PML
 * shell (0 inside it), and the adjoint of the additive sources (nt * N). */
int oracle_adj_backward(const oracle_adj_args *a, const double *fa, const double *fb,
                        const double *u_hist, const double *resid, double *g_vp,
                        double *g_eps, double *g_del, double *f_adj);
/* Tangent-linear run about the base trajectory u_hist (u^k before each step,
 * nt * N): records (nt * hx * hy) of the response to additive sources extra
 * (nt * N); with live = 1 the perturbation of S through the unit normal is
 * included, so that oracle_adj_backward (same live, f_adj) is its transpose. */
int oracle_adj_tlm(const oracle_adj_args *a, const double *fa, const double *fb,
                   const double *u_hist, const double *extra, double *record);

#ifdef __cplusplus
}
#endif
#endif
