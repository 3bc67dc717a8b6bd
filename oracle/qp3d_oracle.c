/*
 * qp3d_oracle.c -- CPU oracle for the 3D pure-qP VTI time-stepping loop.
 *
 * TEST INFRASTRUCTURE ONLY (see qp3d_oracle.h).  Build with
 * -ffp-contract=off: the FP32 variants state every rounding explicitly and a
 * compiler that fuses a*b+c would change them (gcc fuses by default on Arm).
 *
 * Reference files cited below are paths inside hlc0216/Gpu-c_3dqmodeling.
 */
#include "qp3d_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define R 5                 /* stencil radius M/2, M = 10 (CPU_function.c:7) */
#define EPSN 2.22e-17       /* CPU_function.c:8, GPU_kernel.cu:7 */

enum { FL = 0, FR, FF, FBK, FT, FBO };                 /* PML faces */
enum { W11 = 0, W12, W13, W21, W31, W32, W33, P1, P2, P3 };

typedef struct {
    size_t fsz[6];
    size_t off[6][10];
    size_t total;
} pml_layout;

static void layout_init(pml_layout *L, int nx, int ny, int nz, int pml)
{
    size_t xf = (size_t)pml * ny * nz, yf = (size_t)pml * nx * nz,
           zf = (size_t)pml * nx * ny;
    size_t s[6] = {xf, xf, yf, yf, zf, zf};
    size_t o = 0;
    for (int f = 0; f < 6; f++) {
        L->fsz[f] = s[f];
        for (int a = 0; a < 10; a++) {
            L->off[f][a] = o;
            o += s[f];
        }
    }
    L->total = o;
}

size_t oracle_pml_state_size(int nx, int ny, int nz, int pml)
{
    pml_layout L;
    layout_init(&L, nx, ny, nz, pml);
    return L.total;
}

/* Face index of cell (z,x,y) (GPU_kernel.cu:568,580,592,604,616,628). */
static inline size_t face_index(int f, int z, int x, int y, int nx, int ny,
                                int nz, int pml)
{
    switch (f) {
    case FL: return (size_t)z * ny * pml + (size_t)x * ny + y;
    case FR: return (size_t)z * ny * pml + (size_t)(x - nx + pml) * ny + y;
    case FF: return (size_t)z * nx * pml + (size_t)x * pml + y;
    case FBK: return (size_t)z * nx * pml + (size_t)x * pml + (y - ny + pml);
    case FT: return (size_t)z * nx * ny + (size_t)x * ny + y;
    default: return (size_t)(z - nz + pml) * ny * nx + (size_t)x * ny + y;
    }
}

/* Region of a cell inside [5,n-5)^3: -1 interior, else the first matching
 * face in the reference's priority order (GPU_kernel.cu:558-626). */
static inline int region(int z, int x, int y, int nx, int ny, int nz, int pml)
{
    if (x >= pml && x < nx - pml && y >= pml && y < ny - pml && z >= pml &&
        z < nz - pml)
        return -1;
    if (x < pml) return FL;
    if (x >= nx - pml) return FR;
    if (y < pml) return FF;
    if (y >= ny - pml) return FBK;
    if (z < pml) return FT;
    return FBO;
}

/* Layer index into the damping profile (GPU_kernel.cu:569,581,593,605,617,629). */
static inline int layer(int f, int z, int x, int y, int nx, int ny, int nz,
                        int pml)
{
    switch (f) {
    case FL: return pml - x;
    case FR: return x - nx + pml;
    case FF: return pml - y;
    case FBK: return y - ny + pml;
    case FT: return pml - z;
    default: return z - nz + pml;
    }
}

static int set_threads(int n)
{
#ifdef _OPENMP
    int prev = omp_get_max_threads();
    if (n > 0) omp_set_num_threads(n);
    return prev;
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Host utilities (restated)                                                 */
/* ------------------------------------------------------------------------- */

float oracle_absmax(const float *a, size_t n)
{   /* CPU_function.c:10-22: Max starts at 0, ">=" keeps the last equal */
    float m = 0.0f;
    for (size_t i = 0; i < n; i++)
        if (fabsf(a[i]) >= m) m = fabsf(a[i]);
    return m;
}

void oracle_fdcoff1(float *c)
{   /* CPU_function.c:111-128 (only [31..35] are used by the M=10 scheme) */
    c[7] = 0.5f;
    c[13] = 0.667f; c[14] = -0.083f;
    c[19] = 0.75f; c[20] = -0.15f; c[21] = 0.0167f;
    c[25] = 0.8f; c[26] = -0.2f; c[27] = 0.038f; c[28] = -0.0036f;
    c[31] = 0.833f; c[32] = -0.2381f; c[33] = 0.059f; c[34] = -0.0099f;
    c[35] = 0.00079f;
}

void oracle_fdcoff2(float *c)
{   /* CPU_function.c:131-148 */
    c[7] = 1.0f;
    c[13] = (float)(4.0 / 3.0); c[14] = (float)(-1.0 / 12.0);
    c[19] = 1.5f; c[20] = -0.15f; c[21] = (float)(1.0 / 90.0);
    c[25] = 1.6f; c[26] = -0.2f; c[27] = (float)(8.0 / 315.0);
    c[28] = (float)(-1.0 / 560);
    c[31] = 1.6667f; c[32] = -0.2381f; c[33] = 0.0397f; c[34] = -0.0050f;
    c[35] = 0.0003f;
}

void oracle_pmlcoff(int pml, float vpmax, float dx, float dy, float dz,
                    float *dlr, float *ddlr, float *dtb, float *ddtb,
                    float *dfb, float *ddfb)
{   /* CPU_function.c:150-169; pow() on float args promotes to double */
    float Rc = 0.00001f, widlr = pml * dx, widtb = pml * dz, widfb = pml * dy;
    float lg = logf(1 / Rc);
    for (int i = 0; i < pml; i++) {
        float widx = (i + 1) * dx, widz = (i + 1) * dz, widy = (i + 1) * dy;
        dlr[i] = (float)(4 * vpmax / (2 * widlr) * pow(widx / widlr, 3) * lg);
        ddlr[i] = (float)(6 * vpmax * widx * widx / pow(widlr, 4) * lg);
        dtb[i] = (float)(4 * vpmax / (2 * widtb) * pow(widz / widtb, 3) * lg);
        ddtb[i] = (float)(6 * vpmax * widz * widz / pow(widtb, 4) * lg);
        dfb[i] = (float)(4 * vpmax / (2 * widfb) * pow(widy / widfb, 3) * lg);
        ddfb[i] = (float)(6 * vpmax * widy * widy / pow(widfb, 4) * lg);
    }
}

void oracle_source(int sx, int sy, int sz, float fm, float amp, float alpha,
                   float dt, float dx, float dy, float dz, float t0, int nt,
                   int nx, int ny, int nz, float *source, float *wavelet)
{   /* CPU_function.c:37-64 */
    const double pi = 3.1415926535898;
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < nx; j++)
            for (int k = 0; k < ny; k++)
                source[(size_t)i * nx * ny + (size_t)j * ny + k] =
                    (float)(amp * exp(-pow(alpha, 2) *
                                      (pow((j - sx) * dx, 2) +
                                       pow((k - sy) * dy, 2) +
                                       pow((i - sz) * dz, 2))));
    for (int k = 0; k < nt; k++) {
        float t = k * dt;
        float temp = (float)pow(pi * fm * (t - t0), 2);
        wavelet[k] = (1 - 2 * temp) * expf(-temp);   /* exp(float) is expf in C++ */
    }
}

void oracle_extend_model(const float *in, float *out, int nx, int ny, int nz,
                         int pml)
{   /* CPU_function.c:67-108: copy interior, then replicate edges z, x, y */
    size_t sxy = (size_t)nx * ny;
    int hx = nx - 2 * pml, hy = ny - 2 * pml;
    for (int i = pml; i < nz - pml; i++)
        for (int j = pml; j < nx - pml; j++)
            for (int k = pml; k < ny - pml; k++)
                out[i * sxy + (size_t)j * ny + k] =
                    in[(size_t)(i - pml) * hx * hy + (size_t)(j - pml) * hy + k - pml];
    for (int i = 0; i < pml; i++)
        for (int j = pml; j < nx - pml; j++)
            for (int k = pml; k < ny - pml; k++)
                out[i * sxy + (size_t)j * ny + k] = out[pml * sxy + (size_t)j * ny + k];
    for (int i = nz - pml; i < nz; i++)
        for (int j = pml; j < nx - pml; j++)
            for (int k = pml; k < ny - pml; k++)
                out[i * sxy + (size_t)j * ny + k] =
                    out[(size_t)(nz - pml - 1) * sxy + (size_t)j * ny + k];
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < pml; j++)
            for (int k = pml; k < ny - pml; k++)
                out[i * sxy + (size_t)j * ny + k] = out[i * sxy + (size_t)pml * ny + k];
    for (int i = 0; i < nz; i++)
        for (int j = nx - pml; j < nx; j++)
            for (int k = pml; k < ny - pml; k++)
                out[i * sxy + (size_t)j * ny + k] =
                    out[i * sxy + (size_t)(nx - pml - 1) * ny + k];
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < nx; j++)
            for (int k = 0; k < pml; k++)
                out[i * sxy + (size_t)j * ny + k] = out[i * sxy + (size_t)j * ny + pml];
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < nx; j++)
            for (int k = ny - pml; k < ny; k++)
                out[i * sxy + (size_t)j * ny + k] =
                    out[i * sxy + (size_t)j * ny + ny - pml - 1];
}

/* ------------------------------------------------------------------------- */
/* Threshold helpers (mirror variant)                                        */
/* ------------------------------------------------------------------------- */

float oracle_threshold_f(float uxyzmax)
{   /* (double)mode > 1.0e-02*uxyzMax  <=>  mode > T for float mode, T = the
     * largest float not above the double product (GPU_kernel.cu:99). */
    double td = 1.0e-02 * (double)uxyzmax;
    float t = (float)td;
    if ((double)t > td) t = nextafterf(t, -INFINITY);
    return t;
}

float oracle_threshold_m2(float uxyzmax)
{   /* sqrtf(m2) > T  <=>  m2 > T2, T2 = max{x : sqrtf(x) <= T}. */
    float t = oracle_threshold_f(uxyzmax);
    if (!(t >= 0.0f)) return t;
    float x = t * t;
    while (x > 0.0f && sqrtf(x) > t) x = nextafterf(x, 0.0f);
    for (;;) {
        float nx_ = nextafterf(x, INFINITY);
        if (isinf(nx_) || sqrtf(nx_) > t) break;
        x = nx_;
    }
    return x;
}

/* ------------------------------------------------------------------------- */
/* FP32 state shared by REF32 and MIRROR                                     */
/* ------------------------------------------------------------------------- */

typedef struct {
    int nx, ny, nz, pml;
    size_t N;
    float *u1, *u2, *u3, *ux, *uy, *uz, *S;
    float *st;               /* canonical PML state */
    pml_layout L;
} st32;

typedef struct {
    int nx, ny, nz, pml;
    size_t N;
    double *u1, *u2, *u3, *ux, *uy, *uz, *S;
    double *st;
    pml_layout L;
} st64;

#define IX(z, x, y) ((size_t)(z) * nx * ny + (size_t)(x) * ny + (y))

/* ---- REF32: CPU_function.c:301-324 ------------------------------------- */
static void ref32_grad(st32 *s, const float *c, float dx, float dy, float dz)
{
    int nx = s->nx, ny = s->ny, nz = s->nz;
    const float *u2 = s->u2;
#pragma omp parallel for schedule(static)
    for (int i = R; i < nz - R; i++)
        for (int j = R; j < nx - R; j++)
            for (int k = R; k < ny - R; k++) {
                float Ux = 0.0f, Uy = 0.0f, Uz = 0.0f;
                for (int m = 1; m <= R; m++) {
                    Ux = Ux + c[30 + m] * (u2[IX(i, j + m, k)] - u2[IX(i, j - m, k)]) / dx;
                    Uy = Uy + c[30 + m] * (u2[IX(i, j, k + m)] - u2[IX(i, j, k - m)]) / dy;
                    Uz = Uz + c[30 + m] * (u2[IX(i + m, j, k)] - u2[IX(i - m, j, k)]) / dz;
                }
                s->ux[IX(i, j, k)] = Ux;
                s->uy[IX(i, j, k)] = Uy;
                s->uz[IX(i, j, k)] = Uz;
            }
}

/* absMaxval over the whole volume, three times, then the two ternaries of
 * modeling3D.c:54-59.  Max is order independent, so chunks are combined. */
static float absmax_par(const float *a, size_t n)
{
    float m = 0.0f;
#pragma omp parallel
    {
        float lm = 0.0f;
#pragma omp for schedule(static) nowait
        for (size_t i = 0; i < n; i++)
            if (fabsf(a[i]) >= lm) lm = fabsf(a[i]);
#pragma omp critical
        if (lm >= m) m = lm;
    }
    return m;
}

static float uxyz_max32(st32 *s)
{
    float a = absmax_par(s->ux, s->N), b = absmax_par(s->uy, s->N),
          c = absmax_par(s->uz, s->N);
    float m = (a > b) ? a : b;
    return (m > c) ? m : c;
}

/* ---- REF32: CPU_function.c:339-370 ------------------------------------- */
static void ref32_scalar(st32 *s, float uxyzMax, const float *epsilon,
                         const float *delta)
{
    int nx = s->nx, ny = s->ny, nz = s->nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++) {
                size_t i = IX(z, x, y);
                s->S[i] = 1.0f;
                if (y >= 5 && y < ny - 5 && x >= 5 && x < nx - 5 && z >= 5 && z < nz - 5) {
                    float ux = s->ux[i], uy = s->uy[i], uz = s->uz[i];
                    float mode = sqrtf(ux * ux + uy * uy + uz * uz);
                    float nxv, nyv, nzv;
                    if ((double)mode > 1.0e-02 * (double)uxyzMax) {
                        nxv = (float)((double)ux / ((double)mode + EPSN));
                        nyv = (float)((double)uy / ((double)mode + EPSN));
                        nzv = (float)((double)uz / ((double)mode + EPSN));
                    } else {
                        nxv = nyv = nzv = 0.0f;
                    }
                    float e = epsilon[i], d = delta[i];
                    float aa = nxv * nxv + nyv * nyv;
                    float num = 8 * (e - d) * aa * nzv * nzv;
                    float base = 1 + 2 * e * aa;
                    double den = (double)base * (double)base;     /* pow(float,2) */
                    s->S[i] = (float)(0.5 * (1 + sqrt(1 - (double)num / den)));
                }
            }
}

/* ---- REF32: CPU_function.c:371-480 ------------------------------------- */
static void ref32_update(st32 *s, const oracle_args *a)
{
    int nx = s->nx, ny = s->ny, nz = s->nz, pml = s->pml;
    const float *c2 = a->c2, *eps = a->epsilon, *vp = a->vp;
    float dx = a->dx, dy = a->dy, dz = a->dz, dt = a->dt;
    const float *u1 = s->u1, *u2 = s->u2;
    float *u3 = s->u3, *st = s->st;
#pragma omp parallel for schedule(static)
    for (int z = R; z < nz - R; z++)
        for (int x = R; x < nx - R; x++)
            for (int y = R; y < ny - R; y++) {
                size_t i = IX(z, x, y);
                float Uxx = 0.0f, Uyy = 0.0f, Uzz = 0.0f;
                for (int m = 1; m <= R; m++) {
                    Uxx = Uxx + c2[30 + m] * (u2[IX(z, x + m, y)] - 2 * u2[i] + u2[IX(z, x - m, y)]) / (dx * dx);
                    Uyy = Uyy + c2[30 + m] * (u2[IX(z, x, y + m)] - 2 * u2[i] + u2[IX(z, x, y - m)]) / (dy * dy);
                    Uzz = Uzz + c2[30 + m] * (u2[IX(z + m, x, y)] - 2 * u2[i] + u2[IX(z - m, x, y)]) / (dz * dz);
                }
                int f = region(z, x, y, nx, ny, nz, pml);
                float S = s->S[i], e = eps[i];
                if (f < 0) {
                    u3[i] = 2 * u2[i] - u1[i] + dt * dt * ((1 + 2 * e) * (Uxx + Uyy) + Uzz) * S * vp[i] * vp[i];
                    continue;
                }
                const float *dp, *ddp;
                float Unn, Un, tang;
                double An;     /* normal coefficient, (e2*S) or S, times (vp*dt)^2 */
                double At;     /* tangential coefficient */
                float vdt = vp[i] * dt;
                double vdt2 = (double)vdt * (double)vdt;          /* pow(vp*dt,2) */
                if (f == FL || f == FR) {
                    dp = a->dlr; ddp = a->ddlr;
                    An = (double)((1 + 2 * e) * S) * vdt2;
                    Unn = Uxx; Un = s->ux[i];
                    At = (double)S * vdt2; tang = Uzz + (1 + 2 * e) * Uyy;
                } else if (f == FF || f == FBK) {
                    dp = a->dfb; ddp = a->ddfb;
                    An = (double)((1 + 2 * e) * S) * vdt2;
                    Unn = Uyy; Un = s->uy[i];
                    At = (double)S * vdt2; tang = Uzz + (1 + 2 * e) * Uxx;
                } else {
                    dp = a->dtb; ddp = a->ddtb;
                    An = (double)S * vdt2;
                    Unn = Uzz; Un = s->uz[i];
                    At = (double)((1 + 2 * e) * S) * vdt2; tang = Uxx + Uyy;
                }
                int li = layer(f, z, x, y, nx, ny, nz, pml);
                float d = dp[li], dd = ddp[li];
                size_t fi = face_index(f, z, x, y, nx, ny, nz, pml);
                float *w11 = st + s->L.off[f][W11], *w12 = st + s->L.off[f][W12],
                      *w13 = st + s->L.off[f][W13], *w21 = st + s->L.off[f][W21],
                      *w31 = st + s->L.off[f][W31], *w32 = st + s->L.off[f][W32],
                      *w33 = st + s->L.off[f][W33], *p1 = st + s->L.off[f][P1],
                      *p2 = st + s->L.off[f][P2], *p3 = st + s->L.off[f][P3];
                float b1 = d * dt + 1;          /* base of pow((d*dt+1),2) */
                float b2 = 1 + dt * d;          /* base of pow((1+dt*d),2) */
                double t1 = An * (double)Unn - ((double)b1 * b1 - 3) * (double)w12[fi];
                w13[fi] = (float)(t1 + (double)((2 * d * dt - 1) * w11[fi]));
                double q = (3 - (double)b2 * b2) * (double)p2[fi] +
                           (double)((2 * d * dt - 1) * p1[fi]);
                double src = An * (double)dd * (double)Un;
                int minus = (f == FR || f == FBK || f == FBO);
                p3[fi] = (float)(minus ? q - src : q + src);
                w21[fi] = dt * p3[fi] + w21[fi] * (1 - dt * d);
                w33[fi] = (float)(At * (double)tang + (double)(2 * w32[fi]) - (double)w31[fi]);
                u3[i] = w13[fi] + w21[fi] + w33[fi];
            }
}

/* ---- MIRROR: the CUDA kernels' arithmetic, operation by operation ------- */
typedef struct {
    float cx[R], cy[R], cz[R];        /* c[30+m]/h */
    float c2x[R], c2y[R], c2z[R];     /* c2[30+m]/(h*h) */
} mirror_coef;

static void mirror_coef_init(mirror_coef *k, const float *c, const float *c2,
                             float dx, float dy, float dz)
{
    float dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
    for (int m = 0; m < R; m++) {
        k->cx[m] = c[31 + m] / dx;
        k->cy[m] = c[31 + m] / dy;
        k->cz[m] = c[31 + m] / dz;
        k->c2x[m] = c2[31 + m] / dx2;
        k->c2y[m] = c2[31 + m] / dy2;
        k->c2z[m] = c2[31 + m] / dz2;
    }
}

/* Derivatives of u at cell i along one axis with stride st. */
static inline void mirror_axis(const float *u, size_t i, size_t st,
                               const float *cc, const float *c2c, float *U1, float *U2)
{
    float g = 0.0f, l = 0.0f;
    for (int m = 0; m < R; m++) {
        float p = u[i + (m + 1) * st], q = u[i - (m + 1) * st];
        /* second difference in the reference's form (u[+m] - 2u) + u[-m] */
        float dmm = p - q, smm = fmaf(-2.0f, u[i], p) + q;
        g = (m == 0) ? cc[0] * dmm : fmaf(cc[m], dmm, g);
        l = (m == 0) ? c2c[0] * smm : fmaf(c2c[m], smm, l);
    }
    *U1 = g;
    *U2 = l;
}

static float mirror_gradmax(st32 *s, const mirror_coef *k)
{
    int nx = s->nx, ny = s->ny, nz = s->nz;
    const float *u = s->u2;
    float gm = 0.0f;
#pragma omp parallel
    {
        float lm = 0.0f;
#pragma omp for schedule(static) nowait
        for (int z = R; z < nz - R; z++)
            for (int x = R; x < nx - R; x++)
                for (int y = R; y < ny - R; y++) {
                    size_t i = IX(z, x, y);
                    float Ux, Uy, Uz, t;
                    mirror_axis(u, i, (size_t)ny, k->cx, k->c2x, &Ux, &t);
                    mirror_axis(u, i, 1, k->cy, k->c2y, &Uy, &t);
                    mirror_axis(u, i, (size_t)nx * ny, k->cz, k->c2z, &Uz, &t);
                    lm = fmaxf(lm, fmaxf(fabsf(Ux), fmaxf(fabsf(Uy), fabsf(Uz))));
                }
#pragma omp critical
        gm = fmaxf(gm, lm);
    }
    return gm;
}

/* 1/x as the kernels compute it: Newton-Raphson iterations r <- r + r(1 - x r)
 * from the initial guess that negates the exponent of x in its integer
 * representation (the device function rcp_nr, same constant and operation
 * order, each step one fused multiply-add).  Within about 1 ulp of 1/x for
 * normal positive x. */
static inline float mirror_rcp(float x)
{
    uint32_t b;
    float r;
    memcpy(&b, &x, 4);
    b = 0x7EF311C3u - b;
    memcpy(&r, &b, 4);
    for (int it = 0; it < 3; it++) {
        float e = fmaf(-x, r, 1.0f);
        r = fmaf(r, e, r);
    }
    return r;
}

/* Per-layer PML coefficients as the product derives them on the host. */
typedef struct { float a1, a2, a3, dd; } layer_coef;

static void mirror_layer(layer_coef *lc, float d, float dd, float dt)
{
    float b = d * dt + 1.0f;
    lc->a1 = (float)((double)b * (double)b - 3.0);
    lc->a2 = 2.0f * d * dt - 1.0f;
    lc->a3 = 1.0f - dt * d;
    lc->dd = dd;
}

static void mirror_update(st32 *s, const oracle_args *a, const mirror_coef *k,
                          float T2)
{
    int nx = s->nx, ny = s->ny, nz = s->nz, pml = s->pml;
    const float *u1 = s->u1, *u2 = s->u2;
    float *u3 = s->u3, *st = s->st;
    float dt = a->dt;
#pragma omp parallel for schedule(static)
    for (int z = R; z < nz - R; z++)
        for (int x = R; x < nx - R; x++)
            for (int y = R; y < ny - R; y++) {
                size_t i = IX(z, x, y);
                float Ux, Uy, Uz, Uxx, Uyy, Uzz;
                mirror_axis(u2, i, (size_t)ny, k->cx, k->c2x, &Ux, &Uxx);
                mirror_axis(u2, i, 1, k->cy, k->c2y, &Uy, &Uyy);
                mirror_axis(u2, i, (size_t)nx * ny, k->cz, k->c2z, &Uz, &Uzz);
                /* per-cell parameters as stored on the device */
                float vdt = a->vp[i] * dt;
                float K = vdt * vdt;
                float e2x = 2.0f * a->epsilon[i];
                float r8 = 8.0f * (a->epsilon[i] - a->delta[i]);
                /* scalar operator */
                float h2 = Ux * Ux;
                h2 = fmaf(Uy, Uy, h2);
                float m2 = fmaf(Uz, Uz, h2);
                float S = 1.0f;
                if (m2 > T2) {
                    /* a(1-a)/(1+2eps a)^2 = (h2 r)(v2 r), r = 1/(m2 + 2eps h2) */
                    float v2 = Uz * Uz;
                    float r = mirror_rcp(fmaf(e2x, h2, m2));
                    float q = (r8 * (h2 * r)) * (v2 * r);
                    S = fmaf(0.5f, sqrtf(1.0f - q), 0.5f);
                }
                float KS = K * S;
                float e2 = 1.0f + e2x;
                int f = region(z, x, y, nx, ny, nz, pml);
                if (f < 0) {
                    float L = fmaf(e2, Uxx + Uyy, Uzz);
                    u3[i] = fmaf(KS, L, fmaf(2.0f, u2[i], -u1[i]));
                    continue;
                }
                float A, Unn, Un, Bt, Tt;
                const float *dp, *ddp;
                if (f == FL || f == FR) {
                    A = e2 * KS; Unn = Uxx; Un = Ux; Bt = KS; Tt = fmaf(e2, Uyy, Uzz);
                    dp = a->dlr; ddp = a->ddlr;
                } else if (f == FF || f == FBK) {
                    A = e2 * KS; Unn = Uyy; Un = Uy; Bt = KS; Tt = fmaf(e2, Uxx, Uzz);
                    dp = a->dfb; ddp = a->ddfb;
                } else {
                    A = KS; Unn = Uzz; Un = Uz; Bt = e2 * KS; Tt = Uxx + Uyy;
                    dp = a->dtb; ddp = a->ddtb;
                }
                int li = layer(f, z, x, y, nx, ny, nz, pml);
                layer_coef lc;
                mirror_layer(&lc, dp[li], ddp[li], dt);
                size_t fi = face_index(f, z, x, y, nx, ny, nz, pml);
                float *w11 = st + s->L.off[f][W11], *w12 = st + s->L.off[f][W12],
                      *w13 = st + s->L.off[f][W13], *w21 = st + s->L.off[f][W21],
                      *w31 = st + s->L.off[f][W31], *w32 = st + s->L.off[f][W32],
                      *w33 = st + s->L.off[f][W33], *p1 = st + s->L.off[f][P1],
                      *p2 = st + s->L.off[f][P2], *p3 = st + s->L.off[f][P3];
                float nw13 = fmaf(A, Unn, fmaf(-lc.a1, w12[fi], lc.a2 * w11[fi]));
                float Ad = A * lc.dd;
                if (f == FR || f == FBK || f == FBO) Ad = -Ad;
                float np3 = fmaf(Ad, Un, fmaf(-lc.a1, p2[fi], lc.a2 * p1[fi]));
                float nw21 = fmaf(dt, np3, lc.a3 * w21[fi]);
                float nw33 = fmaf(Bt, Tt, fmaf(2.0f, w32[fi], -w31[fi]));
                w13[fi] = nw13; p3[fi] = np3; w21[fi] = nw21; w33[fi] = nw33;
                u3[i] = (nw13 + nw21) + nw33;
            }
}

/* ---- shared FP32 step tail: addsource, exchange, record ----------------- */
static void addsource32(st32 *s, const float *source, float w)
{   /* CPU_function.c:326-338 */
    if (!source) return;
    float *u3 = s->u3;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < s->N; i++) u3[i] += source[i] * w;
}

static void exchange32(st32 *s)
{   /* GPU_kernel.cu:733-812: u1<-u2<-u3 and each PML level 1<-2<-3 by copy */
    memcpy(s->u1, s->u2, s->N * sizeof(float));
    memcpy(s->u2, s->u3, s->N * sizeof(float));
    for (int f = 0; f < 6; f++) {
        size_t n = s->L.fsz[f];
        float *b = s->st;
        memcpy(b + s->L.off[f][W11], b + s->L.off[f][W12], n * sizeof(float));
        memcpy(b + s->L.off[f][W12], b + s->L.off[f][W13], n * sizeof(float));
        memcpy(b + s->L.off[f][W31], b + s->L.off[f][W32], n * sizeof(float));
        memcpy(b + s->L.off[f][W32], b + s->L.off[f][W33], n * sizeof(float));
        memcpy(b + s->L.off[f][P1], b + s->L.off[f][P2], n * sizeof(float));
        memcpy(b + s->L.off[f][P2], b + s->L.off[f][P3], n * sizeof(float));
    }
}

static void record32(st32 *s, int sz, float *rec)
{   /* 3dPureqPModeling_single_shot.cu:333-337 */
    int nx = s->nx, ny = s->ny, pml = s->pml;
    int hy = ny - 2 * pml;
    for (int x = pml; x < nx - pml; x++)
        for (int y = pml; y < ny - pml; y++)
            rec[(size_t)(x - pml) * hy + (y - pml)] = s->u2[IX(sz, x, y)];
}

/* ---- F64: the same scheme in double ------------------------------------ */
static void f64_step(st64 *s, const oracle_args *a, const double *c,
                     const double *c2, const double *vp, const double *eps,
                     const double *del, double *out_max)
{
    int nx = s->nx, ny = s->ny, nz = s->nz, pml = s->pml;
    double dx = a->dx, dy = a->dy, dz = a->dz, dt = a->dt;
    const double *u2 = s->u2, *u1 = s->u1;
    double *u3 = s->u3, *st = s->st;
    /* grad */
#pragma omp parallel for schedule(static)
    for (int i = R; i < nz - R; i++)
        for (int j = R; j < nx - R; j++)
            for (int k = R; k < ny - R; k++) {
                double Ux = 0, Uy = 0, Uz = 0;
                for (int m = 1; m <= R; m++) {
                    Ux += c[30 + m] * (u2[IX(i, j + m, k)] - u2[IX(i, j - m, k)]) / dx;
                    Uy += c[30 + m] * (u2[IX(i, j, k + m)] - u2[IX(i, j, k - m)]) / dy;
                    Uz += c[30 + m] * (u2[IX(i + m, j, k)] - u2[IX(i - m, j, k)]) / dz;
                }
                s->ux[IX(i, j, k)] = Ux;
                s->uy[IX(i, j, k)] = Uy;
                s->uz[IX(i, j, k)] = Uz;
            }
    double M = 0.0;
#pragma omp parallel
    {
        double lm = 0.0;
#pragma omp for schedule(static) nowait
        for (size_t i = 0; i < s->N; i++) {
            double v = fmax(fabs(s->ux[i]), fmax(fabs(s->uy[i]), fabs(s->uz[i])));
            if (v > lm) lm = v;
        }
#pragma omp critical
        if (lm > M) M = lm;
    }
    *out_max = M;
    /* S */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++) {
                size_t i = IX(z, x, y);
                s->S[i] = 1.0;
                if (y >= 5 && y < ny - 5 && x >= 5 && x < nx - 5 && z >= 5 && z < nz - 5) {
                    double ux = s->ux[i], uy = s->uy[i], uz = s->uz[i];
                    double mode = sqrt(ux * ux + uy * uy + uz * uz);
                    double nxv = 0, nyv = 0, nzv = 0;
                    if (mode > 1.0e-02 * M) {
                        nxv = ux / (mode + EPSN);
                        nyv = uy / (mode + EPSN);
                        nzv = uz / (mode + EPSN);
                    }
                    double e = eps[i], d = del[i], aa = nxv * nxv + nyv * nyv;
                    double base = 1 + 2 * e * aa;
                    s->S[i] = 0.5 * (1 + sqrt(1 - 8 * (e - d) * aa * nzv * nzv / (base * base)));
                }
            }
    /* update */
#pragma omp parallel for schedule(static)
    for (int z = R; z < nz - R; z++)
        for (int x = R; x < nx - R; x++)
            for (int y = R; y < ny - R; y++) {
                size_t i = IX(z, x, y);
                double Uxx = 0, Uyy = 0, Uzz = 0;
                for (int m = 1; m <= R; m++) {
                    Uxx += c2[30 + m] * (u2[IX(z, x + m, y)] - 2 * u2[i] + u2[IX(z, x - m, y)]) / (dx * dx);
                    Uyy += c2[30 + m] * (u2[IX(z, x, y + m)] - 2 * u2[i] + u2[IX(z, x, y - m)]) / (dy * dy);
                    Uzz += c2[30 + m] * (u2[IX(z + m, x, y)] - 2 * u2[i] + u2[IX(z - m, x, y)]) / (dz * dz);
                }
                int f = region(z, x, y, nx, ny, nz, pml);
                double S = s->S[i], e = eps[i], v = vp[i];
                if (f < 0) {
                    u3[i] = 2 * u2[i] - u1[i] + dt * dt * ((1 + 2 * e) * (Uxx + Uyy) + Uzz) * S * v * v;
                    continue;
                }
                double An, At, Unn, Un, tang;
                const float *dp, *ddp;
                double vdt2 = (v * dt) * (v * dt);
                if (f == FL || f == FR) {
                    An = (1 + 2 * e) * S * vdt2; Unn = Uxx; Un = s->ux[i];
                    At = S * vdt2; tang = Uzz + (1 + 2 * e) * Uyy;
                    dp = a->dlr; ddp = a->ddlr;
                } else if (f == FF || f == FBK) {
                    An = (1 + 2 * e) * S * vdt2; Unn = Uyy; Un = s->uy[i];
                    At = S * vdt2; tang = Uzz + (1 + 2 * e) * Uxx;
                    dp = a->dfb; ddp = a->ddfb;
                } else {
                    An = S * vdt2; Unn = Uzz; Un = s->uz[i];
                    At = (1 + 2 * e) * S * vdt2; tang = Uxx + Uyy;
                    dp = a->dtb; ddp = a->ddtb;
                }
                int li = layer(f, z, x, y, nx, ny, nz, pml);
                double d = dp[li], dd = ddp[li];
                size_t fi = face_index(f, z, x, y, nx, ny, nz, pml);
                double *w11 = st + s->L.off[f][W11], *w12 = st + s->L.off[f][W12],
                       *w13 = st + s->L.off[f][W13], *w21 = st + s->L.off[f][W21],
                       *w31 = st + s->L.off[f][W31], *w32 = st + s->L.off[f][W32],
                       *w33 = st + s->L.off[f][W33], *p1 = st + s->L.off[f][P1],
                       *p2 = st + s->L.off[f][P2], *p3 = st + s->L.off[f][P3];
                double b = d * dt + 1;
                w13[fi] = An * Unn - (b * b - 3) * w12[fi] + (2 * d * dt - 1) * w11[fi];
                double sgn = (f == FR || f == FBK || f == FBO) ? -1.0 : 1.0;
                p3[fi] = (3 - b * b) * p2[fi] + (2 * d * dt - 1) * p1[fi] + sgn * An * dd * Un;
                w21[fi] = dt * p3[fi] + w21[fi] * (1 - dt * d);
                w33[fi] = At * tang + 2 * w32[fi] - w31[fi];
                u3[i] = w13[fi] + w21[fi] + w33[fi];
            }
}

/* ------------------------------------------------------------------------- */

static int valid_args(const oracle_args *a)
{
    if (!a || !a->vp || !a->epsilon || !a->delta || !a->wavelet || !a->c || !a->c2)
        return 0;
    if (a->nx < 11 || a->ny < 11 || a->nz < 11 || a->pml < 0) return 0;
    if (2 * a->pml > a->nx || 2 * a->pml > a->ny || 2 * a->pml > a->nz) return 0;
    if (a->pml > 0 && (!a->dlr || !a->ddlr || !a->dtb || !a->ddtb || !a->dfb || !a->ddfb))
        return 0;
    if (a->sz < 0 || a->sz >= a->nz) return 0;
    return 1;
}

static int run32(int variant, const oracle_args *a, int k0, int nsteps,
                 float *u1, float *u2, float *u3, float *pml_state,
                 float *record, float *uxyzmax)
{
    st32 s;
    int nx = a->nx, ny = a->ny, nz = a->nz;
    s.nx = nx; s.ny = ny; s.nz = nz; s.pml = a->pml;
    s.N = (size_t)nx * ny * nz;
    layout_init(&s.L, nx, ny, nz, a->pml);
    s.u1 = u1; s.u2 = u2; s.u3 = u3;
    s.ux = calloc(s.N, sizeof(float));
    s.uy = calloc(s.N, sizeof(float));
    s.uz = calloc(s.N, sizeof(float));
    s.S = calloc(s.N, sizeof(float));
    float *own = NULL;
    if (!pml_state) own = pml_state = calloc(s.L.total + 1, sizeof(float));
    s.st = pml_state;
    if (!s.ux || !s.uy || !s.uz || !s.S || !pml_state) {
        free(s.ux); free(s.uy); free(s.uz); free(s.S); free(own);
        return -2;
    }
    mirror_coef mk;
    mirror_coef_init(&mk, a->c, a->c2, a->dx, a->dy, a->dz);
    size_t plane = (size_t)(nx - 2 * a->pml) * (ny - 2 * a->pml);
    for (int k = 0; k < nsteps; k++) {
        float M;
        if (variant == ORACLE_REF32) {
            ref32_grad(&s, a->c, a->dx, a->dy, a->dz);
            M = uxyz_max32(&s);
            ref32_scalar(&s, M, a->epsilon, a->delta);
            ref32_update(&s, a);
        } else {
            M = mirror_gradmax(&s, &mk);
            mirror_update(&s, a, &mk, oracle_threshold_m2(M));
        }
        addsource32(&s, a->source, a->wavelet[k0 + k]);
        exchange32(&s);
        if (record) record32(&s, a->sz, record + (size_t)k * plane);
        if (uxyzmax) uxyzmax[k] = M;
    }
    free(s.ux); free(s.uy); free(s.uz); free(s.S); free(own);
    return 0;
}

static int run64(const oracle_args *a, int k0, int nsteps, double *u1,
                 double *u2, double *u3, double *pml_state, double *record,
                 double *uxyzmax)
{
    st64 s;
    int nx = a->nx, ny = a->ny, nz = a->nz, pml = a->pml;
    s.nx = nx; s.ny = ny; s.nz = nz; s.pml = pml;
    s.N = (size_t)nx * ny * nz;
    layout_init(&s.L, nx, ny, nz, pml);
    s.u1 = u1; s.u2 = u2; s.u3 = u3;
    s.ux = calloc(s.N, sizeof(double));
    s.uy = calloc(s.N, sizeof(double));
    s.uz = calloc(s.N, sizeof(double));
    s.S = calloc(s.N, sizeof(double));
    double *vp = malloc(s.N * sizeof(double)), *eps = malloc(s.N * sizeof(double)),
           *del = malloc(s.N * sizeof(double));
    double *own = NULL;
    if (!pml_state) own = pml_state = calloc(s.L.total + 1, sizeof(double));
    s.st = pml_state;
    int rc = 0;
    if (!s.ux || !s.uy || !s.uz || !s.S || !vp || !eps || !del || !pml_state) {
        rc = -2;
        goto out;
    }
    for (size_t i = 0; i < s.N; i++) {
        vp[i] = a->vp[i];
        eps[i] = a->epsilon[i];
        del[i] = a->delta[i];
    }
    double c[36], c2[36];
    for (int i = 0; i < 36; i++) { c[i] = a->c[i]; c2[i] = a->c2[i]; }
    size_t plane = (size_t)(nx - 2 * pml) * (ny - 2 * pml);
    int hy = ny - 2 * pml;
    for (int k = 0; k < nsteps; k++) {
        double M;
        f64_step(&s, a, c, c2, vp, eps, del, &M);
        if (a->source) {
            double w = a->wavelet[k0 + k];
            for (size_t i = 0; i < s.N; i++) s.u3[i] += (double)a->source[i] * w;
        }
        memcpy(s.u1, s.u2, s.N * sizeof(double));
        memcpy(s.u2, s.u3, s.N * sizeof(double));
        for (int f = 0; f < 6; f++) {
            size_t n = s.L.fsz[f];
            double *b = s.st;
            memcpy(b + s.L.off[f][W11], b + s.L.off[f][W12], n * sizeof(double));
            memcpy(b + s.L.off[f][W12], b + s.L.off[f][W13], n * sizeof(double));
            memcpy(b + s.L.off[f][W31], b + s.L.off[f][W32], n * sizeof(double));
            memcpy(b + s.L.off[f][W32], b + s.L.off[f][W33], n * sizeof(double));
            memcpy(b + s.L.off[f][P1], b + s.L.off[f][P2], n * sizeof(double));
            memcpy(b + s.L.off[f][P2], b + s.L.off[f][P3], n * sizeof(double));
        }
        if (record) {
            double *rec = record + (size_t)k * plane;
            for (int x = pml; x < nx - pml; x++)
                for (int y = pml; y < ny - pml; y++)
                    rec[(size_t)(x - pml) * hy + (y - pml)] = s.u2[IX(a->sz, x, y)];
        }
        if (uxyzmax) uxyzmax[k] = M;
    }
out:
    free(s.ux); free(s.uy); free(s.uz); free(s.S);
    free(vp); free(eps); free(del); free(own);
    return rc;
}

int oracle_run(int variant, const oracle_args *a, int k0, int nsteps,
               void *u1, void *u2, void *u3, void *pml_state, void *record,
               void *uxyzmax)
{
    if (!valid_args(a) || nsteps < 0 || k0 < 0 || !u1 || !u2 || !u3) return -1;
    int prev = set_threads(a->nthreads);
    int rc;
    if (variant == ORACLE_F64)
        rc = run64(a, k0, nsteps, u1, u2, u3, pml_state, record, uxyzmax);
    else if (variant == ORACLE_REF32 || variant == ORACLE_MIRROR)
        rc = run32(variant, a, k0, nsteps, u1, u2, u3, pml_state, record, uxyzmax);
    else
        rc = -1;
    set_threads(prev);
    return rc;
}
