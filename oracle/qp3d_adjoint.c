/* qp3d_adjoint.c -- FP64 adjoint of the time-stepping loop (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the library's qp3d_adjoint, used
 * by tests/ and nothing else.
 *
 * The reference has no adjoint.  The operator differentiated here is the
 * reference's discrete step (CPU_function.c:301-480 in the F64 form of
 * qp3d_oracle.c) with the scalar operator S "frozen": per step and cell the
 * unit-normal factors a = nx^2 + ny^2 and b = nz^2 of a base run are fixed
 * (both 0 where the base run was below the threshold, so S = 1 there), and
 * S = 1/2 (1 + sqrt(1 - 8 (eps - delta) a b / (1 + 2 eps a)^2)) keeps its
 * dependence on eps and delta.  With S frozen the step is linear in the state
 *   s^k = (u^k, u^{k-1}, w1^k, w1^{k-1}, p^k, p^{k-1}, w21^k, w3^k, w3^{k-1})
 * (split-field PML state in shadow volumes), s^{k+1} = T_k(m) s^k + f^k, and
 * the record of step k is R u^{k+1}.  For J = 1/2 sum_k |R u^{k+1} - d_k|^2
 * the adjoint state runs backward, sigma^k = T_k^T (sigma^{k+1} + R^T r_k),
 * and dJ/dm = sum_k <sigma^{k+1} + R^T r_k, (dT_k/dm) s^k>.
 *
 * T_k^T is built exactly: every derivative the update takes of u^k (second
 * derivatives along x, y, z, first derivatives along the PML normal) is
 * multiplied by a per-cell coefficient; the adjoint collects those
 * coefficients times the adjoint of the updated quantity into six fields and
 * applies the transposed stencils (the same stencil for second derivatives,
 * its negative for first derivatives), and the PML recursions are transposed
 * term by term.  The gradient is reported on the cells outside the PML shell
 * (the shell's parameters are extensions of the interior edge and are held
 * fixed).
 *
 * With live = 1 the backward also differentiates S through the unit normal:
 * a = (Ux^2 + Uy^2)/s^2 and b = Uz^2/s^2 (s = |grad u| + 2.22e-17) depend on
 * the first derivatives of u^k, so every cell above the threshold adds
 * sigma dS/dU_c to the first-derivative fields (c = x, y, z), where sigma is
 * the adjoint weight of S in the cell's update (lambda K Lap in the
 * interior; the S-proportional terms of the split-field recursions in the
 * PML).  That is the gradient of the live forward (S recomputed from the
 * perturbed wavefield) except for the threshold decisions, which are
 * discontinuous and held.
 */
#include "qp3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#define R 5
#define EPSN 2.22e-17

#define IX(z, x, y) ((size_t)(z) * (size_t)nx * ny + (size_t)(x) * ny + (y))

enum { FL = 0, FR, FF, FBK, FT, FBO };

static inline int region_a(int z, int x, int y, int nx, int ny, int nz, int pml)
{
    if (x < pml) return FL;
    if (x >= nx - pml) return FR;
    if (y < pml) return FF;
    if (y >= ny - pml) return FBK;
    if (z < pml) return FT;
    if (z >= nz - pml) return FBO;
    return -1;
}

static inline int layer_a(int f, int z, int x, int y, int nx, int ny, int nz, int pml)
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

static inline int updated(int z, int x, int y, int nx, int ny, int nz)
{
    return x >= R && x < nx - R && y >= R && y < ny - R && z >= R && z < nz - R;
}

typedef struct {
    double cx[R + 1], c2x[R + 1], cy[R + 1], c2y[R + 1], cz[R + 1], c2z[R + 1];
} dcoef;

static void dcoef_init(dcoef *k, const oracle_adj_args *a)
{
    for (int m = 1; m <= R; m++) {
        k->cx[m] = a->c[30 + m] / a->dx;
        k->cy[m] = a->c[30 + m] / a->dy;
        k->cz[m] = a->c[30 + m] / a->dz;
        k->c2x[m] = a->c2[30 + m] / (a->dx * a->dx);
        k->c2y[m] = a->c2[30 + m] / (a->dy * a->dy);
        k->c2z[m] = a->c2[30 + m] / (a->dz * a->dz);
    }
}

/* derivatives of u at an updated cell (F64 forms of CPU_function.c:301-324, 371-400) */
static inline void derivs(const double *u, int z, int x, int y, int nx, int ny,
                          const dcoef *k, double d[6])
{
    size_t i = IX(z, x, y);
    double Ux = 0, Uy = 0, Uz = 0, Uxx = 0, Uyy = 0, Uzz = 0;
    for (int m = 1; m <= R; m++) {
        double xp = u[IX(z, x + m, y)], xm = u[IX(z, x - m, y)];
        double yp = u[IX(z, x, y + m)], ym = u[IX(z, x, y - m)];
        double zp = u[IX(z + m, x, y)], zm = u[IX(z - m, x, y)];
        Ux += k->cx[m] * (xp - xm);
        Uy += k->cy[m] * (yp - ym);
        Uz += k->cz[m] * (zp - zm);
        Uxx += k->c2x[m] * (xp - 2 * u[i] + xm);
        Uyy += k->c2y[m] * (yp - 2 * u[i] + ym);
        Uzz += k->c2z[m] * (zp - 2 * u[i] + zm);
    }
    d[0] = Ux; d[1] = Uy; d[2] = Uz; d[3] = Uxx; d[4] = Uyy; d[5] = Uzz;
}

/* frozen S and its derivatives in eps, delta */
static inline void frozen_s(double a, double b, double e, double dl, double *S, double *dSe,
                            double *dSd)
{
    double D = 1 + 2 * e * a;
    double q = 8 * (e - dl) * a * b / (D * D);
    double r = sqrt(1 - q);
    *S = 0.5 * (1 + r);
    if (dSe) {
        double dq_de = 8 * a * b / (D * D) * (1 - 4 * a * (e - dl) / D);
        double dq_dd = -8 * a * b / (D * D);
        double dS_dq = (a * b != 0.0) ? -0.25 / r : 0.0;
        *dSe = dS_dq * dq_de;
        *dSd = dS_dq * dq_dd;
    }
}

/* dS/dUx, dS/dUy, dS/dUz of an above-threshold cell: S of frozen_s through
 * a = (Ux^2 + Uy^2)/s^2 and b = Uz^2/s^2, s = |grad u| + EPSN (the forms of
 * step_fwd). */
static inline void s_grad(const double d[6], double e, double dl, double g[3])
{
    double h2 = d[0] * d[0] + d[1] * d[1], v2 = d[2] * d[2];
    double mode = sqrt(h2 + v2), s = mode + EPSN;
    double a = h2 / (s * s), b = v2 / (s * s);
    double D = 1 + 2 * e * a, R8 = 8 * (e - dl);
    double q = R8 * a * b / (D * D), r = sqrt(1 - q);
    double dSdq = -0.25 / r;
    double dqa = R8 * b * (D - 4 * e * a) / (D * D * D), dqb = R8 * a / (D * D);
    for (int c = 0; c < 3; c++) {
        double common = d[c] / (mode * s * s * s);
        double ac = (c < 2 ? 2 * d[c] / (s * s) : 0.0) - 2 * h2 * common;
        double bc = (c == 2 ? 2 * d[c] / (s * s) : 0.0) - 2 * v2 * common;
        g[c] = dSdq * (dqa * ac + dqb * bc);
    }
}

typedef struct {
    double A, At, dd, sgn, a1, a2, a3;
    int f;
} pml_coef;

static inline void pml_cell_coef(const oracle_adj_args *a, int f, int li, double S, double e,
                                 double v, pml_coef *c)
{
    double dt = a->dt, vdt2 = (v * dt) * (v * dt), e2 = 1 + 2 * e;
    const float *dp, *ddp;
    if (f == FL || f == FR) {
        c->A = e2 * S * vdt2; c->At = S * vdt2; dp = a->dlr; ddp = a->ddlr;
    } else if (f == FF || f == FBK) {
        c->A = e2 * S * vdt2; c->At = S * vdt2; dp = a->dfb; ddp = a->ddfb;
    } else {
        c->A = S * vdt2; c->At = e2 * S * vdt2; dp = a->dtb; ddp = a->ddtb;
    }
    double d = dp[li], b = d * dt + 1;
    c->dd = ddp[li];
    c->a1 = b * b - 3;           /* w1' = A Unn - a1 w1 + a2 w1o */
    c->a2 = 2 * d * dt - 1;
    c->a3 = 1 - dt * d;
    c->sgn = (f == FR || f == FBK || f == FBO) ? -1.0 : 1.0;
    c->f = f;
}

typedef struct {
    double *u, *up, *w1, *w1o, *p, *po, *w21, *w3, *w3o;
} state;

static int state_alloc(state *s, size_t N)
{
    double **v[] = {&s->u, &s->up, &s->w1, &s->w1o, &s->p, &s->po, &s->w21, &s->w3, &s->w3o};
    int ok = 1;
    for (int i = 0; i < 9; i++) {
        *v[i] = calloc(N, sizeof(double));
        ok = ok && *v[i];
    }
    return ok;
}

static void state_free(state *s)
{
    double *v[] = {s->u, s->up, s->w1, s->w1o, s->p, s->po, s->w21, s->w3, s->w3o};
    for (int i = 0; i < 9; i++) free(v[i]);
}

static int valid(const oracle_adj_args *a)
{
    if (!a || !a->vp || !a->eps || !a->del || !a->wavelet || !a->c || !a->c2) return 0;
    if (a->nx < 11 || a->ny < 11 || a->nz < 11 || a->pml < 0 || a->nt < 1) return 0;
    if (2 * a->pml > a->nx || 2 * a->pml > a->ny || 2 * a->pml > a->nz) return 0;
    if (a->pml > 0 && (!a->dlr || !a->ddlr || !a->dtb || !a->ddtb || !a->dfb || !a->ddfb))
        return 0;
    return a->sz >= 0 && a->sz < a->nz;
}

/* One forward step from s (u^k ...) into n (u^{k+1} ...).  fa/fb: frozen
 * factors of this step, or NULL for the live S (recorded into rec_a/rec_b). */
static void step_fwd(const oracle_adj_args *a, const dcoef *kc, const state *s, state *n,
                     const double *fa, const double *fb, double *rec_a, double *rec_b,
                     double w, const double *extra)
{
    int nx = a->nx, ny = a->ny, nz = a->nz, pml = a->pml;
    size_t N = (size_t)nx * ny * nz;
    double dt = a->dt;
    double M = 0.0;
    if (!fa) {   /* live S: the max over the updated box first */
#pragma omp parallel for reduction(max : M) schedule(static)
        for (int z = R; z < nz - R; z++)
            for (int x = R; x < nx - R; x++)
                for (int y = R; y < ny - R; y++) {
                    double d[6];
                    derivs(s->u, z, x, y, nx, ny, kc, d);
                    double v = fmax(fabs(d[0]), fmax(fabs(d[1]), fabs(d[2])));
                    if (v > M) M = v;
                }
    }
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++) {
                size_t i = IX(z, x, y);
                double un;
                n->w1[i] = n->w1o[i] = n->p[i] = n->po[i] = 0;
                n->w21[i] = n->w3[i] = n->w3o[i] = 0;
                if (!updated(z, x, y, nx, ny, nz)) {
                    un = s->u[i];
                } else {
                    double d[6];
                    derivs(s->u, z, x, y, nx, ny, kc, d);
                    double A_, B_;
                    if (fa) {
                        A_ = fa[i];
                        B_ = fb[i];
                    } else {
                        double mode = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                        double nxv = 0, nyv = 0, nzv = 0;
                        if (mode > 1.0e-02 * M) {
                            nxv = d[0] / (mode + EPSN);
                            nyv = d[1] / (mode + EPSN);
                            nzv = d[2] / (mode + EPSN);
                        }
                        A_ = nxv * nxv + nyv * nyv;
                        B_ = nzv * nzv;
                        if (rec_a) { rec_a[i] = A_; rec_b[i] = B_; }
                    }
                    double e = a->eps[i], dl = a->del[i], v = a->vp[i], S;
                    frozen_s(A_, B_, e, dl, &S, NULL, NULL);
                    int f = region_a(z, x, y, nx, ny, nz, pml);
                    if (f < 0) {
                        double K = (v * dt) * (v * dt);
                        un = 2 * s->u[i] - s->up[i] +
                             K * S * ((1 + 2 * e) * (d[3] + d[4]) + d[5]);
                    } else {
                        pml_coef c;
                        pml_cell_coef(a, f, layer_a(f, z, x, y, nx, ny, nz, pml), S, e, v, &c);
                        double Unn, Un, tang, e2 = 1 + 2 * e;
                        if (f <= FR) { Unn = d[3]; Un = d[0]; tang = d[5] + e2 * d[4]; }
                        else if (f <= FBK) { Unn = d[4]; Un = d[1]; tang = d[5] + e2 * d[3]; }
                        else { Unn = d[5]; Un = d[2]; tang = d[3] + d[4]; }
                        double w1n = c.A * Unn - c.a1 * s->w1[i] + c.a2 * s->w1o[i];
                        double pn = -c.a1 * s->p[i] + c.a2 * s->po[i] + c.sgn * c.A * c.dd * Un;
                        double w21n = dt * pn + c.a3 * s->w21[i];
                        double w3n = c.At * tang + 2 * s->w3[i] - s->w3o[i];
                        n->w1[i] = w1n; n->w1o[i] = s->w1[i];
                        n->p[i] = pn; n->po[i] = s->p[i];
                        n->w21[i] = w21n;
                        n->w3[i] = w3n; n->w3o[i] = s->w3[i];
                        un = w1n + w21n + w3n;
                    }
                }
                if (a->source) un += (double)a->source[i] * w;
                if (extra) un += extra[i];
                n->u[i] = un;
                n->up[i] = s->u[i];
            }
    (void)N;
}

static void record_plane(const oracle_adj_args *a, const double *u, double *rec)
{
    int nx = a->nx, ny = a->ny, pml = a->pml, hy = ny - 2 * pml;
    for (int x = pml; x < nx - pml; x++)
        for (int y = pml; y < ny - pml; y++)
            rec[(size_t)(x - pml) * hy + (y - pml)] = u[IX(a->sz, x, y)];
}

static void swap_state(state *a, state *b)
{
    state t = *a;
    *a = *b;
    *b = t;
}

int oracle_adj_freeze(const oracle_adj_args *a, double *fa, double *fb)
{
    if (!valid(a) || !fa || !fb) return -1;
    size_t N = (size_t)a->nx * a->ny * a->nz;
    int prev = omp_get_max_threads();
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
    dcoef kc;
    dcoef_init(&kc, a);
    state s, n;
    int rc = 0;
    if (!state_alloc(&s, N) || !state_alloc(&n, N)) {
        rc = -2;
        goto out;
    }
    for (int k = 0; k < a->nt; k++) {
        memset(fa + (size_t)k * N, 0, N * sizeof(double));
        memset(fb + (size_t)k * N, 0, N * sizeof(double));
        step_fwd(a, &kc, &s, &n, NULL, NULL, fa + (size_t)k * N, fb + (size_t)k * N,
                 a->wavelet[k], NULL);
        swap_state(&s, &n);
    }
out:
    state_free(&s);
    state_free(&n);
    omp_set_num_threads(prev);
    return rc;
}

int oracle_adj_forward(const oracle_adj_args *a, const double *fa, const double *fb,
                       const double *extra, double *record, double *u_hist)
{
    if (!valid(a) || !fa || !fb) return -1;
    size_t N = (size_t)a->nx * a->ny * a->nz;
    size_t plane = (size_t)(a->nx - 2 * a->pml) * (a->ny - 2 * a->pml);
    int prev = omp_get_max_threads();
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
    dcoef kc;
    dcoef_init(&kc, a);
    state s, n;
    int rc = 0;
    if (!state_alloc(&s, N) || !state_alloc(&n, N)) {
        rc = -2;
        goto out;
    }
    for (int k = 0; k < a->nt; k++) {
        if (u_hist) memcpy(u_hist + (size_t)k * N, s.u, N * sizeof(double));
        step_fwd(a, &kc, &s, &n, fa + (size_t)k * N, fb + (size_t)k * N, NULL, NULL,
                 a->wavelet[k], extra ? extra + (size_t)k * N : NULL);
        swap_state(&s, &n);
        if (record) record_plane(a, s.u, record + (size_t)k * plane);
    }
out:
    state_free(&s);
    state_free(&n);
    omp_set_num_threads(prev);
    return rc;
}

/* One tangent-linear step about the base wavefield ub = u^k: the frozen step
 * of the perturbation s (no source: it does not depend on the state) plus,
 * with live, the perturbation of S through the unit normal, dS = sum_c
 * dS/dU_c (base) D_c du, times the S-proportional terms of the base update. */
static void tlm_step(const oracle_adj_args *a, const dcoef *kc, const state *s, state *n,
                     const double *fa, const double *fb, const double *ub, const double *extra)
{
    int nx = a->nx, ny = a->ny, nz = a->nz, pml = a->pml;
    double dt = a->dt;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++) {
                size_t i = IX(z, x, y);
                double un;
                n->w1[i] = n->w1o[i] = n->p[i] = n->po[i] = 0;
                n->w21[i] = n->w3[i] = n->w3o[i] = 0;
                if (!updated(z, x, y, nx, ny, nz)) {
                    un = s->u[i];
                } else {
                    double d[6], db[6], gs[3], dS = 0.0;
                    derivs(s->u, z, x, y, nx, ny, kc, d);
                    derivs(ub, z, x, y, nx, ny, kc, db);
                    double e = a->eps[i], dl = a->del[i], v = a->vp[i], S;
                    frozen_s(fa[i], fb[i], e, dl, &S, NULL, NULL);
                    int live_on = a->live && (fa[i] != 0.0 || fb[i] != 0.0);
                    if (live_on) {
                        s_grad(db, e, dl, gs);
                        dS = gs[0] * d[0] + gs[1] * d[1] + gs[2] * d[2];
                    }
                    int f = region_a(z, x, y, nx, ny, nz, pml);
                    double e2 = 1 + 2 * e;
                    if (f < 0) {
                        double K = (v * dt) * (v * dt);
                        un = 2 * s->u[i] - s->up[i] + K * S * (e2 * (d[3] + d[4]) + d[5]);
                        if (live_on) un += K * (e2 * (db[3] + db[4]) + db[5]) * dS;
                    } else {
                        pml_coef c;
                        pml_cell_coef(a, f, layer_a(f, z, x, y, nx, ny, nz, pml), S, e, v, &c);
                        double Unn, Un, tang, Unb, Ub, tb;
                        if (f <= FR) {
                            Unn = d[3]; Un = d[0]; tang = d[5] + e2 * d[4];
                            Unb = db[3]; Ub = db[0]; tb = db[5] + e2 * db[4];
                        } else if (f <= FBK) {
                            Unn = d[4]; Un = d[1]; tang = d[5] + e2 * d[3];
                            Unb = db[4]; Ub = db[1]; tb = db[5] + e2 * db[3];
                        } else {
                            Unn = d[5]; Un = d[2]; tang = d[3] + d[4];
                            Unb = db[5]; Ub = db[2]; tb = db[3] + db[4];
                        }
                        double w1n = c.A * Unn - c.a1 * s->w1[i] + c.a2 * s->w1o[i];
                        double pn = -c.a1 * s->p[i] + c.a2 * s->po[i] + c.sgn * c.A * c.dd * Un;
                        double w3n = c.At * tang + 2 * s->w3[i] - s->w3o[i];
                        if (live_on) {   /* A and At are proportional to S */
                            w1n += c.A / S * Unb * dS;
                            pn += c.sgn * c.A / S * c.dd * Ub * dS;
                            w3n += c.At / S * tb * dS;
                        }
                        double w21n = dt * pn + c.a3 * s->w21[i];
                        n->w1[i] = w1n; n->w1o[i] = s->w1[i];
                        n->p[i] = pn; n->po[i] = s->p[i];
                        n->w21[i] = w21n;
                        n->w3[i] = w3n; n->w3o[i] = s->w3[i];
                        un = w1n + w21n + w3n;
                    }
                }
                if (extra) un += extra[i];
                n->u[i] = un;
                n->up[i] = s->u[i];
            }
}

int oracle_adj_tlm(const oracle_adj_args *a, const double *fa, const double *fb,
                   const double *u_hist, const double *extra, double *record)
{
    if (!valid(a) || !fa || !fb || !u_hist || !record) return -1;
    size_t N = (size_t)a->nx * a->ny * a->nz;
    size_t plane = (size_t)(a->nx - 2 * a->pml) * (a->ny - 2 * a->pml);
    int prev = omp_get_max_threads();
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
    dcoef kc;
    dcoef_init(&kc, a);
    state s, n;
    int rc = 0;
    if (!state_alloc(&s, N) || !state_alloc(&n, N)) {
        rc = -2;
        goto out;
    }
    for (int k = 0; k < a->nt; k++) {
        tlm_step(a, &kc, &s, &n, fa + (size_t)k * N, fb + (size_t)k * N, u_hist + (size_t)k * N,
                 extra ? extra + (size_t)k * N : NULL);
        swap_state(&s, &n);
        record_plane(a, s.u, record + (size_t)k * plane);
    }
out:
    state_free(&s);
    state_free(&n);
    omp_set_num_threads(prev);
    return rc;
}

int oracle_adj_backward(const oracle_adj_args *a, const double *fa, const double *fb,
                        const double *u_hist, const double *resid, double *g_vp,
                        double *g_eps, double *g_del, double *f_adj)
{
    if (!valid(a) || !fa || !fb || !u_hist || !resid) return -1;
    int nx = a->nx, ny = a->ny, nz = a->nz, pml = a->pml, hy = ny - 2 * pml;
    size_t N = (size_t)nx * ny * nz;
    size_t plane = (size_t)(nx - 2 * pml) * (ny - 2 * pml);
    double dt = a->dt;
    int prev = omp_get_max_threads();
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
    dcoef kc;
    dcoef_init(&kc, a);
    state L, NL;
    double *C[6], *gK = calloc(N, sizeof(double)), *ge = calloc(N, sizeof(double)),
           *gd = calloc(N, sizeof(double)), *lam = calloc(N, sizeof(double));
    int rc = 0, ok = state_alloc(&L, N) && state_alloc(&NL, N) && gK && ge && gd && lam;
    for (int i = 0; i < 6; i++) {
        C[i] = calloc(N, sizeof(double));
        ok = ok && C[i];
    }
    if (!ok) {
        rc = -2;
        goto out;
    }
    for (int k = a->nt - 1; k >= 0; k--) {
        const double *u = u_hist + (size_t)k * N;
        const double *Fa = fa + (size_t)k * N, *Fb = fb + (size_t)k * N;
        const double *rk = resid + (size_t)k * plane;
        /* lambda = adjoint of u^{k+1}, with the record misfit injected */
        memcpy(lam, L.u, N * sizeof(double));
        for (int x = pml; x < nx - pml; x++)
            for (int y = pml; y < ny - pml; y++)
                lam[IX(a->sz, x, y)] += rk[(size_t)(x - pml) * hy + (y - pml)];
        if (f_adj) memcpy(f_adj + (size_t)k * N, lam, N * sizeof(double));
        for (int i = 0; i < 6; i++) memset(C[i], 0, N * sizeof(double));
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; z++)
            for (int x = 0; x < nx; x++)
                for (int y = 0; y < ny; y++) {
                    size_t i = IX(z, x, y);
                    double l = lam[i];
                    NL.u[i] = L.up[i];      /* s^{k+1}.up is u^k */
                    NL.up[i] = 0;
                    NL.w1[i] = NL.w1o[i] = NL.p[i] = NL.po[i] = 0;
                    NL.w21[i] = NL.w3[i] = NL.w3o[i] = 0;
                    if (!updated(z, x, y, nx, ny, nz)) {
                        NL.u[i] += l;       /* never-updated cell: u^{k+1} = u^k */
                        continue;
                    }
                    double e = a->eps[i], dl = a->del[i], v = a->vp[i], S, dSe, dSd;
                    frozen_s(Fa[i], Fb[i], e, dl, &S, &dSe, &dSd);
                    double e2 = 1 + 2 * e, K = (v * dt) * (v * dt);
                    int f = region_a(z, x, y, nx, ny, nz, pml);
                    if (f < 0) {
                        NL.u[i] += 2 * l;
                        NL.up[i] = -l;
                        C[3][i] = K * S * e2 * l;
                        C[4][i] = K * S * e2 * l;
                        C[5][i] = K * S * l;
                        /* gradient: lambda (dT/dm) s^k */
                        double d[6];
                        derivs(u, z, x, y, nx, ny, &kc, d);
                        double Lap = e2 * (d[3] + d[4]) + d[5];
                        if (a->live && (Fa[i] != 0.0 || Fb[i] != 0.0)) {
                            double gs[3], sig = l * K * Lap;
                            s_grad(d, e, dl, gs);
                            C[0][i] += sig * gs[0];
                            C[1][i] += sig * gs[1];
                            C[2][i] += sig * gs[2];
                        }
                        gK[i] += l * S * Lap;
                        ge[i] += l * K * (2 * S * (d[3] + d[4]) + dSe * Lap);
                        gd[i] += l * K * dSd * Lap;
                        continue;
                    }
                    pml_coef c;
                    pml_cell_coef(a, f, layer_a(f, z, x, y, nx, ny, nz, pml), S, e, v, &c);
                    double W1 = L.w1[i] + l, W21 = L.w21[i] + l, W3 = L.w3[i] + l;
                    double P = L.p[i] + dt * W21;
                    NL.w1[i] = -c.a1 * W1 + L.w1o[i];
                    NL.w1o[i] = c.a2 * W1;
                    NL.p[i] = -c.a1 * P + L.po[i];
                    NL.po[i] = c.a2 * P;
                    NL.w21[i] = c.a3 * W21;
                    NL.w3[i] = 2 * W3 + L.w3o[i];
                    NL.w3o[i] = -W3;
                    double cn = c.A * W1, c1 = c.sgn * c.A * c.dd * P, ct = c.At * W3;
                    if (f <= FR) { C[3][i] += cn; C[0][i] += c1; C[4][i] += ct * e2; C[5][i] += ct; }
                    else if (f <= FBK) { C[4][i] += cn; C[1][i] += c1; C[3][i] += ct * e2; C[5][i] += ct; }
                    else { C[5][i] += cn; C[2][i] += c1; C[3][i] += ct; C[4][i] += ct; }
                    if (a->live && (Fa[i] != 0.0 || Fb[i] != 0.0)) {
                        /* the S-proportional terms of w1', p' and w3' */
                        double d[6], gs[3], Unn, Un, tang;
                        derivs(u, z, x, y, nx, ny, &kc, d);
                        if (f <= FR) { Unn = d[3]; Un = d[0]; tang = d[5] + e2 * d[4]; }
                        else if (f <= FBK) { Unn = d[4]; Un = d[1]; tang = d[5] + e2 * d[3]; }
                        else { Unn = d[5]; Un = d[2]; tang = d[3] + d[4]; }
                        double sig = (cn * Unn + c1 * Un + ct * tang) / S;
                        s_grad(d, e, dl, gs);
                        C[0][i] += sig * gs[0];
                        C[1][i] += sig * gs[1];
                        C[2][i] += sig * gs[2];
                    }
                }
        /* transposed stencils: second derivatives symmetric, first antisymmetric */
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; z++)
            for (int x = 0; x < nx; x++)
                for (int y = 0; y < ny; y++) {
                    size_t i = IX(z, x, y);
                    double acc = 0;
                    for (int m = 1; m <= R; m++) {
                        double sxx = 0, syy = 0, szz = 0, sx = 0, sy = 0, sz = 0;
                        if (x + m < nx) { sxx += C[3][IX(z, x + m, y)]; sx -= C[0][IX(z, x + m, y)]; }
                        if (x - m >= 0) { sxx += C[3][IX(z, x - m, y)]; sx += C[0][IX(z, x - m, y)]; }
                        if (y + m < ny) { syy += C[4][IX(z, x, y + m)]; sy -= C[1][IX(z, x, y + m)]; }
                        if (y - m >= 0) { syy += C[4][IX(z, x, y - m)]; sy += C[1][IX(z, x, y - m)]; }
                        if (z + m < nz) { szz += C[5][IX(z + m, x, y)]; sz -= C[2][IX(z + m, x, y)]; }
                        if (z - m >= 0) { szz += C[5][IX(z - m, x, y)]; sz += C[2][IX(z - m, x, y)]; }
                        acc += kc.c2x[m] * (sxx - 2 * C[3][i]) + kc.c2y[m] * (syy - 2 * C[4][i]) +
                               kc.c2z[m] * (szz - 2 * C[5][i]) + kc.cx[m] * sx + kc.cy[m] * sy +
                               kc.cz[m] * sz;
                    }
                    NL.u[i] += acc;
                }
        swap_state(&L, &NL);
    }
    for (size_t i = 0; i < N; i++) {
        int z = (int)(i / ((size_t)nx * ny)), x = (int)(i / ny % nx), y = (int)(i % ny);
        int inside = x >= pml && x < nx - pml && y >= pml && y < ny - pml && z >= pml &&
                     z < nz - pml;
        double v = a->vp[i];
        if (g_vp) g_vp[i] = inside ? gK[i] * 2 * v * dt * dt : 0.0;
        if (g_eps) g_eps[i] = inside ? ge[i] : 0.0;
        if (g_del) g_del[i] = inside ? gd[i] : 0.0;
    }
out:
    state_free(&L);
    state_free(&NL);
    for (int i = 0; i < 6; i++) free(C[i]);
    free(gK); free(ge); free(gd); free(lam);
    omp_set_num_threads(prev);
    return rc;
}
