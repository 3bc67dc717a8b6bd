/*
 * ref_harness.cpp -- drives the reference's own CPU operators.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled together with the reference's
 * CPU_function.c, straight from the reference checkout (oracle/build.py), into
 * oracle/_ref/libqp3d_ref.so.  The reference source is not copied.
 *
 * The shipped CPU driver (modeling3D.c:17-153) cannot be used as is: its
 * exchange() never sets its index (CPU_function.c:497), its buffers are not
 * zeroed (modeling3D.c:34-48) and several PML buffers are mis-sized
 * (modeling3D.c:38-45).  This harness keeps the reference's step sequence
 * (modeling3D.c:53-87) and operators unchanged and supplies what is missing:
 * zeroed buffers sized as 3dPureqPModeling_single_shot.cu:100-186 sizes them,
 * and the copy rotation of GPU_kernel.cu:733-812.  The reference exchange is
 * renamed at compile time (-Dexchange=...) so it is neither called nor linked
 * against the harness.
 *
 * The state buffers use the canonical layout of oracle/qp3d_oracle.h.
 */
#include <cstddef>
#include <cstdlib>
#include <cstring>

#include "CPU_function.h"   /* reference header, from the reference checkout */

namespace {

enum { FL = 0, FR, FF, FBK, FT, FBO };

struct Layout {
    size_t fsz[6];
    size_t off[6][10];
    size_t total;
};

void layout_init(Layout &L, int nx, int ny, int nz, int pml)
{
    size_t xf = (size_t)pml * ny * nz, yf = (size_t)pml * nx * nz,
           zf = (size_t)pml * nx * ny;
    size_t s[6] = {xf, xf, yf, yf, zf, zf};
    size_t o = 0;
    for (int f = 0; f < 6; f++) {
        L.fsz[f] = s[f];
        for (int a = 0; a < 10; a++) {
            L.off[f][a] = o;
            o += s[f];
        }
    }
    L.total = o;
}

}  // namespace

extern "C" size_t ref_pml_state_size(int nx, int ny, int nz, int pml)
{
    Layout L;
    layout_init(L, nx, ny, nz, pml);
    return L.total;
}

/* Same argument meaning as oracle_run() with variant ORACLE_REF32. */
extern "C" int ref_run(int nx, int ny, int nz, int pml, int sz, float dx,
                       float dy, float dz, float dt, const float *vp,
                       const float *epsilon, const float *delta,
                       const float *source, const float *wavelet,
                       const float *dlr, const float *ddlr, const float *dtb,
                       const float *ddtb, const float *dfb, const float *ddfb,
                       const float *c, const float *c2, int k0, int nsteps,
                       float *u1, float *u2, float *u3, float *pml_state,
                       float *record, float *uxyzmax)
{
    if (nx < 11 || ny < 11 || nz < 11 || pml < 0 || nsteps < 0) return -1;
    size_t N = (size_t)nx * ny * nz;
    Layout L;
    layout_init(L, nx, ny, nz, pml);
    float *ux = (float *)calloc(N, sizeof(float));
    float *uy = (float *)calloc(N, sizeof(float));
    float *uz = (float *)calloc(N, sizeof(float));
    float *S = (float *)calloc(N, sizeof(float));
    float *own = nullptr;
    if (!pml_state) own = pml_state = (float *)calloc(L.total + 1, sizeof(float));
    if (!ux || !uy || !uz || !S || !pml_state) {
        free(ux); free(uy); free(uz); free(S); free(own);
        return -2;
    }
    float *p[6][10];
    for (int f = 0; f < 6; f++)
        for (int a = 0; a < 10; a++) p[f][a] = pml_state + L.off[f][a];
    float *zero = (float *)calloc(N, sizeof(float));
    float *src = source ? const_cast<float *>(source) : zero;
    size_t plane = (size_t)(nx - 2 * pml) * (ny - 2 * pml);
    int hy = ny - 2 * pml;
    float *cc = const_cast<float *>(c), *cc2 = const_cast<float *>(c2);

    for (int k = 0; k < nsteps; k++) {
        /* modeling3D.c:53-59 */
        grad(u2, ux, uy, uz, cc, nx, ny, nz, dx, dy, dz);
        float uxMax = absMaxval(ux, nx, ny, nz);
        float uyMax = absMaxval(uy, nx, ny, nz);
        float uzMax = absMaxval(uz, nx, ny, nz);
        float uxyzMax = (uxMax > uyMax) ? uxMax : uyMax;
        uxyzMax = (uxyzMax > uzMax) ? uxyzMax : uzMax;
        /* modeling3D.c:63-73 */
        scalar_operator(uxyzMax, ux, uy, uz, const_cast<float *>(epsilon),
                        const_cast<float *>(delta), S, nx, ny, nz);
        wavefield_update(cc, cc2, const_cast<float *>(dlr), const_cast<float *>(ddlr),
                         const_cast<float *>(dtb), const_cast<float *>(ddtb),
                         const_cast<float *>(dfb), const_cast<float *>(ddfb),
                         const_cast<float *>(epsilon), const_cast<float *>(delta),
                         const_cast<float *>(vp), dx, dy, dz, dt, nx, ny, nz, pml, sz,
                         ux, uy, uz, u1, u3, u2, S,
                         p[FL][0], p[FL][1], p[FL][2], p[FL][3], p[FL][4], p[FL][5], p[FL][6], p[FL][7], p[FL][8], p[FL][9],
                         p[FR][0], p[FR][1], p[FR][2], p[FR][3], p[FR][4], p[FR][5], p[FR][6], p[FR][7], p[FR][8], p[FR][9],
                         p[FT][0], p[FT][1], p[FT][2], p[FT][3], p[FT][4], p[FT][5], p[FT][6], p[FT][7], p[FT][8], p[FT][9],
                         p[FBO][0], p[FBO][1], p[FBO][2], p[FBO][3], p[FBO][4], p[FBO][5], p[FBO][6], p[FBO][7], p[FBO][8], p[FBO][9],
                         p[FF][0], p[FF][1], p[FF][2], p[FF][3], p[FF][4], p[FF][5], p[FF][6], p[FF][7], p[FF][8], p[FF][9],
                         p[FBK][0], p[FBK][1], p[FBK][2], p[FBK][3], p[FBK][4], p[FBK][5], p[FBK][6], p[FBK][7], p[FBK][8], p[FBK][9]);
        addsource(src, wavelet[k0 + k], u3, nx, ny, nz);
        /* rotation as GPU_kernel.cu:748-809 (copies) */
        memcpy(u1, u2, N * sizeof(float));
        memcpy(u2, u3, N * sizeof(float));
        for (int f = 0; f < 6; f++) {
            size_t n = L.fsz[f] * sizeof(float);
            memcpy(p[f][0], p[f][1], n); memcpy(p[f][1], p[f][2], n);   /* w11<-w12<-w13 */
            memcpy(p[f][4], p[f][5], n); memcpy(p[f][5], p[f][6], n);   /* w31<-w32<-w33 */
            memcpy(p[f][7], p[f][8], n); memcpy(p[f][8], p[f][9], n);   /* p1<-p2<-p3 */
        }
        /* 3dPureqPModeling_single_shot.cu:333-337 */
        if (record) {
            float *rec = record + (size_t)k * plane;
            for (int x = pml; x < nx - pml; x++)
                for (int y = pml; y < ny - pml; y++)
                    rec[(size_t)(x - pml) * hy + (y - pml)] =
                        u2[(size_t)sz * nx * ny + (size_t)x * ny + y];
        }
        if (uxyzmax) uxyzmax[k] = uxyzMax;
    }
    free(ux); free(uy); free(uz); free(S); free(own); free(zero);
    return 0;
}

/* The reference's host utilities, exported for input-parity checks. */
extern "C" void ref_fdcoff(float *c, float *c2) { fdcoff1(c); fdcoff2(c2); }
extern "C" void ref_pmlcoff(int pml, float vpmax, float dx, float dy, float dz,
                            float *dlr, float *ddlr, float *dtb, float *ddtb,
                            float *dfb, float *ddfb)
{
    pmlcoff(pml, vpmax, dx, dy, dz, dlr, ddlr, dtb, ddtb, dfb, ddfb);
}
extern "C" void ref_source(int sx, int sy, int sz, float fm, float amp,
                           float alpha, float dt, float dx, float dy, float dz,
                           float t0, int nt, int nx, int ny, int nz,
                           float *source, float *wavelet)
{
    Source(sx, sy, sz, fm, amp, alpha, dt, dx, dy, dz, t0, nt, nx, ny, nz, source, wavelet);
}
extern "C" void ref_extend_model(float *in, float *out, int nx, int ny, int nz, int pml)
{
    extend_model(in, out, nx, ny, nz, pml);
}
extern "C" float ref_absmax(float *a, int nx, int ny, int nz) { return absMaxval(a, nx, ny, nz); }
