// exact_emul.cpp -- the library's exact-arithmetic header (csrc/qp3d_exact.h)
// compiled for the CPU and run as a whole time loop, so that the tests can
// compare it with the oracle's restatement of the reference operators bit
// for bit.  Test code: built by tests/test_exact_arith.py.
//
// The loop has the structure of the reference's per-step sequence
// (grad -> max -> scalar_operator -> wavefield_update -> addsource ->
// exchange -> record) and the oracle's data layout (qp3d_oracle.h); all
// arithmetic comes from the header.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "qp3d_exact.h"
#include "qp3d_oracle.h"

using namespace qp3d::xr;

namespace {

struct Counts {
    long long s_fp64, unit_fp64, pml_fp64, s_cells, pml_cells;
};

inline size_t IX(int z, int x, int y, int nx, int ny)
{
    return (size_t)z * nx * ny + (size_t)x * ny + y;
}

float threshold_f(float m)
{   // largest float not above 0.01 * (double)m
    double td = 1.0e-02 * (double)m;
    float t = (float)td;
    if ((double)t > td) t = nextafterf(t, -INFINITY);
    return t;
}

}  // namespace

extern "C" int emul_run(const oracle_args *a, int k0, int nsteps, float *u1, float *u2,
                        float *u3, float *st, float *record, float *uxyzmax, long long *counts)
{
    const int nx = a->nx, ny = a->ny, nz = a->nz, pml = a->pml;
    const size_t N = (size_t)nx * ny * nz;
    std::vector<float> ux(N, 0.0f), uy(N, 0.0f), uz(N, 0.0f), S(N, 1.0f);
    const size_t fs[6] = {(size_t)pml * ny * nz, (size_t)pml * ny * nz, (size_t)pml * nx * nz,
                          (size_t)pml * nx * nz, (size_t)pml * nx * ny, (size_t)pml * nx * ny};
    size_t off[6][10], o = 0;
    for (int f = 0; f < 6; ++f)
        for (int j = 0; j < 10; ++j) {
            off[f][j] = o;
            o += fs[f];
        }
    const float dx = a->dx, dy = a->dy, dz = a->dz, dt = a->dt;
    const float hx = dx, hy = dy, hz = dz;
    const float hx2 = dx * dx, hy2 = dy * dy, hz2 = dz * dz;
    const float *c = a->c + 31, *c2 = a->c2 + 31;
    const float dt2 = dt * dt;
    Counts cnt{};
    const size_t plane = (size_t)(nx - 2 * pml) * (ny - 2 * pml);
    const float *dprof[3] = {a->dlr, a->dfb, a->dtb}, *ddprof[3] = {a->ddlr, a->ddfb, a->ddtb};

    for (int k = 0; k < nsteps; ++k) {
        // grad over [5, n-5)^3 (the rest stays zero)
#pragma omp parallel for schedule(static)
        for (int z = 5; z < nz - 5; ++z)
            for (int x = 5; x < nx - 5; ++x)
                for (int y = 5; y < ny - 5; ++y) {
                    float A[5], B[5];
                    for (int m = 0; m < 5; ++m) {
                        A[m] = u2[IX(z, x + m + 1, y, nx, ny)];
                        B[m] = u2[IX(z, x - m - 1, y, nx, ny)];
                    }
                    const size_t i = IX(z, x, y, nx, ny);
                    ux[i] = grad_axis(A, B, c, hx);
                    for (int m = 0; m < 5; ++m) {
                        A[m] = u2[i + m + 1];
                        B[m] = u2[i - m - 1];
                    }
                    uy[i] = grad_axis(A, B, c, hy);
                    for (int m = 0; m < 5; ++m) {
                        A[m] = u2[IX(z + m + 1, x, y, nx, ny)];
                        B[m] = u2[IX(z - m - 1, x, y, nx, ny)];
                    }
                    uz[i] = grad_axis(A, B, c, hz);
                }
        float M = 0.0f;
        for (size_t i = 0; i < N; ++i)
            M = fmaxf(M, fmaxf(fabsf(ux[i]), fmaxf(fabsf(uy[i]), fabsf(uz[i]))));
        const float Tf = threshold_f(M);
        long long s64 = 0, u64 = 0, scells = 0, p64 = 0, pcells = 0;
        // scalar operator
#pragma omp parallel for schedule(static) reduction(+ : s64, u64, scells)
        for (int z = 5; z < nz - 5; ++z)
            for (int x = 5; x < nx - 5; ++x)
                for (int y = 5; y < ny - 5; ++y) {
                    const size_t i = IX(z, x, y, nx, ny);
                    const float m2 = grad_m2(ux[i], uy[i], uz[i]);
                    // (double)sqrtf(m2) > 0.01 * (double)M  <=>  sqrtf(m2) > Tf
                    if (!(sqrt_ieee(m2) > Tf)) {
                        S[i] = 1.0f;
                        continue;
                    }
                    const float e = a->epsilon[i], d = a->delta[i];
                    S[i] = scalar_s(ux[i], uy[i], uz[i], m2, mul(2.0f, e), mul(8.0f, sub(e, d)));
                    ++scells;
                }
        // update
#pragma omp parallel for schedule(static) reduction(+ : p64, pcells)
        for (int z = 5; z < nz - 5; ++z)
            for (int x = 5; x < nx - 5; ++x)
                for (int y = 5; y < ny - 5; ++y) {
                    const size_t i = IX(z, x, y, nx, ny);
                    float A[5], B[5];
                    const float u0 = u2[i];
                    for (int m = 0; m < 5; ++m) {
                        A[m] = u2[IX(z, x + m + 1, y, nx, ny)];
                        B[m] = u2[IX(z, x - m - 1, y, nx, ny)];
                    }
                    const float Uxx = lap_axis(A, B, u0, c2, hx2);
                    for (int m = 0; m < 5; ++m) {
                        A[m] = u2[i + m + 1];
                        B[m] = u2[i - m - 1];
                    }
                    const float Uyy = lap_axis(A, B, u0, c2, hy2);
                    for (int m = 0; m < 5; ++m) {
                        A[m] = u2[IX(z + m + 1, x, y, nx, ny)];
                        B[m] = u2[IX(z - m - 1, x, y, nx, ny)];
                    }
                    const float Uzz = lap_axis(A, B, u0, c2, hz2);
                    const float e1 = add(1.0f, mul(2.0f, a->epsilon[i]));
                    const bool inner = x >= pml && x < nx - pml && y >= pml && y < ny - pml &&
                                       z >= pml && z < nz - pml;
                    if (inner) {
                        u3[i] = interior_update(u0, u1[i], Uxx, Uyy, Uzz, e1, S[i], a->vp[i], dt2);
                        continue;
                    }
                    int f, li, axis;
                    size_t fi;
                    if (x < pml) { f = 0; li = pml - x; axis = 0; fi = (size_t)z * ny * pml + (size_t)x * ny + y; }
                    else if (x >= nx - pml) { f = 1; li = x - nx + pml; axis = 0; fi = (size_t)z * ny * pml + (size_t)(x - nx + pml) * ny + y; }
                    else if (y < pml) { f = 2; li = pml - y; axis = 1; fi = (size_t)z * nx * pml + (size_t)x * pml + y; }
                    else if (y >= ny - pml) { f = 3; li = y - ny + pml; axis = 1; fi = (size_t)z * nx * pml + (size_t)x * pml + (y - ny + pml); }
                    else if (z < pml) { f = 4; li = pml - z; axis = 2; fi = (size_t)z * nx * ny + (size_t)x * ny + y; }
                    else { f = 5; li = z - nz + pml; axis = 2; fi = (size_t)(z - nz + pml) * ny * nx + (size_t)x * ny + y; }
                    const PmlLayer L = pml_layer(dprof[axis][li], ddprof[axis][li], dt);
                    const float Unn = axis == 0 ? Uxx : (axis == 1 ? Uyy : Uzz);
                    const float Un = axis == 0 ? ux[i] : (axis == 1 ? uy[i] : uz[i]);
                    const float tang = axis == 0 ? add(Uzz, mul(e1, Uyy))
                                     : (axis == 1 ? add(Uzz, mul(e1, Uxx)) : add(Uxx, Uyy));
                    const float vdt = mul(a->vp[i], dt);
                    float *w11 = st + off[f][0], *w12 = st + off[f][1], *w13 = st + off[f][2],
                          *w21 = st + off[f][3], *w31 = st + off[f][4], *w32 = st + off[f][5],
                          *w33 = st + off[f][6], *p1 = st + off[f][7], *p2 = st + off[f][8],
                          *p3 = st + off[f][9];
                    PmlOut r = pml_update(axis == 2, (f & 1) != 0, S[i], e1, vdt, Unn, Un, tang, dt,
                                          L, w11[fi], w12[fi], w21[fi], w31[fi], w32[fi], p1[fi],
                                          p2[fi]);
                    w13[fi] = r.w13;
                    p3[fi] = r.p3;
                    w21[fi] = r.w21;
                    w33[fi] = r.w33;
                    u3[i] = r.u3;
                    ++pcells;
                }
        // addsource (CPU_function.c:326-338) on every cell
        const float w = a->wavelet[k0 + k];
        if (a->source)
            for (size_t i = 0; i < N; ++i) u3[i] += a->source[i] * w;
        // exchange (GPU_kernel.cu:733-812): copy rotation of u and the levels
        memcpy(u1, u2, N * sizeof(float));
        memcpy(u2, u3, N * sizeof(float));
        for (int f = 0; f < 6; ++f) {
            memcpy(st + off[f][0], st + off[f][1], fs[f] * sizeof(float));
            memcpy(st + off[f][1], st + off[f][2], fs[f] * sizeof(float));
            memcpy(st + off[f][4], st + off[f][5], fs[f] * sizeof(float));
            memcpy(st + off[f][5], st + off[f][6], fs[f] * sizeof(float));
            memcpy(st + off[f][7], st + off[f][8], fs[f] * sizeof(float));
            memcpy(st + off[f][8], st + off[f][9], fs[f] * sizeof(float));
        }
        if (record)
            for (int x = pml; x < nx - pml; ++x)
                memcpy(record + k * plane + (size_t)(x - pml) * (ny - 2 * pml),
                       u2 + IX(a->sz, x, pml, nx, ny), (ny - 2 * pml) * sizeof(float));
        if (uxyzmax) uxyzmax[k] = M;
        cnt.s_cells += scells;
        cnt.pml_cells += pcells;
        (void)s64; (void)u64; (void)p64;
    }
    if (counts) {
        counts[0] = cnt.s_cells;
        counts[1] = cnt.pml_cells;
    }
    return 0;
}

// Rates of the FP64 fallbacks over sampled inputs of the scalar operator
// and the PML update (for the tests' statements of how rare they are).
extern "C" void emul_fallback_rates(const float *ux, const float *uy, const float *uz,
                                    const float *e2, const float *r8, long long n,
                                    long long *unit_fb, long long *s_fb)
{
    long long u = 0, s = 0;
    for (long long i = 0; i < n; ++i) {
        const float m2 = grad_m2(ux[i], uy[i], uz[i]);
        const float mode = sqrt_ieee(m2);
        float y = rcp_approx(mode);
        y = fma_(fma_(-mode, y, 1.0f), y, y);
        float nx_, ny_, nz_;
        const bool ok = unit_comp(ux[i], mode, y, nx_) && unit_comp(uy[i], mode, y, ny_) &&
                        unit_comp(uz[i], mode, y, nz_);
        if (!ok) {
            ++u;
            nx_ = unit_comp_fp64(ux[i], mode);
            ny_ = unit_comp_fp64(uy[i], mode);
            nz_ = unit_comp_fp64(uz[i], mode);
        }
        const float aa = add(mul(nx_, nx_), mul(ny_, ny_));
        const float num = mul(mul(mul(r8[i], aa), nz_), nz_);
        const float base = add(1.0f, mul(e2[i], aa));
        float S;
        if (!s_value(num, base, S)) ++s;
    }
    *unit_fb = u;
    *s_fb = s;
}

// The same decisions, checked one by one against the reference expressions
// evaluated directly (double arithmetic as the reference writes it).
extern "C" long long emul_check_scalar(const float *ux, const float *uy, const float *uz,
                                       const float *e2, const float *r8, long long n,
                                       float *got, float *want)
{
    long long bad = 0;
    for (long long i = 0; i < n; ++i) {
        const float m2 = grad_m2(ux[i], uy[i], uz[i]);
        const float g = scalar_s(ux[i], uy[i], uz[i], m2, e2[i], r8[i]);
        const float mode = sqrtf(m2);
        const float nxv = (float)((double)ux[i] / ((double)mode + kEpsN));
        const float nyv = (float)((double)uy[i] / ((double)mode + kEpsN));
        const float nzv = (float)((double)uz[i] / ((double)mode + kEpsN));
        const float aa = nxv * nxv + nyv * nyv;
        const float num = r8[i] * aa * nzv * nzv;
        const float base = 1 + e2[i] * aa;
        const double den = (double)base * (double)base;
        const float w = (float)(0.5 * (1 + sqrt(1 - (double)num / den)));
        got[i] = g;
        want[i] = w;
        uint32_t gb, wb;
        memcpy(&gb, &g, 4);
        memcpy(&wb, &w, 4);
        if (gb != wb) ++bad;
    }
    return bad;
}
