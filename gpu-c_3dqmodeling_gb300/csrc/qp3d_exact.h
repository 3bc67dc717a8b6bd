// qp3d_exact.h -- the reference CPU operators' arithmetic, bit for bit.
//
// The reference's CPU operators (CPU_function.c:301-480, compiled by g++ as
// C++ without contraction) round every float operation separately, divide
// every stencil tap by dx (or dx*dx), and evaluate parts of the scalar
// operator and of the PML update in double precision:
//
//   grad      Ux = sum_m  c[m]*(u[+m]-u[-m]) / dx              (float, in order)
//   laplacian Uxx = sum_m c2[m]*((u[+m]-2u) + u[-m]) / (dx*dx)  (float, in order)
//   S         n = u/(mode + 2.22e-17)     (double, rounded to float)
//             S = 0.5*(1 + sqrt(1 - num/base^2))                (double -> float)
//   PML       w13, p3, w33 of each face                         (double -> float)
//
// This header restates those operations so that FP32 hardware reproduces
// the reference's results exactly:
//   * float operations are the same IEEE operations, each rounded once, in
//     the reference's order; the divisions stay IEEE divisions (a multiply by
//     a rounded reciprocal with a fused correction is exact for normal
//     quotients only, and the subnormal quotients of the tiny values ahead of
//     a wavefront grow with it into the signal);
//   * expressions evaluated in double are computed as unevaluated sums of two
//     floats with a bound on their error.  Where the float nearest to the
//     double result is certain, it is taken; otherwise (a few cells per
//     million) the expression is evaluated in FP64 exactly as the reference
//     does.  FP64 arithmetic (IEEE add, multiply, divide, square root) is the
//     same on the GPU and on the host.
//
// Everything here is __host__ __device__: the tests compile this header for
// the CPU and compare it with the oracle's restatement of the reference,
// operation by operation and over whole runs.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define QP3D_HD __host__ __device__ __forceinline__
#define QP3D_HD_NOINLINE static __host__ __device__ __noinline__
#else
#define QP3D_HD inline
#define QP3D_HD_NOINLINE static inline
#endif

namespace qp3d {
namespace xr {

constexpr double kEpsN = 2.22e-17;   // CPU_function.c:8, GPU_kernel.cu:7

// ---------------------------------------------------------------------------
// Primitives: one IEEE round-to-nearest operation each.
// ---------------------------------------------------------------------------
#if defined(__CUDA_ARCH__)
QP3D_HD float add(float a, float b) { return __fadd_rn(a, b); }
QP3D_HD float sub(float a, float b) { return __fsub_rn(a, b); }
QP3D_HD float mul(float a, float b) { return __fmul_rn(a, b); }
QP3D_HD float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
QP3D_HD float div_ieee(float a, float b) { return __fdiv_rn(a, b); }
QP3D_HD float sqrt_ieee(float a) { return __fsqrt_rn(a); }
// approximations (relative error below 2^-21 for normal inputs)
QP3D_HD float rcp_approx(float a)
{
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
QP3D_HD float rsqrt_approx(float a)
{
    float r;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
QP3D_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
QP3D_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
QP3D_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
QP3D_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
QP3D_HD double dsqrt(double a) { return __dsqrt_rn(a); }
QP3D_HD float d2f(double a) { return __double2float_rn(a); }
QP3D_HD uint32_t fbits(float a) { return __float_as_uint(a); }
QP3D_HD float ffrom(uint32_t u) { return __uint_as_float(u); }
#else
// Host: compiled with contraction off, so each expression is one rounding.
// QP3D_XR_APPROX_SKEW (tests) perturbs the approximations by up to that
// relative amount, to exercise the error bounds the device relies on.
#ifndef QP3D_XR_APPROX_SKEW
#define QP3D_XR_APPROX_SKEW 0.0
#endif
inline float add(float a, float b) { return a + b; }
inline float sub(float a, float b) { return a - b; }
inline float mul(float a, float b) { return a * b; }
inline float fma_(float a, float b, float c) { return fmaf(a, b, c); }
inline float div_ieee(float a, float b) { return a / b; }
inline float sqrt_ieee(float a) { return sqrtf(a); }
inline float skew(float r, float a)
{
    if (QP3D_XR_APPROX_SKEW == 0.0) return r;
    uint32_t u;
    memcpy(&u, &a, 4);
    u = u * 2654435761u;   // a deterministic pseudo-random sign and size per input
    double f = ((double)(u >> 8) / (double)(1u << 24)) * 2.0 - 1.0;
    return (float)((double)r * (1.0 + f * QP3D_XR_APPROX_SKEW));
}
inline float rcp_approx(float a) { return skew(1.0f / a, a); }
inline float rsqrt_approx(float a) { return skew(1.0f / sqrtf(a), a); }
inline double dadd(double a, double b) { return a + b; }
inline double dsub(double a, double b) { return a - b; }
inline double dmul(double a, double b) { return a * b; }
inline double ddiv(double a, double b) { return a / b; }
inline double dsqrt(double a) { return sqrt(a); }
inline float d2f(double a) { return (float)a; }
inline uint32_t fbits(float a)
{
    uint32_t u;
    memcpy(&u, &a, 4);
    return u;
}
inline float ffrom(uint32_t u)
{
    float a;
    memcpy(&a, &u, 4);
    return a;
}
#endif

// ---------------------------------------------------------------------------
// Helpers for the rounding decisions
// ---------------------------------------------------------------------------
// Half an ulp of |x| above and below |x| (x normal, |x| >= 2^-100).
QP3D_HD void half_ulps(float x, float &hup, float &hdn)
{
    const uint32_t e = fbits(x) & 0x7f800000u;
    hup = mul(ffrom(e), 5.9604644775390625e-08f);   // 2^-24
    hdn = (fbits(x) & 0x007fffffu) ? hup : mul(hup, 0.5f);
}

// Exact sum s + e = a + b (|a| >= |b| or a == 0).
QP3D_HD void fast_two_sum(float a, float b, float &s, float &e)
{
    s = add(a, b);
    e = sub(b, sub(s, a));
}

// Exact sum s + e = a + b (any order).
QP3D_HD void two_sum(float a, float b, float &s, float &e)
{
    s = add(a, b);
    const float bb = sub(s, a);
    e = add(sub(a, sub(s, bb)), sub(b, bb));
}

// float-float value hi + lo
struct FF {
    float hi, lo;
};

// (x.hi + x.lo) * f with error below 2^-47 |x f|
QP3D_HD FF ff_mul_f(FF x, float f)
{
    FF r;
    r.hi = mul(x.hi, f);
    r.lo = fma_(x.lo, f, fma_(x.hi, f, -r.hi));
    return r;
}

// x + y with error below 2^-47 (|x| + |y|)
QP3D_HD FF ff_add(FF x, FF y)
{
    float s, e;
    two_sum(x.hi, y.hi, s, e);
    e = add(e, add(x.lo, y.lo));
    FF r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

QP3D_HD FF ff_add_f(FF x, float f)
{
    float s, e;
    two_sum(x.hi, f, s, e);
    e = add(e, x.lo);
    FF r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

QP3D_HD FF ff_neg(FF x) { return FF{-x.hi, -x.lo}; }

// The float nearest to v = x.hi + x.lo when v is known within err (absolute),
// and the double computation that v approximates is within err of v too:
// returns false when v lies within 2 err of a rounding boundary (midpoint
// between floats), or when |v| is too small for the bound to hold (parts
// of it may have underflowed; a result of exactly zero is the caller's to
// handle).  Normalized input (|lo| <= ulp(hi)/2 up to rounding) as produced
// by ff_add.
QP3D_HD bool ff_round(FF x, float err, float &out)
{
    const float ah = fabsf(x.hi);
    if (!(ah >= 7.88860905e-31f) || !(ah < 1.0e30f)) return false;   // 2^-100
    float hup, hdn;
    half_ulps(ah, hup, hdn);
    // lo pointing away from zero: the boundary is hup away, else hdn
    const bool away = (x.lo > 0.0f) == (x.hi > 0.0f);
    const float lim = away ? hup : hdn;
    const float m = add(fabsf(x.lo), mul(2.0f, err));
    if (!(m < lim)) return false;
    out = x.hi;
    return true;
}

// ---------------------------------------------------------------------------
// Scalar operator: the unit-normal components (CPU_function.c:355-357)
//   n = (float)((double)u / ((double)mode + 2.22e-17))
// q = RN(u/mode) from a reciprocal y of mode and Markstein corrections, its
// exact remainder, and a test that (double)u/(mode + eps) rounds to q too.
// Returns false when that is not certain (the caller then uses FP64).
// ---------------------------------------------------------------------------
QP3D_HD bool unit_comp(float u, float mode, float y, float &out)
{
    if (u == 0.0f) {
        out = u;   // +-0 / positive = +-0
        return true;
    }
    const float q0 = mul(u, y);
    const float r0 = fma_(-q0, mode, u);
    const float q1 = fma_(r0, y, q0);
    const float r1 = fma_(-q1, mode, u);    // exact when q1 = RN(u/mode)
    const float A = fabsf(u), Q = fabsf(q1);
    if (!(A >= 7.88860905e-31f) || !(Q >= 7.88860905e-31f) || !(Q < 1.0e30f)) return false;
    const float R = (u > 0.0f) ? r1 : -r1;  // remainder of |u| / mode
    float hup, hdn;
    half_ulps(Q, hup, hdn);
    // |u|/mode lies in [Q - hdn, Q + hup] iff -hdn*mode <= R <= hup*mode; the
    // reference's quotient is |u|/mode' with mode <= mode' <= mode (1 + eta),
    // eta <= 2.22e-17/mode + 2^-53, then rounded to double (2^-53).
    // above: hup*mode - R > 2^-52 |u|  (factor 2 covers this test's roundings)
    const float up = sub(mul(hup, mode), R);
    if (!(up > mul(A, 2.22044605e-16f))) return false;                 // 2^-52
    // below: R + hdn*mode > |u| (eta + 2^-53): |u| eta <= Q (1 + 2^-23) 2.22e-17 + |u| 2^-53
    const float dn = add(R, mul(hdn, mode));
    const float lim = fma_(Q, 4.44100009e-17f, mul(A, 4.44089210e-16f));   // 2x, 2^-51
    if (!(dn > lim)) return false;
    out = (u > 0.0f) ? Q : -Q;
    return true;
}

QP3D_HD_NOINLINE float unit_comp_fp64(float u, float mode)
{
    return d2f(ddiv((double)u, dadd((double)mode, kEpsN)));
}

// S = (float)(0.5 * (1 + sqrt(1 - (double)num / ((double)base * base))))
// (CPU_function.c:365; pow(float, 2) is the exact double square).
QP3D_HD_NOINLINE float s_value_fp64(float num, float base)
{
    const double den = dmul((double)base, (double)base);
    return d2f(dmul(0.5, dadd(1.0, dsqrt(dsub(1.0, ddiv((double)num, den))))));
}

QP3D_HD bool s_value(float num, float base, float &out)
{
    if (num == 0.0f) {   // 1 - 0 = 1, sqrt 1 = 1, 0.5 * 2 = 1
        out = 1.0f;
        return true;
    }
    if (!(num > 0.0f) || !(base >= 0.5f) || !(base < 4.0f)) return false;
    // x = num / base^2 as xh + xl (error < 2^-45 x)
    const float bh = mul(base, base), bl = fma_(base, base, -bh);
    const float rb = rcp_approx(bh);
    const float x0 = mul(num, rb);
    const float xh = fma_(fma_(-x0, bh, num), rb, x0);
    const float e1 = fma_(-xh, bh, num);
    const float xl = mul(fma_(-xh, bl, e1), rb);
    // y = 1 - x as yh + yl
    const float yh = sub(1.0f, xh);
    if (!(yh > 0.0625f)) return false;
    const float yl = sub(sub(sub(1.0f, yh), xh), xl);
    // s = sqrt(y) as sh + sl
    const float rs = rsqrt_approx(yh);
    const float hrs = mul(0.5f, rs);
    const float s0 = mul(yh, rs);
    const float s1 = fma_(fma_(-s0, s0, yh), hrs, s0);
    const float sl = mul(add(fma_(-s1, s1, yh), yl), hrs);
    // t = 1 + s, V = t / 2
    float th, tl;
    fast_two_sum(1.0f, s1, th, tl);
    tl = add(tl, sl);
    FF v;
    fast_two_sum(mul(0.5f, th), mul(0.5f, tl), v.hi, v.lo);
    // float-float error ~2^-44, the reference's double roundings ~2^-51
    return ff_round(v, 2.8421709e-14f /* 2^-45 */, out);
}

// ---------------------------------------------------------------------------
// The whole scalar operator of one cell above the threshold, given its
// gradient (CPU_function.c:351-365).  e2 = 2 eps, r8 = 8 (eps - delta), both
// exact multiples of the inputs.
// ---------------------------------------------------------------------------
QP3D_HD float scalar_s(float ux, float uy, float uz, float m2, float e2, float r8)
{
    const float mode = sqrt_ieee(m2);
    // reciprocal of mode good to ~1 ulp: approximation + one Newton step
    float y = rcp_approx(mode);
    y = fma_(fma_(-mode, y, 1.0f), y, y);
    float nxv, nyv, nzv;
    const bool okx = unit_comp(ux, mode, y, nxv);
    const bool oky = unit_comp(uy, mode, y, nyv);
    const bool okz = unit_comp(uz, mode, y, nzv);
    if (!(okx && oky && okz)) {
        nxv = unit_comp_fp64(ux, mode);
        nyv = unit_comp_fp64(uy, mode);
        nzv = unit_comp_fp64(uz, mode);
    }
    const float aa = add(mul(nxv, nxv), mul(nyv, nyv));
    const float num = mul(mul(mul(r8, aa), nzv), nzv);
    const float base = add(1.0f, mul(e2, aa));
    float S;
    if (!s_value(num, base, S)) S = s_value_fp64(num, base);
    return S;
}

// ---------------------------------------------------------------------------
// Stencil along one axis (CPU_function.c:314-316, 393-395), scalar form:
// a[m] = u at +(m+1), b[m] = u at -(m+1), c = c[31..35] or c2[31..35].
// The kernels perform the same operations two cells at a time.
// ---------------------------------------------------------------------------
QP3D_HD float grad_axis(const float *a, const float *b, const float *c, float h)
{
    float g = 0.0f;
    for (int m = 0; m < 5; ++m) g = add(g, div_ieee(mul(c[m], sub(a[m], b[m])), h));
    return g;
}

QP3D_HD float lap_axis(const float *a, const float *b, float u0, const float *c2, float h2)
{
    float l = 0.0f;
    for (int m = 0; m < 5; ++m)
        l = add(l, div_ieee(mul(c2[m], add(fma_(-2.0f, u0, a[m]), b[m])), h2));
    return l;
}

// m2 = ux*ux + uy*uy + uz*uz in the reference's order
QP3D_HD float grad_m2(float ux, float uy, float uz)
{
    return add(add(mul(ux, ux), mul(uy, uy)), mul(uz, uz));
}

// ---------------------------------------------------------------------------
// Interior update (CPU_function.c:392):
//   u3 = 2*u2 - u1 + dt*dt*((1 + 2*eps)*(Uxx + Uyy) + Uzz)*S*vp*vp
// dt2 = RN(dt*dt), e1 = RN(1 + 2 eps).
// ---------------------------------------------------------------------------
QP3D_HD float interior_update(float u2, float u1, float Uxx, float Uyy, float Uzz, float e1,
                              float S, float vp, float dt2)
{
    const float X = add(mul(e1, add(Uxx, Uyy)), Uzz);
    const float B = mul(mul(mul(mul(dt2, X), S), vp), vp);
    return add(fma_(2.0f, u2, -u1), B);
}

// ---------------------------------------------------------------------------
// PML update of one cell (CPU_function.c:400-478).  Per layer the reference
// uses d = damping profile, dd its second profile, and
//   b = d*dt + 1 (= 1 + dt*d),  a1 = b^2 - 3 (exact in double),
//   a2 = 2*d*dt - 1 (float),    a3 = 1 - dt*d (float).
// a1 is carried as a1h + a1l (exact).  Face kinds: normal along x, y or z;
// the odd faces (right, back, bottom) subtract the dd*u_n term.
// ---------------------------------------------------------------------------
struct PmlLayer {
    float a1h, a1l, a2, a3, dd;
};

struct PmlOut {
    float w13, w21, w33, p3, u3;
};

// An = (double)F * vdt^2 as a float-float (vdt^2 = vh + vl exactly)
QP3D_HD FF coef_times_v2(float F, float vh, float vl)
{
    FF r;
    r.hi = mul(F, vh);
    r.lo = fma_(F, vl, fma_(F, vh, -r.hi));
    return r;
}

QP3D_HD_NOINLINE PmlOut pml_update_fp64(bool zface, bool minus, float S, float e1, float vdt,
                                        float Unn, float Un, float tang, float dt,
                                        const PmlLayer &L, float w11, float w12, float w21,
                                        float w31, float w32, float p1, float p2)
{
    const double vdt2 = dmul((double)vdt, (double)vdt);
    const float eS = mul(e1, S);
    const double An = dmul((double)(zface ? S : eS), vdt2);
    const double At = dmul((double)(zface ? eS : S), vdt2);
    const double a1 = (double)L.a1h + (double)L.a1l;   // exact
    PmlOut o;
    const double t1 = dsub(dmul(An, (double)Unn), dmul(a1, (double)w12));
    o.w13 = d2f(dadd(t1, (double)mul(L.a2, w11)));
    const double q = dadd(dmul(-a1, (double)p2), (double)mul(L.a2, p1));
    const double src = dmul(dmul(An, (double)L.dd), (double)Un);
    o.p3 = d2f(minus ? dsub(q, src) : dadd(q, src));
    o.w21 = add(mul(dt, o.p3), mul(w21, L.a3));
    o.w33 = d2f(dsub(dadd(dmul(At, (double)tang), (double)mul(2.0f, w32)), (double)w31));
    o.u3 = add(add(o.w13, o.w21), o.w33);
    return o;
}

// zface: the face's normal is z (top/bottom), which swaps the roles of
// S and (1 + 2 eps) S; minus: right, back or bottom face.
// A result whose terms are all exactly zero is the signed zero that IEEE
// arithmetic gives on those zeros; it is computed directly, in the
// reference's order of operations.
QP3D_HD PmlOut pml_update(bool zface, bool minus, float S, float e1, float vdt, float Unn,
                          float Un, float tang, float dt, const PmlLayer &L, float w11,
                          float w12, float w21, float w31, float w32, float p1, float p2)
{
    const float vh = mul(vdt, vdt), vl = fma_(vdt, vdt, -vh);
    const float eS = mul(e1, S);
    const FF An = coef_times_v2(zface ? S : eS, vh, vl);
    const FF At = coef_times_v2(zface ? eS : S, vh, vl);
    const FF a1 = {L.a1h, L.a1l};
    const bool an0 = An.hi == 0.0f && An.lo == 0.0f, at0 = At.hi == 0.0f && At.lo == 0.0f;
    PmlOut o;
    bool ok = true;
    // w13 = (float)(An*Unn - a1*w12 + (float)(a2*w11))
    {
        const float F2 = mul(L.a2, w11);
        if ((an0 || Unn == 0.0f) && w12 == 0.0f && F2 == 0.0f) {
            o.w13 = add(sub(mul(An.hi, Unn), mul(a1.hi, w12)), F2);
        } else {
            const FF t = ff_add(ff_mul_f(An, Unn), ff_neg(ff_mul_f(a1, w12)));
            const FF w = ff_add_f(t, F2);
            const float mag = add(add(fabsf(mul(An.hi, Unn)), fabsf(mul(a1.hi, w12))), fabsf(F2));
            ok = ok && ff_round(w, mul(mag, 1.42108547e-14f /* 2^-46 */), o.w13);
        }
    }
    // p3 = (float)((-a1)*p2 + (float)(a2*p1) +- An*dd*Un)
    {
        const float F3 = mul(L.a2, p1);
        if (p2 == 0.0f && F3 == 0.0f && (an0 || L.dd == 0.0f || Un == 0.0f)) {
            const float q = add(mul(-a1.hi, p2), F3), src = mul(mul(An.hi, L.dd), Un);
            o.p3 = minus ? sub(q, src) : add(q, src);
        } else {
            const FF q = ff_add_f(ff_neg(ff_mul_f(a1, p2)), F3);
            FF src = ff_mul_f(ff_mul_f(An, L.dd), Un);
            if (minus) src = ff_neg(src);
            const FF w = ff_add(q, src);
            const float mag = add(add(fabsf(mul(a1.hi, p2)), fabsf(F3)), fabsf(src.hi));
            ok = ok && ff_round(w, mul(mag, 1.42108547e-14f), o.p3);
        }
    }
    // w33 = (float)(At*tang + (float)(2*w32) - w31)
    {
        const float F4 = mul(2.0f, w32);
        if ((at0 || tang == 0.0f) && F4 == 0.0f && w31 == 0.0f) {
            o.w33 = sub(add(mul(At.hi, tang), F4), w31);
        } else {
            const FF w = ff_add_f(ff_add_f(ff_mul_f(At, tang), F4), -w31);
            const float mag = add(add(fabsf(mul(At.hi, tang)), fabsf(F4)), fabsf(w31));
            ok = ok && ff_round(w, mul(mag, 1.42108547e-14f), o.w33);
        }
    }
    if (!ok)
        return pml_update_fp64(zface, minus, S, e1, vdt, Unn, Un, tang, dt, L, w11, w12, w21,
                               w31, w32, p1, p2);
    o.w21 = add(mul(dt, o.p3), mul(w21, L.a3));
    o.u3 = add(add(o.w13, o.w21), o.w33);
    return o;
}

// Per-layer constants of a damping profile value d (host or device).
QP3D_HD PmlLayer pml_layer(float d, float dd, float dt)
{
    PmlLayer L;
    const float b = add(mul(d, dt), 1.0f);
    // a1 = b*b - 3 exactly: b*b = bh + bl exactly, then bh - 3 is exact
    // (bh in [1, 4)), so a1 = (bh - 3) + bl, renormalized
    const float bh = mul(b, b), bl = fma_(b, b, -bh);
    fast_two_sum(sub(bh, 3.0f), bl, L.a1h, L.a1l);
    L.a2 = sub(mul(mul(2.0f, d), dt), 1.0f);
    L.a3 = sub(1.0f, mul(dt, d));
    L.dd = dd;
    return L;
}

}  // namespace xr
}  // namespace qp3d
