// qp3d_kernels.cu -- sm_103a kernels for the 3D pure-qP VTI time step.
//
// One time step of the reference (3dPureqPModeling_single_shot.cu:282-320:
// grad -> D2H + host absMaxval -> scalar_operator -> wavefield_update ->
// addsource -> exchange -> D2H + record crop) becomes:
//
//   qp3d_step_kernel      everything in one pass: gradient, scalar operator S
//                         (GPU_kernel.cu:87-115), Laplacians, interior
//                         leapfrog and the six split-field PML faces
//                         (GPU_kernel.cu:534-639), source injection
//                         (GPU_kernel.cu:720-731), the receiver plane
//                         (3dPureqPModeling_single_shot.cu:333-337), and the
//                         step's own max|grad u| (atomicMax on the float bits:
//                         all values are >= 0, so bit order is value order).
//                         The time-level rotation (GPU_kernel.cu:733-812) is
//                         done by the host swapping buffer indices.
//   the threshold         S needs the max of the step before any cell is
//                         updated: either qp3d_gradmax_kernel computes it
//                         first (GPU_kernel.cu:14-33 + CPU_function.c:10-22),
//                         or the step runs speculatively with a predicted
//                         window and qp3d_resolve / compact / fixup_kernel
//                         settle the cells whose decision waited (a gated
//                         exact re-run when the prediction missed).
//
// The same tile bodies run in the batched persistent kernels (many shots per
// launch), and the adjoint kernels at the end of the file transpose the step.
//
// Both kernels march along z.  A CTA owns a tile of tile_x rows (x) by 32
// cells (y) and a chunk of z planes.  Each thread owns one row and four
// consecutive y cells (a "quad", one float4).  Planes of u(k), with a 5-row
// and 8-column halo, are staged into a ring of kRing shared-memory slots by
// TMA (cp.async.bulk.tensor.3d) and completed on one mbarrier per slot; the
// stencil reads all 30 taps from shared memory.  Loads of the next planes
// overlap the arithmetic of the current one.
//
// Arithmetic.  The 1/h factors of the reference (each tap divided by dx or
// dx*dx, CPU_function.c:314-316,393-395) are folded into the coefficient
// tables, and a*b+c is fused where written as fmaf().  This translation unit
// is compiled with -fmad=false so that no other fusion happens: the result is
// bit-identical to the mirror variant of the CPU oracle.  The division of the
// scalar operator is a Newton-Raphson reciprocal (rcp_nr2: fused
// multiply-adds only, so the oracle reproduces it exactly); the square root
// is IEEE (sqrt.rn).
#include "qp3d_internal.h"
#include "qp3d_exact.h"

#include <math.h>

namespace qp3d {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + TMA
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after limit_ns of wall time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  unsigned long long limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int c0, int c1,
                                            int c2, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float4 lds4(const float *p)
{
    return *reinterpret_cast<const float4 *>(p);
}

__device__ __forceinline__ float f4(const float4 &v, int j)
{
    return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w;
}

// ---------------------------------------------------------------------------
// Shared-memory layout of both plane kernels
// ---------------------------------------------------------------------------
struct SmemLayout {
    size_t slot_floats;   // one staged plane, padded to 128 B
    size_t ring_bytes;
    size_t bar_off;       // kRing mbarriers
    size_t tab_off;       // 3 * pml float4 layer coefficients
    size_t src_off;       // fused source entries of this CTA
    size_t misc_off;      // scalars
    size_t total;
};

__host__ __device__ inline SmemLayout smem_layout(int tile_x, int pml,
                                                  int nsrc = kMaxFusedSources)
{
    SmemLayout L;
    size_t box = (size_t)(tile_x + 2 * kRadius) * kBoxY;
    L.slot_floats = (box + 31) & ~(size_t)31;
    L.ring_bytes = L.slot_floats * 4 * kRing;
    L.bar_off = L.ring_bytes;
    L.tab_off = L.bar_off + 16 * kRing;   // full[kRing], empty[kRing]
    L.tab_off = (L.tab_off + 15) & ~(size_t)15;
    L.src_off = L.tab_off + 16 * 3 * (size_t)(pml > 0 ? pml : 1);
    L.misc_off = L.src_off + sizeof(SrcEntry) * (size_t)(nsrc > 0 ? nsrc : 1);
    L.misc_off = (L.misc_off + 15) & ~(size_t)15;
    L.total = L.misc_off + 64;
    return L;
}

size_t plane_smem_bytes(int tile_x, int pml, int nsrc) { return smem_layout(tile_x, pml, nsrc).total; }

// ---------------------------------------------------------------------------
// Threshold of the scalar operator, GPU_kernel.cu:99.
//   (double)mode > 1.0e-02 * uxyzMax  <=>  mode > Tf, Tf = largest float not
//   above the double product;  mode = sqrtf(m2) > Tf  <=>  m2 > T2 with
//   T2 = max{x : sqrtf(x) <= Tf}.  The oracle derives T2 the same way.
// ---------------------------------------------------------------------------
__device__ float threshold_m2(float gmax)
{
    double td = 1.0e-02 * (double)gmax;
    float t = __double2float_rd(td);
    if (!(t >= 0.0f)) return t;
    float x = __fmul_rn(t, t);
    for (int it = 0; it < 64 && x > 0.0f && __fsqrt_rn(x) > t; ++it) x = nextafterf(x, 0.0f);
    for (int it = 0; it < 64; ++it) {
        float n = nextafterf(x, INFINITY);
        if (isinf(n) || __fsqrt_rn(n) > t) break;
        x = n;
    }
    return x;
}

// ---------------------------------------------------------------------------
// Stencil over one quad: first and second derivatives along x, y, z of the
// four cells (x, y..y+3, z) from the staged planes.  Cells (0,1) and (2,3)
// are processed as pairs with the packed FP32x2 instructions (add/mul/fma
// .rn.f32x2, round-to-nearest per lane, so every lane is bit-identical to
// the scalar operation it replaces).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
}

// slot of staged plane (base + d), base already reduced modulo kRing
__device__ __forceinline__ int slot_add(int s, int d)
{
    s += d;
    if (s >= kRing) s -= kRing;
    if (s < 0) s += kRing;
    return s;
}

// One second-difference tap in the reference's form, (u[+m] - 2u) + u[-m]
// (CPU_function.c:393-395), two cells at a time.  Summing c2[m] times these
// keeps a constant field's Laplacian exactly zero; the form with the centre
// weight folded into one coefficient, -2 sum(c2[m]) u + sum c2[m](u[+m] +
// u[-m]), does not (its rounded coefficients leave a term proportional to u),
// and that systematic term grew to 1.6e-5 relative L2 against the reference
// arithmetic over a 1000-step shot, against 6.7e-6 with this form.
__device__ __forceinline__ float2 lap_tap2(float2 a, float2 b, float2 u0)
{
    return __fadd2_rn(__ffma2_rn(make_float2(-2.0f, -2.0f), u0, a), b);
}

template <bool SECOND>
__device__ __forceinline__ void quad_derivs(const float *ring, size_t slot_floats, int t, int rc,
                                            const Coefs &k, float Ux[4], float Uy[4],
                                            float Uz[4], float Uxx[4], float Uyy[4],
                                            float Uzz[4], float u0[4])
{
    const int sc = (t + kRadius) % kRing;
    const float *pc = ring + (size_t)sc * slot_floats;
    // the z taps: planes sc +- (m + 1) of the ring, wrapped by one ring length
    const float *pcr = pc + rc;
    const float *pcr_lo = pcr - kRing * (int)slot_floats;
    const float *pcr_hi = pcr + kRing * (int)slot_floats;
    // y taps: columns c-8 .. c+11 of the centre plane
    float Y[20];
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        float4 v = lds4(pc + rc - 8 + 4 * b);
        Y[4 * b] = v.x; Y[4 * b + 1] = v.y; Y[4 * b + 2] = v.z; Y[4 * b + 3] = v.w;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j0 = 2 * h, j1 = 2 * h + 1;
        const float2 c0 = f2(Y[8 + j0], Y[8 + j1]);
        u0[j0] = c0.x;
        u0[j1] = c0.y;
        float2 g = f2(0.0f, 0.0f), l = f2(0.0f, 0.0f);
#pragma unroll
        for (int m = 0; m < kRadius; ++m) {
            const float2 a = f2(Y[8 + j0 + m + 1], Y[8 + j1 + m + 1]);
            const float2 b = f2(Y[8 + j0 - m - 1], Y[8 + j1 - m - 1]);
            const float2 d = sub2(a, b);
            g = (m == 0) ? __fmul2_rn(k.cy2[0], d) : __ffma2_rn(k.cy2[m], d, g);
            if (SECOND) l = (m == 0) ? __fmul2_rn(k.c2y2[0], lap_tap2(a, b, c0))
                                     : __ffma2_rn(k.c2y2[m], lap_tap2(a, b, c0), l);
        }
        Uy[j0] = g.x; Uy[j1] = g.y;
        if (SECOND) { Uyy[j0] = l.x; Uyy[j1] = l.y; }
    }
    // x taps: rows r +- m of the centre plane
    const float2 uc[2] = {f2(u0[0], u0[1]), f2(u0[2], u0[3])};
    float2 gx[2] = {f2(0.f, 0.f), f2(0.f, 0.f)}, lx[2] = {f2(0.f, 0.f), f2(0.f, 0.f)};
#pragma unroll
    for (int m = 0; m < kRadius; ++m) {
        const float4 a = lds4(pc + rc + (m + 1) * kBoxY);
        const float4 b = lds4(pc + rc - (m + 1) * kBoxY);
        const float2 a2[2] = {f2(a.x, a.y), f2(a.z, a.w)}, b2[2] = {f2(b.x, b.y), f2(b.z, b.w)};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2 d = sub2(a2[h], b2[h]);
            gx[h] = (m == 0) ? __fmul2_rn(k.cx2[0], d) : __ffma2_rn(k.cx2[m], d, gx[h]);
            if (SECOND) lx[h] = (m == 0) ? __fmul2_rn(k.c2x2[0], lap_tap2(a2[h], b2[h], uc[h]))
                                         : __ffma2_rn(k.c2x2[m], lap_tap2(a2[h], b2[h], uc[h]),
                                                      lx[h]);
        }
    }
    Ux[0] = gx[0].x; Ux[1] = gx[0].y; Ux[2] = gx[1].x; Ux[3] = gx[1].y;
    if (SECOND) { Uxx[0] = lx[0].x; Uxx[1] = lx[0].y; Uxx[2] = lx[1].x; Uxx[3] = lx[1].y; }
    // z taps: planes t+5 +- m
    float2 gz[2] = {f2(0.f, 0.f), f2(0.f, 0.f)}, lz[2] = {f2(0.f, 0.f), f2(0.f, 0.f)};
#pragma unroll
    for (int m = 0; m < kRadius; ++m) {
        const int d = (m + 1) * (int)slot_floats;
        const float4 a = lds4((sc + m + 1 < kRing ? pcr : pcr_lo) + d);
        const float4 b = lds4((sc >= m + 1 ? pcr : pcr_hi) - d);
        const float2 a2[2] = {f2(a.x, a.y), f2(a.z, a.w)}, b2[2] = {f2(b.x, b.y), f2(b.z, b.w)};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float2 d = sub2(a2[h], b2[h]);
            gz[h] = (m == 0) ? __fmul2_rn(k.cz2[0], d) : __ffma2_rn(k.cz2[m], d, gz[h]);
            if (SECOND) lz[h] = (m == 0) ? __fmul2_rn(k.c2z2[0], lap_tap2(a2[h], b2[h], uc[h]))
                                         : __ffma2_rn(k.c2z2[m], lap_tap2(a2[h], b2[h], uc[h]),
                                                      lz[h]);
        }
    }
    Uz[0] = gz[0].x; Uz[1] = gz[0].y; Uz[2] = gz[1].x; Uz[3] = gz[1].y;
    if (SECOND) { Uzz[0] = lz[0].x; Uzz[1] = lz[0].y; Uzz[2] = lz[1].x; Uzz[3] = lz[1].y; }
}

// ---------------------------------------------------------------------------
// The same derivatives in the reference's arithmetic (CPU_function.c:314-316,
// 393-395; qp3d_exact.h): per tap c*(u[+m]-u[-m]) / h and
// c2*((u[+m]-2u) + u[-m]) / h^2, each operation rounded, IEEE division, the
// taps summed in order from 0.  Products and sums two cells at a time with
// the packed FP32x2 instructions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 div2(float2 p, float h)
{
    return make_float2(__fdiv_rn(p.x, h), __fdiv_rn(p.y, h));
}

// one tap of both derivatives for a pair of cells: a = u[+m], b = u[-m]
__device__ __forceinline__ void tap2(float2 a, float2 b, float2 u0, float2 c, float2 c2, float h,
                                     float h2, float2 &g, float2 &l)
{
    g = __fadd2_rn(g, div2(__fmul2_rn(c, sub2(a, b)), h));
    l = __fadd2_rn(l, div2(__fmul2_rn(c2, lap_tap2(a, b, u0)), h2));
}

__device__ __forceinline__ void quad_derivs_ref(const float *ring, size_t slot_floats, int t,
                                                int rc, const Coefs &k, float Ux[4], float Uy[4],
                                                float Uz[4], float Uxx[4], float Uyy[4],
                                                float Uzz[4], float u0[4])
{
    const int sc = (t + kRadius) % kRing;
    const float *pc = ring + (size_t)sc * slot_floats;
    const float2 zero = make_float2(0.0f, 0.0f);
    float Y[20];
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        float4 v = lds4(pc + rc - 8 + 4 * b);
        Y[4 * b] = v.x; Y[4 * b + 1] = v.y; Y[4 * b + 2] = v.z; Y[4 * b + 3] = v.w;
    }
    float2 c0[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j0 = 2 * h, j1 = 2 * h + 1;
        c0[h] = f2(Y[8 + j0], Y[8 + j1]);
        u0[j0] = c0[h].x;
        u0[j1] = c0[h].y;
        float2 g = zero, l = zero;
#pragma unroll
        for (int m = 0; m < kRadius; ++m)
            tap2(f2(Y[8 + j0 + m + 1], Y[8 + j1 + m + 1]), f2(Y[8 + j0 - m - 1], Y[8 + j1 - m - 1]),
                 c0[h], k.rc[m], k.rc2[m], k.rh[1], k.rh2[1], g, l);
        Uy[j0] = g.x; Uy[j1] = g.y;
        Uyy[j0] = l.x; Uyy[j1] = l.y;
    }
    float2 gx[2] = {zero, zero}, lx[2] = {zero, zero};
#pragma unroll
    for (int m = 0; m < kRadius; ++m) {
        const float4 a = lds4(pc + rc + (m + 1) * kBoxY);
        const float4 b = lds4(pc + rc - (m + 1) * kBoxY);
        const float2 a2[2] = {f2(a.x, a.y), f2(a.z, a.w)}, b2[2] = {f2(b.x, b.y), f2(b.z, b.w)};
#pragma unroll
        for (int h = 0; h < 2; ++h)
            tap2(a2[h], b2[h], c0[h], k.rc[m], k.rc2[m], k.rh[0], k.rh2[0], gx[h], lx[h]);
    }
    Ux[0] = gx[0].x; Ux[1] = gx[0].y; Ux[2] = gx[1].x; Ux[3] = gx[1].y;
    Uxx[0] = lx[0].x; Uxx[1] = lx[0].y; Uxx[2] = lx[1].x; Uxx[3] = lx[1].y;
    float2 gz[2] = {zero, zero}, lz[2] = {zero, zero};
#pragma unroll
    for (int m = 0; m < kRadius; ++m) {
        const float *pp = ring + (size_t)slot_add(sc, m + 1) * slot_floats;
        const float *pm = ring + (size_t)slot_add(sc, -m - 1) * slot_floats;
        const float4 a = lds4(pp + rc);
        const float4 b = lds4(pm + rc);
        const float2 a2[2] = {f2(a.x, a.y), f2(a.z, a.w)}, b2[2] = {f2(b.x, b.y), f2(b.z, b.w)};
#pragma unroll
        for (int h = 0; h < 2; ++h)
            tap2(a2[h], b2[h], c0[h], k.rc[m], k.rc2[m], k.rh[2], k.rh2[2], gz[h], lz[h]);
    }
    Uz[0] = gz[0].x; Uz[1] = gz[0].y; Uz[2] = gz[1].x; Uz[3] = gz[1].y;
    Uzz[0] = lz[0].x; Uzz[1] = lz[0].y; Uzz[2] = lz[1].x; Uzz[3] = lz[1].y;
}

// First derivatives only, for the gradmax kernels.
__device__ __forceinline__ void quad_grad_ref(const float *ring, size_t slot_floats, int t, int rc,
                                              const Coefs &k, float Ux[4], float Uy[4],
                                              float Uz[4])
{
    const int sc = (t + kRadius) % kRing;
    const float *pc = ring + (size_t)sc * slot_floats;
    const float2 zero = make_float2(0.0f, 0.0f);
    float Y[20];
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        float4 v = lds4(pc + rc - 8 + 4 * b);
        Y[4 * b] = v.x; Y[4 * b + 1] = v.y; Y[4 * b + 2] = v.z; Y[4 * b + 3] = v.w;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j0 = 2 * h, j1 = 2 * h + 1;
        float2 g = zero;
#pragma unroll
        for (int m = 0; m < kRadius; ++m) {
            const float2 d = sub2(f2(Y[8 + j0 + m + 1], Y[8 + j1 + m + 1]),
                                  f2(Y[8 + j0 - m - 1], Y[8 + j1 - m - 1]));
            g = __fadd2_rn(g, div2(__fmul2_rn(k.rc[m], d), k.rh[1]));
        }
        Uy[j0] = g.x; Uy[j1] = g.y;
    }
    float2 gx[2] = {zero, zero}, gz[2] = {zero, zero};
#pragma unroll
    for (int m = 0; m < kRadius; ++m) {
        const float4 a = lds4(pc + rc + (m + 1) * kBoxY);
        const float4 b = lds4(pc + rc - (m + 1) * kBoxY);
        const float4 za = lds4(ring + (size_t)slot_add(sc, m + 1) * slot_floats + rc);
        const float4 zb = lds4(ring + (size_t)slot_add(sc, -m - 1) * slot_floats + rc);
        const float2 a2[2] = {f2(a.x, a.y), f2(a.z, a.w)}, b2[2] = {f2(b.x, b.y), f2(b.z, b.w)};
        const float2 za2[2] = {f2(za.x, za.y), f2(za.z, za.w)},
                     zb2[2] = {f2(zb.x, zb.y), f2(zb.z, zb.w)};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            gx[h] = __fadd2_rn(gx[h], div2(__fmul2_rn(k.rc[m], sub2(a2[h], b2[h])), k.rh[0]));
            gz[h] = __fadd2_rn(gz[h], div2(__fmul2_rn(k.rc[m], sub2(za2[h], zb2[h])), k.rh[2]));
        }
    }
    Ux[0] = gx[0].x; Ux[1] = gx[0].y; Ux[2] = gx[1].x; Ux[3] = gx[1].y;
    Uz[0] = gz[0].x; Uz[1] = gz[0].y; Uz[2] = gz[1].x; Uz[3] = gz[1].y;
}

// ---------------------------------------------------------------------------
// Plane pipeline.  Staged plane i of a chunk holds z = zfirst + i, in slot
// s = i % kRing.  full[s] completes when the TMA load of a plane into s has
// landed (one arrival + transaction bytes); empty[s] completes when every
// consumer warp has finished with the plane in s.  Plane i is last read by
// iteration t = i (as the z-5 tap of plane z = zfirst + i + 5), so warps
// release slot t % kRing after iteration t and thread 0 refills it with plane
// t + kRing.  No CTA-wide barrier in the plane loop.
// ---------------------------------------------------------------------------
struct Pipe {
    float *ring;
    uint64_t *full, *empty;
    size_t slot_floats;
    unsigned box_bytes;
    int nplanes;     // planes to stage for this chunk
    int zfirst;      // z of staged plane 0
    int c0, c1;      // TMA coordinates of the box (y, x)
    int ncw;         // consumer warps
    unsigned long long wait_ns;   // limit of every wait
    int hold;        // test hook: plane never issued (-1: none)
};

__device__ __forceinline__ void pipe_issue(const Pipe &P, const CUtensorMap *tm, int i)
{
    if (i == P.hold) return;   // test hook: the waits for this plane run out
    int s = i % kRing;
    mbar_arrive_expect_tx(&P.full[s], P.box_bytes);
    tma_load_3d(P.ring + (size_t)s * P.slot_floats, tm, P.c0, P.c1, P.zfirst + i, &P.full[s]);
}

__device__ __forceinline__ bool pipe_wait(const Pipe &P, int i)
{
    return mbar_wait_bounded(&P.full[i % kRing], (unsigned)((i / kRing) & 1), P.wait_ns);
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Consumer warp: release the slot of plane i.
__device__ __forceinline__ void pipe_release(const Pipe &P, int i)
{
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&P.empty[i % kRing]);
}

__device__ void pipe_init(const Pipe &P)
{
    for (int s = 0; s < kRing; ++s) {
        mbar_init(&P.full[s], 1);
        mbar_init(&P.empty[s], P.ncw);
    }
    fence_barrier_init();
    // a CTA that takes another tile reuses shared memory its threads read
    // and wrote (generic proxy) as TMA destination (async proxy)
    fence_proxy_async();
}

// Refills, done by thread 0 of the CTA (which also computes).  Before
// iteration t it issues every plane whose slot has been released, and blocks
// only for the plane iteration t needs (t + 10) -- i.e. only when some warp
// is more than two planes behind.  That wait needs planes <= t + 7, all
// issued earlier, so it cannot deadlock.  Returns false on a timed-out wait.
__device__ bool pipe_refill(const Pipe &P, const CUtensorMap *tm, int t, int &next_issue)
{
    while (next_issue < P.nplanes) {
        const int i = next_issue;
        uint64_t *e = &P.empty[i % kRing];
        const unsigned par = (unsigned)(((i - kRing) / kRing) & 1);
        if (i <= t + 2 * kRadius) {
            if (!mbar_wait_bounded(e, par, P.wait_ns)) return false;
        } else if (!mbar_try_wait(e, par)) {
            break;
        }
        fence_proxy_async();
        pipe_issue(P, tm, i);
        ++next_issue;
    }
    return true;
}

// After an aborted loop (thread 0): wait, bounded, for the loads still in
// flight so that none lands in shared memory after the CTA has exited.
__device__ void pipe_drain(const Pipe &P, int next_issue)
{
    for (int j = max(0, next_issue - kRing); j < next_issue; ++j) (void)pipe_wait(P, j);
}

__device__ __forceinline__ void pipe_setup(Pipe &P, unsigned char *smem, int tile_x, int pml,
                                           int y0, int x0, int z0, int nzc)
{
    const SmemLayout L = smem_layout(tile_x, pml);
    P.ring = reinterpret_cast<float *>(smem);
    P.full = reinterpret_cast<uint64_t *>(smem + L.bar_off);
    P.empty = P.full + kRing;
    P.slot_floats = L.slot_floats;
    P.box_bytes = (unsigned)((tile_x + 2 * kRadius) * kBoxY * 4);
    P.nplanes = nzc + 2 * kRadius;
    P.zfirst = z0 - kRadius;
    P.c0 = y0 - kHaloY;
    P.c1 = x0 - kRadius;
    P.ncw = blockDim.x >> 5;   // every warp of the CTA releases every slot
    P.wait_ns = 2000000000ull;
    P.hold = -1;
}

// The wait limit of the launch (0: 2 s) and the plane-withholding test hook,
// which applies to the first CTA of a grid launch only.
__device__ __forceinline__ void pipe_hooks(Pipe &P, const PlaneParams &p)
{
    if (p.wait_ns) P.wait_ns = p.wait_ns;
    if (p.hold_plane > 0 && (blockIdx.x | blockIdx.y | blockIdx.z) == 0) P.hold = p.hold_plane - 1;
}

__device__ __forceinline__ void pipe_setup(Pipe &P, unsigned char *smem, const PlaneParams &p,
                                           int y0, int x0, int z0, int nzc)
{
    pipe_setup(P, smem, p.tile_x, p.pml, y0, x0, z0, nzc);
    pipe_hooks(P, p);
}

// Before a CTA reuses its barriers for another tile (thread 0, after a CTA
// barrier; every load of the previous tile has been waited for).
__device__ void pipe_inval(const Pipe &P)
{
    for (int s = 0; s < kRing; ++s) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&P.full[s])) : "memory");
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&P.empty[s])) : "memory");
    }
}

// ---------------------------------------------------------------------------
// gradmax kernel.  With QUEUE the thread keeps its own column of the last 11
// planes in registers (loop unrolled by 11 so the queue never moves), which
// leaves 16 shared-memory vector loads per quad and plane instead of 25.
// ---------------------------------------------------------------------------
template <bool QUEUE, int AR>
__global__ void __launch_bounds__(kThreads, 2)
    qp3d_gradmax_kernel(const __grid_constant__ CUtensorMap tm_u, const PlaneParams p)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int q = tid & (kQuadsY - 1), r = tid / kQuadsY;
    const int y0 = blockIdx.x * kTileY, x0 = kRadius + blockIdx.y * p.tile_x;
    const int z0 = kRadius + blockIdx.z * p.chunk_z;
    const int z1 = min(z0 + p.chunk_z, p.nz - kRadius);
    if (z0 >= z1) return;
    const int nzc = z1 - z0;
    Pipe P;
    pipe_setup(P, smem, p, y0, x0, z0, nzc);
    int next_issue = 0;
    if (tid == 0) {
        pipe_init(P);
        next_issue = min(kRing, P.nplanes);
        for (int i = 0; i < next_issue; ++i) pipe_issue(P, &tm_u, i);
    }
    __syncthreads();
    const int x = x0 + r, yq = y0 + 4 * q;
    const bool row_ok = (r < p.tile_x) && (x < p.nx - kRadius);
    bool cell_ok[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) cell_ok[j] = row_ok && (yq + j >= kRadius) && (yq + j < p.ny - kRadius);
    const int rc = (r + kRadius) * kBoxY + kHaloY + 4 * q;
    const Coefs &k = p.k;

    float mx = 0.0f;
    bool ok = true;
    if (QUEUE) {
        float4 zq[2 * kRadius + 1];
#pragma unroll
        for (int i = 0; i < 2 * kRadius; ++i) {
            ok = ok && pipe_wait(P, i);
            zq[i] = lds4(P.ring + (size_t)(i % kRing) * P.slot_floats + rc);
        }
        for (int t0 = 0; t0 < nzc && ok; t0 += 2 * kRadius + 1) {
#pragma unroll
            for (int u = 0; u < 2 * kRadius + 1; ++u) {
                const int t = t0 + u;
                if (t >= nzc) break;
                if (tid == 0 && t >= kPrefetch + 1 && !pipe_refill(P, &tm_u, t, next_issue)) {
                    ok = false;
                    break;
                }
                if (!pipe_wait(P, t + 2 * kRadius)) {
                    ok = false;
                    break;
                }
                zq[(u + 2 * kRadius) % 11] =
                    lds4(P.ring + (size_t)((t + 2 * kRadius) % kRing) * P.slot_floats + rc);
                const float *pc = P.ring + (size_t)((t + kRadius) % kRing) * P.slot_floats;
                if (row_ok) {
                    float Ux[4], Uy[4], Uz[4];
                    float Y[20];
#pragma unroll
                    for (int b = 0; b < 5; ++b) {
                        float4 v = lds4(pc + rc - 8 + 4 * b);
                        Y[4 * b] = v.x; Y[4 * b + 1] = v.y; Y[4 * b + 2] = v.z; Y[4 * b + 3] = v.w;
                    }
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float g = 0.0f;
#pragma unroll
                        for (int m = 0; m < kRadius; ++m) {
                            float d = __fsub_rn(Y[8 + j + m + 1], Y[8 + j - m - 1]);
                            g = (m == 0) ? __fmul_rn(k.cy[0], d) : fmaf(k.cy[m], d, g);
                        }
                        Uy[j] = g;
                    }
#pragma unroll
                    for (int m = 0; m < kRadius; ++m) {
                        float4 a = lds4(pc + rc + (m + 1) * kBoxY);
                        float4 b = lds4(pc + rc - (m + 1) * kBoxY);
                        float4 za = zq[(u + kRadius + m + 1) % 11];
                        float4 zb = zq[(u + kRadius - m - 1 + 11) % 11];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            float dx_ = __fsub_rn(f4(a, j), f4(b, j));
                            float dz_ = __fsub_rn(f4(za, j), f4(zb, j));
                            Ux[j] = (m == 0) ? __fmul_rn(k.cx[0], dx_) : fmaf(k.cx[m], dx_, Ux[j]);
                            Uz[j] = (m == 0) ? __fmul_rn(k.cz[0], dz_) : fmaf(k.cz[m], dz_, Uz[j]);
                        }
                    }
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (cell_ok[j])
                            mx = fmaxf(mx, fmaxf(fabsf(Ux[j]), fmaxf(fabsf(Uy[j]), fabsf(Uz[j]))));
                }
                pipe_release(P, t);
            }
        }
    } else {
        int waited = 0;
        for (int t = 0; t < nzc; ++t) {
            if (tid == 0 && t >= kPrefetch + 1 && !pipe_refill(P, &tm_u, t, next_issue)) {
                ok = false;
                break;
            }
            while (ok && waited <= t + 2 * kRadius) {
                ok = pipe_wait(P, waited);
                if (ok) ++waited;
            }
            if (!ok) break;
            if (row_ok) {
                float Ux[4], Uy[4], Uz[4], Uxx[4], Uyy[4], Uzz[4], u0[4];
                if (AR == kArithRef)
                    quad_grad_ref(P.ring, P.slot_floats, t, rc, k, Ux, Uy, Uz);
                else
                    quad_derivs<false>(P.ring, P.slot_floats, t, rc, k, Ux, Uy, Uz, Uxx, Uyy,
                                       Uzz, u0);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (cell_ok[j])
                        mx = fmaxf(mx, fmaxf(fabsf(Ux[j]), fmaxf(fabsf(Uy[j]), fabsf(Uz[j]))));
            }
            pipe_release(P, t);
        }
    }
    if (!ok) {
        atomicOr(p.err, kErrWaitTimeout);
        if (tid == 0) pipe_drain(P, next_issue);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0 && mx > 0.0f)
        atomicMax(reinterpret_cast<unsigned *>(p.gmax + p.step), __float_as_uint(mx));
}

// ---------------------------------------------------------------------------
// gradmax of one tile column [z0, z1) for the batched launches: the
// arithmetic of qp3d_gradmax_kernel<false>.  With REUSE the CTA's barriers
// are invalidated at the end so that it can take another tile; the return
// value (false: a wait timed out) is then the same in every thread.
// ---------------------------------------------------------------------------
template <bool REUSE, int AR = kArithFast>
__device__ __forceinline__ bool gradmax_tile(const CUtensorMap *tm, const PlaneParams &p,
                                             const Coefs &k, int tile_x, int y0, int x0, int z0,
                                             int z1, unsigned char *smem)
{
    const int tid = threadIdx.x;
    const int q = tid & (kQuadsY - 1), r = tid / kQuadsY;
    const int nzc = z1 - z0;
    Pipe P;
    pipe_setup(P, smem, tile_x, p.pml, y0, x0, z0, nzc);
    if (!REUSE) pipe_hooks(P, p);
    int next_issue = 0;
    if (tid == 0) {
        pipe_init(P);
        next_issue = min(kRing, P.nplanes);
        for (int i = 0; i < next_issue; ++i) pipe_issue(P, tm, i);
    }
    __syncthreads();
    const int x = x0 + r, yq = y0 + 4 * q;
    const bool row_ok = (r < tile_x) && (x < p.nx - kRadius);
    bool cell_ok[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) cell_ok[j] = row_ok && (yq + j >= kRadius) && (yq + j < p.ny - kRadius);
    const int rc = (r + kRadius) * kBoxY + kHaloY + 4 * q;
    float mx = 0.0f;
    bool ok = true;
    int waited = 0;
    for (int t = 0; t < nzc; ++t) {
        if (tid == 0 && t >= kPrefetch + 1 && !pipe_refill(P, tm, t, next_issue)) ok = false;
        while (ok && waited <= t + 2 * kRadius) {
            ok = pipe_wait(P, waited);
            if (ok) ++waited;
        }
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
        if (row_ok) {
            float Ux[4], Uy[4], Uz[4], Uxx[4], Uyy[4], Uzz[4], u0[4];
            if (AR == kArithRef)
                quad_grad_ref(P.ring, P.slot_floats, t, rc, k, Ux, Uy, Uz);
            else
                quad_derivs<false>(P.ring, P.slot_floats, t, rc, k, Ux, Uy, Uz, Uxx, Uyy, Uzz, u0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (cell_ok[j])
                    mx = fmaxf(mx, fmaxf(fabsf(Ux[j]), fmaxf(fabsf(Uy[j]), fabsf(Uz[j]))));
        }
        pipe_release(P, t);
    }
    if (!ok) {
        atomicOr(p.err, kErrWaitTimeout);
        if (tid == 0) pipe_drain(P, next_issue);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0 && mx > 0.0f)
        atomicMax(reinterpret_cast<unsigned *>(p.gmax + p.step), __float_as_uint(mx));
    if (REUSE) {
        ok = __syncthreads_and(ok) != 0;
        if (tid == 0 && ok) pipe_inval(P);
    }
    return ok;
}

// ---------------------------------------------------------------------------
// gradmax with per-CTA partial results: the same staging and arithmetic as
// qp3d_gradmax_kernel<false>, but each CTA writes its own maximum to
// partial[linear CTA index] (every CTA writes its slot, also when it has no
// cell), for callers that supply the partial array themselves.
// ---------------------------------------------------------------------------
template <int AR>
__global__ void __launch_bounds__(kThreads, 2)
    qp3d_gradmax_partial_kernel(const __grid_constant__ CUtensorMap tm_u, const PlaneParams p,
                                float *partial)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ float wmax[kThreads / 32];
    const int tid = threadIdx.x;
    const unsigned cta = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int q = tid & (kQuadsY - 1), r = tid / kQuadsY;
    const int y0 = blockIdx.x * kTileY, x0 = kRadius + blockIdx.y * p.tile_x;
    const int z0 = kRadius + blockIdx.z * p.chunk_z;
    const int z1 = min(z0 + p.chunk_z, p.nz - kRadius);
    if (z0 >= z1) {
        if (tid == 0) partial[cta] = 0.0f;
        return;
    }
    const int nzc = z1 - z0;
    Pipe P;
    pipe_setup(P, smem, p, y0, x0, z0, nzc);
    int next_issue = 0;
    if (tid == 0) {
        pipe_init(P);
        next_issue = min(kRing, P.nplanes);
        for (int i = 0; i < next_issue; ++i) pipe_issue(P, &tm_u, i);
    }
    __syncthreads();
    const int x = x0 + r, yq = y0 + 4 * q;
    const bool row_ok = (r < p.tile_x) && (x < p.nx - kRadius);
    bool cell_ok[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) cell_ok[j] = row_ok && (yq + j >= kRadius) && (yq + j < p.ny - kRadius);
    const int rc = (r + kRadius) * kBoxY + kHaloY + 4 * q;
    float mx = 0.0f;
    bool ok = true;
    int waited = 0;
    for (int t = 0; t < nzc; ++t) {
        if (tid == 0 && t >= kPrefetch + 1 && !pipe_refill(P, &tm_u, t, next_issue)) ok = false;
        while (ok && waited <= t + 2 * kRadius) {
            ok = pipe_wait(P, waited);
            if (ok) ++waited;
        }
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
        if (row_ok) {
            float Ux[4], Uy[4], Uz[4], Uxx[4], Uyy[4], Uzz[4], u0[4];
            if (AR == kArithRef)
                quad_grad_ref(P.ring, P.slot_floats, t, rc, p.k, Ux, Uy, Uz);
            else
                quad_derivs<false>(P.ring, P.slot_floats, t, rc, p.k, Ux, Uy, Uz, Uxx, Uyy, Uzz,
                                   u0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (cell_ok[j])
                    mx = fmaxf(mx, fmaxf(fabsf(Ux[j]), fmaxf(fabsf(Uy[j]), fabsf(Uz[j]))));
        }
        pipe_release(P, t);
    }
    if (!ok) {
        atomicOr(p.err, kErrWaitTimeout);
        if (tid == 0) pipe_drain(P, next_issue);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) wmax[tid / 32] = mx;
    __syncthreads();
    if (tid == 0) {
        float m = 0.0f;
        for (int w = 0; w < (int)blockDim.x / 32; ++w) m = fmaxf(m, wmax[w]);
        partial[cta] = m;
    }
}

// One block: out[0] = max(partial[0..n)), or NaN when *err is set.
__global__ void qp3d_reduce_max_kernel(const float *partial, unsigned n, const unsigned *err,
                                       float *out)
{
    __shared__ float wmax[32];
    float m = 0.0f;
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, partial[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x / 32] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = 0.0f;
        for (int w = 0; w < (int)blockDim.x / 32; ++w) r = fmaxf(r, wmax[w]);
        out[0] = (err && *err) ? __int_as_float(0x7fc00000) : r;
    }
}

// ---------------------------------------------------------------------------
// PML update of one cell (GPU_kernel.cu:566-637 restated with per-layer
// coefficients a1 = (d*dt+1)^2-3, a2 = 2*d*dt-1, a3 = 1-dt*d).  Face codes
// L=0 R=1 F=2 Bk=3 T=4 Bo=5; the odd faces take the minus sign on the
// dd*u_n term.  Written with selects only.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pml_cell(int f, float4 lc, float KS, float e2, float Ux,
                                          float Uy, float Uz, float Uxx, float Uyy, float Uzz,
                                          float dt, float w11, float w12, float w21, float w31,
                                          float w32, float p1, float p2, float &nw13,
                                          float &nw21, float &nw33, float &np3)
{
    const bool isx = f < 2, isz = f >= 4;
    const float e2KS = __fmul_rn(e2, KS);
    const float A = isz ? KS : e2KS;
    const float Unn = isx ? Uxx : (isz ? Uzz : Uyy);
    const float Un = isx ? Ux : (isz ? Uz : Uy);
    const float Bt = isz ? e2KS : KS;
    const float Tt = isz ? __fadd_rn(Uxx, Uyy) : fmaf(e2, isx ? Uyy : Uxx, Uzz);
    const float a1 = lc.x, a2 = lc.y, a3 = lc.z, dd = lc.w;
    nw13 = fmaf(A, Unn, fmaf(-a1, w12, __fmul_rn(a2, w11)));
    float Ad = __fmul_rn(A, dd);
    Ad = (f & 1) ? -Ad : Ad;
    np3 = fmaf(Ad, Un, fmaf(-a1, p2, __fmul_rn(a2, p1)));
    nw21 = fmaf(dt, np3, __fmul_rn(a3, w21));
    nw33 = fmaf(Bt, Tt, fmaf(2.0f, w32, -w31));
    return __fadd_rn(__fadd_rn(nw13, nw21), nw33);
}

// The same update with two scalar operators, KS and KS1 (S = 1): the terms
// that do not depend on S are shared, and each result equals pml_cell's with
// that operator bit for bit.  The second set of outputs goes to a1x.
__device__ __forceinline__ float pml_cell2(int f, float4 lc, float KS, float KS1, float e2,
                                           float Ux, float Uy, float Uz, float Uxx, float Uyy,
                                           float Uzz, float dt, float w11, float w12, float w21,
                                           float w31, float w32, float p1, float p2,
                                           float &nw13, float &nw21, float &nw33, float &np3,
                                           float &v1, float4 &a1x)
{
    const bool isx = f < 2, isz = f >= 4;
    const float Unn = isx ? Uxx : (isz ? Uzz : Uyy);
    const float Un = isx ? Ux : (isz ? Uz : Uy);
    const float Tt = isz ? __fadd_rn(Uxx, Uyy) : fmaf(e2, isx ? Uyy : Uxx, Uzz);
    const float a1 = lc.x, a2 = lc.y, a3 = lc.z, dd = lc.w;
    const float X1 = fmaf(-a1, w12, __fmul_rn(a2, w11));
    const float X2 = fmaf(-a1, p2, __fmul_rn(a2, p1));
    const float X3 = fmaf(2.0f, w32, -w31);
    const float W = __fmul_rn(a3, w21);
    float out[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const float ks = s ? KS1 : KS;
        const float e2KS = __fmul_rn(e2, ks);
        const float A = isz ? ks : e2KS, Bt = isz ? e2KS : ks;
        float Ad = __fmul_rn(A, dd);
        Ad = (f & 1) ? -Ad : Ad;
        const float n13 = fmaf(A, Unn, X1), n3 = fmaf(Ad, Un, X2);
        const float n21 = fmaf(dt, n3, W), n33 = fmaf(Bt, Tt, X3);
        out[s] = __fadd_rn(__fadd_rn(n13, n21), n33);
        if (s) a1x = make_float4(n13, n21, n33, n3);
        else nw13 = n13, nw21 = n21, nw33 = n33, np3 = n3;
    }
    v1 = out[1];
    return out[0];
}

__device__ __forceinline__ float4 ldg4(const float *p)
{
    return __ldg(reinterpret_cast<const float4 *>(p));
}

__device__ __forceinline__ float4 ld4(const float *p)
{
    return *reinterpret_cast<const float4 *>(p);
}

// Face code and layer index of a cell from its x/y/z face parts (-1: none),
// in the reference's priority order.
__device__ __forceinline__ void cell_face(int fx, int lix, int fy, int liy, int fz, int liz,
                                          int &f, int &li)
{
    f = fx >= 0 ? fx : (fy >= 0 ? fy : fz);
    li = fx >= 0 ? lix : (fy >= 0 ? liy : liz);
}

// ---------------------------------------------------------------------------
// step kernel.
//   SPEC = false ("exact"): the threshold comes from gmax[step], already
//     known (gradmax kernel, or a speculative pass of the same step).  With a
//     gate the kernel runs only when *gate != 0 (the re-run of a step whose
//     speculation failed).
//   SPEC = true: the max of the step is not known yet.  It is predicted from
//     the two previous steps with a window [M_lo, M_hi]; a cell whose m2 lies
//     in (T2(M_lo), T2(M_hi)] has an uncertain decision: the kernel computes
//     it as "above", marks it in the deferred-cell bitmask with its m2 and
//     S = 1 value, and reduces the true max of the step into gmax[step] on
//     the way.  The resolution, compaction and fix-up kernels then give the
//     S = 1 result to the marked cells that turn out to be below the
//     threshold, or ask for the exact re-run when the max fell outside the
//     window.  The step never overwrites its inputs, so both are possible.
//     Both modes write bit-identical results.
// ---------------------------------------------------------------------------
__device__ void spec_window(const PlaneParams &p, float &lo, float &hi, float &pred)
{
    const int k = p.step;
    const float m1 = k >= 1 ? p.gmax[k - 1] : 0.0f;
    const float m0 = k >= 2 ? p.gmax[k - 2] : 0.0f;
    float r = (m0 > 0.0f) ? __fdiv_rn(m1, m0) : 1.0f;
    r = fminf(fmaxf(r, 0.5f), 2.0f);
    // half the last trend: late in a shot the max moves by a few tenths of a
    // percent per step with changing sign, which a full extrapolation doubles
    pred = __fmul_rn(m1, fmaf(0.5f, __fsub_rn(r, 1.0f), 1.0f));
    // cover both "the max keeps its trend" and "the max stays where it was",
    // widened by 1.5x the largest of the recent prediction errors
    float e = 0.0f;
#pragma unroll
    for (int i = 0; i < kSpecHist; ++i) e = fmaxf(e, p.spec_err[i]);
    const float d = fminf(0.25f, fmaxf(p.delta_min, __fmul_rn(1.5f, e)));
    lo = __fmul_rn(fminf(pred, m1), __fsub_rn(1.0f, d));
    hi = __fmul_rn(fmaxf(pred, m1), __fadd_rn(1.0f, d));
    if (p.spec_bias != 0.0f) {   // test hook: a window that misses on purpose
        lo = __fmul_rn(lo, __fadd_rn(1.0f, p.spec_bias));
        hi = __fmul_rn(hi, __fadd_rn(1.0f, p.spec_bias));
    }
}

// 1/x for normal positive x, within about 1 ulp: Newton-Raphson steps
// r <- r + r (1 - x r) from an initial guess that negates the exponent of x in
// its integer representation (the integer-subtraction trick known from the
// fast inverse square root).  Three steps take the guess's ~12% error below
// float rounding.  About a third of the instructions of an IEEE division,
// which dominated the scalar operator once most cells are above the
// threshold; the mirror oracle performs the same operations:
//   r = bits(0x7EF311C3 - bits(x)); 3 x { e = fma(-x, r, 1); r = fma(r, e, r) }
// Two cells at a time with the packed FP32x2 instructions (round-to-nearest
// per lane: each lane performs the scalar operations above).
__device__ __forceinline__ float2 rcp_nr2(float2 x)
{
    float2 r = make_float2(__uint_as_float(0x7EF311C3u - __float_as_uint(x.x)),
                           __uint_as_float(0x7EF311C3u - __float_as_uint(x.y)));
    const float2 nx = make_float2(-x.x, -x.y), one = make_float2(1.0f, 1.0f);
#pragma unroll
    for (int it = 0; it < 3; ++it) {
        const float2 e = __ffma2_rn(nx, r, one);
        r = __ffma2_rn(r, e, r);
    }
    return r;
}

// S of two cells (GPU_kernel.cu:100-111), given they are above the threshold.
// With a = (nx^2 + ny^2) = h2/m2, nz^2 = 1 - a = v2/m2 (v2 = Uz^2),
// S = 1/2 + 1/2 sqrt(1 - 8(eps-delta) a (1-a) / (1 + 2 eps a)^2)
//   = 1/2 + 1/2 sqrt(1 - 8(eps-delta) (h2 r) (v2 r)),  r = 1 / (m2 + 2 eps h2):
// one reciprocal per cell, and both factors h2 r, v2 r lie in [0, 1].
__device__ __forceinline__ float2 aniso_s2(float2 h2, float2 m2, float2 v2, float2 e2x, float2 r8)
{
    const float2 one = make_float2(1.0f, 1.0f), half = make_float2(0.5f, 0.5f);
    const float2 r = rcp_nr2(__ffma2_rn(e2x, h2, m2));
    const float2 qq = __fmul2_rn(__fmul2_rn(r8, __fmul2_rn(h2, r)), __fmul2_rn(v2, r));
    const float2 t = __fadd2_rn(one, make_float2(-qq.x, -qq.y));
    return __ffma2_rn(half, make_float2(__fsqrt_rn(t.x), __fsqrt_rn(t.y)), half);
}

// Per-cell parameters of a quad from half-precision vp, eps, delta, with the
// operations of qp3d_params_dense_kernel: vp, 2 eps, 8 (eps - delta).
__device__ __forceinline__ void quad_params_half(uint2 hv, uint2 he, uint2 hd, float4 &V,
                                                 float4 &E2, float4 &R8)
{
    const float2 v0 = __half22float2(*reinterpret_cast<const __half2 *>(&hv.x));
    const float2 v1 = __half22float2(*reinterpret_cast<const __half2 *>(&hv.y));
    const float2 e0 = __half22float2(*reinterpret_cast<const __half2 *>(&he.x));
    const float2 e1 = __half22float2(*reinterpret_cast<const __half2 *>(&he.y));
    const float2 d0 = __half22float2(*reinterpret_cast<const __half2 *>(&hd.x));
    const float2 d1 = __half22float2(*reinterpret_cast<const __half2 *>(&hd.y));
    const float ep[4] = {e0.x, e0.y, e1.x, e1.y}, de[4] = {d0.x, d0.y, d1.x, d1.y};
    float e[4], r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        e[j] = __fmul_rn(2.0f, ep[j]);
        r[j] = __fmul_rn(8.0f, __fsub_rn(ep[j], de[j]));
    }
    V = make_float4(v0.x, v0.y, v1.x, v1.y);
    E2 = make_float4(e[0], e[1], e[2], e[3]);
    R8 = make_float4(r[0], r[1], r[2], r[3]);
}

// (vp dt)^2 of the fast arithmetic
__device__ __forceinline__ float k_of_vp(float vp, float dt)
{
    const float vdt = __fmul_rn(vp, dt);
    return __fmul_rn(vdt, vdt);
}

// The fast arithmetic's layer coefficients from the stored (a1h, a1l, d*dt, dd):
// a1 = RN(a1h + a1l) = a1h, a2 = 2*d*dt - 1, a3 = 1 - d*dt.
__device__ __forceinline__ float4 fast_layer(float4 t)
{
    return make_float4(t.x, __fmaf_rn(2.0f, t.z, -1.0f), __fsub_rn(1.0f, t.z), t.w);
}

// One tile column [z0, z1) of the step.  The grid kernel below runs one per
// CTA; the batched kernel runs many per CTA (REUSE: barriers invalidated at
// the end, return value uniform over the CTA; false = a wait timed out).
// AR: kArithRef (the reference CPU operators' roundings, qp3d_exact.h) or
// kArithFast (folded coefficients, fused multiply-adds, one reciprocal in S).
template <bool SPEC, bool REUSE, bool HALF = false, int AR = kArithFast>
__device__ __forceinline__ bool step_tile(const CUtensorMap *tm, const PlaneParams &p,
                                          const Coefs &k, int tile_x, int y0, int x0, int z0,
                                          int z1, bool win_writer, unsigned char *smem)
{
    const SmemLayout L = smem_layout(tile_x, p.pml, p.nsrc);
    float4 *tab = reinterpret_cast<float4 *>(smem + L.tab_off);
    SrcEntry *csrc = reinterpret_cast<SrcEntry *>(smem + L.src_off);
    float *misc = reinterpret_cast<float *>(smem + L.misc_off);
    int *misc_i = reinterpret_cast<int *>(smem + L.misc_off + 16);

    const int tid = threadIdx.x, lane = tid & 31;
    const int q = tid & (kQuadsY - 1), r = tid / kQuadsY;
    const int nzc = z1 - z0;
    Pipe P;
    pipe_setup(P, smem, tile_x, p.pml, y0, x0, z0, nzc);
    if (!REUSE) pipe_hooks(P, p);
    const int nx = p.nx, ny = p.ny, nz = p.nz, pml = p.pml;
    int next_issue = 0;
    if (tid == 0) {
        pipe_init(P);
        next_issue = min(kRing, P.nplanes);
        for (int i = 0; i < next_issue; ++i) pipe_issue(P, tm, i);
        if (SPEC) {
            float lo, hi, pred;
            spec_window(p, lo, hi, pred);
            misc[0] = threshold_m2(lo);
            misc[1] = threshold_m2(hi);
            if (win_writer) {
                p.win[0] = lo;
                p.win[1] = hi;
                p.win[2] = pred;
            }
        } else {
            misc[0] = misc[1] = threshold_m2(p.gmax[p.step]);
        }
        int n = 0;
        for (int e = 0; e < p.nsrc; ++e) {
            SrcEntry s = p.src[e];
            if (s.x >= x0 && s.x < x0 + tile_x && s.y >= y0 && s.y < y0 + kTileY && s.z >= z0 &&
                s.z < z1 && n < p.nsrc)
                csrc[n++] = s;
        }
        misc_i[0] = n;
    }
    for (int i = tid; i < 3 * pml; i += blockDim.x) tab[i] = p.layers[i];
    __syncthreads();
    const float T2lo = misc[0], T2hi = misc[1];
    const int ncsrc = misc_i[0];

    const int x = x0 + r, yq = y0 + 4 * q;
    const bool row_ok = (r < tile_x) && (x < nx - kRadius);
    // quads wholly in the row padding (y >= ny, the last y tile) neither load
    // nor store: their cells are not part of the volume
    const bool mem_ok = row_ok && (yq < ny);
    bool cell_ok[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) cell_ok[j] = row_ok && (yq + j >= kRadius) && (yq + j < ny - kRadius);
    const int rc = (r + kRadius) * kBoxY + kHaloY + 4 * q;
    // x and y face parts, constant along z
    const int fx = x < pml ? 0 : (x >= nx - pml ? 1 : -1);
    const int lix = x < pml ? pml - x : x - nx + pml;
    int fy[4], liy[4];
    bool any_fy = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int y = yq + j;
        fy[j] = y < pml ? 2 : (y >= ny - pml ? 3 : -1);
        liy[j] = y < pml ? pml - y : y - ny + pml;
        any_fy = any_fy || (cell_ok[j] && fy[j] >= 0);
    }
    const bool xy_face = row_ok && (fx >= 0 || any_fy);
    const int hy = ny - 2 * pml;
    const float dt = p.dt;
    const float dt2 = __fmul_rn(dt, dt);
    // the reference adds source * wavelet to every cell (CPU_function.c:326-338):
    // a cell without a source gets +-0, which turns a -0 into +0 when the
    // product is +0
    const float zw = __fmul_rn(0.0f, p.wavelet);
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);

    float mx = 0.0f;
    bool ok = true;
    int waited = 0;
    long long base = (long long)z0 * p.plane + (long long)x * p.ldy + yq;
    for (int t = 0; t < nzc; ++t, base += p.plane) {
        const int z = z0 + t;
        const int fz = z < pml ? 4 : (z >= nz - pml ? 5 : -1);
        const int liz = z < pml ? pml - z : z - nz + pml;
        const bool pml_quad = xy_face || (row_ok && fz >= 0);
        float4 u1v = zero4, Vv = zero4, Ev = zero4, Rv = zero4;
        uint2 hv = make_uint2(0u, 0u), he = hv, hd = hv;
        if (mem_ok) {
            u1v = ldg4(p.u_prev + base);
            if (HALF) {   // widened after the stencil, when the loads have landed
                hv = __ldg(reinterpret_cast<const uint2 *>(p.h_vp + base));
                he = __ldg(reinterpret_cast<const uint2 *>(p.h_eps + base));
                hd = __ldg(reinterpret_cast<const uint2 *>(p.h_del + base));
            } else {
                Vv = ldg4(p.prm_v + base);
                Ev = ldg4(p.prm_e + base);
                Rv = ldg4(p.prm_r + base);
            }
        }
        float4 w11 = zero4, w12 = zero4, w31 = zero4, w32 = zero4, p1 = zero4, p2 = zero4,
               w21 = zero4;
        if (pml_quad && mem_ok) {
            w11 = ldg4(p.w1o + base); w12 = ldg4(p.w1c + base);
            w31 = ldg4(p.w3o + base); w32 = ldg4(p.w3c + base);
            p1 = ldg4(p.po + base);   p2 = ldg4(p.pc + base);
            w21 = ldg4(p.w21o + base);
        }
        if (tid == 0 && t >= kPrefetch + 1 && !pipe_refill(P, tm, t, next_issue)) ok = false;
        while (ok && waited <= t + 2 * kRadius) {
            ok = pipe_wait(P, waited);
            if (ok) ++waited;
        }
        ok = __all_sync(0xffffffffu, ok);   // warps stay converged for the collectives below
        if (!ok) break;
        float Ux[4], Uy[4], Uz[4], Uxx[4], Uyy[4], Uzz[4], u0[4];
        if (AR == kArithRef)
            quad_derivs_ref(P.ring, P.slot_floats, t, rc, k, Ux, Uy, Uz, Uxx, Uyy, Uzz, u0);
        else
            quad_derivs<true>(P.ring, P.slot_floats, t, rc, k, Ux, Uy, Uz, Uxx, Uyy, Uzz, u0);
        if (HALF) quad_params_half(hv, he, hd, Vv, Ev, Rv);
        // scalar operator, GPU_kernel.cu:93-111 / CPU_function.c:339-370
        float h2[4], m2[4];
        bool above[4], amb[4];
        bool any_above = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (AR == kArithRef) {
                m2[j] = xr::grad_m2(Ux[j], Uy[j], Uz[j]);
                h2[j] = 0.0f;
            } else {
                h2[j] = fmaf(Uy[j], Uy[j], __fmul_rn(Ux[j], Ux[j]));
                m2[j] = fmaf(Uz[j], Uz[j], h2[j]);
            }
            if (SPEC && cell_ok[j]) {   // three-input max: one instruction fewer per cell
                float t;
                asm("max.f32 %0, %1, %2, %3;" : "=f"(t) : "f"(mx), "f"(fabsf(Ux[j])), "f"(fabsf(Uy[j])));
                mx = fmaxf(t, fabsf(Uz[j]));
            }
            above[j] = m2[j] > T2lo;
            if (!SPEC && p.dec_in && row_ok) above[j] = (p.dec_in[base >> 5] >> (4 * q + j)) & 1u;
            amb[j] = SPEC && cell_ok[j] && above[j] && !(m2[j] > T2hi);
            any_above = any_above || (row_ok && above[j]);
        }
        float S[4], e1[4];   // S; 1 + 2 eps
        float KS[4];         // fast arithmetic: (vp dt)^2 S
#pragma unroll
        for (int j = 0; j < 4; ++j) e1[j] = __fadd_rn(1.0f, f4(Ev, j));
        if (AR == kArithRef) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                S[j] = 1.0f;
                if (cell_ok[j] && above[j])
                    S[j] = xr::scalar_s(Ux[j], Uy[j], Uz[j], m2[j], f4(Ev, j), f4(Rv, j));
            }
        } else if (__any_sync(0xffffffffu, any_above)) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {   // cells (0,1) and (2,3) as pairs
                const int j0 = 2 * h, j1 = 2 * h + 1;
                const float2 s = aniso_s2(make_float2(h2[j0], h2[j1]), make_float2(m2[j0], m2[j1]),
                                          __fmul2_rn(make_float2(Uz[j0], Uz[j1]),
                                                     make_float2(Uz[j0], Uz[j1])),
                                          make_float2(f4(Ev, j0), f4(Ev, j1)),
                                          make_float2(f4(Rv, j0), f4(Rv, j1)));
                KS[j0] = __fmul_rn(k_of_vp(f4(Vv, j0), dt), above[j0] ? s.x : 1.0f);
                KS[j1] = __fmul_rn(k_of_vp(f4(Vv, j1), dt), above[j1] ? s.y : 1.0f);
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) KS[j] = __fmul_rn(k_of_vp(f4(Vv, j), dt), 1.0f);
        }
        float out[4], alt[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (AR == kArithRef) {
                out[j] = xr::interior_update(u0[j], f4(u1v, j), Uxx[j], Uyy[j], Uzz[j], e1[j],
                                             S[j], f4(Vv, j), dt2);
                alt[j] = xr::interior_update(u0[j], f4(u1v, j), Uxx[j], Uyy[j], Uzz[j], e1[j],
                                             1.0f, f4(Vv, j), dt2);   // S = 1, deferred cells
            } else {
                const float Lp = fmaf(e1[j], __fadd_rn(Uxx[j], Uyy[j]), Uzz[j]);
                const float lin = fmaf(2.0f, u0[j], -f4(u1v, j));
                out[j] = fmaf(KS[j], Lp, lin);
                alt[j] = fmaf(__fmul_rn(k_of_vp(f4(Vv, j), dt), 1.0f), Lp, lin);
            }
        }
        if (__any_sync(0xffffffffu, pml_quad)) {
            float n13[4], n21[4], n33[4], n3[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int f, li;
                cell_face(fx, lix, fy[j], liy[j], fz, liz, f, li);
                const bool is_pml = pml_quad && cell_ok[j] && f >= 0;
                const float4 lt = tab[is_pml ? (f >> 1) * pml + li : 0];
                if (AR == kArithRef) {
                    n13[j] = n33[j] = n3[j] = 0.0f;
                    n21[j] = f4(w21, j);
                    if (is_pml) {
                        const bool isx = f < 2, isz = f >= 4;
                        xr::PmlLayer Lr;
                        Lr.a1h = lt.x; Lr.a1l = lt.y;
                        Lr.a2 = __fmaf_rn(2.0f, lt.z, -1.0f);
                        Lr.a3 = __fsub_rn(1.0f, lt.z);
                        Lr.dd = lt.w;
                        const float Unn = isx ? Uxx[j] : (isz ? Uzz[j] : Uyy[j]);
                        const float Un = isx ? Ux[j] : (isz ? Uz[j] : Uy[j]);
                        const float tang = isz ? __fadd_rn(Uxx[j], Uyy[j])
                                               : __fadd_rn(Uzz[j], __fmul_rn(e1[j], isx ? Uyy[j] : Uxx[j]));
                        const float vdt = __fmul_rn(f4(Vv, j), dt);
                        const xr::PmlOut o = xr::pml_update(isz, (f & 1) != 0, S[j], e1[j], vdt,
                                                            Unn, Un, tang, dt, Lr, f4(w11, j),
                                                            f4(w12, j), f4(w21, j), f4(w31, j),
                                                            f4(w32, j), f4(p1, j), f4(p2, j));
                        out[j] = o.u3;
                        n13[j] = o.w13; n21[j] = o.w21; n33[j] = o.w33; n3[j] = o.p3;
                        if (SPEC && amb[j]) {   // the S = 1 update, kept for the fix-up
                            const xr::PmlOut o1 = xr::pml_update(isz, (f & 1) != 0, 1.0f, e1[j],
                                                                 vdt, Unn, Un, tang, dt, Lr,
                                                                 f4(w11, j), f4(w12, j),
                                                                 f4(w21, j), f4(w31, j),
                                                                 f4(w32, j), f4(p1, j), f4(p2, j));
                            alt[j] = o1.u3;
                            p.apml[base + j] = make_float4(o1.w13, o1.w21, o1.w33, o1.p3);
                        }
                    }
                } else {
                    const float4 lc = fast_layer(lt);
                    const float v = pml_cell(f < 0 ? 0 : f, lc, KS[j], e1[j], Ux[j], Uy[j], Uz[j],
                                             Uxx[j], Uyy[j], Uzz[j], dt, f4(w11, j), f4(w12, j),
                                             f4(w21, j), f4(w31, j), f4(w32, j), f4(p1, j),
                                             f4(p2, j), n13[j], n21[j], n33[j], n3[j]);
                    if (SPEC && is_pml && amb[j]) {
                        // the S = 1 update of a deferred cell and its split-field
                        // outputs, kept for the fix-up
                        float a13, a21, a33, a3;
                        alt[j] = pml_cell(f, lc, __fmul_rn(k_of_vp(f4(Vv, j), dt), 1.0f), e1[j],
                                          Ux[j], Uy[j], Uz[j], Uxx[j], Uyy[j], Uzz[j], dt,
                                          f4(w11, j), f4(w12, j), f4(w21, j), f4(w31, j),
                                          f4(w32, j), f4(p1, j), f4(p2, j), a13, a21, a33, a3);
                        p.apml[base + j] = make_float4(a13, a21, a33, a3);
                    }
                    out[j] = is_pml ? v : out[j];
                    n13[j] = is_pml ? n13[j] : 0.0f;
                    n33[j] = is_pml ? n33[j] : 0.0f;
                    n3[j] = is_pml ? n3[j] : 0.0f;
                    n21[j] = is_pml ? n21[j] : f4(w21, j);
                }
            }
            if (pml_quad && mem_ok) {
                *reinterpret_cast<float4 *>(p.w1n + base) = make_float4(n13[0], n13[1], n13[2], n13[3]);
                *reinterpret_cast<float4 *>(p.w3n + base) = make_float4(n33[0], n33[1], n33[2], n33[3]);
                *reinterpret_cast<float4 *>(p.pn + base) = make_float4(n3[0], n3[1], n3[2], n3[3]);
                *reinterpret_cast<float4 *>(p.w21n + base) = make_float4(n21[0], n21[1], n21[2], n21[3]);
            }
        }
        // source injection (GPU_kernel.cu:727, CPU_function.c:334): u3 += source * wavelet
        bool has_src[4] = {false, false, false, false};
        for (int e = 0; e < ncsrc; ++e) {
            const SrcEntry s = csrc[e];
            if (s.z == z && s.x == x) {
                const int js = s.y - yq;
                const float add = __fmul_rn(s.v, p.wavelet);
#pragma unroll
                for (int jj = 0; jj < 4; ++jj)
                    if (jj == js) {
                        out[jj] = __fadd_rn(out[jj], add);
                        alt[jj] = __fadd_rn(alt[jj], add);
                        has_src[jj] = true;
                    }
            }
        }
        if (AR == kArithRef) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (!has_src[j]) {
                    out[j] = __fadd_rn(out[j], zw);
                    alt[j] = __fadd_rn(alt[j], zw);
                }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) out[j] = cell_ok[j] ? out[j] : u0[j];   // never updated
        if (mem_ok) {
            *reinterpret_cast<float4 *>(p.u_out + base) = make_float4(out[0], out[1], out[2], out[3]);
            // receiver plane (3dPureqPModeling_single_shot.cu:333-337)
            if (p.record && z == p.sz && x >= pml && x < nx - pml) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int y = yq + j;
                    if (cell_ok[j] && y >= pml && y < ny - pml)
                        p.record[(long long)(x - pml) * hy + (y - pml)] = out[j];
                }
            }
        }
        // the step's decisions, when asked for (same word layout as the
        // deferred-cell mask below)
        if (!SPEC && p.dec_out) {
            const unsigned nib = (unsigned)(cell_ok[0] && above[0]) |
                                 ((unsigned)(cell_ok[1] && above[1]) << 1) |
                                 ((unsigned)(cell_ok[2] && above[2]) << 2) |
                                 ((unsigned)(cell_ok[3] && above[3]) << 3);
            unsigned w = nib << (4 * q);
            w |= __shfl_xor_sync(0xffffffffu, w, 1);
            w |= __shfl_xor_sync(0xffffffffu, w, 2);
            w |= __shfl_xor_sync(0xffffffffu, w, 4);
            if (q == 0 && row_ok) p.dec_out[base >> 5] = w;
        }
        // deferred cells: the row's bitmask word (the 8 lanes of a row combine
        // their 4 bits; written every step, so stale bits never survive), and
        // for a quad with any deferred cell its m2 and S = 1 values
        if (SPEC) {
            const unsigned nib = (unsigned)amb[0] | ((unsigned)amb[1] << 1) |
                                 ((unsigned)amb[2] << 2) | ((unsigned)amb[3] << 3);
            if (nib) {
                *reinterpret_cast<float4 *>(p.am2 + base) = make_float4(m2[0], m2[1], m2[2], m2[3]);
                *reinterpret_cast<float4 *>(p.av + base) = make_float4(alt[0], alt[1], alt[2], alt[3]);
            }
            unsigned w = nib << (4 * q);
            w |= __shfl_xor_sync(0xffffffffu, w, 1);
            w |= __shfl_xor_sync(0xffffffffu, w, 2);
            w |= __shfl_xor_sync(0xffffffffu, w, 4);
            if (q == 0 && row_ok) p.amask[base >> 5] = w;
        }
        pipe_release(P, t);
    }
    if (!ok) {
        atomicOr(p.err, kErrWaitTimeout);
        if (tid == 0) pipe_drain(P, next_issue);
    }
    if (SPEC) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0 && mx > 0.0f &&
            mx > *reinterpret_cast<const volatile float *>(p.gmax + p.step))
            atomicMax(reinterpret_cast<unsigned *>(p.gmax + p.step), __float_as_uint(mx));
    }
    if (REUSE) {
        ok = __syncthreads_and(ok) != 0;
        if (tid == 0 && ok) pipe_inval(P);
    }
    return ok;
}

template <bool SPEC, bool HALF, int AR>
__global__ void __launch_bounds__(kThreads, 2)
    qp3d_step_kernel(const __grid_constant__ CUtensorMap tm_u, const PlaneParams p)
{
    if (!SPEC && p.gate && *p.gate == 0) return;
    extern __shared__ __align__(128) unsigned char smem[];
    const int y0 = blockIdx.x * kTileY, x0 = kRadius + blockIdx.y * p.tile_x;
    const int z0 = kRadius + blockIdx.z * p.chunk_z;
    const int z1 = min(z0 + p.chunk_z, p.nz - kRadius);
    if (z0 >= z1) return;
    step_tile<SPEC, false, HALF, AR>(&tm_u, p, p.k, p.tile_x, y0, x0, z0, z1,
                                     blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0, smem);
}

// Resolution and compaction of a speculative step, over the deferred-cell
// bitmask (four words per thread).  Every block derives from the true max M
// whether it fell in the predicted window and the threshold T2 of M (thread 0,
// while the others load their words); block 0 also sets the re-run flag and
// shifts the history of the prediction's relative errors.  *p.alt_count ends as the number of deferred
// cells of the step; when M is inside the window, the deferred cells below
// the threshold are listed in p.alist and counted in *p.fix_count.
__device__ __forceinline__ void compact_body(const PlaneParams &p, unsigned block, int *redo,
                                             float *spec_err)
{
    __shared__ unsigned s_warp[32], s_def[32];
    __shared__ unsigned s_base;
    const float M = p.gmax[p.step];   // complete: the step kernel has finished
    const bool inside = (M >= p.win[0]) && (M <= p.win[1]);
    __shared__ float s_T2;
    if (threadIdx.x == 0) s_T2 = threshold_m2(M);
    if (block == 0 && threadIdx.x == 0) {
        *redo = inside ? 0 : 1;   // the fix-up sets it too when the list overflows
        const float pred = p.win[2];
#pragma unroll
        for (int i = kSpecHist - 1; i > 0; --i) spec_err[i] = spec_err[i - 1];
        spec_err[0] = pred > 0.0f ? fabsf(__fdiv_rn(M, pred) - 1.0f) : 1.0f;
    }
    const unsigned nwords = (unsigned)defer_mask_words(p.plane * p.nz);   // a multiple of 4
    const unsigned w0 = (block * blockDim.x + threadIdx.x) * 4u;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint4 wv = make_uint4(0u, 0u, 0u, 0u);
    if (w0 < nwords) wv = *reinterpret_cast<const uint4 *>(p.amask + w0);
    __syncthreads();
    const float T2 = s_T2;
    const unsigned ws[4] = {wv.x, wv.y, wv.z, wv.w};
    unsigned fix[4] = {0u, 0u, 0u, 0u};
    unsigned c = 0, dcnt = 0;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        const unsigned w = ws[h];
        dcnt += __popc(w);
        if (w && inside) {
            const float4 *m = reinterpret_cast<const float4 *>(p.am2 + (size_t)(w0 + h) * 32);
#pragma unroll
            for (int q4 = 0; q4 < 8; ++q4) {
                const unsigned nib = (w >> (4 * q4)) & 15u;
                if (!nib) continue;
                const float4 v = m[q4];
                const unsigned below = (unsigned)!(v.x > T2) | ((unsigned)!(v.y > T2) << 1) |
                                       ((unsigned)!(v.z > T2) << 2) | ((unsigned)!(v.w > T2) << 3);
                fix[h] |= (nib & below) << (4 * q4);
            }
        }
        c += __popc(fix[h]);
    }
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += v;
        dcnt += __shfl_xor_sync(0xffffffffu, dcnt, o);
    }
    if (lane == 31) s_warp[warp] = incl;
    if (lane == 0) s_def[warp] = dcnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0, d = 0;
        for (unsigned i = 0; i < (blockDim.x >> 5); ++i) {
            const unsigned v = s_warp[i];
            s_warp[i] = t;
            t += v;
            d += s_def[i];
        }
        if (d) atomicAdd(p.alt_count, d);
        s_base = t ? atomicAdd(p.fix_count, t) : 0u;
    }
    __syncthreads();
    unsigned pos = s_base + s_warp[warp] + incl - c;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        unsigned bits = fix[h];
        while (bits) {
            const int bit = __ffs(bits) - 1;
            bits &= bits - 1;
            if (pos < p.alist_cap) p.alist[pos] = (w0 + h) * 32u + (unsigned)bit;
            ++pos;
        }
    }
}

__global__ void qp3d_compact_kernel(const PlaneParams p, int *redo, float *spec_err)
{
    compact_body(p, blockIdx.x, redo, spec_err);
}

// Fix-up of a speculative step: every listed cell (deferred and below the
// true threshold) gets the S = 1 results the step kernel stored for it
// (u(k+1), and at PML cells the split-field state).  Only called when the max
// fell in the window and the list did not overflow.
__device__ __forceinline__ void fixup_cells(const PlaneParams &p, unsigned n, unsigned first,
                                            unsigned stride)
{
    const int nx = p.nx, ny = p.ny, nz = p.nz, pml = p.pml, hy = ny - 2 * pml;
    const unsigned plane = (unsigned)p.plane, ldy = (unsigned)p.ldy;
    for (unsigned i = first; i < n; i += stride) {
        const unsigned idx = p.alist[i];
        const int z = (int)(idx / plane);
        const unsigned rem = idx - (unsigned)z * plane;
        const int x = (int)(rem / ldy), y = (int)(rem - (unsigned)x * ldy);
        const bool in_pml = x < pml || x >= nx - pml || y < pml || y >= ny - pml || z < pml ||
                            z >= nz - pml;
        const float out = p.av[idx];   // the step kernel's S = 1 value, source included
        if (in_pml) {                  // and a PML cell's split-field outputs
            const float4 s = p.apml[idx];
            p.w1n[idx] = s.x;
            p.w21n[idx] = s.y;
            p.w3n[idx] = s.z;
            p.pn[idx] = s.w;
        }
        p.u_out[idx] = out;
        if (p.record && z == p.sz && x >= pml && x < nx - pml && y >= pml && y < ny - pml)
            p.record[(long long)(x - pml) * hy + (y - pml)] = out;
    }
}

// The fix-up of a speculative step, or its exact re-run when the max fell
// outside the predicted window (*p.gate, set by the compaction) or the list
// overflowed: one persistent grid of one CTA per SM.  The re-run takes the
// step's tile columns in turn, so a step that needs none costs one short
// wave instead of a full grid of CTAs that each read the gate and exit.
template <bool HALF, int AR>
__global__ void __launch_bounds__(kThreads, 1)
    qp3d_fix_or_rerun_kernel(const __grid_constant__ CUtensorMap tm_u, const PlaneParams p)
{
    const unsigned n = *p.fix_count;
    const bool rerun = *p.gate != 0 || n > p.alist_cap;
    if (!rerun) {
        fixup_cells(p, n, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *const_cast<int *>(p.gate) = 1;   // overflow: count it
    extern __shared__ __align__(128) unsigned char smem[];
    const int nyt = (p.ny - kRadius - 1) / kTileY + 1;
    const int nxt = (p.nx - 2 * kRadius + p.tile_x - 1) / p.tile_x;
    const int nch = (p.nz - 2 * kRadius + p.chunk_z - 1) / p.chunk_z;
    const int ntiles = nyt * nxt * nch;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int by = t % nyt, bx = (t / nyt) % nxt, bz = t / (nyt * nxt);
        const int z0 = kRadius + bz * p.chunk_z;
        const int z1 = min(z0 + p.chunk_z, p.nz - kRadius);
        if (z0 >= z1) continue;
        if (!step_tile<false, true, HALF, AR>(&tm_u, p, p.k, p.tile_x, by * kTileY,
                                              kRadius + bx * p.tile_x, z0, z1, false, smem))
            return;
    }
}

// ---------------------------------------------------------------------------
// Small kernels
// ---------------------------------------------------------------------------

// Sources outside the updated box [5,n-5)^3: the reference never updates
// those cells, so u3 there is its previous value plus the source
// (CPU_function.c:326-338 on a cell wavefield_update skips); with two
// buffers that previous value is u(k).
__global__ void qp3d_band_source_kernel(float *u_new, const float *u_cur, const SrcEntry *src,
                                        int n, long long plane, int ldy, float w)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    SrcEntry s = src[e];
    long long i = (long long)s.z * plane + (long long)s.x * ldy + s.y;
    u_new[i] = __fadd_rn(u_cur[i], __fmul_rn(s.v, w));
}

// All sources, after the step kernel (used when there are too many to fuse).
__global__ void qp3d_all_source_kernel(float *u_new, const float *u_cur, const SrcEntry *src,
                                       int n, long long plane, int ldy, int nx, int ny, int nz,
                                       float w)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    SrcEntry s = src[e];
    long long i = (long long)s.z * plane + (long long)s.x * ldy + s.y;
    bool inside = s.x >= kRadius && s.x < nx - kRadius && s.y >= kRadius && s.y < ny - kRadius &&
                  s.z >= kRadius && s.z < nz - kRadius;
    float prev = inside ? u_new[i] : u_cur[i];
    u_new[i] = __fadd_rn(prev, __fmul_rn(s.v, w));
}

__global__ void qp3d_record_kernel(const float *u, float *rec, int nx, int ny, int pml, int sz,
                                   int ldy, long long plane)
{
    int hx = nx - 2 * pml, hy = ny - 2 * pml;
    long long n = (long long)hx * hy;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int xi = (int)(i / hy), yi = (int)(i % hy);
        rec[i] = u[(long long)sz * plane + (long long)(xi + pml) * ldy + yi + pml];
    }
}

__global__ void qp3d_crop_kernel(const float *u, float *out, int x0, int x1, int y0, int y1,
                                 int z0, int z1, int ldy, long long plane)
{
    long long nyc = y1 - y0, nxc = x1 - x0, nzc = z1 - z0;
    long long n = nxc * nyc * nzc;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        long long yi = i % nyc, xi = (i / nyc) % nxc, zi = i / (nyc * nxc);
        out[i] = u[(zi + z0) * plane + (xi + x0) * ldy + yi + y0];
    }
}

// Per-cell parameters vp, 2 eps, 8 (eps - delta) from dense [nz][nx][ny]
// volumes (the caller's layout) into the pitched layout, one thread per
// pitched cell, row padding zero; and the same layout change for
// half-precision storage.
__global__ void qp3d_params_dense_kernel(const float *vp, const float *eps, const float *del,
                                         float *VP, float *E2, float *R8, int ny,
                                         long long vol, int ldy)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < vol;
         i += (long long)gridDim.x * blockDim.x) {
        const long long row = i / ldy;
        const int y = (int)(i - row * ldy);
        float v = 0.0f, e2 = 0.0f, r8 = 0.0f;
        if (y < ny) {
            const long long j = row * ny + y;
            const float e = eps[j], d = del[j];
            v = vp[j];
            e2 = __fmul_rn(2.0f, e);
            r8 = __fmul_rn(8.0f, __fsub_rn(e, d));
        }
        VP[i] = v;
        E2[i] = e2;
        R8[i] = r8;
    }
}

__global__ void qp3d_to_half_dense_kernel(const float *a, __half *h, int ny, long long vol,
                                          int ldy)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < vol;
         i += (long long)gridDim.x * blockDim.x) {
        const long long row = i / ldy;
        const int y = (int)(i - row * ldy);
        h[i] = __float2half_rn(y < ny ? a[row * ny + y] : 0.0f);
    }
}

// ---------------------------------------------------------------------------
// Batched shots.  Per time step:
//   qp3d_batch_prepare_kernel   reads the step counter k, writes every shot's
//                               PlaneParams of step k (buffer rotation,
//                               wavelet[k], record plane, per-step slots),
//                               zeroes the work queues, sets the counter to
//                               k + 1.  The step is therefore the same
//                               sequence of launches for every k and can be
//                               captured once in a CUDA graph.
//   qp3d_batch_plane_kernel     persistent CTAs (as many as are resident)
//                               take work items -- one tile column of one
//                               shot -- from an atomic queue and run the
//                               gradmax or step tile body on it; uneven shot
//                               sizes mix in one launch.
//   qp3d_batch_compact_kernel,  the speculative resolution, compaction
//   qp3d_batch_fixup_kernel     and fix-up, blockIdx.y = shot.
// ---------------------------------------------------------------------------
__global__ void qp3d_batch_prepare_kernel(const BatchShot *shots, int nshots, PlaneParams *pp,
                                          int *ctr, int *queues, int spec)
{
    const int k = *ctr;
    for (int s = threadIdx.x; s < nshots; s += blockDim.x) {
        const BatchShot &b = shots[s];
        PlaneParams p;
        memset(&p, 0, sizeof(p));
        p.nx = b.nx; p.ny = b.ny; p.nz = b.nz; p.ldy = b.ldy; p.pml = b.pml; p.sz = b.sz;
        p.plane = b.plane;
        p.dt = b.dt;
        p.step = k;
        p.err = b.err;
        p.active = k < b.nt ? 1 : 0;
        if (p.active) {
            // the host's rotation of qp3d_shot_advance from a reset shot
            const int a = (3 - k % 3) % 3, bb = (a + 1) % 3, c = (a + 2) % 3;
            p.ucur = a;
            p.u_cur = b.U[a]; p.u_prev = b.U[bb]; p.u_out = b.U[c];
            p.prm_v = b.VP; p.prm_e = b.E2; p.prm_r = b.R8;
            const int lo = k % 3, lc = (k + 1) % 3, ln = (k + 2) % 3;
            p.w1o = b.W1[lo]; p.w1c = b.W1[lc]; p.w1n = b.W1[ln];
            p.w3o = b.W3[lo]; p.w3c = b.W3[lc]; p.w3n = b.W3[ln];
            p.po = b.P[lo];   p.pc = b.P[lc];   p.pn = b.P[ln];
            p.w21o = b.W21[k % 2];
            p.w21n = b.W21[(k + 1) % 2];
            p.layers = b.layers;
            p.gmax = b.gmax;
            p.record = b.record + (long long)k * b.hx * b.hy;
            p.src = b.src;
            p.nsrc = b.nsrc;
            p.wavelet = b.wavelet[k];
            p.spec = spec;
            p.gate = spec ? b.redo + k : nullptr;
            p.win = b.win + 3 * (long long)k;
            p.spec_err = b.spec_err;
            p.delta_min = b.delta_min;
            p.spec_bias = b.spec_bias;
            p.amask = b.amask;
            p.am2 = b.am2;
            p.av = b.av;
            p.apml = b.apml;
            p.alt_count = b.alt_count + k;
            p.alist = b.alist;
            p.alist_cap = b.alist_cap;
            p.fix_count = b.fix_count + k;
        }
        pp[s] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        queues[0] = queues[1] = queues[2] = queues[3] = 0;
        *ctr = k + 1;
    }
}

constexpr size_t kParamBytes = (sizeof(PlaneParams) + 127) & ~(size_t)127;

size_t batch_smem_bytes(int tile_x, int pml, int nsrc)
{
    return kParamBytes + plane_smem_bytes(tile_x, pml, nsrc);
}

// KIND 0: gradmax, 1: exact step (skipped for shots whose gate is 0),
// 2: speculative step.  Bounded for one CTA of kThreads per SM: the per-shot
// parameters live in shared memory rather than in the constant bank, and held
// to the two-CTA budget of 128 registers the step body spills (measured: 15 %
// fewer shots/s).  The shape tuner then picks the tile height, which sets how
// many CTAs share an SM (three of 128 threads at 16 rows).
template <int KIND, int AR>
__global__ void __launch_bounds__(kThreads, 1) qp3d_batch_plane_kernel(const __grid_constant__ BatchArgs b)
{
    extern __shared__ __align__(128) unsigned char smem[];
    // item slot double-buffered by iteration: thread 0 can run one iteration
    // ahead of the others only on the skip path, which has no second barrier
    __shared__ int s_item[2], s_run[2];
    PlaneParams *sp = reinterpret_cast<PlaneParams *>(smem);
    unsigned char *body = smem + kParamBytes;
    for (int iter = 0;; ++iter) {
        const int slot = iter & 1;
        if (threadIdx.x == 0) {
            const int it = atomicAdd(b.queue, 1);
            int run = 0;
            if (it < b.nwork) {
                const PlaneParams &g = b.pp[b.work[it].shot];
                run = g.active != 0;
                if (KIND == 1) run = run && !(g.gate && *g.gate == 0);
            }
            s_item[slot] = it;
            s_run[slot] = run;
        }
        __syncthreads();
        const int it = s_item[slot];
        if (it >= b.nwork) return;
        if (!s_run[slot]) continue;
        const WorkItem w = b.work[it];
        {
            const unsigned *src = reinterpret_cast<const unsigned *>(b.pp + w.shot);
            unsigned *dst = reinterpret_cast<unsigned *>(sp);
            for (int i = threadIdx.x; i < (int)(sizeof(PlaneParams) / 4); i += blockDim.x)
                dst[i] = src[i];
        }
        const CUtensorMap *tm = b.tm + 3 * w.shot;
        if (threadIdx.x == 0)   // maps written by the host before the launch
            for (int i = 0; i < 3; ++i)
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tm + i)
                             : "memory");
        __syncthreads();
        const PlaneParams &p = *sp;
        tm += p.ucur;
        bool ok;
        if (KIND == 0) {
            ok = gradmax_tile<true, AR>(tm, p, b.k, w.tile_x, w.y0, w.x0, w.z0, w.z1, body);
        } else {
            const bool first = w.y0 == 0 && w.x0 == kRadius && w.z0 == kRadius;
            ok = step_tile<KIND == 2, true, false, AR>(tm, p, b.k, w.tile_x, w.y0, w.x0, w.z0,
                                                       w.z1, first, body);
        }
        if (!ok) return;
    }
}

__global__ void qp3d_batch_compact_kernel(const __grid_constant__ BatchArgs b)
{
    const PlaneParams &p = b.pp[blockIdx.y];
    if (!p.active || !p.spec) return;
    if ((long long)blockIdx.x * blockDim.x * 4 >= defer_mask_words(p.plane * p.nz)) return;
    compact_body(p, blockIdx.x, const_cast<int *>(p.gate), const_cast<float *>(p.spec_err));
}

// Fix-up of the shots whose max fell in their window; a shot whose list
// overflowed is marked for the exact pass instead.
__global__ void qp3d_batch_fixup_kernel(const __grid_constant__ BatchArgs b)
{
    const PlaneParams &p = b.pp[blockIdx.y];
    if (!p.active || !p.spec || *p.gate) return;
    const unsigned n = *p.fix_count;
    if (n > p.alist_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *const_cast<int *>(p.gate) = 1;
        return;
    }
    fixup_cells(p, n, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// ---------------------------------------------------------------------------
// Adjoint (qp3d_adjoint.cu drives them).  Pass A, per cell: the residual of
// the step is injected at the receivers; the scalar operator of step k is
// rebuilt from u^k (frozen: its decision and unit normal are those of the
// forward, its eps/delta dependence is differentiated); the PML recursions
// and the interior leapfrog are transposed term by term; each derivative the
// update took of u^k leaves a coefficient field; the gradient terms
// lambda * (d update / d m) are summed.  Pass B, per cell: the transposed
// stencils of the six coefficient fields (second derivatives: the stencil
// itself; first derivatives: its negative), zero outside the volume.
// Pass A writes only what a cell can make non-zero (PML state and first-
// derivative fields at PML cells, u_prev and second-derivative fields at
// updated cells); the caller zeroes every buffer once, so the entries never
// written stay zero in both buffers of each pair.
// The gradient is checked against the FP64 adjoint by cosine, not bit for
// bit, so these kernels take the cheaper arithmetic: fast division
// (__fdividef, 2 ulp) in S and its derivatives, fused multiply-adds in the
// transposed stencils.  Both passes are bound by the L1 load path and
// instruction issue (31 and 63 gathered taps per cell), so each thread takes
// four consecutive y cells with 16-byte loads (a quarter of the load
// instructions); a shared-memory z-marching form (register queue along z)
// was measured slower on GB300.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float4 ldg4_or0(const float *f, long long j, bool ok)
{
    return ok ? __ldg(reinterpret_cast<const float4 *>(f + j)) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// The 20 values y-8 .. y+11 of a field around a quad (zero off the row).
__device__ __forceinline__ void row_window(const float *f, long long i, int y, int ldy, float w[20])
{
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        const int yb = y - 8 + 4 * b;
        const float4 v = ldg4_or0(f, i - 8 + 4 * b, yb >= 0 && yb < ldy);
        w[4 * b] = v.x; w[4 * b + 1] = v.y; w[4 * b + 2] = v.z; w[4 * b + 3] = v.w;
    }
}

// 16 bytes global -> shared through L2 (cp.async.cg), completed by
// adj_pf_wait in the same thread
__device__ __forceinline__ void adj_pf(float4 *dst, const float *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void adj_pf_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void adj_pf_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Pass A, four consecutive y cells (a quad) per thread, block and warp
// shapes as pass B.  The derivatives of u^k take the operation order of
// quad_derivs; the streamed volumes move as 16-byte loads and stores.  Every
// entry a quad writes that its cells leave unchanged is written as zero,
// which it already is (padding, PML state at interior cells, u_prev and
// gradient at PML cells).
#define QP3D_ST4(ptr, v) *reinterpret_cast<float4 *>((ptr) + i) = make_float4(v[0], v[1], v[2], v[3])
__global__ void __launch_bounds__(256, 2) qp3d_adj_a_kernel(const AdjParams a)
{
    const int q = threadIdx.x & 7, r = threadIdx.x >> 3;
    const int y = blockIdx.x * 32 + 4 * q, x = blockIdx.y * 32 + r, z = blockIdx.z;
    if (y >= a.ny || x >= a.nx) return;
    const long long i = (long long)z * a.plane + (long long)x * a.ldy + y;
    const int nx = a.nx, ny = a.ny, nz = a.nz, pml = a.pml;
    const Coefs &k = a.k;
    const float4 lu = ldg4_or0(a.Lu, i, true), lup = ldg4_or0(a.Lup, i, true);
    float l[4] = {lu.x, lu.y, lu.z, lu.w}, nu[4] = {lup.x, lup.y, lup.z, lup.w};
    if (a.resid && z == a.sz && x >= pml && x < nx - pml) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (y + j >= pml && y + j < ny - pml)
                l[j] += a.resid[(long long)(x - pml) * a.hy + (y + j - pml)];
    }
    const bool row_upd = x >= kRadius && x < nx - kRadius && z >= kRadius && z < nz - kRadius;
    const int fx = x < pml ? 0 : (x >= nx - pml ? 1 : -1);
    const int fz = z < pml ? 4 : (z >= nz - pml ? 5 : -1);
    const int lix = x < pml ? pml - x : x - nx + pml, liz = z < pml ? pml - z : z - nz + pml;
    bool upd[4];
    int f[4], li[4];
    bool any_int = false, any_pml = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int yj = y + j;
        upd[j] = row_upd && yj >= kRadius && yj < ny - kRadius;
        const int fy = yj < pml ? 2 : (yj >= ny - pml ? 3 : -1);
        cell_face(fx, lix, fy, yj < pml ? pml - yj : yj - ny + pml, fz, liz, f[j], li[j]);
        any_int = any_int || (upd[j] && f[j] < 0);
        any_pml = any_pml || (upd[j] && f[j] >= 0);
        if (!upd[j]) nu[j] += l[j];   // a never-updated cell keeps its value
    }
    float c3[4] = {0.f, 0.f, 0.f, 0.f}, c4[4] = {0.f, 0.f, 0.f, 0.f}, c5[4] = {0.f, 0.f, 0.f, 0.f};
    float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f}, c2[4] = {0.f, 0.f, 0.f, 0.f};
    if (any_int || any_pml) {
        // derivatives of u^k (all taps in range for updated cells)
        float Ux[4], Uy[4], Uz[4], Uxx[4], Uyy[4], Uzz[4], u0[4];
        {
            float w[20];
            row_window(a.u, i, y, a.ldy, w);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                u0[j] = w[8 + j];
                float g = 0.0f, l2 = __fmul_rn(k.ky, u0[j]);
#pragma unroll
                for (int m = 0; m < kRadius; ++m) {
                    const float pa = w[8 + j + m + 1], pb = w[8 + j - m - 1];
                    const float d = __fsub_rn(pa, pb);
                    g = (m == 0) ? __fmul_rn(k.cy[0], d) : fmaf(k.cy[m], d, g);
                    l2 = fmaf(k.c2y[m], __fadd_rn(pa, pb), l2);
                }
                Uy[j] = g;
                Uyy[j] = l2;
                Ux[j] = Uz[j] = 0.0f;
                Uxx[j] = __fmul_rn(k.kx, u0[j]);
                Uzz[j] = __fmul_rn(k.kz, u0[j]);
            }
        }
#pragma unroll
        for (int m = 0; m < kRadius; ++m) {
            const long long dx = (long long)(m + 1) * a.ldy, dz = (long long)(m + 1) * a.plane;
            const float4 xp = ldg4_or0(a.u, i + dx, true), xm = ldg4_or0(a.u, i - dx, true);
            const float4 zp = ldg4_or0(a.u, i + dz, true), zm = ldg4_or0(a.u, i - dz, true);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float ddx = __fsub_rn(f4(xp, j), f4(xm, j));
                const float ddz = __fsub_rn(f4(zp, j), f4(zm, j));
                Ux[j] = (m == 0) ? __fmul_rn(k.cx[0], ddx) : fmaf(k.cx[m], ddx, Ux[j]);
                Uz[j] = (m == 0) ? __fmul_rn(k.cz[0], ddz) : fmaf(k.cz[m], ddz, Uz[j]);
                Uxx[j] = fmaf(k.c2x[m], __fadd_rn(f4(xp, j), f4(xm, j)), Uxx[j]);
                Uzz[j] = fmaf(k.c2z[m], __fadd_rn(f4(zp, j), f4(zm, j)), Uzz[j]);
            }
        }
        // frozen scalar operator and its eps / delta derivatives
        const float4 Vv = ldg4_or0(a.VP, i, true), Ev = ldg4_or0(a.E2, i, true),
                     Rv = ldg4_or0(a.R8, i, true);
        const float4 Kv = make_float4(k_of_vp(Vv.x, a.dt), k_of_vp(Vv.y, a.dt),
                                      k_of_vp(Vv.z, a.dt), k_of_vp(Vv.w, a.dt));
        const float T2 = *a.T2;
        // wa: with the live operator, dS/da times 2 / m2, so that the
        // derivatives of S in Ux, Uy, Uz are wa (Ux (1 - a), Uy (1 - a), -Uz a)
        // (a = h2 / m2 = nx^2 + ny^2, h2 = Ux^2 + Uy^2, m2 = h2 + Uz^2; no
        // power of m2 above the first, which could leave the float range)
        float KS[4], e2[4], S[4], dSe[4], dSd[4], wa[4], av[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float E2 = f4(Ev, j), R8 = f4(Rv, j);
            e2[j] = 1.0f + E2;
            const float h2 = fmaf(Uy[j], Uy[j], Ux[j] * Ux[j]), m2 = fmaf(Uz[j], Uz[j], h2);
            S[j] = 1.0f;
            dSe[j] = dSd[j] = wa[j] = av[j] = 0.0f;
            const bool on = a.dec ? ((a.dec[i >> 5] >> ((unsigned)(i & 31) + j)) & 1u) != 0
                                  : (m2 > T2);
            if (on) {
                const float aa = __fdividef(h2, m2), bb = 1.0f - aa, D = fmaf(E2, aa, 1.0f);
                const float iD = __fdividef(1.0f, D);
                const float ab8 = 8.0f * aa * bb * iD * iD;
                const float qq = 0.125f * R8 * ab8;
                const float rr = sqrtf(fmaxf(1.0f - qq, 0.0f));
                S[j] = 0.5f + 0.5f * rr;
                const float dSdq = rr > 0.0f ? __fdividef(-0.25f, rr) : 0.0f;
                dSe[j] = dSdq * ab8 * (1.0f - 0.5f * aa * R8 * iD);
                dSd[j] = -dSdq * ab8;
                if (a.live) {   // dq/da = R8 ((1 - 2a) D - 2 E2 a (1 - a)) / D^3
                    const float dqda = R8 * ((1.0f - 2.0f * aa) * D - 2.0f * E2 * aa * bb) * iD * iD * iD;
                    wa[j] = __fdividef(2.0f * dSdq * dqda, m2);
                    av[j] = aa;
                }
            }
            KS[j] = f4(Kv, j) * S[j];
        }
        if (any_int) {   // interior leapfrog and the gradient sums
            const float4 vK = ldg4_or0(a.gK, i, true), vE = ldg4_or0(a.gE, i, true),
                         vD = ldg4_or0(a.gD, i, true);
            float gK[4] = {vK.x, vK.y, vK.z, vK.w}, gE[4] = {vE.x, vE.y, vE.z, vE.w},
                  gD[4] = {vD.x, vD.y, vD.z, vD.w}, nup[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!(upd[j] && f[j] < 0)) continue;
                nu[j] += 2.0f * l[j];
                nup[j] = -l[j];
                c3[j] = KS[j] * e2[j] * l[j];
                c4[j] = c3[j];
                c5[j] = KS[j] * l[j];
                const float Lh = Uxx[j] + Uyy[j], Lap = fmaf(e2[j], Lh, Uzz[j]);
                const float Kc = f4(Kv, j);
                gK[j] += l[j] * S[j] * Lap;
                gE[j] += l[j] * Kc * (2.0f * S[j] * Lh + dSe[j] * Lap);
                gD[j] += l[j] * Kc * dSd[j] * Lap;
                // live operator: S's dependence on grad u, through the
                // transposed first derivatives (zero where S = 1)
                const float w = l[j] * Kc * Lap * wa[j], bv = 1.0f - av[j];
                c0[j] = w * Ux[j] * bv;
                c1[j] = w * Uy[j] * bv;
                c2[j] = -w * Uz[j] * av[j];
            }
            QP3D_ST4(a.gK, gK); QP3D_ST4(a.gE, gE); QP3D_ST4(a.gD, gD); QP3D_ST4(a.Nup, nup);
        }
        if (any_pml) {   // transposed split-field recursions
            const float4 vw1 = ldg4_or0(a.Lw1, i, true), vw21 = ldg4_or0(a.Lw21, i, true),
                         vw3 = ldg4_or0(a.Lw3, i, true), vp = ldg4_or0(a.Lp, i, true),
                         vw1o = ldg4_or0(a.Lw1o, i, true), vpo = ldg4_or0(a.Lpo, i, true),
                         vw3o = ldg4_or0(a.Lw3o, i, true);
            float nw1[4], nw1o[4], np_[4], npo[4], nw21[4], nw3[4], nw3o[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                nw1[j] = nw1o[j] = np_[j] = npo[j] = nw21[j] = nw3[j] = nw3o[j] = 0.0f;
                if (!(upd[j] && f[j] >= 0)) continue;
                const float4 lc = fast_layer(a.layers[(f[j] >> 1) * pml + li[j]]);
                const bool isz = f[j] >= 4;
                const float A = isz ? KS[j] : e2[j] * KS[j], Bt = isz ? e2[j] * KS[j] : KS[j];
                const float sgn = (f[j] & 1) ? -1.0f : 1.0f;
                const float W1 = f4(vw1, j) + l[j], W21 = f4(vw21, j) + l[j], W3 = f4(vw3, j) + l[j];
                const float P = fmaf(a.dt, W21, f4(vp, j));
                nw1[j] = fmaf(-lc.x, W1, f4(vw1o, j));
                nw1o[j] = lc.y * W1;
                np_[j] = fmaf(-lc.x, P, f4(vpo, j));
                npo[j] = lc.y * P;
                nw21[j] = lc.z * W21;
                nw3[j] = fmaf(2.0f, W3, f4(vw3o, j));
                nw3o[j] = -W3;
                const float cn = A * W1, cf = sgn * A * lc.w * P, ct = Bt * W3;
                if (f[j] < 2) { c3[j] = cn; c0[j] = cf; c4[j] = ct * e2[j]; c5[j] = ct; }
                else if (f[j] < 4) { c4[j] = cn; c1[j] = cf; c3[j] = ct * e2[j]; c5[j] = ct; }
                else { c5[j] = cn; c2[j] = cf; c3[j] = ct; c4[j] = ct; }
                if (a.live && wa[j] != 0.0f) {
                    // the S-proportional terms of w1', p' and w3' (their
                    // weights cn, cf, ct over S) times dS/d(grad u)
                    const float Unn = f[j] < 2 ? Uxx[j] : (isz ? Uzz[j] : Uyy[j]);
                    const float Un = f[j] < 2 ? Ux[j] : (isz ? Uz[j] : Uy[j]);
                    const float tang = isz ? Uxx[j] + Uyy[j]
                                           : fmaf(e2[j], f[j] < 2 ? Uyy[j] : Uxx[j], Uzz[j]);
                    const float w = __fdividef(cn * Unn + cf * Un + ct * tang, S[j]) * wa[j];
                    const float bv = 1.0f - av[j];
                    c0[j] += w * Ux[j] * bv;
                    c1[j] += w * Uy[j] * bv;
                    c2[j] -= w * Uz[j] * av[j];
                }
            }
            QP3D_ST4(a.Nw1, nw1); QP3D_ST4(a.Nw1o, nw1o); QP3D_ST4(a.Np, np_);
            QP3D_ST4(a.Npo, npo); QP3D_ST4(a.Nw21, nw21); QP3D_ST4(a.Nw3, nw3);
            QP3D_ST4(a.Nw3o, nw3o);
        }
        if (any_pml || a.live) {
            QP3D_ST4(a.C[0], c0); QP3D_ST4(a.C[1], c1); QP3D_ST4(a.C[2], c2);
        }
        QP3D_ST4(a.C[3], c3); QP3D_ST4(a.C[4], c4); QP3D_ST4(a.C[5], c5);
    }
    QP3D_ST4(a.Nu, nu);
#undef QP3D_ST4
}

// Pass B: Nu += the transposed stencils of the six coefficient fields, four
// consecutive y cells (a quad) per thread with 16-byte loads; a block is 8
// quads (32 y) x 32 rows, a warp 8 quads x 4 rows.  Taps outside the volume
// read zero (the coefficient fields are zero in the row padding).  Outside
// the PML shell the first-derivative fields Cx, Cy, Cz are zero and Cyy
// equals Cxx (qp3d_adj_a_kernel), so a warp whose whole footprint (its cells
// and 5 around them) lies inside reads two fields.
__global__ void __launch_bounds__(256) qp3d_adj_b_kernel(const AdjParams a)
{
    const int q = threadIdx.x & 7, r = threadIdx.x >> 3;
    const int y = blockIdx.x * 32 + 4 * q, x = blockIdx.y * 32 + r, z = blockIdx.z;
    if (y >= a.ny || x >= a.nx) return;
    const int xw = blockIdx.y * 32 + ((threadIdx.x >> 5) << 2), yw = blockIdx.x * 32;
    const long long i = (long long)z * a.plane + (long long)x * a.ldy + y;
    const Coefs &k = a.k;
    // the quad's Nu, read-modified-written at the end, moves to shared memory
    // while the taps are gathered (7% of the pass on a 240x240x190 grid)
    __shared__ __align__(16) float4 pnu[256];
    const bool vec_nu = y + 3 < a.ny;
    if (vec_nu) {
        adj_pf(&pnu[threadIdx.x], a.Nu + i);
        adj_pf_commit();
    }
    const bool inside = !a.live && xw - kRadius >= a.pml && xw + 4 + kRadius <= a.nx - a.pml &&
                        yw - kRadius >= a.pml && yw + 32 + kRadius <= a.ny - a.pml &&
                        z - kRadius >= a.pml && z + kRadius < a.nz - a.pml;
    float acc[4];
    if (inside) {
        const float *H = a.C[3], *V = a.C[5];
        float w[20];
        row_window(H, i, y, a.ldy, w);
        const float4 v0 = ldg4_or0(V, i, true);
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = k.kx * w[8 + j] + k.ky * w[8 + j] + k.kz * f4(v0, j);
#pragma unroll
        for (int m = 0; m < kRadius; ++m) {
            const int d = m + 1;
            const long long dx = (long long)d * a.ldy, dz = (long long)d * a.plane;
            const float4 hp = ldg4_or0(H, i + dx, true), hm = ldg4_or0(H, i - dx, true);
            const float4 vp = ldg4_or0(V, i + dz, true), vm = ldg4_or0(V, i - dz, true);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                acc[j] = fmaf(k.c2x[m], f4(hp, j) + f4(hm, j), acc[j]);
                acc[j] = fmaf(k.c2y[m], w[8 + j + d] + w[8 + j - d], acc[j]);
                acc[j] = fmaf(k.c2z[m], f4(vp, j) + f4(vm, j), acc[j]);
            }
        }
    } else {
        const float *Cx = a.C[0], *Cy = a.C[1], *Cz = a.C[2], *Cxx = a.C[3], *Cyy = a.C[4],
                    *Czz = a.C[5];
        {
            float wyy[20];
            row_window(Cyy, i, y, a.ldy, wyy);
            const float4 xx0 = ldg4_or0(Cxx, i, true), zz0 = ldg4_or0(Czz, i, true);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                acc[j] = k.kx * f4(xx0, j) + k.ky * wyy[8 + j] + k.kz * f4(zz0, j);
#pragma unroll
            for (int m = 0; m < kRadius; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    acc[j] = fmaf(k.c2y[m], wyy[8 + j + m + 1] + wyy[8 + j - m - 1], acc[j]);
        }
        {
            float wy[20];
            row_window(Cy, i, y, a.ldy, wy);
#pragma unroll
            for (int m = 0; m < kRadius; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    acc[j] = fmaf(k.cy[m], wy[8 + j - m - 1] - wy[8 + j + m + 1], acc[j]);
        }
#pragma unroll
        for (int m = 0; m < kRadius; ++m) {
            const int d = m + 1;
            const long long dx = (long long)d * a.ldy, dz = (long long)d * a.plane;
            const bool xp = x + d < a.nx, xm = x - d >= 0, zp = z + d < a.nz, zm = z - d >= 0;
            const float4 xxp = ldg4_or0(Cxx, i + dx, xp), xxm = ldg4_or0(Cxx, i - dx, xm);
            const float4 x1p = ldg4_or0(Cx, i + dx, xp), x1m = ldg4_or0(Cx, i - dx, xm);
            const float4 zzp = ldg4_or0(Czz, i + dz, zp), zzm = ldg4_or0(Czz, i - dz, zm);
            const float4 z1p = ldg4_or0(Cz, i + dz, zp), z1m = ldg4_or0(Cz, i - dz, zm);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                acc[j] = fmaf(k.c2x[m], f4(xxp, j) + f4(xxm, j), acc[j]);
                acc[j] = fmaf(k.c2z[m], f4(zzp, j) + f4(zzm, j), acc[j]);
                acc[j] = fmaf(k.cx[m], f4(x1m, j) - f4(x1p, j), acc[j]);
                acc[j] = fmaf(k.cz[m], f4(z1m, j) - f4(z1p, j), acc[j]);
            }
        }
    }
    float *nu = a.Nu + i;
    if (vec_nu) {
        adj_pf_wait();
        float4 v = pnu[threadIdx.x];
        v.x += acc[0]; v.y += acc[1]; v.z += acc[2]; v.w += acc[3];
        *reinterpret_cast<float4 *>(nu) = v;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (y + j < a.ny) nu[j] += acc[j];
    }
}

__global__ void qp3d_threshold_kernel(const float *gmax, float *T2, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) T2[i] = threshold_m2(gmax[i]);
}

// Record residual r = record - d_obs and the misfit 1/2 sum r^2 (FP64, one
// atomic per block).
__global__ void qp3d_residual_kernel(const float *rec, const float *dobs, float *r, long long n,
                                     double *misfit)
{
    __shared__ double s[32];
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float v = rec[i] - dobs[i];
        r[i] = v;
        acc += 0.5 * (double)v * (double)v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        atomicAdd(misfit, t);
    }
}

__global__ void qp3d_to_bf16_kernel(const float *a, __nv_bfloat16 *h, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        h[i] = __float2bfloat16_rn(a[i]);
}

__global__ void qp3d_from_bf16_kernel(const __nv_bfloat16 *h, float *a, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        a[i] = __bfloat162float(h[i]);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <typename F>
static cudaError_t set_smem(F *fn, int bytes)
{
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t configure_kernels()
{
    const int bytes = 200 * 1024;
    cudaError_t e;
    if ((e = set_smem(qp3d_batch_plane_kernel<0, kArithFast>, bytes)) ||
        (e = set_smem(qp3d_batch_plane_kernel<1, kArithFast>, bytes)) ||
        (e = set_smem(qp3d_batch_plane_kernel<2, kArithFast>, bytes)) ||
        (e = set_smem(qp3d_batch_plane_kernel<0, kArithRef>, bytes)) ||
        (e = set_smem(qp3d_batch_plane_kernel<1, kArithRef>, bytes)) ||
        (e = set_smem(qp3d_batch_plane_kernel<2, kArithRef>, bytes)))
        return e;
#define QP3D_STEP_SMEM(AR)                                                                   \
    if ((e = set_smem(qp3d_step_kernel<true, false, AR>, bytes)) ||                         \
        (e = set_smem(qp3d_step_kernel<false, false, AR>, bytes)) ||                        \
        (e = set_smem(qp3d_step_kernel<true, true, AR>, bytes)) ||                          \
        (e = set_smem(qp3d_step_kernel<false, true, AR>, bytes)) ||                         \
        (e = set_smem(qp3d_gradmax_kernel<false, AR>, bytes)) ||                            \
        (e = set_smem(qp3d_fix_or_rerun_kernel<false, AR>, bytes)) ||                              \
        (e = set_smem(qp3d_fix_or_rerun_kernel<true, AR>, bytes)))                                 \
        return e;
    QP3D_STEP_SMEM(kArithFast)
    QP3D_STEP_SMEM(kArithRef)
#undef QP3D_STEP_SMEM
    return set_smem(qp3d_gradmax_kernel<true, kArithFast>, bytes);
}

// whole warps: rows past tile_x are idle, so every warp collective sees 32 lanes
static inline int plane_threads(int tile_x) { return (kQuadsY * tile_x + 31) & ~31; }

cudaError_t launch_gradmax(const CUtensorMap &tm_u, const PlaneParams &p, dim3 grid, size_t smem,
                           cudaStream_t stream, int variant)
{
    const int t = plane_threads(p.tile_x);
    if (p.arith == kArithRef)
        qp3d_gradmax_kernel<false, kArithRef><<<grid, t, smem, stream>>>(tm_u, p);
    else if (variant == 0)
        qp3d_gradmax_kernel<false, kArithFast><<<grid, t, smem, stream>>>(tm_u, p);
    else
        qp3d_gradmax_kernel<true, kArithFast><<<grid, t, smem, stream>>>(tm_u, p);
    return cudaGetLastError();
}

template <int AR>
static void launch_step_t(const CUtensorMap &tm_u, const PlaneParams &p, dim3 grid, int t,
                          size_t smem, cudaStream_t stream)
{
    if (p.half_params) {
        if (p.spec) qp3d_step_kernel<true, true, AR><<<grid, t, smem, stream>>>(tm_u, p);
        else qp3d_step_kernel<false, true, AR><<<grid, t, smem, stream>>>(tm_u, p);
    } else {
        if (p.spec) qp3d_step_kernel<true, false, AR><<<grid, t, smem, stream>>>(tm_u, p);
        else qp3d_step_kernel<false, false, AR><<<grid, t, smem, stream>>>(tm_u, p);
    }
}

cudaError_t launch_step(const CUtensorMap &tm_u, const PlaneParams &p, dim3 grid, size_t smem,
                        cudaStream_t stream)
{
    const int t = plane_threads(p.tile_x);
    if (p.arith == kArithRef) launch_step_t<kArithRef>(tm_u, p, grid, t, smem, stream);
    else launch_step_t<kArithFast>(tm_u, p, grid, t, smem, stream);
    return cudaGetLastError();
}

cudaError_t configure_gradmax_partial()
{
    cudaError_t e;
    if ((e = set_smem(qp3d_gradmax_partial_kernel<kArithFast>, 200 * 1024))) return e;
    return set_smem(qp3d_gradmax_partial_kernel<kArithRef>, 200 * 1024);
}

cudaError_t launch_gradmax_partial(const CUtensorMap &tm_u, const PlaneParams &p, dim3 grid,
                                   size_t smem, cudaStream_t stream, float *partial,
                                   unsigned nblocks, float *out)
{
    const int t = plane_threads(p.tile_x);
    if (p.arith == kArithRef)
        qp3d_gradmax_partial_kernel<kArithRef><<<grid, t, smem, stream>>>(tm_u, p, partial);
    else
        qp3d_gradmax_partial_kernel<kArithFast><<<grid, t, smem, stream>>>(tm_u, p, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    qp3d_reduce_max_kernel<<<1, 1024, 0, stream>>>(partial, nblocks, p.err, out);
    return cudaGetLastError();
}

cudaError_t launch_compact(const PlaneParams &p, int *redo, float *spec_err, cudaStream_t stream)
{
    const long long words = defer_mask_words(p.plane * p.nz);
    qp3d_compact_kernel<<<(unsigned)((words / 4 + 255) / 256), 256, 0, stream>>>(p, redo,
                                                                                 spec_err);
    return cudaGetLastError();
}

template <int AR>
static void launch_fix_or_rerun_t(const CUtensorMap &tm_u, const PlaneParams &p, int grid, int t,
                                  size_t smem, cudaStream_t stream)
{
    if (p.half_params) qp3d_fix_or_rerun_kernel<true, AR><<<grid, t, smem, stream>>>(tm_u, p);
    else qp3d_fix_or_rerun_kernel<false, AR><<<grid, t, smem, stream>>>(tm_u, p);
}

cudaError_t launch_fix_or_rerun(const CUtensorMap &tm_u, const PlaneParams &p, int nsm,
                                size_t smem, cudaStream_t stream)
{
    const int t = plane_threads(p.tile_x);
    if (p.arith == kArithRef) launch_fix_or_rerun_t<kArithRef>(tm_u, p, nsm, t, smem, stream);
    else launch_fix_or_rerun_t<kArithFast>(tm_u, p, nsm, t, smem, stream);
    return cudaGetLastError();
}

int batch_plane_threads(int tile_x) { return plane_threads(tile_x); }

cudaError_t launch_batch_prepare(const BatchShot *shots, int nshots, PlaneParams *pp, int *ctr,
                                 int *queues, int spec, cudaStream_t stream)
{
    qp3d_batch_prepare_kernel<<<1, 128, 0, stream>>>(shots, nshots, pp, ctr, queues, spec);
    return cudaGetLastError();
}

static const void *batch_plane_fn(int kind, int arith)
{
    if (arith == kArithRef)
        return kind == 0 ? (const void *)qp3d_batch_plane_kernel<0, kArithRef>
             : kind == 1 ? (const void *)qp3d_batch_plane_kernel<1, kArithRef>
                         : (const void *)qp3d_batch_plane_kernel<2, kArithRef>;
    return kind == 0 ? (const void *)qp3d_batch_plane_kernel<0, kArithFast>
         : kind == 1 ? (const void *)qp3d_batch_plane_kernel<1, kArithFast>
                     : (const void *)qp3d_batch_plane_kernel<2, kArithFast>;
}

cudaError_t batch_ctas_per_sm(int kind, int arith, int threads, size_t smem, int *n)
{
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, batch_plane_fn(kind, arith), threads,
                                                         smem);
}

cudaError_t launch_batch_plane(int kind, const BatchArgs &b, int grid, int threads, size_t smem,
                               cudaStream_t stream)
{
    void *args[] = {const_cast<BatchArgs *>(&b)};
    return cudaLaunchKernel(batch_plane_fn(kind, b.arith), dim3(grid), dim3(threads), args, smem,
                            stream);
}

cudaError_t launch_batch_fixup(const BatchArgs &b, int nshots, int blocks_per_shot,
                               long long max_words, cudaStream_t stream)
{
    qp3d_batch_compact_kernel<<<dim3((unsigned)((max_words / 4 + 255) / 256), nshots), 256, 0,
                                stream>>>(b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    qp3d_batch_fixup_kernel<<<dim3(blocks_per_shot, nshots), 256, 0, stream>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_band_sources(float *u_new, const float *u_cur, const SrcEntry *src, int n,
                                long long plane, int ldy, float w, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    qp3d_band_source_kernel<<<(n + 127) / 128, 128, 0, stream>>>(u_new, u_cur, src, n, plane, ldy,
                                                                 w);
    return cudaGetLastError();
}

cudaError_t launch_all_sources(float *u_new, const float *u_cur, const SrcEntry *src, int n,
                               long long plane, int ldy, int nx, int ny, int nz, float w,
                               cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    qp3d_all_source_kernel<<<(n + 255) / 256, 256, 0, stream>>>(u_new, u_cur, src, n, plane, ldy,
                                                                nx, ny, nz, w);
    return cudaGetLastError();
}

cudaError_t launch_record(const float *u, float *rec, int nx, int ny, int pml, int sz, int ldy,
                          long long plane, cudaStream_t stream)
{
    long long n = (long long)(nx - 2 * pml) * (ny - 2 * pml);
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    qp3d_record_kernel<<<blocks, 256, 0, stream>>>(u, rec, nx, ny, pml, sz, ldy, plane);
    return cudaGetLastError();
}

cudaError_t launch_crop(const float *u, float *out, int x0, int x1, int y0, int y1, int z0, int z1,
                        int ldy, long long plane, cudaStream_t stream)
{
    long long n = (long long)(x1 - x0) * (y1 - y0) * (z1 - z0);
    if (n <= 0) return cudaSuccess;
    long long b = (n + 255) / 256;
    int blocks = (int)(b > 8192 ? 8192 : b);
    qp3d_crop_kernel<<<blocks, 256, 0, stream>>>(u, out, x0, x1, y0, y1, z0, z1, ldy, plane);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_step(const AdjParams &a, cudaStream_t stream)
{
    // one thread per quad of 4 y cells; a block is 8 quads x 32 rows
    const dim3 grid((a.ny + 31) / 32, (a.nx + 31) / 32, a.nz);
    qp3d_adj_a_kernel<<<grid, 256, 0, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    qp3d_adj_b_kernel<<<grid, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_threshold(const float *gmax, float *T2, int n, cudaStream_t stream)
{
    qp3d_threshold_kernel<<<1, 256, 0, stream>>>(gmax, T2, n);
    return cudaGetLastError();
}

cudaError_t launch_residual(const float *rec, const float *dobs, float *r, long long n,
                            double *misfit, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    long long b = (n + 255) / 256;
    qp3d_residual_kernel<<<(int)(b > 4096 ? 4096 : b), 256, 0, stream>>>(rec, dobs, r, n, misfit);
    return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float *a, __nv_bfloat16 *h, long long n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    long long b = (n + 255) / 256;
    qp3d_to_bf16_kernel<<<(int)(b > 8192 ? 8192 : b), 256, 0, stream>>>(a, h, n);
    return cudaGetLastError();
}

cudaError_t launch_from_bf16(const __nv_bfloat16 *h, float *a, long long n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    long long b = (n + 255) / 256;
    qp3d_from_bf16_kernel<<<(int)(b > 8192 ? 8192 : b), 256, 0, stream>>>(h, a, n);
    return cudaGetLastError();
}

cudaError_t launch_params_dense(const float *vp, const float *eps, const float *del, float *VP,
                                float *E2, float *R8, int nx, int ny, int nz, int ldy,
                                cudaStream_t stream)
{
    const long long vol = (long long)nz * nx * ldy;
    const long long b = (vol + 255) / 256;
    qp3d_params_dense_kernel<<<(int)(b > 16384 ? 16384 : b), 256, 0, stream>>>(
        vp, eps, del, VP, E2, R8, ny, vol, ldy);
    return cudaGetLastError();
}

cudaError_t launch_to_half_dense(const float *a, __half *h, int nx, int ny, int nz, int ldy,
                                 cudaStream_t stream)
{
    const long long vol = (long long)nz * nx * ldy;
    const long long b = (vol + 255) / 256;
    qp3d_to_half_dense_kernel<<<(int)(b > 16384 ? 16384 : b), 256, 0, stream>>>(a, h, ny, vol,
                                                                                ldy);
    return cudaGetLastError();
}

}  // namespace qp3d
