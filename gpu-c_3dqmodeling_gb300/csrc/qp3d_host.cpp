// qp3d_host.cpp -- host side of the library: the derived coefficient tables
// the kernels use, the reference's host utilities (C ABI), and the
// C++-linkage modeling3d drop-in.
//
// Compiled with -ffp-contract=off: the derivations below state each float
// rounding, and the CPU oracle's mirror variant derives the same tables the
// same way, so kernel results can be compared bit for bit.
#include "qp3d.h"
#include "qp3d_modeling3d.h"
#include "qp3d_internal.h"
#include "qp3d_exact.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace qp3d {

// The reference adds the whole source volume every step
// (CPU_function.c:326-338); its non-zero samples are the sparse source.
// Planes are split over up to 16 threads and the lists joined in plane
// order, so the order is that of one sequential scan.
void scan_source_volume(const float *s, int nx, int ny, int nz, std::vector<SrcEntry> &out)
{
    out.clear();
    const unsigned hw = std::thread::hardware_concurrency();
    const int nth = (int)std::max(1u, std::min(16u, hw ? hw : 1u));
    std::vector<std::vector<SrcEntry>> part(nth);
    auto work = [&](int t) {
        const int z0 = (int)((long long)nz * t / nth), z1 = (int)((long long)nz * (t + 1) / nth);
        for (int z = z0; z < z1; ++z)
            for (int x = 0; x < nx; ++x) {
                const float *row = s + ((size_t)z * nx + x) * ny;
                for (int y = 0; y < ny; ++y)
                    if (row[y] != 0.0f) part[t].push_back(SrcEntry{x, y, z, row[y]});
            }
    };
    std::vector<std::thread> th;
    int started = 1;
    try {
        for (int t = 1; t < nth; ++t, ++started) th.emplace_back(work, t);
    } catch (...) {   // no more threads: this one scans the rest
    }
    work(0);
    for (auto &t : th) t.join();
    for (int t = started; t < nth; ++t) work(t);
    for (auto &p : part) out.insert(out.end(), p.begin(), p.end());
}

// FD tables with the 1/h factors folded in.  The reference divides every tap
// by dx (first derivative, CPU_function.c:314-316) or dx*dx (second,
// CPU_function.c:393-395); c[31..35] / c2[31..35] are the M=10 weights.
void derive_coefs(const float *c, const float *c2, float dx, float dy, float dz, Coefs *k)
{
    float dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (int m = 0; m < kRadius; m++) {
        k->cx[m] = c[31 + m] / dx;
        k->cy[m] = c[31 + m] / dy;
        k->cz[m] = c[31 + m] / dz;
        k->c2x[m] = c2[31 + m] / dx2;
        k->c2y[m] = c2[31 + m] / dy2;
        k->c2z[m] = c2[31 + m] / dz2;
        sx = sx + k->c2x[m];
        sy = sy + k->c2y[m];
        sz = sz + k->c2z[m];
    }
    k->kx = -(2.0f * sx);
    k->ky = -(2.0f * sy);
    k->kz = -(2.0f * sz);
    for (int m = 0; m < kRadius; m++) {
        k->cx2[m] = make_float2(k->cx[m], k->cx[m]);
        k->cy2[m] = make_float2(k->cy[m], k->cy[m]);
        k->cz2[m] = make_float2(k->cz[m], k->cz[m]);
        k->c2x2[m] = make_float2(k->c2x[m], k->c2x[m]);
        k->c2y2[m] = make_float2(k->c2y[m], k->c2y[m]);
        k->c2z2[m] = make_float2(k->c2z[m], k->c2z[m]);
    }
    k->kx2 = make_float2(k->kx, k->kx);
    k->ky2 = make_float2(k->ky, k->ky);
    k->kz2 = make_float2(k->kz, k->kz);
    // reference arithmetic: the tables as they are, and the divisors
    for (int m = 0; m < kRadius; m++) {
        k->rc[m] = make_float2(c[31 + m], c[31 + m]);
        k->rc2[m] = make_float2(c2[31 + m], c2[31 + m]);
    }
    const float h[3] = {dx, dy, dz}, h2[3] = {dx2, dy2, dz2};
    for (int a = 0; a < 3; a++) {
        k->rh[a] = h[a];
        k->rh2[a] = h2[a];
    }
}

// Per-layer PML recursion coefficients (GPU_kernel.cu:569-572,
// CPU_function.c:400-404): a1 = (d*dt+1)^2 - 3, which the reference squares
// in double (pow(float,int)), is exact as the float pair (a1h, a1l); with
// t = d*dt the other two are a2 = 2*d*dt - 1 = fma(2, t, -1) and
// a3 = 1 - dt*d = 1 - t; dd is the second profile.  Stored (a1h, a1l, t, dd).
void derive_layers(const float *d, const float *dd, int pml, float dt, float4 *out)
{
    for (int i = 0; i < pml; i++) {
        const xr::PmlLayer L = xr::pml_layer(d[i], dd[i], dt);
        out[i] = make_float4(L.a1h, L.a1l, d[i] * dt, dd[i]);
    }
}

}  // namespace qp3d

// ---------------------------------------------------------------------------
// Host utilities (restating CPU_function.c)
// ---------------------------------------------------------------------------
extern "C" float qp3d_absmax(const float *a, size_t n)
{   // CPU_function.c:10-22: Max starts at 0 and NaNs never compare >=
    float m = 0.0f;
    for (size_t i = 0; i < n; i++)
        if (std::fabs(a[i]) >= m) m = std::fabs(a[i]);
    return m;
}

extern "C" void qp3d_fdcoff1(float *c)
{   // CPU_function.c:111-128
    c[7] = 0.5f;
    c[13] = 0.667f; c[14] = -0.083f;
    c[19] = 0.75f; c[20] = -0.15f; c[21] = 0.0167f;
    c[25] = 0.8f; c[26] = -0.2f; c[27] = 0.038f; c[28] = -0.0036f;
    c[31] = 0.833f; c[32] = -0.2381f; c[33] = 0.059f; c[34] = -0.0099f; c[35] = 0.00079f;
}

extern "C" void qp3d_fdcoff2(float *c)
{   // CPU_function.c:131-148
    c[7] = 1.0f;
    c[13] = (float)(4.0 / 3.0); c[14] = (float)(-1.0 / 12.0);
    c[19] = 1.5f; c[20] = -0.15f; c[21] = (float)(1.0 / 90.0);
    c[25] = 1.6f; c[26] = -0.2f; c[27] = (float)(8.0 / 315.0); c[28] = (float)(-1.0 / 560);
    c[31] = 1.6667f; c[32] = -0.2381f; c[33] = 0.0397f; c[34] = -0.0050f; c[35] = 0.0003f;
}

extern "C" void qp3d_pmlcoff(int pml, float vpmax, float dx, float dy, float dz, float *dlr,
                             float *ddlr, float *dtb, float *ddtb, float *dfb, float *ddfb)
{   // CPU_function.c:150-169: d = 4 vmax/(2W) (x/W)^3 ln(1/R), dd = 6 vmax x^2/W^4 ln(1/R)
    const float R = 0.00001f;
    const float wlr = pml * dx, wtb = pml * dz, wfb = pml * dy;
    const float lg = logf(1 / R);
    for (int i = 0; i < pml; i++) {
        float wx = (i + 1) * dx, wz = (i + 1) * dz, wy = (i + 1) * dy;
        dlr[i] = (float)(4 * vpmax / (2 * wlr) * std::pow((double)(wx / wlr), 3.0) * lg);
        ddlr[i] = (float)(6 * vpmax * wx * wx / std::pow((double)wlr, 4.0) * lg);
        dtb[i] = (float)(4 * vpmax / (2 * wtb) * std::pow((double)(wz / wtb), 3.0) * lg);
        ddtb[i] = (float)(6 * vpmax * wz * wz / std::pow((double)wtb, 4.0) * lg);
        dfb[i] = (float)(4 * vpmax / (2 * wfb) * std::pow((double)(wy / wfb), 3.0) * lg);
        ddfb[i] = (float)(6 * vpmax * wy * wy / std::pow((double)wfb, 4.0) * lg);
    }
}

extern "C" void qp3d_source(int sx, int sy, int sz, float fm, float amp, float alpha, float dt,
                            float dx, float dy, float dz, float t0, int nt, int nx, int ny, int nz,
                            float *source, float *wavelet)
{   // CPU_function.c:37-64: Gaussian spatial source and Ricker wavelet
    const double pi = 3.1415926535898;
    const double a2 = (double)alpha * (double)alpha;
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < nx; j++) {
            double rx = (double)((j - sx) * dx), rz = (double)((i - sz) * dz);
            for (int k = 0; k < ny; k++) {
                double ry = (double)((k - sy) * dy);
                source[((size_t)i * nx + j) * ny + k] =
                    (float)(amp * std::exp(-a2 * (rx * rx + ry * ry + rz * rz)));
            }
        }
    for (int k = 0; k < nt; k++) {
        float t = k * dt;
        float temp = (float)std::pow(pi * fm * (t - t0), 2.0);
        wavelet[k] = (1 - 2 * temp) * std::exp(-temp);   // float overload, as in C++
    }
}

extern "C" void qp3d_extend_model(const float *in, float *out, int nx, int ny, int nz, int pml)
{   // CPU_function.c:67-108: edge replication into the PML shell (clamped index)
    const int hx = nx - 2 * pml, hy = ny - 2 * pml, hz = nz - 2 * pml;
    for (int i = 0; i < nz; i++) {
        int zi = i < pml ? 0 : (i >= nz - pml ? hz - 1 : i - pml);
        for (int j = 0; j < nx; j++) {
            int xi = j < pml ? 0 : (j >= nx - pml ? hx - 1 : j - pml);
            const float *src = in + ((size_t)zi * hx + xi) * hy;
            float *dst = out + ((size_t)i * nx + j) * ny;
            for (int k = 0; k < ny; k++) {
                int yi = k < pml ? 0 : (k >= ny - pml ? hy - 1 : k - pml);
                dst[k] = src[yi];
            }
        }
    }
}

extern "C" int qp3d_readmodel3d(const char *filename, float *a, int ny, int nx, int nz, int fny,
                                int fnx, int fnz, int vny, int vnx, int vnz)
{   // CPU_function.c:234-261: window of a [vny][vnx][vnz] file, transposed to [z][x][y]
    if (!filename || !a || nx <= 0 || ny <= 0 || nz <= 0) return QP3D_ERR_ARG;
    if (fny < 0 || fnx < 0 || fnz < 0 || fny + ny > vny || fnx + nx > vnx || fnz + nz > vnz)
        return QP3D_ERR_ARG;
    FILE *fp = fopen(filename, "rb");
    if (!fp) return QP3D_ERR_IO;
    std::vector<float> col(nz);
    int rc = QP3D_OK;
    for (int i = 0; i < ny && rc == QP3D_OK; i++)
        for (int j = 0; j < nx; j++) {
            long long off = (((long long)(fny + i) * vnx + fnx + j) * vnz + fnz) * (long long)sizeof(float);
            if (fseeko(fp, (off_t)off, SEEK_SET) != 0 ||
                fread(col.data(), sizeof(float), nz, fp) != (size_t)nz) {
                rc = QP3D_ERR_IO;
                break;
            }
            for (int k = 0; k < nz; k++) a[((size_t)k * nx + j) * ny + i] = col[k];
        }
    fclose(fp);
    return rc;
}

// ---------------------------------------------------------------------------
// modeling3d drop-in (C++ linkage, 3dPureqPModeling_single_shot.h:4-6)
// ---------------------------------------------------------------------------
namespace qp3d {

// Snapshot file names of 3dPureqPModeling_single_shot.cu:342-345:
// <prefix><k>.dat and <prefix>_xz/_yz/_xy<k>.dat.
std::string snapshot_file_name(const std::string &prefix, int kind, int step)
{
    static const char *suffix[4] = {"", "_xz", "_yz", "_xy"};
    return prefix + suffix[kind < 0 || kind > 3 ? 0 : kind] + std::to_string(step) + ".dat";
}

// Snapshot files as raw native floats (read_write.c:29-52); user points to
// the prefix (std::string).
int write_snapshot_files(void *user, int step, int kind, const float *data, int n0, int n1,
                         int n2)
{
    const std::string *prefix = static_cast<const std::string *>(user);
    if (kind < 0 || kind > 3) return -1;
    const std::string name = snapshot_file_name(*prefix, kind, step);
    FILE *fp = fopen(name.c_str(), "wb");
    if (!fp) return -1;
    const size_t n = (size_t)n0 * n1 * n2;
    const size_t w = fwrite(data, sizeof(float), n, fp);
    return (fclose(fp) == 0 && w == n) ? 0 : -1;
}

}  // namespace qp3d

namespace {

qp3d_ctx *g_ctx = nullptr;

}  // namespace

void modeling3d(int nx, int ny, int nz, int nt, int ntsnap, float dx, float dy, float dz, float dt,
                int pml, int snapflag, int sx, int sy, int sz, float *vp, float *epsilon,
                float *delta, float *source, float *wavelet, float *record, float *dlr,
                float *ddlr, float *dtb, float *ddtb, float *dfb, float *ddfb, float *c, float *c2,
                const char *snap_file)
{
    (void)sx;
    (void)sy;   // unused by the reference kernel as well
    int rc = QP3D_OK;
    if (!g_ctx) {
        rc = qp3d_ctx_create(0, &g_ctx);   // the reference always uses device 0
        if (rc) {
            fprintf(stderr, "modeling3d: no CUDA device (%s)\n", qp3d_strerror(rc));
            return;
        }
    }
    qp3d_geom g;
    g.nx = nx; g.ny = ny; g.nz = nz; g.nt = nt; g.pml = pml; g.sz = sz;
    g.dx = dx; g.dy = dy; g.dz = dz; g.dt = dt;
    qp3d_model m;
    m.vp = vp; m.epsilon = epsilon; m.delta = delta; m.source = source; m.wavelet = wavelet;
    m.dlr = dlr; m.ddlr = ddlr; m.dtb = dtb; m.ddtb = ddtb; m.dfb = dfb; m.ddfb = ddfb;
    m.c = c; m.c2 = c2;
    std::string prefix(snap_file ? snap_file : "");
    qp3d_snap snap;
    snap.ntsnap = ntsnap;
    snap.kinds = 0xFu;
    snap.fn = qp3d::write_snapshot_files;
    snap.user = &prefix;
    rc = qp3d_forward(g_ctx, &g, &m, record, (snapflag == 1 && ntsnap > 0) ? &snap : nullptr);
    if (rc)
        fprintf(stderr, "modeling3d: %s: %s\n", qp3d_strerror(rc), qp3d_ctx_last_error(g_ctx));
}
