// qp3d_api.cu -- the C ABI of include/qp3d.h: context, shot buffers, the
// per-step launch sequence and state I/O.
//
// The reference's per-shot driver (3dPureqPModeling_single_shot.cu:26-447)
// allocates 70 device buffers per call, copies three full volumes to the host
// every step to find max|grad u| on one CPU core, and copies the whole
// wavefield back every step to take one receiver plane.  Here the model stays
// resident, the maximum is a device reduction, the receiver plane is written
// by the step kernel, and nothing crosses the host link inside the time loop
// except optional snapshots.
#include "qp3d_ctx.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace qp3d;

extern "C" int qp3d_version(void) { return 10000; }

extern "C" const char *qp3d_strerror(int code)
{
    switch (code) {
    case QP3D_OK: return "ok";
    case QP3D_ERR_ARG: return "invalid argument";
    case QP3D_ERR_CUDA: return "CUDA error";
    case QP3D_ERR_NOMEM: return "out of memory";
    case QP3D_ERR_TIMEOUT: return "device wait timed out";
    case QP3D_ERR_STATE: return "invalid call order";
    case QP3D_ERR_IO: return "file I/O error";
    case QP3D_ERR_CALLBACK: return "snapshot callback failed";
    default: return "unknown error";
    }
}

extern "C" const char *qp3d_ctx_last_error(const qp3d_ctx *ctx) { return ctx ? ctx->err : ""; }

static void free_shot(qp3d_ctx *ctx)
{
    cudaSetDevice(ctx->device);
    float **bufs[] = {&ctx->U[0],  &ctx->U[1],  &ctx->U[2],  &ctx->VP,     &ctx->E2,
                      &ctx->R8,    &ctx->W1[0], &ctx->W1[1], &ctx->W1[2], &ctx->W3[0],
                      &ctx->W3[1], &ctx->W3[2], &ctx->P[0],  &ctx->P[1],  &ctx->P[2],
                      &ctx->W21[0], &ctx->W21[1], &ctx->record, &ctx->gmax, &ctx->snap_dev,
                      &ctx->win,   &ctx->spec_err, &ctx->am2, &ctx->av};
    for (float **b : bufs) {
        if (*b) cudaFree(*b);
        *b = nullptr;
    }
    if (ctx->redo) cudaFree(ctx->redo);
    if (ctx->alt_count) cudaFree(ctx->alt_count);
    if (ctx->amask) cudaFree(ctx->amask);
    if (ctx->apml) cudaFree(ctx->apml);
    ctx->apml = nullptr;
    if (ctx->alist) cudaFree(ctx->alist);
    if (ctx->fix_count) cudaFree(ctx->fix_count);
    ctx->fix_count = nullptr;
    ctx->redo = nullptr;
    ctx->alt_count = nullptr;
    ctx->amask = nullptr;
    ctx->alist = nullptr;
    ctx->alist_cap = 0;
    __half **halves[] = {&ctx->h_vp, &ctx->h_eps, &ctx->h_del};
    for (__half **h : halves) {
        if (*h) cudaFree(*h);
        *h = nullptr;
    }
    if (ctx->layers) cudaFree(ctx->layers);
    if (ctx->src_fused) cudaFree(ctx->src_fused);
    if (ctx->src_band) cudaFree(ctx->src_band);
    if (ctx->src_all) cudaFree(ctx->src_all);
    if (ctx->snap_host) cudaFreeHost(ctx->snap_host);
    ctx->layers = nullptr;
    ctx->src_fused = ctx->src_band = ctx->src_all = nullptr;
    ctx->snap_host = nullptr;
    ctx->snap_cap = 0;
    ctx->loaded = false;
}

extern "C" int qp3d_ctx_create(int device, qp3d_ctx **out)
{
    if (!out) return QP3D_ERR_ARG;
    *out = nullptr;
    qp3d_ctx *ctx = new (std::nothrow) qp3d_ctx();
    if (!ctx) return QP3D_ERR_NOMEM;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= 0 || device < 0 || device >= ndev) {
        delete ctx;
        return QP3D_ERR_CUDA;
    }
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        configure_kernels() != cudaSuccess) {
        delete ctx;
        return QP3D_ERR_CUDA;
    }
    for (auto &ev : ctx->ev) cudaEventCreate(&ev);
    for (auto &ev : ctx->uev) cudaEventCreate(&ev);
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        qp3d_ctx_destroy(ctx);
        return QP3D_ERR_CUDA;
    }
    ctx->encode = reinterpret_cast<EncodeTiledFn>(fn);
    *out = ctx;
    return QP3D_OK;
}

extern "C" void qp3d_ctx_destroy(qp3d_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_shot(ctx);
    batch_free(ctx->batch);
    ctx->batch = nullptr;
    adjoint_free(ctx->adj);
    ctx->adj = nullptr;
    if (ctx->errword) cudaFree(ctx->errword);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (auto &sl : ctx->sring) {
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.ready) cudaEventDestroy(sl.ready);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->copy_ev) cudaEventDestroy(ctx->copy_ev);
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : ctx->uev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// ---------------------------------------------------------------------------
static int check_geom(qp3d_ctx *ctx, const qp3d_geom *g)
{
    if (!g) return ctx_fail(ctx, QP3D_ERR_ARG, "null geometry");
    if (g->nx < 11 || g->ny < 11 || g->nz < 11)
        return ctx_fail(ctx, QP3D_ERR_ARG, "grid %dx%dx%d smaller than 11 cells", g->nx, g->ny, g->nz);
    if (g->pml < 0 || g->pml > kMaxPml || 2 * g->pml >= g->nx || 2 * g->pml >= g->ny ||
        2 * g->pml >= g->nz)
        return ctx_fail(ctx, QP3D_ERR_ARG, "pml %d invalid for grid %dx%dx%d", g->pml, g->nx, g->ny,
                    g->nz);
    if (g->nt < 0) return ctx_fail(ctx, QP3D_ERR_ARG, "nt < 0");
    if (g->sz < 0 || g->sz >= g->nz) return ctx_fail(ctx, QP3D_ERR_ARG, "sz %d outside [0,%d)", g->sz, g->nz);
    if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0) || !(g->dt > 0))
        return ctx_fail(ctx, QP3D_ERR_ARG, "non-positive spacing or time step");
    long long n = (long long)g->nx * g->ny * g->nz;
    if (n > (1ll << 40)) return ctx_fail(ctx, QP3D_ERR_ARG, "grid too large");
    return QP3D_OK;
}

static int make_tmap(qp3d_ctx *ctx, float *base, CUtensorMap *tm)
{
    const qp3d_geom &g = ctx->g;
    cuuint64_t dims[3] = {(cuuint64_t)g.ny, (cuuint64_t)g.nx, (cuuint64_t)g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)ctx->ldy * 4, (cuuint64_t)ctx->plane * 4};
    cuuint32_t box[3] = {(cuuint32_t)kBoxY, (cuuint32_t)(ctx->tile_x + 2 * kRadius), 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = ctx->encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return ctx_fail(ctx, QP3D_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return QP3D_OK;
}

static void plan_launch(qp3d_ctx *ctx)
{
    const qp3d_geom &g = ctx->g;
    int ncx = g.nx - 2 * kRadius;
    int ntx = (ncx + kMaxTileX - 1) / kMaxTileX;
    ctx->tile_x = (ncx + ntx - 1) / ntx;
    if (ctx->tune_tile_x > 0) ctx->tile_x = std::min(ctx->tune_tile_x, kMaxTileX);
    ctx->nxt = (ncx + ctx->tile_x - 1) / ctx->tile_x;
    ctx->nyt = (g.ny - kRadius - 1) / kTileY + 1;   // last tile starts below ny-5
    int ncz = g.nz - 2 * kRadius;
    long long tiles = (long long)ctx->nxt * ctx->nyt;
    long long target = 18ll * ctx->nsm;              // ~9 waves at 2 CTAs/SM
    int nch = (int)((target + tiles - 1) / tiles);
    int maxch = std::max(1, ncz / 24);
    nch = std::max(1, std::min(nch, maxch));
    if (ctx->tune_chunks > 0) nch = std::min(ctx->tune_chunks, ncz);
    ctx->chunk_z = (ncz + nch - 1) / nch;
    ctx->nchunks = (ncz + ctx->chunk_z - 1) / ctx->chunk_z;
    ctx->smem = plane_smem_bytes(ctx->tile_x, g.pml, ctx->fuse_sources ? ctx->n_fused : 0);
}

static int alloc_vol(qp3d_ctx *ctx, float **p)
{
    CK(cudaMalloc(p, (size_t)ctx->vol * sizeof(float)));
    return QP3D_OK;
}

// Copy a dense [nz][nx][ny] host volume into the pitched device layout.
static int upload_vol(qp3d_ctx *ctx, float *dst, const float *src)
{
    const qp3d_geom &g = ctx->g;
    CK(cudaMemcpy2DAsync(dst, (size_t)ctx->ldy * 4, src, (size_t)g.ny * 4, (size_t)g.ny * 4,
                         (size_t)g.nx * g.nz, cudaMemcpyHostToDevice, ctx->stream));
    return QP3D_OK;
}

static int download_vol(qp3d_ctx *ctx, float *dst, const float *src)
{
    const qp3d_geom &g = ctx->g;
    CK(cudaMemcpy2DAsync(dst, (size_t)g.ny * 4, src, (size_t)ctx->ldy * 4, (size_t)g.ny * 4,
                         (size_t)g.nx * g.nz, cudaMemcpyDeviceToHost, ctx->stream));
    return QP3D_OK;
}

extern "C" int qp3d_shot_load(qp3d_ctx *ctx, const qp3d_geom *g, const qp3d_model *m)
{
    if (!ctx) return QP3D_ERR_ARG;
    int rc = check_geom(ctx, g);
    if (rc) return rc;
    if (!m || !m->vp || !m->epsilon || !m->delta || !m->wavelet || !m->c || !m->c2)
        return ctx_fail(ctx, QP3D_ERR_ARG, "missing model input");
    if (g->pml > 0 && (!m->dlr || !m->ddlr || !m->dtb || !m->ddtb || !m->dfb || !m->ddfb))
        return ctx_fail(ctx, QP3D_ERR_ARG, "missing PML profiles");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));

    const bool half = ctx->param_fp16 != 0;
    bool same = ctx->loaded && ctx->g.nx == g->nx && ctx->g.ny == g->ny && ctx->g.nz == g->nz &&
                ctx->g.nt == g->nt && ctx->g.pml == g->pml && ctx->half_loaded == half;
    if (!same) free_shot(ctx);
    ctx->g = *g;
    ctx->ldy = (g->ny + 31) & ~31;
    ctx->plane = (long long)g->nx * ctx->ldy;
    ctx->vol = ctx->plane * g->nz;
    ctx->hx = g->nx - 2 * g->pml;
    ctx->hy = g->ny - 2 * g->pml;

    if (!same) {
        float **vols[] = {&ctx->U[0],  &ctx->U[1],  &ctx->U[2],  &ctx->W1[0], &ctx->W1[1],
                          &ctx->W1[2], &ctx->W3[0], &ctx->W3[1], &ctx->W3[2], &ctx->P[0],
                          &ctx->P[1],  &ctx->P[2],  &ctx->W21[0], &ctx->W21[1],
                          &ctx->VP,     &ctx->E2,    &ctx->R8};
        const int nvols = half ? 14 : 17;   // half storage: no FP32 parameter volumes
        for (int v = 0; v < nvols; ++v)
            if ((rc = alloc_vol(ctx, vols[v]))) {
                free_shot(ctx);
                return rc;
            }
        if (half) {
            __half **hs[] = {&ctx->h_vp, &ctx->h_eps, &ctx->h_del};
            for (__half **h : hs) CK(cudaMalloc(h, (size_t)ctx->vol * sizeof(__half)));
        }
        ctx->half_loaded = half;
        size_t nrec = (size_t)std::max(g->nt, 1) * ctx->hx * ctx->hy;
        CK(cudaMalloc(&ctx->record, nrec * sizeof(float)));
        CK(cudaMalloc(&ctx->gmax, (size_t)std::max(g->nt, 1) * sizeof(float)));
        CK(cudaMalloc(&ctx->layers, sizeof(float4) * 3 * std::max(g->pml, 1)));
        if (!ctx->errword) CK(cudaMalloc(&ctx->errword, sizeof(unsigned)));
        size_t ntb = (size_t)std::max(g->nt, 1);
        CK(cudaMalloc(&ctx->win, 3 * ntb * sizeof(float)));
        CK(cudaMalloc(&ctx->redo, ntb * sizeof(int)));
        CK(cudaMalloc(&ctx->alt_count, ntb * sizeof(unsigned)));
        CK(cudaMalloc(&ctx->spec_err, kSpecHist * sizeof(float)));
        // deferred cells of a speculative step: one bit per cell (vol is a
        // multiple of 32), m2 and the alternative value at the cell's index
        CK(cudaMalloc(&ctx->amask, (size_t)defer_mask_words(ctx->vol) * sizeof(unsigned)));
        CK(cudaMalloc(&ctx->am2, (size_t)ctx->vol * sizeof(float)));
        CK(cudaMalloc(&ctx->av, (size_t)ctx->vol * sizeof(float)));
        CK(cudaMalloc(&ctx->apml, (size_t)ctx->vol * sizeof(float4)));
        CK(cudaMalloc(&ctx->fix_count, ntb * sizeof(unsigned)));
        // compacted list: a quarter of the cells (more deferred cells than
        // that make the step re-run exactly)
        ctx->alist_cap = (unsigned)std::min<long long>(std::max(1ll << 16, ctx->vol / 4), 0x7fffffff);
        CK(cudaMalloc(&ctx->alist, (size_t)ctx->alist_cap * sizeof(unsigned)));
    }
    // vp, eps, delta go to the device in one piece each (the wavefield buffers
    // serve as staging; the reset below zeroes them) and are laid out pitched
    // on the device: as IEEE half, or as the per-cell parameters
    {
        const float *src[3] = {m->vp, m->epsilon, m->delta};
        const size_t dense = (size_t)g->nx * g->ny * g->nz * sizeof(float);
        for (int i = 0; i < 3; ++i)
            CK(cudaMemcpyAsync(ctx->U[i], src[i], dense, cudaMemcpyHostToDevice, ctx->stream));
        if (half) {
            __half *dst[3] = {ctx->h_vp, ctx->h_eps, ctx->h_del};
            for (int i = 0; i < 3; ++i)
                CKL(launch_to_half_dense(ctx->U[i], dst[i], g->nx, g->ny, g->nz, ctx->ldy,
                                         ctx->stream));
        } else {
            CKL(launch_params_dense(ctx->U[0], ctx->U[1], ctx->U[2], ctx->VP, ctx->E2, ctx->R8,
                                    g->nx, g->ny, g->nz, ctx->ldy, ctx->stream));
        }
    }
    // coefficient tables
    derive_coefs(m->c, m->c2, g->dx, g->dy, g->dz, &ctx->coefs);
    if (g->pml > 0) {
        std::vector<float4> tab(3 * g->pml);
        derive_layers(m->dlr, m->ddlr, g->pml, g->dt, tab.data());
        derive_layers(m->dfb, m->ddfb, g->pml, g->dt, tab.data() + g->pml);
        derive_layers(m->dtb, m->ddtb, g->pml, g->dt, tab.data() + 2 * g->pml);
        CK(cudaMemcpyAsync(ctx->layers, tab.data(), sizeof(float4) * tab.size(),
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    ctx->wavelet.assign(m->wavelet, m->wavelet + g->nt);
    // sparse source: every non-zero sample (CPU_function.c:326-338 adds all)
    std::vector<SrcEntry> fused, band, all;
    if (m->source) scan_source_volume(m->source, g->nx, g->ny, g->nz, all);
    for (const SrcEntry &e : all) {
        const bool inside = e.x >= kRadius && e.x < g->nx - kRadius && e.y >= kRadius &&
                            e.y < g->ny - kRadius && e.z >= kRadius && e.z < g->nz - kRadius;
        (inside ? fused : band).push_back(e);
    }
    if (ctx->src_fused) cudaFree(ctx->src_fused);
    if (ctx->src_band) cudaFree(ctx->src_band);
    if (ctx->src_all) cudaFree(ctx->src_all);
    ctx->src_fused = ctx->src_band = ctx->src_all = nullptr;
    ctx->fuse_sources = fused.size() <= (size_t)kMaxFusedSources;
    ctx->n_fused = (int)fused.size();
    ctx->n_band = (int)band.size();
    ctx->n_all = (int)all.size();
    auto up = [&](std::vector<SrcEntry> &v, SrcEntry **d) -> int {
        if (v.empty()) return QP3D_OK;
        CK(cudaMalloc(d, v.size() * sizeof(SrcEntry)));
        CK(cudaMemcpy(*d, v.data(), v.size() * sizeof(SrcEntry), cudaMemcpyHostToDevice));
        return QP3D_OK;
    };
    if ((rc = up(fused, &ctx->src_fused)) || (rc = up(band, &ctx->src_band)) ||
        (rc = up(all, &ctx->src_all)))
        return rc;
    // the receiver plane is written by the step kernel when every record cell
    // lies inside the updated box
    ctx->rec_fused = g->pml >= kRadius && g->sz >= kRadius && g->sz < g->nz - kRadius &&
                     ctx->fuse_sources && ctx->n_band == 0;
    plan_launch(ctx);   // after the sources: the per-CTA source list is in shared memory
    for (int i = 0; i < 3; ++i)
        if ((rc = make_tmap(ctx, ctx->U[i], &ctx->tm[i]))) return rc;
    ctx->loaded = true;
    return qp3d_shot_reset(ctx);
}

extern "C" int qp3d_shot_reset(qp3d_ctx *ctx)
{
    if (!ctx) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    CK(cudaSetDevice(ctx->device));
    size_t vb = (size_t)ctx->vol * sizeof(float);
    float *zero[] = {ctx->U[0],  ctx->U[1],  ctx->U[2],  ctx->W1[0], ctx->W1[1], ctx->W1[2],
                     ctx->W3[0], ctx->W3[1], ctx->W3[2], ctx->P[0],  ctx->P[1],  ctx->P[2],
                     ctx->W21[0], ctx->W21[1]};
    for (float *p : zero) CK(cudaMemsetAsync(p, 0, vb, ctx->stream));
    size_t ntb = (size_t)std::max(ctx->g.nt, 1);
    CK(cudaMemsetAsync(ctx->win, 0, 3 * ntb * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(ctx->redo, 0, ntb * sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->alt_count, 0, ntb * sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->fix_count, 0, ntb * sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->amask, 0, (size_t)defer_mask_words(ctx->vol) * sizeof(unsigned),
                       ctx->stream));
    // error history: no prediction yet (1.0 opens the widest window once)
    static const float first[kSpecHist] = {1.0f};
    CK(cudaMemcpyAsync(ctx->spec_err, first, sizeof(first), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->gmax, 0, sizeof(float) * std::max(ctx->g.nt, 1), ctx->stream));
    CK(cudaMemsetAsync(ctx->record, 0,
                       sizeof(float) * (size_t)std::max(ctx->g.nt, 1) * ctx->hx * ctx->hy,
                       ctx->stream));
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(unsigned), ctx->stream));
    ctx->step = 0;
    ctx->cur = 0;
    ctx->prev = 1;
    return QP3D_OK;
}

// Speculative threshold handling is used from this step on (the window is
// predicted from the two previous maxima).
constexpr int kSpecFirstStep = 3;

static bool use_spec(const qp3d_ctx *ctx, int k)
{
    return ctx->threshold_mode == 1 && ctx->dec_mode == 0 && k >= kSpecFirstStep &&
           ctx->vol < (1ll << 32);
}

// Enqueue one time step.  ev_* are optional events bracketing the main step
// kernel (s) and the threshold overhead kernels (g: gradmax, or fix-up plus
// the gated exact re-run).
static int enqueue_step(qp3d_ctx *ctx, cudaEvent_t ev_g0, cudaEvent_t ev_g1, cudaEvent_t ev_s0,
                        cudaEvent_t ev_s1)
{
    const qp3d_geom &g = ctx->g;
    const int k = ctx->step;
    const int a = ctx->cur, b = ctx->prev, c = 3 - a - b;
    PlaneParams p;
    memset(&p, 0, sizeof(p));
    p.nx = g.nx; p.ny = g.ny; p.nz = g.nz; p.ldy = ctx->ldy; p.pml = g.pml; p.sz = g.sz;
    p.tile_x = ctx->tile_x;
    p.chunk_z = ctx->chunk_z;
    p.plane = ctx->plane;
    p.k = ctx->coefs;
    p.dt = g.dt;
    p.step = k;
    p.wavelet = ctx->wavelet[k];
    p.u_cur = ctx->U[a];
    p.u_prev = ctx->U[b];
    p.u_out = ctx->U[c];
    p.prm_v = ctx->VP; p.prm_e = ctx->E2; p.prm_r = ctx->R8;
    p.h_vp = ctx->h_vp; p.h_eps = ctx->h_eps; p.h_del = ctx->h_del;
    p.half_params = ctx->half_loaded ? 1 : 0;
    const int lo = k % 3, lc = (k + 1) % 3, ln = (k + 2) % 3;
    p.w1o = ctx->W1[lo]; p.w1c = ctx->W1[lc]; p.w1n = ctx->W1[ln];
    p.w3o = ctx->W3[lo]; p.w3c = ctx->W3[lc]; p.w3n = ctx->W3[ln];
    p.po = ctx->P[lo];   p.pc = ctx->P[lc];   p.pn = ctx->P[ln];
    p.w21o = ctx->W21[k % 2];
    p.w21n = ctx->W21[(k + 1) % 2];
    p.layers = ctx->layers;
    p.arith = ctx->arith;
    p.wait_ns = ctx->wait_ns;
    p.hold_plane = ctx->hold_plane;
    if (ctx->dec_mode == 1) p.dec_out = ctx->dec_base + (size_t)k * ctx->dec_words;
    if (ctx->dec_mode == 2) p.dec_in = ctx->dec_base + (size_t)k * ctx->dec_words;
    p.gmax = ctx->gmax;
    float *rec_plane = ctx->record + (size_t)k * ctx->hx * ctx->hy;
    p.record = ctx->rec_fused ? rec_plane : nullptr;
    p.src = ctx->fuse_sources ? ctx->src_fused : nullptr;
    p.nsrc = ctx->fuse_sources ? ctx->n_fused : 0;
    p.err = ctx->errword;
    p.delta_min = ctx->delta_min;
    dim3 grid(ctx->nyt, ctx->nxt, ctx->nchunks);

    if (use_spec(ctx, k)) {
        p.spec = 1;
        p.win = ctx->win + 3 * (size_t)k;
        p.spec_err = ctx->spec_err;
        p.spec_bias = ctx->spec_bias;
        p.amask = ctx->amask;
        p.am2 = ctx->am2;
        p.av = ctx->av;
        p.apml = ctx->apml;
        p.alt_count = ctx->alt_count + k;
        p.alist = ctx->alist;
        p.alist_cap = ctx->alist_cap;
        p.fix_count = ctx->fix_count + k;
        if (ev_s0) CK(cudaEventRecord(ev_s0, ctx->stream));
        CKL(launch_step(ctx->tm[a], p, grid, ctx->smem, ctx->stream));
        if (ev_s1) CK(cudaEventRecord(ev_s1, ctx->stream));
        if (ev_g0) CK(cudaEventRecord(ev_g0, ctx->stream));
        CKL(launch_compact(p, ctx->redo + k, ctx->spec_err, ctx->stream));
        PlaneParams pe = p;
        pe.spec = 0;
        pe.gate = ctx->redo + k;
        CKL(launch_fix_or_rerun(ctx->tm[a], pe, ctx->nsm, ctx->smem, ctx->stream));
        if (ev_g1) CK(cudaEventRecord(ev_g1, ctx->stream));
    } else {
        if (ev_g0) CK(cudaEventRecord(ev_g0, ctx->stream));
        CKL(launch_gradmax(ctx->tm[a], p, grid, ctx->smem, ctx->stream, ctx->gradmax_variant));
        if (ev_g1) CK(cudaEventRecord(ev_g1, ctx->stream));
        if (ev_s0) CK(cudaEventRecord(ev_s0, ctx->stream));
        CKL(launch_step(ctx->tm[a], p, grid, ctx->smem, ctx->stream));
        if (ev_s1) CK(cudaEventRecord(ev_s1, ctx->stream));
    }
    if (ctx->fuse_sources) {
        if (ctx->n_band > 0)
            CKL(launch_band_sources(ctx->U[c], ctx->U[a], ctx->src_band, ctx->n_band, ctx->plane,
                               ctx->ldy, p.wavelet, ctx->stream));
    } else if (ctx->n_all > 0) {
        CKL(launch_all_sources(ctx->U[c], ctx->U[a], ctx->src_all, ctx->n_all, ctx->plane, ctx->ldy,
                              g.nx, g.ny, g.nz, p.wavelet, ctx->stream));
    }
    if (!ctx->rec_fused)
        CKL(launch_record(ctx->U[c], rec_plane, g.nx, g.ny, g.pml, g.sz, ctx->ldy, ctx->plane,
                         ctx->stream));
    ctx->prev = a;
    ctx->cur = c;
    ctx->step = k + 1;
    return QP3D_OK;
}

// For qp3d_adjoint.cu: one step of the loaded shot, and a jump back to the
// start of step `step` (rotation as from a reset; the per-step bookkeeping
// of the steps to come is cleared; the caller restores the state volumes).
int qp3d_internal_enqueue_step(qp3d_ctx *ctx)
{
    if (ctx->step >= ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_STATE, "step past nt");
    return enqueue_step(ctx, nullptr, nullptr, nullptr, nullptr);
}

// Wavefield buffers chosen by the caller for the next step (qp3d_adjoint keeps
// every u^k in an array of its own): the step reads u(k-1) from u_prev and
// u(k) from u_cur (its TMA map is encoded for that buffer) and writes u(k+1)
// to u_next.  Launches already enqueued keep the maps they were given.
int qp3d_internal_bind_wavefields(qp3d_ctx *ctx, float *u_prev, float *u_cur, float *u_next)
{
    const int a = ctx->cur, b = ctx->prev, c = 3 - a - b;
    ctx->U[a] = u_cur;
    ctx->U[b] = u_prev;
    ctx->U[c] = u_next;
    return make_tmap(ctx, u_cur, &ctx->tm[a]);
}

// The shot's own three wavefield buffers back in place, with their maps.
int qp3d_internal_restore_wavefields(qp3d_ctx *ctx, float *const U[3])
{
    int rc = QP3D_OK;
    for (int i = 0; i < 3; ++i) {
        ctx->U[i] = U[i];
        const int r = make_tmap(ctx, U[i], &ctx->tm[i]);
        if (r && !rc) rc = r;
    }
    return rc;
}

int qp3d_internal_restore_step(qp3d_ctx *ctx, int step)
{
    if (step < 0 || step >= ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_ARG, "bad step %d", step);
    const size_t n = (size_t)(ctx->g.nt - step);
    CK(cudaMemsetAsync(ctx->gmax + step, 0, n * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(ctx->win + 3 * (size_t)step, 0, 3 * n * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(ctx->redo + step, 0, n * sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->alt_count + step, 0, n * sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->fix_count + step, 0, n * sizeof(unsigned), ctx->stream));
    ctx->step = step;
    ctx->cur = (3 - step % 3) % 3;
    ctx->prev = (ctx->cur + 1) % 3;
    return QP3D_OK;
}

extern "C" int qp3d_shot_launches_per_step(const qp3d_ctx *ctx)
{
    if (!ctx || !ctx->loaded) return 0;
    int n = use_spec(ctx, ctx->step) ? 3 : 2;   // step, compaction, fix-up or re-run
    if (ctx->fuse_sources) n += ctx->n_band > 0 ? 1 : 0;
    else n += ctx->n_all > 0 ? 1 : 0;
    if (!ctx->rec_fused) n += 1;
    return n;
}

extern "C" int qp3d_shot_advance(qp3d_ctx *ctx, int nsteps)
{
    if (!ctx || nsteps < 0) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    if (ctx->step + nsteps > ctx->g.nt)
        return ctx_fail(ctx, QP3D_ERR_ARG, "advance past nt (%d + %d > %d)", ctx->step, nsteps, ctx->g.nt);
    CK(cudaSetDevice(ctx->device));
    for (int i = 0; i < nsteps; ++i) {
        int rc = enqueue_step(ctx, nullptr, nullptr, nullptr, nullptr);
        if (rc) return rc;
    }
    return QP3D_OK;
}

extern "C" int qp3d_shot_sync(qp3d_ctx *ctx)
{
    if (!ctx) return QP3D_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->errword) {
        unsigned e = 0;
        CK(cudaMemcpy(&e, ctx->errword, sizeof(e), cudaMemcpyDeviceToHost));
        if (e) return ctx_fail(ctx, QP3D_ERR_TIMEOUT, "device wait timed out (flags 0x%x)", e);
    }
    return QP3D_OK;
}

extern "C" int qp3d_shot_step(const qp3d_ctx *ctx) { return ctx ? ctx->step : -1; }

extern "C" int qp3d_shot_read_record(qp3d_ctx *ctx, int k0, int nsteps, float *out)
{
    if (!ctx || !out || k0 < 0 || nsteps < 0) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    if (k0 + nsteps > ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_ARG, "record range past nt");
    int rc = qp3d_shot_sync(ctx);
    if (rc) return rc;
    size_t row = (size_t)ctx->hx * ctx->hy;
    CK(cudaMemcpy(out, ctx->record + (size_t)k0 * row, row * nsteps * sizeof(float),
                  cudaMemcpyDeviceToHost));
    return QP3D_OK;
}

extern "C" int qp3d_shot_read_uxyzmax(qp3d_ctx *ctx, int k0, int nsteps, float *out)
{
    if (!ctx || !out || k0 < 0 || nsteps < 0) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    if (k0 + nsteps > ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_ARG, "range past nt");
    int rc = qp3d_shot_sync(ctx);
    if (rc) return rc;
    CK(cudaMemcpy(out, ctx->gmax + k0, nsteps * sizeof(float), cudaMemcpyDeviceToHost));
    return QP3D_OK;
}

// ---------------------------------------------------------------------------
// State in the reference layout
// ---------------------------------------------------------------------------
namespace {
struct FaceLayout {
    size_t fsz[6];
    size_t off[6][10];
    size_t total;
};
FaceLayout face_layout(int nx, int ny, int nz, int pml)
{
    FaceLayout L;
    size_t xf = (size_t)pml * ny * nz, yf = (size_t)pml * nx * nz, zf = (size_t)pml * nx * ny;
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
    return L;
}
// cell (z,x,y) -> face-local index, or -1 when the cell is not in face f
long long face_index(int f, int z, int x, int y, int nx, int ny, int nz, int pml)
{
    switch (f) {
    case 0: return x < pml ? (long long)z * ny * pml + (long long)x * ny + y : -1;
    case 1: return x >= nx - pml ? (long long)z * ny * pml + (long long)(x - nx + pml) * ny + y : -1;
    case 2: return y < pml ? (long long)z * nx * pml + (long long)x * pml + y : -1;
    case 3: return y >= ny - pml ? (long long)z * nx * pml + (long long)x * pml + (y - ny + pml) : -1;
    case 4: return z < pml ? (long long)z * nx * ny + (long long)x * ny + y : -1;
    default: return z >= nz - pml ? (long long)(z - nz + pml) * ny * nx + (long long)x * ny + y : -1;
    }
}
int region(int x, int y, int z, int nx, int ny, int nz, int pml)
{
    if (x < pml) return 0;
    if (x >= nx - pml) return 1;
    if (y < pml) return 2;
    if (y >= ny - pml) return 3;
    if (z < pml) return 4;
    if (z >= nz - pml) return 5;
    return -1;
}
}  // namespace

extern "C" size_t qp3d_pml_state_size(int nx, int ny, int nz, int pml)
{
    if (nx <= 0 || ny <= 0 || nz <= 0 || pml < 0) return 0;
    return face_layout(nx, ny, nz, pml).total;
}

// shadow-volume arrays in the order of the face arrays (w11..p3) for step k
static void level_arrays(qp3d_ctx *ctx, int k, float *arr[10])
{
    const int lo = k % 3, lc = (k + 1) % 3, ln = (k + 2) % 3;
    arr[0] = ctx->W1[lo]; arr[1] = ctx->W1[lc]; arr[2] = ctx->W1[ln]; arr[3] = ctx->W21[k % 2];
    arr[4] = ctx->W3[lo]; arr[5] = ctx->W3[lc]; arr[6] = ctx->W3[ln];
    arr[7] = ctx->P[lo];  arr[8] = ctx->P[lc];  arr[9] = ctx->P[ln];
}

extern "C" int qp3d_shot_write_state(qp3d_ctx *ctx, int step, const float *u_prev,
                                     const float *u_cur, const float *pml_state)
{
    if (!ctx) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    if (step < 0 || step > ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_ARG, "step out of range");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->step = step;
    int rc;
    if (u_prev && (rc = upload_vol(ctx, ctx->U[ctx->prev], u_prev))) return rc;
    if (u_cur && (rc = upload_vol(ctx, ctx->U[ctx->cur], u_cur))) return rc;
    if (pml_state) {
        const qp3d_geom &g = ctx->g;
        FaceLayout L = face_layout(g.nx, g.ny, g.nz, g.pml);
        float *arr[10];
        level_arrays(ctx, step, arr);
        std::vector<float> tmp((size_t)ctx->vol);
        for (int a = 0; a < 10; ++a) {
            std::fill(tmp.begin(), tmp.end(), 0.0f);
            for (int z = 0; z < g.nz; ++z)
                for (int x = 0; x < g.nx; ++x)
                    for (int y = 0; y < g.ny; ++y) {
                        int f = region(x, y, z, g.nx, g.ny, g.nz, g.pml);
                        if (f < 0) continue;
                        long long fi = face_index(f, z, x, y, g.nx, g.ny, g.nz, g.pml);
                        tmp[(size_t)z * ctx->plane + (size_t)x * ctx->ldy + y] =
                            pml_state[L.off[f][a] + fi];
                    }
            CK(cudaMemcpy(arr[a], tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return QP3D_OK;
}

extern "C" int qp3d_shot_read_state(qp3d_ctx *ctx, float *u_prev, float *u_cur, float *pml_state)
{
    if (!ctx) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    int rc = qp3d_shot_sync(ctx);
    if (rc) return rc;
    if (u_prev && (rc = download_vol(ctx, u_prev, ctx->U[ctx->prev]))) return rc;
    if (u_cur && (rc = download_vol(ctx, u_cur, ctx->U[ctx->cur]))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    if (pml_state) {
        const qp3d_geom &g = ctx->g;
        FaceLayout L = face_layout(g.nx, g.ny, g.nz, g.pml);
        memset(pml_state, 0, L.total * sizeof(float));
        // levels as the next step will read them: w11 = w(k-1), w12 = w(k)
        float *arr[10];
        level_arrays(ctx, ctx->step, arr);
        std::vector<float> tmp((size_t)ctx->vol);
        for (int a = 0; a < 10; ++a) {
            CK(cudaMemcpy(tmp.data(), arr[a], tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
            for (int z = 0; z < g.nz; ++z)
                for (int x = 0; x < g.nx; ++x)
                    for (int y = 0; y < g.ny; ++y) {
                        int f = region(x, y, z, g.nx, g.ny, g.nz, g.pml);
                        if (f < 0) continue;
                        long long fi = face_index(f, z, x, y, g.nx, g.ny, g.nz, g.pml);
                        pml_state[L.off[f][a] + fi] =
                            tmp[(size_t)z * ctx->plane + (size_t)x * ctx->ldy + y];
                    }
        }
        // after the reference's exchange w13 == w12, w33 == w32, p3 == p2
        for (int f = 0; f < 6; ++f) {
            memcpy(pml_state + L.off[f][2], pml_state + L.off[f][1], L.fsz[f] * sizeof(float));
            memcpy(pml_state + L.off[f][6], pml_state + L.off[f][5], L.fsz[f] * sizeof(float));
            memcpy(pml_state + L.off[f][9], pml_state + L.off[f][8], L.fsz[f] * sizeof(float));
        }
    }
    return QP3D_OK;
}

// ---------------------------------------------------------------------------
// Snapshots
// ---------------------------------------------------------------------------
static int ensure_snap(qp3d_ctx *ctx, size_t n)
{
    if (n <= ctx->snap_cap) return QP3D_OK;
    if (ctx->snap_dev) cudaFree(ctx->snap_dev);
    if (ctx->snap_host) cudaFreeHost(ctx->snap_host);
    ctx->snap_dev = nullptr;
    ctx->snap_host = nullptr;
    ctx->snap_cap = 0;
    CK(cudaMalloc(&ctx->snap_dev, n * sizeof(float)));
    CK(cudaMallocHost(&ctx->snap_host, n * sizeof(float)));
    ctx->snap_cap = n;
    return QP3D_OK;
}

// The four snapshot regions of the reference (3dPureqPModeling_single_shot.cu:340-377):
// the interior volume and its mid xz, yz and xy slices.
struct SnapReq {
    int kind, x0, x1, y0, y1, z0, z1, n0, n1, n2;
    size_t size() const { return (size_t)(x1 - x0) * (y1 - y0) * (z1 - z0); }
};

static void snap_requests(const qp3d_ctx *ctx, SnapReq reqs[4])
{
    const int pml = ctx->g.pml, hx = ctx->hx, hy = ctx->hy, hz = ctx->g.nz - 2 * pml;
    reqs[0] = {QP3D_SNAP_VOLUME, pml, pml + hx, pml, pml + hy, pml, pml + hz, hz, hx, hy};
    reqs[1] = {QP3D_SNAP_XZ, pml, pml + hx, pml + (hy - 1) / 2, pml + (hy - 1) / 2 + 1, pml, pml + hz,
               hz, hx, 1};
    reqs[2] = {QP3D_SNAP_YZ, pml + (hx - 1) / 2, pml + (hx - 1) / 2 + 1, pml, pml + hy, pml, pml + hz,
               hz, hy, 1};
    reqs[3] = {QP3D_SNAP_XY, pml, pml + hx, pml, pml + hy, pml + (hz - 1) / 2, pml + (hz - 1) / 2 + 1,
               hx, hy, 1};
}

extern "C" int qp3d_shot_snapshot(qp3d_ctx *ctx, const qp3d_snap *snap)
{
    if (!ctx || !snap || !snap->fn) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    const float *u = ctx->U[ctx->cur];
    const int k = ctx->step - 1;
    SnapReq reqs[4];
    snap_requests(ctx, reqs);
    for (const SnapReq &r : reqs) {
        if (!(snap->kinds & (1u << r.kind))) continue;
        size_t n = r.size();
        int rc = ensure_snap(ctx, n);
        if (rc) return rc;
        CKL(launch_crop(u, ctx->snap_dev, r.x0, r.x1, r.y0, r.y1, r.z0, r.z1, ctx->ldy, ctx->plane,
                       ctx->stream));
        CK(cudaMemcpyAsync(ctx->snap_host, ctx->snap_dev, n * sizeof(float), cudaMemcpyDeviceToHost,
                           ctx->stream));
        rc = qp3d_shot_sync(ctx);
        if (rc) return rc;
        if (snap->fn(snap->user, k, r.kind, ctx->snap_host, r.n0, r.n1, r.n2) != 0)
            return ctx_fail(ctx, QP3D_ERR_CALLBACK, "snapshot callback failed at step %d", k);
    }
    return QP3D_OK;
}

// Snapshots of qp3d_forward without stopping the time loop.  A snapshot after
// step k crops its slices on the step stream into a device slot (the crop
// runs before step k + 2 overwrites u(k)), and copy_stream moves the slot to
// its page-locked host twin; the host delivers the slots in step order as
// their copies land, polling between pieces of steps, and waits only when
// every slot is taken.  The callbacks therefore see the same data at the same
// step numbers as with qp3d_shot_snapshot, while later steps already run.
static int snap_slots(size_t floats)
{
    const size_t budget = (size_t)512 << 20;   // bytes of device (and host) slots
    const size_t n = budget / std::max<size_t>(floats * sizeof(float), 1);
    return (int)std::max<size_t>(1, std::min<size_t>(n, qp3d_ctx::kSnapSlots));
}

static int snap_deliver(qp3d_ctx *ctx, const qp3d_snap *snap, int nslots, bool wait)
{
    SnapReq reqs[4];
    snap_requests(ctx, reqs);
    while (ctx->snap_count > 0) {
        qp3d_ctx::SnapSlot &sl = ctx->sring[ctx->snap_head];
        if (!wait) {
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) break;
            CK(q);
        } else {
            CK(cudaEventSynchronize(sl.done));
        }
        size_t off = 0;
        for (const SnapReq &r : reqs) {
            if (!(sl.kinds & (1u << r.kind))) continue;
            if (snap->fn(snap->user, sl.step, r.kind, sl.host + off, r.n0, r.n1, r.n2) != 0)
                return ctx_fail(ctx, QP3D_ERR_CALLBACK, "snapshot callback failed at step %d",
                                sl.step);
            off += r.size();
        }
        ctx->snap_head = (ctx->snap_head + 1) % nslots;
        --ctx->snap_count;
    }
    return QP3D_OK;
}

static int snap_enqueue(qp3d_ctx *ctx, const qp3d_snap *snap, int nslots)
{
    SnapReq reqs[4];
    snap_requests(ctx, reqs);
    size_t total = 0;
    for (const SnapReq &r : reqs)
        if (snap->kinds & (1u << r.kind)) total += r.size();
    if (ctx->snap_count == nslots) {
        // every slot is taken: wait for the oldest, then deliver what has landed
        CK(cudaEventSynchronize(ctx->sring[ctx->snap_head].done));
        const int rc = snap_deliver(ctx, snap, nslots, false);
        if (rc) return rc;
    }
    qp3d_ctx::SnapSlot &sl = ctx->sring[(ctx->snap_head + ctx->snap_count) % nslots];
    if (!sl.ready) {
        CK(cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
    }
    if (sl.cap < total) {
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        sl.dev = sl.host = nullptr;
        sl.cap = 0;
        CK(cudaMalloc(&sl.dev, total * sizeof(float)));
        CK(cudaMallocHost(&sl.host, total * sizeof(float)));
        sl.cap = total;
    }
    const float *u = ctx->U[ctx->cur];
    size_t off = 0;
    for (const SnapReq &r : reqs) {
        if (!(snap->kinds & (1u << r.kind))) continue;
        CKL(launch_crop(u, sl.dev + off, r.x0, r.x1, r.y0, r.y1, r.z0, r.z1, ctx->ldy, ctx->plane,
                        ctx->stream));
        off += r.size();
    }
    CK(cudaEventRecord(sl.ready, ctx->stream));
    CK(cudaStreamWaitEvent(ctx->copy_stream, sl.ready, 0));
    CK(cudaMemcpyAsync(sl.host, sl.dev, total * sizeof(float), cudaMemcpyDeviceToHost,
                       ctx->copy_stream));
    CK(cudaEventRecord(sl.done, ctx->copy_stream));
    sl.step = ctx->step - 1;
    sl.kinds = snap->kinds;
    ++ctx->snap_count;
    return QP3D_OK;
}

// ---------------------------------------------------------------------------
extern "C" int qp3d_forward(qp3d_ctx *ctx, const qp3d_geom *g, const qp3d_model *m, float *record,
                            const qp3d_snap *snap)
{
    if (!ctx || !record) return QP3D_ERR_ARG;
    int rc = qp3d_shot_load(ctx, g, m);
    if (rc) return rc;
    // A page-locked record buffer is filled while the time loop runs: the
    // planes of each finished piece of steps go to the host on a second
    // stream (the reference copies the whole wavefield back every step,
    // 3dPureqPModeling_single_shot.cu:320); a pageable one is read at the end.
    cudaPointerAttributes attr;
    const bool pinned = cudaPointerGetAttributes(&attr, record) == cudaSuccess &&
                        attr.type == cudaMemoryTypeHost;
    (void)cudaGetLastError();
    const bool snaps = snap && snap->fn && snap->ntsnap > 0 && snap->kinds;
    if ((pinned || snaps) && !ctx->copy_stream) {
        CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->copy_ev, cudaEventDisableTiming));
    }
    const size_t row = (size_t)ctx->hx * ctx->hy;
    int nslots = 1;
    if (snaps) {
        SnapReq reqs[4];
        snap_requests(ctx, reqs);
        size_t total = 0;
        for (const SnapReq &r : reqs)
            if (snap->kinds & (1u << r.kind)) total += r.size();
        nslots = snap_slots(total);
        ctx->snap_head = ctx->snap_count = 0;
    }
    constexpr int kChunk = 100;   // steps per streamed piece of the record
    int k = 0, sent = 0;
    while (k < g->nt && rc == QP3D_OK) {
        int n = std::min(g->nt - k, kChunk);
        if (snaps) {
            // the reference snapshots after step k when k % ntsnap == 0
            int next = (k % snap->ntsnap == 0) ? k : (k / snap->ntsnap + 1) * snap->ntsnap;
            n = std::min(n, next - k + 1);
        }
        if ((rc = qp3d_shot_advance(ctx, n))) break;
        k += n;
        if (pinned && (k - sent >= kChunk || k == g->nt)) {
            cudaError_t e = cudaEventRecord(ctx->copy_ev, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev, 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(record + (size_t)sent * row, ctx->record + (size_t)sent * row,
                                    (size_t)(k - sent) * row * sizeof(float),
                                    cudaMemcpyDeviceToHost, ctx->copy_stream);
            if (e != cudaSuccess) {
                rc = ctx_fail(ctx, QP3D_ERR_CUDA, "record copy: %s", cudaGetErrorString(e));
                break;
            }
            sent = k;
        }
        if (snaps && (k - 1) % snap->ntsnap == 0) rc = snap_enqueue(ctx, snap, nslots);
        if (snaps && !rc) rc = snap_deliver(ctx, snap, nslots, false);
    }
    if (snaps && !rc) rc = snap_deliver(ctx, snap, nslots, true);
    if (snaps) ctx->snap_count = 0;   // after an error: the pending slots are dropped
    if (!pinned) {
        if (snaps) (void)cudaStreamSynchronize(ctx->copy_stream);
        return rc ? rc : qp3d_shot_read_record(ctx, 0, g->nt, record);
    }
    // no copy into the caller's buffer may outlive the call, also on error
    const cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
    if (rc) return rc;
    if ((rc = qp3d_shot_sync(ctx))) return rc;
    if (e != cudaSuccess)
        return ctx_fail(ctx, QP3D_ERR_CUDA, "record copy: %s", cudaGetErrorString(e));
    return QP3D_OK;
}

// ---------------------------------------------------------------------------
extern "C" int qp3d_shot_time(qp3d_ctx *ctx, int nsteps, float *ms_total, float *ms_step,
                              float *ms_gradmax)
{
    if (!ctx || nsteps < 0) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    if (ctx->step + nsteps > ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_ARG, "advance past nt");
    CK(cudaSetDevice(ctx->device));
    const bool per_kernel = ms_step || ms_gradmax;
    std::vector<cudaEvent_t> evs;
    if (per_kernel) {
        evs.resize((size_t)4 * nsteps);
        for (auto &e : evs) CK(cudaEventCreate(&e));
    }
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    for (int i = 0; i < nsteps; ++i) {
        int rc = per_kernel ? enqueue_step(ctx, evs[4 * i], evs[4 * i + 1], evs[4 * i + 2], evs[4 * i + 3])
                            : enqueue_step(ctx, nullptr, nullptr, nullptr, nullptr);
        if (rc) return rc;
    }
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    int rc = qp3d_shot_sync(ctx);
    if (rc) return rc;
    float t = 0;
    CK(cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
    if (ms_total) *ms_total = t;
    if (per_kernel) {
        float sg = 0, ss = 0;
        for (int i = 0; i < nsteps; ++i) {
            float a = 0, b = 0;
            CK(cudaEventElapsedTime(&a, evs[4 * i], evs[4 * i + 1]));
            CK(cudaEventElapsedTime(&b, evs[4 * i + 2], evs[4 * i + 3]));
            sg += a;
            ss += b;
        }
        for (auto &e : evs) cudaEventDestroy(e);
        if (ms_step) *ms_step = ss;
        if (ms_gradmax) *ms_gradmax = sg;
    }
    return QP3D_OK;
}

// ---------------------------------------------------------------------------
extern "C" int qp3d_event_record(qp3d_ctx *ctx, int slot)
{
    if (!ctx || slot < 0 || slot >= 8) return QP3D_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaEventRecord(ctx->uev[slot], ctx->stream));
    return QP3D_OK;
}

extern "C" int qp3d_event_elapsed(qp3d_ctx *ctx, int a, int b, float *ms)
{
    if (!ctx || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return QP3D_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaEventSynchronize(ctx->uev[b]));
    CK(cudaEventElapsedTime(ms, ctx->uev[a], ctx->uev[b]));
    return QP3D_OK;
}

extern "C" void *qp3d_host_alloc(size_t bytes)
{
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}

extern "C" void qp3d_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

namespace qp3d {
int noalloc_tune(const char *key, int value);   // qp3d_noalloc.cu
}

extern "C" int qp3d_tune(qp3d_ctx *ctx, const char *key, int value)
{
    if (!ctx && key) return noalloc_tune(key, value);
    if (!ctx || !key) return QP3D_ERR_ARG;
    if (!strcmp(key, "gradmax_variant") && (value == 0 || value == 1)) ctx->gradmax_variant = value;
    else if (!strcmp(key, "tile_x") && value >= 0 && value <= kMaxTileX) ctx->tune_tile_x = value;
    else if (!strcmp(key, "chunks") && value >= 0) ctx->tune_chunks = value;
    else if (!strcmp(key, "threshold_mode") && (value == 0 || value == 1)) ctx->threshold_mode = value;
    else if (!strcmp(key, "spec_delta_ppm") && value >= 0 && value <= 250000)
        ctx->delta_min = value * 1e-6f, ctx->delta_min_set = true;
    else if (!strcmp(key, "batch_graph") && (value == 0 || value == 1)) ctx->batch_graph = value;
    else if (!strcmp(key, "batch_tune") && (value == 0 || value == 1)) ctx->batch_tune = value;
    else if (!strcmp(key, "batch_candidate") && value >= -1 && value < 16)
        ctx->batch_candidate = value;
    else if (!strcmp(key, "batch_mem_mb") && value >= 0) ctx->batch_mem_mb = value;
    else if (!strcmp(key, "spec_bias_ppm") && value >= -500000 && value <= 1000000)
        ctx->spec_bias = value * 1e-6f;
    else if (!strcmp(key, "param_fp16") && (value == 0 || value == 1)) ctx->param_fp16 = value;
    else if (!strcmp(key, "arith") && (value == kArithRef || value == kArithFast)) ctx->arith = value;
    else if (!strcmp(key, "wait_limit_us") && value >= 0) ctx->wait_ns = 1000ull * (unsigned)value;
    else if (!strcmp(key, "test_hold_plane") && value >= -1) ctx->hold_plane = value + 1;
    else if (!strcmp(key, "adj_ckpt_bf16") && (value == 0 || value == 1)) ctx->adj_bf16 = value;
    else if (!strcmp(key, "adj_keep_all") && value >= -1 && value <= 1) ctx->adj_keep = value;
    else if (!strcmp(key, "adj_live") && (value == 0 || value == 1)) ctx->adj_live = value;
    else return ctx_fail(ctx, QP3D_ERR_ARG, "unknown tuning key or value: %s=%d", key, value);
    if (ctx->loaded && (!strcmp(key, "tile_x") || !strcmp(key, "chunks"))) {
        CK(cudaSetDevice(ctx->device));
        CK(cudaStreamSynchronize(ctx->stream));
        plan_launch(ctx);
        int rc;
        for (int i = 0; i < 3; ++i)
            if ((rc = make_tmap(ctx, ctx->U[i], &ctx->tm[i]))) return rc;
    }
    return QP3D_OK;
}

extern "C" int qp3d_tune_get(const qp3d_ctx *ctx, const char *key)
{
    if (!ctx || !key) return QP3D_ERR_ARG;
    if (!strcmp(key, "gradmax_variant")) return ctx->gradmax_variant;
    if (!strcmp(key, "tile_x")) return ctx->loaded ? ctx->tile_x : ctx->tune_tile_x;
    if (!strcmp(key, "chunks")) return ctx->loaded ? ctx->nchunks : ctx->tune_chunks;
    if (!strcmp(key, "threshold_mode")) return ctx->threshold_mode;
    if (!strcmp(key, "spec_delta_ppm")) return (int)(ctx->delta_min * 1e6f + 0.5f);
    if (!strcmp(key, "spec_bias_ppm")) return (int)lrintf(ctx->spec_bias * 1e6f);
    if (!strcmp(key, "param_fp16")) return ctx->param_fp16;
    if (!strcmp(key, "arith")) return ctx->arith;
    if (!strcmp(key, "wait_limit_us"))
        return (int)((ctx->wait_ns ? ctx->wait_ns : 2000000000ull) / 1000ull);
    if (!strcmp(key, "test_hold_plane")) return ctx->hold_plane - 1;
    if (!strcmp(key, "adj_ckpt_bf16")) return ctx->adj_bf16;
    if (!strcmp(key, "adj_keep_all")) return ctx->adj_keep;
    if (!strcmp(key, "adj_live")) return ctx->adj_live;
    if (!strcmp(key, "batch_graph")) return ctx->batch_graph;
    if (!strcmp(key, "batch_tune")) return ctx->batch_tune;
    if (!strcmp(key, "batch_candidate")) return ctx->batch_candidate;
    if (!strcmp(key, "batch_mem_mb")) return (int)ctx->batch_mem_mb;
    return QP3D_ERR_ARG;
}

extern "C" int qp3d_shot_read_stats(qp3d_ctx *ctx, int k0, int nsteps, int *redo, unsigned *alt)
{
    if (!ctx || k0 < 0 || nsteps < 0) return QP3D_ERR_ARG;
    if (!ctx->loaded) return ctx_fail(ctx, QP3D_ERR_STATE, "no shot loaded");
    if (k0 + nsteps > ctx->g.nt) return ctx_fail(ctx, QP3D_ERR_ARG, "range past nt");
    int rc = qp3d_shot_sync(ctx);
    if (rc) return rc;
    if (redo) CK(cudaMemcpy(redo, ctx->redo + k0, nsteps * sizeof(int), cudaMemcpyDeviceToHost));
    if (alt)
        CK(cudaMemcpy(alt, ctx->alt_count + k0, nsteps * sizeof(unsigned), cudaMemcpyDeviceToHost));
    return QP3D_OK;
}

extern "C" long long qp3d_ctx_launch_count(const qp3d_ctx *ctx) { return ctx ? ctx->launches : -1; }
