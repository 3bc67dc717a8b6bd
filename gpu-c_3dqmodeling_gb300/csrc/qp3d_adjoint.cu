// qp3d_adjoint.cu -- gradient of the L2 record misfit (qp3d_adjoint of
// include/qp3d.h).  No counterpart in the reference.
//
// Operator: the forward step with its scalar operator S frozen per step and
// cell (decision and unit normal from the forward wavefield, dependence on
// eps and delta differentiated); with S frozen the step is linear in the
// state (u, u_prev and the split-field PML state), and the adjoint is its
// exact transpose (kernels qp3d_adj_a/b_kernel).  The FP64 oracle
// (oracle/qp3d_adjoint.c) implements the same operator and passes
// dot-product and finite-difference tests.
//
// Schedule: the adjoint step reads u^k (S and its derivatives) and nothing
// else of the forward state.  When the nt wavefields fit in device memory
// (240x240x190 padded cells x 2000 steps is 88 GB) the forward pass keeps
// every u^k and the backward pass runs straight through.  Otherwise the
// forward pass stores the state every C = ceil(sqrt(nt)) steps (nine volumes:
// u, u_prev and the seven live PML levels) and the backward pass restores
// each checkpoint, recomputes its C steps keeping u^k, and runs the C adjoint
// steps backward.  By default ("adj_ckpt_bf16" = 1) the seven PML levels of a
// checkpoint are stored in BF16 (22 instead of 36 bytes per cell and
// checkpoint) and the forward pass also records every step's threshold
// decisions (one bit per cell and step), which the recomputation replays
// instead of re-deciding: the rounded PML levels then change the recomputed
// wavefield by rounding-sized amounts but never flip a decision of S, whose
// threshold is a discontinuity of the operator and dominated the delta
// gradient's error without the replay (cosine against FP32 checkpoints 0.91
// on 16 shots of 240x240x190).  u and u_prev stay FP32: S depends on the
// direction of grad u, a difference of neighbouring values that BF16
// rounding of a smooth wavefield would destroy.  With "adj_ckpt_bf16" = 0 the
// checkpoints are FP32 and the recomputation is bit-identical to the forward.
// Device memory: ~27 volumes plus nt (all kept) or C volumes, the checkpoints
// and nt/32 volumes of decision bits.  Gradients are summed per shot in FP32
// on the device and added to the caller's FP64 arrays.
#include "qp3d_ctx.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

using namespace qp3d;

// qp3d_api.cu
int qp3d_internal_enqueue_step(qp3d_ctx *ctx);
int qp3d_internal_restore_step(qp3d_ctx *ctx, int step);
int qp3d_internal_bind_wavefields(qp3d_ctx *ctx, float *u_prev, float *u_cur, float *u_next);
int qp3d_internal_restore_wavefields(qp3d_ctx *ctx, float *const U[3]);

namespace qp3d {

struct AdjState {
    long long vol = 0;
    int nt = 0, C = 0, nck = 0, bf16 = 1, keep = 0;
    float *L[9] = {}, *N[9] = {}, *Cf[6] = {}, *g[3] = {};
    float *seg = nullptr;          // C volumes: u^k of the segment (keep: C = nt)
    void *ck = nullptr;            // nck checkpoints x 9 volumes
    float *resid = nullptr;        // nt * hx * hy: d_obs, then the residual
    float *T2 = nullptr;           // thresholds of a segment
    unsigned *dec = nullptr;       // checkpoint schedule: every step's decisions
    double *misfit = nullptr;
};

void adjoint_free(AdjState *s)
{
    if (!s) return;
    for (auto *p : s->L) cudaFree(p);
    for (auto *p : s->N) cudaFree(p);
    for (auto *p : s->Cf) cudaFree(p);
    for (auto *p : s->g) cudaFree(p);
    cudaFree(s->seg);
    cudaFree(s->ck);
    cudaFree(s->resid);
    cudaFree(s->T2);
    cudaFree(s->dec);
    cudaFree(s->misfit);
    delete s;
}

}  // namespace qp3d

namespace {

// The nine live state volumes at the start of step k (the rotation of
// enqueue_step: PML levels k % 3 (old) and (k + 1) % 3 (current), W21 k % 2).
void live_state(qp3d_ctx *ctx, int k, float *v[9])
{
    v[0] = ctx->U[ctx->cur];
    v[1] = ctx->U[ctx->prev];
    v[2] = ctx->W1[(k + 1) % 3];
    v[3] = ctx->W1[k % 3];
    v[4] = ctx->P[(k + 1) % 3];
    v[5] = ctx->P[k % 3];
    v[6] = ctx->W21[k % 2];
    v[7] = ctx->W3[(k + 1) % 3];
    v[8] = ctx->W3[k % 3];
}

int alloc_state(qp3d_ctx *ctx, AdjState *s, int C, int nck, int bf16, int keep, size_t rec)
{
    const size_t vb = (size_t)s->vol * sizeof(float);
    for (int i = 0; i < 9; ++i) {
        CK(cudaMalloc(&s->L[i], vb));
        CK(cudaMalloc(&s->N[i], vb));
    }
    for (auto *&p : s->Cf) CK(cudaMalloc(&p, vb));
    for (auto *&p : s->g) CK(cudaMalloc(&p, vb));
    CK(cudaMalloc(&s->seg, vb * C));
    // the row padding of a wavefield is never written by a step: zero it once
    CK(cudaMemset(s->seg, 0, vb * C));
    const size_t per = (size_t)s->vol * (bf16 ? 2 * sizeof(float) + 7 * sizeof(__nv_bfloat16)
                                              : 9 * sizeof(float));
    if (nck) CK(cudaMalloc(&s->ck, per * nck));
    CK(cudaMalloc(&s->resid, rec * sizeof(float)));
    CK(cudaMalloc(&s->T2, sizeof(float) * C));
    if (nck) {   // one bit per cell and step: the forward's threshold decisions
        const size_t db = (size_t)s->nt * (size_t)(s->vol / 32) * sizeof(unsigned);
        CK(cudaMalloc(&s->dec, db));
        CK(cudaMemset(s->dec, 0, db));
    }
    CK(cudaMalloc(&s->misfit, sizeof(double)));
    s->C = C;
    s->nck = nck;
    s->bf16 = bf16;
    s->keep = keep;
    return QP3D_OK;
}

}  // namespace

extern "C" int qp3d_adjoint(qp3d_ctx *ctx, const qp3d_geom *g, const qp3d_model *m,
                            const float *d_obs, double *grad_vp, double *grad_eps,
                            double *grad_del, double *misfit)
{
    if (!ctx) return QP3D_ERR_ARG;
    if (!g || !m || !d_obs) return ctx_fail(ctx, QP3D_ERR_ARG, "missing input");
    if (ctx->param_fp16) return ctx_fail(ctx, QP3D_ERR_ARG, "qp3d_adjoint needs FP32 parameters");
    int rc = qp3d_shot_load(ctx, g, m);
    if (rc) return rc;
    if (!ctx->fuse_sources || ctx->n_band > 0 || !ctx->rec_fused)
        return ctx_fail(ctx, QP3D_ERR_ARG,
                        "qp3d_adjoint: sources and receivers must lie inside the updated box");
    const int nt = g->nt;
    if (nt == 0) {   // no record: zero misfit, nothing added to the gradient
        if (misfit) *misfit = 0.0;
        return QP3D_OK;
    }
    const long long vol = ctx->vol;
    const size_t rec = (size_t)nt * ctx->hx * ctx->hy;
    const size_t vb = (size_t)vol * sizeof(float);
    // state buffers, reused when the geometry and the schedule repeat
    AdjState *&S = ctx->adj;
    if (S && (S->vol != vol || S->nt != nt || S->bf16 != ctx->adj_bf16 ||
              (ctx->adj_keep >= 0 && S->keep != ctx->adj_keep))) {
        adjoint_free(S);
        S = nullptr;
    }
    int keep = S ? S->keep : ctx->adj_keep;
    if (keep < 0) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        const size_t need = (size_t)nt * vb + 32 * vb + rec * sizeof(float);
        keep = fr > need + (8ull << 30) ? 1 : 0;
    }
    const int C = keep ? std::max(nt, 1)
                       : std::max(1, (int)std::ceil(std::sqrt((double)std::max(nt, 1))));
    const int nck = keep ? 0 : (nt + C - 1) / C;
    if (!S) {
        S = new (std::nothrow) AdjState();
        if (!S) return ctx_fail(ctx, QP3D_ERR_NOMEM, "out of host memory");
        S->vol = vol;
        S->nt = nt;
        if ((rc = alloc_state(ctx, S, C, nck, ctx->adj_bf16, keep, rec))) {
            adjoint_free(S);
            S = nullptr;
            return rc;
        }
    }
    // checkpoint c: volumes 0, 1 (u, u_prev) FP32, 2..8 FP32 or BF16
    const size_t hb = S->bf16 ? (size_t)vol * sizeof(__nv_bfloat16) : vb;
    auto ck_slot = [&](int c, int j) {
        return static_cast<char *>(S->ck) + (size_t)c * (2 * vb + 7 * hb) +
               (j < 2 ? (size_t)j * vb : 2 * vb + (size_t)(j - 2) * hb);
    };

    // The checkpoint schedule records every step's threshold decisions in the
    // forward pass and replays them in the recomputation and the adjoint
    // steps, so that a recomputation from rounded (BF16) checkpoints keeps
    // the forward's S = 1 / anisotropic split; the decision is a
    // discontinuity of S, and a flipped cell changes the delta gradient far
    // more than the rounding itself.
    struct DecGuard {
        qp3d_ctx *c;
        ~DecGuard() { c->dec_mode = 0; c->dec_base = nullptr; }
    } dec_guard{ctx};
    if (!keep) {
        ctx->dec_base = S->dec;
        ctx->dec_words = vol / 32;
        ctx->dec_mode = 1;
    }
    // ---- forward, keeping u^k or checkpoints.  Keeping every u^k, the steps
    // write u(k+1) straight into its slot of the kept array (no copy per
    // step); the shot's own buffers serve as u(-1) (zero after the reset) and
    // receive u(nt), and are put back afterwards, also on an error.
    float *const own[3] = {ctx->U[0], ctx->U[1], ctx->U[2]};
    struct OwnGuard {
        qp3d_ctx *c;
        float *const *u;
        bool on;
        ~OwnGuard() { if (on) (void)qp3d_internal_restore_wavefields(c, u); }
    } own_guard{ctx, own, keep != 0};
    if (keep) CK(cudaMemsetAsync(S->seg, 0, vb, ctx->stream));   // u^0
    for (int k = 0; k < nt; ++k) {
        if (keep) {
            float *u_prev = k ? S->seg + (size_t)(k - 1) * vol : ctx->U[ctx->prev];
            float *u_next = k + 1 < nt ? S->seg + (size_t)(k + 1) * vol : own[3 - ctx->cur - ctx->prev];
            if (k == 0) u_prev = own[ctx->prev];
            if ((rc = qp3d_internal_bind_wavefields(ctx, u_prev, S->seg + (size_t)k * vol, u_next)))
                return rc;
        } else if (k % C == 0) {
            float *v[9];
            live_state(ctx, k, v);
            for (int j = 0; j < 9; ++j) {
                if (S->bf16 && j >= 2)
                    CKL(launch_to_bf16(v[j], reinterpret_cast<__nv_bfloat16 *>(ck_slot(k / C, j)),
                                       vol, ctx->stream));
                else
                    CK(cudaMemcpyAsync(ck_slot(k / C, j), v[j], vb, cudaMemcpyDeviceToDevice,
                                       ctx->stream));
            }
        }
        if ((rc = qp3d_internal_enqueue_step(ctx))) return rc;
    }
    // ---- residual and misfit, on the device
    CK(cudaMemcpyAsync(S->resid, d_obs, rec * sizeof(float), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemsetAsync(S->misfit, 0, sizeof(double), ctx->stream));
    CKL(launch_residual(ctx->record, S->resid, S->resid, (long long)rec, S->misfit, ctx->stream));
    double J = 0.0;
    CK(cudaMemcpyAsync(&J, S->misfit, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    // every entry the adjoint kernels never write must be zero in both
    // buffers of each pair (see qp3d_adj_a_kernel)
    for (auto *p : S->L) CK(cudaMemsetAsync(p, 0, vb, ctx->stream));
    for (auto *p : S->N) CK(cudaMemsetAsync(p, 0, vb, ctx->stream));
    for (auto *p : S->Cf) CK(cudaMemsetAsync(p, 0, vb, ctx->stream));
    for (auto *p : S->g) CK(cudaMemsetAsync(p, 0, vb, ctx->stream));

    // ---- backward, one checkpoint segment at a time
    AdjParams a;
    memset(&a, 0, sizeof(a));
    a.nx = g->nx; a.ny = g->ny; a.nz = g->nz; a.ldy = ctx->ldy; a.pml = g->pml; a.sz = g->sz;
    a.hx = ctx->hx; a.hy = ctx->hy; a.plane = ctx->plane; a.k = ctx->coefs; a.dt = g->dt;
    a.VP = ctx->VP; a.E2 = ctx->E2; a.R8 = ctx->R8; a.layers = ctx->layers;
    a.live = ctx->adj_live;
    for (int c = (keep ? 1 : nck) - 1; c >= 0; --c) {
        const int k0 = c * C, k1 = std::min(nt, k0 + C);
        if (!keep) {   // restore the checkpoint, recompute keeping u^k
            ctx->dec_mode = 2;
            if ((rc = qp3d_internal_restore_step(ctx, k0))) return rc;
            float *v[9];
            live_state(ctx, k0, v);
            for (int j = 0; j < 9; ++j) {
                if (S->bf16 && j >= 2)
                    CKL(launch_from_bf16(
                        reinterpret_cast<const __nv_bfloat16 *>(ck_slot(c, j)), v[j], vol,
                        ctx->stream));
                else
                    CK(cudaMemcpyAsync(v[j], ck_slot(c, j), vb, cudaMemcpyDeviceToDevice,
                                       ctx->stream));
            }
            for (int k = k0; k < k1; ++k) {
                CK(cudaMemcpyAsync(S->seg + (size_t)(k - k0) * vol, ctx->U[ctx->cur], vb,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
                if ((rc = qp3d_internal_enqueue_step(ctx))) return rc;
            }
        }
        CKL(launch_threshold(ctx->gmax + k0, S->T2, k1 - k0, ctx->stream));
        for (int k = k1 - 1; k >= k0; --k) {
            a.T2 = S->T2 + (k - k0);
            a.dec = keep ? nullptr : S->dec + (size_t)k * (size_t)(vol / 32);
            a.u = S->seg + (size_t)(k - k0) * vol;
            a.resid = S->resid + (size_t)k * ctx->hx * ctx->hy;
            const float **Lc[9] = {&a.Lu, &a.Lup, &a.Lw1, &a.Lw1o, &a.Lp, &a.Lpo, &a.Lw21,
                                   &a.Lw3, &a.Lw3o};
            float **Nc[9] = {&a.Nu, &a.Nup, &a.Nw1, &a.Nw1o, &a.Np, &a.Npo, &a.Nw21, &a.Nw3,
                             &a.Nw3o};
            for (int j = 0; j < 9; ++j) {
                *Lc[j] = S->L[j];
                *Nc[j] = S->N[j];
            }
            for (int j = 0; j < 6; ++j) a.C[j] = S->Cf[j];
            a.gK = S->g[0]; a.gE = S->g[1]; a.gD = S->g[2];
            CKL(launch_adjoint_step(a, ctx->stream));
            ++ctx->launches;   // two passes
            for (int j = 0; j < 9; ++j) std::swap(S->L[j], S->N[j]);
        }
    }
    // ---- gradient: interior cells, added to the caller's FP64 arrays
    const int nx = g->nx, ny = g->ny, nz = g->nz, pml = g->pml;
    std::vector<float> hg((size_t)nx * ny * nz);
    double *outs[3] = {grad_vp, grad_eps, grad_del};
    for (int q = 0; q < 3; ++q) {
        if (!outs[q]) continue;
        CK(cudaMemcpy2DAsync(hg.data(), (size_t)ny * 4, S->g[q], (size_t)ctx->ldy * 4,
                             (size_t)ny * 4, (size_t)nx * nz, cudaMemcpyDeviceToHost,
                             ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        // every cell on its own, so host threads take z slabs
        double *out = outs[q];
        auto add = [&](int za, int zb) {
            for (int z = za; z < zb; ++z)
                for (int x = pml; x < nx - pml; ++x)
                    for (int y = pml; y < ny - pml; ++y) {
                        const size_t i = ((size_t)z * nx + x) * ny + y;
                        double gi = hg[i];
                        if (q == 0) gi *= 2.0 * (double)m->vp[i] * (double)g->dt * (double)g->dt;
                        out[i] += gi;
                    }
        };
        const unsigned hw = std::thread::hardware_concurrency();
        const int nth = (int)std::max(1u, std::min(16u, hw ? hw : 1u));
        const int hz = nz - 2 * pml;
        std::vector<std::thread> th;
        int started = 1;
        try {
            for (int t = 1; t < nth; ++t, ++started)
                th.emplace_back(add, pml + (int)((long long)hz * t / nth),
                                pml + (int)((long long)hz * (t + 1) / nth));
        } catch (...) {   // no more threads: this one adds the rest
        }
        add(pml, pml + (int)((long long)hz / nth));
        for (auto &t : th) t.join();
        for (int t = started; t < nth; ++t)
            add(pml + (int)((long long)hz * t / nth), pml + (int)((long long)hz * (t + 1) / nth));
    }
    rc = qp3d_shot_sync(ctx);
    if (!rc && misfit) *misfit = J;
    return rc;
}
