// qp3d_ctx.h -- the library context (internal to libqp3d).
#pragma once

#include "qp3d_internal.h"
#include "qp3d.h"

#include <cstdarg>
#include <cstdio>
#include <vector>

namespace qp3d {
// qp3d_host.cpp: host derivations shared with the drop-in driver.
void derive_coefs(const float *c, const float *c2, float dx, float dy, float dz, Coefs *k);
void derive_layers(const float *d, const float *dd, int pml, float dt, float4 *out);
struct BatchState;                 // qp3d_batch.cu
void batch_free(BatchState *b);
struct AdjState;                   // qp3d_adjoint.cu
void adjoint_free(AdjState *s);
}  // namespace qp3d

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

struct qp3d_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // record pieces to page-locked host memory
    cudaEvent_t copy_ev = nullptr;
    EncodeTiledFn encode = nullptr;
    char err[512] = {0};

    // shot
    bool loaded = false;
    qp3d_geom g{};
    int ldy = 0;
    long long plane = 0, vol = 0;
    int hx = 0, hy = 0;
    int tile_x = 0, nxt = 0, nyt = 0, nchunks = 0, chunk_z = 0;
    size_t smem = 0;
    bool rec_fused = true;
    float *U[3] = {nullptr, nullptr, nullptr};
    float *VP = nullptr, *E2 = nullptr, *R8 = nullptr;   // vp, 2 eps, 8 (eps - delta)
    __half *h_vp = nullptr, *h_eps = nullptr, *h_del = nullptr;   // param_fp16 storage
    bool half_loaded = false;        // the loaded shot stores its parameters as half
    float *W1[3] = {}, *W3[3] = {}, *P[3] = {}, *W21[2] = {};
    float *record = nullptr;
    float *gmax = nullptr;
    // speculative threshold: per-step window, re-run flags, deferred-cell counts
    float *win = nullptr;
    int *redo = nullptr;
    unsigned *alt_count = nullptr;
    float *spec_err = nullptr;
    unsigned *amask = nullptr;       // deferred-cell bits, vol / 32 words
    float *am2 = nullptr, *av = nullptr;
    float4 *apml = nullptr;
    unsigned *fix_count = nullptr;   // per step: deferred cells below the threshold
    unsigned *alist = nullptr;       // compacted deferred cells
    unsigned alist_cap = 0;
    float4 *layers = nullptr;
    qp3d::SrcEntry *src_fused = nullptr, *src_band = nullptr, *src_all = nullptr;
    int n_fused = 0, n_band = 0, n_all = 0;
    bool fuse_sources = true;
    unsigned *errword = nullptr;
    CUtensorMap tm[3];
    qp3d::Coefs coefs{};
    std::vector<float> wavelet;
    int step = 0;
    int cur = 0;           // U[cur] holds u(step)
    int prev = 1;          // U[prev] holds u(step-1); the third buffer receives u(step+1)
    // snapshot staging (qp3d_shot_snapshot)
    float *snap_dev = nullptr;
    float *snap_host = nullptr;
    size_t snap_cap = 0;
    // snapshots of qp3d_forward: a ring of slots whose slices are cropped on
    // the step stream and copied to page-locked memory on copy_stream while
    // the time loop goes on; the callbacks run in step order once a slot's
    // copy has landed
    struct SnapSlot {
        float *dev = nullptr, *host = nullptr;
        size_t cap = 0;                       // floats
        cudaEvent_t ready = nullptr, done = nullptr;
        int step = -1;
        unsigned kinds = 0;
    };
    static constexpr int kSnapSlots = 4;
    SnapSlot sring[kSnapSlots];
    int snap_head = 0, snap_count = 0;        // FIFO of slots waiting for delivery
    cudaEvent_t ev[4] = {};
    cudaEvent_t uev[8] = {};
    // tuning
    int gradmax_variant = 0, tune_tile_x = 0, tune_chunks = 0;
    int threshold_mode = 1;          // 0: gradmax pre-pass every step, 1: speculative
    // smallest half-width of the predicted window: 1% for single shots, 2% for
    // batched ones (their small grids make the max jumpier: measured on 64
    // uneven shots of ~11 M cells, 2000 steps: 3417 exact re-runs at 1%, 1013
    // at 2%, 1.7% faster) unless set with "spec_delta_ppm"
    float delta_min = 0.01f;
    bool delta_min_set = false;
    float spec_bias = 0.0f;          // test hook: shifts the predicted window
    int param_fp16 = 0;              // store vp, eps, delta as IEEE half (next load)
    // arithmetic of the step: the fast folded form (default) or the reference
    // CPU operators' roundings, bit for bit ("arith" tuning key)
    int arith = qp3d::kArithFast;
    // bounded device waits: limit (0: 2 s) and the withheld-plane test hook
    // (plane index + 1 in the first CTA of each grid launch; 0: none)
    unsigned long long wait_ns = 0;
    int hold_plane = 0;
    // threshold decisions of each step (qp3d_adjoint): 1 = record them into
    // dec_base + step * dec_words, 2 = replay them; steps then run exactly
    // (gradmax pre-pass), not speculatively
    int dec_mode = 0;
    unsigned *dec_base = nullptr;
    long long dec_words = 0;
    long long launches = 0;          // kernels launched by this context
    // batched shots (qp3d_batch)
    qp3d::BatchState *batch = nullptr;
    int batch_graph = 1;             // replay speculative steps from a captured graph
    int batch_tune = 1;              // choose the tile / z-block shape by timing
    int batch_candidate = -1;        // fixed shape (when not tuning), -1: default
    long long batch_mem_mb = 0;      // device memory for one group of shots, 0: auto
    // adjoint (qp3d_adjoint)
    qp3d::AdjState *adj = nullptr;
    int adj_bf16 = 1;                // 1: PML levels of the checkpoints in BF16
    int adj_keep = -1;               // 1: keep every u^k, 0: checkpoints, -1: by free memory
    int adj_live = 1;                // 1: gradient of the live operator (dS/du included), 0: S frozen
};
inline int ctx_fail(qp3d_ctx *c, int code, const char *fmt, ...)
{
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->err, sizeof(c->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return ctx_fail(ctx, e_ == cudaErrorMemoryAllocation ? QP3D_ERR_NOMEM : QP3D_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// launch a library kernel: check it and count it
#define CKL(call)                                                                          \
    do {                                                                                   \
        CK(call);                                                                          \
        ++ctx->launches;                                                                   \
    } while (0)

