// qp3d_batch.cu -- many shots in one time loop (qp3d_batch of include/qp3d.h).
//
// The reference runs its shots one after another, one modeling3d call each
// (3dPureqPModeling1.0.c:225-277): every call allocates, steps and frees on
// its own, so a shot of ~10 M cells leaves most of the GPU idle between the
// short launches of each step.  Here all shots that fit in device memory are
// resident at once.  Per time step there is one launch of each plane kernel
// for all of them; its persistent CTAs take work items (one tile column of one
// shot) from a device queue, so shots of uneven size share the SMs.  The
// per-step parameters of every shot are written on the device
// (qp3d_batch_prepare_kernel), so one step is the same sequence of launches
// for every k and the speculative steps are replayed from a captured graph.
//
// Shape tuning: the tile height and the number of z blocks of a column change
// only the schedule, never a result.  The first steps after the three
// gradmax steps time each candidate shape (forward, then backward order, to
// cancel the slow drift of the step cost) and the rest of the run uses the
// fastest; the choice is cached per set of shot sizes.
#include "qp3d_ctx.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

using namespace qp3d;

namespace qp3d {

namespace {

struct Cand {
    int tile_rows;   // largest tile height (x rows)
    int zblocks;     // z blocks per tile column
};
constexpr Cand kCands[] = {{32, 1}, {32, 2}, {32, 4}, {16, 1}, {16, 2}};
constexpr int kNumCands = (int)(sizeof(kCands) / sizeof(kCands[0]));
constexpr int kDefaultCand = 4;   // 16 rows: three CTAs per SM
constexpr int kTuneSteps = 2;       // steps per candidate and pass (two passes)
constexpr int kGraphSteps = 8;      // steps per captured graph
constexpr int kSpecFirst = 3;       // as the single-shot path

// Host view of one batched shot.
struct Plan {
    int idx = 0;                    // index in the caller's array
    qp3d_geom g{};
    int ldy = 0, hx = 0, hy = 0;
    long long plane = 0, vol = 0;
    std::vector<SrcEntry> src;
    size_t bytes = 0;               // device bytes of this shot
    BatchShot d{};                  // device pointers, filled per group
};

}  // namespace

struct BatchState {
    void *arena = nullptr;
    size_t arena_bytes = 0;
    BatchShot *d_shots = nullptr;
    PlaneParams *d_pp = nullptr;
    int shots_cap = 0;
    int *d_ctr = nullptr;           // [0] step counter, [4..8) work queues
    WorkItem *d_work[kNumCands] = {};
    size_t work_cap[kNumCands] = {};
    CUtensorMap *d_tm[kNumCands] = {};
    size_t tm_cap[kNumCands] = {};
    std::map<std::string, int> tuned;
    qp3d_batch_stats stats{};
};

void batch_free(BatchState *b)
{
    if (!b) return;
    if (b->arena) cudaFree(b->arena);
    if (b->d_shots) cudaFree(b->d_shots);
    if (b->d_pp) cudaFree(b->d_pp);
    if (b->d_ctr) cudaFree(b->d_ctr);
    for (int c = 0; c < kNumCands; ++c) {
        if (b->d_work[c]) cudaFree(b->d_work[c]);
        if (b->d_tm[c]) cudaFree(b->d_tm[c]);
    }
    delete b;
}

}  // namespace qp3d

namespace {

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// Device bytes of one shot; the same walk lays the buffers out (carve).
struct Carver {
    char *base;
    size_t off = 0;
    template <class T> T *take(size_t count)
    {
        T *p = reinterpret_cast<T *>(base ? base + off : nullptr);
        off += align256(count * sizeof(T));
        return p;
    }
};

// Lays out one shot at c (base null: only counts).  The state that starts at
// zero comes first, in one span of zero_bytes.
void carve(Plan &s, Carver &c, size_t *zero_bytes)
{
    const size_t vol = (size_t)s.vol, nt = (size_t)std::max(s.g.nt, 1);
    const size_t start = c.off;
    BatchShot &d = s.d;
    for (int i = 0; i < 3; ++i) d.U[i] = c.take<float>(vol);
    for (int i = 0; i < 3; ++i) d.W1[i] = c.take<float>(vol);
    for (int i = 0; i < 3; ++i) d.W3[i] = c.take<float>(vol);
    for (int i = 0; i < 3; ++i) d.P[i] = c.take<float>(vol);
    for (int i = 0; i < 2; ++i) d.W21[i] = c.take<float>(vol);
    d.record = c.take<float>(nt * s.hx * s.hy);
    d.gmax = c.take<float>(nt);
    d.win = c.take<float>(3 * nt);
    d.redo = c.take<int>(nt);
    d.alt_count = c.take<unsigned>(nt);
    d.fix_count = c.take<unsigned>(nt);
    d.amask = c.take<unsigned>((size_t)defer_mask_words((long long)vol));
    if (zero_bytes) *zero_bytes = c.off - start;
    d.VP = c.take<float>(vol);
    d.E2 = c.take<float>(vol);
    d.R8 = c.take<float>(vol);
    d.spec_err = c.take<float>(kSpecHist);
    d.am2 = c.take<float>(vol);
    d.av = c.take<float>(vol);
    d.apml = c.take<float4>(vol);
    d.alist_cap = (unsigned)std::min<size_t>(std::max<size_t>(1u << 16, vol / 4), 0x7fffffff);
    d.alist = c.take<unsigned>(d.alist_cap);
    d.layers = c.take<float4>(3 * (size_t)std::max(s.g.pml, 1));
    d.wavelet = c.take<float>(nt);
    d.src = c.take<SrcEntry>(std::max<size_t>(s.src.size(), 1));
}

int tile_height(int nx, int rows)
{
    const int ncx = nx - 2 * kRadius;
    const int ntx = (ncx + rows - 1) / rows;
    return (ncx + ntx - 1) / ntx;
}

int make_tmap(qp3d_ctx *ctx, const Plan &s, float *base, int tile_x, CUtensorMap *tm)
{
    cuuint64_t dims[3] = {(cuuint64_t)s.g.ny, (cuuint64_t)s.g.nx, (cuuint64_t)s.g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)s.ldy * 4, (cuuint64_t)s.plane * 4};
    cuuint32_t box[3] = {(cuuint32_t)kBoxY, (cuuint32_t)(tile_x + 2 * kRadius), 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = ctx->encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return ctx_fail(ctx, QP3D_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return QP3D_OK;
}

template <class T> int ensure(qp3d_ctx *ctx, T **p, size_t *cap, size_t n)
{
    if (*cap >= n && *p) return QP3D_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    CK(cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T)));
    *cap = n;
    return QP3D_OK;
}

// One candidate's launch configuration for a group.
struct Launch {
    int nwork = 0, threads = 0, grid = 0;
    size_t smem = 0;
};

bool same_coefs(const Coefs &a, const Coefs &b) { return !memcmp(&a, &b, sizeof(Coefs)); }

class Runner {
  public:
    Runner(qp3d_ctx *ctx, BatchState *B) : ctx(ctx), B(B) {}
    int run_group(std::vector<Plan *> &G, const Coefs &kc, const qp3d_shot *shots);

  private:
    qp3d_ctx *ctx;
    BatchState *B;
    Launch L[kNumCands];
    int nshots = 0;
    long long max_words = 0;   // largest deferred-cell bitmask of the group
    Coefs coefs{};

    int build_candidate(int c, std::vector<Plan *> &G);
    BatchArgs args(int c, int queue) const
    {
        BatchArgs a;
        a.k = coefs;
        a.pp = B->d_pp;
        a.tm = B->d_tm[c];
        a.work = B->d_work[c];
        a.nwork = L[c].nwork;
        a.queue = B->d_ctr + 4 + queue;
        a.arith = ctx->arith;
        return a;
    }
    int enqueue_step(int c, bool spec);
};

int Runner::build_candidate(int c, std::vector<Plan *> &G)
{
    std::vector<WorkItem> items;
    std::vector<CUtensorMap> tms(3 * G.size());
    int max_tile = 1;
    size_t smem = 0;
    for (size_t s = 0; s < G.size(); ++s) {
        const Plan &P = *G[s];
        const int tx = tile_height(P.g.nx, kCands[c].tile_rows);
        max_tile = std::max(max_tile, tx);
        smem = std::max(smem, batch_smem_bytes(tx, P.g.pml, (int)P.src.size()));
        const int nxt = (P.g.nx - 2 * kRadius + tx - 1) / tx;
        const int nyt = (P.g.ny - kRadius - 1) / kTileY + 1;
        const int ncz = P.g.nz - 2 * kRadius;
        const int zb = std::min(kCands[c].zblocks, ncz);
        const int cz = (ncz + zb - 1) / zb;
        for (int z0 = kRadius; z0 < P.g.nz - kRadius; z0 += cz)
            for (int xt = 0; xt < nxt; ++xt)
                for (int yt = 0; yt < nyt; ++yt) {
                    WorkItem w;
                    w.shot = (int)s;
                    w.tile_x = tx;
                    w.y0 = yt * kTileY;
                    w.x0 = kRadius + xt * tx;
                    w.z0 = z0;
                    w.z1 = std::min(z0 + cz, P.g.nz - kRadius);
                    items.push_back(w);
                }
        for (int i = 0; i < 3; ++i) {
            int rc = make_tmap(ctx, P, P.d.U[i], tx, &tms[3 * s + i]);
            if (rc) return rc;
        }
    }
    // longest columns first: the queue hands them out before the short ones
    std::stable_sort(items.begin(), items.end(), [](const WorkItem &a, const WorkItem &b) {
        return (a.z1 - a.z0) > (b.z1 - b.z0);
    });
    int rc;
    if ((rc = ensure(ctx, &B->d_work[c], &B->work_cap[c], items.size())) ||
        (rc = ensure(ctx, &B->d_tm[c], &B->tm_cap[c], tms.size())))
        return rc;
    CK(cudaMemcpyAsync(B->d_work[c], items.data(), items.size() * sizeof(WorkItem),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(B->d_tm[c], tms.data(), tms.size() * sizeof(CUtensorMap),
                       cudaMemcpyHostToDevice, ctx->stream));
    Launch &l = L[c];
    l.nwork = (int)items.size();
    l.threads = batch_plane_threads(max_tile);
    l.smem = smem;
    int per_sm = 0;
    CK(batch_ctas_per_sm(2, ctx->arith, l.threads, l.smem, &per_sm));
    if (per_sm < 1) return ctx_fail(ctx, QP3D_ERR_CUDA, "batched step kernel does not fit an SM");
    l.grid = std::max(1, std::min(l.nwork, per_sm * ctx->nsm));
    return QP3D_OK;
}

int Runner::enqueue_step(int c, bool spec)
{
    const Launch &l = L[c];
    CKL(launch_batch_prepare(B->d_shots, nshots, B->d_pp, B->d_ctr, B->d_ctr + 4, spec ? 1 : 0,
                             ctx->stream));
    if (spec) {
        CKL(launch_batch_plane(2, args(c, 1), l.grid, l.threads, l.smem, ctx->stream));
        const int per_shot = std::max(2, 8 * ctx->nsm / std::max(nshots, 1));
        CKL(launch_batch_fixup(args(c, 1), nshots, per_shot, max_words, ctx->stream));
        ctx->launches += 1;   // compaction and fix-up
        CKL(launch_batch_plane(1, args(c, 2), l.grid, l.threads, l.smem, ctx->stream));
    } else {
        CKL(launch_batch_plane(0, args(c, 0), l.grid, l.threads, l.smem, ctx->stream));
        CKL(launch_batch_plane(1, args(c, 1), l.grid, l.threads, l.smem, ctx->stream));
    }
    return QP3D_OK;
}

int Runner::run_group(std::vector<Plan *> &G, const Coefs &kc, const qp3d_shot *shots)
{
    int rc;
    nshots = (int)G.size();
    coefs = kc;
    max_words = 0;
    for (Plan *p : G) max_words = std::max(max_words, defer_mask_words(p->vol));
    // ---- device memory: one arena for the group
    size_t total = 0;
    for (Plan *p : G) total += p->bytes;
    if (B->arena_bytes < total) {
        if (B->arena) cudaFree(B->arena);
        B->arena = nullptr;
        B->arena_bytes = 0;
        CK(cudaMalloc(&B->arena, total));
        B->arena_bytes = total;
    }
    if (B->shots_cap < nshots) {
        if (B->d_shots) cudaFree(B->d_shots);
        if (B->d_pp) cudaFree(B->d_pp);
        B->d_shots = nullptr;
        B->d_pp = nullptr;
        B->shots_cap = 0;
        CK(cudaMalloc(&B->d_shots, sizeof(BatchShot) * nshots));
        CK(cudaMalloc(&B->d_pp, sizeof(PlaneParams) * nshots));
        B->shots_cap = nshots;
    }
    if (!B->d_ctr) CK(cudaMalloc(&B->d_ctr, 8 * sizeof(int)));
    if (!ctx->errword) CK(cudaMalloc(&ctx->errword, sizeof(unsigned)));
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(unsigned), ctx->stream));

    // ---- per shot: layout, model upload, derived inputs, zero state
    Carver cv{static_cast<char *>(B->arena)};
    std::vector<BatchShot> hshots(nshots);
    int nt_max = 0;
    for (int s = 0; s < nshots; ++s) {
        Plan &P = *G[s];
        const qp3d_model &m = shots[P.idx].model;
        size_t zero_bytes = 0;
        const size_t start = cv.off;
        carve(P, cv, &zero_bytes);
        BatchShot &d = P.d;
        d.nx = P.g.nx; d.ny = P.g.ny; d.nz = P.g.nz; d.ldy = P.ldy; d.pml = P.g.pml;
        d.sz = P.g.sz; d.nt = P.g.nt; d.hx = P.hx; d.hy = P.hy; d.plane = P.plane;
        d.dt = P.g.dt;
        d.delta_min = ctx->delta_min_set ? ctx->delta_min : 0.02f;
        d.nsrc = (int)P.src.size();
        d.spec_bias = ctx->spec_bias;
        d.err = ctx->errword;
        nt_max = std::max(nt_max, P.g.nt);
        CK(cudaMemsetAsync(static_cast<char *>(B->arena) + start, 0, zero_bytes, ctx->stream));
        // vp, eps, delta in one piece each to the wavefield buffers (staging,
        // zeroed again after), then the per-cell parameters, pitched
        {
            const float *src[3] = {m.vp, m.epsilon, m.delta};
            const size_t dense = (size_t)P.g.nx * P.g.ny * P.g.nz * sizeof(float);
            for (int i = 0; i < 3; ++i)
                CK(cudaMemcpyAsync(d.U[i], src[i], dense, cudaMemcpyHostToDevice, ctx->stream));
            CKL(launch_params_dense(d.U[0], d.U[1], d.U[2], const_cast<float *>(d.VP),
                                    const_cast<float *>(d.E2), const_cast<float *>(d.R8),
                                    P.g.nx, P.g.ny, P.g.nz, P.ldy, ctx->stream));
            for (int i = 0; i < 3; ++i)
                CK(cudaMemsetAsync(d.U[i], 0, (size_t)P.vol * sizeof(float), ctx->stream));
        }
        static const float first[kSpecHist] = {1.0f};   // no prediction yet
        CK(cudaMemcpyAsync(d.spec_err, first, sizeof(first), cudaMemcpyHostToDevice,
                           ctx->stream));
        if (P.g.pml > 0) {
            std::vector<float4> tab(3 * P.g.pml);
            derive_layers(m.dlr, m.ddlr, P.g.pml, P.g.dt, tab.data());
            derive_layers(m.dfb, m.ddfb, P.g.pml, P.g.dt, tab.data() + P.g.pml);
            derive_layers(m.dtb, m.ddtb, P.g.pml, P.g.dt, tab.data() + 2 * P.g.pml);
            // pageable source: staged before the call returns, ordered on the stream
            CK(cudaMemcpyAsync(const_cast<float4 *>(d.layers), tab.data(),
                               sizeof(float4) * tab.size(), cudaMemcpyHostToDevice, ctx->stream));
        }
        if (P.g.nt > 0)
            CK(cudaMemcpyAsync(const_cast<float *>(d.wavelet), m.wavelet, sizeof(float) * P.g.nt,
                               cudaMemcpyHostToDevice, ctx->stream));
        if (!P.src.empty())
            CK(cudaMemcpyAsync(const_cast<SrcEntry *>(d.src), P.src.data(),
                               sizeof(SrcEntry) * P.src.size(), cudaMemcpyHostToDevice,
                               ctx->stream));
        hshots[s] = d;
    }
    CK(cudaMemcpyAsync(B->d_shots, hshots.data(), sizeof(BatchShot) * nshots,
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(B->d_ctr, 0, 8 * sizeof(int), ctx->stream));
    for (int c = 0; c < kNumCands; ++c)
        if ((rc = build_candidate(c, G))) return rc;

    // ---- choose the shape: cache, fixed, or timed on the run's own steps
    std::string key = ctx->threshold_mode ? "s" : "g";
    for (Plan *p : G) {
        char buf[64];
        snprintf(buf, sizeof(buf), "|%d,%d,%d,%d", p->g.nx, p->g.ny, p->g.nz, p->g.pml);
        key += buf;
    }
    qp3d_batch_stats &st = B->stats;
    const bool spec_mode = ctx->threshold_mode == 1;
    const int spec_from = spec_mode ? kSpecFirst : nt_max;
    int cand = ctx->batch_candidate >= 0 ? std::min(ctx->batch_candidate, kNumCands - 1)
                                          : kDefaultCand;
    bool tune = false;
    if (ctx->batch_candidate < 0) {
        auto it = B->tuned.find(key);
        if (it != B->tuned.end()) cand = it->second;
        else tune = ctx->batch_tune && spec_mode &&
                    nt_max >= spec_from + 4 * kTuneSteps * kNumCands;
    }

    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } evg{e0, e1};
    CK(cudaEventRecord(e0, ctx->stream));

    int k = 0;
    for (; k < std::min(spec_from, nt_max); ++k)
        if ((rc = enqueue_step(cand, false))) return rc;
    if (tune) {
        const int nsteps = 2 * kTuneSteps * kNumCands;
        std::vector<cudaEvent_t> ev(nsteps + 1);
        for (auto &e : ev) CK(cudaEventCreate(&e));
        struct Guard {
            std::vector<cudaEvent_t> &v;
            ~Guard() { for (auto e : v) cudaEventDestroy(e); }
        } g{ev};
        std::vector<int> order;
        for (int c = 0; c < kNumCands; ++c) order.push_back(c);
        for (int c = kNumCands - 1; c >= 0; --c) order.push_back(c);
        int i = 0;
        CK(cudaEventRecord(ev[0], ctx->stream));
        for (int c : order)
            for (int r = 0; r < kTuneSteps; ++r, ++i, ++k) {
                if ((rc = enqueue_step(c, true))) return rc;
                CK(cudaEventRecord(ev[i + 1], ctx->stream));
            }
        CK(cudaEventSynchronize(ev[nsteps]));
        float sum[kNumCands] = {};
        i = 0;
        for (int c : order)
            for (int r = 0; r < kTuneSteps; ++r, ++i) {
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
                sum[c] += ms;
            }
        cand = 0;
        for (int c = 0; c < kNumCands; ++c) {
            st.cand_ms[c] = sum[c] / (2 * kTuneSteps);
            if (sum[c] < sum[cand]) cand = c;
        }
        st.ncand = kNumCands;
        st.tuned = 1;
        B->tuned[key] = cand;
    }
    // speculative steps: from a captured graph of kGraphSteps steps
    if (spec_mode && ctx->batch_graph && nt_max - k >= kGraphSteps) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const long long launches0 = ctx->launches;
        int crc = QP3D_OK;
        for (int i = 0; i < kGraphSteps && !crc; ++i) crc = enqueue_step(cand, true);
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        const long long per_graph = ctx->launches - launches0;
        ctx->launches = launches0;
        if (crc) {
            if (graph) cudaGraphDestroy(graph);
            return crc;
        }
        CK(ce);
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CK(ie);
        struct ExecGuard {
            cudaGraphExec_t e;
            ~ExecGuard() { cudaGraphExecDestroy(e); }
        } xg{exec};
        for (; k + kGraphSteps <= nt_max; k += kGraphSteps) {
            CK(cudaGraphLaunch(exec, ctx->stream));
            ctx->launches += per_graph;
            st.graph_steps += kGraphSteps;
        }
        for (; k < nt_max; ++k)
            if ((rc = enqueue_step(cand, true))) return rc;
        CK(cudaEventRecord(e1, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    } else {
        for (; k < nt_max; ++k)
            if ((rc = enqueue_step(cand, spec_mode && k >= spec_from))) return rc;
        CK(cudaEventRecord(e1, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    st.run_ms += ms;
    unsigned e = 0;
    CK(cudaMemcpy(&e, ctx->errword, sizeof(e), cudaMemcpyDeviceToHost));
    if (e) return ctx_fail(ctx, QP3D_ERR_TIMEOUT, "device wait timed out (flags 0x%x)", e);

    // ---- results
    for (int s = 0; s < nshots; ++s) {
        Plan &P = *G[s];
        float *out = shots[P.idx].record;
        if (P.g.nt > 0 && out)
            CK(cudaMemcpy(out, P.d.record, sizeof(float) * (size_t)P.g.nt * P.hx * P.hy,
                          cudaMemcpyDeviceToHost));
        if (P.g.nt > 0) {
            std::vector<int> redo(P.g.nt);
            CK(cudaMemcpy(redo.data(), P.d.redo, sizeof(int) * P.g.nt, cudaMemcpyDeviceToHost));
            for (int v : redo) st.redo_steps += v != 0;
        }
    }
    st.candidate = cand;
    st.tile_rows = kCands[cand].tile_rows;
    st.zblocks = kCands[cand].zblocks;
    st.work_items = L[cand].nwork;
    st.ctas = L[cand].grid;
    st.groups += 1;
    st.batched_shots += nshots;
    return QP3D_OK;
}

// Whether a shot can run in the batched launches: fused sources and receiver
// plane (as the single-shot path decides), 32-bit cell indices.
bool batchable(const qp3d_geom &g, const std::vector<SrcEntry> &src, bool band)
{
    if (band || src.size() > (size_t)kMaxFusedSources) return false;
    if (g.pml < kRadius || g.sz < kRadius || g.sz >= g.nz - kRadius) return false;
    const long long ldy = (g.ny + 31) & ~31;
    return (long long)g.nx * ldy * g.nz < (1ll << 32);
}

}  // namespace

extern "C" int qp3d_batch(qp3d_ctx *ctx, int nshots, const qp3d_shot *shots)
{
    if (!ctx) return QP3D_ERR_ARG;
    if (nshots < 0 || (nshots > 0 && !shots)) return ctx_fail(ctx, QP3D_ERR_ARG, "bad shot list");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!ctx->batch) ctx->batch = new (std::nothrow) BatchState();
    if (!ctx->batch) return ctx_fail(ctx, QP3D_ERR_NOMEM, "out of host memory");
    BatchState *B = ctx->batch;
    B->stats = qp3d_batch_stats{};
    B->stats.candidate = -1;

    // ---- validate, classify
    std::vector<Plan> plans(nshots);
    std::vector<Coefs> coefs(nshots);
    std::vector<int> single;
    for (int i = 0; i < nshots; ++i) {
        const qp3d_geom &g = shots[i].geom;
        const qp3d_model &m = shots[i].model;
        if (g.nx < 11 || g.ny < 11 || g.nz < 11 || g.pml < 0 || g.pml > kMaxPml ||
            2 * g.pml >= g.nx || 2 * g.pml >= g.ny || 2 * g.pml >= g.nz || g.nt < 0 ||
            g.sz < 0 || g.sz >= g.nz || !(g.dx > 0) || !(g.dy > 0) || !(g.dz > 0) || !(g.dt > 0))
            return ctx_fail(ctx, QP3D_ERR_ARG, "shot %d: invalid geometry", i);
        if (!m.vp || !m.epsilon || !m.delta || !m.wavelet || !m.c || !m.c2 || !shots[i].record)
            return ctx_fail(ctx, QP3D_ERR_ARG, "shot %d: missing model input or record", i);
        if (g.pml > 0 && (!m.dlr || !m.ddlr || !m.dtb || !m.ddtb || !m.dfb || !m.ddfb))
            return ctx_fail(ctx, QP3D_ERR_ARG, "shot %d: missing PML profiles", i);
        Plan &P = plans[i];
        P.idx = i;
        P.g = g;
        P.ldy = (g.ny + 31) & ~31;
        P.plane = (long long)g.nx * P.ldy;
        P.vol = P.plane * g.nz;
        P.hx = g.nx - 2 * g.pml;
        P.hy = g.ny - 2 * g.pml;
        bool band = false;
        if (m.source) {
            std::vector<SrcEntry> all;
            scan_source_volume(m.source, g.nx, g.ny, g.nz, all);
            for (const SrcEntry &e : all) {
                const bool inside = e.x >= kRadius && e.x < g.nx - kRadius && e.y >= kRadius &&
                                    e.y < g.ny - kRadius && e.z >= kRadius && e.z < g.nz - kRadius;
                if (!inside) band = true;
                else if (P.src.size() <= (size_t)kMaxFusedSources) P.src.push_back(e);
            }
        }
        derive_coefs(m.c, m.c2, g.dx, g.dy, g.dz, &coefs[i]);
        Carver cv{nullptr};
        carve(P, cv, nullptr);
        P.bytes = cv.off;
        if (!batchable(g, P.src, band)) single.push_back(i);
    }

    // ---- batched classes (same coefficient tables), groups that fit memory
    std::vector<bool> done(nshots, false);
    for (int i : single) done[i] = true;
    Runner R(ctx, B);
    for (int lead = 0; lead < nshots; ++lead) {
        if (done[lead]) continue;
        std::vector<Plan *> cls;
        for (int i = lead; i < nshots; ++i)
            if (!done[i] && same_coefs(coefs[i], coefs[lead])) {
                cls.push_back(&plans[i]);
                done[i] = true;
            }
        size_t pos = 0;
        while (pos < cls.size()) {
            size_t fr = 0, tot = 0;
            CK(cudaMemGetInfo(&fr, &tot));
            size_t budget = fr + B->arena_bytes;
            budget = budget > (2ull << 30) ? budget - (2ull << 30) : 0;
            budget = budget / 20 * 19;
            if (ctx->batch_mem_mb > 0) budget = (size_t)ctx->batch_mem_mb << 20;
            std::vector<Plan *> G;
            size_t used = 0;
            while (pos < cls.size() && (G.empty() || used + cls[pos]->bytes <= budget)) {
                used += cls[pos]->bytes;
                G.push_back(cls[pos++]);
            }
            int rc = R.run_group(G, coefs[lead], shots);
            if (rc) return rc;
        }
    }
    // ---- the rest one by one
    for (int i : single) {
        int rc = qp3d_forward(ctx, &shots[i].geom, &shots[i].model, shots[i].record, nullptr);
        if (rc) return rc;
        B->stats.single_shots += 1;
    }
    return QP3D_OK;
}

extern "C" int qp3d_batch_get_stats(const qp3d_ctx *ctx, qp3d_batch_stats *out)
{
    if (!ctx || !out) return QP3D_ERR_ARG;
    if (!ctx->batch) {
        *out = qp3d_batch_stats{};
        out->candidate = -1;
        return QP3D_OK;
    }
    *out = ctx->batch->stats;
    return QP3D_OK;
}
