// qp3d_internal.h -- shared definitions between the host API and the kernels.
//
// Device layout of one shot (all float32, row pitch ldy = ny rounded up to 32
// so every row starts on a 128-byte boundary):
//   U[3]            wavefields u(k-1), u(k), u(k+1), rotated by index: a step
//                   never overwrites its inputs
//   VP, E2, R8      per-cell parameters vp, 2*eps, 8*(eps-delta)
//   W1[3],W3[3],P[3] PML split fields, three time levels each, and W21[2],
//                   rotated by index (no copies).  These are full "shadow"
//                   volumes: only PML cells are ever touched, so a cell's
//                   state lives at the cell's own index whatever face owns it.
//   record          nt * hx * hy receiver samples
//   gmax            nt floats: max|grad u| of each step (bits, atomicMax)
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace qp3d {

constexpr int kRadius = 5;        // 10th-order stencil (M/2 with M = 10)
constexpr int kTileY = 32;        // y cells per tile = 8 quads of 4 cells
constexpr int kQuadsY = kTileY / 4;
constexpr int kHaloY = 8;         // y halo rounded up to 16 bytes
constexpr int kBoxY = kTileY + 2 * kHaloY;   // 48 floats per staged row
// Planes loaded ahead of use.  One is enough to cover the TMA latency; every
// further slot costs 8 KB of shared memory per CTA, and the L1 share of the
// SM (where the per-cell global loads wait for DRAM) shrinks with it: two
// CTAs of 32-row tiles with a 12-slot ring fit the 196 KiB shared-memory
// carveout (60 KiB left for L1), a 13-slot ring needs the 228 KiB carveout
// (28 KiB of L1) and runs the step about 17% slower.
constexpr int kPrefetch = 1;
constexpr int kRing = 2 * kRadius + 1 + kPrefetch;   // staged planes
constexpr int kMaxTileX = 32;
constexpr int kThreads = kQuadsY * kMaxTileX;        // 256
constexpr int kMaxFusedSources = 64;
// Relative prediction errors of the step max kept for the speculative window
// (most recent first).
constexpr int kSpecHist = 8;
constexpr int kMaxPml = 256;

// Error bits written to the device error word.
constexpr unsigned kErrWaitTimeout = 1u;

struct Coefs {
    float cx[kRadius], cy[kRadius], cz[kRadius];      // c[31+m]/h
    float c2x[kRadius], c2y[kRadius], c2z[kRadius];   // c2[31+m]/h^2
    float kx, ky, kz;                                  // -2*sum(c2?)
    // the same values duplicated in both lanes, for the paired FP32x2 stencil
    float2 cx2[kRadius], cy2[kRadius], cz2[kRadius];
    float2 c2x2[kRadius], c2y2[kRadius], c2z2[kRadius];
    float2 kx2, ky2, kz2;
    // Reference arithmetic (qp3d_exact.h): the tables as given (both lanes
    // alike) and per axis the divisors of the first and second derivatives,
    // h and h*h rounded.
    float2 rc[kRadius], rc2[kRadius];                  // c[31+m], c2[31+m]
    float rh[3], rh2[3];                               // x, y, z
};

// Arithmetic of the step: the reference CPU operators' roundings
// (qp3d_exact.h, bit-identical to CPU_function.c) or the folded fast form.
enum Arith { kArithRef = 0, kArithFast = 1 };

// One source sample: padded coordinates and the amplitude.
struct SrcEntry {
    int x, y, z;
    float v;
};

// Words of the deferred-cell bitmask of a volume of vol cells (vol is a
// multiple of 32), rounded up to a multiple of 4 for 16-byte loads; the
// padding words stay zero.
__host__ __device__ inline long long defer_mask_words(long long vol) { return ((vol >> 5) + 3) & ~3ll; }

struct PlaneParams {
    // geometry
    int nx, ny, nz, ldy, pml, sz;
    int tile_x;          // rows per tile (<= kMaxTileX)
    int chunk_z;         // planes per z chunk
    long long plane;     // nx * ldy
    Coefs k;
    float dt;
    int step;            // time step index k
    float wavelet;       // wavelet[k]
    // wavefields: u(k) is staged by TMA (and read directly by the fix-up);
    // u(k-1) read, u(k+1) written
    const float *u_cur;
    const float *u_prev;
    float *u_out;
    const float *prm_v, *prm_e, *prm_r;   // vp, 2 eps, 8 (eps - delta)
    // half-precision parameter storage (half_params != 0): vp, eps, delta as
    // IEEE half, widened in the kernels; prm_* are unused then
    const __half *h_vp, *h_eps, *h_del;
    int half_params;
    const float *w1o, *w1c; float *w1n;   // w11, w12 -> w13
    const float *w3o, *w3c; float *w3n;   // w31, w32 -> w33
    const float *po, *pc; float *pn;      // p1, p2 -> p3
    const float *w21o; float *w21n;       // w21 -> w21'
    const float4 *layers;     // [3][pml] (a1h, a1l, d*dt, dd) for lr, fb, tb: the
                              // reference's a1 = (d*dt+1)^2 - 3 as an exact float
                              // pair; a2 = 2*d*dt - 1 and a3 = 1 - d*dt follow
    int arith;                // Arith of this launch
    float *gmax;              // gmax[0..nt): max|grad u| per step
    float *record;            // record plane of this step, or null
    const SrcEntry *src;      // sources inside the updated box, fused
    int nsrc;
    unsigned *err;
    // threshold decisions of the step, one bit per cell in the layout of amask
    // (exact steps only): written to dec_out, or read from dec_in instead of
    // being taken (the gradient's recomputation replays the forward's)
    unsigned *dec_out;
    const unsigned *dec_in;
    unsigned long long wait_ns;   // limit of every bounded device wait (0: 2 s)
    int hold_plane;           // test hook: plane hold_plane - 1 of the first CTA is
                              // never loaded, so its waits run out (0: none)
    // threshold handling of the step kernel
    int spec;                 // 1: predicted window, own max, deferred cells
    const int *gate;          // exact mode: run only if *gate != 0 (null: always)
    float *win;               // spec: &win[3*step] = (M_lo, M_hi, M_pred)
    const float *spec_err;    // kSpecHist last relative prediction errors of the max
    float delta_min;          // smallest half-width of the window
    float spec_bias;          // relative shift of the window (test hook, 0)
    // Cells whose decision waits for the exact max of the step ("deferred"):
    // one bit per cell, 32 y-cells per word (word = pitched index / 32), and
    // at the cell's own index its m2 and its alternative value: u(k+1) with
    // S = 1 (source included); a PML cell also keeps the split-field outputs
    // of S = 1 {w13, w21, w33, p3} in apml.
    unsigned *amask;
    float *am2, *av;
    float4 *apml;
    unsigned *alt_count;      // &alt_count[step]: deferred cells (compaction)
    unsigned *fix_count;      // &fix_count[step]: of them below the threshold
    unsigned *alist;          // their pitched indices (compaction -> fix-up)
    unsigned alist_cap;
    // batched launches only
    int ucur;                 // index of u(k) among the shot's three buffers
    int active;               // 0 once the shot has run all its steps
};

// One shot of a batched run, as the host lays it out in device memory; the
// per-step PlaneParams are derived from it on the device
// (qp3d_batch_prepare_kernel), so a captured step can be replayed.
struct BatchShot {
    int nx, ny, nz, ldy, pml, sz, nt, hx, hy;
    long long plane;
    float dt, delta_min;
    float *U[3];
    const float *VP, *E2, *R8;
    float *W1[3], *W3[3], *P[3], *W21[2];
    const float4 *layers;
    float *gmax;
    float *record;
    const SrcEntry *src;
    int nsrc;
    const float *wavelet;     // nt samples
    float *win;               // 3 * nt
    int *redo;                // nt
    unsigned *alt_count;      // nt
    float *spec_err;
    unsigned *amask;          // vol / 32 words
    float *am2, *av;          // vol each
    float4 *apml;             // vol
    unsigned *fix_count;      // nt
    unsigned *alist;          // alist_cap entries
    unsigned alist_cap;
    float spec_bias;
    unsigned *err;
};

// A unit of work of a batched launch: one tile column of one shot.
struct WorkItem {
    int shot, tile_x, y0, x0, z0, z1;
};

// Kernel arguments of the batched plane kernels.  The coefficient tables are
// shared by all shots of a batch (same spacing and FD tables).
struct BatchArgs {
    Coefs k;
    const PlaneParams *pp;    // per shot, the current step
    const CUtensorMap *tm;    // per shot three maps (one per u buffer)
    const WorkItem *work;
    int nwork;
    int *queue;               // next work item (zeroed by the prepare kernel)
    int arith;                // Arith of every shot of the batch
};

// One backward step of the adjoint (qp3d_adjoint.cu): the adjoint state of
// s^{k+1} (L*) to that of s^k (N*), with the scalar operator of step k frozen
// from u^k and the step's threshold.  C: coefficient fields of the
// transposed derivatives (x, y, z first; xx, yy, zz second).
struct AdjParams {
    int nx, ny, nz, ldy, pml, sz, hx, hy;
    long long plane;
    Coefs k;
    float dt;
    const float *u;                        // u^k
    const float *VP, *E2, *R8;             // vp, 2 eps, 8 (eps - delta)
    const float4 *layers;
    const float *T2;                       // threshold m2 of step k
    const unsigned *dec;                   // or its decisions, one bit per cell (null: T2)
    const float *resid;                    // record residual of step k (hx * hy)
    const float *Lu, *Lup, *Lw1, *Lw1o, *Lp, *Lpo, *Lw21, *Lw3, *Lw3o;
    float *Nu, *Nup, *Nw1, *Nw1o, *Np, *Npo, *Nw21, *Nw3, *Nw3o;
    float *C[6];
    float *gK, *gE, *gD;                   // gradient sums over the steps
    int live;                              // 1: S's dependence on grad u included
};

cudaError_t launch_adjoint_step(const AdjParams &a, cudaStream_t stream);
cudaError_t launch_threshold(const float *gmax, float *T2, int n, cudaStream_t stream);
cudaError_t launch_residual(const float *rec, const float *dobs, float *r, long long n,
                            double *misfit, cudaStream_t stream);
cudaError_t launch_to_bf16(const float *a, __nv_bfloat16 *h, long long n, cudaStream_t stream);
cudaError_t launch_from_bf16(const __nv_bfloat16 *h, float *a, long long n, cudaStream_t stream);

// Launchers (qp3d_kernels.cu).  All enqueue on `stream` and return the
// launch error.
cudaError_t launch_gradmax(const CUtensorMap &tm_u, const PlaneParams &p,
                           dim3 grid, size_t smem, cudaStream_t stream, int variant);
cudaError_t launch_step(const CUtensorMap &tm_u, const PlaneParams &p,
                        dim3 grid, size_t smem, cudaStream_t stream);
// Speculative step resolution: compaction of the deferred-cell bitmask into a
// list, then the fix-up of the listed cells.
// resolution and compaction of a speculative step, then its fix-up or (when
// the max fell outside the window) its exact re-run, a persistent grid of
// nsm CTAs
cudaError_t launch_compact(const PlaneParams &p, int *redo, float *spec_err, cudaStream_t stream);
cudaError_t launch_fix_or_rerun(const CUtensorMap &tm_u, const PlaneParams &p, int nsm,
                                size_t smem, cudaStream_t stream);
cudaError_t launch_band_sources(float *u_new, const float *u_cur,
                                const SrcEntry *src, int n, long long plane,
                                int ldy, float w, cudaStream_t stream);
cudaError_t launch_all_sources(float *u_new, const float *u_cur,
                               const SrcEntry *src, int n, long long plane,
                               int ldy, int nx, int ny, int nz, float w,
                               cudaStream_t stream);
cudaError_t launch_record(const float *u, float *rec, int nx, int ny, int pml,
                          int sz, int ldy, long long plane,
                          cudaStream_t stream);
cudaError_t launch_crop(const float *u, float *out, int x0, int x1, int y0,
                        int y1, int z0, int z1, int ldy, long long plane,
                        cudaStream_t stream);
// Per-cell parameters vp, 2 eps, 8 (eps - delta), or vp, eps, delta as
// IEEE half (round to nearest even), from dense [nz][nx][ny] volumes (the
// caller's layout, copied to the device in one piece) into the pitched
// layout, row padding zero.
cudaError_t launch_params_dense(const float *vp, const float *eps, const float *del, float *VP,
                                float *E2, float *R8, int nx, int ny, int nz, int ldy,
                                cudaStream_t stream);
cudaError_t launch_to_half_dense(const float *a, __half *h, int nx, int ny, int nz, int ldy,
                                 cudaStream_t stream);
// Every non-zero sample of a dense [nz][nx][ny] source volume, in index order
// (z, then x, then y), scanned by several host threads.
void scan_source_volume(const float *s, int nx, int ny, int nz, std::vector<SrcEntry> &out);
// Dynamic shared memory of a plane kernel; nsrc = fused sources of the shot
// (the per-CTA source list has room for all of them).
size_t plane_smem_bytes(int tile_x, int pml, int nsrc = kMaxFusedSources);

// Batched launches (persistent CTAs pulling work items).  kind: 0 gradmax,
// 1 exact step (gated per shot), 2 speculative step.
size_t batch_smem_bytes(int tile_x, int pml, int nsrc);
cudaError_t launch_batch_prepare(const BatchShot *shots, int nshots, PlaneParams *pp, int *ctr,
                                 int *queues, int spec, cudaStream_t stream);
cudaError_t launch_batch_plane(int kind, const BatchArgs &b, int grid, int threads, size_t smem,
                               cudaStream_t stream);
cudaError_t launch_batch_fixup(const BatchArgs &b, int nshots, int blocks_per_shot,
                               long long max_words, cudaStream_t stream);
int batch_plane_threads(int tile_x);
cudaError_t batch_ctas_per_sm(int kind, int arith, int threads, size_t smem, int *n);
cudaError_t configure_gradmax_partial();
cudaError_t launch_gradmax_partial(const CUtensorMap &tm_u, const PlaneParams &p, dim3 grid,
                                   size_t smem, cudaStream_t stream, float *partial,
                                   unsigned nblocks, float *out);
cudaError_t configure_kernels();

}  // namespace qp3d
