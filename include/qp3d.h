/*
 * qp3d.h -- C ABI of the GB300 implementation of the 3D pure-qP VTI
 * finite-difference modeling loop of hlc0216/Gpu-c_3dqmodeling.
 *
 * Plain C: pointers and sizes only.  All host pointers are caller-owned; the
 * library owns every device buffer (one reusable context per device and
 * host thread).  Every entry point returns QP3D_OK (0) or a negative code;
 * nothing calls exit().
 *
 * Grid convention (as the reference, array_new.c:2 and Main.c:125): padded
 * sizes nx = hx + 2*pml, ny = hy + 2*pml, nz = Nz0 + 2*pml; volumes are
 * [nz][nx][ny] float32 with y fastest.  The record is [nt][hx][hy].
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   qp3d_forward ............ modeling3d, 3dPureqPModeling_single_shot.h:4-6
 *                             (GPU impl 3dPureqPModeling_single_shot.cu:26-447,
 *                             CPU impl modeling3D.c:17-153)
 *   qp3d_shot_* ............. the same call split into load / advance / read
 *                             so that callers can keep the model resident
 *   qp3d_adjoint ............ no counterpart (gradient of the record misfit)
 *   qp3d_batch .............. the shot loop of the main programs
 *                             (3dPureqPModeling1.0.c:225-277, Main.c:181-231),
 *                             one modeling3d call per shot there
 *   qp3d_fdcoff1/2 .......... fdcoff1/fdcoff2, CPU_function.c:111-148
 *   qp3d_pmlcoff ............ pmlcoff, CPU_function.c:150-169
 *   qp3d_source ............. Source, CPU_function.c:37-64
 *   qp3d_extend_model ....... extend_model, CPU_function.c:67-108
 *   qp3d_readmodel3d ........ readmodel3d, CPU_function.c:234-261
 *   qp3d_absmax ............. absMaxval, CPU_function.c:10-22
 * The C++-linkage symbol modeling3d itself is declared in qp3d_modeling3d.h.
 */
#ifndef QP3D_H
#define QP3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QP3D_OK 0
#define QP3D_ERR_ARG (-1)       /* invalid argument or geometry */
#define QP3D_ERR_CUDA (-2)      /* CUDA runtime/driver error */
#define QP3D_ERR_NOMEM (-3)     /* device or host allocation failed */
#define QP3D_ERR_TIMEOUT (-4)   /* a bounded device wait expired */
#define QP3D_ERR_STATE (-5)     /* call out of order (no shot loaded, ...) */
#define QP3D_ERR_IO (-6)        /* file could not be read or written */
#define QP3D_ERR_CALLBACK (-7)  /* a snapshot callback returned non-zero */

typedef struct qp3d_ctx qp3d_ctx;

typedef struct {
    int nx, ny, nz;   /* padded grid (cells) */
    int nt;           /* time steps */
    int pml;          /* absorbing layer thickness (cells) */
    int sz;           /* receiver depth, padded z index */
    float dx, dy, dz; /* spacing (m) */
    float dt;         /* time step (s) */
} qp3d_geom;

typedef struct {
    const float *vp, *epsilon, *delta;   /* padded volumes */
    const float *source;                 /* padded source volume, or NULL */
    const float *wavelet;                /* nt amplitudes */
    const float *dlr, *ddlr;             /* x-face damping profiles, pml each */
    const float *dtb, *ddtb;             /* z-face */
    const float *dfb, *ddfb;             /* y-face */
    const float *c, *c2;                 /* 36-entry tables of fdcoff1/fdcoff2 */
} qp3d_model;

/* Snapshots (3dPureqPModeling_single_shot.cu:340-377): every ntsnap steps,
 * after the step, the interior wavefield and/or its mid slices. */
enum {
    QP3D_SNAP_VOLUME = 0,   /* [Nz0][hx][hy] */
    QP3D_SNAP_XZ = 1,       /* [Nz0][hx] at y = (hy-1)/2 */
    QP3D_SNAP_YZ = 2,       /* [Nz0][hy] at x = (hx-1)/2 */
    QP3D_SNAP_XY = 3        /* [hx][hy]  at z = (Nz0-1)/2 */
};
typedef int (*qp3d_snap_fn)(void *user, int step, int kind, const float *data,
                            int n0, int n1, int n2);
typedef struct {
    int ntsnap;             /* 0: no snapshots */
    unsigned kinds;         /* bit mask of (1u << QP3D_SNAP_*) */
    qp3d_snap_fn fn;
    void *user;
} qp3d_snap;

int qp3d_version(void);
const char *qp3d_strerror(int code);

/* Context: binds a device and a stream.  Not thread-safe per context. */
int qp3d_ctx_create(int device, qp3d_ctx **out);
void qp3d_ctx_destroy(qp3d_ctx *ctx);
const char *qp3d_ctx_last_error(const qp3d_ctx *ctx);

/* One shot, host buffers in and out: the replacement of modeling3d.
 * record: caller-allocated nt*hx*hy floats, fully overwritten.
 * snap: NULL for none. */
int qp3d_forward(qp3d_ctx *ctx, const qp3d_geom *g, const qp3d_model *m,
                 float *record, const qp3d_snap *snap);

/* Many independent shots (each its own grid, model window, source, receiver
 * depth and nt): the replacement of the main programs' loop of modeling3d
 * calls.  Records are the same, bit for bit, as qp3d_forward's for each shot.
 * All shots that fit in device memory are resident at once and every time
 * step of all of them is one launch of a persistent kernel that takes work
 * items (one tile column of one shot) from a device queue; steps after the
 * first three are replayed from a captured CUDA graph.  The tile height and
 * the number of z blocks per column are chosen by timing a few candidate
 * shapes on the first steps of the run (results do not depend on the shape;
 * the choice is cached per set of shot sizes).  Shots whose sources or
 * receivers lie in the never-updated outer 5 cells, with more than 64 source
 * cells, or with FD tables or spacings different from the first shot's run
 * through qp3d_forward instead.  No snapshots.  Uses the context's stream and
 * replaces any shot loaded with qp3d_shot_load. */
typedef struct {
    qp3d_geom geom;
    qp3d_model model;
    float *record;        /* out: nt*hx*hy floats, fully overwritten */
} qp3d_shot;

int qp3d_batch(qp3d_ctx *ctx, int nshots, const qp3d_shot *shots);

typedef struct {
    int groups;           /* groups of resident shots, run one after another */
    int batched_shots;    /* shots run by the batched launches */
    int single_shots;     /* shots run through qp3d_forward */
    int candidate;        /* tile / z-block shape used in the last group */
    int tile_rows;        /* its largest tile height (x rows per tile) */
    int zblocks;          /* its z blocks per tile column */
    int tuned;            /* 1: chosen by timing in this call */
    int ncand;            /* candidates timed (tuned calls) */
    float cand_ms[8];     /* mean step time of each candidate (tuned calls) */
    int graph_steps;      /* steps replayed from the captured graph */
    int redo_steps;       /* shot-steps whose speculation missed (re-run) */
    int work_items;       /* work items per launch (last group) */
    int ctas;             /* persistent CTAs per launch (last group) */
    float run_ms;         /* device time of the time loop, summed over groups */
} qp3d_batch_stats;
int qp3d_batch_get_stats(const qp3d_ctx *ctx, qp3d_batch_stats *out);

/* Gradient of the record misfit J = 1/2 sum |record - d_obs|^2 of one shot
 * with respect to vp, epsilon and delta, by the adjoint-state method.  No
 * counterpart in the reference.  The forward is the qp3d_forward step; the
 * adjoint is the transpose of its linearization, split-field PML included:
 * S's dependence on epsilon and delta and (by default, "adj_live" = 1) on
 * the unit normal of the wavefield gradient are differentiated, so the
 * result is the gradient of the forward as it runs; only the threshold
 * decisions (S = 1 below 1% of the step's max |grad u|), which are
 * discontinuous, are held.  "adj_live" = 0 holds the unit normal as well
 * (S frozen per step and cell).  The backward pass needs u^k of every step: when
 * all nt wavefields fit in device memory the forward keeps them
 * ("adj_keep_all", default -1: decided by free memory), otherwise it stores
 * checkpoints every ceil(sqrt(nt)) steps and the backward recomputes each
 * segment.  By default ("adj_ckpt_bf16" = 1) a checkpoint keeps the seven PML
 * state levels in BF16 (u and u_prev stay FP32) and the recomputation replays
 * the forward's threshold decisions, recorded as one bit per cell and step;
 * with "adj_ckpt_bf16" = 0 the checkpoints are FP32 and the recomputation is
 * bit-identical to the forward, so that both schedules give the same
 * gradient bit for bit.  The gradient is added (+=) to the caller's padded [nz][nx][ny]
 * FP64 arrays on the cells outside the PML shell (the shell's parameters
 * extend the interior edge and are held fixed); NULL skips one.  misfit:
 * out, J (may be NULL).  Needs FP32 parameter storage and sources and
 * receivers inside the updated box; replaces the loaded shot. */
int qp3d_adjoint(qp3d_ctx *ctx, const qp3d_geom *g, const qp3d_model *m,
                 const float *d_obs, double *grad_vp, double *grad_eps,
                 double *grad_del, double *misfit);

/* Staged form of the same shot. */
int qp3d_shot_load(qp3d_ctx *ctx, const qp3d_geom *g, const qp3d_model *m);
int qp3d_shot_reset(qp3d_ctx *ctx);                 /* zero state, step 0 */
int qp3d_shot_advance(qp3d_ctx *ctx, int nsteps);   /* enqueue, asynchronous */
int qp3d_shot_sync(qp3d_ctx *ctx);                  /* wait, check errors */
int qp3d_shot_step(const qp3d_ctx *ctx);            /* steps done */
int qp3d_shot_read_record(qp3d_ctx *ctx, int k0, int nsteps, float *out);
int qp3d_shot_read_uxyzmax(qp3d_ctx *ctx, int k0, int nsteps, float *out);
/* Snapshot of the current step through the same callback as qp3d_forward. */
int qp3d_shot_snapshot(qp3d_ctx *ctx, const qp3d_snap *snap);

/* Full state in the reference's own layout (test and checkpoint use):
 * u_prev = u(k-1), u_cur = u(k) as padded volumes; pml_state as six faces
 * L,R,F,B,T,Bo (GPU_kernel.cu:568-628 indexing), each ten arrays
 * w11,w12,w13,w21,w31,w32,w33,p1,p2,p3; only w11,w12,w21,w31,w32,p1,p2 are
 * live between steps.  NULL pointers are skipped. */
size_t qp3d_pml_state_size(int nx, int ny, int nz, int pml);
int qp3d_shot_write_state(qp3d_ctx *ctx, int step, const float *u_prev,
                          const float *u_cur, const float *pml_state);
int qp3d_shot_read_state(qp3d_ctx *ctx, float *u_prev, float *u_cur,
                         float *pml_state);

/* Threshold bookkeeping of steps [k0, k0+nsteps): redo[i] = 1 when the
 * step's predicted max window missed and the step was re-run exactly;
 * alt[i] = number of cells whose decision waited for the exact max.
 * Steps computed with the gradmax pre-pass report 0 for both. */
int qp3d_shot_read_stats(qp3d_ctx *ctx, int k0, int nsteps, int *redo,
                         unsigned *alt);

/* Device timing of nsteps further steps with CUDA events on the context's
 * stream.  ms_total: whole interval; ms_step: sum of the fused step kernel's
 * launch durations; ms_gradmax: sum of the threshold overhead per step (the
 * gradmax pre-pass, or the fix-up and gated re-run of a speculative step).
 * NULL per-kernel pointers skip the per-kernel events. */
int qp3d_shot_time(qp3d_ctx *ctx, int nsteps, float *ms_total, float *ms_step,
                   float *ms_gradmax);
/* Number of kernels the library launches per time step for the loaded shot
 * at its current step, and the total number of kernels this context has
 * launched since it was created. */
int qp3d_shot_launches_per_step(const qp3d_ctx *ctx);
long long qp3d_ctx_launch_count(const qp3d_ctx *ctx);

/* Launch tuning.  Keys: "gradmax_variant" (0: shared-memory z taps,
 * 1: register queue), "tile_x" (rows per tile, 0 = automatic),
 * "chunks" (z chunks, 0 = automatic), "threshold_mode" (0: gradmax pre-pass
 * every step, 1: speculative threshold), "spec_delta_ppm" (smallest
 * half-width of the predicted max window; default 1% for single shots, 2% in
 * qp3d_batch), "spec_bias_ppm" (test hook: shifts the predicted window so that
 * predictions miss and steps re-run).  Single shots: takes effect at the next
 * qp3d_shot_load, or immediately for the loaded shot.  qp3d_batch:
 * "batch_graph" (1: replay steps from a captured graph), "batch_tune"
 * (1: time the candidate shapes), "batch_candidate" (shape index used when
 * not tuning, -1 = default), "batch_mem_mb" (device memory for one group of
 * resident shots, 0 = what is free).  All these settings compute identical
 * results.  "param_fp16" (1: the next qp3d_shot_load / qp3d_forward stores
 * vp, epsilon and delta as IEEE half, rounded to nearest; the stencil stays
 * FP32, and the results equal an FP32 run on the rounded model bit for bit;
 * qp3d_batch always stores FP32).  "adj_ckpt_bf16" (qp3d_adjoint
 * checkpoint storage of the PML state, 0: FP32, 1: BF16 with the forward's
 * threshold decisions replayed (default)).
 * "adj_keep_all" (qp3d_adjoint schedule, 1: keep u^k of every step,
 * 0: checkpoints and recomputation, -1: keep all when nt wavefields fit in
 * the free device memory less 8 GiB).  "adj_live" (qp3d_adjoint, 1: S's
 * dependence on grad u included (default), 0: S frozen per step and cell).
 * "arith" (arithmetic of the step, any time): 1 = fast (default: folded
 * 1/h coefficients and fused multiply-adds; within 1e-5 relative L2 of the
 * reference arithmetic over a 1000-step shot), 0 = the reference CPU
 * operators' roundings, operation by operation (CPU_function.c:301-480),
 * so that records, maxima and states equal the reference's bit for bit.
 * "wait_limit_us" (limit of the kernels' bounded waits, 0: 2 s) and
 * "test_hold_plane" (test hook: a plane index that the first CTA of each
 * launch never loads, so that its waits run out and the step reports
 * QP3D_ERR_TIMEOUT; -1: none). */
int qp3d_tune(qp3d_ctx *ctx, const char *key, int value);
int qp3d_tune_get(const qp3d_ctx *ctx, const char *key);

/* CUDA events on the context's stream, for timing any sequence of library
 * calls on the stream the kernels run on.  slot in [0, 8). */
int qp3d_event_record(qp3d_ctx *ctx, int slot);
int qp3d_event_elapsed(qp3d_ctx *ctx, int slot_start, int slot_end, float *ms);

/* Page-locked host memory (cudaMallocHost), for inputs and records that
 * cross the host link at full speed.  NULL on failure. */
void *qp3d_host_alloc(size_t bytes);
void qp3d_host_free(void *p);

/* max over [5,n-5)^3 of max(|du/dx|,|du/dy|,|du/dz|) of a wavefield the
 * caller keeps in device memory, computed without allocating any device
 * memory.  No counterpart in the reference (there the maximum is a host scan,
 * 3dPureqPModeling_single_shot.cu:284-292); it serves callers that cannot let
 * a library allocate: a framework that already holds the device memory in
 * its own pool, or a loop that forbids allocation after start-up.  Same
 * arithmetic as the library's default path.
 *   d_u    device pointer, [nz][nx][ldy] float32, 16-byte aligned,
 *          ldy >= ny and a multiple of 4
 *   c      host pointer to the 36-entry fdcoff1 table
 *   d_max  device pointer to one float; NaN if a device wait timed out
 *   stream cudaStream_t (NULL: legacy default stream); the call waits for
 *          the stream before it returns
 *   err    optional message buffer (NULL to skip)
 * Returns QP3D_ERR_TIMEOUT when a bounded device wait ran out.
 * Limits: the grid may need at most 65536 tiles of 32x32 cells per z chunk
 * (nx*ny up to about 64 M cells), and at most 65535 tiles along x and z
 * chunks; larger grids return QP3D_ERR_ARG.
 * Its scratch is a fixed device array that every GPU loading the library
 * holds until exit and that all calls share: calls that overlap on the GPU
 * race.  The first call on each device sets up the scratch addresses and the
 * kernel attributes; make it before any stream capture.  Test hooks, set with
 * qp3d_tune(NULL, key, value): "noalloc_wait_limit_us" (limit of the bounded
 * waits, 0: 2 s) and "noalloc_test_hold_plane" (a plane the first CTA never
 * loads, so that its waits run out; -1: none). */
int qp3d_gradmax_noalloc(const float *d_u, int nx, int ny, int nz, int ldy,
                         float dx, float dy, float dz, const float *c,
                         float *d_max, void *stream, char *err, size_t errlen);

/* Host utilities, restating the reference's (see the list above). */
void qp3d_fdcoff1(float *c);
void qp3d_fdcoff2(float *c2);
void qp3d_pmlcoff(int pml, float vpmax, float dx, float dy, float dz,
                  float *dlr, float *ddlr, float *dtb, float *ddtb,
                  float *dfb, float *ddfb);
void qp3d_source(int sx, int sy, int sz, float fm, float amp, float alpha,
                 float dt, float dx, float dy, float dz, float t0, int nt,
                 int nx, int ny, int nz, float *source, float *wavelet);
void qp3d_extend_model(const float *in, float *out, int nx, int ny, int nz,
                       int pml);
float qp3d_absmax(const float *a, size_t n);
/* Window [fny,fny+ny) x [fnx,fnx+nx) x [fnz,fnz+nz) of a file stored
 * [vny][vnx][vnz] (z fastest) into a[nz][nx][ny].  Unlike the reference it
 * fails with QP3D_ERR_IO on a missing file or a short read. */
int qp3d_readmodel3d(const char *filename, float *a, int ny, int nx, int nz,
                     int fny, int fnx, int fnz, int vny, int vnx, int vnz);

#ifdef __cplusplus
}
#endif
#endif /* QP3D_H */
