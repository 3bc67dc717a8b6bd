/*
 * qp3d_modeling3d.h -- drop-in for the reference's per-shot entry point.
 *
 * Same C++-linkage symbol, signature and behaviour as modeling3d in
 * 3dPureqPModeling_single_shot.h:4-6 (implementations
 * 3dPureqPModeling_single_shot.cu:26-447 and modeling3D.c:17-153), so the
 * reference's own main programs (3dPureqPModeling1.0.c:202,267, Main.c:172,202)
 * link against libqp3d unchanged:
 *   - all pointers are host, caller-owned; vp/epsilon/delta/source are padded
 *     [nz][nx][ny] volumes, wavelet has nt entries, record receives
 *     nt*(nx-2*pml)*(ny-2*pml) samples of the plane z = sz;
 *   - sx, sy are accepted and unused, as in the reference;
 *   - with snapflag == 1, every ntsnap steps it writes <snap_file><k>.dat
 *     (interior volume) and <snap_file>_xz/_yz/_xy<k>.dat slices.
 * Runs on CUDA device 0 like the reference.  It has no return value; errors
 * are reported on stderr (use qp3d_forward for status codes).  Like the
 * reference it is not re-entrant: all calls share one library context that
 * keeps the device buffers between calls of the same grid size; call it from
 * one host thread at a time.
 */
#ifndef QP3D_MODELING3D_H
#define QP3D_MODELING3D_H

#ifdef __cplusplus
void modeling3d(int nx, int ny, int nz, int nt, int ntsnap, float dx, float dy, float dz,
                float dt, int pml, int snapflag, int sx, int sy, int sz, float *vp,
                float *epsilon, float *delta, float *source, float *wavelet, float *record,
                float *dlr, float *ddlr, float *dtb, float *ddtb, float *dfb, float *ddfb,
                float *c, float *c2, const char *snap_file);
#endif

#endif
