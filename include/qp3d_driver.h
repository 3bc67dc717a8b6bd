/*
 * qp3d_driver.h -- the modeling program around qp3d_forward: parameter file,
 * model windows, shot loop, direct-wave muting and the reference's output
 * files.  Replaces the main programs 3dPureqPModeling1.0.c:21-378 (GPU build)
 * and Main.c:15-255 (CPU build); the executable bin/qp3d_modeling is a thin
 * wrapper around qp3d_run_parameter_file.
 */
#ifndef QP3D_DRIVER_H
#define QP3D_DRIVER_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QP3D_PATH_MAX 256

/* Contents of parameter.txt in the reference's fixed order
 * (3dPureqPModeling1.0.c:41-95): each value line follows one header line. */
typedef struct {
    float dt;
    int nt, ntsnap;
    int Nx0, Ny0, Nz0;             /* model size (cells) */
    float dx, dy, dz;
    float fm, amp, alpha;          /* Ricker frequency, amplitude, Gaussian decay */
    int sx0, sy0, sz0;             /* first shot (model cells) */
    int gx0, gy0, gz0;             /* read, unused (as in the reference) */
    int nxshot, nyshot, dxshot, dyshot;
    int hx, hy;                    /* aperture window (cells) */
    int pml;
    char vp_file[QP3D_PATH_MAX], eps_file[QP3D_PATH_MAX], del_file[QP3D_PATH_MAX];
    char recfull_file[QP3D_PATH_MAX], recdir_file[QP3D_PATH_MAX], recmut_file[QP3D_PATH_MAX];
    char recxz_file[QP3D_PATH_MAX], recyz_file[QP3D_PATH_MAX];
    char snap_direct[QP3D_PATH_MAX], snap_full[QP3D_PATH_MAX];
    int multishot, muteflag, snapflag_full, snapflag_direct;
} qp3d_parameters;

/* Direct-wave model used when muteflag == 1.  The reference leaves its direct
 * model zero-filled (3dPureqPModeling1.0.c:105,181-188 commented out), so its
 * "direct wave" is computed with vp = 0; QP3D_DIRECT_ZERO reproduces that.
 * QP3D_DIRECT_SOURCE_CELL (default) uses a homogeneous model with the vp,
 * epsilon, delta of the first shot's model at its source cell, and
 * QP3D_DIRECT_VALUES the values given in the options. */
enum { QP3D_DIRECT_SOURCE_CELL = 0, QP3D_DIRECT_ZERO = 1, QP3D_DIRECT_VALUES = 2 };

typedef struct {
    int device;                    /* CUDA device (the reference uses 0) */
    int direct_model;              /* QP3D_DIRECT_* */
    float direct_vp, direct_eps, direct_del;
    int verbose;                   /* progress lines on stdout */
    int shots_per_call;            /* 0: shots go through qp3d_batch in groups that
                                      fit 16 GB of host memory (one by one when
                                      full-wave snapshots are requested);
                                      1: one qp3d_forward per shot, as the
                                      reference; N > 1: at most N per call */
    int write_rsf;                 /* 1: an RSF header beside every file the job
                                      writes (qp3d_write_rsf_header) */
} qp3d_run_options;

/* Madagascar RSF header for a raw native-float file, in the form of the
 * reference's model/grey3_tmp.rsf: in="<datafile>", data_format, esize, then
 * n, d, o (0) and label of each axis, fastest axis first.  The header is
 * <datafile> with its ".dat" suffix replaced by ".rsf" (".rsf" appended when
 * there is none); in= holds datafile as given.  Returns QP3D_OK,
 * QP3D_ERR_ARG (no name, naxes outside 1..9, an axis n < 1) or QP3D_ERR_IO. */
int qp3d_write_rsf_header(const char *datafile, int naxes, const long long *n, const float *d,
                          const char *const *labels);

/* Parse a parameter file.  Returns QP3D_OK, QP3D_ERR_IO (cannot open) or
 * QP3D_ERR_ARG (a value is missing or out of range); err receives a message. */
int qp3d_parse_parameter_file(const char *path, qp3d_parameters *out, char *err, size_t errlen);

/* Run the whole modeling job a parameter file describes, writing the same
 * files as the reference program: Record_fullwave and Record_mute appended
 * shot after shot (read_write.c:66-77), Record_direct, the first shot's xz/yz
 * record slices, and snapshots through modeling3d's naming.  With write_rsf
 * each gets an RSF header: records [shot][t][x][y] (n4 counts every shot the
 * appended file holds), record slices [t][x] and [t][y], snapshot volumes
 * [z][x][y] and slices [z][x], [z][y], [x][y].  The records do
 * not depend on shots_per_call.  Unlike the
 * reference it stops with an error when a model window leaves the model or a
 * file cannot be read or written.  opt may be NULL (defaults). */
int qp3d_run_parameter_file(const char *path, const qp3d_run_options *opt, char *err,
                            size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
