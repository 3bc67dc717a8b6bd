// qp3d_driver.cpp -- the modeling program around qp3d_forward (see
// include/qp3d_driver.h).  Follows the shot loop of Main.c:148-247 /
// 3dPureqPModeling1.0.c:225-312 with the library's own host utilities.
#include "qp3d.h"
#include "qp3d_driver.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <string>
#include <utility>
#include <vector>

namespace qp3d {
int write_snapshot_files(void *user, int step, int kind, const float *data, int n0, int n1,
                         int n2);
std::string snapshot_file_name(const std::string &prefix, int kind, int step);
}

namespace {

int fail(char *err, size_t errlen, int code, const char *fmt, ...)
{
    if (err && errlen) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, errlen, fmt, ap);
        va_end(ap);
    }
    return code;
}

// One parameter-file reader state: the reference skips a header line before
// every value line and the rest of each value line after its values.
struct Reader {
    FILE *fp;
    bool ok = true;
    int section = 0;
    void skip_line()
    {
        int ch;
        while ((ch = fgetc(fp)) != EOF && ch != '\n') {
        }
    }
    void header()
    {
        skip_line();
        ++section;
    }
    void i(int *v) { ok = ok && fscanf(fp, "%d", v) == 1; }
    void f(float *v) { ok = ok && fscanf(fp, "%f", v) == 1; }
    void s(char *v) { ok = ok && fscanf(fp, "%255s", v) == 1; }
};

int write_file(const char *name, const float *d, size_t n, const char *mode)
{   // read_write.c:29-77: raw native floats, "wb+" or "ab+"
    FILE *fp = fopen(name, mode);
    if (!fp) return -1;
    size_t w = fwrite(d, sizeof(float), n, fp);
    int rc = fclose(fp);
    return (w == n && rc == 0) ? 0 : -1;
}

struct ShotInputs {
    std::vector<float> vp, eps, del, source, wavelet, prof[6];
};

// Window of the three model files for one shot, padded into the PML shell
// (3dPureqPModeling1.0.c:234-250).
int read_shot_model(const qp3d_parameters &P, int sx, int sy, ShotInputs &in, char *err,
                    size_t errlen)
{
    const int nx = P.hx + 2 * P.pml, ny = P.hy + 2 * P.pml, nz = P.Nz0 + 2 * P.pml;
    const int fny = sy - (P.hy - 1) / 2, fnx = sx - (P.hx - 1) / 2;
    if (fny < 0 || fnx < 0 || fny + P.hy > P.Ny0 || fnx + P.hx > P.Nx0)
        return fail(err, errlen, QP3D_ERR_ARG,
                    "shot at (%d,%d): window [%d,%d)x[%d,%d) leaves the %dx%d model", sx, sy, fnx,
                    fnx + P.hx, fny, fny + P.hy, P.Nx0, P.Ny0);
    const char *files[3] = {P.vp_file, P.eps_file, P.del_file};
    std::vector<float> *dst[3] = {&in.vp, &in.eps, &in.del};
    std::vector<float> win((size_t)P.hx * P.hy * P.Nz0);
    for (int a = 0; a < 3; ++a) {
        int rc = qp3d_readmodel3d(files[a], win.data(), P.hy, P.hx, P.Nz0, fny, fnx, 0, P.Ny0,
                                  P.Nx0, P.Nz0);
        if (rc) return fail(err, errlen, rc, "cannot read %s (window at %d,%d)", files[a], fnx, fny);
        dst[a]->assign((size_t)nx * ny * nz, 0.0f);
        qp3d_extend_model(win.data(), dst[a]->data(), nx, ny, nz, P.pml);
    }
    return QP3D_OK;
}

// PML profiles and source for the model in `in` (3dPureqPModeling1.0.c:261-266).
void shot_source(const qp3d_parameters &P, ShotInputs &in)
{
    const int nx = P.hx + 2 * P.pml, ny = P.hy + 2 * P.pml, nz = P.Nz0 + 2 * P.pml;
    const size_t n = (size_t)nx * ny * nz;
    const float vpmax = (1 + 2 * qp3d_absmax(in.eps.data(), n)) * qp3d_absmax(in.vp.data(), n);
    for (auto &pr : in.prof) pr.assign(std::max(P.pml, 1), 0.0f);
    qp3d_pmlcoff(P.pml, vpmax, P.dx, P.dy, P.dz, in.prof[0].data(), in.prof[1].data(),
                 in.prof[2].data(), in.prof[3].data(), in.prof[4].data(), in.prof[5].data());
    const int sx1 = (P.hx - 1) / 2 + P.pml, sy1 = (P.hy - 1) / 2 + P.pml, sz1 = P.pml;
    in.source.assign(n, 0.0f);
    in.wavelet.assign(P.nt, 0.0f);
    qp3d_source(sx1, sy1, sz1, P.fm, P.amp, P.alpha, P.dt, P.dx, P.dy, P.dz, 1.0f / P.fm, P.nt,
                nx, ny, nz, in.source.data(), in.wavelet.data());
}

// Geometry and model of one shot (receivers on the top of the window, as
// 3dPureqPModeling1.0.c:267 passes sz = pml).
void shot_geom_model(const qp3d_parameters &P, ShotInputs &in, const float *c, const float *c2,
                     qp3d_geom &g, qp3d_model &m)
{
    g.nx = P.hx + 2 * P.pml; g.ny = P.hy + 2 * P.pml; g.nz = P.Nz0 + 2 * P.pml;
    g.nt = P.nt; g.pml = P.pml; g.sz = P.pml;
    g.dx = P.dx; g.dy = P.dy; g.dz = P.dz; g.dt = P.dt;
    m.vp = in.vp.data(); m.epsilon = in.eps.data(); m.delta = in.del.data();
    m.source = in.source.data(); m.wavelet = in.wavelet.data();
    m.dlr = in.prof[0].data(); m.ddlr = in.prof[1].data(); m.dtb = in.prof[2].data();
    m.ddtb = in.prof[3].data(); m.dfb = in.prof[4].data(); m.ddfb = in.prof[5].data();
    m.c = c; m.c2 = c2;
}

// RSF header of a file of [n_k]...[n_1] floats, axes given fastest first.
int rsf(const char *file, std::initializer_list<std::pair<long long, float>> ax,
        std::initializer_list<const char *> labels)
{
    long long n[4];
    float d[4];
    const char *lab[4];
    int k = 0;
    for (const auto &a : ax) n[k] = a.first, d[k] = a.second, ++k;
    k = 0;
    for (const char *l : labels) lab[k++] = l;
    return qp3d_write_rsf_header(file, (int)ax.size(), n, d, lab);
}

// Snapshot callback: the files of write_snapshot_files, plus their RSF
// headers when asked for.
struct SnapFiles {
    std::string prefix;
    bool rsf;
    float dx, dy, dz;
};

int snapshot_with_headers(void *user, int step, int kind, const float *data, int n0, int n1,
                          int n2)
{
    const SnapFiles *s = static_cast<const SnapFiles *>(user);
    std::string prefix = s->prefix;
    if (qp3d::write_snapshot_files(&prefix, step, kind, data, n0, n1, n2)) return -1;
    if (!s->rsf) return 0;
    const std::string name = qp3d::snapshot_file_name(s->prefix, kind, step);
    switch (kind) {
    case QP3D_SNAP_VOLUME:   // [z][x][y]
        return rsf(name.c_str(), {{n2, s->dy}, {n1, s->dx}, {n0, s->dz}}, {"y", "x", "z"});
    case QP3D_SNAP_XZ:       // [z][x]
        return rsf(name.c_str(), {{n1, s->dx}, {n0, s->dz}}, {"x", "z"});
    case QP3D_SNAP_YZ:       // [z][y]
        return rsf(name.c_str(), {{n1, s->dy}, {n0, s->dz}}, {"y", "z"});
    default:                 // [x][y]
        return rsf(name.c_str(), {{n1, s->dy}, {n0, s->dx}}, {"y", "x"});
    }
}

int model_shot(qp3d_ctx *ctx, const qp3d_parameters &P, ShotInputs &in, const float *c,
               const float *c2, int snapflag, const char *snap_prefix, bool write_rsf,
               float *record, char *err, size_t errlen)
{
    qp3d_geom g;
    qp3d_model m;
    shot_geom_model(P, in, c, c2, g, m);
    SnapFiles files{std::string(snap_prefix), write_rsf, P.dx, P.dy, P.dz};
    qp3d_snap snap;
    snap.ntsnap = P.ntsnap;
    snap.kinds = 0xFu;
    snap.fn = snapshot_with_headers;
    snap.user = &files;
    int rc = qp3d_forward(ctx, &g, &m, record, (snapflag == 1 && P.ntsnap > 0) ? &snap : nullptr);
    if (rc) return fail(err, errlen, rc, "modeling failed: %s", qp3d_ctx_last_error(ctx));
    return QP3D_OK;
}

}  // namespace

extern "C" int qp3d_parse_parameter_file(const char *path, qp3d_parameters *P, char *err,
                                         size_t errlen)
{
    if (!path || !P) return fail(err, errlen, QP3D_ERR_ARG, "null argument");
    memset(P, 0, sizeof(*P));
    FILE *fp = fopen(path, "r");
    if (!fp) return fail(err, errlen, QP3D_ERR_IO, "cannot open %s", path);
    Reader r{fp};
    r.header(); r.f(&P->dt); r.i(&P->nt); r.i(&P->ntsnap); r.skip_line();
    r.header(); r.i(&P->Nx0); r.i(&P->Ny0); r.i(&P->Nz0); r.skip_line();
    r.header(); r.f(&P->dx); r.f(&P->dy); r.f(&P->dz); r.skip_line();
    r.header(); r.f(&P->fm); r.f(&P->amp); r.f(&P->alpha); r.skip_line();
    r.header(); r.i(&P->sx0); r.i(&P->sy0); r.i(&P->sz0); r.skip_line();
    r.header(); r.i(&P->gx0); r.i(&P->gy0); r.i(&P->gz0); r.skip_line();
    r.header(); r.i(&P->nxshot); r.i(&P->nyshot); r.i(&P->dxshot); r.i(&P->dyshot); r.skip_line();
    r.header(); r.i(&P->hx); r.i(&P->hy); r.skip_line();
    r.header(); r.i(&P->pml); r.skip_line();
    r.header(); r.s(P->vp_file); r.s(P->eps_file); r.s(P->del_file); r.skip_line();
    r.header(); r.s(P->recfull_file); r.s(P->recdir_file); r.s(P->recmut_file); r.skip_line();
    r.header(); r.s(P->recxz_file); r.s(P->recyz_file); r.skip_line();
    r.header(); r.s(P->snap_direct); r.s(P->snap_full); r.skip_line();
    r.header(); r.i(&P->multishot); r.skip_line();
    r.header(); r.i(&P->muteflag); r.skip_line();
    r.header(); r.i(&P->snapflag_full); r.skip_line();
    r.header(); r.i(&P->snapflag_direct);
    fclose(fp);
    if (!r.ok)
        return fail(err, errlen, QP3D_ERR_ARG, "%s: missing or malformed value in section %d",
                    path, r.section);
    if (P->nt < 1 || !(P->dt > 0) || !(P->dx > 0) || !(P->dy > 0) || !(P->dz > 0) || !(P->fm > 0))
        return fail(err, errlen, QP3D_ERR_ARG, "%s: nt, dt, spacing and fm must be positive", path);
    if (P->Nx0 < 1 || P->Ny0 < 1 || P->Nz0 < 1 || P->hx < 1 || P->hy < 1 || P->pml < 0 ||
        P->hx > P->Nx0 || P->hy > P->Ny0)
        return fail(err, errlen, QP3D_ERR_ARG, "%s: model, window or pml size invalid", path);
    if (P->nxshot < 0 || P->nyshot < 0)
        return fail(err, errlen, QP3D_ERR_ARG, "%s: negative shot count", path);
    if ((P->snapflag_full == 1 || P->snapflag_direct == 1) && P->ntsnap <= 0)
        return fail(err, errlen, QP3D_ERR_ARG, "%s: snapshots requested with ntsnap <= 0", path);
    return QP3D_OK;
}

extern "C" int qp3d_run_parameter_file(const char *path, const qp3d_run_options *opt, char *err,
                                       size_t errlen)
{
    qp3d_run_options o{0, QP3D_DIRECT_SOURCE_CELL, 0.f, 0.f, 0.f, 0, 0, 0};
    if (opt) o = *opt;
    qp3d_parameters P;
    int rc = qp3d_parse_parameter_file(path, &P, err, errlen);
    if (rc) return rc;
    const int nx = P.hx + 2 * P.pml, ny = P.hy + 2 * P.pml, nz = P.Nz0 + 2 * P.pml;
    const size_t n = (size_t)nx * ny * nz, nrec = (size_t)P.nt * P.hx * P.hy;
    float c[36] = {0}, c2[36] = {0};
    qp3d_fdcoff1(c);
    qp3d_fdcoff2(c2);
    qp3d_ctx *ctx = nullptr;
    rc = qp3d_ctx_create(o.device, &ctx);
    if (rc) return fail(err, errlen, rc, "no CUDA device %d", o.device);
    std::vector<float> rec_direct(nrec, 0.0f), rec_mute(nrec);
    ShotInputs in;

    // direct wave (Main.c:148-160), once before the shot loop
    if (P.muteflag == 1) {
        float vd = 0.f, ed = 0.f, dd = 0.f;
        if (o.direct_model == QP3D_DIRECT_SOURCE_CELL) {
            if ((rc = read_shot_model(P, P.sx0, P.sy0, in, err, errlen))) goto done;
            const size_t sc = ((size_t)P.pml * nx + (P.hx - 1) / 2 + P.pml) * ny + (P.hy - 1) / 2 + P.pml;
            vd = in.vp[sc]; ed = in.eps[sc]; dd = in.del[sc];
        } else if (o.direct_model == QP3D_DIRECT_VALUES) {
            vd = o.direct_vp; ed = o.direct_eps; dd = o.direct_del;
        }
        in.vp.assign(n, vd);
        in.eps.assign(n, ed);
        in.del.assign(n, dd);
        shot_source(P, in);
        if (o.verbose) printf("direct wave: vp %g eps %g delta %g\n", vd, ed, dd);
        if ((rc = model_shot(ctx, P, in, c, c2, P.snapflag_direct, P.snap_direct,
                             o.write_rsf == 1, rec_direct.data(), err, errlen)))
            goto done;
        if (write_file(P.recdir_file, rec_direct.data(), nrec, "wb")) {
            rc = fail(err, errlen, QP3D_ERR_IO, "cannot write %s", P.recdir_file);
            goto done;
        }
    }
    // shot loop (Main.c:162-246): x slow, y fast.  Without per-shot
    // snapshots the shots go through qp3d_batch in groups that fit the host
    // memory budget; the output files are written in the same order.
    {
        std::vector<std::pair<int, int>> pos;
        for (int ix = 0; ix < P.nxshot; ++ix)
            for (int iy = 0; iy < P.nyshot; ++iy)
                pos.push_back({P.sx0 + ix * P.dxshot, P.sy0 + iy * P.dyshot});
        const bool batched = !(P.snapflag_full == 1 && P.ntsnap > 0) && o.shots_per_call != 1;
        const size_t per_shot = (4 * n + nrec + (size_t)P.nt) * sizeof(float);
        size_t group = 1;
        if (batched)
            group = o.shots_per_call > 1 ? (size_t)o.shots_per_call
                                         : std::max<size_t>(1, (16ull << 30) / per_shot);
        for (size_t g0 = 0; g0 < pos.size(); g0 += group) {
            const size_t cnt = std::min(group, pos.size() - g0);
            std::vector<ShotInputs> ins(cnt);
            std::vector<std::vector<float>> recs(cnt, std::vector<float>(nrec));
            for (size_t i = 0; i < cnt; ++i) {
                const int sx = pos[g0 + i].first, sy = pos[g0 + i].second;
                if (o.verbose) printf("shot %zu at (%d,%d)\n", g0 + i, sx, sy);
                if ((rc = read_shot_model(P, sx, sy, ins[i], err, errlen))) goto done;
                shot_source(P, ins[i]);
            }
            if (batched) {
                std::vector<qp3d_shot> shots(cnt);
                for (size_t i = 0; i < cnt; ++i) {
                    shot_geom_model(P, ins[i], c, c2, shots[i].geom, shots[i].model);
                    shots[i].record = recs[i].data();
                }
                if ((rc = qp3d_batch(ctx, (int)cnt, shots.data()))) {
                    rc = fail(err, errlen, rc, "modeling failed: %s", qp3d_ctx_last_error(ctx));
                    goto done;
                }
            } else if ((rc = model_shot(ctx, P, ins[0], c, c2, P.snapflag_full, P.snap_full,
                                        o.write_rsf == 1, recs[0].data(), err, errlen))) {
                goto done;
            }
            for (size_t i = 0; i < cnt; ++i) {
                const std::vector<float> &rec_full = recs[i];
                for (size_t j = 0; j < nrec; ++j) rec_mute[j] = rec_full[j] - rec_direct[j];
                if (write_file(P.recfull_file, rec_full.data(), nrec, "ab") ||
                    write_file(P.recmut_file, rec_mute.data(), nrec, "ab")) {
                    rc = fail(err, errlen, QP3D_ERR_IO, "cannot append %s / %s", P.recfull_file,
                              P.recmut_file);
                    goto done;
                }
                if (g0 + i == 0) {
                    // the reference writes the muted slices, then overwrites
                    // the same files with the full-wave slices (Main.c:216-245)
                    const int jy = (P.hy - 1) / 2, ixs = (P.hx - 1) / 2;
                    std::vector<float> xz((size_t)P.nt * P.hx), yz((size_t)P.nt * P.hy);
                    for (int k = 0; k < P.nt; ++k) {
                        for (int x = 0; x < P.hx; ++x)
                            xz[(size_t)k * P.hx + x] = rec_full[((size_t)k * P.hx + x) * P.hy + jy];
                        for (int y = 0; y < P.hy; ++y)
                            yz[(size_t)k * P.hy + y] = rec_full[((size_t)k * P.hx + ixs) * P.hy + y];
                    }
                    if (write_file(P.recxz_file, xz.data(), xz.size(), "wb") ||
                        write_file(P.recyz_file, yz.data(), yz.size(), "wb")) {
                        rc = fail(err, errlen, QP3D_ERR_IO, "cannot write the record slices");
                        goto done;
                    }
                }
            }
        }
    }
    // RSF headers of the record files; the appended files count every shot
    // they hold
    if (o.write_rsf == 1) {
        const long long per = (long long)nrec * sizeof(float);
        const std::pair<long long, float> y{P.hy, P.dy}, x{P.hx, P.dx}, t{P.nt, P.dt};
        bool ok = true;
        for (const char *f : {P.recfull_file, P.recmut_file}) {
            FILE *fp = fopen(f, "rb");
            long long size = -1;
            if (fp && fseek(fp, 0, SEEK_END) == 0) size = ftell(fp);
            if (fp) fclose(fp);
            ok = ok && size > 0 && size % per == 0 &&
                 !rsf(f, {y, x, t, {size / per, 1.0f}}, {"y", "x", "t", "shot"});
        }
        if (P.muteflag == 1) ok = ok && !rsf(P.recdir_file, {y, x, t}, {"y", "x", "t"});
        ok = ok && !rsf(P.recxz_file, {x, t}, {"x", "t"}) &&
             !rsf(P.recyz_file, {y, t}, {"y", "t"});
        if (!ok) rc = fail(err, errlen, QP3D_ERR_IO, "cannot write the RSF headers");
    }
done:
    qp3d_ctx_destroy(ctx);
    return rc;
}

extern "C" int qp3d_write_rsf_header(const char *datafile, int naxes, const long long *n,
                                     const float *d, const char *const *labels)
{
    if (!datafile || !*datafile || !n || naxes < 1 || naxes > 9) return QP3D_ERR_ARG;
    for (int a = 0; a < naxes; ++a)
        if (n[a] < 1) return QP3D_ERR_ARG;
    std::string h(datafile);
    if (h.size() >= 4 && h.compare(h.size() - 4, 4, ".dat") == 0) h.resize(h.size() - 4);
    h += ".rsf";
    FILE *fp = fopen(h.c_str(), "w");
    if (!fp) return QP3D_ERR_IO;
    fprintf(fp, "in=\"%s\"\ndata_format=\"native_float\"\nesize=4\n", datafile);
    for (int a = 0; a < naxes; ++a) {
        fprintf(fp, "n%d=%lld\n", a + 1, n[a]);
        if (d) fprintf(fp, "d%d=%.9g\no%d=0\n", a + 1, (double)d[a], a + 1);
        if (labels && labels[a]) fprintf(fp, "label%d=\"%s\"\n", a + 1, labels[a]);
    }
    return (ferror(fp) | fclose(fp)) ? QP3D_ERR_IO : QP3D_OK;
}
