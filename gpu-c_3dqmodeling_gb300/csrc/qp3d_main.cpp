// qp3d_main.cpp -- bin/qp3d_modeling: the modeling program of the reference
// (3dPureqPModeling1.0.c, Main.c) on the GB300 library.
//
//   qp3d_modeling [parameter_file] [--device N] [--direct-model source|zero|VP,EPS,DEL]
//                 [--shots-per-call N] [--rsf] [--quiet]
//
// parameter_file defaults to ./input/parameter.txt; paths inside it are
// relative to the working directory, as in the reference.  --rsf writes an
// RSF header beside every output file.
#include "qp3d.h"
#include "qp3d_driver.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

int main(int argc, char **argv)
{
    const char *path = "./input/parameter.txt";
    qp3d_run_options o{0, QP3D_DIRECT_SOURCE_CELL, 0.f, 0.f, 0.f, 1, 0, 0};
    for (int a = 1; a < argc; ++a) {
        if (!strcmp(argv[a], "--device") && a + 1 < argc) {
            o.device = atoi(argv[++a]);
        } else if (!strcmp(argv[a], "--direct-model") && a + 1 < argc) {
            const char *v = argv[++a];
            if (!strcmp(v, "source")) {
                o.direct_model = QP3D_DIRECT_SOURCE_CELL;
            } else if (!strcmp(v, "zero")) {
                o.direct_model = QP3D_DIRECT_ZERO;
            } else if (sscanf(v, "%f,%f,%f", &o.direct_vp, &o.direct_eps, &o.direct_del) == 3) {
                o.direct_model = QP3D_DIRECT_VALUES;
            } else {
                fprintf(stderr, "bad --direct-model %s\n", v);
                return 2;
            }
        } else if (!strcmp(argv[a], "--shots-per-call") && a + 1 < argc) {
            o.shots_per_call = atoi(argv[++a]);
        } else if (!strcmp(argv[a], "--rsf")) {
            o.write_rsf = 1;
        } else if (!strcmp(argv[a], "--quiet")) {
            o.verbose = 0;
        } else if (argv[a][0] == '-') {
            fprintf(stderr, "usage: %s [parameter_file] [--device N] "
                            "[--direct-model source|zero|VP,EPS,DEL] [--shots-per-call N] "
                            "[--rsf] [--quiet]\n", argv[0]);
            return 2;
        } else {
            path = argv[a];
        }
    }
    char err[512];
    int rc = qp3d_run_parameter_file(path, &o, err, sizeof(err));
    if (rc) {
        fprintf(stderr, "qp3d_modeling: %s (%s)\n", err, qp3d_strerror(rc));
        return 1;
    }
    return 0;
}
