/*
 * A plain C caller of the library's C ABI (include/des_gpu.h,
 * include/des_workload.h): builds a seeded box, its topology and boundary
 * normals, creates the device state, runs init() and the loop, and writes
 * every loop field at three points to a binary file.  tests/test_abi_harness.py
 * compiles it, runs it on config 1 and compares the fields with the golden
 * hashes of the reference's own functions.
 *
 *   abi_harness PARAMS NX NY NZ XL YL ZL JITTER SEED T_TOP T_BOTTOM OUT
 *
 * PARAMS holds a des_params (sizeof bytes); OUT receives, for step 0, 100 and
 * 2000, the 20 fields in the order of FIELDS below, then time, dt, steps.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "des_gpu.h"
#include "des_workload.h"

static int fail(const char *what, int rc)
{
    fprintf(stderr, "%s: %s (%d)\n", what, des_gpu_error_string(rc), rc);
    return 1;
}

#define CK(call)                              \
    do {                                      \
        int rc_ = (call);                     \
        if (rc_) return fail(#call, rc_);     \
    } while (0)

static void put(FILE *f, const double *a, size_t n) { fwrite(a, sizeof(double), n, f); }

int main(int argc, char **argv)
{
    if (argc != 13) {
        fprintf(stderr, "usage: %s PARAMS NX NY NZ XL YL ZL JITTER SEED T_TOP T_BOTTOM OUT\n", argv[0]);
        return 2;
    }
    des_params p;
    FILE *pf = fopen(argv[1], "rb");
    if (!pf || fread(&p, sizeof p, 1, pf) != 1) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(pf);
    des_box_spec box = {atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), atof(argv[5]), atof(argv[6]),
                        atof(argv[7]), atof(argv[8]), strtoull(argv[9], NULL, 10)};
    const double t_top = atof(argv[10]), t_bottom = atof(argv[11]);

    int nn, ne, ns;
    CK(des_box_sizes(&box, &nn, &ne, &ns));
    const size_t N = (size_t)nn, E = (size_t)ne;
    double *coord = calloc(3 * N, sizeof(double));
    int *conn = calloc(4 * E, sizeof(int));
    int *seg = calloc(3 * (size_t)ns, sizeof(int));
    int *segflag = calloc((size_t)ns, sizeof(int));
    int *markers = calloc(E, sizeof(int));
    CK(des_box_fill(&box, coord, conn, seg, segflag));
    const int mattype = 0;
    const double no_depth = 0.0;
    CK(des_markers_layered(ne, 1, coord, conn, 4, box.zlength, 1, &mattype, &no_depth, box.seed + 1,
                           markers));

    des_mesh_view mesh = {nn, ne, ns, 1, conn, seg, segflag, markers};
    des_topology *topo = NULL;
    CK(des_topology_build(&mesh, &topo));
    CK(des_boundary_normals(topo, conn, coord, &p));

    /* the loop state in the reference layout */
    double *node3[4], *node1[5], *elem1[7], *elem6[3], *elem4[3], *tmp12;
    for (int i = 0; i < 4; ++i) node3[i] = calloc(3 * N, sizeof(double));
    for (int i = 0; i < 5; ++i) node1[i] = calloc(N, sizeof(double));
    for (int i = 0; i < 7; ++i) elem1[i] = calloc(E, sizeof(double));
    for (int i = 0; i < 3; ++i) elem6[i] = calloc(6 * E, sizeof(double));
    for (int i = 0; i < 3; ++i) elem4[i] = calloc(4 * E, sizeof(double));
    tmp12 = calloc(12 * E, sizeof(double));
    des_state_view s = {nn, ne,
                        node3[0], node3[1], node3[2], node3[3],           /* coord vel force coord0 */
                        node1[0], node1[1], node1[2], node1[3], node1[4], /* T mass tmass volume_n ntmp */
                        elem1[0], elem1[1], elem1[2],                     /* volume volume_old edvoldt */
                        elem1[3], elem1[4], elem1[5], elem1[6],           /* plstrain dpls dpressure sg */
                        elem6[0], elem6[1], elem6[2],                     /* stress strain strain_rate */
                        elem4[0], elem4[1], elem4[2], tmp12, 0.0, 0.0, 0};
    memcpy(s.coord, coord, sizeof(double) * 3 * N);
    CK(des_temperature_linear(nn, coord, box.zlength, t_top, t_bottom, 0.0, 0, s.temperature));

    des_gpu *g = NULL;
    CK(des_gpu_create(&mesh, &p, 0, &g));
    CK(des_gpu_upload(g, &s, DES_F_COORD | DES_F_TEMPERATURE | DES_F_PLSTRAIN));
    CK(des_gpu_init_fields(g));

    FILE *out = fopen(argv[12], "wb");
    if (!out) return 2;
    const int at[3] = {0, 100, 2000};
    int done = 0;
    for (int k = 0; k < 3; ++k) {
        des_step_report r;
        if (at[k] > done) CK(des_gpu_step(g, at[k] - done, &r));
        done = at[k];
        CK(des_gpu_download(g, &s, DES_F_ALL));
        /* FIELDS: coord vel force temperature mass tmass volume_n ntmp volume
         * volume_old edvoldt plstrain delta_plstrain dpressure stress strain
         * strain_rate shpdx shpdy shpdz */
        put(out, s.coord, 3 * N);
        put(out, s.vel, 3 * N);
        put(out, s.force, 3 * N);
        put(out, s.temperature, N);
        put(out, s.mass, N);
        put(out, s.tmass, N);
        put(out, s.volume_n, N);
        put(out, s.ntmp, N);
        put(out, s.volume, E);
        put(out, s.volume_old, E);
        put(out, s.edvoldt, E);
        put(out, s.plstrain, E);
        put(out, s.delta_plstrain, E);
        put(out, s.dpressure, E);
        put(out, s.stress, 6 * E);
        put(out, s.strain, 6 * E);
        put(out, s.strain_rate, 6 * E);
        put(out, s.shpdx, 4 * E);
        put(out, s.shpdy, 4 * E);
        put(out, s.shpdz, 4 * E);
        double sc[3] = {s.time, s.dt, (double)s.steps};
        put(out, sc, 3);
    }
    fclose(out);
    CK(des_gpu_destroy(g));
    des_topology_free(topo);
    printf("abi_harness: %d tets, %d steps\n", ne, done);
    return 0;
}
