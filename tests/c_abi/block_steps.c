/* A plain C99 user of the C ABI: the block-step loop of
 * Hermite4GPU_integration.cpp:81-99 through include/gravidy_gb300.h.
 *
 *   block_steps <state.bin> <t_end> <mode>
 *
 * state.bin: uint32 n, double e2, float eta, then n h4_double4 positions
 * (w = mass) and n h4_double4 velocities.  Prints one line:
 *   steps <k> itime <t> atime <t> energy <E> r0 <x> <y> <z>
 * with %a (exact) floating-point values.  With no arguments it only checks
 * that an invalid creation is refused with a status and a message, which
 * needs no GPU. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gravidy_gb300.h"

static int fail(const char *what, int st) {
    fprintf(stderr, "%s: %s (%s)\n", what, h4_status_string(st), h4_last_error());
    return 1;
}

int main(int argc, char **argv) {
    h4_handle h = NULL;
    if (argc < 4) {
        int st = h4_create(&h, 0u, 1e-4, 0.01f, NULL, NULL, H4_FORCE_FP64);
        if (st != H4_ERR_ARG || h4_last_error()[0] == '\0') return 2;
        printf("refused %d %s\n", st, h4_last_error());
        return 0;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    unsigned int n = 0;
    double e2 = 0.0;
    float eta = 0.f;
    if (fread(&n, sizeof n, 1, f) != 1 || fread(&e2, sizeof e2, 1, f) != 1 || fread(&eta, sizeof eta, 1, f) != 1) {
        fclose(f);
        return 3;
    }
    h4_double4 *r = (h4_double4 *)malloc(sizeof(h4_double4) * n);
    h4_double4 *v = (h4_double4 *)malloc(sizeof(h4_double4) * n);
    if (!r || !v || fread(r, sizeof(h4_double4), n, f) != n || fread(v, sizeof(h4_double4), n, f) != n) {
        fclose(f);
        return 3;
    }
    fclose(f);
    const double t_end = atof(argv[2]);
    const int mode = strcmp(argv[3], "mixed") == 0 ? H4_FORCE_MIXED
                     : strcmp(argv[3], "exact") == 0 ? H4_FORCE_EXACT : H4_FORCE_FP64;

    int st = h4_create(&h, n, e2, eta, r, v, mode);
    if (st) return fail("h4_create", st);
    if ((st = h4_init_acc_jrk(h))) return fail("h4_init_acc_jrk", st);
    double atime = 1.0e10, itime = 0.0;
    if ((st = h4_init_dt(h, &atime, 0.01f, itime))) return fail("h4_init_dt", st);
    unsigned long long steps = 0;
    while (itime < t_end) {
        unsigned int nact = 0;
        itime = atime;
        if ((st = h4_find_particles_to_move(h, itime, &nact))) return fail("find", st);
        if ((st = h4_save_old_acc_jrk(h, nact))) return fail("save_old", st);
        if ((st = h4_predicted_pos_vel(h, itime))) return fail("predict", st);
        if ((st = h4_update_acc_jrk(h, nact))) return fail("update", st);
        if ((st = h4_correction_pos_vel(h, itime, nact))) return fail("correct", st);
        if ((st = h4_next_integration_time(h, &atime))) return fail("next_time", st);
        steps++;
    }
    double ek, ep, e;
    if ((st = h4_get_energy(h, &ek, &ep, &e))) return fail("energy", st);
    if ((st = h4_download(h, r, v, NULL, NULL, NULL, NULL, NULL, NULL, NULL))) return fail("download", st);
    printf("steps %llu itime %a atime %a energy %a r0 %a %a %a\n", steps, itime, atime, e, r[0].x, r[0].y, r[0].z);
    h4_destroy(h);
    free(r);
    free(v);
    return 0;
}
