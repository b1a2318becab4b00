/* h4_oracle.c -- CPU restatement of the reference GraviDy Hermite4 CPU path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the CPU
 * baseline timed by bench.py.  Nothing in the product library uses it.
 *
 * Each function names the reference routine it restates (paths relative to
 * the GraviDy source tree).  The floating-point operations are written in the
 * reference's order and the file is compiled with -ffp-contract=off, so that
 * every result is bit-identical to the reference built with g++ on x86-64
 * (where no FMA contraction happens) on any host, x86-64 or AArch64.
 * Parallel loops only split independent per-particle work; every sum keeps
 * the reference's serial order, so results do not depend on the thread count.
 */
#include "h4_oracle.h"
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_D_TIME_MIN 1.1920928955078125e-07 /* common.hpp:122, 2^-23 */
#define ORC_D_TIME_MAX 0.125                  /* common.hpp:129, 2^-3 */
static const float ORC_ETA_S = 0.01f;         /* common.hpp:114 */

double orc_e2_from_softening(float softening)
{
    /* NbodySystem.cpp:50 -- e2 = op.softening * op.softening, a float product */
    float e2f = softening * softening;
    return (double)e2f;
}

int orc_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

orc_system *orc_create(unsigned int n, double e2, float eta,
                       const orc_double4 *r, const orc_double4 *v)
{
    orc_system *s = (orc_system *)calloc(1, sizeof(orc_system));
    if (!s) return NULL;
    s->n = n;
    s->e2 = e2;
    s->eta = eta;
    s->dt_min = ORC_D_TIME_MIN;
    s->dt_max = ORC_D_TIME_MAX;
    size_t nn = n ? n : 1;
    s->r = (orc_double4 *)calloc(nn, sizeof(orc_double4));
    s->v = (orc_double4 *)calloc(nn, sizeof(orc_double4));
    s->f = (orc_forces *)calloc(nn, sizeof(orc_forces));
    s->old = (orc_forces *)calloc(nn, sizeof(orc_forces));
    s->a2 = (orc_double3 *)calloc(nn, sizeof(orc_double3));
    s->a3 = (orc_double3 *)calloc(nn, sizeof(orc_double3));
    s->t = (double *)calloc(nn, sizeof(double));
    s->dt = (double *)calloc(nn, sizeof(double));
    s->move = (unsigned int *)calloc(nn, sizeof(unsigned int));
    s->p = (orc_predictor *)calloc(nn, sizeof(orc_predictor));
    s->epot_i = (double *)calloc(nn, sizeof(double));
    if (!s->r || !s->v || !s->f || !s->old || !s->a2 || !s->a3 || !s->t ||
        !s->dt || !s->move || !s->p || !s->epot_i) {
        orc_destroy(s);
        return NULL;
    }
    if (n) {
        memcpy(s->r, r, n * sizeof(orc_double4));
        memcpy(s->v, v, n * sizeof(orc_double4));
    }
    /* Hermite4::init_data, Hermite4.cpp:194-240: predictors from r, v, m;
     * everything else zero.  (NbodySystem's max_mass starts at 0,
     * NbodySystem.cpp:84.) */
    for (unsigned int i = 0; i < n; i++) {
        double mass = s->r[i].w;
        s->p[i].m = (float)mass;
        s->p[i].r[0] = s->r[i].x;
        s->p[i].r[1] = s->r[i].y;
        s->p[i].r[2] = s->r[i].z;
        s->p[i].v[0] = s->v[i].x;
        s->p[i].v[1] = s->v[i].y;
        s->p[i].v[2] = s->v[i].z;
    }
    s->max_mass = 0.0;
    return s;
}

void orc_destroy(orc_system *s)
{
    if (!s) return;
    free(s->r); free(s->v); free(s->f); free(s->old); free(s->a2); free(s->a3);
    free(s->t); free(s->dt); free(s->move); free(s->p); free(s->epot_i);
    free(s);
}

void orc_set_dt_limits(orc_system *s, double dt_min, double dt_max)
{
    s->dt_min = dt_min;
    s->dt_max = dt_max;
}

/* Hermite4::find_particles_to_move, Hermite4.cpp:63-84 */
unsigned int orc_find_particles_to_move(orc_system *s, double itime)
{
    unsigned int j = 0;
    for (unsigned int i = 0; i < s->n; i++) {
        s->move[i] = (unsigned int)-1;
        if (s->r[i].w > (double)(float)s->max_mass)
            s->max_mass = (float)s->r[i].w;
        double tmp_time = s->t[i] + s->dt[i];
        if (fabs(itime - tmp_time) < 2 * DBL_EPSILON) {
            s->move[j] = i;
            j++;
        }
    }
    return j;
}

/* Hermite4::next_integration_time, Hermite4.cpp:90-102 */
void orc_next_integration_time(orc_system *s, double *ctime)
{
    *ctime = s->t[0] + s->dt[0];
    for (unsigned int i = 1; i < s->n; i++) {
        double time = s->t[i] + s->dt[i];
        if (time < *ctime) *ctime = time;
    }
}

/* (int) of a double as x86-64 cvttsd2si does it: NaN and out-of-range values
 * give INT_MIN.  The reference relies on this when |jerk| is zero
 * (Hermite4.cpp:124); C leaves it undefined, so it is spelled out here. */
static int orc_trunc_to_int(double x)
{
    if (!(x > -2147483649.0 && x < 2147483648.0)) return INT_MIN;
    return (int)x;
}

/* Hermite4::init_dt, Hermite4.cpp:108-140 */
void orc_init_dt(orc_system *s, double *ctime, float eta, double itime)
{
    for (unsigned int i = 0; i < s->n; i++) {
        const orc_forces *f = &s->f[i];
        double a2 = orc_get_magnitude(f->a[0], f->a[1], f->a[2]);
        double j2 = orc_get_magnitude(f->a1[0], f->a1[1], f->a1[2]);
        double tmp_dt = eta * (a2 / j2);
        int ex = orc_trunc_to_int(ceil(log(tmp_dt) / log(2.0)) - 1);
        tmp_dt = pow(2, ex);
        if (tmp_dt < s->dt_min)
            tmp_dt = s->dt_min;
        else if (tmp_dt > s->dt_max)
            tmp_dt = s->dt_max;
        s->dt[i] = tmp_dt;
        s->t[i] = itime;
        if (tmp_dt < *ctime) *ctime = tmp_dt;
    }
}

/* Hermite4::save_old_acc_jrk, Hermite4.cpp:145-153 */
void orc_save_old_acc_jrk(orc_system *s, unsigned int nact)
{
    for (unsigned int k = 0; k < nact; k++) {
        unsigned int i = s->move[k];
        s->old[i] = s->f[i];
    }
}

/* Hermite4CPU::force_calculation, Hermite4CPU.cpp:55-82 */
void orc_force_calculation(const orc_predictor *pi, const orc_predictor *pj,
                           orc_forces *fi, double e2)
{
    double rx = pj->r[0] - pi->r[0];
    double ry = pj->r[1] - pi->r[1];
    double rz = pj->r[2] - pi->r[2];
    double vx = pj->v[0] - pi->v[0];
    double vy = pj->v[1] - pi->v[1];
    double vz = pj->v[2] - pi->v[2];
    double r2 = rx * rx + ry * ry + rz * rz + e2;
    double rinv = 1.0 / sqrt(r2);
    double r2inv = rinv * rinv;
    double r3inv = r2inv * rinv;
    double r5inv = r2inv * r3inv;
    double mr3inv = r3inv * pj->m;
    double mr5inv = r5inv * pj->m;
    double rv = rx * vx + ry * vy + rz * vz;
    fi->a[0] += (rx * mr3inv);
    fi->a[1] += (ry * mr3inv);
    fi->a[2] += (rz * mr3inv);
    fi->a1[0] += (vx * mr3inv - (3 * rv) * rx * mr5inv);
    fi->a1[1] += (vy * mr3inv - (3 * rv) * ry * mr5inv);
    fi->a1[2] += (vz * mr3inv - (3 * rv) * rz * mr5inv);
}

/* Hermite4CPU::init_acc_jrk, Hermite4CPU.cpp:289-304 (accumulates into f,
 * which Hermite4::init_data left at zero). */
void orc_init_acc_jrk(orc_system *s)
{
    long n = (long)s->n;
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < n; i++) {
        for (long j = 0; j < n; j++) {
            if (i == j) continue;
            orc_force_calculation(&s->p[i], &s->p[j], &s->f[i], s->e2);
        }
    }
}

void orc_forces_for(unsigned int n, const orc_predictor *p, double e2,
                    unsigned int nact, const unsigned int *move, orc_forces *out)
{
    long na = (long)nact;
#pragma omp parallel for schedule(dynamic, 4)
    for (long k = 0; k < na; k++) {
        unsigned int i = move[k];
        orc_forces f;
        memset(&f, 0, sizeof(f));
        for (unsigned int j = 0; j < n; j++) {
            if (i == j) continue;
            orc_force_calculation(&p[i], &p[j], &f, e2);
        }
        out[k] = f;
    }
}

/* Hermite4CPU::update_acc_jrk, Hermite4CPU.cpp:309-336 */
void orc_update_acc_jrk(orc_system *s, unsigned int nact)
{
    long na = (long)nact;
#pragma omp parallel for schedule(dynamic, 4)
    for (long k = 0; k < na; k++) {
        unsigned int i = s->move[k];
        orc_forces *fi = &s->f[i];
        memset(fi, 0, sizeof(*fi));
        for (unsigned int j = 0; j < s->n; j++) {
            if (i == j) continue;
            orc_force_calculation(&s->p[i], &s->p[j], fi, s->e2);
        }
    }
}

/* Hermite4CPU::predicted_pos_vel, Hermite4CPU.cpp:340-365 */
void orc_predicted_pos_vel(orc_system *s, double itime)
{
    long n = (long)s->n;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double dt = itime - s->t[i];
        double dt2 = (dt * dt);
        double dt3 = (dt2 * dt);
        double dt2c = dt2 / 2.0;
        double dt3c = dt3 / 6.0;
        const orc_forces *f = &s->f[i];
        orc_predictor *p = &s->p[i];
        p->r[0] = (dt3c * f->a1[0]) + (dt2c * f->a[0]) + (dt * s->v[i].x) + s->r[i].x;
        p->r[1] = (dt3c * f->a1[1]) + (dt2c * f->a[1]) + (dt * s->v[i].y) + s->r[i].y;
        p->r[2] = (dt3c * f->a1[2]) + (dt2c * f->a[2]) + (dt * s->v[i].z) + s->r[i].z;
        p->v[0] = (dt2c * f->a1[0]) + (dt * f->a[0]) + s->v[i].x;
        p->v[1] = (dt2c * f->a1[1]) + (dt * f->a[1]) + s->v[i].y;
        p->v[2] = (dt2c * f->a1[2]) + (dt * f->a[2]) + s->v[i].z;
        p->m = (float)s->r[i].w;
    }
}

/* NbodyUtils::get_magnitude, NbodyUtils.cpp:331-334 */
double orc_get_magnitude(double x, double y, double z)
{
    return sqrt(x * x + y * y + z * z);
}

/* NbodyUtils::get_timestep_normal, NbodyUtils.cpp:337-365 */
double orc_get_timestep_normal(const orc_system *s, unsigned int i, float eta)
{
    const orc_double3 *a2 = &s->a2[i];
    const orc_double3 *a3 = &s->a3[i];
    const orc_forces *f = &s->f[i];
    double ax1_2 = a2->x + s->dt[i] * a3->x;
    double ay1_2 = a2->y + s->dt[i] * a3->y;
    double az1_2 = a2->z + s->dt[i] * a3->z;
    double abs_a1 = orc_get_magnitude(f->a[0], f->a[1], f->a[2]);
    double abs_j1 = orc_get_magnitude(f->a1[0], f->a1[1], f->a1[2]);
    double abs_j12 = abs_j1 * abs_j1;
    double abs_a1_3 = orc_get_magnitude(a3->x, a3->y, a3->z);
    double abs_a1_2 = orc_get_magnitude(ax1_2, ay1_2, az1_2);
    double abs_a1_22 = abs_a1_2 * abs_a1_2;
    return sqrt(eta * ((abs_a1 * abs_a1_2 + abs_j12) / (abs_j1 * abs_a1_3 + abs_a1_22)));
}

/* NbodyUtils::normalize_dt, NbodyUtils.cpp:371-424 */
double orc_normalize_dt(const orc_system *s, double new_dt, double old_dt, double t)
{
    if (new_dt <= old_dt / 8) {
        new_dt = ORC_D_TIME_MIN;
    } else if (old_dt / 8 < new_dt && new_dt <= old_dt / 4) {
        new_dt = old_dt / 8;
    } else if (old_dt / 4 < new_dt && new_dt <= old_dt / 2) {
        new_dt = old_dt / 4;
    } else if (old_dt / 2 < new_dt && new_dt <= old_dt) {
        new_dt = old_dt / 2;
    } else if (old_dt < new_dt && new_dt <= old_dt * 2) {
        new_dt = old_dt;
    } else if (2 * old_dt < new_dt) {
        double val = t / (2 * old_dt);
        if (ceil(val) == val)
            new_dt = 2.0 * old_dt;
        else
            new_dt = old_dt;
    } else {
        new_dt = old_dt;
    }
    if (new_dt < s->dt_min)
        new_dt = s->dt_min;
    else if (new_dt > s->dt_max)
        new_dt = s->dt_max;
    return new_dt;
}

/* Hermite4CPU::correction_pos_vel, Hermite4CPU.cpp:370-411 */
void orc_correction_pos_vel(orc_system *s, double itime, unsigned int nact)
{
    long na = (long)nact;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < na; k++) {
        int i = (int)s->move[k];
        const orc_forces *f = &s->f[i];
        const orc_forces *o = &s->old[i];
        orc_double3 *a2 = &s->a2[i];
        orc_double3 *a3 = &s->a3[i];
        const orc_predictor *p = &s->p[i];
        double dt1 = s->dt[i];
        double dt2 = dt1 * dt1;
        double dt3 = dt2 * dt1;
        double dt4 = dt2 * dt2;
        double dt5 = dt4 * dt1;

        a2->x = (-6 * (o->a[0] - f->a[0]) - dt1 * (4 * o->a1[0] + 2 * f->a1[0])) / dt2;
        a2->y = (-6 * (o->a[1] - f->a[1]) - dt1 * (4 * o->a1[1] + 2 * f->a1[1])) / dt2;
        a2->z = (-6 * (o->a[2] - f->a[2]) - dt1 * (4 * o->a1[2] + 2 * f->a1[2])) / dt2;

        a3->x = (12 * (o->a[0] - f->a[0]) + 6 * dt1 * (o->a1[0] + f->a1[0])) / dt3;
        a3->y = (12 * (o->a[1] - f->a[1]) + 6 * dt1 * (o->a1[1] + f->a1[1])) / dt3;
        a3->z = (12 * (o->a[2] - f->a[2]) + 6 * dt1 * (o->a1[2] + f->a1[2])) / dt3;

        s->r[i].x = p->r[0] + (dt4 / 24) * a2->x + (dt5 / 120) * a3->x;
        s->r[i].y = p->r[1] + (dt4 / 24) * a2->y + (dt5 / 120) * a3->y;
        s->r[i].z = p->r[2] + (dt4 / 24) * a2->z + (dt5 / 120) * a3->z;

        s->v[i].x = p->v[0] + (dt3 / 6) * a2->x + (dt4 / 24) * a3->x;
        s->v[i].y = p->v[1] + (dt3 / 6) * a2->y + (dt4 / 24) * a3->y;
        s->v[i].z = p->v[2] + (dt3 / 6) * a2->z + (dt4 / 24) * a3->z;

        s->t[i] = itime;
        double normal_dt = orc_get_timestep_normal(s, (unsigned int)i, s->eta);
        normal_dt = orc_normalize_dt(s, normal_dt, s->dt[i], s->t[i]);
        s->dt[i] = normal_dt;
    }
}

/* NbodyUtils::get_energy, NbodyUtils.cpp:427-529 (PN terms compiled out).
 * The reference adds the per-i partial sums with omp atomic; with one thread
 * that is i order, which is the order used here for any thread count. */
double orc_get_energy(orc_system *s, double *ekin, double *epot)
{
    long n = (long)s->n;
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < n; i++) {
        double epot_tmp = 0.0;
        for (long j = i + 1; j < n; j++) {
            double rx = s->r[j].x - s->r[i].x;
            double ry = s->r[j].y - s->r[i].y;
            double rz = s->r[j].z - s->r[i].z;
            double r2 = rx * rx + ry * ry + rz * rz;
            epot_tmp -= (s->r[i].w * s->r[j].w) / sqrt(r2);
        }
        s->epot_i[i] = epot_tmp;
    }
    double kinetic = 0.0, potential = 0.0;
    for (long i = 0; i < n; i++) {
        double vvx = s->v[i].x * s->v[i].x;
        double vvy = s->v[i].y * s->v[i].y;
        double vvz = s->v[i].z * s->v[i].z;
        double vv2 = vvx + vvy + vvz;
        double ekin_tmp = 0.5 * s->r[i].w * vv2;
        kinetic += ekin_tmp;
        potential += s->epot_i[i];
    }
    if (ekin) *ekin = kinetic;
    if (epot) *epot = potential;
    return kinetic + potential + 0.0;
}

/* One pass of the loop body of Hermite4CPU_integration.cpp:81-99. */
unsigned int orc_block_step(orc_system *s, double *itime, double *atime)
{
    *itime = *atime;
    unsigned int nact = orc_find_particles_to_move(s, *itime);
    orc_save_old_acc_jrk(s, nact);
    orc_predicted_pos_vel(s, *itime);
    orc_update_acc_jrk(s, nact);
    orc_correction_pos_vel(s, *itime, nact);
    orc_next_integration_time(s, atime);
    return nact;
}

/* Hermite4CPU_integration.cpp:38-124 without nbody_attributes, snapshots and
 * the info file (diagnostic outputs that do not feed back into the state). */
int orc_integrate(orc_system *s, float t_end, float interval, orc_run_stats *st,
                  double *rows, int max_rows)
{
    double atime = 1.0e+10;
    double itime = 0.0;
    unsigned int output_factor = 1;
    int nrows = 0;
    long long nsteps = 0, iterations = 0, interactions = 0;

    orc_init_acc_jrk(s);
    orc_init_dt(s, &atime, ORC_ETA_S, itime);
    double e_ini = orc_get_energy(s, NULL, NULL);
    double e_last = e_ini;
    if (rows && nrows < max_rows) {
        rows[4 * nrows + 0] = itime;
        rows[4 * nrows + 1] = 0.0;
        rows[4 * nrows + 2] = 0.0;
        rows[4 * nrows + 3] = e_ini;
        nrows++;
    }
    while (itime < t_end) {
        unsigned int nact = orc_block_step(s, &itime, &atime);
        interactions += (long long)nact * s->n;
        if (itime >= interval * output_factor) {
            e_last = orc_get_energy(s, NULL, NULL);
            if (rows && nrows < max_rows) {
                rows[4 * nrows + 0] = itime;
                rows[4 * nrows + 1] = (double)iterations;
                rows[4 * nrows + 2] = (double)nsteps;
                rows[4 * nrows + 3] = e_last;
                nrows++;
            }
            output_factor += 1;
        }
        nsteps += nact;
        iterations++;
    }
    if (st) {
        st->itime = itime;
        st->atime = atime;
        st->iterations = iterations;
        st->nsteps = nsteps;
        st->interactions = interactions;
        st->e_ini = e_ini;
        st->e_last = e_last;
    }
    return nrows;
}

unsigned long long orc_fnv1a(const void *p, size_t nbytes, unsigned long long h)
{
    const unsigned char *b = (const unsigned char *)p;
    for (size_t k = 0; k < nbytes; k++) {
        h ^= b[k];
        h *= 1099511628211ULL;
    }
    return h;
}

void orc_state_record(const orc_system *s, double *out)
{
    for (unsigned int i = 0; i < s->n; i++) {
        double *rec = out + 15 * (size_t)i;
        rec[0] = s->r[i].x; rec[1] = s->r[i].y; rec[2] = s->r[i].z; rec[3] = s->r[i].w;
        rec[4] = s->v[i].x; rec[5] = s->v[i].y; rec[6] = s->v[i].z;
        rec[7] = s->f[i].a[0]; rec[8] = s->f[i].a[1]; rec[9] = s->f[i].a[2];
        rec[10] = s->f[i].a1[0]; rec[11] = s->f[i].a1[1]; rec[12] = s->f[i].a1[2];
        rec[13] = s->t[i]; rec[14] = s->dt[i];
    }
}

unsigned long long orc_state_hash(const orc_system *s)
{
    unsigned long long h = 14695981039346656037ULL;
    double rec[15];
    for (unsigned int i = 0; i < s->n; i++) {
        rec[0] = s->r[i].x; rec[1] = s->r[i].y; rec[2] = s->r[i].z; rec[3] = s->r[i].w;
        rec[4] = s->v[i].x; rec[5] = s->v[i].y; rec[6] = s->v[i].z;
        rec[7] = s->f[i].a[0]; rec[8] = s->f[i].a[1]; rec[9] = s->f[i].a[2];
        rec[10] = s->f[i].a1[0]; rec[11] = s->f[i].a1[1]; rec[12] = s->f[i].a1[2];
        rec[13] = s->t[i]; rec[14] = s->dt[i];
        h = orc_fnv1a(rec, sizeof(rec), h);
    }
    return h;
}

/* ---- diagnostics (NbodyUtils.cpp:59-328) ------------------------------------ */

#define ORC_PI 3.14159265358979323846   /* M_PI of the reference's <cmath> */

typedef struct { int index; double value; } orc_distance;

static int orc_cmp_distance(const void *a, const void *b)
{
    const double x = ((const orc_distance *)a)->value, y = ((const orc_distance *)b)->value;
    return (x < y) ? -1 : (x > y) ? 1 : 0;
}

float orc_total_mass(const orc_system *s)
{
    float m = 0.0f;   /* NbodySystem.cpp:182: float += float (the parsed mass) */
    for (unsigned int i = 0; i < s->n; i++) m += (float)s->r[i].w;
    return m;
}

/* NbodyUtils::get_center_of_density, NbodyUtils.cpp:163-220 (J = 6,
 * common.hpp:94): density from the 6th neighbour distance, float radius and
 * density, float sum of the densities. */
void orc_center_of_density(const orc_system *s, double cod[3])
{
    const unsigned int n = s->n;
    const int J = 6;
    double *p = (double *)calloc(n ? n : 1, sizeof(double));
    long nn = (long)n;
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < nn; i++) {
        /* the J+1 smallest entries of d (self = 0 included), kept sorted */
        double best[7];
        for (int k = 0; k < 7; k++) best[k] = INFINITY;
        best[0] = 0.0;   /* d[i] keeps the zero-valued default entry */
        int cnt = 1;
        for (unsigned int j = 0; j < n; j++) {
            if ((long)j == i) continue;
            double rx = (s->r[j].x - s->r[i].x);
            double ry = (s->r[j].y - s->r[i].y);
            double rz = (s->r[j].z - s->r[i].z);
            double v = sqrt(rx * rx + ry * ry + rz * rz);
            if (cnt < 7 || v < best[6]) {
                int k = cnt < 7 ? cnt++ : 6;
                while (k > 0 && best[k - 1] > v) { best[k] = best[k - 1]; k--; }
                best[k] = v;
            }
        }
        float radius = (float)best[J];
        float aa = (J - 1) * s->r[i].w;
        float bb = (4.0 * ORC_PI * radius * radius * radius) / 3.0;
        p[i] = aa / bb;
    }
    double cx = 0.0, cy = 0.0, cz = 0.0;
    float dsum = 0.0f;
    for (unsigned int i = 0; i < n; i++) {
        dsum += p[i];
        cx += s->r[i].x * p[i];
        cy += s->r[i].y * p[i];
        cz += s->r[i].z * p[i];
    }
    cod[0] = cx / dsum;
    cod[1] = cy / dsum;
    cod[2] = cz / dsum;
    free(p);
}

/* get_core_radius (:108-143), get_halfmass_radius (:223-260) and
 * get_radii + get_layers (:285-328) about `center`.  The reference's layer
 * loop runs past its 6 layers; this one stops there. */
void orc_mass_radii(const orc_system *s, const double center[3], float total_mass, double *core,
                    double *halfmass, double lagrange[6])
{
    static const float LAGRANGE[6] = {0.01f, 0.05f, 0.1f, 0.2f, 0.5f, 0.75f};
    const float CORE_MASS = 0.1f;
    const unsigned int n = s->n;
    orc_distance *d = (orc_distance *)malloc(sizeof(orc_distance) * (n ? n : 1));
    for (unsigned int i = 0; i < n; i++) {
        double rx = s->r[i].x - center[0];
        double ry = s->r[i].y - center[1];
        double rz = s->r[i].z - center[2];
        d[i].index = (int)i;
        d[i].value = sqrt(rx * rx + ry * ry + rz * rz);
    }
    qsort(d, n, sizeof(orc_distance), orc_cmp_distance);
    /* core radius */
    double core_mass = 0.0, radius = 0.0;
    for (unsigned int i = 0; i < n; i++) {
        if (core_mass > total_mass * CORE_MASS) {
            radius = d[i - 1].value;
            break;
        }
        core_mass += s->r[d[i].index].w;
    }
    *core = radius;
    /* half-mass radius */
    float half_mass = 0.0f;
    unsigned int jh = 0;
    for (unsigned int i = 0; i < n; i++) {
        if (half_mass >= total_mass / 2.0) {
            jh = i;
            break;
        }
        half_mass += s->r[d[i].index].w;
    }
    *halfmass = jh > 0 ? d[jh - 1].value : 0.0;
    /* Lagrange radii */
    float tmp_mass = 0.0f;
    unsigned int layer = 0;
    for (int k = 0; k < 6; k++) lagrange[k] = 0.0;
    for (unsigned int i = 0; i < n && layer < 6; i++) {
        if (tmp_mass >= total_mass) break;
        if (tmp_mass > LAGRANGE[layer]) {
            lagrange[layer] = d[i].value;
            layer += 1;
        }
        tmp_mass += s->r[d[i].index].w;
    }
    free(d);
}

/* NbodyUtils::nbody_attributes, NbodyUtils.cpp:59-78, with
 * get_virial_radius (:81-86), get_crossing_time (:88-97),
 * get_close_encounter_radius/_timestep (:99-110) and
 * get_half_mass_relaxation_time (:145-160). */
void orc_nbody_attributes(const orc_system *s, double e_ini, float total_mass, double cod_state[3],
                          orc_attributes *out)
{
    const int G = 1;
    const unsigned int n = s->n;
    double lag[6], core, core2, half;
    float r_virial = (-G * total_mass * total_mass) / (4 * e_ini);
    float M = total_mass;
    float Rv3 = (double)r_virial * (double)r_virial * (double)r_virial;
    float Ut = sqrt(Rv3 / (G * M));
    float t_cr = 2 * sqrt(2) * Ut;
    double r_cl = (4.0 * (double)r_virial) / n;
    float r_cl3 = r_cl * r_cl * r_cl;
    double dt_cl = 0.04 * sqrt(r_cl3 * n);
    /* core radius about the NbodyUtils::cod held on entry */
    orc_mass_radii(s, cod_state, total_mass, &core, &half, lag);
    /* relaxation time: center of density first, then the half-mass radius */
    orc_center_of_density(s, cod_state);
    orc_mass_radii(s, cod_state, total_mass, &core2, &half, lag);
    float r_h = half;
    float a = sqrt((n * r_h * r_h * r_h) / (G * (total_mass / (n))));
    float b = 1 / log(0.11 * n);
    float t_rh = 0.138 * a * b;
    out->r_virial = r_virial;
    out->t_cr = t_cr;
    out->r_cl = r_cl;
    out->dt_cl = dt_cl;
    out->r_core = core;
    out->t_rlx = t_rh;
    out->r_hm = r_h;
    out->cod[0] = cod_state[0];
    out->cod[1] = cod_state[1];
    out->cod[2] = cod_state[2];
}
