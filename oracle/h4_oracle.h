/* h4_oracle -- CPU restatement of the reference GraviDy Hermite4 CPU path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * and the timed CPU baseline of bench.py; the product library never links,
 * loads or calls it.  Parity of this restatement with the reference itself is
 * pinned by tests/test_oracle_golden.py against fixtures produced by the
 * reference sources compiled unmodified (oracle/Makefile, target "ref").
 *
 * Every routine keeps the reference's floating-point operation order
 * (compiled with -ffp-contract=off, no fast-math), so results are
 * bit-identical to the reference CPU build on the same inputs.  Float
 * parameters (eta, ETA_S, softening, masses) stay float as in the reference.
 */
#ifndef H4_ORACLE_H
#define H4_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Layouts of src/include/common.hpp:67-77 (double4/double3) and :213-231. */
typedef struct { double x, y, z, w; } orc_double4;
typedef struct { double x, y, z; } orc_double3;
typedef struct { double r[3]; double v[3]; float m; } orc_predictor;
typedef struct { double a[3]; double a1[3]; } orc_forces;

typedef struct orc_system {
    unsigned int n;
    double e2;          /* NbodySystem::e2 (float product, NbodySystem.cpp:50) */
    float eta;          /* NbodySystem::eta, -e flag */
    double dt_min;      /* D_TIME_MIN, common.hpp:122 */
    double dt_max;      /* D_TIME_MAX, common.hpp:129 */
    orc_double4 *r, *v;
    orc_forces *f, *old;
    orc_double3 *a2, *a3;
    double *t, *dt;
    unsigned int *move;
    orc_predictor *p;
    double *epot_i;     /* per-i potential partial sums (scratch) */
    double max_mass;
} orc_system;

/* e2 exactly as NbodySystem.cpp:50: float softening squared in float. */
double orc_e2_from_softening(float softening);

orc_system *orc_create(unsigned int n, double e2, float eta,
                       const orc_double4 *r, const orc_double4 *v);
void orc_destroy(orc_system *s);
void orc_set_dt_limits(orc_system *s, double dt_min, double dt_max);
int orc_set_threads(int nthreads);

/* Hermite4 base (src/include/Hermite4.cpp) */
unsigned int orc_find_particles_to_move(orc_system *s, double itime);
void orc_next_integration_time(orc_system *s, double *ctime);
void orc_init_dt(orc_system *s, double *ctime, float eta, double itime);
void orc_save_old_acc_jrk(orc_system *s, unsigned int nact);

/* Hermite4CPU (src/include/cpu/Hermite4CPU.cpp) */
void orc_force_calculation(const orc_predictor *pi, const orc_predictor *pj,
                           orc_forces *fi, double e2);
void orc_init_acc_jrk(orc_system *s);
void orc_update_acc_jrk(orc_system *s, unsigned int nact);
void orc_predicted_pos_vel(orc_system *s, double itime);
void orc_correction_pos_vel(orc_system *s, double itime, unsigned int nact);

/* NbodyUtils (src/include/utils/NbodyUtils.cpp) */
double orc_get_magnitude(double x, double y, double z);
double orc_get_timestep_normal(const orc_system *s, unsigned int i, float eta);
double orc_normalize_dt(const orc_system *s, double new_dt, double old_dt, double t);
double orc_get_energy(orc_system *s, double *ekin, double *epot);

/* Stateless force sum over an arbitrary active list (update_acc_jrk body). */
void orc_forces_for(unsigned int n, const orc_predictor *p, double e2,
                    unsigned int nact, const unsigned int *move, orc_forces *out);

/* Whole block-step loop body of Hermite4CPU_integration.cpp:81-99. */
unsigned int orc_block_step(orc_system *s, double *itime, double *atime);

/* The integration loop (Hermite4CPU_integration.cpp:49-124) without the
 * diagnostic side outputs.  For every energy log point it appends
 * (itime, iterations, nsteps, energy) to rows[4*k..] (at most max_rows). */
typedef struct {
    double itime;
    double atime;
    long long iterations;
    long long nsteps;
    long long interactions;
    double e_ini;
    double e_last;
} orc_run_stats;
int orc_integrate(orc_system *s, float t_end, float interval, orc_run_stats *st,
                  double *rows, int max_rows);

/* Diagnostics of NbodyUtils (src/include/utils/NbodyUtils.cpp:59-328), with
 * the reference's float/double types.  total_mass is NbodySystem::total_mass
 * (a float summed in input order, NbodySystem.cpp:182).  Need n >= 8 (the
 * reference reads the 6th neighbour, and crashes below that). */
float orc_total_mass(const orc_system *s);
void orc_center_of_density(const orc_system *s, double cod[3]);
/* Core radius (mass fraction CORE_MASS = 0.1, strict), half-mass radius and
 * Lagrange radii (LAGRANGE_RADII = 0.01 .. 0.75) about `center`. */
void orc_mass_radii(const orc_system *s, const double center[3], float total_mass, double *core,
                    double *halfmass, double lagrange[6]);
typedef struct {
    double r_virial, t_cr, r_cl, dt_cl, r_core, t_rlx, r_hm;
    double cod[3];
} orc_attributes;
/* NbodyUtils::nbody_attributes: cod_state is NbodyUtils::cod, in and out
 * (the core radius uses its value on entry, then it is recomputed). */
void orc_nbody_attributes(const orc_system *s, double e_ini, float total_mass, double cod_state[3],
                          orc_attributes *out);

/* FNV-1a 64 over raw bytes, and over the state record
 * (r.x r.y r.z r.w v.x v.y v.z a[3] a1[3] t dt per particle, 15 doubles),
 * the layout written by oracle/ref_harness.cpp. */
unsigned long long orc_fnv1a(const void *p, size_t nbytes, unsigned long long h);
unsigned long long orc_state_hash(const orc_system *s);
void orc_state_record(const orc_system *s, double *out /* 15*n */);

#ifdef __cplusplus
}
#endif
#endif
