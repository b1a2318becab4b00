/* Full-precision trace driver for the reference GraviDy CPU path.
 *
 * Test infrastructure only.  Compiled together with the unmodified reference
 * sources (src/include/Hermite4.cpp, NbodySystem.cpp, utils/NbodyUtils.cpp,
 * utils/Logger.cpp, cpu/Hermite4CPU.cpp) into oracle/_ref/ref_harness by
 * oracle/Makefile.  The reference's own snapshots keep 4 significant digits
 * (src/include/utils/Logger.cpp:84-85), so this driver replays the block-step
 * loop of src/include/cpu/Hermite4CPU_integration.cpp:49-124 call for call and
 * writes the state bit for bit.  The Hermite4CPU methods are private
 * (cpu/Hermite4CPU.hpp:58-68); the Makefile compiles this file with
 * -Dprivate=public to reach them.  Diagnostics that do not touch the dynamics
 * (nbody_attributes, snapshots, info file) are skipped.
 *
 * Usage:
 *   ref_harness -i <input> [-s soft] [-e eta] [-t tend] [-z interval]
 *               -d <outdir> [-K nfull] [-D step,step,...]
 * Writes into <outdir>:
 *   init.bin   : forces after init_acc_jrk, dt after init_dt (little endian)
 *   steps.txt  : per block step "step itime nact fnv(move) fnv(state)"
 *                for the first nfull steps and for every logged step
 *   energy.txt : "itime energy" at t=0 and at every log time (hex floats)
 *   state_<k>.bin for each requested step k (and 'final' at the end)
 *   attributes.txt : for N >= 8, NbodyUtils::nbody_attributes and
 *                lagrange_radii (NbodyUtils.cpp:59-78, 246-328) after the
 *                initial energy and again at the end, in the reference's
 *                call order (hex floats)
 */
#include "cpu/Hermite4CPU.hpp"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <stdint.h>

static uint64_t fnv1a(const void *p, size_t nbytes, uint64_t h)
{
    const unsigned char *b = (const unsigned char *)p;
    for (size_t k = 0; k < nbytes; k++) {
        h ^= b[k];
        h *= 1099511628211ULL;
    }
    return h;
}
static const uint64_t FNV0 = 14695981039346656037ULL;

/* Hash of the integrator state in a fixed layout: r (x,y,z,m), v (x,y,z),
 * a[3], a1[3], t, dt for every particle. */
static uint64_t state_hash(NbodySystem *ns)
{
    uint64_t h = FNV0;
    for (unsigned int i = 0; i < ns->n; i++) {
        double rec[15] = {ns->h_r[i].x, ns->h_r[i].y, ns->h_r[i].z, ns->h_r[i].w,
                          ns->h_v[i].x, ns->h_v[i].y, ns->h_v[i].z,
                          ns->h_f[i].a[0], ns->h_f[i].a[1], ns->h_f[i].a[2],
                          ns->h_f[i].a1[0], ns->h_f[i].a1[1], ns->h_f[i].a1[2],
                          ns->h_t[i], ns->h_dt[i]};
        h = fnv1a(rec, sizeof(rec), h);
    }
    return h;
}

static void write_attributes(FILE *fa, const char *tag, NbodySystem *ns, NbodyUtils *nu)
{
    nu->nbody_attributes();
    std::fprintf(fa, "%s_attr %a %a %a %a %a %a %a %a %a %a\n", tag, (double)ns->r_virial, (double)ns->t_cr,
                 ns->r_cl, ns->dt_cl, ns->r_core, (double)ns->t_rlx, (double)ns->r_hm, nu->cod.x, nu->cod.y,
                 nu->cod.z);
    nu->lagrange_radii();
    std::fprintf(fa, "%s_lagr", tag);
    for (size_t k = 0; k < nu->layers_radii.size(); k++) std::fprintf(fa, " %a", nu->layers_radii[k]);
    std::fprintf(fa, " %a %a %a\n", nu->cod.x, nu->cod.y, nu->cod.z);
}

static void write_state(NbodySystem *ns, const std::string &path)
{
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) { std::perror(path.c_str()); std::exit(2); }
    for (unsigned int i = 0; i < ns->n; i++) {
        double rec[15] = {ns->h_r[i].x, ns->h_r[i].y, ns->h_r[i].z, ns->h_r[i].w,
                          ns->h_v[i].x, ns->h_v[i].y, ns->h_v[i].z,
                          ns->h_f[i].a[0], ns->h_f[i].a[1], ns->h_f[i].a[2],
                          ns->h_f[i].a1[0], ns->h_f[i].a1[1], ns->h_f[i].a1[2],
                          ns->h_t[i], ns->h_dt[i]};
        std::fwrite(rec, sizeof(double), 15, fp);
    }
    std::fclose(fp);
}

int main(int argc, char *argv[])
{
    /* Split our own flags (-d, -K, -D) from the reference flags. */
    std::string outdir;
    long nfull = 200;
    std::set<long> dump_steps;
    std::vector<char *> rargv;
    rargv.push_back(argv[0]);
    for (int k = 1; k < argc; k++) {
        if (!std::strcmp(argv[k], "-d") && k + 1 < argc) { outdir = argv[++k]; }
        else if (!std::strcmp(argv[k], "-K") && k + 1 < argc) { nfull = std::atol(argv[++k]); }
        else if (!std::strcmp(argv[k], "-D") && k + 1 < argc) {
            char *s = argv[++k];
            while (*s) {
                dump_steps.insert(std::strtol(s, &s, 10));
                if (*s == ',') s++;
            }
        } else rargv.push_back(argv[k]);
    }
    if (outdir.empty()) { std::fprintf(stderr, "ref_harness: -d <outdir> required\n"); return 2; }

    OptionsParser op((int)rargv.size(), &rargv[0]);
    if (!op.check_options()) return 1;
    NbodySystem ns(op);
    ns.read_input_file();
    ns.alloc_base_attributes(0);
    ns.copy_input_data();
    Logger logger(&ns);
    NbodyUtils nu(&ns);
    Hermite4CPU h4(&ns, &logger, &nu);

    /* Hermite4CPU_integration.cpp:41-53 */
    double ATIME = 1.0e+10;
    double ITIME = ns.snapshot_time;
    unsigned int nact = 0;
    unsigned int nsteps = 0;
    long long interactions = 0;
    unsigned int output_factor = 1;

    h4.init_acc_jrk();
    h4.init_dt(ATIME, ETA_S, ITIME);
    {
        std::string path = outdir + "/init.bin";
        FILE *fp = std::fopen(path.c_str(), "wb");
        if (!fp) { std::perror(path.c_str()); return 2; }
        for (unsigned int i = 0; i < ns.n; i++) std::fwrite(&ns.h_f[i], sizeof(Forces), 1, fp);
        std::fwrite(ns.h_dt, sizeof(double), ns.n, fp);
        std::fwrite(&ATIME, sizeof(double), 1, fp);
        std::fclose(fp);
    }
    ns.en.ini = nu.get_energy(0);
    ns.en.tmp = ns.en.ini;
    FILE *fa = 0;
    if (ns.n >= 8) {
        std::string apath = outdir + "/attributes.txt";
        fa = std::fopen(apath.c_str(), "w");
        if (!fa) { std::perror("attributes"); return 2; }
        std::fprintf(fa, "total_mass %a\n", (double)ns.total_mass);
        write_attributes(fa, "t0", &ns, &nu);
    }

    std::string spath = outdir + "/steps.txt";
    std::string epath = outdir + "/energy.txt";
    FILE *fs = std::fopen(spath.c_str(), "w");
    FILE *fe = std::fopen(epath.c_str(), "w");
    if (!fs || !fe) { std::perror("open"); return 2; }
    std::fprintf(fe, "%a %a\n", ITIME, ns.en.ini);

    long step = 0;
    while (ITIME < ns.integration_time) {
        ITIME = ATIME;
        nact = h4.find_particles_to_move(ITIME);
        h4.save_old_acc_jrk(nact);
        h4.predicted_pos_vel(ITIME);
        h4.update_acc_jrk(nact);
        h4.correction_pos_vel(ITIME, nact);
        interactions += (long long)nact * ns.n;
        h4.next_integration_time(ATIME);
        bool logged = false;
        if (ITIME >= ns.interval_time * output_factor) {
            double e = nu.get_energy(0);
            std::fprintf(fe, "%a %a\n", ITIME, e);
            output_factor += 1;
            logged = true;
        }
        nsteps += nact;
        ns.iterations++;
        if (step < nfull || logged) {
            std::fprintf(fs, "%ld %a %u %016llx %016llx\n", step, ITIME, nact,
                         (unsigned long long)fnv1a(ns.h_move, sizeof(unsigned int) * nact, FNV0),
                         (unsigned long long)state_hash(&ns));
        }
        if (dump_steps.count(step)) {
            char name[64];
            std::snprintf(name, sizeof(name), "/state_%ld.bin", step);
            write_state(&ns, outdir + name);
        }
        step++;
    }
    write_state(&ns, outdir + "/state_final.bin");
    if (fa) {
        write_attributes(fa, "end", &ns, &nu);
        std::fclose(fa);
    }
    std::fprintf(fs, "# steps %ld nsteps %u interactions %lld\n", step, nsteps, interactions);
    std::fclose(fs);
    std::fclose(fe);
    return 0;
}
