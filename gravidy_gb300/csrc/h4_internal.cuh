// Internal device-side layout and kernel entry points of the Hermite4 block
// step.  Host code (h4_capi.cu) owns the allocations; kernels get the arrays
// through H4Dev, passed by value.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace h4 {

// 32-byte aligned double4: one 256-bit access per element on sm_100+.
typedef double4_32a dbl4;
__host__ __device__ __forceinline__ dbl4 make_dbl4(double x, double y, double z, double w) {
    dbl4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}

// Per-system control block in device memory.  Every block-time quantity of a
// step lives here, so a step can run without the host reading anything back.
struct H4Ctrl {
    double itime;                  // current block time (ITIME)
    unsigned long long atime_bits; // next block time (ATIME), as the bit
                                   // pattern of a non-negative double, so
                                   // atomicMin on it is a min on the value
    unsigned int nact;             // active particles of the current step
    unsigned int work_next;        // work-queue head of the force kernel
    unsigned int work_total;       // work items of the current force launch
    unsigned int force_split;      // j-chunks per active group (S)
    unsigned int n_blocks_flag;    // blocks of the active-set kernels
    unsigned int err;              // sticky error bits (H4_ERRBIT_*)
    // h4_advance bookkeeping
    double t_stop;                 // stop when itime >= t_stop
    double t_log;                  // stop when itime >= t_log
    unsigned long long steps;      // block steps done
    unsigned long long psteps;     // sum of nact
    unsigned long long inter;      // sum of nact * n
    unsigned long long max_steps;  // hard bound on steps of one advance call
    unsigned long long nact_hist[32]; // block steps by floor(log2(nact)), since creation
    int running;                   // 1 while the device loop continues
    unsigned int bounds_site;      // first failing check of the bounds-checked build (0 = none)
};

enum : unsigned int {
    H4_ERRBIT_NONFINITE = 1u,      // non-finite value met in the corrector
    H4_ERRBIT_SPLIT = 2u,          // partial-force scratch too small
    H4_ERRBIT_STEPCAP = 4u,        // device loop reached its step bound
    H4_ERRBIT_TIMEOUT = 8u,        // a bounded wait (mbarrier) gave up
    H4_ERRBIT_BOUNDS = 16u,        // an index check of the bounds-checked build failed
};

// ---- bounds-checked build -----------------------------------------------------
// Compiled with -DH4_BOUNDS_CHECK, every kernel checks the index ranges it is
// about to touch (the active list and the particle indices in it, the j range
// and the partial-force area of a work item, a system's particle range in an
// ensemble) before touching them.  A violation sets H4_ERRBIT_BOUNDS, keeps
// the first failing site, and the access is skipped instead of made; the
// host reports it as an error.  This stands in for a memory checker.  In the
// normal build kBoundsCheck is false and every check folds away.
#ifdef H4_BOUNDS_CHECK
constexpr bool kBoundsCheck = true;
#else
constexpr bool kBoundsCheck = false;
#endif

// Sites of the checks (the value kept in bounds_site).
enum : unsigned int {
    BS_NACT = 1,          // active count within the particle count
    BS_SCATTER = 2,       // active-list writes of the ordered compaction
    BS_MOVE = 3,          // a particle index read from the active list
    BS_PART = 4,          // partial-force area of a work item or of the reduction
    BS_FP64_J = 5,        // j range of an FP64 warp item
    BS_FP64_K = 6,        // active-list range of an FP64 warp item
    BS_MIXED_J = 7,       // j range (tiles) of a mixed tiled item
    BS_MIXED_K = 8,       // active-list range of a mixed item
    BS_MIXED_WJ = 9,      // j range of a mixed warp item
    BS_ENERGY = 10,       // pair range of the energy kernel
    BS_ENS_SYS = 11,      // an ensemble system's particle range
    BS_ENS_ITEM = 12,     // an ensemble force item's ranges
    BS_ENS_PART = 13,     // an ensemble system's partial-force area
    BS_NOALLOC = 14,      // ranges of the allocation-free force sum
    BS_DIAG = 15,         // diagnostics kernels
};

// [lo, hi) within [0, cap).  Always true in the normal build.
__device__ __forceinline__ bool range_ok(unsigned *err, unsigned *site, unsigned code, long long lo,
                                         long long hi, long long cap) {
    if (!kBoundsCheck) return true;
    if (lo >= 0 && lo <= hi && hi <= cap) return true;
    atomicOr(err, (unsigned)H4_ERRBIT_BOUNDS);
    atomicCAS(site, 0u, code);
    return false;
}

// Device clock in ns (%globaltimer).
__device__ __forceinline__ unsigned long long device_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits until *word differs from `old`, for at most timeout_ns; false on
// timeout.  Every inter-block wait of this library goes through here, so no
// wait can run forever: the caller records an error bit and returns.
__device__ __forceinline__ bool bounded_wait_change(const volatile unsigned *word, unsigned old,
                                                    unsigned long long timeout_ns) {
    const unsigned long long t0 = device_ns();
    while (*word == old) {
        if (device_ns() - t0 > timeout_ns) return false;
        __nanosleep(100);
    }
    return true;
}

struct H4Dev {
    int n;          // particles
    int n_pad;      // predicted arrays are padded to a multiple of 256
    double e2;      // softening squared
    double eta;     // timestep parameter (float value held in double)
    double dt_min, dt_max;
    dbl4 *r, *v;         // corrected position (w = mass) and velocity
    double *f, *old;        // [6n] acc/jerk, Forces layout (a[3], a1[3])
    double *a2, *a3;        // [3n] double3 layout
    double *t, *dt;         // [n]
    dbl4 *pr, *pv;       // [n_pad] predicted position (w = mass), velocity
    float4 *jf0, *jf1, *jf2; // [n_pad] predicted j data for the mixed kernels:
                             // (x_hi, y_hi, z_hi, m), (x_lo, y_lo, z_lo, 0), (vx, vy, vz, 0)
    float4 *jd;              // [5][n_pad] the same j data with every value twice, for
                             // packed f32x2 arithmetic: (xh,xh,yh,yh), (zh,zh,m,m),
                             // (xl,xl,yl,yl), (zl,zl,vx,vx), (vy,vy,vz,vz)
    int mixed;              // mixed form selected: the predictor also writes jf0..2 and jd
    unsigned int *move;     // [n] active list
    unsigned int *blk_cnt;  // [n_blocks_flag] active count per chunk
    double *part;           // partial forces, [S][6][nact] for the current step
    size_t part_cap;        // capacity of part in doubles
    double *epot_i;         // [n] per-particle potential (energy kernel)
    double *energy_out;     // [2] kinetic, potential
    H4Ctrl *ctrl;
};

__device__ __forceinline__ bool range_ok(const H4Dev &d, unsigned code, long long lo, long long hi,
                                         long long cap) {
    return range_ok(&d.ctrl->err, &d.ctrl->bounds_site, code, lo, hi, cap);
}

constexpr int FLAG_THREADS = 256;
constexpr int FLAG_ITEMS = 8;                       // elements per thread
constexpr int FLAG_CHUNK = FLAG_THREADS * FLAG_ITEMS;

// ---- exact-order kernels (h4_step_kernels.cu) ------------------------------
void launch_find_active(const H4Dev &d, bool host_itime, double itime, cudaStream_t s);
void launch_save_old(const H4Dev &d, cudaStream_t s);
void launch_predict(const H4Dev &d, bool host_itime, double itime, cudaStream_t s);
void launch_reduce_forces(const H4Dev &d, bool save_old, cudaStream_t s);
void launch_correct(const H4Dev &d, bool host_itime, double itime, bool fused_reduce, cudaStream_t s);
void launch_next_time(const H4Dev &d, bool reset, cudaStream_t s);
// Device-resident step: active set + predictor in the first pass (2 kernels),
// and the next block time with the loop's bookkeeping (1 kernel).
void launch_find_active_predict(const H4Dev &d, cudaStream_t s);
void launch_next_time_bookkeeping(const H4Dev &d, cudaGraphConditionalHandle cond, cudaStream_t s);
void launch_init_dt(const H4Dev &d, float eta, double itime, cudaStream_t s);
void launch_identity_move(const H4Dev &d, cudaStream_t s);
void launch_set_nact(const H4Dev &d, unsigned nact, cudaStream_t s);
void launch_set_atime(const H4Dev &d, double atime, cudaStream_t s);
void launch_reduce_to(const H4Dev &d, double *out, cudaStream_t s);
void launch_set_pred_from_state(const H4Dev &d, cudaStream_t s);
void launch_pad_predicted(const H4Dev &d, cudaStream_t s);
// The mixed form's j data (jf0..2, jd) from the predicted arrays pr, pv.
void launch_pack_j(const H4Dev &d, cudaStream_t s);

// ---- force kernels -----------------------------------------------------------
// Active list and count come from d.move / d.ctrl->nact; results are written
// as partial sums into d.part (reduced by launch_reduce_forces/correct).
void launch_force_fp64(const H4Dev &d, int grid_warps, cudaStream_t s);
void launch_force_exact(const H4Dev &d, cudaStream_t s);   // writes d.part with S = 1
// Returns the number of kernels launched (1 or 2).
int launch_force_mixed(const H4Dev &d, int num_sms, unsigned threshold, long long known_nact, cudaStream_t s);

int force_fp64_grid_warps(int num_sms);

// ---- energy (h4_energy.cu) --------------------------------------------------
void launch_energy(const H4Dev &d, cudaStream_t s);

// ---- peaks -------------------------------------------------------------------
cudaError_t probe_peaks(double *fp64, double *fp32);
cudaError_t selftest_bounded_wait(double seconds, int *timed_out);

}  // namespace h4
