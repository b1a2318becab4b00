// Batched ensemble: many independent N-body systems (star clusters of uneven
// N), each with its own block time and active set, advanced together by one
// persistent fused kernel per graph iteration.
//
// The per-system arithmetic is the single-system path's (exact-order
// predictor/corrector/timestep of h4_exact.cuh, force items of h4_pair.cuh;
// the mixed form's predictor and corrector in their own FP32/FMA forms below);
// what changes is the schedule.  One iteration of k_ensemble does one block
// step of every unfinished system, in four phases separated by grid-wide
// barriers:
//   A  per system (one block): next block time (the least t + dt, kept by
//      the corrector and the last compaction), the reference's loop
//      condition, ordered active set (integer work on the bits of t + dt),
//      force work layout for its (N, N_act) from the tuning table: warp items
//      (lanes over j), or in the mixed form block-tiled items (lanes over i,
//      j tiles in shared memory);
//   B  all threads: predictor of every particle of the stepping systems;
//   C  all blocks: the force sums -- block-tiled items (j tiles brought into
//      shared memory by TMA bulk copies, three stages on full/empty
//      mbarriers; packed f32x2) then warp items (j through a per-warp TMA
//      ring), each kind from one global work queue (the systems' item counts
//      are prefix-summed in shared memory, an item finds its system by binary
//      search);
//   D  all threads: fixed-order reduction of the partial forces, corrector
//      and new timestep of every active particle.
// The O(N) and O(N_act) phases are spread over the whole GPU: FP64
// prediction and correction of a large system on one SM would otherwise set
// the pace of every iteration.
// The kernel is launched cooperatively (all blocks resident), and its grid
// barriers are bounded waits on the global timer: a barrier that waits longer
// than BARRIER_TIMEOUT_NS records H4_ERRBIT_TIMEOUT and every block leaves.
// A CUDA graph with a device-side while loop relaunches the kernel until
// every system has reached its end time.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gravidy_gb300.h"
#include "h4_exact.cuh"
#include "h4_internal.cuh"
#include "h4_pair.cuh"
#include "h4_tma.cuh"

namespace h4 {
namespace ens {

// Resident blocks per SM the register allocation must allow: two in the
// mixed form (16 warps per SM for the FP32 force items; every phase fits 128
// registers a thread), one in the FP64 and exact forms (their FP64 warp items
// need more registers).  Build knob for the mixed form.
#ifndef H4_ENS_MIN_BLOCKS_MIXED
#define H4_ENS_MIN_BLOCKS_MIXED 2
#endif
template <int MODE>
constexpr int kMinBlocks = MODE == H4_FORCE_MIXED ? H4_ENS_MIN_BLOCKS_MIXED : 1;
constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int NB_N = H4_ENS_TUNE_NB_N;
constexpr int NB_A = H4_ENS_TUNE_NB_A;
constexpr unsigned long long BARRIER_TIMEOUT_NS = 60ull * 1000000000ull;
constexpr int ITERS_PER_LAUNCH = 16;
constexpr unsigned MAX_SYSTEMS = 4096;
// Block-tiled items (mixed form): BTI active particles (BTI / 2 packed pairs)
// x one j-chunk, the chunk streamed through shared memory in tiles of JT j,
// JT in {128, 256} (one instantiation each).  The block's 256 threads are
// P = BTI / 2 pairs x Q = 256 / P j-lanes: thread (p, q) takes tile entries
// q, q + Q, ...; each j-lane's sum is a partial of its own (partial index
// s * Q + q), so no reduction inside the block.
constexpr int JT_MAX = 256;
constexpr unsigned BTI_MIN = 16, BTI_MAX = 2 * THREADS;
constexpr unsigned WAIT_LIMIT = 1u << 26;  // mbarrier polls before a tile wait gives up
// Stages in flight: NS block-item tiles per block; per warp, WARP_STAGES
// stages of WARP_STAGE_J j for the warp items.  The two share one shared-memory
// area (a block runs its block items, then its warp items).  Two stages of
// 128 j per warp (four j per lane per stage) measured faster than three or
// four of 64: fewer stage waits and refills, and four independent pairs per
// lane between them.
constexpr unsigned NS = 3;          // block-item tile stages
constexpr int WARP_STAGES = 2;      // warp-item stages (per warp)
constexpr int WARP_STAGE_J = 128;   // j per warp-item stage (four per lane)
constexpr size_t BLOCK_TILE_BYTES = (size_t)NS * 5 * JT_MAX * sizeof(float4);
constexpr size_t WARP_RING_BYTES = (size_t)WARP_STAGES * 3 * WARP_STAGE_J * sizeof(float4);
constexpr size_t TILE_AREA_BYTES =
    BLOCK_TILE_BYTES > WARPS * WARP_RING_BYTES ? BLOCK_TILE_BYTES : WARPS * WARP_RING_BYTES;

struct System {
    int off, n;                  // particle offset and count
    int joff, npad;              // offset and length (n rounded up to JT_MAX) of its block-item j data
    double e2, eta, dt_min, dt_max;
    double t_end;
    double itime, atime;         // last block time, next block time
    unsigned nact;
    unsigned ig, chunk, split, n_groups, items;
    // block-tiled items (mixed form): count, j tile, j-lanes, j-chunks
    // (split = bsplit * q partials per particle)
    unsigned bitems, jt, q, bsplit;
    unsigned done, err;
    // the next block time without a scan (bit patterns of tn): the least tn
    // of the particles that did not step (phase A's compaction) and of those
    // corrected since (phase D, atomic minimum)
    unsigned long long tmin_idle, tmin_stepped;
    size_t part_off, part_cap;   // partial-force area (doubles)
    unsigned long long steps, psteps, inter;
};

struct Dev {
    int nsys, total;
    System *sys;
    dbl4 *r, *v, *pr, *pv;
    double *f, *t, *dt;          // forces (a, jerk), time, timestep
    double *tn;                  // t + dt of every particle (exact::add), set by the corrector
    float4 *jf0, *jf1, *jf2;
    float4 *cs;                  // [4][total] mixed form: corrected state in FP32 form (store_cs)
    float4 *jd;                  // [5][jtotal] duplicated j data of the block-tiled items, each system's
                                 // at joff, padded to npad with zero-mass far-away particles
    int jtotal;
    unsigned *move;
    double *part;
    unsigned *queue;             // force work-queue head (warp items)
    unsigned *queue_b;           // force work-queue head (block items)
    unsigned *bar_count, *bar_gen;
    unsigned *err;               // [2]: global error bits, first failing bounds-check site
    size_t part_total;           // doubles in part
    unsigned *tune_ig, *tune_chunk, *tune_jt;   // [NB_N * NB_A]
    unsigned long long *bucket;  // [NB_N * NB_A][2]: block steps, interactions per (N, N_act) bucket
    unsigned *forced_nact;       // tuning probe: active count forced on every system (0 = off)
    unsigned long long *launches;     // persistent-kernel launches so far
    unsigned long long *phase_ns;     // [4] device time of phases A, B, C, D since creation
    unsigned long long max_launches;
    double *epot_i, *energy;     // energy: per particle, per system (kin, pot)
    int mode;
};

// Bounds-checked build: [lo, hi) within [0, cap) (always true otherwise).
__device__ __forceinline__ bool in_range(const Dev &d, unsigned code, long long lo, long long hi, long long cap) {
    return range_ok(d.err, d.err + 1, code, lo, hi, cap);
}

// Bounds-checked build: a system's particle range and partial-force area.
__device__ __forceinline__ bool system_ok(const Dev &d, const System &S) {
    return in_range(d, BS_ENS_SYS, S.off, (long long)S.off + S.n, d.total) &&
           in_range(d, BS_ENS_PART, (long long)S.part_off, (long long)(S.part_off + S.part_cap),
                    (long long)d.part_total);
}

// Bounds-checked build: the ranges of one force item of system S -- its slice
// of the active list ([k0, k0 + cnt) of nact <= n), its j range, its slice of
// the system's partial-force area, and (lanes < cnt) the particle indices.
__device__ bool item_ok(const Dev &d, const System &S, unsigned s, unsigned k0, unsigned cnt, int jb, int je,
                        unsigned lane) {
    bool ok = system_ok(d, S) && in_range(d, BS_ENS_ITEM, 0, S.nact, S.n) &&
              in_range(d, BS_ENS_ITEM, k0, (long long)k0 + cnt, S.nact) && in_range(d, BS_ENS_ITEM, jb, je, S.n) &&
              in_range(d, BS_ENS_PART, 6ll * S.nact * s, 6ll * S.nact * (s + 1), (long long)S.part_cap);
    if (ok && lane < cnt) {
        const unsigned i = d.move[S.off + k0 + lane];
        ok = in_range(d, BS_MOVE, i, i + 1ll, S.n);
    }
    return ok;
}

// Grid-wide barrier of a cooperative launch, bounded in time.
__device__ bool grid_sync(const Dev &d) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = d.bar_gen;
        const unsigned g0 = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(d.bar_count, 1u) + 1u;
        if (arrived == gridDim.x) {
            *d.bar_count = 0u;
            __threadfence();
            atomicAdd((unsigned *)d.bar_gen, 1u);
        } else if (!bounded_wait_change(gen, g0, BARRIER_TIMEOUT_NS)) {
            atomicOr(d.err, (unsigned)H4_ERRBIT_TIMEOUT);
        }
        __threadfence();
    }
    __syncthreads();
    return (*(volatile unsigned *)d.err & H4_ERRBIT_TIMEOUT) == 0u;
}

// Partials of a particle summed by a warp (the fixed order of
// exact::sum_partials_warp) from this many j-chunks on, by its thread (chunk
// order) below: higher than the single-system path's threshold, so that the
// 32-63-chunk splits of mid-sized warp-item steps stay on the thread path
// (measured: the corrector phase of C4 355 against 491 ms, with the groups
// of the warp path moved to the last blocks).
constexpr unsigned ENS_WARP_REDUCE_MIN_S = 64;
__device__ __forceinline__ bool warp_reduce(unsigned S) { return S >= ENS_WARP_REDUCE_MIN_S; }

__device__ __forceinline__ int n_bucket(int n) {
    int b = 0;
    for (int lim = 512; b < NB_N - 1 && n > lim; lim <<= 1) b++;
    return b;
}
__device__ __forceinline__ int a_bucket(unsigned nact) {
    // 1 | 2-3 | 4-15 | 16-63 | 64-255 | 256-1023 | 1024-4095 | >= 4096
    if (nact <= 1) return 0;
    int b = 1;
    for (unsigned lim = 4; b < NB_A - 1 && nact >= lim; lim <<= 2) b++;
    return b;
}

__device__ unsigned block_sum_u(unsigned x, unsigned *red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    __syncthreads();
    if (lane == 0) red[w] = x;
    __syncthreads();
    unsigned s = 0;
    for (int k = 0; k < WARPS; k++) s += red[k];
    __syncthreads();
    return s;
}

// Exclusive scan of one value per thread (THREADS threads).
__device__ unsigned block_scan_u(unsigned x, unsigned *red, unsigned *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    __syncthreads();
    if (lane == 31) red[w] = incl;
    __syncthreads();
    unsigned before = 0, all = 0;
    for (int k = 0; k < WARPS; k++) {
        if (k < w) before += red[k];
        all += red[k];
    }
    *total = all;
    __syncthreads();
    return before + incl - x;
}

// ---- phase A (one block per system): next block time, ordered active set,
// bookkeeping and force work layout -------------------------------------------
template <int MODE>
__device__ void phaseA(const Dev &d, int c, bool init, unsigned *red, double *redd) {
    System &S = d.sys[c];
    const int off = S.off, n = S.n;
    const unsigned forced = *d.forced_nact;
    unsigned nact = 0;
    double itime = 0.0;
    if (!system_ok(d, S)) {   // bounds-checked build only
        if (threadIdx.x == 0) { S.items = 0; S.bitems = 0; S.nact = 0; S.done = 1u; }
        return;
    }
    if (init || forced) {
        if (!init && S.done) {
            if (threadIdx.x == 0) { S.items = 0; S.bitems = 0; S.nact = 0; }
            return;
        }
        const int na = init ? n : (int)min((unsigned)n, forced);
        for (int i = threadIdx.x; i < na; i += THREADS) d.move[off + i] = (unsigned)i;
        nact = (unsigned)na;
        itime = init ? 0.0 : S.itime;
        if (init && threadIdx.x == 0) {   // every particle is corrected: its tn enters tmin_stepped
            S.tmin_idle = exact::INF_BITS;
            S.tmin_stepped = exact::INF_BITS;
        }
    } else {
        if (S.done) {
            if (threadIdx.x == 0) { S.items = 0; S.bitems = 0; S.nact = 0; }
            return;
        }
        // Hermite4::next_integration_time (Hermite4.cpp:90-102) for this
        // system: the least t + dt over its particles, as the least bit
        // pattern of the stored tn (t + dt > 0; a NaN pattern sorts above
        // +inf, as fmin ignores NaN): the least over the particles that did
        // not step last time (recorded by the last compaction) and over those
        // corrected since (atomic minimum of the corrector) -- integer work
        // and no scan, where FP64 adds and minima on one SM would take longer
        // than the rest of the phase
        const unsigned long long *tnb = reinterpret_cast<const unsigned long long *>(d.tn + off);
        const double m = exact::bits_to_double(min(S.tmin_idle, S.tmin_stepped));
        // the reference's loop condition, on the last step's block time
        const bool stop = S.err != 0u || !(S.itime < S.t_end);
        if (stop) {
            if (threadIdx.x == 0) { S.atime = m; S.done = 1u; S.items = 0; S.bitems = 0; S.nact = 0; }
            return;
        }
        itime = m;
        // Hermite4::find_particles_to_move (Hermite4.cpp:64-88): the test
        // |itime - tn| < 2^-51 as a window of bit patterns
        unsigned long long wlo = 0, whi = 0;
        const bool window = exact::active_window(itime, wlo, whi);
        // ascending compaction and the least tn of the particles that do not
        // step, in rounds of 8 x 1024 particles: warp w takes the segment
        // [base + 1024 w, + 1024) as 32 rows of 32 (coalesced loads), lane q
        // keeps row q's ballot, a block scan of the eight warp counts places
        // the segments, and each row is written at its running offset
        unsigned long long idle = exact::INF_BITS;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int base = 0; base < n; base += THREADS * 32) {
            const int seg = base + w * 1024;
            unsigned long long b[32];
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const int i = seg + q * 32 + lane;
                b[q] = i < n ? tnb[i] : exact::INF_BITS;
            }
            unsigned row = 0, cnt = 0;
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const int i = seg + q * 32 + lane;
                const bool act = i < n && (window ? b[q] - wlo <= whi - wlo
                                                  : exact::is_active_tn(itime, exact::bits_to_double(b[q])));
                if (!act) idle = min(idle, b[q]);
                const unsigned m = __ballot_sync(0xffffffffu, act);
                if (lane == q) row = m;
                cnt += (unsigned)__popc(m);
            }
            unsigned tot;
            unsigned pos = nact + block_scan_u(lane == 0 ? cnt : 0u, red, &tot);
            pos = __shfl_sync(0xffffffffu, pos, 0);
            if (cnt && !in_range(d, BS_SCATTER, pos, (long long)pos + cnt, n)) row = 0;
            const unsigned lt = (1u << lane) - 1u;
#pragma unroll 4
            for (int q = 0; q < 32; q++) {
                const unsigned m = __shfl_sync(0xffffffffu, row, q);
                if (m & (1u << lane)) d.move[off + pos + (unsigned)__popc(m & lt)] = (unsigned)(seg + q * 32 + lane);
                pos += (unsigned)__popc(m);
            }
            nact += tot;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) idle = min(idle, __shfl_down_sync(0xffffffffu, idle, o));
        unsigned long long *redb = reinterpret_cast<unsigned long long *>(redd);
        if (lane == 0) redb[w] = idle;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 1; k < WARPS; k++) idle = min(idle, redb[k]);
            S.tmin_idle = idle;
            S.tmin_stepped = exact::INF_BITS;
        }
    }
    if (threadIdx.x == 0) {
        if (!forced) S.itime = itime;   // a tuning probe leaves the block time alone
        if (!init && !forced) {
            S.atime = itime;
            S.steps += 1;
            S.psteps += nact;
            S.inter += (unsigned long long)nact * (unsigned long long)n;
        }
        S.nact = nact;
        unsigned ig, chunk, split, jt = JT_MAX, q = 1, bsplit = 0;
        bool block = false;
        if (MODE == H4_FORCE_EXACT) {
            ig = 32; chunk = (unsigned)n; split = 1;
        } else {
            const int t = n_bucket(n) * NB_A + a_bucket(nact);
            if (!init && !forced) {
                atomicAdd(&d.bucket[2 * t], 1ull);
                atomicAdd(&d.bucket[2 * t + 1], (unsigned long long)nact * (unsigned long long)n);
            }
            ig = d.tune_ig[t];
            chunk = d.tune_chunk[t];
            if (MODE == H4_FORCE_MIXED && S.e2 > 0.0 && ig >= BTI_MIN && ig <= BTI_MAX && (ig & (ig - 1)) == 0) {
                // block-tiled items of ig active particles; the j-chunk is a
                // whole number of tiles; the partials (bsplit * q per
                // particle) must fit the system's area, else wider items
                // (fewer j-lanes)
                block = true;
                jt = d.tune_jt[t] == 128u ? 128u : (unsigned)JT_MAX;
                chunk = max(jt, (chunk + jt - 1) / jt * jt);
                const unsigned npad = (unsigned)S.npad;
                for (;;) {
                    q = (unsigned)THREADS / (ig / 2);
                    bsplit = (npad + chunk - 1) / chunk;
                    const unsigned cap = nact ? (unsigned)(S.part_cap / (6ull * nact * q)) : 1u;
                    if (cap >= 1u || ig >= BTI_MAX) {
                        if (bsplit > cap) {
                            bsplit = max(1u, cap);
                            chunk = ((npad + bsplit - 1) / bsplit + jt - 1) / jt * jt;
                            bsplit = (npad + chunk - 1) / chunk;
                        }
                        break;
                    }
                    ig *= 2;
                }
                split = bsplit * q;
            } else {
                // warp items: 1, 2 or 4 particles (FP64); 1, 2 (a packed
                // pair) or 4 (two packed pairs) in the mixed form
                if (ig != 1 && ig != 2 && ig != 4) ig = MODE == H4_FORCE_MIXED ? 2 : 4;
                chunk = max(32u, (chunk + 31u) & ~31u);
                split = ((unsigned)n + chunk - 1) / chunk;
                const unsigned cap = nact ? (unsigned)(S.part_cap / (6ull * nact)) : 1u;
                if (split > cap) {
                    split = max(1u, cap);
                    chunk = (((unsigned)n + split - 1) / split + 31u) & ~31u;
                    split = ((unsigned)n + chunk - 1) / chunk;
                }
            }
        }
        S.ig = ig;
        S.chunk = chunk;
        S.split = split;
        S.jt = jt;
        S.q = q;
        S.bsplit = bsplit;
        S.n_groups = nact ? (nact + ig - 1) / ig : 0;
        if (block) {
            S.bitems = S.n_groups * bsplit;
            S.items = 0;
        } else {
            S.bitems = 0;
            S.items = S.n_groups * split;
        }
    }
    __syncthreads();
}

// ---- phase B (grid-wide): predictor of one particle of a stepping system ----
// The mixed form's corrector predictor: the same Taylor polynomials in FP64,
// evaluated with fused multiply-adds and 1/6 as a multiplication (about half
// the FP64 instructions of the reference-order form, which the FP64 and exact
// forms keep for parity).
__device__ __forceinline__ void predict_fma(double itime, double t, const double *f, const dbl4 &r, const dbl4 &v,
                                            dbl4 &pr, dbl4 &pv) {
    const double dt = itime - t;
    const double dt2c = 0.5 * dt * dt;
    const double dt3c = dt2c * dt * (1.0 / 3.0);
    pr.x = fma(dt3c, f[3], fma(dt2c, f[0], fma(dt, v.x, r.x)));
    pr.y = fma(dt3c, f[4], fma(dt2c, f[1], fma(dt, v.y, r.y)));
    pr.z = fma(dt3c, f[5], fma(dt2c, f[2], fma(dt, v.z, r.z)));
    pr.w = (double)(float)r.w;
    pv.x = fma(dt2c, f[3], fma(dt, f[0], v.x));
    pv.y = fma(dt2c, f[4], fma(dt, f[1], v.y));
    pv.z = fma(dt2c, f[5], fma(dt, f[2], v.z));
    pv.w = 0.0;
}

// Mixed form: the corrected state of particle g in FP32 form, written by the
// corrector for its particles only -- position as a double-single hi/lo pair
// (exact::ds_split), mass, and velocity, acceleration and jerk rounded to
// FP32, in four planes of the cs array:
//   (x_hi, y_hi, z_hi, m) (x_lo, y_lo, z_lo, vx) (vy, vz, ax, ay) (az, jx, jy, jz)
__device__ __forceinline__ void store_cs(const Dev &d, size_t g, const dbl4 &r, const dbl4 &v, const double f[6]) {
    const size_t tp = (size_t)d.total;
    float4 c0, c1;
    exact::ds_split(r.x, c0.x, c1.x);
    exact::ds_split(r.y, c0.y, c1.y);
    exact::ds_split(r.z, c0.z, c1.z);
    c0.w = (float)r.w;
    c1.w = (float)v.x;
    d.cs[g] = c0;
    d.cs[tp + g] = c1;
    d.cs[2 * tp + g] = make_float4((float)v.y, (float)v.z, (float)f[0], (float)f[1]);
    d.cs[3 * tp + g] = make_float4((float)f[2], (float)f[3], (float)f[4], (float)f[5]);
}

// hi + lo + x as a renormalised double-single pair: Knuth's two-sum of hi and
// x, the low parts added, then a fast two-sum (|s| >= |l|).
__device__ __forceinline__ void ds_add(float hi, float lo, float x, float &ohi, float &olo) {
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    const float l = __fadd_rn(lo, e);
    ohi = __fadd_rn(s, l);
    olo = __fsub_rn(l, __fsub_rn(ohi, s));
}

// Mixed form: the j data of particle g at the block time from its FP32-form
// state -- the Taylor terms of the displacement and the velocity in FP32 (the
// step dt = itime - t formed in FP64), the displacement added to the
// double-single position.  The terms carry FP32 rounding relative to the
// displacement since the particle's last step, far below the FP32 error of
// a pair's force, so the predictor needs no FP64 arithmetic: every particle
// of every stepping system goes through it each iteration.
__device__ __forceinline__ void predict_ds(const float4 &c0, const float4 &c1, const float4 &c2, const float4 &c3,
                                           float dt, float4 &a, float4 &b, float4 &c) {
    const float dt2 = 0.5f * dt * dt;
    const float dt3 = dt2 * dt * (1.0f / 3.0f);
    ds_add(c0.x, c1.x, fmaf(dt3, c3.y, fmaf(dt2, c2.z, dt * c1.w)), a.x, b.x);
    ds_add(c0.y, c1.y, fmaf(dt3, c3.z, fmaf(dt2, c2.w, dt * c2.x)), a.y, b.y);
    ds_add(c0.z, c1.z, fmaf(dt3, c3.w, fmaf(dt2, c3.x, dt * c2.y)), a.z, b.z);
    a.w = c0.w;
    b.w = 0.f;
    c = make_float4(fmaf(dt2, c3.y, fmaf(dt, c2.z, c1.w)), fmaf(dt2, c3.z, fmaf(dt, c2.w, c2.x)),
                    fmaf(dt2, c3.w, fmaf(dt, c3.x, c2.y)), 0.f);
}

// Last c with pre[c] <= x, over pre[0..m] (pre[0] = 0, nondecreasing).
__device__ __forceinline__ int find_seg(const unsigned *pre, int m, unsigned x) {
    int lo = 0, hi = m;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pre[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

// Writes particle g's j data (a, b, c: the jf0-jf2 records) in the layouts
// this step's force items of its system read.
__device__ __forceinline__ void store_jdata(const Dev &d, const System &S, size_t g, const float4 &a, const float4 &b,
                                            const float4 &cc) {
    // jf0-jf2 (the warp items' j, every force item's i particles), and the
    // duplicated planes only when this step's force work is block-tiled items
    d.jf0[g] = a;
    d.jf1[g] = b;
    d.jf2[g] = cc;
    if (S.bitems) {
        const size_t tp = (size_t)d.jtotal, gj = (size_t)S.joff + (g - (size_t)S.off);
        d.jd[gj] = make_float4(a.x, a.x, a.y, a.y);
        d.jd[tp + gj] = make_float4(a.z, a.z, a.w, a.w);
        d.jd[2 * tp + gj] = make_float4(b.x, b.x, b.y, b.y);
        d.jd[3 * tp + gj] = make_float4(b.z, b.z, cc.x, cc.x);
        d.jd[4 * tp + gj] = make_float4(cc.y, cc.y, cc.z, cc.z);
    }
}

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

template <int MODE>
__device__ __forceinline__ void predict_one(const Dev &d, const System &S, size_t g, bool from_state) {
    if (MODE != H4_FORCE_MIXED) {
        dbl4 pr, pv;
        if (from_state) {   // Hermite4::init_data predictors (Hermite4.cpp:202-214)
            pr = d.r[g];
            pr.w = (double)(float)pr.w;
            pv = d.v[g];
            pv.w = 0.0;
        } else {
            exact::predict(S.itime, d.t[g], d.f + 6 * g, d.r[g], d.v[g], pr, pv);
        }
        d.pr[g] = pr;
        d.pv[g] = pv;
        return;
    }
    float4 a, b, cc;
    if (from_state) {   // the initial forces or a tuning probe
        dbl4 pr = d.r[g], pv = d.v[g];
        pr.w = (double)(float)pr.w;
        exact::pack_jf(pr, pv, a, b, cc);
    } else {
        const size_t tp = (size_t)d.total;
        predict_ds(d.cs[g], d.cs[tp + g], d.cs[2 * tp + g], d.cs[3 * tp + g],
                   __double2float_rn(exact::sub(S.itime, d.t[g])), a, b, cc);
    }
    store_jdata(d, S, g, a, b, cc);
}


// ---- P1 (mixed form): one block-tiled item --------------------------------------
// S.ig active particles (P = S.ig / 2 packed pairs, one per thread of each of
// the Q = S.q j-lanes) against one j-chunk of the system's padded j data; the
// chunk streams through shared memory in tiles of JT j, each tile brought in
// by five 1-D bulk copies (TMA, one per plane of the duplicated j data) that
// complete on the stage's `full` mbarrier.  NS stages rotate across the
// block's items; a warp done with a tile arrives on the stage's `empty`
// mbarrier, and thread 0 refills a stage once all warps have released it, so
// the warps of a block may drift apart by up to NS - 1 tiles instead of
// meeting at a barrier after every tile.  j past the system's end are
// zero-mass padding (exact zero terms); needs e2 > 0 (the self term is then
// an exact zero).  Sums as k_force_mixed_tiled_x2: FP32 over runs of at most
// 64 j per thread, Kahan across runs, stored as doubles, j-lane q of chunk s
// as partial s * Q + q.  gt counts the tiles this block has consumed (stage
// gt % NS, phase parity (gt / NS) & 1).  Returns false when a wait timed out
// (the error bit is then set); the block meets at one barrier per item.

// Thread 0: tile t of the item (global tile g of this block) into stage
// g % NS, once every warp has released that stage's previous tile.
template <int JT>
__device__ __forceinline__ bool issue_tile(float4 (*sj)[5][JT_MAX], uint64_t *full, uint64_t *empty, unsigned g,
                                           const float4 *src, size_t jtp, int t) {
    const unsigned b = g % NS;
    if (g >= NS && !tma::wait_bounded(&empty[b], ((g / NS) - 1u) & 1u, WAIT_LIMIT)) return false;
    tma::fence_proxy_async();
    tma::mbar_arrive_expect_tx(&full[b], 5 * JT * (unsigned)sizeof(float4));
#pragma unroll
    for (int pl = 0; pl < 5; pl++)
        tma::load_1d(&sj[b][pl][0], src + pl * jtp + (size_t)t * JT, JT * (unsigned)sizeof(float4), &full[b]);
    return true;
}

template <int JT>
__device__ bool block_item(const Dev &d, const System &S, unsigned local, float4 (*sj)[5][JT_MAX], uint64_t *full,
                           uint64_t *empty, unsigned &gt) {
    using namespace pair;
    const unsigned s = local / S.n_groups;
    const unsigned g = local - s * S.n_groups;
    const unsigned nact = S.nact, P = S.ig / 2, Q = S.q;
    const unsigned p = threadIdx.x & (P - 1), qq = threadIdx.x / P;
    const int jb = (int)(s * S.chunk);
    const int je = min(S.npad, jb + (int)S.chunk);
    const int ntiles = (je - jb) / JT;
    const unsigned kb = g * S.ig, k0 = kb + p, k1 = k0 + P;
    const unsigned *move = d.move + S.off;
    if (kBoundsCheck) {   // block-uniform ranges, then this thread's two particle indices
        const unsigned cnt = min(S.ig, nact - kb);
        if (!__syncthreads_and(
                system_ok(d, S) && in_range(d, BS_ENS_ITEM, 0, nact, S.n) &&
                in_range(d, BS_ENS_ITEM, kb, (long long)kb + cnt, nact) && in_range(d, BS_ENS_ITEM, jb, je, S.npad) &&
                in_range(d, BS_ENS_ITEM, 0, (je - jb) % JT, 1) &&
                in_range(d, BS_ENS_ITEM, (long long)S.joff + jb, (long long)S.joff + je, d.jtotal) &&
                in_range(d, BS_ENS_PART, 6ll * nact * s * Q, 6ll * nact * (s + 1) * Q, (long long)S.part_cap)))
            return true;
        const unsigned i0 = move[min(k0, nact - 1)], i1 = move[min(k1, nact - 1)];
        if (!__syncthreads_and(in_range(d, BS_MOVE, i0, i0 + 1ll, S.n) && in_range(d, BS_MOVE, i1, i1 + 1ll, S.n)))
            return true;
    }
    const float4 *jf0 = d.jf0 + S.off, *jf1 = d.jf1 + S.off, *jf2 = d.jf2 + S.off;
    const IPair ip = pack_pair(load_i(jf0, jf1, jf2, move[min(k0, nact - 1)]),
                               load_i(jf0, jf1, jf2, move[min(k1, nact - 1)]));
    const size_t jtp = (size_t)d.jtotal;
    const float e2f = (float)S.e2;
    const f2 e2 = pk2(e2f, e2f), m3 = pk2(-3.0f, -3.0f);
    f2 Sum[6], Cmp[6];
#pragma unroll
    for (int c = 0; c < 6; c++) { Sum[c] = 0ull; Cmp[c] = 0ull; }
    const float4 *src = d.jd + (size_t)S.joff + jb;
    const unsigned g0 = gt;   // the item's first tile
    bool ok = true;
    if (threadIdx.x == 0)     // the item's first NS tiles
        for (int t = 0; t < (int)NS && t < ntiles && ok; t++) ok = issue_tile<JT>(sj, full, empty, g0 + t, src, jtp, t);
    const int per = JT / (int)Q;          // j per thread per tile
    const int sub = per > 64 ? 64 : per;  // j per FP32 run
    int t = 0;
    for (; t < ntiles && ok; t++) {
        const unsigned gg = g0 + (unsigned)t, b = gg % NS;
        const bool mine = ok && tma::wait_bounded(&full[b], (gg / NS) & 1u, WAIT_LIMIT);
        ok = __all_sync(0xffffffffu, mine);   // warp-uniform (thread 0 also reports its refills)
        if (!ok) break;
        for (int sb = 0; sb < per; sb += sub) {
            f2 part[6];
#pragma unroll
            for (int c = 0; c < 6; c++) part[c] = 0ull;
#pragma unroll 32   // measured: 7.9e11 pairs/s against 7.7e11 (16), 7.5e11 (8) and 7.1e11 (4)
            for (int u = 0; u < sub; u++) {
                const int jj = (int)qq + (sb + u) * (int)Q;
                const f2 *q0 = (const f2 *)&sj[b][0][jj], *q1 = (const f2 *)&sj[b][1][jj],
                         *q2 = (const f2 *)&sj[b][2][jj], *q3 = (const f2 *)&sj[b][3][jj],
                         *q4 = (const f2 *)&sj[b][4][jj];
                pair_x2(ip, q0[0], q0[1], q1[0], q1[1], q2[0], q2[1], q3[0], q3[1], q4[0], q4[1], e2, m3, part);
            }
#pragma unroll
            for (int c = 0; c < 6; c++) kahan2(Sum[c], Cmp[c], part[c]);
        }
        __syncwarp();
        if ((threadIdx.x & 31) == 0) tma::mbar_arrive(&empty[b]);   // this warp is done with stage b
        if (threadIdx.x == 0 && t + (int)NS < ntiles) ok = issue_tile<JT>(sj, full, empty, gg + NS, src, jtp, t + NS);
    }
    // the block meets once per item: every warp has finished (or given up)
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            // copies of this item possibly still in flight: tiles t .. t + NS - 1
            for (int k = t; k < ntiles && k < t + (int)NS; k++)
                tma::wait_bounded(&full[(g0 + k) % NS], ((g0 + k) / NS) & 1u, WAIT_LIMIT);
            atomicOr(d.err, (unsigned)H4_ERRBIT_TIMEOUT);
        }
        return false;
    }
    gt = g0 + (unsigned)ntiles;
    double *part_s = d.part + S.part_off + (size_t)(s * Q + qq) * 6 * nact;
#pragma unroll
    for (int c = 0; c < 6; c++) {
        if (k0 < nact) part_s[(size_t)c * nact + k0] = (double)lo2(Sum[c]) - (double)lo2(Cmp[c]);
        if (k1 < nact) part_s[(size_t)c * nact + k1] = (double)hi2(Sum[c]) - (double)hi2(Cmp[c]);
    }
    return true;
}

// ---- P1 (mixed form, e2 > 0): one warp item through a per-warp TMA ring ------
// The warp item of pair::mixed_warp_item (NI = 1) or mixed_warp_item_x2
// (NI = 2) with its j data brought into shared memory instead of loaded by
// every lane from L2: stages of WARP_STAGE_J consecutive j (three 1-D bulk
// copies, one per plane of jf0/jf1/jf2, issued by lane 0 and completing on
// the stage's mbarrier), WARP_STAGES of them in flight, so the L2 latency is
// hidden behind the pair arithmetic of the stages before.  Lane l takes the
// stage's j l, l + 32, l + 64, l + 96 -- the same j in the same order as the
// L2 form, so the sums are the same.  gw counts the stages this warp has consumed.
// Returns false when a wait timed out (the error bit is then set).
__device__ __forceinline__ void issue_stage(float4 (*ring)[3][WARP_STAGE_J], uint64_t *wfull, unsigned gs,
                                            const float4 *jf0, const float4 *jf1, const float4 *jf2, int j0, int cnt) {
    const unsigned st = gs % WARP_STAGES;
    const unsigned bytes = (unsigned)cnt * (unsigned)sizeof(float4);
    tma::fence_proxy_async();
    tma::mbar_arrive_expect_tx(&wfull[st], 3 * bytes);
    tma::load_1d(&ring[st][0][0], jf0 + j0, bytes, &wfull[st]);
    tma::load_1d(&ring[st][1][0], jf1 + j0, bytes, &wfull[st]);
    tma::load_1d(&ring[st][2][0], jf2 + j0, bytes, &wfull[st]);
}

template <int NI>
__device__ bool ring_warp_item(const Dev &d, const System &S, const unsigned *move, unsigned nact, unsigned k0, int jb,
                               int je, double *part_s, float4 (*ring)[3][WARP_STAGE_J], uint64_t *wfull, unsigned &gw,
                               int lane) {
    using namespace pair;
    const float4 *jf0 = d.jf0 + S.off, *jf1 = d.jf1 + S.off, *jf2 = d.jf2 + S.off;
    const float e2f = (float)S.e2;
    const int nst = (je - jb + WARP_STAGE_J - 1) / WARP_STAGE_J;
    const unsigned gs0 = gw;
    if (lane == 0)
        for (int k = 0; k < WARP_STAGES && k < nst; k++)
            issue_stage(ring, wfull, gs0 + k, jf0, jf1, jf2, jb + k * WARP_STAGE_J,
                        min(WARP_STAGE_J, je - jb - k * WARP_STAGE_J));
    constexpr int RUN = 512 / WARP_STAGE_J;   // stages per FP32 run (16 j per lane)
    IPair ip;
    IParticle i1;
    if (NI == 2)
        ip = pack_pair(load_i(jf0, jf1, jf2, move[k0]), load_i(jf0, jf1, jf2, move[k0 + 1]));
    else
        i1 = load_i(jf0, jf1, jf2, move[k0]);
    const f2 e2 = pk2(e2f, e2f), m3 = pk2(-3.0f, -3.0f);
    f2 Sx[6], Cx[6], px[6];
    float S1[6], C1[6], p1[6];
#pragma unroll
    for (int c = 0; c < 6; c++) { Sx[c] = 0ull; Cx[c] = 0ull; px[c] = 0ull; S1[c] = 0.f; C1[c] = 0.f; p1[c] = 0.f; }
    bool ok = true;
    int k = 0;
    for (; k < nst; k++) {
        const unsigned gs = gs0 + (unsigned)k, st = gs % WARP_STAGES;
        ok = __all_sync(0xffffffffu, tma::wait_bounded(&wfull[st], (gs / WARP_STAGES) & 1u, WAIT_LIMIT));
        if (!ok) break;
        const int j0 = jb + k * WARP_STAGE_J;
#pragma unroll
        for (int h = 0; h < WARP_STAGE_J / 32; h++) {
            const int jj = lane + 32 * h;
            if (j0 + jj < je) {
                const float4 a = ring[st][0][jj], b = ring[st][1][jj], c = ring[st][2][jj];
                if (NI == 2)
                    pair_x2(ip, pk2(a.x, a.x), pk2(a.y, a.y), pk2(a.z, a.z), pk2(a.w, a.w), pk2(b.x, b.x),
                            pk2(b.y, b.y), pk2(b.z, b.z), pk2(c.x, c.x), pk2(c.y, c.y), pk2(c.z, c.z), e2, m3, px);
                else
                    pair_mixed<false>(i1, a, b, c, e2f, false, p1);
            }
        }
        __syncwarp();
        if (lane == 0 && k + WARP_STAGES < nst)
            issue_stage(ring, wfull, gs + WARP_STAGES, jf0, jf1, jf2, j0 + WARP_STAGES * WARP_STAGE_J,
                        min(WARP_STAGE_J, je - j0 - WARP_STAGES * WARP_STAGE_J));
        if ((k % RUN) == RUN - 1 || k == nst - 1) {
#pragma unroll
            for (int c = 0; c < 6; c++) {
                if (NI == 2) { kahan2(Sx[c], Cx[c], px[c]); px[c] = 0ull; }
                else { kahan_add(S1[c], C1[c], p1[c]); p1[c] = 0.f; }
            }
        }
    }
    if (!ok) {
        if (lane == 0) {   // stages possibly still in flight: k .. k + WARP_STAGES - 1
            for (int q = k; q < nst && q < k + WARP_STAGES; q++)
                tma::wait_bounded(&wfull[(gs0 + q) % WARP_STAGES], ((gs0 + q) / WARP_STAGES) & 1u, WAIT_LIMIT);
            atomicOr(d.err, (unsigned)H4_ERRBIT_TIMEOUT);
        }
        return false;
    }
    gw = gs0 + (unsigned)nst;
    // Kahan pairs (value S - C) summed over the lanes in double-single FP32
    constexpr int V = NI == 2 ? 16 : 8;
    float h[V], l[V];
#pragma unroll
    for (int c = 0; c < 6; c++) {
        if (NI == 2) {
            h[2 * c] = lo2(Sx[c]); h[2 * c + 1] = hi2(Sx[c]);
            l[2 * c] = -lo2(Cx[c]); l[2 * c + 1] = -hi2(Cx[c]);
        } else {
            h[c] = S1[c];
            l[c] = -C1[c];
        }
    }
#pragma unroll
    for (int x = 6 * NI; x < V; x++) { h[x] = 0.f; l[x] = 0.f; }
    rs_sum_ds<V, 16>(h, l, lane);
    const int x = rs_index<V>(lane);
    if (rs_first<V>(lane) && x < 6 * NI) part_s[(size_t)(x / NI) * nact + k0 + (x % NI)] = (double)h[0] + (double)l[0];
    return true;
}

// The same for four active particles k0 .. k0 + 3 as two packed pairs: every
// j a lane loads, and the duplication of its values into register pairs, then
// serves both pairs, and every stage wait and refill four particles.  To fit
// the registers, each lane sums its j of the chunk in plain FP32 (chunk / 32
// terms, no runs or Kahan pairs); the lanes' sums are then added in
// double-single as the other items do.
__device__ bool ring_warp_item4(const Dev &d, const System &S, const unsigned *move, unsigned nact, unsigned k0,
                                int jb, int je, double *part_s, float4 (*ring)[3][WARP_STAGE_J], uint64_t *wfull,
                                unsigned &gw, int lane) {
    using namespace pair;
    const float4 *jf0 = d.jf0 + S.off, *jf1 = d.jf1 + S.off, *jf2 = d.jf2 + S.off;
    const float e2f = (float)S.e2;
    const int nst = (je - jb + WARP_STAGE_J - 1) / WARP_STAGE_J;
    const unsigned gs0 = gw;
    if (lane == 0)
        for (int k = 0; k < WARP_STAGES && k < nst; k++)
            issue_stage(ring, wfull, gs0 + k, jf0, jf1, jf2, jb + k * WARP_STAGE_J,
                        min(WARP_STAGE_J, je - jb - k * WARP_STAGE_J));
    const IPair ip0 = pack_pair(load_i(jf0, jf1, jf2, move[k0]), load_i(jf0, jf1, jf2, move[k0 + 1]));
    const IPair ip1 = pack_pair(load_i(jf0, jf1, jf2, move[k0 + 2]), load_i(jf0, jf1, jf2, move[k0 + 3]));
    const f2 e2 = pk2(e2f, e2f), m3 = pk2(-3.0f, -3.0f);
    f2 T0[6], T1[6];
#pragma unroll
    for (int c = 0; c < 6; c++) { T0[c] = 0ull; T1[c] = 0ull; }
    bool ok = true;
    int k = 0;
    for (; k < nst; k++) {
        const unsigned gs = gs0 + (unsigned)k, st = gs % WARP_STAGES;
        ok = __all_sync(0xffffffffu, tma::wait_bounded(&wfull[st], (gs / WARP_STAGES) & 1u, WAIT_LIMIT));
        if (!ok) break;
        const int j0 = jb + k * WARP_STAGE_J;
#pragma unroll
        for (int h = 0; h < WARP_STAGE_J / 32; h++) {
            const int jj = lane + 32 * h;
            if (j0 + jj < je) {
                const float4 a = ring[st][0][jj], b = ring[st][1][jj], c = ring[st][2][jj];
                const f2 xh = pk2(a.x, a.x), yh = pk2(a.y, a.y), zh = pk2(a.z, a.z), m = pk2(a.w, a.w);
                const f2 xl = pk2(b.x, b.x), yl = pk2(b.y, b.y), zl = pk2(b.z, b.z);
                const f2 vx = pk2(c.x, c.x), vy = pk2(c.y, c.y), vz = pk2(c.z, c.z);
                pair_x2(ip0, xh, yh, zh, m, xl, yl, zl, vx, vy, vz, e2, m3, T0);
                pair_x2(ip1, xh, yh, zh, m, xl, yl, zl, vx, vy, vz, e2, m3, T1);
            }
        }
        __syncwarp();
        if (lane == 0 && k + WARP_STAGES < nst)
            issue_stage(ring, wfull, gs + WARP_STAGES, jf0, jf1, jf2, j0 + WARP_STAGES * WARP_STAGE_J,
                        min(WARP_STAGE_J, je - j0 - WARP_STAGES * WARP_STAGE_J));
    }
    if (!ok) {
        if (lane == 0) {   // stages possibly still in flight: k .. k + WARP_STAGES - 1
            for (int q = k; q < nst && q < k + WARP_STAGES; q++)
                tma::wait_bounded(&wfull[(gs0 + q) % WARP_STAGES], ((gs0 + q) / WARP_STAGES) & 1u, WAIT_LIMIT);
            atomicOr(d.err, (unsigned)H4_ERRBIT_TIMEOUT);
        }
        return false;
    }
    gw = gs0 + (unsigned)nst;
    // the lanes' totals summed in double-single FP32, three components at a
    // time: value 4c' + q is component 3 half + c' of particle k0 + q
    constexpr int V = 16;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        float h[V], l[V];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int cc = 3 * half + c;
            h[4 * c] = lo2(T0[cc]); h[4 * c + 1] = hi2(T0[cc]);
            h[4 * c + 2] = lo2(T1[cc]); h[4 * c + 3] = hi2(T1[cc]);
        }
#pragma unroll
        for (int x = 0; x < V; x++) {
            l[x] = 0.f;
            if (x >= 12) h[x] = 0.f;
        }
        rs_sum_ds<V, 16>(h, l, lane);
        const int x = rs_index<V>(lane);
        if (rs_first<V>(lane) && x < 12)
            part_s[(size_t)(3 * half + x / 4) * nact + k0 + (x % 4)] = (double)h[0] + (double)l[0];
    }
    return true;
}

// ---- P1: one warp item of some system's force sum ---------------------------
template <int MODE>
__device__ bool force_item(const Dev &d, const System &S, unsigned local, int lane, float4 (*ring)[3][WARP_STAGE_J],
                           uint64_t *wfull, unsigned &gw) {
    const unsigned s = local / S.n_groups;
    const unsigned g = local - s * S.n_groups;
    const int off = S.off;
    const int jb = (int)(s * S.chunk);
    const int je = min(S.n, jb + (int)S.chunk);
    const unsigned nact = S.nact;
    double *part_s = d.part + S.part_off + (size_t)s * 6 * nact;
    const unsigned *move = d.move + off;
    if (MODE == H4_FORCE_EXACT) {
        const unsigned k = g * 32 + lane;
        const unsigned cnt = min(32u, nact - g * 32);
        if (kBoundsCheck && !__all_sync(0xffffffffu, item_ok(d, S, s, g * 32, cnt, 0, S.n, (unsigned)lane))) return true;
        if (k < nact) {
            double f[6];
            pair::exact_sum(d.pr + off, d.pv + off, S.n, move[k], S.e2, f);
#pragma unroll
            for (int c = 0; c < 6; c++) part_s[(size_t)c * nact + k] = f[c];
        }
        return true;
    }
    const unsigned k0 = g * S.ig;
    const unsigned cnt = min(S.ig, nact - k0);
    if (kBoundsCheck && !__all_sync(0xffffffffu, item_ok(d, S, s, k0, cnt, jb, je, (unsigned)lane))) return true;
    if (MODE == H4_FORCE_FP64) {
        const dbl4 *pr = d.pr + off, *pv = d.pv + off;
        if (cnt == 4) {
            pair::fp64_warp_item<4>(pr, pv, move, nact, k0, jb, je, S.e2, part_s, lane);
        } else {
            unsigned k = k0;
            if (cnt >= 2) { pair::fp64_warp_item<2>(pr, pv, move, nact, k, jb, je, S.e2, part_s, lane); k += 2; }
            if (cnt & 1) pair::fp64_warp_item<1>(pr, pv, move, nact, k, jb, je, S.e2, part_s, lane);
        }
    } else {
        const float4 *a = d.jf0 + off, *b = d.jf1 + off, *c = d.jf2 + off;
        const float e2 = (float)S.e2;
        if (S.e2 > 0.0)   // a packed pair, or one particle, j through the warp's ring
        {   // four particles (two packed pairs), a packed pair, or one; j through the warp's ring
            if (cnt == 4) return ring_warp_item4(d, S, move, nact, k0, jb, je, part_s, ring, wfull, gw, lane);
            unsigned k = k0;
            if (cnt >= 2) {
                if (!ring_warp_item<2>(d, S, move, nact, k, jb, je, part_s, ring, wfull, gw, lane)) return false;
                k += 2;
            }
            if (cnt & 1) return ring_warp_item<1>(d, S, move, nact, k, jb, je, part_s, ring, wfull, gw, lane);
            return true;
        }
        {   // e2 = 0: the self term masked, j from L2
            unsigned k = k0;
            while (k < k0 + cnt) {
                pair::mixed_warp_item<1, true>(a, b, c, move, nact, k, jb, je, e2, part_s, lane);
                k++;
            }
        }
    }
    return true;
}

// ---- phase D (grid-wide): reduction, corrector and timestep of one active
// particle (init: forces and the initial timestep) -----------------------------
// Bounds-checked build: the ranges the reduction and corrector of active
// particle k of system S touch.
__device__ __forceinline__ bool correct_ok(const Dev &d, const System &S, unsigned k) {
    if (!kBoundsCheck) return true;
    if (!(system_ok(d, S) && in_range(d, BS_ENS_ITEM, k, k + 1ll, S.nact) &&
          in_range(d, BS_ENS_PART, 0, 6ll * S.nact * S.split, (long long)S.part_cap)))
        return false;
    const unsigned i = d.move[S.off + k];
    return in_range(d, BS_MOVE, i, i + 1ll, S.n);
}

// Mixed form's corrector: the quantities of Hermite4CPU::correction_pos_vel
// (Hermite4CPU.cpp:370-411), NbodyUtils::get_timestep_normal
// (NbodyUtils.cpp:337-365) and NbodyUtils::normalize_dt (NbodyUtils.cpp:371-
// 424) as exact::correct forms them, evaluated with fused multiply-adds and
// reciprocal powers of dt, and the timestep test on the square of the
// criterion, q = eta (|a| |a2| + |j|^2) / (|j| |a3| + |a2|^2), against the
// squares of the candidate steps: q in FP32 where its inputs allow (the
// quantised step then differs from an FP64 q only within FP32 rounding of a
// power-of-two boundary), else two FP64 square roots and one division, where
// the reference order takes five and one.  A NaN q fails every test, as a NaN
// step does in the reference (the old step is kept).
__device__ __forceinline__ double normalize_dt_sq(double q, double old_dt, double t, double dt_min, double dt_max) {
    const double s1 = old_dt * old_dt;   // squares of old_dt / 8, / 4, / 2, x 1, x 2
    const double s8 = s1 * 0.015625, s4 = s1 * 0.0625, s2 = s1 * 0.25, s2x = s1 * 4.0;
    double nd;
    if (q <= s8) {
        nd = exact::D_TIME_MIN_REF;
    } else if (s8 < q && q <= s4) {
        nd = old_dt * 0.125;
    } else if (s4 < q && q <= s2) {
        nd = old_dt * 0.25;
    } else if (s2 < q && q <= s1) {
        nd = old_dt * 0.5;
    } else if (s1 < q && q <= s2x) {
        nd = old_dt;
    } else if (s2x < q) {
        const double o2x = old_dt * 2.0;
        const double val = exact::is_pow2(o2x) ? t * exact::recip_pow2(o2x) : t / o2x;
        nd = (ceil(val) == val) ? o2x : old_dt;
    } else {
        nd = old_dt;
    }
    return nd < dt_min ? dt_min : (nd > dt_max ? dt_max : nd);
}

__device__ __forceinline__ bool correct_mixed(double itime, double eta, double dt_min, double dt_max, const double f[6],
                                              const double o[6], const dbl4 &p, const dbl4 &pv, double dt1, dbl4 &r,
                                              dbl4 &v, double a2[3], double a3[3], double &new_dt) {
    const double dt2 = dt1 * dt1, dt3 = dt2 * dt1, dt4 = dt2 * dt2, dt5 = dt4 * dt1;
    double i2, i3;
    if (exact::is_pow2(dt1) && exact::is_pow2(dt5)) {   // block steps: exact reciprocals
        i2 = exact::recip_pow2(dt2);
        i3 = exact::recip_pow2(dt3);
    } else {
        const double i1 = 1.0 / dt1;
        i2 = i1 * i1;
        i3 = i2 * i1;
    }
    const double dt6 = 6.0 * dt1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const double da = o[c] - f[c];
        a2[c] = fma(-6.0, da, -dt1 * fma(4.0, o[3 + c], 2.0 * f[3 + c])) * i2;
        a3[c] = fma(12.0, da, dt6 * (o[3 + c] + f[3 + c])) * i3;
    }
    const double c24 = dt4 * (1.0 / 24.0), c120 = dt5 * (1.0 / 120.0), c6 = dt3 * (1.0 / 6.0);
    r.x = fma(c120, a3[0], fma(c24, a2[0], p.x));
    r.y = fma(c120, a3[1], fma(c24, a2[1], p.y));
    r.z = fma(c120, a3[2], fma(c24, a2[2], p.z));
    v.x = fma(c24, a3[0], fma(c6, a2[0], pv.x));
    v.y = fma(c24, a3[1], fma(c6, a2[1], pv.y));
    v.z = fma(c24, a3[2], fma(c6, a2[2], pv.z));
    // the criterion at the end of the step: a2 + dt a3
    const double bx = fma(dt1, a3[0], a2[0]), by = fma(dt1, a3[1], a2[1]), bz = fma(dt1, a3[2], a2[2]);
    const double A2 = fma(f[0], f[0], fma(f[1], f[1], f[2] * f[2]));
    const double J2 = fma(f[3], f[3], fma(f[4], f[4], f[5] * f[5]));
    const double B2 = fma(bx, bx, fma(by, by, bz * bz));
    const double C2 = fma(a3[0], a3[0], fma(a3[1], a3[1], a3[2] * a3[2]));
    // the criterion in FP32 where the four squares and their products lie
    // well inside its range (exponents within 2^+-60, tested on the bits),
    // else in FP64
    const auto in_f32 = [](double x) {
        const unsigned e = (unsigned)(exact::double_to_bits(x) >> 52);   // sign 0: x >= 0
        return e >= 1023u - 60u && e <= 1023u + 60u;
    };
    double q;
    if (in_f32(A2) && in_f32(J2) && in_f32(B2) && in_f32(C2)) {
        const float a = (float)A2, j = (float)J2, b = (float)B2, c = (float)C2;
        q = (double)((float)eta * (sqrtf(a * b) + j) / (sqrtf(j * c) + b));
    } else {
        q = eta * (sqrt(A2 * B2) + J2) / (sqrt(J2 * C2) + B2);
    }
    new_dt = normalize_dt_sq(q, dt1, itime, dt_min, dt_max);
    return isfinite(r.x) && isfinite(r.y) && isfinite(r.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
}

// fn: the sum of the particle's partial forces (exact::sum_partials_*).
template <int MODE>
// Returns the bit pattern of the particle's new tn = t + dt.
__device__ __forceinline__ unsigned long long correct_one(const Dev &d, System &S, unsigned k, bool init,
                                                          const double fn[6]) {
    const unsigned i = d.move[S.off + k];
    const size_t g = (size_t)S.off + i;
    double *fp = d.f + 6 * g;
    if (init) {
#pragma unroll
        for (int q = 0; q < 6; q++) fp[q] = fn[q];
        const double dt0 = exact::init_dt(fn, (double)0.01f, S.dt_min, S.dt_max);
        d.dt[g] = dt0;
        d.t[g] = 0.0;
        const double tn0 = exact::add(0.0, dt0);
        d.tn[g] = tn0;
        if (MODE == H4_FORCE_MIXED) store_cs(d, g, d.r[g], d.v[g], fn);
        return exact::double_to_bits(tn0);
    }
    double o[6];   // the old forces (the reference's old_a/old_a1), read before they are replaced
#pragma unroll
    for (int q = 0; q < 6; q++) { o[q] = fp[q]; fp[q] = fn[q]; }
    dbl4 r = d.r[g], v = d.v[g];
    double a2[3], a3[3], ndt;
    dbl4 pr, pv;
    if (MODE == H4_FORCE_MIXED) {   // phase B's predictor of this particle, from the same inputs
        predict_fma(S.itime, d.t[g], o, r, v, pr, pv);
    } else {
        pr = d.pr[g];
        pv = d.pv[g];
    }
    const bool ok = MODE == H4_FORCE_MIXED
                        ? correct_mixed(S.itime, S.eta, S.dt_min, S.dt_max, fn, o, pr, pv, d.dt[g], r, v, a2, a3, ndt)
                        : exact::correct(S.itime, S.eta, S.dt_min, S.dt_max, fn, o, pr, pv, d.dt[g], r, v, a2, a3,
                                         ndt);
    d.r[g] = r;
    d.v[g] = v;
    d.t[g] = S.itime;
    d.dt[g] = ndt;
    const double tn = exact::add(S.itime, ndt);
    d.tn[g] = tn;
    if (MODE == H4_FORCE_MIXED) store_cs(d, g, r, v, fn);
    if (!ok) {
        atomicOr(&S.err, (unsigned)H4_ERRBIT_NONFINITE);
        atomicOr(d.err, (unsigned)H4_ERRBIT_NONFINITE);
    }
    return exact::double_to_bits(tn);
}

// The corrected particles' tn into their systems' tmin_stepped: one atomic
// per warp when its lanes share a system (c < 0: lane without a particle).
// Called by every lane of the warp.
__device__ __forceinline__ void fold_tmin(const Dev &d, int c, unsigned long long tnb) {
    const int c0 = __shfl_sync(0xffffffffu, c, 0);
    if (__all_sync(0xffffffffu, c == c0 || c < 0)) {
        unsigned long long m = c < 0 ? exact::INF_BITS : tnb;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_down_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0 && c0 >= 0) atomicMin(&d.sys[c0].tmin_stepped, m);
    } else if (c >= 0) {
        atomicMin(&d.sys[c].tmin_stepped, tnb);
    }
}

// Phase timer: block 0 reads %globaltimer after every grid barrier and adds
// the time since the previous one to its phase.  A barrier ends when the
// last block reaches it, so this is the phase's duration on the whole GPU.
__device__ __forceinline__ void phase_mark(const Dev &d, int phase, unsigned long long &t_prev) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long t = device_ns();
        d.phase_ns[phase] += t - t_prev;
        t_prev = t;
    }
}

template <int MODE>
__global__ void __launch_bounds__(THREADS, kMinBlocks<MODE>) k_ensemble(Dev d, int iters, int init, int force_only) {
    // dynamic shared memory: the mixed form's tile area (block-item j tiles,
    // or the warps' j rings), then per-system prefix sums, [nsys + 1] each:
    // particle offsets, warp items, block items, and the active particles of
    // the systems whose partials a warp per particle reduces, and of the rest
    extern __shared__ __align__(128) unsigned char s_raw[];
    constexpr size_t tile_area = MODE == H4_FORCE_MIXED ? TILE_AREA_BYTES : 0;
    float4(*sj)[5][JT_MAX] = reinterpret_cast<float4(*)[5][JT_MAX]>(s_raw);
    float4(*ring)[3][WARP_STAGE_J] =
        reinterpret_cast<float4(*)[3][WARP_STAGE_J]>(s_raw + (threadIdx.x >> 5) * WARP_RING_BYTES);
    unsigned *s_dyn = reinterpret_cast<unsigned *>(s_raw + tile_area);
    unsigned *s_off = s_dyn;
    unsigned *s_prefix = s_off + d.nsys + 1;
    unsigned *s_prefix_b = s_prefix + d.nsys + 1;
    unsigned *s_actw = s_prefix_b + d.nsys + 1;
    unsigned *s_actt = s_actw + d.nsys + 1;
    __shared__ unsigned red[WARPS];
    __shared__ double redd[WARPS];
    __shared__ unsigned s_item[WARPS];
    __shared__ double s_fn[32][6];   // phase D: reduced forces of a group of warp-reduced particles
    __shared__ unsigned s_bitem;
    // barriers of the block-item stages and of the warps' rings
    __shared__ __align__(8) uint64_t s_full[NS], s_empty[NS], s_wfull[WARPS][WARP_STAGES];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned gt = 0;   // block-item tiles consumed by this block
    unsigned gw = 0;   // warp-item stages consumed by this warp
    if (MODE == H4_FORCE_MIXED) {
        if (threadIdx.x == 0) {
            for (unsigned b = 0; b < NS; b++) {
                tma::mbar_init(&s_full[b], 1);
                tma::mbar_init(&s_empty[b], WARPS);
            }
            for (int q = 0; q < WARPS; q++)
                for (int st = 0; st < WARP_STAGES; st++) tma::mbar_init(&s_wfull[q][st], 1);
            tma::mbar_init_fence();
        }
        __syncthreads();
    }
    const bool from_state = init || (*d.forced_nact != 0u);
    const unsigned nthreads = gridDim.x * THREADS;
    const unsigned gtid = blockIdx.x * THREADS + threadIdx.x;
    unsigned long long t_prev = (blockIdx.x == 0 && threadIdx.x == 0) ? device_ns() : 0ull;
    for (int it = 0; it < iters; it++) {
        // A: per system
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *d.queue = 0u;
            *d.queue_b = 0u;
            __threadfence();
        }
        for (int c = blockIdx.x; c < d.nsys; c += gridDim.x) phaseA<MODE>(d, c, init != 0, red, redd);
        if (!grid_sync(d)) return;
        phase_mark(d, 0, t_prev);
        // prefix sums of the systems' counts
        unsigned c_off = 0, c_w = 0, c_b = 0, c_aw = 0, c_at = 0;
        for (int base = 0; base < d.nsys; base += THREADS) {
            const int c = base + threadIdx.x;
            const bool v = c < d.nsys;
            const unsigned x_off = v ? (unsigned)d.sys[c].n : 0u;
            const unsigned x_w = v ? d.sys[c].items : 0u;
            const unsigned x_b = v ? d.sys[c].bitems : 0u;
            const unsigned x_a = v ? d.sys[c].nact : 0u;
            const unsigned x_aw = (v && warp_reduce(d.sys[c].split)) ? x_a : 0u;
            unsigned t0, t1, t2, t3, t4;
            const unsigned e0 = block_scan_u(x_off, red, &t0);
            const unsigned e1 = block_scan_u(x_w, red, &t1);
            const unsigned e2 = block_scan_u(x_b, red, &t2);
            const unsigned e3 = block_scan_u(x_aw, red, &t3);
            const unsigned e4 = block_scan_u(x_a - x_aw, red, &t4);
            if (v) {
                s_off[c] = c_off + e0;
                s_prefix[c] = c_w + e1;
                s_prefix_b[c] = c_b + e2;
                s_actw[c] = c_aw + e3;
                s_actt[c] = c_at + e4;
            }
            c_off += t0; c_w += t1; c_b += t2; c_aw += t3; c_at += t4;
        }
        if (threadIdx.x == 0) {
            s_off[d.nsys] = c_off; s_prefix[d.nsys] = c_w; s_prefix_b[d.nsys] = c_b;
            s_actw[d.nsys] = c_aw; s_actt[d.nsys] = c_at;
        }
        __syncthreads();
        // B: predictor of every particle of the systems taking a step (the
        // mixed form's inputs of a thread's next particle prefetched into L2
        // meanwhile: its chain of loads would otherwise wait out the latency)
        for (unsigned g = gtid; g < (unsigned)d.total; g += nthreads) {
            if (MODE == H4_FORCE_MIXED && !from_state && g + nthreads < (unsigned)d.total) {
                const size_t gn = (size_t)g + nthreads, tp = (size_t)d.total;
                prefetch_l2(d.cs + gn);
                prefetch_l2(d.cs + tp + gn);
                prefetch_l2(d.cs + 2 * tp + gn);
                prefetch_l2(d.cs + 3 * tp + gn);
                prefetch_l2(d.t + gn);
            }
            const int c = find_seg(s_off, d.nsys, g);
            const System &S = d.sys[c];
            if (S.nact == 0u) continue;
            predict_one<MODE>(d, S, g, from_state);
        }
        if (!grid_sync(d)) return;
        phase_mark(d, 1, t_prev);
        // C: force sums
        bool tiles_ok = true;
        if constexpr (MODE == H4_FORCE_MIXED) {
            const unsigned total_b = c_b;
            for (;;) {
                if (threadIdx.x == 0) s_bitem = atomicAdd(d.queue_b, 1u);
                __syncthreads();
                const unsigned item = s_bitem;
                __syncthreads();
                if (item >= total_b) break;
                const int c = find_seg(s_prefix_b, d.nsys, item);
                const System &S = d.sys[c];
                tiles_ok = S.jt == 128u ? block_item<128>(d, S, item - s_prefix_b[c], sj, s_full, s_empty, gt)
                                        : block_item<JT_MAX>(d, S, item - s_prefix_b[c], sj, s_full, s_empty, gt);
                if (!tiles_ok) break;   // a tile wait timed out: straight to the barrier, which fails
            }
        }
        const unsigned total = tiles_ok ? c_w : 0u;
        for (;;) {
            if (lane == 0) s_item[w] = atomicAdd(d.queue, 1u);
            __syncwarp();
            const unsigned item = s_item[w];
            __syncwarp();
            if (item >= total) break;
            const int c = find_seg(s_prefix, d.nsys, item);
            if (!force_item<MODE>(d, d.sys[c], item - s_prefix[c], lane, ring, s_wfull[w], gw))
                break;   // a stage wait timed out: straight to the barrier, which fails
        }
        if (!grid_sync(d)) return;
        phase_mark(d, 2, t_prev);
        if (force_only) return;
        // D: corrector of every active particle; the partial forces of
        // systems with many j-chunks are summed by a warp per particle
        // (lane 0 corrects), the others by a thread per particle
        // (groups of 32 particles per block: each warp reduces four into
        // shared memory, then one warp corrects the 32 with every lane busy
        // -- an FP64 corrector on one lane of a warp takes the FP64 pipe as
        // long as a full warp)
        // (groups taken from the last block down: the thread path below
        // gives particle a to thread a, so when the active particles do not
        // fill the grid the last blocks have none, and the groups then run
        // beside the thread path instead of after it on the same blocks)
        for (unsigned grp = gridDim.x - 1u - blockIdx.x; grp * 32u < c_aw; grp += gridDim.x) {
            for (unsigned q = (unsigned)w; q < 32u; q += WARPS) {
                const unsigned a = grp * 32u + q;
                if (a >= c_aw) break;
                const int c = find_seg(s_actw, d.nsys, a);
                const System &S = d.sys[c];
                const unsigned k = a - s_actw[c];
                if (!__all_sync(0xffffffffu, correct_ok(d, S, k))) continue;
                double fn[6];
                exact::sum_partials_warp(d.part + S.part_off, S.nact, k, S.split, lane, fn);
                if (lane == 0)
#pragma unroll
                    for (int x = 0; x < 6; x++) s_fn[q][x] = fn[x];
            }
            __syncthreads();
            if (w == 0) {
                const unsigned a = grp * 32u + (unsigned)lane;
                int cs = -1;
                unsigned long long tnb = exact::INF_BITS;
                if (a < c_aw) {
                    const int c = find_seg(s_actw, d.nsys, a);
                    System &S = d.sys[c];
                    const unsigned k = a - s_actw[c];
                    if (correct_ok(d, S, k)) {
                        tnb = correct_one<MODE>(d, S, k, init != 0, s_fn[lane]);
                        cs = c;
                    }
                }
                fold_tmin(d, cs, tnb);
            }
            __syncthreads();
        }
        // (warp-uniform trip count, for fold_tmin)
        for (unsigned a0 = gtid - (unsigned)lane; a0 < c_at; a0 += nthreads) {
            const unsigned a = a0 + (unsigned)lane;
            int cs = -1;
            unsigned long long tnb = exact::INF_BITS;
            if (a < c_at) {
                const int c = find_seg(s_actt, d.nsys, a);
                System &S = d.sys[c];
                const unsigned k = a - s_actt[c];
                if (correct_ok(d, S, k)) {
                    double fn[6];
                    exact::sum_partials_thread(d.part + S.part_off, S.nact, k, S.split, fn);
                    tnb = correct_one<MODE>(d, S, k, init != 0, fn);
                    cs = c;
                }
            }
            fold_tmin(d, cs, tnb);
        }
        if (!grid_sync(d)) return;
        phase_mark(d, 3, t_prev);
        if (init) {
            // Hermite4::init_dt's CTIME and the first loop condition
            for (int c = blockIdx.x; c < d.nsys; c += gridDim.x) {
                System &S = d.sys[c];
                double m = __longlong_as_double((long long)exact::INF_BITS);
                for (int i = threadIdx.x; i < S.n; i += THREADS) m = fmin(m, d.dt[S.off + i]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
                __syncthreads();
                if (lane == 0) redd[w] = m;
                __syncthreads();
                if (threadIdx.x == 0) {
                    for (int k = 1; k < WARPS; k++) m = fmin(m, redd[k]);
                    S.atime = m;
                    S.itime = 0.0;
                    S.done = (0.0 < S.t_end) ? 0u : 1u;
                }
                __syncthreads();
            }
        }
    }
}

// Padding of every system's block-item j data past its n (to npad): zero
// mass, far away, at rest -- each such j contributes exactly zero.  Written
// once at creation; the predictor writes only the first n entries.
__global__ void k_ens_pad_jd(Dev d) {
    const size_t tp = (size_t)d.jtotal;
    for (int c = blockIdx.x; c < d.nsys; c += gridDim.x) {
        const System &S = d.sys[c];
        for (int i = S.n + (int)threadIdx.x; i < S.npad; i += blockDim.x) {
            const size_t gj = (size_t)S.joff + i;
            d.jd[gj] = make_float4(1.0e15f, 1.0e15f, 1.0e15f, 1.0e15f);
            d.jd[tp + gj] = make_float4(1.0e15f, 1.0e15f, 0.f, 0.f);
            d.jd[2 * tp + gj] = make_float4(0.f, 0.f, 0.f, 0.f);
            d.jd[3 * tp + gj] = make_float4(0.f, 0.f, 0.f, 0.f);
            d.jd[4 * tp + gj] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// Loop condition of the graph: continue while a system is unfinished, no
// error was recorded and the launch bound is not reached.
__global__ void k_ens_check(Dev d, cudaGraphConditionalHandle cond) {
    __shared__ unsigned any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < d.nsys; c += blockDim.x)
        if (!d.sys[c].done) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long l = ++*d.launches;
        // a system that went non-finite stops alone (phase A); a timed-out
        // barrier or the launch bound stops everything
        unsigned go = any && ((*d.err & (H4_ERRBIT_TIMEOUT | H4_ERRBIT_STEPCAP)) == 0u);
        if (go && l >= d.max_launches) {
            atomicOr(d.err, (unsigned)H4_ERRBIT_STEPCAP);
            go = 0;
        }
        cudaGraphSetConditional(cond, go);
    }
}

// Energy of every system: ring pairing (as h4_energy.cu) over warp items of
// 4 particles, then a fixed-order sum per system (one block per system).
__global__ void __launch_bounds__(THREADS) k_ens_energy_pairs(Dev d) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
    const int nw = gridDim.x * WARPS;
    int item = gw;
    for (int c = 0; c < d.nsys; c++) {
        const System &S = d.sys[c];
        const int n = S.n, off = S.off;
        const int groups = (n + 3) / 4;
        for (; item < groups; item += nw) {
            const int i0 = item * 4;
            const int half = n / 2;
            const bool even = (n % 2) == 0;
            double acc[4];
            int ie[4];
            double xi[4], yi[4], zi[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                ie[q] = min(i0 + q, n - 1);
                const dbl4 r = d.r[off + ie[q]];
                xi[q] = r.x; yi[q] = r.y; zi[q] = r.z;
                acc[q] = 0.0;
            }
            for (int o = 1 + lane; o <= half; o += 32) {
                const double wgt = (even && o == half) ? 0.5 : 1.0;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    int j = ie[q] + o;
                    if (j >= n) j -= n;
                    const dbl4 rj = d.r[off + j];
                    const double dx = rj.x - xi[q], dy = rj.y - yi[q], dz = rj.z - zi[q];
                    acc[q] = fma(wgt * rj.w, pair::rsqrt_refined(fma(dx, dx, fma(dy, dy, dz * dz))), acc[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                double a = acc[q];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
                if (lane == 0 && i0 + q < n) d.epot_i[off + i0 + q] = n > 1 ? -a * d.r[off + i0 + q].w : 0.0;
            }
        }
        item -= groups;
    }
}

__global__ void __launch_bounds__(THREADS) k_ens_energy_sum(Dev d) {
    __shared__ double sk[THREADS], sp[THREADS];
    for (int c = blockIdx.x; c < d.nsys; c += gridDim.x) {
        const System &S = d.sys[c];
        double ek = 0.0, ep = 0.0;
        for (int i = threadIdx.x; i < S.n; i += THREADS) {
            const dbl4 v = d.v[S.off + i];
            ek += 0.5 * d.r[S.off + i].w * (v.x * v.x + v.y * v.y + v.z * v.z);
            ep += d.epot_i[S.off + i];
        }
        sk[threadIdx.x] = ek;
        sp[threadIdx.x] = ep;
        __syncthreads();
        for (int s = THREADS / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) {
                sk[threadIdx.x] += sk[threadIdx.x + s];
                sp[threadIdx.x] += sp[threadIdx.x + s];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            d.energy[2 * c] = sk[0];
            d.energy[2 * c + 1] = sp[0];
        }
        __syncthreads();
    }
}

}  // namespace ens
}  // namespace h4

// ============================== host side =====================================
using namespace h4;
using namespace h4::ens;

namespace {
thread_local std::string g_ens_err;
int efail(int st, const std::string &m) {
    g_ens_err = m;
    return st;
}
int ecuda(cudaError_t e, const char *what) {
    g_ens_err = std::string(what) + ": " + cudaGetErrorString(e);
    return H4_ERR_CUDA;
}
#define ENS_TRY(call, what)                        \
    do {                                           \
        cudaError_t e__ = (call);                  \
        if (e__ != cudaSuccess) return ecuda(e__, what); \
    } while (0)
}  // namespace

struct h4_ensemble_s {
    Dev d{};
    int nsys = 0, total = 0, mode = 0, num_sms = 0, grid = 0;
    size_t smem = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    std::vector<System> host_sys;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float last_ms = 0.f;
    unsigned long long launches = 0;
    bool initialised = false;
    std::vector<void *> allocs;
};

namespace {

template <int MODE>
const void *ens_kernel() { return (const void *)k_ensemble<MODE>; }

const void *kernel_for(int mode) {
    switch (mode) {
    case H4_FORCE_EXACT: return ens_kernel<H4_FORCE_EXACT>();
    case H4_FORCE_MIXED: return ens_kernel<H4_FORCE_MIXED>();
    default: return ens_kernel<H4_FORCE_FP64>();
    }
}

cudaError_t launch_persistent(h4_ensemble_s *E, cudaStream_t s, int iters, int init, int force_only) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)E->grid);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = E->smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {(void *)&E->d, (void *)&iters, (void *)&init, (void *)&force_only};
    return cudaLaunchKernelExC(&cfg, kernel_for(E->mode), args);
}

template <typename T>
cudaError_t dalloc(h4_ensemble_s *E, T **p, size_t count) {
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) E->allocs.push_back((void *)*p);
    return e;
}

void ens_free(h4_ensemble_s *E) {
    if (E->exec) cudaGraphExecDestroy(E->exec);
    if (E->graph) cudaGraphDestroy(E->graph);
    if (E->cap) cudaStreamDestroy(E->cap);
    if (E->e0) cudaEventDestroy(E->e0);
    if (E->e1) cudaEventDestroy(E->e1);
    for (void *p : E->allocs) cudaFree(p);
    if (E->own) cudaStreamDestroy(E->own);
}

// Default tuning table (used until a tuned table is loaded).  FP64: up to 4
// particles per warp item; j-chunks short for small active sets (more
// items), the whole system for large ones.  Mixed: warp items of two packed
// pairs below 1024 active particles (one pair below 4) against 1024-j chunks
// (128 for the smallest steps), block-tiled items of 512 particles above,
// 1024 j per block item (many items per step: in an ensemble few systems
// take a large step in the same iteration), tiles of 256.
void default_tuning(int mode, unsigned *ig, unsigned *chunk, unsigned *jt) {
    static const unsigned ch[NB_A] = {128, 128, 256, 512, 1024, 2048, 4096, 8192};
    static const unsigned mixed_ig[NB_A] = {1, 2, 4, 4, 4, 4, 512, 512};
    static const unsigned mixed_ch[NB_A] = {128, 128, 1024, 1024, 1024, 1024, 1024, 1024};
    for (int b = 0; b < NB_N; b++) {
        for (int a = 0; a < NB_A; a++) {
            const int t = b * NB_A + a;
            jt[t] = JT_MAX;
            if (mode == H4_FORCE_MIXED) {
                ig[t] = mixed_ig[a];
                chunk[t] = mixed_ch[a];
            } else {
                ig[t] = 4;
                chunk[t] = ch[a];
            }
        }
    }
}

// Partial-force area of a system of n particles (doubles): room for
// `splits` j-chunks of every particle, so that a step with all particles
// active still splits into enough items to fill the GPU (a block step of one
// large system often runs with few other systems stepping), and for 4096
// partials beyond that for the many-chunk splits of small active sets.
// splits = 16, fewer for ensembles of more than 2^22 particles (about 0.8 GB
// of partials at 2^22; at least one chunk per particle).
size_t part_splits_for(size_t total) {
    const size_t s = ((size_t)1 << 26) / (total ? total : 1);
    return s < 1 ? 1 : (s > 16 ? 16 : s);
}
size_t part_cap_for(unsigned n, size_t splits) { return 6 * (splits * (size_t)n + 4096); }

// Checks a tuning table for the ensemble's force mode (see h4_ens_set_tuning).
bool tuning_valid(int mode, const unsigned *ig, const unsigned *chunk, const unsigned *jt) {
    for (int t = 0; t < NB_N * NB_A; t++) {
        const bool warp = ig[t] == 1 || ig[t] == 2 || ig[t] == 4;
        const bool block = mode == H4_FORCE_MIXED && ig[t] >= BTI_MIN && ig[t] <= BTI_MAX && (ig[t] & (ig[t] - 1)) == 0;
        if (!(warp || block) || chunk[t] < 32 || chunk[t] > (1u << 24)) return false;
        if (jt && jt[t] != 128 && jt[t] != 256) return false;
    }
    return true;
}

int build_ens_graph(h4_ensemble_s *E) {
    if (E->exec) return H4_OK;
    if (!E->cap) ENS_TRY(cudaStreamCreateWithFlags(&E->cap, cudaStreamNonBlocking), "ensemble capture stream");
    ENS_TRY(cudaGraphCreate(&E->graph, 0), "cudaGraphCreate");
    cudaGraphConditionalHandle cond;
    ENS_TRY(cudaGraphConditionalHandleCreate(&cond, E->graph, 1u, cudaGraphCondAssignDefault), "conditional handle");
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    ENS_TRY(cudaGraphAddNode(&node, E->graph, nullptr, nullptr, 0, &cp), "while node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    ENS_TRY(cudaStreamBeginCaptureToGraph(E->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
            "begin capture");
    cudaError_t e = launch_persistent(E, E->cap, ITERS_PER_LAUNCH, 0, 0);
    if (e == cudaSuccess) {
        k_ens_check<<<1, 256, 0, E->cap>>>(E->d, cond);
        e = cudaGetLastError();
    }
    cudaGraph_t out = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(E->cap, &out);
    if (e != cudaSuccess) return ecuda(e, "capture ensemble step");
    if (e2 != cudaSuccess) return ecuda(e2, "end capture");
    ENS_TRY(cudaGraphInstantiate(&E->exec, E->graph, 0), "instantiate ensemble graph");
    return H4_OK;
}

int pull_systems(h4_ensemble_s *E) {
    ENS_TRY(cudaMemcpyAsync(E->host_sys.data(), E->d.sys, sizeof(System) * E->nsys, cudaMemcpyDeviceToHost,
                            E->stream),
            "copy systems");
    ENS_TRY(cudaStreamSynchronize(E->stream), "synchronize");
    return H4_OK;
}

}  // namespace

extern "C" {

const char *h4_ens_last_error(void) { return g_ens_err.c_str(); }

int h4_ens_create(h4_ens_handle *out, unsigned int nsys, const unsigned int *n, const double *e2, const float *eta,
                  const h4_double4 *r, const h4_double4 *v, int mode) {
    if (!out) return efail(H4_ERR_ARG, "h4_ens_create: out is NULL");
    *out = nullptr;
    if (nsys < 1 || nsys > MAX_SYSTEMS) return efail(H4_ERR_ARG, "h4_ens_create: nsys must be in [1, 4096]");
    if (!n || !e2 || !eta || !r || !v) return efail(H4_ERR_ARG, "h4_ens_create: null array");
    if (mode < H4_FORCE_FP64 || mode > H4_FORCE_MIXED) return efail(H4_ERR_ARG, "h4_ens_create: unknown mode");
    size_t total = 0, part_total = 0;
    for (unsigned c = 0; c < nsys; c++) {
        if (n[c] < 1 || n[c] > (1u << 24)) return efail(H4_ERR_ARG, "h4_ens_create: system size out of range");
        if (!(e2[c] >= 0.0) || !(eta[c] > 0.f)) return efail(H4_ERR_ARG, "h4_ens_create: bad e2 or eta");
        total += n[c];
    }
    const size_t splits = part_splits_for(total);
    for (unsigned c = 0; c < nsys; c++) part_total += part_cap_for(n[c], splits);
    if (total > (1u << 28)) return efail(H4_ERR_ARG, "h4_ens_create: too many particles");
    for (size_t i = 0; i < total; i++)
        if (!std::isfinite(r[i].x) || !std::isfinite(r[i].y) || !std::isfinite(r[i].z) || !std::isfinite(r[i].w) ||
            !std::isfinite(v[i].x) || !std::isfinite(v[i].y) || !std::isfinite(v[i].z))
            return efail(H4_ERR_NONFINITE, "h4_ens_create: non-finite input at particle " + std::to_string(i));
    h4_ensemble_s *E = new (std::nothrow) h4_ensemble_s();
    if (!E) return efail(H4_ERR_ALLOC, "h4_ens_create: host allocation");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&E->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { delete E; return ecuda(e, "h4_ens_create: no CUDA device"); }
    E->nsys = (int)nsys;
    E->total = (int)total;
    E->mode = mode;
    Dev &d = E->d;
    d.nsys = (int)nsys;
    d.total = (int)total;
    d.mode = mode;
    E->host_sys.resize(nsys);
    size_t off = 0, poff = 0, joff = 0;
    for (unsigned c = 0; c < nsys; c++) {
        System S{};
        S.off = (int)off;
        S.n = (int)n[c];
        S.joff = (int)joff;
        S.npad = (int)((n[c] + JT_MAX - 1) / JT_MAX * JT_MAX);
        joff += (size_t)S.npad;
        S.e2 = e2[c];
        S.eta = (double)eta[c];
        S.dt_min = 1.1920928955078125e-07;
        S.dt_max = 0.125;
        S.t_end = 0.0;
        S.part_off = poff;
        S.part_cap = part_cap_for(n[c], splits);
        E->host_sys[c] = S;
        off += n[c];
        poff += S.part_cap;
    }
    d.jtotal = (int)joff;
    e = cudaSuccess;
#define EA(p, cnt) if (e == cudaSuccess) e = dalloc(E, &p, cnt)
    EA(d.sys, nsys); EA(d.r, total); EA(d.v, total); EA(d.pr, total); EA(d.pv, total);
    EA(d.f, 6 * total);
    d.part_total = part_total;
    EA(d.t, total); EA(d.dt, total); EA(d.tn, total); EA(d.move, total); EA(d.part, part_total);
    EA(d.queue, 1); EA(d.queue_b, 1); EA(d.bar_count, 1); EA(d.bar_gen, 1); EA(d.err, 2);
    EA(d.tune_ig, NB_N * NB_A); EA(d.tune_chunk, NB_N * NB_A); EA(d.tune_jt, NB_N * NB_A);
    EA(d.bucket, 2 * NB_N * NB_A); EA(d.forced_nact, 1); EA(d.launches, 1);
    EA(d.phase_ns, 4);
    EA(d.epot_i, total); EA(d.energy, 2 * nsys);
    if (mode == H4_FORCE_MIXED) {
        EA(d.jf0, total); EA(d.jf1, total); EA(d.jf2, total); EA(d.jd, 5 * joff); EA(d.cs, 4 * total);
    }
#undef EA
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E->own, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&E->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&E->e1);
    if (e != cudaSuccess) { ens_free(E); delete E; return efail(H4_ERR_ALLOC, std::string("h4_ens_create: ") + cudaGetErrorString(e)); }
    E->stream = E->own;
    cudaStream_t s = E->stream;
    std::vector<h4_double4> rr(r, r + total);
    for (auto &p : rr) p.w = (double)(float)p.w;   // masses are floats in the reference
    std::vector<unsigned> tig(NB_N * NB_A), tch(NB_N * NB_A), tjt(NB_N * NB_A);
    default_tuning(mode, tig.data(), tch.data(), tjt.data());
    e = cudaMemcpy(d.sys, E->host_sys.data(), sizeof(System) * nsys, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.r, rr.data(), sizeof(dbl4) * total, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.v, v, sizeof(dbl4) * total, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.tune_ig, tig.data(), sizeof(unsigned) * tig.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.tune_chunk, tch.data(), sizeof(unsigned) * tch.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.tune_jt, tjt.data(), sizeof(unsigned) * tjt.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.bucket, 0, sizeof(unsigned long long) * 2 * NB_N * NB_A, s);
    if (e == cudaSuccess && mode == H4_FORCE_MIXED) {   // zero-mass padding of the block items' j data
        k_ens_pad_jd<<<std::min(nsys, 4096u), THREADS, 0, s>>>(d);
        e = cudaGetLastError();
    }
    void *zero[] = {d.f, d.t, d.dt, d.tn};
    size_t zb[] = {48 * total, 8 * total, 8 * total, 8 * total};
    for (int k = 0; k < 4 && e == cudaSuccess; k++) e = cudaMemsetAsync(zero[k], 0, zb[k], s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.queue, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.queue_b, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.bar_count, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.bar_gen, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.err, 0, 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.forced_nact, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.launches, 0, 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.phase_ns, 0, 32, s);
    // persistent grid: every block resident (cooperative launch)
    E->smem = (mode == H4_FORCE_MIXED ? TILE_AREA_BYTES : 0) + sizeof(unsigned) * 5 * (nsys + 1);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel_for(mode), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel_for(mode), THREADS, E->smem);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || per_sm < 1) {
        ens_free(E);
        delete E;
        return e != cudaSuccess ? ecuda(e, "h4_ens_create: setup") : efail(H4_ERR_CUDA, "h4_ens_create: kernel does not fit an SM");
    }
    E->grid = E->num_sms * std::min(per_sm, 2);
    *out = E;
    return H4_OK;
}

int h4_ens_destroy(h4_ens_handle E) {
    if (!E) return H4_OK;
    cudaStreamSynchronize(E->stream);
    ens_free(E);
    delete E;
    return H4_OK;
}

int h4_ens_set_stream(h4_ens_handle E, void *stream) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    ENS_TRY(cudaStreamSynchronize(E->stream), "synchronize");
    E->stream = stream ? (cudaStream_t)stream : E->own;
    return H4_OK;
}

int h4_ens_set_tuning(h4_ens_handle E, const unsigned int *ig, const unsigned int *chunk, const unsigned int *jtile) {
    if (!E || !ig || !chunk) return efail(H4_ERR_ARG, "h4_ens_set_tuning: null argument");
    if (!tuning_valid(E->mode, ig, chunk, jtile))
        return efail(H4_ERR_ARG, E->mode == H4_FORCE_MIXED
                                     ? "h4_ens_set_tuning: ig must be 1, 2 or 4 (warp items) or a power of two in "
                                       "[16, 512] (block items), chunk in [32, 2^24], jtile 128 or 256"
                                     : "h4_ens_set_tuning: ig must be 1, 2 or 4 and chunk in [32, 2^24]");
    std::vector<unsigned> jt(NB_N * NB_A, (unsigned)JT_MAX);
    if (jtile) jt.assign(jtile, jtile + NB_N * NB_A);
    ENS_TRY(cudaMemcpyAsync(E->d.tune_ig, ig, sizeof(unsigned) * NB_N * NB_A, cudaMemcpyHostToDevice, E->stream), "tuning");
    ENS_TRY(cudaMemcpyAsync(E->d.tune_chunk, chunk, sizeof(unsigned) * NB_N * NB_A, cudaMemcpyHostToDevice, E->stream), "tuning");
    ENS_TRY(cudaMemcpyAsync(E->d.tune_jt, jt.data(), sizeof(unsigned) * NB_N * NB_A, cudaMemcpyHostToDevice, E->stream),
            "tuning");
    ENS_TRY(cudaStreamSynchronize(E->stream), "tuning");
    return H4_OK;
}

int h4_ens_bucket_stats(h4_ens_handle E, unsigned long long *steps, unsigned long long *inter) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    std::vector<unsigned long long> b(2 * NB_N * NB_A);
    ENS_TRY(cudaMemcpyAsync(b.data(), E->d.bucket, sizeof(unsigned long long) * b.size(), cudaMemcpyDeviceToHost,
                            E->stream), "bucket statistics");
    ENS_TRY(cudaStreamSynchronize(E->stream), "bucket statistics");
    for (int t = 0; t < NB_N * NB_A; t++) {
        if (steps) steps[t] = b[2 * t];
        if (inter) inter[t] = b[2 * t + 1];
    }
    return H4_OK;
}

int h4_ens_set_dt_limits(h4_ens_handle E, double dt_min, double dt_max) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    int ex1, ex2;
    if (!(dt_min > 0) || !(dt_max >= dt_min) || std::frexp(dt_min, &ex1) != 0.5 || std::frexp(dt_max, &ex2) != 0.5)
        return efail(H4_ERR_ARG, "h4_ens_set_dt_limits: powers of two with dt_min <= dt_max");
    int st = pull_systems(E);
    if (st) return st;
    for (auto &S : E->host_sys) { S.dt_min = dt_min; S.dt_max = dt_max; }
    ENS_TRY(cudaMemcpyAsync(E->d.sys, E->host_sys.data(), sizeof(System) * E->nsys, cudaMemcpyHostToDevice, E->stream), "systems");
    ENS_TRY(cudaStreamSynchronize(E->stream), "systems");
    return H4_OK;
}

int h4_ens_init(h4_ens_handle E) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    int st = pull_systems(E);
    if (st) return st;
    for (auto &S : E->host_sys) { S.done = 0; S.t_end = 1.0; S.steps = S.psteps = S.inter = 0; S.err = 0; }
    ENS_TRY(cudaMemcpyAsync(E->d.sys, E->host_sys.data(), sizeof(System) * E->nsys, cudaMemcpyHostToDevice, E->stream), "systems");
    ENS_TRY(launch_persistent(E, E->stream, 1, 1, 0), "h4_ens_init launch");
    E->launches += 1;
    ENS_TRY(cudaStreamSynchronize(E->stream), "h4_ens_init");
    unsigned err = 0;
    ENS_TRY(cudaMemcpy(&err, E->d.err, 4, cudaMemcpyDeviceToHost), "error word");
    if (err) return efail(H4_ERR_CUDA, "h4_ens_init: device error bits " + std::to_string(err));
    E->initialised = true;
    return H4_OK;
}

int h4_ens_advance(h4_ens_handle E, const double *t_end, double stats[4]) {
    if (!E || !t_end) return efail(H4_ERR_ARG, "h4_ens_advance: null argument");
    if (!E->initialised) return efail(H4_ERR_STATE, "h4_ens_advance: call h4_ens_init first");
    int st = pull_systems(E);
    if (st) return st;
    unsigned long long before_steps = 0;
    double span = 0.0, dtmin = 1.0;
    for (int c = 0; c < E->nsys; c++) {
        System &S = E->host_sys[c];
        before_steps += S.steps;
        S.t_end = t_end[c];
        S.done = (S.err || !(S.itime < S.t_end)) ? 1u : 0u;
        if (S.steps == 0) S.done = (S.t_end > 0.0 && !S.err) ? 0u : 1u;
        span = std::max(span, S.t_end - S.itime);
        dtmin = std::min(dtmin, S.dt_min);
    }
    ENS_TRY(cudaMemcpyAsync(E->d.sys, E->host_sys.data(), sizeof(System) * E->nsys, cudaMemcpyHostToDevice, E->stream), "systems");
    // Launch bound: every iteration advances each unfinished system by at
    // least dt_min, so span/dt_min iterations always suffice.
    const double iters = span / dtmin + 16.0;
    E->d.max_launches = (unsigned long long)std::min(iters / ITERS_PER_LAUNCH + 2.0, 1.0e12);
    ENS_TRY(cudaMemsetAsync(E->d.launches, 0, 8, E->stream), "launch counter");
    if (E->exec) { cudaGraphExecDestroy(E->exec); E->exec = nullptr; cudaGraphDestroy(E->graph); E->graph = nullptr; }
    st = build_ens_graph(E);
    if (st) return st;
    cudaEventRecord(E->e0, E->stream);
    ENS_TRY(cudaGraphLaunch(E->exec, E->stream), "ensemble graph launch");
    cudaEventRecord(E->e1, E->stream);
    if ((st = pull_systems(E))) return st;
    cudaEventElapsedTime(&E->last_ms, E->e0, E->e1);
    unsigned long long nl = 0;
    unsigned err = 0;
    ENS_TRY(cudaMemcpy(&nl, E->d.launches, 8, cudaMemcpyDeviceToHost), "launch counter");
    ENS_TRY(cudaMemcpy(&err, E->d.err, 4, cudaMemcpyDeviceToHost), "error word");
    E->launches += 2 * nl;
    unsigned long long steps = 0, ps = 0, inter = 0;
    for (auto &S : E->host_sys) { steps += S.steps; ps += S.psteps; inter += S.inter; }
    if (stats) {
        stats[0] = (double)(steps - before_steps);
        stats[1] = (double)ps;
        stats[2] = (double)inter;
        stats[3] = (double)nl;
    }
    if (err & H4_ERRBIT_BOUNDS) {
        unsigned w[2] = {0, 0};
        ENS_TRY(cudaMemcpy(w, E->d.err, 8, cudaMemcpyDeviceToHost), "error word");
        return efail(H4_ERR_STATE, "h4_ens_advance: bounds check failed at site " + std::to_string(w[1]));
    }
    if (err & H4_ERRBIT_TIMEOUT) return efail(H4_ERR_CUDA, "h4_ens_advance: a grid barrier timed out");
    if (err & H4_ERRBIT_NONFINITE) return efail(H4_ERR_NONFINITE, "h4_ens_advance: non-finite state in a system");
    if (err & H4_ERRBIT_STEPCAP) return efail(H4_ERR_STATE, "h4_ens_advance: launch bound reached");
    return H4_OK;
}

int h4_ens_energy(h4_ens_handle E, double *ekin, double *epot) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    k_ens_energy_pairs<<<E->num_sms * 8, THREADS, 0, E->stream>>>(E->d);
    k_ens_energy_sum<<<std::min(E->nsys, 4096), THREADS, 0, E->stream>>>(E->d);
    E->launches += 2;
    ENS_TRY(cudaGetLastError(), "h4_ens_energy launch");
    std::vector<double> en(2 * (size_t)E->nsys);
    ENS_TRY(cudaMemcpyAsync(en.data(), E->d.energy, sizeof(double) * en.size(), cudaMemcpyDeviceToHost, E->stream), "energy");
    ENS_TRY(cudaStreamSynchronize(E->stream), "energy");
    for (int c = 0; c < E->nsys; c++) {
        if (ekin) ekin[c] = en[2 * c];
        if (epot) epot[c] = en[2 * c + 1];
    }
    return H4_OK;
}

int h4_ens_download(h4_ens_handle E, h4_double4 *r, h4_double4 *v, h4_forces *f, double *t, double *dt) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    const size_t N = E->total;
    cudaStream_t s = E->stream;
    if (r) ENS_TRY(cudaMemcpyAsync(r, E->d.r, 32 * N, cudaMemcpyDeviceToHost, s), "download r");
    if (v) ENS_TRY(cudaMemcpyAsync(v, E->d.v, 32 * N, cudaMemcpyDeviceToHost, s), "download v");
    if (f) ENS_TRY(cudaMemcpyAsync(f, E->d.f, 48 * N, cudaMemcpyDeviceToHost, s), "download f");
    if (t) ENS_TRY(cudaMemcpyAsync(t, E->d.t, 8 * N, cudaMemcpyDeviceToHost, s), "download t");
    if (dt) ENS_TRY(cudaMemcpyAsync(dt, E->d.dt, 8 * N, cudaMemcpyDeviceToHost, s), "download dt");
    ENS_TRY(cudaStreamSynchronize(s), "download");
    return H4_OK;
}

int h4_ens_system_stats(h4_ens_handle E, double *itime, double *atime, unsigned long long *steps,
                        unsigned long long *psteps, unsigned long long *inter) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    int st = pull_systems(E);
    if (st) return st;
    for (int c = 0; c < E->nsys; c++) {
        const System &S = E->host_sys[c];
        if (itime) itime[c] = S.itime;
        if (atime) atime[c] = S.atime;
        if (steps) steps[c] = S.steps;
        if (psteps) psteps[c] = S.psteps;
        if (inter) inter[c] = S.inter;
    }
    return H4_OK;
}

int h4_ens_tune_force(h4_ens_handle E, unsigned int nact, unsigned int ig, unsigned int chunk, unsigned int jtile,
                      float *ms) {
    if (!E || !ms) return efail(H4_ERR_ARG, "null argument");
    if (nact < 1) return efail(H4_ERR_ARG, "nact must be >= 1");
    std::vector<unsigned> tig(NB_N * NB_A, ig), tch(NB_N * NB_A, chunk), tjt(NB_N * NB_A, jtile ? jtile : JT_MAX);
    int st = h4_ens_set_tuning(E, tig.data(), tch.data(), tjt.data());
    if (st) return st;
    if ((st = pull_systems(E))) return st;
    for (auto &S : E->host_sys) S.done = 0;
    ENS_TRY(cudaMemcpyAsync(E->d.sys, E->host_sys.data(), sizeof(System) * E->nsys, cudaMemcpyHostToDevice, E->stream), "systems");
    ENS_TRY(cudaMemcpyAsync(E->d.forced_nact, &nact, 4, cudaMemcpyHostToDevice, E->stream), "forced nact");
    cudaEventRecord(E->e0, E->stream);
    ENS_TRY(launch_persistent(E, E->stream, 1, 0, 1), "tune launch");
    cudaEventRecord(E->e1, E->stream);
    E->launches += 1;
    const unsigned zero = 0;
    ENS_TRY(cudaMemcpyAsync(E->d.forced_nact, &zero, 4, cudaMemcpyHostToDevice, E->stream), "forced nact");
    ENS_TRY(cudaStreamSynchronize(E->stream), "tune");
    cudaEventElapsedTime(ms, E->e0, E->e1);
    unsigned err = 0;
    ENS_TRY(cudaMemcpy(&err, E->d.err, 4, cudaMemcpyDeviceToHost), "error word");
    if (err) return efail(H4_ERR_CUDA, "h4_ens_tune_force: device error bits " + std::to_string(err));
    return H4_OK;
}

int h4_ens_phase_times(h4_ens_handle E, double ms[4]) {
    if (!E || !ms) return efail(H4_ERR_ARG, "h4_ens_phase_times: null argument");
    unsigned long long ns[4];
    ENS_TRY(cudaStreamSynchronize(E->stream), "h4_ens_phase_times");
    ENS_TRY(cudaMemcpy(ns, E->d.phase_ns, sizeof(ns), cudaMemcpyDeviceToHost), "phase timers");
    for (int k = 0; k < 4; k++) ms[k] = ns[k] * 1e-6;
    return H4_OK;
}

int h4_ens_timings(h4_ens_handle E, float *advance_ms, unsigned long long *kernel_launches) {
    if (!E) return efail(H4_ERR_ARG, "null handle");
    if (advance_ms) *advance_ms = E->last_ms;
    if (kernel_launches) *kernel_launches = E->launches;
    return H4_OK;
}

}  // extern "C"
