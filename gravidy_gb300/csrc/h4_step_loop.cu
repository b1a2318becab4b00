// Device-resident block-step loop of one system in a single persistent
// kernel (FP64 and exact forms, small N).
//
// At small N a block step is a handful of tiny passes -- active set, predictor,
// force sum of a few active particles, corrector, next block time -- and the
// launch latency of one kernel per pass sets the step time (Hermite4GPU_
// integration.cpp:81-124 pays six host<->device round trips per step
// instead).  Here one cooperative kernel, one block per SM, runs the steps of
// h4_advance back to back; four grid-wide barriers per step separate
//   P1  predictor of every particle at the block time, active count per
//       chunk, and the minimum of t + dt over the particles that stay inactive;
//   P2  ordered scatter of the active list (ascending i);
//   P3  force sum: the FP64 warp items of k_force_fp64 with the j-split sized
//       for that kernel's launch (so the same items and summation order), or
//       the exact per-particle sum;
//   P4  fused reduction + corrector + new timestep of the active particles,
//       and the minimum of their new t + dt;
// and the last block to reach the fourth barrier does the step's
// bookkeeping (counters, the loop condition) before releasing the others, so
// every block sees the same decision.  The arithmetic of every phase is that
// of the multi-kernel step (h4_step_kernels.cu, h4_force_fp64.cu), so the
// results are bit-identical to it.  Every barrier wait is bounded in time
// (H4_ERRBIT_TIMEOUT, then every block leaves, and the while-loop condition is
// cleared so the graph stops); after max_iters steps, or when the loop
// condition fails, the kernel sets the CUDA graph's while-loop condition and
// returns.
#include "../../include/gravidy_gb300.h"
#include "h4_exact.cuh"
#include "h4_force_fp64.cuh"
#include "h4_internal.cuh"
#include "h4_step_device.cuh"

namespace h4 {
namespace {

using exact::add;
using exact::bits_to_double;
using exact::double_to_bits;
using exact::INF_BITS;
using exact::is_active;

constexpr int LT = FLAG_THREADS;   // threads per block: one chunk of FLAG_CHUNK particles per block pass
constexpr unsigned long long BARRIER_TIMEOUT_NS = 10ull * 1000000000ull;

__device__ unsigned block_sum_u(unsigned x, unsigned *red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    __syncthreads();
    if (lane == 0) red[w] = x;
    __syncthreads();
    unsigned s = 0;
    for (int k = 0; k < LT / 32; k++) s += red[k];
    __syncthreads();
    return s;
}

__device__ unsigned block_scan_u(unsigned x, unsigned *red) {   // exclusive
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
    unsigned before = 0;
    for (int k = 0; k < w; k++) before += red[k];
    __syncthreads();
    return before + incl - x;
}

__device__ double block_min_d(double m, double *red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
    __syncthreads();
    if (lane == 0) red[w] = m;
    __syncthreads();
    m = red[0];
    for (int k = 1; k < LT / 32; k++) m = fmin(m, red[k]);
    __syncthreads();
    return m;
}

// Per-step bookkeeping of h4_advance (as advance_bookkeeping of the
// multi-kernel step) and the loop condition; one thread, with every block's
// work of the step complete.
__device__ void step_bookkeeping(const H4Dev &d) {
    H4Ctrl *c = d.ctrl;
    const unsigned nact = c->nact;
    c->steps += 1;
    c->psteps += nact;
    if (nact) c->nact_hist[31 - __clz(nact)] += 1;
    c->inter += (unsigned long long)nact * (unsigned long long)d.n;
    const double itime = c->itime;
    int go = (itime < c->t_stop) && (itime < c->t_log) && (c->err == 0u);
    if (go && c->steps >= c->max_steps) {   // every step advances time by >= dt_min
        c->err |= H4_ERRBIT_STEPCAP;
        go = 0;
    }
    c->running = go;
}

// Grid-wide barrier of the cooperative launch, bounded in time.  With
// `decide`, the last block to arrive runs the step's bookkeeping before it
// releases the others.  False after a timeout (error bit set).
__device__ bool loop_barrier(const H4Dev &d, bool decide) {
    H4Ctrl *c = d.ctrl;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &c->bar_gen;
        const unsigned g0 = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(&c->bar_count, 1u) + 1u;
        if (arrived == gridDim.x) {
            c->bar_count = 0u;
            if (decide) step_bookkeeping(d);
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            // short spin first: a barrier of ~150 blocks completes in about a
            // microsecond
            int spins = 0;
            while (*gen == g0 && ++spins < 4096) {
            }
            if (*gen == g0 && !bounded_wait_change(gen, g0, BARRIER_TIMEOUT_NS))
                atomicOr(&c->err, (unsigned)H4_ERRBIT_TIMEOUT);
        }
        __threadfence();
    }
    __syncthreads();
    return (*(volatile unsigned *)&c->err & H4_ERRBIT_TIMEOUT) == 0u;
}

template <int MODE>
__global__ void __launch_bounds__(LT, 1)
    k_step_loop(H4Dev d, int max_iters, unsigned split_warps, cudaGraphConditionalHandle cond) {
    __shared__ unsigned red[LT / 32];
    __shared__ double redd[LT / 32];
    H4Ctrl *c = d.ctrl;
    const unsigned nthreads = gridDim.x * LT;
    const unsigned gtid = blockIdx.x * LT + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int nchunks = (d.n + FLAG_CHUNK - 1) / FLAG_CHUNK;
    int go = *(volatile int *)&c->running;
    bool ok = true;   // false once a barrier timed out: leave, and stop the graph's loop
    if (gtid == 0) c->loop_launches += 1;
    for (int it = 0; it < max_iters && go; it++) {
        // P1: block time, predictor, active counts, min(t + dt) of the inactive
        const double itime = bits_to_double(c->atime_bits);
        double m = bits_to_double(INF_BITS);
        for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
            const int base = ch * FLAG_CHUNK + threadIdx.x * FLAG_ITEMS;
            unsigned cnt = 0;
#pragma unroll
            for (int q = 0; q < FLAG_ITEMS; q++) {
                const int i = base + q;
                if (i < d.n && is_active(itime, d.t[i], d.dt[i])) cnt++;
            }
            cnt = block_sum_u(cnt, red);
            if (threadIdx.x == 0) d.blk_cnt[ch] = cnt;
        }
        for (unsigned i = gtid; i < (unsigned)d.n; i += nthreads) {
            const double t = d.t[i], dt = d.dt[i];
            if (!is_active(itime, t, dt)) m = fmin(m, add(t, dt));
            step::predict_particle(d, (int)i, itime);
        }
        if (gtid == 0) {
            c->itime = itime;
            c->work_next = 0u;
        }
        if (!(ok = loop_barrier(d, false))) break;
        // P2: ordered scatter of the active list, active count
        unsigned nact = 0;
        for (int b = threadIdx.x; b < nchunks; b += LT) nact += d.blk_cnt[b];
        nact = block_sum_u(nact, red);
        for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
            unsigned before = 0;
            for (int b = threadIdx.x; b < ch; b += LT) before += d.blk_cnt[b];
            before = block_sum_u(before, red);
            const int base = ch * FLAG_CHUNK + threadIdx.x * FLAG_ITEMS;
            unsigned flags = 0, cnt = 0;
#pragma unroll
            for (int q = 0; q < FLAG_ITEMS; q++) {
                const int i = base + q;
                if (i < d.n && is_active(itime, d.t[i], d.dt[i])) { flags |= 1u << q; cnt++; }
            }
            unsigned off = before + block_scan_u(cnt, red);
            if (cnt && !range_ok(d, BS_SCATTER, off, (long long)off + cnt, d.n)) flags = 0;
#pragma unroll
            for (int q = 0; q < FLAG_ITEMS; q++)
                if (flags & (1u << q)) d.move[off++] = (unsigned)(base + q);
        }
        if (gtid == 0) {
            c->nact = nact;
            c->atime_bits = INF_BITS;   // read by every block in P1 only
        }
        if (!(ok = loop_barrier(d, false))) break;
        // P3: force sum of the active particles
        if (MODE == H4_FORCE_EXACT) {
            if (gtid == 0) c->force_split = 1u;
            for (unsigned k = gtid; k < nact; k += nthreads) fp64::exact_particle(d, nact, k);
        } else {
            fp64::force_items(d, split_warps, lane, gtid == 0);
        }
        if (!(ok = loop_barrier(d, false))) break;
        // P4: reduction + corrector + new timestep; min(t + dt) of the active
        const unsigned S = c->force_split;
        if (step::reduce_ranges_ok(d, nact, S)) {
            step::for_each_reduced(d, nact, S, [&](unsigned k, const double *fn) {
                step::correct_particle(d, k, itime, fn);
                const unsigned i = d.move[k];
                if (range_ok(d, BS_MOVE, i, i + 1ll, d.n)) m = fmin(m, add(d.t[i], d.dt[i]));
            });
        }
        m = block_min_d(m, redd);
        if (threadIdx.x == 0) atomicMin(&c->atime_bits, double_to_bits(m));
        if (!(ok = loop_barrier(d, true))) break;
        go = *(volatile int *)&c->running;
    }
    if (gtid == 0) cudaGraphSetConditional(cond, (ok && go) ? 1u : 0u);
}

}  // namespace

int step_loop_supported(int mode) { return mode == H4_FORCE_FP64 || mode == H4_FORCE_EXACT; }

cudaError_t launch_step_loop(const H4Dev &d, int mode, int grid, int max_iters, unsigned split_warps,
                             cudaGraphConditionalHandle cond, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(LT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (mode == H4_FORCE_EXACT)
        return cudaLaunchKernelEx(&cfg, k_step_loop<H4_FORCE_EXACT>, d, max_iters, split_warps, cond);
    return cudaLaunchKernelEx(&cfg, k_step_loop<H4_FORCE_FP64>, d, max_iters, split_warps, cond);
}

cudaError_t step_loop_max_grid(int mode, int num_sms, int *grid) {
    int per_sm = 0;
    cudaError_t e = mode == H4_FORCE_EXACT
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_loop<H4_FORCE_EXACT>, LT, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_loop<H4_FORCE_FP64>, LT, 0);
    *grid = per_sm > 0 ? num_sms : 0;   // one block per SM (all resident: cooperative launch)
    return e;
}

}  // namespace h4
