// Block-step kernels of the Hermite4 integrator, other than the force sum.
//
// These kernels restate the reference's host-side integrator arithmetic
// (src/include/cpu/Hermite4CPU.cpp:340-411, src/include/Hermite4.cpp:63-140,
// src/include/utils/NbodyUtils.cpp:331-424) with every floating-point
// operation spelled out as an IEEE round-to-nearest intrinsic in the
// reference's order.  nvcc would otherwise contract a*b+c into one FMA, which
// the reference build (g++ on x86-64) never does; with the intrinsics the
// predictor, corrector, timestep and active-set results are bit-identical to
// the reference's for identical inputs.
#include "h4_exact.cuh"
#include "h4_internal.cuh"
#include "h4_step_device.cuh"

namespace h4 {
namespace {

using namespace step;
using exact::add;
using exact::bits_to_double;
using exact::double_to_bits;
using exact::dvd;
using exact::INF_BITS;
using exact::is_active;
using exact::mul;
using exact::sub;

// Block-wide exclusive scan of one unsigned per thread (FLAG_THREADS threads).
__device__ unsigned block_exclusive_scan(unsigned x) {
    __shared__ unsigned warp_sums[FLAG_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = (lane < FLAG_THREADS / 32) ? warp_sums[lane] : 0u;
        unsigned wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < FLAG_THREADS / 32) warp_sums[lane] = wi - w;  // exclusive
    }
    __syncthreads();
    unsigned res = warp_sums[warp] + incl - x;
    __syncthreads();
    return res;
}

__device__ unsigned block_sum(unsigned x) {
    __shared__ unsigned red[FLAG_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp] = x;
    __syncthreads();
    unsigned s = 0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < FLAG_THREADS / 32; w++) s += red[w];
        red[0] = s;
    }
    __syncthreads();
    s = red[0];
    __syncthreads();
    return s;
}

// ---- active set (Hermite4::find_particles_to_move) --------------------------
// Pass 1: active count of each chunk of FLAG_CHUNK particles.
__device__ __forceinline__ void flag_count_chunk(const H4Dev &d, double itime) {
    const int base = blockIdx.x * FLAG_CHUNK + threadIdx.x * FLAG_ITEMS;
    unsigned c = 0;
#pragma unroll
    for (int q = 0; q < FLAG_ITEMS; q++) {
        int i = base + q;
        if (i < d.n && is_active(itime, d.t[i], d.dt[i])) c++;
    }
    c = block_sum(c);
    if (threadIdx.x == 0) {
        d.blk_cnt[blockIdx.x] = c;
        if (blockIdx.x == 0) d.ctrl->itime = itime;
    }
}

__global__ void __launch_bounds__(FLAG_THREADS)
k_flag_count(H4Dev d, int host_itime, double itime_in) {
    flag_count_chunk(d, host_itime ? itime_in : bits_to_double(d.ctrl->atime_bits));
}

// Pass 2: ordered scatter of the active indices (ascending i, as the
// reference's sequential loop produces them).
__global__ void __launch_bounds__(FLAG_THREADS)
k_flag_scatter(H4Dev d, int nblocks) {
    const double itime = d.ctrl->itime;
    unsigned before = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += FLAG_THREADS) before += d.blk_cnt[b];
    before = block_sum(before);
    const int base = blockIdx.x * FLAG_CHUNK + threadIdx.x * FLAG_ITEMS;
    unsigned flags = 0, c = 0;
#pragma unroll
    for (int q = 0; q < FLAG_ITEMS; q++) {
        int i = base + q;
        if (i < d.n && is_active(itime, d.t[i], d.dt[i])) { flags |= 1u << q; c++; }
    }
    unsigned off = before + block_exclusive_scan(c);
    if (c && !range_ok(d, BS_SCATTER, off, (long long)off + c, d.n)) flags = 0;
#pragma unroll
    for (int q = 0; q < FLAG_ITEMS; q++)
        if (flags & (1u << q)) d.move[off++] = (unsigned)(base + q);
    if (blockIdx.x == 0) {
        unsigned all = 0;
        for (int b = threadIdx.x; b < nblocks; b += FLAG_THREADS) all += d.blk_cnt[b];
        all = block_sum(all);
        if (threadIdx.x == 0) {
            d.ctrl->nact = all;
            d.ctrl->work_next = 0;
            d.ctrl->atime_bits = INF_BITS;
        }
    }
}

// ---- Hermite4::save_old_acc_jrk (Hermite4.cpp:145-153) ----------------------
__global__ void k_save_old(H4Dev d) {
    const unsigned nact = d.ctrl->nact;
    if (!range_ok(d, BS_NACT, 0, nact, d.n)) return;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nact; k += gridDim.x * blockDim.x) {
        const unsigned i = d.move[k];
        if (!range_ok(d, BS_MOVE, i, i + 1ll, d.n)) continue;
#pragma unroll
        for (int c = 0; c < 6; c++) d.old[6 * (size_t)i + c] = d.f[6 * (size_t)i + c];
    }
}

// ---- Hermite4CPU::predicted_pos_vel (Hermite4CPU.cpp:340-365) ---------------
__global__ void __launch_bounds__(256) k_predict(H4Dev d, int host_itime, double itime_in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    predict_particle(d, i, host_itime ? itime_in : d.ctrl->itime);
}

// The device-resident step's first pass: the active counts of the chunks
// (the first nb_flag blocks, one chunk each) and the predictor of every
// particle at the next block time (the control block's atime; one particle
// per thread, all blocks), in one launch.  Same arithmetic as k_flag_count
// then k_predict.
__global__ void __launch_bounds__(FLAG_THREADS) k_flag_count_predict(H4Dev d, int nb_flag) {
    const double itime = bits_to_double(d.ctrl->atime_bits);
    if ((int)blockIdx.x < nb_flag) flag_count_chunk(d, itime);
    const int i = blockIdx.x * FLAG_THREADS + threadIdx.x;
    if (i < d.n) predict_particle(d, i, itime);
}

// Predictors straight from the state (Hermite4::init_data, Hermite4.cpp:
// 202-214), used before init_acc_jrk.
__global__ void k_pred_from_state(H4Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    dbl4 r = d.r[i], v = d.v[i];
    r.w = (double)(float)r.w;
    v.w = 0.0;
    d.pr[i] = r;
    d.pv[i] = v;
    if (d.mixed) write_jf(d, i, r, v);
}

__global__ void k_pack_j(H4Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.n) write_jf(d, i, d.pr[i], d.pv[i]);
}

// Padding of the predicted arrays past n: zero mass, far away, at rest.
// A padded j contributes exactly zero to every sum, so tiled kernels may
// process whole tiles without bounds checks.
__global__ void k_pad_predicted(H4Dev d) {
    const int i = d.n + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n_pad) return;
    d.pr[i] = make_dbl4(1.0e15, 1.0e15, 1.0e15, 0.0);
    d.pv[i] = make_dbl4(0.0, 0.0, 0.0, 0.0);
    if (d.jf0) write_jf(d, i, d.pr[i], d.pv[i]);
}

__global__ void k_identity_move(H4Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.n) d.move[i] = (unsigned)i;
    if (i == 0) {
        d.ctrl->nact = (unsigned)d.n;
        d.ctrl->work_next = 0;
    }
}

__global__ void k_reduce_forces(H4Dev d, int save_old) {
    const unsigned nact = d.ctrl->nact, S = d.ctrl->force_split;
    if (!reduce_ranges_ok(d, nact, S)) return;
    for_each_reduced(d, nact, S, [&](unsigned k, const double *fn) {
        const unsigned i = d.move[k];
        if (!range_ok(d, BS_MOVE, i, i + 1ll, d.n)) return;
        double *f = d.f + 6 * (size_t)i;
        if (save_old) {
#pragma unroll
            for (int c = 0; c < 6; c++) d.old[6 * (size_t)i + c] = f[c];
        }
#pragma unroll
        for (int c = 0; c < 6; c++) f[c] = fn[c];
    });
}

__global__ void __launch_bounds__(128) k_correct(H4Dev d, int host_itime, double itime_in, int fused_reduce) {
    const unsigned nact = d.ctrl->nact;
    const double itime = host_itime ? itime_in : d.ctrl->itime;
    if (fused_reduce) {
        const unsigned S = d.ctrl->force_split;
        if (!reduce_ranges_ok(d, nact, S)) return;
        for_each_reduced(d, nact, S, [&](unsigned k, const double *fn) { correct_particle(d, k, itime, fn); });
    } else {
        if (!reduce_ranges_ok(d, nact, 0u)) return;
        for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nact; k += gridDim.x * blockDim.x)
            correct_particle(d, k, itime, nullptr);
    }
}

// ---- Hermite4::next_integration_time (Hermite4.cpp:90-102) ------------------
__global__ void k_reset_atime(H4Dev d) { d.ctrl->atime_bits = INF_BITS; }

__device__ void advance_bookkeeping(const H4Dev &d, cudaGraphConditionalHandle cond, int use_cond);

// bookkeep: also the per-step bookkeeping of the device-resident loop (one
// thread), which needs nothing this kernel computes.
__global__ void __launch_bounds__(256) k_next_time(H4Dev d, int bookkeep, cudaGraphConditionalHandle cond) {
    if (bookkeep && blockIdx.x == 0 && threadIdx.x == 0) advance_bookkeeping(d, cond, 1);
    double m = __longlong_as_double((long long)INF_BITS);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x)
        m = fmin(m, add(d.t[i], d.dt[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmin(m, red[w]);
        atomicMin(&d.ctrl->atime_bits, double_to_bits(m));
    }
}

// ---- Hermite4::init_dt (Hermite4.cpp:108-140) -------------------------------
__global__ void k_init_dt(H4Dev d, double eta, double itime) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double tmp = __longlong_as_double((long long)INF_BITS);
    if (i < d.n) {
        tmp = exact::init_dt(d.f + 6 * (size_t)i, eta, d.dt_min, d.dt_max);
        d.dt[i] = tmp;
        d.t[i] = itime;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tmp = fmin(tmp, __shfl_down_sync(0xffffffffu, tmp, o));
    if ((threadIdx.x & 31) == 0) atomicMin(&d.ctrl->atime_bits, double_to_bits(tmp));
}

__global__ void k_set_nact(H4Dev d, unsigned nact) {
    d.ctrl->nact = nact;
    d.ctrl->work_next = 0;
}

__global__ void k_set_atime(H4Dev d, double atime) { d.ctrl->atime_bits = double_to_bits(atime); }

// Fixed-order sum of the partial forces into out[6k + c] (Forces layout).
__global__ void k_reduce_to(H4Dev d, double *out) {
    const unsigned nact = d.ctrl->nact, S = d.ctrl->force_split;
    if (!reduce_ranges_ok(d, nact, S)) return;
    for_each_reduced(d, nact, S, [&](unsigned k, const double *fn) {
#pragma unroll
        for (int c = 0; c < 6; c++) out[6 * (size_t)k + c] = fn[c];
    });
}

// ---- per-step bookkeeping of the device-resident loop ------------------------
__device__ void advance_bookkeeping(const H4Dev &d, cudaGraphConditionalHandle cond, int use_cond) {
    H4Ctrl *c = d.ctrl;
    const unsigned nact = c->nact;
    c->steps += 1;
    c->psteps += nact;
    if (nact) c->nact_hist[31 - __clz(nact)] += 1;
    c->inter += (unsigned long long)nact * (unsigned long long)d.n;
    const double itime = c->itime;
    // Every step advances the block time by at least dt_min (times are
    // multiples of dt_min), so max_steps bounds the loop; reaching it is an
    // error, never an endless loop.
    int go = (itime < c->t_stop) && (itime < c->t_log) && (c->err == 0u);
    if (go && c->steps >= c->max_steps) {
        c->err |= H4_ERRBIT_STEPCAP;
        go = 0;
    }
    c->running = go;
    if (use_cond) cudaGraphSetConditional(cond, go ? 1u : 0u);
}


}  // namespace

static inline int blocks_for(int n, int t) { return (n + t - 1) / t > 0 ? (n + t - 1) / t : 1; }

void launch_find_active(const H4Dev &d, bool host_itime, double itime, cudaStream_t s) {
    const int nb = blocks_for(d.n, FLAG_CHUNK);
    k_flag_count<<<nb, FLAG_THREADS, 0, s>>>(d, host_itime ? 1 : 0, itime);
    k_flag_scatter<<<nb, FLAG_THREADS, 0, s>>>(d, nb);
}

void launch_save_old(const H4Dev &d, cudaStream_t s) {
    k_save_old<<<blocks_for(d.n, 256), 256, 0, s>>>(d);
}

void launch_predict(const H4Dev &d, bool host_itime, double itime, cudaStream_t s) {
    k_predict<<<blocks_for(d.n, 256), 256, 0, s>>>(d, host_itime ? 1 : 0, itime);
}

void launch_reduce_forces(const H4Dev &d, bool save_old, cudaStream_t s) {
    k_reduce_forces<<<blocks_for(d.n, 256), 256, 0, s>>>(d, save_old ? 1 : 0);
}

void launch_correct(const H4Dev &d, bool host_itime, double itime, bool fused_reduce, cudaStream_t s) {
    k_correct<<<blocks_for(d.n, 128), 128, 0, s>>>(d, host_itime ? 1 : 0, itime, fused_reduce ? 1 : 0);
}

void launch_next_time(const H4Dev &d, bool reset, cudaStream_t s) {
    if (reset) k_reset_atime<<<1, 1, 0, s>>>(d);
    int nb = blocks_for(d.n, 256);
    if (nb > 1024) nb = 1024;
    k_next_time<<<nb, 256, 0, s>>>(d, 0, cudaGraphConditionalHandle{});
}

void launch_next_time_bookkeeping(const H4Dev &d, cudaGraphConditionalHandle cond, cudaStream_t s) {
    int nb = blocks_for(d.n, 256);
    if (nb > 1024) nb = 1024;
    k_next_time<<<nb, 256, 0, s>>>(d, 1, cond);
}

void launch_find_active_predict(const H4Dev &d, cudaStream_t s) {
    const int nb = blocks_for(d.n, FLAG_CHUNK);
    const int np = blocks_for(d.n, FLAG_THREADS);   // >= nb
    k_flag_count_predict<<<np, FLAG_THREADS, 0, s>>>(d, nb);
    k_flag_scatter<<<nb, FLAG_THREADS, 0, s>>>(d, nb);
}

void launch_init_dt(const H4Dev &d, float eta, double itime, cudaStream_t s) {
    k_reset_atime<<<1, 1, 0, s>>>(d);
    k_init_dt<<<blocks_for(d.n, 256), 256, 0, s>>>(d, (double)eta, itime);
}

void launch_identity_move(const H4Dev &d, cudaStream_t s) {
    k_identity_move<<<blocks_for(d.n, 256), 256, 0, s>>>(d);
}

void launch_set_pred_from_state(const H4Dev &d, cudaStream_t s) {
    k_pred_from_state<<<blocks_for(d.n, 256), 256, 0, s>>>(d);
}

void launch_pack_j(const H4Dev &d, cudaStream_t s) {
    k_pack_j<<<blocks_for(d.n, 256), 256, 0, s>>>(d);
}

void launch_pad_predicted(const H4Dev &d, cudaStream_t s) {
    if (d.n_pad > d.n) k_pad_predicted<<<blocks_for(d.n_pad - d.n, 256), 256, 0, s>>>(d);
}

void launch_set_nact(const H4Dev &d, unsigned nact, cudaStream_t s) { k_set_nact<<<1, 1, 0, s>>>(d, nact); }

void launch_set_atime(const H4Dev &d, double atime, cudaStream_t s) { k_set_atime<<<1, 1, 0, s>>>(d, atime); }

void launch_reduce_to(const H4Dev &d, double *out, cudaStream_t s) {
    k_reduce_to<<<blocks_for(d.n, 256), 256, 0, s>>>(d, out);
}


}  // namespace h4
