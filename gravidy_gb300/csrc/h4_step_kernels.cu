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
#include "h4_internal.cuh"

namespace h4 {
namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double bits_to_double(unsigned long long b) {
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long double_to_bits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
constexpr unsigned long long INF_BITS = 0x7FF0000000000000ull;

// NbodyUtils::get_magnitude (NbodyUtils.cpp:331-334): sqrt(x*x + y*y + z*z).
__device__ __forceinline__ double magnitude(double x, double y, double z) {
    return __dsqrt_rn(add(add(mul(x, x), mul(y, y)), mul(z, z)));
}

// Active test of Hermite4::find_particles_to_move (Hermite4.cpp:74-76):
// |ITIME - (t + dt)| < 2 * DBL_EPSILON.
__device__ __forceinline__ bool is_active(double itime, double t, double dt) {
    double tmp = add(t, dt);
    return fabs(sub(itime, tmp)) < 4.440892098500626e-16;
}

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

// Double-single split of a double: hi = fl32(x), lo = fl32(x - hi).
__device__ __forceinline__ void ds_split(double x, float &hi, float &lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(__dadd_rn(x, -(double)hi));
}

// Packed FP32 j data of the mixed kernels, from predicted position/velocity.
__device__ __forceinline__ void write_jf(const H4Dev &d, int i, const dbl4 &pr, const dbl4 &pv) {
    float4 a, b, c;
    ds_split(pr.x, a.x, b.x);
    ds_split(pr.y, a.y, b.y);
    ds_split(pr.z, a.z, b.z);
    a.w = (float)pr.w;
    b.w = 0.f;
    c = make_float4((float)pv.x, (float)pv.y, (float)pv.z, 0.f);
    d.jf0[i] = a;
    d.jf1[i] = b;
    d.jf2[i] = c;
}

// ---- active set (Hermite4::find_particles_to_move) --------------------------
// Pass 1: active count of each chunk of FLAG_CHUNK particles.
__global__ void __launch_bounds__(FLAG_THREADS)
k_flag_count(H4Dev d, int host_itime, double itime_in) {
    double itime = host_itime ? itime_in : bits_to_double(d.ctrl->atime_bits);
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
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nact; k += gridDim.x * blockDim.x) {
        const unsigned i = d.move[k];
#pragma unroll
        for (int c = 0; c < 6; c++) d.old[6 * (size_t)i + c] = d.f[6 * (size_t)i + c];
    }
}

// ---- Hermite4CPU::predicted_pos_vel (Hermite4CPU.cpp:340-365) ---------------
__global__ void __launch_bounds__(256) k_predict(H4Dev d, int host_itime, double itime_in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const double itime = host_itime ? itime_in : d.ctrl->itime;
    const double dt = sub(itime, d.t[i]);
    const double dt2 = mul(dt, dt);
    const double dt3 = mul(dt2, dt);
    const double dt2c = dvd(dt2, 2.0);
    const double dt3c = dvd(dt3, 6.0);
    const double *f = d.f + 6 * (size_t)i;
    const dbl4 r = d.r[i], v = d.v[i];
    dbl4 pr, pv;
    pr.x = add(add(add(mul(dt3c, f[3]), mul(dt2c, f[0])), mul(dt, v.x)), r.x);
    pr.y = add(add(add(mul(dt3c, f[4]), mul(dt2c, f[1])), mul(dt, v.y)), r.y);
    pr.z = add(add(add(mul(dt3c, f[5]), mul(dt2c, f[2])), mul(dt, v.z)), r.z);
    pr.w = (double)(float)r.w;   // Predictor::m is a float (common.hpp:216)
    pv.x = add(add(mul(dt2c, f[3]), mul(dt, f[0])), v.x);
    pv.y = add(add(mul(dt2c, f[4]), mul(dt, f[1])), v.y);
    pv.z = add(add(mul(dt2c, f[5]), mul(dt, f[2])), v.z);
    pv.w = 0.0;
    d.pr[i] = pr;
    d.pv[i] = pv;
    if (d.jf0) write_jf(d, i, pr, pv);
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
    if (d.jf0) write_jf(d, i, r, v);
}

// Padding of the predicted arrays past n: zero mass, far away, at rest.
// A padded j contributes exactly zero to every sum, so tiled kernels may
// process whole tiles without bounds checks.
__global__ void k_pad_predicted(H4Dev d) {
    const int i = d.n + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n_pad) return;
    d.pr[i] = make_dbl4(1.0e15, 1.0e15, 1.0e15, 0.0);
    d.pv[i] = make_dbl4(0.0, 0.0, 0.0, 0.0);
    if (d.jf0) {
        d.jf0[i] = make_float4(1.0e15f, 1.0e15f, 1.0e15f, 0.f);
        d.jf1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        d.jf2[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void k_identity_move(H4Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.n) d.move[i] = (unsigned)i;
    if (i == 0) {
        d.ctrl->nact = (unsigned)d.n;
        d.ctrl->work_next = 0;
    }
}

// Sum of the j-split partial forces of active particle k, in chunk order.
__device__ __forceinline__ void reduce_partials(const H4Dev &d, unsigned k, unsigned nact,
                                                unsigned S, double out[6]) {
#pragma unroll
    for (int c = 0; c < 6; c++) out[c] = 0.0;
    for (unsigned s = 0; s < S; s++) {
        const double *p = d.part + (size_t)s * 6 * nact;
#pragma unroll
        for (int c = 0; c < 6; c++) out[c] = add(out[c], p[(size_t)c * nact + k]);
    }
}

__global__ void k_reduce_forces(H4Dev d, int save_old) {
    const unsigned nact = d.ctrl->nact, S = d.ctrl->force_split;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nact; k += gridDim.x * blockDim.x) {
        const unsigned i = d.move[k];
        double fn[6];
        reduce_partials(d, k, nact, S, fn);
        double *f = d.f + 6 * (size_t)i;
        if (save_old) {
#pragma unroll
            for (int c = 0; c < 6; c++) d.old[6 * (size_t)i + c] = f[c];
        }
#pragma unroll
        for (int c = 0; c < 6; c++) f[c] = fn[c];
    }
}

// NbodyUtils::normalize_dt (NbodyUtils.cpp:371-424).
__device__ double normalize_dt(const H4Dev &d, double new_dt, double old_dt, double t) {
    const double o8 = dvd(old_dt, 8.0), o4 = dvd(old_dt, 4.0), o2 = dvd(old_dt, 2.0);
    const double o2x = mul(old_dt, 2.0), x2o = mul(2.0, old_dt);
    if (new_dt <= o8) {
        new_dt = 1.1920928955078125e-07;  // D_TIME_MIN (common.hpp:122), not the handle's bound
    } else if (o8 < new_dt && new_dt <= o4) {
        new_dt = o8;
    } else if (o4 < new_dt && new_dt <= o2) {
        new_dt = o4;
    } else if (o2 < new_dt && new_dt <= old_dt) {
        new_dt = o2;
    } else if (old_dt < new_dt && new_dt <= o2x) {
        new_dt = old_dt;
    } else if (x2o < new_dt) {
        const double val = dvd(t, x2o);
        new_dt = (ceil(val) == val) ? mul(2.0, old_dt) : old_dt;
    } else {
        new_dt = old_dt;
    }
    if (new_dt < d.dt_min)
        new_dt = d.dt_min;
    else if (new_dt > d.dt_max)
        new_dt = d.dt_max;
    return new_dt;
}

// ---- Hermite4CPU::correction_pos_vel (Hermite4CPU.cpp:370-411) --------------
// with NbodyUtils::get_timestep_normal (NbodyUtils.cpp:337-365).
__global__ void __launch_bounds__(128) k_correct(H4Dev d, int host_itime, double itime_in, int fused_reduce) {
    const unsigned nact = d.ctrl->nact;
    const double itime = host_itime ? itime_in : d.ctrl->itime;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nact; k += gridDim.x * blockDim.x) {
        const unsigned i = d.move[k];
        double *fp = d.f + 6 * (size_t)i;
        double *op = d.old + 6 * (size_t)i;
        double f[6], o[6];
        if (fused_reduce) {
            reduce_partials(d, k, nact, d.ctrl->force_split, f);
#pragma unroll
            for (int c = 0; c < 6; c++) { o[c] = fp[c]; op[c] = o[c]; fp[c] = f[c]; }
        } else {
#pragma unroll
            for (int c = 0; c < 6; c++) { f[c] = fp[c]; o[c] = op[c]; }
        }
        const dbl4 p = d.pr[i], pv = d.pv[i];
        const double dt1 = d.dt[i];
        const double dt2 = mul(dt1, dt1);
        const double dt3 = mul(dt2, dt1);
        const double dt4 = mul(dt2, dt2);
        const double dt5 = mul(dt4, dt1);
        double a2[3], a3[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            // (-6 (a0 - a1) - dt (4 j0 + 2 j1)) / dt^2
            a2[c] = dvd(sub(mul(-6.0, sub(o[c], f[c])),
                            mul(dt1, add(mul(4.0, o[3 + c]), mul(2.0, f[3 + c])))), dt2);
            // (12 (a0 - a1) + 6 dt (j0 + j1)) / dt^3
            a3[c] = dvd(add(mul(12.0, sub(o[c], f[c])),
                            mul(mul(6.0, dt1), add(o[3 + c], f[3 + c]))), dt3);
        }
        const double c24 = dvd(dt4, 24.0), c120 = dvd(dt5, 120.0), c6 = dvd(dt3, 6.0);
        dbl4 r = d.r[i], v = d.v[i];
        r.x = add(add(p.x, mul(c24, a2[0])), mul(c120, a3[0]));
        r.y = add(add(p.y, mul(c24, a2[1])), mul(c120, a3[1]));
        r.z = add(add(p.z, mul(c24, a2[2])), mul(c120, a3[2]));
        v.x = add(add(pv.x, mul(c6, a2[0])), mul(c24, a3[0]));
        v.y = add(add(pv.y, mul(c6, a2[1])), mul(c24, a3[1]));
        v.z = add(add(pv.z, mul(c6, a2[2])), mul(c24, a3[2]));
        d.r[i] = r;
        d.v[i] = v;
#pragma unroll
        for (int c = 0; c < 3; c++) { d.a2[3 * (size_t)i + c] = a2[c]; d.a3[3 * (size_t)i + c] = a3[c]; }
        d.t[i] = itime;

        // get_timestep_normal, with the step's old dt as the reference uses it.
        const double ax1 = add(a2[0], mul(dt1, a3[0]));
        const double ay1 = add(a2[1], mul(dt1, a3[1]));
        const double az1 = add(a2[2], mul(dt1, a3[2]));
        const double abs_a1 = magnitude(f[0], f[1], f[2]);
        const double abs_j1 = magnitude(f[3], f[4], f[5]);
        const double abs_j12 = mul(abs_j1, abs_j1);
        const double abs_a1_3 = magnitude(a3[0], a3[1], a3[2]);
        const double abs_a1_2 = magnitude(ax1, ay1, az1);
        const double abs_a1_22 = mul(abs_a1_2, abs_a1_2);
        const double normal_dt = __dsqrt_rn(mul(d.eta, dvd(add(mul(abs_a1, abs_a1_2), abs_j12),
                                                            add(mul(abs_j1, abs_a1_3), abs_a1_22))));
        const double ndt = normalize_dt(d, normal_dt, dt1, itime);
        d.dt[i] = ndt;
        if (!isfinite(r.x) || !isfinite(r.y) || !isfinite(r.z) || !isfinite(v.x) ||
            !isfinite(v.y) || !isfinite(v.z))
            atomicOr(&d.ctrl->err, (unsigned)H4_ERRBIT_NONFINITE);
    }
}

// ---- Hermite4::next_integration_time (Hermite4.cpp:90-102) ------------------
__global__ void k_reset_atime(H4Dev d) { d.ctrl->atime_bits = INF_BITS; }

__global__ void __launch_bounds__(256) k_next_time(H4Dev d) {
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

// (int) of a double as x86-64 converts it (NaN and out-of-range -> INT_MIN);
// the reference relies on that for particles without jerk (Hermite4.cpp:124).
__device__ __forceinline__ int trunc_to_int_x86(double x) {
    if (!(x > -2147483649.0 && x < 2147483648.0)) return INT_MIN;
    return (int)x;
}

// ---- Hermite4::init_dt (Hermite4.cpp:108-140) -------------------------------
__global__ void k_init_dt(H4Dev d, double eta, double itime) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double tmp = __longlong_as_double((long long)INF_BITS);
    if (i < d.n) {
        const double *f = d.f + 6 * (size_t)i;
        const double a2 = magnitude(f[0], f[1], f[2]);
        const double j2 = magnitude(f[3], f[4], f[5]);
        tmp = mul(eta, dvd(a2, j2));
        // log(2.0), correctly rounded: 0x3FE62E42FEFA39EF
        const int ex = trunc_to_int_x86(sub(ceil(dvd(log(tmp), 0x1.62e42fefa39efp-1)), 1.0));
        tmp = ldexp(1.0, ex);   // pow(2, ex): exact
        if (tmp < d.dt_min)
            tmp = d.dt_min;
        else if (tmp > d.dt_max)
            tmp = d.dt_max;
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
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < nact; k += gridDim.x * blockDim.x) {
        double fn[6];
        reduce_partials(d, k, nact, S, fn);
#pragma unroll
        for (int c = 0; c < 6; c++) out[6 * (size_t)k + c] = fn[c];
    }
}

// ---- per-step bookkeeping of the device-resident loop ------------------------
__global__ void k_advance_bookkeeping(H4Dev d, cudaGraphConditionalHandle cond, int use_cond) {
    H4Ctrl *c = d.ctrl;
    const unsigned nact = c->nact;
    c->steps += 1;
    c->psteps += nact;
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

int kernels_per_step() { return 6; }

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
    k_next_time<<<nb, 256, 0, s>>>(d);
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

void launch_pad_predicted(const H4Dev &d, cudaStream_t s) {
    if (d.n_pad > d.n) k_pad_predicted<<<blocks_for(d.n_pad - d.n, 256), 256, 0, s>>>(d);
}

void launch_set_nact(const H4Dev &d, unsigned nact, cudaStream_t s) { k_set_nact<<<1, 1, 0, s>>>(d, nact); }

void launch_set_atime(const H4Dev &d, double atime, cudaStream_t s) { k_set_atime<<<1, 1, 0, s>>>(d, atime); }

void launch_reduce_to(const H4Dev &d, double *out, cudaStream_t s) {
    k_reduce_to<<<blocks_for(d.n, 256), 256, 0, s>>>(d, out);
}

void launch_advance_bookkeeping(const H4Dev &d, cudaGraphConditionalHandle cond, bool use_cond,
                                cudaStream_t s) {
    k_advance_bookkeeping<<<1, 1, 0, s>>>(d, cond, use_cond ? 1 : 0);
}

}  // namespace h4
