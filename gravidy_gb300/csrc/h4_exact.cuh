// Per-particle integrator arithmetic in the reference's exact operation
// order (IEEE round-to-nearest intrinsics, no FMA contraction), shared by the
// single-system kernels and the ensemble kernel.  Each function names the
// reference routine it restates.
#pragma once
#include "h4_internal.cuh"

namespace h4 {
namespace exact {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

constexpr unsigned long long INF_BITS = 0x7FF0000000000000ull;
constexpr double D_TIME_MIN_REF = 1.1920928955078125e-07;   // common.hpp:122

__device__ __forceinline__ double bits_to_double(unsigned long long b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ unsigned long long double_to_bits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}

// NbodyUtils::get_magnitude (NbodyUtils.cpp:331-334)
__device__ __forceinline__ double magnitude(double x, double y, double z) {
    return __dsqrt_rn(add(add(mul(x, x), mul(y, y)), mul(z, z)));
}

// Hermite4::find_particles_to_move test (Hermite4.cpp:74-76)
constexpr double ACTIVE_EPS = 4.440892098500626e-16;   // 2^-51
__device__ __forceinline__ bool is_active(double itime, double t, double dt) {
    return fabs(sub(itime, add(t, dt))) < ACTIVE_EPS;
}
// The same test on a stored tn = add(t, dt).
__device__ __forceinline__ bool is_active_tn(double itime, double tn) { return fabs(sub(itime, tn)) < ACTIVE_EPS; }

// The bit patterns [lo, hi] of exactly the doubles tn that pass
// is_active_tn(itime, tn), for 2^-48 <= itime < inf (returns false
// otherwise; callers then test each tn).  A tn within 2^-51 of such an itime
// lies in [itime / 2, 2 itime], where itime - tn is exact (Sterbenz), so the
// test is the real inequality |itime - tn| < 2^-51; any other tn misses by
// far more than a rounding.  Positive doubles order like their bit patterns,
// and no non-positive or NaN pattern falls in [lo, hi].
__device__ __forceinline__ bool active_window(double itime, unsigned long long &lo, unsigned long long &hi) {
    if (!(itime >= 0x1p-48 && itime < bits_to_double(INF_BITS))) return false;
    unsigned long long a = double_to_bits(__dadd_ru(itime, -ACTIVE_EPS));
    if (__dadd_rd(itime, -ACTIVE_EPS) == bits_to_double(a)) a++;   // itime - 2^-51 itself fails the test
    unsigned long long b = double_to_bits(__dadd_rd(itime, ACTIVE_EPS));
    if (__dadd_ru(itime, ACTIVE_EPS) == bits_to_double(b)) b--;
    lo = a;
    hi = b;
    return true;
}

// Hermite4CPU::predicted_pos_vel (Hermite4CPU.cpp:344-362) for one particle.
__device__ __forceinline__ void predict(double itime, double t, const double *f, const dbl4 &r, const dbl4 &v,
                                        dbl4 &pr, dbl4 &pv) {
    const double dt = sub(itime, t);
    const double dt2 = mul(dt, dt);
    const double dt3 = mul(dt2, dt);
    const double dt2c = mul(dt2, 0.5);   // == dt2 / 2.0 for every double (scaling by 2^-1)
    const double dt3c = dvd(dt3, 6.0);
    pr.x = add(add(add(mul(dt3c, f[3]), mul(dt2c, f[0])), mul(dt, v.x)), r.x);
    pr.y = add(add(add(mul(dt3c, f[4]), mul(dt2c, f[1])), mul(dt, v.y)), r.y);
    pr.z = add(add(add(mul(dt3c, f[5]), mul(dt2c, f[2])), mul(dt, v.z)), r.z);
    pr.w = (double)(float)r.w;   // Predictor::m is a float (common.hpp:216)
    pv.x = add(add(mul(dt2c, f[3]), mul(dt, f[0])), v.x);
    pv.y = add(add(mul(dt2c, f[4]), mul(dt, f[1])), v.y);
    pv.z = add(add(mul(dt2c, f[5]), mul(dt, f[2])), v.z);
    pv.w = 0.0;
}

// Double-single split of a double: hi = fl32(x), lo = fl32(x - hi).
__device__ __forceinline__ void ds_split(double x, float &hi, float &lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(__dadd_rn(x, -(double)hi));
}

// Packed FP32 j data of the mixed kernels.
__device__ __forceinline__ void pack_jf(const dbl4 &pr, const dbl4 &pv, float4 &a, float4 &b, float4 &c) {
    ds_split(pr.x, a.x, b.x);
    ds_split(pr.y, a.y, b.y);
    ds_split(pr.z, a.z, b.z);
    a.w = (float)pr.w;
    b.w = 0.f;
    c = make_float4((float)pv.x, (float)pv.y, (float)pv.z, 0.f);
}

// x is a normal power of two (zero mantissa bits).
__device__ __forceinline__ bool is_pow2(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long e = (b >> 52) & 0x7FFull;
    return (b & 0x000FFFFFFFFFFFFFull) == 0ull && e != 0ull && e != 0x7FFull && (b >> 63) == 0ull;
}

// 1/x of a normal power of two x, exactly (exponent arithmetic); requires
// 1/x to be normal as well.
__device__ __forceinline__ double recip_pow2(double x) {
    const long long e = (long long)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FFull);
    return __longlong_as_double((long long)((unsigned long long)(2046 - e) << 52));
}

// NbodyUtils::normalize_dt (NbodyUtils.cpp:371-424); dt_min/dt_max are the
// clamp bounds (D_TIME_MIN/D_TIME_MAX by default).
__device__ __forceinline__ double normalize_dt(double new_dt, double old_dt, double t, double dt_min,
                                               double dt_max) {
    // x / 2^k == x * 2^-k for every double x: scaling by a power of two
    const double o8 = mul(old_dt, 0.125), o4 = mul(old_dt, 0.25), o2 = mul(old_dt, 0.5);
    const double o2x = mul(old_dt, 2.0);
    if (new_dt <= o8) {
        new_dt = D_TIME_MIN_REF;
    } else if (o8 < new_dt && new_dt <= o4) {
        new_dt = o8;
    } else if (o4 < new_dt && new_dt <= o2) {
        new_dt = o4;
    } else if (o2 < new_dt && new_dt <= old_dt) {
        new_dt = o2;
    } else if (old_dt < new_dt && new_dt <= o2x) {
        new_dt = old_dt;
    } else if (o2x < new_dt) {
        const double val = is_pow2(o2x) ? mul(t, recip_pow2(o2x)) : dvd(t, o2x);
        new_dt = (ceil(val) == val) ? mul(2.0, old_dt) : old_dt;
    } else {
        new_dt = old_dt;
    }
    if (new_dt < dt_min)
        new_dt = dt_min;
    else if (new_dt > dt_max)
        new_dt = dt_max;
    return new_dt;
}

// Hermite4CPU::correction_pos_vel (Hermite4CPU.cpp:370-411) with
// NbodyUtils::get_timestep_normal (NbodyUtils.cpp:337-365) for one particle:
// new r, v, a2, a3 and the new block timestep.  Returns false if r or v came
// out non-finite.
__device__ __forceinline__ bool correct(double itime, double eta, double dt_min, double dt_max, const double f[6],
                                        const double o[6], const dbl4 &p, const dbl4 &pv, double dt1, dbl4 &r,
                                        dbl4 &v, double a2[3], double a3[3], double &new_dt) {
    const double dt2 = mul(dt1, dt1);
    const double dt3 = mul(dt2, dt1);
    const double dt4 = mul(dt2, dt2);
    const double dt5 = mul(dt4, dt1);
    // Block timesteps are powers of two, so dt^k is one too (dt >= 2^-23 keeps
    // every power normal): x / dt^k is then x * (1/dt^k) exactly, and
    // dt^k / 24 = dt^k * RN(1/24) exactly, since RN(2^m / 3) = 2^m RN(1/3)
    // (likewise 1/6 and 1/120 = 2^-3 / 15).  Identical results to the
    // divisions, without the FP64 division sequences; any other dt takes the
    // divisions.
    const bool p2 = is_pow2(dt1) && is_pow2(dt5);
    const double i2 = p2 ? recip_pow2(dt2) : 0.0, i3 = p2 ? recip_pow2(dt3) : 0.0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        // (-6 (a0 - a1) - dt (4 j0 + 2 j1)) / dt^2
        const double n2 = sub(mul(-6.0, sub(o[c], f[c])), mul(dt1, add(mul(4.0, o[3 + c]), mul(2.0, f[3 + c]))));
        // (12 (a0 - a1) + 6 dt (j0 + j1)) / dt^3
        const double n3 = add(mul(12.0, sub(o[c], f[c])), mul(mul(6.0, dt1), add(o[3 + c], f[3 + c])));
        a2[c] = p2 ? mul(n2, i2) : dvd(n2, dt2);
        a3[c] = p2 ? mul(n3, i3) : dvd(n3, dt3);
    }
    const double c24 = p2 ? mul(dt4, 0x1.5555555555555p-5) : dvd(dt4, 24.0);
    const double c120 = p2 ? mul(dt5, 0x1.1111111111111p-7) : dvd(dt5, 120.0);
    const double c6 = p2 ? mul(dt3, 0x1.5555555555555p-3) : dvd(dt3, 6.0);
    r.x = add(add(p.x, mul(c24, a2[0])), mul(c120, a3[0]));
    r.y = add(add(p.y, mul(c24, a2[1])), mul(c120, a3[1]));
    r.z = add(add(p.z, mul(c24, a2[2])), mul(c120, a3[2]));
    v.x = add(add(pv.x, mul(c6, a2[0])), mul(c24, a3[0]));
    v.y = add(add(pv.y, mul(c6, a2[1])), mul(c24, a3[1]));
    v.z = add(add(pv.z, mul(c6, a2[2])), mul(c24, a3[2]));
    // get_timestep_normal with the step's old dt
    const double ax1 = add(a2[0], mul(dt1, a3[0]));
    const double ay1 = add(a2[1], mul(dt1, a3[1]));
    const double az1 = add(a2[2], mul(dt1, a3[2]));
    const double abs_a1 = magnitude(f[0], f[1], f[2]);
    const double abs_j1 = magnitude(f[3], f[4], f[5]);
    const double abs_j12 = mul(abs_j1, abs_j1);
    const double abs_a1_3 = magnitude(a3[0], a3[1], a3[2]);
    const double abs_a1_2 = magnitude(ax1, ay1, az1);
    const double abs_a1_22 = mul(abs_a1_2, abs_a1_2);
    const double normal_dt =
        __dsqrt_rn(mul(eta, dvd(add(mul(abs_a1, abs_a1_2), abs_j12), add(mul(abs_j1, abs_a1_3), abs_a1_22))));
    new_dt = normalize_dt(normal_dt, dt1, itime, dt_min, dt_max);
    return isfinite(r.x) && isfinite(r.y) && isfinite(r.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
}

// (int) of a double as x86-64 converts it (NaN and out-of-range -> INT_MIN);
// the reference relies on that for particles without jerk (Hermite4.cpp:124).
__device__ __forceinline__ int trunc_to_int_x86(double x) {
    if (!(x > -2147483649.0 && x < 2147483648.0)) return INT_MIN;
    return (int)x;
}

// Hermite4::init_dt (Hermite4.cpp:112-131) for one particle.
__device__ __forceinline__ double init_dt(const double *f, double eta, double dt_min, double dt_max) {
    const double a2 = magnitude(f[0], f[1], f[2]);
    const double j2 = magnitude(f[3], f[4], f[5]);
    double tmp = mul(eta, dvd(a2, j2));
    // log(2.0), correctly rounded: 0x3FE62E42FEFA39EF
    const int ex = trunc_to_int_x86(sub(ceil(dvd(log(tmp), 0x1.62e42fefa39efp-1)), 1.0));
    tmp = ldexp(1.0, ex);   // pow(2, ex): exact
    if (tmp < dt_min)
        tmp = dt_min;
    else if (tmp > dt_max)
        tmp = dt_max;
    return tmp;
}

// ---- j-split partial forces -------------------------------------------------
// The force kernels leave, for active particle k and j-chunk s, the partial sum
// of component c at part[(s * 6 + c) * nact + k].  Their sum is formed in one
// of two fixed orders, chosen by the chunk count S alone:
//  * a thread per particle adds the chunks in chunk order;
//  * with many chunks (S >= WARP_REDUCE_MIN_S, small active sets) a warp per
//    particle does it: lane l adds chunks l, l + 32, ... in order, then a
//    fixed shuffle tree.  A chain of S dependent FP64 additions per thread
//    would otherwise, at GB300's FP64 rate, take longer than the force sum
//    of a small active set.
constexpr unsigned WARP_REDUCE_MIN_S = 32;

__device__ __forceinline__ bool warp_reduce(unsigned S) { return S >= WARP_REDUCE_MIN_S; }

__device__ __forceinline__ void sum_partials_thread(const double *part, unsigned nact, unsigned k, unsigned S,
                                                    double out[6]) {
#pragma unroll
    for (int c = 0; c < 6; c++) out[c] = 0.0;
    for (unsigned s = 0; s < S; s++) {
        const double *p = part + (size_t)s * 6 * nact;
#pragma unroll
        for (int c = 0; c < 6; c++) out[c] = add(out[c], p[(size_t)c * nact + k]);
    }
}

// All 32 lanes call it with the same k; the sum is in lane 0.
__device__ __forceinline__ void sum_partials_warp(const double *part, unsigned nact, unsigned k, unsigned S, int lane,
                                                  double out[6]) {
#pragma unroll
    for (int c = 0; c < 6; c++) out[c] = 0.0;
    for (unsigned s = lane; s < S; s += 32) {
        const double *p = part + (size_t)s * 6 * nact;
#pragma unroll
        for (int c = 0; c < 6; c++) out[c] = add(out[c], p[(size_t)c * nact + k]);
    }
#pragma unroll
    for (int c = 0; c < 6; c++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) out[c] = add(out[c], __shfl_down_sync(0xffffffffu, out[c], o));
}

}  // namespace exact
}  // namespace h4
