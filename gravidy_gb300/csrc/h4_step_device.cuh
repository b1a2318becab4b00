// Per-particle pieces of the block step (h4_step_kernels.cu): the predictor,
// the fused reduction + corrector, and the j data of the mixed form.
// Grid-wide loops use the launch's gridDim/blockDim.
#pragma once
#include "h4_exact.cuh"
#include "h4_internal.cuh"

namespace h4 {
namespace step {

// Packed FP32 j data of the mixed kernels, from predicted position/velocity.
__device__ __forceinline__ void write_jf(const H4Dev &d, int i, const dbl4 &pr, const dbl4 &pv) {
    float4 a, b, c;
    exact::pack_jf(pr, pv, a, b, c);
    d.jf0[i] = a;
    d.jf1[i] = b;
    d.jf2[i] = c;
    if (d.jd) {
        const size_t np = (size_t)d.n_pad;
        d.jd[i] = make_float4(a.x, a.x, a.y, a.y);
        d.jd[np + i] = make_float4(a.z, a.z, a.w, a.w);
        d.jd[2 * np + i] = make_float4(b.x, b.x, b.y, b.y);
        d.jd[3 * np + i] = make_float4(b.z, b.z, c.x, c.x);
        d.jd[4 * np + i] = make_float4(c.y, c.y, c.z, c.z);
    }
}

// ---- Hermite4CPU::predicted_pos_vel (Hermite4CPU.cpp:340-365) ---------------
__device__ __forceinline__ void predict_particle(const H4Dev &d, int i, double itime) {
    dbl4 pr, pv;
    exact::predict(itime, d.t[i], d.f + 6 * (size_t)i, d.r[i], d.v[i], pr, pv);
    d.pr[i] = pr;
    d.pv[i] = pv;
    if (d.mixed) write_jf(d, i, pr, pv);
}

// Calls body(k, f) for every active particle k with the sum f of its j-split
// partial forces, over the whole grid: a thread per particle, or a warp per
// particle with body called by lane 0 (exact::warp_reduce(S)).  blockDim is a
// multiple of 32.
template <class Body>
__device__ __forceinline__ void for_each_reduced(const H4Dev &d, unsigned nact, unsigned S, Body body) {
    const unsigned gt = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    if (exact::warp_reduce(S)) {
        const int lane = threadIdx.x & 31;
        for (unsigned k = gt >> 5; k < nact; k += nt >> 5) {
            double f[6];
            exact::sum_partials_warp(d.part, nact, k, S, lane, f);
            if (lane == 0) body(k, f);
        }
    } else {
        for (unsigned k = gt; k < nact; k += nt) {
            double f[6];
            exact::sum_partials_thread(d.part, nact, k, S, f);
            body(k, f);
        }
    }
}

// The active list and the partial-force area the reduction reads (checked
// build only).
__device__ __forceinline__ bool reduce_ranges_ok(const H4Dev &d, unsigned nact, unsigned S) {
    return range_ok(d, BS_NACT, 0, nact, d.n) && range_ok(d, BS_PART, 0, 6ll * nact * S, (long long)d.part_cap);
}

// ---- Hermite4CPU::correction_pos_vel (Hermite4CPU.cpp:370-411) --------------
// with NbodyUtils::get_timestep_normal (NbodyUtils.cpp:337-365).
// fn: the new forces when the reduction is fused here, else null (the forces
// were reduced into d.f and the old ones saved by k_reduce_forces).
__device__ __forceinline__ void correct_particle(const H4Dev &d, unsigned k, double itime, const double *fn) {
    const unsigned i = d.move[k];
    if (!range_ok(d, BS_MOVE, i, i + 1ll, d.n)) return;
    double *fp = d.f + 6 * (size_t)i;
    double *op = d.old + 6 * (size_t)i;
    double f[6], o[6];
    if (fn) {
#pragma unroll
        for (int c = 0; c < 6; c++) { f[c] = fn[c]; o[c] = fp[c]; op[c] = o[c]; fp[c] = f[c]; }
    } else {
#pragma unroll
        for (int c = 0; c < 6; c++) { f[c] = fp[c]; o[c] = op[c]; }
    }
    dbl4 r = d.r[i], v = d.v[i];
    double a2[3], a3[3], ndt;
    const bool ok = exact::correct(itime, d.eta, d.dt_min, d.dt_max, f, o, d.pr[i], d.pv[i], d.dt[i], r, v,
                                   a2, a3, ndt);
    d.r[i] = r;
    d.v[i] = v;
#pragma unroll
    for (int c = 0; c < 3; c++) { d.a2[3 * (size_t)i + c] = a2[c]; d.a3[3 * (size_t)i + c] = a3[c]; }
    d.t[i] = itime;
    d.dt[i] = ndt;
    if (!ok) atomicOr(&d.ctrl->err, (unsigned)H4_ERRBIT_NONFINITE);
}

}  // namespace step
}  // namespace h4
