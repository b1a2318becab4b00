// Pair arithmetic and warp work items of the force sum, shared by the
// single-system force kernels and the ensemble kernel.
//
// A warp item is (up to 4 active particles, one j range): the 32 lanes take
// interleaved j, every lane keeps the sums of all the item's particles, and a
// fixed butterfly reduce-scatter combines the lanes at the end
// (deterministic).  Results
// go to part_s[c * nact + k] (component c of active particle k, for this
// j-chunk).  Indices in `move` and j are relative to the arrays passed.
#pragma once
#include "h4_internal.cuh"

// j-loop unroll of the FP64 and mixed warp items (build knobs, defaults as
// measured best on GB300: 1 and 2).
#ifndef H4_FP64_JUNROLL
#define H4_FP64_JUNROLL 1
#endif
#ifndef H4_MIXED_JUNROLL
#define H4_MIXED_JUNROLL 2
#endif
// j-loop unroll of the packed-pair mixed warp item (1: it then fits the
// 128 registers a thread of the two-blocks-per-SM ensemble kernel has).
#ifndef H4_MIXED_X2_JUNROLL
#define H4_MIXED_X2_JUNROLL 1
#endif

namespace h4 {
namespace pair {

constexpr int kFp64JUnroll = H4_FP64_JUNROLL;
constexpr int kMixedJUnroll = H4_MIXED_JUNROLL;
constexpr int kMixedX2JUnroll = H4_MIXED_X2_JUNROLL;

// 1/sqrt(x) in FP64: hardware reciprocal-square-root approximation
// (rsqrt.approx.f64) refined by one cubic Householder step,
// y = y0 (1 + e/2 + 3e^2/8) with e = 1 - x y0^2.
__device__ __forceinline__ double rsqrt_refined(double x) {
    double y0;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
    const double e = fma(-x, y0 * y0, 1.0);
    return fma(y0 * e, fma(e, 0.375, 0.5), y0);
}

// FP64 pair (Hermite4CPU::force_calculation, Hermite4CPU.cpp:55-82), written
// as a = A dr, a1 = A (dv - 3 (dr.dv)/r^2 dr), A = m / r^3: 31 FP64
// instructions.  The self pair (j == i) is skipped by a select, as the
// reference skips it (Hermite4CPU.cpp:328).
__device__ __forceinline__ void pair_fp64(double xi, double yi, double zi, double vxi, double vyi, double vzi,
                                          const dbl4 &pj, const dbl4 &vj, double e2, bool self, double acc[6]) {
    const double dx = pj.x - xi, dy = pj.y - yi, dz = pj.z - zi;
    const double dvx = vj.x - vxi, dvy = vj.y - vyi, dvz = vj.z - vzi;
    double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, e2)));
    double m = pj.w;
    r2 = self ? 1.0 : r2;
    m = self ? 0.0 : m;
    const double rinv = rsqrt_refined(r2);
    const double r2inv = rinv * rinv;
    const double A = (m * rinv) * r2inv;
    const double rv = fma(dx, dvx, fma(dy, dvy, dz * dvz));
    const double eta = rv * (-3.0 * r2inv);
    acc[0] = fma(A, dx, acc[0]);
    acc[1] = fma(A, dy, acc[1]);
    acc[2] = fma(A, dz, acc[2]);
    acc[3] = fma(A, fma(eta, dx, dvx), acc[3]);
    acc[4] = fma(A, fma(eta, dy, dvy), acc[4]);
    acc[5] = fma(A, fma(eta, dz, dvz), acc[5]);
}

// ---- lane sums of a warp item ---------------------------------------------------
// A warp item ends with 6 * NI sums per lane to be added over the 32 lanes.
// A shuffle tree per value costs 5 additions per value; a butterfly
// reduce-scatter costs 31 in all for 32 values: at offset o each lane keeps
// half of its values, adds the partner's copies of them, and sends the other
// half.  With V = 2^L values, lane t ends holding the total of value
// t >> (5 - L) (the lanes that share it hold the same total), in a fixed
// order.  On GB300 this matters: the FP64 pipe runs a warp-wide addition at
// 1/64 of the FP32 rate, and the per-value trees cost as much as the pair
// arithmetic of a short j-chunk.

// Smallest power of two >= x (x <= 32).
__host__ __device__ constexpr int pow2_ceil(int x) { return x <= 1 ? 1 : 2 * pow2_ceil((x + 1) / 2); }
__host__ __device__ constexpr int log2_exact(int x) { return x <= 1 ? 0 : 1 + log2_exact(x / 2); }

template <int V, int O>
__device__ __forceinline__ void rs_sum_f64(double *v, int lane) {
    if constexpr (O > 0) {
        if constexpr (V > 1) {
            const bool upper = (lane & O) != 0;
#pragma unroll
            for (int k = 0; k < V / 2; k++) {
                const double send = upper ? v[k] : v[k + V / 2];
                const double keep = upper ? v[k + V / 2] : v[k];
                v[k] = keep + __shfl_xor_sync(0xffffffffu, send, O);
            }
            rs_sum_f64<V / 2, O / 2>(v, lane);
        } else {
            v[0] = v[0] + __shfl_xor_sync(0xffffffffu, v[0], O);
            rs_sum_f64<1, O / 2>(v, lane);
        }
    }
}

// Error-free sum (Knuth's TwoSum): s + e == a + b exactly, for any order of
// magnitudes.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// (h + l) += (h2 + l2) in double-single arithmetic (a float pair), renormalised.
__device__ __forceinline__ void ds_add(float &h, float &l, float h2, float l2) {
    float s, e;
    two_sum(h, h2, s, e);
    e = e + (l + l2);
    h = s + e;
    l = e - (h - s);
}

template <int V, int O>
__device__ __forceinline__ void rs_sum_ds(float *h, float *l, int lane) {
    if constexpr (O > 0) {
        if constexpr (V > 1) {
            const bool upper = (lane & O) != 0;
#pragma unroll
            for (int k = 0; k < V / 2; k++) {
                const float sh = upper ? h[k] : h[k + V / 2], sl = upper ? l[k] : l[k + V / 2];
                float kh = upper ? h[k + V / 2] : h[k], kl = upper ? l[k + V / 2] : l[k];
                ds_add(kh, kl, __shfl_xor_sync(0xffffffffu, sh, O), __shfl_xor_sync(0xffffffffu, sl, O));
                h[k] = kh;
                l[k] = kl;
            }
            rs_sum_ds<V / 2, O / 2>(h, l, lane);
        } else {
            ds_add(h[0], l[0], __shfl_xor_sync(0xffffffffu, h[0], O), __shfl_xor_sync(0xffffffffu, l[0], O));
            rs_sum_ds<1, O / 2>(h, l, lane);
        }
    }
}

// Value index held by `lane` after a reduce-scatter of V values, and whether
// the lane is the first of those holding it.
template <int V>
__device__ __forceinline__ int rs_index(int lane) { return lane >> (5 - log2_exact(V)); }
template <int V>
__device__ __forceinline__ bool rs_first(int lane) { return (lane & ((32 / V) - 1)) == 0; }

template <int NI>
__device__ __forceinline__ void fp64_warp_item(const dbl4 *__restrict__ pr, const dbl4 *__restrict__ pv,
                                               const unsigned *__restrict__ move, unsigned nact, unsigned k0,
                                               int j_begin, int j_end, double e2, double *part_s, int lane) {
    double xi[NI], yi[NI], zi[NI], vxi[NI], vyi[NI], vzi[NI];
    unsigned idx[NI];
    double acc[NI][6];
#pragma unroll
    for (int q = 0; q < NI; q++) {
        idx[q] = move[k0 + q];
        const dbl4 p = pr[idx[q]], v = pv[idx[q]];
        xi[q] = p.x; yi[q] = p.y; zi[q] = p.z;
        vxi[q] = v.x; vyi[q] = v.y; vzi[q] = v.z;
#pragma unroll
        for (int c = 0; c < 6; c++) acc[q][c] = 0.0;
    }
#pragma unroll kFp64JUnroll
    for (int j = j_begin + lane; j < j_end; j += 32) {
        const dbl4 pj = pr[j], vj = pv[j];
#pragma unroll
        for (int q = 0; q < NI; q++)
            pair_fp64(xi[q], yi[q], zi[q], vxi[q], vyi[q], vzi[q], pj, vj, e2, (unsigned)j == idx[q], acc[q]);
    }
    // value c * NI + q = component c of particle q; zero padding to V
    constexpr int V = pow2_ceil(6 * NI);
    double val[V];
#pragma unroll
    for (int x = 0; x < V; x++) val[x] = x < 6 * NI ? acc[x % NI][x / NI] : 0.0;
    rs_sum_f64<V, 16>(val, lane);
    const int x = rs_index<V>(lane);
    if (rs_first<V>(lane) && x < 6 * NI) part_s[(size_t)(x / NI) * nact + k0 + (x % NI)] = val[0];
}

// Bounds-checked build: every range one single-system warp item touches --
// its slice of the active list, the particle indices in it, its j range and
// its slice of the partial-force area ([S][6][nact]).  Warp-uniform result.
__device__ __forceinline__ bool warp_item_ok(const H4Dev &d, unsigned nact, unsigned k0, unsigned cnt, int j_begin,
                                             int j_end, unsigned s, int lane, unsigned site_j) {
    bool ok = range_ok(d, BS_NACT, 0, nact, d.n) && range_ok(d, BS_FP64_K, k0, (long long)k0 + cnt, nact) &&
              range_ok(d, site_j, j_begin, j_end, d.n) &&
              range_ok(d, BS_PART, 6ll * nact * s, 6ll * nact * (s + 1), (long long)d.part_cap);
    if (ok && (unsigned)lane < cnt) {
        const unsigned i = d.move[k0 + lane];
        ok = range_ok(d, BS_MOVE, i, i + 1ll, d.n);
    }
    return __all_sync(0xffffffffu, ok);
}

// Bit-identical restatement of the reference's per-particle sum (one thread,
// j ascending, the reference's operation order, IEEE sqrt and division).
__device__ __forceinline__ void exact_sum(const dbl4 *__restrict__ pr, const dbl4 *__restrict__ pv, int n,
                                          unsigned i, double e2, double f[6]) {
    const dbl4 pi = pr[i], vi = pv[i];
#pragma unroll
    for (int c = 0; c < 6; c++) f[c] = 0.0;
    for (int j = 0; j < n; j++) {
        if ((unsigned)j == i) continue;
        const dbl4 pj = pr[j], vj = pv[j];
        const double rx = __dadd_rn(pj.x, -pi.x), ry = __dadd_rn(pj.y, -pi.y), rz = __dadd_rn(pj.z, -pi.z);
        const double vx = __dadd_rn(vj.x, -vi.x), vy = __dadd_rn(vj.y, -vi.y), vz = __dadd_rn(vj.z, -vi.z);
        const double r2 =
            __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)), e2);
        const double rinv = __ddiv_rn(1.0, __dsqrt_rn(r2));
        const double r2inv = __dmul_rn(rinv, rinv);
        const double r3inv = __dmul_rn(r2inv, rinv);
        const double r5inv = __dmul_rn(r2inv, r3inv);
        const double mr3inv = __dmul_rn(r3inv, pj.w);
        const double mr5inv = __dmul_rn(r5inv, pj.w);
        const double rv = __dadd_rn(__dadd_rn(__dmul_rn(rx, vx), __dmul_rn(ry, vy)), __dmul_rn(rz, vz));
        const double rv3 = __dmul_rn(3.0, rv);
        f[0] = __dadd_rn(f[0], __dmul_rn(rx, mr3inv));
        f[1] = __dadd_rn(f[1], __dmul_rn(ry, mr3inv));
        f[2] = __dadd_rn(f[2], __dmul_rn(rz, mr3inv));
        f[3] = __dadd_rn(f[3], __dadd_rn(__dmul_rn(vx, mr3inv), -__dmul_rn(__dmul_rn(rv3, rx), mr5inv)));
        f[4] = __dadd_rn(f[4], __dadd_rn(__dmul_rn(vy, mr3inv), -__dmul_rn(__dmul_rn(rv3, ry), mr5inv)));
        f[5] = __dadd_rn(f[5], __dadd_rn(__dmul_rn(vz, mr3inv), -__dmul_rn(__dmul_rn(rv3, rz), mr5inv)));
    }
}

// ---- mixed precision ----------------------------------------------------------

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

struct IParticle {
    float xh, yh, zh, xl, yl, zl, vx, vy, vz;
};

__device__ __forceinline__ IParticle load_i(const float4 *jf0, const float4 *jf1, const float4 *jf2, unsigned i) {
    const float4 a = jf0[i], b = jf1[i], c = jf2[i];
    IParticle p;
    p.xh = a.x; p.yh = a.y; p.zh = a.z;
    p.xl = b.x; p.yl = b.y; p.zl = b.z;
    p.vx = c.x; p.vy = c.y; p.vz = c.z;
    return p;
}

// One pair, FP32 after the double-single difference of the positions.  With
// e2 = 0 the self term is masked explicitly; with e2 > 0 it is an exact zero
// (dr = dv = 0).
template <bool MASK_SELF>
__device__ __forceinline__ void pair_mixed(const IParticle &p, float4 j0, float4 j1, float4 j2, float e2,
                                           bool self, float sum[6]) {
    const float dx = (j0.x - p.xh) + (j1.x - p.xl);
    const float dy = (j0.y - p.yh) + (j1.y - p.yl);
    const float dz = (j0.z - p.zh) + (j1.z - p.zl);
    const float dvx = j2.x - p.vx, dvy = j2.y - p.vy, dvz = j2.z - p.vz;
    float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, e2)));
    float m = j0.w;
    if (MASK_SELF) {
        r2 = self ? 1.0f : r2;
        m = self ? 0.0f : m;
    }
    float rinv;   // hardware approximation (MUFU), no denormal range handling
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rinv) : "f"(r2));
    const float r2inv = rinv * rinv;
    const float A = (m * rinv) * r2inv;
    const float rv = fmaf(dx, dvx, fmaf(dy, dvy, dz * dvz));
    const float eta = rv * (-3.0f * r2inv);
    sum[0] = fmaf(A, dx, sum[0]);
    sum[1] = fmaf(A, dy, sum[1]);
    sum[2] = fmaf(A, dz, sum[2]);
    sum[3] = fmaf(A, fmaf(eta, dx, dvx), sum[3]);
    sum[4] = fmaf(A, fmaf(eta, dy, dvy), sum[4]);
    sum[5] = fmaf(A, fmaf(eta, dz, dvz), sum[5]);
}

// Mixed warp item: FP32 lane sums over runs of 16 j, Kahan-compensated
// across runs, double-single reduce-scatter across lanes, one FP64 value per
// lane at the end.
template <int NI, bool MASK_SELF>
__device__ __forceinline__ void mixed_warp_item(const float4 *__restrict__ jf0, const float4 *__restrict__ jf1,
                                                const float4 *__restrict__ jf2, const unsigned *__restrict__ move,
                                                unsigned nact, unsigned k0, int j_begin, int j_end, float e2,
                                                double *part_s, int lane) {
    IParticle ip[NI];
    unsigned idx[NI];
    float S[NI][6], C[NI][6];
#pragma unroll
    for (int q = 0; q < NI; q++) {
        idx[q] = move[k0 + q];
        ip[q] = load_i(jf0, jf1, jf2, idx[q]);
#pragma unroll
        for (int c = 0; c < 6; c++) { S[q][c] = 0.f; C[q][c] = 0.f; }
    }
    for (int jb = j_begin; jb < j_end; jb += 32 * 16) {
        float part[NI][6];
#pragma unroll
        for (int q = 0; q < NI; q++)
#pragma unroll
            for (int c = 0; c < 6; c++) part[q][c] = 0.f;
        const int jl = min(j_end, jb + 32 * 16);
#pragma unroll kMixedJUnroll
        for (int j = jb + lane; j < jl; j += 32) {
            const float4 j0 = jf0[j], j1 = jf1[j], j2 = jf2[j];
#pragma unroll
            for (int q = 0; q < NI; q++) pair_mixed<MASK_SELF>(ip[q], j0, j1, j2, e2, (unsigned)j == idx[q], part[q]);
        }
#pragma unroll
        for (int q = 0; q < NI; q++)
#pragma unroll
            for (int c = 0; c < 6; c++) kahan_add(S[q][c], C[q][c], part[q][c]);
    }
    // Kahan pairs (value S - C) summed over the lanes in double-single FP32;
    // value c * NI + q = component c of particle q; zero padding to V
    constexpr int V = pow2_ceil(6 * NI);
    float h[V], l[V];
#pragma unroll
    for (int x = 0; x < V; x++) {
        h[x] = x < 6 * NI ? S[x % NI][x / NI] : 0.f;
        l[x] = x < 6 * NI ? -C[x % NI][x / NI] : 0.f;
    }
    rs_sum_ds<V, 16>(h, l, lane);
    const int x = rs_index<V>(lane);
    if (rs_first<V>(lane) && x < 6 * NI)
        part_s[(size_t)(x / NI) * nact + k0 + (x % NI)] = (double)h[0] + (double)l[0];
}

// ---- packed f32x2 arithmetic (sm_100+) ---------------------------------------
// Two active particles share one 64-bit register pair; every FP32 operation of
// pair_mixed becomes one packed instruction.  Same arithmetic per lane.

typedef unsigned long long f2;

__device__ __forceinline__ f2 pk2(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float lo2(f2 v) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return a;
}
__device__ __forceinline__ float hi2(f2 v) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return b;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f2 rsqrt2(f2 v) {
    float a, b, ra, rb;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(ra) : "f"(a));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(b));
    return pk2(ra, rb);
}
struct IPair {   // two active particles, packed
    f2 xh, yh, zh, xl, yl, zl, vx, vy, vz;
};

__device__ __forceinline__ void kahan2(f2 &s, f2 &c, f2 x) {
    const f2 y = sub2(x, c);
    const f2 t = add2(s, y);
    c = sub2(sub2(t, s), y);
    s = t;
}

__device__ __forceinline__ IPair pack_pair(const IParticle &a, const IParticle &b) {
    IPair p;
    p.xh = pk2(a.xh, b.xh); p.yh = pk2(a.yh, b.yh); p.zh = pk2(a.zh, b.zh);
    p.xl = pk2(a.xl, b.xl); p.yl = pk2(a.yl, b.yl); p.zl = pk2(a.zl, b.zl);
    p.vx = pk2(a.vx, b.vx); p.vy = pk2(a.vy, b.vy); p.vz = pk2(a.vz, b.vz);
    return p;
}

__device__ __forceinline__ void pair_x2(const IPair &p, f2 jxh, f2 jyh, f2 jzh, f2 jm, f2 jxl, f2 jyl, f2 jzl,
                                        f2 jvx, f2 jvy, f2 jvz, f2 e2, f2 m3, f2 sum[6]) {
    const f2 dx = add2(sub2(jxh, p.xh), sub2(jxl, p.xl));
    const f2 dy = add2(sub2(jyh, p.yh), sub2(jyl, p.yl));
    const f2 dz = add2(sub2(jzh, p.zh), sub2(jzl, p.zl));
    const f2 dvx = sub2(jvx, p.vx), dvy = sub2(jvy, p.vy), dvz = sub2(jvz, p.vz);
    const f2 r2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
    const f2 rinv = rsqrt2(r2);
    const f2 r2inv = mul2(rinv, rinv);
    const f2 A = mul2(mul2(jm, rinv), r2inv);
    const f2 rv = fma2(dx, dvx, fma2(dy, dvy, mul2(dz, dvz)));
    const f2 eta = mul2(rv, mul2(m3, r2inv));
    sum[0] = fma2(A, dx, sum[0]);
    sum[1] = fma2(A, dy, sum[1]);
    sum[2] = fma2(A, dz, sum[2]);
    sum[3] = fma2(A, fma2(eta, dx, dvx), sum[3]);
    sum[4] = fma2(A, fma2(eta, dy, dvy), sum[4]);
    sum[5] = fma2(A, fma2(eta, dz, dvz), sum[5]);
}

// Mixed warp item of two active particles (k0, k0 + 1) held as one packed
// f32x2 pair: the lanes take interleaved j straight from L2 as
// mixed_warp_item does, and every FP32 operation of the pair formula is one
// packed instruction for both particles (the j values are duplicated into
// both halves of a register pair).  Needs e2 > 0 (the self term is then an
// exact zero).  Same sums as mixed_warp_item: FP32 over runs of 16 j per
// lane, Kahan across runs, double-single reduce-scatter across lanes.
__device__ __forceinline__ void mixed_warp_item_x2(const float4 *__restrict__ jf0, const float4 *__restrict__ jf1,
                                                   const float4 *__restrict__ jf2, const unsigned *__restrict__ move,
                                                   unsigned nact, unsigned k0, int j_begin, int j_end, float e2f,
                                                   double *part_s, int lane) {
    const IPair ip = pack_pair(load_i(jf0, jf1, jf2, move[k0]), load_i(jf0, jf1, jf2, move[k0 + 1]));
    const f2 e2 = pk2(e2f, e2f), m3 = pk2(-3.0f, -3.0f);
    f2 S[6], Cc[6];
#pragma unroll
    for (int c = 0; c < 6; c++) { S[c] = 0ull; Cc[c] = 0ull; }
    for (int jb = j_begin; jb < j_end; jb += 32 * 16) {
        f2 part[6];
#pragma unroll
        for (int c = 0; c < 6; c++) part[c] = 0ull;
        const int jl = min(j_end, jb + 32 * 16);
#pragma unroll kMixedX2JUnroll
        for (int j = jb + lane; j < jl; j += 32) {
            const float4 a = jf0[j], b = jf1[j], c = jf2[j];
            pair_x2(ip, pk2(a.x, a.x), pk2(a.y, a.y), pk2(a.z, a.z), pk2(a.w, a.w), pk2(b.x, b.x), pk2(b.y, b.y),
                    pk2(b.z, b.z), pk2(c.x, c.x), pk2(c.y, c.y), pk2(c.z, c.z), e2, m3, part);
        }
#pragma unroll
        for (int c = 0; c < 6; c++) kahan2(S[c], Cc[c], part[c]);
    }
    // value c * 2 + q = component c of particle q; zero padding to 16
    float h[16], l[16];
#pragma unroll
    for (int c = 0; c < 6; c++) {
        h[2 * c] = lo2(S[c]);
        h[2 * c + 1] = hi2(S[c]);
        l[2 * c] = -lo2(Cc[c]);
        l[2 * c + 1] = -hi2(Cc[c]);
    }
#pragma unroll
    for (int x = 12; x < 16; x++) { h[x] = 0.f; l[x] = 0.f; }
    rs_sum_ds<16, 16>(h, l, lane);
    const int x = rs_index<16>(lane);
    if (rs_first<16>(lane) && x < 12) part_s[(size_t)(x >> 1) * nact + k0 + (x & 1)] = (double)h[0] + (double)l[0];
}

}  // namespace pair
}  // namespace h4
