// Cluster diagnostics on the device: center of density, core, half-mass and
// Lagrange radii (src/include/utils/NbodyUtils.cpp:108-328).
//
// The reference computes the center of density by sorting, for every
// particle, its distances to all others (O(N^2 log N) on the host) to take
// the 6th neighbour.  Here one thread per particle scans all j (j tiles in
// shared memory) and keeps its 8 nearest candidates by an FP32 squared
// distance taken from double-single positions; the 8 candidates' distances are
// then recomputed in FP64 exactly as the reference does and ranked, so the
// 6th-neighbour distance is the reference's value (the FP32 pass only has to
// keep the true 6 among 8, i.e. fail only for three distances within ~1e-7
// of each other).  The density and the mass-radius scans keep the reference's
// float/double types and sequential summation order (single-thread passes:
// the float sums are order dependent), and the radii are ordered by a bitonic
// sort.  Diagnostics only: nothing here feeds back into the dynamics.
#include <cmath>
#include <string>

#include "../../include/gravidy_gb300.h"
#include "h4_internal.cuh"

namespace h4 {
namespace diag {

constexpr int T = 256;
constexpr int KNN = 8;

__global__ void k_pack_positions(const dbl4 *r, float4 *hi, float4 *lo, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const dbl4 p = r[i];
    float4 a, b;
    a.x = __double2float_rn(p.x); b.x = __double2float_rn(p.x - (double)a.x);
    a.y = __double2float_rn(p.y); b.y = __double2float_rn(p.y - (double)a.y);
    a.z = __double2float_rn(p.z); b.z = __double2float_rn(p.z - (double)a.z);
    a.w = 0.f; b.w = 0.f;
    hi[i] = a;
    lo[i] = b;
}

// Density of every particle from its 6th-neighbour distance
// (get_center_of_density, NbodyUtils.cpp:172-200), float as the reference.
__global__ void __launch_bounds__(T) k_knn_density(const dbl4 *r, const float4 *hi, const float4 *lo, int n,
                                                   double *p) {
    __shared__ float4 sh[T], sl[T];
    const int i = blockIdx.x * T + threadIdx.x;
    const bool valid = i < n;
    float4 ih = make_float4(0.f, 0.f, 0.f, 0.f), il = ih;
    if (valid) { ih = hi[i]; il = lo[i]; }
    float bd[KNN];
    int bj[KNN];
#pragma unroll
    for (int k = 0; k < KNN; k++) { bd[k] = INFINITY; bj[k] = -1; }
    for (int j0 = 0; j0 < n; j0 += T) {
        const int jl = j0 + threadIdx.x;
        if (jl < n) { sh[threadIdx.x] = hi[jl]; sl[threadIdx.x] = lo[jl]; }
        __syncthreads();
        const int cnt = min(T, n - j0);
        for (int jj = 0; jj < cnt; jj++) {
            const float4 a = sh[jj], b = sl[jj];
            const float dx = (a.x - ih.x) + (b.x - il.x);
            const float dy = (a.y - ih.y) + (b.y - il.y);
            const float dz = (a.z - ih.z) + (b.z - il.z);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const int j = j0 + jj;
            if (d2 < bd[KNN - 1] && j != i) {
                // insert into the sorted candidate list
                float v = d2;
                int vj = j;
#pragma unroll
                for (int k = 0; k < KNN; k++) {
                    if (v < bd[k]) {
                        const float tv = bd[k]; const int tj = bj[k];
                        bd[k] = v; bj[k] = vj;
                        v = tv; vj = tj;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!valid) return;
    // exact distances of the candidates, as the reference computes them
    double e[KNN];
    const dbl4 pi = r[i];
#pragma unroll
    for (int k = 0; k < KNN; k++) {
        if (bj[k] < 0) { e[k] = INFINITY; continue; }
        const dbl4 pj = r[bj[k]];
        const double rx = __dadd_rn(pj.x, -pi.x), ry = __dadd_rn(pj.y, -pi.y), rz = __dadd_rn(pj.z, -pi.z);
        e[k] = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)));
    }
    // the 6th smallest (d[J] with the self entry at d[0], J = 6)
#pragma unroll
    for (int a = 0; a < KNN; a++)
#pragma unroll
        for (int b = 0; b < KNN - 1 - a; b++)
            if (e[b] > e[b + 1]) { const double t = e[b]; e[b] = e[b + 1]; e[b + 1] = t; }
    const float radius = (float)e[5];
    const float aa = (float)(5.0 * pi.w);                       // (J - 1) * m
    const double bbd = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, 3.14159265358979323846),
                                                               (double)radius), (double)radius), (double)radius),
                                 3.0);
    const float bb = (float)bbd;
    p[i] = (double)__fdiv_rn(aa, bb);
}

// Center of density: float sum of the densities, double weighted positions,
// in particle order (NbodyUtils.cpp:203-219).
__global__ void k_cod_seq(const dbl4 *r, const double *p, int n, double *cod) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double cx = 0.0, cy = 0.0, cz = 0.0;
    float dsum = 0.f;
    for (int i = 0; i < n; i++) {
        const double w = p[i];
        const dbl4 x = r[i];
        dsum = (float)__dadd_rn((double)dsum, w);
        cx = __dadd_rn(cx, __dmul_rn(x.x, w));
        cy = __dadd_rn(cy, __dmul_rn(x.y, w));
        cz = __dadd_rn(cz, __dmul_rn(x.z, w));
    }
    cod[0] = __ddiv_rn(cx, (double)dsum);
    cod[1] = __ddiv_rn(cy, (double)dsum);
    cod[2] = __ddiv_rn(cz, (double)dsum);
}

// Distances to the center (get_radii, NbodyUtils.cpp:285-296), padded to a
// power of two with +inf for the sort.
__global__ void k_radii(const dbl4 *r, int n, int npow, double cx, double cy, double cz, double *key,
                        unsigned *val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npow) return;
    if (i < n) {
        const dbl4 p = r[i];
        const double rx = __dadd_rn(p.x, -cx), ry = __dadd_rn(p.y, -cy), rz = __dadd_rn(p.z, -cz);
        key[i] = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)));
        val[i] = (unsigned)i;
    } else {
        key[i] = INFINITY;
        val[i] = 0xFFFFFFFFu;
    }
}

// One compare-exchange pass of a bitonic sort (ascending by key, then index).
__global__ void k_bitonic(double *key, unsigned *val, int npow, int j, int k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npow) return;
    const int l = i ^ j;
    if (l <= i) return;
    const double ki = key[i], kl = key[l];
    const unsigned vi = val[i], vl = val[l];
    const bool gt = (ki > kl) || (ki == kl && vi > vl);
    const bool up = (i & k) == 0;
    if (up == gt) {
        key[i] = kl; key[l] = ki;
        val[i] = vl; val[l] = vi;
    }
}

// Core radius (> CORE_MASS of the mass, double sum), half-mass radius (>= half,
// float sum) and Lagrange radii (float sum, at most one layer per particle)
// over the sorted radii (NbodyUtils.cpp:108-143, 223-260, 299-328).
__global__ void k_radii_scan(const double *key, const unsigned *val, const dbl4 *r, int n, float total_mass,
                             double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float lag[6] = {0.01f, 0.05f, 0.1f, 0.2f, 0.5f, 0.75f};
    const float core_lim = total_mass * 0.1f;
    const double half_lim = (double)total_mass / 2.0;
    double core_mass = 0.0, core = 0.0;
    bool core_done = false, half_done = false;
    float half_mass = 0.f, tmp_mass = 0.f;
    int jh = 0, layer = 0;
    bool lag_done = false;
    double layers[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++) {
        const double m = r[val[i]].w;
        if (!core_done) {
            if (core_mass > (double)core_lim) { core = key[i - 1]; core_done = true; }
            else core_mass = __dadd_rn(core_mass, m);
        }
        if (!half_done) {
            if ((double)half_mass >= half_lim) { jh = i; half_done = true; }
            else half_mass = (float)__dadd_rn((double)half_mass, m);
        }
        if (!lag_done) {
            if (tmp_mass >= total_mass || layer >= 6) {
                lag_done = true;
            } else {
                if (tmp_mass > lag[layer]) { layers[layer] = key[i]; layer++; }
                tmp_mass = (float)__dadd_rn((double)tmp_mass, m);
            }
        }
        if (core_done && half_done && lag_done) break;
    }
    out[0] = core;
    out[1] = jh > 0 ? key[jh - 1] : 0.0;
    for (int k = 0; k < 6; k++) out[2 + k] = layers[k];
}

}  // namespace diag
}  // namespace h4

using namespace h4;

namespace {
thread_local std::string g_diag_err;
int dfail(int st, const std::string &m) {
    g_diag_err = m;
    return st;
}
}  // namespace

// The handle's device state is reached through the C ABI's download
// functions' counterpart: h4_internal_state (h4_capi.cu).
extern "C" int h4_internal_positions(h4_handle h, const void **r, int *n, void **stream);

extern "C" const char *h4_diag_last_error(void) { return g_diag_err.c_str(); }

extern "C" int h4_center_of_density(h4_handle h, double cod[3]) {
    if (!h || !cod) return dfail(H4_ERR_ARG, "h4_center_of_density: null argument");
    const void *rp = nullptr;
    int n = 0;
    void *sp = nullptr;
    int st = h4_internal_positions(h, &rp, &n, &sp);
    if (st) return st;
    if (n < 8) return dfail(H4_ERR_ARG, "h4_center_of_density: needs n >= 8 (6th neighbour)");
    const dbl4 *r = (const dbl4 *)rp;
    cudaStream_t s = (cudaStream_t)sp;
    float4 *hi = nullptr, *lo = nullptr;
    double *p = nullptr, *dc = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&hi, sizeof(float4) * n, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&lo, sizeof(float4) * n, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&p, sizeof(double) * n, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dc, sizeof(double) * 3, s);
    if (e == cudaSuccess) {
        const int b = (n + diag::T - 1) / diag::T;
        diag::k_pack_positions<<<b, diag::T, 0, s>>>(r, hi, lo, n);
        diag::k_knn_density<<<b, diag::T, 0, s>>>(r, hi, lo, n, p);
        diag::k_cod_seq<<<1, 32, 0, s>>>(r, p, n, dc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cod, dc, sizeof(double) * 3, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(hi, s);
    cudaFreeAsync(lo, s);
    cudaFreeAsync(p, s);
    cudaFreeAsync(dc, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return dfail(H4_ERR_CUDA, std::string("h4_center_of_density: ") + cudaGetErrorString(e));
    return H4_OK;
}

extern "C" int h4_mass_radii(h4_handle h, const double center[3], float total_mass, double *core, double *halfmass,
                             double lagrange[6]) {
    if (!h || !center) return dfail(H4_ERR_ARG, "h4_mass_radii: null argument");
    const void *rp = nullptr;
    int n = 0;
    void *sp = nullptr;
    int st = h4_internal_positions(h, &rp, &n, &sp);
    if (st) return st;
    const dbl4 *r = (const dbl4 *)rp;
    cudaStream_t s = (cudaStream_t)sp;
    int npow = 1;
    while (npow < n) npow <<= 1;
    double *key = nullptr, *dout = nullptr;
    unsigned *val = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&key, sizeof(double) * npow, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&val, sizeof(unsigned) * npow, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dout, sizeof(double) * 8, s);
    if (e == cudaSuccess) {
        const int b = (npow + diag::T - 1) / diag::T;
        diag::k_radii<<<b, diag::T, 0, s>>>(r, n, npow, center[0], center[1], center[2], key, val);
        for (int k = 2; k <= npow; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) diag::k_bitonic<<<b, diag::T, 0, s>>>(key, val, npow, j, k);
        diag::k_radii_scan<<<1, 32, 0, s>>>(key, val, r, n, total_mass, dout);
        e = cudaGetLastError();
    }
    double out[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, sizeof(double) * 8, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(key, s);
    cudaFreeAsync(val, s);
    cudaFreeAsync(dout, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return dfail(H4_ERR_CUDA, std::string("h4_mass_radii: ") + cudaGetErrorString(e));
    if (core) *core = out[0];
    if (halfmass) *halfmass = out[1];
    if (lagrange)
        for (int k = 0; k < 6; k++) lagrange[k] = out[2 + k];
    return H4_OK;
}
