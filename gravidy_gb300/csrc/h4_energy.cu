// Total energy of the corrected state: kinetic plus unsoftened potential.
//
// Reference: NbodyUtils::get_energy (src/include/utils/NbodyUtils.cpp:427-529)
// and Hermite4GPU::get_energy_gpu + k_energy (Hermite4GPU.cu:540-592,
// Hermite4GPU_kernels.cu:250-288):
//   E = sum_i m_i v_i^2 / 2  -  sum_{i<j} m_i m_j / |r_i - r_j|
// The reference's GPU kernel gives each i the j > i triangle, so the work per
// thread ranges from N-1 pairs to none.  Here every unordered pair is visited
// once through a ring: particle i takes j = i+1 .. i+N/2 (mod N), which is the
// same count for every i; for even N the pair at distance N/2 is met from
// both ends and weighted 1/2.  One warp handles four consecutive i with its
// lanes over the ring offset; per-particle sums are combined in a fixed order
// (deterministic for a given N).
#include "h4_internal.cuh"

namespace h4 {
namespace {

constexpr int EW = 4;  // warps per block
constexpr int EI = 4;  // particles per warp item

__device__ __forceinline__ double rsqrt_refined_e(double x) {
    double y0;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
    const double e = fma(-x, y0 * y0, 1.0);
    return fma(y0 * e, fma(e, 0.375, 0.5), y0);
}

__global__ void __launch_bounds__(EW * 32) k_energy_pairs(H4Dev d) {
    const int n = d.n;
    const int lane = threadIdx.x & 31;
    const int half = n / 2;                    // last ring offset
    const bool even = (n % 2) == 0;
    const int n_items = (n + EI - 1) / EI;
    for (int item = blockIdx.x * EW + (threadIdx.x >> 5); item < n_items; item += gridDim.x * EW) {
        const int i0 = item * EI;
        double xi[EI], yi[EI], zi[EI], acc[EI];
        int ieff[EI];   // rows past n repeat the last particle; never stored
#pragma unroll
        for (int q = 0; q < EI; q++) {
            const int i = min(i0 + q, n - 1);
            ieff[q] = i;
            const dbl4 r = d.r[i];
            xi[q] = r.x; yi[q] = r.y; zi[q] = r.z;
            acc[q] = 0.0;
        }
        for (int off = 1 + lane; off <= half; off += 32) {
            const double w = (even && off == half) ? 0.5 : 1.0;
#pragma unroll
            for (int q = 0; q < EI; q++) {
                int j = ieff[q] + off;   // < 3n/2
                if (j >= n) j -= n;
                if (!range_ok(d, BS_ENERGY, j, j + 1ll, n)) continue;
                const dbl4 rj = d.r[j];
                const double dx = rj.x - xi[q], dy = rj.y - yi[q], dz = rj.z - zi[q];
                const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
                acc[q] = fma(w * rj.w, rsqrt_refined_e(r2), acc[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < EI; q++) {
            double a = acc[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0 && i0 + q < n) d.epot_i[i0 + q] = -a * d.r[i0 + q].w;
        }
    }
}

// Fixed-order sum of the per-particle potential and kinetic terms.
__global__ void __launch_bounds__(1024) k_energy_sum(H4Dev d) {
    __shared__ double sk[1024], sp[1024];
    double ek = 0.0, ep = 0.0;
    for (int i = threadIdx.x; i < d.n; i += 1024) {
        const dbl4 v = d.v[i];
        const double vv2 = v.x * v.x + v.y * v.y + v.z * v.z;
        ek += 0.5 * d.r[i].w * vv2;
        ep += d.epot_i[i];
    }
    sk[threadIdx.x] = ek;
    sp[threadIdx.x] = ep;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sk[threadIdx.x] += sk[threadIdx.x + s];
            sp[threadIdx.x] += sp[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        d.energy_out[0] = sk[0];
        d.energy_out[1] = sp[0];
    }
}

}  // namespace

void launch_energy(const H4Dev &d, cudaStream_t s) {
    if (d.n >= 2) {
        const int items = (d.n + EI - 1) / EI;
        int blocks = (items + EW - 1) / EW;
        if (blocks > 152 * 16) blocks = 152 * 16;
        k_energy_pairs<<<blocks, EW * 32, 0, s>>>(d);
    } else {
        cudaMemsetAsync(d.epot_i, 0, sizeof(double) * (size_t)(d.n > 0 ? d.n : 1), s);
    }
    k_energy_sum<<<1, 1024, 0, s>>>(d);
}

}  // namespace h4
