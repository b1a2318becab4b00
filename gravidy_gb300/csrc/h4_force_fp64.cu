// FP64 acc+jerk force sum of the active particles (update_acc_jrk).
//
// Reference: Hermite4GPU::update_acc_jrk (src/include/gpu/Hermite4GPU.cu:
// 385-535) with k_update / k_reduce (Hermite4GPU_kernels.cu:165-248), and the
// pair arithmetic of Hermite4CPU::force_calculation (Hermite4CPU.cpp:55-82):
//   dr = rj - ri, dv = vj - vi, r2 = |dr|^2 + e2, A = mj / r2^(3/2)
//   a  += A dr
//   a1 += A dv - 3 (dr.dv) A / r2 dr
//
// On GB300 the FP64 pipe is the bottleneck by a wide margin (2 DFMA per clock
// per SM against 128 FFMA), so this kernel is shaped around the FP64
// instruction count, not around memory:
//  * one warp per work item = (up to 4 active particles, one j-chunk); the 32
//    lanes take interleaved j of the chunk, so no lane idles when few
//    particles are active, and every lane runs 4 independent i chains;
//  * the j data (predicted position+mass, velocity: 64 B) comes straight from
//    L2 -- the whole predicted system of N <= 1M particles (64 MB) stays
//    resident in GB300's L2;
//  * 1/sqrt(r2): hardware FP64 reciprocal-square-root approximation
//    (rsqrt.approx.f64) refined by one cubic Householder step,
//    y = y0 (1 + e/2 + 3e^2/8), e = 1 - r2 y0^2, which is accurate to the last
//    bits of a double;
//  * jerk as A (dv - 3 (dr.dv)/r2 dr): 31 FP64 instructions per pair;
//  * the 32 lane sums are combined with a fixed shuffle tree, the j-chunks of
//    one particle in chunk order by the reduction kernel: deterministic.
// Work items are handed out through an atomic counter in the control block
// (reset by the active-set kernel of the step).
#include "h4_internal.cuh"

namespace h4 {
namespace {

constexpr int WARPS = 4;        // warps per block
constexpr int IG = 4;           // active particles per work item
constexpr int ITEMS_PER_WARP = 12;

__device__ __forceinline__ double rsqrt_approx(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}

// 1/sqrt(x): hardware seed + one cubic Householder step.
__device__ __forceinline__ double rsqrt_refined(double x) {
    const double y0 = rsqrt_approx(x);
    const double e = fma(-x, y0 * y0, 1.0);
    const double c = fma(e, 0.375, 0.5);
    return fma(y0 * e, c, y0);
}

template <int NI>
__device__ __forceinline__ void force_item(const H4Dev &d, unsigned nact, unsigned k0,
                                           int j_begin, int j_end, unsigned split, unsigned s,
                                           int lane) {
    double xi[NI], yi[NI], zi[NI], vxi[NI], vyi[NI], vzi[NI];
    unsigned idx[NI];
    double acc[NI][6];
#pragma unroll
    for (int q = 0; q < NI; q++) {
        idx[q] = d.move[k0 + q];
        const dbl4 p = d.pr[idx[q]], v = d.pv[idx[q]];
        xi[q] = p.x; yi[q] = p.y; zi[q] = p.z;
        vxi[q] = v.x; vyi[q] = v.y; vzi[q] = v.z;
#pragma unroll
        for (int c = 0; c < 6; c++) acc[q][c] = 0.0;
    }
    const double e2 = d.e2;
    for (int j = j_begin + lane; j < j_end; j += 32) {
        const dbl4 pj = d.pr[j], vj = d.pv[j];
#pragma unroll
        for (int q = 0; q < NI; q++) {
            const double dx = pj.x - xi[q], dy = pj.y - yi[q], dz = pj.z - zi[q];
            const double dvx = vj.x - vxi[q], dvy = vj.y - vyi[q], dvz = vj.z - vzi[q];
            double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, e2)));
            double m = pj.w;
            const bool self = (unsigned)j == idx[q];   // the reference skips i == j
            r2 = self ? 1.0 : r2;
            m = self ? 0.0 : m;
            const double rinv = rsqrt_refined(r2);
            const double r2inv = rinv * rinv;
            const double A = (m * rinv) * r2inv;
            const double rv = fma(dx, dvx, fma(dy, dvy, dz * dvz));
            const double eta = rv * (-3.0 * r2inv);
            acc[q][0] = fma(A, dx, acc[q][0]);
            acc[q][1] = fma(A, dy, acc[q][1]);
            acc[q][2] = fma(A, dz, acc[q][2]);
            acc[q][3] = fma(A, fma(eta, dx, dvx), acc[q][3]);
            acc[q][4] = fma(A, fma(eta, dy, dvy), acc[q][4]);
            acc[q][5] = fma(A, fma(eta, dz, dvz), acc[q][5]);
        }
    }
#pragma unroll
    for (int q = 0; q < NI; q++) {
#pragma unroll
        for (int c = 0; c < 6; c++) {
            double a = acc[q][c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            acc[q][c] = a;
        }
    }
    if (lane == 0) {
        double *p = d.part + (size_t)s * 6 * nact;
#pragma unroll
        for (int q = 0; q < NI; q++) {
#pragma unroll
            for (int c = 0; c < 6; c++) p[(size_t)c * nact + k0 + q] = acc[q][c];
        }
    }
    (void)split;
}

__global__ void __launch_bounds__(WARPS * 32) k_force_fp64(H4Dev d) {
    const unsigned nact = d.ctrl->nact;
    if (nact == 0) return;
    const int lane = threadIdx.x & 31;
    const unsigned total_warps = gridDim.x * WARPS;
    const unsigned n_groups = (nact + IG - 1) / IG;
    // j-split: enough items for every warp to take several, chunks of at
    // least 64 j, and the partial sums must fit the scratch buffer.
    unsigned split = (total_warps * ITEMS_PER_WARP + n_groups - 1) / n_groups;
    unsigned max_split = (unsigned)((d.n + 63) / 64);
    if (split > max_split) split = max_split;
    const unsigned cap_split = (unsigned)(d.part_cap / (6ull * nact));
    if (split > cap_split) split = cap_split;
    if (split < 1) split = 1;
    int chunk = (d.n + (int)split - 1) / (int)split;
    chunk = (chunk + 31) & ~31;
    split = (unsigned)((d.n + chunk - 1) / chunk);
    const unsigned total = n_groups * split;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        d.ctrl->force_split = split;
        d.ctrl->work_total = total;
    }
    for (;;) {
        unsigned item;
        if (lane == 0) item = atomicAdd(&d.ctrl->work_next, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        const unsigned s = item / n_groups;
        const unsigned g = item - s * n_groups;
        const int j_begin = (int)s * chunk;
        const int j_end = min(d.n, j_begin + chunk);
        const unsigned k0 = g * IG;
        const unsigned cnt = min((unsigned)IG, nact - k0);
        if (cnt == 4) {
            force_item<4>(d, nact, k0, j_begin, j_end, split, s, lane);
        } else {
            unsigned k = k0;
            if (cnt >= 2) { force_item<2>(d, nact, k, j_begin, j_end, split, s, lane); k += 2; }
            if (cnt & 1) force_item<1>(d, nact, k, j_begin, j_end, split, s, lane);
        }
    }
}

// Bit-identical restatement of Hermite4CPU::update_acc_jrk: one thread per
// active particle, j in ascending order, the reference's operation order with
// no FMA contraction, IEEE sqrt and division.  A validation mode, not fast.
__global__ void __launch_bounds__(128) k_force_exact(H4Dev d) {
    const unsigned nact = d.ctrl->nact;
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) d.ctrl->force_split = 1;
    if (k >= nact) return;
    const unsigned i = d.move[k];
    const dbl4 pi = d.pr[i], vi = d.pv[i];
    double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const double e2 = d.e2;
    for (int j = 0; j < d.n; j++) {
        if ((unsigned)j == i) continue;
        const dbl4 pj = d.pr[j], vj = d.pv[j];
        const double rx = __dadd_rn(pj.x, -pi.x), ry = __dadd_rn(pj.y, -pi.y), rz = __dadd_rn(pj.z, -pi.z);
        const double vx = __dadd_rn(vj.x, -vi.x), vy = __dadd_rn(vj.y, -vi.y), vz = __dadd_rn(vj.z, -vi.z);
        const double r2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)), e2);
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
#pragma unroll
    for (int c = 0; c < 6; c++) d.part[(size_t)c * nact + k] = f[c];
}

}  // namespace

int force_fp64_grid_warps(int num_sms) { return num_sms * 2 * WARPS; }

void launch_force_fp64(const H4Dev &d, int grid_warps, cudaStream_t s) {
    int blocks = grid_warps / WARPS;
    if (blocks < 1) blocks = 1;
    k_force_fp64<<<blocks, WARPS * 32, 0, s>>>(d);
}

void launch_force_exact(const H4Dev &d, cudaStream_t s) {
    int blocks = (d.n + 127) / 128;
    k_force_exact<<<blocks, 128, 0, s>>>(d);
}

}  // namespace h4
