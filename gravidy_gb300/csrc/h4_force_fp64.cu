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
//  * the lane sums are combined by a fixed butterfly reduce-scatter, the
//    j-chunks of one particle in a fixed order by the reduction kernel:
//    deterministic.
// Work items are handed out through an atomic counter in the control block
// (reset by the active-set kernel of the step).
#include "h4_internal.cuh"
#include "h4_pair.cuh"

namespace h4 {
namespace {

#ifndef H4_FP64_IG
#define H4_FP64_IG 4
#endif
#ifndef H4_FP64_BPS
#define H4_FP64_BPS 2
#endif
constexpr int WARPS = 4;        // warps per block
constexpr int IG = H4_FP64_IG;  // active particles per work item (build knob: 2, 4 or 8)
constexpr int ITEMS_PER_WARP = 12;

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
        double *part_s = d.part + (size_t)s * 6 * nact;
        if (kBoundsCheck && !pair::warp_item_ok(d, nact, k0, cnt, j_begin, j_end, s, lane, BS_FP64_J)) continue;
        if (cnt == (unsigned)IG) {
            pair::fp64_warp_item<IG>(d.pr, d.pv, d.move, nact, k0, j_begin, j_end, d.e2, part_s, lane);
        } else {
            unsigned k = k0, left = cnt;
            if (IG > 4 && left >= 4) {
                pair::fp64_warp_item<4>(d.pr, d.pv, d.move, nact, k, j_begin, j_end, d.e2, part_s, lane);
                k += 4; left -= 4;
            }
            if (left >= 2) {
                pair::fp64_warp_item<2>(d.pr, d.pv, d.move, nact, k, j_begin, j_end, d.e2, part_s, lane);
                k += 2; left -= 2;
            }
            if (left & 1) pair::fp64_warp_item<1>(d.pr, d.pv, d.move, nact, k, j_begin, j_end, d.e2, part_s, lane);
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
    if (!range_ok(d, BS_NACT, 0, nact, d.n) || !range_ok(d, BS_PART, 0, 6ll * nact, (long long)d.part_cap) ||
        !range_ok(d, BS_MOVE, d.move[k], d.move[k] + 1ll, d.n))
        return;
    double f[6];
    pair::exact_sum(d.pr, d.pv, d.n, d.move[k], d.e2, f);
#pragma unroll
    for (int c = 0; c < 6; c++) d.part[(size_t)c * nact + k] = f[c];
}

}  // namespace

int force_fp64_grid_warps(int num_sms) { return num_sms * H4_FP64_BPS * WARPS; }

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
