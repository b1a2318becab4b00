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
#include "h4_force_fp64.cuh"
#include "h4_internal.cuh"
#include "h4_pair.cuh"

namespace h4 {
namespace {

using namespace fp64;

__global__ void __launch_bounds__(WARPS * 32) k_force_fp64(H4Dev d) {
    force_items(d, gridDim.x * WARPS, threadIdx.x & 31, blockIdx.x == 0 && threadIdx.x == 0);
}

// Bit-identical restatement of Hermite4CPU::update_acc_jrk: one thread per
// active particle (fp64::exact_particle).  A validation mode, not fast.
__global__ void __launch_bounds__(128) k_force_exact(H4Dev d) {
    const unsigned nact = d.ctrl->nact;
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) d.ctrl->force_split = 1;
    if (k < nact) exact_particle(d, nact, k);
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
