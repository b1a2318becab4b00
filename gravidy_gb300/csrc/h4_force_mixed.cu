// Mixed-precision acc+jerk force sum (H4_FORCE_MIXED).
//
// Same quantity as Hermite4CPU::force_calculation (src/include/cpu/
// Hermite4CPU.cpp:55-82) summed as in Hermite4GPU::update_acc_jrk
// (src/include/gpu/Hermite4GPU.cu:385-535), with the arithmetic split by need:
//  * positions are held as double-single pairs (hi + lo floats); the
//    difference rj - ri is taken on both parts before it is rounded to float,
//    so close pairs keep their separation to ~2^-48 of |r|;
//  * everything else of the pair (r^2, 1/sqrt, A = m/r^3, the jerk term) is
//    FP32 on the FP32 pipe, 64x the FP64 pipe's rate on GB300;
//  * each particle's terms are summed in FP32 over sub-tiles of 64 j, and the
//    sub-tile sums are added into Kahan-compensated FP32 accumulators; the
//    compensated sum of each j-chunk is stored as a double and the chunks are
//    added in FP64, in chunk order, by the reduction/corrector kernel.
// The j data come from three float4 arrays written by the predictor:
//   jf0 = (x_hi, y_hi, z_hi, m), jf1 = (x_lo, y_lo, z_lo, 0), jf2 = (vx, vy, vz, 0)
// padded to a multiple of 256 with zero-mass particles (exact zero terms).
//
// Two shapes, chosen per launch from the active count:
//  * tiled: a block owns a group of active particles (lanes over i) and one
//    j-chunk; the chunk streams through shared memory in tiles of 256 j,
//    each tile brought in by TMA bulk copies (cp.async.bulk) that complete on
//    an mbarrier, double buffered.  The packed form (e2 > 0) holds two active
//    particles per thread in f32x2 registers (256 per block); the scalar form
//    (e2 = 0, explicit self mask) four per thread;
//  * warp items (small active sets): a warp owns up to 4 active particles and
//    one j-chunk, its lanes take interleaved j straight from L2, and the lane
//    sums are combined by a reduce-scatter in double-single FP32.
// Every wait on an mbarrier is bounded; on timeout the block waits (bounded)
// for its copies still in flight, records H4_ERRBIT_TIMEOUT in the control
// block and leaves.
#include <stdint.h>

#include "h4_internal.cuh"
#include "h4_pair.cuh"
#include "h4_tma.cuh"

namespace h4 {
namespace {

constexpr int MT = 128;                 // threads per block (tiled shape)
constexpr int IPT = 4;                  // active particles per thread
constexpr int TI = MT * IPT;            // active particles per tile item
constexpr int JT = 256;                 // j per shared-memory tile
constexpr int SUB = 64;                 // j per FP32 partial sum
constexpr int WARPS_W = 4;              // warps per block (warp-item shape)
constexpr int IGW = 4;                  // active particles per warp item
constexpr unsigned WAIT_LIMIT = 1u << 26;

using tma::smem_addr;
using tma::mbar_arrive_expect_tx;
using tma::mbar_init;
using tma::mbar_try_wait;

__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    tma::load_1d(dst, src, bytes, bar);
}

using pair::IParticle;
using pair::kahan_add;
using pair::pair_mixed;

__device__ __forceinline__ IParticle load_i(const H4Dev &d, unsigned i) {
    return pair::load_i(d.jf0, d.jf1, d.jf2, i);
}

struct MixedSplit {
    unsigned split, total, n_groups;
    int chunk;
};

// j-split of the tiled shape: chunks are whole tiles of the padded arrays.
__device__ __forceinline__ MixedSplit tiled_split(const H4Dev &d, unsigned nact, unsigned blocks, unsigned ti) {
    MixedSplit s;
    s.n_groups = (nact + ti - 1) / ti;
    unsigned split = (blocks * 6 + s.n_groups - 1) / s.n_groups;
    const unsigned tiles = (unsigned)(d.n_pad / JT);
    if (split > tiles) split = tiles;
    const unsigned cap = (unsigned)(d.part_cap / (6ull * nact));
    if (split > cap) split = cap;
    if (split < 1) split = 1;
    const unsigned tiles_per_chunk = (tiles + split - 1) / split;
    s.chunk = (int)(tiles_per_chunk * JT);
    s.split = (unsigned)((d.n_pad + s.chunk - 1) / s.chunk);
    s.total = s.n_groups * s.split;
    return s;
}

// Bounds-checked build: the ranges of one tiled item -- whole tiles of the
// padded j arrays, its slice of the partial-force area.  Block-uniform.
__device__ __forceinline__ bool tiled_item_ok(const H4Dev &d, unsigned nact, unsigned s, int j_begin, int j_end) {
    return range_ok(d, BS_NACT, 0, nact, d.n) && range_ok(d, BS_MIXED_J, j_begin, j_end, d.n_pad) &&
           range_ok(d, BS_MIXED_J, 0, (j_end - j_begin) % JT, 1) &&
           range_ok(d, BS_PART, 6ll * nact * s, 6ll * nact * (s + 1), (long long)d.part_cap);
}

// Bounds-checked build: a particle index of the active list (skipped: 0).
__device__ __forceinline__ unsigned checked_move(const H4Dev &d, unsigned k) {
    const unsigned i = d.move[k];
    return range_ok(d, BS_MOVE, i, i + 1ll, d.n) ? i : 0u;
}

template <bool MASK_SELF>
__global__ void __launch_bounds__(MT, 3) k_force_mixed_tiled(H4Dev d, unsigned threshold) {
    __shared__ __align__(128) float4 sj[2][3][JT];
    __shared__ __align__(8) uint64_t full[2];
    __shared__ unsigned s_item;
    const unsigned nact = d.ctrl->nact;
    if (nact == 0 || nact < threshold) return;   // the warp-item kernel takes small sets
    const MixedSplit sp = tiled_split(d, nact, gridDim.x, TI);
    const int tid = threadIdx.x;
    if (blockIdx.x == 0 && tid == 0) {
        d.ctrl->force_split = sp.split;
        d.ctrl->work_total = sp.total;
    }
    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const float e2 = (float)d.e2;
    unsigned gt = 0;   // tiles consumed by this block so far (buffer = gt & 1, parity = (gt >> 1) & 1)
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&d.ctrl->work_next, 1u);
        __syncthreads();
        const unsigned item = s_item;
        __syncthreads();
        if (item >= sp.total) break;
        const unsigned s = item / sp.n_groups;
        const unsigned g = item - s * sp.n_groups;
        const int j_begin = (int)s * sp.chunk;
        const int j_end = min(d.n_pad, j_begin + sp.chunk);
        const int ntiles = (j_end - j_begin) / JT;
        if (kBoundsCheck && !tiled_item_ok(d, nact, s, j_begin, j_end)) continue;

        IParticle ip[IPT];
        unsigned idx[IPT];
        float S[IPT][6], C[IPT][6];
#pragma unroll
        for (int q = 0; q < IPT; q++) {
            const unsigned k = g * TI + tid + q * MT;
            idx[q] = checked_move(d, k < nact ? k : nact - 1);
            ip[q] = load_i(d, idx[q]);
#pragma unroll
            for (int c = 0; c < 6; c++) { S[q][c] = 0.f; C[q][c] = 0.f; }
        }
        // prefetch the first two tiles
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (int t = 0; t < 2 && t < ntiles; t++) {
                const unsigned b = (gt + t) & 1u;
                const size_t j0 = (size_t)j_begin + (size_t)t * JT;
                mbar_arrive_expect_tx(&full[b], 3 * JT * sizeof(float4));
                tma_load_1d(&sj[b][0][0], d.jf0 + j0, JT * sizeof(float4), &full[b]);
                tma_load_1d(&sj[b][1][0], d.jf1 + j0, JT * sizeof(float4), &full[b]);
                tma_load_1d(&sj[b][2][0], d.jf2 + j0, JT * sizeof(float4), &full[b]);
            }
        }
        for (int t = 0; t < ntiles; t++, gt++) {
            const unsigned b = gt & 1u, parity = (gt >> 1) & 1u;
            unsigned spins = 0;
            bool ok = true;
            while (!mbar_try_wait(&full[b], parity)) {
                if (++spins > WAIT_LIMIT) { ok = false; break; }
            }
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    tma::drain_tiles(full, gt, ntiles - t, WAIT_LIMIT);
                    atomicOr(&d.ctrl->err, (unsigned)H4_ERRBIT_TIMEOUT);
                }
                return;
            }
            const int jt0 = j_begin + t * JT;
#pragma unroll 1
            for (int sb = 0; sb < JT; sb += SUB) {
                float part[IPT][6];
#pragma unroll
                for (int q = 0; q < IPT; q++)
#pragma unroll
                    for (int c = 0; c < 6; c++) part[q][c] = 0.f;
#pragma unroll 4
                for (int jj = sb; jj < sb + SUB; jj++) {
                    const float4 j0 = sj[b][0][jj], j1 = sj[b][1][jj], j2 = sj[b][2][jj];
#pragma unroll
                    for (int q = 0; q < IPT; q++)
                        pair_mixed<MASK_SELF>(ip[q], j0, j1, j2, e2, (unsigned)(jt0 + jj) == idx[q], part[q]);
                }
#pragma unroll
                for (int q = 0; q < IPT; q++)
#pragma unroll
                    for (int c = 0; c < 6; c++) kahan_add(S[q][c], C[q][c], part[q][c]);
            }
            __syncthreads();   // every thread is done with buffer b
            if (tid == 0 && t + 2 < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const size_t j0 = (size_t)j_begin + (size_t)(t + 2) * JT;
                mbar_arrive_expect_tx(&full[b], 3 * JT * sizeof(float4));
                tma_load_1d(&sj[b][0][0], d.jf0 + j0, JT * sizeof(float4), &full[b]);
                tma_load_1d(&sj[b][1][0], d.jf1 + j0, JT * sizeof(float4), &full[b]);
                tma_load_1d(&sj[b][2][0], d.jf2 + j0, JT * sizeof(float4), &full[b]);
            }
        }
        double *p = d.part + (size_t)s * 6 * nact;
#pragma unroll
        for (int q = 0; q < IPT; q++) {
            const unsigned k = g * TI + tid + q * MT;
            if (k < nact) {
#pragma unroll
                for (int c = 0; c < 6; c++) p[(size_t)c * nact + k] = (double)S[q][c] - (double)C[q][c];
            }
        }
    }
}

// ---- packed f32x2 variant of the tiled shape (e2 > 0) ----------------------------
// Two active particles share one 64-bit register pair and every FP32
// operation of the pair formula is one packed f32x2 instruction (sm_100+),
// which halves the issue slots the tiled kernel is bound by.  The j data come
// pre-duplicated from d.jd, so one 128-bit shared load gives two packed
// operands.  Same arithmetic per lane as pair_mixed (and hence the same
// results up to the order of the FP32 partial sums, which is identical here).

using pair::f2;
using pair::pk2;
using pair::lo2;
using pair::hi2;
using pair::IPair;
using pair::kahan2;
using pair::pair_x2;

// 128-bit shared load as two packed operands.  A plain load lets the
// compiler fold the tile offsets into the instruction and schedule the loads
// of the unrolled j loop freely (build knob H4_X2_ASM_LDS=1: the inline-PTX
// form, kept for comparison).
#ifndef H4_X2_ASM_LDS
#define H4_X2_ASM_LDS 0
#endif
__device__ __forceinline__ void lds2(const float4 *p, f2 &a, f2 &b) {
#if H4_X2_ASM_LDS
    asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "r"(smem_addr(p)));
#else
    const ulonglong2 q = *reinterpret_cast<const ulonglong2 *>(p);
    a = q.x;
    b = q.y;
#endif
}

// Shape of the packed kernel (build knobs; defaults as measured best on GB300):
// packed pairs of active particles per thread, j-loop unroll, blocks per SM.
// Measured (N = 16384 .. 2^20): one packed pair per thread at 4 blocks per SM
// (120 registers, 16 warps per SM) beats two pairs at 3 blocks (168
// registers, 12 warps) by 10-16 %: the FMA pipe's latency is hidden by more
// warps better than by more independent pairs per warp.
#ifndef H4_X2_NPK
#define H4_X2_NPK 1
#endif
#ifndef H4_X2_UNROLL
#define H4_X2_UNROLL 16
#endif
#ifndef H4_X2_BPS
#define H4_X2_BPS 4
#endif
constexpr int NPK = H4_X2_NPK;
constexpr int IPT2 = 2 * NPK;      // active particles per thread
constexpr int TI2 = MT * IPT2;     // active particles per tile item
constexpr int kX2Unroll = H4_X2_UNROLL;

__global__ void __launch_bounds__(MT, H4_X2_BPS) k_force_mixed_tiled_x2(H4Dev d, unsigned threshold) {
    __shared__ __align__(128) float4 sj[2][5][JT];
    __shared__ __align__(8) uint64_t full[2];
    __shared__ unsigned s_item;
    const unsigned nact = d.ctrl->nact;
    if (nact == 0 || nact < threshold) return;
    const MixedSplit sp = tiled_split(d, nact, gridDim.x, TI2);
    const int tid = threadIdx.x;
    if (blockIdx.x == 0 && tid == 0) {
        d.ctrl->force_split = sp.split;
        d.ctrl->work_total = sp.total;
    }
    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const float e2f = (float)d.e2;
    const f2 e2 = pk2(e2f, e2f), m3 = pk2(-3.0f, -3.0f);
    const size_t np = (size_t)d.n_pad;
    unsigned gt = 0;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&d.ctrl->work_next, 1u);
        __syncthreads();
        const unsigned item = s_item;
        __syncthreads();
        if (item >= sp.total) break;
        const unsigned s = item / sp.n_groups;
        const unsigned g = item - s * sp.n_groups;
        const int j_begin = (int)s * sp.chunk;
        const int j_end = min(d.n_pad, j_begin + sp.chunk);
        const int ntiles = (j_end - j_begin) / JT;
        if (kBoundsCheck && !tiled_item_ok(d, nact, s, j_begin, j_end)) continue;

        IPair ip[NPK];
        f2 S[NPK][6], Cc[NPK][6];
#pragma unroll
        for (int q = 0; q < NPK; q++) {
            const unsigned k0 = g * TI2 + tid + (2 * q) * MT, k1 = k0 + MT;
            const IParticle a = load_i(d, checked_move(d, k0 < nact ? k0 : nact - 1));
            const IParticle b = load_i(d, checked_move(d, k1 < nact ? k1 : nact - 1));
            ip[q].xh = pk2(a.xh, b.xh); ip[q].yh = pk2(a.yh, b.yh); ip[q].zh = pk2(a.zh, b.zh);
            ip[q].xl = pk2(a.xl, b.xl); ip[q].yl = pk2(a.yl, b.yl); ip[q].zl = pk2(a.zl, b.zl);
            ip[q].vx = pk2(a.vx, b.vx); ip[q].vy = pk2(a.vy, b.vy); ip[q].vz = pk2(a.vz, b.vz);
#pragma unroll
            for (int c = 0; c < 6; c++) { S[q][c] = 0ull; Cc[q][c] = 0ull; }
        }
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (int t = 0; t < 2 && t < ntiles; t++) {
                const unsigned b = (gt + t) & 1u;
                const size_t j0 = (size_t)j_begin + (size_t)t * JT;
                mbar_arrive_expect_tx(&full[b], 5 * JT * sizeof(float4));
#pragma unroll
                for (int pl = 0; pl < 5; pl++)
                    tma_load_1d(&sj[b][pl][0], d.jd + pl * np + j0, JT * sizeof(float4), &full[b]);
            }
        }
        for (int t = 0; t < ntiles; t++, gt++) {
            const unsigned b = gt & 1u, parity = (gt >> 1) & 1u;
            unsigned spins = 0;
            bool ok = true;
            while (!mbar_try_wait(&full[b], parity)) {
                if (++spins > WAIT_LIMIT) { ok = false; break; }
            }
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    tma::drain_tiles(full, gt, ntiles - t, WAIT_LIMIT);
                    atomicOr(&d.ctrl->err, (unsigned)H4_ERRBIT_TIMEOUT);
                }
                return;
            }
#pragma unroll 1
            for (int sb = 0; sb < JT; sb += SUB) {
                f2 part[NPK][6];
#pragma unroll
                for (int q = 0; q < NPK; q++)
#pragma unroll
                    for (int c = 0; c < 6; c++) part[q][c] = 0ull;
#pragma unroll kX2Unroll
                for (int jj = sb; jj < sb + SUB; jj++) {
                    f2 jxh, jyh, jzh, jm, jxl, jyl, jzl, jvx, jvy, jvz;
                    lds2(&sj[b][0][jj], jxh, jyh);
                    lds2(&sj[b][1][jj], jzh, jm);
                    lds2(&sj[b][2][jj], jxl, jyl);
                    lds2(&sj[b][3][jj], jzl, jvx);
                    lds2(&sj[b][4][jj], jvy, jvz);
#pragma unroll
                    for (int q = 0; q < NPK; q++)
                        pair_x2(ip[q], jxh, jyh, jzh, jm, jxl, jyl, jzl, jvx, jvy, jvz, e2, m3, part[q]);
                }
#pragma unroll
                for (int q = 0; q < NPK; q++)
#pragma unroll
                    for (int c = 0; c < 6; c++) kahan2(S[q][c], Cc[q][c], part[q][c]);
            }
            __syncthreads();   // every thread is done with buffer b
            if (tid == 0 && t + 2 < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const size_t j0 = (size_t)j_begin + (size_t)(t + 2) * JT;
                mbar_arrive_expect_tx(&full[b], 5 * JT * sizeof(float4));
#pragma unroll
                for (int pl = 0; pl < 5; pl++)
                    tma_load_1d(&sj[b][pl][0], d.jd + pl * np + j0, JT * sizeof(float4), &full[b]);
            }
        }
        double *p = d.part + (size_t)s * 6 * nact;
#pragma unroll
        for (int q = 0; q < NPK; q++) {
            const unsigned k0 = g * TI2 + tid + (2 * q) * MT, k1 = k0 + MT;
#pragma unroll
            for (int c = 0; c < 6; c++) {
                if (k0 < nact) p[(size_t)c * nact + k0] = (double)lo2(S[q][c]) - (double)lo2(Cc[q][c]);
                if (k1 < nact) p[(size_t)c * nact + k1] = (double)hi2(S[q][c]) - (double)hi2(Cc[q][c]);
            }
        }
    }
}

// ---- warp items: small active sets --------------------------------------------
__device__ __forceinline__ MixedSplit warp_split(const H4Dev &d, unsigned nact, unsigned total_warps) {
    MixedSplit s;
    s.n_groups = (nact + IGW - 1) / IGW;
    unsigned split = (total_warps * 8 + s.n_groups - 1) / s.n_groups;
    const unsigned max_split = (unsigned)((d.n + 127) / 128);
    if (split > max_split) split = max_split;
    const unsigned cap = (unsigned)(d.part_cap / (6ull * nact));
    if (split > cap) split = cap;
    if (split < 1) split = 1;
    int chunk = (d.n + (int)split - 1) / (int)split;
    chunk = (chunk + 31) & ~31;
    s.chunk = chunk;
    s.split = (unsigned)((d.n + chunk - 1) / chunk);
    s.total = s.n_groups * s.split;
    return s;
}

template <bool MASK_SELF>
__global__ void __launch_bounds__(WARPS_W * 32) k_force_mixed_warp(H4Dev d, unsigned threshold) {
    const unsigned nact = d.ctrl->nact;
    if (nact == 0 || nact >= threshold) return;   // the tiled kernel takes large sets
    const int lane = threadIdx.x & 31;
    const MixedSplit sp = warp_split(d, nact, gridDim.x * WARPS_W);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        d.ctrl->force_split = sp.split;
        d.ctrl->work_total = sp.total;
    }
    const float e2 = (float)d.e2;
    for (;;) {
        unsigned item;
        if (lane == 0) item = atomicAdd(&d.ctrl->work_next, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= sp.total) break;
        const unsigned s = item / sp.n_groups;
        const unsigned g = item - s * sp.n_groups;
        const int j_begin = (int)s * sp.chunk;
        const int j_end = min(d.n, j_begin + sp.chunk);
        const unsigned k0 = g * IGW;
        const unsigned cnt = min((unsigned)IGW, nact - k0);
        double *part_s = d.part + (size_t)s * 6 * nact;
        if (kBoundsCheck && !pair::warp_item_ok(d, nact, k0, cnt, j_begin, j_end, s, lane, BS_MIXED_WJ)) continue;
        if (cnt == 4) {
            pair::mixed_warp_item<4, MASK_SELF>(d.jf0, d.jf1, d.jf2, d.move, nact, k0, j_begin, j_end, e2, part_s, lane);
        } else {
            unsigned k = k0;
            if (cnt >= 2) {
                pair::mixed_warp_item<2, MASK_SELF>(d.jf0, d.jf1, d.jf2, d.move, nact, k, j_begin, j_end, e2, part_s,
                                                    lane);
                k += 2;
            }
            if (cnt & 1)
                pair::mixed_warp_item<1, MASK_SELF>(d.jf0, d.jf1, d.jf2, d.move, nact, k, j_begin, j_end, e2, part_s,
                                                    lane);
        }
    }
}

}  // namespace

// Both shapes are launched when the active count is only known on the device
// (the captured block step); the one not chosen returns at once.  When the
// host knows the count (known_nact >= 0) only the chosen one is launched.
int launch_force_mixed(const H4Dev &d, int num_sms, unsigned threshold, long long known_nact, cudaStream_t s) {
    const bool mask = !(d.e2 > 0.0);
    int launched = 0;
    const bool want_tiled = known_nact < 0 || (unsigned long long)known_nact >= threshold;
    const bool want_warp = known_nact < 0 || (unsigned long long)known_nact < threshold;
    if (want_tiled) {
        if (mask)
            k_force_mixed_tiled<true><<<num_sms * 3, MT, 0, s>>>(d, threshold);
        else if (d.jd)
            k_force_mixed_tiled_x2<<<num_sms * H4_X2_BPS, MT, 0, s>>>(d, threshold);
        else
            k_force_mixed_tiled<false><<<num_sms * 3, MT, 0, s>>>(d, threshold);
        launched++;
    }
    if (want_warp) {
        if (mask)
            k_force_mixed_warp<true><<<num_sms * 4, WARPS_W * 32, 0, s>>>(d, threshold);
        else
            k_force_mixed_warp<false><<<num_sms * 4, WARPS_W * 32, 0, s>>>(d, threshold);
        launched++;
    }
    return launched;
}

}  // namespace h4
