// FP64 force sum of the active particles as device routines (the work-item
// loop of k_force_fp64 and the exact per-particle sum of k_force_exact); any
// launch shape yields the same items, and hence the same summation order,
// from the same active set.
#pragma once
#include "h4_internal.cuh"
#include "h4_pair.cuh"

namespace h4 {
namespace fp64 {

#ifndef H4_FP64_IG
#define H4_FP64_IG 4
#endif
#ifndef H4_FP64_BPS
#define H4_FP64_BPS 2
#endif
constexpr int WARPS = 4;        // warps per block of the force kernel
constexpr int IG = H4_FP64_IG;  // active particles per work item (build knob: 2, 4 or 8)
constexpr int ITEMS_PER_WARP = 12;
// Smaller items for small steps (build knob; 0 = always IG particles, >= 64 j).
#ifndef H4_FP64_SMALL_SPLIT
#define H4_FP64_SMALL_SPLIT 1
#endif
constexpr bool kFp64SmallSplit = H4_FP64_SMALL_SPLIT != 0;

// The queue loop for items of G particles (G a compile-time constant, so
// the common all-IG shape keeps fully unrolled items).
template <int G>
__device__ __forceinline__ void items_loop(const H4Dev &d, unsigned nact, unsigned n_groups, unsigned total, int chunk,
                                           int lane) {
    for (;;) {
        unsigned item;
        if (lane == 0) item = atomicAdd(&d.ctrl->work_next, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        const unsigned s = item / n_groups;
        const unsigned g = item - s * n_groups;
        const int j_begin = (int)s * chunk;
        const int j_end = min(d.n, j_begin + chunk);
        const unsigned k0 = g * G;
        const unsigned cnt = min((unsigned)G, nact - k0);
        double *part_s = d.part + (size_t)s * 6 * nact;
        if (kBoundsCheck && !pair::warp_item_ok(d, nact, k0, cnt, j_begin, j_end, s, lane, BS_FP64_J)) continue;
        if (cnt == (unsigned)G) {
            pair::fp64_warp_item<G>(d.pr, d.pv, d.move, nact, k0, j_begin, j_end, d.e2, part_s, lane);
        } else {
            unsigned k = k0, left = cnt;
            if (G > 4 && left >= 4) {
                pair::fp64_warp_item<4>(d.pr, d.pv, d.move, nact, k, j_begin, j_end, d.e2, part_s, lane);
                k += 4; left -= 4;
            }
            if (G > 2 && left >= 2) {
                pair::fp64_warp_item<2>(d.pr, d.pv, d.move, nact, k, j_begin, j_end, d.e2, part_s, lane);
                k += 2; left -= 2;
            }
            if (left & 1) pair::fp64_warp_item<1>(d.pr, d.pv, d.move, nact, k, j_begin, j_end, d.e2, part_s, lane);
        }
    }
}

// Small steps' items (1 or 2 particles), out of line so that the common
// shape's loop keeps its register allocation.
static __device__ __noinline__ void small_items(const H4Dev &d, unsigned nact, unsigned n_groups, unsigned total, int chunk,
                                         int lane, unsigned ig) {
    if (ig >= 2)
        items_loop<2>(d, nact, n_groups, total, chunk, lane);
    else
        items_loop<1>(d, nact, n_groups, total, chunk, lane);
}

// Warp lane `lane` takes work items from the queue in the control block
// until it is empty.  The j-split is fixed by nact, n and `split_warps` (the
// warp count the split is sized for: enough items for every warp to take
// several, chunks of at least 64 j, partial sums within the scratch), not by
// the warps that actually run, so any launch shape gives the same items.
// first: this caller publishes the split.
__device__ __forceinline__ void force_items(const H4Dev &d, unsigned split_warps, int lane, bool first) {
    const unsigned nact = d.ctrl->nact;
    if (nact == 0) return;
    // Small steps (too few items of IG particles and >= 64 j to give every
    // warp one): fewer particles per item, then chunks down to 32 j, so that
    // each warp's FP64 chain is short -- at 1/64 of the FP32 rate the step is
    // then bound by the longest chain, not by the total work.
    unsigned ig = IG, min_chunk = 64;
    if (kFp64SmallSplit) {
        while (ig > 1 && ((nact + ig - 1) / ig) * (unsigned)((d.n + 63) / 64) < split_warps) ig >>= 1;
        if (ig == 1 && nact * (unsigned)((d.n + 63) / 64) < split_warps) min_chunk = 32;
    }
    const unsigned n_groups = (nact + ig - 1) / ig;
    unsigned split = (split_warps * ITEMS_PER_WARP + n_groups - 1) / n_groups;
    unsigned max_split = (unsigned)((d.n + min_chunk - 1) / min_chunk);
    if (split > max_split) split = max_split;
    const unsigned cap_split = (unsigned)(d.part_cap / (6ull * nact));
    if (split > cap_split) split = cap_split;
    if (split < 1) split = 1;
    int chunk = (d.n + (int)split - 1) / (int)split;
    chunk = (chunk + 31) & ~31;
    split = (unsigned)((d.n + chunk - 1) / chunk);
    const unsigned total = n_groups * split;
    if (first) {
        d.ctrl->force_split = split;
        d.ctrl->work_total = total;
    }
    if (ig == (unsigned)IG)
        items_loop<IG>(d, nact, n_groups, total, chunk, lane);
    else
        small_items(d, nact, n_groups, total, chunk, lane, ig);
}

// Bit-identical restatement of Hermite4CPU::update_acc_jrk for active
// particle k: one thread, j in ascending order, the reference's operation
// order with no FMA contraction, IEEE sqrt and division (S = 1).
__device__ __forceinline__ void exact_particle(const H4Dev &d, unsigned nact, unsigned k) {
    if (!range_ok(d, BS_NACT, 0, nact, d.n) || !range_ok(d, BS_PART, 0, 6ll * nact, (long long)d.part_cap) ||
        !range_ok(d, BS_MOVE, d.move[k], d.move[k] + 1ll, d.n))
        return;
    double f[6];
    pair::exact_sum(d.pr, d.pv, d.n, d.move[k], d.e2, f);
#pragma unroll
    for (int c = 0; c < 6; c++) d.part[(size_t)c * nact + k] = f[c];
}

}  // namespace fp64
}  // namespace h4
