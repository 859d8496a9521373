// Device-resident progressive-refinement shooting loop for GB300 (sm_103a).
//
// One shooter step of the reference (parallelRadiosity, src/rad.cpp:406-451)
// is two kernels:
//
//   k_setup  (1 CTA)   reduce the previous step's per-CTA (key, slot) maxima
//                      to the shooter (listCanditate, rad.cpp:387-404) and
//                      build the shooter record: centre, normal, area, unshot
//                      energy and, for a source whose longest squared edge is
//                      >= 0.1, the two halves AdaptCalFF shoots from
//                      (shade.cpp:76-99, 141-168).
//   k_shoot  (N/80 CTAs) for every receiver slot: the three corner form
//                      factors (CalFF, shade.cpp:107-127) with the octree
//                      walk (RayHitted, raycast.cpp:335-360), the deposit in
//                      the reference's v-outer / c-inner order (CalRadiosity,
//                      shade.cpp:244-259), the shooters' unshot energy zeroed,
//                      and the next step's selection key reduced per CTA.
//
// Lane layout of k_shoot: a warp owns 10 consecutive slots, lanes 3r..3r+2
// are the three corners of slot r (lanes 30, 31 idle).  Each lane casts its
// corner's ray(s); the three form factors meet by warp shuffle and each lane
// updates its own vertex's accB while lane 3r keeps the slot's deltaB sum in
// the reference's order, so the result is independent of ray timing.
//
// Exactness: compiled with -fmad=false (no contraction), IEEE division and
// square root, and FP64 exactly where the reference promotes (its double
// literals 0.0001, 0.1, 1.0, PI, 2.0, 3.0 and the (double) casts).  The
// FP32 solver then reproduces the reference's FP32 build bit for bit; with
// T = double it is the all-FP64 form.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "capi_internal.h"
#include "prep_workspace.h"

#include "rad_kernels.cuh"

namespace radgb {
namespace dev {

// Persistent: each warp takes 10-slot groups from the step's queue until it
// is empty, so warps that finish early take more work; once all its warps are
// done, thread 0 writes the CTA's (key, slot) maximum.
//
// FUSED (one shooter per step): the last CTA of the grid to finish also does
// the next step's selection -- it reduces the per-CTA partials, builds the
// next shooter record and advances the step -- so a step is one kernel.
// Several shooters per step keep the separate k_setup.
// a group is split in the next step when its item took longer than this
// fraction of the step (an item that was already split: the second figure)
constexpr double kHeavyFrac = 0.55, kHeavyFracSplit = 0.27;
// ... and longer than this multiple of the step's mean group time
constexpr double kHeavyMeanMult = 3.0;
// a group shot whole that took longer than this multiple of the step's mean
// group time starts early in the next step
constexpr double kEarlyMeanMult = 1.5;
// Two forms of the single-shooter kernel, picked per scene (layout):
//   1 (tail-bound: a step is about one wave of groups) -- a split group's
//     items cast each corner with 4 lanes that share the list scans, so a
//     long walk ends sooner; 4 CTAs per SM (64 registers) in FP32, 3 (80) in
//     FP64, which spills far more at 64;
//   2 (throughput-bound: many groups per warp, e.g. 400k triangles) -- 4 CTAs
//     per SM, 64 registers, split items keep one lane per corner (3 slots
//     per item) so the walk is inlined once.
// Measured: the 61k-triangle room 10.1k vs 8.2k shots/s (flushed) in form 1
// vs 2; the 422k-triangle hall 794 vs 1,087 shots/s.  Form 1 at 3 CTAs per SM
// (80 registers) measured 9.5k on the room.
// The counting kernels and the several-shooters kernel (which cannot re-read
// the deposit inputs after the walk) stay at 3 CTAs per SM.
template <typename T>
constexpr int kForm1MinBlocks = std::is_same<T, float>::value ? 4 : 3;
template <int HL>
__host__ __device__ constexpr int heavy_slots() { return HL == 1 ? 3 : 32 / (3 * HL); }
template <int HL>
__host__ __device__ constexpr int heavy_items() { return (kSlotsPerWarp + heavy_slots<HL>() - 1) / heavy_slots<HL>(); }
template <typename T, bool COUNT, bool FUSED, int MINB, int HL>
__global__ void __launch_bounds__(kShootThreads, MINB)
k_shoot(Slots<T> S, Grid<T> G, Shooter<T>* shooters, State* st, Partial* __restrict__ part, T conv) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned long long wkey[kShootThreads / 32];
    __shared__ int wslot[kShootThreads / 32];
    __shared__ int ndone;
    if (st->done || st->paused) return;
    if (FUSED && threadIdx.x == 0) atomicMin(&st->t_start, global_ns());
    const int nsh = st->nsh;
    Shooter<T>* sh = reinterpret_cast<Shooter<T>*>(smem);
    T* thr = reinterpret_cast<T*>(smem + kMaxShooterBytes<T>(nsh));
    {
        const int words = nsh * (int)(sizeof(Shooter<T>) / 4);
        const int* srcw = reinterpret_cast<const int*>(shooters);
        int* dstw = reinterpret_cast<int*>(smem);
        for (int q = threadIdx.x; q < words; q += blockDim.x) dstw[q] = srcw[q];
        for (int q = threadIdx.x; q < G.n_thr; q += blockDim.x) thr[q] = G.thr[q];
        if (threadIdx.x == 0) ndone = 0;
    }
    __syncthreads();
    Grid<T> Gs = G;
    Gs.thr = thr;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int n_groups = (S.n + kSlotsPerWarp - 1) / kSlotsPerWarp;
    unsigned long long kk = 0;
    int ks = -1;
    Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
    // the queue: the heavy groups' one-slot items first, then the other groups
    const bool split = !COUNT && FUSED && st->heavy_on;
    const int s = (int)st->steps;
    constexpr int kHeavySlots = heavy_slots<HL>(), kHeavyItems = heavy_items<HL>();
    const int n_heavy_items = split ? st->heavy_n[s & 1] * kHeavyItems : 0;
    const int n_early = split ? st->early_n[s & 1] : 0;
    // The last groups of the slot order go out as split items (4 lanes per
    // corner, kHeavySlots slots each), like the heavy ones: handed out when
    // the queue is nearly empty, a whole group would start long walks that
    // the rest of the grid, idle by then, waits for; split, its walks spread
    // over the idle warps.  One group per 16 resident warps, at most a
    // twentieth of the groups; only where split items use several lanes and
    // a step is about one wave of groups (at most two per resident warp: on
    // the 61k-slot room the step fell from 95.5 to 94.7 us flushed and from
    // 87.6 to 84.4 us in graph chunks).  With many groups per warp the slow
    // groups' own split (the heavy part) serves better: the 422k-slot hall
    // in form 1 fell from 812 to 663 shots/s with a tail.  (Form 1 on the hall
    // measures 690 against 810 shots/s even without one, from the registers
    // this code takes; the hall runs form 2, unchanged at 1,066.)
    const int n_warps = (int)gridDim.x * (kShootThreads / 32);
    const int n_tail = (split && HL > 1 && n_groups <= 2 * n_warps) ? imin(n_groups / 20, n_warps / 16) : 0;
    const int n_whole = n_groups - n_tail;
    // each warp's first item is its own index; later ones come from the queue
    int first = (int)blockIdx.x * (kShootThreads / 32) + wid;
    for (;;) {
        int g = first;
        if (first < 0) {
            if (lane == 0) g = atomicAdd(&st->work, 1) + n_warps;
            g = __shfl_sync(kFull, g, 0);
        }
        first = -1;
        int grp, i0, n_item;
        const unsigned long long t_item = global_ns();
        bool tail = false;
        if (g < n_heavy_items) {
            grp = st->heavy[(s & 1) * n_groups + g / kHeavyItems];
            const int part = (g % kHeavyItems) * kHeavySlots;
            i0 = grp * kSlotsPerWarp + part;
            n_item = imin(kHeavySlots, kSlotsPerWarp - part);
        } else {
            const int j = g - n_heavy_items;
            int q = 0;
            if (j < n_early) {
                grp = st->early[(s & 1) * n_groups + j];
            } else if (j - n_early < n_whole) {
                grp = j - n_early;
                if (split && __ldcg(&st->estamp[grp]) >= s) continue;   // it was in the early part
            } else {                                                     // the tail's split items
                q = j - n_early - n_whole;
                if (q >= n_tail * kHeavyItems) break;
                grp = n_whole + q / kHeavyItems;
                tail = true;
                if (__ldcg(&st->estamp[grp]) >= s) continue;
            }
            if (split && __ldcg(&st->stamp[grp]) >= s) continue;   // its items are in the heavy part
            if (tail) {
                const int part = (q % kHeavyItems) * kHeavySlots;
                i0 = grp * kSlotsPerWarp + part;
                n_item = imin(kHeavySlots, kSlotsPerWarp - part);
            } else {
                i0 = grp * kSlotsPerWarp;
                n_item = kSlotsPerWarp;
            }
        }
        // one call site when every item is cast one lane per corner: the
        // walk is inlined once, which keeps the register count down
        // FUSED: at most one shooter per step.  Items then re-read the
        // deposit's inputs after the walk instead of holding them in
        // registers (ONE): 3-4% faster in form 2 and in the batched kernel,
        // and what lets form 1 run 4 CTAs per SM (6% faster on the 61k room
        // than 3 CTAs per SM without it).  At 3 CTAs per SM (FP64) the 4-lane
        // items keep their registers: 20-25% slower otherwise.
        constexpr bool kOneHeavy = FUSED && MINB >= 4;
        if constexpr (HL == 1 || COUNT) {
            shoot_item<T, COUNT, 1, FUSED>(S, Gs, sh, nsh, i0, n_item, lane, conv, kk, ks, c);
        } else {
            if (g < n_heavy_items || tail)
                shoot_item<T, false, HL, kOneHeavy>(S, Gs, sh, nsh, i0, n_item, lane, conv, kk, ks, c);
            else
                shoot_item<T, COUNT, 1, FUSED>(S, Gs, sh, nsh, i0, n_item, lane, conv, kk, ks, c);
        }
        if (split && lane == 0) {
            const long long dt = (long long)(global_ns() - t_item);
            if (g >= n_heavy_items && !tail) {
                atomicAdd(&st->item_ns, (unsigned long long)dt);
                atomicAdd(&st->items, 1u);
            }
            // a tail group is not marked: its later items read its stamp to
            // tell whether the heavy part already shot it, and the tail
            // splits it again in the next step
            if (!tail && dt > (g < n_heavy_items ? st->heavy_ns_split : st->heavy_ns)) {
                if (atomicMax(&st->stamp[grp], s + 1) < s + 1) {
                    const int q = atomicAdd(&st->heavy_n[(s + 1) & 1], 1);
                    st->heavy[((s + 1) & 1) * n_groups + q] = grp;
                }
            } else if (!tail && g >= n_heavy_items && dt > st->early_ns) {
                st->estamp[grp] = s + 1;
                const int q = atomicAdd(&st->early_n[(s + 1) & 1], 1);
                st->early[((s + 1) & 1) * n_groups + q] = grp;
            }
        }
    }
    warp_max(kk, ks);
    flush_counters<COUNT>(st, c, lane);
    constexpr bool kPacked = FUSED && std::is_same<T, float>::value;
    if constexpr (kPacked) {
        // One shooter in FP32: the (key, slot) maximum fits one 64-bit word
        // (ties: the larger slot, as part_less orders them), so each CTA
        // posts its own and the grid's last CTA reads the word, instead of
        // reducing per-CTA partials.
        if (lane == 0) wkey[wid] = ks >= 0 ? (kk << 32) | (unsigned long long)(unsigned)ks : 0ull;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long b = 0;
            for (int w = 0; w < kShootThreads / 32; w++) b = wkey[w] > b ? wkey[w] : b;
            if (b) atomicMax(&st->best, b);
            __threadfence();
            ndone = atomicAdd(&st->ctas_done, 1) == (int)gridDim.x - 1;
        }
        __syncthreads();
        if (!ndone || threadIdx.x != 0) return;
        __threadfence();
        const unsigned long long b = atomicExch(&st->best, 0ull);   // read and reset at L2
        kk = b >> 32;
        ks = b ? (int)(unsigned)(b & 0xffffffffull) : -1;
    } else {
        if (lane == 0) {
            wkey[wid] = kk;
            wslot[wid] = ks;
        }
        // The queue is empty: the CTA's warps meet (the early ones have nothing
        // left to do) and thread 0 writes the CTA partial.
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long bk = 0;
            int bs = -1;
            for (int w = 0; w < kShootThreads / 32; w++)
                if (part_less(bk, bs, wkey[w], wslot[w])) { bk = wkey[w]; bs = wslot[w]; }
            part[blockIdx.x].key = bk;
            part[blockIdx.x].slot = bs;
            if (FUSED) {
                __threadfence();
                ndone = atomicAdd(&st->ctas_done, 1) == (int)gridDim.x - 1;
            }
        }
        if (!FUSED) return;
        __syncthreads();
        if (!ndone) return;
        // the grid's last CTA: select the next step's shooter (listCanditate for
        // one shooter), every thread reading a few CTA partials
        __threadfence();
        kk = 0;
        ks = -1;
        for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
            const unsigned long long qk = __ldcg(&part[q].key);
            const int qs = __ldcg(&part[q].slot);
            if (part_less(kk, ks, qk, qs)) { kk = qk; ks = qs; }
        }
        warp_max(kk, ks);
        __syncthreads();          // wkey / wslot are reused
        if (lane == 0) {
            wkey[wid] = kk;
            wslot[wid] = ks;
        }
        __syncthreads();
        if (threadIdx.x != 0) return;
        kk = 0;
        ks = -1;
        for (int w = 0; w < kShootThreads / 32; w++)
            if (part_less(kk, ks, wkey[w], wslot[w])) { kk = wkey[w]; ks = wslot[w]; }
    }
    // thread 0 of the grid's last CTA
    {
        long long steps = st->steps + (nsh > 0 ? 1 : 0);    // the step just shot is complete
        if (!kk) {
            st->done = 1;
            st->nsh = 0;
        } else {
            build_shooter(S, ks, shooters[0]);
            if (steps < st->trace_cap) st->trace[steps] = ks;
            st->nsh = 1;
            if (steps >= st->step_limit) st->paused = 1;
        }
        st->steps = steps;
        st->work = 0;
        st->ctas_done = 0;
        st->heavy_n[(steps + 1) & 1] = 0;   // consumed by this step, refilled by the next
        st->early_n[(steps + 1) & 1] = 0;
        // the next step's split limits, from this step's duration
        const long long took = (long long)(global_ns() - st->t_start);
        if (nsh > 0 && !COUNT && st->items > 0) {
            const double mean = (double)st->item_ns / (double)st->items;
            st->heavy_ns = (long long)fmax(st->frac * (double)took, st->mean_mult * mean);
            st->heavy_ns_split = (long long)(st->frac_split * (double)took);
            st->early_ns = (long long)(st->early_mult * mean);
        }
        st->t_start = ~0ull;
        st->item_ns = 0;
        st->items = 0;
    }
}

// ------------------------------------------------------------------ k_setup
template <typename T>
__global__ void __launch_bounds__(kSetupThreads)
k_setup(Slots<T> S, Shooter<T>* shooters, State* st, const Partial* __restrict__ part, int nparts, T conv, int P) {
    __shared__ unsigned long long bk[kSetupThreads / 32];
    __shared__ int bs[kSetupThreads / 32];
    __shared__ int chosen[kMaxShooters];
    __shared__ int nch;
    if (st->done || st->paused) return;
    if (st->steps >= st->step_limit) {
        if (threadIdx.x == 0) st->paused = 1;
        return;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (P == 1) {
        unsigned long long kk = 0;
        int ks = -1;
        for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
            const Partial q = part[b];
            if (part_less(kk, ks, q.key, q.slot)) { kk = q.key; ks = q.slot; }
        }
        warp_max(kk, ks);
        if (lane == 0) { bk[wid] = kk; bs[wid] = ks; }
        __syncthreads();
        if (wid == 0) {
            kk = bk[lane];
            ks = bs[lane];
            warp_max(kk, ks);
            if (lane == 0) { nch = kk ? 1 : 0; chosen[0] = ks; }
        }
        __syncthreads();
    } else {
        // listCanditate for P > 1: the n = min((|C|+4)/5, P) largest pairs
        const int n = cta_top_shooters(S, conv, P, chosen);
        if (threadIdx.x == 0) nch = n;
        __syncthreads();
    }
    const int n = nch;
    if (n == 0) {
        if (threadIdx.x == 0) st->done = 1;
        return;
    }
    if ((int)threadIdx.x < n) build_shooter(S, chosen[threadIdx.x], shooters[threadIdx.x]);
    if (threadIdx.x == 0) {
        const long long base = st->steps * (long long)P;
        for (int j = 0; j < P; j++)
            if (base + j < st->trace_cap) st->trace[base + j] = j < n ? chosen[j] : -1;
        st->nsh = n;
        st->work = 0;
        st->steps += 1;
    }
}

// ------------------------------------------------------------------ unshot power
// The total unshot power, sum over live slots of (dB_r + dB_g + dB_b) * area,
// in FP64: each thread sums its slots in index order, each CTA reduces in a
// fixed tree, one warp adds the CTA partials in a fixed order -- the same
// value on every call for the same state.  A monitor only: selection keeps the
// reference's FP32 key.
constexpr int kUnshotCtas = 304, kUnshotThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kUnshotThreads) k_unshot(Slots<T> S, double* part) {
    __shared__ double red[kUnshotThreads];
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) {
        const Q4<T> fr = S.frgb[i];
        if ((int)fr.w < 0) continue;
        const Q4<T> db = S.deltaB[i];
        acc += ((double)db.x + (double)db.y + (double)db.z) * (double)S.ctr[i].w;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kUnshotThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// one warp: lane l adds partials l, l+32, ... in order, then a fixed tree
__global__ void k_unshot_total(const double* part, int n, double* out) {
    const int lane = threadIdx.x & 31;
    double t = 0;
    for (int i = lane; i < n; i += 32) t += part[i];
#pragma unroll
    for (int d = 16; d; d >>= 1) t += __shfl_xor_sync(kFull, t, d);
    if (threadIdx.x == 0) *out = t;
}

// ------------------------------------------------------------------ queries
template <typename T>
__global__ void k_ray_hit(Grid<T> G, const T* __restrict__ p, const T* __restrict__ v, const int* __restrict__ ban,
                          int n, int* __restrict__ out, State* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < n) {
        const T pp[3] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
        const T vv[3] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        out[i] = walk<T, false>(G, pp, vv, ban[i], c);
    }
    if (c.capped) atomicAdd(&st->capped, (unsigned long long)c.capped);
    if (c.loops) atomicAdd(&st->loops, (unsigned long long)c.loops);
}

template <typename T>
__global__ void k_build_one(Slots<T> S, int slot, Shooter<T>* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) build_shooter(S, slot, *out);
}

template <typename T>
__global__ void k_form_factors(Slots<T> S, Grid<T> G, const Shooter<T>* __restrict__ shp, const int* __restrict__ rcv,
                               int n, T* __restrict__ ff, State* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
    if (t < 3 * n) {
        const Shooter<T> s = *shp;
        const int i = rcv[t / 3], v = t % 3;
        const Q4<T> pp = S.vtx[i * 3 + v], nn = S.nrm[i], fr = S.frgb[i];
        const T pv[3] = {pp.x, pp.y, pp.z}, nd[3] = {nn.x, nn.y, nn.z};
        ff[t] = corner_ff<T, false>(s, pv, nd, nn.w, (int)fr.w, G, c);
    }
    if (c.capped) atomicAdd(&st->capped, (unsigned long long)c.capped);
    if (c.loops) atomicAdd(&st->loops, (unsigned long long)c.loops);
}

// ------------------------------------------------------------------ no-allocation variant
// Shooter records for rad_dev_form_factors_noalloc live in this fixed array
// instead of memory allocated per call.  Sized for the FP64 record, so it
// serves both precisions.
constexpr int kNoAllocMaxShooters = 64;
static __device__ __align__(256) unsigned char g_noalloc_shooters[kNoAllocMaxShooters * sizeof(Shooter<double>)];
static_assert(sizeof(Shooter<float>) <= sizeof(Shooter<double>) && alignof(Shooter<double>) <= 256 &&
                  alignof(Shooter<float>) <= 256,
              "the fixed array holds 64 records of either precision");

struct ShooterSlots { int slot[kNoAllocMaxShooters]; };

template <typename T>
__global__ void k_build_many(Slots<T> S, ShooterSlots src, int n_src, Shooter<T>* out) {
    const int j = threadIdx.x;
    if (j < n_src) build_shooter(S, src.slot[j], out[j]);
}

// ff[(s * n_rcv + i) * 3 + v] for shooter s, receiver rcv[i], corner v;
// receivers outside [0, n_slots) give NaN
template <typename T>
__global__ void k_form_factors_many(Slots<T> S, Grid<T> G, const Shooter<T>* __restrict__ sh, int n_src,
                                    const int* __restrict__ rcv, int n_rcv, T* __restrict__ ff, State* st) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
    if (t < 3LL * n_rcv * n_src) {
        const int s = (int)(t / (3LL * n_rcv));
        const int rem = (int)(t - (long long)s * 3 * n_rcv);
        const int i = rcv[rem / 3], v = rem % 3;
        if (i < 0 || i >= S.n) {
            ff[t] = (T)NAN;
        } else {
            const Q4<T> pp = S.vtx[i * 3 + v], nn = S.nrm[i], fr = S.frgb[i];
            const T pv[3] = {pp.x, pp.y, pp.z}, nd[3] = {nn.x, nn.y, nn.z};
            ff[t] = corner_ff<T, false>(sh[s], pv, nd, nn.w, (int)fr.w, G, c);
        }
    }
    if (c.capped) atomicAdd(&st->capped, (unsigned long long)c.capped);
    if (c.loops) atomicAdd(&st->loops, (unsigned long long)c.loops);
}

}  // namespace dev
}  // namespace radgb

// ==================================================================== host
using namespace radgb;
using namespace radgb::dev;

namespace {

#define CU(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(RAD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct DevBase {
    virtual ~DevBase() {}
};

template <typename T>
struct DevImpl : DevBase {
    using Real = T;
    int device = 0;
    cudaStream_t stream = nullptr;
    Slots<T> S{};
    Grid<T> G{};
    Shooter<T>* d_shooters = nullptr;
    State* d_state = nullptr;
    Partial* d_part = nullptr;
    double* d_unshot = nullptr;   // kUnshotCtas partials, then the total
    int* d_trace = nullptr;
    long long trace_cap = 0;
    bool trace_own = false;   // d_trace is its own allocation (after a growth), not part of the block
    int n_cta = 0;          // CTAs of the current layout's kernel
    int n_cta1 = 0, n_cta2 = 0;
    int n_cta_nf = 0;       // the counting kernels and the several-shooters kernel (3 CTAs per SM)
    int n_cta_of(int l) const { return l == 2 ? n_cta2 : n_cta1; }
    int layout = 1;         // 1 tail-bound form, 2 throughput form (FP32, one shooter per step)
    int P = 1;
    T conv = 0;
    bool counting = false;
    cudaGraphExec_t graphs[3][2][33] = {};   // [layout][counting][steps per launch]
    bool graph_seen[3][2][33] = {};          // a chunk of that shape has run once
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::vector<void*> allocs;
    size_t bytes = 0;
    long long h2d_bytes = 0;   // host -> device copies of the upload
    State host{};   // mirror after the last synchronisation

    ~DevImpl() override {
        for (auto& plane : graphs)
            for (auto& row : plane)
                for (auto& g : row)
                    if (g) cudaGraphExecDestroy(g);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (void* p : allocs) cudaFree(p);
        if (d_trace && trace_own) cudaFree(d_trace);
        if (stream) cudaStreamDestroy(stream);
    }
    // one cudaMalloc for every array of a DevBlock, carved at its offsets
    int alloc_block(DevBlock& b) {
        void* q = nullptr;
        CU(cudaMalloc(&q, std::max<size_t>(b.size, 16)));
        allocs.push_back(q);
        bytes += b.size;
        b.carve(q);
        return RAD_OK;
    }
    template <typename U>
    int alloc(U** p, size_t count) {
        void* q = nullptr;
        size_t b = count * sizeof(U);
        if (b == 0) b = 16;
        CU(cudaMalloc(&q, b));
        allocs.push_back(q);
        bytes += b;
        *p = (U*)q;
        return RAD_OK;
    }
    int n_thr = 0;
    size_t shoot_smem() const { return kMaxShooterBytes<T>(P) + (size_t)n_thr * sizeof(T); }
};

// 1 + the largest triangle a list entry names (0 without entries), the
// entries split over the host pool when there are many
inline int max_entry_tri(const std::vector<int32_t>& ent, int jobs) {
    const int n = (int)ent.size();
    const int parts = pack_jobs(n, jobs);
    std::vector<int> best((size_t)parts, 0);
    split_range(parts, parts, [&](int a, int b) {
        for (int k = a; k < b; k++) {
            int m = 0;
            const int lo = (int)((long long)n * k / parts), hi = (int)((long long)n * (k + 1) / parts);
            for (int i = lo; i < hi; i++) m = std::max(m, ent[(size_t)i] + 1);
            best[(size_t)k] = m;
        }
    });
    return parts ? *std::max_element(best.begin(), best.end()) : 0;
}

// Resident CTAs per SM of each k_shoot form at a dynamic shared memory size,
// and the SM count: the same for every handle of a device and size, so kept
// for the process (with the kernels' shared-memory limits raised once per
// device), not queried again at each handle's creation.
struct ShootShape {
    int sms = 0, per1 = 0, per_nf = 0, per2 = 0;
};

template <typename T>
int shoot_shape(int device, size_t smem, ShootShape* out) {
    struct Known {
        int device;
        size_t smem;
        ShootShape shape;
    };
    static std::mutex m;
    static std::vector<Known> known;
    static std::vector<size_t> smem_allowed;   // per device: the kernels' dynamic shared memory limit
    std::lock_guard<std::mutex> g(m);
    for (const Known& k : known)
        if (k.device == device && k.smem == smem) {
            *out = k.shape;
            return RAD_OK;
        }
    if ((int)smem_allowed.size() <= device) smem_allowed.resize((size_t)device + 1, 48 * 1024);
    if (smem > smem_allowed[(size_t)device]) {
        CU(cudaFuncSetAttribute(k_shoot<T, false, false, 3, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CU(cudaFuncSetAttribute(k_shoot<T, true, false, 3, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CU(cudaFuncSetAttribute(k_shoot<T, false, true, kForm1MinBlocks<T>, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
        CU(cudaFuncSetAttribute(k_shoot<T, true, true, 3, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if constexpr (std::is_same<T, float>::value)
            CU(cudaFuncSetAttribute(k_shoot<T, false, true, 4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        smem_allowed[(size_t)device] = smem;
    }
    ShootShape sh;
    CU(cudaDeviceGetAttribute(&sh.sms, cudaDevAttrMultiProcessorCount, device));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh.per1, k_shoot<T, false, true, kForm1MinBlocks<T>, 4>,
                                                     kShootThreads, smem));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh.per_nf, k_shoot<T, false, false, 3, 4>, kShootThreads, smem));
    if constexpr (std::is_same<T, float>::value)
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh.per2, k_shoot<T, false, true, 4, 1>, kShootThreads, smem));
    else
        sh.per2 = sh.per1;
    known.push_back({device, smem, sh});
    *out = sh;
    return RAD_OK;
}

template <typename T>
int upload(const Scene<T>& s, const Octree<T>& o, const rad_options& opt, int device, DevImpl<T>& d) {
    d.device = device;
    CU(cudaSetDevice(device));
    CU(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
    d.P = opt.parallel_src < 1 ? 1 : opt.parallel_src;
    if (d.P > kMaxShooters) return fail(RAD_ERR_CAPACITY, "-parallel_src above 256 is not supported");
    d.conv = (T)opt.converge;
    const int n = s.trinum;
    if (n < 0) return fail(RAD_ERR_ARG, "negative slot count");
    if (!thresholds_consistent(o)) return fail(RAD_ERR_ARG, "octree cell thresholds do not match its dimensions");
    const int n_tri = max_entry_tri(o.entry_tri, opt.jobs);
    if (n_tri > n) return fail(RAD_ERR_ARG, "octree names a triangle beyond the scene");
    const long long n_cell = (long long)o.cell_leaf.size(), n_ent = (long long)o.entry_tri.size();
    const size_t n_rec = (size_t)n * 10;            // vtx 3, acc 3, nrm, ctr, frgb, db per slot
    const size_t n_trec = (size_t)n_tri * 5;

    // the kernels' launch shapes: k_shoot is persistent, as many CTAs as fit at once
    d.n_thr = (int)o.thr.size();
    const int n_groups = (n + kSlotsPerWarp - 1) / kSlotsPerWarp;
    {
        ShootShape sh;
        int rc0;
        if ((rc0 = shoot_shape<T>(device, d.shoot_smem(), &sh))) return rc0;
        const int want = (n_groups + kShootThreads / 32 - 1) / (kShootThreads / 32);
        d.n_cta1 = std::max(1, std::min(want, std::max(1, sh.sms * sh.per1)));
        d.n_cta_nf = std::max(1, std::min(want, std::max(1, sh.sms * sh.per_nf)));
        d.n_cta2 = std::max(1, std::min(want, std::max(1, sh.sms * sh.per2)));
        // the throughput form once there are over 4 groups per resident warp
        const long long warps2 = (long long)sh.sms * std::max(sh.per2, 1) * (kShootThreads / 32);
        d.layout = (std::is_same<T, float>::value && d.P == 1 && n_groups > 4 * warps2) ? 2 : 1;
        d.n_cta = d.n_cta_of(d.layout);
    }

    // Every array the handle keeps, carved from one device allocation.
    Q4<T>* d_rec;
    Q4<T>* d_ent;
    CellRec<T>* d_cell;
    T* d_thr;
    int *d_heavy, *d_stamp, *d_early, *d_estamp;
    DevBlock blk;
    blk.add(&d_rec, n_rec);
    blk.add(&d_thr, o.thr.size());
    blk.add(&d_cell, (size_t)n_cell);
    blk.add(&d_ent, (size_t)n_ent * 5);
    blk.add(&d.d_shooters, (size_t)d.P);
    blk.add(&d.d_state, 1);
    blk.add(&d.d_part, (size_t)std::max({d.n_cta1, d.n_cta2, d.n_cta_nf}));
    blk.add(&d_heavy, 2 * (size_t)n_groups);
    blk.add(&d_stamp, (size_t)n_groups);
    blk.add(&d.d_unshot, (size_t)kUnshotCtas + 1);
    blk.add(&d_early, 2 * (size_t)n_groups);
    blk.add(&d_estamp, (size_t)n_groups);
    d.trace_cap = 1 << 16;
    blk.add(&d.d_trace, (size_t)d.trace_cap);
    int rc;
    if ((rc = d.alloc_block(blk))) return rc;
    Q4<T>* d_vtx = d_rec;
    Q4<T>* d_acc = d_vtx + (size_t)n * 3;
    Q4<T>* d_nrm = d_acc + (size_t)n * 3;
    Q4<T>* d_ctr = d_nrm + n;
    Q4<T>* d_frgb = d_ctr + n;
    Q4<T>* d_db = d_frgb + n;

    // The records are packed on the host into this thread's pinned staging
    // (reused between handles, so no page faults) on the host pool's threads,
    // and copied from there in three pieces: the six per-slot arrays into the
    // handle's block; the walk's triangle records with the octree's compact
    // tables, laid out as in the staging, into this thread's preparation
    // scratch, where k_expand_cells and k_gather_entries build the cell table
    // and the list entries the handle keeps; and the cell thresholds.
    HostLayout lay;
    const size_t o_rec = lay.add(n_rec * sizeof(Q4<T>));
    const size_t o_trec = lay.add(n_trec * sizeof(Q4<T>));
    const size_t o_cleaf = lay.add(o.cell_leaf.size() * 4);
    const size_t o_lbox = lay.add(o.leaf_box.size() * sizeof(T));
    const size_t o_lrange = lay.add(o.leaf_range.size() * 4);
    const size_t o_etri = lay.add(o.entry_tri.size() * 4);
    const size_t o_tab_end = lay.size;
    const size_t o_thr = lay.add(o.thr.size() * sizeof(T));
    void* stage_p = nullptr;
    CU(pinned_stage().get(lay.size, &stage_p));
    char* stage = static_cast<char*>(stage_p);
    Q4<T>* h_vtx = reinterpret_cast<Q4<T>*>(stage + o_rec);
    Q4<T>* h_acc = h_vtx + (size_t)n * 3;
    Q4<T>* h_nrm = h_acc + (size_t)n * 3;
    Q4<T>* h_ctr = h_nrm + n;
    Q4<T>* h_frgb = h_ctr + n;
    Q4<T>* h_db = h_frgb + n;
    Q4<T>* h_trec = reinterpret_cast<Q4<T>*>(stage + o_trec);
    // slots [a, b): their records, and the walk's triangle records of the
    // triangles among them that a list names (five per triangle)
    auto pack = [&](int a, int b) {
        for (int i = a; i < b; i++) {
            const Slot<T>& t = s.slots[i];
            for (int v = 0; v < 3; v++) {
                h_vtx[(size_t)i * 3 + v] = {t.p[v][0], t.p[v][1], t.p[v][2], 0};
                h_acc[(size_t)i * 3 + v] = {t.accB[v][0], t.accB[v][1], t.accB[v][2], 0};
            }
            const T nl = (T)std::sqrt(t.n[0] * t.n[0] + t.n[1] * t.n[1] + t.n[2] * t.n[2]);
            h_nrm[i] = {t.n[0], t.n[1], t.n[2], nl};
            h_ctr[i] = {t.c[0], t.c[1], t.c[2], t.area};
            h_frgb[i] = {(T)t.Frgb[0], (T)t.Frgb[1], (T)t.Frgb[2], (T)t.parent};
            h_db[i] = {t.deltaB[0], t.deltaB[1], t.deltaB[2], 0};
            if (i < n_tri) {
                Q4<T>* r = &h_trec[(size_t)i * 5];
                r[0] = {t.n[0], t.n[1], t.n[2], pack_int<T>(i)};
                r[1] = {t.c[0], t.c[1], t.c[2], 0};
                for (int e = 0; e < 3; e++) r[2 + e] = {t.se[e][0], t.se[e][1], t.se[e][2], t.se[e][3]};
            }
        }
    };
    // memory-bound passes: large scenes split them over the host pool
    const int jobs = pack_jobs(n, opt.jobs);
    split_range(n, jobs, pack);
    copy_segments({{stage + o_cleaf, o.cell_leaf.data(), o.cell_leaf.size() * 4},
                   {stage + o_lbox, o.leaf_box.data(), o.leaf_box.size() * sizeof(T)},
                   {stage + o_lrange, o.leaf_range.data(), o.leaf_range.size() * 4},
                   {stage + o_etri, o.entry_tri.data(), o.entry_tri.size() * 4},
                   {stage + o_thr, o.thr.data(), o.thr.size() * sizeof(T)}},
                  jobs);
    auto h2d = [&](void* dst, const void* src, size_t bytes) -> int {
        if (bytes) CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, d.stream));
        d.h2d_bytes += (long long)bytes;
        return RAD_OK;
    };
    PrepWorkspace& ws = prep_workspace(device);
    void* scratch;
    CU(ws.buffer(8, std::max<size_t>(o_tab_end - o_trec, 16), &scratch));
    auto tab = [&](size_t off) { return static_cast<char*>(scratch) + (off - o_trec); };   // staging offsets
    if ((rc = h2d(d_rec, stage + o_rec, n_rec * sizeof(Q4<T>))) ||
        (rc = h2d(tab(o_trec), stage + o_trec, o_tab_end - o_trec)) ||
        (rc = h2d(d_thr, stage + o_thr, o.thr.size() * sizeof(T))))
        return rc;
    if (n_cell > 0)
        k_expand_cells<T><<<(int)std::min<long long>((n_cell + 255) / 256, 4096), 256, 0, d.stream>>>(
            reinterpret_cast<const int32_t*>(tab(o_cleaf)), reinterpret_cast<const T*>(tab(o_lbox)),
            reinterpret_cast<const int32_t*>(tab(o_lrange)), n_cell, d_cell);
    if (n_ent > 0)
        k_gather_entries<T><<<(int)std::min<long long>((n_ent * 5 + 255) / 256, 4096), 256, 0, d.stream>>>(
            reinterpret_cast<const int32_t*>(tab(o_etri)), reinterpret_cast<const Q4<T>*>(tab(o_trec)), n_ent, d_ent);
    CU(cudaGetLastError());
    d.S = Slots<T>{n, d_vtx, d_nrm, d_ctr, d_frgb, d_acc, d_db};
    Grid<T> G = grid_params(o, opt.walk_cap);
    G.thr = d_thr;
    G.cell = d_cell;
    G.entry = d_ent;
    d.G = G;

    // per-step state
    CU(cudaMemsetAsync(d_stamp, 0xff, (size_t)n_groups * sizeof(int), d.stream));
    CU(cudaMemsetAsync(d_estamp, 0xff, (size_t)n_groups * sizeof(int), d.stream));
    State st{};
    st.step_limit = 0;
    st.trace = d.d_trace;
    st.trace_cap = d.trace_cap;
    st.heavy = d_heavy;
    st.stamp = d_stamp;
    st.heavy_on = d.P == 1;
    st.heavy_ns = 0x7fffffffffffffffLL;   // no split before a step has been timed
    st.heavy_ns_split = 0x7fffffffffffffffLL;
    st.early = d_early;
    st.estamp = d_estamp;
    st.early_ns = 0x7fffffffffffffffLL;
    st.frac = kHeavyFrac;
    st.frac_split = kHeavyFracSplit;
    st.mean_mult = kHeavyMeanMult;
    st.early_mult = kEarlyMeanMult;
    st.t_start = ~0ull;
    CU(cudaMemcpyAsync(d.d_state, &st, sizeof st, cudaMemcpyHostToDevice, d.stream));
    d.h2d_bytes += (long long)sizeof st;
    CU(cudaMemsetAsync(d.d_shooters, 0, sizeof(Shooter<T>) * d.P, d.stream));
    CU(cudaMemsetAsync(d.d_part, 0, sizeof(Partial) * std::max({d.n_cta1, d.n_cta2, d.n_cta_nf}), d.stream));
    // initial selection keys: a step with no shooter only reduces the keys
    CU(launch_shoot(d, d.stream));
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(&st, d.d_state, sizeof st, cudaMemcpyDeviceToHost, d.stream));
    CU(cudaStreamSynchronize(d.stream));
    d.host = st;
    return RAD_OK;
}

// the shooting kernel of one step; with one shooter per step it also selects the next
template <typename T>
cudaError_t launch_shoot(DevImpl<T>& d, cudaStream_t s) {
    const bool fused = d.P == 1;
    const size_t sm = d.shoot_smem();
    // counting and several shooters per step use the tail-bound form at 3
    // CTAs per SM (they cannot re-read the deposit inputs); FP64 uses form 1
    if (d.counting && fused)
        k_shoot<T, true, true, 3, 4><<<d.n_cta_nf, kShootThreads, sm, s>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
    else if (d.counting)
        k_shoot<T, true, false, 3, 4><<<d.n_cta_nf, kShootThreads, sm, s>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
    else if (fused && d.layout == 2) {
        if constexpr (std::is_same<T, float>::value)
            k_shoot<T, false, true, 4, 1><<<d.n_cta2, kShootThreads, sm, s>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part,
                                                                           d.conv);
    } else if (fused)
        k_shoot<T, false, true, kForm1MinBlocks<T>, 4><<<d.n_cta1, kShootThreads, sm, s>>>(d.S, d.G, d.d_shooters, d.d_state,
                                                                                          d.d_part, d.conv);
    else
        k_shoot<T, false, false, 3, 4><<<d.n_cta_nf, kShootThreads, sm, s>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
    return cudaGetLastError();
}

template <typename T>
int launch_step(DevImpl<T>& d, cudaStream_t s) {
    if (d.P > 1) k_setup<T><<<1, kSetupThreads, 0, s>>>(d.S, d.d_shooters, d.d_state, d.d_part, d.n_cta_nf, d.conv, d.P);
    CU(launch_shoot(d, s));
    CU(cudaGetLastError());
    return RAD_OK;
}

// The graph of a chunk of `steps` steps, built the second time a chunk of
// that shape runs; null the first time, when the caller launches the steps
// one by one: a step's kernel outlasts its launch, so the launches overlap the
// device's work, while capturing and instantiating a graph would delay it.
template <typename T>
int graph_for(DevImpl<T>& d, int steps, cudaGraphExec_t* out) {
    cudaGraphExec_t& slot = d.graphs[d.layout][d.counting ? 1 : 0][steps];
    bool& seen = d.graph_seen[d.layout][d.counting ? 1 : 0][steps];
    if (!slot && !seen) {
        seen = true;
        *out = nullptr;
        return RAD_OK;
    }
    if (!slot) {
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < steps; k++) {
            int rc = launch_step(d, d.stream);
            if (rc) { cudaStreamEndCapture(d.stream, &g); return rc; }
        }
        CU(cudaStreamEndCapture(d.stream, &g));
        cudaError_t e = cudaGraphInstantiate(&slot, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { slot = nullptr; return fail(RAD_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)); }
    }
    *out = slot;
    return RAD_OK;
}

template <typename T>
int grow_trace(DevImpl<T>& d, long long need) {
    if (need <= d.trace_cap) return RAD_OK;
    long long cap = d.trace_cap;
    while (cap < need) cap *= 2;
    int* nt = nullptr;
    CU(cudaMalloc(&nt, (size_t)cap * 4));
    CU(cudaMemcpyAsync(nt, d.d_trace, (size_t)d.trace_cap * 4, cudaMemcpyDeviceToDevice, d.stream));
    CU(cudaStreamSynchronize(d.stream));
    if (d.trace_own) cudaFree(d.d_trace);
    d.d_trace = nt;
    d.trace_own = true;
    d.trace_cap = cap;
    CU(cudaMemcpyAsync(&d.d_state->trace, &nt, sizeof(int*), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(&d.d_state->trace_cap, &cap, sizeof(long long), cudaMemcpyHostToDevice, d.stream));
    CU(cudaStreamSynchronize(d.stream));
    return RAD_OK;
}

constexpr int kChunk = 32;   // steps per graph launch

// mode 0: graphs; mode 1: graphs with events around each launch;
// mode 2: one kernel at a time with events around each kernel
template <typename T>
int run(DevImpl<T>& d, long long max_steps, long long* done_steps, int* converged, int mode, double* ms_a,
        double* ms_b) {
    CU(cudaSetDevice(d.device));
    if (ms_a) *ms_a = 0;
    if (ms_b) *ms_b = 0;
    long long start = d.host.steps;
    if (d.host.done || max_steps <= 0) {
        if (done_steps) *done_steps = 0;
        if (converged) *converged = d.host.done;
        return RAD_OK;
    }
    if (mode && !d.ev[0])
        for (auto& e : d.ev) CU(cudaEventCreate(&e));
    const long long limit = start + max_steps;
    const int zero = 0;
    CU(cudaMemcpyAsync(&d.d_state->step_limit, &limit, sizeof limit, cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(&d.d_state->paused, &zero, sizeof zero, cudaMemcpyHostToDevice, d.stream));
    int rc;
    for (;;) {
        const long long left = limit - d.host.steps;
        const int chunk = (int)std::min<long long>(kChunk, std::max<long long>(left, 1));
        if ((rc = grow_trace(d, (d.host.steps + chunk + 1) * d.P))) return rc;
        if (mode == 2) {
            // one step per iteration, kernels timed separately
            CU(cudaEventRecord(d.ev[0], d.stream));
            if (d.P > 1) k_setup<T><<<1, kSetupThreads, 0, d.stream>>>(d.S, d.d_shooters, d.d_state, d.d_part, d.n_cta_nf, d.conv, d.P);
            CU(cudaEventRecord(d.ev[1], d.stream));
            CU(launch_shoot(d, d.stream));
            CU(cudaGetLastError());
            CU(cudaEventRecord(d.ev[2], d.stream));
        } else {
            cudaGraphExec_t g;
            if ((rc = graph_for(d, chunk, &g))) return rc;
            if (mode) CU(cudaEventRecord(d.ev[0], d.stream));
            if (g) {
                CU(cudaGraphLaunch(g, d.stream));
            } else {
                for (int k = 0; k < chunk; k++)
                    if ((rc = launch_step(d, d.stream))) return rc;
            }
            if (mode) CU(cudaEventRecord(d.ev[2], d.stream));
        }
        CU(cudaMemcpyAsync(&d.host, d.d_state, sizeof(State), cudaMemcpyDeviceToHost, d.stream));
        CU(cudaStreamSynchronize(d.stream));
        if (mode == 1) {
            float ms = 0;
            CU(cudaEventElapsedTime(&ms, d.ev[0], d.ev[2]));
            if (ms_a) *ms_a += ms;
        } else if (mode == 2) {
            float a = 0, b = 0;
            CU(cudaEventElapsedTime(&a, d.ev[0], d.ev[1]));
            CU(cudaEventElapsedTime(&b, d.ev[1], d.ev[2]));
            if (ms_a) *ms_a += a;
            if (ms_b) *ms_b += b;
        }
        if (d.host.done || d.host.paused) break;
    }
    if (done_steps) *done_steps = d.host.steps - start;
    if (converged) *converged = d.host.done;
    if (d.host.capped) return fail(RAD_ERR_WALK, "a visibility walk reached walk_cap");
    return RAD_OK;
}

template <typename T>
int download(DevImpl<T>& d, Scene<T>& s) {
    const int n = d.S.n;
    if (n != s.trinum) return fail(RAD_ERR_ARG, "scene slot count differs from the device copy");
    CU(cudaSetDevice(d.device));
    // through this thread's pinned staging: accB (3 records per slot), deltaB (1)
    void* stage_p = nullptr;
    CU(pinned_stage().get((size_t)n * 4 * sizeof(Q4<T>), &stage_p));
    Q4<T>* acc = static_cast<Q4<T>*>(stage_p);
    Q4<T>* db = acc + (size_t)n * 3;
    if (n) {
        CU(cudaMemcpyAsync(acc, d.S.accB, (size_t)n * 3 * sizeof(Q4<T>), cudaMemcpyDeviceToHost, d.stream));
        CU(cudaMemcpyAsync(db, d.S.deltaB, (size_t)n * sizeof(Q4<T>), cudaMemcpyDeviceToHost, d.stream));
    }
    CU(cudaStreamSynchronize(d.stream));
    split_range(n, pack_jobs(n, s.opt.jobs), [&](int a, int b) {
        for (int i = a; i < b; i++) {
            Slot<T>& t = s.slots[i];
            for (int v = 0; v < 3; v++) {
                t.accB[v][0] = acc[i * 3 + v].x; t.accB[v][1] = acc[i * 3 + v].y; t.accB[v][2] = acc[i * 3 + v].z;
            }
            t.deltaB[0] = db[i].x; t.deltaB[1] = db[i].y; t.deltaB[2] = db[i].z;
        }
    });
    return RAD_OK;
}

template <typename T>
int ray_hit(DevImpl<T>& d, const T* p, const T* v, const int32_t* ban, int n, int32_t* hit) {
    if (n <= 0) return RAD_OK;
    CU(cudaSetDevice(d.device));
    T *dp, *dv;
    int *db, *dh;
    CU(cudaMallocAsync(&dp, (size_t)n * 3 * sizeof(T), d.stream));
    CU(cudaMallocAsync(&dv, (size_t)n * 3 * sizeof(T), d.stream));
    CU(cudaMallocAsync(&db, (size_t)n * 4, d.stream));
    CU(cudaMallocAsync(&dh, (size_t)n * 4, d.stream));
    CU(cudaMemcpyAsync(dp, p, (size_t)n * 3 * sizeof(T), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(dv, v, (size_t)n * 3 * sizeof(T), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(db, ban, (size_t)n * 4, cudaMemcpyHostToDevice, d.stream));
    k_ray_hit<T><<<(n + 255) / 256, 256, 0, d.stream>>>(d.G, dp, dv, db, n, dh, d.d_state);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(hit, dh, (size_t)n * 4, cudaMemcpyDeviceToHost, d.stream));
    CU(cudaFreeAsync(dp, d.stream));
    CU(cudaFreeAsync(dv, d.stream));
    CU(cudaFreeAsync(db, d.stream));
    CU(cudaFreeAsync(dh, d.stream));
    CU(cudaStreamSynchronize(d.stream));
    return RAD_OK;
}

template <typename T>
int form_factors(DevImpl<T>& d, int src, const int32_t* rcv, int n, T* ff) {
    if (src < 0 || src >= d.S.n) return fail(RAD_ERR_ARG, "shooter slot out of range");
    for (int i = 0; i < n; i++)
        if (rcv[i] < 0 || rcv[i] >= d.S.n) return fail(RAD_ERR_ARG, "receiver slot out of range");
    if (n <= 0) return RAD_OK;
    CU(cudaSetDevice(d.device));
    Shooter<T>* ds;
    int* dr;
    T* df;
    CU(cudaMallocAsync(&ds, sizeof(Shooter<T>), d.stream));
    CU(cudaMallocAsync(&dr, (size_t)n * 4, d.stream));
    CU(cudaMallocAsync(&df, (size_t)n * 3 * sizeof(T), d.stream));
    CU(cudaMemcpyAsync(dr, rcv, (size_t)n * 4, cudaMemcpyHostToDevice, d.stream));
    k_build_one<T><<<1, 32, 0, d.stream>>>(d.S, src, ds);
    k_form_factors<T><<<(3 * n + 255) / 256, 256, 0, d.stream>>>(d.S, d.G, ds, dr, n, df, d.d_state);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(ff, df, (size_t)n * 3 * sizeof(T), cudaMemcpyDeviceToHost, d.stream));
    CU(cudaFreeAsync(ds, d.stream));
    CU(cudaFreeAsync(dr, d.stream));
    CU(cudaFreeAsync(df, d.stream));
    CU(cudaStreamSynchronize(d.stream));
    return RAD_OK;
}

// Device address of g_noalloc_shooters, looked up once per device with that
// device current (a host-side use of the symbol's name is not a device address).
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};

int noalloc_scratch(int device, void** out) {
    if (device < 0 || device >= 64) return fail(RAD_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        int cur = 0;
        CU(cudaGetDevice(&cur));
        if (cur != device) CU(cudaSetDevice(device));
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_shooters);
        if (cur != device) cudaSetDevice(cur);
        if (e != cudaSuccess) return fail(RAD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return RAD_OK;
}

template <typename T>
int form_factors_noalloc(DevImpl<T>& d, const int32_t* src, int n_src, const int32_t* d_rcv, int n_rcv, T* d_ff,
                         cudaStream_t stream) {
    if (n_src < 1 || n_src > kNoAllocMaxShooters)
        return fail(RAD_ERR_CAPACITY, "rad_dev_form_factors_noalloc: 1 to 64 shooters per call");
    if (n_rcv < 0 || (n_rcv > 0 && (!d_rcv || !d_ff)) || !src)
        return fail(RAD_ERR_ARG, "rad_dev_form_factors_noalloc: bad argument");
    if ((long long)n_src * n_rcv * 3 > 0x7fffffffLL)
        return fail(RAD_ERR_CAPACITY, "rad_dev_form_factors_noalloc: n_src * n_rcv * 3 exceeds 2^31-1");
    ShooterSlots slots{};
    for (int j = 0; j < n_src; j++) {
        if (src[j] < 0 || src[j] >= d.S.n) return fail(RAD_ERR_ARG, "shooter slot out of range");
        slots.slot[j] = src[j];
    }
    // the handle's device is made current for the launches; the caller's
    // current device is restored on every path out
    int caller_dev = 0;
    CU(cudaGetDevice(&caller_dev));
    struct Restore {
        int dev;
        bool on;
        ~Restore() { if (on) cudaSetDevice(dev); }
    } restore{caller_dev, caller_dev != d.device};
    if (caller_dev != d.device) CU(cudaSetDevice(d.device));
    void* scratch = nullptr;
    int rc = noalloc_scratch(d.device, &scratch);
    if (rc) return rc;
    Shooter<T>* sh = reinterpret_cast<Shooter<T>*>(scratch);
    k_build_many<T><<<1, kNoAllocMaxShooters, 0, stream>>>(d.S, slots, n_src, sh);
    const long long work = 3LL * n_rcv * n_src;
    if (work > 0)
        k_form_factors_many<T><<<(unsigned)((work + 255) / 256), 256, 0, stream>>>(d.S, d.G, sh, n_src, d_rcv, n_rcv,
                                                                                 d_ff, d.d_state);
    CU(cudaGetLastError());
    return RAD_OK;
}

}  // namespace

struct rad_dev {
    int precision = 32;
    DevImpl<float>* d32 = nullptr;
    DevImpl<double>* d64 = nullptr;
    ~rad_dev() { delete d32; delete d64; }
};

extern "C" {

int rad_dev_create(const rad_scene* s, const rad_octree* t, const rad_options* o, int32_t device, rad_dev** out) {
    if (!s || !t || !o || !out) return fail(RAD_ERR_ARG, "rad_dev_create: null argument");
    if (s->precision != t->precision) return fail(RAD_ERR_ARG, "scene and octree precision differ");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RAD_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(RAD_ERR_ARG, "device index out of range");
    rad_dev* h = new rad_dev();
    h->precision = s->precision;
    int rc;
    if (s->precision == 32) {
        h->d32 = new DevImpl<float>();
        rc = upload(s->s32, t->o32, *o, device, *h->d32);
    } else {
        h->d64 = new DevImpl<double>();
        rc = upload(s->s64, t->o64, *o, device, *h->d64);
    }
    if (rc) { delete h; return rc; }
    *out = h;
    return RAD_OK;
}

int rad_dev_run(rad_dev* h, int64_t max_steps, int64_t* steps_done, int32_t* converged) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_run: null handle");
    long long sd = 0;
    int cv = 0;
    int rc = h->d32 ? run(*h->d32, max_steps, &sd, &cv, 0, nullptr, nullptr)
                    : run(*h->d64, max_steps, &sd, &cv, 0, nullptr, nullptr);
    if (steps_done) *steps_done = sd;
    if (converged) *converged = cv;
    return rc;
}

int rad_dev_stream(const rad_dev* h, void** stream) {
    if (!h || !stream) return fail(RAD_ERR_ARG, "rad_dev_stream: null argument");
    *stream = h->d32 ? (void*)h->d32->stream : (void*)h->d64->stream;
    return RAD_OK;
}

int rad_dev_run_timed(rad_dev* h, int64_t max_steps, int64_t* steps_done, int32_t* converged, double* device_ms) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_run_timed: null handle");
    long long sd = 0;
    int cv = 0;
    double ms = 0;
    int rc = h->d32 ? run(*h->d32, max_steps, &sd, &cv, 1, &ms, nullptr)
                    : run(*h->d64, max_steps, &sd, &cv, 1, &ms, nullptr);
    if (steps_done) *steps_done = sd;
    if (converged) *converged = cv;
    if (device_ms) *device_ms = ms;
    return rc;
}

int rad_dev_run_profiled(rad_dev* h, int64_t max_steps, int64_t* steps_done, int32_t* converged, double* ms_setup,
                         double* ms_shoot) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_run_profiled: null handle");
    long long sd = 0;
    int cv = 0;
    int rc = h->d32 ? run(*h->d32, max_steps, &sd, &cv, 2, ms_setup, ms_shoot)
                    : run(*h->d64, max_steps, &sd, &cv, 2, ms_setup, ms_shoot);
    if (steps_done) *steps_done = sd;
    if (converged) *converged = cv;
    return rc;
}

int rad_dev_download(rad_dev* h, rad_scene* s) {
    if (!h || !s) return fail(RAD_ERR_ARG, "rad_dev_download: null argument");
    if (s->precision != h->precision) return fail(RAD_ERR_ARG, "precision differs");
    return h->d32 ? download(*h->d32, s->s32) : download(*h->d64, s->s64);
}

int rad_dev_trace(const rad_dev* h, int32_t* out, int64_t cap, int64_t* n) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_trace: null handle");
    auto go = [&](auto& d) -> int {
        long long have = std::min<long long>(d.host.steps * d.P, d.trace_cap);
        if (n) *n = have;
        if (!out || cap <= 0) return RAD_OK;
        long long k = std::min<long long>(have, cap);
        CU(cudaSetDevice(d.device));
        CU(cudaMemcpy(out, d.d_trace, (size_t)k * 4, cudaMemcpyDeviceToHost));
        return RAD_OK;
    };
    return h->d32 ? go(*h->d32) : go(*h->d64);
}

int rad_dev_stats(const rad_dev* h, rad_stats* st) {
    if (!h || !st) return fail(RAD_ERR_ARG, "rad_dev_stats: null argument");
    auto go = [&](auto& d) -> int {
        CU(cudaSetDevice(d.device));
        CU(cudaMemcpyAsync(&d.host, d.d_state, sizeof(State), cudaMemcpyDeviceToHost, d.stream));
        CU(cudaStreamSynchronize(d.stream));
        std::memset(st, 0, sizeof *st);
        st->steps = d.host.steps;
        st->shots = 0;
        st->rays = (int64_t)d.host.rays;
        st->rays_ref = (int64_t)d.host.rays_ref;
        st->cells = (int64_t)d.host.cells;
        st->tri_tests = (int64_t)d.host.tris;
        st->se_tests = (int64_t)d.host.se;
        st->prec_steps = (int64_t)d.host.prec;
        st->walk_cap_hits = (int64_t)d.host.capped;
        st->walk_loops = (int64_t)d.host.loops;
        st->converged = d.host.done;
        st->n_slots = d.S.n;
        st->device_bytes = (int64_t)(d.bytes + (d.trace_own ? d.trace_cap * 4 : 0));
        st->h2d_bytes = (int64_t)d.h2d_bytes;
        using TT = typename std::remove_reference<decltype(d)>::type::Real;
        k_unshot<TT><<<kUnshotCtas, kUnshotThreads, 0, d.stream>>>(d.S, d.d_unshot);
        k_unshot_total<<<1, 32, 0, d.stream>>>(d.d_unshot, kUnshotCtas, d.d_unshot + kUnshotCtas);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(&st->unshot_power, d.d_unshot + kUnshotCtas, sizeof(double), cudaMemcpyDeviceToHost,
                           d.stream));
        CU(cudaStreamSynchronize(d.stream));
        return RAD_OK;
    };
    int rc = h->d32 ? go(*h->d32) : go(*h->d64);
    if (rc) return rc;
    // shooters processed: count the trace entries that name a slot
    const long long steps = st->steps;
    const int P = h->d32 ? h->d32->P : h->d64->P;
    if (P == 1) {
        st->shots = steps;
    } else {
        std::vector<int32_t> tr((size_t)steps * P);
        int64_t n = 0;
        if ((rc = rad_dev_trace(h, tr.data(), (int64_t)tr.size(), &n))) return rc;
        for (int64_t k = 0; k < n; k++) st->shots += tr[k] >= 0;
    }
    return RAD_OK;
}

int rad_dev_set_schedule(rad_dev* h, double split_frac, double split_frac_split, double split_mean_mult,
                         double early_mean_mult) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_set_schedule: null handle");
    if (!(split_frac >= 0) || !(split_frac_split >= 0) || !(split_mean_mult >= 0) || !(early_mean_mult >= 0))
        return fail(RAD_ERR_ARG, "rad_dev_set_schedule: limits must be >= 0");
    auto go = [&](auto& d) -> int {
        CU(cudaSetDevice(d.device));
        const double v[4] = {split_frac, split_frac_split, split_mean_mult, early_mean_mult};
        CU(cudaMemcpyAsync(&d.d_state->frac, v, sizeof v, cudaMemcpyHostToDevice, d.stream));
        CU(cudaStreamSynchronize(d.stream));
        return RAD_OK;
    };
    return h->d32 ? go(*h->d32) : go(*h->d64);
}

int rad_dev_autotune(rad_dev* h, int32_t steps_per_trial, int64_t max_steps, int64_t* steps_done,
                     int32_t* converged, int32_t* chosen) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_autotune: null handle");
    if (steps_per_trial < 1 || steps_per_trial > 32) return fail(RAD_ERR_ARG, "rad_dev_autotune: steps_per_trial must be 1..32");
    long long total = 0;
    int cv = 0, walk_rc = RAD_OK;
    // a capped walk (RAD_ERR_WALK) is reported at the end, as rad_dev_run does
    auto go_run = [&](auto& d, long long n, double* ms) -> int {
        long long sd = 0;
        int c = 0;
        int rc = run(d, n, &sd, &c, ms ? 1 : 0, ms, nullptr);
        total += sd;
        if (c) cv = 1;
        if (rc == RAD_ERR_WALK) {
            walk_rc = rc;
            rc = RAD_OK;
        }
        return rc;
    };
    if (h->d32 && h->d32->P == 1 && !h->d32->counting) {
        DevImpl<float>& d = *h->d32;
        const int before = d.layout;
        // one untimed step per form (first launches), then trials of both
        // forms in alternating order until max_steps is used up
        double ms[3] = {0, 0, 0};
        long long n[3] = {0, 0, 0};
        for (int r = 0; !cv && total < max_steps; r++) {
            for (int k = 0; k < 2 && !cv && total < max_steps; k++) {
                const int layout = ((r + k) & 1) ? 2 : 1;
                d.layout = layout;
                d.n_cta = d.n_cta_of(layout);
                if (r == 0) {
                    int rc = go_run(d, 1, nullptr);
                    if (rc) return rc;
                    continue;
                }
                const long long want = std::min<long long>(steps_per_trial, max_steps - total);
                const long long had = total;
                double t = 0;
                int rc = go_run(d, want, &t);
                if (rc) return rc;
                ms[layout] += t;
                n[layout] += total - had;
            }
        }
        int best = before;
        if (n[1] > 0 && n[2] > 0) best = ms[2] / (double)n[2] < ms[1] / (double)n[1] ? 2 : 1;
        d.layout = best;
        d.n_cta = d.n_cta_of(best);
    } else if (max_steps > 0) {
        // one form only: the steps run as rad_dev_run would run them
        int rc = h->d32 ? go_run(*h->d32, max_steps, nullptr) : go_run(*h->d64, max_steps, nullptr);
        if (rc) return rc;
    }
    if (steps_done) *steps_done = total;
    if (converged) *converged = cv;
    if (chosen) *chosen = h->d32 ? h->d32->layout : 1;
    return walk_rc;
}

int rad_dev_set_layout(rad_dev* h, int32_t layout) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_set_layout: null handle");
    if (layout < 0 || layout > 2) return fail(RAD_ERR_ARG, "rad_dev_set_layout: layout must be 0, 1 or 2");
    if (h->d32) {
        DevImpl<float>& d = *h->d32;
        if (layout == 0) {
            int sms = 0, per2 = 0;
            CU(cudaSetDevice(d.device));
            CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d.device));
            CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_shoot<float, false, true, 4, 1>, kShootThreads,
                                                             d.shoot_smem()));
            const int n_groups = (d.S.n + kSlotsPerWarp - 1) / kSlotsPerWarp;
            const long long warps2 = (long long)sms * std::max(per2, 1) * (kShootThreads / 32);
            layout = (d.P == 1 && n_groups > 4 * warps2) ? 2 : 1;
        }
        if (layout == 2 && d.P != 1) layout = 1;
        d.layout = layout;
        d.n_cta = d.n_cta_of(layout);
    }
    return RAD_OK;   // the FP64 solver has only the tail-bound form
}

int rad_dev_layout(const rad_dev* h) {
    if (!h) return 0;
    return h->d32 ? h->d32->layout : 1;
}

int rad_dev_set_counting(rad_dev* h, int32_t on) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_set_counting: null handle");
    if (h->d32) h->d32->counting = on != 0; else h->d64->counting = on != 0;
    return RAD_OK;
}

int rad_dev_ray_hit(rad_dev* h, const void* p, const void* v, const int32_t* ban, int32_t n, int32_t* hit) {
    if (!h || (n > 0 && (!p || !v || !ban || !hit))) return fail(RAD_ERR_ARG, "rad_dev_ray_hit: null argument");
    return h->d32 ? ray_hit(*h->d32, (const float*)p, (const float*)v, ban, n, hit)
                  : ray_hit(*h->d64, (const double*)p, (const double*)v, ban, n, hit);
}

int rad_dev_form_factors(rad_dev* h, int32_t src, const int32_t* rcv, int32_t n, void* ff) {
    if (!h || (n > 0 && (!rcv || !ff))) return fail(RAD_ERR_ARG, "rad_dev_form_factors: null argument");
    return h->d32 ? form_factors(*h->d32, src, rcv, n, (float*)ff) : form_factors(*h->d64, src, rcv, n, (double*)ff);
}

int rad_dev_form_factors_noalloc(rad_dev* h, const int32_t* src, int32_t n_src, const int32_t* d_rcv, int32_t n_rcv,
                                 void* d_ff, void* stream) {
    if (!h) return fail(RAD_ERR_ARG, "rad_dev_form_factors_noalloc: null handle");
    cudaStream_t s = (cudaStream_t)stream;
    return h->d32 ? form_factors_noalloc(*h->d32, src, n_src, d_rcv, n_rcv, (float*)d_ff, s)
                  : form_factors_noalloc(*h->d64, src, n_src, d_rcv, n_rcv, (double*)d_ff, s);
}

void rad_dev_destroy(rad_dev* h) { delete h; }

}  // extern "C"
