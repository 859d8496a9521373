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

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "capi_internal.h"

namespace radgb {
namespace dev {

constexpr int kShootThreads = 256;
constexpr int kSlotsPerWarp = 10;
constexpr int kSlotsPerCta = kSlotsPerWarp * (kShootThreads / 32);   // 80
constexpr int kSetupThreads = 1024;
constexpr int kMaxShooters = 256;
constexpr double kPiD = 3.1415926535897932;
constexpr unsigned kFull = 0xffffffffu;

template <typename T> struct alignas(4 * sizeof(T)) Q4 { T x, y, z, w; };

// integers carried in the 4th lane of a record, bit-exact
__host__ __device__ inline float int_to_real(int v, float*) {
#ifdef __CUDA_ARCH__
    return __int_as_float(v);
#else
    float f; std::memcpy(&f, &v, 4); return f;
#endif
}
__host__ __device__ inline double int_to_real(int v, double*) {
    long long w = v;
#ifdef __CUDA_ARCH__
    return __longlong_as_double(w);
#else
    double d; std::memcpy(&d, &w, 8); return d;
#endif
}
__device__ __forceinline__ int real_to_int(float f) { return __float_as_int(f); }
__device__ __forceinline__ int real_to_int(double d) { return (int)__double_as_longlong(d); }
template <typename T> inline T pack_int(int v) { return int_to_real(v, (T*)nullptr); }

// order-preserving integer image of a key (+0 and -0 equal, as in the
// reference's pair<float,int> comparison); candidates always map above 0
__device__ __forceinline__ unsigned long long key_order(float f) {
    unsigned u = __float_as_uint(f == 0.0f ? 0.0f : f);
    return (u & 0x80000000u) ? (unsigned long long)(~u) : (unsigned long long)(u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long key_order(double f) {
    unsigned long long u = (unsigned long long)__double_as_longlong(f == 0.0 ? 0.0 : f);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// Visibility structure (kernel parameter; constant for a handle).
template <typename T>
struct Grid {
    T g0[3], g1[3];
    T inv_grid;                              // 1 / MinGridLen, for the first guess only
    T t_eps, v_eps;                          // exact FP32 images of the 0.0001 and 1e-6 tests
    int dims[3];
    int thr_off[3];
    int n_thr;
    const T* thr;                            // cell-coordinate thresholds (global; staged to smem)
    const int32_t* __restrict__ cell_leaf;   // cell coordinate triple -> leaf
    const Q4<T>* __restrict__ leaf;          // 2 per leaf: (g0, begin) (g1, end)
    const Q4<T>* __restrict__ entry;         // 5 per list entry: (n, id) (c, 0) se0 se1 se2
    int walk_cap;
};

// Slot store, SoA of 4-wide records.
template <typename T>
struct Slots {
    int n;
    const Q4<T>* __restrict__ vtx;   // 3 per slot
    const Q4<T>* __restrict__ nrm;   // normal, w = |n| (norm() of the reference)
    const Q4<T>* __restrict__ ctr;   // centre, w = area
    const Q4<T>* __restrict__ frgb;  // reflectance 0..255, w = parent
    Q4<T>* accB;                     // 3 per slot (w unused)
    Q4<T>* deltaB;                   // 1 per slot (w unused)
};

template <typename T>
struct Patch { T c[3]; T area; };

template <typename T>
struct Shooter {
    int slot, logsrc, split, pad;
    T n[3];
    T nlen;
    T deltaB[3];
    T pad2;
    Patch<T> part[3];   // whole source, half 1, half 2
};

struct Partial { unsigned long long key; int slot; int pad; };

// dynamic shared memory of k_shoot: shooter records, then the thresholds
template <typename T>
__host__ __device__ inline size_t kMaxShooterBytes(int nsh) {
    return ((size_t)nsh * sizeof(Shooter<T>) + 15) & ~(size_t)15;
}

struct State {
    int work;               // next 10-slot group of the current step (k_shoot queue)
    int done;               // a selection found no candidate
    int paused;             // step limit reached
    int nsh;                // shooters of the current step
    int err;
    long long steps;
    long long step_limit;
    long long trace_cap;
    int* trace;
    unsigned long long rays, rays_ref, cells, tris, se, prec, capped;
};

struct Cnt { unsigned rays, rays_ref, cells, tris, se, prec, capped; };

// Cell coordinate along one axis: a first guess in T, corrected against the
// thresholds so the result equals the reference's FP64 expression exactly.
template <typename T>
__device__ __forceinline__ int cell_axis(T q, T g0, T inv, const T* th, int D) {
    int k = (int)((q - g0) * inv);
    k = min(max(k, 0), D - 1);
    while (k + 1 < D && q >= th[k + 1]) ++k;
    while (k > 0 && q < th[k]) --k;
    return k;
}

// ------------------------------------------------------------------ walk
// RayHitted (raycast.cpp:335-360) with TreeNodeNum (254-281) as a table
// lookup, TriListHitted/TriHitted (283-333) and NextPoint (235-251).
template <typename T, bool COUNT>
__device__ __forceinline__ int walk(const Grid<T>& G, const T p[3], const T v[3], int ban, Cnt& c) {
    T t = 0;
    int prev = -1;
    T q0 = p[0], q1 = p[1], q2 = p[2];
    for (int it = 0; it < G.walk_cap; ++it) {
        if (q0 < G.g0[0] || q0 > G.g1[0] || q1 < G.g0[1] || q1 > G.g1[1] || q2 < G.g0[2] || q2 > G.g1[2])
            return -1;
        if (COUNT) c.cells++;
        // (int)(((double)q - G0) / MinGridLen) per axis, found exactly from the thresholds
        const int gx = cell_axis(q0, G.g0[0], G.inv_grid, G.thr + G.thr_off[0], G.dims[0]);
        const int gy = cell_axis(q1, G.g0[1], G.inv_grid, G.thr + G.thr_off[1], G.dims[1]);
        const int gz = cell_axis(q2, G.g0[2], G.inv_grid, G.thr + G.thr_off[2], G.dims[2]);
        const int leaf = __ldg(&G.cell_leaf[(gx * G.dims[1] + gy) * G.dims[2] + gz]);
        if (leaf == prev) {          // "Precision Exceeded": step one unit of t
            if (COUNT) c.prec++;
            t = (T)((double)t + 1.0);
            q0 = p[0] + t * v[0]; q1 = p[1] + t * v[1]; q2 = p[2] + t * v[2];
            continue;
        }
        const Q4<T> lo = G.leaf[2 * leaf], hi = G.leaf[2 * leaf + 1];
        const int b = real_to_int(lo.w), e = real_to_int(hi.w);
        T tmin = (T)1000000.0;
        int best = -1;
        for (int k = b; k < e; ++k) {
            const Q4<T> en = G.entry[5 * k];
            const int id = real_to_int(en.w);
            if (id == ban) continue;
            const Q4<T> ec = G.entry[5 * k + 1];
            if (COUNT) c.tris++;
            const T a1 = v[0] * en.x + v[1] * en.y + v[2] * en.z;
            const T w0 = ec.x - p[0], w1 = ec.y - p[1], w2 = ec.z - p[2];
            const T a2 = w0 * en.x + w1 * en.y + w2 * en.z;
            const T tt = a2 / a1;
            if (tt < G.t_eps) continue;            // (double)t < 0.0001
            if (tt >= tmin) continue;
            if (COUNT) c.se++;
            const T x = p[0] + tt * v[0], y = p[1] + tt * v[1], z = p[2] + tt * v[2];
            const Q4<T> s0 = G.entry[5 * k + 2];
            if ((x * s0.x + y * s0.y + z * s0.z + s0.w) < 0.0) continue;
            const Q4<T> s1 = G.entry[5 * k + 3];
            if ((x * s1.x + y * s1.y + z * s1.z + s1.w) < 0.0) continue;
            const Q4<T> s2 = G.entry[5 * k + 4];
            if ((x * s2.x + y * s2.y + z * s2.z + s2.w) < 0.0) continue;
            tmin = tt;
            best = id;
        }
        if (best >= 0) return best;
        prev = leaf;
        // NextPoint: leave the cell from the ray origin, overshoot by 0.1 in t
        const T bl[3] = {lo.x, lo.y, lo.z}, bh[3] = {hi.x, hi.y, hi.z};
        T tm = (T)1000000.0;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (fabs(v[a]) > G.v_eps) {             // fabs((double)v) > 1e-6
                const T s = (v[a] > 0) ? (bh[a] - p[a]) / v[a] : (bl[a] - p[a]) / v[a];
                tm = (s < tm) ? s : tm;
            }
        }
        tm = (T)((double)tm + 0.1);
        q0 = p[0] + tm * v[0]; q1 = p[1] + tm * v[1]; q2 = p[2] + tm * v[2];
        t = tm;
    }
    c.capped++;
    return -2;
}

template <typename T> __device__ __forceinline__ T rsqrt_exact(T x);
template <> __device__ __forceinline__ float rsqrt_exact<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double rsqrt_exact<double>(double x) { return sqrt(x); }

// CalFF, shade.cpp:107-127: the pre-test is cheap, the walk is not
template <typename T, bool COUNT, bool WALK>
__device__ __forceinline__ T point_ff(const Shooter<T>& s, const Patch<T>& src, const T p[3], const T nd[3], T ndlen,
                                      int logdes, const Grid<T>& G, Cnt& c) {
    const T d[3] = {src.c[0] - p[0], src.c[1] - p[1], src.c[2] - p[2]};
    const T ds = d[0] * s.n[0] + d[1] * s.n[1] + d[2] * s.n[2];
    const T dd = -(d[0] * nd[0] + d[1] * nd[1] + d[2] * nd[2]);
    if ((ds < 0) != (dd < 0)) return 0;
    const T d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const T dl = rsqrt_exact<T>(d2);
    const T c1 = ds / dl / s.nlen;
    const T c2 = dd / dl / ndlen;
    T ff = c1 * c2;
    if (ff <= 0.0) return 0;
    ff = (T)((double)ff * ((double)src.area / ((double)d2 * kPiD)));
    if (ff <= 0.0) return 0;
    if (!WALK) return ff;   // pre-test only (reference ray accounting)
    c.rays++;
    return walk<T, COUNT>(G, p, d, logdes, c) == s.logsrc ? ff : (T)0;
}

// Shade's per-corner AdaptCalFF(CalFF(...)), shade.cpp:442-450 with the
// stray ';' at shade.cpp:164: a split source returns ff(half1)+ff(half2); the
// whole-source result is discarded, so its walk is not cast.
template <typename T, bool COUNT>
__device__ __forceinline__ T corner_ff(const Shooter<T>& s, const T p[3], const T nd[3], T ndlen, int logdes,
                                       const Grid<T>& G, Cnt& c) {
    const unsigned before = c.rays;
    if (!s.split) {
        const T f = point_ff<T, COUNT, true>(s, s.part[0], p, nd, ndlen, logdes, G, c);
        if (COUNT) c.rays_ref += c.rays - before;
        return f;
    }
    if (COUNT && point_ff<T, COUNT, false>(s, s.part[0], p, nd, ndlen, logdes, G, c) > (T)0) c.rays_ref++;
    const T f1 = point_ff<T, COUNT, true>(s, s.part[1], p, nd, ndlen, logdes, G, c);
    const T f2 = point_ff<T, COUNT, true>(s, s.part[2], p, nd, ndlen, logdes, G, c);
    if (COUNT) c.rays_ref += c.rays - before;
    return f1 + f2;
}

template <typename T>
__device__ __forceinline__ T shfl(T v, int src) { return __shfl_sync(kFull, v, src); }

__device__ __forceinline__ bool part_less(unsigned long long ka, int ia, unsigned long long kb, int ib) {
    return ka < kb || (ka == kb && ia < ib);
}

__device__ __forceinline__ void warp_max(unsigned long long& k, int& i) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        unsigned long long k2 = __shfl_xor_sync(kFull, k, o);
        int i2 = __shfl_xor_sync(kFull, i, o);
        if (part_less(k, i, k2, i2)) { k = k2; i = i2; }
    }
}

template <bool COUNT>
__device__ __forceinline__ void flush_counters(State* st, Cnt& c, int lane) {
    unsigned v[7] = {c.rays, c.rays_ref, c.cells, c.tris, c.se, c.prec, c.capped};
    unsigned long long* dst[7] = {&st->rays, &st->rays_ref, &st->cells, &st->tris, &st->se, &st->prec, &st->capped};
    const int nc = COUNT ? 7 : 1;
#pragma unroll
    for (int q = 0; q < 7; q++) {
        if (q >= nc && q != 6) continue;
        unsigned s = __reduce_add_sync(kFull, v[q]);
        if (lane == 0 && s) atomicAdd(dst[q], (unsigned long long)s);
    }
}

// ------------------------------------------------------------------ k_shoot
// One 10-slot group: lanes 3r+v are corner v of slot g*10+r.
template <typename T, bool COUNT>
__device__ __forceinline__ void shoot_group(const Slots<T>& S, const Grid<T>& G, const Shooter<T>* sh, int nsh,
                                            int g, int lane, T conv, unsigned long long& kk, int& ks, Cnt& c) {
    const int r = lane / 3, v = lane - 3 * r;
    const int i = g * kSlotsPerWarp + r;
    const bool own = lane < 3 * kSlotsPerWarp && i < S.n;

    Q4<T> fr = {0, 0, 0, (T)-1}, acc = {0, 0, 0, 0}, db = {0, 0, 0, 0};
    if (own) {
        fr = S.frgb[i];
        acc = S.accB[i * 3 + v];
    }
    const int parent = (int)fr.w;
    const bool live = own && parent >= 0;
    bool is_src = false;
    for (int j = 0; j < nsh; j++) is_src |= (sh[j].slot == i);
    // a receiver is skipped only when all nine accB components are >= 255
    const bool open_v = live && (acc.x < (T)255 || acc.y < (T)255 || acc.z < (T)255);
    const unsigned ballot = __ballot_sync(kFull, open_v);
    const int base = 3 * min(r, kSlotsPerWarp - 1);
    const bool open = ((ballot >> base) & 7u) != 0;
    const bool active = live && !is_src && open && nsh > 0;
    if (live && v == 0) db = S.deltaB[i];

    T pv[3] = {0, 0, 0}, nd[3] = {0, 0, 0}, ndlen = 1;
    if (active) {
        const Q4<T> pp = S.vtx[i * 3 + v];
        const Q4<T> nn = S.nrm[i];
        pv[0] = pp.x; pv[1] = pp.y; pv[2] = pp.z;
        nd[0] = nn.x; nd[1] = nn.y; nd[2] = nn.z;
        ndlen = nn.w;
    }
    const T k = (T)(0.5 / 255.0);   // RefRatio / 255.0, shade.cpp:246
    T a0 = acc.x, a1 = acc.y, a2 = acc.z;
    T d0 = db.x, d1 = db.y, d2 = db.z;
    for (int j = 0; j < nsh; j++) {
        T ff = 0;
        if (active) ff = corner_ff<T, COUNT>(sh[j], pv, nd, ndlen, parent, G, c);
        const T f0 = shfl(ff, base), f1 = shfl(ff, base + 1), f2 = shfl(ff, base + 2);
        if (active) {
            const T lo0 = fr.x * k * sh[j].deltaB[0] / 3;
            const T lo1 = fr.y * k * sh[j].deltaB[1] / 3;
            const T lo2 = fr.z * k * sh[j].deltaB[2] / 3;
            a0 += lo0 * ff; a1 += lo1 * ff; a2 += lo2 * ff;
            if (v == 0) {
                d0 += lo0 * f0; d0 += lo0 * f1; d0 += lo0 * f2;
                d1 += lo1 * f0; d1 += lo1 * f1; d1 += lo1 * f2;
                d2 += lo2 * f0; d2 += lo2 * f1; d2 += lo2 * f2;
            }
        }
    }
    if (active) {
        Q4<T> o = {a0, a1, a2, acc.w};
        S.accB[i * 3 + v] = o;
        if (v == 0) { Q4<T> q = {d0, d1, d2, db.w}; S.deltaB[i] = q; }
    }
    if (live && is_src && v == 0) {       // rad.cpp:446-449
        d0 = d1 = d2 = 0;
        Q4<T> q = {0, 0, 0, db.w};
        S.deltaB[i] = q;
    }
    // next selection: key = (dB0 + dB1) + dB2 (rad.cpp:394), candidates > converge
    if (live && v == 0) {
        const T key = (d0 + d1) + d2;
        if (key > conv) {
            const unsigned long long o = key_order(key);
            if (part_less(kk, ks, o, i)) { kk = o; ks = i; }
        }
    }
}

// Persistent: each warp takes 10-slot groups from the step's queue until it
// is empty, so warps that finish early take more work; the CTA's (key, slot)
// maximum is written by whichever of its warps finishes last.
template <typename T, bool COUNT>
__global__ void __launch_bounds__(kShootThreads)
k_shoot(Slots<T> S, Grid<T> G, const Shooter<T>* __restrict__ shooters, State* st, Partial* __restrict__ part, T conv) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned long long wkey[kShootThreads / 32];
    __shared__ int wslot[kShootThreads / 32];
    __shared__ int ndone;
    if (st->done || st->paused) return;
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
    Cnt c = {0, 0, 0, 0, 0, 0, 0};
    for (;;) {
        int g = 0;
        if (lane == 0) g = atomicAdd(&st->work, 1);
        g = __shfl_sync(kFull, g, 0);
        if (g >= n_groups) break;
        shoot_group<T, COUNT>(S, Gs, sh, nsh, g, lane, conv, kk, ks, c);
    }
    warp_max(kk, ks);
    flush_counters<COUNT>(st, c, lane);
    if (lane == 0) {
        wkey[wid] = kk;
        wslot[wid] = ks;
        __threadfence_block();
        if (atomicAdd(&ndone, 1) == kShootThreads / 32 - 1) {
            volatile unsigned long long* vk = wkey;
            volatile int* vs = wslot;
            unsigned long long bk = 0;
            int bs = -1;
            for (int w = 0; w < kShootThreads / 32; w++)
                if (part_less(bk, bs, vk[w], vs[w])) { bk = vk[w]; bs = vs[w]; }
            part[blockIdx.x].key = bk;
            part[blockIdx.x].slot = bs;
        }
    }
}

// ------------------------------------------------------------------ k_setup
template <typename T>
__device__ void build_shooter(const Slots<T>& S, int slot, Shooter<T>& s) {
    const Q4<T> fr = S.frgb[slot], nn = S.nrm[slot], cc = S.ctr[slot], db = S.deltaB[slot];
    T p[3][3];
    for (int v = 0; v < 3; v++) {
        const Q4<T> q = S.vtx[slot * 3 + v];
        p[v][0] = q.x; p[v][1] = q.y; p[v][2] = q.z;
    }
    s.slot = slot;
    s.logsrc = (int)fr.w;
    s.pad = 0;
    s.n[0] = nn.x; s.n[1] = nn.y; s.n[2] = nn.z;
    s.nlen = nn.w;
    s.deltaB[0] = db.x; s.deltaB[1] = db.y; s.deltaB[2] = db.z;
    s.pad2 = 0;
    s.part[0].c[0] = cc.x; s.part[0].c[1] = cc.y; s.part[0].c[2] = cc.z;
    s.part[0].area = cc.w;
    // AdaptCalFF's split decision (shade.cpp:143-156): first longest edge
    int e = 0;
    T longest = 0;
    for (int v = 0; v < 3; v++) {
        const T l0 = p[(v + 1) % 3][0] - p[v][0], l1 = p[(v + 1) % 3][1] - p[v][1], l2 = p[(v + 1) % 3][2] - p[v][2];
        const T len = l0 * l0 + l1 * l1 + l2 * l2;
        if (longest < len) { longest = len; e = v; }
    }
    s.split = !((double)longest < 0.1);
    if (s.split) {   // PartitionSource, shade.cpp:76-99
        const int i0 = e, i1 = (e + 1) % 3, i2 = (e + 2) % 3;
        T m[3];
        for (int q = 0; q < 3; q++) m[q] = (T)((double)(p[i0][q] + p[i1][q]) / 2.0);
        for (int q = 0; q < 3; q++) {
            s.part[1].c[q] = (T)((double)(m[q] + p[i2][q] + p[i0][q]) / 3.0);
            s.part[2].c[q] = (T)((double)(m[q] + p[i1][q] + p[i2][q]) / 3.0);
        }
        s.part[1].area = s.part[2].area = (T)((double)cc.w / 2.0);
    } else {
        for (int h = 1; h < 3; h++) {
            for (int q = 0; q < 3; q++) s.part[h].c[q] = 0;
            s.part[h].area = 0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kSetupThreads)
k_setup(Slots<T> S, Shooter<T>* shooters, State* st, const Partial* __restrict__ part, int nparts, T conv, int P) {
    __shared__ unsigned long long bk[kSetupThreads / 32];
    __shared__ int bs[kSetupThreads / 32];
    __shared__ int bc[kSetupThreads / 32];
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
        // listCanditate for P > 1: n = min((|C|+4)/5, P) largest (key, slot)
        // pairs, descending; one block-wide argmax per rank
        unsigned long long lim_k = ~0ull;
        int lim_s = 0x7fffffff;
        int n_take = 0;
        for (int rank = 0; rank < P; rank++) {
            unsigned long long kk = 0;
            int ks = -1, cnt = 0;
            for (int i = threadIdx.x; i < S.n; i += blockDim.x) {
                const Q4<T> fr = S.frgb[i];
                if ((int)fr.w < 0) continue;
                const Q4<T> db = S.deltaB[i];
                const T key = (db.x + db.y) + db.z;
                if (!(key > conv)) continue;
                const unsigned long long o = key_order(key);
                cnt++;
                if (part_less(o, i, lim_k, lim_s) && part_less(kk, ks, o, i)) { kk = o; ks = i; }
            }
            warp_max(kk, ks);
            cnt = __reduce_add_sync(kFull, cnt);
            if (lane == 0) { bk[wid] = kk; bs[wid] = ks; bc[wid] = cnt; }
            __syncthreads();
            if (wid == 0) {
                kk = bk[lane];
                ks = bs[lane];
                int cc = __reduce_add_sync(kFull, bc[lane]);
                warp_max(kk, ks);
                if (lane == 0) {
                    if (rank == 0) nch = min((cc + 4) / 5, P);
                    chosen[rank] = ks;
                    bk[0] = kk;
                    bs[0] = ks;
                }
            }
            __syncthreads();
            lim_k = bk[0];
            lim_s = bs[0];
            n_take = nch;
            __syncthreads();
            if (rank + 1 >= n_take) break;
        }
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

// ------------------------------------------------------------------ queries
template <typename T>
__global__ void k_ray_hit(Grid<T> G, const T* __restrict__ p, const T* __restrict__ v, const int* __restrict__ ban,
                          int n, int* __restrict__ out, State* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    Cnt c = {0, 0, 0, 0, 0, 0, 0};
    if (i < n) {
        const T pp[3] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
        const T vv[3] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        out[i] = walk<T, false>(G, pp, vv, ban[i], c);
    }
    if (c.capped) atomicAdd(&st->capped, (unsigned long long)c.capped);
}

template <typename T>
__global__ void k_build_one(Slots<T> S, int slot, Shooter<T>* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) build_shooter(S, slot, *out);
}

template <typename T>
__global__ void k_form_factors(Slots<T> S, Grid<T> G, const Shooter<T>* __restrict__ shp, const int* __restrict__ rcv,
                               int n, T* __restrict__ ff, State* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    Cnt c = {0, 0, 0, 0, 0, 0, 0};
    if (t < 3 * n) {
        const Shooter<T> s = *shp;
        const int i = rcv[t / 3], v = t % 3;
        const Q4<T> pp = S.vtx[i * 3 + v], nn = S.nrm[i], fr = S.frgb[i];
        const T pv[3] = {pp.x, pp.y, pp.z}, nd[3] = {nn.x, nn.y, nn.z};
        ff[t] = corner_ff<T, false>(s, pv, nd, nn.w, (int)fr.w, G, c);
    }
    if (c.capped) atomicAdd(&st->capped, (unsigned long long)c.capped);
}

// ------------------------------------------------------------------ no-allocation variant
// Shooter records for rad_dev_form_factors_noalloc live in this fixed array
// instead of memory allocated per call.  Sized for the FP64 record, so it
// serves both precisions.
constexpr int kNoAllocMaxShooters = 64;
static __device__ __align__(256) unsigned char g_noalloc_shooters[kNoAllocMaxShooters * sizeof(Shooter<double>)];

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
    Cnt c = {0, 0, 0, 0, 0, 0, 0};
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
    int device = 0;
    cudaStream_t stream = nullptr;
    Slots<T> S{};
    Grid<T> G{};
    Shooter<T>* d_shooters = nullptr;
    State* d_state = nullptr;
    Partial* d_part = nullptr;
    int* d_trace = nullptr;
    long long trace_cap = 0;
    int n_cta = 0;
    int P = 1;
    T conv = 0;
    bool counting = false;
    cudaGraphExec_t graphs[2][33] = {};   // [counting][steps per launch]
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::vector<void*> allocs;
    size_t bytes = 0;
    State host{};   // mirror after the last synchronisation

    ~DevImpl() override {
        for (auto& row : graphs)
            for (auto& g : row)
                if (g) cudaGraphExecDestroy(g);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (void* p : allocs) cudaFree(p);
        if (d_trace) cudaFree(d_trace);
        if (stream) cudaStreamDestroy(stream);
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
    // slot records
    std::vector<Q4<T>> vtx((size_t)n * 3), nrm(n), ctr(n), frgb(n), acc((size_t)n * 3), db(n);
    for (int i = 0; i < n; i++) {
        const Slot<T>& t = s.slots[i];
        for (int v = 0; v < 3; v++) {
            vtx[i * 3 + v] = {t.p[v][0], t.p[v][1], t.p[v][2], 0};
            acc[i * 3 + v] = {t.accB[v][0], t.accB[v][1], t.accB[v][2], 0};
        }
        const T nl = (T)std::sqrt(t.n[0] * t.n[0] + t.n[1] * t.n[1] + t.n[2] * t.n[2]);
        nrm[i] = {t.n[0], t.n[1], t.n[2], nl};
        ctr[i] = {t.c[0], t.c[1], t.c[2], t.area};
        frgb[i] = {(T)t.Frgb[0], (T)t.Frgb[1], (T)t.Frgb[2], (T)t.parent};
        db[i] = {t.deltaB[0], t.deltaB[1], t.deltaB[2], 0};
    }
    Q4<T> *d_vtx, *d_nrm, *d_ctr, *d_frgb, *d_acc, *d_db;
    int rc;
    if ((rc = d.alloc(&d_vtx, vtx.size())) || (rc = d.alloc(&d_nrm, nrm.size())) || (rc = d.alloc(&d_ctr, ctr.size())) ||
        (rc = d.alloc(&d_frgb, frgb.size())) || (rc = d.alloc(&d_acc, acc.size())) || (rc = d.alloc(&d_db, db.size())))
        return rc;
    CU(cudaMemcpyAsync(d_vtx, vtx.data(), vtx.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_nrm, nrm.data(), nrm.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_ctr, ctr.data(), ctr.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_frgb, frgb.data(), frgb.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_acc, acc.data(), acc.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_db, db.data(), db.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    d.S = Slots<T>{n, d_vtx, d_nrm, d_ctr, d_frgb, d_acc, d_db};

    if (!thresholds_consistent(o)) return fail(RAD_ERR_ARG, "octree cell thresholds do not match its dimensions");
    // visibility structure; the walk's triangle records come from the current slots
    const int n_leaves = (int)(o.leaf_range.size() / 2);
    const size_t n_ent = o.entry_tri.size();
    std::vector<Q4<T>> leaf((size_t)n_leaves * 2), ent(n_ent * 5);
    for (int l = 0; l < n_leaves; l++) {
        const T* b = &o.leaf_box[(size_t)l * 8];
        leaf[2 * l] = {b[0], b[1], b[2], pack_int<T>(o.leaf_range[2 * l])};
        leaf[2 * l + 1] = {b[4], b[5], b[6], pack_int<T>(o.leaf_range[2 * l + 1])};
    }
    for (size_t k = 0; k < n_ent; k++) {
        const int id = o.entry_tri[k];
        const Slot<T>& t = s.slots[id];
        ent[5 * k] = {t.n[0], t.n[1], t.n[2], pack_int<T>(id)};
        ent[5 * k + 1] = {t.c[0], t.c[1], t.c[2], 0};
        for (int e = 0; e < 3; e++) ent[5 * k + 2 + e] = {t.se[e][0], t.se[e][1], t.se[e][2], t.se[e][3]};
    }
    Q4<T> *d_leaf, *d_ent;
    int32_t* d_cell;
    if ((rc = d.alloc(&d_leaf, leaf.size())) || (rc = d.alloc(&d_ent, ent.size())) ||
        (rc = d.alloc(&d_cell, o.cell_leaf.size())))
        return rc;
    CU(cudaMemcpyAsync(d_leaf, leaf.data(), leaf.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_ent, ent.data(), ent.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemcpyAsync(d_cell, o.cell_leaf.data(), o.cell_leaf.size() * 4, cudaMemcpyHostToDevice, d.stream));
    T* d_thr;
    if ((rc = d.alloc(&d_thr, o.thr.size()))) return rc;
    CU(cudaMemcpyAsync(d_thr, o.thr.data(), o.thr.size() * sizeof(T), cudaMemcpyHostToDevice, d.stream));
    Grid<T> G{};
    for (int k = 0; k < 3; k++) {
        G.g0[k] = o.G0[k]; G.g1[k] = o.G1[k]; G.dims[k] = o.dims[k]; G.thr_off[k] = o.thr_off[k];
    }
    G.inv_grid = (T)(1.0 / (double)o.min_grid);
    G.t_eps = o.t_eps;
    G.v_eps = o.v_eps;
    G.n_thr = (int)o.thr.size();
    G.thr = d_thr;
    G.cell_leaf = d_cell;
    G.leaf = d_leaf;
    G.entry = d_ent;
    G.walk_cap = opt.walk_cap > 0 ? opt.walk_cap : (1 << 20);
    d.G = G;

    // per-step state; k_shoot is persistent: as many CTAs as fit at once
    d.n_thr = (int)o.thr.size();
    if (d.shoot_smem() > 48 * 1024) {
        CU(cudaFuncSetAttribute(k_shoot<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.shoot_smem()));
        CU(cudaFuncSetAttribute(k_shoot<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.shoot_smem()));
    }
    {
        int sms = 0, per_sm = 0;
        CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shoot<T, false>, kShootThreads, d.shoot_smem()));
        const int n_groups = (n + kSlotsPerWarp - 1) / kSlotsPerWarp;
        const int want = (n_groups + kShootThreads / 32 - 1) / (kShootThreads / 32);
        d.n_cta = std::max(1, std::min(want, std::max(1, sms * per_sm)));
    }
    if ((rc = d.alloc(&d.d_shooters, (size_t)d.P)) || (rc = d.alloc(&d.d_state, 1)) ||
        (rc = d.alloc(&d.d_part, (size_t)d.n_cta)))
        return rc;
    d.trace_cap = 1 << 16;
    CU(cudaMalloc(&d.d_trace, (size_t)d.trace_cap * 4));
    State st{};
    st.step_limit = 0;
    st.trace = d.d_trace;
    st.trace_cap = d.trace_cap;
    CU(cudaMemcpyAsync(d.d_state, &st, sizeof st, cudaMemcpyHostToDevice, d.stream));
    CU(cudaMemsetAsync(d.d_shooters, 0, sizeof(Shooter<T>) * d.P, d.stream));
    CU(cudaMemsetAsync(d.d_part, 0, sizeof(Partial) * d.n_cta, d.stream));
    // initial selection keys: a step with no shooter only reduces the keys
    k_shoot<T, false><<<d.n_cta, kShootThreads, d.shoot_smem(), d.stream>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(d.stream));
    d.host = st;
    return RAD_OK;
}

template <typename T>
int launch_step(DevImpl<T>& d, cudaStream_t s) {
    k_setup<T><<<1, kSetupThreads, 0, s>>>(d.S, d.d_shooters, d.d_state, d.d_part, d.n_cta, d.conv, d.P);
    if (d.counting)
        k_shoot<T, true><<<d.n_cta, kShootThreads, d.shoot_smem(), s>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
    else
        k_shoot<T, false><<<d.n_cta, kShootThreads, d.shoot_smem(), s>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
    CU(cudaGetLastError());
    return RAD_OK;
}

template <typename T>
int graph_for(DevImpl<T>& d, int steps, cudaGraphExec_t* out) {
    cudaGraphExec_t& slot = d.graphs[d.counting ? 1 : 0][steps];
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
    cudaFree(d.d_trace);
    d.d_trace = nt;
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
            k_setup<T><<<1, kSetupThreads, 0, d.stream>>>(d.S, d.d_shooters, d.d_state, d.d_part, d.n_cta, d.conv, d.P);
            CU(cudaEventRecord(d.ev[1], d.stream));
            if (d.counting)
                k_shoot<T, true><<<d.n_cta, kShootThreads, d.shoot_smem(), d.stream>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
            else
                k_shoot<T, false><<<d.n_cta, kShootThreads, d.shoot_smem(), d.stream>>>(d.S, d.G, d.d_shooters, d.d_state, d.d_part, d.conv);
            CU(cudaGetLastError());
            CU(cudaEventRecord(d.ev[2], d.stream));
        } else {
            cudaGraphExec_t g;
            if ((rc = graph_for(d, chunk, &g))) return rc;
            if (mode) CU(cudaEventRecord(d.ev[0], d.stream));
            CU(cudaGraphLaunch(g, d.stream));
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
    std::vector<Q4<T>> acc((size_t)n * 3), db(n);
    CU(cudaSetDevice(d.device));
    CU(cudaMemcpyAsync(acc.data(), d.S.accB, acc.size() * sizeof(Q4<T>), cudaMemcpyDeviceToHost, d.stream));
    CU(cudaMemcpyAsync(db.data(), d.S.deltaB, db.size() * sizeof(Q4<T>), cudaMemcpyDeviceToHost, d.stream));
    CU(cudaStreamSynchronize(d.stream));
    for (int i = 0; i < n; i++) {
        Slot<T>& t = s.slots[i];
        for (int v = 0; v < 3; v++) {
            t.accB[v][0] = acc[i * 3 + v].x; t.accB[v][1] = acc[i * 3 + v].y; t.accB[v][2] = acc[i * 3 + v].z;
        }
        t.deltaB[0] = db[i].x; t.deltaB[1] = db[i].y; t.deltaB[2] = db[i].z;
    }
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
    CU(cudaSetDevice(d.device));
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
        st->converged = d.host.done;
        st->n_slots = d.S.n;
        st->device_bytes = (int64_t)(d.bytes + d.trace_cap * 4);
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
