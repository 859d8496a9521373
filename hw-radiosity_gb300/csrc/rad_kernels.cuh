// Device-side building blocks shared by the single-scene and batched solvers
// (walk, form factors, deposit, selection keys, shooter records).
// See rad_dev.cu for how one shooter step is put together.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "rad_host.h"

namespace radgb {
namespace dev {

constexpr int kShootThreads = 256;
constexpr int kSlotsPerWarp = 10;
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
__host__ __device__ __forceinline__ int real_to_int(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_int(f);
#else
    int v; std::memcpy(&v, &f, 4); return v;
#endif
}
__host__ __device__ __forceinline__ int real_to_int(double d) {
#ifdef __CUDA_ARCH__
    return (int)__double_as_longlong(d);
#else
    long long v; std::memcpy(&v, &d, 8); return (int)v;
#endif
}
// read-only load: the non-coherent path on the device, a plain load on the host
template <typename U>
__host__ __device__ __forceinline__ U ro_load(const U* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}
__host__ __device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
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

// ------------------------------------------------------------------ FP64-free forms
// The reference promotes two hot expressions to double: the walk's overshoot
// (float)((double)t + 0.1) and CalFF's scale (float)((double)ff * ((double)a /
// ((double)d2 * PI))).  FP64 is slow on this GPU (a float->double add->float
// chain measured 191 cycles, a double multiply+divide 642), so both have FP32
// forms that are exact where they answer and fall back to the double
// expression near a float rounding boundary.  Exhaustive and random checks
// against the double expressions are in tests/test_host.py.
__host__ __device__ __forceinline__ unsigned f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

// (float)((double)x + 0.1).  With c = 0.1 (double), s = x + 0.1f rounded and
// e its exact error (TwoSum), the exact sum is s + T, T = e + (c - 0.1f).  For
// s >= 1/16, T lies within one float step of s (|c - 0.1f| = 1.49e-9 is below
// half the spacing under s), so the answer is s or a neighbour, chosen by
// comparing T with the half-spacings above and below s.  Rounding c + x to
// double first moves the sum by at most 2^-30 of the spacing; T is known to
// 2^-24 of it; answers within 2^-18 of a spacing of a midpoint are left to the
// double expression.
__host__ __device__ __forceinline__ float add_tenth(float x) {
    const float c_hi = 0x1.99999ap-4f;          // 0.1f
    const float c_lo = -0x1.99999ap-30f;        // 0.1 - 0.1f, rounded to float
    const float s = x + c_hi;
    const float bv = s - x;
    const float av = s - bv;
    const float e = (x - av) + (c_hi - bv);     // s + e == x + 0.1f exactly
    if (s >= 0.0625f && s < 0x1p100f) {
        const float t = e + c_lo;
        const unsigned bits = f2u(s);
        const float up = u2f((bits & 0x7f800000u) - (23u << 23));   // spacing above s
        const float dn = (bits & 0x007fffffu) ? up : up * 0.5f;     // spacing below s
        const float h_up = up * 0.5f, h_dn = dn * 0.5f, m = up * 0x1p-18f;
        if (fabsf(t - h_up) > m && fabsf(t + h_dn) > m) {
            if (t > h_up) return u2f(bits + 1);
            if (t < -h_dn) return u2f(bits - 1);
            return s;
        }
    }
    return (float)((double)x + 0.1);
}

// (float)((double)f * ((double)a / ((double)d2 * pi))), pi the double constant:
// f*a / (d2*pi) in float-float arithmetic (product errors by fma, pi as a
// float pair, one correction of the quotient), relative error below 2^-42.
// The double expression differs from the exact value by at most 3 * 2^-53, so
// when the float-float value is more than 2^-14 of a float spacing from every
// rounding midpoint both round to the same float.
__host__ __device__ __forceinline__ float ff_scale(float f, float a, float d2) {
    const float pi_hi = 0x1.921fb6p+1f, pi_lo = -0x1.777a5cp-24f;
    const float den_hi = d2 * pi_hi;
    const float den_lo = fmaf(d2, pi_hi, -den_hi) + d2 * pi_lo;
    const float num_hi = f * a;
    const float num_lo = fmaf(f, a, -num_hi);
    const float q1 = num_hi / den_hi;
    if (num_hi >= 0x1p-90f && num_hi <= 0x1p90f && den_hi >= 0x1p-90f && den_hi <= 0x1p90f && q1 >= 0x1p-90f &&
        q1 <= 0x1p90f) {
        const float r = (fmaf(-q1, den_hi, num_hi) + num_lo) - q1 * den_lo;
        const float q2 = r / den_hi;
        const float y = q1 + q2;
        const float bv = y - q1;
        const float z = (q1 - (y - bv)) + (q2 - bv);   // y + z == q1 + q2 exactly
        const unsigned bits = f2u(y);
        const float up = u2f((bits & 0x7f800000u) - (23u << 23));
        const float dn = (bits & 0x007fffffu) ? up : up * 0.5f;
        const float m = up * 0x1p-14f;
        if (z < up * 0.5f - m && z > -dn * 0.5f + m) return y;
    }
    return (float)((double)f * ((double)a / ((double)d2 * kPiD)));
}

// One cell of the dense cell table: the leaf holding it (TreeNodeNum), that
// leaf's triangle-list range and box, so one 48-byte read (FP32) gives the
// walk everything it needs for the cell.
template <typename T>
struct CellRec {
    int4 h;        // (leaf, list begin, list end, 0)
    Q4<T> a, b;    // (lo.x, lo.y, lo.z, hi.x) (hi.y, hi.z, 0, 0)
};

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
    const CellRec<T>* __restrict__ cell;     // cell coordinate triple -> leaf, list range, leaf box
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
    int work;               // next work item of the current step (k_shoot queue)
    int ctas_done;          // CTAs of the current k_shoot that have finished (fused selection)
    int done;               // a selection found no candidate
    int paused;             // step limit reached
    int nsh;                // shooters of the current step
    int err;
    long long steps;
    long long step_limit;
    long long trace_cap;
    int* trace;
    unsigned long long rays, rays_ref, cells, tris, se, prec, capped, loops;
    // Groups whose item took longer than heavy_ns (split items:
    // heavy_ns_split) in step s are listed in heavy[(s+1)&1] and stamped
    // s+1; step s+1 hands each out first, as items of a few slots whose
    // corners are cast by several lanes each.  A group is split when it is
    // long against both the whole step and the typical group: the limit is
    // the larger of a fraction of the previous step's duration (t_start: its
    // first CTA, by %globaltimer) and a multiple of its mean group time
    // (item_ns / items over the groups shot whole).  Only the schedule
    // depends on it, not the results.
    int* heavy;             // 2 x n_groups
    int* stamp;             // per group: the last step it was split in (-1: never)
    int heavy_n[2];
    int heavy_on;           // one shooter per step (the fused kernel)
    long long heavy_ns, heavy_ns_split;
    unsigned long long t_start, item_ns;
    unsigned long long best;  // FP32, one shooter: (ordered key << 32) | slot, the step's maximum
    unsigned items;
    // Groups that took longer than early_ns without being split are stamped
    // (estamp) and listed in early[(s+1)&1]; step s+1 hands them out right
    // after the split items, the rest follow in slot order.
    int* early;             // 2 x n_groups
    int* estamp;            // per group: the last step it was listed early in (-1: never)
    int early_n[2];
    long long early_ns;
    // the schedule's limits (rad_dev_set_schedule): split above
    // max(frac * step, mean_mult * mean), keep split above frac_split * step,
    // start early above early_mult * mean
    double frac, frac_split, mean_mult, early_mult;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct Cnt { unsigned rays, rays_ref, cells, tris, se, prec, capped, loops; };

// Cell coordinate along one axis: a first guess in T, corrected against the
// thresholds so the result equals the reference's FP64 expression exactly.
template <typename T>
__host__ __device__ __forceinline__ int cell_axis(T q, T g0, T inv, const T* th, int D) {
    int k = (int)((q - g0) * inv);
    k = imin(imax(k, 0), D - 1);
    while (k + 1 < D && q >= th[k + 1]) ++k;
    while (k > 0 && q < th[k]) --k;
    return k;
}

// ------------------------------------------------------------------ walk
template <typename T>
struct Cell {
    int leaf, b, e;    // leaf, list [b, e)
    Q4<T> lo, hi;      // leaf box
};

// TreeNodeNum (raycast.cpp:254-281) as a table lookup: the cell holding q;
// the cell coordinate (int)(((double)q - G0) / MinGridLen) per axis is found
// exactly from the thresholds.  The record's three parts load together.
template <typename T>
__host__ __device__ __forceinline__ Cell<T> cell_at(const Grid<T>& G, T q0, T q1, T q2) {
    const int gx = cell_axis(q0, G.g0[0], G.inv_grid, G.thr + G.thr_off[0], G.dims[0]);
    const int gy = cell_axis(q1, G.g0[1], G.inv_grid, G.thr + G.thr_off[1], G.dims[1]);
    const int gz = cell_axis(q2, G.g0[2], G.inv_grid, G.thr + G.thr_off[2], G.dims[2]);
    const CellRec<T>* r = &G.cell[(gx * G.dims[1] + gy) * G.dims[2] + gz];
    const int4 h = ro_load(&r->h);
    const Q4<T> a = r->a, b = r->b;
    Cell<T> out;
    out.leaf = h.x;
    out.b = h.y;
    out.e = h.z;
    out.lo = {a.x, a.y, a.z, 0};
    out.hi = {a.w, b.x, b.y, 0};
    return out;
}

// NextPoint (raycast.cpp:235-251): leave the leaf box [lo, hi] measured from
// the ray origin, overshoot by 0.1 in t; returns the new t.
template <typename T>
__host__ __device__ __forceinline__ T next_t(const Grid<T>& G, const T p[3], const T v[3], const Q4<T>& lo,
                                             const Q4<T>& hi) {
    const T bl[3] = {lo.x, lo.y, lo.z}, bh[3] = {hi.x, hi.y, hi.z};
    T tm = (T)1000000.0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (fabs(v[a]) > G.v_eps) {             // fabs((double)v) > 1e-6
            const T s = (v[a] > 0) ? (bh[a] - p[a]) / v[a] : (bl[a] - p[a]) / v[a];
            tm = (s < tm) ? s : tm;
        }
    }
    if constexpr (std::is_same<T, float>::value)
        return add_tenth(tm);
    else
        return tm + 0.1;
}

// TriListHitted/TriHitted (raycast.cpp:283-333) over entries [b, e) of one
// leaf's list: the nearest hit of the list (first one on ties), or -1.
template <typename T, bool COUNT>
__host__ __device__ __forceinline__ int scan_list(const Grid<T>& G, const T p[3], const T v[3], int ban, int b, int e,
                                                  Cnt& c) {
    T tmin = (T)1000000.0;
    int best = -1;
    // the next entry's (n, id) and (c) records are in flight while this one is tested
    Q4<T> nx_en = {0, 0, 0, 0}, nx_ec = {0, 0, 0, 0};
    if (b < e) { nx_en = G.entry[5 * b]; nx_ec = G.entry[5 * b + 1]; }
    for (int k = b; k < e; ++k) {
        const Q4<T> en = nx_en, ec = nx_ec;
        if (k + 1 < e) { nx_en = G.entry[5 * (k + 1)]; nx_ec = G.entry[5 * (k + 1) + 1]; }
        const int id = real_to_int(en.w);
        if (id == ban) continue;
        if (COUNT) c.tris++;
        const T a1 = v[0] * en.x + v[1] * en.y + v[2] * en.z;
        const T w0 = ec.x - p[0], w1 = ec.y - p[1], w2 = ec.z - p[2];
        const T a2 = w0 * en.x + w1 * en.y + w2 * en.z;
        // a2/a1 is negative or zero when the signs differ or a2 is zero
        // (a1 nonzero): the test below rejects it, so skip the division
        if ((a1 > 0 && a2 <= 0) || (a1 < 0 && a2 >= 0)) continue;
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
    return best;
}

// RayHitted (raycast.cpp:335-360) with TreeNodeNum (254-281) as a table
// lookup, TriListHitted/TriHitted (283-333) and NextPoint (235-251).
//
// The walk's whole state at the top of an iteration is (t, prev): q is
// p + t*v, and everything after depends on q and prev only.  When that state
// repeats, the reference loops forever (it only notices one cell repeated on
// consecutive steps).  This happens when TreeNodeNum returns a leaf that does
// not contain q (GridNum = (int)((G1-G0)/MinGridLen) can truncate to 63 where
// the tree is 64 cells deep, and the bit descent then picks wrong octants):
// the exits measured from the origin can send the walk round a cycle of
// cells, or a "Precision Exceeded" re-step at huge t leaves t unchanged.
// Brent's cycle detection (one saved state, compared every step, replaced at
// powers of two) finds any repeated state; the walk then stops, is counted
// in `loops`, and the ray is treated as blocked (-3).  The state is saved at
// iterations 0, 2, 6, 14, ... (it + 2 a power of two).  A walk the reference
// finishes never repeats a state, so its result is untouched.
// BRENT_IT selects how that schedule is kept, with the same saves and
// results: read off the loop counter, or held in two counters (the power and
// the steps since the last save).  Which one compiles faster depends on the kernel the walk is
// inlined into (measured): the batched kernel takes the loop-counter form
// (120.8k against 119.4k shots/s on the 256-room batch), the single-scene
// kernels the counters (the 422k-slot hall: 1,075 against 987 shots/s).
template <typename T, bool COUNT, bool BRENT_IT = false>
__host__ __device__ __forceinline__ int walk(const Grid<T>& G, const T p[3], const T v[3], int ban, Cnt& c) {
    T t = 0;
    int prev = -1;
    T q0 = p[0], q1 = p[1], q2 = p[2];
    T chk_t = (T)-1;                   // Brent: saved state, power, steps since saved
    int chk_prev = -2, power = 1, lam = 0;
    for (int it = 0; it < G.walk_cap; ++it) {
        if (q0 < G.g0[0] || q0 > G.g1[0] || q1 < G.g0[1] || q1 > G.g1[1] || q2 < G.g0[2] || q2 > G.g1[2])
            return -1;
        if (t == chk_t && prev == chk_prev) {
            c.loops++;
            return -3;
        }
        if constexpr (BRENT_IT) {
            if (((it + 2) & (it + 1)) == 0) { chk_t = t; chk_prev = prev; }
        } else {
            if (++lam == power) { chk_t = t; chk_prev = prev; power <<= 1; lam = 0; }
        }
        if (COUNT) c.cells++;
        const Cell<T> cr = cell_at(G, q0, q1, q2);
        const int leaf = cr.leaf;
        if (leaf == prev) {          // "Precision Exceeded": step one unit of t
            if (COUNT) c.prec++;
            t = (T)((double)t + 1.0);
            q0 = p[0] + t * v[0]; q1 = p[1] + t * v[1]; q2 = p[2] + t * v[2];
            continue;
        }
        const int best = scan_list<T, COUNT>(G, p, v, ban, cr.b, cr.e, c);
        if (best >= 0) return best;
        prev = leaf;
        t = next_t(G, p, v, cr.lo, cr.hi);
        q0 = p[0] + t * v[0]; q1 = p[1] + t * v[1]; q2 = p[2] + t * v[2];
    }
    c.capped++;
    return -2;
}

#ifdef __CUDACC__
// The same walk cast by a group of L lanes (L a power of two, the group's
// lanes in `gmask`, this lane's index in it `sub`).  All L lanes step through
// the cells together; lane `sub` scans entries b+sub, b+sub+L, ... of each
// list with the serial scan's running minimum, and the group then takes the
// smallest (tt, entry index).  The serial scan keeps the first entry with the
// smallest valid tt, so without a NaN the results are equal.  A 0/0 plane
// test (ray in the triangle's plane) makes tt NaN, which the serial scan
// folds in its own way: a list that produces one is scanned serially.
// Ray and cycle counters are kept by lane 0 of the group only.
template <typename T, int L>
__device__ __forceinline__ int walk_lanes(const Grid<T>& G, const T p[3], const T v[3], int ban, int sub,
                                          unsigned gmask, Cnt& c) {
    T t = 0;
    int prev = -1;
    T q0 = p[0], q1 = p[1], q2 = p[2];
    T chk_t = (T)-1;
    int chk_prev = -2, power = 1, lam = 0;
    for (int it = 0; it < G.walk_cap; ++it) {
        if (q0 < G.g0[0] || q0 > G.g1[0] || q1 < G.g0[1] || q1 > G.g1[1] || q2 < G.g0[2] || q2 > G.g1[2])
            return -1;
        if (t == chk_t && prev == chk_prev) {
            if (sub == 0) c.loops++;
            return -3;
        }
        if (++lam == power) { chk_t = t; chk_prev = prev; power <<= 1; lam = 0; }
        const Cell<T> cr = cell_at(G, q0, q1, q2);
        const int leaf = cr.leaf;
        if (leaf == prev) {          // "Precision Exceeded": step one unit of t
            t = (T)((double)t + 1.0);
            q0 = p[0] + t * v[0]; q1 = p[1] + t * v[1]; q2 = p[2] + t * v[2];
            continue;
        }
        const int b = cr.b, e = cr.e;
        if (b == e) {                // empty list: no hit, every lane knows
            prev = leaf;
            t = next_t(G, p, v, cr.lo, cr.hi);
            q0 = p[0] + t * v[0]; q1 = p[1] + t * v[1]; q2 = p[2] + t * v[2];
            continue;
        }
        T tmin = (T)1000000.0;
        int bk = -1;
        bool nan = false;
        Q4<T> nx_en = {0, 0, 0, 0}, nx_ec = {0, 0, 0, 0};
        if (b + sub < e) { nx_en = G.entry[5 * (b + sub)]; nx_ec = G.entry[5 * (b + sub) + 1]; }
        for (int k = b + sub; k < e; k += L) {
            const Q4<T> en = nx_en, ec = nx_ec;
            if (k + L < e) { nx_en = G.entry[5 * (k + L)]; nx_ec = G.entry[5 * (k + L) + 1]; }
            if (real_to_int(en.w) == ban) continue;
            const T a1 = v[0] * en.x + v[1] * en.y + v[2] * en.z;
            const T w0 = ec.x - p[0], w1 = ec.y - p[1], w2 = ec.z - p[2];
            const T a2 = w0 * en.x + w1 * en.y + w2 * en.z;
            if ((a1 > 0 && a2 <= 0) || (a1 < 0 && a2 >= 0)) continue;
            const T tt = a2 / a1;
            if (tt != tt) { nan = true; continue; }
            if (tt < G.t_eps) continue;
            if (tt >= tmin) continue;
            const T x = p[0] + tt * v[0], y = p[1] + tt * v[1], z = p[2] + tt * v[2];
            const Q4<T> s0 = G.entry[5 * k + 2];
            if ((x * s0.x + y * s0.y + z * s0.z + s0.w) < 0.0) continue;
            const Q4<T> s1 = G.entry[5 * k + 3];
            if ((x * s1.x + y * s1.y + z * s1.z + s1.w) < 0.0) continue;
            const Q4<T> s2 = G.entry[5 * k + 4];
            if ((x * s2.x + y * s2.y + z * s2.z + s2.w) < 0.0) continue;
            tmin = tt;
            bk = k;
        }
#pragma unroll
        for (int d = 1; d < L; d <<= 1) {
            const T ot = __shfl_xor_sync(gmask, tmin, d);
            const int ok = __shfl_xor_sync(gmask, bk, d);
            if (ok >= 0 && (bk < 0 || ot < tmin || (ot == tmin && ok < bk))) { tmin = ot; bk = ok; }
        }
        int hit = -1;
        if (__any_sync(gmask, nan))
            hit = scan_list<T, false>(G, p, v, ban, b, e, c);
        else if (bk >= 0)
            hit = real_to_int(G.entry[5 * bk].w);
        if (hit >= 0) return hit;
        prev = leaf;
        t = next_t(G, p, v, cr.lo, cr.hi);
        q0 = p[0] + t * v[0]; q1 = p[1] + t * v[1]; q2 = p[2] + t * v[2];
    }
    if (sub == 0) c.capped++;
    return -2;
}
#endif


template <typename T> __host__ __device__ __forceinline__ T rsqrt_exact(T x);
template <> __host__ __device__ __forceinline__ float rsqrt_exact<float>(float x) { return sqrtf(x); }
template <> __host__ __device__ __forceinline__ double rsqrt_exact<double>(double x) { return sqrt(x); }

// CalFF's unoccluded part, shade.cpp:107-124: false when the pre-test
// rejects the pair (ff 0, no ray); else ff and the ray direction d.
template <typename T>
__host__ __device__ __forceinline__ bool point_pre(const Shooter<T>& s, const Patch<T>& src, const T p[3], const T nd[3],
                                                   T ndlen, T d[3], T& ff) {
    d[0] = src.c[0] - p[0]; d[1] = src.c[1] - p[1]; d[2] = src.c[2] - p[2];
    const T ds = d[0] * s.n[0] + d[1] * s.n[1] + d[2] * s.n[2];
    const T dd = -(d[0] * nd[0] + d[1] * nd[1] + d[2] * nd[2]);
    if ((ds < 0) != (dd < 0)) return false;
    const T d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const T dl = rsqrt_exact<T>(d2);
    const T c1 = ds / dl / s.nlen;
    const T c2 = dd / dl / ndlen;
    ff = c1 * c2;
    if (ff <= 0.0) return false;
    if constexpr (std::is_same<T, float>::value)
        ff = ff_scale(ff, src.area, d2);
    else
        ff = (T)((double)ff * ((double)src.area / ((double)d2 * kPiD)));
    if (ff <= 0.0) return false;
    return true;
}

// CalFF, shade.cpp:107-127: the pre-test is cheap, the walk is not
template <typename T, bool COUNT, bool WALK, bool BRENT_IT = false>
__host__ __device__ __forceinline__ T point_ff(const Shooter<T>& s, const Patch<T>& src, const T p[3], const T nd[3], T ndlen,
                                      int logdes, const Grid<T>& G, Cnt& c) {
    T d[3], ff = 0;
    if (!point_pre(s, src, p, nd, ndlen, d, ff)) return 0;
    if (!WALK) return ff;   // pre-test only (reference ray accounting)
    c.rays++;
    return walk<T, COUNT, BRENT_IT>(G, p, d, logdes, c) == s.logsrc ? ff : (T)0;
}


// Shade's per-corner AdaptCalFF(CalFF(...)), shade.cpp:442-450 with the
// stray ';' at shade.cpp:164: a split source returns ff(half1)+ff(half2); the
// whole-source result is discarded, so its walk is not cast.
template <typename T, bool COUNT, bool BRENT_IT = false>
__host__ __device__ __forceinline__ T corner_ff(const Shooter<T>& s, const T p[3], const T nd[3], T ndlen, int logdes,
                                       const Grid<T>& G, Cnt& c) {
    const unsigned before = c.rays;
    if (!s.split) {
        const T f = point_ff<T, COUNT, true, BRENT_IT>(s, s.part[0], p, nd, ndlen, logdes, G, c);
        if (COUNT) c.rays_ref += c.rays - before;
        return f;
    }
    if (COUNT && point_ff<T, COUNT, false>(s, s.part[0], p, nd, ndlen, logdes, G, c) > (T)0) c.rays_ref++;
    const T f1 = point_ff<T, COUNT, true, BRENT_IT>(s, s.part[1], p, nd, ndlen, logdes, G, c);
    const T f2 = point_ff<T, COUNT, true, BRENT_IT>(s, s.part[2], p, nd, ndlen, logdes, G, c);
    if (COUNT) c.rays_ref += c.rays - before;
    return f1 + f2;
}

#ifdef __CUDACC__
// point_ff / corner_ff (no counting) for a group of L lanes sharing one corner
template <typename T, int L>
__device__ __forceinline__ T point_ff_lanes(const Shooter<T>& s, const Patch<T>& src, const T p[3], const T nd[3],
                                            T ndlen, int logdes, int sub, unsigned gmask, const Grid<T>& G, Cnt& c) {
    T d[3], ff = 0;
    if (!point_pre(s, src, p, nd, ndlen, d, ff)) return 0;
    if (sub == 0) c.rays++;
    return walk_lanes<T, L>(G, p, d, logdes, sub, gmask, c) == s.logsrc ? ff : (T)0;
}

template <typename T, int L>
__device__ __forceinline__ T corner_ff_lanes(const Shooter<T>& s, const T p[3], const T nd[3], T ndlen, int logdes,
                                             int sub, unsigned gmask, const Grid<T>& G, Cnt& c) {
    if (!s.split) return point_ff_lanes<T, L>(s, s.part[0], p, nd, ndlen, logdes, sub, gmask, G, c);
    const T f1 = point_ff_lanes<T, L>(s, s.part[1], p, nd, ndlen, logdes, sub, gmask, G, c);
    const T f2 = point_ff_lanes<T, L>(s, s.part[2], p, nd, ndlen, logdes, sub, gmask, G, c);
    return f1 + f2;
}
#endif

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
    unsigned v[8] = {c.rays, c.rays_ref, c.cells, c.tris, c.se, c.prec, c.capped, c.loops};
    unsigned long long* dst[8] = {&st->rays, &st->rays_ref, &st->cells, &st->tris, &st->se, &st->prec, &st->capped,
                                  &st->loops};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        if (!COUNT && q != 0 && q != 6 && q != 7) continue;
        unsigned s = __reduce_add_sync(kFull, v[q]);
        if (lane == 0 && s) atomicAdd(dst[q], (unsigned long long)s);
    }
}

// ------------------------------------------------------------------ k_shoot
// One work item: n_item consecutive slots from slot i0, each corner's ray cast
// by a group of L lanes.  Lane = L*(3r+v) + sub: corner v of slot i0+r, lane
// `sub` of its group.  L = 1 is the common layout (10 slots, one lane per
// corner); L = 4 serves two slots of a group whose walks were long in the
// previous step.
// The deposit is the same for every layout: the three corners' form factors
// meet by shuffle, the group's lane 0 writes its corner's accB, and corner 0's
// lane 0 keeps the slot's deltaB in the reference's order.
template <typename T, bool COUNT, int L, bool ONE = false, bool BRENT_IT = false>
__device__ __forceinline__ void shoot_item(const Slots<T>& S, const Grid<T>& G, const Shooter<T>* sh, int nsh, int i0,
                                           int n_item, int lane, T conv, unsigned long long& kk, int& ks, Cnt& c) {
    static_assert(L == 1 || !COUNT, "the counting pass uses the serial walk");
    const int ray = lane / L, sub = lane - L * ray;
    const int r = ray / 3, v = ray - 3 * r;
    const int i = i0 + r;
    const bool own = ray < 3 * n_item && i < S.n;
    const unsigned gmask = L == 1 ? 1u << lane : (L == 32 ? kFull : ((1u << L) - 1u) << (lane & ~(L - 1)));
    const bool lead = sub == 0;

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
    const int base = 3 * L * min(r, n_item - 1);   // lane 0 of corner 0 of slot r
    const bool open = (((ballot >> base) | (ballot >> (base + L)) | (ballot >> (base + 2 * L))) & 1u) != 0;
    const bool active = live && !is_src && open && nsh > 0;
    if (ONE) {
        // one shooter: the deposit's inputs are read again after the walk
        // (the warp owns the slot, so they are unchanged) instead of being
        // held in registers across it
        T ff = 0;
        if (active) {
            const Q4<T> pp = S.vtx[i * 3 + v];
            const Q4<T> nn = S.nrm[i];
            const T pv[3] = {pp.x, pp.y, pp.z}, nd[3] = {nn.x, nn.y, nn.z};
            if constexpr (L == 1)
                ff = corner_ff<T, COUNT, BRENT_IT>(sh[0], pv, nd, nn.w, parent, G, c);
            else
                ff = corner_ff_lanes<T, L>(sh[0], pv, nd, nn.w, parent, sub, gmask, G, c);
        }
        const T f0 = shfl(ff, base), f1 = shfl(ff, base + L), f2 = shfl(ff, base + 2 * L);
        T d0 = 0, d1 = 0, d2 = 0;
        if (live && v == 0) { db = S.deltaB[i]; d0 = db.x; d1 = db.y; d2 = db.z; }
        if (active) {
            fr = S.frgb[i];
            acc = S.accB[i * 3 + v];
            const T k = (T)(0.5 / 255.0);   // RefRatio / 255.0, shade.cpp:246
            const T lo0 = fr.x * k * sh[0].deltaB[0] / 3;
            const T lo1 = fr.y * k * sh[0].deltaB[1] / 3;
            const T lo2 = fr.z * k * sh[0].deltaB[2] / 3;
            T a0 = acc.x, a1 = acc.y, a2 = acc.z;
            a0 += lo0 * ff; a1 += lo1 * ff; a2 += lo2 * ff;
            if (v == 0) {
                d0 += lo0 * f0; d0 += lo0 * f1; d0 += lo0 * f2;
                d1 += lo1 * f0; d1 += lo1 * f1; d1 += lo1 * f2;
                d2 += lo2 * f0; d2 += lo2 * f1; d2 += lo2 * f2;
            }
            if (lead) {
                Q4<T> o = {a0, a1, a2, acc.w};
                S.accB[i * 3 + v] = o;
                if (v == 0) { Q4<T> q = {d0, d1, d2, db.w}; S.deltaB[i] = q; }
            }
        }
        if (live && is_src && v == 0) {       // rad.cpp:446-449
            d0 = d1 = d2 = 0;
            if (lead) { Q4<T> q = {0, 0, 0, db.w}; S.deltaB[i] = q; }
        }
        if (live && v == 0 && lead) {
            const T key = (d0 + d1) + d2;
            if (key > conv) {
                const unsigned long long o = key_order(key);
                if (part_less(kk, ks, o, i)) { kk = o; ks = i; }
            }
        }
        return;
    }
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
        if (active) {
            if constexpr (L == 1)
                ff = corner_ff<T, COUNT, BRENT_IT>(sh[j], pv, nd, ndlen, parent, G, c);
            else
                ff = corner_ff_lanes<T, L>(sh[j], pv, nd, ndlen, parent, sub, gmask, G, c);
        }
        const T f0 = shfl(ff, base), f1 = shfl(ff, base + L), f2 = shfl(ff, base + 2 * L);
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
    if (active && lead) {
        Q4<T> o = {a0, a1, a2, acc.w};
        S.accB[i * 3 + v] = o;
        if (v == 0) { Q4<T> q = {d0, d1, d2, db.w}; S.deltaB[i] = q; }
    }
    if (live && is_src && v == 0) {       // rad.cpp:446-449
        d0 = d1 = d2 = 0;
        if (lead) { Q4<T> q = {0, 0, 0, db.w}; S.deltaB[i] = q; }
    }
    // next selection: key = (dB0 + dB1) + dB2 (rad.cpp:394), candidates > converge
    if (live && v == 0 && lead) {
        const T key = (d0 + d1) + d2;
        if (key > conv) {
            const unsigned long long o = key_order(key);
            if (part_less(kk, ks, o, i)) { kk = o; ks = i; }
        }
    }
}

// One 10-slot group in the common layout (lanes 3r+v: corner v of slot g*10+r).
template <typename T, bool COUNT, bool ONE = false, bool BRENT_IT = false>
__device__ __forceinline__ void shoot_group(const Slots<T>& S, const Grid<T>& G, const Shooter<T>* sh, int nsh,
                                            int g, int lane, T conv, unsigned long long& kk, int& ks, Cnt& c) {
    shoot_item<T, COUNT, 1, ONE, BRENT_IT>(S, G, sh, nsh, g * kSlotsPerWarp, kSlotsPerWarp, lane, conv, kk, ks, c);
}

// Shooter record for slot `slot`: normal, |n|, centre, area, unshot energy,
// and AdaptCalFF's split into two halves (shade.cpp:76-99, 141-156).
template <typename T>
__host__ __device__ inline void make_shooter(const T p[3][3], const T c[3], const T n[3], T nlen, T area,
                                             const T deltaB[3], int slot, int logsrc, Shooter<T>& s) {
    s.slot = slot;
    s.logsrc = logsrc;
    s.pad = 0;
    s.n[0] = n[0]; s.n[1] = n[1]; s.n[2] = n[2];
    s.nlen = nlen;
    s.deltaB[0] = deltaB[0]; s.deltaB[1] = deltaB[1]; s.deltaB[2] = deltaB[2];
    s.pad2 = 0;
    s.part[0].c[0] = c[0]; s.part[0].c[1] = c[1]; s.part[0].c[2] = c[2];
    s.part[0].area = area;
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
        s.part[1].area = s.part[2].area = (T)((double)area / 2.0);
    } else {
        for (int h = 1; h < 3; h++) {
            for (int q = 0; q < 3; q++) s.part[h].c[q] = 0;
            s.part[h].area = 0;
        }
    }
}

template <typename T>
__device__ void build_shooter(const Slots<T>& S, int slot, Shooter<T>& s) {
    const Q4<T> fr = S.frgb[slot], nn = S.nrm[slot], cc = S.ctr[slot], db = S.deltaB[slot];
    T p[3][3];
    for (int v = 0; v < 3; v++) {
        const Q4<T> q = S.vtx[slot * 3 + v];
        p[v][0] = q.x; p[v][1] = q.y; p[v][2] = q.z;
    }
    const T c[3] = {cc.x, cc.y, cc.z}, n[3] = {nn.x, nn.y, nn.z}, d[3] = {db.x, db.y, db.z};
    make_shooter(p, c, n, nn.w, cc.w, d, slot, (int)fr.w, s);
}


// listCanditate (rad.cpp:387-404) over one scene's slots, by one CTA of at
// most 1024 threads: the n = min((|C|+4)/5, P) largest (key, slot) pairs,
// descending (ties: higher slot first), where C is the set of live slots whose
// key (dB0 + dB1) + dB2 exceeds conv.  One block-wide argmax per rank, each
// below the previous rank's pair.  chosen (shared, >= P entries) receives the
// slots; returns n (0: converged).  Every thread gets the same n.
template <typename T>
__device__ int cta_top_shooters(const Slots<T>& S, T conv, int P, int* chosen) {
    __shared__ unsigned long long bk[32];
    __shared__ int bs[32], bc[32];
    __shared__ int nch;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    unsigned long long lim_k = ~0ull;
    int lim_s = 0x7fffffff;
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
            kk = lane < nw ? bk[lane] : 0;
            ks = lane < nw ? bs[lane] : -1;
            const int cc = __reduce_add_sync(kFull, lane < nw ? bc[lane] : 0);
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
        const int n_take = nch;
        __syncthreads();
        if (rank + 1 >= n_take) break;
    }
    return nch;
}

// ------------------------------------------------------------------ upload
// The cell table and the list records are expanded on the device from
// compact host arrays: a leaf index per cell, and per triangle one record
// group gathered for each list entry naming it.
template <typename T>
__global__ void k_expand_cells(const int32_t* __restrict__ cell_leaf, const T* __restrict__ leaf_box,
                               const int32_t* __restrict__ leaf_range, long long n_cell, CellRec<T>* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_cell;
         i += (long long)gridDim.x * blockDim.x) {
        const int l = cell_leaf[i];
        const T* b = leaf_box + (size_t)l * 8;
        CellRec<T> r;
        r.h = make_int4(l, leaf_range[2 * l], leaf_range[2 * l + 1], 0);
        r.a = {b[0], b[1], b[2], b[4]};
        r.b = {b[5], b[6], 0, 0};
        out[i] = r;
    }
}

// entry k = the five records of triangle entry_tri[k]
template <typename T>
__global__ void k_gather_entries(const int32_t* __restrict__ entry_tri, const Q4<T>* __restrict__ tri_rec,
                                 long long n_ent, Q4<T>* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_ent * 5;
         i += (long long)gridDim.x * blockDim.x) {
        const long long k = i / 5;
        const int j = (int)(i - 5 * k);
        out[i] = tri_rec[(size_t)entry_tri[k] * 5 + j];
    }
}

// ------------------------------------------------------------------ host packing
// Device records of one scene, appended to growing host arrays so several
// scenes can share one allocation (the batched solver).  Offsets are in
// records.  The walk's triangle records come from the scene's current slots,
// as RayHitted reads TriStore at shooting time.
template <typename T>
struct HostPack {
    std::vector<Q4<T>> vtx, nrm, ctr, frgb, acc, db, ent;
    std::vector<CellRec<T>> cell;
    std::vector<T> thr;
};

struct PackOffsets {
    size_t slot = 0, ent = 0, cell = 0, thr = 0;
    int n = 0;
};

template <typename T>
inline PackOffsets pack_scene(const Scene<T>& s, const Octree<T>& o, HostPack<T>& P) {
    PackOffsets off;
    off.slot = P.frgb.size();
    off.ent = P.ent.size() / 5;
    off.cell = P.cell.size();
    off.thr = P.thr.size();
    off.n = s.trinum;
    for (int i = 0; i < s.trinum; i++) {
        const Slot<T>& t = s.slots[i];
        for (int v = 0; v < 3; v++) {
            P.vtx.push_back({t.p[v][0], t.p[v][1], t.p[v][2], 0});
            P.acc.push_back({t.accB[v][0], t.accB[v][1], t.accB[v][2], 0});
        }
        const T nl = (T)std::sqrt(t.n[0] * t.n[0] + t.n[1] * t.n[1] + t.n[2] * t.n[2]);
        P.nrm.push_back({t.n[0], t.n[1], t.n[2], nl});
        P.ctr.push_back({t.c[0], t.c[1], t.c[2], t.area});
        P.frgb.push_back({(T)t.Frgb[0], (T)t.Frgb[1], (T)t.Frgb[2], (T)t.parent});
        P.db.push_back({t.deltaB[0], t.deltaB[1], t.deltaB[2], 0});
    }
    for (size_t k = 0; k < o.entry_tri.size(); k++) {
        const int id = o.entry_tri[k];
        const Slot<T>& t = s.slots[id];
        P.ent.push_back({t.n[0], t.n[1], t.n[2], pack_int<T>(id)});
        P.ent.push_back({t.c[0], t.c[1], t.c[2], 0});
        for (int e = 0; e < 3; e++) P.ent.push_back({t.se[e][0], t.se[e][1], t.se[e][2], t.se[e][3]});
    }
    for (int32_t l : o.cell_leaf) {
        const T* b = &o.leaf_box[(size_t)l * 8];
        CellRec<T> r;
        r.h = make_int4(l, o.leaf_range[2 * l], o.leaf_range[2 * l + 1], 0);
        r.a = {b[0], b[1], b[2], b[4]};
        r.b = {b[5], b[6], 0, 0};
        P.cell.push_back(r);
    }
    P.thr.insert(P.thr.end(), o.thr.begin(), o.thr.end());
    return off;
}

// Grid parameters of one scene; the pointers are set by the caller
template <typename T>
inline Grid<T> grid_params(const Octree<T>& o, int walk_cap) {
    Grid<T> G{};
    for (int k = 0; k < 3; k++) {
        G.g0[k] = o.G0[k]; G.g1[k] = o.G1[k]; G.dims[k] = o.dims[k]; G.thr_off[k] = o.thr_off[k];
    }
    G.inv_grid = (T)(1.0 / (double)o.min_grid);
    G.t_eps = o.t_eps;
    G.v_eps = o.v_eps;
    G.n_thr = (int)o.thr.size();
    G.walk_cap = walk_cap > 0 ? walk_cap : (1 << 16);
    return G;
}

}  // namespace dev
}  // namespace radgb
