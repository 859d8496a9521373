// Octree construction geometry, shared by the host build (octree.cpp) and the
// device build (rad_octree_dev.cu): the child boxes of a node and the
// triangle-box overlap test of the reference (src/raycast.cpp:24-155, 168-215).
// Both compilers are held to the same arithmetic: no contraction
// (-ffp-contract=off on the host, -fmad=false on the device), IEEE division.
#pragma once

#ifdef __CUDACC__
#define RAD_HD __host__ __device__ __forceinline__
#else
#define RAD_HD inline
#endif

namespace radgb {
namespace geom {

template <typename T>
RAD_HD void swap_ptr(const T*& a, const T*& b) {
    const T* t = a;
    a = b;
    b = t;
}

// segment p0-p1 against the rectangle [g0,g1] in dims (x, y), raycast.cpp:24-60
template <typename T>
RAD_HD bool segment_meets_rect(const T* p0, const T* p1, const T* g0, const T* g1, int x, int y) {
    const unsigned o0 = (p0[x] < g0[x]) | (p0[x] > g1[x]) << 1 | (p0[y] < g0[y]) << 2 | (p0[y] > g1[y]) << 3;
    const unsigned o1 = (p1[x] < g0[x]) | (p1[x] > g1[x]) << 1 | (p1[y] < g0[y]) << 2 | (p1[y] > g1[y]) << 3;
    if (o0 & o1) return false;
    if (!(o0 | o1)) return true;
    const T a = p1[y] - p0[y], b = p1[x] - p0[x];
    const T c00 = a * (g0[x] - p0[x]) - b * (g0[y] - p0[y]);
    if (c00 == 0) return true;
    const bool neg = c00 < 0;
    // the line misses the rectangle iff all four corners lie strictly on one side
    if ((a * (g0[x] - p0[x]) - b * (g1[y] - p0[y]) < 0) != neg) return true;
    if ((a * (g1[x] - p0[x]) - b * (g0[y] - p0[y]) < 0) != neg) return true;
    if ((a * (g1[x] - p0[x]) - b * (g1[y] - p0[y]) < 0) != neg) return true;
    return false;
}

// point on segment hi-lo where coordinate d equals g, raycast.cpp:91-100
template <typename T>
RAD_HD void at_coord(const T* hi, const T* lo, T g, int d, T* out) {
    const T dd = hi[d] - lo[d];
    if (dd == 0.0) { out[0] = hi[0]; out[1] = hi[1]; out[2] = hi[2]; return; }
    const T wa = (g - lo[d]) / dd, wb = (hi[d] - g) / dd;
    for (int k = 0; k < 3; k++) out[k] = wa * hi[k] + wb * lo[k];
}

// does the triangle (p[0], p[1], p[2]) meet the box [g0,g1]; raycast.cpp:109-155
template <typename T>
RAD_HD bool tri_meets_box(const T* p0, const T* p1, const T* p2, const T* g0, const T* g1) {
    const T *hi = p0, *mid = p1, *lo = p2;
    T a[3], b[3];
    for (int x = 0; x < 3; x++) {
        // order the three vertex pointers by coordinate x (raycast.cpp:66-85)
        if (hi[x] < mid[x]) swap_ptr(hi, mid);
        if (hi[x] < lo[x]) swap_ptr(hi, lo);
        if (mid[x] < lo[x]) swap_ptr(mid, lo);
        const int y = (x + 1) % 3, z = (x + 2) % 3;
        if (g1[x] < lo[x]) return false;
        at_coord(hi, lo, g1[x], x, a);
        if (g1[x] < mid[x]) { at_coord(mid, lo, g1[x], x, b); return segment_meets_rect(a, b, g0, g1, y, z); }
        if (g1[x] <= hi[x]) { at_coord(hi, mid, g1[x], x, b); return segment_meets_rect(a, b, g0, g1, y, z); }
        if (g0[x] > hi[x]) return false;
        at_coord(hi, lo, g0[x], x, a);
        if (g0[x] > mid[x]) { at_coord(hi, mid, g0[x], x, b); return segment_meets_rect(a, b, g0, g1, y, z); }
        if (g0[x] >= lo[x]) { at_coord(mid, lo, g0[x], x, b); return segment_meets_rect(a, b, g0, g1, y, z); }
    }
    return true;
}

// child i of the box [b0,b1]: bit j of i picks the upper half on axis j; the
// midpoint is (T)(0.5*g0 + 0.5*g1) in double (raycast.cpp:172-180)
template <typename T>
RAD_HD void child_box(const T* b0, const T* b1, int i, T* c0, T* c1) {
    for (int j = 0; j < 3; j++) {
        const T mid = (T)(0.5 * (double)b0[j] + 0.5 * (double)b1[j]);
        c0[j] = b0[j];
        c1[j] = b1[j];
        if ((i >> j) & 1) c0[j] = mid; else c1[j] = mid;
    }
}

}  // namespace geom
}  // namespace radgb
