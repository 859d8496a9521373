// Host-side scene store and visibility-structure builder (internal C++ API).
//
// The host owns topology work that is sequential by definition (scene input,
// the greedy pre-partition, neighbour links, output); the device owns the
// shooting loop.  Everything is templated on the solver's scalar type T:
// float reproduces the reference's FP32 build, double its float->double build.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <new>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "rad_gb300.h"

namespace radgb {

constexpr double kPi = 3.1415926535897932;   // include/rad.h:5
constexpr int kMaxLevel = 6;                 // include/rad.h:7
constexpr int kMaxTriPerNode = 10;           // include/rad.h:12
constexpr int kMaxTriPool = 1000000;         // include/rad.h:9 (slot pool hard cap)

// One triangle slot with every field the reference's Triangle carries
// (include/rad.h:25-39).  Slots past the live count keep whatever the last
// occupant left, exactly like the reference's static pool, because the
// pre-partition copies whole slots and reads fields it never initialises.
template <typename T>
struct Slot {
    T p[3][3];
    int32_t Frgb[3];
    int32_t Brgb[3];
    T accB[3][3];
    T daccB[3][3];
    T deltaB[3];
    T se[3][4];
    T c[3];
    T n[3];
    T area;
    int32_t parent;
    int32_t nb[3];
};

// Allocator of the slot pool: memory from calloc, and value-initialisation
// that writes nothing, so a pool sized to the -triangle limit (the
// reference's static TriStore of 10^6 slots, rad.h:9) reads as zeros without
// being written -- the operating system maps zero pages as they are first
// touched.  Only for trivially copyable records in vectors that never shrink
// and grow again in place.
template <typename U>
struct ZeroPages {
    using value_type = U;
    ZeroPages() = default;
    template <typename V> ZeroPages(const ZeroPages<V>&) {}
    U* allocate(std::size_t n) {
        void* p = std::calloc(n ? n : 1, sizeof(U));
        if (!p) throw std::bad_alloc();
        return static_cast<U*>(p);
    }
    void deallocate(U* p, std::size_t) { std::free(p); }
    template <typename V, typename... A>
    void construct(V* p, A&&... a) {
        if constexpr (sizeof...(A) > 0) ::new ((void*)p) V(std::forward<A>(a)...);
    }
    template <typename V> bool operator==(const ZeroPages<V>&) const { return true; }
    template <typename V> bool operator!=(const ZeroPages<V>&) const { return false; }
};

template <typename T>
struct Scene {
    static_assert(std::is_trivially_copyable<Slot<T>>::value, "slots are plain records");
    std::vector<Slot<T>, ZeroPages<Slot<T>>> slots;   // pool, zero-filled; [0, trinum) live
    int32_t trinum = 0;           // live slots
    int32_t n_orig = 0;           // triangles read from the input (the octree indexes these)
    T G0[3] = {0, 0, 0};
    T G1[3] = {0, 0, 0};
    T minarea = 0, maxarea = 0;
    rad_options opt{};
    bool alloc_warned = false;
    std::string log;              // info lines the CLI prints
};

// Flattened visibility structure.  Leaves are numbered in the order they
// are created; only their identity matters to the walk (it compares the leaf
// of consecutive steps), and every leaf list keeps the reference's order.
template <typename T>
struct Octree {
    T G0[3], G1[3];
    T min_grid = 0;               // smallest leaf edge (raycast.cpp:184-185)
    int32_t grid_num = 0;         // raycast.cpp:230
    int32_t dims[3] = {0, 0, 0};  // cell-table extent per axis (max cell coordinate + 1)
    std::vector<int32_t> cell_leaf;     // dims[0]*dims[1]*dims[2] -> leaf id
    // thr[off[a] + k] = the smallest value q with cell_coord(q) >= k on axis a
    // (k = 1..dims[a]-1; entries 0 and dims[a] are unused sentinels).  Cell
    // coordinates are monotone in q, so k = #{thresholds <= q}: the device
    // finds it exactly without the reference's FP64 division.
    std::vector<T> thr;
    int32_t thr_off[3] = {0, 0, 0};
    T t_eps = 0;   // smallest T >= 0.0001: (double)t < 0.0001  <=>  t < t_eps
    T v_eps = 0;   // largest T <= 1e-6:    fabs((double)v) > 1e-6  <=>  fabs(v) > v_eps
    std::vector<T> leaf_box;            // 8 per leaf: g0.xyz, 0, g1.xyz, 0
    std::vector<int32_t> leaf_range;    // 2 per leaf: [begin, end) into entry_tri
    std::vector<int32_t> entry_tri;     // triangle id per list entry
    int64_t ref_nodes = 0;        // node and list-slot counts the reference reports
    int64_t ref_list = 0;
};

// Scene input / output, src/rad.cpp:47-111 and 117-242.
template <typename T> int load_tri_text(const char* text, size_t len, const rad_options& o, Scene<T>& s, std::string& err);
template <typename T> int load_arrays(const float* vtx, const int32_t* frgb, const int32_t* brgb, int32_t n,
                                      const rad_options& o, Scene<T>& s, std::string& err);
// links = false leaves the neighbour links to the caller (the device form)
template <typename T> void init_radiosity(Scene<T>& s, bool links = true);   // src/rad.cpp:259-356
template <typename T> void prepartition(Scene<T>& s);                // src/shade.cpp:556-598
template <typename T> int write_fin(const Scene<T>& s, const char* prefix, int loop, std::string& err);
template <typename T> void build_octree(const Scene<T>& s, Octree<T>& o, int threads);  // raycast.cpp:216-233

// PartitionTriangleAndStore (shade.cpp:311-431) on receiver slot sid: out[]
// gets t1..t4 (-1 where not created), *nbid the neighbour split with it (-1
// for none); returns -1 (no split), 0, or 1 (sid now holds a child).
template <typename T> int split_receiver(Scene<T>& s, int32_t sid, int32_t out[4], bool& reshade, int32_t* nbid);
// isFullPool (shade.cpp:26-30)
template <typename T> bool pool_full(const Scene<T>& s, int need);

// The threshold method the device uses for cell coordinates, on the host
// (tests compare it with cell_coord), and the size check run before upload.
template <typename T> int cell_of_thresholds(const Octree<T>& o, int axis, T q);
template <typename T> bool thresholds_consistent(const Octree<T>& o);

// Cell coordinate along one axis, raycast.cpp:263 (shared with the device).
template <typename T>
inline int cell_coord(T q, T g0, T min_grid) {
    return (int)(((double)q - (double)g0) / (double)min_grid);
}

// Float to text with the semantics of include/float2string.h's
// fp::tostring<float>: returns false (and writes nothing) where it would.
bool format_float(float x, char* buf);

}  // namespace radgb
