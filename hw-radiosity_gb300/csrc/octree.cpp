// Visibility structure: the reference's uniform-subdivision octree
// (src/raycast.cpp:168-233), built on the host and flattened for the device.
//
// What the walk needs from the tree is (1) the leaf containing a point and
// (2) each leaf's box and triangle list.  TreeNodeNum (raycast.cpp:254-281)
// finds the leaf by descending on the bits of the integer cell coordinate
// gnum = (int)((q - G0) / MinGridLen), so the leaf is a function of the three
// cell coordinates alone; we tabulate it once for every coordinate triple
// (at most ~65^3 entries for MaxLevel 6) and the device does one lookup
// instead of up to six dependent node reads.
//
// Subtrees below the root are built concurrently; leaves are renumbered
// afterwards.  Leaf numbering is free (the walk only compares the leaves of
// consecutive steps), and each list keeps the reference's order (ascending
// triangle id, as every list is a filtered copy of 0..n-1).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <future>
#include <thread>

#include "octree_build.h"
#include "octree_geom.h"
#include "rad_host.h"

namespace radgb {
namespace {



// order-preserving unsigned image of a float / double
template <typename T> struct OrderedBits;
template <> struct OrderedBits<float> {
    static uint32_t to(float x) {
        uint32_t b; std::memcpy(&b, &x, 4);
        return (b >> 31) ? ~b : (b | 0x80000000u);
    }
    static float from(uint32_t o) {
        uint32_t b = (o >> 31) ? (o & 0x7fffffffu) : ~o;
        float x; std::memcpy(&x, &b, 4);
        return x;
    }
};
template <> struct OrderedBits<double> {
    static uint64_t to(double x) {
        uint64_t b; std::memcpy(&b, &x, 8);
        return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
    }
    static double from(uint64_t o) {
        uint64_t b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
        double x; std::memcpy(&x, &b, 8);
        return x;
    }
};


template <typename T>
struct Builder {
    const Scene<T>& s;

    void child_box(const Box<T>& b, int i, Box<T>& c) const { geom::child_box(b.g0, b.g1, i, c.g0, c.g1); }
    void filter(const std::vector<int32_t>& in, const Box<T>& c, std::vector<int32_t>& out) const {
        out.clear();
        for (int32_t t : in) {
            const auto& p = s.slots[t].p;
            if (geom::tri_meets_box<T>(p[0], p[1], p[2], c.g0, c.g1)) out.push_back(t);
        }
    }
    bool is_leaf(size_t n, int level) const { return n <= (size_t)kMaxTriPerNode || level >= kMaxLevel; }

    int32_t build(Part<T>& P, const std::vector<int32_t>& idx, int level, const Box<T>& b) const {
        const int32_t id = (int32_t)P.nodes.size();
        P.nodes.push_back(Node());
        if (is_leaf(idx.size(), level)) {
            Node& nd = P.nodes[id];
            for (int i = 0; i < 8; i++) nd.child[i] = -1;
            nd.leaf = (int32_t)P.leaf_box.size();
            P.leaf_box.push_back(b);
            P.leaf_begin.push_back((int32_t)P.entries.size());
            P.entries.insert(P.entries.end(), idx.begin(), idx.end());
            P.n_list += (int64_t)idx.size() + 1;
            const T edge0 = b.g1[0] - b.g0[0];
            if (edge0 < P.min_edge) P.min_edge = edge0;
            return id;
        }
        P.nodes[id].leaf = -1;
        std::vector<int32_t> sub;
        for (int i = 0; i < 8; i++) {
            Box<T> c;
            child_box(b, i, c);
            filter(idx, c, sub);
            const int32_t ch = build(P, sub, level + 1, c);
            P.nodes[id].child[i] = ch;
        }
        return id;
    }
};

// append part Q (a subtree) into P; returns Q's root id in P
template <typename T>
int32_t merge(Part<T>& P, const Part<T>& Q) {
    const int32_t noff = (int32_t)P.nodes.size(), loff = (int32_t)P.leaf_box.size();
    const int32_t eoff = (int32_t)P.entries.size();
    for (Node nd : Q.nodes) {
        for (int i = 0; i < 8; i++) if (nd.child[i] >= 0) nd.child[i] += noff;
        if (nd.leaf >= 0) nd.leaf += loff;
        P.nodes.push_back(nd);
    }
    P.leaf_box.insert(P.leaf_box.end(), Q.leaf_box.begin(), Q.leaf_box.end());
    for (int32_t b : Q.leaf_begin) P.leaf_begin.push_back(b + eoff);
    P.entries.insert(P.entries.end(), Q.entries.begin(), Q.entries.end());
    P.n_list += Q.n_list;
    if (Q.min_edge < P.min_edge) P.min_edge = Q.min_edge;
    return noff;
}

}  // namespace

template <typename T>
void build_octree(const Scene<T>& s, Octree<T>& o, int threads) {
    Builder<T> B{s};
    Box<T> root;
    for (int k = 0; k < 3; k++) { root.g0[k] = s.G0[k]; root.g1[k] = s.G1[k]; o.G0[k] = s.G0[k]; o.G1[k] = s.G1[k]; }
    std::vector<int32_t> all((size_t)s.n_orig);
    for (int32_t i = 0; i < s.n_orig; i++) all[i] = i;

    Part<T> P;
    P.min_edge = s.G1[0] - s.G0[0];                       // raycast.cpp:226
    if (B.is_leaf(all.size(), 0) || threads <= 1) {
        B.build(P, all, 0, root);
    } else {
        // root built here; its 8 subtrees (level 1) built concurrently
        P.nodes.push_back(Node());
        P.nodes[0].leaf = -1;
        std::vector<Part<T>> parts(8);
        std::vector<std::future<void>> fut;
        std::vector<Box<T>> cb(8);
        for (int i = 0; i < 8; i++) B.child_box(root, i, cb[i]);
        int nthreads = std::max(1, std::min(threads, 8));
        std::vector<std::thread> pool;
        std::atomic<int> next{0};
        for (int t = 0; t < nthreads; t++)
            pool.emplace_back([&]() {
                std::vector<int32_t> sub;
                for (int i; (i = next.fetch_add(1)) < 8;) {
                    parts[i].min_edge = P.min_edge;
                    B.filter(all, cb[i], sub);
                    B.build(parts[i], sub, 1, cb[i]);
                }
            });
        for (auto& th : pool) th.join();
        for (int i = 0; i < 8; i++) P.nodes[0].child[i] = merge(P, parts[i]);
    }
    finish_octree(s, P, o);
}

template <typename T>
void finish_octree(const Scene<T>& s, Part<T>& P, Octree<T>& o) {
    for (int k = 0; k < 3; k++) { o.G0[k] = s.G0[k]; o.G1[k] = s.G1[k]; }
    const int32_t n_leaves = (int32_t)P.leaf_box.size();
    o.min_grid = P.min_edge;
    o.grid_num = (int32_t)((s.G1[0] - s.G0[0]) / o.min_grid);   // raycast.cpp:230
    o.ref_nodes = (int64_t)P.nodes.size();
    o.ref_list = P.n_list;
    o.leaf_box.assign((size_t)n_leaves * 8, (T)0);
    o.leaf_range.assign((size_t)n_leaves * 2, 0);
    for (int32_t l = 0; l < n_leaves; l++) {
        for (int k = 0; k < 3; k++) { o.leaf_box[l * 8 + k] = P.leaf_box[l].g0[k]; o.leaf_box[l * 8 + 4 + k] = P.leaf_box[l].g1[k]; }
        o.leaf_range[l * 2] = P.leaf_begin[l];
        o.leaf_range[l * 2 + 1] = (l + 1 < n_leaves) ? P.leaf_begin[l + 1] : (int32_t)P.entries.size();
    }
    o.entry_tri = std::move(P.entries);

    for (int a = 0; a < 3; a++) o.dims[a] = cell_coord<T>(s.G1[a], s.G0[a], o.min_grid) + 1;
    // exact cell-coordinate thresholds per axis (binary search over the
    // ordered bit patterns of T between G0 and G1)
    o.thr.clear();
    for (int a = 0; a < 3; a++) {
        o.thr_off[a] = (int32_t)o.thr.size();
        const int D = o.dims[a];
        o.thr.push_back(s.G0[a]);
        for (int k = 1; k < D; k++) {
            auto lo = OrderedBits<T>::to(s.G0[a]), hi = OrderedBits<T>::to(s.G1[a]);
            while (lo < hi) {
                auto mid = lo + (hi - lo) / 2;
                if (cell_coord<T>(OrderedBits<T>::from(mid), s.G0[a], o.min_grid) >= k) hi = mid;
                else lo = mid + 1;
            }
            o.thr.push_back(OrderedBits<T>::from(lo));
        }
        o.thr.push_back(std::numeric_limits<T>::infinity());
    }
    {
        T c = (T)0.0001;
        if ((double)c < 0.0001) c = std::nextafter(c, std::numeric_limits<T>::infinity());
        o.t_eps = c;
        T d = (T)1e-6;
        if ((double)d > 1e-6) d = std::nextafter(d, -std::numeric_limits<T>::infinity());
        o.v_eps = d;
    }

    // cell table: leaf of every cell-coordinate triple (TreeNodeNum's descent)
    const size_t ncell = (size_t)o.dims[0] * o.dims[1] * o.dims[2];
    o.cell_leaf.assign(ncell, -1);
    for (int gx = 0; gx < o.dims[0]; gx++)
        for (int gy = 0; gy < o.dims[1]; gy++)
            for (int gz = 0; gz < o.dims[2]; gz++) {
                int g[3] = {gx, gy, gz};
                int32_t cur = 0;
                int gs = o.grid_num;
                while (P.nodes[cur].leaf < 0) {
                    gs >>= 1;
                    int ix = 0;
                    for (int i = 0; i < 3; i++)
                        if (g[i] >= gs) { ix |= 1 << i; g[i] -= gs; }
                    cur = P.nodes[cur].child[ix];
                }
                o.cell_leaf[((size_t)gx * o.dims[1] + gy) * o.dims[2] + gz] = P.nodes[cur].leaf;
            }
}

template <typename T>
int cell_of_thresholds(const Octree<T>& o, int a, T q) {
    const T* th = o.thr.data() + o.thr_off[a];
    const int D = o.dims[a];
    int k = (int)((q - o.G0[a]) * (T)(1.0 / (double)o.min_grid));
    k = std::min(std::max(k, 0), D - 1);
    while (k + 1 < D && q >= th[k + 1]) ++k;
    while (k > 0 && q < th[k]) --k;
    return k;
}

template <typename T>
bool thresholds_consistent(const Octree<T>& o) {
    size_t need = 0;
    for (int a = 0; a < 3; a++) {
        if (o.dims[a] < 1 || o.thr_off[a] != (int32_t)need) return false;
        need += (size_t)o.dims[a] + 1;
    }
    return need == o.thr.size();
}

template int cell_of_thresholds<float>(const Octree<float>&, int, float);
template int cell_of_thresholds<double>(const Octree<double>&, int, double);
template bool thresholds_consistent<float>(const Octree<float>&);
template bool thresholds_consistent<double>(const Octree<double>&);
template void build_octree<float>(const Scene<float>&, Octree<float>&, int);
template void build_octree<double>(const Scene<double>&, Octree<double>&, int);
template void finish_octree<float>(const Scene<float>&, Part<float>&, Octree<float>&);
template void finish_octree<double>(const Scene<double>&, Part<double>&, Octree<double>&);

}  // namespace radgb
