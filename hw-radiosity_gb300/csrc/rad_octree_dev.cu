// Octree build with the overlap tests on the device (BuildTree,
// src/raycast.cpp:168-233).
//
// The tree is built level by level.  Every (open node, triangle) pair of a
// level is tested against the node's eight child boxes in one kernel launch
// (k_octree_masks, one byte of results per pair); these clipping tests are
// almost all of the build's work.  The host then files each triangle into the
// children its bits name, in ascending triangle order, so every list equals
// the reference's, decides leaf or open by the reference's rule (at most
// kMaxTriPerNode triangles, or level kMaxLevel), and carries the open
// children to the next level.  Nodes and leaves are numbered level by level
// instead of depth first; the walk only compares leaf ids for equality, and
// finish_octree (shared with the host build) derives the cell table, the
// thresholds and the reference's node and list counts from the same tree.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "octree_build.h"
#include "octree_geom.h"
#include "prep_workspace.h"

namespace radgb {
namespace dev {

template <typename T>
__global__ void k_octree_masks(const T* __restrict__ tv, const int32_t* __restrict__ pair_tri,
                               const int32_t* __restrict__ pair_node, const T* __restrict__ node_box,
                               long long n_pairs, uint8_t* __restrict__ mask) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n_pairs;
         j += (long long)gridDim.x * blockDim.x) {
        const T* p = tv + (size_t)pair_tri[j] * 9;
        const T* nb = node_box + (size_t)pair_node[j] * 6;
        T p0[3] = {p[0], p[1], p[2]}, p1[3] = {p[3], p[4], p[5]}, p2[3] = {p[6], p[7], p[8]};
        T b0[3] = {nb[0], nb[1], nb[2]}, b1[3] = {nb[3], nb[4], nb[5]};
        unsigned m = 0;
        for (int i = 0; i < 8; i++) {
            T c0[3], c1[3];
            geom::child_box(b0, b1, i, c0, c1);
            if (geom::tri_meets_box(p0, p1, p2, c0, c1)) m |= 1u << i;
        }
        mask[j] = (uint8_t)m;
    }
}

}  // namespace dev

namespace {

#define CU(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(RAD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// buffer k of this thread's preparation workspace
struct DevBuf {
    PrepWorkspace& ws;
    size_t k;
    void* p = nullptr;
    int ensure(size_t bytes) {
        CU(ws.buffer(k, bytes, &p));
        return RAD_OK;
    }
};

bool is_leaf(size_t n, int level) { return n <= (size_t)kMaxTriPerNode || level >= kMaxLevel; }

template <typename T>
int build_device(const Scene<T>& s, Octree<T>& o, int device) {
    CU(cudaSetDevice(device));
    PrepWorkspace& ws = prep_workspace(device);
    cudaStream_t st = nullptr;
    CU(ws.stream(&st));
    const int n = s.n_orig;
    Part<T> P;
    P.min_edge = s.G1[0] - s.G0[0];                       // raycast.cpp:226
    Box<T> root;
    for (int k = 0; k < 3; k++) { root.g0[k] = s.G0[k]; root.g1[k] = s.G1[k]; }
    auto add_leaf = [&](int32_t id, const Box<T>& b, const int32_t* list, size_t len) {
        Node& nd = P.nodes[id];
        for (int i = 0; i < 8; i++) nd.child[i] = -1;
        nd.leaf = (int32_t)P.leaf_box.size();
        P.leaf_box.push_back(b);
        P.leaf_begin.push_back((int32_t)P.entries.size());
        P.entries.insert(P.entries.end(), list, list + len);
        P.n_list += (int64_t)len + 1;
        const T edge0 = b.g1[0] - b.g0[0];
        if (edge0 < P.min_edge) P.min_edge = edge0;
    };
    P.nodes.push_back(Node());
    std::vector<int32_t> pairs((size_t)n), pair_node((size_t)n, 0);
    for (int32_t i = 0; i < n; i++) pairs[i] = i;
    if (is_leaf(pairs.size(), 0)) {
        add_leaf(0, root, pairs.data(), pairs.size());
        finish_octree(s, P, o);
        return RAD_OK;
    }
    P.nodes[0].leaf = -1;
    // triangle vertices, 9 per original triangle
    std::vector<T> tv((size_t)n * 9);
    for (int i = 0; i < n; i++)
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) tv[(size_t)i * 9 + v * 3 + k] = s.slots[i].p[v][k];
    DevBuf d_tv{ws, 0}, d_tri{ws, 1}, d_node{ws, 2}, d_box{ws, 3}, d_mask{ws, 4};
    if (int rc = d_tv.ensure(tv.size() * sizeof(T))) return rc;
    CU(cudaMemcpyAsync(d_tv.p, tv.data(), tv.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    struct Open { int32_t node; Box<T> box; };
    std::vector<Open> cur = {{0, root}};
    std::vector<size_t> seg = {0, pairs.size()};           // pair range of each open node
    std::vector<uint8_t> mask;
    std::vector<T> boxes;
    for (int level = 0; !cur.empty(); level++) {
        const size_t np = pairs.size();
        boxes.resize(cur.size() * 6);
        for (size_t a = 0; a < cur.size(); a++)
            for (int k = 0; k < 3; k++) { boxes[a * 6 + k] = cur[a].box.g0[k]; boxes[a * 6 + 3 + k] = cur[a].box.g1[k]; }
        int rc;
        if ((rc = d_tri.ensure(np * 4)) || (rc = d_node.ensure(np * 4)) || (rc = d_box.ensure(boxes.size() * sizeof(T))) ||
            (rc = d_mask.ensure(np)))
            return rc;
        CU(cudaMemcpyAsync(d_tri.p, pairs.data(), np * 4, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(d_node.p, pair_node.data(), np * 4, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(d_box.p, boxes.data(), boxes.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        if (np > 0) {
            const int grid = (int)std::min<long long>(((long long)np + 255) / 256, 1 << 16);
            dev::k_octree_masks<T><<<grid, 256, 0, st>>>((const T*)d_tv.p, (const int32_t*)d_tri.p,
                                                        (const int32_t*)d_node.p, (const T*)d_box.p, (long long)np,
                                                        (uint8_t*)d_mask.p);
            CU(cudaGetLastError());
        }
        mask.resize(np);
        CU(cudaMemcpyAsync(mask.data(), d_mask.p, np, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        // file the pairs into the children, in node order and ascending triangle order
        std::vector<Open> next;
        std::vector<int32_t> next_pairs, next_node;
        std::vector<size_t> next_seg = {0};
        std::vector<int32_t> list[8];
        for (size_t a = 0; a < cur.size(); a++) {
            for (auto& l : list) l.clear();
            for (size_t j = seg[a]; j < seg[a + 1]; j++) {
                const unsigned m = mask[j];
                for (int i = 0; i < 8; i++)
                    if ((m >> i) & 1u) list[i].push_back(pairs[j]);
            }
            for (int i = 0; i < 8; i++) {
                Box<T> cb;
                geom::child_box(cur[a].box.g0, cur[a].box.g1, i, cb.g0, cb.g1);
                const int32_t id = (int32_t)P.nodes.size();
                P.nodes.push_back(Node());
                P.nodes[cur[a].node].child[i] = id;
                if (is_leaf(list[i].size(), level + 1)) {
                    add_leaf(id, cb, list[i].data(), list[i].size());
                } else {
                    P.nodes[id].leaf = -1;
                    next.push_back({id, cb});
                    next_pairs.insert(next_pairs.end(), list[i].begin(), list[i].end());
                    next_node.insert(next_node.end(), list[i].size(), (int32_t)(next.size() - 1));
                    next_seg.push_back(next_pairs.size());
                }
            }
        }
        cur.swap(next);
        pairs.swap(next_pairs);
        pair_node.swap(next_node);
        seg.swap(next_seg);
    }
    finish_octree(s, P, o);
    return RAD_OK;
}

}  // namespace
}  // namespace radgb

using namespace radgb;

extern "C" int rad_octree_build_device(const rad_scene* h, int32_t device, rad_octree** out) {
    if (!h || !out) return fail(RAD_ERR_ARG, "rad_octree_build_device: null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RAD_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(RAD_ERR_ARG, "device index out of range");
    rad_octree* t = new (std::nothrow) rad_octree();
    if (!t) return fail(RAD_ERR_CAPACITY, "out of host memory");
    t->precision = h->precision;
    int rc = h->precision == 32 ? build_device(h->s32, t->o32, device) : build_device(h->s64, t->o64, device);
    if (rc) {
        delete t;
        return rc;
    }
    const int32_t* d = h->precision == 32 ? t->o32.dims : t->o64.dims;
    if ((int64_t)d[0] * d[1] * d[2] > (int64_t)1 << 26) {
        delete t;
        return fail(RAD_ERR_CAPACITY, "octree cell table exceeds 2^26 cells");
    }
    *out = t;
    return RAD_OK;
}
