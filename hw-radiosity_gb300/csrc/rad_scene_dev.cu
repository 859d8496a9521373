// Neighbour links on the device (InitRadiosity's pair scan, src/rad.cpp:295-334).
//
// The reference tests every pair of triangles (i, j) and every pair of
// corners (v, n); where corner v of i and corner n of j are the same point
// and the next corner of i lies on j's edge, and the normals are within the
// cosine limit, it writes nb[i][v] = j and j's matching link = i.  Later
// writes win.  Whether a write happens depends only on geometry, never on
// earlier writes, so the final value of a link is the write that comes last
// in the sequential order (i, j, v, n).  Here every candidate write is made
// at once as a 64-bit atomicMax of (order key + 1, neighbour): the largest
// key is the last write.
//
// Candidates share an exact vertex.  Corners are grouped by their exact
// coordinates (+0 and -0 as one, NaN never equal) with a hash table whose
// slots hold one representative corner; each group is a linked list.
#include <cuda_runtime.h>

#include <string>
#include <type_traits>
#include <vector>

#include "capi_internal.h"
#include "prep_workspace.h"

namespace radgb {
namespace dev {

template <typename T> struct KeyBits;
template <> struct KeyBits<float> {
    static __device__ __forceinline__ unsigned long long of(float x) {
        const unsigned u = __float_as_uint(x);
        return u == 0x80000000u ? 0ull : (unsigned long long)u;
    }
};
template <> struct KeyBits<double> {
    static __device__ __forceinline__ unsigned long long of(double x) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(x);
        return u == 0x8000000000000000ull ? 0ull : u;
    }
};

template <typename T>
__device__ __forceinline__ bool same_point(const T* a, const T* b) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {   // splitmix64 finaliser
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

// group each corner with the corners at the same point
template <typename T>
__global__ void k_group_corners(const T* __restrict__ p, int n_corner, int* table, unsigned mask, int* head,
                                int* next, int* err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_corner) return;
    const T* q = p + (size_t)c * 3;
    if (q[0] != q[0] || q[1] != q[1] || q[2] != q[2]) { next[c] = -2; return; }   // NaN: no group
    const unsigned long long h =
        mix64(KeyBits<T>::of(q[0]) * 0x9e3779b97f4a7c15ull ^ mix64(KeyBits<T>::of(q[1]) + 0x632be59bd9b4e019ull) ^
              mix64(KeyBits<T>::of(q[2]) + 0x85157af5ull));
    unsigned slot = (unsigned)h & mask;
    int rep = -1;
    for (unsigned probe = 0; probe <= mask; probe++) {
        int cur = atomicCAS(&table[slot], -1, c);
        if (cur == -1) { rep = c; break; }
        if (same_point(q, p + (size_t)cur * 3)) { rep = cur; break; }
        slot = (slot + 1) & mask;
    }
    if (rep < 0) { atomicExch(err, 1); next[c] = -2; return; }   // cannot happen: the table is never full
    next[c] = atomicExch(&head[rep], c);
}

// every candidate write of InitRadiosity's scan, resolved by the largest
// order key ((i*N + j)*3 + v)*3 + n
template <typename T>
__global__ void k_link_pairs(const T* __restrict__ p, const T* __restrict__ nrm, int N, const int* __restrict__ table,
                             const int* __restrict__ head, const int* __restrict__ next, unsigned mask,
                             unsigned long long* best) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= 3 * N || next[c] == -2) return;
    const int i = c / 3, v = c - 3 * i;
    const T* q = p + (size_t)c * 3;
    // the group's representative is the table entry holding this point
    int rep = -1;
    {
        const unsigned long long h =
            mix64(KeyBits<T>::of(q[0]) * 0x9e3779b97f4a7c15ull ^ mix64(KeyBits<T>::of(q[1]) + 0x632be59bd9b4e019ull) ^
                  mix64(KeyBits<T>::of(q[2]) + 0x85157af5ull));
        unsigned slot = (unsigned)h & mask;
        for (unsigned probe = 0; probe <= mask; probe++) {
            const int cur = table[slot];
            if (cur < 0) break;
            if (same_point(q, p + (size_t)cur * 3)) { rep = cur; break; }
            slot = (slot + 1) & mask;
        }
    }
    if (rep < 0) return;
    const T* ni = nrm + (size_t)i * 3;
    const T* a1 = p + ((size_t)i * 3 + (v + 1) % 3) * 3;
    const T li = (T)sqrt(ni[0] * ni[0] + ni[1] * ni[1] + ni[2] * ni[2]);
    for (int d = head[rep]; d >= 0; d = next[d]) {
        const int j = d / 3, n = d - 3 * j;
        if (j == i) continue;
        const T* nj = nrm + (size_t)j * 3;
        const T lj = (T)sqrt(nj[0] * nj[0] + nj[1] * nj[1] + nj[2] * nj[2]);
        const T cs = (ni[0] * nj[0] + ni[1] * nj[1] + ni[2] * nj[2]) / li / lj;   // CosTheta, include/vector.h:41
        int other = -1;
        if (same_point(a1, p + ((size_t)j * 3 + (n + 1) % 3) * 3)) other = n;
        else if (same_point(a1, p + ((size_t)j * 3 + (n + 2) % 3) * 3)) other = (n + 2) % 3;
        if (other < 0 || !((double)cs > 0.85)) continue;
        const unsigned long long key = ((unsigned long long)i * (unsigned long long)N + (unsigned long long)j) * 9ull +
                                       (unsigned long long)(v * 3 + n) + 1ull;
        atomicMax(&best[(size_t)i * 3 + v], (key << 20) | (unsigned long long)j);
        atomicMax(&best[(size_t)j * 3 + other], (key << 20) | (unsigned long long)i);
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


template <typename T>
int link_neighbours_device(Scene<T>& s, int device) {
    const int N = s.trinum;
    if (N <= 0) return RAD_OK;
    if (N > (1 << 20)) return fail(RAD_ERR_CAPACITY, "device neighbour links take at most 2^20 triangles");
    CU(cudaSetDevice(device));
    std::vector<T> hp((size_t)N * 9), hn((size_t)N * 3);
    for (int i = 0; i < N; i++) {
        const Slot<T>& t = s.slots[i];
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) hp[(size_t)i * 9 + v * 3 + k] = t.p[v][k];
        for (int k = 0; k < 3; k++) hn[(size_t)i * 3 + k] = t.n[k];
    }
    unsigned cap = 1;
    while (cap < 6u * (unsigned)N) cap <<= 1;
    const int nc = 3 * N;
    // this thread's preparation workspace: its stream and buffers 0..6
    PrepWorkspace& ws = prep_workspace(device);
    cudaStream_t st = nullptr;
    CU(ws.stream(&st));
    T *dp, *dn;
    int *table, *head, *next, *err;
    unsigned long long* best;
    auto get = [&](size_t k, auto** q, size_t bytes) -> int {
        void* r = nullptr;
        CU(ws.buffer(k, bytes, &r));
        *q = (std::remove_pointer_t<decltype(q)>)r;
        return RAD_OK;
    };
    int rc;
    if ((rc = get(0, &dp, hp.size() * sizeof(T))) || (rc = get(1, &dn, hn.size() * sizeof(T))) ||
        (rc = get(2, &table, (size_t)cap * 4)) || (rc = get(3, &head, (size_t)nc * 4)) ||
        (rc = get(4, &next, (size_t)nc * 4)) || (rc = get(5, &err, 4)) || (rc = get(6, &best, (size_t)nc * 8)))
        return rc;
    CU(cudaMemcpyAsync(dp, hp.data(), hp.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(dn, hn.data(), hn.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(table, 0xff, (size_t)cap * 4, st));
    CU(cudaMemsetAsync(head, 0xff, (size_t)nc * 4, st));
    CU(cudaMemsetAsync(err, 0, 4, st));
    CU(cudaMemsetAsync(best, 0, (size_t)nc * 8, st));
    const int blocks = (nc + 255) / 256;
    dev::k_group_corners<T><<<blocks, 256, 0, st>>>(dp, nc, table, cap - 1, head, next, err);
    dev::k_link_pairs<T><<<blocks, 256, 0, st>>>(dp, dn, N, table, head, next, cap - 1, best);
    CU(cudaGetLastError());
    std::vector<unsigned long long> hb((size_t)nc);
    int herr = 0;
    CU(cudaMemcpyAsync(hb.data(), best, hb.size() * 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (herr) return fail(RAD_ERR_CAPACITY, "neighbour-link table overflow");
    for (int i = 0; i < N; i++)
        for (int v = 0; v < 3; v++) {
            const unsigned long long b = hb[(size_t)i * 3 + v];
            if (b) s.slots[i].nb[v] = (int32_t)(b & 0xfffffull);
        }
    return RAD_OK;
}

}  // namespace
}  // namespace radgb

using namespace radgb;

extern "C" int rad_scene_init_device(rad_scene* h, int32_t device) {
    if (!h) return fail(RAD_ERR_ARG, "rad_scene_init_device: null scene");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RAD_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(RAD_ERR_ARG, "device index out of range");
    int rc;
    if (h->precision == 32) {
        init_radiosity(h->s32, false);
        rc = link_neighbours_device(h->s32, device);
    } else {
        init_radiosity(h->s64, false);
        rc = link_neighbours_device(h->s64, device);
    }
    take_scene_log(h);
    return rc;
}
