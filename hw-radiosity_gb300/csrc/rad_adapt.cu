// Adaptive split variant of the shooting loop: the reference built with
// include/config.h = ADAPT + ROLLBACK only (serialRadiosity, rad.cpp:452-490,
// and the full Shade, shade.cpp:435-554, whose delta-FF test splits
// receivers).  No pre-partition in this configuration.
//
// A step is sequential by definition: receivers are visited in slot order,
// a split appends slots that the same step visits later, replaces the
// current slot (visited again), or rewrites an earlier neighbour, and the
// sample points come from one global rand() stream.  But almost all the rays
// are independent: the three corner form factors and the centre form factor
// of every receiver against the step's shooter, and the form factors of the
// rand() sample points a receiver draws when those agree.  So each step
//   1. the device computes those four form factors for every slot
//      (k_adapt_ff, one thread per slot and point), runs the delta-FF test of
//      every receiver (k_adapt_test), numbers the sample points of the
//      receivers that pass it by a scan of their counts (the stream
//      compaction of the sampling receivers), and evaluates every one of them
//      at the rand() triple it gets if no receiver breaks its sample loop early
//      (k_adapt_samples, reading a device ring of the host's rand() stream);
//   2. the host runs the reference's receiver loop in order, taking a
//      precomputed value whenever its inputs are unchanged -- the receiver was
//      not written by a split earlier in this step, the shooter slot was not
//      either, and (for sample points) the stream is at the triple the value
//      was drawn from.  When a sample loop broke early or a rewritten receiver
//      drew points, a new speculation starts from the next receiver's first
//      point at the stream's position as soon as the receiver is done
//      (another k_adapt_samples launch, which stops the one before it).  The
//      host takes the points the device has written by the time it needs
//      them and never waits for one.  Points not written yet, and values
//      whose inputs changed -- rewritten or appended receivers, re-shaded
//      neighbours -- are evaluated on the host with the same walk and
//      form-factor code (it is compiled for both).
// The splits themselves (bisection, neighbour links, rollback) stay on the
// host: each one changes what the rest of the step sees.
// The result is bit-identical to the reference's adaptive build: every value
// is computed by the same arithmetic from the same inputs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "rad_kernels.cuh"

namespace radgb {
namespace dev {

// corner v (0..2) or centre (3) form factor of every live slot
template <typename T>
__global__ void k_adapt_ff(Slots<T> S, Grid<T> G, const Shooter<T>* __restrict__ shp, int n, T* __restrict__ ff,
                           State* st) {
    const Shooter<T> sh = *shp;
    Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
    const long long total = 4LL * n;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t >> 2), k = (int)(t & 3);
        const Q4<T> fr = S.frgb[i];
        const int parent = (int)fr.w;
        T out = 0;
        if (parent >= 0) {
            const Q4<T> pp = k < 3 ? S.vtx[i * 3 + k] : S.ctr[i];
            const Q4<T> nn = S.nrm[i];
            const T pv[3] = {pp.x, pp.y, pp.z}, nd[3] = {nn.x, nn.y, nn.z};
            out = corner_ff<T, false>(sh, pv, nd, nn.w, parent, G, c);
        }
        ff[t] = out;
    }
    const unsigned lane = threadIdx.x & 31;
    const unsigned r = __reduce_add_sync(kFull, c.rays), cap = __reduce_add_sync(kFull, c.capped),
                   lp = __reduce_add_sync(kFull, c.loops);
    if (lane == 0) {
        if (r) atomicAdd(&st->rays, (unsigned long long)r);
        if (cap) atomicAdd(&st->capped, (unsigned long long)cap);
        if (lp) atomicAdd(&st->loops, (unsigned long long)lp);
    }
}

// ------------------------------------------------------------------ sample points
// Shade's delta-FF test (shade.cpp:481-508) of every receiver against the
// step's shooter, from its corner and centre form factors: a receiver whose
// corner mean and centre agree draws n = (int)(area / sample_area) rand()
// sample points, unless it is small (area < adapt_area), the pool is full or
// its area is below 1e-8.  ntask[s] = n for those receivers (0 for the others,
// for receivers the host does not visit -- the shooter, dead slots, closed
// ones -- and above kMaxSpecSamples); *n_split counts the receivers whose
// test fails (split candidates).  The exclusive scan of ntask numbers every
// sample point of the step (the stream compaction of the sampling receivers):
// with no split or early break, sample point t of the step is drawn from rand()
// triple base + t.
constexpr int kMaxSpecSamples = 1 << 14;

template <typename T>
__global__ void k_adapt_test(Slots<T> S, int n, const T* __restrict__ ff, const uint8_t* __restrict__ open,
                             float adapt_area, float delta_ff, float sample_area, int pool_full, long long* ntask,
                             unsigned* n_split) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    long long k = 0;
    if (open[s]) {
        const T area = S.ctr[s].w;
        if (!(area < adapt_area) && !pool_full && !((double)area < 1e-8)) {
            const T f0 = ff[4 * s], f1 = ff[4 * s + 1], f2 = ff[4 * s + 2], fc = ff[4 * s + 3];
            const T ground = (T)((double)(f0 + f1 + f2) / 3.0);
            const T dff = (T)fabs((double)(ground - fc));
            if (dff < delta_ff) {
                const T q = area / sample_area;
                if (q >= (T)1 && q < (T)(kMaxSpecSamples + 1)) k = (int)q;
            } else {
                atomicAdd(n_split, 1u);
            }
        }
    }
    ntask[s] = k;
}

// exclusive scan of v[0..n) into out[0..n], out[n] = total: tiles of 1024
// scanned per CTA, the tile sums by one CTA, then the tile offsets added
constexpr int kScanTile = 1024;

__device__ __forceinline__ long long block_excl_scan(long long x, long long* total) {
    __shared__ long long ws[32];
    __shared__ long long wtot;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const long long y = __shfl_up_sync(kFull, inc, d);
        if (lane >= d) inc += y;
    }
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        long long w = lane < nw ? ws[lane] : 0, wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(kFull, wi, d);
            if (lane >= d) wi += y;
        }
        if (lane < nw) ws[lane] = wi - w;
        if (lane == nw - 1) wtot = wi;
    }
    __syncthreads();
    const long long r = ws[wid] + inc - x;
    *total = wtot;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanTile) k_scan_tiles(const long long* v, int n, long long* out, long long* tile_sum) {
    const int i = blockIdx.x * kScanTile + threadIdx.x;
    long long tot;
    const long long e = block_excl_scan(i < n ? v[i] : 0, &tot);
    if (i < n) out[i] = e;
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanTile) k_scan_sums(long long* tile_sum, int tiles, long long* out, int n) {
    long long carry = 0;
    for (int b = 0; b < tiles; b += kScanTile) {
        const int i = b + threadIdx.x;
        long long tot;
        const long long e = block_excl_scan(i < tiles ? tile_sum[i] : 0, &tot);
        if (i < tiles) tile_sum[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void __launch_bounds__(kScanTile) k_scan_add(const long long* tile_off, int n, long long* out) {
    const int i = blockIdx.x * kScanTile + threadIdx.x;
    if (i < n) out[i] += tile_off[blockIdx.x];
}

// Sample points [start, end) of the step (end clipped to the step's total),
// point t drawn from rand() triple base + (t - start) of the ring: the
// receiver (largest s with toff[s] <= t), GetPointInTriangle (shade.cpp:49-68)
// and the point's AdaptCalFF(CalFF(...)) (shade.cpp:499-502).  Written to host
// memory: ff[t] and the walk counters of its rays (rays | capped << 8 |
// loops << 16), added on the host only for points it uses, then, after a
// system-scope fence, tag[t] = gen: the host reads a point as soon as its tag
// shows this speculation, without waiting for the kernel.  A thread stops
// when *live (host memory the host writes) no longer holds gen: the host has
// started a newer speculation and will not read this one's points.
template <typename T>
__global__ void k_adapt_samples(Slots<T> S, Grid<T> G, const Shooter<T>* __restrict__ shp,
                                const long long* __restrict__ toff, int n, long long start, long long end,
                                long long base, const int32_t* __restrict__ ring, long long ring_len,
                                T* __restrict__ out_ff, int* __restrict__ out_code, unsigned* out_tag,
                                const volatile unsigned* live, unsigned gen) {
    const long long total = toff[n];
    if (end > total) end = total;
    const Shooter<T> sh = *shp;
    for (long long t = start + blockIdx.x * (long long)blockDim.x + threadIdx.x; t < end;
         t += (long long)gridDim.x * blockDim.x) {
        if (*live != gen) return;
        int lo = 0, hi = n - 1;        // toff is non-decreasing; toff[0] = 0 <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (toff[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const int s = lo;
        const long long tri = base + (t - start);
        T r1 = (T)ring[(3 * tri) % ring_len], r2 = (T)ring[(3 * tri + 1) % ring_len],
          r3 = (T)ring[(3 * tri + 2) % ring_len];
        const T tot = r1 + r2 + r3;
        r1 /= tot; r2 /= tot; r3 /= tot;
        const Q4<T> p0 = S.vtx[s * 3], p1 = S.vtx[s * 3 + 1], p2 = S.vtx[s * 3 + 2];
        const T pt[3] = {r1 * p0.x + r2 * p1.x + r3 * p2.x, r1 * p0.y + r2 * p1.y + r3 * p2.y,
                         r1 * p0.z + r2 * p1.z + r3 * p2.z};
        const Q4<T> nn = S.nrm[s];
        const T nd[3] = {nn.x, nn.y, nn.z};
        Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
        out_ff[t] = corner_ff<T, false>(sh, pt, nd, nn.w, (int)S.frgb[s].w, G, c);
        out_code[t] = (int)(c.rays | (c.capped << 8) | (c.loops << 16));
        __threadfence_system();
        *(volatile unsigned*)(out_tag + t) = gen;
    }
}

// write the records of changed slots: rec holds vtx[3], nrm, ctr, frgb per slot
template <typename T>
__global__ void k_adapt_scatter(Q4<T>* vtx, Q4<T>* nrm, Q4<T>* ctr, Q4<T>* frgb, const int* __restrict__ idx,
                                const Q4<T>* __restrict__ rec, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = idx[j];
    const Q4<T>* r = rec + 6 * (size_t)j;
    vtx[i * 3] = r[0];
    vtx[i * 3 + 1] = r[1];
    vtx[i * 3 + 2] = r[2];
    nrm[i] = r[3];
    ctr[i] = r[4];
    frgb[i] = r[5];
}

}  // namespace dev
}  // namespace radgb

using namespace radgb;
using namespace radgb::dev;

#define CU(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(RAD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

// glibc's rand() (TYPE_3: x[i] = x[i-3] + x[i-31] mod 2^32, output x >> 1),
// in the front/rear-pointer form of random_r, seeded with 1 as the
// reference never calls srand.
class LibcRand {
    int32_t st_[31];
    int f_ = 3, r_ = 0;

public:
    LibcRand() {
        int32_t w = 1;
        st_[0] = w;
        for (int i = 1; i < 31; i++) {     // 16807 w mod (2^31 - 1), Schrage's method
            const int32_t hi = w / 127773, lo = w % 127773;
            w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            st_[i] = w;
        }
        for (int k = 0; k < 310; k++) next();
    }
    int next() {
        uint32_t v = (uint32_t)st_[f_] + (uint32_t)st_[r_];
        st_[f_] = (int32_t)v;
        if (++f_ >= 31) { f_ = 0; ++r_; }
        else if (++r_ >= 31) r_ = 0;
        return (int)(v >> 1);
    }
};

// The rand() stream with absolute positions: values are generated ahead on
// demand and kept until consumed, so the device can be given future draws.
class RandStream {
    LibcRand g_;
    std::vector<int32_t> buf_;
    long long base_ = 0;   // absolute index of buf_[0]

public:
    long long pos = 0;     // draws consumed so far
    int32_t at(long long i) {
        while (base_ + (long long)buf_.size() <= i) buf_.push_back(g_.next());
        return buf_[(size_t)(i - base_)];
    }
    int next() {
        const int32_t v = at(pos++);
        if (pos - base_ > (1 << 20)) {
            buf_.erase(buf_.begin(), buf_.begin() + (size_t)(pos - base_));
            base_ = pos;
        }
        return v;
    }
};

template <typename T>
inline T slot_nlen(const Slot<T>& t) { return (T)std::sqrt(t.n[0] * t.n[0] + t.n[1] * t.n[1] + t.n[2] * t.n[2]); }

template <typename T>
inline bool is_open(const Slot<T>& t) {   // some accB component < 255 (rad.cpp:471-475)
    for (int v = 0; v < 3; v++)
        for (int c = 0; c < 3; c++)
            if ((double)t.accB[v][c] < 255.0) return true;
    return false;
}

template <typename T>
struct AdaptImpl {
    int device = 0;
    cudaStream_t stream = nullptr;
    Scene<T>* sc = nullptr;
    HostPack<T> pack;          // walk structure (and initial slot records)
    Grid<T> Gh{}, Gd{};        // host / device views of the walk structure
    int cap = 0;               // slot capacity on the device
    Q4<T> *d_vtx = nullptr, *d_nrm = nullptr, *d_ctr = nullptr, *d_frgb = nullptr;
    T* d_ff = nullptr;
    Shooter<T>* d_sh = nullptr;
    State* d_state = nullptr;
    int* d_idx = nullptr;
    Q4<T>* d_rec = nullptr;
    int stage_cap = 0;
    std::vector<void*> allocs;
    size_t bytes = 0;
    std::vector<T> ff;                    // host copy of the step's precomputed values
    std::vector<uint32_t> mod_step;       // step in which a slot was last rewritten by a split
    std::vector<uint8_t> dirty;           // device record out of date
    std::vector<int32_t> dirty_list;
    std::vector<int32_t> trace;
    RandStream rng;
    long long steps = 0;
    bool done = false;
    Cnt hc = {0, 0, 0, 0, 0, 0, 0, 0};    // host-side walks, and the device sample points used
    long long samples = 0, splits = 0, pre_used = 0, host_points = 0;
    uint32_t step_id = 1;

    // Sample points on the device.  Per step: the delta-FF test of every
    // receiver (ntask), its exclusive scan (toff: the first sample point of
    // each receiver), and a speculation -- the sample points of tasks
    // [sp_start, sp_end) drawn from rand() triples sp_base + (t - sp_start).
    // The host uses a receiver's speculated values only when its draws start
    // at exactly that triple; a sample loop that breaks early or a rewritten
    // receiver that draws moves the stream, and a new speculation starts from
    // the next receiver's first point at the stream's position.  Speculations
    // are numbered (sp_gen); the kernel tags each point it writes with its
    // number (h_stag) and stops once *h_live names a newer one.  The host
    // takes a point the kernel has already written and evaluates the others
    // itself, and a superseded speculation frees the GPU at once.
    uint8_t* d_open = nullptr;
    uint8_t* h_open = nullptr;            // pinned
    long long *d_ntask = nullptr, *d_toff = nullptr, *d_tiles = nullptr;
    long long* h_toff = nullptr;          // pinned, cap + 1
    unsigned* d_nsplit = nullptr;
    unsigned* h_nsplit = nullptr;         // pinned
    T* h_sff = nullptr;                   // mapped: sample point form factors, by task
    int* h_scode = nullptr;               // mapped: their walk counters
    T* dm_sff = nullptr;
    int* dm_scode = nullptr;
    long long task_cap = 1 << 21;
    int32_t* d_ring = nullptr;            // rand() values, value i at i % ring_len
    int32_t* h_ring = nullptr;            // pinned staging of the ring
    long long ring_len = 1 << 21, ring_hi = 0;
    long long sp_start = 0, sp_end = 0, sp_base = 0;
    unsigned* h_stag = nullptr;           // mapped: the speculation that wrote each point
    unsigned* h_live = nullptr;           // mapped: the speculation whose points are still wanted
    unsigned* dm_stag = nullptr;
    unsigned* dm_live = nullptr;
    unsigned sp_gen = 0;
    cudaEvent_t copies_done = nullptr;    // the step's test results are on the host
    cudaEvent_t sp_done = nullptr;        // recorded after each speculation
    // 0: the host races the speculation (takes the points already written,
    //    evaluates the others itself, re-speculates as soon as a receiver
    //    moves the stream); 1: the host waits for each new speculation to
    //    finish, started only when the next sampling receiver needs it
    int spec_wait_mode = 0;
    bool sp_finished = false;             // the current speculation has been waited for
    long long dev_samples = 0, spec_launches = 0, split_candidates = 0;
    std::vector<void*> pinned;

    ~AdaptImpl() {
        if (h_live) __atomic_store_n(h_live, sp_gen + 1, __ATOMIC_RELEASE);   // stop a running speculation
        if (stream) cudaStreamSynchronize(stream);
        if (copies_done) cudaEventDestroy(copies_done);
        if (sp_done) cudaEventDestroy(sp_done);
        for (void* p : allocs) cudaFree(p);
        for (void* p : pinned) cudaFreeHost(p);
        if (stream) cudaStreamDestroy(stream);
    }
    template <typename U>
    int host_alloc(U** p, size_t count, unsigned flags) {
        void* q = nullptr;
        CU(cudaHostAlloc(&q, std::max<size_t>(count * sizeof(U), 16), flags));
        pinned.push_back(q);
        *p = (U*)q;
        return RAD_OK;
    }
    template <typename U>
    int alloc(U** p, size_t count) {
        void* q = nullptr;
        size_t b = std::max<size_t>(count * sizeof(U), 16);
        CU(cudaMalloc(&q, b));
        allocs.push_back(q);
        bytes += b;
        *p = (U*)q;
        return RAD_OK;
    }
    void mark(int32_t i) {
        if (i < 0) return;
        mod_step[i] = step_id;
        if (!dirty[i]) { dirty[i] = 1; dirty_list.push_back(i); }
    }
};

template <typename T>
int adapt_upload_dirty(AdaptImpl<T>& a) {
    const int n = (int)a.dirty_list.size();
    if (!n) return RAD_OK;
    if (n > a.stage_cap) {
        int cap = std::max(n, 2 * a.stage_cap);
        int rc;
        if ((rc = a.alloc(&a.d_idx, (size_t)cap)) || (rc = a.alloc(&a.d_rec, (size_t)cap * 6))) return rc;
        a.stage_cap = cap;
    }
    std::vector<Q4<T>> rec((size_t)n * 6);
    for (int j = 0; j < n; j++) {
        const Slot<T>& t = a.sc->slots[a.dirty_list[j]];
        for (int v = 0; v < 3; v++) rec[6 * j + v] = {t.p[v][0], t.p[v][1], t.p[v][2], 0};
        rec[6 * j + 3] = {t.n[0], t.n[1], t.n[2], slot_nlen(t)};
        rec[6 * j + 4] = {t.c[0], t.c[1], t.c[2], t.area};
        rec[6 * j + 5] = {(T)t.Frgb[0], (T)t.Frgb[1], (T)t.Frgb[2], (T)t.parent};
    }
    CU(cudaMemcpyAsync(a.d_idx, a.dirty_list.data(), (size_t)n * 4, cudaMemcpyHostToDevice, a.stream));
    CU(cudaMemcpyAsync(a.d_rec, rec.data(), rec.size() * sizeof(Q4<T>), cudaMemcpyHostToDevice, a.stream));
    k_adapt_scatter<T><<<(n + 127) / 128, 128, 0, a.stream>>>(a.d_vtx, a.d_nrm, a.d_ctr, a.d_frgb, a.d_idx, a.d_rec, n);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(a.stream));   // rec is a host temporary
    for (int32_t i : a.dirty_list) a.dirty[i] = 0;
    a.dirty_list.clear();
    return RAD_OK;
}

template <typename T>
int adapt_create(Scene<T>& s, const Octree<T>& o, const rad_options& opt, int device, AdaptImpl<T>& a) {
    a.device = device;
    a.sc = &s;
    CU(cudaSetDevice(device));
    CU(cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking));
    if (!thresholds_consistent(o)) return fail(RAD_ERR_ARG, "octree cell thresholds do not match its dimensions");
    pack_scene(s, o, a.pack);
    a.Gh = grid_params(o, opt.walk_cap);
    a.Gh.thr = a.pack.thr.data();
    a.Gh.cell = a.pack.cell.data();
    a.Gh.entry = a.pack.ent.data();
    a.cap = (int)s.slots.size();
    int rc;
    auto put = [&](auto** dst, const auto& src) -> int {
        int r = a.alloc(dst, src.size());
        if (r) return r;
        CU(cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice, a.stream));
        return RAD_OK;
    };
    Q4<T>* d_ent;
    CellRec<T>* d_cell;
    T* d_thr;
    if ((rc = put(&d_ent, a.pack.ent)) || (rc = put(&d_cell, a.pack.cell)) ||
        (rc = put(&d_thr, a.pack.thr)))
        return rc;
    a.Gd = a.Gh;
    a.Gd.thr = d_thr;
    a.Gd.cell = d_cell;
    a.Gd.entry = d_ent;
    if ((rc = a.alloc(&a.d_vtx, (size_t)a.cap * 3)) || (rc = a.alloc(&a.d_nrm, (size_t)a.cap)) ||
        (rc = a.alloc(&a.d_ctr, (size_t)a.cap)) || (rc = a.alloc(&a.d_frgb, (size_t)a.cap)) ||
        (rc = a.alloc(&a.d_ff, (size_t)a.cap * 4)) || (rc = a.alloc(&a.d_sh, 1)) || (rc = a.alloc(&a.d_state, 1)))
        return rc;
    CU(cudaMemsetAsync(a.d_state, 0, sizeof(State), a.stream));
    // the sample-point speculation: per-slot test results and offsets, the
    // rand() ring, and the mapped host buffers the sample kernel writes
    const int tiles = (a.cap + kScanTile - 1) / kScanTile;
    if ((rc = a.alloc(&a.d_open, (size_t)a.cap)) || (rc = a.alloc(&a.d_ntask, (size_t)a.cap)) ||
        (rc = a.alloc(&a.d_toff, (size_t)a.cap + 1)) || (rc = a.alloc(&a.d_tiles, (size_t)tiles)) ||
        (rc = a.alloc(&a.d_nsplit, 1)) || (rc = a.alloc(&a.d_ring, (size_t)a.ring_len)) ||
        (rc = a.host_alloc(&a.h_open, (size_t)a.cap, cudaHostAllocDefault)) ||
        (rc = a.host_alloc(&a.h_toff, (size_t)a.cap + 1, cudaHostAllocDefault)) ||
        (rc = a.host_alloc(&a.h_nsplit, 1, cudaHostAllocDefault)) ||
        (rc = a.host_alloc(&a.h_ring, (size_t)a.ring_len, cudaHostAllocDefault)) ||
        (rc = a.host_alloc(&a.h_sff, (size_t)a.task_cap, cudaHostAllocMapped)) ||
        (rc = a.host_alloc(&a.h_scode, (size_t)a.task_cap, cudaHostAllocMapped)) ||
        (rc = a.host_alloc(&a.h_stag, (size_t)a.task_cap, cudaHostAllocMapped)) ||
        (rc = a.host_alloc(&a.h_live, 1, cudaHostAllocMapped)))
        return rc;
    CU(cudaHostGetDevicePointer((void**)&a.dm_sff, a.h_sff, 0));
    CU(cudaHostGetDevicePointer((void**)&a.dm_scode, a.h_scode, 0));
    CU(cudaHostGetDevicePointer((void**)&a.dm_stag, a.h_stag, 0));
    CU(cudaHostGetDevicePointer((void**)&a.dm_live, a.h_live, 0));
    std::memset(a.h_stag, 0, (size_t)a.task_cap * sizeof(unsigned));
    *a.h_live = 0;
    CU(cudaEventCreateWithFlags(&a.copies_done, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&a.sp_done, cudaEventDisableTiming));
    a.ff.assign((size_t)a.cap * 4, (T)0);
    a.mod_step.assign((size_t)a.cap, 0);
    a.dirty.assign((size_t)a.cap, 0);
    for (int32_t i = 0; i < s.trinum; i++) a.mark(i);
    a.step_id = 1;
    return adapt_upload_dirty(a);
}

// keep the device ring holding rand() values [pos, pos + ring_len)
template <typename T>
int ring_top_up(AdaptImpl<T>& a) {
    const long long want = a.rng.pos + a.ring_len;
    if (a.ring_hi >= want) return RAD_OK;
    const long long lo = std::max(a.ring_hi, a.rng.pos);
    for (long long i = lo; i < want; i++) a.h_ring[i % a.ring_len] = a.rng.at(i);
    // one or two contiguous pieces of the ring
    long long i = lo;
    while (i < want) {
        const long long off = i % a.ring_len;
        const long long len = std::min(want - i, a.ring_len - off);
        CU(cudaMemcpyAsync(a.d_ring + off, a.h_ring + off, (size_t)len * 4, cudaMemcpyHostToDevice, a.stream));
        i += len;
    }
    a.ring_hi = want;
    return RAD_OK;
}

// stop every speculation in flight: none of their points will be read
template <typename T>
int spec_cancel(AdaptImpl<T>& a) {
    if (a.sp_gen >= 0xfffffff0u) {      // numbers about to wrap: clear the tags first
        CU(cudaStreamSynchronize(a.stream));
        std::memset(a.h_stag, 0, (size_t)a.task_cap * sizeof(unsigned));
        a.sp_gen = 0;
    }
    a.sp_gen++;
    __atomic_store_n(a.h_live, a.sp_gen, __ATOMIC_RELEASE);
    a.sp_start = a.sp_end = a.sp_base = 0;
    a.sp_finished = false;
    return RAD_OK;
}

// enqueue the sample points of tasks [start, ...) drawn from triples base, ...
// (clipped to the task capacity, the ring and, on the device, the step's
// total), superseding the speculation in flight.  The ring's staging may be
// rewritten while an older copy from it is still queued: that copy then moves
// the newer values, which land in the same ring positions, and only the
// superseded kernel before it could read them.
template <typename T>
int spec_enqueue(AdaptImpl<T>& a, const Slots<T>& S, int n0, long long start, long long base, long long end) {
    int rc;
    if ((rc = spec_cancel(a)) || (rc = ring_top_up(a))) return rc;
    end = std::min(end, a.task_cap);
    end = std::min(end, start + (a.rng.pos + a.ring_len) / 3 - base);
    a.sp_start = start;
    a.sp_base = base;
    a.sp_end = std::max(start, end);
    a.spec_launches++;
    if (a.sp_end <= start || n0 <= 0) return RAD_OK;
    const long long work = a.sp_end - start;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((work + 127) / 128, 152 * 16));
    k_adapt_samples<T><<<blocks, 128, 0, a.stream>>>(S, a.Gd, a.d_sh, a.d_toff, n0, start, a.sp_end, base, a.d_ring,
                                                     a.ring_len, a.dm_sff, a.dm_scode, a.dm_stag, a.dm_live,
                                                     a.sp_gen);
    CU(cudaGetLastError());
    CU(cudaEventRecord(a.sp_done, a.stream));
    return RAD_OK;
}

// Whether point t of the current speculation is on the host.  Racing, the
// host never waits for one: a walk on the GPU takes longer than the same walk
// on the host, so a point the device has not written yet is evaluated on the
// host (the same arithmetic, the same value) while the kernel runs ahead to
// the receivers after it.  Waiting, device_points has already waited for the
// whole speculation, so every point it wrote is there.  A failed kernel is
// reported by the next step's stream synchronisation.
template <typename T>
bool spec_ready(const AdaptImpl<T>& a, long long t) {
    return __atomic_load_n(a.h_stag + t, __ATOMIC_ACQUIRE) == a.sp_gen;
}

template <typename T>
void host_shooter(const Slot<T>& t, int slot, int logsrc, Shooter<T>& sh) {
    make_shooter(t.p, t.c, t.n, slot_nlen(t), t.area, t.deltaB, slot, logsrc, sh);
}

// CalRadiosity, shade.cpp:244-259 (the shooter's unshot energy read live)
template <typename T>
void deposit(const Slot<T>& src, Slot<T>& des, const T ff[3]) {
    const T k = (T)(0.5 / 255.0);
    T lo[3];
    for (int c = 0; c < 3; c++) lo[c] = (T)des.Frgb[c] * k * src.deltaB[c] / 3;
    for (int v = 0; v < 3; v++)
        for (int c = 0; c < 3; c++) {
            const T x = lo[c] * ff[v];
            des.deltaB[c] += x;
            des.accB[v][c] += x;
            des.daccB[v][c] = x;
        }
}

template <typename T>
struct StepCtx {
    AdaptImpl<T>& a;
    int src, logsrc, n0;
    Slots<T> S;               // the device slots as the step started
    bool shooter_changed = false;
    int err = RAD_OK;
    Shooter<T> sh;            // the shooter as the precompute saw it
    Shooter<T> live;          // rebuilt from the slot after a split rewrote it

    // whether the current speculation holds points [t, t + n) drawn from the
    // triples that start at triple cur
    bool covered(long long t, long long n, long long cur) const {
        return t >= a.sp_start && t + n <= a.sp_end && a.sp_base + (t - a.sp_start) == cur;
    }

    // The first task of receiver d's n sample points on the device, when they
    // are the ones it draws now: d is unchanged this step (pre_ok), the
    // device's test gave it n points, and the speculation covering them starts
    // them at the stream's current triple (otherwise a new speculation starts
    // at d).  -1 when d's points are evaluated on the host.
    long long device_points(int d, int n) {
        if (a.rng.pos % 3 != 0) return -1;
        const long long t0 = a.h_toff[d];
        if (a.h_toff[d + 1] - t0 != n) return -1;
        const long long cur = a.rng.pos / 3;
        if (!covered(t0, n, cur)) {
            if (int rc = spec_enqueue(a, S, n0, t0, cur, a.h_toff[n0])) { err = rc; return -1; }
            if (!covered(t0, n, cur)) return -1;
        }
        if (a.spec_wait_mode && !a.sp_finished) {       // the whole speculation, once
            if (cudaEventSynchronize(a.sp_done) != cudaSuccess) {
                err = fail(RAD_ERR_CUDA, "sample-point kernel failed");
                return -1;
            }
            a.sp_finished = true;
        }
        return t0;
    }

    // After receiver d is done: when the stream no longer sits where the
    // speculation puts the next receiver's first point (d broke its sample
    // loop, drew on the host, or drew nothing where the device's test said it
    // would), start the speculation from there now, so that it runs while the
    // host gets to that receiver.
    void respeculate_after(int d) {
        if (a.spec_wait_mode || d + 1 >= n0 || a.rng.pos % 3 != 0) return;
        const long long t = a.h_toff[d + 1];
        if (t >= a.h_toff[n0] || covered(t, 1, a.rng.pos / 3)) return;
        if (int rc = spec_enqueue(a, S, n0, t, a.rng.pos / 3, a.h_toff[n0])) err = rc;
    }

    // AdaptCalFF(CalFF(...)) for point p of receiver d (its normal) with ban logdes
    T ff_host(int d, const T* p, int logdes) {
        const Slot<T>& r = a.sc->slots[d];
        const T nd[3] = {r.n[0], r.n[1], r.n[2]};
        a.host_points++;
        return corner_ff<T, false>(shooter_changed ? live : sh, p, nd, slot_nlen(r), logdes, a.Gh, a.hc);
    }
    bool pre_ok(int d) const { return !shooter_changed && d < n0 && a.mod_step[d] != a.step_id; }
    void touched(int32_t i) {
        a.mark(i);
        if (i == src) {
            shooter_changed = true;
            host_shooter(a.sc->slots[src], src, logsrc, live);
        }
    }

    // Shade, shade.cpp:435-554 (ADAPT, ROLLBACK; no DONT_PARTITION, no PARALLEL)
    int shade(int d, int logdes) {
        Scene<T>& s = *a.sc;
        const rad_options& o = s.opt;
        T f[3];
        const bool pre = pre_ok(d);
        for (int v = 0; v < 3; v++) f[v] = pre ? a.ff[4 * (size_t)d + v] : ff_host(d, s.slots[d].p[v], logdes);
        if (pre) a.pre_used++;
        Slot<T>& des = s.slots[d];
        if (des.area < o.adapt_area) { deposit(s.slots[src], des, f); return 0; }
        if (pool_full(s, 4) || (double)des.area < 1e-8) { deposit(s.slots[src], des, f); return 0; }
        T ground = (T)((double)(f[0] + f[1] + f[2]) / 3.0);
        T ffs = pre ? a.ff[4 * (size_t)d + 3] : ff_host(d, des.c, logdes);
        T dff;
        if ((dff = (T)std::fabs((double)(ground - ffs))) < o.delta_ff) {
            const int n = (int)(des.area / o.sample_area);
            const long long t0 = pre && n > 0 ? device_points(d, n) : -1;
            for (int k = 0; k < n; k++) {
                // GetPointInTriangle, shade.cpp:49-68
                T r1 = (T)a.rng.next(), r2 = (T)a.rng.next(), r3 = (T)a.rng.next();
                const T tot = r1 + r2 + r3;
                r1 /= tot; r2 /= tot; r3 /= tot;
                ground = r1 * f[0] + r2 * f[1] + r3 * f[2];
                a.samples++;
                if (t0 >= 0 && spec_ready(a, t0 + k)) {   // drawn from this very triple on the device
                    const int code = a.h_scode[t0 + k];
                    ffs = a.h_sff[t0 + k];
                    a.hc.rays += code & 0xff;
                    a.hc.capped += (code >> 8) & 0xff;
                    a.hc.loops += (code >> 16) & 0xff;
                    a.dev_samples++;
                } else {
                    T pt[3];
                    for (int q = 0; q < 3; q++) pt[q] = r1 * des.p[0][q] + r2 * des.p[1][q] + r3 * des.p[2][q];
                    ffs = ff_host(d, pt, logdes);
                }
                if ((dff = (T)std::fabs((double)(ground - ffs))) > o.delta_ff) break;
            }
            if (dff < o.delta_ff) { deposit(s.slots[src], des, f); return 0; }
        }
        int32_t out[4], nbid;
        bool reshade;
        const int rep = split_receiver(s, d, out, reshade, &nbid);
        if (rep >= 0) {
            a.splits++;
            touched(d);
            touched(nbid);
            for (int q = 0; q < 4; q++) touched(out[q]);
        }
        if (reshade) {
            const int t4 = out[3];
            for (int v = 0; v < 3; v++) f[v] = ff_host(t4, s.slots[t4].p[v], logdes);
            deposit(s.slots[src], s.slots[t4], f);
        }
        return rep;
    }
};

// MaxDeltaRad, rad.cpp:359-386: the first strict maximum (ties: lowest slot)
template <typename T>
int max_delta(const Scene<T>& s) {
    int best = -1;
    T m = 0;
    for (int i = 0; i < s.trinum; i++) {
        const Slot<T>& t = s.slots[i];
        if (t.parent < 0) continue;
        const T d = t.deltaB[0] + t.deltaB[1] + t.deltaB[2];
        if (d > m && d > (T)s.opt.converge) { best = i; m = d; }
    }
    return best;
}

template <typename T>
int adapt_step(AdaptImpl<T>& a) {
    Scene<T>& s = *a.sc;
    const int src = max_delta(s);
    if (src < 0) { a.done = true; return RAD_OK; }
    a.trace.push_back(src);
    int rc;
    if ((rc = spec_cancel(a)) || (rc = adapt_upload_dirty(a))) return rc;
    const int n0 = s.trinum;
    const Slots<T> S{n0, a.d_vtx, a.d_nrm, a.d_ctr, a.d_frgb, nullptr, nullptr};
    StepCtx<T> cx{a, src, s.slots[src].parent, n0, S};
    host_shooter(s.slots[src], src, cx.logsrc, cx.sh);
    CU(cudaMemcpyAsync(a.d_sh, &cx.sh, sizeof cx.sh, cudaMemcpyHostToDevice, a.stream));
    a.h_toff[0] = 0;
    if (n0 > 0) {
        // the receivers the loop will visit, as the step starts
        for (int d = 0; d < n0; d++) {
            const Slot<T>& t = s.slots[d];
            a.h_open[d] = d != src && t.parent >= 0 && is_open(t);
        }
        CU(cudaMemcpyAsync(a.d_open, a.h_open, (size_t)n0, cudaMemcpyHostToDevice, a.stream));
        CU(cudaMemsetAsync(a.d_nsplit, 0, sizeof(unsigned), a.stream));
        // every slot's corner and centre form factors against this shooter
        const int blocks = (int)std::min<long long>((4LL * n0 + 255) / 256, 152 * 16);
        k_adapt_ff<T><<<blocks, 256, 0, a.stream>>>(S, a.Gd, a.d_sh, n0, a.d_ff, a.d_state);
        // the delta-FF test of every receiver, and its sample points numbered
        const rad_options& o = s.opt;
        k_adapt_test<T><<<(n0 + 255) / 256, 256, 0, a.stream>>>(S, n0, a.d_ff, a.d_open, o.adapt_area, o.delta_ff,
                                                              o.sample_area, pool_full(s, 4) ? 1 : 0, a.d_ntask,
                                                              a.d_nsplit);
        const int tiles = (n0 + kScanTile - 1) / kScanTile;
        k_scan_tiles<<<tiles, kScanTile, 0, a.stream>>>(a.d_ntask, n0, a.d_toff, a.d_tiles);
        k_scan_sums<<<1, kScanTile, 0, a.stream>>>(a.d_tiles, tiles, a.d_toff, n0);
        k_scan_add<<<tiles, kScanTile, 0, a.stream>>>(a.d_tiles, n0, a.d_toff);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(a.ff.data(), a.d_ff, (size_t)n0 * 4 * sizeof(T), cudaMemcpyDeviceToHost, a.stream));
        CU(cudaMemcpyAsync(a.h_toff, a.d_toff, (size_t)(n0 + 1) * sizeof(long long), cudaMemcpyDeviceToHost, a.stream));
        CU(cudaMemcpyAsync(a.h_nsplit, a.d_nsplit, sizeof(unsigned), cudaMemcpyDeviceToHost, a.stream));
        CU(cudaEventRecord(a.copies_done, a.stream));
        // the first speculation: every sample point of the step, as if none
        // broke early; it runs while the host starts the receiver loop
        int rc0;
        if (a.rng.pos % 3 == 0 && (rc0 = spec_enqueue(a, S, n0, 0, a.rng.pos / 3, a.task_cap))) return rc0;
        CU(cudaEventSynchronize(a.copies_done));
        a.sp_end = std::min(a.sp_end, a.h_toff[n0]);
        a.split_candidates += *a.h_nsplit;
    } else {
        CU(cudaStreamSynchronize(a.stream));
    }
    // serialRadiosity's receiver loop, rad.cpp:464-485 (bound re-read: splits append slots)
    for (int d = 0; d < s.trinum; d++) {
        if (d == src) continue;
        const Slot<T>& t = s.slots[d];
        if (t.parent < 0) continue;
        if (!is_open(t)) continue;
        if (cx.shade(d, t.parent)) d--;
        else cx.respeculate_after(d);
        if (cx.err) return cx.err;
    }
    int rc1;
    if ((rc1 = spec_cancel(a))) return rc1;
    Slot<T>& sr = s.slots[src];
    sr.deltaB[0] = sr.deltaB[1] = sr.deltaB[2] = 0;
    a.steps++;
    a.step_id++;
    return RAD_OK;
}

template <typename T>
int adapt_run(AdaptImpl<T>& a, long long max_steps, long long* done_steps, int* converged) {
    CU(cudaSetDevice(a.device));
    long long k = 0;
    int rc;
    while (k < max_steps && !a.done) {
        const long long before = a.steps;
        if ((rc = adapt_step(a))) return rc;
        k += a.steps - before;
    }
    if (done_steps) *done_steps = k;
    if (converged) *converged = a.done;
    State st;
    CU(cudaMemcpy(&st, a.d_state, sizeof st, cudaMemcpyDeviceToHost));
    if (st.capped || a.hc.capped) return fail(RAD_ERR_WALK, "a visibility walk reached walk_cap");
    return RAD_OK;
}

}  // namespace

struct rad_adapt {
    int precision = 32;
    AdaptImpl<float>* a32 = nullptr;
    AdaptImpl<double>* a64 = nullptr;
    ~rad_adapt() { delete a32; delete a64; }
};

extern "C" {

int rad_adapt_create(rad_scene* s, const rad_octree* t, const rad_options* o, int32_t device, rad_adapt** out) {
    if (!s || !t || !o || !out) return fail(RAD_ERR_ARG, "rad_adapt_create: null argument");
    if (s->precision != t->precision) return fail(RAD_ERR_ARG, "scene and octree precision differ");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RAD_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(RAD_ERR_ARG, "device index out of range");
    rad_adapt* h = new rad_adapt();
    h->precision = s->precision;
    int rc;
    if (s->precision == 32) {
        h->a32 = new AdaptImpl<float>();
        rc = adapt_create(s->s32, t->o32, *o, device, *h->a32);
    } else {
        h->a64 = new AdaptImpl<double>();
        rc = adapt_create(s->s64, t->o64, *o, device, *h->a64);
    }
    if (rc) { delete h; return rc; }
    *out = h;
    return RAD_OK;
}

int rad_adapt_run(rad_adapt* h, int64_t max_steps, int64_t* steps_done, int32_t* converged) {
    if (!h) return fail(RAD_ERR_ARG, "rad_adapt_run: null handle");
    long long sd = 0;
    int cv = 0;
    int rc = h->a32 ? adapt_run(*h->a32, max_steps, &sd, &cv) : adapt_run(*h->a64, max_steps, &sd, &cv);
    if (steps_done) *steps_done = sd;
    if (converged) *converged = cv;
    return rc;
}

int rad_adapt_trace(const rad_adapt* h, int32_t* out, int64_t cap, int64_t* n) {
    if (!h) return fail(RAD_ERR_ARG, "rad_adapt_trace: null handle");
    const std::vector<int32_t>& tr = h->a32 ? h->a32->trace : h->a64->trace;
    if (n) *n = (int64_t)tr.size();
    if (out && cap > 0) std::memcpy(out, tr.data(), (size_t)std::min<int64_t>(cap, (int64_t)tr.size()) * 4);
    return RAD_OK;
}

int rad_adapt_stats(const rad_adapt* h, rad_stats* st, int64_t* host_points, int64_t* splits, int64_t* samples) {
    if (!h || !st) return fail(RAD_ERR_ARG, "rad_adapt_stats: null argument");
    auto go = [&](auto& a) -> int {
        State ds;
        CU(cudaSetDevice(a.device));
        CU(cudaMemcpy(&ds, a.d_state, sizeof ds, cudaMemcpyDeviceToHost));
        std::memset(st, 0, sizeof *st);
        st->steps = a.steps;
        st->shots = a.steps;
        st->rays = (int64_t)(ds.rays + a.hc.rays);
        st->walk_cap_hits = (int64_t)(ds.capped + a.hc.capped);
        st->walk_loops = (int64_t)(ds.loops + a.hc.loops);
        st->converged = a.done;
        st->n_slots = a.sc->trinum;
        st->device_bytes = (int64_t)a.bytes;
        if (host_points) *host_points = a.host_points;
        if (splits) *splits = a.splits;
        if (samples) *samples = a.samples;
        return RAD_OK;
    };
    return h->a32 ? go(*h->a32) : go(*h->a64);
}

int rad_adapt_set_speculation(rad_adapt* h, int32_t wait) {
    if (!h) return fail(RAD_ERR_ARG, "rad_adapt_set_speculation: null handle");
    if (wait != 0 && wait != 1) return fail(RAD_ERR_ARG, "rad_adapt_set_speculation: wait is 0 or 1");
    if (h->a32) h->a32->spec_wait_mode = wait;
    else h->a64->spec_wait_mode = wait;
    return RAD_OK;
}

int rad_adapt_device_stats(const rad_adapt* h, int64_t* device_points, int64_t* speculations,
                           int64_t* split_candidates) {
    if (!h) return fail(RAD_ERR_ARG, "rad_adapt_device_stats: null handle");
    auto go = [&](auto& a) {
        if (device_points) *device_points = a.dev_samples;
        if (speculations) *speculations = a.spec_launches;
        if (split_candidates) *split_candidates = a.split_candidates;
        return RAD_OK;
    };
    return h->a32 ? go(*h->a32) : go(*h->a64);
}

void rad_adapt_destroy(rad_adapt* h) { delete h; }

}  // extern "C"
