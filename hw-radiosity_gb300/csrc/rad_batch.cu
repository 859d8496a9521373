// Batched form: many independent scenes shot together, one persistent launch
// per batch iteration.
//
// Every scene keeps its own slots, octree, selection and convergence; in one
// iteration every scene that has not converged does one shooter step of the
// reference's loop (parallelRadiosity, src/rad.cpp:406-451) with its own
// -parallel_src.  All scenes' records are concatenated in HBM; a descriptor
// per scene points into them.
//
// Two pipelines, chosen per batch:
//
//   FP32, one shooter per step (fused, one kernel per iteration)
//     k_batch_shoot  persistent: warps take (scene, 10-slot group) items from
//                    one queue over the groups of the running scenes, run the
//                    single-scene kernel's per-group body on that scene, and
//                    fold the group's selection key into the scene's maximum
//                    with one 64-bit atomicMax ((ordered FP32 key << 32) |
//                    slot, so ties go to the higher slot as in listCanditate).
//                    The grid's last CTA then turns every scene's maximum into
//                    its next shooter record, or marks the scene converged.
//
//   FP64, or several shooters per step (two kernels per iteration)
//     k_batch_select one CTA per scene: listCanditate's top n over the scene's
//                    keys (the single-scene solver's k_setup code) and the
//                    shooter records.
//     k_batch_shoot  as above, without the key maximum.
//
// The queue lists only groups of running scenes; the host rebuilds it between
// graph chunks when scenes finish.  A scene's result is bit-identical to the
// single-scene solver's (same per-group code, same order of every sum).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "capi_internal.h"
#include "prep_workspace.h"
#include "rad_kernels.cuh"

namespace radgb {
namespace dev {

template <typename T>
struct SceneDesc {
    Slots<T> S;
    Grid<T> G;
    T conv;
    int trace_off;     // first trace entry of the scene (P entries per step)
    int trace_cap;     // steps kept in the trace
    int n_groups;
    int sh_off;        // first shooter record of the scene (P records)
};

struct SceneState {
    unsigned long long best;   // fused form: packed selection maximum of the last iteration
    int done;
    int nsh;                   // shooters of the pending step
    long long steps;           // steps selected; the fused form selects one iteration ahead
};

struct BatchCtl {
    int work;                  // next queue item
    int n_items;               // queue length (groups of running scenes)
    int ctas_done;             // fused form: CTAs of the current iteration that have finished
    int n_scenes;
    unsigned long long rays, rays_ref, cells, tris, se, prec, capped, loops;
};

template <bool COUNT>
__device__ __forceinline__ void flush_batch(BatchCtl* bc, Cnt& c, int lane) {
    unsigned v[8] = {c.rays, c.rays_ref, c.cells, c.tris, c.se, c.prec, c.capped, c.loops};
    unsigned long long* dst[8] = {&bc->rays, &bc->rays_ref, &bc->cells, &bc->tris, &bc->se, &bc->prec, &bc->capped,
                                  &bc->loops};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        if (!COUNT && q != 0 && q != 6 && q != 7) continue;
        unsigned s = __reduce_add_sync(kFull, v[q]);
        if (lane == 0 && s) atomicAdd(dst[q], (unsigned long long)s);
    }
}

// The fused form's selection for scene s: the maximum packed by the groups of
// the iteration that just ended becomes the next shooter (listCanditate with
// one shooter, rad.cpp:387-404), or the scene has converged.
__device__ void select_fused(const SceneDesc<float>& d, SceneState& st, Shooter<float>* sh, int* trace) {
    if (st.done) { st.nsh = 0; return; }
    // read and reset at L2: this SM's L1 may hold the record's line from the
    // items' reads of `done` earlier in the launch, before the groups' atomicMax
    const unsigned long long best = atomicExch(&st.best, 0ull);
    if (best == 0) {           // no candidate above the scene's converge limit
        st.done = 1;
        st.nsh = 0;
        return;
    }
    const int slot = (int)(best & 0xffffffffull);
    build_shooter(d.S, slot, sh[d.sh_off]);
    st.nsh = 1;
    if (st.steps < d.trace_cap) trace[d.trace_off + st.steps] = slot;
    st.steps += 1;
}

// Scenes keep every SM busy for the whole launch, so this kernel is bound by
// throughput, not by its slowest group: two forms, 4 CTAs per SM (64
// registers) and 3 (80 registers), chosen by rad_batch_autotune.
template <typename T, bool COUNT, bool ONE, bool FUSED, int MINB>
__global__ void __launch_bounds__(kShootThreads, MINB)
k_batch_shoot(const SceneDesc<T>* __restrict__ desc, SceneState* ss, Shooter<T>* sh, const int2* __restrict__ items,
              BatchCtl* bc, int* trace) {
    static_assert(!FUSED || (ONE && std::is_same<T, float>::value), "the fused form is FP32, one shooter per step");
    __shared__ int last;
    const int lane = threadIdx.x & 31;
    const int n_items = bc->n_items;
    Cnt c = {0, 0, 0, 0, 0, 0, 0, 0};
    for (;;) {
        int g = 0;
        if (lane == 0) g = atomicAdd(&bc->work, 1);
        g = __shfl_sync(kFull, g, 0);
        if (g >= n_items) break;
        const int2 it = items[g];
        const int s = it.x;
        if (ss[s].done) continue;                    // finished earlier in this chunk
        const int nsh = ss[s].nsh;
        // read through the reference: the walk loads the scene's grid fields
        // when it needs them instead of holding the whole descriptor in registers
        const SceneDesc<T>& d = desc[s];
        unsigned long long kk = 0;
        int ks = -1;
        shoot_group<T, COUNT, ONE, true>(d.S, d.G, sh + d.sh_off, nsh, it.y, lane, d.conv, kk, ks, c);
        if (FUSED) {
            warp_max(kk, ks);
            if (lane == 0 && ks >= 0) atomicMax(&ss[s].best, (kk << 32) | (unsigned long long)(unsigned)ks);
        }
    }
    flush_batch<COUNT>(bc, c, lane);
    if constexpr (FUSED) {
        // the grid's last CTA selects every scene's next shooter
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            last = atomicAdd(&bc->ctas_done, 1) == (int)gridDim.x - 1;
        }
        __syncthreads();
        if (!last) return;
        __threadfence();
        const int n_scenes = bc->n_scenes;
        for (int s = threadIdx.x; s < n_scenes; s += blockDim.x) select_fused(desc[s], ss[s], sh, trace);
        if (threadIdx.x == 0) {
            bc->work = 0;
            bc->ctas_done = 0;
        }
    }
}

// FP64 / several shooters per step: one CTA per scene selects its shooters
constexpr int kSelectThreads = 512;

template <typename T>
__global__ void __launch_bounds__(kSelectThreads)
k_batch_select(const SceneDesc<T>* __restrict__ desc, SceneState* ss, Shooter<T>* sh, int P, BatchCtl* bc,
               int* trace) {
    __shared__ int chosen[kMaxShooters];
    if (blockIdx.x == 0 && threadIdx.x == 0) bc->work = 0;
    const int s = blockIdx.x;
    SceneState& st = ss[s];
    if (st.done) return;
    const SceneDesc<T>& d = desc[s];
    const int n = cta_top_shooters(d.S, d.conv, P, chosen);
    if (n == 0) {
        if (threadIdx.x == 0) { st.done = 1; st.nsh = 0; }
        return;
    }
    if ((int)threadIdx.x < n) build_shooter(d.S, chosen[threadIdx.x], sh[d.sh_off + threadIdx.x]);
    if (threadIdx.x == 0) {
        if (st.steps < d.trace_cap) {
            int* tr = trace + d.trace_off + st.steps * (long long)P;
            for (int j = 0; j < P; j++) tr[j] = j < n ? chosen[j] : -1;
        }
        st.nsh = n;
        st.steps += 1;
    }
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

struct BatchBase {
    virtual ~BatchBase() {}
};

struct SceneOff {
    long long slot = 0, ent = 0, cell = 0, thr = 0, lbox = 0, lrange = 0, trec = 0;
    int n = 0;
};

template <typename T>
struct BatchImpl : BatchBase {
    using Real = T;
    int device = 0;
    cudaStream_t stream = nullptr;
    int n_scenes = 0;
    int P = 1;
    bool fused = true;
    bool counting = false;
    int form = 1;                        // 1: 4 CTAs per SM, 2: 3 CTAs per SM
    int n_cta[3] = {0, 1, 1};
    std::vector<void*> allocs;
    size_t bytes = 0;
    long long h2d_bytes = 0;
    std::vector<SceneDesc<T>> desc;      // host copy (device pointers inside)
    std::vector<SceneOff> off;
    SceneDesc<T>* d_desc = nullptr;
    SceneState* d_ss = nullptr;
    Shooter<T>* d_sh = nullptr;
    int2* d_items = nullptr;
    BatchCtl* d_ctl = nullptr;
    int* d_trace = nullptr;
    int trace_cap = 0;
    std::vector<int> done;               // host mirror, per scene
    std::vector<long long> steps;        // steps shot, per scene
    cudaGraphExec_t graphs[3][2][33] = {};   // [form][counting][iterations per launch]
    bool graph_seen[3][2][33] = {};          // a chunk of that shape has run once
    cudaEvent_t ev[2] = {nullptr, nullptr};

    ~BatchImpl() override {
        for (auto& plane : graphs)
            for (auto& row : plane)
                for (auto& g : row)
                    if (g) cudaGraphExecDestroy(g);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (void* p : allocs) cudaFree(p);
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
    template <typename V, typename A>
    int put(V** dst, const std::vector<V, A>& src) {
        int r = alloc(dst, src.size());
        if (r) return r;
        if (!src.empty()) {
            CU(cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(V), cudaMemcpyHostToDevice, stream));
            h2d_bytes += (long long)(src.size() * sizeof(V));
        }
        return RAD_OK;
    }
};

// the shooting kernel of the current form (fused: FP32, one shooter per step)
template <typename T, bool COUNT, bool ONE, bool FUSED>
int launch_shoot_form(BatchImpl<T>& b, cudaStream_t s) {
    if (b.form == 2)
        k_batch_shoot<T, COUNT, ONE, FUSED, 3><<<b.n_cta[2], kShootThreads, 0, s>>>(b.d_desc, b.d_ss, b.d_sh, b.d_items,
                                                                                  b.d_ctl, b.d_trace);
    else
        k_batch_shoot<T, COUNT, ONE, FUSED, 4><<<b.n_cta[1], kShootThreads, 0, s>>>(b.d_desc, b.d_ss, b.d_sh, b.d_items,
                                                                                  b.d_ctl, b.d_trace);
    CU(cudaGetLastError());
    return RAD_OK;
}

template <typename T>
int launch_iter(BatchImpl<T>& b, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        if (b.fused)
            return b.counting ? launch_shoot_form<T, true, true, true>(b, s) : launch_shoot_form<T, false, true, true>(b, s);
    }
    k_batch_select<T><<<b.n_scenes, kSelectThreads, 0, s>>>(b.d_desc, b.d_ss, b.d_sh, b.P, b.d_ctl, b.d_trace);
    CU(cudaGetLastError());
    if (b.P == 1)
        return b.counting ? launch_shoot_form<T, true, true, false>(b, s) : launch_shoot_form<T, false, true, false>(b, s);
    return b.counting ? launch_shoot_form<T, true, false, false>(b, s) : launch_shoot_form<T, false, false, false>(b, s);
}

// The graph of a chunk of `iters` iterations, built the second time a chunk
// of that shape runs; null the first time, when the caller launches the
// iterations one by one (they overlap the device's work; a capture would
// delay it).
template <typename T>
int graph_for(BatchImpl<T>& b, int iters, cudaGraphExec_t* out) {
    cudaGraphExec_t& slot = b.graphs[b.form][b.counting ? 1 : 0][iters];
    bool& seen = b.graph_seen[b.form][b.counting ? 1 : 0][iters];
    if (!slot && !seen) {
        seen = true;
        *out = nullptr;
        return RAD_OK;
    }
    if (!slot) {
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < iters; k++) {
            int rc = launch_iter(b, b.stream);
            if (rc) { cudaStreamEndCapture(b.stream, &g); return rc; }
        }
        CU(cudaStreamEndCapture(b.stream, &g));
        cudaError_t e = cudaGraphInstantiate(&slot, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { slot = nullptr; return fail(RAD_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)); }
    }
    *out = slot;
    return RAD_OK;
}

// queue of (scene, group) items over the scenes still running, the scenes
// with the most groups first: an iteration ends with its last item, and the
// small scenes' short items fill the end (119.5k against 118.0k shots/s on
// the 256-room batch in scene order).  Results do not depend on the order.
template <typename T>
int rebuild_items(BatchImpl<T>& b) {
    std::vector<int2> items;
    std::vector<int> ord(b.n_scenes);
    for (int s = 0; s < b.n_scenes; s++) ord[s] = s;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return b.desc[x].n_groups > b.desc[y].n_groups; });
    for (int s : ord) {
        if (b.done[s]) continue;
        for (int g = 0; g < b.desc[s].n_groups; g++) items.push_back(make_int2(s, g));
    }
    const int n = (int)items.size();
    if (n) CU(cudaMemcpyAsync(b.d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, b.stream));
    CU(cudaMemcpyAsync(&b.d_ctl->n_items, &n, sizeof n, cudaMemcpyHostToDevice, b.stream));
    CU(cudaStreamSynchronize(b.stream));
    return RAD_OK;
}

template <typename T>
int refresh(BatchImpl<T>& b, bool* changed) {
    std::vector<SceneState> ss(b.n_scenes);
    CU(cudaMemcpyAsync(ss.data(), b.d_ss, ss.size() * sizeof(SceneState), cudaMemcpyDeviceToHost, b.stream));
    CU(cudaStreamSynchronize(b.stream));
    *changed = false;
    for (int s = 0; s < b.n_scenes; s++) {
        if (ss[s].done != b.done[s]) *changed = true;
        b.done[s] = ss[s].done;
        // the fused form has already selected the next step's shooter
        b.steps[s] = ss[s].steps - (b.fused ? ss[s].nsh : 0);
    }
    return RAD_OK;
}

constexpr int kBatchChunk = 32;

template <typename T>
int run(BatchImpl<T>& b, long long max_iters, long long* iters_done, int* n_active, double* ms) {
    CU(cudaSetDevice(b.device));
    if (ms) *ms = 0;
    long long done_it = 0;
    int rc;
    auto active = [&]() { int a = 0; for (int d : b.done) a += !d; return a; };
    // iterations in which some scene was running: a running scene has shot in
    // every one of them, a converged one in all but its last
    auto effective = [&]() {
        long long m = 0;
        for (int s = 0; s < b.n_scenes; s++) m = std::max(m, b.steps[s] + b.done[s]);
        return m;
    };
    const long long eff0 = effective();
    if (max_iters > 0 && ms && !b.ev[0])
        for (auto& e : b.ev) CU(cudaEventCreate(&e));
    while (done_it < max_iters && active() > 0) {
        const int chunk = (int)std::min<long long>(kBatchChunk, max_iters - done_it);
        cudaGraphExec_t g;
        if ((rc = graph_for(b, chunk, &g))) return rc;
        if (ms) CU(cudaEventRecord(b.ev[0], b.stream));
        if (g) {
            CU(cudaGraphLaunch(g, b.stream));
        } else {
            for (int k = 0; k < chunk; k++)
                if ((rc = launch_iter(b, b.stream))) return rc;
        }
        if (ms) CU(cudaEventRecord(b.ev[1], b.stream));
        bool changed = false;
        if ((rc = refresh(b, &changed))) return rc;
        if (ms) {
            float t = 0;
            CU(cudaEventElapsedTime(&t, b.ev[0], b.ev[1]));
            *ms += t;
        }
        done_it += chunk;
        if (changed && (rc = rebuild_items(b))) return rc;
    }
    if (iters_done) *iters_done = effective() - eff0;
    if (n_active) *n_active = active();
    BatchCtl ctl;
    CU(cudaMemcpy(&ctl, b.d_ctl, sizeof ctl, cudaMemcpyDeviceToHost));
    if (ctl.capped) return fail(RAD_ERR_WALK, "a visibility walk reached walk_cap");
    return RAD_OK;
}

// The batch's host staging: per-slot records, the thresholds, and the octree
// in the form the device expands (a leaf per cell, leaf boxes and ranges, the
// triangle of each list entry, one five-record group per triangle a list
// names), every scene at its own offsets.  The vectors are sized once with
// zero pages that nothing writes until a scene's thread packs its range, so
// the page faults of the first touch are spread over the packing threads.
template <typename U>
using StageVec = std::vector<U, ZeroPages<U>>;

template <typename T>
struct Staging {
    StageVec<Q4<T>> vtx, nrm, ctr, frgb, acc, db, trec;
    StageVec<T> thr, lbox;
    StageVec<int32_t> cleaf, lrange, etri;
};

// the triangles scene s's lists name: 0 .. n_tri-1 (-1: a list names a triangle beyond the scene)
template <typename T>
int list_triangles(const Scene<T>& s, const Octree<T>& o) {
    int n_tri = 0;
    for (int32_t id : o.entry_tri) n_tri = std::max(n_tri, id + 1);
    return n_tri > s.trinum ? -1 : n_tri;
}

// pack scene s into its ranges of the staging (offsets already set in off)
template <typename T>
void stage_scene(const Scene<T>& s, const Octree<T>& o, int n_tri, Staging<T>& P, const SceneOff& off) {
    const size_t n = (size_t)s.trinum, b3 = (size_t)off.slot * 3, b1 = (size_t)off.slot;
    for (size_t i = 0; i < n; i++) {
        const Slot<T>& t = s.slots[i];
        for (int v = 0; v < 3; v++) {
            P.vtx[b3 + 3 * i + v] = {t.p[v][0], t.p[v][1], t.p[v][2], 0};
            P.acc[b3 + 3 * i + v] = {t.accB[v][0], t.accB[v][1], t.accB[v][2], 0};
        }
        const T nl = (T)std::sqrt(t.n[0] * t.n[0] + t.n[1] * t.n[1] + t.n[2] * t.n[2]);
        P.nrm[b1 + i] = {t.n[0], t.n[1], t.n[2], nl};
        P.ctr[b1 + i] = {t.c[0], t.c[1], t.c[2], t.area};
        P.frgb[b1 + i] = {(T)t.Frgb[0], (T)t.Frgb[1], (T)t.Frgb[2], (T)t.parent};
        P.db[b1 + i] = {t.deltaB[0], t.deltaB[1], t.deltaB[2], 0};
    }
    // the walk's triangle records (as RayHitted reads TriStore at shooting time)
    const size_t bt = (size_t)off.trec * 5;
    for (int id = 0; id < n_tri; id++) {
        const Slot<T>& t = s.slots[id];
        Q4<T>* r = &P.trec[bt + 5 * (size_t)id];
        r[0] = {t.n[0], t.n[1], t.n[2], pack_int<T>(id)};
        r[1] = {t.c[0], t.c[1], t.c[2], 0};
        for (int e = 0; e < 3; e++) r[2 + e] = {t.se[e][0], t.se[e][1], t.se[e][2], t.se[e][3]};
    }
    // indices stay scene-local: the expansion kernels run per scene on offset pointers
    std::copy(o.cell_leaf.begin(), o.cell_leaf.end(), P.cleaf.begin() + off.cell);
    std::copy(o.leaf_box.begin(), o.leaf_box.end(), P.lbox.begin() + off.lbox * 8);
    std::copy(o.leaf_range.begin(), o.leaf_range.end(), P.lrange.begin() + off.lrange * 2);
    std::copy(o.entry_tri.begin(), o.entry_tri.end(), P.etri.begin() + off.ent);
    std::copy(o.thr.begin(), o.thr.end(), P.thr.begin() + off.thr);
}

template <typename T>
const Scene<T>& scene_of(const rad_scene* s);
template <>
const Scene<float>& scene_of<float>(const rad_scene* s) { return s->s32; }
template <>
const Scene<double>& scene_of<double>(const rad_scene* s) { return s->s64; }
template <typename T>
const Octree<T>& tree_of(const rad_octree* t);
template <>
const Octree<float>& tree_of<float>(const rad_octree* t) { return t->o32; }
template <>
const Octree<double>& tree_of<double>(const rad_octree* t) { return t->o64; }

template <typename T>
int batch_create(const rad_scene* const* scenes, const rad_octree* const* trees, const rad_options* opts, int n_scenes,
                 int trace_cap, int device, BatchImpl<T>& b) {
    b.device = device;
    b.n_scenes = n_scenes;
    b.P = std::max(1, opts[0].parallel_src);
    for (int s = 0; s < n_scenes; s++)
        if (std::max(1, opts[s].parallel_src) != b.P)
            return fail(RAD_ERR_ARG, "rad_batch_create: every scene of a batch needs the same -parallel_src");
    if (b.P > kMaxShooters) return fail(RAD_ERR_CAPACITY, "-parallel_src above 256 is not supported");
    b.fused = std::is_same<T, float>::value && b.P == 1;
    b.trace_cap = trace_cap;
    CU(cudaSetDevice(device));
    CU(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
    // offsets of every scene in the staging, then the packing on the -jobs threads
    const int jobs = std::max(1, std::min(opts[0].jobs, 16));
    std::vector<int> n_tri(n_scenes);
    for_each_item(n_scenes, jobs, [&](int s) { n_tri[s] = list_triangles(scene_of<T>(scenes[s]), tree_of<T>(trees[s])); });
    b.off.resize(n_scenes);
    long long total_groups = 0;
    SceneOff end;
    for (int s = 0; s < n_scenes; s++) {
        if (n_tri[s] < 0) return fail(RAD_ERR_ARG, "octree names a triangle beyond the scene");
        const Scene<T>& sc = scene_of<T>(scenes[s]);
        const Octree<T>& tr = tree_of<T>(trees[s]);
        SceneOff& o = b.off[s];
        o = end;
        o.n = sc.trinum;
        end.slot += sc.trinum;
        end.trec += n_tri[s];
        end.cell += (long long)tr.cell_leaf.size();
        end.lbox += (long long)tr.leaf_box.size() / 8;
        end.lrange += (long long)tr.leaf_range.size() / 2;
        end.ent += (long long)tr.entry_tri.size();
        end.thr += (long long)tr.thr.size();
        total_groups += (o.n + kSlotsPerWarp - 1) / kSlotsPerWarp;
    }
    if (total_groups > 0x7fffffffLL || (long long)trace_cap * n_scenes * b.P > 0x7fffffffLL || end.slot > 0x7fffffffLL)
        return fail(RAD_ERR_CAPACITY, "batch too large");
    Staging<T> P;
    P.vtx.resize((size_t)end.slot * 3); P.acc.resize((size_t)end.slot * 3);
    P.nrm.resize((size_t)end.slot); P.ctr.resize((size_t)end.slot); P.frgb.resize((size_t)end.slot);
    P.db.resize((size_t)end.slot); P.trec.resize((size_t)end.trec * 5);
    P.cleaf.resize((size_t)end.cell); P.lbox.resize((size_t)end.lbox * 8); P.lrange.resize((size_t)end.lrange * 2);
    P.etri.resize((size_t)end.ent); P.thr.resize((size_t)end.thr);
    for_each_item(n_scenes, jobs, [&](int s) {
        stage_scene(scene_of<T>(scenes[s]), tree_of<T>(trees[s]), n_tri[s], P, b.off[s]);
    });
    int rc;
    Q4<T> *d_vtx, *d_nrm, *d_ctr, *d_frgb, *d_acc, *d_db, *d_trec, *d_ent;
    CellRec<T>* d_cell;
    T *d_thr, *d_lbox;
    int32_t *d_cleaf, *d_lrange, *d_etri;
    if ((rc = b.put(&d_vtx, P.vtx)) || (rc = b.put(&d_nrm, P.nrm)) || (rc = b.put(&d_ctr, P.ctr)) ||
        (rc = b.put(&d_frgb, P.frgb)) || (rc = b.put(&d_acc, P.acc)) || (rc = b.put(&d_db, P.db)) ||
        (rc = b.put(&d_thr, P.thr)) || (rc = b.put(&d_trec, P.trec)) || (rc = b.put(&d_lbox, P.lbox)) ||
        (rc = b.put(&d_lrange, P.lrange)) || (rc = b.put(&d_cleaf, P.cleaf)) || (rc = b.put(&d_etri, P.etri)) ||
        (rc = b.alloc(&d_cell, P.cleaf.size())) || (rc = b.alloc(&d_ent, P.etri.size() * 5)))
        return rc;
    b.desc.resize(n_scenes);
    for (int s = 0; s < n_scenes; s++) {
        const SceneOff& o = b.off[s];
        const Octree<T>& tr = tree_of<T>(trees[s]);
        const long long n_cell = (long long)tr.cell_leaf.size(), n_ent = (long long)tr.entry_tri.size();
        // expand this scene's cells and list records on the device
        if (n_cell > 0)
            k_expand_cells<T><<<(int)std::min<long long>((n_cell + 255) / 256, 1024), 256, 0, b.stream>>>(
                d_cleaf + o.cell, d_lbox + o.lbox * 8, d_lrange + o.lrange * 2, n_cell, d_cell + o.cell);
        if (n_ent > 0)
            k_gather_entries<T><<<(int)std::min<long long>((n_ent * 5 + 255) / 256, 1024), 256, 0, b.stream>>>(
                d_etri + o.ent, d_trec + o.trec * 5, n_ent, d_ent + o.ent * 5);
        CU(cudaGetLastError());
        SceneDesc<T>& d = b.desc[s];
        d.S = Slots<T>{o.n, d_vtx + o.slot * 3, d_nrm + o.slot, d_ctr + o.slot, d_frgb + o.slot,
                       d_acc + o.slot * 3, d_db + o.slot};
        d.G = grid_params(tr, opts[s].walk_cap);
        d.G.thr = d_thr + o.thr;
        d.G.cell = d_cell + o.cell;
        d.G.entry = d_ent + o.ent * 5;
        d.conv = (T)opts[s].converge;
        d.trace_off = s * trace_cap * b.P;
        d.trace_cap = trace_cap;
        d.n_groups = (o.n + kSlotsPerWarp - 1) / kSlotsPerWarp;
        d.sh_off = s * b.P;
    }
    BatchCtl ctl{};
    ctl.n_scenes = n_scenes;
    if ((rc = b.put(&b.d_desc, b.desc)) || (rc = b.alloc(&b.d_ss, (size_t)n_scenes)) ||
        (rc = b.alloc(&b.d_sh, (size_t)n_scenes * b.P)) ||
        (rc = b.alloc(&b.d_items, (size_t)std::max<long long>(total_groups, 1))) || (rc = b.alloc(&b.d_ctl, 1)) ||
        (rc = b.alloc(&b.d_trace, (size_t)trace_cap * n_scenes * b.P)))
        return rc;
    CU(cudaMemsetAsync(b.d_ss, 0, sizeof(SceneState) * n_scenes, b.stream));
    CU(cudaMemsetAsync(b.d_sh, 0, sizeof(Shooter<T>) * n_scenes * b.P, b.stream));
    CU(cudaMemcpyAsync(b.d_ctl, &ctl, sizeof ctl, cudaMemcpyHostToDevice, b.stream));
    int sms = 0, per4 = 0, per3 = 0;
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per4, k_batch_shoot<T, false, true, false, 4>, kShootThreads, 0));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per3, k_batch_shoot<T, false, true, false, 3>, kShootThreads, 0));
    const long long want = (total_groups + kShootThreads / 32 - 1) / (kShootThreads / 32);
    b.n_cta[1] = (int)std::max<long long>(1, std::min<long long>(want, std::max(1, sms * per4)));
    b.n_cta[2] = (int)std::max<long long>(1, std::min<long long>(want, std::max(1, sms * per3)));
    // FP64 spills at 64 registers: it takes the 3-CTA form unless tuned otherwise
    b.form = std::is_same<T, float>::value ? 1 : 2;
    b.done.assign(n_scenes, 0);
    b.steps.assign(n_scenes, 0);
    if ((rc = rebuild_items(b))) return rc;
    if constexpr (std::is_same<T, float>::value) {
        if (b.fused) {
            // the initial selection keys: every group with no shooter, then the
            // last CTA selects the first shooters
            if ((rc = launch_shoot_form<float, false, true, true>(b, b.stream))) return rc;
            CU(cudaStreamSynchronize(b.stream));
            bool changed = false;
            if ((rc = refresh(b, &changed))) return rc;
            if (changed && (rc = rebuild_items(b))) return rc;
        }
    }
    CU(cudaStreamSynchronize(b.stream));
    return RAD_OK;
}

template <typename T>
int batch_download(BatchImpl<T>& b, int scene, Scene<T>& s) {
    const SceneOff& o = b.off[scene];
    if (o.n != s.trinum) return fail(RAD_ERR_ARG, "scene slot count differs from the batch copy");
    std::vector<Q4<T>> acc((size_t)o.n * 3), db(o.n);
    CU(cudaSetDevice(b.device));
    if (o.n) {
        CU(cudaMemcpyAsync(acc.data(), b.desc[scene].S.accB, acc.size() * sizeof(Q4<T>), cudaMemcpyDeviceToHost, b.stream));
        CU(cudaMemcpyAsync(db.data(), b.desc[scene].S.deltaB, db.size() * sizeof(Q4<T>), cudaMemcpyDeviceToHost, b.stream));
    }
    CU(cudaStreamSynchronize(b.stream));
    for (int i = 0; i < o.n; i++) {
        Slot<T>& t = s.slots[i];
        for (int v = 0; v < 3; v++) {
            t.accB[v][0] = acc[i * 3 + v].x; t.accB[v][1] = acc[i * 3 + v].y; t.accB[v][2] = acc[i * 3 + v].z;
        }
        t.deltaB[0] = db[i].x; t.deltaB[1] = db[i].y; t.deltaB[2] = db[i].z;
    }
    return RAD_OK;
}

template <typename T>
int batch_trace(const BatchImpl<T>& b, int scene, int32_t* out, int64_t cap, int64_t* n) {
    const long long have = std::min<long long>(b.steps[scene], b.desc[scene].trace_cap) * b.P;
    if (n) *n = have;
    if (!out || cap <= 0) return RAD_OK;
    CU(cudaSetDevice(b.device));
    CU(cudaMemcpy(out, b.d_trace + b.desc[scene].trace_off, (size_t)std::min<long long>(have, cap) * 4,
                  cudaMemcpyDeviceToHost));
    return RAD_OK;
}

template <typename T>
int batch_stats(const BatchImpl<T>& b, rad_stats* st) {
    BatchCtl ctl;
    CU(cudaSetDevice(b.device));
    CU(cudaMemcpy(&ctl, b.d_ctl, sizeof ctl, cudaMemcpyDeviceToHost));
    std::memset(st, 0, sizeof *st);
    for (int s = 0; s < b.n_scenes; s++) {
        st->steps += b.steps[s];
        st->n_slots += b.off[s].n;
    }
    if (b.P == 1) {
        st->shots = st->steps;
    } else {
        for (int s = 0; s < b.n_scenes; s++) {
            const long long have = std::min<long long>(b.steps[s], b.desc[s].trace_cap) * b.P;
            std::vector<int32_t> tr((size_t)have);
            if (have) CU(cudaMemcpy(tr.data(), b.d_trace + b.desc[s].trace_off, (size_t)have * 4, cudaMemcpyDeviceToHost));
            for (int32_t x : tr) st->shots += x >= 0;
        }
    }
    st->rays = (int64_t)ctl.rays;
    st->rays_ref = (int64_t)ctl.rays_ref;
    st->cells = (int64_t)ctl.cells;
    st->tri_tests = (int64_t)ctl.tris;
    st->se_tests = (int64_t)ctl.se;
    st->prec_steps = (int64_t)ctl.prec;
    st->walk_cap_hits = (int64_t)ctl.capped;
    st->walk_loops = (int64_t)ctl.loops;
    int active = 0;
    for (int d : b.done) active += !d;
    st->converged = active == 0;
    st->device_bytes = (int64_t)b.bytes;
    st->h2d_bytes = (int64_t)b.h2d_bytes;
    return RAD_OK;
}

// time `iters` iterations in each form, alternating, and keep the faster
template <typename T>
int batch_autotune(BatchImpl<T>& b, int iters_per_trial, int rounds, int* chosen) {
    double ms[3] = {0, 0, 0};
    long long its[3] = {0, 0, 0};
    for (int r = 0; r <= rounds; r++) {
        for (int k = 0; k < 2; k++) {
            const int form = ((r + k) & 1) ? 2 : 1;
            b.form = form;
            long long it = 0;
            int na = 0;
            double t = 0;
            int rc = run(b, r == 0 ? 1 : iters_per_trial, &it, &na, r == 0 ? nullptr : &t);
            if (rc) return rc;
            if (r > 0) { ms[form] += t; its[form] += it; }
            if (na == 0) break;
        }
    }
    int best = b.form;
    if (its[1] > 0 && its[2] > 0) best = ms[2] / (double)its[2] < ms[1] / (double)its[1] ? 2 : 1;
    b.form = best;
    if (chosen) *chosen = best;
    return RAD_OK;
}

}  // namespace

struct rad_batch {
    int precision = 32;
    BatchImpl<float>* b32 = nullptr;
    BatchImpl<double>* b64 = nullptr;
    ~rad_batch() { delete b32; delete b64; }
};

#define BATCH_GO(h, call) ((h)->b32 ? call(*(h)->b32) : call(*(h)->b64))

extern "C" {

int rad_batch_create(const rad_scene* const* scenes, const rad_octree* const* trees, const rad_options* opts,
                     int32_t n_scenes, int32_t trace_cap, int32_t device, rad_batch** out) {
    if (!scenes || !trees || !opts || !out || n_scenes <= 0) return fail(RAD_ERR_ARG, "rad_batch_create: bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RAD_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(RAD_ERR_ARG, "device index out of range");
    if (!scenes[0]) return fail(RAD_ERR_ARG, "null scene or octree");
    const int prec = scenes[0]->precision;
    for (int s = 0; s < n_scenes; s++) {
        if (!scenes[s] || !trees[s]) return fail(RAD_ERR_ARG, "null scene or octree");
        if (scenes[s]->precision != prec || trees[s]->precision != prec || opts[s].precision != prec)
            return fail(RAD_ERR_ARG, "rad_batch_create: scenes, octrees and options need one precision");
        if (!(prec == 32 ? thresholds_consistent(trees[s]->o32) : thresholds_consistent(trees[s]->o64)))
            return fail(RAD_ERR_ARG, "octree thresholds inconsistent");
    }
    if (trace_cap <= 0) trace_cap = 1 << 16;
    rad_batch* h = new rad_batch();
    h->precision = prec;
    int rc;
    if (prec == 32) {
        h->b32 = new BatchImpl<float>();
        rc = batch_create(scenes, trees, opts, n_scenes, trace_cap, device, *h->b32);
    } else {
        h->b64 = new BatchImpl<double>();
        rc = batch_create(scenes, trees, opts, n_scenes, trace_cap, device, *h->b64);
    }
    if (rc) { delete h; return rc; }
    *out = h;
    return RAD_OK;
}

int rad_batch_run(rad_batch* h, int64_t max_iters, int64_t* iters_done, int32_t* n_active) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_run: null handle");
    long long it = 0;
    int na = 0;
    auto go = [&](auto& b) { return run(b, max_iters, &it, &na, nullptr); };
    int rc = BATCH_GO(h, go);
    if (iters_done) *iters_done = it;
    if (n_active) *n_active = na;
    return rc;
}

int rad_batch_run_timed(rad_batch* h, int64_t max_iters, int64_t* iters_done, int32_t* n_active, double* device_ms) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_run_timed: null handle");
    long long it = 0;
    int na = 0;
    double ms = 0;
    auto go = [&](auto& b) { return run(b, max_iters, &it, &na, &ms); };
    int rc = BATCH_GO(h, go);
    if (iters_done) *iters_done = it;
    if (n_active) *n_active = na;
    if (device_ms) *device_ms = ms;
    return rc;
}

int rad_batch_scene_stats(const rad_batch* h, int32_t scene, int64_t* steps, int32_t* converged) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_scene_stats: null handle");
    auto go = [&](auto& b) -> int {
        if (scene < 0 || scene >= b.n_scenes) return fail(RAD_ERR_ARG, "rad_batch_scene_stats: bad argument");
        if (steps) *steps = b.steps[scene];
        if (converged) *converged = b.done[scene];
        return RAD_OK;
    };
    return BATCH_GO(h, go);
}

int rad_batch_download(rad_batch* h, int32_t scene, rad_scene* s) {
    if (!h || !s) return fail(RAD_ERR_ARG, "rad_batch_download: bad argument");
    if (s->precision != h->precision) return fail(RAD_ERR_ARG, "rad_batch_download: precision differs");
    auto go = [&](auto& b) -> int {
        if (scene < 0 || scene >= b.n_scenes) return fail(RAD_ERR_ARG, "rad_batch_download: bad argument");
        using TT = typename std::remove_reference<decltype(b)>::type::Real;
        if constexpr (std::is_same<TT, float>::value)
            return batch_download(b, scene, s->s32);
        else
            return batch_download(b, scene, s->s64);
    };
    return BATCH_GO(h, go);
}

int rad_batch_trace(const rad_batch* h, int32_t scene, int32_t* out, int64_t cap, int64_t* n) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_trace: null handle");
    auto go = [&](auto& b) -> int {
        if (scene < 0 || scene >= b.n_scenes) return fail(RAD_ERR_ARG, "rad_batch_trace: bad argument");
        return batch_trace(b, scene, out, cap, n);
    };
    return BATCH_GO(h, go);
}

int rad_batch_stats(const rad_batch* h, rad_stats* st) {
    if (!h || !st) return fail(RAD_ERR_ARG, "rad_batch_stats: null argument");
    auto go = [&](auto& b) { return batch_stats(b, st); };
    return BATCH_GO(h, go);
}

int rad_batch_set_counting(rad_batch* h, int32_t on) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_set_counting: null handle");
    if (h->b32) h->b32->counting = on != 0; else h->b64->counting = on != 0;
    return RAD_OK;
}

int rad_batch_set_form(rad_batch* h, int32_t form) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_set_form: null handle");
    if (form < 1 || form > 2) return fail(RAD_ERR_ARG, "rad_batch_set_form: form must be 1 or 2");
    if (h->b32) h->b32->form = form; else h->b64->form = form;
    return RAD_OK;
}

int rad_batch_form(const rad_batch* h) {
    if (!h) return 0;
    return h->b32 ? h->b32->form : h->b64->form;
}

int rad_batch_autotune(rad_batch* h, int32_t iters_per_trial, int32_t rounds, int32_t* chosen) {
    if (!h) return fail(RAD_ERR_ARG, "rad_batch_autotune: null handle");
    if (iters_per_trial < 1 || iters_per_trial > 32 || rounds < 1)
        return fail(RAD_ERR_ARG, "rad_batch_autotune: iters_per_trial must be 1..32, rounds >= 1");
    auto go = [&](auto& b) { return batch_autotune(b, iters_per_trial, rounds, chosen); };
    return BATCH_GO(h, go);
}

void rad_batch_destroy(rad_batch* h) { delete h; }

}  // extern "C"
