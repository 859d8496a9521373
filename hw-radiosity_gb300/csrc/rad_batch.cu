// Batched form: many independent scenes shot together, one persistent launch
// per batch iteration (FP32).
//
// Every scene keeps its own slots, octree, selection and convergence; in one
// iteration every scene that has not converged does one shooter step of the
// reference's loop (parallelRadiosity, src/rad.cpp:406-451, one shooter per
// step).  All scenes' records are concatenated in HBM; a descriptor per
// scene points into them.
//
//   k_batch_setup  one thread per scene: take the scene's packed (key, slot)
//                  maximum from the previous iteration, mark the scene done
//                  or build its shooter record.
//   k_batch_shoot  persistent: warps take (scene, 10-slot group) items from a
//                  queue over the groups of the scenes still running, run the
//                  single-scene kernel's per-group body on that scene, and
//                  fold the group's selection key into the scene's maximum
//                  with one 64-bit atomicMax ((ordered FP32 key << 32) | slot,
//                  so ties go to the higher slot as in listCanditate).
//
// The queue lists only groups of running scenes; the host rebuilds it between
// graph chunks when scenes finish.  A scene's result is bit-identical to the
// single-scene solver's (same per-group code, same order of every sum).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "rad_kernels.cuh"

namespace radgb {
namespace dev {

struct SceneDesc {
    Slots<float> S;
    Grid<float> G;
    float conv;
    int trace_off;
    int trace_cap;
    int n_groups;
};

struct SceneState {
    unsigned long long best;   // packed selection maximum of the last iteration
    int done;
    int nsh;                   // 0 before the first step, then 1
    long long steps;
    Shooter<float> sh;
};

struct BatchCtl {
    int work;                  // next queue item
    int n_items;               // queue length (groups of running scenes)
    int pad[2];
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

__global__ void k_batch_setup(const SceneDesc* __restrict__ desc, SceneState* ss, int n_scenes, int* trace,
                              BatchCtl* bc) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) bc->work = 0;
    if (s >= n_scenes) return;
    SceneState& st = ss[s];
    if (st.done) { st.nsh = 0; return; }
    const unsigned long long best = st.best;
    if (best == 0) {           // no candidate above the scene's converge limit
        st.done = 1;
        st.nsh = 0;
        return;
    }
    const int slot = (int)(best & 0xffffffffull);
    build_shooter(desc[s].S, slot, st.sh);
    st.best = 0;
    st.nsh = 1;
    if (st.steps < desc[s].trace_cap) trace[desc[s].trace_off + st.steps] = slot;
    st.steps += 1;
}

// Many scenes keep every SM busy for the whole launch, so this kernel is
// bound by throughput, not by its slowest group: 4 CTAs per SM (64 registers,
// some spilled) measured 14% faster on the 256-room batch than 3 (80
// registers), and 5 or 6 slower again.
#ifndef RAD_BATCH_MIN_BLOCKS
#define RAD_BATCH_MIN_BLOCKS 4
#endif
template <bool COUNT>
__global__ void __launch_bounds__(kShootThreads, RAD_BATCH_MIN_BLOCKS)
k_batch_shoot(const SceneDesc* __restrict__ desc, SceneState* ss, const int2* __restrict__ items, BatchCtl* bc) {
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
        const SceneDesc d = desc[s];
        unsigned long long kk = 0;
        int ks = -1;
        shoot_group<float, COUNT>(d.S, d.G, &ss[s].sh, nsh, it.y, lane, d.conv, kk, ks, c);
        warp_max(kk, ks);
        if (lane == 0 && ks >= 0) atomicMax(&ss[s].best, (kk << 32) | (unsigned long long)(unsigned)ks);
    }
    flush_batch<COUNT>(bc, c, lane);
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

struct rad_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int n_scenes = 0;
    bool counting = false;
    std::vector<void*> allocs;
    size_t bytes = 0;
    std::vector<SceneDesc> desc;        // host copy (device pointers inside)
    std::vector<PackOffsets> off;
    SceneDesc* d_desc = nullptr;
    SceneState* d_ss = nullptr;
    int2* d_items = nullptr;
    BatchCtl* d_ctl = nullptr;
    int* d_trace = nullptr;
    int n_cta = 1;
    std::vector<int> done;              // host mirror, per scene
    std::vector<long long> steps;
    cudaGraphExec_t graphs[2][33] = {};
    cudaEvent_t ev[2] = {nullptr, nullptr};

    ~rad_batch() {
        for (auto& row : graphs)
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
};

namespace {

int launch_iter(rad_batch& b, cudaStream_t s) {
    k_batch_setup<<<(b.n_scenes + 127) / 128, 128, 0, s>>>(b.d_desc, b.d_ss, b.n_scenes, b.d_trace, b.d_ctl);
    if (b.counting)
        k_batch_shoot<true><<<b.n_cta, kShootThreads, 0, s>>>(b.d_desc, b.d_ss, b.d_items, b.d_ctl);
    else
        k_batch_shoot<false><<<b.n_cta, kShootThreads, 0, s>>>(b.d_desc, b.d_ss, b.d_items, b.d_ctl);
    CU(cudaGetLastError());
    return RAD_OK;
}

int graph_for(rad_batch& b, int iters, cudaGraphExec_t* out) {
    cudaGraphExec_t& slot = b.graphs[b.counting ? 1 : 0][iters];
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

// queue of (scene, group) items over the scenes still running
int rebuild_items(rad_batch& b) {
    std::vector<int2> items;
    for (int s = 0; s < b.n_scenes; s++) {
        if (b.done[s]) continue;
        for (int g = 0; g < b.desc[s].n_groups; g++) items.push_back(make_int2(s, g));
    }
    const int n = (int)items.size();
    if (n) CU(cudaMemcpyAsync(b.d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, b.stream));
    CU(cudaMemcpyAsync(&b.d_ctl->n_items, &n, sizeof n, cudaMemcpyHostToDevice, b.stream));
    CU(cudaStreamSynchronize(b.stream));
    return RAD_OK;
}

int refresh(rad_batch& b, bool* changed) {
    std::vector<SceneState> ss(b.n_scenes);
    CU(cudaMemcpyAsync(ss.data(), b.d_ss, ss.size() * sizeof(SceneState), cudaMemcpyDeviceToHost, b.stream));
    CU(cudaStreamSynchronize(b.stream));
    *changed = false;
    for (int s = 0; s < b.n_scenes; s++) {
        if (ss[s].done != b.done[s]) *changed = true;
        b.done[s] = ss[s].done;
        b.steps[s] = ss[s].steps;
    }
    return RAD_OK;
}

constexpr int kBatchChunk = 32;

int run(rad_batch& b, long long max_iters, long long* iters_done, int* n_active, double* ms) {
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
        CU(cudaGraphLaunch(g, b.stream));
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

}  // namespace

extern "C" {

int rad_batch_create(const rad_scene* const* scenes, const rad_octree* const* trees, const rad_options* opts,
                     int32_t n_scenes, int32_t trace_cap, int32_t device, rad_batch** out) {
    if (!scenes || !trees || !opts || !out || n_scenes <= 0) return fail(RAD_ERR_ARG, "rad_batch_create: bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(RAD_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(RAD_ERR_ARG, "device index out of range");
    for (int s = 0; s < n_scenes; s++) {
        if (!scenes[s] || !trees[s]) return fail(RAD_ERR_ARG, "null scene or octree");
        if (scenes[s]->precision != 32 || trees[s]->precision != 32 || opts[s].precision != 32)
            return fail(RAD_ERR_ARG, "the batched form is FP32 only");
        if (opts[s].parallel_src > 1) return fail(RAD_ERR_ARG, "the batched form shoots one shooter per step");
        if (!thresholds_consistent(trees[s]->o32)) return fail(RAD_ERR_ARG, "octree thresholds inconsistent");
    }
    if (trace_cap <= 0) trace_cap = 1 << 16;
    rad_batch* b = new rad_batch();
    auto bail = [&](int rc) { delete b; return rc; };
    b->device = device;
    b->n_scenes = n_scenes;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(RAD_ERR_CUDA, "stream creation failed"));
    HostPack<float> P;
    b->off.resize(n_scenes);
    long long total_groups = 0;
    for (int s = 0; s < n_scenes; s++) {
        b->off[s] = pack_scene(scenes[s]->s32, trees[s]->o32, P);
        total_groups += (b->off[s].n + kSlotsPerWarp - 1) / kSlotsPerWarp;
    }
    if (total_groups > 0x7fffffffLL || (long long)trace_cap * n_scenes > 0x7fffffffLL)
        return bail(fail(RAD_ERR_CAPACITY, "batch too large"));
    Q4<float> *d_vtx, *d_nrm, *d_ctr, *d_frgb, *d_acc, *d_db, *d_ent;
    CellRec<float>* d_cell;
    float* d_thr;
    int rc;
    auto put = [&](auto** dst, const auto& src) -> int {
        int r = b->alloc(dst, src.size());
        if (r) return r;
        CU(cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice, b->stream));
        return RAD_OK;
    };
    if ((rc = put(&d_vtx, P.vtx)) || (rc = put(&d_nrm, P.nrm)) || (rc = put(&d_ctr, P.ctr)) ||
        (rc = put(&d_frgb, P.frgb)) || (rc = put(&d_acc, P.acc)) || (rc = put(&d_db, P.db)) ||
        (rc = put(&d_ent, P.ent)) || (rc = put(&d_cell, P.cell)) ||
        (rc = put(&d_thr, P.thr)))
        return bail(rc);
    b->desc.resize(n_scenes);
    for (int s = 0; s < n_scenes; s++) {
        const PackOffsets& o = b->off[s];
        SceneDesc& d = b->desc[s];
        d.S = Slots<float>{o.n, d_vtx + o.slot * 3, d_nrm + o.slot, d_ctr + o.slot, d_frgb + o.slot,
                           d_acc + o.slot * 3, d_db + o.slot};
        d.G = grid_params(trees[s]->o32, opts[s].walk_cap);
        d.G.thr = d_thr + o.thr;
        d.G.cell = d_cell + o.cell;
        d.G.entry = d_ent + o.ent * 5;
        d.conv = opts[s].converge;
        d.trace_off = s * trace_cap;
        d.trace_cap = trace_cap;
        d.n_groups = (o.n + kSlotsPerWarp - 1) / kSlotsPerWarp;
    }
    if ((rc = put(&b->d_desc, b->desc)) || (rc = b->alloc(&b->d_ss, (size_t)n_scenes)) ||
        (rc = b->alloc(&b->d_items, (size_t)std::max<long long>(total_groups, 1))) || (rc = b->alloc(&b->d_ctl, 1)) ||
        (rc = b->alloc(&b->d_trace, (size_t)trace_cap * n_scenes)))
        return bail(rc);
    if (cudaMemsetAsync(b->d_ss, 0, sizeof(SceneState) * n_scenes, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->d_ctl, 0, sizeof(BatchCtl), b->stream) != cudaSuccess)
        return bail(fail(RAD_ERR_CUDA, "memset failed"));
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_shoot<false>, kShootThreads, 0);
    const long long want = (total_groups + kShootThreads / 32 - 1) / (kShootThreads / 32);
    b->n_cta = (int)std::max<long long>(1, std::min<long long>(want, std::max(1, sms * per_sm)));
    b->done.assign(n_scenes, 0);
    b->steps.assign(n_scenes, 0);
    if ((rc = rebuild_items(*b))) return bail(rc);
    // initial selection keys: every scene's groups with no shooter
    if (cudaMemsetAsync(&b->d_ctl->work, 0, sizeof(int), b->stream) != cudaSuccess) return bail(fail(RAD_ERR_CUDA, "memset"));
    k_batch_shoot<false><<<b->n_cta, kShootThreads, 0, b->stream>>>(b->d_desc, b->d_ss, b->d_items, b->d_ctl);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(b->stream) != cudaSuccess)
        return bail(fail(RAD_ERR_CUDA, "initial selection failed"));
    *out = b;
    return RAD_OK;
}

int rad_batch_run(rad_batch* b, int64_t max_iters, int64_t* iters_done, int32_t* n_active) {
    if (!b) return fail(RAD_ERR_ARG, "rad_batch_run: null handle");
    long long it = 0;
    int na = 0;
    int rc = run(*b, max_iters, &it, &na, nullptr);
    if (iters_done) *iters_done = it;
    if (n_active) *n_active = na;
    return rc;
}

int rad_batch_run_timed(rad_batch* b, int64_t max_iters, int64_t* iters_done, int32_t* n_active, double* device_ms) {
    if (!b) return fail(RAD_ERR_ARG, "rad_batch_run_timed: null handle");
    long long it = 0;
    int na = 0;
    double ms = 0;
    int rc = run(*b, max_iters, &it, &na, &ms);
    if (iters_done) *iters_done = it;
    if (n_active) *n_active = na;
    if (device_ms) *device_ms = ms;
    return rc;
}

int rad_batch_scene_stats(const rad_batch* b, int32_t scene, int64_t* steps, int32_t* converged) {
    if (!b || scene < 0 || scene >= b->n_scenes) return fail(RAD_ERR_ARG, "rad_batch_scene_stats: bad argument");
    if (steps) *steps = b->steps[scene];
    if (converged) *converged = b->done[scene];
    return RAD_OK;
}

int rad_batch_download(rad_batch* b, int32_t scene, rad_scene* s) {
    if (!b || !s || scene < 0 || scene >= b->n_scenes) return fail(RAD_ERR_ARG, "rad_batch_download: bad argument");
    if (s->precision != 32) return fail(RAD_ERR_ARG, "the batched form is FP32 only");
    const PackOffsets& o = b->off[scene];
    if (o.n != s->s32.trinum) return fail(RAD_ERR_ARG, "scene slot count differs from the batch copy");
    std::vector<Q4<float>> acc((size_t)o.n * 3), db(o.n);
    CU(cudaSetDevice(b->device));
    if (o.n) {
        CU(cudaMemcpyAsync(acc.data(), b->desc[scene].S.accB, acc.size() * sizeof(Q4<float>), cudaMemcpyDeviceToHost, b->stream));
        CU(cudaMemcpyAsync(db.data(), b->desc[scene].S.deltaB, db.size() * sizeof(Q4<float>), cudaMemcpyDeviceToHost, b->stream));
    }
    CU(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < o.n; i++) {
        Slot<float>& t = s->s32.slots[i];
        for (int v = 0; v < 3; v++) {
            t.accB[v][0] = acc[i * 3 + v].x; t.accB[v][1] = acc[i * 3 + v].y; t.accB[v][2] = acc[i * 3 + v].z;
        }
        t.deltaB[0] = db[i].x; t.deltaB[1] = db[i].y; t.deltaB[2] = db[i].z;
    }
    return RAD_OK;
}

int rad_batch_trace(const rad_batch* b, int32_t scene, int32_t* out, int64_t cap, int64_t* n) {
    if (!b || scene < 0 || scene >= b->n_scenes) return fail(RAD_ERR_ARG, "rad_batch_trace: bad argument");
    const long long have = std::min<long long>(b->steps[scene], b->desc[scene].trace_cap);
    if (n) *n = have;
    if (!out || cap <= 0) return RAD_OK;
    CU(cudaSetDevice(b->device));
    CU(cudaMemcpy(out, b->d_trace + b->desc[scene].trace_off, (size_t)std::min<long long>(have, cap) * 4,
                  cudaMemcpyDeviceToHost));
    return RAD_OK;
}

int rad_batch_stats(const rad_batch* b, rad_stats* st) {
    if (!b || !st) return fail(RAD_ERR_ARG, "rad_batch_stats: null argument");
    BatchCtl ctl;
    CU(cudaSetDevice(b->device));
    CU(cudaMemcpy(&ctl, b->d_ctl, sizeof ctl, cudaMemcpyDeviceToHost));
    std::memset(st, 0, sizeof *st);
    for (int s = 0; s < b->n_scenes; s++) {
        st->steps += b->steps[s];
        st->n_slots += b->off[s].n;
    }
    st->shots = st->steps;
    st->rays = (int64_t)ctl.rays;
    st->rays_ref = (int64_t)ctl.rays_ref;
    st->cells = (int64_t)ctl.cells;
    st->tri_tests = (int64_t)ctl.tris;
    st->se_tests = (int64_t)ctl.se;
    st->prec_steps = (int64_t)ctl.prec;
    st->walk_cap_hits = (int64_t)ctl.capped;
    st->walk_loops = (int64_t)ctl.loops;
    int active = 0;
    for (int d : b->done) active += !d;
    st->converged = active == 0;
    st->device_bytes = (int64_t)b->bytes;
    return RAD_OK;
}

int rad_batch_set_counting(rad_batch* b, int32_t on) {
    if (!b) return fail(RAD_ERR_ARG, "rad_batch_set_counting: null handle");
    b->counting = on != 0;
    return RAD_OK;
}

void rad_batch_destroy(rad_batch* b) { delete b; }

}  // extern "C"
