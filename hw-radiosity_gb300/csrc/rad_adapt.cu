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
// of every receiver against the step's shooter.  So each step
//   1. the device computes those four form factors for every slot
//      (k_adapt_ff, one thread per slot and point);
//   2. the host runs the reference's receiver loop in order, taking a
//      precomputed value whenever its inputs are unchanged -- the receiver was
//      not written by a split earlier in this step and the shooter slot was
//      not either -- and otherwise evaluating the same walk and form-factor
//      code on the host (it is compiled for both), as for sample points and
//      re-shaded neighbours.
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
    LibcRand rng;
    long long steps = 0;
    bool done = false;
    Cnt hc = {0, 0, 0, 0, 0, 0, 0, 0};    // host-side walks
    long long samples = 0, splits = 0, pre_used = 0, host_points = 0;
    uint32_t step_id = 1;

    ~AdaptImpl() {
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
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
    a.ff.assign((size_t)a.cap * 4, (T)0);
    a.mod_step.assign((size_t)a.cap, 0);
    a.dirty.assign((size_t)a.cap, 0);
    for (int32_t i = 0; i < s.trinum; i++) a.mark(i);
    a.step_id = 1;
    return adapt_upload_dirty(a);
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
    bool shooter_changed = false;
    Shooter<T> sh;            // the shooter as the precompute saw it
    Shooter<T> live;          // rebuilt from the slot after a split rewrote it

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
            for (int k = 0; k < n; k++) {
                // GetPointInTriangle, shade.cpp:49-68
                T r1 = (T)a.rng.next(), r2 = (T)a.rng.next(), r3 = (T)a.rng.next();
                const T tot = r1 + r2 + r3;
                r1 /= tot; r2 /= tot; r3 /= tot;
                T pt[3];
                for (int q = 0; q < 3; q++) pt[q] = r1 * des.p[0][q] + r2 * des.p[1][q] + r3 * des.p[2][q];
                ground = r1 * f[0] + r2 * f[1] + r3 * f[2];
                a.samples++;
                ffs = ff_host(d, pt, logdes);
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
    if ((rc = adapt_upload_dirty(a))) return rc;
    StepCtx<T> cx{a, src, s.slots[src].parent, s.trinum};
    host_shooter(s.slots[src], src, cx.logsrc, cx.sh);
    // every slot's corner and centre form factors against this shooter
    CU(cudaMemcpyAsync(a.d_sh, &cx.sh, sizeof cx.sh, cudaMemcpyHostToDevice, a.stream));
    const Slots<T> S{cx.n0, a.d_vtx, a.d_nrm, a.d_ctr, a.d_frgb, nullptr, nullptr};
    if (cx.n0 > 0) {
        const int blocks = (int)std::min<long long>((4LL * cx.n0 + 255) / 256, 152 * 16);
        k_adapt_ff<T><<<blocks, 256, 0, a.stream>>>(S, a.Gd, a.d_sh, cx.n0, a.d_ff, a.d_state);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(a.ff.data(), a.d_ff, (size_t)cx.n0 * 4 * sizeof(T), cudaMemcpyDeviceToHost, a.stream));
    }
    CU(cudaStreamSynchronize(a.stream));
    // serialRadiosity's receiver loop, rad.cpp:464-485 (bound re-read: splits append slots)
    for (int d = 0; d < s.trinum; d++) {
        if (d == src) continue;
        const Slot<T>& t = s.slots[d];
        if (t.parent < 0) continue;
        if (!is_open(t)) continue;
        if (cx.shade(d, t.parent)) d--;
    }
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

void rad_adapt_destroy(rad_adapt* h) { delete h; }

}  // extern "C"
