// C ABI: host scene store and visibility-structure entry points.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "capi_internal.h"

namespace radgb {
namespace {
thread_local std::string g_err;

// move the scene's tagged log lines ("1|..." stdout, "2|..." stderr) into the handle
template <typename T>
void take_log(rad_scene* h, Scene<T>& s) {
    h->log_out.clear();
    h->log_err.clear();
    size_t a = 0;
    while (a < s.log.size()) {
        size_t b = s.log.find("\n1|", a);
        size_t c = s.log.find("\n2|", a);
        size_t e = std::min(b, c);
        std::string piece = s.log.substr(a, e == std::string::npos ? std::string::npos : e + 1 - a);
        if (piece.size() >= 2 && piece[1] == '|') {
            (piece[0] == '1' ? h->log_out : h->log_err) += piece.substr(2);
        }
        if (e == std::string::npos) break;
        a = e + 1;
    }
    s.log.clear();
}

}  // namespace

void take_scene_log(rad_scene* h) {
    if (h->precision == 32) take_log(h, h->s32); else take_log(h, h->s64);
}

namespace {
template <typename T>
int view_of(const Scene<T>& s, rad_scene_view* v) {
    const size_t n = (size_t)s.trinum;
    static thread_local std::vector<char> buf;
    // slot-major field arrays gathered from the slot structs
    const size_t rs = sizeof(T);
    size_t need = n * (9 + 9 + 3 + 1 + 3 + 3) * rs + n * (1 + 3 + 3 + 3) * 4;
    buf.assign(need, 0);
    char* w = buf.data();
    auto take = [&](size_t bytes) { char* r = w; w += bytes; return r; };
    T* p = (T*)take(n * 9 * rs);
    T* acc = (T*)take(n * 9 * rs);
    T* db = (T*)take(n * 3 * rs);
    T* ar = (T*)take(n * rs);
    T* nr = (T*)take(n * 3 * rs);
    T* ct = (T*)take(n * 3 * rs);
    int32_t* par = (int32_t*)take(n * 4);
    int32_t* fr = (int32_t*)take(n * 12);
    int32_t* br = (int32_t*)take(n * 12);
    int32_t* nb = (int32_t*)take(n * 12);
    for (size_t i = 0; i < n; i++) {
        const Slot<T>& t = s.slots[i];
        std::memcpy(p + i * 9, t.p, 9 * rs);
        std::memcpy(acc + i * 9, t.accB, 9 * rs);
        std::memcpy(db + i * 3, t.deltaB, 3 * rs);
        ar[i] = t.area;
        std::memcpy(nr + i * 3, t.n, 3 * rs);
        std::memcpy(ct + i * 3, t.c, 3 * rs);
        par[i] = t.parent;
        std::memcpy(fr + i * 3, t.Frgb, 12);
        std::memcpy(br + i * 3, t.Brgb, 12);
        std::memcpy(nb + i * 3, t.nb, 12);
    }
    v->n = s.trinum;
    v->n_orig = s.n_orig;
    v->elem_size = (int32_t)rs;
    v->p = p; v->accB = acc; v->deltaB = db; v->area = ar; v->nrm = nr; v->ctr = ct;
    v->parent = par; v->frgb = fr; v->brgb = br; v->nb = nb;
    for (int k = 0; k < 3; k++) { v->G0[k] = (float)s.G0[k]; v->G1[k] = (float)s.G1[k]; }
    v->sample_area = s.opt.sample_area;
    v->min_area = (float)s.minarea;
    v->max_area = (float)s.maxarea;
    return RAD_OK;
}
}  // namespace

void set_error(const std::string& msg) { g_err = msg; }
int fail(int code, const std::string& msg) { g_err = msg; return code; }
}  // namespace radgb

using namespace radgb;

extern "C" {

void rad_options_default(rad_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->debug = 0;
    o->adapt_area = 5.0f;
    o->sample_area = -1.0f;
    o->converge = 1200.0f;
    o->delta_ff = 0.000005f;
    o->write_cycle = 10;
    o->zip = 0;
    o->triangle_limit = 1000000;
    o->light_scale = 1.0f;
    o->interactive = 0;
    o->jobs = 2;
    o->parallel_src = 1;
    o->precision = 32;
    o->walk_cap = 1 << 16;
}

const char* rad_last_error(void) { return g_err.c_str(); }
const char* rad_version(void) { return "hw-radiosity-gb300 0.1 (sm_103a)"; }

int rad_scene_load(const char* path, const rad_options* o, rad_scene** out) {
    if (!path || !o || !out) return fail(RAD_ERR_ARG, "rad_scene_load: null argument");
    if (o->precision != 32 && o->precision != 64) return fail(RAD_ERR_ARG, "precision must be 32 or 64");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(RAD_ERR_IO, std::string("File open error::") + path);
    std::string text;
    char chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) text.append(chunk, k);
    std::fclose(f);
    rad_scene* h = new (std::nothrow) rad_scene();
    if (!h) return fail(RAD_ERR_CAPACITY, "out of host memory");
    h->precision = o->precision;
    std::string err;
    int rc = (o->precision == 32) ? load_tri_text<float>(text.data(), text.size(), *o, h->s32, err)
                                  : load_tri_text<double>(text.data(), text.size(), *o, h->s64, err);
    if (rc != RAD_OK) { delete h; return fail(rc, err); }
    if (h->precision == 32) take_log(h, h->s32); else take_log(h, h->s64);
    *out = h;
    return RAD_OK;
}

int rad_scene_from_arrays(const float* vtx, const int32_t* frgb, const int32_t* brgb, int32_t n,
                          const rad_options* o, rad_scene** out) {
    if (!o || !out) return fail(RAD_ERR_ARG, "rad_scene_from_arrays: null argument");
    if (o->precision != 32 && o->precision != 64) return fail(RAD_ERR_ARG, "precision must be 32 or 64");
    rad_scene* h = new (std::nothrow) rad_scene();
    if (!h) return fail(RAD_ERR_CAPACITY, "out of host memory");
    h->precision = o->precision;
    std::string err;
    int rc = (o->precision == 32) ? load_arrays<float>(vtx, frgb, brgb, n, *o, h->s32, err)
                                  : load_arrays<double>(vtx, frgb, brgb, n, *o, h->s64, err);
    if (rc != RAD_OK) { delete h; return fail(rc, err); }
    if (h->precision == 32) take_log(h, h->s32); else take_log(h, h->s64);
    *out = h;
    return RAD_OK;
}

int rad_scene_init(rad_scene* h) {
    if (!h) return fail(RAD_ERR_ARG, "rad_scene_init: null scene");
    if (h->precision == 32) { init_radiosity(h->s32); take_log(h, h->s32); }
    else { init_radiosity(h->s64); take_log(h, h->s64); }
    return RAD_OK;
}

int rad_scene_prepartition(rad_scene* h) {
    if (!h) return fail(RAD_ERR_ARG, "rad_scene_prepartition: null scene");
    if (h->precision == 32) { prepartition(h->s32); take_log(h, h->s32); }
    else { prepartition(h->s64); take_log(h, h->s64); }
    return RAD_OK;
}

int rad_scene_view_get(const rad_scene* h, rad_scene_view* v) {
    if (!h || !v) return fail(RAD_ERR_ARG, "rad_scene_view_get: null argument");
    return h->precision == 32 ? view_of(h->s32, v) : view_of(h->s64, v);
}

int rad_scene_write_fin(const rad_scene* h, const char* prefix, int32_t loop) {
    if (!h || !prefix) return fail(RAD_ERR_ARG, "rad_scene_write_fin: null argument");
    std::string err;
    int rc = h->precision == 32 ? write_fin(h->s32, prefix, loop, err) : write_fin(h->s64, prefix, loop, err);
    if (rc != RAD_OK) return fail(rc, err);
    if (!err.empty()) set_error(err);
    return RAD_OK;
}

const char* rad_scene_log(const rad_scene* h, int32_t stream) {
    if (!h) return "";
    return stream == 1 ? h->log_out.c_str() : h->log_err.c_str();
}

void rad_scene_free(rad_scene* h) { delete h; }

int rad_octree_build(const rad_scene* h, int32_t threads, rad_octree** out) {
    if (!h || !out) return fail(RAD_ERR_ARG, "rad_octree_build: null argument");
    rad_octree* t = new (std::nothrow) rad_octree();
    if (!t) return fail(RAD_ERR_CAPACITY, "out of host memory");
    t->precision = h->precision;
    if (threads <= 0) threads = (int32_t)std::max(1u, std::thread::hardware_concurrency());
    if (h->precision == 32) build_octree(h->s32, t->o32, threads);
    else build_octree(h->s64, t->o64, threads);
    const int32_t* d = h->precision == 32 ? t->o32.dims : t->o64.dims;
    if ((int64_t)d[0] * d[1] * d[2] > (int64_t)1 << 26) {
        delete t;
        return fail(RAD_ERR_CAPACITY, "octree cell table exceeds 2^26 cells");
    }
    *out = t;
    return RAD_OK;
}

int rad_octree_tables(const rad_octree* t, int32_t* cell_leaf, void* leaf_box, int32_t* leaf_range,
                      int32_t* entry_tri) {
    if (!t) return fail(RAD_ERR_ARG, "rad_octree_tables: null octree");
    auto copy = [&](auto& o) {
        using T = typename std::decay<decltype(o.leaf_box)>::type::value_type;
        if (cell_leaf) std::memcpy(cell_leaf, o.cell_leaf.data(), o.cell_leaf.size() * 4);
        if (leaf_box) std::memcpy(leaf_box, o.leaf_box.data(), o.leaf_box.size() * sizeof(T));
        if (leaf_range) std::memcpy(leaf_range, o.leaf_range.data(), o.leaf_range.size() * 4);
        if (entry_tri) std::memcpy(entry_tri, o.entry_tri.data(), o.entry_tri.size() * 4);
    };
    if (t->precision == 32) copy(t->o32); else copy(t->o64);
    return RAD_OK;
}

int rad_octree_info(const rad_octree* t, int64_t* ref_nodes, int64_t* ref_list, int32_t* n_leaves,
                    int64_t* n_entries, int32_t dims[3]) {
    if (!t) return fail(RAD_ERR_ARG, "rad_octree_info: null octree");
    auto fill = [&](auto& o) {
        if (ref_nodes) *ref_nodes = o.ref_nodes;
        if (ref_list) *ref_list = o.ref_list;
        if (n_leaves) *n_leaves = (int32_t)(o.leaf_range.size() / 2);
        if (n_entries) *n_entries = (int64_t)o.entry_tri.size();
        if (dims) for (int k = 0; k < 3; k++) dims[k] = o.dims[k];
    };
    if (t->precision == 32) fill(t->o32); else fill(t->o64);
    return RAD_OK;
}

int rad_octree_cell_coords(const rad_octree* t, int32_t axis, const void* q, int32_t n, int32_t* out_ref,
                           int32_t* out_fast) {
    if (!t || axis < 0 || axis > 2 || (n > 0 && (!q || !out_ref || !out_fast)))
        return fail(RAD_ERR_ARG, "rad_octree_cell_coords: bad argument");
    auto go = [&](auto& o, auto* qq) {
        for (int32_t i = 0; i < n; i++) {
            out_ref[i] = cell_coord(qq[i], o.G0[axis], o.min_grid);
            out_fast[i] = cell_of_thresholds(o, axis, qq[i]);
        }
    };
    if (t->precision == 32) go(t->o32, (const float*)q);
    else go(t->o64, (const double*)q);
    return RAD_OK;
}

void rad_octree_free(rad_octree* t) { delete t; }

}  // extern "C"
