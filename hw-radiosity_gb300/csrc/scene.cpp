// Host scene store: .tri input, InitRadiosity, PrePartition, .fin output.
//
// Arithmetic follows the reference operation by operation (FP32 values, the
// FP64 promotions its double literals cause); the library is compiled with
// -ffp-contract=off so the compiler fuses no multiply-add (aarch64 GCC would
// otherwise contract by default).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <utility>

#include "rad_host.h"

namespace radgb {
namespace {

template <typename T> inline T dot3(const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename T> inline T len3(const T* a) { return (T)std::sqrt(dot3(a, a)); }
template <typename T> inline void edge(const T* from, const T* to, T* o) {
    o[0] = to[0] - from[0]; o[1] = to[1] - from[1]; o[2] = to[2] - from[2];
}
template <typename T> inline void cross3(const T* a, const T* b, T* o) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}
template <typename T> inline T tmin(T a, T b) { return (b < a) ? b : a; }   // std::min
template <typename T> inline T tmax(T a, T b) { return (a < b) ? b : a; }   // std::max
// CalCenter (include/vector.h:60-63): float sum, double division by 3.0
template <typename T> inline void centre(const T p[3][3], T* c) {
    for (int k = 0; k < 3; k++) c[k] = (T)((double)(p[0][k] + p[1][k] + p[2][k]) / 3.0);
}
template <typename T> inline bool is_light(const Slot<T>& t) {
    return t.Brgb[0] == 255 || t.Brgb[1] == 255 || t.Brgb[2] == 255;
}

// ---------------------------------------------------------------- parsing
struct Cursor {
    const char* p;
    const char* end;
    bool ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
        return p < end;
    }
    static bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }
};

bool read_int(Cursor& c, int32_t& v) {
    if (!c.ws()) return false;
    const char* q = c.p;
    bool neg = false;
    if (q < c.end && (*q == '+' || *q == '-')) { neg = (*q == '-'); q++; }
    if (q >= c.end || *q < '0' || *q > '9') return false;
    int64_t x = 0;
    while (q < c.end && *q >= '0' && *q <= '9') { x = x * 10 + (*q - '0'); if (x > 0x7fffffffLL + 1) x = 0x7fffffffLL + 1; q++; }
    v = (int32_t)(neg ? -x : x);
    c.p = q;
    return true;
}

template <typename T> T parse_real(const char* s, char** e);
template <> float parse_real<float>(const char* s, char** e) { return std::strtof(s, e); }
template <> double parse_real<double>(const char* s, char** e) { return std::strtod(s, e); }

template <typename T>
bool read_real(Cursor& c, T& v, std::string& scratch) {
    if (!c.ws()) return false;
    // strtod needs a terminated string; copy the token (tokens are short)
    const char* q = c.p;
    while (q < c.end && !Cursor::is_ws(*q)) q++;
    scratch.assign(c.p, q);
    char* e = nullptr;
    v = parse_real<T>(scratch.c_str(), &e);
    if (e == scratch.c_str()) return false;
    c.p += (e - scratch.c_str());
    return true;
}

// derived quantities of a freshly read triangle, src/rad.cpp:76-88
template <typename T>
void derive(Slot<T>& t) {
    centre(t.p, t.c);
    T e0[3], e1[3];
    edge(t.p[0], t.p[1], e0);
    edge(t.p[0], t.p[2], e1);
    cross3(e0, e1, t.n);
    t.area = len3(t.n) / 2;
    T l = len3(t.n);
    t.n[0] /= l; t.n[1] /= l; t.n[2] /= l;
    for (int i = 0; i < 3; i++) {
        T e[3], s[3];
        edge(t.p[i], t.p[(i + 1) % 3], e);
        cross3(t.n, e, s);
        t.se[i][0] = s[0]; t.se[i][1] = s[1]; t.se[i][2] = s[2];
        t.se[i][3] = -dot3(t.p[i], s);
    }
}

template <typename T>
void finish_load(Scene<T>& s, const T lo[3], const T hi[3]) {
    T m = 0;
    for (int i = 0; i < 3; i++) m = tmax(m, hi[i] - lo[i]);
    for (int i = 0; i < 3; i++) s.G0[i] = (T)((double)lo[i] - kPi);
    for (int i = 0; i < 3; i++) s.G1[i] = (T)((double)(s.G0[i] + m) + 2 * kPi);
    s.n_orig = s.trinum;
    // the slot pool: live slots plus room for the pre-partition, zero-filled
    int lim = std::min(s.opt.triangle_limit, kMaxTriPool);
    size_t cap = (size_t)std::max(s.trinum, lim) + 8;
    s.slots.resize(cap);
    char buf[256];
    snprintf(buf, sizeof buf, "2|[\x1B[32mINFO\x1B[37m] Read #Triangle \x1B[35m%d\x1B[37m from input file\n", s.trinum);
    s.log += buf;
}

template <typename T>
void bounds_add(const Slot<T>& t, T lo[3], T hi[3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            lo[j] = tmin(lo[j], t.p[i][j]);
            hi[j] = tmax(hi[j], t.p[i][j]);
        }
}

// ---------------------------------------------------------------- float text
}  // namespace

bool format_float(float x, char* buf) {
    uint32_t raw;
    std::memcpy(&raw, &x, 4);
    const bool neg = raw >> 31;
    const int eb = (raw >> 23) & 0xff;
    const uint32_t fr = raw & 0x7fffff;
    if (eb == 0xff || (eb == 0 && fr)) return false;    // Inf, NaN, subnormal
    char* d = buf;
    if (eb == 0) {                                       // +-0
        if (neg) *d++ = '-';
        std::memcpy(d, "0.0", 4);
        return true;
    }
    const int e2 = eb - 150;                             // value = mant * 2^e2
    if (e2 > 0 && e2 >= 41) return false;                // integer part beyond 64 bits
    const uint64_t mant = fr | (1u << 23);
    if (neg) *d++ = '-';
    char digits[24];
    int nd = 0;
    if (e2 < -23) {
        digits[nd++] = '0';
    } else {
        uint64_t iv = e2 > 0 ? mant << e2 : (e2 < 0 ? mant >> -e2 : mant);
        for (; iv; iv /= 10) digits[nd++] = (char)('0' + iv % 10);
    }
    if (!nd) *d++ = '0';
    while (nd) *d++ = digits[--nd];
    *d++ = '.';
    // fraction: value * 2^60 in 64 bits; each step exposes one decimal digit
    // in the top nibble; up to eight digits, truncated, trailing zeros dropped
    const int sh = 60 + e2;
    int keep = 0;
    char fd[8];
    if (sh >= 0 && sh < 60) {
        uint64_t f = mant << sh;
        for (int k = 0; f && k < 8;) {
            f &= 0x0fffffffffffffffULL;
            f *= 10;
            const int dg = (int)(f >> 60);
            fd[k++] = (char)('0' + dg);
            if (dg) keep = k;
        }
    }
    if (!keep) *d++ = '0';
    for (int k = 0; k < keep; k++) *d++ = fd[k];
    *d = 0;
    return true;
}

template <typename T>
int load_tri_text(const char* text, size_t len, const rad_options& o, Scene<T>& s, std::string& err) {
    s = Scene<T>();
    s.opt = o;
    Cursor c{text, text + len};
    T lo[3] = {(T)1000000.0, (T)1000000.0, (T)1000000.0}, hi[3] = {(T)-1000000.0, (T)-1000000.0, (T)-1000000.0};
    std::string scratch;
    s.slots.reserve(len / 64 + 16);
    for (;;) {
        // keyword token; like fscanf("%s") + feof(), a token that runs into the
        // end of the input ends the scan
        if (!c.ws()) break;
        while (c.p < c.end && !Cursor::is_ws(*c.p)) c.p++;
        if (c.p >= c.end) break;
        Slot<T> t;
        std::memset(&t, 0, sizeof t);
        bool ok = true;
        for (int k = 0; k < 3 && ok; k++) ok = read_int(c, t.Frgb[k]);
        for (int k = 0; k < 3 && ok; k++) ok = read_int(c, t.Brgb[k]);
        for (int v = 0; v < 3 && ok; v++)
            for (int k = 0; k < 3 && ok; k++) ok = read_real<T>(c, t.p[v][k], scratch);
        if (!ok) {
            err = "malformed triangle #" + std::to_string(s.trinum) + " in .tri input";
            return RAD_ERR_PARSE;
        }
        derive(t);
        bounds_add(t, lo, hi);
        t.parent = s.trinum;
        t.nb[0] = t.nb[1] = t.nb[2] = -1;
        s.slots.push_back(t);
        s.trinum++;
    }
    finish_load(s, lo, hi);
    return RAD_OK;
}

template <typename T>
int load_arrays(const float* vtx, const int32_t* frgb, const int32_t* brgb, int32_t n, const rad_options& o,
                Scene<T>& s, std::string& err) {
    if (n < 0 || (n > 0 && (!vtx || !frgb || !brgb))) { err = "bad scene arrays"; return RAD_ERR_ARG; }
    s = Scene<T>();
    s.opt = o;
    T lo[3] = {(T)1000000.0, (T)1000000.0, (T)1000000.0}, hi[3] = {(T)-1000000.0, (T)-1000000.0, (T)-1000000.0};
    s.slots.resize((size_t)n);
    for (int32_t i = 0; i < n; i++) {
        Slot<T>& t = s.slots[i];
        std::memset(&t, 0, sizeof t);
        for (int k = 0; k < 3; k++) { t.Frgb[k] = frgb[i * 3 + k]; t.Brgb[k] = brgb[i * 3 + k]; }
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) t.p[v][k] = (T)vtx[i * 9 + v * 3 + k];
        derive(t);
        bounds_add(t, lo, hi);
        t.parent = i;
        t.nb[0] = t.nb[1] = t.nb[2] = -1;
    }
    s.trinum = n;
    finish_load(s, lo, hi);
    return RAD_OK;
}

// ---------------------------------------------------------------- init
namespace {
// exact-coordinate key: +-0 unified (float == treats them as equal)
template <typename T> struct VKey;
template <> struct VKey<float> {
    uint32_t w[3];
    static uint32_t bits(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u == 0x80000000u ? 0u : u; }
};
template <> struct VKey<double> {
    uint64_t w[3];
    static uint64_t bits(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u == 0x8000000000000000ull ? 0ull : u; }
};

template <typename T>
bool same_point(const T* a, const T* b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }

// Neighbour links, src/rad.cpp:295-334.  The reference compares every pair
// (i, j) and lets later writes win.  Candidate pairs share an exact vertex,
// so group corners by vertex (sort on the coordinate bits) and, for each i
// in ascending order, apply its writes in the reference's (j, v, n) order:
// the final links are those of the sequential scan.
template <typename T>
void link_neighbours(Scene<T>& s) {
    const int32_t N = s.trinum;
    struct Corner { decltype(VKey<T>::bits(T(0))) k[3]; int32_t tri; int8_t v; };
    std::vector<Corner> cs;
    cs.reserve((size_t)N * 3);
    for (int32_t i = 0; i < N; i++)
        for (int v = 0; v < 3; v++) {
            const T* p = s.slots[i].p[v];
            if (p[0] != p[0] || p[1] != p[1] || p[2] != p[2]) continue;   // NaN never compares equal
            Corner c;
            for (int k = 0; k < 3; k++) c.k[k] = VKey<T>::bits(p[k]);
            c.tri = i;
            c.v = (int8_t)v;
            cs.push_back(c);
        }
    auto kless = [](const Corner& a, const Corner& b) {
        if (a.k[0] != b.k[0]) return a.k[0] < b.k[0];
        if (a.k[1] != b.k[1]) return a.k[1] < b.k[1];
        if (a.k[2] != b.k[2]) return a.k[2] < b.k[2];
        if (a.tri != b.tri) return a.tri < b.tri;
        return a.v < b.v;
    };
    std::sort(cs.begin(), cs.end(), kless);
    // group id per (tri, corner)
    std::vector<int32_t> grp((size_t)N * 3, -1);
    std::vector<int32_t> gstart;
    for (size_t a = 0; a < cs.size();) {
        size_t b = a + 1;
        while (b < cs.size() && cs[b].k[0] == cs[a].k[0] && cs[b].k[1] == cs[a].k[1] && cs[b].k[2] == cs[a].k[2]) b++;
        int32_t g = (int32_t)gstart.size();
        gstart.push_back((int32_t)a);
        for (size_t q = a; q < b; q++) grp[(size_t)cs[q].tri * 3 + cs[q].v] = g;
        a = b;
    }
    gstart.push_back((int32_t)cs.size());
    struct W { int32_t j; int8_t v, n; };
    std::vector<W> ws;
    for (int32_t i = 0; i < N; i++) {
        ws.clear();
        for (int v = 0; v < 3; v++) {
            int32_t g = grp[(size_t)i * 3 + v];
            if (g < 0) continue;
            for (int32_t q = gstart[g]; q < gstart[g + 1]; q++)
                if (cs[q].tri != i) ws.push_back({cs[q].tri, (int8_t)v, cs[q].v});
        }
        if (ws.empty()) continue;
        std::sort(ws.begin(), ws.end(), [](const W& a, const W& b) {
            if (a.j != b.j) return a.j < b.j;
            if (a.v != b.v) return a.v < b.v;
            return a.n < b.n;
        });
        Slot<T>& tp = s.slots[i];
        for (const W& w : ws) {
            Slot<T>& tn = s.slots[w.j];
            const int v = w.v, n = w.n;
            const T* a1 = tp.p[(v + 1) % 3];
            T cs_ = dot3(tp.n, tn.n) / len3(tp.n) / len3(tn.n);   // CosTheta, include/vector.h:41
            if (same_point(a1, tn.p[(n + 1) % 3])) {
                if ((double)cs_ > 0.85) { tp.nb[v] = w.j; tn.nb[n] = i; }
            } else if (same_point(a1, tn.p[(n + 2) % 3])) {
                if ((double)cs_ > 0.85) { tp.nb[v] = w.j; tn.nb[(n + 2) % 3] = i; }
            }
        }
    }
}
}  // namespace

template <typename T>
void init_radiosity(Scene<T>& s, bool links) {
    T minarea = (T)100000000.0, maxarea = (T)0.0;
    for (int32_t i = 0; i < s.trinum; i++) {
        Slot<T>& tp = s.slots[i];
        minarea = tmin(minarea, tp.area);
        maxarea = tmax(maxarea, tp.area);
        if (is_light(tp)) {
            tp.deltaB[0] = tp.deltaB[1] = tp.deltaB[2] = 0;
            const T scale = (T)s.opt.light_scale;
            for (int v = 0; v < 3; v++) {
                for (int c = 0; c < 3; c++) tp.accB[v][c] = (T)tp.Brgb[c] * scale;
                for (int c = 0; c < 3; c++) tp.deltaB[c] += 100 * tp.accB[v][c] / 3;
            }
        } else {
            std::memset(tp.accB, 0, sizeof tp.accB);
            std::memset(tp.deltaB, 0, sizeof tp.deltaB);
        }
    }
    if (links) link_neighbours(s);
    s.minarea = minarea;
    s.maxarea = maxarea;
    if (s.opt.sample_area < 0.0f) s.opt.sample_area = (float)((double)maxarea / 100.0);
    char b[512];
    const rad_options& o = s.opt;
    snprintf(b, sizeof b, "1|[\x1B[32mINFO\x1B[37m] Max Patch Area = \x1B[35m%f\n\x1B[37m", (double)maxarea); s.log += b;
    snprintf(b, sizeof b, "1|[\x1B[32mINFO\x1B[37m] Min Patch Area = \x1B[35m%f\n\x1B[37m", (double)minarea); s.log += b;
    s.log += "1|[\x1B[32mINFO\x1B[37m] Config Table\n";
    snprintf(b, sizeof b, "1|       -debug          %i\n", o.debug); s.log += b;
    snprintf(b, sizeof b, "1|       -adapt_area     %f\n", (double)o.adapt_area); s.log += b;
    snprintf(b, sizeof b, "1|       -sample_area    %f\n", (double)o.sample_area); s.log += b;
    snprintf(b, sizeof b, "1|       -converge       %f\n", (double)o.converge); s.log += b;
    snprintf(b, sizeof b, "1|       -delta_ff       %f\n", (double)o.delta_ff); s.log += b;
    snprintf(b, sizeof b, "1|       -write_cycle    %d\n", o.write_cycle); s.log += b;
    snprintf(b, sizeof b, "1|       -triangle       %d\n", o.triangle_limit); s.log += b;
    snprintf(b, sizeof b, "1|       -light          %f\n", (double)o.light_scale); s.log += b;
    snprintf(b, sizeof b, "1|       -interactive    %d\n", o.interactive); s.log += b;
    snprintf(b, sizeof b, "1|       -jobs           %d\n", o.jobs); s.log += b;
    snprintf(b, sizeof b, "1|       -parallel_src   %d\n", o.parallel_src); s.log += b;
    s.log += "1|[\x1B[32mINFO\x1B[37m] Complete initialization\n";
}

// ---------------------------------------------------------------- pre-partition
namespace {
template <typename T>
struct Pool {
    Scene<T>& s;
    int32_t limit() const { return std::min(kMaxTriPool, s.opt.triangle_limit); }
    bool full(int need) const { return s.trinum + need >= limit(); }          // shade.cpp:26-30
    int32_t alloc() {                                                          // shade.cpp:14-25
        if (s.trinum == kMaxTriPool || s.trinum == s.opt.triangle_limit) {
            if (!s.alloc_warned) {
                char b[96];
                snprintf(b, sizeof b, "2|\n**** Max Triangle exceed : %i ***\n", s.trinum);
                s.log += b;
                s.alloc_warned = true;
            }
            return -1;
        }
        if ((size_t)s.trinum >= s.slots.size()) s.slots.resize(s.slots.size() * 2 + 8);
        return s.trinum++;
    }
    void release() { s.trinum--; }                                             // shade.cpp:11-13
};

template <typename T>
void relink(Scene<T>& s, int32_t nb, int32_t old_id, int32_t new_id) {      // shade.cpp:33-43
    if (nb < 0) return;
    for (int v = 0; v < 3; v++)
        if (s.slots[nb].nb[v] == old_id) s.slots[nb].nb[v] = new_id;
}

// PartitionDestination (2-way), shade.cpp:171-211.  Only the fields the
// reference writes are written; the rest keep the target slot's old contents.
template <typename T>
void bisect(const Slot<T>& s, Slot<T>& t1, Slot<T>& t2, int e) {
    const int i0 = e, i1 = (e + 1) % 3, i2 = (e + 2) % 3;
    T m[3], a[3];
    for (int k = 0; k < 3; k++) m[k] = (T)((double)(s.p[i0][k] + s.p[i1][k]) / 2.0);
    for (int k = 0; k < 3; k++) a[k] = (T)((double)(s.accB[i0][k] + s.accB[i1][k]) / 2.0);
    const Slot<T> src = s;   // t1/t2 never alias s, but keep the read set explicit
    for (int k = 0; k < 3; k++) {
        t1.p[0][k] = m[k]; t1.p[1][k] = src.p[i2][k]; t1.p[2][k] = src.p[i0][k];
        t1.n[k] = src.n[k]; t1.Frgb[k] = src.Frgb[k]; t1.deltaB[k] = src.deltaB[k];
        t2.p[0][k] = m[k]; t2.p[1][k] = src.p[i1][k]; t2.p[2][k] = src.p[i2][k];
        t2.n[k] = src.n[k]; t2.Frgb[k] = src.Frgb[k]; t2.deltaB[k] = src.deltaB[k];
        t1.accB[0][k] = a[k]; t1.accB[1][k] = src.accB[i2][k]; t1.accB[2][k] = src.accB[i0][k];
        t2.accB[0][k] = a[k]; t2.accB[1][k] = src.accB[i1][k]; t2.accB[2][k] = src.accB[i2][k];
    }
    centre(t1.p, t1.c);
    centre(t2.p, t2.c);
    t1.area = t2.area = (T)((double)src.area / 2.0);
    t1.parent = t2.parent = src.parent;
}

// PartitionTriangleAndStore, shade.cpp:311-431.  out[] receives the slot ids
// of t1..t4 (-1 where not created).
template <typename T>
int split_and_store(Scene<T>& sc, Pool<T>& pool, int32_t sid, int32_t out[4], bool& reshade,
                    int32_t* nbid_out = nullptr) {
    reshade = false;
    out[0] = out[1] = out[2] = out[3] = -1;
    if (nbid_out) *nbid_out = -1;
    if (pool.full(4) || (double)sc.slots[sid].area < 1e-8) return -1;
    int e = 0;
    {
        T longest = 0;
        const Slot<T>& s = sc.slots[sid];
        for (int v = 0; v < 3; v++) {
            T l[3];
            edge(s.p[v], s.p[(v + 1) % 3], l);
            T len = dot3(l, l);
            if (longest < len) { longest = len; e = v; }
        }
        if (longest < 1) return -1;
        int32_t nbid = s.nb[e];
        if (nbid >= 0 && (double)sc.slots[nbid].area < 1e-1) return -1;
    }
    int32_t id1 = pool.alloc(), id2 = pool.alloc();
    const int32_t nbid = sc.slots[sid].nb[e];
    if (nbid_out) *nbid_out = nbid;
    bisect(sc.slots[sid], sc.slots[id1], sc.slots[id2], e);
    int32_t n1, n2;
    sc.slots[id1].nb[1] = n1 = sc.slots[sid].nb[(e + 2) % 3];
    sc.slots[id2].nb[1] = n2 = sc.slots[sid].nb[(e + 1) % 3];
    sc.slots[id1].nb[2] = sc.slots[id2].nb[0] = -1;
    int replaced = 0;
    if (sc.slots[sid].parent == sid) {
        sc.slots[sid].parent = -1;
    } else {
        sc.slots[sid] = sc.slots[id2];
        id2 = sid;
        pool.release();
        replaced = 1;
    }
    relink(sc, n1, sid, id1);
    relink(sc, n2, sid, id2);
    sc.slots[id1].nb[0] = id2;
    sc.slots[id2].nb[2] = id1;
    out[0] = id1;
    out[1] = id2;
    if (nbid < 0) return replaced;

    int32_t id3 = pool.alloc(), id4 = pool.alloc();
    int ne = 0;
    for (int v = 0; v < 3; v++)
        if (sc.slots[nbid].nb[v] == sid) ne = v;
    if (nbid < sid) {
        Slot<T>& nt = sc.slots[nbid];
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) nt.accB[v][k] -= nt.daccB[v][k];
    }
    bisect(sc.slots[nbid], sc.slots[id3], sc.slots[id4], ne);
    sc.slots[id3].nb[1] = n1 = sc.slots[nbid].nb[(ne + 2) % 3];
    sc.slots[id4].nb[1] = n2 = sc.slots[nbid].nb[(ne + 1) % 3];
    if (sc.slots[nbid].parent == nbid) {
        sc.slots[nbid].parent = -1;
    } else {
        sc.slots[nbid] = sc.slots[id4];
        id4 = nbid;
        pool.release();
    }
    relink(sc, n1, nbid, id3);
    relink(sc, n2, nbid, id4);
    sc.slots[id3].nb[0] = id4;
    sc.slots[id4].nb[2] = id3;
    // shade.cpp:416 compares the addresses of two vertex arrays, which are
    // equal only for the same slot and edge
    if (sid == nbid && e == ne) {
        sc.slots[id1].nb[2] = id3; sc.slots[id3].nb[2] = id1;
        sc.slots[id2].nb[0] = id4; sc.slots[id4].nb[0] = id2;
    } else {
        sc.slots[id1].nb[2] = id4; sc.slots[id4].nb[0] = id1;
        sc.slots[id2].nb[0] = id3; sc.slots[id3].nb[2] = id2;
    }
    if (id4 < sid) reshade = true;
    out[2] = id3;
    out[3] = id4;
    return replaced;
}
}  // namespace

template <typename T>
int split_receiver(Scene<T>& s, int32_t sid, int32_t out[4], bool& reshade, int32_t* nbid) {
    Pool<T> pool{s};
    return split_and_store(s, pool, sid, out, reshade, nbid);
}
template int split_receiver<float>(Scene<float>&, int32_t, int32_t*, bool&, int32_t*);
template int split_receiver<double>(Scene<double>&, int32_t, int32_t*, bool&, int32_t*);

template <typename T>
bool pool_full(const Scene<T>& s, int need) {
    return s.trinum + need >= std::min(kMaxTriPool, s.opt.triangle_limit);
}
template bool pool_full<float>(const Scene<float>&, int);
template bool pool_full<double>(const Scene<double>&, int);

template <typename T>
void prepartition(Scene<T>& s) {
    char b[128];
    snprintf(b, sizeof b, "2|[\x1B[31mDEBUG\x1B[37m] Before PrePartitionTriangle %d\n", s.trinum);
    s.log += b;
    Pool<T> pool{s};
    std::set<std::pair<T, int32_t>> S;
    for (int32_t i = 0; i < s.trinum; i++) {
        const Slot<T>& t = s.slots[i];
        if (t.area < 1.f || is_light(t)) continue;
        S.insert(std::make_pair(t.area, i));
    }
    while (!S.empty()) {
        auto top = *S.rbegin();
        S.erase(top);
        const int32_t sid = top.second;
        if (s.slots[sid].area < 1) break;
        int32_t out[4];
        bool reshade;
        if (split_and_store(s, pool, sid, out, reshade) < 0) break;
        if (is_light(s.slots[sid])) {
            const Slot<T> tp = s.slots[sid];
            for (int q = 0; q < 4; q++) {
                if (out[q] < 0 || out[q] == sid) continue;
                Slot<T>& c = s.slots[out[q]];
                for (int k = 0; k < 3; k++) c.Brgb[k] = tp.Brgb[k];
                for (int v = 0; v < 3; v++) {
                    for (int k = 0; k < 3; k++) c.accB[v][k] = tp.accB[v][k];
                    c.deltaB[v] = tp.deltaB[v];
                }
            }
        }
        for (int q = 0; q < 4; q++)
            if (out[q] >= 0) S.insert(std::make_pair(s.slots[out[q]].area, out[q]));
    }
    snprintf(b, sizeof b, "2|[\x1B[31mDEBUG\x1B[37m] After PrePartitionTriangle %d\n", s.trinum);
    s.log += b;
}

// ---------------------------------------------------------------- output
template <typename T>
int write_fin(const Scene<T>& s, const char* prefix, int loop, std::string& err) {
    std::string fn(prefix);
    char tail[32];
    if (loop == 0) snprintf(tail, sizeof tail, ".fin");
    else snprintf(tail, sizeof tail, ".%1d", loop);
    fn += tail;
    FILE* f = std::fopen(fn.c_str(), "w");
    bool to_stdout = false;
    if (!f) {
        err = "Error: output file " + fn + " open failed";
        if (loop != 0) return RAD_ERR_IO;
        f = stdout;
        to_stdout = true;
    }
    // the reference formats through one static buffer that a non-convertible
    // value leaves untouched; keep that state across calls the same way
    static thread_local char fbuf[64] = {0};
    std::string out;
    out.reserve((size_t)s.trinum * 160);
    char line[192];
    for (int32_t i = 0; i < s.trinum; i++) {
        const Slot<T>& t = s.slots[i];
        if (t.parent < 0) continue;
        out += "Triangle \n";
        int col[3];
        for (int j = 0; j < 3; j++) {
            T v = 0;
            for (int k = 0; k < 3; k++) v += t.accB[k][j];
            v /= 3;
            v = ((T)255.0 < v) ? (T)255.0 : v;
            v = (v < (T)0.0) ? (T)0.0 : v;
            if (std::isnan(v)) v = 0;
            col[j] = (int)v;
        }
        snprintf(line, sizeof line, "%d %d %d 0 0 0\n", col[0], col[1], col[2]);
        out += line;
        std::string nrm;
        for (int k = 0; k < 3; k++) {
            format_float((float)t.n[k], fbuf);
            nrm += fbuf;
            nrm += (k < 2) ? " " : "\n";
        }
        for (int j = 0; j < 3; j++) {
            for (int k = 0; k < 3; k++) {
                format_float((float)t.p[j][k], fbuf);
                out += fbuf;
                out += ' ';
            }
            out += nrm;
        }
    }
    std::fwrite(out.data(), 1, out.size(), f);
    if (!to_stdout) std::fclose(f);
    else std::fflush(f);
    return RAD_OK;
}

template int load_tri_text<float>(const char*, size_t, const rad_options&, Scene<float>&, std::string&);
template int load_tri_text<double>(const char*, size_t, const rad_options&, Scene<double>&, std::string&);
template int load_arrays<float>(const float*, const int32_t*, const int32_t*, int32_t, const rad_options&, Scene<float>&, std::string&);
template int load_arrays<double>(const float*, const int32_t*, const int32_t*, int32_t, const rad_options&, Scene<double>&, std::string&);
template void init_radiosity<float>(Scene<float>&, bool);
template void init_radiosity<double>(Scene<double>&, bool);
template void prepartition<float>(Scene<float>&);
template void prepartition<double>(Scene<double>&);
template int write_fin<float>(const Scene<float>&, const char*, int, std::string&);
template int write_fin<double>(const Scene<double>&, const char*, int, std::string&);

}  // namespace radgb
