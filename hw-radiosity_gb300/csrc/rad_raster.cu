// Headless rendering of a result the way the reference's WebGL viewer shows
// it (WebGL_demo/public/index.html with lib/flat.*, lib/gouraud.*), into an
// RGBA8 buffer: no graphics API, a tiled CUDA rasteriser.
//
// Input preparation restates the model converter
// (WebGL_demo/model-converter/main.cpp:167-246, writeColorfulJson 81-150):
// the .fin triangles are read as doubles, the model is scaled so its longest
// side is 10 and shifted by -5, and every position, normal and colour/255
// goes through "%g" and float32, as the JSON and the browser's Float32Array
// do.  Every vertex of a triangle carries the triangle's colour.
//
// The view is the viewer's initial state: a 1024x768 canvas,
// perspective(45 deg, aspect, 0.1, 100), the eye translated by (0, 0, -40),
// the model by (0, 5, 10), then xRot about x and yRot about y (0 by default);
// ambient 0.2, specular and diffuse 0.8, shininess 32, three point lights at
// (-10, 4, -20), (90, -80, -60), (100, 40, -200) in eye space, clear colour
// (0, 0.2, 0.2), depth test LESS.  Flat shading (the viewer's default)
// lights every fragment with the face normal; Gouraud lights the vertices
// and interpolates the colours.
//
// Pipeline (one render): k_vertex transforms and lights the three vertices
// of each triangle and counts the 16x16 tiles its box touches; k_scan turns
// the counts into list offsets; k_bin writes the triangle into each tile's
// list; k_fine runs one CTA per tile, one thread per pixel: the thread keeps
// the smallest (depth, triangle index) over the tile's triangles, which is
// GL's LESS test in draw order, then shades the winner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "capi_internal.h"

namespace radgb {
namespace raster {

constexpr int kTile = 16;

// ------------------------------------------------------------------ host: input
struct FinTri {
    double fc[3];
    double v[3][3];
    double n[3][3];
};

// the viewer's vertex arrays: 9 floats per triangle in each
struct Mesh {
    std::vector<float> pos, nrm, col;
    int n = 0;
};

// the next line of a text held in memory (without its '\n'), as getline
struct Lines {
    const char* p;
    const char* end;
    bool next(const char*& b, const char*& e) {
        if (p >= end) return false;
        b = p;
        while (p < end && *p != '\n') ++p;
        e = p;
        if (p < end) ++p;
        return true;
    }
};

// six numbers from one line, as the converter's readLine (stringstream >> double)
static bool six(const char* b, const char* e, double f[6]) {
    char buf[512];
    const size_t n = std::min((size_t)(e - b), sizeof buf - 1);
    std::memcpy(buf, b, n);
    buf[n] = 0;
    const char* p = buf;
    for (int i = 0; i < 6; i++) {
        char* q = nullptr;
        f[i] = std::strtod(p, &q);
        if (q == p) return false;
        p = q;
    }
    return true;
}

static int parse_fin(const char* path, std::vector<FinTri>& out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(RAD_ERR_IO, std::string("cannot open ") + path);
    std::string text;
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) text.append(chunk, got);
    std::fclose(f);
    Lines L{text.data(), text.data() + text.size()};
    const char *b, *e;
    while (L.next(b, e)) {
        if (std::string(b, e) != "Triangle ") return fail(RAD_ERR_PARSE, "a .fin record must start with \"Triangle \"");
        FinTri t;
        double v[6];
        if (!L.next(b, e) || !six(b, e, v)) return fail(RAD_ERR_PARSE, "bad colour line in .fin");
        for (int i = 0; i < 3; i++) t.fc[i] = v[i];
        for (int k = 0; k < 3; k++) {
            if (!L.next(b, e) || !six(b, e, v)) return fail(RAD_ERR_PARSE, "bad vertex line in .fin");
            for (int i = 0; i < 3; i++) { t.v[k][i] = v[i]; t.n[k][i] = v[i + 3]; }
        }
        out.push_back(t);
    }
    return RAD_OK;
}

// the same triangles from a scene in memory: what write_fin prints, read back
template <typename T>
static void tris_from_scene(const Scene<T>& s, std::vector<FinTri>& out) {
    for (int32_t i = 0; i < s.trinum; i++) {
        const Slot<T>& t = s.slots[i];
        if (t.parent < 0) continue;
        FinTri r;
        for (int j = 0; j < 3; j++) {
            T v = 0;
            for (int k = 0; k < 3; k++) v += t.accB[k][j];
            v /= 3;
            v = ((T)255.0 < v) ? (T)255.0 : v;
            v = (v < (T)0.0) ? (T)0.0 : v;
            if (std::isnan(v)) v = 0;
            r.fc[j] = (double)(int)v;
        }
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++) {
                r.v[k][j] = (double)(float)t.p[k][j];
                r.n[k][j] = (double)(float)t.n[j];
            }
        out.push_back(r);
    }
}

// "%g" then float32, as the JSON text and the browser's Float32Array
static inline float via_g(double x) {
    char b[40];
    std::snprintf(b, sizeof b, "%g", x);
    return (float)std::strtod(b, nullptr);
}

static void convert(const std::vector<FinTri>& in, Mesh& m) {
    const size_t n = in.size();
    m.n = (int)n;
    m.pos.assign(n * 9, 0.f);
    m.nrm.assign(n * 9, 0.f);
    m.col.assign(n * 9, 0.f);
    if (n == 0) return;
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) lo[k] = hi[k] = in[0].v[0][k];
    for (const FinTri& t : in)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], t.v[j][k]);
                hi[k] = std::max(hi[k], t.v[j][k]);
            }
    const double max_side = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    const double view_scale = 10.0;
    const double scale = view_scale / max_side;
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nt; w++)
        th.emplace_back([&, w] {
            for (size_t i = w; i < n; i += nt) {
                const FinTri& t = in[i];
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++) {
                        double v = t.v[j][k];
                        v -= lo[k];
                        v *= scale;
                        v -= 0.5 * view_scale;
                        m.pos[i * 9 + j * 3 + k] = via_g(v);
                        m.nrm[i * 9 + j * 3 + k] = via_g(t.n[j][k]);
                        m.col[i * 9 + j * 3 + k] = via_g(t.fc[k] / 255.0);
                    }
            }
        });
    for (auto& t : th) t.join();
}

// ------------------------------------------------------------------ view
struct Uniforms {
    float P[16], MV[16], N[9];   // column-major, as GL
    float ambient[3], spec[3], diff[3];
    float light[3][3];
    float shininess;
    int width, height, shading;  // 0 flat, 1 gouraud
};

static void mat_mul(const double* a, const double* b, double* o) {   // o = a * b, column-major 4x4
    double r[16];
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a[k * 4 + rr] * b[c * 4 + k];
            r[c * 4 + rr] = s;
        }
    std::memcpy(o, r, sizeof r);
}

static void make_uniforms(const rad_render_options& o, Uniforms& u) {
    const double pi = 3.14159265358979323846;
    const double W = o.width, H = o.height;
    double P[16] = {0};
    const double near = 0.1, far = 100.0;
    const double top = near * std::tan(45.0 * pi / 360.0), right = top * (W / H);
    P[0] = 2 * near / (2 * right);
    P[5] = 2 * near / (2 * top);
    P[10] = -(far + near) / (far - near);
    P[11] = -1;
    P[14] = -(far * near * 2) / (far - near);
    auto ident = [](double* m) { std::memset(m, 0, 16 * sizeof(double)); m[0] = m[5] = m[10] = m[15] = 1; };
    double M[16], T[16];
    ident(M);
    ident(T); T[12] = 0; T[13] = 0; T[14] = -40; mat_mul(M, T, M);
    ident(T); T[12] = 0; T[13] = 5; T[14] = 10; mat_mul(M, T, M);
    const double ax = o.x_rot * pi / 180.0, ay = o.y_rot * pi / 180.0;
    ident(T); T[5] = std::cos(ax); T[6] = std::sin(ax); T[9] = -std::sin(ax); T[10] = std::cos(ax); mat_mul(M, T, M);
    ident(T); T[0] = std::cos(ay); T[2] = -std::sin(ay); T[8] = std::sin(ay); T[10] = std::cos(ay); mat_mul(M, T, M);
    // normal matrix: transpose of the inverse of the upper 3x3
    const double a = M[0], b = M[4], c = M[8], d = M[1], e = M[5], f = M[9], g = M[2], h = M[6], i = M[10];
    const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    const double inv[9] = {(e * i - f * h) / det, (c * h - b * i) / det, (b * f - c * e) / det,
                           (f * g - d * i) / det, (a * i - c * g) / det, (c * d - a * f) / det,
                           (d * h - e * g) / det, (b * g - a * h) / det, (a * e - b * d) / det};   // row-major inverse
    // GL column-major N = transpose(inverse): element (r, c) of N is inv(c, r); stored column-major
    for (int cc = 0; cc < 3; cc++)
        for (int r = 0; r < 3; r++) u.N[cc * 3 + r] = (float)inv[cc * 3 + r];
    for (int k = 0; k < 16; k++) { u.P[k] = (float)P[k]; u.MV[k] = (float)M[k]; }
    for (int k = 0; k < 3; k++) { u.ambient[k] = 0.2f; u.spec[k] = 0.8f; u.diff[k] = 0.8f; }
    const float L[3][3] = {{-10.f, 4.f, -20.f}, {90.f, -80.f, -60.f}, {100.f, 40.f, -200.f}};
    std::memcpy(u.light, L, sizeof L);
    u.shininess = 32.f;
    u.width = o.width;
    u.height = o.height;
    u.shading = o.shading;
}

// ------------------------------------------------------------------ device math
struct V3 { float x, y, z; };
__host__ __device__ inline V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
__host__ __device__ inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline V3 sub3(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline V3 scl3(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ inline V3 norm3(V3 a) {
    const float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return v3(a.x / l, a.y / l, a.z / l);
}
__host__ __device__ inline V3 cross3(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// GLSL reflect(I, N) = I - 2 dot(N, I) N
__host__ __device__ inline V3 reflect3(V3 i, V3 n) { return sub3(i, scl3(n, 2.f * dot3(n, i))); }
// pow(x, 32): five squarings
__host__ __device__ inline float pow32(float x) {
    x = x * x; x = x * x; x = x * x; x = x * x; return x * x;
}
// ambient + specular + diffuse of the three lights (the shaders' loop body)
__host__ __device__ inline V3 light_weight(const Uniforms& u, V3 normal, V3 eye, const V3* ldir) {
    V3 w = v3(0.f, 0.f, 0.f);
    for (int i = 0; i < 3; i++) {
        const V3 r = reflect3(v3(-ldir[i].x, -ldir[i].y, -ldir[i].z), normal);
        const float rd = dot3(r, eye);
        const float spec = pow32(rd > 0.f ? rd : 0.f);
        const float nd = dot3(normal, ldir[i]);
        const float diff = nd > 0.f ? nd : 0.f;
        w.x = w.x + (u.ambient[0] + u.spec[0] * spec + u.diff[0] * diff);
        w.y = w.y + (u.ambient[1] + u.spec[1] * spec + u.diff[1] * diff);
        w.z = w.z + (u.ambient[2] + u.spec[2] * spec + u.diff[2] * diff);
    }
    return w;
}

// per triangle, after setup (window space, counter-clockwise)
struct TriRaster {
    float sx[3], sy[3], sz[3], iw[3];
    float area;
    int x0, y0, x1, y1;   // pixel box, inclusive; x1 < x0 when the triangle is dropped
};
// varyings per vertex: flat = view position (3), the three light directions
// (9), the colour (3); gouraud = the lit colour (3).  tn: flat's face normal
struct TriShade {
    float vary[3][15];
    float tn[3];
};

__device__ inline bool top_left(float ax, float ay, float bx, float by) {
    return (ay == by && bx < ax) || (by < ay);
}

__global__ void k_vertex(Uniforms u, int n, const float* __restrict__ pos, const float* __restrict__ nrm,
                         const float* __restrict__ col, TriRaster* tr, TriShade* ts, int* tile_count, int tiles_x) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    V3 vp[3], vn[3];
    float cx[3], cy[3], cz[3], cw[3];
    bool ok = true;
    for (int k = 0; k < 3; k++) {
        const float x = pos[t * 9 + k * 3], y = pos[t * 9 + k * 3 + 1], z = pos[t * 9 + k * 3 + 2];
        const float* M = u.MV;
        vp[k] = v3(M[0] * x + M[4] * y + M[8] * z + M[12], M[1] * x + M[5] * y + M[9] * z + M[13],
                   M[2] * x + M[6] * y + M[10] * z + M[14]);
        const float* P = u.P;
        cx[k] = P[0] * vp[k].x + P[4] * vp[k].y + P[8] * vp[k].z + P[12];
        cy[k] = P[1] * vp[k].x + P[5] * vp[k].y + P[9] * vp[k].z + P[13];
        cz[k] = P[2] * vp[k].x + P[6] * vp[k].y + P[10] * vp[k].z + P[14];
        cw[k] = P[3] * vp[k].x + P[7] * vp[k].y + P[11] * vp[k].z + P[15];
        const float nx = nrm[t * 9 + k * 3], ny = nrm[t * 9 + k * 3 + 1], nz = nrm[t * 9 + k * 3 + 2];
        const float* N = u.N;
        vn[k] = v3(N[0] * nx + N[3] * ny + N[6] * nz, N[1] * nx + N[4] * ny + N[7] * nz,
                   N[2] * nx + N[5] * ny + N[8] * nz);
        ok &= cw[k] > 0.f;
    }
    TriRaster r;
    int ord[3] = {0, 1, 2};
    r.x0 = 0; r.x1 = -1; r.y0 = 0; r.y1 = -1;
    if (ok) {
        for (int k = 0; k < 3; k++) {
            r.sx[k] = (cx[k] / cw[k] + 1.f) * 0.5f * (float)u.width;
            r.sy[k] = (cy[k] / cw[k] + 1.f) * 0.5f * (float)u.height;
            r.sz[k] = (cz[k] / cw[k] + 1.f) * 0.5f;
            r.iw[k] = 1.f / cw[k];
        }
        float area = (r.sx[1] - r.sx[0]) * (r.sy[2] - r.sy[0]) - (r.sy[1] - r.sy[0]) * (r.sx[2] - r.sx[0]);
        if (area < 0.f) {     // counter-clockwise on screen: swap vertices 1 and 2
            ord[1] = 2; ord[2] = 1;
            float tmp;
            tmp = r.sx[1]; r.sx[1] = r.sx[2]; r.sx[2] = tmp;
            tmp = r.sy[1]; r.sy[1] = r.sy[2]; r.sy[2] = tmp;
            tmp = r.sz[1]; r.sz[1] = r.sz[2]; r.sz[2] = tmp;
            tmp = r.iw[1]; r.iw[1] = r.iw[2]; r.iw[2] = tmp;
            area = -area;
        }
        r.area = area;
        if (area > 0.f) {
            const float mnx = fminf(fminf(r.sx[0], r.sx[1]), r.sx[2]), mxx = fmaxf(fmaxf(r.sx[0], r.sx[1]), r.sx[2]);
            const float mny = fminf(fminf(r.sy[0], r.sy[1]), r.sy[2]), mxy = fmaxf(fmaxf(r.sy[0], r.sy[1]), r.sy[2]);
            if (mxx >= 0.f && mny < (float)u.height && mxy >= 0.f && mnx < (float)u.width) {
                r.x0 = max(0, (int)floorf(mnx));
                r.x1 = min(u.width - 1, (int)ceilf(mxx));
                r.y0 = max(0, (int)floorf(mny));
                r.y1 = min(u.height - 1, (int)ceilf(mxy));
            }
        }
    }
    tr[t] = r;
    if (r.x1 < r.x0 || r.y1 < r.y0) return;
    // varyings in the window-space vertex order
    TriShade s;
    for (int k = 0; k < 3; k++) {
        const int o = ord[k];
        const V3 cc = v3(col[t * 9 + o * 3], col[t * 9 + o * 3 + 1], col[t * 9 + o * 3 + 2]);
        V3 ld[3];
        for (int i = 0; i < 3; i++) ld[i] = norm3(sub3(v3(u.light[i][0], u.light[i][1], u.light[i][2]), vp[o]));
        if (u.shading == 1) {
            const V3 normal = norm3(vn[o]);
            const V3 eye = norm3(v3(-vp[o].x, -vp[o].y, -vp[o].z));
            const V3 w = light_weight(u, normal, eye, ld);
            s.vary[k][0] = cc.x * w.x; s.vary[k][1] = cc.y * w.y; s.vary[k][2] = cc.z * w.z;
        } else {
            s.vary[k][0] = vp[o].x; s.vary[k][1] = vp[o].y; s.vary[k][2] = vp[o].z;
            for (int i = 0; i < 3; i++) { s.vary[k][3 + 3 * i] = ld[i].x; s.vary[k][4 + 3 * i] = ld[i].y; s.vary[k][5 + 3 * i] = ld[i].z; }
            s.vary[k][12] = cc.x; s.vary[k][13] = cc.y; s.vary[k][14] = cc.z;
        }
    }
    // flat: the face normal of the view-space triangle in window order (it faces the eye)
    s.tn[0] = s.tn[1] = s.tn[2] = 0.f;
    if (u.shading == 0) {
        const V3 n = norm3(cross3(sub3(vp[ord[1]], vp[ord[0]]), sub3(vp[ord[2]], vp[ord[0]])));
        s.tn[0] = n.x; s.tn[1] = n.y; s.tn[2] = n.z;
    }
    ts[t] = s;
    for (int ty = r.y0 / kTile; ty <= r.y1 / kTile; ty++)
        for (int tx = r.x0 / kTile; tx <= r.x1 / kTile; tx++) atomicAdd(&tile_count[ty * tiles_x + tx], 1);
}

// exclusive scan of the tile counts (one CTA)
__global__ void k_scan(const int* count, int* start, int* cursor, int n, int* total) {
    __shared__ int part[1024];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(n, b + per);
    int s = 0;
    for (int i = b; i < e; i++) s += count[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int i = 0; i < (int)blockDim.x; i++) { const int v = part[i]; part[i] = acc; acc += v; }
        *total = acc;
    }
    __syncthreads();
    int acc = part[threadIdx.x];
    for (int i = b; i < e; i++) { start[i] = acc; cursor[i] = acc; acc += count[i]; }
}

__global__ void k_bin(int n, const TriRaster* tr, int* cursor, int* list, int tiles_x) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const TriRaster r = tr[t];
    if (r.x1 < r.x0 || r.y1 < r.y0) return;
    for (int ty = r.y0 / kTile; ty <= r.y1 / kTile; ty++)
        for (int tx = r.x0 / kTile; tx <= r.x1 / kTile; tx++) list[atomicAdd(&cursor[ty * tiles_x + tx], 1)] = t;
}

// screen-space barycentrics of pixel centre (px, py); false when outside
// (edge values of zero count only on top and left edges)
__device__ inline bool cover(const TriRaster& r, float px, float py, float& b0, float& b1, float& b2) {
    const float w0 = (r.sx[2] - r.sx[1]) * (py - r.sy[1]) - (r.sy[2] - r.sy[1]) * (px - r.sx[1]);
    const float w1 = (r.sx[0] - r.sx[2]) * (py - r.sy[2]) - (r.sy[0] - r.sy[2]) * (px - r.sx[2]);
    const float w2 = (r.sx[1] - r.sx[0]) * (py - r.sy[0]) - (r.sy[1] - r.sy[0]) * (px - r.sx[0]);
    if (w0 < 0.f || w1 < 0.f || w2 < 0.f) return false;
    if (w0 == 0.f && !top_left(r.sx[1], r.sy[1], r.sx[2], r.sy[2])) return false;
    if (w1 == 0.f && !top_left(r.sx[2], r.sy[2], r.sx[0], r.sy[0])) return false;
    if (w2 == 0.f && !top_left(r.sx[0], r.sy[0], r.sx[1], r.sy[1])) return false;
    b0 = w0 / r.area;
    b1 = w1 / r.area;
    b2 = w2 / r.area;
    return true;
}

__device__ inline unsigned char to8(float c) {
    c = c < 0.f ? 0.f : (c > 1.f ? 1.f : c);
    return (unsigned char)(int)(c * 255.f + 0.5f);
}

__global__ void __launch_bounds__(kTile * kTile) k_fine(Uniforms u, const TriRaster* __restrict__ tr,
                                                        const TriShade* __restrict__ ts, const int* __restrict__ start,
                                                        const int* __restrict__ count, const int* __restrict__ list,
                                                        int tiles_x, unsigned char* rgba) {
    const int tile = blockIdx.x;
    const int x = (tile % tiles_x) * kTile + (int)(threadIdx.x % kTile);
    const int y = (tile / tiles_x) * kTile + (int)(threadIdx.x / kTile);
    const bool in = x < u.width && y < u.height;
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    float bz = 2.f;
    int bt = -1;
    const int b = start[tile], e = b + count[tile];
    for (int k = b; k < e; k++) {
        const int t = list[k];
        const TriRaster& r = tr[t];
        float b0, b1, b2;
        if (!in || x < r.x0 || x > r.x1 || y < r.y0 || y > r.y1 || !cover(r, px, py, b0, b1, b2)) continue;
        const float z = b0 * r.sz[0] + b1 * r.sz[1] + b2 * r.sz[2];
        if (!(z >= 0.f && z <= 1.f)) continue;
        if (z < bz || (z == bz && t < bt)) { bz = z; bt = t; }
    }
    if (!in) return;
    unsigned char* o = rgba + ((size_t)(u.height - 1 - y) * u.width + x) * 4;
    if (bt < 0) {
        o[0] = to8(0.f); o[1] = to8(0.2f); o[2] = to8(0.2f); o[3] = 255;
        return;
    }
    const TriRaster r = tr[bt];
    float b0, b1, b2;
    cover(r, px, py, b0, b1, b2);
    const float q0 = b0 * r.iw[0], q1 = b1 * r.iw[1], q2 = b2 * r.iw[2];
    const float qs = q0 + q1 + q2;
    const TriShade& s = ts[bt];
    float a[15];
    const int na = u.shading == 1 ? 3 : 15;
    for (int i = 0; i < na; i++) a[i] = (q0 * s.vary[0][i] + q1 * s.vary[1][i] + q2 * s.vary[2][i]) / qs;
    float cr, cg, cb;
    if (u.shading == 1) {
        cr = a[0]; cg = a[1]; cb = a[2];
    } else {
        const V3 tn = v3(s.tn[0], s.tn[1], s.tn[2]);
        const V3 eye = norm3(v3(-a[0], -a[1], -a[2]));
        const V3 ld[3] = {v3(a[3], a[4], a[5]), v3(a[6], a[7], a[8]), v3(a[9], a[10], a[11])};
        const V3 w = light_weight(u, tn, eye, ld);
        cr = a[12] * w.x; cg = a[13] * w.y; cb = a[14] * w.z;
    }
    o[0] = to8(cr); o[1] = to8(cg); o[2] = to8(cb); o[3] = 255;
}

}  // namespace raster
}  // namespace radgb

// ==================================================================== host
using namespace radgb;
using namespace radgb::raster;

namespace {

#define CUR(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            rc = fail(RAD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
            goto done;                                                                    \
        }                                                                                 \
    } while (0)

int check_options(const rad_render_options* o) {
    if (!o) return fail(RAD_ERR_ARG, "render: null options");
    if (o->width < 1 || o->height < 1 || o->width > 16384 || o->height > 16384)
        return fail(RAD_ERR_CAPACITY, "render: width and height must be 1..16384");
    if (o->shading != 0 && o->shading != 1) return fail(RAD_ERR_ARG, "render: shading must be 0 (flat) or 1 (gouraud)");
    return RAD_OK;
}

int render(const std::vector<FinTri>& tris, const rad_render_options& o, int device, uint8_t* rgba) {
    Mesh m;
    convert(tris, m);
    Uniforms u;
    make_uniforms(o, u);
    const int tiles_x = (o.width + kTile - 1) / kTile, tiles_y = (o.height + kTile - 1) / kTile;
    const int n_tiles = tiles_x * tiles_y;
    const size_t img = (size_t)o.width * o.height * 4;
    int rc = RAD_OK;
    cudaStream_t st = nullptr;
    float *d_pos = nullptr, *d_nrm = nullptr, *d_col = nullptr;
    TriRaster* d_tr = nullptr;
    TriShade* d_ts = nullptr;
    int *d_count = nullptr, *d_start = nullptr, *d_cursor = nullptr, *d_total = nullptr, *d_list = nullptr;
    unsigned char* d_img = nullptr;
    int total = 0;
    const size_t nt = (size_t)std::max(m.n, 1);
    CUR(cudaSetDevice(device));
    CUR(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CUR(cudaMallocAsync(&d_pos, nt * 9 * 4, st));
    CUR(cudaMallocAsync(&d_nrm, nt * 9 * 4, st));
    CUR(cudaMallocAsync(&d_col, nt * 9 * 4, st));
    CUR(cudaMallocAsync(&d_tr, nt * sizeof(TriRaster), st));
    CUR(cudaMallocAsync(&d_ts, nt * sizeof(TriShade), st));
    CUR(cudaMallocAsync(&d_count, (size_t)n_tiles * 4, st));
    CUR(cudaMallocAsync(&d_start, (size_t)n_tiles * 4, st));
    CUR(cudaMallocAsync(&d_cursor, (size_t)n_tiles * 4, st));
    CUR(cudaMallocAsync(&d_total, 4, st));
    CUR(cudaMallocAsync(&d_img, img, st));
    CUR(cudaMemsetAsync(d_count, 0, (size_t)n_tiles * 4, st));
    if (m.n > 0) {
        CUR(cudaMemcpyAsync(d_pos, m.pos.data(), (size_t)m.n * 36, cudaMemcpyHostToDevice, st));
        CUR(cudaMemcpyAsync(d_nrm, m.nrm.data(), (size_t)m.n * 36, cudaMemcpyHostToDevice, st));
        CUR(cudaMemcpyAsync(d_col, m.col.data(), (size_t)m.n * 36, cudaMemcpyHostToDevice, st));
        k_vertex<<<(m.n + 127) / 128, 128, 0, st>>>(u, m.n, d_pos, d_nrm, d_col, d_tr, d_ts, d_count, tiles_x);
        CUR(cudaGetLastError());
    }
    k_scan<<<1, 1024, 0, st>>>(d_count, d_start, d_cursor, n_tiles, d_total);
    CUR(cudaGetLastError());
    CUR(cudaMemcpyAsync(&total, d_total, 4, cudaMemcpyDeviceToHost, st));
    CUR(cudaStreamSynchronize(st));
    if (total < 0) { rc = fail(RAD_ERR_CAPACITY, "render: too many tile entries"); goto done; }
    CUR(cudaMallocAsync(&d_list, (size_t)std::max(total, 1) * 4, st));
    if (m.n > 0) {
        k_bin<<<(m.n + 127) / 128, 128, 0, st>>>(m.n, d_tr, d_cursor, d_list, tiles_x);
        CUR(cudaGetLastError());
    }
    k_fine<<<n_tiles, kTile * kTile, 0, st>>>(u, d_tr, d_ts, d_start, d_count, d_list, tiles_x, d_img);
    CUR(cudaGetLastError());
    CUR(cudaMemcpyAsync(rgba, d_img, img, cudaMemcpyDeviceToHost, st));
    CUR(cudaStreamSynchronize(st));
done:
    if (st) {
        for (void* p : {(void*)d_pos, (void*)d_nrm, (void*)d_col, (void*)d_tr, (void*)d_ts, (void*)d_count,
                        (void*)d_start, (void*)d_cursor, (void*)d_total, (void*)d_list, (void*)d_img})
            if (p) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    return rc;
}

}  // namespace

extern "C" {

void rad_render_options_default(rad_render_options* o) {
    if (!o) return;
    o->width = 1024;
    o->height = 768;
    o->shading = 0;
    o->pad = 0;
    o->x_rot = 0.f;
    o->y_rot = 0.f;
}

int rad_render_fin(const char* fin_path, const rad_render_options* o, int32_t device, uint8_t* rgba) {
    if (!fin_path || !rgba) return fail(RAD_ERR_ARG, "rad_render_fin: null argument");
    int rc = check_options(o);
    if (rc) return rc;
    std::vector<FinTri> tris;
    if ((rc = parse_fin(fin_path, tris))) return rc;
    return render(tris, *o, device, rgba);
}

int rad_render_scene(const rad_scene* s, const rad_render_options* o, int32_t device, uint8_t* rgba) {
    if (!s || !rgba) return fail(RAD_ERR_ARG, "rad_render_scene: null argument");
    int rc = check_options(o);
    if (rc) return rc;
    std::vector<FinTri> tris;
    if (s->precision == 32)
        tris_from_scene(s->s32, tris);
    else
        tris_from_scene(s->s64, tris);
    return render(tris, *o, device, rgba);
}

}  // extern "C"
