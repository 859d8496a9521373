/* CPU restatement of the reference's result viewer, for checking the CUDA
 * rasteriser (rad_render_*).  ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 *   raster_oracle in.fin out.rgba [width height shading xrot yrot]
 *       renders like rad_render_fin: RGBA8, top row first
 *   raster_oracle --arrays in.fin out.bin
 *       writes the viewer's vertex arrays (float32 positions, normals,
 *       colours, 9 per triangle each, in that order) after the converter
 *       restatement, to compare with the reference converter's JSON
 *
 * Converter: WebGL_demo/model-converter/main.cpp readColorfulTriangle
 * 167-246 (bounding box, longest side scaled to 10, shifted by -5) and
 * writeColorfulJson 81-150 ("%g" text), then float32 as a Float32Array.
 * Viewer: WebGL_demo/public/index.html drawScene 354-380 and defaults
 * 555-600 (canvas 1024x768, perspective 45 deg 0.1..100, eye (0,0,-40),
 * model (0,5,10), xRot/yRot, lights, ambient 0.2, specular/diffuse 0.8,
 * shininess 32, clear (0,0.2,0.2), DEPTH_TEST LESS); lib/gouraud.vs 24-55
 * (per-vertex lighting), lib/flat.vs + flat.fs 22-46 (per-fragment lighting
 * with the face normal, taken here as the normal of the eye-space triangle
 * facing the eye, which is what cross(dFdx, dFdy) of the position gives).
 * Rasterisation: pixel centres, top-left fill rule, perspective-correct
 * varyings, window depth in [0,1], ties in depth to the earlier triangle.
 * Built with -ffp-contract=off; float arithmetic in the same order as the
 * CUDA kernels, so images agree bit for bit. */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

struct Tri { double fc[3], v[3][3], n[3][3]; };

static bool getline_(FILE* f, std::string& s) {
    s.clear();
    int c;
    while ((c = fgetc(f)) != EOF) {
        if (c == '\n') return true;
        s.push_back((char)c);
    }
    return !s.empty();
}

static bool nums6(const std::string& s, double* f) {
    const char* p = s.c_str();
    for (int i = 0; i < 6; i++) {
        char* e;
        f[i] = strtod(p, &e);
        if (e == p) return false;
        p = e;
    }
    return true;
}

static bool read_fin(const char* path, std::vector<Tri>& T) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    std::string s;
    while (getline_(f, s)) {
        if (s != "Triangle ") { fclose(f); return false; }
        Tri t;
        double x[6];
        if (!getline_(f, s) || !nums6(s, x)) { fclose(f); return false; }
        for (int i = 0; i < 3; i++) t.fc[i] = x[i];
        for (int k = 0; k < 3; k++) {
            if (!getline_(f, s) || !nums6(s, x)) { fclose(f); return false; }
            for (int i = 0; i < 3; i++) { t.v[k][i] = x[i]; t.n[k][i] = x[i + 3]; }
        }
        T.push_back(t);
    }
    fclose(f);
    return true;
}

static float g32(double x) {
    char b[40];
    snprintf(b, sizeof b, "%g", x);
    return (float)strtod(b, NULL);
}

/* converter + JSON + Float32Array */
static void arrays(const std::vector<Tri>& T, std::vector<float>& P, std::vector<float>& N, std::vector<float>& C) {
    const size_t n = T.size();
    P.resize(n * 9); N.resize(n * 9); C.resize(n * 9);
    if (!n) return;
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) lo[k] = hi[k] = T[0].v[0][k];
    for (size_t i = 0; i < n; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                if (T[i].v[j][k] < lo[k]) lo[k] = T[i].v[j][k];
                if (T[i].v[j][k] > hi[k]) hi[k] = T[i].v[j][k];
            }
    double side = hi[0] - lo[0];
    if (hi[1] - lo[1] > side) side = hi[1] - lo[1];
    if (hi[2] - lo[2] > side) side = hi[2] - lo[2];
    const double scale = 10.0 / side;
    for (size_t i = 0; i < n; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                double v = T[i].v[j][k];
                v = v - lo[k];
                v = v * scale;
                v = v - 5.0;
                P[i * 9 + j * 3 + k] = g32(v);
                N[i * 9 + j * 3 + k] = g32(T[i].n[j][k]);
                C[i * 9 + j * 3 + k] = g32(T[i].fc[k] / 255.0);
            }
}

struct U {
    float P[16], MV[16], N[9];
    float amb, spc, dif;
    float L[3][3];
    int W, H, shading;
};

static void mul4(const double* a, const double* b, double* o) {
    double r[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a[k * 4 + row] * b[c * 4 + k];
            r[c * 4 + row] = s;
        }
    memcpy(o, r, sizeof r);
}

static void uniforms(int W, int H, int shading, double xr, double yr, U& u) {
    const double pi = 3.14159265358979323846, nr = 0.1, fr = 100.0;
    const double top = nr * tan(45.0 * pi / 360.0), right = top * ((double)W / (double)H);
    double P[16] = {0}, M[16] = {0}, T[16];
    P[0] = 2 * nr / (2 * right);
    P[5] = 2 * nr / (2 * top);
    P[10] = -(fr + nr) / (fr - nr);
    P[11] = -1;
    P[14] = -(fr * nr * 2) / (fr - nr);
    M[0] = M[5] = M[10] = M[15] = 1;
    memset(T, 0, sizeof T); T[0] = T[5] = T[10] = T[15] = 1; T[14] = -40; mul4(M, T, M);
    memset(T, 0, sizeof T); T[0] = T[5] = T[10] = T[15] = 1; T[13] = 5; T[14] = 10; mul4(M, T, M);
    const double ax = xr * pi / 180.0, ay = yr * pi / 180.0;
    memset(T, 0, sizeof T); T[0] = T[15] = 1; T[5] = cos(ax); T[6] = sin(ax); T[9] = -sin(ax); T[10] = cos(ax); mul4(M, T, M);
    memset(T, 0, sizeof T); T[5] = T[15] = 1; T[0] = cos(ay); T[2] = -sin(ay); T[8] = sin(ay); T[10] = cos(ay); mul4(M, T, M);
    /* N = transpose(inverse(upper 3x3)), column-major */
    double A[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) A[r][c] = M[c * 4 + r];
    const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                       A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    double I[3][3];
    I[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
    I[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
    I[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
    I[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
    I[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
    I[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
    I[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
    I[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
    I[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) u.N[c * 3 + r] = (float)I[c][r];   /* N(r,c) = I(c,r) */
    for (int k = 0; k < 16; k++) { u.P[k] = (float)P[k]; u.MV[k] = (float)M[k]; }
    u.amb = 0.2f; u.spc = 0.8f; u.dif = 0.8f;
    const float L[3][3] = {{-10.f, 4.f, -20.f}, {90.f, -80.f, -60.f}, {100.f, 40.f, -200.f}};
    memcpy(u.L, L, sizeof L);
    u.W = W; u.H = H; u.shading = shading;
}

struct V { float x, y, z; };
static V mk(float x, float y, float z) { V r = {x, y, z}; return r; }
static float dt(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V nz(V a) { float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); return mk(a.x / l, a.y / l, a.z / l); }
static V sb(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static V cr(V a, V b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static float p32(float x) { x = x * x; x = x * x; x = x * x; x = x * x; return x * x; }

/* the shaders' light loop: ambient + specular + diffuse per enabled light */
static V lights(const U& u, V n, V e, const V* ld) {
    V w = mk(0.f, 0.f, 0.f);
    for (int i = 0; i < 3; i++) {
        const V I = mk(-ld[i].x, -ld[i].y, -ld[i].z);
        const float k = 2.f * dt(n, I);
        const V r = mk(I.x - n.x * k, I.y - n.y * k, I.z - n.z * k);
        const float rd = dt(r, e);
        const float s = p32(rd > 0.f ? rd : 0.f);
        const float nd = dt(n, ld[i]);
        const float d = nd > 0.f ? nd : 0.f;
        w.x = w.x + (u.amb + u.spc * s + u.dif * d);
        w.y = w.y + (u.amb + u.spc * s + u.dif * d);
        w.z = w.z + (u.amb + u.spc * s + u.dif * d);
    }
    return w;
}

/* The viewer's vertex stage (flat.vs, gouraud.vs): eye-space position MV x v,
 * normal N x n, direction to light i normalize(L_i - position). */
static V eye_pos(const U& u, float x, float y, float z) {
    const float* M = u.MV;
    return mk(M[0] * x + M[4] * y + M[8] * z + M[12], M[1] * x + M[5] * y + M[9] * z + M[13],
              M[2] * x + M[6] * y + M[10] * z + M[14]);
}
static V eye_nrm(const U& u, float a, float b, float c) {
    const float* N = u.N;
    return mk(N[0] * a + N[3] * b + N[6] * c, N[1] * a + N[4] * b + N[7] * c, N[2] * a + N[5] * b + N[8] * c);
}
static V light_dir(const U& u, int i, V vp) { return nz(sb(mk(u.L[i][0], u.L[i][1], u.L[i][2]), vp)); }
/* gouraud.vs's colour of a vertex (eye position vp, eye normal vn, colour cc) */
static V gouraud_colour(const U& u, V vp, V vn, V cc) {
    V ld[3];
    for (int i = 0; i < 3; i++) ld[i] = light_dir(u, i, vp);
    const V w = lights(u, nz(vn), nz(mk(-vp.x, -vp.y, -vp.z)), ld);
    return mk(cc.x * w.x, cc.y * w.y, cc.z * w.z);
}
/* flat.fs's colour of a fragment: face normal tn, interpolated varyings a
 * (eye position 0-2, light directions 3-11, colour 12-14) */
static V flat_colour(const U& u, V tn, const float* a) {
    const V ld[3] = {mk(a[3], a[4], a[5]), mk(a[6], a[7], a[8]), mk(a[9], a[10], a[11])};
    const V w = lights(u, tn, nz(mk(-a[0], -a[1], -a[2])), ld);
    return mk(a[12] * w.x, a[13] * w.y, a[14] * w.z);
}

static bool tl(float ax, float ay, float bx, float by) { return (ay == by && bx < ax) || (by < ay); }

static unsigned char b8(float c) {
    c = c < 0.f ? 0.f : (c > 1.f ? 1.f : c);
    return (unsigned char)(int)(c * 255.f + 0.5f);
}

static void render(const std::vector<float>& Pp, const std::vector<float>& Nn, const std::vector<float>& Cc, const U& u,
                   std::vector<unsigned char>& img) {
    const int n = (int)(Pp.size() / 9), W = u.W, H = u.H;
    std::vector<float> zb((size_t)W * H, 2.f);
    std::vector<int> tb((size_t)W * H, -1);
    struct R { float sx[3], sy[3], sz[3], iw[3], area; int ok, ord[3]; V vp[3], vn[3]; };
    std::vector<R> rs(n);
    for (int t = 0; t < n; t++) {
        R& r = rs[t];
        r.ok = 1;
        float cx[3], cy[3], cz[3], cw[3];
        for (int k = 0; k < 3; k++) {
            const float x = Pp[t * 9 + k * 3], y = Pp[t * 9 + k * 3 + 1], z = Pp[t * 9 + k * 3 + 2];
            r.vp[k] = eye_pos(u, x, y, z);
            const float* P = u.P;
            const V q = r.vp[k];
            cx[k] = P[0] * q.x + P[4] * q.y + P[8] * q.z + P[12];
            cy[k] = P[1] * q.x + P[5] * q.y + P[9] * q.z + P[13];
            cz[k] = P[2] * q.x + P[6] * q.y + P[10] * q.z + P[14];
            cw[k] = P[3] * q.x + P[7] * q.y + P[11] * q.z + P[15];
            r.vn[k] = eye_nrm(u, Nn[t * 9 + k * 3], Nn[t * 9 + k * 3 + 1], Nn[t * 9 + k * 3 + 2]);
            if (!(cw[k] > 0.f)) r.ok = 0;
        }
        r.ord[0] = 0; r.ord[1] = 1; r.ord[2] = 2;
        if (!r.ok) continue;
        for (int k = 0; k < 3; k++) {
            r.sx[k] = (cx[k] / cw[k] + 1.f) * 0.5f * (float)W;
            r.sy[k] = (cy[k] / cw[k] + 1.f) * 0.5f * (float)H;
            r.sz[k] = (cz[k] / cw[k] + 1.f) * 0.5f;
            r.iw[k] = 1.f / cw[k];
        }
        float area = (r.sx[1] - r.sx[0]) * (r.sy[2] - r.sy[0]) - (r.sy[1] - r.sy[0]) * (r.sx[2] - r.sx[0]);
        if (area < 0.f) {
            std::swap(r.sx[1], r.sx[2]); std::swap(r.sy[1], r.sy[2]); std::swap(r.sz[1], r.sz[2]); std::swap(r.iw[1], r.iw[2]);
            r.ord[1] = 2; r.ord[2] = 1;
            area = -area;
        }
        r.area = area;
        if (!(area > 0.f)) { r.ok = 0; continue; }
        const float mnx = std::min(std::min(r.sx[0], r.sx[1]), r.sx[2]), mxx = std::max(std::max(r.sx[0], r.sx[1]), r.sx[2]);
        const float mny = std::min(std::min(r.sy[0], r.sy[1]), r.sy[2]), mxy = std::max(std::max(r.sy[0], r.sy[1]), r.sy[2]);
        if (!(mxx >= 0.f && mny < (float)H && mxy >= 0.f && mnx < (float)W)) { r.ok = 0; continue; }
        const int x0 = std::max(0, (int)floorf(mnx)), x1 = std::min(W - 1, (int)ceilf(mxx));
        const int y0 = std::max(0, (int)floorf(mny)), y1 = std::min(H - 1, (int)ceilf(mxy));
        for (int y = y0; y <= y1; y++)
            for (int x = x0; x <= x1; x++) {
                const float px = (float)x + 0.5f, py = (float)y + 0.5f;
                const float w0 = (r.sx[2] - r.sx[1]) * (py - r.sy[1]) - (r.sy[2] - r.sy[1]) * (px - r.sx[1]);
                const float w1 = (r.sx[0] - r.sx[2]) * (py - r.sy[2]) - (r.sy[0] - r.sy[2]) * (px - r.sx[2]);
                const float w2 = (r.sx[1] - r.sx[0]) * (py - r.sy[0]) - (r.sy[1] - r.sy[0]) * (px - r.sx[0]);
                if (w0 < 0.f || w1 < 0.f || w2 < 0.f) continue;
                if (w0 == 0.f && !tl(r.sx[1], r.sy[1], r.sx[2], r.sy[2])) continue;
                if (w1 == 0.f && !tl(r.sx[2], r.sy[2], r.sx[0], r.sy[0])) continue;
                if (w2 == 0.f && !tl(r.sx[0], r.sy[0], r.sx[1], r.sy[1])) continue;
                const float b0 = w0 / r.area, b1 = w1 / r.area, b2 = w2 / r.area;
                const float z = b0 * r.sz[0] + b1 * r.sz[1] + b2 * r.sz[2];
                if (!(z >= 0.f && z <= 1.f)) continue;
                const size_t o = (size_t)y * W + x;
                if (z < zb[o]) { zb[o] = z; tb[o] = t; }   /* triangles in draw order: LESS */
            }
    }
    img.assign((size_t)W * H * 4, 0);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            unsigned char* o = &img[((size_t)(H - 1 - y) * W + x) * 4];
            const int t = tb[(size_t)y * W + x];
            if (t < 0) { o[0] = b8(0.f); o[1] = b8(0.2f); o[2] = b8(0.2f); o[3] = 255; continue; }
            const R& r = rs[t];
            const float px = (float)x + 0.5f, py = (float)y + 0.5f;
            const float w0 = (r.sx[2] - r.sx[1]) * (py - r.sy[1]) - (r.sy[2] - r.sy[1]) * (px - r.sx[1]);
            const float w1 = (r.sx[0] - r.sx[2]) * (py - r.sy[2]) - (r.sy[0] - r.sy[2]) * (px - r.sx[2]);
            const float w2 = (r.sx[1] - r.sx[0]) * (py - r.sy[0]) - (r.sy[1] - r.sy[0]) * (px - r.sx[0]);
            const float b0 = w0 / r.area, b1 = w1 / r.area, b2 = w2 / r.area;
            const float q0 = b0 * r.iw[0], q1 = b1 * r.iw[1], q2 = b2 * r.iw[2];
            const float qs = q0 + q1 + q2;
            /* vertex outputs in window order */
            float vary[3][15];
            for (int k = 0; k < 3; k++) {
                const int s = r.ord[k];
                const V cc = mk(Cc[t * 9 + s * 3], Cc[t * 9 + s * 3 + 1], Cc[t * 9 + s * 3 + 2]);
                if (u.shading == 1) {
                    const V g = gouraud_colour(u, r.vp[s], r.vn[s], cc);
                    vary[k][0] = g.x; vary[k][1] = g.y; vary[k][2] = g.z;
                } else {
                    vary[k][0] = r.vp[s].x; vary[k][1] = r.vp[s].y; vary[k][2] = r.vp[s].z;
                    for (int i = 0; i < 3; i++) {
                        const V ld = light_dir(u, i, r.vp[s]);
                        vary[k][3 + 3 * i] = ld.x; vary[k][4 + 3 * i] = ld.y; vary[k][5 + 3 * i] = ld.z;
                    }
                    vary[k][12] = cc.x; vary[k][13] = cc.y; vary[k][14] = cc.z;
                }
            }
            float a[15];
            const int na = u.shading == 1 ? 3 : 15;
            for (int i = 0; i < na; i++) a[i] = (q0 * vary[0][i] + q1 * vary[1][i] + q2 * vary[2][i]) / qs;
            float c0, c1, c2;
            if (u.shading == 1) {
                c0 = a[0]; c1 = a[1]; c2 = a[2];
            } else {
                const V tn = nz(cr(sb(r.vp[r.ord[1]], r.vp[r.ord[0]]), sb(r.vp[r.ord[2]], r.vp[r.ord[0]])));
                const V c = flat_colour(u, tn, a);
                c0 = c.x; c1 = c.y; c2 = c.z;
            }
            o[0] = b8(c0); o[1] = b8(c1); o[2] = b8(c2); o[3] = 255;
        }
}

int main(int argc, char** argv) {
    if (argc == 4 && !strcmp(argv[1], "--arrays")) {
        std::vector<Tri> T;
        if (!read_fin(argv[2], T)) { fprintf(stderr, "cannot read %s\n", argv[2]); return 1; }
        std::vector<float> P, N, C;
        arrays(T, P, N, C);
        FILE* f = fopen(argv[3], "wb");
        if (!f) return 1;
        fwrite(P.data(), 4, P.size(), f);
        fwrite(N.data(), 4, N.size(), f);
        fwrite(C.data(), 4, C.size(), f);
        fclose(f);
        return 0;
    }
    if (argc != 3 && argc != 8) {
        fprintf(stderr, "usage: raster_oracle in.fin out.rgba [width height shading xrot yrot] | --arrays in.fin out.bin\n");
        return 2;
    }
    const int W = argc == 8 ? atoi(argv[3]) : 1024, H = argc == 8 ? atoi(argv[4]) : 768;
    const int shading = argc == 8 ? atoi(argv[5]) : 0;
    const double xr = argc == 8 ? atof(argv[6]) : 0.0, yr = argc == 8 ? atof(argv[7]) : 0.0;
    std::vector<Tri> T;
    if (!read_fin(argv[1], T)) { fprintf(stderr, "cannot read %s\n", argv[1]); return 1; }
    std::vector<float> P, N, C;
    arrays(T, P, N, C);
    U u;
    uniforms(W, H, shading, xr, yr, u);
    std::vector<unsigned char> img;
    render(P, N, C, u, img);
    FILE* f = fopen(argv[2], "wb");
    if (!f) return 1;
    fwrite(img.data(), 1, img.size(), f);
    fclose(f);
    return 0;
}
