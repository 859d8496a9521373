/* The viewer's own shader sources against the raster restatement.
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * oracle/stage_ref.py stages the reference's lib/gouraud.vs, lib/flat.vs and
 * lib/flat.fs (WebGL_demo/public) into oracle/_ref/src_shaders with
 * syntax-only edits (the #extension and precision lines dropped, swizzles
 * written as calls); this program compiles them as C++ against
 * oracle/glsl_shim.h and runs them beside the restatement's vertex and
 * fragment stages (oracle/raster_oracle.cpp, the functions its render()
 * calls), on seeded inputs with the viewer's initial uniforms:
 *
 *   gouraud.vs   fragcolor.rgb            vs gouraud_colour(eye_pos, eye_nrm)
 *   flat.vs      vVertexPosition,         vs eye_pos
 *                vLightDirection[0..2],   vs light_dir
 *                vFragcolor               vs the vertex colour
 *   flat.fs      gl_FragColor.rgb         vs flat_colour, with dFdx and dFdy
 *                                            the triangle's eye-space edges
 *
 * Every output must be equal bit for bit.  gl_Position is compared too, but
 * only reported, as the largest difference of window position in pixels:
 * the shader writes (P x MV) x v, the restatement (and the CUDA rasteriser)
 * P x (MV x v), which rounds differently.
 *
 *   shader_pin [samples]   prints one line of counts; exit 0 when equal */
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#define main raster_oracle_main
#include "raster_oracle.cpp"
#undef main

#include "glsl_shim.h"

namespace gouraud_vs {
using namespace glsl;
vec4 gl_Position;
#include "gouraud.vs"
}  // namespace gouraud_vs

namespace flat_vs {
using namespace glsl;
vec4 gl_Position;
#include "flat.vs"
}  // namespace flat_vs

namespace flat_fs {
using namespace glsl;
vec4 gl_FragColor;
#include "flat.fs"
}  // namespace flat_fs

namespace {

uint64_t rng_state = 0x9e3779b97f4a7c15ull;
float uniform01() {   // xorshift64*, 24 random bits
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return (float)((rng_state * 0x2545f4914f6cdd1dull) >> 40) * (1.0f / 16777216.0f);
}
float in(float lo, float hi) { return lo + (hi - lo) * uniform01(); }

bool same(float a, float b) { return std::memcmp(&a, &b, 4) == 0; }
bool same3(const V& a, const glsl::vec3& b) { return same(a.x, b.x) && same(a.y, b.y) && same(a.z, b.z); }

template <typename M4>
void set4(M4& m, const float* f) { for (int k = 0; k < 16; k++) m.m[k] = f[k]; }

// the viewer's initial uniforms, as the restatement builds them
template <typename NS_MV, typename NS_P, typename NS_N>
void matrices(const U& u, NS_MV& mv, NS_P& p, NS_N& n) {
    set4(mv, u.MV);
    set4(p, u.P);
    for (int k = 0; k < 9; k++) n.m[k] = u.N[k];
}

}  // namespace

int main(int argc, char** argv) {
    const long samples = argc > 1 ? atol(argv[1]) : 200000;
    long bad_gouraud = 0, bad_flat_vs = 0, bad_flat_fs = 0, n_pos = 0;
    double max_pos_rel = 0;
    for (int view = 0; view < 3; view++) {
        const double xr[3] = {0.0, 30.0, -75.0}, yr[3] = {0.0, 45.0, 200.0};
        U u;
        uniforms(1024, 768, 0, xr[view], yr[view], u);
        {
            using namespace gouraud_vs;
            matrices(u, uMVMatrix, uPMatrix, uNMatrix);
            uMaterialShininess = 32.0f;
            uAmbientColor = glsl::vec3(u.amb, u.amb, u.amb);
            uPointLightingSpecularColor = glsl::vec3(u.spc, u.spc, u.spc);
            uPointLightingDiffuseColor = glsl::vec3(u.dif, u.dif, u.dif);
            for (int i = 0; i < 3; i++) {
                uPointLightingLocation[i] = glsl::vec3(u.L[i][0], u.L[i][1], u.L[i][2]);
                uPointEnabled[i] = 1.0f;
            }
            uTriangleColor = 1;
        }
        {
            using namespace flat_vs;
            matrices(u, uMVMatrix, uPMatrix, uNMatrix);
            for (int i = 0; i < 3; i++) uPointLightingLocation[i] = glsl::vec3(u.L[i][0], u.L[i][1], u.L[i][2]);
            uTriangleColor = 1;
        }
        {
            using namespace flat_fs;
            uMaterialShininess = 32.0f;
            uAmbientColor = glsl::vec3(u.amb, u.amb, u.amb);
            uPointLightingSpecularColor = glsl::vec3(u.spc, u.spc, u.spc);
            uPointLightingDiffuseColor = glsl::vec3(u.dif, u.dif, u.dif);
            for (int i = 0; i < 3; i++) uPointEnabled[i] = 1.0f;
        }
        for (long k = 0; k < samples; k++) {
            // a triangle of the converted model (inside [-5, 5]^3) with unit-ish normals and colours
            float pos[3][3], nrm[3][3], col[3][3];
            for (int v = 0; v < 3; v++)
                for (int c = 0; c < 3; c++) {
                    pos[v][c] = in(-5.f, 5.f);
                    nrm[v][c] = in(-1.f, 1.f);
                    col[v][c] = in(0.f, 1.f);
                }
            V vp[3];
            for (int v = 0; v < 3; v++) {
                vp[v] = eye_pos(u, pos[v][0], pos[v][1], pos[v][2]);
                const V vn = eye_nrm(u, nrm[v][0], nrm[v][1], nrm[v][2]);
                const V cc = mk(col[v][0], col[v][1], col[v][2]);
                // gouraud.vs
                gouraud_vs::aVertexPosition = glsl::vec3(pos[v][0], pos[v][1], pos[v][2]);
                gouraud_vs::aVertexNormal = glsl::vec3(nrm[v][0], nrm[v][1], nrm[v][2]);
                gouraud_vs::aVertexFrontColor = glsl::vec3(col[v][0], col[v][1], col[v][2]);
                gouraud_vs::main();
                const V g = gouraud_colour(u, vp[v], vn, cc);
                if (!same3(g, gouraud_vs::fragcolor.rgb()) || !same(gouraud_vs::fragcolor.a(), 1.0f)) bad_gouraud++;
                // gl_Position: reported only
                const float* P = u.P;
                const V q = vp[v];
                const float cp[4] = {P[0] * q.x + P[4] * q.y + P[8] * q.z + P[12],
                                     P[1] * q.x + P[5] * q.y + P[9] * q.z + P[13],
                                     P[2] * q.x + P[6] * q.y + P[10] * q.z + P[14],
                                     P[3] * q.x + P[7] * q.y + P[11] * q.z + P[15]};
                // window position (pixels of the 1024 x 768 canvas) of both
                const glsl::vec4& sp = gouraud_vs::gl_Position;
                if (cp[3] > 0.f && sp.w > 0.f) {
                    const double dx = ((double)sp.x / sp.w - (double)cp[0] / cp[3]) * 512.0;
                    const double dy = ((double)sp.y / sp.w - (double)cp[1] / cp[3]) * 384.0;
                    const double d = std::fmax(std::fabs(dx), std::fabs(dy));
                    if (d > max_pos_rel) max_pos_rel = d;
                    n_pos++;
                }
                // flat.vs
                flat_vs::aVertexPosition = gouraud_vs::aVertexPosition;
                flat_vs::aVertexNormal = gouraud_vs::aVertexNormal;
                flat_vs::aVertexFrontColor = gouraud_vs::aVertexFrontColor;
                flat_vs::main();
                bool ok = same3(vp[v], flat_vs::vVertexPosition);
                for (int i = 0; i < 3; i++) ok = ok && same3(light_dir(u, i, vp[v]), flat_vs::vLightDirection[i]);
                ok = ok && same3(cc, flat_vs::vFragcolor.rgb()) && same(flat_vs::vFragcolor.a(), 1.0f);
                if (!ok) bad_flat_vs++;
            }
            // flat.fs at a point inside the triangle: varyings interpolated
            // with weights b, face derivatives along the eye-space edges
            float b0 = uniform01(), b1 = uniform01() * (1.f - b0);
            const float b2 = 1.f - b0 - b1;
            float a[15];
            for (int c = 0; c < 15; c++) {
                float x[3];
                for (int v = 0; v < 3; v++) {
                    const V ld0 = light_dir(u, 0, vp[v]), ld1 = light_dir(u, 1, vp[v]), ld2 = light_dir(u, 2, vp[v]);
                    const float all[15] = {vp[v].x, vp[v].y, vp[v].z, ld0.x, ld0.y, ld0.z, ld1.x, ld1.y, ld1.z,
                                           ld2.x, ld2.y, ld2.z, col[v][0], col[v][1], col[v][2]};
                    x[v] = all[c];
                }
                a[c] = b0 * x[0] + b1 * x[1] + b2 * x[2];
            }
            const V e1 = sb(vp[1], vp[0]), e2 = sb(vp[2], vp[0]);
            glsl::ddx = glsl::vec3(e1.x, e1.y, e1.z);
            glsl::ddy = glsl::vec3(e2.x, e2.y, e2.z);
            flat_fs::vVertexPosition = glsl::vec3(a[0], a[1], a[2]);
            for (int i = 0; i < 3; i++) flat_fs::vLightDirection[i] = glsl::vec3(a[3 + 3 * i], a[4 + 3 * i], a[5 + 3 * i]);
            flat_fs::vFragcolor = glsl::vec4(a[12], a[13], a[14], 1.0f);
            flat_fs::main();
            const V want = flat_colour(u, nz(cr(e1, e2)), a);
            if (!same3(want, flat_fs::gl_FragColor.rgb()) || !same(flat_fs::gl_FragColor.a(), 1.0f)) bad_flat_fs++;
        }
    }
    printf("samples %ld gouraud_vs_mismatch %ld flat_vs_mismatch %ld flat_fs_mismatch %ld "
           "gl_position_max_window_diff_px %.3g over %ld vertices in front of the eye\n",
           samples * 3, bad_gouraud, bad_flat_vs, bad_flat_fs, max_pos_rel, n_pos);
    return (bad_gouraud || bad_flat_vs || bad_flat_fs) ? 1 : 0;
}
