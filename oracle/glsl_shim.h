/* Just enough GLSL ES 1.0 to compile the viewer's shader sources as C++, so
 * the raster restatement can be checked against the shaders' own text.
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Types: vec2/vec3/vec4 with component-wise operators, mat3/mat4 stored
 * column-major (GL's layout, as the viewer uploads them), swizzles .xyz .rgb
 * .a .s .t as member functions (the staging script rewrites `v.xyz` to
 * `v.xyz()`).  Qualifiers (attribute, uniform, varying) are empty.
 *
 * Arithmetic is IEEE single precision, built without FP contraction, in the
 * order the shader text writes it.  Builtins, with the choices a GLSL
 * implementation is free to make stated here (the restatement makes the same
 * ones):
 *   dot(a, b)       a.x*b.x + a.y*b.y + a.z*b.z, left to right
 *   normalize(v)    v / sqrt(dot(v, v)), each component divided by the length
 *   cross(a, b)     the usual determinant form
 *   reflect(I, N)   I - (2.0 * dot(N, I)) * N   (GLSL ES 1.0 spec, 8.4)
 *   pow(x, y)       x^32 by five squarings when y == 32 (the viewer's
 *                   shininess), the C library's powf otherwise
 *   max(x, y)       y if x < y, else x
 *   mat * vec       column-major, column 0 first: M[0]*v.x + M[4]*v.y + ...
 *   mat * mat       column-major, k = 0..3 summed in order
 *   dFdx, dFdy      the values the harness sets in glsl::ddx, glsl::ddy
 *   texture2D       the harness's glsl::tex (the viewer samples no texture
 *                   when uTriangleColor != 0) */
#ifndef GLSL_SHIM_H
#define GLSL_SHIM_H
#include <cmath>

namespace glsl {

struct vec3;
struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
    float s() const { return x; }
    float t() const { return y; }
};
struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3 xyz() const { return *this; }
    vec3 rgb() const { return *this; }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
};
struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
    vec3 rgb() const { return vec3(x, y, z); }
    float a() const { return w; }
};
struct mat3 { float m[9]; };
struct mat4 { float m[16]; };
struct sampler2D { int unit; };

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float k) { return vec3(a.x * k, a.y * k, a.z * k); }
inline vec3 operator*(float k, const vec3& a) { return vec3(k * a.x, k * a.y, k * a.z); }
inline vec3 operator/(const vec3& a, float k) { return vec3(a.x / k, a.y / k, a.z / k); }

inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 normalize(const vec3& v) { return v / std::sqrt(dot(v, v)); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline vec3 reflect(const vec3& I, const vec3& N) { return I - (2.0f * dot(N, I)) * N; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float pow(float x, float y) {
    if (y == 32.0f) {
        x = x * x; x = x * x; x = x * x; x = x * x;
        return x * x;
    }
    return std::pow(x, y);
}
inline vec4 operator*(const mat4& M, const vec4& v) {
    const float* m = M.m;
    return vec4(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w, m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
                m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w,
                m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w);
}
inline mat4 operator*(const mat4& A, const mat4& B) {
    mat4 R;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) {
            float s = A.m[r] * B.m[c * 4];
            for (int k = 1; k < 4; k++) s = s + A.m[k * 4 + r] * B.m[c * 4 + k];
            R.m[c * 4 + r] = s;
        }
    return R;
}
inline vec3 operator*(const mat3& N, const vec3& v) {
    const float* m = N.m;
    return vec3(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
                m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

// set by the harness for the fragment being shaded
inline vec3 ddx, ddy;
inline vec4 tex;
inline vec3 dFdx(const vec3&) { return ddx; }
inline vec3 dFdy(const vec3&) { return ddy; }
inline vec4 texture2D(const sampler2D&, const vec2&) { return tex; }

}  // namespace glsl

#define attribute
#define uniform
#define varying

#endif
