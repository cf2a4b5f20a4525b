// oracle_math.h — TEST INFRASTRUCTURE: vector math of the CPU oracle.
//
// Restates the glm operations the reference kernels use, with glm's evaluation order, so that the
// oracle's float results can be compared bit-for-bit with the CUDA path (both sides are compiled
// without FMA contraction: -ffp-contract=off here, --fmad=false for the CUDA library; the stretch
// and bend projections use explicit fused multiply-adds, the same ones on both sides).
//   dot(a,b)      = (a.x*b.x + a.y*b.y) + a.z*b.z          (glm compute_dot for vec3)
//   cross(x,y)    = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
//   length(v)     = sqrt(dot(v,v));  normalize(v) = v * (1 / sqrt(dot(v,v)))
// MathFunctions::min/max/Clamp are the ternaries of xrtailor/include/xrtailor/math/MathFunctions.cuh:23-78.
#pragma once
#include <cmath>
#include <cstdint>
#include <cfloat>

namespace orc {

struct V3 {
  float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
static inline V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
static inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
static inline V3& operator-=(V3& a, V3 b) { a = a - b; return a; }
static inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 cross(V3 x, V3 y) {
  return V3{x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
static inline float length(V3 v) { return std::sqrt(dot(v, v)); }
static inline V3 normalize(V3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }
static inline float get(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
static inline void set(V3& v, int i, float s) {
  if (i == 0) v.x = s; else if (i == 1) v.y = s; else v.z = s;
}

template <typename T> static inline T mmin(T a, T b) { return a < b ? a : b; }
template <typename T> static inline T mmax(T a, T b) { return a > b ? a : b; }
template <typename T> static inline T mmin3(T a, T b, T c) { return mmin(a, mmin(b, c)); }
template <typename T> static inline T mmax3(T a, T b, T c) { return mmax(a, mmax(b, c)); }
template <typename T> static inline T clampf(T x, T a, T b) { return x < a ? a : (x > b ? b : x); }
template <typename T> static inline T mabs(T x) { return x < T(0) ? -x : x; }

static const float kEps = 1e-6f;       // EPSILON, core/Scalar.hpp:39
static const float kScalarMax = FLT_MAX;  // SCALAR_MAX, core/Scalar.cuh:10

// Fused forms of the stretch and bend projections (the CUDA library's fdot / fcross / fmad): one
// std::fma (rounded once) per product-plus-term, in the same expression tree on both sides.
static inline float fma1(float a, float b, float c) { return std::fma(a, b, c); }
static inline float fdot(V3 a, V3 b) { return fma1(a.z, b.z, fma1(a.y, b.y, a.x * b.x)); }
static inline V3 fcross(V3 a, V3 b) {
  return V3{fma1(a.y, b.z, -(b.y * a.z)), fma1(a.z, b.x, -(b.z * a.x)),
            fma1(a.x, b.y, -(b.x * a.y))};
}
static inline V3 fmad(V3 a, float s, V3 b) {
  return V3{fma1(a.x, s, b.x), fma1(a.y, s, b.y), fma1(a.z, s, b.z)};
}

// arccos on [0, 1]: Abramowitz & Stegun 4.4.46, |error| <= 2e-8, Horner steps fused (the CUDA
// library evaluates the same polynomial in its bend kernel, so both sides round identically).
static inline float acos_as(float x) {
  float p = -0.0012624911f;
  p = fma1(p, x, 0.0066700901f);
  p = fma1(p, x, -0.0170881256f);
  p = fma1(p, x, 0.0308918810f);
  p = fma1(p, x, -0.0501743046f);
  p = fma1(p, x, 0.0889789874f);
  p = fma1(p, x, -0.2145988016f);
  p = fma1(p, x, 1.5707963050f);
  return std::sqrt(1.0f - x) * p;
}

// MathFunctions::FaceNormal (src/math/MathFunctions.cu:14-20)
static inline V3 face_normal(V3 a, V3 b, V3 c) { return normalize(cross(b - a, c - a)); }

// glm mat4 * vec4(p, 1) for a column-major matrix, glm's association: (c0 x + c1 y) + (c2 z + c3 w).
static inline V3 transform_point(const float* m, V3 p) {
  float r[3];
  for (int k = 0; k < 3; ++k) {
    float a0 = m[0 + k] * p.x, a1 = m[4 + k] * p.y, a2 = m[8 + k] * p.z, a3 = m[12 + k] * 1.0f;
    r[k] = (a0 + a1) + (a2 + a3);
  }
  return V3{r[0], r[1], r[2]};
}

}  // namespace orc
