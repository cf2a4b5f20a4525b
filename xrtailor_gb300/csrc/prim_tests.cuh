// prim_tests.cuh — narrow-phase primitive tests of the Swift contact kernels, restated for the
// device with the reference's operation order:
//   NearestPoint             xrtailor/src/math/BasicPrimitiveTests.cu:6-100
//   RayIntersect             xrtailor/src/math/BasicPrimitiveTests.cu:242-284
//   ClosestPtSegmentSegment  xrtailor/src/math/BasicPrimitiveTests.cu:303-361
#pragma once
#include "common.cuh"

namespace xrt {

__device__ __forceinline__ float nearest_point(f3 p, f3 a, f3 b, f3 c, f3& qs) {
  const f3 e1 = b - a, e2 = c - a, e3 = c - b;
  const f3 v1 = p - a;
  const float d1 = dot(e1, v1), d2 = dot(e2, v1);
  if (d1 <= 0 && d2 <= 0) {
    qs = a;
    return length(p - qs);
  }
  const f3 v2 = p - b;
  const float d3 = dot(e1, v2), d4 = dot(e2, v2);
  if (d3 >= 0 && d4 <= d3) {
    qs = b;
    return length(p - qs);
  }
  const float vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    const float v = d1 / (d1 - d3);
    qs = a + v * e1;
    return length(p - qs);
  }
  const f3 v3 = p - c;
  const float d5 = dot(e1, v3), d6 = dot(e2, v3);
  if (d6 >= 0 && d5 <= d6) {
    qs = c;
    return length(p - qs);
  }
  const float vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    const float w = d2 / (d2 - d6);
    qs = a + w * e2;
    return length(p - qs);
  }
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    qs = b + w * e3;
    return length(p - qs);
  }
  const float d = 1 / (va + vb + vc);
  const float v = vb * d;
  const float w = vc * d;
  qs = a + e1 * v + e2 * w;
  return length(p - qs);
}

__device__ __forceinline__ float ray_intersect(f3 o, f3 d, float ray_length, f3 a, f3 b, f3 c) {
  const f3 e1 = b - a, e2 = c - a;
  const f3 n = cross(d, e2);
  const float det = dot(e1, n);
  if (tabs(det) < kEps) return kScalarMax;
  const float inv_det = 1 / det;
  const f3 t = o - a;
  const float u = dot(t, n) * inv_det;
  if (u < 0 || u > 1) return kScalarMax;
  const f3 q = cross(t, e1);
  const float v = dot(d, q) * inv_det;
  if (v < 0 || v + u > 1) return kScalarMax;
  const float s = dot(e2, q) * inv_det;
  if (s > 0 && s < ray_length) return s;
  return __int_as_float(0x7f800000);  // INFINITY
}

__device__ __forceinline__ float closest_seg_seg(f3 p1, f3 q1, f3 p2, f3 q2, float& s, float& t,
                                                 f3& c1, f3& c2) {
  const f3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
  const float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
  if (a <= kEps && e <= kEps) {
    s = t = 0;
    c1 = p1;
    c2 = p2;
    return length(c1 - c2);
  }
  if (a <= kEps) {
    s = 0;
    t = f / e;
    t = tclamp(t, 0.0f, 1.0f);
  } else {
    const float c = dot(d1, r);
    if (e <= kEps) {
      t = 0;
      s = tclamp(-c / a, 0.0f, 1.0f);
    } else {
      const float b = dot(d1, d2);
      const float denom = a * e - b * b;
      if (denom > kEps) s = tclamp((b * f - c * e) / denom, 0.0f, 1.0f);
      else s = 0;
      t = (b * s + f) / e;
      if (t < kEps) {
        t = 0;
        s = tclamp(-c / a, 0.0f, 1.0f);
      } else if (t > 1) {
        t = 1;
        s = tclamp((b - c) / a, 0.0f, 1.0f);
      }
    }
  }
  c1 = p1 + d1 * s;
  c2 = p2 + d2 * t;
  return length(c1 - c2);
}

}  // namespace xrt
