// Stand-in for the CUDA Samples header helper_math.h, which the reference
// includes (fluidparams.cuh:6, fluidintegrator.cuh:6, fluidphysics.cu:5,
// fluidutil.cu:8, hash.cuh:13) but which is not part of the reference tree
// nor of this container.  Only the float3 helpers the reference calls are
// provided, with the documented semantics of that header:
//   component-wise + - * / and compound forms, scalar*vector, make_float3(s),
//   dot, length = sqrtf(dot), normalize = v * rsqrtf(dot(v,v)),
//   fabs / fmaxf / fminf applied per component.
// Used only to compile the reference's own device code for the oracle pins.
#ifndef SPH_REF_HELPER_MATH_H
#define SPH_REF_HELPER_MATH_H

#include <cuda_runtime.h>
#include <math.h>

#define HM_FN inline __host__ __device__

HM_FN float3 make_float3(float s) { return make_float3(s, s, s); }
HM_FN float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
HM_FN float3 operator+(const float3& a, const float3& b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
HM_FN float3 operator-(const float3& a, const float3& b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
HM_FN float3 operator*(const float3& a, const float3& b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
HM_FN float3 operator/(const float3& a, const float3& b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
HM_FN float3 operator*(const float3& a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
HM_FN float3 operator*(float s, const float3& a) { return make_float3(s * a.x, s * a.y, s * a.z); }
HM_FN float3 operator/(const float3& a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
HM_FN float3 operator+(const float3& a, float s) { return make_float3(a.x + s, a.y + s, a.z + s); }
HM_FN float3 operator-(const float3& a, float s) { return make_float3(a.x - s, a.y - s, a.z - s); }
HM_FN void operator+=(float3& a, const float3& b) { a.x += b.x; a.y += b.y; a.z += b.z; }
HM_FN void operator-=(float3& a, const float3& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
HM_FN void operator*=(float3& a, float s) { a.x *= s; a.y *= s; a.z *= s; }
HM_FN void operator/=(float3& a, float s) { a.x /= s; a.y /= s; a.z /= s; }

HM_FN float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HM_FN float length(const float3& v) { return sqrtf(dot(v, v)); }
HM_FN float3 fabs(const float3& v) { return make_float3(fabsf(v.x), fabsf(v.y), fabsf(v.z)); }
HM_FN float3 fmaxf(const float3& a, const float3& b) { return make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
HM_FN float3 fminf(const float3& a, const float3& b) { return make_float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }

#ifdef __CUDACC__
inline __device__ float3 normalize(const float3& v) { return v * rsqrtf(dot(v, v)); }
#endif

#endif
