/*
 * OpenCL-C shim for compiling the reference's own kernel sources
 * (synchrad/kernel_farfield.cl, synchrad/kernel_nearfield.cl) as host C++.
 *
 * TEST INFRASTRUCTURE ONLY: this header is part of the oracle.  It is used by
 * oracle/build_ref.sh to turn the reference kernels into a CPU library under
 * oracle/_ref/ that pins the C restatement in oracle/sr_oracle.c.  Nothing in
 * the product links it.
 *
 * What the kernels need from OpenCL C, and how it is provided here:
 *   - `uint`, `__kernel`, `__global`, the `#pragma OPENCL EXTENSION` line;
 *   - 3-component vectors `double3` / `float3` with members s0, s1, s2, built
 *     with the compound-literal form `(double3){a, b, c}` (a GNU C++ extension
 *     for aggregates), elementwise + - and scalar * ;
 *   - `dot` (evaluated left to right: s0*s0 + s1*s1 + s2*s2), `rsqrt` (as
 *     1/sqrt, correctly rounded parts), `sin`, `cos`, `sqrt`, `fabs` and the
 *     `native_` spellings of them (the oracle has no approximate variants);
 *   - `get_global_id(0)`, read from a thread-local work-item id that the driver
 *     (oracle/ref_driver.cpp) sets before each call.  It must be a single
 *     extern object: a header-local `static` would give every translation unit
 *     its own copy.
 */
#pragma once
#include <cmath>
#include <cstddef>

typedef unsigned int uint;

#define __kernel
#define __global

extern thread_local unsigned int sr_cl_gid;
#define get_global_id(dim) ((size_t)sr_cl_gid)

template <typename T>
struct sr_cl_vec3 {
  T s0, s1, s2;
};
typedef sr_cl_vec3<double> double3;
typedef sr_cl_vec3<float> float3;

template <typename T>
static inline sr_cl_vec3<T> operator+(sr_cl_vec3<T> a, sr_cl_vec3<T> b) {
  return sr_cl_vec3<T>{a.s0 + b.s0, a.s1 + b.s1, a.s2 + b.s2};
}
template <typename T>
static inline sr_cl_vec3<T> operator-(sr_cl_vec3<T> a, sr_cl_vec3<T> b) {
  return sr_cl_vec3<T>{a.s0 - b.s0, a.s1 - b.s1, a.s2 - b.s2};
}
template <typename T>
static inline sr_cl_vec3<T> operator-(sr_cl_vec3<T> a) {
  return sr_cl_vec3<T>{-a.s0, -a.s1, -a.s2};
}
template <typename T>
static inline sr_cl_vec3<T> operator*(T s, sr_cl_vec3<T> a) {
  return sr_cl_vec3<T>{s * a.s0, s * a.s1, s * a.s2};
}
template <typename T>
static inline sr_cl_vec3<T> operator*(sr_cl_vec3<T> a, T s) {
  return sr_cl_vec3<T>{a.s0 * s, a.s1 * s, a.s2 * s};
}
template <typename T>
static inline sr_cl_vec3<T>& operator+=(sr_cl_vec3<T>& a, sr_cl_vec3<T> b) {
  a.s0 += b.s0; a.s1 += b.s1; a.s2 += b.s2;
  return a;
}
template <typename T>
static inline sr_cl_vec3<T>& operator*=(sr_cl_vec3<T>& a, T s) {
  a.s0 *= s; a.s1 *= s; a.s2 *= s;
  return a;
}
template <typename T>
static inline T dot(sr_cl_vec3<T> a, sr_cl_vec3<T> b) {
  return a.s0 * b.s0 + a.s1 * b.s1 + a.s2 * b.s2;
}

static inline double sr_cl_rsqrt(double v) { return 1.0 / std::sqrt(v); }
static inline float sr_cl_rsqrt(float v) { return 1.0f / std::sqrt(v); }
static inline double sr_cl_sin(double v) { return std::sin(v); }
static inline float sr_cl_sin(float v) { return std::sin(v); }
static inline double sr_cl_cos(double v) { return std::cos(v); }
static inline float sr_cl_cos(float v) { return std::cos(v); }
static inline double sr_cl_sqrt(double v) { return std::sqrt(v); }
static inline float sr_cl_sqrt(float v) { return std::sqrt(v); }
static inline double sr_cl_fabs(double v) { return std::fabs(v); }
static inline float sr_cl_fabs(float v) { return std::fabs(v); }

#define rsqrt(v) sr_cl_rsqrt(v)
#define sin(v) sr_cl_sin(v)
#define cos(v) sr_cl_cos(v)
#define sqrt(v) sr_cl_sqrt(v)
#define fabs(v) sr_cl_fabs(v)
#define native_rsqrt(v) sr_cl_rsqrt(v)
#define native_sin(v) sr_cl_sin(v)
#define native_cos(v) sr_cl_cos(v)
#define native_sqrt(v) sr_cl_sqrt(v)
