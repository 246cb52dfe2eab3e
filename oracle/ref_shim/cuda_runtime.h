// Host stand-in for <cuda_runtime.h>, used only to compile the reference's
// device functions (src/sim.cuh) as host code for the oracle cross-check.
// TEST INFRASTRUCTURE: never part of the GPU library.
#pragma once
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>

#define __device__
#define __host__
#define __shared__
#define __global__ static inline

struct double3 { double x, y, z; };
static inline double3 make_double3(double x, double y, double z) { return double3{x, y, z}; }
struct merc_dim3 { unsigned x, y, z; };
// threadIdx / blockDim of the emulated thread (set by refhost_driver.cpp)
extern thread_local merc_dim3 threadIdx;
extern thread_local merc_dim3 blockDim;

using std::cbrt;
static inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
static inline double norm3d(double a, double b, double c) { return std::sqrt(std::fma(a, a, std::fma(b, b, c * c))); }

// r_crit scale: the reference's Hill radius is a*cbrt(m/3) (sim.cuh:163), the
// only cbrt call of the file; scaling cbrt scales r_crit by the changeover
// factor without touching the reference source.
extern double merc_ref_hill_factor;
static inline double merc_ref_cbrt(double x) { return std::cbrt(x) * merc_ref_hill_factor; }

typedef int cudaError_t;
