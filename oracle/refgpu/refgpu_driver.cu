// refgpu_driver.cu - launches the reference's own mercurius_solver kernel on the
// GPU (TEST INFRASTRUCTURE: a measurement and correctness anchor, never part of
// libmerc.so).
//
// Compiled against the patched copy of the reference's src/sim.cuh that
// oracle/refgpu/prepare.py writes (the two compile fixes, BATCH_SIZE set at run
// time, one barrier before the kernel's exit).  The launch reproduces the
// reference host program (src/mercurius.cu:43-69, 73-164, 182-198): clusters
// of 16 blocks of N/16 threads, one cluster per sweep, SWEEPS_PER_GPU (4)
// sweeps per launch, dynamic shared memory of N/16 x (2 double3 + double)
// bytes, the six element arrays per sweep in HBM, elements written back by
// the kernel's epilogue and read again by the next launch's prologue.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "sim.cuh"

namespace {
constexpr int kCluster = 16;

int fail(char* err, int errlen, const char* what, cudaError_t e) {
  if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s: %s", what, cudaGetErrorString(e));
  return 2;
}
}  // namespace

#define RCK(call)                                                   \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) return fail(err, errlen, #call, e_);     \
  } while (0)

extern "C" {

int refgpu_sweeps(void) { return SWEEPS_PER_GPU; }

// n bodies per sweep (massive first, nm of them), elements[SWEEPS_PER_GPU][6][n]
// in the order inclination, node, argument of perihelion, mean anomaly,
// eccentricity, semi-major axis; masses[n].  Runs `launches` kernel launches of
// `steps` steps each with time step dt.  Outputs: out_pos[SWEEPS_PER_GPU][n][3]
// (the kernel's output positions after the last launch), out_elements
// (same layout as elements, after the last launch's epilogue; may be NULL),
// ms[launches] (CUDA-event time of each launch; may be NULL).
// Returns 0, 1 for a shape the reference's launch does not accept, 2 for a
// CUDA error (message in err).
int refgpu_run(int device, int n, int nm, const double* elements, const double* masses, double dt, long steps,
               int launches, double* out_pos, double* out_elements, float* ms, char* err, int errlen) {
  if (n <= 0 || n % kCluster != 0 || n / kCluster > 1024 || nm < 0 || nm > n / kCluster || steps < 1 ||
      launches < 1) {
    if (err && errlen > 0) snprintf(err, (size_t)errlen, "shape not accepted: n %% 16 == 0, n/16 <= 1024, nm <= n/16");
    return 1;
  }
  RCK(cudaSetDevice(device));
  const int S = SWEEPS_PER_GPU;
  cudaLaunchConfig_t config = {};
  RCK(cudaFuncSetAttribute((void*)mercurius_solver, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  config.blockDim = dim3(n / kCluster, 1, 1);
  config.gridDim = dim3(kCluster * S, 1, 1);
  config.dynamicSmemBytes = config.blockDim.x * (sizeof(double3) * 2 + sizeof(double));
  RCK(cudaFuncSetAttribute((void*)mercurius_solver, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)config.dynamicSmemBytes));
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  config.numAttrs = 1;
  config.attrs = attr;
  int clusters = 0;
  RCK(cudaOccupancyMaxActiveClusters(&clusters, (void*)mercurius_solver, &config));
  if (clusters < 1) {
    if (err && errlen > 0) snprintf(err, (size_t)errlen, "no cluster of 16 blocks fits on this device");
    return 2;
  }
  long steps_h = steps;
  RCK(cudaMemcpyToSymbol(merc_ref_batch_steps_d, &steps_h, sizeof(long)));

  const size_t nn = (size_t)n * S;
  // element arrays in the kernel's argument order: peri, M, e, a, inc, node
  const int arg_row[6] = {2, 3, 4, 5, 0, 1};
  double* d_el[6] = {};
  double* d_m = nullptr;
  double3* d_out = nullptr;
  for (int k = 0; k < 6; k++) RCK(cudaMalloc(&d_el[k], nn * sizeof(double)));
  RCK(cudaMalloc(&d_m, (size_t)n * sizeof(double)));
  RCK(cudaMalloc(&d_out, nn * sizeof(double3)));
  std::vector<double> h((size_t)n);
  for (int k = 0; k < 6; k++)
    for (int s = 0; s < S; s++) {
      const double* src = elements + ((size_t)s * 6 + arg_row[k]) * n;
      RCK(cudaMemcpy(d_el[k] + (size_t)s * n, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    }
  RCK(cudaMemcpy(d_m, masses, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  cudaEvent_t e0, e1;
  RCK(cudaEventCreate(&e0));
  RCK(cudaEventCreate(&e1));
  for (int b = 0; b < launches; b++) {
    RCK(cudaEventRecord(e0));
    RCK(cudaLaunchKernelEx(&config, mercurius_solver, d_el[0], d_el[1], d_el[2], d_el[3], d_el[4], d_el[5], d_m,
                           d_out, nm, b, dt));
    RCK(cudaGetLastError());
    RCK(cudaEventRecord(e1));
    RCK(cudaEventSynchronize(e1));
    float t = 0.f;
    RCK(cudaEventElapsedTime(&t, e0, e1));
    if (ms) ms[b] = t;
  }
  RCK(cudaDeviceSynchronize());
  std::vector<double3> out(nn);
  RCK(cudaMemcpy(out.data(), d_out, nn * sizeof(double3), cudaMemcpyDeviceToHost));
  for (size_t j = 0; j < nn; j++) {
    out_pos[3 * j + 0] = out[j].x;
    out_pos[3 * j + 1] = out[j].y;
    out_pos[3 * j + 2] = out[j].z;
  }
  if (out_elements)
    for (int k = 0; k < 6; k++)
      for (int s = 0; s < S; s++)
        RCK(cudaMemcpy(out_elements + ((size_t)s * 6 + arg_row[k]) * n, d_el[k] + (size_t)s * n,
                       (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int k = 0; k < 6; k++) cudaFree(d_el[k]);
  cudaFree(d_m);
  cudaFree(d_out);
  return 0;
}

}  // extern "C"
