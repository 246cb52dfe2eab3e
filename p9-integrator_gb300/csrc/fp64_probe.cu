// fp64_probe.cu - throughput of the FP64 pipe on this GPU and the cost of
// common FP64 operations in FP64-FMA issue slots.  A measurement tool for the
// design of the kernels (not part of libmerc.so):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 fp64_probe.cu -o fp64_probe && ./fp64_probe
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s line %d\n", cudaGetErrorString(e), __LINE__); return 1;}}while(0)

__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0+x1+x2+x3+x4+x5+x6+x7;
}
__global__ void k_ffma(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; i++) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0+x1+x2+x3+x4+x5+x6+x7;
}
// dependent-chain latency of DFMA: one thread
__global__ void k_dlat(double* out, int iters, double a, double b) {
  double x = threadIdx.x;
  for (int i = 0; i < iters; i++) x = fma(x, a, b);
  out[blockIdx.x * blockDim.x + threadIdx.x] = x;
}
template <int OP>
__global__ void k_fn(double* out, int iters) {
  double x0 = 1.0 + threadIdx.x * 1e-4, x1 = x0 + 0.25, x2 = x0 + 0.5, x3 = x0 + 0.75;
  double s = 0;
  for (int i = 0; i < iters; i++) {
    if (OP == 0) { x0 = sqrt(x0) + 1.0; x1 = sqrt(x1) + 1.0; x2 = sqrt(x2) + 1.0; x3 = sqrt(x3) + 1.0; }
    if (OP == 1) { x0 = 3.0 / x0 + 1.0; x1 = 3.0 / x1 + 1.0; x2 = 3.0 / x2 + 1.0; x3 = 3.0 / x3 + 1.0; }
    if (OP == 2) { x0 = rsqrt(x0) + 1.0; x1 = rsqrt(x1) + 1.0; x2 = rsqrt(x2) + 1.0; x3 = rsqrt(x3) + 1.0; }
    if (OP == 3) { double c0,c1,c2,c3; sincos(x0,&x0,&c0); sincos(x1,&x1,&c1); sincos(x2,&x2,&c2); sincos(x3,&x3,&c3); x0+=c0+1; x1+=c1+1; x2+=c2+1; x3+=c3+1; }
    if (OP == 4) { x0 = cbrt(x0) + 1.0; x1 = cbrt(x1) + 1.0; x2 = cbrt(x2) + 1.0; x3 = cbrt(x3) + 1.0; }
    if (OP == 5) { x0 = (double)rsqrtf((float)x0) + 1.0; x1 = (double)rsqrtf((float)x1) + 1.0; x2 = (double)rsqrtf((float)x2) + 1.0; x3 = (double)rsqrtf((float)x3) + 1.0; }
    if (OP == 6) { x0 = x0 + 1.0; x1 = x1 + 1.0; x2 = x2 + 1.0; x3 = x3 + 1.0; }
    if (OP == 7) { x0 = acos(0.5/x0) + 1.0; x1 = acos(0.5/x1) + 1.0; x2 = acos(0.5/x2) + 1.0; x3 = acos(0.5/x3) + 1.0; }
    if (OP == 8) { x0 = sinh(x0*1e-3) + 1.0; x1 = sinh(x1*1e-3) + 1.0; x2 = sinh(x2*1e-3) + 1.0; x3 = sinh(x3*1e-3) + 1.0; }
    if (OP == 9) { x0 = atan2(x0, 2.0) + 1.0; x1 = atan2(x1, 2.0) + 1.0; x2 = atan2(x2, 2.0) + 1.0; x3 = atan2(x3, 2.0) + 1.0; }
    if (OP == 10) { x0 = log(x0) + 1.0; x1 = log(x1) + 1.0; x2 = log(x2) + 1.0; x3 = log(x3) + 1.0; }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + s;
}
int main() {
  int dev = 0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, dev));
  int clk=0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
  printf("%s SMs=%d clk(kHz)=%d smem/block optin=%zu\n", p.name, p.multiProcessorCount, clk, p.sharedMemPerBlockOptin);
  int nsm = p.multiProcessorCount;
  double* d; CK(cudaMalloc(&d, sizeof(double) * nsm * 1024 * 8));
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  for (int tpb : {128, 256, 512}) {
    int iters = 20000, blocks = nsm * 4;
    k_dfma<<<blocks, tpb>>>(d, 100, 1.0000001, 1e-9); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); k_dfma<<<blocks, tpb>>>(d, iters, 1.0000001, 1e-9); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    double fl = 2.0 * 8 * (double)iters * blocks * tpb;
    printf("DFMA tpb=%d: %.3f TFLOP/s (%.3f ms)\n", tpb, fl / ms / 1e9, ms);
  }
  {
    int iters = 20000, blocks = nsm * 4, tpb = 256;
    k_ffma<<<blocks, tpb>>>((float*)d, 100, 1.0000001f, 1e-9f); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); k_ffma<<<blocks, tpb>>>((float*)d, iters, 1.0000001f, 1e-9f); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("FFMA: %.3f TFLOP/s\n", 2.0 * 8 * (double)iters * blocks * tpb / ms / 1e9);
  }
  {
    int iters = 100000;
    k_dlat<<<1, 1>>>(d, 100, 1.0000001, 1e-9); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); k_dlat<<<1, 1>>>(d, iters, 1.0000001, 1e-9); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("DFMA dependent latency: %.2f ns/op (%.1f cycles at %d MHz)\n", ms * 1e6 / iters, ms * 1e6 / iters * clk / 1e6, clk/1000);
  }
  double dfma_rate = 0;  // FP64 FMA instructions per second, whole GPU
  {
    int iters = 20000, blocks = nsm * 4, tpb = 256;
    cudaEventRecord(e0); k_dfma<<<blocks, tpb>>>(d, iters, 1.0000001, 1e-9); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    dfma_rate = 8.0 * (double)iters * blocks * tpb / (ms * 1e-3);
  }
  const char* names[] = {"sqrt","div","rsqrt","sincos","cbrt","f32rsqrt+cvt","dadd","acos(div)","sinh","atan2","log"};
  for (int op = 0; op < 11; op++) {
    int iters = 2000, blocks = nsm * 4, tpb = 256;
    auto launch = [&](int it) {
      switch (op) {
        case 0: k_fn<0><<<blocks, tpb>>>(d, it); break; case 1: k_fn<1><<<blocks, tpb>>>(d, it); break;
        case 2: k_fn<2><<<blocks, tpb>>>(d, it); break; case 3: k_fn<3><<<blocks, tpb>>>(d, it); break;
        case 4: k_fn<4><<<blocks, tpb>>>(d, it); break; case 5: k_fn<5><<<blocks, tpb>>>(d, it); break;
        case 6: k_fn<6><<<blocks, tpb>>>(d, it); break; case 7: k_fn<7><<<blocks, tpb>>>(d, it); break;
        case 8: k_fn<8><<<blocks, tpb>>>(d, it); break; case 9: k_fn<9><<<blocks, tpb>>>(d, it); break;
        case 10: k_fn<10><<<blocks, tpb>>>(d, it); break;
      }
    };
    launch(10); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); launch(iters); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    double calls = 4.0 * iters * blocks * tpb;
    // each call also does one FP64 add (the loop-carried +1.0 or acos's divide input)
    printf("%-14s %8.3f Gcalls/s  -> %5.1f FP64-FMA slots per call (incl. one add)\n", names[op], calls / ms / 1e6,
           dfma_rate / (calls / (ms * 1e-3)));
  }
  return 0;
}
