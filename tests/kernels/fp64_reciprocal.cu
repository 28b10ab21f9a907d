// Test program (tests/test_fp64_reciprocal.py): the soil solver's FP64
// reciprocal rcp64 (cbm_physics.cuh) against CUDA's FP64 division 1.0 / x on
// the GPU, over 2^22 values spread log-uniformly over 1e-20..1e20 plus the
// range of the soil systems' pivots and saturation deficits.  Prints the
// largest difference in units in the last place and the largest relative
// error; exit status 0 if both are within the bounds given on the command
// line.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <vector>
#include "cbm_physics.cuh"

__global__ void recip(const double* __restrict__ x, double* __restrict__ mine, double* __restrict__ cuda, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  mine[i] = cg::rcp64(x[i]);
  cuda[i] = 1.0 / x[i];
}

int main(int argc, char** argv) {
  const double max_ulp = argc > 1 ? atof(argv[1]) : 2.0;
  const double max_rel = argc > 2 ? atof(argv[2]) : 4.5e-16;
  const int n = 1 << 22;
  std::vector<double> x(n), a(n), b(n);
  uint64_t s = 0x9E3779B97F4A7C15ull;
  for (int i = 0; i < n; ++i) {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    const double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
    // half over 1e-20..1e20, half over 1e-3..1e4 (the solver's pivots)
    const double lg = (i & 1) ? (-20.0 + 40.0 * u) : (-3.0 + 7.0 * u);
    x[i] = std::pow(10.0, lg) * ((i & 2) ? -1.0 : 1.0);
  }
  double *dx, *da, *db;
  if (cudaMalloc(&dx, n * sizeof(double)) || cudaMalloc(&da, n * sizeof(double)) || cudaMalloc(&db, n * sizeof(double)))
    return 2;
  cudaMemcpy(dx, x.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  recip<<<(n + 255) / 256, 256>>>(dx, da, db, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 2;
  cudaMemcpy(a.data(), da, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(b.data(), db, n * sizeof(double), cudaMemcpyDeviceToHost);
  double worst_ulp = 0.0, worst_rel = 0.0;
  for (int i = 0; i < n; ++i) {
    const double ulp = std::nextafter(std::fabs(b[i]), INFINITY) - std::fabs(b[i]);
    worst_ulp = std::fmax(worst_ulp, std::fabs(a[i] - b[i]) / ulp);
    worst_rel = std::fmax(worst_rel, std::fabs(a[i] * x[i] - 1.0));
  }
  printf("max_ulp %.3f max_rel %.3e\n", worst_ulp, worst_rel);
  cudaFree(dx); cudaFree(da); cudaFree(db);
  return (worst_ulp <= max_ulp && worst_rel <= max_rel) ? 0 : 1;
}
