// Test program (tests/test_fp64_reciprocal.py): the soil solver's FP64
// Thomas elimination trimb64 (cbm_physics.cuh) on the GPU against the same
// elimination in long double on the host, for 2^18 systems of 6 rows (the
// soil column) and 2^18 of 9 rows (snow and soil), built like the soil
// systems: FP32 off-diagonals a, c <= 0 with magnitudes log-uniform over
// 1e-4..1e4, b = 1 - a - c, a surface term db0 on half of them, and
// right-hand sides near 273 (temperatures) or in 0..1 (liquid fractions).
// The host also runs the elimination in double with IEEE division, the
// reference's own arithmetic.  Prints the largest error of each, relative to
// the system's largest solution value (strongly coupled systems are
// ill-conditioned: the host double elimination itself departs by ~1e-12);
// exit status 0 if the GPU's largest error is within the factor given on the
// command line of the host double elimination's.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <vector>
#include "cbm_physics.cuh"

template <int N>
__global__ void solve(const float* __restrict__ a, const float* __restrict__ c, const double* __restrict__ db0,
                      double* __restrict__ x, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float ar[N], cr[N];
  double r[N];
#pragma unroll
  for (int k = 0; k < N; ++k) { ar[k] = a[(size_t)i * N + k]; cr[k] = c[(size_t)i * N + k]; r[k] = x[(size_t)i * N + k]; }
  cg::trimb64<N>(ar, cr, db0[i], r);
#pragma unroll
  for (int k = 0; k < N; ++k) x[(size_t)i * N + k] = r[k];
}

template <int N>
double run(int n, uint64_t seed, double* host64) {
  std::vector<float> a((size_t)n * N), c((size_t)n * N);
  std::vector<double> db0(n), x((size_t)n * N), ref((size_t)n * N), hd((size_t)n * N);
  uint64_t s = seed;
  auto uni = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return (double)(s >> 11) * (1.0 / 9007199254740992.0); };
  for (int i = 0; i < n; ++i) {
    const bool temp = i & 1;
    for (int k = 0; k < N; ++k) {
      a[(size_t)i * N + k] = k == 0 ? 0.f : -(float)std::pow(10.0, -4.0 + 8.0 * uni());
      c[(size_t)i * N + k] = k == N - 1 ? 0.f : -(float)std::pow(10.0, -4.0 + 8.0 * uni());
      x[(size_t)i * N + k] = temp ? 250.0 + 40.0 * uni() : uni();
    }
    db0[i] = (i & 2) ? std::pow(10.0, -3.0 + 3.0 * uni()) : 0.0;
    // long double elimination of the same system
    long double e[N], g[N], sol[N];
    for (int k = 0; k < N; ++k) {
      const long double ak = a[(size_t)i * N + k], ck = c[(size_t)i * N + k];
      long double b = 1.0L - ak - ck + (k == 0 ? (long double)db0[i] : 0.0L);
      const long double piv = k == 0 ? b : b - ak * e[k - 1];
      e[k] = ck / piv;
      g[k] = ((long double)x[(size_t)i * N + k] - (k == 0 ? 0.0L : ak * g[k - 1])) / piv;
    }
    sol[N - 1] = g[N - 1];
    for (int k = N - 2; k >= 0; --k) sol[k] = g[k] - e[k] * sol[k + 1];
    for (int k = 0; k < N; ++k) ref[(size_t)i * N + k] = (double)sol[k];
    // double elimination with IEEE division
    double ed[N], gd[N];
    for (int k = 0; k < N; ++k) {
      const double ak = a[(size_t)i * N + k], ck = c[(size_t)i * N + k];
      const double b = (1.0 - ak - ck) + (k == 0 ? db0[i] : 0.0);
      const double piv = k == 0 ? b : b - ak * ed[k - 1];
      ed[k] = ck / piv;
      gd[k] = (x[(size_t)i * N + k] - (k == 0 ? 0.0 : ak * gd[k - 1])) / piv;
    }
    hd[(size_t)i * N + N - 1] = gd[N - 1];
    for (int k = N - 2; k >= 0; --k) hd[(size_t)i * N + k] = gd[k] - ed[k] * hd[(size_t)i * N + k + 1];
  }
  float *da, *dc;
  double *ddb, *dx;
  if (cudaMalloc(&da, a.size() * 4) || cudaMalloc(&dc, c.size() * 4) || cudaMalloc(&ddb, n * 8) ||
      cudaMalloc(&dx, x.size() * 8))
    return 1e30;
  cudaMemcpy(da, a.data(), a.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dc, c.data(), c.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(ddb, db0.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x.data(), x.size() * 8, cudaMemcpyHostToDevice);
  solve<N><<<(n + 127) / 128, 128>>>(da, dc, ddb, dx, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 1e30;
  cudaMemcpy(x.data(), dx, x.size() * 8, cudaMemcpyDeviceToHost);
  cudaFree(da); cudaFree(dc); cudaFree(ddb); cudaFree(dx);
  double worst = 0.0, worst_h = 0.0;
  for (int i = 0; i < n; ++i) {
    double scale = 0.0;
    for (int k = 0; k < N; ++k) scale = std::fmax(scale, std::fabs(ref[(size_t)i * N + k]));
    for (int k = 0; k < N; ++k) {
      worst = std::fmax(worst, std::fabs(x[(size_t)i * N + k] - ref[(size_t)i * N + k]) / scale);
      worst_h = std::fmax(worst_h, std::fabs(hd[(size_t)i * N + k] - ref[(size_t)i * N + k]) / scale);
    }
  }
  *host64 = worst_h;
  return worst;
}

int main(int argc, char** argv) {
  const double factor = argc > 1 ? atof(argv[1]) : 2.0;
  double h6 = 0.0, h9 = 0.0;
  const double w6 = run<6>(1 << 18, 0x243F6A8885A308D3ull, &h6);
  const double w9 = run<9>(1 << 18, 0x13198A2E03707344ull, &h9);
  printf("max relative error, GPU trimb64: 6 rows %.3e, 9 rows %.3e; host double: %.3e, %.3e\n", w6, w9, h6, h9);
  return (w6 <= factor * h6 && w9 <= factor * h9) ? 0 : 1;
}
