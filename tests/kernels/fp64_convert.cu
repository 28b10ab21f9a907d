// Test program (tests/test_fp64_reciprocal.py): the soil solver's
// FP32 <-> FP64 conversions on the integer pipe (f2d, d2f in
// cbm_physics.cuh) against the hardware conversion instructions on the GPU,
// bit for bit: every float bit pattern class (random 32-bit patterns,
// including infinities and NaNs, plus zeros and the normal range's ends) and
// doubles of every class, doubles inside the float range with random
// fractions, and rounding ties to even and odd.  f2d turns a subnormal
// float into zero of its sign and keeps a NaN's fraction (any NaN is a
// match); everything else must be bitwise equal.  Prints the number of
// mismatches; exit status 0 if there are none.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include "cbm_physics.cuh"

__global__ void conv(const float* __restrict__ xf, const double* __restrict__ xd, unsigned long long* __restrict__ out,
                     int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[4 * (size_t)i + 0] = (unsigned long long)__double_as_longlong(cg::f2d(xf[i]));
  out[4 * (size_t)i + 1] = (unsigned long long)__double_as_longlong((double)xf[i]);
  out[4 * (size_t)i + 2] = __float_as_uint(cg::d2f(xd[i]));
  out[4 * (size_t)i + 3] = __float_as_uint((float)xd[i]);
}

int main() {
  const int n = 1 << 23;
  std::vector<float> xf(n);
  std::vector<double> xd(n);
  uint64_t s = 0x853C49E6748FEA9Bull;
  auto next = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  for (int i = 0; i < n; ++i) {
    uint32_t fb = (uint32_t)next();
    uint64_t db = next();
    switch (i & 7) {
      case 0: break;                                                      // random patterns
      case 1: fb &= 0x807fffffu; db &= 0x800fffffffffffffull; break;     // float subnormals / double subnormals
      case 2: fb |= 0x7f800000u; db |= 0x7ff0000000000000ull; break;     // inf / NaN
      case 3: {                                                           // doubles in the float normal range
        const uint64_t e = 897 + (next() % 254);
        db = (db & 0x800fffffffffffffull) | (e << 52);
        break;
      }
      case 4: {                                                           // ties: dropped bits exactly half
        const uint64_t e = 897 + (next() % 254);
        db = (db & 0x800fffffe0000000ull) | (e << 52) | 0x10000000ull;
        break;
      }
      case 5: {                                                           // float-range ends, and beyond
        const uint64_t e = (next() & 1) ? 893 + (next() % 6) : 1148 + (next() % 6);
        db = (db & 0x800fffffffffffffull) | (e << 52);
        fb = (fb & 0x807fffffu) | ((next() & 1) ? 0x00800000u : 0x7f000000u);
        break;
      }
      case 6: fb &= 0x80000000u; db &= 0x8000000000000000ull; break;     // signed zeros
      default: {                                                          // values of the soil systems
        const float v = (float)((double)(next() >> 11) * (1.0 / 9007199254740992.0) * 400.0 - 100.0);
        std::memcpy(&fb, &v, 4);
        const double w = (double)(next() >> 11) * (1.0 / 9007199254740992.0) * 300.0;
        std::memcpy(&db, &w, 8);
      }
    }
    std::memcpy(&xf[i], &fb, 4);
    std::memcpy(&xd[i], &db, 8);
  }
  float* dxf;
  double* dxd;
  unsigned long long* dout;
  if (cudaMalloc(&dxf, n * 4) || cudaMalloc(&dxd, n * 8) || cudaMalloc(&dout, (size_t)n * 32)) return 2;
  cudaMemcpy(dxf, xf.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dxd, xd.data(), n * 8, cudaMemcpyHostToDevice);
  conv<<<(n + 255) / 256, 256>>>(dxf, dxd, dout, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 2;
  std::vector<unsigned long long> out((size_t)n * 4);
  cudaMemcpy(out.data(), dout, (size_t)n * 32, cudaMemcpyDeviceToHost);
  long long bad_f2d = 0, bad_d2f = 0;
  for (int i = 0; i < n; ++i) {
    uint32_t fb;
    std::memcpy(&fb, &xf[i], 4);
    const uint32_t mag = fb & 0x7fffffffu;
    uint64_t want = out[4 * (size_t)i + 1];
    if (mag != 0 && mag < 0x00800000u) want = (uint64_t)(fb & 0x80000000u) << 32;   // subnormal -> signed zero
    const bool nan_in = mag > 0x7f800000u;
    const uint64_t got = out[4 * (size_t)i];
    const bool got_nan = (got & 0x7ff0000000000000ull) == 0x7ff0000000000000ull && (got & 0x000fffffffffffffull);
    bad_f2d += nan_in ? !got_nan : got != want;
    bad_d2f += out[4 * (size_t)i + 2] != out[4 * (size_t)i + 3];
  }
  printf("f2d mismatches %lld, d2f mismatches %lld of %d\n", bad_f2d, bad_d2f, n);
  cudaFree(dxf); cudaFree(dxd); cudaFree(dout);
  return (bad_f2d == 0 && bad_d2f == 0) ? 0 : 1;
}
