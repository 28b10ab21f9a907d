// In-kernel synthetic met forcing: the seeded stand-in for the reference's
// netCDF site forcing, generated per (tile, step) inside the timestep kernel
// so no forcing bytes move through HBM.
//
// Derivation rules follow the reference driver:
//   SW split 50/50 VIS/NIR          src/offline/cable_input.F90:1880-1883
//   precip_sn = precip if tk<=tfrz  src/offline/cable_input.F90:2666-2674
//   coszen = sinbet(doy, lat, hod)  src/offline/cable_input.F90:2677,
//                                   src/science/radiation/cbl_sinbet.F90:8-28
// Random numbers: Philox-4x32-10 (Salmon et al., SC'11) with counter
// (tile, step, stream, 0) and a 64-bit key, so every value is reproducible
// independently of launch shape and tile order.
#pragma once
#include <cstdint>

#define CG_NFORC 13
enum { CGF_FSD1, CGF_FSD2, CGF_FLD, CGF_PRECIP, CGF_PRECIP_SN, CGF_TK, CGF_PMB, CGF_UA, CGF_QV, CGF_CA,
       CGF_COSZEN, CGF_DOY, CGF_HOD };

struct CgForcingSpec {
  unsigned long long seed;
  int doy0;
  float dels;
};

__device__ __forceinline__ void cg_philox(uint32_t c[4], unsigned long long seed) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t o0 = hi1 ^ c[1] ^ k0, o2 = hi0 ^ c[3] ^ k1;
    c[0] = o0; c[1] = lo1; c[2] = o2; c[3] = lo0;
  }
}

__device__ __forceinline__ float cg_u01(uint32_t x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// f[CG_NFORC] for one tile-step.  lat: degrees north; lonphase: local-time
// offset (h); tbase: base air temperature (K); swscale: shortwave scale.
__device__ __forceinline__ void cg_forcing(const CgForcingSpec& spec, float lat, float lonphase, float tbase,
                                           float swscale, uint32_t tile, uint32_t step, float f[CG_NFORC]) {
  const float TWO_PI = 6.2831853f, PI = 3.1415927f, PI180 = 3.1415927f / 180.0f;
  float thours = (float)step * (spec.dels / 3600.0f) + lonphase;
  float day = floorf(thours / 24.0f);
  float hod = thours - 24.0f * day;
  int iday = (spec.doy0 - 1 + (int)day) % 365;
  float doy = (float)(1 + iday);
  uint32_t c0[4] = {tile, step, 0u, 0u};
  uint32_t c1[4] = {tile, step, 1u, 0u};
  cg_philox(c0, spec.seed);
  cg_philox(c1, spec.seed);
  float u_cloud = cg_u01(c0[0]), u_lw1 = cg_u01(c0[1]), u_lw2 = cg_u01(c0[2]), u_rh = cg_u01(c0[3]);
  float u_w1 = cg_u01(c1[0]), u_w2 = cg_u01(c1[1]), u_pb = cg_u01(c1[2]), u_pe = cg_u01(c1[3]);
  // sinbet (cbl_sinbet.F90:22-26)
  float sindec = -sinf(23.45f * PI180) * cosf(2.f * PI * (doy + 10.0f) / 365.0f);
  float sinb = sinf(PI180 * lat) * sindec + cosf(PI180 * lat) * sqrtf(1.f - sindec * sindec) * cosf(PI * (hod - 12.0f) / 12.0f);
  sinb = sinb > 1e-8f ? sinb : 1e-8f;
  float sw = fmaxf(0.0f, 900.0f * sinb) * (0.3f + 0.7f * u_cloud) * swscale;
  float z_lw = sqrtf(-2.0f * logf(u_lw1)) * cosf(TWO_PI * u_lw2);
  float z_w = sqrtf(-2.0f * logf(u_w1)) * cosf(TWO_PI * u_w2);
  float season = cosf(TWO_PI * (doy - 196.0f) / 365.0f);
  if (lat < 0.0f) season = -season;
  float tk = tbase + 8.0f * sinf(TWO_PI * (hod - 9.0f) / 24.0f) + 10.0f * season;
  float rh = 0.3f + 0.6f * u_rh;
  float tc = tk - 273.16f;
  float qsat = (0.018016f / 0.02897f) * (6.106f * expf(17.27f * tc / (237.3f + tc))) / 1000.0f;
  float precip = (u_pb < 0.05f) ? -2.0f * logf(u_pe) : 0.0f;
  f[CGF_FSD1] = 0.5f * sw;
  f[CGF_FSD2] = 0.5f * sw;
  f[CGF_FLD] = 300.0f + 30.0f * z_lw;
  f[CGF_PRECIP] = precip;
  f[CGF_PRECIP_SN] = (tk <= 273.16f) ? precip : 0.0f;
  f[CGF_TK] = tk;
  f[CGF_PMB] = 1000.0f;
  f[CGF_UA] = expf(1.0986123f - 0.125f + 0.5f * z_w);
  f[CGF_QV] = rh * qsat;
  f[CGF_CA] = 400.0e-6f;
  f[CGF_COSZEN] = sinb;
  f[CGF_DOY] = doy;
  f[CGF_HOD] = hod;
}
