// ORACLE / TEST INFRASTRUCTURE ONLY.
// CPU version of the seeded synthetic met forcing that stands in for the
// reference's netCDF site forcing (the TumbaFluxnet file is not available).
// The GPU generator in cable_gb300/csrc/forcing.cuh implements the same
// specification; tests compare the two within a few float ulps.
//
// Derivation rules follow the reference driver:
//   SW split 50/50 VIS/NIR          src/offline/cable_input.F90:1880-1883
//   precip_sn = precip if tk<=tfrz  src/offline/cable_input.F90:2666-2674
//   coszen = sinbet(doy, lat, hod)  src/offline/cable_input.F90:2677,
//                                   src/science/radiation/cbl_sinbet.F90:8-28
// Random numbers: Philox-4x32-10 (Salmon et al., SC'11), counter =
// (tile, step, stream, 0), key = 64-bit seed.
#pragma once
#include <cmath>
#include <cstdint>

namespace cbmref {

struct Philox {
  static inline void round(uint32_t c[4], const uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t o0 = hi1 ^ c[1] ^ k[0], o1 = lo1, o2 = hi0 ^ c[3] ^ k[1], o3 = lo0;
    c[0] = o0; c[1] = o1; c[2] = o2; c[3] = o3;
  }
  static inline void gen(uint32_t ctr[4], uint64_t seed) {
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int r = 0; r < 10; ++r) {
      if (r) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
      round(ctr, k);
    }
  }
};

// uniform in (0,1), exact in float: ((x >> 8) + 0.5) * 2^-24
static inline float u01(uint32_t x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// per-tile forcing parameters (the jitter of the synthetic generator)
struct TileForcingParams {
  float lat;       // degrees north
  float lonphase;  // local-time offset in hours, [0, 24)
  float tbase;     // base air temperature (K)
  float swscale;   // shortwave scale factor
};

struct ForcingSpec {
  uint64_t seed = 12345;
  int doy0 = 1;          // day of year at step 0
  float dels = 1800.f;   // step length (s)
};

// The reference's sinbet (cbl_sinbet.F90:8-28) in float.
static inline float sinbet_f(float doy, float xslat, float hod) {
  const float PI = 3.1415927f, PI180 = 3.1415927f / 180.0f;
  float sindec = -std::sin(23.45f * PI180) * std::cos(2.f * PI * (doy + 10.0f) / 365.0f);
  float z = std::sin(PI180 * xslat) * sindec + std::cos(PI180 * xslat) * std::sqrt(1.f - sindec * sindec) *
                                                    std::cos(PI * (hod - 12.0f) / 12.0f);
  return z > 1e-8f ? z : 1e-8f;
}

// Forcing fields, in this order (13 floats per tile-step)
enum { F_FSD1, F_FSD2, F_FLD, F_PRECIP, F_PRECIP_SN, F_TK, F_PMB, F_UA, F_QV, F_CA, F_COSZEN, F_DOY, F_HOD, F_NFIELDS };

static inline void forcing_at(const ForcingSpec& spec, const TileForcingParams& tp, uint32_t tile, uint32_t step,
                              float out[F_NFIELDS]) {
  const float TWO_PI = 6.2831853f;
  // local time
  float thours = (float)step * (spec.dels / 3600.0f) + tp.lonphase;
  float day = std::floor(thours / 24.0f);
  float hod = thours - 24.0f * day;
  int iday = (spec.doy0 - 1 + (int)day) % 365;
  float doy = (float)(1 + iday);
  uint32_t c0[4] = {tile, step, 0u, 0u};
  uint32_t c1[4] = {tile, step, 1u, 0u};
  Philox::gen(c0, spec.seed);
  Philox::gen(c1, spec.seed);
  float u_cloud = u01(c0[0]), u_lw1 = u01(c0[1]), u_lw2 = u01(c0[2]), u_rh = u01(c0[3]);
  float u_w1 = u01(c1[0]), u_w2 = u01(c1[1]), u_pb = u01(c1[2]), u_pe = u01(c1[3]);
  float sinb = sinbet_f(doy, tp.lat, hod);
  float sw = std::fmax(0.0f, 900.0f * sinb) * (0.3f + 0.7f * u_cloud) * tp.swscale;
  float z_lw = std::sqrt(-2.0f * std::log(u_lw1)) * std::cos(TWO_PI * u_lw2);
  float z_w = std::sqrt(-2.0f * std::log(u_w1)) * std::cos(TWO_PI * u_w2);
  float season = std::cos(TWO_PI * (doy - 196.0f) / 365.0f);
  if (tp.lat < 0.0f) season = -season;
  float tk = tp.tbase + 8.0f * std::sin(TWO_PI * (hod - 9.0f) / 24.0f) + 10.0f * season;
  float rh = 0.3f + 0.6f * u_rh;
  float tc = tk - 273.16f;
  float qsat = (0.018016f / 0.02897f) * (6.106f * std::exp(17.27f * tc / (237.3f + tc))) / 1000.0f;
  float precip = (u_pb < 0.05f) ? -2.0f * std::log(u_pe) : 0.0f;
  out[F_FSD1] = 0.5f * sw;
  out[F_FSD2] = 0.5f * sw;
  out[F_FLD] = 300.0f + 30.0f * z_lw;
  out[F_PRECIP] = precip;
  out[F_PRECIP_SN] = (tk <= 273.16f) ? precip : 0.0f;
  out[F_TK] = tk;
  out[F_PMB] = 1000.0f;
  out[F_UA] = std::exp(1.0986123f - 0.125f + 0.5f * z_w);   // lognormal, mean 3 m/s, sigma 0.5
  out[F_QV] = rh * qsat;
  out[F_CA] = 400.0e-6f;
  out[F_COSZEN] = sinb;
  out[F_DOY] = doy;
  out[F_HOD] = hod;
}

}  // namespace cbmref
