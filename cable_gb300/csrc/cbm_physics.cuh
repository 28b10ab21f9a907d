// Device-side restatement of CABLE's offline cbm() timestep for one tile
// (src/offline/cbl_model_driver_offline.F90:38-231) with the offline driver's
// rescaling and balance checks (src/offline/cable_serial.F90:573-728,
// src/offline/cable_checks.F90:472-618).  One thread owns one tile for the
// whole timestep; every call-site below cites the reference routine it
// restates.
//
// Precision policy (GB300: FP64 runs at a small fraction of the FP32 rate):
//   * FP32 for radiation, canopy energy balance, photosynthesis, snow, soil
//     fluxes, the coefficients of the soil systems, and carbon;
//   * FP64-class storage for soil water / ice (ssnow%wb, ssnow%wbice:
//     double-FP32 pairs, a 48-bit significand) and FP64 for the layer-1 heat
//     capacity;
//   * the two tridiagonal (Thomas) solves of soil heat and soil moisture in
//     FP64 on the reference's direct form (trimb64, the default), or in FP32
//     on the step's change (trid_correction, selectable); FP64 for the
//     energy / water balance accumulators.
//
// Switch set: the reference offline defaults (cable.nml): soil_struc
// 'default', fwsoil 'standard', ssnow_potev 'HDM', gs_switch 'leuning'
// (medlyn selectable), litter / or_evap / gw_model / l_rev_corr /
// call_climate / soil_thermal_fix / redistrb off, diag_soil_resp 'ON',
// icycle 0.
#pragma once
#include <cstdint>
#include "tables.h"
#include "forcing.cuh"

namespace cg {

// physical constants (src/params/cable_phys_constants_mod.F90 and friends)
constexpr float TFRZ = 273.16f, SBOLTZ = 5.67e-8f, EMSOIL = 1.0f, EMLEAF = 1.0f, CAPP = 1004.64f;
// litter conductivity (W/m/K) and vapour diffusivity (m2/s) of cable_canopy.F90:203-204
constexpr float KTH_LITT = 0.3f, DV_LITT = 3.1415841138194147e-05f;
constexpr float HL = 2.5014e6f, HLF = 0.334e6f, DHEAT = 21.5e-6f, GRAV = 9.8086f, RGAS = 8.3143f;
constexpr float RMAIR = 0.02897f, RMH2O = 0.018016f, CGSNOW = 2090.0f, CSICE = 2.100e3f, CSWAT = 4.218e3f;
constexpr float DLIQ = 1000.0f, DICE = 921.0f, TETENA = 6.106f, TETENB = 17.27f, TETENC = 237.3f;
constexpr float VONK = 0.40f, A33 = 1.25f, CSW = 0.50f, CTL = 0.40f, APOL = 0.70f, PRANDT = 0.71f;
constexpr float CRD = 0.3f, CSD = 0.003f, CCD = 15.0f, CCW_C = 2.0f, USUHM = 0.3f, ZETNEG = -15.0f;
constexpr float ZETPOS = 1.0f, ZDLIN = 1.0f, UMIN = 0.1f, GAM0 = 28.0e-6f, GAM1 = 0.0509f, GAM2 = 0.0010f;
constexpr float RGBWC = 1.32f, RGSWC = 1.57f, TREFK = 298.2f, LAI_THRESH = 0.001f, RAD_THRESH = 0.001f;
constexpr float COSZEN_TOLS = 1.0e-4f, PI_C = 3.1415927f, MAX_GLACIER_SNOWD = 1100.0f, SNOW_CCNSW = 2.0f;
constexpr float MAX_SSDN = 750.0f, MAX_SCONDS = 2.51f, FROZEN_LIMIT = 0.85f, SNMIN = 1.0f;
constexpr float GW0 = 0.308f, GW1 = 0.514f, GW2 = 0.178f;
constexpr int LAKES = 16, ICE_SURF = 17, ICE_SOIL = 9, MAXITER = 20, NITER = 4;
// per-tile status bits (the public CABLEGPU_TILE_* values)
constexpr uint8_t CG_TS_NONFINITE = 1, CG_TS_DRYLEAF_NOCONV = 2, CG_TS_FORCING_RANGE = 4, CG_TS_OUTPUT_RANGE = 8,
                  CG_TS_EVAPFBL = 16;
// x outside [lo, hi], or not a number (the range checks of cable_checks.F90)
__device__ __forceinline__ bool out_of(float x, float lo, float hi) { return !(x >= lo && x <= hi); }

// Number / order of the optional per-tile diagnostics (debug output).
#define CG_NDIAG 63
// Headline outputs written every step: fe fh fgpp frday tv rnet ga trad
#define CG_NOUT 8

// Device view of every per-tile array ([layer][ld] structure of arrays).
struct CgDev {
  int mp, ld;
  // static per tile (device slot order; tile_id = the caller's tile index)
  const int* tile_id;
  const uint8_t* iveg;
  const uint8_t* isoilm;
  const float* vlai;
  const float* lat;
  const float* lonphase;
  const float* tbase;
  const float* swscale;
  const float* albsoil;    // VIS bare-soil albedo, soil%albsoil(:,1)
  // prognostic state
  float* wb;         // [6] as double-FP32 pairs: hi layers 0..5, lo layers 6..11
  float* wbice;      // [6] likewise
  double* gammzz1;   // layer-1 heat capacity (J/m2/K)
  float* tgg;        // [6]
  float* tggsn;      // [3]
  float* ssdn;       // [3]
  float* smass;      // [3]
  float* sdepth;     // [3]
  uint8_t* flags;    // bit0 isflag, bit1 soil_snow first call pending
  float* snowd;
  float* ssdnn;
  float* snage;
  float* pudsto;
  float* owetfac;
  float* rtsoil;
  float* tss;
  float* wb_lake;
  float* wbtot1;
  float* wbtot2;
  float* cansto;
  float* cplant;     // [3]
  float* csoil;      // [2]
  double* owb;
  double* ebal_tot;
  double* wbal_tot;
  float* vlaiw;      // snow-reduced LAI carried between coupled calls (canopy%vlaiw)
  // outputs
  float* out;              // [CG_NOUT]
  uint8_t* tile_status;    // per-tile status bits (CG_TS_*), OR-ed by the kernels, cleared by the caller
  float* out_caller;       // [CG_NOUT][mp] copy of out for the host-I/O steps, or null
  int out_caller_order;    // 1: out_caller in the caller's tile order, 0: in device order
  float* diag;             // [CG_NDIAG] or null
  float* work_a;           // phase A -> B, C handoff record
  float* work_b;           // phase B -> C handoff record
  float* work_c;           // phase C1 -> C2 -> C3 handoff record
  const float* forcing_in; // [CG_NFORC] host-provided forcing, or null (synthetic)
  int forcing_caller_order; // layout of forcing_in: 0 [CG_NFORC][ld] device order, 1 [CG_NFORC][mp]
                            // in the caller's tile order, 2 [CG_NFORC][mp] in device order
  float* forcing_out;      // [CG_NFORC] copy of the forcing used, or null
  unsigned int* status;    // bit0: non-finite output seen, bit1: surrogate network failed
  // dryLeaf training-row harvest (null when off): rows of 12 features and 3
  // targets (sur:: layout), one per sampled (tile, step, MO iteration)
  float* harvest;
  unsigned long long* harvest_n;
  long long harvest_cap;
  float harvest_prob;
  unsigned long long harvest_seed;
  // dryLeaf surrogate (null when off): the network kernel's predicted leaf
  // temperature change of the first Monin-Obukhov iteration
  const float* sur_dt;             // [ld]
  float sur_gate;                  // K: closure test of the prediction
  int sur_strict;                  // 1: a prediction that does not close restarts the plain iteration
  unsigned long long* sur_stats;   // [0] tiles that started from a prediction, [1] closed in one pass
};

struct CgTables {
  CgPftTable pft;
  CgSoilTable soil;
};

__device__ __forceinline__ float sqf(float x) { return x * x; }

// ---------------------------------------------------------------- double-FP32 state
// Soil water and ice (REAL(r_2) in the reference) are carried as unevaluated
// sums hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2: a 48-bit
// significand (relative precision ~4e-15), updated with error-free FP32
// transformations (Knuth's two-sum, Dekker's fast two-sum and FMA-based
// products), so the soil kernels keep FP64-class state without issuing FP64
// instructions, which GB300 executes at a small fraction of the FP32 rate.
// Field layout: [2 * n][ld] floats, hi of layer k at row k, lo at row n + k.
struct df32 {
  float hi, lo;
};
__device__ __forceinline__ df32 df_load(const float* p, int n, int ld, int k, int t) {
  return {p[k * ld + t], p[(n + k) * ld + t]};
}
__device__ __forceinline__ void df_store(float* p, int n, int ld, int k, int t, df32 v) {
  p[k * ld + t] = v.hi;
  p[(n + k) * ld + t] = v.lo;
}
__device__ __forceinline__ df32 df_norm(float s, float e) {   // fast two-sum, |s| >= |e|
  const float hi = s + e;
  return {hi, e - (hi - s)};
}
// a + b for an FP32 b
__device__ __forceinline__ df32 df_add(df32 a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b - bb);
  return df_norm(s, e + a.lo);
}
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  return df_norm(s, e + (a.lo + b.lo));
}
// a * c for an FP32 c
__device__ __forceinline__ df32 df_mul(df32 a, float c) {
  const float p = a.hi * c;
  const float e = fmaf(a.hi, c, -p);
  return df_norm(p, fmaf(a.lo, c, e));
}
// a - b rounded to FP32
__device__ __forceinline__ float df_sub(df32 a, df32 b) { return (a.hi - b.hi) + (a.lo - b.lo); }
__device__ __forceinline__ bool df_lt(df32 a, df32 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ double f2d(float x);
__device__ __forceinline__ float d2f(double x);
__device__ __forceinline__ double df_to_double(df32 a) { return f2d(a.hi) + f2d(a.lo); }
__device__ __forceinline__ df32 df_from_double(double d) {
  const float hi = d2f(d);
  return {hi, d2f(d - f2d(hi))};
}
// A double as double-FP32 without FP64 instructions: hi = x truncated to 24
// significant bits, lo = its next 23 bits (the rest, below 2^-47 of x, is
// dropped), both built with integer operations on the IEEE-754 fields.  For
// |x| < 2^127; below 2^-80 (and zero) the result is a zero of x's sign.
__device__ __forceinline__ df32 df_split(double x) {
  const unsigned int h = (unsigned int)__double2hiint(x), l = (unsigned int)__double2loint(x);
  const unsigned int mh = h & 0x7fffffffu, sign = h & 0x80000000u;
  const bool tiny = mh < (943u << 20);
  const float hi = __uint_as_float(sign | (tiny ? 0u : ((mh - (896u << 20)) << 3) | (l >> 29)));
  // the low 29 fraction bits, top 23 of them, as the integer they spell
  // (2^23 + m - 2^23, exact), scaled by 2^(e - 1069)
  const float m = __fsub_rn(__uint_as_float(0x4B000000u | ((l & 0x1fffffffu) >> 6)), 8388608.0f);
  const float lo = tiny ? 0.f : __fmul_rn(m, __uint_as_float(((mh >> 20) - 1069u + 127u) << 23));
  return {hi, sign ? -lo : lo};
}
// x / s for a double-FP32 x and an FP32 s != 0, as double-FP32 to about
// 2^-46: q1 = x.hi / s approximately, then the remainder x - q1 s with the
// product's exact error (Sterbenz: x.hi - q1 s is exact) divided by s.
__device__ __forceinline__ df32 df_div(df32 x, float s) {
  const float r = __fdividef(1.0f, s);
  const float q1 = __fmul_rn(x.hi, r);
  const float p = __fmul_rn(q1, s);
  const float rem = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, p), __fmaf_rn(q1, s, -p)), x.lo);
  return df_norm(q1, __fmul_rn(rem, r));
}
__device__ __forceinline__ float pow4(float x) { float y = x * x; return y * y; }
__device__ __forceinline__ float fsignf(float a, float b) { return signbit(b) ? -fabsf(a) : fabsf(a); }

// cbl_qsat.F90:46-50 (tair in deg C)
__device__ __forceinline__ float qsatfjh(float tair, float pmb) {
  return (RMH2O / RMAIR) * (TETENA * expf(TETENB * tair / (TETENC + tair))) / pmb;
}
// cbl_friction_vel.F90:112-166
__device__ __forceinline__ float psim(float zeta) {
  const float gu = 16.0f, b = 0.667f, xc = 5.0f, d = 0.35f;
  float z = 0.5f + fsignf(0.5f, zeta);
  float stable = -zeta - b * (zeta - xc / d) * expf(-d * zeta) - b * xc / d;
  float x = sqrtf(sqrtf(1.0f + gu * fabsf(zeta)));
  float unstable = logf((1.0f + x * x) * sqf(1.0f + x) / 8.0f) - 2.0f * atanf(x) + PI_C * 0.5f;
  return z * stable + (1.0f - z) * unstable;
}
// cbl_friction_vel.F90:168-221
__device__ __forceinline__ float psis(float zeta) {
  const float gu = 16.0f, b = 0.667f, c = 5.0f, d = 0.35f;
  float z = 0.5f + fsignf(0.5f, zeta);
  float stz = fmaxf(0.f, zeta);
  float w = 1.f + 2.f / 3.f * stz;
  float stable = -(w * sqrtf(w)) - b * (stz - c / d) * expf(-d * stz) - b * c / d + 1.f;
  float y = sqrtf(1.0f + gu * fabsf(zeta));
  float unstable = 2.0f * logf((1.f + y) * 0.5f);
  return z * stable + (1.0f - z) * unstable;
}

// The canopy kernel is built without implicit multiply-add contraction
// (-fmad=false): the compiler's choice of which products to fuse depends on
// the code around them, so it differs between the kernel's instantiations
// (diagnostics on or off, the surrogate's and coupled variants), which must
// compute identical results.  Its hot arithmetic below is written with
// explicit fused multiply-adds (__fmaf_rn) instead.

// Positive root of a*x^2 + b*x + c = 0 as the reference writes it,
// (-b + sqrt(max(0, b^2 - 4ac))) / (2a), evaluated without cancellation:
// for b > 0 the algebraically identical 2c / (-b - sqrt(...)) is used.
__device__ __forceinline__ float qroot(float a, float b, float c) {
  float disc = sqrtf(fmaxf(0.0f, __fmaf_rn(b, b, -4.0f * c * a)));
  if (b > 0.0f) {
    float den = -b - disc;
    return (den != 0.0f) ? (2.0f * c) / den : 0.0f;
  }
  return (-b + disc) / (2.0f * a);
}

// cbl_photosynthesis.F90:52-213 for one leaf (masks applied by the caller):
// the Rubisco-, RuBP- and sink-limited net assimilation as roots of the
// reference's three quadratics, their coefficients grouped into
// multiply-adds (1 - csx gs, the common term vcmxt3 cx2 / 2 + cx1 (rdx -
// vcmxt4), and gmf factored out of the sink constant term).
__device__ __forceinline__ float photosynthesis_leaf(float csx, float cx1, float cx2, float gswmin, float rdx,
                                                     float vcmxt3, float vcmxt4, float vx3, float vx4, float gs_coeff,
                                                     float fwsoil) {
  const float effc4 = 4000.0f;
  const float gmf = gswmin * fwsoil / RGSWC;
  const float one_m = __fmaf_rn(-csx, gs_coeff, 1.0f);   // 1 - csx gs_coeff
  const float hc2 = 0.5f * cx2;
  float anrubisco = 0.f, anrubp, ansink = 0.f, ci, coef0, coef1, coef2;
  float tt = __fmaf_rn(vcmxt3, hc2, cx1 * (rdx - vcmxt4));
  coef2 = __fmaf_rn(gs_coeff, vcmxt3 - (rdx - vcmxt4), gmf);
  coef1 = __fmaf_rn(one_m, vcmxt3 + vcmxt4 - rdx, __fmaf_rn(gmf, cx1 - csx, -gs_coeff * tt));
  coef0 = __fmaf_rn(-one_m, tt, -(gmf * cx1) * csx);
  if (fabsf(coef2) > 1.0e-9f && fabsf(coef1) < 1.0e-9f) anrubisco = 99999.0f;
  if (fabsf(coef2) < 1.e-9f && fabsf(coef1) >= 1e-9f) {
    ci = fmaxf(0.0f, -coef0 / coef1);
    anrubisco = __fmaf_rn(vcmxt3, (ci - hc2) / (ci + cx1), vcmxt4 - rdx);
  }
  if (fabsf(coef2) >= 1.e-9f) {
    ci = fmaxf(0.0f, qroot(coef2, coef1, coef0));
    anrubisco = __fmaf_rn(vcmxt3, (ci - hc2) / (ci + cx1), vcmxt4 - rdx);
  }
  tt = __fmaf_rn(vx3, hc2, cx2 * (rdx - vx4));
  coef2 = __fmaf_rn(gs_coeff, vx3 - (rdx - vx4), gmf);
  coef1 = __fmaf_rn(one_m, vx3 + vx4 - rdx, __fmaf_rn(gmf, cx2 - csx, -gs_coeff * tt));
  coef0 = __fmaf_rn(-one_m, tt, -(gmf * cx2) * csx);
  anrubp = 99999.0f;
  if (fabsf(coef2) < 1.e-9f && fabsf(coef1) >= 1.e-9f) {
    ci = fmaxf(0.0f, -coef0 / coef1);
    anrubp = __fmaf_rn(vx3, (ci - hc2) / (ci + cx2), vx4 - rdx);
  }
  if (fabsf(coef2) >= 1.e-9f) {
    ci = fmaxf(0.0f, qroot(coef2, coef1, coef0));
    anrubp = __fmaf_rn(vx3, (ci - hc2) / (ci + cx2), vx4 - rdx);
  }
  // sink: coef1 = gmf + gs (rdx - vcmxt3 / 2) + effc4 vcmxt4 (1 - gs csx),
  // coef0 = gmf (rdx - vcmxt3 / 2 - csx effc4 vcmxt4)
  const float u = __fmaf_rn(-0.5f, vcmxt3, rdx), e4v = effc4 * vcmxt4;
  coef2 = gs_coeff;
  coef1 = __fmaf_rn(e4v, one_m, __fmaf_rn(gs_coeff, u, gmf));
  coef0 = gmf * __fmaf_rn(-csx, e4v, u);
  if (fabsf(coef2) < 1.0e-9f && fabsf(coef1) < 1.0e-9f) ansink = 99999.0f;
  if (fabsf(coef2) < 1.e-9f && fabsf(coef1) >= 1.e-9f) ansink = -coef0 / coef1;
  if (fabsf(coef2) >= 1.e-9f) ansink = qroot(coef2, coef1, coef0);
  return fminf(fminf(anrubisco, anrubp), ansink);
}

// cbl_dryLeaf.F90:779-877.  alpha * parx is fixed over a dryLeaf call and x
// changes every pass: the sum is one explicitly rounded multiply-add, so it
// is computed the same wherever the pass runs.
__device__ __forceinline__ float ej3x(float parx, float alpha, float convex, float x) {
  float s = __fmaf_rn(alpha, parx, x);
  return fmaxf(0.0f, 0.25f * ((s - sqrtf(__fmaf_rn(s, s, -(4.0f * convex * alpha * parx) * x))) / (2.0f * convex)));
}
__device__ __forceinline__ float ej4x(float parx, float alpha, float convex, float x) {
  float s = __fmaf_rn(alpha, parx, x);
  return fmaxf(0.0f, (s - sqrtf(__fmaf_rn(s, s, -(4.0f * convex * alpha * parx) * x))) / (2.0f * convex));
}
__device__ __forceinline__ float xvcmxt4(float x) {
  return exp2f(__fmaf_rn(0.1f, x, -2.5f)) / ((1.0f + expf(0.3f * (13.0f - x))) * (1.0f + expf(0.3f * (x - 36.0f))));
}
__device__ __forceinline__ float xvcmxt3(float x) {
  float num = 1.17461f * expf((73637.0f / (RGAS * TREFK)) * (1.f - TREFK / x));
  float den = 1.0f + expf(__fmaf_rn(486.0f, x, -149252.0f) / (RGAS * x));
  return fmaxf(0.0f, num / den);
}
__device__ __forceinline__ float xejmxt3(float x) {
  float num = 1.16715f * expf((50300.0f / (RGAS * TREFK)) * (1.f - TREFK / x));
  float den = 1.0f + expf(__fmaf_rn(495.0f, x, -152044.0f) / (RGAS * x));
  return fmaxf(0.0f, num / den);
}

// FP32 <-> FP64 conversions on the integer pipe.  GB300 issues the
// conversion instructions at the FP64 rate (a warp's conversion occupies the
// FP64 pipe as long as a fused multiply-add), and the soil kernels' FP64
// solves widen every FP32 coefficient and right-hand side and round every
// result.  These build the other format's bit pattern from the IEEE-754
// fields instead.  f2d: float -> double moves the 8-bit exponent (rebiased
// by 1023 - 127 = 896) and the 23-bit fraction into place, exactly, with no
// conversion instruction at all (a fallback in a branch was if-converted by
// the compiler, which then issued the conversion for every value);
// infinities and NaNs keep their class (the exponent field is rebiased to
// all ones), zeros their sign, and subnormal floats, which the soil
// systems' coefficients and states never come near (their magnitudes are
// above 1e-30), become zero of the same sign.  d2f: double -> float
// rebiases, keeps 23 fraction bits and rounds to nearest, ties to even, on
// the 29 bits dropped (a carry out of the fraction increments the exponent,
// as rounding requires); zero is handled in place and doubles outside the
// float normal range (and infinities, NaNs) take the hardware conversion in
// a branch that stays a branch.  Both are bitwise the conversion
// instructions' results for every input but f2d's subnormals
// (tests/test_fp64_reciprocal.py).
__device__ __forceinline__ double f2d(float x) {
  const unsigned int b = __float_as_uint(x);
  const unsigned int mag = b & 0x7fffffffu;
  const bool zero = mag < 0x00800000u;                 // zero or subnormal
  unsigned int hi = (mag >> 3) + (mag >= 0x7f800000u ? 0x70000000u : 0x38000000u);
  hi = (zero ? 0u : hi) | (b & 0x80000000u);
  return __hiloint2double((int)hi, zero ? 0 : (int)(b << 29));
}
__device__ __forceinline__ float d2f(double x) {
  const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
  const unsigned int mh = hi & 0x7fffffffu;
  if (mh - (897u << 20) >= ((1151u - 897u) << 20)) {   // exponent outside [897, 1150]
    if ((mh | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    return (float)x;
  }
  unsigned int f = ((mh - (896u << 20)) << 3) | (lo >> 29);
  const unsigned int rem = lo & 0x1fffffffu;
  f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
  return __uint_as_float(f | (hi & 0x80000000u));
}

// 1/x in FP64 from two fused multiply-adds.  R, the FP32 reciprocal of x's
// leading 24 bits (df_split: integer operations), is within about 2^-22 of
// 1/x; widened exactly (f2d) it has 29 zero fraction bits at the bottom.
// With t = 1 - x R (the first FMA; exact before its one rounding),
// 1/x = R (1 + t + t^2 + ...).  c = R (1 + t^2) is R's bit pattern plus the
// integer k = R t^2 / ulp(R), rounded, formed on the FP32 pipe from t
// truncated to FP32 (k < 2^10, so it lands in R's zero bits: no carry, no
// normalisation); r = R t + c is the second FMA.  The error is below one
// ulp (the roundings of k and of the second FMA; t^3 is below 2^-64):
// faithfully rounded.  Two FP64-pipe instructions, against three for a
// Newton step from a double-float seed (1/(1 - t) is the geometric series;
// the t^2 term rides in the addend's spare bits).  For 2^-80 <= |x| < 2^126 (the soil systems' pivots are >= 1).  Tested against
// CUDA's FP64 division (tests/test_fp64_reciprocal.py).
__device__ __forceinline__ double rcp64(double x) {
  const float r = __fdividef(1.0f, df_split(x).hi);
  const double rd = f2d(r);
  const double t = fma(-x, rd, 1.0);
  const float tf = df_split(t).hi;
  const float mf = __uint_as_float((__float_as_uint(r) & 0x007fffffu) | 0x3f800000u);   // R's significand
  // k + 2^23 in the float whose ulp is 1: k = round(t^2 mf 2^52)
  const float kf = __fmaf_rn(__fmul_rn(__fmul_rn(tf, tf), mf), 4503599627370496.0f, 8388608.0f);
  const unsigned int k = __float_as_uint(kf) - 0x4B000000u;
  const double c = __hiloint2double(__double2hiint(rd), (int)((unsigned int)__double2loint(rd) + k));
  return fma(rd, t, c);
}

// cbl_trimb.F90:17-53 in FP64, as the reference solves both soil systems,
// for their diffusion form: the Thomas algorithm on
//   a(k) u(k-1) + b(k) u(k) + c(k) u(k+1) = rhs(k),  b(k) = 1 - a(k) - c(k)
// (cbl_stempv.F90:100-124, cbl_smoisturev.F90:256), plus db0 on the first
// row (the surface coupling of the heat system, cbl_stempv.F90:129, :197).
// The off-diagonals come as FP32 coefficients and are widened exactly; the
// diagonal, the right-hand side and the elimination are FP64.  rhs is
// replaced by the solution.  The reference's steps: e(1) = c(1)/b(1),
// g(1) = rhs(1)/b(1); temp(k) = 1/(b(k) - a(k) e(k-1)), e(k) = c(k) temp(k),
// g(k) = (rhs(k) - a(k) g(k-1)) temp(k) for k = 2..N-1; the last row
// divided by its own pivot; back substitution.  Row 1's two divisions by
// b(1) are one reciprocal here, every division a multiplication by an FP64
// reciprocal (rcp64, within an ulp of the division), and g(k) overwrites
// rhs(k), so only e and the solution are live in FP64.
// Both are written with explicit fused multiply-adds, so their rounding does
// not depend on where the compiler inlines them: a soil column solves to the
// same bits in either (the heat kernel's warps choose between them).
// trimb64_s: the same with db added to the diagonal of row srow, 0 or S
// (the surface row of a system whose first S rows may be identity rows):
// adding 0.0 to the other candidate row changes nothing.
template <int N, int S>
__device__ __forceinline__ void trimb64_s(const float* a, const float* c, double db, bool s_first, double* rhs) {
  double e[N - 1];
  const double ib = rcp64((1.0 - f2d(a[0]) - f2d(c[0])) + (s_first ? db : 0.0));
  e[0] = f2d(c[0]) * ib;
  rhs[0] = rhs[0] * ib;
#pragma unroll
  for (int k = 1; k < N - 1; ++k) {
    const double ak = f2d(a[k]), ck = f2d(c[k]);
    const double bk = (k == S) ? (1.0 - ak - ck) + (s_first ? 0.0 : db) : (1.0 - ak - ck);
    const double temp = rcp64(fma(-ak, e[k - 1], bk));
    e[k] = ck * temp;
    rhs[k] = fma(-ak, rhs[k - 1], rhs[k]) * temp;
  }
  {
    const double ak = f2d(a[N - 1]), ck = f2d(c[N - 1]);
    rhs[N - 1] = fma(-ak, rhs[N - 2], rhs[N - 1]) * rcp64(fma(-ak, e[N - 2], 1.0 - ak - ck));
  }
#pragma unroll
  for (int k = N - 2; k >= 0; --k) rhs[k] = fma(-e[k], rhs[k + 1], rhs[k]);
}

// kDb0 false: no surface term (db0 is ignored), one FP64 addition fewer.
template <int N, bool kDb0 = true>
__device__ __forceinline__ void trimb64(const float* a, const float* c, double db0, double* rhs) {
  double e[N - 1];
  const double b0 = 1.0 - f2d(a[0]) - f2d(c[0]);
  const double ib = rcp64(kDb0 ? b0 + db0 : b0);
  e[0] = f2d(c[0]) * ib;
  rhs[0] = rhs[0] * ib;
#pragma unroll
  for (int k = 1; k < N - 1; ++k) {
    const double ak = f2d(a[k]), ck = f2d(c[k]);
    const double temp = rcp64(fma(-ak, e[k - 1], 1.0 - ak - ck));
    e[k] = ck * temp;
    rhs[k] = fma(-ak, rhs[k - 1], rhs[k]) * temp;
  }
  {
    const double ak = f2d(a[N - 1]), ck = f2d(c[N - 1]);
    rhs[N - 1] = fma(-ak, rhs[N - 2], rhs[N - 1]) * rcp64(fma(-ak, e[N - 2], 1.0 - ak - ck));
  }
#pragma unroll
  for (int k = N - 2; k >= 0; --k) rhs[k] = fma(-e[k], rhs[k + 1], rhs[k]);
}

// Tridiagonal solve in correction form (the elimination of cbl_trimb.F90:17-53
// applied to the step's change rather than to the new state).  The soil heat
// and moisture systems are A x_new = rhs with A = I + M, M the diffusion
// operator; with x_new = x_old + d the change solves A d = rhs - A x_old,
// whose right-hand side is the step's source term minus M x_old, formed from
// differences of the old state (exact in FP32 for temperatures; from FP64
// differences for soil water).  d is O(the step's change) instead of
// O(the state), so FP32 elimination leaves an error of ~1e-7 of the change,
// far below the FP32 rounding of the stored temperatures, and d = 0 exactly
// when the state is at equilibrium: no drift from rounding.  A is
// diagonally dominant (an M-matrix), so elimination without pivoting is
// stable.  r holds the right-hand side on entry and d on exit.
template <int N>
__device__ __forceinline__ void trid_correction(const float* a, const float* b, const float* c, float* r) {
  float e[N];
  float t = 1.0f / b[0];
  e[0] = c[0] * t;
  r[0] = r[0] * t;
#pragma unroll
  for (int k = 1; k < N; ++k) {
    t = 1.0f / (b[k] - a[k] * e[k - 1]);
    e[k] = c[k] * t;
    r[k] = (r[k] - a[k] * r[k - 1]) * t;
  }
#pragma unroll
  for (int k = N - 2; k >= 0; --k) r[k] = r[k] - e[k] * r[k + 1];
}

}  // namespace cg
