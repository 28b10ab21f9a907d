// The cbm() timestep as five kernels per step, one thread per tile in each:
//   phase A   ruff_resist, define_air, masks, init_radiation, albedo,
//             Surf_wetness_fact, radiation
//   phase B   define_canopy: 4 Monin-Obukhov iterations of dryLeaf / wetLeaf /
//             within-canopy / soil evaporation, screen diagnostics, canopy
//             water budget, soil-coupling derivatives, energy balance
//   phase C1  soil_snow's snow pack: snowcheck, density, accumulation, melt,
//             layer adjustment
//   phase C2  soil heat: the stempv tridiagonal solve (FP64 on the direct
//             form by default, or FP32 on the step's change), melt,
//             remove_trans, soilfreeze
//   phase C3  soil water: the smoisturev tridiagonal solve (likewise),
//             surfbv, snow_aging, carbon, water balance
// Splitting keeps each kernel's code and register footprint small enough
// for the instruction cache and for several resident warps per scheduler;
// the phases hand over per-tile records through HBM (structure of arrays).
#pragma once
#include "cbm_physics.cuh"

namespace cg {

struct StepParams {
  int ktau;          // 1-based step counter of the run (mass_balance init / totals)
  float dels;        // step length (s)
  int medlyn;        // gs_switch: 0 leuning, 1 medlyn
  int thermal_fix;   // cable_user%soil_thermal_fix
  int litter;        // cable_user%litter
  int rev_corr;      // cable_user%l_rev_corr
  int fwsoil_mode;   // fwsoil_switch: 0 standard, 1 non-linear extrapolation, 2 Lai and Ktaul 2000
  int potev_pm;      // ssnow_potev = 'P-M'
  int reduce_soilevp;  // cable_user%l_new_reduce_soilevp
  int runoff_speed;  // cable_user%l_new_runoff_speed
  int soil_resp_off; // diag_soil_resp = 'OFF'
  CgForcingSpec forc;
  int step_index;    // 0-based counter for the synthetic forcing
  // ACCESS coupling (src/coupled/AM3/control/cable/CM3/cbl_cbm_mod.F90):
  // 0 the offline cbm(), 1 cbm_expl (radiation and canopy; the canopy water,
  // wetness factor and surface temperature are left as they were), 2 cbm_impl
  int mode;
  int final_cycle;   // cbm_impl: 1 on the last implicit cycle of the step (cycleno == numcycles)
  int canopy_pool;   // 1: the canopy kernel runs the block's dryLeaf passes as a
                     // shared-memory pool; 0: each thread its own tile's
  int solve64;       // 1: the soil heat and moisture Thomas solves in FP64 on the
                     // reference's direct form; 0: in FP32 on the step's change
  int lai_refresh;   // cbm_expl: the host model's radiation call ran, so the
                     // snow-reduced LAI is recomputed rather than carried
};

__device__ __forceinline__ float ldf(const float* p, int i) { return __ldg(p + i); }


// half-depths between layer centres (cable_parameters.F90:1828-1831) of the
// constant layer thicknesses, as immediates: zshh(1) = zse(1)/2,
// zshh(k) = (zse(k-1) + zse(k))/2, zshh(ms+1) = zse(ms)/2 (the table's values)
__device__ constexpr float ZSE_C[CG_MS] = {0.022f, 0.058f, 0.154f, 0.409f, 1.085f, 2.872f};
__device__ constexpr float ZSHH[CG_MS + 1] = {0.5f * ZSE_C[0], 0.5f * (ZSE_C[0] + ZSE_C[1]), 0.5f * (ZSE_C[1] + ZSE_C[2]),
                                   0.5f * (ZSE_C[2] + ZSE_C[3]), 0.5f * (ZSE_C[3] + ZSE_C[4]),
                                   0.5f * (ZSE_C[4] + ZSE_C[5]), 0.5f * ZSE_C[5]};

// Phase A record (per tile, [CG_NA][ld]): forcing, roughness, air, radiation,
// interception and the soil liquid water seen by dryLeaf.
#define CG_NA 52
// Phase B record (per tile, [CG_NB][ld]): what soil_snow, carbon and the
// water balance need from define_canopy.
#define CG_NB 19
// rows CG_NB.. of the same record, written only by the canopy kernel of an
// implicit coupled call: dfh_dtg, dfe_dtg, dfn_dtg (the soil-surface flux
// derivatives of the online energy-balance corrections)
#define CG_NB_ALLOC 22
// Soil-snow record (per tile, [CG_NC][ld]) handed from the snow-pack kernel
// to the soil-heat kernel and on to the soil-water kernel.
#define CG_NC 12
// row CG_NC: ssnow%dtmlt(:,1) of an implicit coupled call, summed by the
// snow-pack and soil-heat kernels, read by the soil-water kernel
#define CG_NC_ALLOC 13

template <bool kDiag, bool kCoupled = false>
__device__ __forceinline__ void phase_a(const CgDev& D, const CgTables* __restrict__ T, const StepParams& P, int t) {
  // the coupled-call code exists only in the kCoupled instantiation
  const int mode = kCoupled ? P.mode : 0;
  const int ld = D.ld;
  const float dels = P.dels;
  // ---------------------------------------------------------------- static
  const int iveg = D.iveg[t], isoilm = D.isoilm[t];
  const int v = iveg - 1, so = isoilm - 1;
  const CgPftTable& V = T->pft;
  const CgSoilTable& S = T->soil;
  const float vlai = (iveg >= 14) ? 0.0f : D.vlai[t];   // cable_serial.F90:575
  const float hc = ldf(V.hc, v), canst1 = ldf(V.canst1, v), dleaf = ldf(V.dleaf, v), extkn = ldf(V.extkn, v);
  const float xfang = ldf(V.xfang, v);
  const float refl[2] = {ldf(V.refl1, v), ldf(V.refl2, v)}, taul[2] = {ldf(V.taul1, v), ldf(V.taul2, v)};
  float froot[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) froot[k] = ldf(V.froot[k], v);
  const float ssat = ldf(S.ssat, so), sfc = ldf(S.sfc, so), swilt = ldf(S.swilt, so), css = ldf(S.css, so);
  const float rhosoil = ldf(S.rhosoil, so);
  // soil layer thicknesses (m), cable_parameters.F90:1241: model constants,
  // the same values as the table's, as immediates rather than registers
  constexpr float zse[CG_MS] = {0.022f, 0.058f, 0.154f, 0.409f, 1.085f, 2.872f};

  // ---------------------------------------------------------------- state
  df32 wb[CG_MS], wbice[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wb[k] = df_load(D.wb, CG_MS, ld, k, t); wbice[k] = df_load(D.wbice, CG_MS, ld, k, t); }
  float tgg[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) tgg[k] = D.tgg[k * ld + t];
  float tggsn[3], ssdn[3], smass[3], sdepth[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tggsn[k] = D.tggsn[k * ld + t]; ssdn[k] = D.ssdn[k * ld + t];
    smass[k] = D.smass[k * ld + t]; sdepth[k] = D.sdepth[k * ld + t];
  }
  uint8_t flags = D.flags[t];
  int isflag = flags & 1;
  float snowd = D.snowd[t], ssdnn = D.ssdnn[t], snage = D.snage[t];
  const float owetfac_in = D.owetfac[t];
  float wb_lake = D.wb_lake[t], wbtot1 = D.wbtot1[t], wbtot2 = D.wbtot2[t];
  const float oldcansto = D.cansto[t];

  // ---------------------------------------------------------------- forcing
  float F[CG_NFORC];
  if (D.forcing_in) {
    // device tile order, or the caller's order straight from the host-I/O
    // staging buffer (one gather instead of a reordering pass)
    const size_t base = D.forcing_caller_order == 1 ? (size_t)D.tile_id[t] : (size_t)t;
    const size_t stride = D.forcing_caller_order ? (size_t)D.mp : (size_t)ld;
#pragma unroll
    for (int i = 0; i < CG_NFORC; ++i) F[i] = D.forcing_in[i * stride + base];
  } else {
    cg_forcing(P.forc, D.lat[t], D.lonphase[t], D.tbase[t], D.swscale[t], (uint32_t)D.tile_id[t],
               (uint32_t)P.step_index, F);
  }
  if (D.forcing_out) {
#pragma unroll
    for (int i = 0; i < CG_NFORC; ++i) D.forcing_out[i * ld + t] = F[i];
  }
  const float fsd0 = F[CGF_FSD1], fsd1 = F[CGF_FSD2], fld = F[CGF_FLD], precip = F[CGF_PRECIP];
  const float precip_sn = F[CGF_PRECIP_SN], tk = F[CGF_TK], pmb = F[CGF_PMB], ua = F[CGF_UA], qv = F[CGF_QV];
  const float ca = F[CGF_CA], coszen = F[CGF_COSZEN], doy = F[CGF_DOY];
  const float tvrad = tk;
  // the driver's forcing checks (cable_input.F90:2683-2689; ranges
  // cable_checks.F90:60-70): SWdown, LWdown, Qair, Rainf, Wind, Tair, PSurf
  if (out_of(fsd0 + fsd1, 0.f, 1360.f) || out_of(fld, 0.f, 950.f) || out_of(qv, 0.f, 0.1f) ||
      out_of(precip / P.dels, 0.f, 0.1f) || out_of(ua, 0.f, 75.f) || out_of(tk, 200.f, 333.f) ||
      out_of(pmb, 500.f, 1100.f))
    D.tile_status[t] |= CG_TS_FORCING_RANGE;

  // wbliq as left by the previous soil_snow call
  float wbliq0[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) wbliq0[k] = df_sub(wb[k], wbice[k]);

  // lakes top-layer fix (cbl_model_driver_offline.F90:116-121); the
  // coupled cbm_expl / cbm_impl have none
  const bool offline = mode == 0;
  if (offline) {
    if (iveg == LAKES && df_lt(wb[0], df32{sfc, 0.f})) {
      wbtot1 = wb[0].hi * DLIQ * zse[0];
      wb[0] = df32{sfc, 0.f};
      wbtot2 = wb[0].hi * DLIQ * zse[0];
    }
    wb_lake = wb_lake + fmaxf(wbtot2 - wbtot1, 0.f);
  }

  // ---------------------------------------------------------------- ruff_resist
  // cable_roughness.F90:64-332, roughnessHGT_effLAI_cbl.F90:42-149
  float hruff, vlaiw, z0soilsn, z0m, disp, zref_uv, zref_tq, zruffs, rt0us, rt1usa, rt1usb, usuh, coexp;
  {
    float den_eff = fmaxf(100.0f, ssdnn);
    hruff = fmaxf(1.0e-6f, hc - (1.2f * snowd / den_eff));
    vlaiw = vlai * (hruff / fmaxf(0.01f, hc));
    // coupled calls: ruff_resist leaves canopy%vlaiw alone
    // (cable_roughness.F90:176-186); it holds the LAI_eff of the host
    // model's last radiation call (cable_land_albedo_mod_cbl.F90:263,
    // cbl_um_update_canopy.F90:27), the same function of the snow state
    if (mode != 0) {
      if (P.lai_refresh) D.vlaiw[t] = vlaiw;
      else vlaiw = D.vlaiw[t];
    }
    float z0soil = 0.0009f * fminf(1.0f, vlaiw) + 1.e-4f;
    z0soilsn = z0soil;
    if (snowd > 0.01f) z0soilsn = fmaxf(1.e-7f, z0soil - z0soil * fminf(snowd, 10.f) / 10.f);
    if (snowd > 0.01f && iveg == ICE_SURF) z0soilsn = fmaxf(z0soilsn, 1.e-4f);
    usuh = fminf(sqrtf(CSD + CRD * (vlaiw * 0.5f)), USUHM);
    float xx = sqrtf(CCD * fmaxf(vlaiw * 0.5f, 0.0005f));
    float dh = 1.0f - (1.0f - expf(-xx)) / xx;
    coexp = usuh / (VONK * CCW_C * (1.0f - dh));
    if (vlaiw <= LAI_THRESH || hruff < z0soilsn) {
      z0m = z0soilsn; rt0us = 0.f; disp = 0.f;
      zref_uv = fmaxf(fmaxf(3.5f + z0m, 40.0f), hruff - disp);
      zref_tq = zref_uv;
      zruffs = 0.f; rt1usa = 0.f; rt1usb = 0.f;
    } else {
      disp = dh * hruff;
      z0m = ((1.0f - dh) * expf(logf(CCW_C) - 1.f + 1.f / CCW_C - VONK / usuh)) * hruff;
      zref_uv = fmaxf(fmaxf(3.5f + z0m, 40.0f), hruff - disp);
      zref_tq = zref_uv;
      const float e2 = expf(2.f * CSW * vlaiw);
      float term2 = expf(2.f * CSW * vlaiw * (1.f - disp / hruff));
      float term3 = A33 * A33 * CTL * 2.f * CSW * vlaiw;
      float term5 = fmaxf((2.f / 3.f) * hruff / disp, 1.0f);
      rt0us = term5 * (ZDLIN * logf(ZDLIN * disp / z0soilsn) + (1.f - ZDLIN)) * (e2 - term2) / term3;
      zruffs = disp + hruff * A33 * A33 * CTL / VONK / term5;
      rt1usa = term5 * (term2 - 1.0f) / term3;
      rt1usb = term5 * (fminf(zref_tq + disp, zruffs) - hruff) / (A33 * A33 * CTL * hruff);
      rt1usb = fmaxf(rt1usb, 0.0f);
    }
  }

  // define_air (cable_air.F90:51-97) with tvair = tk
  float rho, cmolar, epsi, visc, psyc, dsatdk;
  const float rlam = HL;
  {
    float tc = tk - TFRZ;
    float es = TETENA * expf(TETENB * tc / (TETENC + tc));
    cmolar = pmb * 100.0f / (RGAS * tk);
    rho = fminf(1.3f, RMAIR * cmolar);
    epsi = (rlam / CAPP) * (RMH2O / RMAIR) * es * TETENB * TETENC / sqf(TETENC + tc) / pmb;
    visc = 1e-5f * fmaxf(1.0f, 1.35f + 0.0092f * tc);
    psyc = pmb * 100.0f * CAPP * RMAIR / rlam / RMH2O;
    dsatdk = 100.0f * (TETENA * TETENB * TETENC) / sqf(tc + TETENC) * expf(TETENB * tc / (tc + TETENC));
  }
  const bool veg_mask = vlaiw > LAI_THRESH;
  const bool sunlit_veg = veg_mask && (fsd0 + fsd1) > RAD_THRESH;

  // ---------------------------------------------------------------- init_radiation + albedo
  // cbl_init_radiation.F90:30-392, cbl_spitter.F90, cbl_rhoch.F90,
  // cbl_albedo.F90:56-386, cbl_snow_albedo.F90:36-161
  float extkb, extkd, extkbm[2], extkdm[2], fbeam[2], albsoilsn[2], reffdf[2], reffbm[2], cexpkbm[2], cexpkdm[2];
  float albedo[2];
  {
    float xphi1 = 0.f, xphi2 = 0.f;
    if (veg_mask) {
      xphi1 = 0.5f - xfang * (0.633f + 0.33f * xfang);
      xphi2 = 0.877f * (1.0f - 2.0f * xphi1);
    }
    const float cos3[3] = {0.96592583f, 0.70710678f, 0.25881905f};   // cos(15, 45, 75 deg)
    float xk[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) xk[b] = veg_mask ? xphi1 / cos3[b] + xphi2 : 0.0f;
    float c1[2], rhoch[2];
#pragma unroll
    for (int b = 0; b < 2; ++b) { c1[b] = sqrtf(1.0f - taul[b] - refl[b]); rhoch[b] = (1.0f - c1[b]) / (1.0f + c1[b]); }
    extkb = 0.5f; extkd = 0.7f;
    if (veg_mask)
      extkd = -logf(GW0 * expf(-xk[0] * vlaiw) + GW1 * expf(-xk[1] * vlaiw) + GW2 * expf(-xk[2] * vlaiw)) / vlaiw;
    if (veg_mask && coszen > COSZEN_TOLS * 1e-2f) extkb = xphi1 / coszen + xphi2;
    if (coszen < COSZEN_TOLS * 1e-2f) extkb = 1.0e5f;
    if (fabsf(extkb - extkd) < 0.001f) extkb = extkd + 0.001f;
#pragma unroll
    for (int b = 0; b < 2; ++b) { extkbm[b] = veg_mask ? extkb * c1[b] : 0.0f; extkdm[b] = extkd * c1[b]; }
    // spitter (cbl_spitter.F90:36-76)
    {
      float fsd = fsd0 + fsd1;
      float tmpr = 0.847f + coszen * (1.04f * coszen - 1.61f);
      float tmpk = (1.47f - tmpr) / 1.66f;
      float tmprat = 0.0f;
      if (coszen > 1.0e-10f && fsd > 10.0f)
        tmprat = fsd / (1370.0f * (1.0f + 0.033f * cosf(2.0f * PI_C * ((float)(int)doy - 10.0f) / 365.0f)) * coszen);
      float fb = 0.0f;
      if (tmprat > 0.22f) fb = 6.4f * sqf(tmprat - 0.22f);
      if (tmprat > 0.35f) fb = fminf(1.66f * tmprat - 0.4728f, 1.0f);
      if (tmprat > tmpk) fb = fmaxf(1.0f - tmpr, 0.0f);
      if (coszen < COSZEN_TOLS * 1e2f) fb = 0.0f;
      fbeam[0] = fb; fbeam[1] = fb;
    }
    // surface_albedosn
    float soilalb = D.albsoil[t];
    if (iveg == LAKES) soilalb = -0.022f * (fminf(275.0f, fmaxf(260.0f, tgg[0])) - 260.0f) + 0.45f;
    if (snowd > 1.0f && iveg == LAKES) soilalb = 0.85f;
    float sfact = 0.68f;
    if (soilalb <= 0.14f) sfact = 0.5f;
    else if (soilalb <= 0.20f) sfact = 0.62f;
    albsoilsn[1] = 2.0f * soilalb / (1.0f + sfact);
    albsoilsn[0] = sfact * albsoilsn[1];
    float snrat = 0.f, alir = 0.f, alv = 0.f;
    if (snowd > 1.0f) {
      float tmp = snowd / fmaxf(ssdnn, 200.0f);
      snrat = fminf(1.0f, tmp / (tmp + 0.1f));
      float fage = 1.0f - 1.0f / (1.0f + snage);
      tmp = fmaxf(0.17365f, coszen);
      float fzenm = fmaxf(0.0f, (tmp > 0.5f) ? 0.0f : 1.5f / (1.0f + 4.0f * tmp) - 0.5f);
      tmp = 0.95f * (1.0f - 0.2f * fage);
      alv = 0.4f * fzenm * (1.0f - tmp) + tmp;
      tmp = 0.70f * (1.0f - 0.5f * fage);
      alir = 0.4f * fzenm * (1.0f - tmp) + tmp;
    }
    albsoilsn[1] = fminf(0.70f, (1.0f - snrat) * albsoilsn[1] + snrat * alir);
    albsoilsn[0] = fminf(0.95f, (1.0f - snrat) * albsoilsn[0] + snrat * alv);
    if (isoilm == ICE_SOIL) { albsoilsn[0] = 0.95f - 0.05f; albsoilsn[1] = 0.70f - 0.05f; }
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      float rhocbm = veg_mask ? 2.0f * extkb / (extkb + extkd) * rhoch[b] : 0.0f;
      float rhocdf = rhoch[b] * 2.0f * (GW0 * xk[0] / (xk[0] + extkd) + GW1 * xk[1] / (xk[1] + extkd) +
                                        GW2 * xk[2] / (xk[2] + extkd));
      cexpkbm[b] = veg_mask ? expf(-fminf(extkbm[b] * vlaiw, 20.0f)) : 0.0f;
      cexpkdm[b] = expf(-(extkdm[b] * vlaiw));
      reffdf[b] = albsoilsn[b]; reffbm[b] = albsoilsn[b]; albedo[b] = albsoilsn[b];
      if (veg_mask) {
        reffdf[b] = rhocdf + (albsoilsn[b] - rhocdf) * sqf(cexpkdm[b]);
        reffbm[b] = rhocbm + (albsoilsn[b] - rhocbm) * sqf(cexpkbm[b]);
        albedo[b] = (1.0f - fbeam[b]) * reffdf[b] + fbeam[b] * reffbm[b];
      }
    }
  }

  // ================================================================ define_canopy
  // cable_canopy.F90:10-1048
  float cansto = oldcansto;
  const float cansat = canst1 * vlaiw;
  // Surf_wetness_fact (cbl_SurfaceWetness.F90:10-79)
  float through, fwet, wetfac;
  {
    float upper = 4.0f * fminf(dels, 1800.0f) / (60.0f * 1440.0f);
    float ftemp = fminf(precip - precip_sn, upper);
    upper = fmaxf(cansat - cansto, 0.0f);
    float wcint = (ftemp > 0.0f && tk > TFRZ) ? fminf(upper, ftemp) : 0.0f;
    through = precip_sn + fminf(precip - precip_sn, fmaxf(0.0f, precip - precip_sn - wcint));
    cansto = cansto + wcint;
    fwet = fmaxf(0.0f, fminf(0.9f, 0.8f * cansto / fmaxf(cansat, 0.01f)));
    // initialize_wetfac (cbl_init_wetfac_mod.F90:9-116)
    float wilting_pt = swilt / 2.0f;
    float den = fmaxf(0.0830f, sfc - wilting_pt);
    wetfac = fmaxf(0.0f, fminf(1.0f, (wb[0].hi - wilting_pt) / den));
    if (wbice[0].hi > 0.0f) {
      // (wbice / wb)^2 in FP32: the quotient of the FP32-rounded values is
      // within a few ulp of the reference's r_2 quotient rounded to REAL
      const float q = wbice[0].hi / wb[0].hi;
      float ice_ratio = q * q;
      float ice_factor = fmaxf(0.5f, 1.0f - fminf(0.2f, ice_ratio));
      wetfac = wetfac * ice_factor;
    }
    if (snowd > 0.1f) wetfac = 0.9f;
    if (iveg == LAKES) wetfac = (tk >= TFRZ + 5.f) ? 1.0f : 0.7f;
    wetfac = 0.5f * (wetfac + owetfac_in);
  }
  // working variables of the canopy iteration
  float tvair = tk, qvair = qv;
  float qstvair = qsatfjh(tvair - TFRZ, pmb);
  float dva = (qstvair - qvair) * RMAIR / RMH2O * pmb * 100.0f;
  float dsx = fmaxf(dva, 0.0f);
  float evapfbl[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) evapfbl[k] = 0.0f;
  float tss = (float)(1 - isflag) * tgg[0] + (float)isflag * tggsn[0];
  const float tss4 = pow4(tss);
  // radiation (cbl_radiation.F90:30-218)
  float transd, transb, flws, qssabs, fvlai[2], scalex[2], rniso[2], gradis[2], qcan_par[2], swcan;
  {
    float cf2n = expf(-extkn * vlaiw);
    transd = veg_mask ? expf(-extkd * vlaiw) : 1.0f;
    transb = expf(-fminf(extkb * vlaiw, 30.f));
    float flpwb = SBOLTZ * pow4(tvrad);
    float flwv = EMLEAF * flpwb;
    flws = SBOLTZ * EMSOIL * pow4(tss);
    float emair = fld / flpwb;
    float qlw[2] = {0.f, 0.f};
    gradis[0] = 0.f; gradis[1] = 0.f;
    if (veg_mask) {
      gradis[0] = (4.0f * EMLEAF / (CAPP * rho)) * flpwb / tvrad * extkd *
                  ((1.0f - transb * transd) / (extkb + extkd) + (transd - transb) / (extkb - extkd));
      gradis[1] = (8.0f * EMLEAF / (CAPP * rho)) * flpwb / tvrad * extkd * (1.0f - transd) / extkd - gradis[0];
      qlw[0] = (flws - flwv) * extkd * (transd - transb) / (extkb - extkd) +
               (emair - EMLEAF) * extkd * flpwb * (1.0f - transd * transb) / (extkb + extkd);
      qlw[1] = (1.0f - transd) * (flws + fld - 2.0f * flwv) - qlw[0];
    }
    gradis[0] = fmaxf(1.0e-3f, cmolar * gradis[0]);
    gradis[1] = fmaxf(1.0e-3f, cmolar * gradis[1]);
    float qsw[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    if (sunlit_veg) {
      const float fsdb[2] = {fsd0, fsd1};
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        float cf1 = (1.0f - transb * cexpkdm[b]) / (extkb + extkdm[b]);
        float cf3 = (1.0f - transb * cexpkbm[b]) / (extkb + extkbm[b]);
        float direct = fbeam[b] * (1.0f - taul[b] - refl[b]) * extkb *
                       ((1.f - transb) / extkb - (1.f - transb * transb) / (extkb + extkb));
        qsw[0][b] = fsdb[b] * ((1.0f - fbeam[b]) * (1.0f - reffdf[b]) * extkdm[b] * cf1 +
                               fbeam[b] * (1.0f - reffbm[b]) * extkbm[b] * cf3 + direct);
        qsw[1][b] = fsdb[b] * ((1.0f - fbeam[b]) * (1.0f - reffdf[b]) * extkdm[b] * ((1.0f - cexpkdm[b]) / extkdm[b] - cf1) +
                               fbeam[b] * (1.f - reffbm[b]) * extkbm[b] * ((1.0f - cexpkbm[b]) / extkbm[b] - cf3) - direct);
      }
      qssabs = fsd0 * (fbeam[0] * (1.f - reffbm[0]) * expf(-fminf(extkbm[0] * vlaiw, 20.f)) +
                       (1.f - fbeam[0]) * (1.f - reffdf[0]) * expf(-fminf(extkdm[0] * vlaiw, 20.f))) +
               fsd1 * (fbeam[1] * (1.f - reffbm[1]) * cexpkbm[1] + (1.f - fbeam[1]) * (1.f - reffdf[1]) * cexpkdm[1]);
      scalex[0] = (1.0f - transb * cf2n) / (extkb + extkn);
      fvlai[0] = (1.0f - transb) / extkb;
      fvlai[1] = vlaiw - fvlai[0];
    } else {
      qssabs = (1.0f - albsoilsn[0]) * fsd0 + (1.0f - albsoilsn[1]) * fsd1;
      scalex[0] = 0.f; fvlai[0] = 0.f; fvlai[1] = vlaiw;
    }
    scalex[1] = (1.0f - cf2n) / extkn - scalex[0];
    qcan_par[0] = qsw[0][0]; qcan_par[1] = qsw[1][0];
    rniso[0] = qsw[0][0] + qsw[0][1] + qlw[0];
    rniso[1] = qsw[1][0] + qsw[1][1] + qlw[1];
    swcan = qsw[0][0] + qsw[1][0] + qsw[0][1] + qsw[1][1];
  }
  const float sum_rad_rniso = rniso[0] + rniso[1];

  (void)sunlit_veg;
  {
    const float rec[CG_NA] = {tk, qv, pmb, ua, fld, ca, precip, precip_sn, vlaiw, hruff, z0soilsn, z0m, disp, zref_uv, zruffs, rt0us, rt1usa, rt1usb, usuh, coexp, rho, cmolar, epsi, visc, psyc, dsatdk, extkb, transd, flws, qssabs, fvlai[0], fvlai[1], scalex[0], scalex[1], rniso[0], rniso[1], gradis[0], gradis[1], qcan_par[0], qcan_par[1], swcan, cansto, through, fwet, wetfac, tss, wbliq0[0], wbliq0[1], wbliq0[2], wbliq0[3], wbliq0[4], wbliq0[5]};
#pragma unroll
    for (int i = 0; i < CG_NA; ++i) D.work_a[i * ld + t] = rec[i];
  }
  if (offline) {
    if (iveg == LAKES) df_store(D.wb, CG_MS, ld, 0, t, wb[0]);
    D.wb_lake[t] = wb_lake; D.wbtot1[t] = wbtot1; D.wbtot2[t] = wbtot2;
  }
  if (kDiag) {
    D.diag[29 * ld + t] = albedo[0]; D.diag[30 * ld + t] = albedo[1]; D.diag[31 * ld + t] = transd;
    D.diag[47 * ld + t] = qssabs; D.diag[48 * ld + t] = sum_rad_rniso; D.diag[49 * ld + t] = vlaiw;
  }
}

// The plant-type table the canopy kernel re-reads inside its dryLeaf
// iteration, in constant memory (one copy per translation unit that includes
// this header; phase_b.cu uploads its copy, upload_canopy_pft_table).  Tiles
// are grouped by plant type, so a warp's reads are almost always of one
// address: a constant-cache broadcast rather than an L1 load on the
// iteration's dependency chain.  The table is the same for every context.
static __constant__ CgPftTable c_pft;
// A read of c_pft.  Constant-bank loads are cheap for the compiler to
// re-issue where a value is used, so unlike ldv's reads these need no
// protection against being hoisted into registers.
__device__ __forceinline__ float ldk(const float& x) { return x; }

// kHarvest: sampled tiles append a training row for the surrogate network
// (features at the start of the first Monin-Obukhov iteration's dryLeaf and
// its converged result) to D.harvest.  kSur: the first
// iteration's dryLeaf starts from the network's leaf temperature (the
// surrogate; see the comment at its use).
// A read of a read-only table entry that the compiler may not hoist or keep
// in a register: re-reading it where it is used costs an L1 hit, holding it
// live through the dryLeaf iteration costs the canopy kernel registers.
__device__ __forceinline__ float ldv(const float* p) {
  float r;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(r) : "l"(p));
  return r;
}

// transp_soil_water (cbl_remove_trans.F90:43-93): root-weighted extraction of
// fe_mm (mm of transpiration over the step) from the layers, each layer's
// deficit carried to the next; returns the total.  Explicitly rounded
// operations, so a given fe_mm yields the same layer amounts wherever this is
// evaluated: the canopy iteration keeps only fe_mm of the latest extracting
// pass and of its best iterate, and rebuilds both layer arrays afterwards.
__device__ __forceinline__ float transp_extract(float fe_mm, const float (&froot)[CG_MS], const float (&avail)[CG_MS],
                                                float (&ev)[CG_MS]) {
  float diffp = 0.f, se = 0.f;
#pragma unroll
  for (int kk = 0; kk < CG_MS; ++kk) {
    const float xx = __fadd_rn(__fmul_rn(fe_mm, froot[kk]), diffp);
    const float xxd = __fsub_rn(xx, avail[kk]);
    if (xxd > 0.0f) { ev[kk] = avail[kk]; diffp = xxd; }
    else { ev[kk] = xx; diffp = 0.0f; }
    se = __fadd_rn(se, ev[kk]);
  }
  return se;
}

// kPool: the dryLeaf passes of the block's tiles run as a pool in shared
// memory sm (dryleaf.cuh); every thread of the block must then call this
// (threads beyond the last tile call dl_pool_idle instead).
}  // namespace cg
// the dryLeaf pass and its schedules (uses c_pft, ldk and transp_extract above)
#include "dryleaf.cuh"
namespace cg {

template <bool kDiag, bool kHarvest = false, bool kSur = false, bool kCoupled = false, bool kPool = false>
__device__ __forceinline__ void phase_b(const CgDev& D, const CgTables* __restrict__ T, const StepParams& P, int t_in,
                                        float* sm = nullptr) {
  // A pooling block's threads beyond the last tile ("ghosts") run the last
  // tile's code path and store nothing, so every thread of the block reaches
  // the pool's barriers and votes on one path; they leave after the
  // Monin-Obukhov loop, the last code with barriers.
  const bool ghost = kPool && t_in >= D.mp;
  const int t = ghost ? D.mp - 1 : t_in;
  // the coupled-call code exists only in the kCoupled instantiation
  const int mode = kCoupled ? P.mode : 0;
  const int ld = D.ld;
  const float dels = P.dels;
  const int iveg = D.iveg[t], isoilm = D.isoilm[t];
  const int v = iveg - 1, so = isoilm - 1;
  (void)isoilm;
  const CgPftTable& V = T->pft;
  const CgSoilTable& S = T->soil;
  float froot[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) froot[k] = ldf(V.froot[k], v);
  const float sfc = ldf(S.sfc, so), swilt = ldf(S.swilt, so);
  // soil layer thicknesses (m), cable_parameters.F90:1241: model constants,
  // the same values as the table's, as immediates rather than registers
  constexpr float zse[CG_MS] = {0.022f, 0.058f, 0.154f, 0.409f, 1.085f, 2.872f};
  // phase A record
  const float* WA = D.work_a;
  auto A = [&](int i) { return WA[i * ld + t]; };
  const float tk = A(0), qv = A(1), pmb = A(2), ua = A(3), fld = A(4), ca = A(5);
  const float vlaiw = A(8), hruff = A(9), z0soilsn = A(10), z0m = A(11), disp = A(12), zref_uv = A(13);
  const float zref_tq = zref_uv, zruffs = A(14), rt0us = A(15), rt1usa = A(16), rt1usb = A(17), usuh = A(18);
  const float coexp = A(19), rghlai = vlaiw;
  const float rho = A(20), cmolar = A(21), epsi = A(22), visc = A(23), psyc = A(24), dsatdk = A(25);
  const float rlam = HL;
  const float extkb = A(26), transd = A(27), flws = A(28), qssabs = A(29);
  const float fvlai[2] = {A(30), A(31)}, scalex[2] = {A(32), A(33)}, rniso[2] = {A(34), A(35)};
  const float gradis[2] = {A(36), A(37)}, qcan_par[2] = {A(38), A(39)};
  const float swcan = A(40);
  float cansto = A(41), through = A(42);
  const float fwet = A(43);
  float wetfac = A(44);
  const float tss = A(45);
  float wbliq0[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) wbliq0[k] = A(46 + k);
  const float cansat = ldf(V.canst1, v) * vlaiw;
  const bool veg_mask = vlaiw > LAI_THRESH;
  const float sum_rad_rniso = rniso[0] + rniso[1];
  const float sum_rad_gradis = gradis[0] + gradis[1];
  const float tss4 = pow4(tss);
  const float tvrad = tk;
  // litter resistances to heat and vapour (cable_canopy.F90:471-476,
  // :987-988), zero unless the litter switch is on; rho is fixed over the
  // iteration, so they are too.  Recomputed where used rather than kept
  // live through the dryLeaf iteration.
  auto litter_resist = [&](float& rhlitt, float& relitt) {
    rhlitt = 0.f; relitt = 0.f;
    if (P.litter) {
      const float cl = (float)(1 - (D.flags[t] & 1)) * ldf(V.clitt, v) * 0.003f;
      rhlitt = cl / KTH_LITT / (rho * CAPP);
      relitt = cl / DV_LITT;
    }
  };
  // state read by define_canopy
  const float oldcansto = D.cansto[t], ortsoil = D.rtsoil[t], snowd = D.snowd[t], pudsto = D.pudsto[t];
  const float tgg[1] = {D.tgg[t]};
  const df32 wb[1] = {df_load(D.wb, CG_MS, ld, 0, t)}, wbice[1] = {df_load(D.wbice, CG_MS, ld, 0, t)};
  const float pudsmx = 0.0f;
  // working variables of the canopy iteration (cable_canopy.F90:183-215)
  float tvair = tk, qvair = qv, tv = tk;
  float qstvair = qsatfjh(tvair - TFRZ, pmb);
  float dva = (qstvair - qvair) * RMAIR / RMH2O * pmb * 100.0f;
  float dsx = fmaxf(dva, 0.0f);
  float tlfx = tk, tlfy = tk;
  float csx[2] = {ca, ca};
  float gswx[2] = {1e-3f, 1e-3f};
  float gbhu[2] = {1e-3f, 1e-3f}, gbhf[2] = {1e-3f, 1e-3f};
  float evapfbl[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) evapfbl[k] = 0.0f;
  // per-PFT photosynthesis parameters (gathered once)
  // per-PFT photosynthesis parameters: re-read from the (L1-resident) table
  // where used instead of being held in registers through the iteration
  const float vbeta = ldf(V.vbeta, v), shelrb = ldf(V.shelrb, v);

  // stability parameter of the current Monin-Obukhov iteration (canopy%zetar:
  // 0 for the first, then each iteration's update_zetar result)
  float zeta = 0.0f;
  float us = 0.f, rt0 = 0.f, rt1 = 0.f, rt1usc = 0.f, rtsoil = ortsoil, cls = 1.f;
  float fev = 0.f, fhv = 0.f, fnv = 0.f, fns = 0.f, fhs = 0.f, fe = 0.f, fh = 0.f, potev = 0.f;
  // canopy%ga persists between steps; read before it is set only by ssnow_potev = 'P-M' (the
  // output row "ga" holds the last step's value)
  float ga = P.potev_pm ? D.out[6 * ld + t] : 0.f;
  float fes = 0.f, fess = 0.f, fesp = 0.f, fevw = 0.f, fhvw = 0.f, fevw_pot = 0.f, fevc = 0.f, epot = 0.f;
  float ecy = 0.f, hcy = 0.f, rny = 0.f, frday = 0.f, fpn = 0.f, fwsoil = 1.0f, qstss = 0.f;
  int passes_total = 0;
  // surrogate and harvest bookkeeping
  unsigned int sur_tried = 0, sur_accepted = 0;
  const bool harvesting = kHarvest && D.harvest != nullptr;
  // soil water limitation of stomatal conductance, computed once in the
  // first Monin-Obukhov iteration of the reference (cbl_dryLeaf.F90:168-181)
  if (P.fwsoil_mode == 0) {   // fwsoil_calc_std (cbl_fwsoil.F90:13-38)
    float rwater = 0.f;
#pragma unroll
    for (int k = 0; k < CG_MS; ++k)
      rwater += froot[k] * fmaxf(1.0e-9f, fminf(1.0f, (wbliq0[k] - swilt) / (sfc - swilt)));
    rwater = fmaxf(1.0e-9f, rwater);
    fwsoil = P.medlyn ? fmaxf(1.0e-4f, fminf(1.0f, rwater)) : fmaxf(1.0e-9f, fminf(1.0f, vbeta * rwater));
  } else if (P.fwsoil_mode == 1) {
    // fwsoil_calc_non_linear (cbl_fwsoil.F90:44-88): quadratic through
    // (swilt, 0), (midpoint, 0.9), (sfc, 1) of the root-weighted water
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) sum += froot[k] * fmaxf(0.0f, fminf(1.0f, wbliq0[k] - swilt));
    float rwater = fmaxf(1.0e-9f, sum / (sfc - swilt));
    rwater = swilt + rwater * (sfc - swilt);
    const float x1 = swilt, x2 = swilt + (sfc - swilt) / 2.0f, x3 = sfc;
    const float s2 = (rwater - x1) / (x2 - x1) * (rwater - x3) / (x2 - x3);
    const float s3 = (rwater - x1) / (x3 - x1) * (rwater - x2) / (x3 - x2);
    fwsoil = (rwater < sfc - 0.02f) ? fmaxf(0.f, fminf(1.f, 0.9f * s2 + s3)) : 1.0f;
  } else {
    // fwsoil_calc_Lai_Ktaul (cbl_fwsoil.F90:90-112); a layer drier than
    // wilting takes the 1e-4 floor (a negative base to a non-integer
    // power in the reference, compiler-dependent there)
    const float ssat = ldf(S.ssat, so);
    float fw = 0.f;
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) {
      const float avail = wbliq0[k] - swilt;
      const float dummy = 0.01f / fmaxf(1.0e-3f, avail);
      const float base = avail / ssat;
      const float frw = (base > 0.f) ? fmaxf(1.0e-4f, __powf(base, dummy)) : 1.0e-4f;
      fw = fminf(1.0f, fmaxf(fw, frw));
    }
    fwsoil = fw;
  }
  // water each layer can give to transpiration, fixed over the step
  // (transp_soil_water, cbl_remove_trans.F90:62-63)
  float dk_avail[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) dk_avail[k] = fmaxf(0.0f, wbliq0[k] - 1.1f * swilt) * zse[k] * DLIQ;
  for (int iter = 1; iter <= NITER; ++iter) {
    const float zi = zeta;
    // comp_friction_vel (cbl_friction_vel.F90:19-108)
    {
      float psim_1 = psim(zi * zref_uv / zref_tq);
      float rescale = VONK * fmaxf(ua, UMIN);
      float psim_2 = psim(zi * z0m / zref_tq);
      us = fminf(fmaxf(1.e-6f, rescale / (logf(zref_uv / z0m) - psim_1 + psim_2)), 10.0f);
    }
    // resistances (cable_canopy.F90:276-363)
    {
      float xx = 0.5f + fsignf(0.5f, zref_tq + disp - zruffs);
      float zr = fmaxf(zruffs - disp, z0soilsn);
      rt1usc = xx * (logf(zref_tq / zr) - psis(zi) + psis(zi * zr / zref_tq)) / VONK;
      rt0 = fmaxf(5.f, rt0us / us);
      rt1 = fmaxf(5.f, (rt1usa + rt1usb + rt1usc) / us);
      rtsoil = veg_mask ? rt0 : rt0 + rt1;
      rtsoil = fmaxf(5.f, rtsoil);
      if (rtsoil > 2.f * ortsoil || rtsoil < 0.5f * ortsoil) rtsoil = fmaxf(5.f, 0.5f * (rtsoil + ortsoil));
    }
    // boundary-layer conductance (:374-397)
    if (veg_mask) {
      const float dl = ldk(c_pft.dleaf[v]);
      float gbvtop = cmolar * APOL * visc / PRANDT / dl * sqrtf(us / fmaxf(usuh, 1.e-6f) * dl / visc) *
                     0.89194175f /* prandt**(1/3) */ / shelrb;
      gbvtop = fmaxf(0.05f, gbvtop);
      gbhu[0] = gbvtop * (1.0f - expf(-fminf(vlaiw * (0.5f * coexp + extkb), 20.0f))) / (extkb + 0.5f * coexp);
      gbhu[1] = (2.0f / coexp) * gbvtop * (1.0f - expf(-fminf(0.5f * coexp * vlaiw, 20.0f))) - gbhu[0];
    }
    // ------------------------------------------------ dryLeaf (cbl_dryLeaf.F90:10-666)
    {
      // surrogate inputs: the state the first iteration starts from
      const float tlf_entry = tlfx;
      bool sampled = false;
      if (harvesting && iter == 1 && veg_mask && !ghost) {
        uint32_t c4[4] = {(uint32_t)D.tile_id[t], (uint32_t)P.step_index, 0xD1EAF001u, 0u};
        cg_philox(c4, D.harvest_seed);
        sampled = cg_u01(c4[0]) < D.harvest_prob;
      }
      float feat[12];
      if (sampled) {
        const float sc = scalex[0] + scalex[1];
        feat[0] = qcan_par[0]; feat[1] = qcan_par[1]; feat[2] = tlfx; feat[3] = dsx; feat[4] = ca;
        feat[5] = ldk(c_pft.vcmax[v]) * sc; feat[6] = ldk(c_pft.ejmax[v]) * (1.0f - ldk(c_pft.frac4[v])) * sc; feat[7] = P.medlyn ? ldk(c_pft.g1[v]) : ldk(c_pft.a1gs[v]);
        feat[8] = fwsoil; feat[9] = vlaiw; feat[10] = ua; feat[11] = tk;
      }
      bool sur_try = false;
      float tlf_sur = tlfx;
      if (kSur && iter == 1 && veg_mask) {
        const float dt = D.sur_dt[t];
        if (isfinite(dt)) { sur_try = true; tlf_sur = tlf_entry + dt; }
      }
      // the call's inputs and the iteration's start (cbl_dryLeaf.F90:183-237)
      DlCtx c;
      c.v = v; c.tk = tk; c.ca = ca; c.cmolar = cmolar; c.psyc = psyc; c.dsatdk = dsatdk; c.fwet = fwet;
      c.fwsoil = fwsoil;
#pragma unroll
      for (int l = 0; l < 2; ++l) {
        c.scalex[l] = scalex[l]; c.fvlai[l] = fvlai[l]; c.gradis[l] = gradis[l]; c.rniso[l] = rniso[l];
        c.qcan_par[l] = qcan_par[l]; c.gbhu[l] = gbhu[l];
      }
#pragma unroll
      for (int q = 0; q < CG_MS; ++q) c.dk_avail[q] = dk_avail[q];
      c.tvair = tvair; c.dva = dva; c.conv = 0.1f;
      DlState st;
      st.tlfx = tlfx; st.dsx = dsx;
#pragma unroll
      for (int l = 0; l < 2; ++l) { st.csx[l] = csx[l]; st.gswx[l] = gswx[l]; st.gbhf[l] = gbhf[l]; st.psycst[l] = psyc; }
      st.abs_deltlf = 999.0f; st.deltlfy = 999.0f; st.ecx = sum_rad_rniso;
      st.rny = sum_rad_rniso; st.hcy = 0.f; st.ecy = sum_rad_rniso; st.tlfy = tlfy;
      st.rdy_sum = 0.f; st.an_y_sum = 0.f; st.fe_mm_best = 0.f; st.fe_mm_last = 0.f; st.k = 0;
      // With the surrogate the first iteration starts from the network's
      // leaf temperature.  The first pass is the closure test of the
      // prediction: when the leaf energy balance evaluated there moves the
      // leaf temperature by at most D.sur_gate the tile is done in one pass.
      // Otherwise, in strict mode the tile restarts the plain iteration from
      // its usual start (bitwise the plain result); in warm mode the plain
      // iteration continues from the prediction to the gate as its
      // convergence test (cbl_dryLeaf.F90 uses 0.1 K).
      const DlState entry = st;
      if (sur_try) {
        ++sur_tried;
        st.tlfx = tlf_sur;
        st.dsx = fmaxf(dva + dsatdk * (st.tlfx - tvair), 0.0f);
        c.conv = D.sur_gate;
      }
      bool restarted = false;
      if constexpr (kPool) {
        // the block's tiles iterate together (dryleaf.cuh): park this tile's
        // inputs and state in its slot, run the rounds, take the result back
        const DlPool<kSur> pool{sm, (int)blockDim.x};
        const int slot = threadIdx.x;
        __syncthreads();   // the previous call's slots and round counters are free
        if (veg_mask) {
          if (iter == 1) pool.put_step(slot, c);
          if (kSur && sur_try) pool.put_entry(slot, entry);
          pool.put_call(slot, c, st, (kSur && sur_try) ? dlp::SUR_TRY : 0);
        }
        if (threadIdx.x == 0) { int* cn = pool.cnt(); cn[0] = 0; cn[1] = 0; cn[2] = 0; }
        __syncthreads();
        pool.run(veg_mask, P.medlyn, dels, D.sur_strict);
        if (veg_mask) {
          pool.get_state(slot, st);
          const int bits = pool.kv(slot);
          if (kSur && (bits & dlp::SUR_ACC)) ++sur_accepted;
          if (kSur && (bits & dlp::SUR_RESTART)) { restarted = true; ++passes_total; }
        }
      } else if (veg_mask) {
        bool more = true, first_sur = sur_try;
        while (more) {
          more = dl_pass(c, st, froot, P.medlyn, dels);
          if (kSur && first_sur) {
            first_sur = false;
            if (st.abs_deltlf <= c.conv) {
              ++sur_accepted;
            } else if (D.sur_strict) {
              // strict: the prediction did not close, so the tile runs the
              // plain iteration from its usual start, exactly as without the
              // surrogate
              passes_total += st.k;
              const float keep_psycst[2] = {st.psycst[0], st.psycst[1]};
              const float keep_rny = st.rny, keep_ecy = st.ecy, keep_tlfy = st.tlfy;
              st = entry;
              st.psycst[0] = keep_psycst[0]; st.psycst[1] = keep_psycst[1];
              st.rny = keep_rny; st.ecy = keep_ecy; st.tlfy = keep_tlfy;
              c.conv = 0.1f;
              restarted = true;
              more = true;
            }
          }
        }
      }
      if (!veg_mask) {
        // no pass: the best-iterate store of the first (inactive) pass
        st.tlfy = st.tlfx; st.rny = 0.f; st.hcy = 0.f; st.ecy = 0.f; st.rdy_sum = 0.f; st.an_y_sum = 0.f;
        st.fe_mm_best = 0.f; st.fe_mm_last = 0.f; st.ecx = 0.f; st.abs_deltlf = 0.f;
      }
      passes_total += st.k;
      const float conv = restarted ? 0.1f : c.conv;
      tlfx = st.tlfx; dsx = st.dsx; tlfy = st.tlfy;
#pragma unroll
      for (int l = 0; l < 2; ++l) { csx[l] = st.csx[l]; gswx[l] = st.gswx[l]; gbhf[l] = st.gbhf[l]; }
      rny = st.rny; hcy = st.hcy; ecy = st.ecy;
      const float ecx = st.ecx, abs_deltlf = st.abs_deltlf;
      const float rdy_sum = st.rdy_sum, an_y_sum = st.an_y_sum, fe_mm_last = st.fe_mm_last, fe_mm_best = st.fe_mm_best;
      // status bits of this iteration, recorded with diagnostics on (they cost
      // the fast kernel registers in its hottest loop): pass limit reached
      // unconverged; the reference's 'oldevapfbl not right' condition
      uint8_t it_bits = (kDiag && veg_mask && abs_deltlf > conv) ? CG_TS_DRYLEAF_NOCONV : 0;
      // the layer amounts of the latest extracting pass (zero if none)
      if (fe_mm_last > 0.f) {
        transp_extract(fe_mm_last, froot, dk_avail, evapfbl);
      } else {
#pragma unroll
        for (int kk = 0; kk < CG_MS; ++kk) evapfbl[kk] = 0.f;
      }
      fevc = (1.0f - fwet) * ecy;
      if (ecy > 0.0f && fwet < 1.0f && fabsf(ecy - ecx) > 1.0e-6f) {
        // the best iterate's layer amounts replace them when they match its
        // transpiration (cbl_dryLeaf.F90:626-645)
        float oldevapfbl[CG_MS] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float so2 = (fe_mm_best > 0.f) ? transp_extract(fe_mm_best, froot, dk_avail, oldevapfbl) : 0.f;
        if (!(fabsf(fevc - so2 * rlam / dels) > 1.0e-4f)) {
#pragma unroll
          for (int kk = 0; kk < CG_MS; ++kk) evapfbl[kk] = oldevapfbl[kk];
        } else {
          if (kDiag) it_bits |= CG_TS_EVAPFBL;
        }
      }
      if (kDiag && it_bits && !ghost) D.tile_status[t] |= it_bits;
      frday = 12.0f * rdy_sum;
      fpn = fminf(-12.0f * an_y_sum, frday);
      // training row: features at entry, converged stomatal conductance,
      // net assimilation and leaf temperature change
      if (sampled) {
        const unsigned long long slot = atomicAdd(D.harvest_n, 1ull);
        if (slot < (unsigned long long)D.harvest_cap) {
          float4* r = reinterpret_cast<float4*>(D.harvest + slot * 16);
          r[0] = make_float4(feat[0], feat[1], feat[2], feat[3]);
          r[1] = make_float4(feat[4], feat[5], feat[6], feat[7]);
          r[2] = make_float4(feat[8], feat[9], feat[10], feat[11]);
          r[3] = make_float4(gswx[0] + gswx[1], an_y_sum, tlfy - tlf_entry, 0.f);
        }
      }
    }
    // ------------------------------------------------ wetLeaf (cbl_wetleaf.F90:9-111)
    fevw = 0.f; fhvw = 0.f;
    if (veg_mask) {
      float sum_gbh = gbhu[0] + gbhf[0] + gbhu[1] + gbhf[1];
      float ghwet = 2.0f * sum_gbh, gwwet = 1.075f * sum_gbh;
      float ghrwet = sum_rad_gradis + ghwet;
      float ccfevw = fminf(cansto * rlam / dels, 2.0f / (1440.0f / (dels / 60.0f)) * rlam);
      const float cpr = CAPP * RMAIR;
      float num = dsatdk * (sum_rad_rniso - cpr * (tvair - tk) * sum_rad_gradis) + cpr * dva * ghrwet;
      float den = dsatdk + psyc * ghrwet / gwwet;
      fevw = fminf(fwet * num / den, ccfevw);
      fevw_pot = num / den;
      fhvw = fwet * (sum_rad_rniso - cpr * (tlfy - tk) * sum_rad_gradis) - fevw;
    }
    fev = fevc + fevw;
    fhv = (1.0f - fwet) * hcy + fhvw;
    fnv = (1.0f - fwet) * rny + fevw + fhvw;
    // canopy temperature from the longwave balance (:425-450)
    if (veg_mask && hruff > z0soilsn) {
      float lwabv = CAPP * RMAIR * (tlfy - tk) * sum_rad_gradis;
      float arg = lwabv / (2.0f * (1.0f - transd) * SBOLTZ * EMLEAF) + pow4(tvrad);
      tv = (arg > 0.0f) ? sqrtf(sqrtf(arg)) : tvrad;
    } else {
      tv = tvrad;
    }
    fns = qssabs + transd * fld + (1.0f - transd) * EMLEAF * SBOLTZ * pow4(tv) - EMSOIL * SBOLTZ * tss4;
    // two passes of soil evaporation, separated by the within-canopy update
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      qstss = qsatfjh(tss - TFRZ, pmb);
      // Humidity_deficit_method (cbl_pot_evap_snow.F90:79-167)
      float dq = qstss - (pass == 0 ? qv : qvair);
      if (snowd > 1.0f || tgg[0] == TFRZ) dq = fmaxf(-0.1e-3f, dq);
      float rhlitt, relitt;
      litter_resist(rhlitt, relitt);
      if (P.potev_pm) {
        // Penman_Monteith (cbl_pot_evap_snow.F90:9-78): soil available
        // energy fns - ga (ga of the previous iteration or step) and the
        // canopy-air humidity deficit
        const float cc1 = dsatdk / (dsatdk + psyc), cc2 = psyc / (dsatdk + psyc);
        const float qsatfvar = qsatfjh(tvair - TFRZ, pmb);
        potev = cc1 * (fns - ga) + cc2 * rho * rlam * (qsatfvar - qvair) / (rtsoil + relitt);
      } else {
        potev = rho * rlam * dq / (rtsoil + relitt);
      }
      // Latent_heat_flux (cbl_latent_heat.F90:15-285)
      {
        if (potev < 0.f) wetfac = 1.0f;
        fess = wetfac * potev;
        float pwet = fmaxf(0.f, fminf(0.2f, pudsto / fmaxf(1.f, pudsmx)));
        fess = fess * (1.f - pwet);
        float frescale = zse[0] * DLIQ * rlam / dels;
        if (snowd < 0.1f && fess > 0.0f) {
          float flower = P.reduce_soilevp ? wb[0].hi - swilt : wb[0].hi - swilt / 2.0f;
          float fupper = fmaxf(0.f, flower * frescale - evapfbl[0] * rlam / dels);
          fess = fminf(fess, fupper);
          fupper = fmaxf(((wb[0].hi - wbice[0].hi / FROZEN_LIMIT) + (wb[0].lo - wbice[0].lo / FROZEN_LIMIT)) * frescale, 0.f);
          fess = fminf(fess, fupper);
        }
        cls = 1.f;
        if (snowd >= 0.1f) { cls = 1.1335f; fess = cls * potev; }
        if (snowd < 0.1f && potev < 0.f && tss < TFRZ) { cls = 1.1335f; fess = cls * potev; }
        if (snowd >= 0.1f && potev > 0.f) { cls = 1.1335f; fess = fminf((wetfac * potev) * cls, snowd / dels * rlam * cls); }
        fesp = fminf(pudsto / dels * rlam, fmaxf(pwet * potev, 0.f));
        fes = fess + fesp;
      }
      // the litter branch's first soil sensible heat uses the
      // reference-height air temperature (cable_canopy.F90:521-534)
      fhs = rho * CAPP * (tss - ((P.litter && pass == 0) ? tk : tvair)) / (rtsoil + rhlitt);
      if (pass == 0) {
        // within_canopy (cbl_within_canopy.F90:10-159)
        float rrbw = (gbhu[0] + gbhf[0] + gbhu[1] + gbhf[1]) / cmolar;
        float rrsw = (gswx[0] + gswx[1]) / cmolar;
        float fix_eqn = cls, fix_eqn2 = 1.f;
        if (P.litter) { fix_eqn = cls * rt0 / (rt0 + relitt); fix_eqn2 = rt0 / (rt0 + rhlitt); }
        if (potev > 0.f) fix_eqn = fix_eqn * wetfac;
        if (veg_mask && hruff > z0soilsn) {
          float r01 = rt0 * rt1, bs = rrbw * rrsw, g = (1.f + epsi) * rrsw + rrbw;
          float dmah = (rt0 + fix_eqn2 * rt1) * g + epsi * r01 * bs;
          float dmbh = (-rlam / CAPP) * r01 * bs;
          float dmch = g * r01 * (fhv + fhs) / (rho * CAPP);
          float dmae = (-epsi * CAPP / rlam) * r01 * bs;
          float dmbe = (rt0 + fix_eqn * rt1) * g + r01 * bs;
          float dmce = g * r01 * (fev + fes / cls) / (rho * rlam);
          float det = dmah * dmbe - dmae * dmbh + 1.0e-12f;
          tvair = tk + (dmbe * dmch - dmbh * dmce) / det;
          tvair = fminf(fmaxf(tvair, fminf(tss, tk) - 5.0f), fmaxf(tss, tk) + 5.0f);
          qvair = fmaxf(0.0f, qv + (dmah * dmce - dmae * dmch) / det);
          qvair = fminf(fmaxf(qvair, fminf(qstss, qv)), fmaxf(qstss, qv));
          qstvair = qsatfjh(tvair - TFRZ, pmb);
          dva = (qstvair - qvair) * RMAIR / RMH2O * pmb * 100.f;
        }
      }
    }
    ga = fns - fhs - fes;
    fe = fev + fes;
    fh = fhv + fhs;
    potev = (potev >= 0.f) ? fmaxf(0.00001f, potev) : fminf(-0.0002f, potev);
    fevw_pot = (fevw_pot >= 0.f) ? fmaxf(0.000001f, fevw_pot) : fminf(-0.002f, fevw_pot);
    epot = (fevw_pot + potev / cls) * dels / rlam;
    // update_zetar (cbl_zetar.F90:13-159)
    if (iter < NITER) {
      float z = -(VONK * GRAV * zref_tq * (fh + 0.07f * fe)) / (rho * CAPP * tk * us * us * us);
      zeta = fmaxf(ZETNEG, fminf(ZETPOS, z));
    }
  }

  if (ghost) return;
  // ---------------------------------------------------------------- post-loop (:684-1038)
  const float z4 = zeta;   // the last iteration's
  const float cduv = us * us / sqf(fmaxf(ua, UMIN));
  float cdtq = 0.f;
  if (kDiag)
    cdtq = cduv * (logf(zref_uv / z0m) - psim(z4 * zref_uv / zref_tq) + psim(z4 * z0m / zref_tq)) /
           (logf(zref_tq / (0.1f * z0m)) - psis(z4) + psis(z4 * 0.1f * z0m / zref_tq));
  float tscrn, qscrn;
  {
    float tstar = -fh / (rho * CAPP * us);
    float qstar = -fe / (rho * rlam * us * cls);
    float zscrn = fmaxf(z0m, 2.0f - disp);
    float ftemp = (logf(zref_tq / zscrn) - psis(z4) + psis(z4 * zscrn / zref_tq)) / VONK;
    tscrn = tk - TFRZ - tstar * ftemp;
    qscrn = qv - qstar * ftemp;
    const bool scr = veg_mask && hruff > 0.01f;
    float r_sc = 0.f, rsum = 1.f;
    if (scr) {
      float term1 = 0.f, term2 = 0.f, term5 = 0.f;
      float zscl = fmaxf(z0soilsn, 2.0f);
      const float e2 = expf(2.f * CSW * rghlai);
      if (disp > 0.0f) {
        term1 = expf(2.f * CSW * rghlai * (1.f - zscl / hruff));
        term2 = expf(2.f * CSW * rghlai * (1.f - disp / hruff));
        term5 = fmaxf(2.f / 3.f * hruff / disp, 1.f);
      }
      float term3 = A33 * A33 * CTL * 2.f * CSW * rghlai;
      if (zscl < disp) {
        r_sc = term5 * logf(zscl / z0soilsn) * (e2 - term2) / term3 + term5 * logf(disp / zscl) * (e2 - term1) / term3;
      } else if (zscl < hruff) {
        r_sc = rt0us + term5 * (term2 - term1) / term3;
      } else if (zscl < zruffs) {
        r_sc = rt0us + rt1usa + term5 * (zscl - hruff) / (A33 * A33 * CTL * hruff);
      } else {
        r_sc = rt0us + rt1usa + rt1usb +
               (logf((zscl - disp) / fmaxf(zruffs - disp, z0soilsn)) - psis((zscl - disp) * z4 / zref_tq) +
                psis((zruffs - disp) * z4 / zref_tq)) / VONK;
      }
      const float rsum0 = rt0us + rt1usa + rt1usb + rt1usc;
      rsum = fminf(1.f, r_sc / fmaxf(1.f, rsum0));
      float rsum_h = rsum;
      if (P.litter) {   // :808-812, :848-854
        float rhlitt, relitt;
        litter_resist(rhlitt, relitt);
        rsum_h = fminf(1.f, (r_sc + rhlitt * us) / fmaxf(1.f, rsum0 + rhlitt * us));
        rsum = fminf(1.f, (r_sc + relitt * us) / fmaxf(1.f, rsum0 + relitt * us));
      }
      tscrn = tss + (tk - tss) * rsum_h - TFRZ;
    }
    float rsts = qsatfjh(tscrn, pmb);
    float qtgnet = rsts * wetfac - qv;
    float qsurf = (qtgnet > 0.f) ? rsts * wetfac : 0.1f * rsts * wetfac + 0.9f * qv;
    if (scr) qscrn = qsurf + (qv - qsurf) * rsum;
  }
  // canopy water budget (:881-906)
  {
    float dewmm = -(fminf(0.0f, fevw) + fminf(0.0f, fevc)) * dels / rlam;
    cansto = cansto + dewmm;
    cansto = fmaxf(cansto - fmaxf(0.0f, fevw) * dels / rlam, 0.0f);
    float spill = fmaxf(0.0f, cansto - cansat);
    through = through + spill;
    cansto = cansto - spill;
  }
  const float precis0 = fmaxf(0.f, through);
  const float delwc = cansto - oldcansto;
  // soil-coupling derivative (:913-1027, default and litter branches, with
  // the l_rev_corr revisions :916-922, :993-1014)
  float dgdtg;
  {
    const float dfn_dtg = -4.f * EMSOIL * SBOLTZ * tss4 / tss;
    float rttsoil = rtsoil;
    if (P.rev_corr && veg_mask) rttsoil = rttsoil + rt1;
    float rhlitt, relitt;
    litter_resist(rhlitt, relitt);
    float dfh_dtg = rho * CAPP / (rttsoil + rhlitt);
    float dfe_ddq = wetfac * rho * rlam * cls / (rttsoil + relitt);
    if (P.rev_corr && potev < 0.f) dfe_ddq = rho * rlam * cls / (rttsoil + relitt);
    float tc = tss - TFRZ;
    float ddq_dtg = (RMH2O / RMAIR) / pmb * TETENA * TETENB * TETENC / sqf(TETENC + tc) * expf(TETENB * tc / (TETENC + tc));
    dgdtg = dfn_dtg - dfh_dtg - dfe_ddq * ddq_dtg;
    if (mode == 2) {
      D.work_b[CG_NB * ld + t] = dfh_dtg;
      D.work_b[(CG_NB + 1) * ld + t] = dfe_ddq * ddq_dtg;   // ssnow%dfe_dtg (:1026)
      D.work_b[(CG_NB + 2) * ld + t] = dfn_dtg;
    }
  }
  const float drybal = (ecy + hcy) - sum_rad_rniso + CAPP * RMAIR * (tlfy - tk) * sum_rad_gradis;
  const float wetbal = fevw + fhvw - sum_rad_rniso * fwet + CAPP * RMAIR * (tlfy - tk) * sum_rad_gradis * fwet;
  const float swnet = swcan + qssabs;
  const float lwnet = fld - SBOLTZ * EMLEAF * pow4(tv) * (1.f - transd) - flws * transd;
  const float owetfac_out = wetfac;   // cbm:192
  const bool cls_snow = (cls == 1.1335f);

  (void)cls_snow;
  // energy balance (cable_checks.F90:565-618); fev = fevc + fevw is the same
  // sum before and after remove_trans moves negative fevc into fevw
  const float ebal = swnet + fld - SBOLTZ * EMLEAF * pow4(tv) * (1.f - transd) - flws * transd - fev - fes - fh - ga;
  if (kSur && D.sur_stats) {
    // warp totals, one atomic per warp
    const unsigned int a = __reduce_add_sync(__activemask(), sur_tried);
    const unsigned int b = __reduce_add_sync(__activemask(), sur_accepted);
    if ((threadIdx.x & 31) == (__ffs(__activemask()) - 1)) {
      if (a) atomicAdd(&D.sur_stats[0], (unsigned long long)a);
      if (b) atomicAdd(&D.sur_stats[1], (unsigned long long)b);
    }
  }
  // the coupled calls run no balance checks; cbm_expl restores the canopy
  // water and wetness factor (cbl_cbm_mod.F90:150-152), so the step's
  // state is what the implicit call leaves
  if (mode == 0) D.ebal_tot[t] = D.ebal_tot[t] + f2d(ebal);
  if (mode != 1) {
    D.cansto[t] = cansto;
    D.owetfac[t] = owetfac_out;
  }
  D.rtsoil[t] = rtsoil;
  if (mode != 1) {
    const float rec[CG_NB] = {ga, dgdtg, fes, fess, fesp, fevc, fevw, cls, precis0, evapfbl[0], evapfbl[1], evapfbl[2],
                              evapfbl[3], evapfbl[4], evapfbl[5], delwc, fpn, frday, tv};
#pragma unroll
    for (int i = 0; i < CG_NB; ++i) D.work_b[i * ld + t] = rec[i];
  }
  const float rnet = fns + fnv;
  const float fgpp = -fpn + frday;
  const float outv[7] = {fe, fh, fgpp, frday, tv, rnet, ga};
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 7; ++i) { D.out[i * ld + t] = outv[i]; finite = finite && isfinite(outv[i]); }
  if (D.out_caller) {
    const size_t o = D.out_caller_order ? (size_t)D.tile_id[t] : (size_t)t;
#pragma unroll
    for (int i = 0; i < 7; ++i) D.out_caller[(size_t)i * D.mp + o] = outv[i];
  }
  {
    // output ranges of the reference's output checks (cable_checks.F90:71-123):
    // Qle, Qh, Qg, Rnet, VegT
    uint8_t bits = finite ? 0 : CG_TS_NONFINITE;
    if (!finite) atomicOr(D.status, 1u);
    if (out_of(fe, -2500.f, 2500.f) || out_of(fh, -2000.f, 2000.f) || out_of(ga, -4000.f, 4000.f) ||
        out_of(rnet, -500.f, 1250.f) || out_of(tv, 213.f, 353.f))
      bits |= CG_TS_OUTPUT_RANGE;
    if (bits) D.tile_status[t] |= bits;
  }
  if (kDiag) {
    const int idx[39] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 18, 20, 21, 22, 32, 33, 34, 35,
                         36, 43, 44, 45, 50, 51, 52, 53, 55, 56, 57, 58, 59, 60};
    const float val[39] = {fe, fh, fev, fhv, fhs, fns, fnv, ga, tv, tscrn, qscrn, rnet, us, cduv, cdtq, epot, fes,
                           dgdtg, fpn, frday, fgpp, precis0, through, fwet, owetfac_out, potev, drybal, wetbal, ebal,
                           tvair, qvair, swnet, lwnet, gswx[0], gswx[1], fwsoil, (float)passes_total, delwc, cls};
#pragma unroll
    for (int i = 0; i < 39; ++i) D.diag[idx[i] * ld + t] = val[i];
  }
}

// cbm_expl's radiative temperature (cbl_cbm_mod.F90:172-179) after the
// canopy kernel of an explicit call: emissivities 1, the surface temperature
// of the start of the step, and no correction term (canopy%fns_cor is zeroed
// by define_canopy, cable_canopy.F90:233).
__device__ __forceinline__ void explicit_trad(const CgDev& D, int t) {
  const int ld = D.ld;
  const float tv = D.out[4 * ld + t];
  const float transd = D.work_a[27 * ld + t], tss = D.work_a[45 * ld + t];
  const float trad = sqrtf(sqrtf((1.f - transd) * pow4(tv) + transd * pow4(tss)));
  D.out[7 * ld + t] = trad;
  if (D.out_caller) D.out_caller[(size_t)7 * D.mp + (D.out_caller_order ? (size_t)D.tile_id[t] : (size_t)t)] = trad;
  if (!isfinite(trad)) { atomicOr(D.status, 1u); D.tile_status[t] |= CG_TS_NONFINITE; }
}

template <bool kDiag, bool kCoupled = false>
__device__ __forceinline__ void phase_c1(const CgDev& D, const CgTables* __restrict__ T, const StepParams& P, int t) {
  // the coupled-call code exists only in the kCoupled instantiation
  const int mode = kCoupled ? P.mode : 0;
  const int ld = D.ld;
  const float dels = P.dels;
  const int iveg = D.iveg[t], isoilm = D.isoilm[t];
  const int v = iveg - 1, so = isoilm - 1;
  const CgPftTable& V = T->pft;
  const CgSoilTable& S = T->soil;
  float froot[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) froot[k] = ldf(V.froot[k], v);
  const float ssat = ldf(S.ssat, so), sfc = ldf(S.sfc, so), swilt = ldf(S.swilt, so), css = ldf(S.css, so);
  const float rhosoil = ldf(S.rhosoil, so);
  // soil layer thicknesses (m), cable_parameters.F90:1241: model constants,
  // the same values as the table's, as immediates rather than registers
  constexpr float zse[CG_MS] = {0.022f, 0.058f, 0.154f, 0.409f, 1.085f, 2.872f};
  // state
  df32 wb[CG_MS], wbice[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wb[k] = df_load(D.wb, CG_MS, ld, k, t); wbice[k] = df_load(D.wbice, CG_MS, ld, k, t); }
  // FP32 shadows of soil water and ice for thresholds and fluxes; every
  // change to the state is mirrored into them
  float wbf[CG_MS], wbicef[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wbf[k] = wb[k].hi; wbicef[k] = wbice[k].hi; }
  float tgg[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) tgg[k] = D.tgg[k * ld + t];
  float tggsn[3], ssdn[3], smass[3], sdepth[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tggsn[k] = D.tggsn[k * ld + t]; ssdn[k] = D.ssdn[k * ld + t];
    smass[k] = D.smass[k * ld + t]; sdepth[k] = D.sdepth[k * ld + t];
  }
  const uint8_t flags = D.flags[t];
  int isflag = flags & 1;
  bool first_call = (flags & 2) != 0;
  double gammzz1 = D.gammzz1[t];
  float snowd = D.snowd[t], ssdnn = D.ssdnn[t];
  // phase A and B records
  const float precip_sn = D.work_a[7 * ld + t];
  auto Bv = [&](int i) { return D.work_b[i * ld + t]; };
  const float ga = Bv(0), dgdtg = Bv(1), fes = Bv(2), fess = Bv(3), fesp = Bv(4);
  float fevc = Bv(5), fevw = Bv(6);
  const float cls = Bv(7), precis0 = Bv(8);
  float evapfbl[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) evapfbl[k] = Bv(9 + k);
  const float delwc = Bv(15), fpn = Bv(16), frday = Bv(17), tv = Bv(18);
  const bool cls_snow = (cls == 1.1335f);
  // ================================================================ soil_snow
  // cbl_soilsnow_main.F90:28-207
  float precis = precis0;
  float hcll = fmaxf(0.01f, css * rhosoil);
  const float t_snwlr = 0.05f;
  float dtmlt0 = 0.f;
  const float osnowd = snowd;
  if (first_call) {
    const double wb0 = df_to_double(wb[0]), wbice0 = df_to_double(wbice[0]);
    gammzz1 = fmax((double)((1.0f - ssat) * css * rhosoil) + (wb0 - wbice0) * (double)(CSWAT * DLIQ) +
                       wbice0 * (double)(CSICE * DICE), (double)(css * rhosoil)) * (double)zse[0] +
              (double)((float)(1 - isflag) * CGSNOW * snowd);
    first_call = false;
  }
  float g1f = d2f(gammzz1);   // layer-1 heat capacity, FP32 working copy
  float wblf[CG_MS], wbfice[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    wblf[k] = fmaxf(0.01f, wbf[k] - wbicef[k]) / ssat;
    wbfice[k] = wbicef[k] / ssat;
  }
  float sconds[3] = {0.f, 0.f, 0.f};
  // snowcheck (cbl_snowCheck.F90:9-100)
  if (snowd <= 0.0f) {
    isflag = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) { ssdn[k] = 120.0f; tggsn[k] = TFRZ; }
    ssdnn = 120.0f;
    sdepth[0] = snowd / ssdn[0]; sdepth[1] = 0.f; sdepth[2] = 0.f;
    smass[0] = snowd; smass[1] = 0.f; smass[2] = 0.f;
  } else if (snowd < SNMIN * ssdnn) {
    if (isflag == 1) { ssdn[0] = ssdnn; tgg[0] = tggsn[0]; }
    isflag = 0;
    ssdnn = fminf(400.0f, fmaxf(120.0f, ssdn[0]));
    float tm = fminf(TFRZ, tgg[0]);
    tggsn[0] = tm; tggsn[1] = tm; tggsn[2] = tm;
    sdepth[0] = snowd / ssdn[0]; sdepth[1] = 0.f; sdepth[2] = 0.f;
    smass[0] = snowd; smass[1] = 0.f; smass[2] = 0.f;
    ssdn[0] = ssdnn; ssdn[1] = ssdnn; ssdn[2] = ssdnn;
  } else {
    if (isflag == 0) {
      float tm = fminf(TFRZ, tgg[0]);
      tggsn[0] = tm; tggsn[1] = tm; tggsn[2] = tm;
      ssdn[1] = ssdn[0]; ssdn[2] = ssdn[0];
      sdepth[0] = t_snwlr;
      smass[0] = t_snwlr * ssdn[0];
      smass[1] = (snowd - smass[0]) * 0.4f;
      smass[2] = (snowd - smass[0]) * 0.6f;
      sdepth[1] = smass[1] / ssdn[1];
      sdepth[2] = smass[2] / ssdn[2];
      ssdnn = (ssdn[0] * smass[0] + ssdn[1] * smass[1] + ssdn[2] * smass[2]) / snowd;
    }
    isflag = 1;
  }
  // snowdensity (cbl_snowDensity.F90:9-102)
  if (snowd > 0.1f && isflag == 0) {
    float tmin1 = fminf(TFRZ, tgg[0]);
    float s0 = ssdn[0];
    s0 = fminf(MAX_SSDN, fmaxf(120.0f, s0 + dels * s0 * 3.1e-6f * expf(-0.03f * (273.15f - tmin1) -
                                                                           ((s0 >= 150.0f) ? 0.046f : 0.0f) * (s0 - 150.0f))));
    s0 = fminf(MAX_SSDN, s0 + dels * 9.806f * s0 * 0.75f * snowd / (3.0e7f * expf(0.021f * s0 + 0.081f * (273.15f - tmin1))));
    if (isoilm != 9) s0 = fminf(450.0f, s0);
    sconds[0] = fmaxf(0.2f, fminf(2.876e-6f * s0 * s0 + 0.074f, MAX_SCONDS));
    sconds[1] = sconds[0]; sconds[2] = sconds[0];
    ssdnn = s0;
    ssdn[0] = s0; ssdn[1] = s0; ssdn[2] = s0;
  }
  if (isflag == 1) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
      ssdn[k] = ssdn[k] + dels * ssdn[k] * 3.1e-6f *
                              expf(-0.03f * (273.15f - fminf(TFRZ, tggsn[k])) - ((ssdn[k] >= 150.0f) ? 0.046f : 0.0f) * (ssdn[k] - 150.0f));
    // overburden compaction; layers 2 and 3 see the updated top-layer density
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float ov = t_snwlr * ssdn[0];
      if (k >= 1) ov += (k == 1) ? 0.5f * smass[1] : smass[1] + 0.5f * smass[2];
      ssdn[k] = ssdn[k] + dels * 9.806f * ssdn[k] * ov / (3.0e7f * expf(0.021f * ssdn[k] + 0.081f * (273.15f - fminf(TFRZ, tggsn[k]))));
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) sdepth[k] = smass[k] / ssdn[k];
    ssdnn = (ssdn[0] * smass[0] + ssdn[1] * smass[1] + ssdn[2] * smass[2]) / snowd;
#pragma unroll
    for (int k = 0; k < 3; ++k) sconds[k] = fmaxf(0.2f, fminf(2.876e-6f * ssdn[k] * ssdn[k] + 0.074f, MAX_SCONDS));
  }
  // snow_accum (cbl_snowAccum.F90:10-188)
  float segg;
  {
    if (precis > 0.0f && isflag == 0) {
      snowd = fmaxf(snowd + precip_sn, 0.0f);
      precis = precis - precip_sn;
      ssdn[0] = fmaxf(120.0f, ssdn[0] * osnowd / fmaxf(0.01f, snowd) + 120.0f * precip_sn / fmaxf(0.01f, snowd));
      ssdnn = ssdn[0];
      if (precis > 0.0f && tgg[0] < TFRZ) {
        snowd = fmaxf(snowd + precis, 0.0f);
        float dT = precis * HLF / (g1f + CSWAT * precis);
        tgg[0] = tgg[0] + dT;
        dtmlt0 = dtmlt0 + dT;
        ssdn[0] = fminf(MAX_SSDN, fmaxf(120.0f, ssdn[0] * osnowd / fmaxf(0.01f, snowd) + DLIQ * precis / fmaxf(0.01f, snowd)));
        if (isoilm != 9) ssdn[0] = fminf(450.0f, ssdn[0]);
        precis = 0.0f;
        ssdnn = ssdn[0];
      }
    }
    if (precis > 0.0f && isflag > 0) {
      snowd = fmaxf(snowd + precip_sn, 0.0f);
      precis = precis - precip_sn;
      float osm = smass[0];
      smass[0] = smass[0] + precip_sn;
      ssdn[0] = fmaxf(120.0f, ssdn[0] * osm / smass[0] + 120.0f * precip_sn / smass[0]);
      sdepth[0] = fmaxf(0.02f, smass[0] / ssdn[0]);
      if (precis > 0.0f) {
        snowd = fmaxf(snowd + precis, 0.0f);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          float sgamm = ssdn[k] * CGSNOW * sdepth[k];
          osm = smass[k];
          float dT = precis * HLF * osm / (sgamm * osnowd);
          tggsn[k] = tggsn[k] + dT;
          if (k == 0) dtmlt0 = dtmlt0 + dT;
          smass[k] = smass[k] + precis * osm / osnowd;
          ssdn[k] = fmaxf(120.0f, fminf(ssdn[k] * osm / smass[k] + DLIQ * (1.0f - osm / smass[k]), MAX_SSDN));
          if (isoilm != 9) ssdn[k] = fminf(450.0f, ssdn[k]);
          sdepth[k] = smass[k] / ssdn[k];
        }
        precis = 0.0f;
      }
    }
    segg = fess / HL;
    if (cls_snow) {
      float evapsn = dels * fess / (HL + HLF);
      float xxx = evapsn;
      if (isflag == 0 && fess > 0.0f) evapsn = fminf(snowd, xxx);
      if (isflag > 0 && fess > 0.0f) evapsn = fminf(0.9f * smass[0], xxx);
      snowd = snowd - evapsn;
      if (isflag > 0) {
        smass[0] = smass[0] - evapsn;
        sdepth[0] = fmaxf(0.02f, smass[0] / ssdn[0]);
      }
      segg = (HL + HLF) * (xxx - evapsn) / HL / dels;
    }
  }
  // snow_melting (cbl_snowMelt.F90:9-120), first and second call share code
  auto snow_melting = [&]() -> float {
    float snowmlt = 0.f;
    if (snowd > 0.0f && isflag == 0 && tgg[0] >= TFRZ) {
      float snowflx = (tgg[0] - TFRZ) * g1f;
      snowmlt = fminf(snowflx / HLF, snowd);
      dtmlt0 = dtmlt0 + snowmlt * HLF / g1f;
      snowd = snowd - snowmlt;
      tgg[0] = tgg[0] - snowmlt * HLF / g1f;
    }
    if (snowd > 0.0f && isflag > 0) {
      float sm_prev = 0.f;   // smelt1(:,k-1)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float sgamm = ssdn[k] * CGSNOW * sdepth[k];
        float snowflx = sm_prev * HLF / dels;
        tggsn[k] = tggsn[k] + (snowflx * dels + sm_prev * CSWAT * (TFRZ - tggsn[k])) / (sgamm + CSWAT * sm_prev);
        float osm = smass[k];
        smass[k] = smass[k] + sm_prev;
        ssdn[k] = fmaxf(120.0f, fminf(ssdn[k] * osm / smass[k] + DLIQ * (1.0f - osm / smass[k]), MAX_SSDN));
        if (isoilm != 9) ssdn[k] = fminf(450.0f, ssdn[k]);
        sdepth[k] = smass[k] / ssdn[k];
        sgamm = smass[k] * CGSNOW;
        float sm = 0.f;
        if (tggsn[k] > TFRZ) {
          snowflx = (tggsn[k] - TFRZ) * sgamm;
          sm = fminf(snowflx / HLF, 0.6f * smass[k]);
          if (k == 0) dtmlt0 = dtmlt0 + sm * HLF / sgamm;
          smass[k] = smass[k] - sm;
          tggsn[k] = tggsn[k] - sm * HLF / sgamm;
          sdepth[k] = smass[k] / ssdn[k];
        }
        sm_prev = sm;
      }
      // melt of layers 1 and 2 refreezes into the layer below; only the
      // bottom layer's melt leaves the pack
      snowmlt = sm_prev;
      snowd = snowd - snowmlt;
    }
    return snowmlt;
  };
  float smelt = snow_melting();
  // snowl_adjust (cbl_snowl_adjust.F90:9-156)
  if (isflag > 0) {
    if (sdepth[0] > t_snwlr) {
      float excd = sdepth[0] - t_snwlr;
      float excm = excd * ssdn[0];
      sdepth[0] = sdepth[0] - excd;
      smass[0] = smass[0] - excm;
      float osm = smass[1];
      smass[1] = fmaxf(0.01f, smass[1] + excm);
      ssdn[1] = fmaxf(120.0f, fminf(MAX_SSDN, ssdn[1] * osm / smass[1] + ssdn[0] * excm / smass[1]));
      sdepth[1] = smass[1] / ssdn[1];
      tggsn[1] = tggsn[1] * osm / smass[1] + tggsn[0] * excm / smass[1];
      smass[2] = fmaxf(0.01f, snowd - smass[0] - smass[1]);
    } else {
      float excd = t_snwlr - sdepth[0];
      float excm = excd * ssdn[1];
      float osm = smass[0];
      smass[0] = smass[0] + excm;
      sdepth[0] = t_snwlr;
      ssdn[0] = fmaxf(120.0f, fminf(MAX_SSDN, ssdn[0] * osm / smass[0] + ssdn[1] * excm / smass[0]));
      tggsn[0] = tggsn[0] * osm / smass[0] + tggsn[1] * excm / smass[0];
      smass[1] = fmaxf(0.01f, smass[1] - excm);
      sdepth[1] = smass[1] / ssdn[1];
      smass[2] = fmaxf(0.01f, snowd - smass[0] - smass[1]);
    }
    float frac = smass[1] / fmaxf(0.02f, smass[2]);
    float xfrac = 2.0f / 3.0f / frac;
    if (xfrac > 1.0f) {
      float excm = (xfrac - 1.0f) * smass[1];
      float osm = smass[1];
      smass[1] = fmaxf(0.01f, smass[1] + excm);
      tggsn[1] = tggsn[1] * osm / smass[1] + tggsn[2] * excm / smass[1];
      ssdn[1] = fmaxf(120.0f, fminf(MAX_SSDN, ssdn[1] * osm / smass[1] + ssdn[2] * excm / smass[1]));
      smass[2] = fmaxf(0.01f, snowd - smass[0] - smass[1]);
      sdepth[2] = fmaxf(0.02f, smass[2] / ssdn[2]);
    } else {
      float excm = (1.f - xfrac) * smass[1];
      smass[1] = fmaxf(0.01f, smass[1] - excm);
      sdepth[1] = fmaxf(0.02f, smass[1] / ssdn[1]);
      float osm = smass[2];
      smass[2] = fmaxf(0.01f, snowd - smass[0] - smass[1]);
      tggsn[2] = tggsn[2] * osm / smass[2] + tggsn[1] * excm / smass[2];
      ssdn[2] = fmaxf(120.0f, fminf(MAX_SSDN, ssdn[2] * osm / smass[2] + ssdn[1] * excm / smass[2]));
      sdepth[2] = smass[2] / ssdn[2];
    }
    isflag = 1;
    ssdnn = (ssdn[0] * sdepth[0] + ssdn[1] * sdepth[1] + ssdn[2] * sdepth[2]) / (sdepth[0] + sdepth[1] + sdepth[2]);
  }
  // store: snow pack, layer-1 temperature, heat capacity and the C1 record
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    D.tggsn[k * ld + t] = tggsn[k]; D.ssdn[k * ld + t] = ssdn[k]; D.smass[k * ld + t] = smass[k];
    D.sdepth[k * ld + t] = sdepth[k];
  }
  D.tgg[t] = tgg[0];
  D.flags[t] = (uint8_t)(isflag | (first_call ? 2 : 0));
  D.gammzz1[t] = f2d(g1f);
  D.snowd[t] = snowd; D.ssdnn[t] = ssdnn;
  D.work_c[0 * ld + t] = osnowd;
  D.work_c[1 * ld + t] = precis;
  D.work_c[2 * ld + t] = segg;
  D.work_c[3 * ld + t] = smelt;
  if (mode == 2) D.work_c[CG_NC * ld + t] = dtmlt0;
  (void)sconds; (void)hcll; (void)wblf; (void)wbfice;
}

// snow pack state that snow_melting updates
struct CgSnowPack {
  float tggsn[3], ssdn[3], smass[3], sdepth[3];
  float snowd, tgg0, dtmlt0;
};

// snow_melting (cbl_snowMelt.F90:9-120): melt of the snow lumped with soil
// layer 1 (isflag 0) or of the 3-layer pack, returning the melt that leaves
// the pack.  g1f: layer-1 heat capacity (J/m2/K).
static __device__ __noinline__ float cg_snow_melting(CgSnowPack& p, int isflag, int isoilm, float g1f, float dels) {
  float snowmlt = 0.f;
  if (p.snowd > 0.0f && isflag == 0 && p.tgg0 >= TFRZ) {
    float snowflx = (p.tgg0 - TFRZ) * g1f;
    snowmlt = fminf(snowflx / HLF, p.snowd);
    p.dtmlt0 = p.dtmlt0 + snowmlt * HLF / g1f;
    p.snowd = p.snowd - snowmlt;
    p.tgg0 = p.tgg0 - snowmlt * HLF / g1f;
  }
  if (p.snowd > 0.0f && isflag > 0) {
    float sm_prev = 0.f;   // smelt1(:,k-1)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float sgamm = p.ssdn[k] * CGSNOW * p.sdepth[k];
      float snowflx = sm_prev * HLF / dels;
      p.tggsn[k] = p.tggsn[k] + (snowflx * dels + sm_prev * CSWAT * (TFRZ - p.tggsn[k])) / (sgamm + CSWAT * sm_prev);
      float osm = p.smass[k];
      p.smass[k] = p.smass[k] + sm_prev;
      p.ssdn[k] = fmaxf(120.0f, fminf(p.ssdn[k] * osm / p.smass[k] + DLIQ * (1.0f - osm / p.smass[k]), MAX_SSDN));
      if (isoilm != 9) p.ssdn[k] = fminf(450.0f, p.ssdn[k]);
      p.sdepth[k] = p.smass[k] / p.ssdn[k];
      sgamm = p.smass[k] * CGSNOW;
      float sm = 0.f;
      if (p.tggsn[k] > TFRZ) {
        snowflx = (p.tggsn[k] - TFRZ) * sgamm;
        sm = fminf(snowflx / HLF, 0.6f * p.smass[k]);
        if (k == 0) p.dtmlt0 = p.dtmlt0 + sm * HLF / sgamm;
        p.smass[k] = p.smass[k] - sm;
        p.tggsn[k] = p.tggsn[k] - sm * HLF / sgamm;
        p.sdepth[k] = p.smass[k] / p.ssdn[k];
      }
      sm_prev = sm;
    }
    // melt of layers 1 and 2 refreezes into the layer below; only the
    // bottom layer's melt leaves the pack
    snowmlt = sm_prev;
    p.snowd = p.snowd - snowmlt;
  }
  return snowmlt;
}

// kS64: the heat solve in FP64 on the reference's direct form (trimb64, as
// cbl_stempv.F90:201-214 calls cbl_trimb.F90); otherwise in FP32 on the
// step's change (trid_correction).
template <bool kDiag, bool kCoupled = false, bool kS64 = true>
__device__ __forceinline__ void phase_c2(const CgDev& D, const CgTables* __restrict__ T, const StepParams& P, int t) {
  // the coupled-call code exists only in the kCoupled instantiation
  const int mode = kCoupled ? P.mode : 0;
  const int ld = D.ld;
  const float dels = P.dels;
  const int iveg = D.iveg[t], isoilm = D.isoilm[t];
  const int v = iveg - 1, so = isoilm - 1;
  const CgPftTable& V = T->pft;
  const CgSoilTable& S = T->soil;
  float froot[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) froot[k] = ldf(V.froot[k], v);
  const float ssat = ldf(S.ssat, so), sfc = ldf(S.sfc, so), swilt = ldf(S.swilt, so), css = ldf(S.css, so);
  const float rhosoil = ldf(S.rhosoil, so);
  // soil layer thicknesses (m), cable_parameters.F90:1241: model constants,
  // the same values as the table's, as immediates rather than registers
  constexpr float zse[CG_MS] = {0.022f, 0.058f, 0.154f, 0.409f, 1.085f, 2.872f};
  // state
  df32 wb[CG_MS], wbice[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wb[k] = df_load(D.wb, CG_MS, ld, k, t); wbice[k] = df_load(D.wbice, CG_MS, ld, k, t); }
  // FP32 shadows of soil water and ice for thresholds and fluxes; every
  // change to the state is mirrored into them
  float wbf[CG_MS], wbicef[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wbf[k] = wb[k].hi; wbicef[k] = wbice[k].hi; }
  float tgg[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) tgg[k] = D.tgg[k * ld + t];
  float tggsn[3], ssdn[3], smass[3], sdepth[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tggsn[k] = D.tggsn[k * ld + t]; ssdn[k] = D.ssdn[k * ld + t];
    smass[k] = D.smass[k * ld + t]; sdepth[k] = D.sdepth[k * ld + t];
  }
  const uint8_t flags = D.flags[t];
  int isflag = flags & 1;
  bool first_call = (flags & 2) != 0;
  double gammzz1 = D.gammzz1[t];
  float snowd = D.snowd[t], ssdnn = D.ssdnn[t];
  // phase A and B records
  auto Bv = [&](int i) { return D.work_b[i * ld + t]; };
  const float ga = Bv(0), dgdtg = Bv(1), fes = Bv(2), fess = Bv(3), fesp = Bv(4);
  float fevc = Bv(5), fevw = Bv(6);
  const float cls = Bv(7), precis0 = Bv(8);
  float evapfbl[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) evapfbl[k] = Bv(9 + k);
  const float delwc = Bv(15), fpn = Bv(16), frday = Bv(17), tv = Bv(18);
  float tss;
  // soil_snow, heat part (cbl_soilsnow_main.F90:125-136)
  float hcll = fmaxf(0.01f, css * rhosoil);
  // dtmlt(:,1) so far this step (the snow-pack kernel's part); only the
  // implicit coupled call uses it
  float dtmlt0 = mode == 2 ? D.work_c[CG_NC * ld + t] : 0.f;
  float g1f = d2f(gammzz1);
  float smelt = D.work_c[3 * ld + t];
  float wblf[CG_MS], wbfice[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    wblf[k] = fmaxf(0.01f, wbf[k] - wbicef[k]) / ssat;
    wbfice[k] = wbicef[k] / ssat;
  }
  float sconds[3] = {0.f, 0.f, 0.f};
  // snow_melting (cbl_snowMelt.F90:9-120): called twice, kept out of line
  // (one copy of its code keeps the kernel's instruction working set small)
  CgSnowPack sp;
#pragma unroll
  for (int k = 0; k < 3; ++k) { sp.tggsn[k] = tggsn[k]; sp.ssdn[k] = ssdn[k]; sp.smass[k] = smass[k]; sp.sdepth[k] = sdepth[k]; }
  auto snow_melting = [&]() -> float {
    sp.snowd = snowd; sp.tgg0 = tgg[0]; sp.dtmlt0 = dtmlt0;
#pragma unroll
    for (int k = 0; k < 3; ++k) { sp.tggsn[k] = tggsn[k]; sp.ssdn[k] = ssdn[k]; sp.smass[k] = smass[k]; sp.sdepth[k] = sdepth[k]; }
    const float m = cg_snow_melting(sp, isflag, isoilm, g1f, dels);
    snowd = sp.snowd; tgg[0] = sp.tgg0; dtmlt0 = sp.dtmlt0;
#pragma unroll
    for (int k = 0; k < 3; ++k) { tggsn[k] = sp.tggsn[k]; ssdn[k] = sp.ssdn[k]; smass[k] = sp.smass[k]; sdepth[k] = sp.sdepth[k]; }
    return m;
  };
  // stempv (cbl_stempv.F90:13-221) with old_soil_conductivity
  // (cbl_Oldconductivity.F90:7-59), or total_soil_conductivity
  // (cbl_conductivity.F90:10-85) under soil_thermal_fix (cbl_stempv.F90:57-61)
  float ghflux, sghflux = 0.f;
  float gf[CG_MS];   // soil layer heat capacities (ssnow%gammzz), J/m2/K
  {
    float ccnsw[CG_MS];
    if (P.thermal_fix) {
      const float ktmp = ldf(S.ktmp, so), cnsdv = ldf(S.cnsdv, so);
      const bool snowy = isflag != 0 || snowd >= 0.1f;
#pragma unroll
      for (int k = 0; k < CG_MS; ++k) {
        if (isoilm == 9) {
          ccnsw[k] = SNOW_CCNSW;
        } else {
          const float w = wbf[k], wi = wbicef[k];
          const float liq = (w >= 1.0e-15f) ? fminf(1.f, fmaxf(0.f, (w - wi) / w)) : 0.f;
          // Ksat = Ktmp 2.2^(ssat (1 - liq)) 0.57^liq
          const float ksat = ktmp * exp2f(ssat * (1.f - liq) * 1.13750352f + liq * -0.810966176f);
          const float sr = fminf(0.9999f, fmaxf(0.f, w - 0.01f) / (ssat - 0.01f));
          float ke = (sr >= 0.05f) ? 0.7f * log10f(sr) + 1.f : 0.f;
          if (wi > 0.f || tgg[k] < TFRZ || snowy) ke = sr;
          ccnsw[k] = fminf(ksat, fmaxf(cnsdv, ke * ksat + (1.f - ke) * cnsdv));
        }
      }
    } else {
    const float cnsd = ldf(S.cnsd, so);
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) {
      if (isoilm == 9) {
        ccnsw[k] = SNOW_CCNSW;
      } else {
        float ew = wblf[k] * ssat;
        float exp_arg = ew * 4.0943446f /* log 60 */ + wbfice[k] * ssat * 5.5214609f /* log 250 */;
        float f2 = fmaxf(1.0f, sqrtf(fminf(2.0f, 0.5f * ssat / fminf(ew, 0.5f * ssat))));
        ccnsw[k] = (exp_arg > 30.f) ? 1.5f * f2 : fminf(cnsd * __expf(exp_arg), 1.5f) * f2;
      }
    }
    }
    float coeff[CG_MS + 1];   // coeff(1..ms+1) of the reference, coeff[ms] = 0
    float coefb;
    float snowz = 0.f;
    if (isflag == 0) {
      snowz = fmaxf(0.f, snowd / ssdnn);
      ccnsw[0] = (ccnsw[0] - 0.2f) * (zse[0] / (zse[0] + snowz)) + 0.2f;
      coeff[0] = 0.f;
    }
#pragma unroll
    for (int k = 2; k <= CG_MS; ++k) coeff[k - 1] = 2.0f / (zse[k - 2] / ccnsw[k - 2] + zse[k - 1] / ccnsw[k - 1]);
    coeff[CG_MS] = 0.f;
    if (isflag == 0) {
      coeff[1] = 2.0f / ((zse[0] + snowz) / ccnsw[0] + zse[1] / ccnsw[1]);
      coefb = coeff[1];
    }
    float csn[3];
    if (isflag != 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) sconds[k] = fmaxf(0.2f, fminf(2.876e-6f * ssdn[k] * ssdn[k] + 0.074f, MAX_SCONDS));
      csn[0] = 2.0f / (sdepth[0] / sconds[0] + sdepth[1] / sconds[1]);
      csn[1] = 2.0f / (sdepth[1] / sconds[1] + sdepth[2] / sconds[2]);
      coeff[0] = 2.0f / (sdepth[2] / sconds[2] + zse[0] / ccnsw[0]);
      coefb = coeff[0];
    }
    // heat capacity of the soil layers
#pragma unroll
    for (int k = 0; k < CG_MS; ++k)
      gf[k] = fmaxf(hcll, (1.0f - ssat) * css * rhosoil + ssat * (wblf[k] * CSWAT * DLIQ + wbfice[k] * CSICE * DICE)) * zse[k];
    if (isflag == 0) gf[0] = gf[0] + CGSNOW * snowd;
    // Implicit heat conduction (cbl_stempv.F90:98-217).  Row k of the
    // reference's system is a_k T_{k-1} + b_k T_k + c_k T_{k+1} = rhs_k with
    // b_k = 1 - a_k - c_k, minus dgdtg * dtg on the surface row, and rhs the
    // old temperatures after the explicit surface update
    // T_1 + (ga - T_1 dgdtg) dtg (:129-131, :201-204).
    //   kS64: that system in FP64 (coefficients formed in FP32 and widened,
    //   b and the elimination in FP64), the explicit update in FP32 as the
    //   reference's REAL arithmetic, the solution rounded to the FP32 state.
    //   Otherwise: solved for the temperature change of the step
    //   (trid_correction).  Subtracting A T_old leaves ga * dtg on the
    //   surface row and -a_k (T_{k-1} - T_k) - c_k (T_{k+1} - T_k)
    //   everywhere: the surface-coupling terms in dgdtg cancel exactly.
    // kS64: a warp whose tiles all lack snow layers solves the 6 soil rows;
    // a warp with a snow-layered tile solves the 9-row system for each of
    // its tiles, the others with identity snow rows (zero coefficients and
    // right-hand side) and the surface coupling on soil row 1, which gives
    // them the soil temperatures of their 6-row solve to the bit (the
    // identity rows add exact zeros) instead of running both solves one
    // after the other in the warp.
    const bool rows9 = kS64 ? __any_sync(__activemask(), isflag != 0) : (isflag != 0);
    if (!rows9) {
      // soil-only system: the snow rows of the reference's 9-row system are
      // identity rows decoupled from the soil (coeff(1) = 0), so the 6-row
      // solve gives the same soil temperatures
      float a[CG_MS], c[CG_MS];
      const float dtg0 = dels / gf[0];
#pragma unroll
      for (int k = 0; k < CG_MS; ++k) {
        const float dtg = dels / gf[k];
        a[k] = -dtg * coeff[k];
        c[k] = -dtg * coeff[k + 1];
      }
      if constexpr (kS64) {
        double rd[CG_MS];
#pragma unroll
        for (int k = 1; k < CG_MS; ++k) rd[k] = f2d(tgg[k]);
        // the explicit surface update T_1 + (ga - T_1 dgdtg) dtg, rounded
        // the same in both solves
        rd[0] = f2d(__fmaf_rn(__fmaf_rn(-tgg[0], dgdtg, ga), dtg0, tgg[0]));
        trimb64<CG_MS>(a, c, -f2d(dgdtg) * f2d(dtg0), rd);
#pragma unroll
        for (int k = 0; k < CG_MS; ++k) tgg[k] = d2f(rd[k]);
      } else {
        float b[CG_MS], r[CG_MS];
#pragma unroll
        for (int k = 0; k < CG_MS; ++k) {
          b[k] = 1.0f - a[k] - c[k];
          const float up = (k > 0) ? tgg[k - 1] - tgg[k] : 0.f;
          const float dn = (k < CG_MS - 1) ? tgg[k + 1] - tgg[k] : 0.f;
          r[k] = -(a[k] * up + c[k] * dn);
        }
        b[0] = b[0] - dgdtg * dtg0;
        r[0] = r[0] + ga * dtg0;
        trid_correction<CG_MS>(a, b, c, r);
#pragma unroll
        for (int k = 0; k < CG_MS; ++k) tgg[k] = tgg[k] + r[k];
      }
      ghflux = coefb * (tgg[0] - tgg[1]);
    } else {
      // rows 0-2 snow layers (identity rows for a tile without them), 3-8
      // soil layers
      const bool snow = isflag != 0;
      const float csnow[4] = {0.f, csn[0], csn[1], coeff[0]};   // coeff(-2..1)
      float x[9], a[9], c[9];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = snow ? tggsn[k] : 0.f;
        const float dtg = snow ? dels / (ssdn[k] * CGSNOW * sdepth[k]) : 0.f;
        a[k] = snow ? -dtg * csnow[k] : 0.f;
        c[k] = snow ? -dtg * csnow[k + 1] : 0.f;
      }
#pragma unroll
      for (int k = 0; k < CG_MS; ++k) {
        x[3 + k] = tgg[k];
        const float dtg = dels / gf[k];
        a[3 + k] = -dtg * coeff[k];
        c[3 + k] = -dtg * coeff[k + 1];
      }
      if constexpr (kS64) {
        // the surface row: the top snow layer, or soil layer 1
        const float dtg0 = snow ? dels / (ssdn[0] * CGSNOW * sdepth[0]) : dels / gf[0];
        const int s0 = snow ? 0 : 3;
        double rd[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) rd[k] = f2d(x[k]);
        rd[s0] = f2d(__fmaf_rn(__fmaf_rn(-x[s0], dgdtg, ga), dtg0, x[s0]));
        trimb64_s<9, 3>(a, c, -f2d(dgdtg) * f2d(dtg0), snow, rd);
        if (snow) {
#pragma unroll
          for (int k = 0; k < 3; ++k) tggsn[k] = d2f(rd[k]);
        }
#pragma unroll
        for (int k = 0; k < CG_MS; ++k) tgg[k] = d2f(rd[3 + k]);
      } else {
        const float dtg0 = dels / (ssdn[0] * CGSNOW * sdepth[0]);
        float b[9], r[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          b[k] = 1.0f - a[k] - c[k];
          const float up = (k > 0) ? x[k - 1] - x[k] : 0.f;
          const float dn = (k < 8) ? x[k + 1] - x[k] : 0.f;
          r[k] = -(a[k] * up + c[k] * dn);
        }
        b[0] = b[0] - dgdtg * dtg0;
        r[0] = r[0] + ga * dtg0;
        trid_correction<9>(a, b, c, r);
#pragma unroll
        for (int k = 0; k < 3; ++k) tggsn[k] = x[k] + r[k];
#pragma unroll
        for (int k = 0; k < CG_MS; ++k) tgg[k] = x[3 + k] + r[3 + k];
      }
      if (snow) sghflux = csn[0] * (tggsn[0] - tggsn[1]);
      ghflux = coefb * (tgg[0] - tgg[1]);
    }
  }
  g1f = gf[0];
  tss = (float)(1 - isflag) * tgg[0] + (float)isflag * tggsn[0];
  smelt = smelt + snow_melting();
  // remove_trans (cbl_remove_trans.F90:9-40)
  if (fevc < 0.0f) { fevw = fevw + fevc; fevc = 0.0f; }
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    const float dw = evapfbl[k] / (zse[k] * DLIQ);
    wb[k] = df_add(wb[k], -dw);
    wbf[k] = wb[k].hi;
  }
  // soilfreeze (cbl_soilfreeze.F90:9-81)
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    const float rzd = 1.0f / (zse[k] * DICE), rzl = 1.0f / (zse[k] * DLIQ);
    const bool freeze = tgg[k] < TFRZ && FROZEN_LIMIT * wbf[k] - wbicef[k] > .001f;
    const bool thaw = !freeze && tgg[k] > TFRZ && wbicef[k] > 0.f;
    if (freeze || thaw) {
      float amt;   // ice mass frozen (> 0) or melted (< 0), kg/m2
      if (freeze) {
        float sf = fminf(FROZEN_LIMIT * wbf[k] - wbicef[k], (ssat - wbf[k]) / (1.0f - DICE / DLIQ));
        amt = fminf(fmaxf(0.0f, sf) * zse[k] * DICE, (TFRZ - tgg[k]) * gf[k] / HLF);
      } else {
        amt = -fminf(wbicef[k] * zse[k] * DICE, (tgg[k] - TFRZ) * gf[k] / HLF);
      }
      df32 wbice_new = df_add(wbice[k], amt * rzd);
      if (freeze) {
        const df32 cap = df_mul(wb[k], FROZEN_LIMIT);
        if (df_lt(cap, wbice_new)) wbice_new = cap;
      } else if (wbice_new.hi < 0.f) {
        wbice_new = df32{0.f, 0.f};
      }
      wbice[k] = wbice_new;
      wb[k] = df_add(wb[k], amt * rzd - amt * rzl);
      wbf[k] = wb[k].hi;
      wbicef[k] = wbice[k].hi;
      gf[k] = fmaxf(hcll, (1.0f - ssat) * css * rhosoil + (wbf[k] - wbicef[k]) * (CSWAT * DLIQ) + wbicef[k] * (CSICE * DICE)) * zse[k];
      if (k == 0 && isflag == 0) gf[k] = gf[k] + CGSNOW * snowd;
      tgg[k] = tgg[k] + amt * HLF / gf[k];
    }
  }
  g1f = gf[0];
  // store: temperatures, snow pack, soil water / ice and the C2 record
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    df_store(D.wb, CG_MS, ld, k, t, wb[k]);
    df_store(D.wbice, CG_MS, ld, k, t, wbice[k]);
    D.tgg[k * ld + t] = tgg[k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    D.tggsn[k * ld + t] = tggsn[k]; D.ssdn[k * ld + t] = ssdn[k]; D.smass[k * ld + t] = smass[k];
    D.sdepth[k * ld + t] = sdepth[k];
  }
  D.gammzz1[t] = f2d(g1f);
  D.snowd[t] = snowd;
  D.work_c[3 * ld + t] = smelt;
  D.work_c[4 * ld + t] = ghflux;
  D.work_c[5 * ld + t] = sghflux;
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) D.work_c[(6 + k) * ld + t] = gf[k];
  if (mode == 2) D.work_c[CG_NC * ld + t] = dtmlt0;
  (void)tss; (void)first_call;
}

// kS64: the moisture solve in FP64 on the reference's direct form (trimb64
// on wblf, as cbl_smoisturev.F90:422 calls cbl_trimb.F90); otherwise in FP32
// on the step's change (trid_correction) with a flux-form state update.
template <bool kDiag, bool kCoupled = false, bool kS64 = true>
__device__ __forceinline__ void phase_c3(const CgDev& D, const CgTables* __restrict__ T, const StepParams& P, int t) {
  // the coupled-call code exists only in the kCoupled instantiation
  const int mode = kCoupled ? P.mode : 0;
  const int ld = D.ld;
  const float dels = P.dels;
  const int iveg = D.iveg[t], isoilm = D.isoilm[t];
  const int v = iveg - 1, so = isoilm - 1;
  const CgPftTable& V = T->pft;
  const CgSoilTable& S = T->soil;
  const float vlai = (iveg >= 14) ? 0.0f : D.vlai[t];
  const float ssat = ldf(S.ssat, so), sfc = ldf(S.sfc, so), swilt = ldf(S.swilt, so), css = ldf(S.css, so);
  const float rhosoil = ldf(S.rhosoil, so);
  // soil layer thicknesses (m), cable_parameters.F90:1241: model constants,
  // the same values as the table's, as immediates rather than registers
  constexpr float zse[CG_MS] = {0.022f, 0.058f, 0.154f, 0.409f, 1.085f, 2.872f};
  // state
  df32 wb[CG_MS], wbice[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wb[k] = df_load(D.wb, CG_MS, ld, k, t); wbice[k] = df_load(D.wbice, CG_MS, ld, k, t); }
  // FP32 shadows of soil water and ice for thresholds and fluxes; every
  // change to the state is mirrored into them
  float wbf[CG_MS], wbicef[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) { wbf[k] = wb[k].hi; wbicef[k] = wbice[k].hi; }
  float tgg[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) tgg[k] = D.tgg[k * ld + t];
  float tggsn[3], ssdn[3], smass[3], sdepth[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tggsn[k] = D.tggsn[k * ld + t]; ssdn[k] = D.ssdn[k * ld + t];
    smass[k] = D.smass[k * ld + t]; sdepth[k] = D.sdepth[k * ld + t];
  }
  const uint8_t flags = D.flags[t];
  int isflag = flags & 1;
  bool first_call = (flags & 2) != 0;
  double gammzz1 = D.gammzz1[t];
  float snowd = D.snowd[t], ssdnn = D.ssdnn[t], snage = D.snage[t], pudsto = D.pudsto[t];
  float wb_lake = D.wb_lake[t];
  const float pudsmx = 0.0f;
  const float rlam = HL;
  // phase A and B records
  const float tk = D.work_a[0 * ld + t], precip = D.work_a[6 * ld + t];
  const float transd = D.work_a[27 * ld + t];
  auto Bv = [&](int i) { return D.work_b[i * ld + t]; };
  const float ga = Bv(0), dgdtg = Bv(1), fes = Bv(2), fess = Bv(3), fesp = Bv(4);
  float fevc = Bv(5), fevw = Bv(6);
  const float cls = Bv(7), precis0 = Bv(8);
  float evapfbl[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) evapfbl[k] = Bv(9 + k);
  const float delwc = Bv(15), fpn = Bv(16), frday = Bv(17), tv = Bv(18);
  float tss;
  // soil_snow, water part (cbl_soilsnow_main.F90:139-203), then snow_aging,
  // carbon and the balances
  const float osnowd = D.work_c[0 * ld + t];
  float precis = D.work_c[1 * ld + t];
  const float segg = D.work_c[2 * ld + t];
  float smelt = D.work_c[3 * ld + t];
  const float ghflux = D.work_c[4 * ld + t], sghflux = D.work_c[5 * ld + t];
  float gf[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) gf[k] = D.work_c[(6 + k) * ld + t];
  float g1f = d2f(gammzz1);
  // remove_trans moved negative transpiration into wet-canopy evaporation
  if (fevc < 0.0f) { fevw = fevw + fevc; fevc = 0.0f; }
  // infiltration (cbl_soilsnow_main.F90:139-159)
  float rnof1, rnof2;
  float fwtop[3];
  {
    float weting = precis + smelt + fmaxf(0.f, pudsto - fesp / HL * dels);
    float sinfil[3];
    float rem = weting;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sinfil[k] = fminf(0.95f * (ssat - wbf[k]) * zse[k] * DLIQ, rem);
      rem = rem - sinfil[k];
    }
    fwtop[0] = sinfil[0] / dels - segg;
    fwtop[1] = sinfil[1] / dels;
    fwtop[2] = sinfil[2] / dels;
    pudsto = fmaxf(0.f, weting - sinfil[0] - sinfil[1] - sinfil[2]);
    rnof1 = fmaxf(0.f, pudsto - pudsmx);
    pudsto = pudsto - rnof1;
  }
  // surfbv -> smoisturev (cbl_surfbv.F90:9-146, cbl_smoisturev.F90:11-444, nmeth = -1)
  {
    const float hyds = ldf(S.hyds, so), i2bp3 = ldf(S.i2bp3, so), ibp2 = ldf(S.ibp2, so), hsbh = ldf(S.hsbh, so);
    const float pwb_min = ldf(S.pwb_min, so);
    float fluxh[CG_MS + 1];
    fluxh[0] = 0.f; fluxh[CG_MS] = 0.f;
    float delt_prev = 0.f;
    const float wbl_min = P.runoff_speed ? 0.001f : 0.01f;   // l_new_runoff_speed (cbl_smoisturev.F90:112)
#pragma unroll
    for (int k = 1; k <= CG_MS - 1; ++k) {
      float wbl_k = fmaxf(wbl_min, wbf[k - 1] - wbicef[k - 1]);
      float wbl_kp = fmaxf(wbl_min, wbf[k] - wbicef[k]);
      float delt = wbl_kp - wbl_k;
      float wh = fminf(wbl_k, wbl_kp);
      if (wbicef[k - 1] > 0.05f || wbicef[k] > 0.01f) wh = 0.9f * wbl_k + 0.1f * wbl_kp;
      float speed_k = hyds * __powf(wh / ssat, i2bp3 - 1.f);
      float rat = delt_prev / (delt + fsignf(1.0e-20f, delt));
      float phi = fmaxf(fmaxf(0.0f, fminf(1.0f, 2.0f * rat)), fminf(2.0f, rat));
      speed_k = fminf(speed_k, 0.5f * zse[k - 1] / dels);
      fluxh[k] = speed_k * (wbl_k + phi * (wh - wbl_k));
      delt_prev = delt;
    }
    if (wbf[CG_MS - 1] > sfc) {
      float wbl_k = fmaxf(0.001f, wbf[CG_MS - 1] - wbicef[CG_MS - 1]);
      float wbl_kp = fmaxf(0.001f, ssat - wbicef[CG_MS - 1]);
      float wh = fminf(wbl_k, wbl_kp);
      if (wbicef[CG_MS - 1] > 0.05f) wh = 0.9f * wbl_k + 0.1f * wbl_kp;
      float speed_k = hyds * __powf(wh / ssat, i2bp3 - 1.f);
      if (P.runoff_speed) {   // cbl_smoisturev.F90:180-197
        speed_k = speed_k / (1.f - fminf(0.5f, 10.f * wbicef[CG_MS - 1]));
        speed_k = fminf(speed_k, 0.5f * zse[CG_MS - 1] / dels);
      } else {
        speed_k = 0.5f * speed_k / (1.f - fminf(0.5f, 10.f * wbicef[CG_MS - 1]));
        speed_k = fminf(0.5f * speed_k, 0.5f * zse[CG_MS - 1] / dels);
      }
      fluxh[CG_MS] = fmaxf(0.0f, speed_k * wbl_k);
    }
    // drainage step (cbl_smoisturev.F90, nmeth = -1 explicit part); its
    // FP32 increments join the diffusion increments below in one FP64
    // update of the state
    float dwd[CG_MS];
#pragma unroll
    for (int k = CG_MS; k >= 1; --k) {
      fluxh[k - 1] = fminf(fluxh[k - 1], (ssat - wbf[k - 1]) * zse[k - 1] / dels + fluxh[k]);
      dwd[k - 1] = dels * (fluxh[k - 1] - fluxh[k]) / zse[k - 1];
      wbf[k - 1] = wbf[k - 1] + dwd[k - 1];
    }
    rnof2 = dels * fluxh[CG_MS] * DLIQ;
    if constexpr (kS64) {
      // Implicit diffusion of the liquid fraction wblf = (wb - wbice) /
      // (ssat - wbice) on the reference's direct form
      // (cbl_smoisturev.F90:200-262, :422-427), the elimination (trimb64) in
      // FP64.  Its right-hand side is formed at the soil water state's own
      // precision, double-FP32 (48-bit significand), on the FP32 pipe: the
      // liquid water after the explicit drainage, wb + dwd - wbice, with
      // error-free FP32 operations, divided by the pore space (df_div,
      // ~2^-46), plus the top layers' infiltration source, then widened to
      // FP64 once.  The solution goes back the same way: wb = wblf
      // (ssat - wbice) + wbice as a double-FP32 product and sum (df_split,
      // df_mul), the state's storage format.  The pore space ssat - wbice
      // is the FP32 value (ssat is REAL in the reference) in wblf, in
      // dtt = dels / (zse (ssat - wbice)) and in the product, so the scaling
      // in and out of wblf is inverse to the state's precision.  The matrix
      // coefficients dtt z3 are FP32 (bulk arithmetic, widened exactly).
      double rd[CG_MS];
      float sat[CG_MS], xf[CG_MS], dtt[CG_MS];
#pragma unroll
      for (int k = 0; k < CG_MS; ++k) {
        sat[k] = ssat - wbicef[k];
        const df32 liq = df_add(df_add(wb[k], dwd[k]), df32{-wbice[k].hi, -wbice[k].lo});
        df32 q = df_div(liq, sat[k]);
        xf[k] = q.hi;   // the conductivity's weighting, FP32
        dtt[k] = dels / (zse[k] * sat[k]);
        if (k < 3) q = df_add(q, dtt[k] * fwtop[k] / DLIQ);
        rd[k] = df_to_double(q);
      }
      float a[CG_MS], c[CG_MS];
      a[0] = 0.f; c[CG_MS - 1] = 0.f;
#pragma unroll
      for (int k = 2; k <= CG_MS; ++k) {
        float wbh_k = (zse[k - 1] * xf[k - 2] + zse[k - 2] * xf[k - 1]) / (zse[k - 1] + zse[k - 2]);
        float fact = __powf(wbh_k, ibp2 - 1.f);
        float icef = fmaxf(wbicef[k - 2] / fmaxf(0.01f, wbf[k - 2]), wbicef[k - 1] / fmaxf(0.01f, wbf[k - 1]));
        float pwb_wbh = (hsbh * (1.f - fminf(2.f * fminf(0.1f, icef), 0.1f))) * fmaxf(pwb_min, wbh_k * fact);
        const float z3 = pwb_wbh / ZSHH[k - 1];
        a[k - 1] = -dtt[k - 1] * z3;
        c[k - 2] = -dtt[k - 2] * z3;
      }
      trimb64<CG_MS, false>(a, c, 0.0, rd);
#pragma unroll
      for (int k = 0; k < CG_MS; ++k) {
        wb[k] = df_add(df_mul(df_split(rd[k]), sat[k]), wbice[k]);
        wbf[k] = wb[k].hi;
      }
    } else {
    // Implicit diffusion of the liquid fraction x = (wb - wbice) /
    // (ssat - wbice) (cbl_smoisturev.F90, trimb on wblfsp), solved for the
    // change of x (trid_correction): the right-hand side is the top layers'
    // infiltration source minus M x_old, with the differences of x between
    // layers formed from FP64 differences of the state, so they are exact
    // to FP32 rounding and zero for a uniform column.
    float sat[CG_MS], x[CG_MS], dtt[CG_MS];
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) {
      sat[k] = ssat - wbicef[k];
      x[k] = (wbf[k] - wbicef[k]) / sat[k];   // conductivity weighting only
      dtt[k] = dels / (zse[k] * sat[k]);
    }
    // dx[k] = x_{k-1} - x_k = (liq_{k-1} - liq_k) / sat_{k-1}
    //         + x_k (wbice_{k-1} - wbice_k) / sat_{k-1},
    // liq_{k-1} - liq_k = (wb_{k-1} - wb_k) + (dw_{k-1} - dw_k) - di
    float dx[CG_MS + 1];
    dx[0] = 0.f; dx[CG_MS] = 0.f;
#pragma unroll
    for (int k = 1; k < CG_MS; ++k) {
      const float di = (wbicef[k - 1] != 0.f || wbicef[k] != 0.f) ? df_sub(wbice[k - 1], wbice[k]) : 0.f;
      const float dl = df_sub(wb[k - 1], wb[k]) + (dwd[k - 1] - dwd[k]) - di;
      dx[k] = (dl + x[k] * di) / sat[k - 1];
    }
    float a[CG_MS], b[CG_MS], c[CG_MS], r[CG_MS];
    float z3[CG_MS];   // z3[k]: conductance of the interface between layers k-1 and k
    a[0] = 0.f; c[CG_MS - 1] = 0.f;
#pragma unroll
    for (int k = 2; k <= CG_MS; ++k) {
      float wbh_k = (zse[k - 1] * x[k - 2] + zse[k - 2] * x[k - 1]) / (zse[k - 1] + zse[k - 2]);
      float fact = __powf(wbh_k, ibp2 - 1.f);
      float icef = fmaxf(wbicef[k - 2] / fmaxf(0.01f, wbf[k - 2]), wbicef[k - 1] / fmaxf(0.01f, wbf[k - 1]));
      float pwb_wbh = (hsbh * (1.f - fminf(2.f * fminf(0.1f, icef), 0.1f))) * fmaxf(pwb_min, wbh_k * fact);
      z3[k - 1] = pwb_wbh / ZSHH[k - 1];
      a[k - 1] = -dtt[k - 1] * z3[k - 1];
      c[k - 2] = -dtt[k - 2] * z3[k - 1];
    }
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) {
      b[k] = 1.0f - a[k] - c[k];
      r[k] = -a[k] * dx[k] + c[k] * dx[k + 1];
      if (k < 3) r[k] = r[k] + dtt[k] * fwtop[k] / DLIQ;
    }
    trid_correction<CG_MS>(a, b, c, r);
    // Row k of the solve reads d_k = dtt_k (G_k - G_{k+1} + src_k) with the
    // interface flux G_k = z3_k (dx_k + d_{k-1} - d_k), and dtt_k sat_k =
    // dels / zse_k.  The state is updated in that flux form: each interface
    // carries one FP32 amount (explicit drainage plus implicit diffusion, m
    // of water per step) that leaves one layer and enters the next, so the
    // column total changes by exactly the top sources and the bottom
    // drainage.  (Applying d_k sat_k directly loses conservation in
    // proportion to |a| |d|, which for the stiff, highly conductive soils is
    // ~1e-3 mm per step.)
    float H[CG_MS + 1];
    H[0] = dels * fluxh[0];
    H[CG_MS] = dels * fluxh[CG_MS];
#pragma unroll
    for (int k = 1; k < CG_MS; ++k) H[k] = dels * (fluxh[k] + z3[k] * (dx[k] + r[k - 1] - r[k]));
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) {
      float net = H[k] - H[k + 1];
      if (k < 3) net = net + dels * fwtop[k] / DLIQ;
      wb[k] = df_add(wb[k], net / zse[k]);
      wbf[k] = wb[k].hi;
    }
    }
    const float dfactor = 1.0f - DICE / DLIQ;
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) {
      if (wbicef[k] > FROZEN_LIMIT * wbf[k]) {
        const float sm = df_sub(wbice[k], df_mul(wb[k], FROZEN_LIMIT)) * (1.0f / (1.0f - FROZEN_LIMIT * dfactor));
        wbice[k] = df_add(wbice[k], -sm);
        wb[k] = df_add(wb[k], -dfactor * sm);
        wbf[k] = wb[k].hi;
        wbicef[k] = wbice[k].hi;
        tgg[k] = tgg[k] - sm * zse[k] * DICE * HLF / gf[k];
      }
    }
  }
  // surfbv remainder
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    if (wbf[k] > ssat) {
      // the excess over saturation, low word included, leaves as runoff
      rnof1 = rnof1 + df_sub(wb[k], df32{ssat, 0.f}) * (DLIQ * zse[k]);
      wb[k] = df32{ssat, 0.f};
      wbf[k] = ssat;
    } else if (wbf[k] < swilt / 4.0f) {
      wb[k] = df32{swilt / 4.0f, 0.f};
      wbf[k] = swilt / 4.0f;
    }
  }
  float rnof5 = 0.f;
  {
    float smasstot = 0.f;
    float sm1[3] = {0.f, 0.f, 0.f};
    if (snowd > MAX_GLACIER_SNOWD) {
      rnof5 = fminf(0.1f, snowd - MAX_GLACIER_SNOWD);
      if (isflag == 0) {
        tgg[0] = tgg[0] - rnof5 * HLF / g1f;
        snowd = snowd - rnof5;
      } else {
        smasstot = smass[0] + smass[1] + smass[2];
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (snowd > MAX_GLACIER_SNOWD && isflag > 0) {
        sm1[k] = fminf(rnof5 * smass[k] / smasstot, 0.2f * smass[k]);
        smass[k] = smass[k] - sm1[k];
        snowd = snowd - sm1[k];
      }
    }
    if (isflag > 0) rnof5 = sm1[0] + sm1[1] + sm1[2];
  }
  if (iveg == LAKES) {
    float sinfil = fminf(rnof1, wb_lake);
    rnof1 = fmaxf(0.0f, rnof1 - sinfil);
    wb_lake = fmaxf(0.0f, wb_lake - sinfil);
    sinfil = fminf(rnof2, wb_lake);
    rnof2 = fmaxf(0.0f, rnof2 - sinfil);
    wb_lake = fmaxf(0.0f, wb_lake - sinfil);
    float xl = fmaxf(0.0f, df_sub(wb[CG_MS - 1], df32{sfc, 0.f}) * (zse[CG_MS - 1] * DLIQ));
    sinfil = fminf(xl, wb_lake);
    wb[CG_MS - 1] = df_add(wb[CG_MS - 1], -(sinfil / (zse[CG_MS - 1] * DLIQ)));
    wb_lake = fmaxf(0.0f, wb_lake - sinfil);
    xl = fmaxf(0.0f, df_sub(wb[CG_MS - 1], df32{0.5f * (sfc + swilt), 0.f}) * (zse[CG_MS - 1] * DLIQ));
    sinfil = fminf(xl, wb_lake);
    wb[CG_MS - 1] = df_add(wb[CG_MS - 1], -(sinfil / (zse[CG_MS - 1] * DLIQ)));
    wb_lake = fmaxf(0.0f, wb_lake - sinfil);
    wbf[CG_MS - 1] = wb[CG_MS - 1].hi;
  }
  rnof1 = rnof1 / dels + rnof5 / dels;
  rnof2 = rnof2 / dels;
  tss = (float)(1 - isflag) * tgg[0] + (float)isflag * tggsn[0];
  // column water (mm): sum of zse (DLIQ (wb - wbice) + DICE wbice)
  constexpr double ZL[CG_MS] = {(double)0.022f * DLIQ, (double)0.058f * DLIQ, (double)0.154f * DLIQ,
                                (double)0.409f * DLIQ, (double)1.085f * DLIQ, (double)2.872f * DLIQ};
  constexpr double ZI[CG_MS] = {(double)0.022f * (DICE - DLIQ), (double)0.058f * (DICE - DLIQ),
                                (double)0.154f * (DICE - DLIQ), (double)0.409f * (DICE - DLIQ),
                                (double)1.085f * (DICE - DLIQ), (double)2.872f * (DICE - DLIQ)};
  // summed in double-FP32 (weights rounded to FP32 once; the same every
  // step, so the step-to-step change the water balance uses is unaffected)
  df32 wsum{0.f, 0.f};
#pragma unroll
  for (int k = 0; k < CG_MS; ++k)
    wsum = df_add(df_add(wsum, df_mul(wb[k], (float)ZL[k])), df_mul(wbice[k], (float)ZI[k]));
  const double wbtot = df_to_double(wsum);

  // snow_aging (cbl_snow_aging.F90:11-83)
  if (snowd > 1.0f) {
    float dnsnow = fminf(1.0f, 0.1f * fmaxf(0.0f, snowd - osnowd));
    float tmp = fminf((float)isflag * tggsn[0] + (float)(1 - isflag) * tgg[0], TFRZ);
    float ar1 = 5000.0f * (1.0f / (TFRZ - 0.01f) - 1.0f / tmp);
    float ar3;
    if (isoilm == ICE_SOIL) { ar3 = 0.0000001f; dnsnow = 1.0f; }
    else ar3 = 0.1f;
    float dtau = 1.0e-6f * (__expf(ar1) + __expf(10.0f * ar1) + ar3) * dels;
    snage = fmaxf(0.0f, (snage + dtau) * (1.0f - dnsnow));
  }
  float trad;
  if (mode != 2) {
    trad = sqrtf(sqrtf((1.f - transd) * pow4(tv) + transd * pow4(tss)));
  } else {
    // implicit coupled call: the online energy-balance corrections of
    // soil_snow (cbl_soilsnow_main.F90:164-183, melt-driven) and of cbm_impl
    // (cbl_cbm_mod.F90:317-357, surface-temperature-driven; the temperature
    // is reset to the start of the step first on a cycle that is not the
    // last, :307-311), applied to the canopy kernel's fe, fh, rnet and ga;
    // then cbm_impl's radiative temperature (:374-381): emissivities 1, the
    // start-of-step surface temperature and the correction fns_cor / sigma
    const float otss = D.tss[t];
    if (!P.final_cycle) tss = otss;
    const float dfh_dtg = Bv(CG_NB), dfe_dtg = Bv(CG_NB + 1), dfn_dtg = Bv(CG_NB + 2);
    const float dtm = D.work_c[CG_NC * ld + t];
    const float dT = tss - otss;
    const size_t oc = D.out_caller_order ? (size_t)D.tile_id[t] : (size_t)t;
    auto add_out = [&](int i, float dv) {
      const float x = D.out[i * ld + t] + dv;
      D.out[i * ld + t] = x;
      if (D.out_caller) D.out_caller[(size_t)i * D.mp + oc] = x;
    };
    add_out(0, dtm * dfe_dtg + dT * dfe_dtg);   // fe = fev + fes
    add_out(1, dtm * dfh_dtg + dT * dfh_dtg);   // fh = fhv + fhs
    float fns_cor = 0.f;
    if (P.rev_corr) {
      fns_cor = dtm * dfn_dtg + dT * dfn_dtg;
      add_out(5, fns_cor);                      // rnet = fns + fnv
      add_out(6, dtm * dgdtg + dT * dgdtg);     // ga
    }
    trad = sqrtf(sqrtf((1.f - transd) * pow4(tv) + transd * pow4(otss) + fns_cor / SBOLTZ));
  }

  // carbon, icycle == 0 (cable_carbon.F90:38-360, cbm:214-229)
  // root fractions, used only by the carbon routines below
  float froot[CG_MS];
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) froot[k] = ldf(V.froot[k], v);
  float frp, frpw, frpr, frs;
  float cplant[3], csoil[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) cplant[k] = D.cplant[k * ld + t];
  csoil[0] = D.csoil[t]; csoil[1] = D.csoil[ld + t];
  {
    const float rc0 = V.ratecp[0], rc1 = V.ratecp[1], rc2 = V.ratecp[2];
    float tot = rc0 * cplant[0] + rc1 * cplant[1] + rc2 * cplant[2];
    float pc1 = tot - rc0 * cplant[0];
    float pc1w = pc1 - rc2 * cplant[2];
    float pc1r = pc1 - rc1 * cplant[1];
    float tmp1 = fmaxf(3.22f - 0.046f * (tk - TFRZ), 1e-6f);
    float tmp3 = __powf(tmp1, 0.1f * (tk - TFRZ - 20.0f));
    float c = ldf(V.rp20, v) * tmp3 / 31536000.0f;
    frp = c * pc1; frpw = c * pc1w; frpr = c * pc1r;
  }
  if (P.soil_resp_off) {
    // diag_soil_resp = 'OFF' (cable_carbon.F90:256-276): rs20 scheme
    float avgwrs = 0.f, sumt = 0.f;
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) { avgwrs += froot[k] * wbf[k]; sumt += froot[k] * tgg[k]; }
    const float avgtrs = fmaxf(0.0f, sumt - TFRZ);
    frs = ldf(V.rs20, v) *
          fminf(1.0f, fmaxf(0.0f, fminf(-0.0178f + 0.2883f * avgwrs + 5.0176f * avgwrs * avgwrs -
                                             4.5128f * avgwrs * avgwrs * avgwrs,
                                         0.3320f + 22.6726f * __expf(-5.8184f * avgwrs)))) *
          fminf(1.0f, fmaxf(0.0f, fminf(0.0104f * __powf(avgtrs, 1.3053f), 5.5956f - 0.1189f * avgtrs)));
    frs = frs * (V.ratecs[0] * csoil[0] + V.ratecs[1] * csoil[1]) / (365.0f * 24.0f * 3600.0f);
    if (snowd > 1.f) frs = frs / fmaxf(0.001f, fminf(100.f, snowd));
  } else {
    float den = fmaxf(0.07f, sfc - swilt);
    float rswc = fmaxf(0.0001f, froot[0] * (wbf[1] - swilt)) / den;
    float tsoil = froot[0] * tgg[1] - TFRZ;
    float tref = fmaxf(0.f, tgg[CG_MS - 1] - (TFRZ - .05f));
#pragma unroll
    for (int k = 1; k < CG_MS; ++k) {
      rswc += fmaxf(0.0001f, froot[k] * (wbf[k] - swilt)) / den;
      tsoil += froot[k] * tgg[k];
    }
    rswc = fminf(1.f, rswc);
    tsoil = fmaxf(-46.f + 2.f, tsoil);
    float e0rswc = 52.4f + 285.f * rswc;
    float ftsoil = fminf(0.0015f, 1.f / (tref + 46.f) - 1.f / (tsoil + 46.f));
    float sss = fmaxf(-15.f, fminf(1.f, e0rswc * ftsoil));
    frs = ldf(V.vegcf, v) * (144.0f / 44.0e6f) * fminf(1.f, 1.4f * fmaxf(.3f, .0278f * tsoil + .5f)) * __expf(sss) * rswc /
          (0.16f + rswc);
  }
  {
    float coef_cold = __expf(fminf(1.f, -(tv - ldf(V.tvclst, v))));
    float wbav = 0.f;
#pragma unroll
    for (int k = 0; k < CG_MS; ++k) wbav += froot[k] * wbf[k];
    wbav = fmaxf(0.01f, wbav);
    float campbell = 2.0f - ldf(S.ibp2, so);
    float esw = fmaxf(1.0f, __powf(wbav, campbell) - 1.0f);
    float eswilt = __powf(swilt, campbell) - 1.0f;
    float relstress = fminf(1.0f, esw / eswilt - 1.0f);
    float coef_cd = (coef_cold + __expf(5.0f * relstress)) * 2.0e-7f;
    float fcl = __expf(-ldf(V.tfcl, v) * vlai);
    float clitt = (coef_cd + 3.17e-8f) * cplant[0];
    cplant[0] = cplant[0] - dels * (fpn * fcl + clitt);
    float fr = fminf(1.f, __expf(-ldf(V.rw, v) * 0.9f * 0.0001f * cplant[2] / fmaxf(cplant[1], 0.01f)) / 0.9f);
    float cfwd = 6.342e-10f * cplant[1];
    cplant[1] = cplant[1] - dels * (fpn * (1.f - fcl) * (1.f - fr) + frpw + cfwd);
    float cfrts = 4.53e-9f * cplant[2];
    cplant[2] = cplant[2] - dels * (fpn * (1.f - fcl) * fr + cfrts + frpr);
    float cfsf = 1.057e-10f * csoil[0];
    csoil[0] = csoil[0] + dels * (0.98f * clitt + 0.9f * cfrts + cfwd - cfsf - 0.98f * frs);
    csoil[1] = csoil[1] + dels * (0.02f * clitt + 0.1f * cfrts + cfsf - 0.02f * frs);
#pragma unroll
    for (int k = 0; k < 3; ++k) cplant[k] = fmaxf(0.f, cplant[k]);
    csoil[0] = fmaxf(0.f, csoil[0]); csoil[1] = fmaxf(0.f, csoil[1]);
  }

  // driver rescaling (cable_serial.F90:602-605) and balances (cable_checks.F90)
  // rounded operations throughout: the compiler may not fuse a product into
  // the sums here differently in the kernels with and without diagnostics
  const float runoff_mm = __fmul_rn(__fadd_rn(rnof1, rnof2), dels);
  const float evap_mm = __fdiv_rn(__fmul_rn(__fadd_rn(__fadd_rn(fevw, fevc), __fdiv_rn(fes, cls)), dels), rlam);
  double owb = D.owb[t];
  if (P.ktau == 1) owb = wbtot;
  const double delwb = wbtot - owb;
  const float wbal = d2f(f2d(precip - delwc - snowd + osnowd - runoff_mm - evap_mm) - delwb);
  double wbal_tot = D.wbal_tot[t];
  if (P.ktau == 1) wbal_tot = 0.0;
  if (P.ktau > 10) wbal_tot += f2d(wbal);

  // store
#pragma unroll
  for (int k = 0; k < CG_MS; ++k) {
    df_store(D.wb, CG_MS, ld, k, t, wb[k]);
    df_store(D.wbice, CG_MS, ld, k, t, wbice[k]);
    D.tgg[k * ld + t] = tgg[k];
  }
  (void)first_call; (void)isoilm;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    D.tggsn[k * ld + t] = tggsn[k]; D.ssdn[k * ld + t] = ssdn[k]; D.smass[k * ld + t] = smass[k];
    D.sdepth[k * ld + t] = sdepth[k]; D.cplant[k * ld + t] = cplant[k];
  }
  D.csoil[t] = csoil[0]; D.csoil[ld + t] = csoil[1];
  D.snowd[t] = snowd; D.ssdnn[t] = ssdnn; D.snage[t] = snage; D.pudsto[t] = pudsto;
  D.tss[t] = tss; D.wb_lake[t] = wb_lake;
  if (mode == 0) { D.owb[t] = wbtot; D.wbal_tot[t] = wbal_tot; }   // no balance checks in coupled calls
  D.out[7 * ld + t] = trad;
  if (D.out_caller) D.out_caller[(size_t)7 * D.mp + (D.out_caller_order ? (size_t)D.tile_id[t] : (size_t)t)] = trad;
  {
    uint8_t bits = 0;
    if (!isfinite(trad)) { atomicOr(D.status, 1u); bits |= CG_TS_NONFINITE; }
    // RadT and SoilTemp ranges (cable_checks.F90:81-104)
    float tlo = tgg[0], thi = tgg[0];
#pragma unroll
    for (int k = 1; k < CG_MS; ++k) { tlo = fminf(tlo, tgg[k]); thi = fmaxf(thi, tgg[k]); }
    if (out_of(trad, 200.f, 373.f) || out_of(tlo, 213.f, 353.f) || out_of(thi, 213.f, 353.f))
      bits |= CG_TS_OUTPUT_RANGE;
    if (bits) D.tile_status[t] |= bits;
  }
  if (kDiag) {
    const int idx[18] = {17, 19, 23, 24, 25, 26, 27, 28, 37, 38, 39, 40, 41, 42, 46, 54, 61, 62};
    const float val[18] = {fevc, fevw, -fpn - frp, fpn + frs + frp, frp + frday, frp, frs, trad, runoff_mm,
                           rnof1 * dels, rnof2 * dels, smelt, ghflux, sghflux, wbal, (float)wbtot, frpw, frpr};
#pragma unroll
    for (int i = 0; i < 18; ++i) D.diag[idx[i] * ld + t] = val[i];
  }
}

}  // namespace cg
