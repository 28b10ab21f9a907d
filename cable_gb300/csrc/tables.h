// Per-PFT and per-soil parameter tables of the CABLE offline defaults, with
// every per-type derived quantity precomputed on the host so the timestep
// kernel only gathers them.
//
// Data sources (values, not code):
//   src/offline/pft_params.nml:2-61            17 plant functional types
//   src/offline/cable_soilparm.nml:3-22        9 soil types
//   src/science/misc/cable_carbon.F90:129-140  carbon turnover tables (17 types)
// Derivations (restated in build_tables below):
//   dleaf = sqrt(width*length)                       cable_pft_params.F90:110
//   ejmax = 2*vcmax                                  cable_parameters.F90:1543
//   froot from rootbeta (Jackson et al. 1996)        cable_parameters.F90:3331-3343
//   hsbh, ibp2, i2bp3, pwb_min                       cable_parameters.F90:2236-2245
//   cnsd = 0.3 sand + 0.25 clay + 0.265 silt         cable_parameters.F90:2230
//   zshh                                             cable_parameters.F90:1828-1831
//   soil_thermal_fix set: cnsdv, and css, rhosoil,   cable_parameters.F90:2165-2227
//   cnsd rewritten (cg_apply_soil_thermal_fix);
//   ktmp, the saturated-conductivity factor of        cbl_conductivity.F90:36-43
//   total_soil_conductivity
// Soil albedo is not in the reference tables (it is read from the gridded
// soil file); the VIS/NIR pair per soil type below is this library's choice.
#pragma once

#define CG_NPFT 17
#define CG_NSOIL 9
#define CG_MS 6
#define CG_MSN 3

// Structure-of-arrays so a warp's divergent gather touches few cache lines.
struct CgPftTable {
  float canst1[CG_NPFT], dleaf[CG_NPFT], ejmax[CG_NPFT], frac4[CG_NPFT], hc[CG_NPFT], vbeta[CG_NPFT];
  float rp20[CG_NPFT], vegcf[CG_NPFT], extkn[CG_NPFT], a1gs[CG_NPFT], d0gs[CG_NPFT];
  float alpha[CG_NPFT], convex[CG_NPFT], cfrd[CG_NPFT], gswmin[CG_NPFT], conkc0[CG_NPFT], conko0[CG_NPFT];
  float ekc[CG_NPFT], eko[CG_NPFT], g0[CG_NPFT], g1[CG_NPFT], vcmax[CG_NPFT], xfang[CG_NPFT], shelrb[CG_NPFT];
  float refl1[CG_NPFT], refl2[CG_NPFT], taul1[CG_NPFT], taul2[CG_NPFT];
  float froot[CG_MS][CG_NPFT];
  float rw[CG_NPFT], tfcl[CG_NPFT], tvclst[CG_NPFT];
  float clitt[CG_NPFT];   // litter carbon, used by the litter switch
  float rs20[CG_NPFT];    // soil respiration at 20 C, used by diag_soil_resp = 'OFF'
  float cplant0[3][CG_NPFT], csoil0[2][CG_NPFT];
  float ratecp[3], ratecs[2];
};

struct CgSoilTable {
  float bch[CG_NSOIL], css[CG_NSOIL], hyds[CG_NSOIL], rhosoil[CG_NSOIL], sfc[CG_NSOIL], ssat[CG_NSOIL];
  float sucs[CG_NSOIL], swilt[CG_NSOIL], cnsd[CG_NSOIL], hsbh[CG_NSOIL], ibp2[CG_NSOIL], i2bp3[CG_NSOIL];
  float pwb_min[CG_NSOIL], albsoil_vis[CG_NSOIL], albsoil_nir[CG_NSOIL];
  float sand[CG_NSOIL], clay[CG_NSOIL], silt[CG_NSOIL];
  float zse[CG_MS], zshh[CG_MS + 1];
  // soil_thermal_fix: dry conductivity cnsd_vec and Ktmp = ((7.7^q Ko^(1-q))^(1-ssat),
  // q the quartz fraction (both unused unless the switch is on)
  float cnsdv[CG_NSOIL], ktmp[CG_NSOIL];
};

// Fills both tables; implemented in tables.cpp (host only).
void cg_build_tables(CgPftTable* pft, CgSoilTable* soil);
// Rewrites css, rhosoil and cnsd as the reference's parameter set-up does
// under soil_thermal_fix (rhosoil / (1 - ssat), css from the texture
// regression, cnsd = cnsd_vec).
void cg_apply_soil_thermal_fix(CgSoilTable* soil);
