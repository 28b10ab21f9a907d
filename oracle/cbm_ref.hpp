// ORACLE / TEST INFRASTRUCTURE ONLY.
// CPU restatement of CABLE's offline cbm() timestep for ONE tile, templated on
// the reference's two real kinds:  R = default REAL, R2 = REAL(r_2).
//   cbm_ref<double,double>  : the FP64 parity oracle
//   cbm_ref<float,double>   : the reference's own precision mix (offline build:
//                             REAL is 4-byte, r_2 is 8-byte;
//                             src/offline/cable_define_types.F90:55-61)
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg may use
// anything under oracle/; the product never links it.
//
// Parity status: unpinned by the reference's own tests (there are no golden
// vectors for this path and the Fortran cannot be compiled here); pinned to
// physical invariants (energy/water closure, leaf energy balance, closed-form
// unit checks) by tests/test_oracle.py.
//
// Switch set (offline defaults, src/offline/cable.nml + cable_runtime_opts_mod):
//   soil_struc='default', fwsoil_switch='standard', ssnow_potev='HDM',
//   gs_switch='leuning' (medlyn selectable), l_rev_corr=F, litter=F,
//   or_evap=F, gw_model=F, call_climate=F, soil_thermal_fix=F, redistrb=F,
//   l_new_roughness_soil=F, l_new_runoff_speed=F, l_new_reduce_soilevp=F,
//   diag_soil_resp='ON', icycle=0, snmin=1, cable_runtime%offline=T.
//
// Every routine below cites the reference file:line it restates.  Fortran
// semantics kept: REAL() narrowing, default-REAL literals (written R(x)),
// array-WHERE order, SIGN/MERGE/NINT, and the in/out persistence of
// intent(inout) module arrays.  Tiles never interact inside cbm(), so the
// whole timestep is restated per tile.
#pragma once
#include <cmath>
#include <algorithm>
#include "cbm_ref_tables.hpp"

namespace cbmref {

template <class T> static inline T sq(T x) { return x * x; }
template <class T> static inline T fsign(T a, T b) { return std::signbit(b) ? -std::fabs(a) : std::fabs(a); }
template <class A, class B> static inline auto mx(A a, B b) { using C = decltype(a + b); return C(a) > C(b) ? C(a) : C(b); }
template <class A, class B> static inline auto mn(A a, B b) { using C = decltype(a + b); return C(a) < C(b) ? C(a) : C(b); }

// --------------------------------------------------------------------------
// Per-tile static parameters (derived at set-up from the PFT / soil tables).
template <class R, class R2>
struct Params {
  int iveg = 1, isoilm = 1;
  R vlai = 0;                     // LAI (zeroed for iveg >= 14, cable_serial.F90:575)
  R lat = 0;
  // veg (cable_parameters.F90:3277-3345, init_veg_from_vegin)
  R canst1, dleaf, ejmax, frac4, hc, vbeta, rp20, rs20, shelrb, vegcf, extkn;
  R a1gs, d0gs, alpha, convex, cfrd, gswmin, conkc0, conko0, ekc, eko, g0, g1, vcmax, xfang;
  R refl[3], taul[3], froot[MS], meth;
  R rw, tfcl, tvclst;             // carbon tables (cable_carbon.F90:129-140)
  R2 clitt;                       // litter carbon (veg%clitt, cable_parameters.F90:3330)
  R ratecp[3], ratecs[2];
  // soil (cable_parameters.F90:1511-1522 and derived_parameters :2236-2245)
  R bch, css, hyds, rhosoil, sfc, ssat, sucs, swilt, sand, clay, silt;
  R2 cnsd, pwb_min;
  // soil_thermal_fix inputs of total_soil_conductivity (cbl_conductivity.F90:10-85):
  // the layer vectors are the soil-type values spread over the layers
  // (cable_parameters.F90:1689, :1516-1529), cnsd_vec rewritten at :2184-2186
  R2 ssat_vec, sand_vec, cnsd_vec, watr;
  R hsbh, ibp2, i2bp3;
  R albsoil[3];
  R zse[MS], zshh[MS + 1];
  R2 zse_vec[MS], swilt_vec[MS], sfc_vec[MS];
  R za_uv = R(40.0), za_tq = R(40.0);
};

// Per-tile prognostic state (persists from step to step).
template <class R, class R2>
struct State {
  R2 wb[MS], wbice[MS], gammzz[MS];
  R tgg[MS], tggsn[MSN], ssdn[MSN], smass[MSN], sdepth[MSN];
  int isflag = 0;
  R snowd, osnowd, ssdnn, snage, pudsto, pudsmx, owetfac, rtsoil, tss, wb_lake, wbtot1, wbtot2;
  R cansto;
  R ga = 0;                        // canopy%ga of the last step (read by ssnow_potev='P-M')
  R cplant[3], csoil[2];
  // balances (cable_checks.F90 mass_balance SAVE owb; energy/water totals)
  R2 owb, ebal_tot, wbal_tot;
  bool first_soilsnow_call = true;  // soil_snow SAVE ktau (cbl_soilsnow_main.F90:60-62)
  R vlaiw = 0;                      // canopy%vlaiw carried between coupled calls
};

// Per-step forcing (met_type fields set by the driver, cable_input.F90).
template <class R>
struct Forcing {
  R fsd[2], fld, precip, precip_sn, tk, pmb, ua, qv, ca, coszen, doy, hod;
};

// Per-step diagnostics written by one cbm() call.
template <class R, class R2>
struct Diag {
  R fe, fh, fev, fhv, fhs, fns, fnv, ga, tv, tscrn, qscrn, rnet, us, cduv, cdtq, epot;
  R2 fes, fevc, dgdtg;
  R fevw, fpn, frday, fgpp, fnpp, fnee, fra, frp, frs, trad, albedo[2], transd;
  R precis, through, fwet, wetfac, potev, runoff, rnof1, rnof2, smelt, ghflux, sghflux;
  R drybal, wetbal, ebal, wbal, qssabs, rniso, vlaiw, tvair, qvair, swnet, lwnet;
  R2 wbtot;
  R gswx[2], fwsoil;
  int dryleaf_passes;            // total dryLeaf passes over the 4 MO iterations
  int dryleaf_noconv;            // MO iterations whose dryLeaf loop ended unconverged at the pass limit
  int evapfbl_err;               // MO iterations with the reference's 'oldevapfbl not right' message
  // read by the offline driver after cbm(): canopy%delwc (mass_balance,
  // cable_checks.F90:472-551), ssnow%cls (the balances), canopy%frpw and
  // frpr (sumcflux)
  R delwc, cls, frpw, frpr;
};

// ==========================================================================
template <class R, class R2>
struct CbmRef {
  using P = Params<R, R2>;
  using S = State<R, R2>;
  using F = Forcing<R>;
  using D = Diag<R, R2>;
  bool medlyn = false;             // gs_switch; 'leuning' per cable.nml:62
  bool soil_thermal_fix = false;   // cable_user%soil_thermal_fix (cable_runtime_opts_mod.F90:31)
  bool litter = false;             // cable_user%litter: litter resistances in define_canopy
  bool l_rev_corr = false;         // cable_user%l_rev_corr (cable_runtime_opts_mod.F90:28)
  int fwsoil_mode = 0;             // fwsoil_switch: 0 'standard', 1 'non-linear extrapolation',
                                   // 2 'Lai and Ktaul 2000' (cbl_dryLeaf.F90:170-181)
  bool potev_pm = false;           // ssnow_potev = 'P-M' (cable_canopy.F90:480, :553)
  bool new_reduce_soilevp = false; // cable_user%l_new_reduce_soilevp (cbl_latent_heat.F90:205-210)
  bool new_runoff_speed = false;   // cable_user%l_new_runoff_speed (cbl_smoisturev.F90:112, :153)
  bool diag_soil_resp_off = false; // diag_soil_resp = 'OFF' (cable_carbon.F90:256-276)
  // litter conductivity / vapour diffusivity (cable_canopy.F90:203-204)
  static constexpr double KTH_LITT = 0.3, DV_LITT = 3.1415841138194147e-05;

  // ---- met / air working copies (met_type, air_type)
  struct Met { R fsd[3], fld, precip, precip_sn, tk, tvair, tvrad, pmb, ua, qv, qvair, dva, ca, coszen, doy; };
  struct Air { R rho, volm, rlam, qsat, epsi, visc, psyc, dsatdk, cmolar; };
  struct Rough {
    R disp, hruff, rt0us, rt1usa, rt1usb, rt1, z0m, zref_uv, zref_tq, zruffs, z0soilsn, z0soil;
    R coexp, usuh, term2, term3, term5, term6, term6a;
  };
  struct Rad {
    R transb, extkb, extkd, flws, qssabs, transd, lwabv, swnet, lwnet;
    R fvlai[2], rhocdf[3], rniso[2], scalex[2], albedo[3], reffdf[3], reffbm[3];
    R extkbm[3], extkdm[3], fbeam[3], cexpkbm[3], cexpkdm[3], rhocbm[3], gradis[2];
    R qcan[2][3];
  };

  // ------------------------------------------------------------------ qsat
  // cbl_qsat.F90:46-50 (qsatfjh), tair in deg C
  static R qsatfjh(R tair, R pmb) {
    return (R(RMH2O) / R(RMAIR)) * (R(TETENA) * std::exp(R(TETENB) * tair / (R(TETENC) + tair))) / pmb;
  }

  // ------------------------------------------------------- stability funcs
  // cbl_friction_vel.F90:112-166
  static R psim(R zeta) {
    const R gu = R(16.0), a = R(1.0), b = R(0.667), xc = R(5.0), d = R(0.35);
    R z = R(0.5) + fsign(R(0.5), zeta);
    R stable = -a * zeta - b * (zeta - xc / d) * std::exp(-d * zeta) - b * xc / d;
    R x = std::pow(R(1.0) + gu * std::fabs(zeta), R(0.25));
    R unstable = std::log((R(1.0) + x * x) * sq(R(1.0) + x) / R(8)) - R(2.0) * std::atan(x) + R(PI_C) * R(0.5);
    return z * stable + (R(1.0) - z) * unstable;
  }
  // cbl_friction_vel.F90:168-221
  static R psis(R zeta) {
    const R gu = R(16.0), a = R(1.0), b = R(0.667), c = R(5.0), d = R(0.35);
    R z = R(0.5) + fsign(R(0.5), zeta);
    R stzeta = mx(R(0.), zeta);
    R stable = -std::pow(R(1.) + R(2.) / R(3.) * a * stzeta, R(3.) / R(2.)) - b * (stzeta - c / d) * std::exp(-d * stzeta) - b * c / d + R(1.);
    R y = std::pow(R(1.0) + gu * std::fabs(zeta), R(0.5));
    R unstable = R(2.0) * std::log((R(1) + y) * R(0.5));
    return z * stable + (R(1.0) - z) * unstable;
  }

  // ------------------------------------------------------------ define_air
  // cable_air.F90:51-97
  static void define_air(const Met& met, Air& air) {
    R tc = met.tvair - R(TFRZ);
    R es = R(TETENA) * std::exp(R(TETENB) * tc / (R(TETENC) + tc));
    air.cmolar = met.pmb * R(100.0) / (R(RGAS) * met.tvair);
    air.rho = mn(R(1.3), R(RMAIR) * air.cmolar);
    air.volm = R(RGAS) * met.tvair / (R(100.0) * met.pmb);
    air.rlam = R(HL);
    air.qsat = (R(RMH2O) / R(RMAIR)) * es / met.pmb;
    air.epsi = (air.rlam / R(CAPP)) * (R(RMH2O) / R(RMAIR)) * es * R(TETENB) * R(TETENC) / sq(R(TETENC) + tc) / met.pmb;
    air.visc = R(1e-5) * mx(R(1.0), R(1.35) + R(0.0092) * tc);
    air.psyc = met.pmb * R(100.0) * R(CAPP) * R(RMAIR) / air.rlam / R(RMH2O);
    air.dsatdk = R(100.0) * (R(TETENA) * R(TETENB) * R(TETENC)) / sq(tc + R(TETENC)) * std::exp(R(TETENB) * tc / (tc + R(TETENC)));
  }

  // ------------------------------------------------------------ ruff_resist
  // cable_roughness.F90:64-332 (+ roughnessHGT_effLAI_cbl.F90:42-149)
  // vlaiw_in: the coupled calls' carried canopy%vlaiw, which ruff_resist
  // then leaves alone (cable_roughness.F90:176-186), or null
  static void ruff_resist(const P& p, const S& s, Rough& r, R& vlaiw, R& rghlai, const R* vlaiw_in = nullptr) {
    const R z0soilsn_min = R(1.e-7), z0soilsn_min_PF = R(1.e-4);
    // HgtAboveSnow (roughnessHGT_effLAI_cbl.F90:71-95)
    R snowden_eff = mx(R(100.0), s.ssdnn);
    R hmin = R(10.0) * z0soilsn_min;
    R hcomp = p.hc - (R(1.2) * s.snowd / snowden_eff);
    R has = mx(hmin, hcomp);
    r.hruff = has;
    // LAI_eff (:123-126)
    vlaiw = p.vlai * (has / mx(R(0.01), p.hc));
    if (vlaiw_in) vlaiw = *vlaiw_in;
    rghlai = vlaiw;
    // :193-205
    r.z0soil = R(0.0009) * mn(R(1.0), vlaiw) + R(1.e-4);
    r.z0soilsn = r.z0soil;
    if (s.snowd > R(0.01)) r.z0soilsn = mx(z0soilsn_min, r.z0soil - r.z0soil * mn(s.snowd, R(10.)) / R(10.));
    if (s.snowd > R(0.01) && p.iveg == ICE_SURF) r.z0soilsn = mx(r.z0soilsn, z0soilsn_min_PF);
    // :220-317
    if (vlaiw <= R(LAI_THRESH) || r.hruff < r.z0soilsn) {
      r.z0m = r.z0soilsn;
      r.rt0us = 0; r.disp = 0;
      r.zref_uv = mx(R(3.5) + r.z0m, p.za_uv);
      r.zref_tq = mx(R(3.5) + r.z0m, p.za_tq);
      r.zref_uv = mx(r.zref_uv, r.hruff - r.disp);
      r.zref_tq = mx(r.zref_tq, r.hruff - r.disp);
      r.zruffs = 0; r.rt1usa = 0; r.rt1usb = 0;
      r.usuh = mn(std::sqrt(R(CSD) + R(CRD) * (vlaiw * R(0.5))), R(USUHM));
      R xx = std::sqrt(R(CCD) * mx(vlaiw * R(0.5), R(0.0005)));
      R dh = R(1.0) - (R(1.0) - std::exp(-xx)) / xx;
      r.coexp = r.usuh / (R(VONK) * R(CCW_C) * (R(1.0) - dh));
    } else {
      r.usuh = mn(std::sqrt(R(CSD) + R(CRD) * (rghlai * R(0.5))), R(USUHM));
      R xx = std::sqrt(R(CCD) * mx(rghlai * R(0.5), R(0.0005)));
      R dh = R(1.0) - (R(1.0) - std::exp(-xx)) / xx;
      r.disp = dh * r.hruff;
      r.z0m = ((R(1.0) - dh) * std::exp(std::log(R(CCW_C)) - R(1.) + R(1.) / R(CCW_C) - R(VONK) / r.usuh)) * r.hruff;
      r.zref_uv = mx(R(3.5) + r.z0m, p.za_uv);
      r.zref_tq = mx(R(3.5) + r.z0m, p.za_tq);
      r.zref_uv = mx(r.zref_uv, r.hruff - r.disp);
      r.zref_tq = mx(r.zref_tq, r.hruff - r.disp);
      r.coexp = r.usuh / (R(VONK) * R(CCW_C) * (R(1.0) - dh));
      r.term2 = std::exp(R(2) * R(CSW) * rghlai * (R(1) - r.disp / r.hruff));
      r.term3 = R(A33) * R(A33) * R(CTL) * R(2) * R(CSW) * rghlai;
      r.term5 = mx((R(2.) / R(3.)) * r.hruff / r.disp, R(1.0));
      r.term6 = std::exp(R(3.) * r.coexp * (r.disp / r.hruff - R(1.)));
      r.term6a = std::exp(r.coexp * (R(0.1) * r.hruff / r.hruff - R(1.)));
      r.rt0us = r.term5 * (R(ZDLIN) * std::log(R(ZDLIN) * r.disp / r.z0soilsn) + (R(1) - R(ZDLIN))) *
                (std::exp(R(2) * R(CSW) * rghlai) - r.term2) / r.term3;
      r.zruffs = r.disp + r.hruff * R(A33) * R(A33) * R(CTL) / R(VONK) / r.term5;
      r.rt1usa = r.term5 * (r.term2 - R(1.0)) / r.term3;
      r.rt1usb = r.term5 * (mn(r.zref_tq + r.disp, r.zruffs) - r.hruff) / (R(A33) * R(A33) * R(CTL) * r.hruff);
      r.rt1usb = mx(r.rt1usb, R(0.0));
    }
  }

  // ------------------------------------------------------------ spitter
  // cbl_spitter.F90:36-76
  static R spitter(int doy, R coszen, R fsd) {
    const R solcon = R(1370.0);
    R fbeam = 0;
    R tmpr = R(0.847) + coszen * (R(1.04) * coszen - R(1.61));
    R tmpk = (R(1.47) - tmpr) / R(1.66);
    R tmprat;
    if (coszen > R(1.0e-10) && fsd > R(10.0))
      tmprat = fsd / (solcon * (R(1.0) + R(0.033) * std::cos(R(2.0) * R(PI_C) * (R(doy) - R(10.0)) / R(365.0))) * coszen);
    else
      tmprat = 0;
    if (tmprat > R(0.22)) fbeam = R(6.4) * sq(tmprat - R(0.22));
    if (tmprat > R(0.35)) fbeam = mn(R(1.66) * tmprat - R(0.4728), R(1.0));
    if (tmprat > tmpk) fbeam = mx(R(1.0) - tmpr, R(0.0));
    return fbeam;
  }

  // --------------------------------------------- init_radiation + albedo
  // cbl_init_radiation.F90:30-392, cbl_rhoch.F90:38-62,
  // cbl_albedo.F90:56-386, cbl_snow_albedo.F90:36-161
  static void init_radiation_albedo(const P& p, const S& s, const Met& met, R vlaiw, bool veg_mask,
                                    Rad& rad, R albsoilsn[3], R c1[3], R rhoch[3], R xk[3]) {
    for (int b = 0; b < 3; ++b) { c1[b] = 0; rhoch[b] = 0; xk[b] = 0; rad.extkbm[b] = 0; rad.extkdm[b] = 0; }
    rad.extkb = 0; rad.extkd = 0;
    // Common_InitRad_Scalings (:132-218)
    R cos3[3];
    const R angles[3] = {R(15.0), R(45.0), R(75.0)};
    for (int b = 0; b < 3; ++b) cos3[b] = std::cos(R(PI180) * angles[b]);
    R xphi1 = 0, xphi2 = 0;
    if (veg_mask) {
      xphi1 = R(0.5) - p.xfang * (R(0.633) + R(0.33) * p.xfang);
      xphi2 = R(0.877) * (R(1.0) - R(2.0) * xphi1);
    }
    for (int b = 0; b < 3; ++b) xk[b] = (vlaiw > R(LAI_THRESH)) ? xphi1 / cos3[b] + xphi2 : R(0.0);
    // calc_rhoch
    c1[0] = std::sqrt(R(1.0) - p.taul[0] - p.refl[0]);
    c1[1] = std::sqrt(R(1.0) - p.taul[1] - p.refl[1]);
    c1[2] = R(1.0);
    for (int b = 0; b < 3; ++b) rhoch[b] = (R(1.0) - c1[b]) / (R(1.0) + c1[b]);
    const R cz_huge = R(COSZEN_TOLS) * R(1e2), cz_tiny = R(COSZEN_TOLS) * R(1e-2);
    // ExtinctionCoeff (:222-283)
    rad.extkb = R(0.5);
    rad.extkd = R(0.7);
    if (veg_mask) {
      R sum = 0;
      for (int b = 0; b < 3; ++b) sum += R(GAUSS_W[b]) * std::exp(-xk[b] * vlaiw);
      rad.extkd = -std::log(sum) / vlaiw;
    }
    if (veg_mask && met.coszen > cz_tiny) rad.extkb = xphi1 / met.coszen + xphi2;
    if (met.coszen < cz_tiny) rad.extkb = R(1.0e5);
    if (std::fabs(rad.extkb - rad.extkd) < R(0.001)) rad.extkb = rad.extkd + R(0.001);
    // EffectiveExtinctCoeffs (:287-354)
    for (int b = 0; b < 2; ++b) {
      if (veg_mask) rad.extkbm[b] = rad.extkb * c1[b];
      rad.extkdm[b] = rad.extkd * c1[b];
    }
    // BeamFraction (:358-392)
    rad.fbeam[0] = spitter((int)met.doy, met.coszen, met.fsd[0] + met.fsd[1]);
    rad.fbeam[1] = rad.fbeam[0];
    rad.fbeam[2] = 0;
    if (met.coszen < cz_huge) { rad.fbeam[0] = 0; rad.fbeam[1] = 0; }

    // ---- albedo: surface_albedosn (cbl_snow_albedo.F90:85-157)
    const R alvo = R(0.95), aliro = R(0.70);
    R soilalb = p.albsoil[0];
    if (p.iveg == LAKES) soilalb = R(-0.022) * (mn(R(275.0), mx(R(260.0), s.tgg[0])) - R(260.0)) + R(0.45);
    if (s.snowd > R(SNOW_DEPTH_THRESH) && p.iveg == LAKES) soilalb = R(0.85);
    R sfact = R(0.68);
    if (soilalb <= R(0.14)) sfact = R(0.5);
    else if (soilalb > R(0.14) && soilalb <= R(0.20)) sfact = R(0.62);
    albsoilsn[1] = R(2.0) * soilalb / (R(1.0) + sfact);
    albsoilsn[0] = sfact * albsoilsn[1];
    albsoilsn[2] = 0;
    R snrat = 0, alir = 0, alv = 0;
    if (s.snowd > R(SNOW_DEPTH_THRESH)) {
      R tmp = s.snowd / mx(s.ssdnn, R(200.0));
      snrat = mn(R(1.0), tmp / (tmp + R(0.1)));
      R fage = R(1.0) - R(1.0) / (R(1.0) + s.snage);
      tmp = mx(R(0.17365), met.coszen);
      R fzenm = mx(R(0.0), (tmp > R(0.5)) ? R(0.0) : R(1.5) / (R(1.0) + R(4.0) * tmp) - R(0.5));
      tmp = alvo * (R(1.0) - R(0.2) * fage);
      alv = R(0.4) * fzenm * (R(1.0) - tmp) + tmp;
      tmp = aliro * (R(1.0) - R(0.5) * fage);
      alir = R(0.4) * fzenm * (R(1.0) - tmp) + tmp;
    }
    albsoilsn[1] = mn(aliro, (R(1.0) - snrat) * albsoilsn[1] + snrat * alir);
    albsoilsn[0] = mn(alvo, (R(1.0) - snrat) * albsoilsn[0] + snrat * alv);
    if (p.isoilm == ICE_SOIL) { albsoilsn[0] = alvo - R(0.05); albsoilsn[1] = aliro - R(0.05); }
    // CanopyReflectance (cbl_albedo.F90:196-240)
    for (int b = 0; b < 3; ++b) { rad.rhocbm[b] = 0; rad.rhocdf[b] = 0; }
    for (int b = 0; b < 2; ++b) {
      if (veg_mask) rad.rhocbm[b] = R(2.0) * rad.extkb / (rad.extkb + rad.extkd) * rhoch[b];
      rad.rhocdf[b] = rhoch[b] * R(2.0) *
          (R(GAUSS_W[0]) * xk[0] / (xk[0] + rad.extkd) + R(GAUSS_W[1]) * xk[1] / (xk[1] + rad.extkd) +
           R(GAUSS_W[2]) * xk[2] / (xk[2] + rad.extkd));
    }
    // CanopyTransmitance (:244-283); non-vegetated beam values are never read
    for (int b = 0; b < 3; ++b) { rad.cexpkbm[b] = 0; rad.cexpkdm[b] = 0; }
    for (int b = 0; b < 2; ++b) {
      if (veg_mask) rad.cexpkbm[b] = std::exp(R(-1.0) * mn(rad.extkbm[b] * vlaiw, R(20.0)));
      rad.cexpkdm[b] = std::exp(R(-1.0) * (rad.extkdm[b] * vlaiw));
    }
    // EffectiveSurfaceReflectance (:287-350)
    for (int b = 0; b < 3; ++b) { rad.reffbm[b] = albsoilsn[b]; rad.reffdf[b] = albsoilsn[b]; }
    for (int b = 0; b < 2; ++b) {
      if (veg_mask) {
        rad.reffdf[b] = rad.rhocdf[b] + (albsoilsn[b] - rad.rhocdf[b]) * sq(rad.cexpkdm[b]);
        rad.reffbm[b] = rad.rhocbm[b] + (albsoilsn[b] - rad.rhocbm[b]) * sq(rad.cexpkbm[b]);
      }
    }
    // FbeamRadAlbedo (:354-386)
    for (int b = 0; b < 3; ++b) rad.albedo[b] = albsoilsn[b];
    for (int b = 0; b < 2; ++b)
      if (veg_mask) rad.albedo[b] = (R(1.0) - rad.fbeam[b]) * rad.reffdf[b] + rad.fbeam[b] * rad.reffbm[b];
  }

  // ------------------------------------------------------------ radiation
  // cbl_radiation.F90:30-218
  static void radiation(const P& p, const Met& met, const Air& air, R vlaiw, R tss, bool sunlit_veg,
                        const R albsoilsn[3], Rad& rad) {
    R cf2n = std::exp(-p.extkn * vlaiw);
    rad.transd = R(1.0);
    if (vlaiw > R(LAI_THRESH)) rad.transd = std::exp(-rad.extkd * vlaiw);
    R dummy2 = mn(rad.extkb * vlaiw, R(30.));
    rad.transb = std::exp(-dummy2);
    R flpwb = R(SBOLTZ) * std::pow(met.tvrad, 4);
    R flwv = R(EMLEAF) * flpwb;
    rad.flws = R(SBOLTZ) * R(EMSOIL) * std::pow(tss, 4);
    R emair = met.fld / flpwb;
    rad.gradis[0] = rad.gradis[1] = 0;
    for (int l = 0; l < 2; ++l) for (int b = 0; b < 3; ++b) rad.qcan[l][b] = 0;
    if (vlaiw > R(LAI_THRESH)) {
      rad.gradis[0] = (R(4.0) * R(EMLEAF) / (R(CAPP) * air.rho)) * flpwb / met.tvrad * rad.extkd *
                      ((R(1.0) - rad.transb * rad.transd) / (rad.extkb + rad.extkd) +
                       (rad.transd - rad.transb) / (rad.extkb - rad.extkd));
      rad.gradis[1] = (R(8.0) * R(EMLEAF) / (R(CAPP) * air.rho)) * flpwb / met.tvrad * rad.extkd *
                      (R(1.0) - rad.transd) / rad.extkd - rad.gradis[0];
      rad.qcan[0][2] = (rad.flws - flwv) * rad.extkd * (rad.transd - rad.transb) / (rad.extkb - rad.extkd) +
                       (emair - R(EMLEAF)) * rad.extkd * flpwb * (R(1.0) - rad.transd * rad.transb) / (rad.extkb + rad.extkd);
      rad.qcan[1][2] = (R(1.0) - rad.transd) * (rad.flws + met.fld - R(2.0) * flwv) - rad.qcan[0][2];
    }
    for (int l = 0; l < 2; ++l) {
      rad.gradis[l] = air.cmolar * rad.gradis[l];
      rad.gradis[l] = R(mx(R2(1.0e-3), R2(rad.gradis[l])));
    }
    for (int b = 0; b < 2; ++b) {
      if (sunlit_veg) {
        R cf1 = (R(1.0) - rad.transb * rad.cexpkdm[b]) / (rad.extkb + rad.extkdm[b]);
        R cf3 = (R(1.0) - rad.transb * rad.cexpkbm[b]) / (rad.extkb + rad.extkbm[b]);
        R direct = rad.fbeam[b] * (R(1.0) - p.taul[b] - p.refl[b]) * rad.extkb *
                   ((R(1) - rad.transb) / rad.extkb - (R(1) - sq(rad.transb)) / (rad.extkb + rad.extkb));
        rad.qcan[0][b] = met.fsd[b] * ((R(1.0) - rad.fbeam[b]) * (R(1.0) - rad.reffdf[b]) * rad.extkdm[b] * cf1 +
                                      rad.fbeam[b] * (R(1.0) - rad.reffbm[b]) * rad.extkbm[b] * cf3 + direct);
        rad.qcan[1][b] = met.fsd[b] * ((R(1.0) - rad.fbeam[b]) * (R(1.0) - rad.reffdf[b]) * rad.extkdm[b] *
                                          ((R(1.0) - rad.cexpkdm[b]) / rad.extkdm[b] - cf1) +
                                      rad.fbeam[b] * (R(1.) - rad.reffbm[b]) * rad.extkbm[b] *
                                          ((R(1.0) - rad.cexpkbm[b]) / rad.extkbm[b] - cf3) - direct);
      }
    }
    rad.qssabs = 0;
    if (sunlit_veg) {
      rad.qssabs = met.fsd[0] * (rad.fbeam[0] * (R(1.) - rad.reffbm[0]) * std::exp(-mn(rad.extkbm[0] * vlaiw, R(20.))) +
                                 (R(1.) - rad.fbeam[0]) * (R(1.) - rad.reffdf[0]) * std::exp(-mn(rad.extkdm[0] * vlaiw, R(20.)))) +
                   met.fsd[1] * (rad.fbeam[1] * (R(1.) - rad.reffbm[1]) * rad.cexpkbm[1] +
                                 (R(1.) - rad.fbeam[1]) * (R(1.) - rad.reffdf[1]) * rad.cexpkdm[1]);
      rad.scalex[0] = (R(1.0) - rad.transb * cf2n) / (rad.extkb + p.extkn);
      rad.fvlai[0] = (R(1.0) - rad.transb) / rad.extkb;
      rad.fvlai[1] = vlaiw - rad.fvlai[0];
    } else {
      rad.qssabs = (R(1.0) - albsoilsn[0]) * met.fsd[0] + (R(1.0) - albsoilsn[1]) * met.fsd[1];
      rad.scalex[0] = 0;
      rad.fvlai[0] = 0;
      rad.fvlai[1] = vlaiw;
    }
    rad.scalex[1] = (R(1.0) - cf2n) / p.extkn - rad.scalex[0];
    for (int l = 0; l < 2; ++l) rad.rniso[l] = rad.qcan[l][0] + rad.qcan[l][1] + rad.qcan[l][2];
  }

  // ----------------------------------------------- dryLeaf helper functions
  // cbl_dryLeaf.F90:779-877
  static R ej3x(R parx, R alpha, R convex, R x) {
    return mx(R(0.0), R(0.25) * ((alpha * parx + x - std::sqrt(sq(alpha * parx + x) - R(4.0) * convex * alpha * parx * x)) /
                                 (R(2.0) * convex)));
  }
  static R ej4x(R parx, R alpha, R convex, R x) {
    return mx(R(0.0), (alpha * parx + x - std::sqrt(sq(alpha * parx + x) - R(4.0) * convex * alpha * parx * x)) /
                          (R(2.0) * convex));
  }
  static R xvcmxt4(R x) {
    const R q10c4 = R(2.0);
    return std::pow(q10c4, R(0.1) * x - R(2.5)) /
           ((R(1.0) + std::exp(R(0.3) * (R(13.0) - x))) * (R(1.0) + std::exp(R(0.3) * (x - R(36.0)))));
  }
  static R xvcmxt3(R x) {
    const R EHaVc = R(73637.0), EHdVc = R(149252.0), EntropVc = R(486.0), xVccoef = R(1.17461);
    R xvcnum = xVccoef * std::exp((EHaVc / (R(RGAS) * R(TREFK))) * (R(1.) - R(TREFK) / x));
    R xvcden = R(1.0) + std::exp((EntropVc * x - EHdVc) / (R(RGAS) * x));
    return mx(R(0.0), xvcnum / xvcden);
  }
  static R xejmxt3(R x) {
    const R EHaJx = R(50300.0), EHdJx = R(152044.0), EntropJx = R(495.0), xjxcoef = R(1.16715);
    R xjxnum = xjxcoef * std::exp((EHaJx / (R(RGAS) * R(TREFK))) * (R(1.) - R(TREFK) / x));
    R xjxden = R(1.0) + std::exp((EntropJx * x - EHdJx) / (R(RGAS) * x));
    return mx(R(0.0), xjxnum / xjxden);
  }

  // ------------------------------------------------------ transp_soil_water
  // cbl_remove_trans.F90:43-93
  static void transp_soil_water(R dels, const P& p, R2 fevc, const R2 wbliq[MS], R2 evapfbl[MS]) {
    R2 xx = 0, xxd = 0, diff_prev = 0;
    if (fevc > 0.0) {
      for (int k = 0; k < MS; ++k) {
        xx = fevc * dels / R(HL) * p.froot[k] + diff_prev;
        R2 diffk = mx(R2(0.0), wbliq[k] - R(1.1) * p.swilt_vec[k]) * p.zse_vec[k] * R(DENSITY_LIQ);
        xxd = xx - diffk;
        if (xxd > 0.0) { evapfbl[k] = diffk; diff_prev = xxd; }
        else { evapfbl[k] = xx; diff_prev = 0.0; }
      }
    }
  }

  // ---------------------------------------------------------- photosynthesis
  // cbl_photosynthesis.F90:10-226 (one leaf; the caller applies the masks)
  static R photosynthesis_leaf(R2 csx, R cx1, R cx2, R gswmin, R rdx, R vcmxt3, R vcmxt4, R vx3, R vx4,
                               R gs_coeff, R fwsoil) {
    const R effc4 = R(4000.0);
    R2 anrubisco = 0, anrubp = 0, ansink = 0, ci, coef0, coef1, coef2, delcx;
    // Rubisco limited
    coef2 = gswmin * fwsoil / R(RGSWC) + gs_coeff * (vcmxt3 - (rdx - vcmxt4));
    coef1 = (R(1.0) - csx * gs_coeff) * (vcmxt3 + vcmxt4 - rdx) + (gswmin * fwsoil / R(RGSWC)) * (cx1 - csx) -
            gs_coeff * (vcmxt3 * cx2 / R(2.0) + cx1 * (rdx - vcmxt4));
    coef0 = -(R(1.0) - csx * gs_coeff) * (vcmxt3 * cx2 / R(2.0) + cx1 * (rdx - vcmxt4)) -
            (gswmin * fwsoil / R(RGSWC)) * cx1 * csx;
    if (std::fabs(coef2) > 1.0e-9 && std::fabs(coef1) < 1.0e-9) { ci = 99999.0; anrubisco = 99999.0; }
    if (std::fabs(coef2) < 1.e-9 && std::fabs(coef1) >= 1e-9) {
      ci = -1.0 * coef0 / coef1;
      ci = mx(R2(0.0), ci);
      anrubisco = vcmxt3 * (ci - cx2 / R(2.0)) / (ci + cx1) + vcmxt4 - rdx;
    }
    if (std::fabs(coef2) >= 1.e-9) {
      delcx = sq(coef1) - R(4.0) * coef0 * coef2;
      ci = (-coef1 + std::sqrt(mx(R2(0.0), delcx))) / (R(2.0) * coef2);
      ci = mx(R2(0.0), ci);
      anrubisco = vcmxt3 * (ci - cx2 / R(2.0)) / (ci + cx1) + vcmxt4 - rdx;
    }
    // RuBP limited
    coef2 = gswmin * fwsoil / R(RGSWC) + gs_coeff * (vx3 - (rdx - vx4));
    coef1 = (R(1.0) - csx * gs_coeff) * (vx3 + vx4 - rdx) + (gswmin * fwsoil / R(RGSWC)) * (cx2 - csx) -
            gs_coeff * (vx3 * cx2 / R(2.0) + cx2 * (rdx - vx4));
    coef0 = -(R(1.0) - csx * gs_coeff) * (vx3 * cx2 / R(2.0) + cx2 * (rdx - vx4)) -
            (gswmin * fwsoil / R(RGSWC)) * cx2 * csx;
    ci = 99999.0;
    anrubp = 99999.0;
    if (std::fabs(coef2) < 1.e-9 && std::fabs(coef1) >= 1.e-9) {
      ci = -1.0 * coef0 / coef1;
      ci = mx(R2(0.0), ci);
      anrubp = vx3 * (ci - cx2 / R(2.0)) / (ci + cx2) + vx4 - rdx;
    }
    if (std::fabs(coef2) >= 1.e-9) {
      delcx = sq(coef1) - R(4.0) * coef0 * coef2;
      ci = (-coef1 + std::sqrt(mx(R2(0.0), delcx))) / (R(2.0) * coef2);
      ci = mx(R2(0.0), ci);
      anrubp = vx3 * (ci - cx2 / R(2.0)) / (ci + cx2) + vx4 - rdx;
    }
    // sink limited
    coef2 = gs_coeff;
    coef1 = gswmin * fwsoil / R(RGSWC) + gs_coeff * (rdx - R(0.5) * vcmxt3) + effc4 * vcmxt4 -
            gs_coeff * csx * effc4 * vcmxt4;
    coef0 = -(gswmin * fwsoil / R(RGSWC)) * csx * effc4 * vcmxt4 + (rdx - R(0.5) * vcmxt3) * gswmin * fwsoil / R(RGSWC);
    if (std::fabs(coef2) < 1.0e-9 && std::fabs(coef1) < 1.0e-9) { ci = 99999.0; ansink = 99999.0; }
    if (std::fabs(coef2) < 1.e-9 && std::fabs(coef1) >= 1.e-9) { ci = -1.0 * coef0 / coef1; ansink = ci; }
    if (std::fabs(coef2) >= 1.e-9) {
      delcx = sq(coef1) - R(4.0) * coef0 * coef2;
      ci = (-coef1 + std::sqrt(mx(R2(0.0), delcx))) / (R(2.0) * coef2);
      ansink = ci;
    }
    return R(mn(mn(anrubisco, anrubp), ansink));
  }

  // ---------------------------------------------------------------- dryLeaf
  // cbl_dryLeaf.F90:10-666 (one tile)
  struct LeafIter {
    R dsx, fwsoil, tlfx, tlfy;
    R2 ecy, hcy, rny, ghwet;
    R2 gbhu[2], gbhf[2], csx[2];
    R gswx[2];
    R2 fevc;
    R fevw, fhvw;
    R frday, fpn;
    R2 evapfbl[MS];
    int passes;
    int noconv = 0;     // MO iterations whose dryLeaf loop hit the pass limit unconverged
    int evapfbl_err = 0;  // MO iterations where the reference prints 'oldevapfbl not right'
  };

  void dryLeaf(R dels, const P& p, const Rad& rad, const Met& met, const Air& air, R vlaiw, R cansto, R fwet,
               const R2 wbliq[MS], LeafIter& L, int iter, R sum_rad_gradis, R sum_rad_rniso) const {
    const R co2cp3 = R(0.0), jtomol = R(4.6e-6);
    R gs_coeff[2] = {0, 0};
    if (iter == 1 && fwsoil_mode == 0) {
      // fwsoil_calc_std (cbl_fwsoil.F90:13-38)
      R rwater = 0;
      for (int k = 0; k < MS; ++k)
        rwater += p.froot[k] * mx(R(1.0e-9), mn(R(1.0), R((wbliq[k] - p.swilt_vec[k]) / (p.sfc_vec[k] - p.swilt_vec[k]))));
      rwater = mx(R(1.0e-9), rwater);
      if (medlyn) L.fwsoil = mx(R(1.0e-4), mn(R(1.0), rwater));
      else L.fwsoil = mx(R(1.0e-9), mn(R(1.0), p.vbeta * rwater));
    } else if (iter == 1 && fwsoil_mode == 1) {
      // fwsoil_calc_non_linear (cbl_fwsoil.F90:44-88): the root-weighted
      // available water mapped through a quadratic through (swilt, 0),
      // (midpoint, 0.9), (sfc, 1)
      R sum = 0;
      for (int k = 0; k < MS; ++k) sum += p.froot[k] * mx(R(0.0), mn(R(1.0), R(wbliq[k] - R2(p.swilt))));
      R rwater = mx(R(1.0e-9), sum / (p.sfc - p.swilt));
      L.fwsoil = R(1.);
      rwater = p.swilt + rwater * (p.sfc - p.swilt);
      const R x1 = p.swilt, x2 = p.swilt + (p.sfc - p.swilt) / R(2.0), x3 = p.sfc;
      const R s1 = (rwater - x2) / (x1 - x2) * (rwater - x3) / (x1 - x3);
      const R s2 = (rwater - x1) / (x2 - x1) * (rwater - x3) / (x2 - x3);
      const R s3 = (rwater - x1) / (x3 - x1) * (rwater - x2) / (x3 - x2);
      if (rwater < p.sfc - R(0.02)) L.fwsoil = mx(R(0.), mn(R(1.), R(0.) * s1 + R(0.9) * s2 + R(1.0) * s3));
    } else if (iter == 1 && fwsoil_mode == 2) {
      // fwsoil_calc_Lai_Ktaul (cbl_fwsoil.F90:90-112), r_2 arithmetic.  A
      // layer drier than wilting raises a negative base to a non-integer
      // power (NaN in IEEE arithmetic) whose MAX with the 1e-4 floor is
      // compiler-dependent in the reference; here it takes the floor.
      const R2 rootgamma = R2(0.01f);
      R fw = R(0.0);
      for (int k = 0; k < MS; ++k) {
        const R2 avail = wbliq[k] - p.swilt_vec[k];
        const R dummy = R(rootgamma / mx(R2(1.0e-3), avail));
        const R2 base = avail / p.ssat_vec;
        const R2 frwater = base > R2(0.0) ? mx(R2(1.0e-4), std::pow(base, R2(dummy))) : R2(1.0e-4);
        fw = mn(R(1.0), mx(fw, R(frwater)));
      }
      L.fwsoil = fw;
    }
    const R fwsoil = L.fwsoil;
    R gswmin[2];
    for (int l = 0; l < 2; ++l) gswmin[l] = mx(R(1.e-6), rad.scalex[l] * p.gswmin);
    R gw[2] = {R(1.0e-3), R(1.0e-3)}, gh[2] = {R(1.0e-3), R(1.0e-3)}, ghr[2] = {R(1.0e-3), R(1.0e-3)};
    R rdx[2] = {0, 0}, anx[2] = {0, 0}, an_y[2] = {0, 0}, rdy[2] = {0, 0};
    R2 rnx = sum_rad_rniso, ecx = sum_rad_rniso, hcx = 0;
    R abs_deltlf = R(999.0), deltlf = 0;
    L.hcy = 0;
    R tlfxx = L.tlfx;
    R psycst[2] = {air.psyc, air.psyc};
    L.fevc = 0;
    for (int k = 0; k < MS; ++k) L.evapfbl[k] = 0;
    L.ghwet = R2(1.0e-3);
    L.fevw = 0; L.fhvw = 0;
    R sum_gbh = R(L.gbhu[0] + L.gbhf[0] + L.gbhu[1] + L.gbhf[1]);
    if (vlaiw <= R(LAI_THRESH)) {
      rnx = 0; ecx = 0; L.ecy = ecx; abs_deltlf = 0; L.rny = rnx;
    }
    R deltlfy = abs_deltlf;
    R vcmxt3[2] = {0, 0}, vcmxt4[2] = {0, 0}, ejmxt3[2] = {0, 0}, vx3[2] = {0, 0}, vx4[2] = {0, 0};
    R cx1 = 0, cx2 = 0;
    R oldevapfbl[MS];
    int k = 0;
    L.passes = 0;
    while (k < MAXITER) {
      k = k + 1;
      const bool active = vlaiw > R(LAI_THRESH) && abs_deltlf > R(0.1);
      if (active) {
        L.passes++;
        L.ghwet = R(2.0) * sum_gbh;
        R gras = mx(R(1.0e-6), R(1.595E8) * std::fabs(L.tlfx - met.tvair) * std::pow(p.dleaf, R(3.0)));
        for (int l = 0; l < 2; ++l) {
          L.gbhf[l] = rad.fvlai[l] * air.cmolar * R(0.5) * R(DHEAT) * std::pow(gras, R(0.25)) / p.dleaf;
          L.gbhf[l] = mx(R2(1.e-6), L.gbhf[l]);
          gh[l] = R(2.0 * (L.gbhu[l] + L.gbhf[l]));
          ghr[l] = rad.gradis[l] + gh[l];
        }
        R temp = xvcmxt3(L.tlfx) * p.vcmax * (R(1.0) - p.frac4);
        vcmxt3[0] = rad.scalex[0] * temp; vcmxt3[1] = rad.scalex[1] * temp;
        temp = xvcmxt4(L.tlfx - R(TFRZ)) * p.vcmax * p.frac4;
        vcmxt4[0] = rad.scalex[0] * temp; vcmxt4[1] = rad.scalex[1] * temp;
        temp = xejmxt3(L.tlfx) * p.ejmax * (R(1.0) - p.frac4);
        ejmxt3[0] = rad.scalex[0] * temp; ejmxt3[1] = rad.scalex[1] * temp;
        R tdiff = L.tlfx - R(TREFK);
        R conkct = p.conkc0 * std::exp((p.ekc / (R(RGAS) * R(TREFK))) * (R(1.0) - R(TREFK) / L.tlfx));
        R conkot = p.conko0 * std::exp((p.eko / (R(RGAS) * R(TREFK))) * (R(1.0) - R(TREFK) / L.tlfx));
        tlfxx = L.tlfx;
        cx1 = conkct * (R(1.0) + R(0.21) / conkot);
        cx2 = R(2.0) * R(GAM0) * (R(1.0) + R(GAM1) * tdiff + R(GAM2) * tdiff * tdiff);
        for (int l = 0; l < 2; ++l) {
          R t2 = rad.qcan[l][0] * jtomol * (R(1.0) - p.frac4);
          vx3[l] = ej3x(t2, p.alpha, p.convex, ejmxt3[l]);
          t2 = rad.qcan[l][0] * jtomol * p.frac4;
          vx4[l] = ej4x(t2, p.alpha, p.convex, vcmxt4[l]);
          rdx[l] = (p.cfrd * vcmxt3[l] + p.cfrd * vcmxt4[l]);
        }
        if (!medlyn) {
          for (int l = 0; l < 2; ++l)
            gs_coeff[l] = R((fwsoil / (L.csx[l] - co2cp3)) * (p.a1gs / (R(1.0) + L.dsx / p.d0gs)));
        } else {
          for (int l = 0; l < 2; ++l) gswmin[l] = p.g0;
          R vpd = (L.dsx < R(50.0)) ? R(0.05) : L.dsx * R(1E-03);
          R g1 = p.g1;
          for (int l = 0; l < 2; ++l) gs_coeff[l] = R((R(1.0) + (g1 * fwsoil) / std::sqrt(vpd)) / L.csx[l]);
          const R medlyn_lim = R(0.05);
          if (fwsoil <= medlyn_lim)
            for (int l = 0; l < 2; ++l)
              gs_coeff[l] = R((fwsoil / medlyn_lim + (g1 * fwsoil) / std::sqrt(vpd)) / L.csx[l]);
        }
      }
      // photosynthesis: anx zeroed for every tile, computed under the masks
      anx[0] = anx[1] = 0;
      if (rad.fvlai[0] + rad.fvlai[1] > R(LAI_THRESH)) {
        for (int l = 0; l < 2; ++l)
          if (rad.fvlai[l] > R(LAI_THRESH) && abs_deltlf > R(0.1))
            anx[l] = photosynthesis_leaf(L.csx[l], cx1, cx2, gswmin[l], rdx[l], vcmxt3[l], vcmxt4[l], vx3[l], vx4[l],
                                         gs_coeff[l], fwsoil);
      }
      if (active) {
        for (int l = 0; l < 2; ++l) {
          if (rad.fvlai[l] > R(LAI_THRESH)) {
            L.csx[l] = met.ca - R(RGBWC) * anx[l] / (L.gbhu[l] + L.gbhf[l]);
            L.csx[l] = mx(R2(1.0e-4), L.csx[l]);
            L.gswx[l] = mx(R(1.e-3), gswmin[l] * fwsoil + mx(R(0.0), R(RGSWC) * gs_coeff[l] * anx[l]));
            gw[l] = R(R(1.0) / (R(1.0) / L.gswx[l] + R(1.0) / (R(1.075) * (L.gbhu[l] + L.gbhf[l]))));
            gw[l] = mx(gw[l], R(0.00001));
            psycst[l] = air.psyc * R(ghr[l] / gw[l]);
          }
        }
        ecx = (air.dsatdk * (rad.rniso[0] - R(CAPP) * R(RMAIR) * (met.tvair - met.tk) * rad.gradis[0]) +
               R(CAPP) * R(RMAIR) * met.dva * ghr[0]) / (air.dsatdk + psycst[0]) +
              (air.dsatdk * (rad.rniso[1] - R(CAPP) * R(RMAIR) * (met.tvair - met.tk) * rad.gradis[1]) +
               R(CAPP) * R(RMAIR) * met.dva * ghr[1]) / (air.dsatdk + psycst[1]);
        R2 local_fevc = (R(1.0) - fwet) * R(ecx);
        if (local_fevc > 0.0) {
          transp_soil_water(dels, p, local_fevc, wbliq, L.evapfbl);
          R2 se = 0;
          for (int kk = 0; kk < MS; ++kk) se += L.evapfbl[kk];
          L.fevc = se * air.rlam / dels;
          ecx = L.fevc / (R(1.0) - fwet);
        }
        hcx = (sum_rad_rniso - ecx - R(CAPP) * R(RMAIR) * (met.tvair - met.tk) * sum_rad_gradis) *
              (gh[0] + gh[1]) / (ghr[0] + ghr[1]);
        L.tlfx = met.tvair + R(hcx) / (R(CAPP) * R(RMAIR) * (gh[0] + gh[1]));
        rnx = sum_rad_rniso - R(CAPP) * R(RMAIR) * (L.tlfx - met.tk) * sum_rad_gradis;
        L.dsx = met.dva + air.dsatdk * (L.tlfx - met.tvair);
        L.dsx = mx(L.dsx, R(0.0));
        deltlf = tlfxx - L.tlfx;
        abs_deltlf = std::fabs(deltlf);
      }
      // keep the best iterate (:565-582)
      if (abs_deltlf < std::fabs(deltlfy)) {
        deltlfy = deltlf;
        L.tlfy = L.tlfx; L.rny = rnx; L.hcy = hcx; L.ecy = ecx;
        rdy[0] = rdx[0]; rdy[1] = rdx[1]; an_y[0] = anx[0]; an_y[1] = anx[1];
        for (int kk = 0; kk < MS; ++kk) oldevapfbl[kk] = R(L.evapfbl[kk]);
      }
      // damping once k > 5 (:584-590); MAX(0,k-5) is integer, k-4.9999 real
      if (abs_deltlf > R(0.1)) {
        R fac = R(0.5) * (R(std::max(0, k - 5)) / (R(k) - R(4.9999)));
        L.tlfx = fac * tlfxx + (R(1.0) - fac) * L.tlfx;
      }
      if (k == 1) {
        L.tlfy = L.tlfx; L.rny = rnx; L.hcy = hcx; L.ecy = ecx;
        rdy[0] = rdx[0]; rdy[1] = rdx[1]; an_y[0] = anx[0]; an_y[1] = anx[1];
        for (int kk = 0; kk < MS; ++kk) oldevapfbl[kk] = R(L.evapfbl[kk]);
      }
      // Once a tile stops iterating nothing above changes again (converged
      // tiles are exact no-ops), so leaving the loop early is exact.
      if (!(vlaiw > R(LAI_THRESH) && abs_deltlf > R(0.1))) break;
    }
    if (vlaiw > R(LAI_THRESH) && abs_deltlf > R(0.1)) L.noconv++;
    L.fevc = (R(1.0) - fwet) * L.ecy;
    if (L.ecy > 0.0 && fwet < R(1.0)) {
      if (std::fabs(L.ecy - ecx) > 1.0e-6) {
        R2 so = 0;
        for (int kk = 0; kk < MS; ++kk) so += oldevapfbl[kk];
        if (std::fabs(L.fevc - (so * air.rlam / dels)) > 1.0e-4) {
          // the reference prints a diagnostic and keeps evapfbl
          L.evapfbl_err++;
        } else {
          for (int kk = 0; kk < MS; ++kk) L.evapfbl[kk] = oldevapfbl[kk];
        }
      }
    }
    L.frday = R(12.0) * (rdy[0] + rdy[1]);
    L.fpn = mn(R(-12.0) * (an_y[0] + an_y[1]), L.frday);
  }

  // ------------------------------------------------------- Latent_heat_flux
  // cbl_latent_heat.F90:15-285
  void latent_heat_flux(R dels, const P& p, R rlam, const S& s, R potev, R& wetfac, R2 evapfbl1, R& cls,
                               R tss, R2& fes, R2& fess, R2& fesp, R& pwet) const {
    if (potev < R(0.)) wetfac = R(1.0);
    fess = wetfac * potev;
    pwet = mx(R(0.), mn(R(0.2), s.pudsto / mx(R(1.), s.pudsmx)));
    fess = fess * (R(1.) - pwet);
    R frescale = p.zse[0] * R(DENSITY_LIQ) * rlam / dels;
    if (s.snowd < R(0.1) && fess > 0.0) {
      R flower = new_reduce_soilevp ? R(s.wb[0]) - p.swilt : R(s.wb[0]) - p.swilt / R(2.0);
      R fupper = R(mx(R2(0.), flower * frescale - evapfbl1 * rlam / dels));
      fess = mn(fess, R2(fupper));
      fupper = R(s.wb[0] - s.wbice[0] / R(FROZEN_LIMIT)) * frescale;
      fupper = R(mx(R2(fupper), R(0.)));
      fess = mn(fess, R2(fupper));
    }
    cls = R(1.);
    if (s.snowd >= R(0.1)) { cls = R(1.1335); fess = cls * potev; }
    if (s.snowd < R(0.1) && potev < R(0.) && tss < R(TFRZ)) { cls = R(1.1335); fess = cls * potev; }
    if (s.snowd >= R(0.1) && potev > R(0.)) {
      cls = R(1.1335);
      fess = mn((wetfac * potev) * cls, s.snowd / dels * rlam * cls);
    }
    fesp = mn(s.pudsto / dels * rlam, mx(pwet * potev, R(0.)));
    fes = fess + fesp;
  }

  // ------------------------------------------------ Humidity_deficit_method
  // cbl_pot_evap_snow.F90:79-167 (default branch)
  static R hdm(R rho, R rlam, R dq, R rtsoil, R snowd, R tgg1) {
    if (snowd > R(1.0) || tgg1 == R(TFRZ)) dq = mx(R(-0.1e-3), dq);
    return rho * rlam * dq / rtsoil;
  }
  // litter branch of Humidity_deficit_method (cbl_pot_evap_snow.F90:155-157):
  // the litter vapour resistance added in default-REAL arithmetic
  static R hdm_litter(R rho, R rlam, R dq, R rtsoil, R snowd, R tgg1, int isflag, R2 clitt) {
    if (snowd > R(1.0) || tgg1 == R(TFRZ)) dq = mx(R(-0.1e-3), dq);
    return rho * rlam * dq / (rtsoil + R(1 - isflag) * R(clitt) * R(0.003f) / R(DV_LITT));
  }
  // Penman_Monteith (cbl_pot_evap_snow.F90:9-78): the latent heat of soil
  // potential evaporation from the soil available energy (fns - ga, ga the
  // latest value of canopy%ga) and the canopy-air humidity deficit
  R penman_monteith(const Air& air, const Met& met, R ga_prev, R fns, R rtsoil, int isflag, R2 clitt) const {
    const R sss = air.dsatdk;
    const R cc1 = sss / (sss + air.psyc), cc2 = air.psyc / (sss + air.psyc);
    const R qsatfvar = qsatfjh(met.tvair - R(TFRZ), met.pmb);
    const R rs = litter ? rtsoil + R(1 - isflag) * R(clitt) * R(0.003f) / R(DV_LITT) : rtsoil;
    return cc1 * (fns - ga_prev) + cc2 * air.rho * air.rlam * (qsatfvar - met.qvair) / rs;
  }
  // litter resistances to heat and vapour (cable_canopy.F90:471-476, :987-988)
  static void litter_resist(R2 clitt, int isflag, R rho, R& rhlitt, R& relitt) {
    rhlitt = R(R2(R(1 - isflag)) * clitt * R2(0.003f) / R2(KTH_LITT) / R2(rho * R(CAPP)));
    relitt = R(R2(R(1 - isflag)) * clitt * R2(0.003f) / R2(DV_LITT));
  }

  // ======================================================================
  // one cbm() timestep for one tile, followed by the offline driver's
  // rescaling and balance checks (cable_serial.F90:573-728)
  // mode 0: the offline cbm() (cbl_model_driver_offline.F90:38-231).
  // ACCESS coupling (src/coupled/AM3/control/cable/CM3/cbl_cbm_mod.F90):
  // mode 1 cbm_expl (:10-182), lai_refresh when the host model's radiation
  // call recomputed canopy%vlaiw (cable_land_albedo_mod_cbl.F90:263,
  // cbl_um_update_canopy.F90:27); mode 2 cbm_impl (:184-396) for cycle
  // cycleno of numcycles, with the driver's prognostic bank: stored before
  // the call and reinstated after every cycle but the last
  // (cable_implicit_main.F90:190-213, cbl_prognostic_bank.F90:26-165).
  void step(const P& p, S& s, const F& f, D& d, int ktau, R dels, int mode = 0, bool final_cycle = true,
            bool lai_refresh = false) const {
    if (mode == 2 && !final_cycle) {
      const S bank = s;
      step_body(p, s, f, d, ktau, dels, mode, final_cycle, lai_refresh);
      reinstate(s, bank);
      return;
    }
    step_body(p, s, f, d, ktau, dels, mode, final_cycle, lai_refresh);
  }

  // cable_reinstate_prognostics (cbl_prognostic_bank.F90:119-165), default soil
  static void reinstate(S& s, const S& pb) {
    for (int k = 0; k < MS; ++k) { s.tgg[k] = pb.tgg[k]; s.wb[k] = pb.wb[k]; s.wbice[k] = pb.wbice[k]; }
    for (int k = 0; k < MSN; ++k) {
      s.sdepth[k] = pb.sdepth[k]; s.smass[k] = pb.smass[k]; s.tggsn[k] = pb.tggsn[k]; s.ssdn[k] = pb.ssdn[k];
    }
    s.ssdnn = pb.ssdnn; s.snage = pb.snage; s.isflag = pb.isflag; s.snowd = pb.snowd; s.pudsto = pb.pudsto;
    s.rtsoil = pb.rtsoil; s.owetfac = pb.owetfac; s.wb_lake = pb.wb_lake; s.tss = pb.tss;
    s.cansto = pb.cansto;   // canopy%oldcansto, the next call's starting canopy water
    for (int k = 0; k < 3; ++k) s.cplant[k] = pb.cplant[k];
    for (int k = 0; k < 2; ++k) s.csoil[k] = pb.csoil[k];
  }

  void step_body(const P& p, S& s, const F& f, D& d, int ktau, R dels, int mode, bool final_cycle,
                 bool lai_refresh) const {
    Met met;
    met.fsd[0] = f.fsd[0]; met.fsd[1] = f.fsd[1]; met.fsd[2] = 0;
    met.fld = f.fld; met.precip = f.precip; met.precip_sn = f.precip_sn; met.tk = f.tk;
    met.tvair = f.tk; met.tvrad = f.tk;   // cable_input.F90:2679-2680
    met.pmb = f.pmb; met.ua = f.ua; met.qv = f.qv; met.qvair = f.qv; met.ca = f.ca;
    met.coszen = f.coszen; met.doy = f.doy; met.dva = 0;
    const R oldcansto = s.cansto;          // cable_serial.F90:573
    // ssnow%wbliq as left by the previous soil_snow call (wb - wbice); the
    // lakes fix below changes wb but not wbliq before dryLeaf reads it
    R2 wbliq0[MS];
    for (int k = 0; k < MS; ++k) wbliq0[k] = s.wb[k] - s.wbice[k];

    // lakes top-layer fix (cbl_model_driver_offline.F90:116-121); not in
    // the coupled calls
    if (mode == 0) {
      if (p.iveg == LAKES && s.wb[0] < p.sfc) {
        s.wbtot1 = R(s.wb[0]) * R(DENSITY_LIQ) * p.zse[0];
        s.wb[0] = p.sfc;
        s.wbtot2 = R(s.wb[0]) * R(DENSITY_LIQ) * p.zse[0];
      }
      s.wb_lake = s.wb_lake + mx(s.wbtot2 - s.wbtot1, R(0.));
    }

    Rough rough{};
    R vlaiw, rghlai;
    const bool carried = mode != 0 && !(mode == 1 && lai_refresh);
    ruff_resist(p, s, rough, vlaiw, rghlai, carried ? &s.vlaiw : nullptr);
    if (mode == 1 && lai_refresh) s.vlaiw = vlaiw;
    Air air;
    define_air(met, air);
    const bool veg_mask = vlaiw > R(LAI_THRESH);
    const bool sunlit_mask = (met.fsd[0] + met.fsd[1]) > R(RAD_THRESH);
    const bool sunlit_veg = veg_mask && sunlit_mask;
    Rad rad{};
    R albsoilsn[3], c1[3], rhoch[3], xk[3];
    init_radiation_albedo(p, s, met, vlaiw, veg_mask, rad, albsoilsn, c1, rhoch, xk);
    const R otss = s.tss;

    // ================= define_canopy (cable_canopy.F90:10-1048)
    R cansto = oldcansto;
    const R cansat = p.canst1 * vlaiw;
    // Surf_wetness_fact (cbl_SurfaceWetness.F90:10-79)
    R upper_limit = R(4.0) * mn(dels, R(1800.0)) / (R(60.0) * R(1440.0));
    R ftemp = mn(met.precip - met.precip_sn, upper_limit);
    R lower_limit = cansat - cansto;
    upper_limit = mx(lower_limit, R(0.0));
    R wcint = (ftemp > R(0.0) && met.tk > R(TFRZ)) ? mn(upper_limit, ftemp) : R(0.0);
    R through = met.precip_sn + mn(met.precip - met.precip_sn, mx(R(0.0), met.precip - met.precip_sn - wcint));
    cansto = cansto + wcint;
    const R fwet = mx(R(0.0), mn(R(0.9), R(0.8) * cansto / mx(cansat, R(0.01))));
    // initialize_wetfac (cbl_init_wetfac_mod.F90:9-116)
    R wetfac;
    {
      R wilting_pt = p.swilt / R(WILT_LIMITFACTOR);
      R num = R(s.wb[0]) - wilting_pt;
      R den = R(p.sfc - wilting_pt);
      den = mx(R(0.0830), den);
      wetfac = num / den;
      wetfac = mn(R(1.0), wetfac);
      wetfac = mx(R(0.0), wetfac);
      if (s.wbice[0] > 0.0) {
        R ice_ratio = R(sq(s.wbice[0] / s.wb[0]));
        R ice_factor = R(R2(1.0) - mn(R2(0.2), R2(ice_ratio)));
        ice_factor = R(mx(R2(0.5), R2(ice_factor)));
        wetfac = wetfac * ice_factor;
      }
      if (s.snowd > R(0.1)) wetfac = R(0.9);
      if (p.iveg == LAKES) {
        if (met.tk >= R(TFRZ) + R(5.)) wetfac = R(1.0);
        if (met.tk < R(TFRZ) + R(5.)) wetfac = R(0.7);
      }
    }
    wetfac = R(0.5) * (wetfac + s.owetfac);

    R fevw_pot = 0;
    LeafIter L{};
    L.gswx[0] = L.gswx[1] = R(1e-3);
    L.gbhf[0] = L.gbhf[1] = R2(1e-3);
    L.gbhu[0] = L.gbhu[1] = R2(1e-3);
    R2 evapfbl[MS];
    for (int k = 0; k < MS; ++k) evapfbl[k] = 0;
    L.csx[0] = L.csx[1] = met.ca;
    met.tvair = met.tk;
    met.qvair = met.qv;
    R tv = met.tvair;
    L.fwsoil = R(1.0);
    define_air(met, air);
    R qstvair = qsatfjh(met.tvair - R(TFRZ), met.pmb);
    met.dva = (qstvair - met.qvair) * R(RMAIR) / R(RMH2O) * met.pmb * R(100.0);
    L.dsx = met.dva;
    L.dsx = mx(L.dsx, R(0.0));
    L.tlfx = met.tk;
    L.tlfy = met.tk;
    const R ortsoil = s.rtsoil;
    s.tss = R(1 - s.isflag) * s.tgg[0] + R(s.isflag) * s.tggsn[0];
    const R tss4 = std::pow(s.tss, 4);
    R2 fes = 0, fess = 0, fesp = 0;
    R potev = 0;
    fevw_pot = 0;
    radiation(p, met, air, vlaiw, s.tss, sunlit_veg, albsoilsn, rad);
    R zetar[NITER];
    zetar[0] = R(ZETA0);
    zetar[1] = R(ZETPOS) + R(1);
    zetar[2] = zetar[3] = 0;
    const R sum_rad_rniso = rad.rniso[0] + rad.rniso[1];
    const R sum_rad_gradis = rad.gradis[0] + rad.gradis[1];
    R us = 0, rt0 = 0, rt1usc = 0, rtsoil = s.rtsoil, cls = R(1);
    R rhlitt = 0, relitt = 0;   // cable_canopy.F90:239-240
    R fev = 0, fhv = 0, fnv = 0, fns = 0, fhs = 0, fe = 0, fh = 0, rnet = 0, epot = 0, qstss = 0;
    R ga = s.ga;   // canopy%ga persists between steps (read before it is set only by P-M)
    R fevw = 0, fhvw = 0;
    R2 ghwet = 0;
    int iterplus = 1;
    int passes_total = 0;
    R pwet = 0;
    for (int iter = 1; iter <= NITER; ++iter) {
      // comp_friction_vel (cbl_friction_vel.F90:19-108)
      {
        R zi = zetar[iter - 1];
        R psim_1 = psim(zi * rough.zref_uv / rough.zref_tq);
        R rescale = R(VONK) * mx(met.ua, R(UMIN));
        R z_eff = rough.zref_uv / rough.z0m;
        R psim_2 = psim(zi * rough.z0m / rough.zref_tq);
        R ll = rescale / (std::log(z_eff) - psim_1 + psim_2);
        us = mn(mx(R(1.e-6), ll), R(10.0));
      }
      // :276-363
      R xx = R(0.5) + fsign(R(0.5), rough.zref_tq + rough.disp - rough.zruffs);
      R zr = mx(rough.zruffs - rough.disp, rough.z0soilsn);
      rt1usc = xx * (std::log(rough.zref_tq / zr) - psis(zetar[iter - 1]) +
                     psis(zetar[iter - 1] * zr / rough.zref_tq)) / R(VONK);
      const R rt_min = R(5.);
      rt0 = mx(rt_min, rough.rt0us / us);
      rough.rt1 = mx(R(5.), (rough.rt1usa + rough.rt1usb + rt1usc) / us);
      rtsoil = (vlaiw > R(LAI_THRESH)) ? rt0 : rt0 + rough.rt1;
      rtsoil = mx(rt_min, rtsoil);
      if (rtsoil > R(2.) * ortsoil || rtsoil < R(0.5) * ortsoil) rtsoil = mx(rt_min, R(0.5) * (rtsoil + ortsoil));
      // :374-397
      if (vlaiw > R(LAI_THRESH)) {
        R2 gbvtop = air.cmolar * R(APOL) * air.visc / R(PRANDT) / p.dleaf *
                    std::pow(us / mx(rough.usuh, R(1.e-6)) * p.dleaf / air.visc, R(0.5)) *
                    std::pow(R(PRANDT), R(1.0) / R(3.0)) / p.shelrb;
        gbvtop = mx(R2(0.05), gbvtop);
        L.gbhu[0] = gbvtop * (R(1.0) - std::exp(-mn(vlaiw * (R(0.5) * rough.coexp + rad.extkb), R(20.0)))) /
                    (rad.extkb + R(0.5) * rough.coexp);
        L.gbhu[1] = (R(2.0) / rough.coexp) * gbvtop * (R(1.0) - std::exp(-mn(R(0.5) * rough.coexp * vlaiw, R(20.0)))) -
                    L.gbhu[0];
      }
      L.rny = sum_rad_rniso;
      L.hcy = 0.0;
      L.ecy = L.rny - L.hcy;
      dryLeaf(dels, p, rad, met, air, vlaiw, cansto, fwet, wbliq0, L, iter, sum_rad_gradis, sum_rad_rniso);
      passes_total += L.passes;
      for (int k = 0; k < MS; ++k) evapfbl[k] = L.evapfbl[k];
      // wetLeaf (cbl_wetleaf.F90:9-111)
      {
        ghwet = R2(1.0e-3);
        R gwwet = R(1.0e-3), ghrwet = R(1.0e-3);
        fevw = 0; fhvw = 0;
        R sum_gbh = R(L.gbhu[0] + L.gbhf[0] + L.gbhu[1] + L.gbhf[1]);
        if (vlaiw > R(LAI_THRESH)) {
          ghwet = R(2.0) * sum_gbh;
          gwwet = R(1.075) * sum_gbh;
          ghrwet = sum_rad_gradis + R(ghwet);
          R ccfevw = mn(cansto * air.rlam / dels, R(2.0) / (R(1440.0) / (dels / R(60.0))) * air.rlam);
          R num = air.dsatdk * (sum_rad_rniso - R(CAPP) * R(RMAIR) * (met.tvair - met.tk) * sum_rad_gradis) +
                  R(CAPP) * R(RMAIR) * met.dva * ghrwet;
          R den = air.dsatdk + air.psyc * ghrwet / gwwet;
          fevw = mn(fwet * num / den, ccfevw);
          fevw_pot = num / den;
          fhvw = fwet * (sum_rad_rniso - R(CAPP) * R(RMAIR) * (L.tlfy - met.tk) * sum_rad_gradis) - fevw;
        }
      }
      fev = R(L.fevc + fevw);
      ftemp = (R(1.0) - fwet) * R(L.hcy) + fhvw;
      fhv = ftemp;
      ftemp = (R(1.0) - fwet) * R(L.rny) + fevw + fhvw;
      fnv = ftemp;
      // :425-450
      if (vlaiw > R(LAI_THRESH) && rough.hruff > rough.z0soilsn) {
        rad.lwabv = R(CAPP) * R(RMAIR) * (L.tlfy - met.tk) * sum_rad_gradis;
        R arg = rad.lwabv / (R(2.0) * (R(1.0) - rad.transd) * R(SBOLTZ) * R(EMLEAF)) + std::pow(met.tvrad, 4);
        tv = (arg > R(0.0)) ? std::pow(arg, R(0.25)) : met.tvrad;
      } else {
        tv = met.tvrad;
      }
      fns = rad.qssabs + rad.transd * met.fld + (R(1.0) - rad.transd) * R(EMLEAF) * R(SBOLTZ) * std::pow(tv, 4) -
            R(EMSOIL) * R(SBOLTZ) * tss4;
      qstss = qsatfjh(s.tss - R(TFRZ), met.pmb);
      if (litter) litter_resist(p.clitt, s.isflag, air.rho, rhlitt, relitt);
      if (potev_pm) {
        potev = penman_monteith(air, met, ga, fns, rtsoil, s.isflag, p.clitt);
      } else {
        R dq = qstss - met.qv;
        potev = litter ? hdm_litter(air.rho, air.rlam, dq, rtsoil, s.snowd, s.tgg[0], s.isflag, p.clitt)
                       : hdm(air.rho, air.rlam, dq, rtsoil, s.snowd, s.tgg[0]);
      }
      latent_heat_flux(dels, p, air.rlam, s, potev, wetfac, evapfbl[0], cls, s.tss, fes, fess, fesp, pwet);
      // :521-534: the litter branch uses the reference-height air temperature
      if (litter) fhs = air.rho * R(CAPP) * (s.tss - met.tk) / (rtsoil + rhlitt);
      else fhs = air.rho * R(CAPP) * (s.tss - met.tvair) / rtsoil;
      // within_canopy (cbl_within_canopy.F90:10-159)
      {
        R rrbw = R(L.gbhu[0] + L.gbhf[0] + L.gbhu[1] + L.gbhf[1]) / air.cmolar;
        R rrsw = (L.gswx[0] + L.gswx[1]) / air.cmolar;
        R fix_eqn = cls * rt0 / (rt0 + relitt);
        if (potev > R(0.)) fix_eqn = fix_eqn * wetfac;
        R fix_eqn2 = rt0 / (rt0 + rhlitt);
        if (p.meth > R(0) && vlaiw > R(LAI_THRESH) && rough.hruff > rough.z0soilsn) {
          const R rt1 = rough.rt1;
          R dmah = (rt0 + fix_eqn2 * rt1) * ((R(1.) + air.epsi) * rrsw + rrbw) + air.epsi * (rt0 * rt1) * (rrbw * rrsw);
          R dmbh = (-air.rlam / R(CAPP)) * (rt0 * rt1) * (rrbw * rrsw);
          R dmch = ((R(1.) + air.epsi) * rrsw + rrbw) * rt0 * rt1 * (fhv + fhs) / (air.rho * R(CAPP));
          R dmae = (-air.epsi * R(CAPP) / air.rlam) * (rt0 * rt1) * (rrbw * rrsw);
          R dmbe = (rt0 + fix_eqn * rt1) * ((R(1.) + air.epsi) * rrsw + rrbw) + (rt0 * rt1) * (rrbw * rrsw);
          R dmce = R(((R(1.) + air.epsi) * rrsw + rrbw) * rt0 * rt1 * (fev + fes / cls) / (air.rho * air.rlam));
          met.tvair = met.tk + (dmbe * dmch - dmbh * dmce) / (dmah * dmbe - dmae * dmbh + R(1.0e-12));
          R lo = mn(s.tss, met.tk) - R(5.0), hi = mx(s.tss, met.tk) + R(5.0);
          met.tvair = mx(met.tvair, lo);
          met.tvair = mn(met.tvair, hi);
          met.qvair = met.qv + (dmah * dmce - dmae * dmch) / (dmah * dmbe - dmae * dmbh + R(1.0e-12));
          met.qvair = mx(R(0.0), met.qvair);
          lo = mn(qstss, met.qv); hi = mx(qstss, met.qv);
          met.qvair = mx(met.qvair, lo);
          met.qvair = mn(met.qvair, hi);
          qstvair = qsatfjh(met.tvair - R(TFRZ), met.pmb);
          met.dva = (qstvair - met.qvair) * R(RMAIR) / R(RMH2O) * met.pmb * R(100.);
        }
      }
      qstss = qsatfjh(s.tss - R(TFRZ), met.pmb);
      if (potev_pm) {
        potev = penman_monteith(air, met, ga, fns, rtsoil, s.isflag, p.clitt);
      } else {
        R dq = qstss - met.qvair;
        potev = litter ? hdm_litter(air.rho, air.rlam, dq, rtsoil, s.snowd, s.tgg[0], s.isflag, p.clitt)
                       : hdm(air.rho, air.rlam, dq, rtsoil, s.snowd, s.tgg[0]);
      }
      latent_heat_flux(dels, p, air.rlam, s, potev, wetfac, evapfbl[0], cls, s.tss, fes, fess, fesp, pwet);
      if (litter) fhs = air.rho * R(CAPP) * (s.tss - met.tvair) / (rtsoil + rhlitt);
      else fhs = air.rho * R(CAPP) * (s.tss - met.tvair) / rtsoil;
      ga = fns - fhs - R(fes);
      fe = R(fev + fes);
      fh = fhv + fhs;
      // :627-641
      if (potev >= R(0.)) potev = mx(R(0.00001), potev);
      else potev = mn(R(-0.0002), potev);
      if (fevw_pot >= R(0.)) fevw_pot = mx(R(0.000001), fevw_pot);
      else fevw_pot = mn(R(-0.002), fevw_pot);
      rnet = fnv + fns;
      epot = (fevw_pot + potev / cls) * dels / air.rlam;
      // wetfac_cs (:657-669) is diagnostic only and not carried
      // update_zetar (cbl_zetar.F90:13-159)
      if (iter < NITER) {
        iterplus = std::max(iter + 1, 2);
        R z = -(R(VONK) * R(GRAV) * rough.zref_tq * (fh + R(0.07) * fe)) / (air.rho * R(CAPP) * met.tk * us * us * us);
        z = mn(R(ZETPOS), z);
        z = mx(R(ZETNEG), z);
        zetar[iterplus - 1] = z;
      }
    }
    // post-loop (:684-1038)
    d.cduv = us * us / sq(mx(met.ua, R(UMIN)));
    const R z4 = zetar[NITER - 1];
    d.cdtq = d.cduv * (std::log(rough.zref_uv / rough.z0m) - psim(z4 * rough.zref_uv / rough.zref_tq) +
                       psim(z4 * rough.z0m / rough.zref_tq)) /
             (std::log(rough.zref_tq / (R(0.1) * rough.z0m)) - psis(z4) + psis(z4 * R(0.1) * rough.z0m / rough.zref_tq));
    const R zip = zetar[iterplus - 1];
    R tstar = -fh / (air.rho * R(CAPP) * us);
    R qstar = -fe / (air.rho * air.rlam * us * cls);
    R zscrn = mx(rough.z0m, R(2.0) - rough.disp);
    ftemp = (std::log(rough.zref_tq / zscrn) - psis(zip) + psis(zip * zscrn / rough.zref_tq)) / R(VONK);
    R tscrn = met.tk - R(TFRZ) - tstar * ftemp;
    R term1 = 0, term2 = 0, term5 = 0, term3 = 0, r_sc = 0;
    R zscl = mx(rough.z0soilsn, R(2.0));
    const bool screen_canopy = vlaiw > R(LAI_THRESH) && rough.hruff > R(0.01);
    if (screen_canopy) {
      if (rough.disp > R(0.0)) {
        term1 = std::exp(R(2) * R(CSW) * rghlai * (R(1) - zscl / rough.hruff));
        term2 = std::exp(R(2) * R(CSW) * rghlai * (R(1) - rough.disp / rough.hruff));
        term5 = mx(R(2.) / R(3.) * rough.hruff / rough.disp, R(1.));
      }
      term3 = R(A33) * R(A33) * R(CTL) * R(2) * R(CSW) * rghlai;
      if (zscl < rough.disp) {
        r_sc = term5 * std::log(zscl / rough.z0soilsn) * (std::exp(R(2) * R(CSW) * rghlai) - term2) / term3;
        r_sc = r_sc + term5 * std::log(rough.disp / zscl) * (std::exp(R(2) * R(CSW) * rghlai) - term1) / term3;
      } else if (rough.disp <= zscl && zscl < rough.hruff) {
        r_sc = rough.rt0us + term5 * (term2 - term1) / term3;
      } else if (rough.hruff <= zscl && zscl < rough.zruffs) {
        r_sc = rough.rt0us + rough.rt1usa + term5 * (zscl - rough.hruff) / (R(A33) * R(A33) * R(CTL) * rough.hruff);
      } else if (zscl >= rough.zruffs) {
        r_sc = rough.rt0us + rough.rt1usa + rough.rt1usb +
               (std::log((zscl - rough.disp) / mx(rough.zruffs - rough.disp, rough.z0soilsn)) -
                psis((zscl - rough.disp) * zip / rough.zref_tq) + psis((rough.zruffs - rough.disp) * zip / rough.zref_tq)) /
                   R(VONK);
      }
      if (litter)   // :808-812
        tscrn = s.tss + (met.tk - s.tss) *
                            mn(R(1.), ((r_sc + rhlitt * us) /
                                       mx(R(1.), rough.rt0us + rough.rt1usa + rough.rt1usb + rt1usc + rhlitt * us))) -
                R(TFRZ);
      else
        tscrn = s.tss + (met.tk - s.tss) *
                            mn(R(1.), (r_sc / mx(R(1.), rough.rt0us + rough.rt1usa + rough.rt1usb + rt1usc))) -
                R(TFRZ);
    }
    R rsts = qsatfjh(tscrn, met.pmb);
    R qtgnet = rsts * wetfac - met.qv;
    R qsurf = (qtgnet > R(0.)) ? rsts * wetfac : R(0.1) * rsts * wetfac + R(0.9) * met.qv;
    R qscrn = met.qv - qstar * ftemp;
    if (screen_canopy && litter)   // :848-854
      qscrn = qsurf + (met.qv - qsurf) *
                          mn(R(1.), ((r_sc + relitt * us) /
                                     mx(R(1.), rough.rt0us + rough.rt1usa + rough.rt1usb + rt1usc + relitt * us)));
    else if (screen_canopy)
      qscrn = qsurf + (met.qv - qsurf) * mn(R(1.), (r_sc / mx(R(1.), rough.rt0us + rough.rt1usa + rough.rt1usb + rt1usc)));
    // canopy water budget (:881-906)
    R dewmm = R(-(mn(R(0.0), fevw) + mn(R2(0.0), L.fevc)) * dels / air.rlam);
    cansto = cansto + dewmm;
    cansto = mx(cansto - mx(R(0.0), fevw) * dels / air.rlam, R(0.0));
    R spill = mx(R(0.0), cansto - cansat);
    through = through + spill;
    R precis = mx(R(0.), through);
    cansto = cansto - spill;
    R delwc = cansto - oldcansto;
    // soil-coupling derivatives (:913-1027): default and litter branches,
    // with the l_rev_corr revisions (:916-922, :993-1014)
    R dfn_dtg = R(-1.) * R(4.) * R(EMSOIL) * R(SBOLTZ) * tss4 / s.tss;
    R rttsoil = rtsoil;
    if (l_rev_corr && vlaiw > R(LAI_THRESH)) rttsoil = rttsoil + rough.rt1;
    R dfh_dtg, dfe_ddq;
    if (litter) {
      litter_resist(p.clitt, s.isflag, air.rho, rhlitt, relitt);
      dfh_dtg = air.rho * R(CAPP) / (rttsoil + rhlitt);
      dfe_ddq = wetfac * air.rho * air.rlam * cls / (rttsoil + relitt);
    } else {
      dfh_dtg = air.rho * R(CAPP) / rttsoil;
      dfe_ddq = wetfac * air.rho * air.rlam * cls / rttsoil;
    }
    if (l_rev_corr && potev < R(0.)) dfe_ddq = air.rho * air.rlam * cls / (rttsoil + relitt);
    R ddq_dtg = (R(RMH2O) / R(RMAIR)) / met.pmb * R(TETENA) * R(TETENB) * R(TETENC) / (sq(R(TETENC) + s.tss - R(TFRZ))) *
                std::exp(R(TETENB) * (s.tss - R(TFRZ)) / (R(TETENC) + s.tss - R(TFRZ)));
    R dfe_dtg = dfe_ddq * ddq_dtg;
    R2 dgdtg = dfn_dtg - dfh_dtg - dfe_dtg;
    d.drybal = R(L.ecy + L.hcy) - sum_rad_rniso + R(CAPP) * R(RMAIR) * (L.tlfy - met.tk) * sum_rad_gradis;
    d.wetbal = fevw + fhvw - sum_rad_rniso * fwet + R(CAPP) * R(RMAIR) * (L.tlfy - met.tk) * sum_rad_gradis * fwet;
    rad.swnet = rad.qcan[0][0] + rad.qcan[1][0] + rad.qcan[0][1] + rad.qcan[1][1] + rad.qssabs;
    rad.lwnet = met.fld - R(SBOLTZ) * R(EMLEAF) * std::pow(tv, 4) * (R(1) - rad.transd) - rad.flws * rad.transd;
    s.rtsoil = rtsoil;
    R2 fevc = L.fevc;
    // cbm_expl puts back the canopy water and wetness factor
    // (cbl_cbm_mod.F90:150-152)
    if (mode != 1) s.cansto = cansto;
    s.ga = ga;
    // ================= end define_canopy
    if (mode != 1) s.owetfac = wetfac;     // cbm:192

    SoilOut so{};
    if (mode != 1)
      soil_snow(p, s, dels, precis, fes, fess, fesp, fevc, fevw, ga, dgdtg, evapfbl, met, cls == R(1.1335), so);

    // snow_aging (cbl_snow_aging.F90:11-83)
    if (mode != 1 && s.snowd > R(SNOW_DEPTH_THRESH)) {
      R dnsnow = mn(R(1.0), R(0.1) * mx(R(0.0), s.snowd - s.osnowd));
      R tmp = R(s.isflag) * s.tggsn[0] + R(1 - s.isflag) * s.tgg[0];
      tmp = mn(tmp, R(TFRZ));
      R ar1 = R(5000.0) * (R(1.0) / (R(TFRZ) - R(0.01)) - R(1.0) / tmp);
      R ar2 = R(10.0) * ar1, ar3;
      if (p.isoilm == ICE_SOIL) { ar3 = R(0.0000001); dnsnow = R(1.0); }
      else ar3 = R(0.1);
      R dtau = R(1.0e-6) * (std::exp(ar1) + std::exp(ar2) + ar3) * dels;
      s.snage = mx(R(0.0), (s.snage + dtau) * (R(1.0) - dnsnow));
    }
    R trad;
    if (mode == 0) {
      fev = R(fevc + fevw);
      fe = R(fev + fes);
      rnet = fns + fnv;
      trad = std::pow((R(1.) - rad.transd) * std::pow(tv, 4) + rad.transd * std::pow(s.tss, 4), R(0.25));
    } else {
      R fns_cor = 0;   // zeroed by define_canopy (cable_canopy.F90:233)
      if (mode == 2) {
        // soil_snow's online corrections (cbl_soilsnow_main.F90:164-183)
        const R fhs_cor = so.dtmlt1 * dfh_dtg;
        const R2 fes_cor = so.dtmlt1 * dfe_dtg;
        fhs = fhs + fhs_cor;
        fes = fes + fes_cor;
        if (l_rev_corr) {
          fns_cor = so.dtmlt1 * dfn_dtg;
          fns = fns + fns_cor;
          ga = R(ga + so.dtmlt1 * dgdtg);
          fess = fess + fes_cor;
        }
        // cbm_impl (cbl_cbm_mod.F90:307-357): tss reset on a cycle that is
        // not the last, then the corrections for the change of tss
        if (!final_cycle) s.tss = otss;
        const R dT = s.tss - otss;
        fhs = fhs + dT * dfh_dtg;
        fh = fhv + fhs;
        fes = fes + dT * dfe_dtg;
        if (l_rev_corr) {
          fns_cor = fns_cor + dT * dfn_dtg;
          fns = fns + dT * dfn_dtg;
          ga = R(ga + dT * dgdtg);
          fess = fess + dT * dfe_dtg;
        }
        s.ga = ga;
      }
      fev = R(fevc + fevw);
      fe = R(fev + fes);
      rnet = fns + fnv;
      // emissivities 1 (cable_phys_constants_mod.F90:26-27), the surface
      // temperature of the start of the step (cbl_cbm_mod.F90:172-179, :374-381)
      trad = std::pow((R(1.) - rad.transd) * std::pow(tv, 4) + rad.transd * std::pow(otss, 4) + fns_cor / R(SBOLTZ),
                      R(0.25));
    }

    // carbon, icycle == 0 (cable_carbon.F90:38-360 and cbm:214-229)
    R frp, frpw, frpr, frs;
    {
      R tot = p.ratecp[0] * s.cplant[0] + p.ratecp[1] * s.cplant[1] + p.ratecp[2] * s.cplant[2];
      R pc1 = tot - p.ratecp[0] * s.cplant[0];
      R pc1w = tot - p.ratecp[0] * s.cplant[0] - p.ratecp[2] * s.cplant[2];
      R pc1r = tot - p.ratecp[0] * s.cplant[0] - p.ratecp[1] * s.cplant[1];
      R tmp1 = mx(R(3.22) - R(0.046) * (met.tk - R(TFRZ)), R(1e-6));
      R tmp2 = R(0.1) * (met.tk - R(TFRZ) - R(20.0));
      R tmp3 = std::pow(tmp1, tmp2);
      const R spy = R(365.0) * R(24.0) * R(3600.0);
      frp = p.rp20 * tmp3 * pc1 / spy;
      frpw = p.rp20 * tmp3 * pc1w / spy;
      frpr = p.rp20 * tmp3 * pc1r / spy;
    }
    if (diag_soil_resp_off) {
      // diag_soil_resp = 'OFF' (cable_carbon.F90:256-276): rs20 scheme
      R avgwrs = 0, sumt = 0;
      for (int k = 0; k < MS; ++k) { avgwrs += p.froot[k] * R(s.wb[k]); sumt += p.froot[k] * s.tgg[k]; }
      const R avgtrs = mx(R(0.0), sumt - R(TFRZ));
      frs = p.rs20 *
            mn(R(1.0), mx(R(0.0), mn(R(-0.0178) + R(0.2883) * avgwrs + R(5.0176) * avgwrs * avgwrs -
                                         R(4.5128) * avgwrs * avgwrs * avgwrs,
                                     R(0.3320) + R(22.6726) * std::exp(R(-5.8184) * avgwrs)))) *
            mn(R(1.0), mx(R(0.0), mn(R(0.0104) * std::pow(avgtrs, R(1.3053)), R(5.5956) - R(0.1189) * avgtrs)));
      frs = frs * (p.ratecs[0] * s.csoil[0] + p.ratecs[1] * s.csoil[1]) / (R(365.0) * R(24.0) * R(3600.0));
      if (s.snowd > R(1.)) frs = frs / mx(R(0.001), mn(R(100.), s.snowd));
    } else {
      const R rswch = R(0.16), soilcf = R(1.0), t0 = R(-46.0);
      R den = mx(R(0.07), p.sfc - p.swilt);
      R rswc = mx(R(0.0001), p.froot[0] * (R(s.wb[1]) - p.swilt)) / den;
      R tsoil = p.froot[0] * s.tgg[1] - R(TFRZ);
      R tref = mx(R(0.), s.tgg[MS - 1] - (R(TFRZ) - R(.05)));
      for (int k = 1; k < MS; ++k) {
        rswc = rswc + mx(R(0.0001), p.froot[k] * (R(s.wb[k]) - p.swilt)) / den;
        tsoil = tsoil + p.froot[k] * s.tgg[k];
      }
      rswc = mn(R(1.), rswc);
      tsoil = mx(t0 + R(2.), tsoil);
      R e0rswc = R(52.4) + R(285.) * rswc;
      R ftsoil = mn(R(0.0015), R(1.) / (tref - t0) - R(1.) / (tsoil - t0));
      R sss = mx(R(-15.), mn(R(1.), e0rswc * ftsoil));
      R ftsrs = std::exp(sss);
      frs = p.vegcf * (R(144.0) / R(44.0e6)) * soilcf * mn(R(1.), R(1.4) * mx(R(.3), R(.0278) * tsoil + R(.5))) * ftsrs *
            rswc / (rswch + rswc);
    }
    if (mode != 1) {   // carbon_pl; cbm_expl has no carbon
      const R beta = R(0.9);
      const R trnl = R(3.17e-8), trnr = R(4.53e-9), trnsf = R(1.057e-10), trnw = R(6.342e-10);
      R coef_cold = std::exp(mn(R(1.), -(tv - p.tvclst)));
      R wbav = 0;
      for (int k = 0; k < MS; ++k) wbav += p.froot[k] * R(s.wb[k]);
      wbav = mx(R(0.01), wbav);
      R campbell = R(2.0) - p.ibp2;
      R esw = std::pow(wbav, campbell) - R(1.0);
      esw = mx(R(1.0), esw);
      R eswilt = std::pow(p.swilt, campbell) - R(1.0);
      R relstress = esw / eswilt - R(1.0);
      relstress = mn(R(1.0), relstress);
      R coef_drght = std::exp(R(5.0) * relstress);
      R coef_cd = (coef_cold + coef_drght) * R(2.0e-7);
      R fcl = std::exp(-p.tfcl * p.vlai);
      R clitt = (coef_cd + trnl) * s.cplant[0];
      s.cplant[0] = s.cplant[0] - dels * (L.fpn * fcl + clitt);
      R fr = mn(R(1.), std::exp(-p.rw * beta * R(0.0001) * s.cplant[2] / mx(s.cplant[1], R(0.01))) / beta);
      R cfwd = trnw * s.cplant[1];
      s.cplant[1] = s.cplant[1] - dels * (L.fpn * (R(1.) - fcl) * (R(1.) - fr) + frpw + cfwd);
      R cfrts = trnr * s.cplant[2];
      s.cplant[2] = s.cplant[2] - dels * (L.fpn * (R(1.) - fcl) * fr + cfrts + frpr);
      R cfsf = trnsf * s.csoil[0];
      s.csoil[0] = s.csoil[0] + dels * (R(0.98) * clitt + R(0.9) * cfrts + cfwd - cfsf - R(0.98) * frs);
      s.csoil[1] = s.csoil[1] + dels * (R(0.02) * clitt + R(0.1) * cfrts + cfsf - R(0.02) * frs);
      for (int k = 0; k < 3; ++k) s.cplant[k] = mx(R(0.00), s.cplant[k]);
      for (int k = 0; k < 2; ++k) s.csoil[k] = mx(R(0.00), s.csoil[k]);
    }

    // driver rescaling (cable_serial.F90:602-605)
    const R smelt = so.smelt * dels;
    const R rnof1 = so.rnof1 * dels, rnof2 = so.rnof2 * dels, runoff = so.runoff * dels;

    // the offline driver's balance checks; the coupled calls run none
    R wbal = 0, ebal = 0;
    if (mode == 0) {
      // mass_balance (cable_checks.F90:472-551)
      if (ktau == 1) s.owb = so.wbtot;
      R2 delwb = so.wbtot - s.owb;
      s.owb = so.wbtot;
      wbal = R(met.precip - delwc - s.snowd + s.osnowd - runoff - (fevw + fevc + fes / cls) * dels / air.rlam - delwb - R(0));
      if (ktau == 1) s.wbal_tot = 0;
      if (ktau > 10) s.wbal_tot = s.wbal_tot + wbal;
      // energy_balance (cable_checks.F90:565-618)
      ebal = rad.qcan[0][0] + rad.qcan[1][0] + rad.qcan[0][1] + rad.qcan[1][1] + rad.qssabs + met.fld -
             R(SBOLTZ) * R(EMLEAF) * std::pow(tv, 4) * (R(1) - rad.transd) - rad.flws * rad.transd - fev - R(fes) - fh - ga;
      s.ebal_tot = s.ebal_tot + ebal;
    }

    // ---- diagnostics
    d.fe = fe; d.fh = fh; d.fev = fev; d.fhv = fhv; d.fhs = fhs; d.fns = fns; d.fnv = fnv; d.ga = ga; d.tv = tv;
    d.tscrn = tscrn; d.qscrn = qscrn; d.rnet = rnet; d.us = us; d.epot = epot;
    d.fes = fes; d.fevc = fevc; d.dgdtg = dgdtg; d.fevw = fevw;
    d.fpn = L.fpn; d.frday = L.frday;
    d.fnpp = R(-1.0) * L.fpn - frp;
    d.fgpp = R(-1.0) * L.fpn + L.frday;
    d.fnee = L.fpn + frs + frp;
    d.fra = frp + L.frday;
    d.frp = frp; d.frs = frs; d.trad = trad;
    d.frpw = frpw; d.frpr = frpr; d.delwc = delwc; d.cls = cls;
    d.albedo[0] = rad.albedo[0]; d.albedo[1] = rad.albedo[1]; d.transd = rad.transd;
    d.precis = precis; d.through = through; d.fwet = fwet; d.wetfac = wetfac; d.potev = potev;
    d.runoff = runoff; d.rnof1 = rnof1; d.rnof2 = rnof2; d.smelt = smelt;
    d.ghflux = so.ghflux; d.sghflux = so.sghflux;
    d.ebal = ebal; d.wbal = wbal; d.qssabs = rad.qssabs; d.rniso = sum_rad_rniso; d.vlaiw = vlaiw;
    d.tvair = met.tvair; d.qvair = met.qvair; d.swnet = rad.swnet; d.lwnet = rad.lwnet;
    d.wbtot = so.wbtot; d.gswx[0] = L.gswx[0]; d.gswx[1] = L.gswx[1]; d.fwsoil = L.fwsoil;
    d.dryleaf_passes = passes_total;
    d.dryleaf_noconv = L.noconv;
    d.evapfbl_err = L.evapfbl_err;
  }

  // ====================================================================
  // soil_snow (cbl_soilsnow_main.F90:28-207) and its callees
  struct SoilOut { R smelt, rnof1, rnof2, runoff, ghflux, sghflux; R2 wbtot; R dtmlt1; };

  static void trimb(const R2* a, const R2* b, const R2* c, R2* rhs, int kmax) {
    // cbl_trimb.F90:17-53
    R2 e[9], temp[9], g[9];
    e[0] = c[0] / b[0];
    for (int k = 1; k < kmax - 1; ++k) {
      temp[k] = 1. / (b[k] - a[k] * e[k - 1]);
      e[k] = c[k] * temp[k];
    }
    g[0] = rhs[0] / b[0];
    for (int k = 1; k < kmax - 1; ++k) g[k] = (rhs[k] - a[k] * g[k - 1]) * temp[k];
    rhs[kmax - 1] = (rhs[kmax - 1] - a[kmax - 1] * g[kmax - 2]) / (b[kmax - 1] - a[kmax - 1] * e[kmax - 2]);
    for (int k = kmax - 2; k >= 0; --k) rhs[k] = g[k] - e[k] * rhs[k + 1];
  }

  void soil_snow(const P& p, S& s, R dels, R precis, R2 fes, R2 fess, R2 fesp, R2& fevc, R& fevw, R ga, R2 dgdtg,
                 R2 evapfbl[MS], const Met& met, bool cls_snow, SoilOut& o) const {
    (void)fes;
    R hcll[MS];
    for (int k = 0; k < MS; ++k) hcll[k] = mx(R(0.01), p.css * p.rhosoil);
    const R t_snwlr = R(0.05);
    R fwtop1 = 0, fwtop2 = 0, fwtop3 = 0, rnof1 = 0, rnof2 = 0, smelt = 0;
    R dtmlt[3] = {0, 0, 0};
    s.osnowd = s.snowd;
    R2 wbliq[MS], wblf[MS], wbfice[MS];
    for (int k = 0; k < MS; ++k) wbliq[k] = s.wb[k] - s.wbice[k];
    if (s.first_soilsnow_call) {
      R xx = p.css * p.rhosoil;
      s.gammzz[0] = mx((R(1.0) - p.ssat) * p.css * p.rhosoil + (s.wb[0] - s.wbice[0]) * R(CSWAT) * R(DENSITY_LIQ) +
                           s.wbice[0] * R(CSICE) * R(DENSITY_ICE), R2(xx)) * p.zse[0] +
                    R(1. - s.isflag) * R(CGSNOW) * s.snowd;
      s.first_soilsnow_call = false;
    }
    for (int k = 0; k < MS; ++k) {
      wblf[k] = mx(R2(0.01), (s.wb[k] - s.wbice[k])) / R2(p.ssat);
      wbfice[k] = R(s.wbice[k]) / p.ssat;
    }
    // ---- snowcheck (cbl_snowCheck.F90:9-100)
    if (s.snowd <= R(0.0)) {
      s.isflag = 0;
      for (int k = 0; k < 3; ++k) { s.ssdn[k] = R(120.0); s.tggsn[k] = R(TFRZ); }
      s.ssdnn = R(120.0);
      s.sdepth[0] = s.snowd / s.ssdn[0]; s.sdepth[1] = 0; s.sdepth[2] = 0;
      s.smass[0] = s.snowd; s.smass[1] = 0; s.smass[2] = 0;
    } else if (s.snowd < R(SNMIN) * s.ssdnn) {
      if (s.isflag == 1) { s.ssdn[0] = s.ssdnn; s.tgg[0] = s.tggsn[0]; }
      s.isflag = 0;
      s.ssdnn = mn(R(400.0), mx(R(120.0), s.ssdn[0]));
      for (int k = 0; k < 3; ++k) s.tggsn[k] = mn(R(TFRZ), s.tgg[0]);
      s.sdepth[0] = s.snowd / s.ssdn[0]; s.sdepth[1] = 0; s.sdepth[2] = 0;
      s.smass[0] = s.snowd; s.smass[1] = 0; s.smass[2] = 0;
      for (int k = 0; k < 3; ++k) s.ssdn[k] = s.ssdnn;
    } else {
      if (s.isflag == 0) {
        for (int k = 0; k < 3; ++k) s.tggsn[k] = mn(R(TFRZ), s.tgg[0]);
        s.ssdn[1] = s.ssdn[0]; s.ssdn[2] = s.ssdn[0];
        s.sdepth[0] = t_snwlr;
        s.smass[0] = t_snwlr * s.ssdn[0];
        s.smass[1] = (s.snowd - s.smass[0]) * R(0.4);
        s.smass[2] = (s.snowd - s.smass[0]) * R(0.6);
        s.sdepth[1] = s.smass[1] / s.ssdn[1];
        s.sdepth[2] = s.smass[2] / s.ssdn[2];
        s.ssdnn = (s.ssdn[0] * s.smass[0] + s.ssdn[1] * s.smass[1] + s.ssdn[2] * s.smass[2]) / s.snowd;
      }
      s.isflag = 1;
    }
    // ---- snowdensity (cbl_snowDensity.F90:9-102)
    R sconds[3] = {0, 0, 0};
    {
      R tmin1 = mn(R(TFRZ), s.tgg[0]);
      if (s.snowd > R(0.1) && s.isflag == 0) {
        s.ssdn[0] = mn(R(MAX_SSDN), mx(R(120.0), s.ssdn[0] + dels * s.ssdn[0] * R(3.1e-6) *
                                                         std::exp(R(-0.03) * (R(273.15) - tmin1) -
                                                                  ((s.ssdn[0] >= R(150.0)) ? R(0.046) : R(0.0)) * (s.ssdn[0] - R(150.0)))));
        s.ssdn[0] = mn(R(MAX_SSDN), s.ssdn[0] + dels * R(9.806) * s.ssdn[0] * R(0.75) * s.snowd /
                                                    (R(3.0e7) * std::exp(R(0.021) * s.ssdn[0] + R(0.081) * (R(273.15) - mn(R(TFRZ), s.tgg[0])))));
        if (p.isoilm != 9) s.ssdn[0] = mn(R(450.0), s.ssdn[0]);
        sconds[0] = mx(R(0.2), mn(R(2.876e-6) * sq(s.ssdn[0]) + R(0.074), R(MAX_SCONDS)));
        sconds[1] = sconds[0]; sconds[2] = sconds[0];
        s.ssdnn = s.ssdn[0];
        s.ssdn[1] = s.ssdn[0]; s.ssdn[2] = s.ssdn[0];
      }
      if (s.isflag == 1) {
        for (int k = 0; k < 3; ++k)
          s.ssdn[k] = s.ssdn[k] + dels * s.ssdn[k] * R(3.1e-6) *
                                      std::exp(R(-0.03) * (R(273.15) - mn(R(TFRZ), s.tggsn[k])) -
                                               ((s.ssdn[k] >= R(150.0)) ? R(0.046) : R(0.0)) * (s.ssdn[k] - R(150.0)));
        s.ssdn[0] = s.ssdn[0] + dels * R(9.806) * s.ssdn[0] * t_snwlr * s.ssdn[0] /
                                    (R(3.0e7) * std::exp(R(.021) * s.ssdn[0] + R(0.081) * (R(273.15) - mn(R(TFRZ), s.tggsn[0]))));
        s.ssdn[1] = s.ssdn[1] + dels * R(9.806) * s.ssdn[1] * (t_snwlr * s.ssdn[0] + R(0.5) * s.smass[1]) /
                                    (R(3.0e7) * std::exp(R(.021) * s.ssdn[1] + R(0.081) * (R(273.15) - mn(R(TFRZ), s.tggsn[1]))));
        s.ssdn[2] = s.ssdn[2] + dels * R(9.806) * s.ssdn[2] * (t_snwlr * s.ssdn[0] + s.smass[1] + R(0.5) * s.smass[2]) /
                                    (R(3.0e7) * std::exp(R(.021) * s.ssdn[2] + R(0.081) * (R(273.15) - mn(R(TFRZ), s.tggsn[2]))));
        for (int k = 0; k < 3; ++k) s.sdepth[k] = s.smass[k] / s.ssdn[k];
        s.ssdnn = (s.ssdn[0] * s.smass[0] + s.ssdn[1] * s.smass[1] + s.ssdn[2] * s.smass[2]) / s.snowd;
        for (int k = 0; k < 3; ++k) sconds[k] = mx(R(0.2), mn(R(2.876e-6) * sq(s.ssdn[k]) + R(0.074), R(MAX_SCONDS)));
      }
    }
    // ---- snow_accum (cbl_snowAccum.F90:10-188)
    R segg;
    {
      if (precis > R(0.0) && s.isflag == 0) {
        s.snowd = mx(s.snowd + met.precip_sn, R(0.0));
        precis = precis - met.precip_sn;
        s.ssdn[0] = mx(R(120.0), s.ssdn[0] * s.osnowd / mx(R(0.01), s.snowd) + R(120.0) * met.precip_sn / mx(R(0.01), s.snowd));
        s.ssdnn = s.ssdn[0];
        if (precis > R(0.0) && s.tgg[0] < R(TFRZ)) {
          s.snowd = mx(s.snowd + precis, R(0.0));
          s.tgg[0] = s.tgg[0] + precis * R(HLF) / (R(s.gammzz[0]) + R(CSWAT) * precis);
          dtmlt[0] = dtmlt[0] + precis * R(HLF) / (R(s.gammzz[0]) + R(CSWAT) * precis);
          s.ssdn[0] = mn(R(MAX_SSDN), mx(R(120.0), s.ssdn[0] * s.osnowd / mx(R(0.01), s.snowd) +
                                                        R(DENSITY_LIQ) * precis / mx(R(0.01), s.snowd)));
          if (p.isoilm != 9) s.ssdn[0] = mn(R(450.0), s.ssdn[0]);
          precis = R(0.0);
          s.ssdnn = s.ssdn[0];
        }
      }
      if (precis > R(0.0) && s.isflag > 0) {
        s.snowd = mx(s.snowd + met.precip_sn, R(0.0));
        precis = precis - met.precip_sn;
        R osm = s.smass[0];
        s.smass[0] = s.smass[0] + met.precip_sn;
        s.ssdn[0] = mx(R(120.0), s.ssdn[0] * osm / s.smass[0] + R(120.0) * met.precip_sn / s.smass[0]);
        s.sdepth[0] = mx(R(0.02), s.smass[0] / s.ssdn[0]);
        if (precis > R(0.0)) {
          s.snowd = mx(s.snowd + precis, R(0.0));
          R sgamm = s.ssdn[0] * R(CGSNOW) * s.sdepth[0];
          osm = s.smass[0];
          s.tggsn[0] = s.tggsn[0] + precis * R(HLF) * osm / (sgamm * s.osnowd);
          dtmlt[0] = dtmlt[0] + precis * R(HLF) * osm / (sgamm * s.osnowd);
          s.smass[0] = s.smass[0] + precis * osm / s.osnowd;
          s.ssdn[0] = mx(R(120.0), mn(s.ssdn[0] * osm / s.smass[0] + R(DENSITY_LIQ) * (R(1.0) - osm / s.smass[0]), R(MAX_SSDN)));
          if (p.isoilm != 9) s.ssdn[0] = mn(R(450.0), s.ssdn[0]);
          s.sdepth[0] = s.smass[0] / s.ssdn[0];
          for (int k = 1; k < 3; ++k) {
            sgamm = s.ssdn[k] * R(CGSNOW) * s.sdepth[k];
            osm = s.smass[k];
            s.tggsn[k] = s.tggsn[k] + precis * R(HLF) * osm / (sgamm * s.osnowd);
            s.smass[k] = s.smass[k] + precis * osm / s.osnowd;
            s.ssdn[k] = mx(R(120.0), mn(s.ssdn[k] * osm / s.smass[k] + R(DENSITY_LIQ) * (R(1.0) - osm / s.smass[k]), R(MAX_SSDN)));
            if (p.isoilm != 9) s.ssdn[k] = mn(R(450.0), s.ssdn[k]);
            s.sdepth[k] = s.smass[k] / s.ssdn[k];
          }
          precis = R(0.0);
        }
      }
      segg = R((fess + R2(0)) / R(HL));   // fes_cor is zero offline
      if (cls_snow) {
        R evapsn = R(dels * (fess + R2(0)) / (R(HL) + R(HLF)));
        R xxx = evapsn;
        if (s.isflag == 0 && fess + R2(0) > 0.0) evapsn = mn(s.snowd, xxx);
        if (s.isflag > 0 && fess + R2(0) > 0.0) evapsn = mn(R(0.9) * s.smass[0], xxx);
        s.snowd = s.snowd - evapsn;
        if (s.isflag > 0) {
          s.smass[0] = s.smass[0] - evapsn;
          s.sdepth[0] = mx(R(0.02), s.smass[0] / s.ssdn[0]);
        }
        segg = (R(HL) + R(HLF)) * (xxx - evapsn) / R(HL) / dels;
      }
    }
    // ---- snow_melting (cbl_snowMelt.F90:9-120), first call
    R snowmlt = snow_melting(p, s, dels, dtmlt);
    smelt = snowmlt;
    // ---- snowl_adjust (cbl_snowl_adjust.F90:9-156)
    if (s.isflag > 0) {
      R2 excd, excm;
      R osm;
      if (s.sdepth[0] > t_snwlr) {
        excd = s.sdepth[0] - t_snwlr;
        excm = excd * s.ssdn[0];
        s.sdepth[0] = s.sdepth[0] - R(excd);
        osm = s.smass[0];
        s.smass[0] = s.smass[0] - R(excm);
        osm = s.smass[1];
        s.smass[1] = mx(R(0.01), s.smass[1] + R(excm));
        s.ssdn[1] = R(mx(R2(120.0), mn(R2(MAX_SSDN), s.ssdn[1] * osm / s.smass[1] + s.ssdn[0] * excm / s.smass[1])));
        s.sdepth[1] = s.smass[1] / s.ssdn[1];
        s.tggsn[1] = R(s.tggsn[1] * osm / s.smass[1] + s.tggsn[0] * excm / s.smass[1]);
        s.smass[2] = mx(R(0.01), s.snowd - s.smass[0] - s.smass[1]);
      } else {
        excd = t_snwlr - s.sdepth[0];
        excm = excd * s.ssdn[1];
        osm = s.smass[0];
        s.smass[0] = s.smass[0] + R(excm);
        s.sdepth[0] = t_snwlr;
        s.ssdn[0] = R(mx(R2(120.0), mn(R2(MAX_SSDN), s.ssdn[0] * osm / s.smass[0] + s.ssdn[1] * excm / s.smass[0])));
        s.tggsn[0] = R(s.tggsn[0] * osm / s.smass[0] + s.tggsn[1] * excm / s.smass[0]);
        s.smass[1] = mx(R(0.01), s.smass[1] - R(excm));
        s.sdepth[1] = s.smass[1] / s.ssdn[1];
        s.smass[2] = mx(R(0.01), s.snowd - s.smass[0] - s.smass[1]);
      }
      R2 frac = s.smass[1] / mx(R(0.02), s.smass[2]);
      R2 xfrac = R(2.0) / R(3.0) / frac;
      if (xfrac > 1.0) {
        excm = (xfrac - 1.0) * s.smass[1];
        osm = s.smass[1];
        s.smass[1] = mx(R(0.01), s.smass[1] + R(excm));
        s.tggsn[1] = s.tggsn[1] * osm / s.smass[1] + s.tggsn[2] * R(excm) / s.smass[1];
        s.ssdn[1] = mx(R(120.0), mn(R(MAX_SSDN), s.ssdn[1] * osm / s.smass[1] + s.ssdn[2] * R(excm) / s.smass[1]));
        s.smass[2] = mx(R(0.01), s.snowd - s.smass[0] - s.smass[1]);
        s.sdepth[2] = mx(R(0.02), s.smass[2] / s.ssdn[2]);
      } else {
        excm = (1 - xfrac) * s.smass[1];
        s.smass[1] = mx(R(0.01), s.smass[1] - R(excm));
        s.sdepth[1] = mx(R(0.02), s.smass[1] / s.ssdn[1]);
        osm = s.smass[2];
        s.smass[2] = mx(R(0.01), s.snowd - s.smass[0] - s.smass[1]);
        s.tggsn[2] = s.tggsn[2] * osm / s.smass[2] + s.tggsn[1] * R(excm) / s.smass[2];
        s.ssdn[2] = mx(R(120.0), mn(R(MAX_SSDN), s.ssdn[2] * osm / s.smass[2] + s.ssdn[1] * R(excm) / s.smass[2]));
        s.sdepth[2] = s.smass[2] / s.ssdn[2];
      }
      s.isflag = 1;
      s.ssdnn = (s.ssdn[0] * s.sdepth[0] + s.ssdn[1] * s.sdepth[1] + s.ssdn[2] * s.sdepth[2]) /
                (s.sdepth[0] + s.sdepth[1] + s.sdepth[2]);
    }
    // ---- stempv (cbl_stempv.F90:13-221)
    {
      R2 ccnsw[MS];
      // total_soil_conductivity (cbl_conductivity.F90:10-85), cbl_stempv.F90:57-61;
      // r_2 arithmetic with default-REAL literals promoted
      for (int k = 0; k < MS && soil_thermal_fix; ++k) {
        if (p.isoilm == 9) {
          ccnsw[k] = R2(R(SNOW_CCNSW));
          continue;
        }
        const R2 quartz = mx(R2(0.0), mn(R2(0.8f), p.sand_vec * R2(0.92f)));
        const R2 Ko = quartz > R2(0.2f) ? R2(2.0) : R2(3.0);
        const R2 Ktmp = std::pow(std::pow(R2(7.7f), quartz) * std::pow(Ko, R2(1.0) - quartz), R2(1.0) - p.ssat_vec);
        const R2 wbliq = s.wb[k] - s.wbice[k];   // cbl_soilsnow_main.F90:87
        const R2 liq_frac = s.wb[k] >= R2(1.0e-15f) ? mn(R2(1.0), mx(R2(0.0), wbliq / s.wb[k])) : R2(0.0);
        const R2 Ksat = Ktmp * std::pow(R2(2.2f), p.ssat_vec * (R2(1.0) - liq_frac)) * std::pow(R2(0.57f), liq_frac);
        const R2 Sr = mn(R2(0.9999f), mx(R2(0.0), s.wb[k] - p.watr) / (p.ssat_vec - p.watr));
        R2 Ke = Sr >= R2(0.05f) ? R2(0.7f) * std::log10(Sr) + R2(1.0) : R2(0.0);
        if (s.wbice[k] > R2(0.0) || s.tgg[k] < R(TFRZ) || s.isflag != 0 || s.snowd >= R(0.1f)) Ke = Sr;
        const R2 kk = Ke * Ksat + (R2(1.0) - Ke) * p.cnsd_vec;
        ccnsw[k] = mn(Ksat, mx(p.cnsd_vec, kk));
      }
      for (int k = 0; k < MS && !soil_thermal_fix; ++k) {   // old_soil_conductivity (cbl_Oldconductivity.F90:7-59)
        if (p.isoilm == 9) {
          ccnsw[k] = R(SNOW_CCNSW);
        } else {
          R ew = R(wblf[k] * p.ssat);
          R exp_arg = R(R2(ew * std::log(R(60.0))) + wbfice[k] * p.ssat * std::log(R(250.0)));
          R2 f2 = mx(R2(1.0), std::sqrt(mn(R2(2.0), R2(R(0.5) * p.ssat) / mn(R2(ew), R2(0.5) * p.ssat))));
          if (exp_arg > R(30)) ccnsw[k] = R(1.5) * f2;
          else ccnsw[k] = mn(p.cnsd * std::exp(exp_arg), R2(1.5)) * f2;
        }
      }
      R2 at[9], bt[9], ct[9], coeff[10];
      for (int k = 0; k < 9; ++k) { at[k] = 0.0; bt[k] = 1.0; ct[k] = 0.0; }
      for (int k = 0; k < 10; ++k) coeff[k] = 0.0;
      // row index j = k + 2 for soil layer k (k=1..ms), j = k-1 for snow layer k=1..3 (rows -2..0)
      // coeff index m = i + 2 for Fortran coeff(i), i = -2..ms+1
      auto C = [&](int i) -> R2& { return coeff[i + 2]; };
      auto A = [&](int i) -> R2& { return at[i + 2]; };
      auto B = [&](int i) -> R2& { return bt[i + 2]; };
      auto Cc = [&](int i) -> R2& { return ct[i + 2]; };
      R coefa = 0, coefb = 0;
      R2 xx = 0;
      if (s.isflag == 0) {
        xx = mx(R(0.), s.snowd / s.ssdnn);
        ccnsw[0] = (ccnsw[0] - R(0.2)) * (p.zse[0] / (p.zse[0] + xx)) + R(0.2);
        for (int k = 3; k <= MS; ++k) C(k) = 2.0 / (p.zse[k - 2] / ccnsw[k - 2] + p.zse[k - 1] / ccnsw[k - 1]);
        C(2) = 2.0 / ((p.zse[0] + xx) / ccnsw[0] + p.zse[1] / ccnsw[1]);
        coefa = 0.0;
        coefb = R(C(2));
        s.gammzz[0] = mx(R2(hcll[0]), (R(1.0) - p.ssat) * p.css * p.rhosoil +
                                           p.ssat * (wblf[0] * R(CSWAT) * R(DENSITY_LIQ) + wbfice[0] * R(CSICE) * R(DENSITY_ICE))) * p.zse[0];
        s.gammzz[0] = s.gammzz[0] + R(CGSNOW) * s.snowd;
        R2 dtg = dels / s.gammzz[0];
        A(1) = -dtg * C(1); Cc(1) = -dtg * C(2); B(1) = 1.0 - A(1) - Cc(1);
        for (int k = 2; k <= MS; ++k) {
          s.gammzz[k - 1] = mx(R2(hcll[k - 1]), (R(1.0) - p.ssat) * p.css * p.rhosoil +
                                                    p.ssat * (wblf[k - 1] * R(CSWAT) * R(DENSITY_LIQ) + wbfice[k - 1] * R(CSICE) * R(DENSITY_ICE))) * p.zse[k - 1];
          dtg = dels / s.gammzz[k - 1];
          A(k) = -dtg * C(k); Cc(k) = -dtg * C(k + 1); B(k) = 1.0 - A(k) - Cc(k);
        }
        B(1) = B(1) - dgdtg * dels / s.gammzz[0];
        s.tgg[0] = s.tgg[0] + (ga - s.tgg[0] * R(dgdtg)) * dels / R(s.gammzz[0]);
      }
      C(-2) = 0.0;
      if (s.isflag != 0) {
        for (int k = 0; k < 3; ++k) sconds[k] = mx(R(0.2), mn(R(2.876e-6) * sq(s.ssdn[k]) + R(0.074), R(MAX_SCONDS)));
        C(-1) = 2.0 / (s.sdepth[0] / sconds[0] + s.sdepth[1] / sconds[1]);
        C(0) = 2.0 / (s.sdepth[1] / sconds[1] + s.sdepth[2] / sconds[2]);
        C(1) = 2.0 / (s.sdepth[2] / sconds[2] + p.zse[0] / ccnsw[0]);
        for (int k = 2; k <= MS; ++k) C(k) = 2.0 / (p.zse[k - 2] / ccnsw[k - 2] + p.zse[k - 1] / ccnsw[k - 1]);
        coefa = R(C(-1));
        coefb = R(C(1));
        for (int k = 1; k <= 3; ++k) {
          R sgamm = s.ssdn[k - 1] * R(CGSNOW) * s.sdepth[k - 1];
          R2 dtg = dels / sgamm;
          A(k - 3) = -dtg * C(k - 3); Cc(k - 3) = -dtg * C(k - 2); B(k - 3) = 1.0 - A(k - 3) - Cc(k - 3);
        }
        for (int k = 1; k <= MS; ++k) {
          s.gammzz[k - 1] = mx((R(1.0) - p.ssat) * p.css * p.rhosoil +
                                   p.ssat * (wblf[k - 1] * R(CSWAT) * R(DENSITY_LIQ) + wbfice[k - 1] * R(CSICE) * R(DENSITY_ICE)),
                               R2(hcll[k - 1])) * p.zse[k - 1];
          R2 dtg = dels / s.gammzz[k - 1];
          A(k) = -dtg * C(k); Cc(k) = -dtg * C(k + 1); B(k) = 1.0 - A(k) - Cc(k);
        }
        R sgamm = s.ssdn[0] * R(CGSNOW) * s.sdepth[0];
        B(-2) = B(-2) - dgdtg * dels / sgamm;
        s.tggsn[0] = s.tggsn[0] + (ga - s.tggsn[0] * R(dgdtg)) * dels / sgamm;
      }
      R2 tmp_mat[9];
      for (int k = 0; k < 3; ++k) tmp_mat[k] = R2(s.tggsn[k]);
      for (int k = 0; k < MS; ++k) tmp_mat[3 + k] = R2(s.tgg[k]);
      trimb(at, bt, ct, tmp_mat, MS + 3);
      for (int k = 0; k < 3; ++k) s.tggsn[k] = R(tmp_mat[k]);
      for (int k = 0; k < MS; ++k) s.tgg[k] = R(tmp_mat[3 + k]);
      o.sghflux = coefa * (s.tggsn[0] - s.tggsn[1]);
      o.ghflux = coefb * (s.tgg[0] - s.tgg[1]);
    }
    s.tss = R(1 - s.isflag) * s.tgg[0] + R(s.isflag) * s.tggsn[0];
    // ---- snow_melting, second call
    snowmlt = snow_melting(p, s, dels, dtmlt);
    smelt = smelt + snowmlt;
    // ---- remove_trans (cbl_remove_trans.F90:9-40)
    if (fevc < 0.0) { fevw = R(fevw + fevc); fevc = 0.0; }
    for (int k = 0; k < MS; ++k) {
      wbliq[k] = wbliq[k] - evapfbl[k] / (p.zse_vec[k] * R(DENSITY_LIQ));
      s.wb[k] = wbliq[k] + s.wbice[k];
    }
    // ---- soilfreeze (cbl_soilfreeze.F90:9-81)
    for (int k = 0; k < MS; ++k) {
      if (s.tgg[k] < R(TFRZ) && R(FROZEN_LIMIT) * s.wb[k] - s.wbice[k] > .001) {
        R2 sicefreeze = mn(R(FROZEN_LIMIT) * s.wb[k] - s.wbice[k],
                           (p.ssat - s.wb[k]) / mx(R(1.0) - R(DENSITY_ICE) / R(DENSITY_LIQ), R(1.0E-3)));
        sicefreeze = mn(mx(R2(0.0), sicefreeze) * p.zse[k] * R(DENSITY_ICE), (R(TFRZ) - s.tgg[k]) * s.gammzz[k] / R(HLF));
        s.wbice[k] = mn(s.wbice[k] + sicefreeze / (p.zse[k] * R(DENSITY_ICE)), R(FROZEN_LIMIT) * s.wb[k]);
        s.wb[k] = s.wb[k] + sicefreeze / (p.zse[k] * R(DENSITY_ICE)) - sicefreeze / (p.zse[k] * R(DENSITY_LIQ));
        R max_arg1 = hcll[k];
        R max_arg2 = R(R2((R(1.0) - p.ssat) * p.css * p.rhosoil) + (s.wb[k] - s.wbice[k]) * R2(R(CSWAT) * R(DENSITY_LIQ)) +
                       s.wbice[k] * R2(R(CSICE) * R(DENSITY_ICE)));
        s.gammzz[k] = mx(max_arg1, max_arg2) * R2(p.zse[k]);
        if (k == 0 && s.isflag == 0) s.gammzz[k] = s.gammzz[k] + R(CGSNOW) * s.snowd;
        s.tgg[k] = s.tgg[k] + R(sicefreeze) * R(HLF) / R(s.gammzz[k]);
      } else if (s.tgg[k] > R(TFRZ) && s.wbice[k] > 0.) {
        R2 sicemelt = mn(s.wbice[k] * p.zse[k] * R(DENSITY_ICE), (s.tgg[k] - R(TFRZ)) * s.gammzz[k] / R(HLF));
        s.wbice[k] = mx(R2(0.0), s.wbice[k] - sicemelt / (p.zse[k] * R(DENSITY_ICE)));
        s.wb[k] = s.wb[k] - sicemelt / (p.zse[k] * R(DENSITY_ICE)) + sicemelt / (p.zse[k] * R(DENSITY_LIQ));
        R max_arg1 = hcll[k];
        R max_arg2 = R(R2((R(1.0) - p.ssat) * p.css * p.rhosoil) + (s.wb[k] - s.wbice[k]) * R2(R(CSWAT) * R(DENSITY_LIQ)) +
                       s.wbice[k] * R2(R(CSICE) * R(DENSITY_ICE)));
        s.gammzz[k] = mx(max_arg1, max_arg2) * R2(p.zse[k]);
        if (k == 0 && s.isflag == 0) s.gammzz[k] = s.gammzz[k] + R(CGSNOW) * s.snowd;
        s.tgg[k] = s.tgg[k] - R(sicemelt) * R(HLF) / R(s.gammzz[k]);
      }
    }
    // ---- infiltration (cbl_soilsnow_main.F90:139-159)
    R totwet = precis + smelt;
    R weting = R(totwet + mx(R2(0.), s.pudsto - fesp / R(HL) * dels));
    R2 xxx = p.ssat - s.wb[0];
    R2 sinfil1 = mn(R(0.95) * xxx * p.zse[0] * R(DENSITY_LIQ), R2(weting));
    xxx = p.ssat - s.wb[1];
    R2 sinfil2 = mn(R(0.95) * xxx * p.zse[1] * R(DENSITY_LIQ), R2(weting - R(sinfil1)));
    xxx = p.ssat - s.wb[2];
    R2 sinfil3 = mn(R(0.95) * xxx * p.zse[2] * R(DENSITY_LIQ), R2(weting - R(sinfil1) - R(sinfil2)));
    fwtop1 = R(sinfil1 / dels - segg);
    fwtop2 = R(sinfil2 / dels);
    fwtop3 = R(sinfil3 / dels);
    s.pudsto = R(mx(R2(0.), weting - sinfil1 - sinfil2 - sinfil3));
    rnof1 = mx(R(0.), s.pudsto - s.pudsmx);
    s.pudsto = s.pudsto - rnof1;
    // ---- surfbv (cbl_surfbv.F90:9-146) -> smoisturev (cbl_smoisturev.F90:11-444, nmeth = -1)
    {
      R2 at[MS], bt[MS], ct[MS], fluxh[MS + 1], delt[MS + 1], dtt[MS];
      for (int k = 0; k < MS; ++k) { at[k] = 0.0; bt[k] = 1.0; ct[k] = 0.0; }
      delt[0] = 0.0; fluxh[0] = 0.0; fluxh[MS] = 0.0;
      const R2 wbl_min = new_runoff_speed ? R2(0.001) : R2(0.01);
      for (int k = 1; k <= MS - 1; ++k) {
        R2 wbl_k = mx(wbl_min, s.wb[k - 1] - s.wbice[k - 1]);
        R2 wbl_kp = mx(wbl_min, s.wb[k] - s.wbice[k]);
        delt[k] = wbl_kp - wbl_k;
        R2 wh = mn(wbl_k, wbl_kp);
        if (s.wbice[k - 1] > 0.05 || s.wbice[k] > 0.01) wh = 0.9 * wbl_k + 0.1 * wbl_kp;
        R2 hydss = p.hyds;
        R2 speed_k = hydss * std::pow(wh / p.ssat, R2(p.i2bp3 - R(1)));
        R2 rat = delt[k - 1] / (delt[k] + fsign(R2(R(1.0e-20)), delt[k]));
        R2 phi = mx(mx(R2(0.0), mn(R2(1.0), R2(2.0) * rat)), mn(R2(2.0), rat));
        R2 fluxhi = wh, fluxlo = wbl_k;
        speed_k = mn(speed_k, R2(R(0.5) * p.zse[k - 1] / dels));
        fluxh[k] = speed_k * (fluxlo + phi * (fluxhi - fluxlo));
      }
      if (s.wb[MS - 1] > p.sfc) {
        R2 wbl_k = mx(R2(0.001), s.wb[MS - 1] - s.wbice[MS - 1]);
        R2 wbl_kp = mx(R2(0.001), p.ssat - s.wbice[MS - 1]);
        R2 wh = mn(wbl_k, wbl_kp);
        if (s.wbice[MS - 1] > 0.05) wh = 0.9 * wbl_k + 0.1 * wbl_kp;
        R2 speed_k = p.hyds * std::pow(wh / p.ssat, R2(p.i2bp3 - R(1)));
        if (new_runoff_speed) {   // :180-197
          speed_k = speed_k / (1. - mn(R2(0.5), 10. * s.wbice[MS - 1]));
          speed_k = mn(speed_k, R2(R(0.5) * p.zse[MS - 1] / dels));
        } else {
          speed_k = 0.5 * speed_k / (1. - mn(R2(0.5), 10. * s.wbice[MS - 1]));
          speed_k = mn(0.5 * speed_k, R2(0.5) * p.zse[MS - 1] / dels);
        }
        R2 fluxlo = wbl_k;
        fluxh[MS] = mx(R2(0.0), speed_k * fluxlo);
      }
      for (int k = MS; k >= 1; --k) {
        fluxh[k - 1] = mn(fluxh[k - 1], (p.ssat - s.wb[k - 1]) * p.zse[k - 1] / dels + fluxh[k]);
        s.wb[k - 1] = s.wb[k - 1] + dels * (fluxh[k - 1] - fluxh[k]) / p.zse[k - 1];
        R2 ssatcurr_k = p.ssat - s.wbice[k - 1];
        dtt[k - 1] = dels / (p.zse[k - 1] * ssatcurr_k);
        wblf[k - 1] = (s.wb[k - 1] - s.wbice[k - 1]) / ssatcurr_k;
      }
      rnof2 = dels * R(fluxh[MS]) * R(DENSITY_LIQ);
      for (int k = 2; k <= MS; ++k) {
        R2 wbh_k = (p.zse[k - 1] * wblf[k - 2] + p.zse[k - 2] * wblf[k - 1]) / (p.zse[k - 1] + p.zse[k - 2]);
        R2 fact = std::pow(wbh_k, R2(p.ibp2 - R(1)));
        R2 icef = mx(s.wbice[k - 2] / mx(R2(0.01), s.wb[k - 2]), s.wbice[k - 1] / mx(R2(0.01), s.wb[k - 1]));
        R2 pwb_wbh = (p.hsbh * (1. - mn(2. * mn(R2(0.1), icef), R2(0.1)))) * mx(p.pwb_min, wbh_k * fact);
        R2 z3_k = pwb_wbh / p.zshh[k - 1];
        at[k - 1] = -dtt[k - 1] * z3_k;
        ct[k - 2] = -dtt[k - 2] * z3_k;
      }
      for (int k = 0; k < MS; ++k) bt[k] = 1. - at[k] - ct[k];
      wblf[0] = wblf[0] + dtt[0] * fwtop1 / R(DENSITY_LIQ);
      wblf[1] = wblf[1] + dtt[1] * fwtop2 / R(DENSITY_LIQ);
      wblf[2] = wblf[2] + dtt[2] * fwtop3 / R(DENSITY_LIQ);
      trimb(at, bt, ct, wblf, MS);
      for (int k = 0; k < MS; ++k) {
        R2 ssatcurr = p.ssat - s.wbice[k];
        s.wb[k] = wblf[k] * ssatcurr + s.wbice[k];
      }
      const R dfactor = R(1.0) - R(DENSITY_ICE) / R(DENSITY_LIQ);
      for (int k = 0; k < MS; ++k) {
        if (s.wbice[k] > R(FROZEN_LIMIT) * s.wb[k]) {
          R sicemelt = R((s.wbice[k] - R(FROZEN_LIMIT) * s.wb[k]) / (R(1.0) - R(FROZEN_LIMIT) * dfactor));
          s.wbice[k] = s.wbice[k] - sicemelt;
          s.wb[k] = s.wb[k] - dfactor * sicemelt;
          s.tgg[k] = s.tgg[k] - sicemelt * p.zse[k] * R(DENSITY_ICE) * R(HLF) / R(s.gammzz[k]);
        }
      }
    }
    // surfbv remainder
    for (int k = 0; k < MS; ++k) {
      R2 xs = R2(p.ssat);
      rnof1 = rnof1 + R(mx(s.wb[k] - xs, R2(0.0)) * R(DENSITY_LIQ)) * p.zse[k];
      s.wb[k] = mx(R2(p.swilt / (R(2.) * R(WILT_LIMITFACTOR))), mn(s.wb[k], xs));
    }
    R rnof5 = 0;
    {
      R smelt1[3] = {0, 0, 0};
      R smasstot = 0;
      if (s.snowd > R(MAX_GLACIER_SNOWD)) {
        rnof5 = mn(R(0.1), s.snowd - R(MAX_GLACIER_SNOWD));
        if (s.isflag == 0) {
          smasstot = 0.0;
          s.tgg[0] = s.tgg[0] - rnof5 * R(HLF) / R(s.gammzz[0]);
          s.snowd = s.snowd - rnof5;
        } else {
          smasstot = s.smass[0] + s.smass[1] + s.smass[2];
        }
      }
      for (int k = 0; k < 3; ++k) {
        if (s.snowd > R(MAX_GLACIER_SNOWD) && s.isflag > 0) {
          smelt1[k] = mn(rnof5 * s.smass[k] / smasstot, R(0.2) * s.smass[k]);
          s.smass[k] = s.smass[k] - smelt1[k];
          s.snowd = s.snowd - smelt1[k];
        }
      }
      if (s.isflag > 0) rnof5 = smelt1[0] + smelt1[1] + smelt1[2];
    }
    if (p.iveg == LAKES) {
      R sinfil = mn(rnof1, s.wb_lake);
      rnof1 = mx(R(0.0), rnof1 - sinfil);
      s.wb_lake = mx(R(0.0), s.wb_lake - sinfil);
      sinfil = mn(rnof2, s.wb_lake);
      rnof2 = mx(R(0.0), rnof2 - sinfil);
      s.wb_lake = mx(R(0.0), s.wb_lake - sinfil);
      R2 xl = mx(R2(0.0), (s.wb[MS - 1] - R2(p.sfc)) * p.zse[MS - 1] * R(DENSITY_LIQ));
      sinfil = mn(R(xl), s.wb_lake);
      s.wb[MS - 1] = s.wb[MS - 1] - R2(sinfil / (p.zse[MS - 1] * R(DENSITY_LIQ)));
      s.wb_lake = mx(R(0.0), s.wb_lake - sinfil);
      xl = mx(R2(0.0), (s.wb[MS - 1] - R(0.5) * (p.sfc + p.swilt)) * p.zse[MS - 1] * R(DENSITY_LIQ));
      sinfil = mn(R(xl), s.wb_lake);
      s.wb[MS - 1] = s.wb[MS - 1] - sinfil / (p.zse[MS - 1] * R(DENSITY_LIQ));
      s.wb_lake = mx(R(0.0), s.wb_lake - sinfil);
    }
    rnof1 = rnof1 / dels + rnof5 / dels;
    rnof2 = rnof2 / dels;
    o.rnof1 = rnof1; o.rnof2 = rnof2; o.runoff = rnof1 + rnof2;
    o.smelt = smelt / dels;
    s.tss = R(1 - s.isflag) * s.tgg[0] + R(s.isflag) * s.tggsn[0];
    R2 wbtot = 0;
    for (int k = 0; k < MS; ++k) {
      R2 wl = s.wb[k] - s.wbice[k];
      wbtot = wbtot + (wl * R(DENSITY_LIQ) + s.wbice[k] * R(DENSITY_ICE)) * p.zse[k];
    }
    o.wbtot = wbtot;
    o.dtmlt1 = dtmlt[0];   // ssnow%dtmlt(:,1), read by the coupled corrections
  }

  // snow_melting (cbl_snowMelt.F90:9-120); returns snowmlt
  static R snow_melting(const P& p, S& s, R dels, R dtmlt[3]) {
    R snowmlt = 0;
    R smelt1[4] = {0, 0, 0, 0};
    if (s.snowd > R(0.0) && s.isflag == 0 && s.tgg[0] >= R(TFRZ)) {
      R snowflx = R((s.tgg[0] - R(TFRZ)) * s.gammzz[0]);
      snowmlt = mn(snowflx / R(HLF), s.snowd);
      dtmlt[0] = R(dtmlt[0] + snowmlt * R(HLF) / s.gammzz[0]);
      s.snowd = s.snowd - snowmlt;
      s.tgg[0] = R(s.tgg[0] - snowmlt * R(HLF) / s.gammzz[0]);
    }
    smelt1[0] = 0.0;
    for (int k = 1; k <= 3; ++k) {
      if (s.snowd > R(0.0) && s.isflag > 0) {
        R sgamm = s.ssdn[k - 1] * R(CGSNOW) * s.sdepth[k - 1];
        R snowflx = smelt1[k - 1] * R(HLF) / dels;
        s.tggsn[k - 1] = s.tggsn[k - 1] + (snowflx * dels + smelt1[k - 1] * R(CSWAT) * (R(TFRZ) - s.tggsn[k - 1])) /
                                              (sgamm + R(CSWAT) * smelt1[k - 1]);
        R osm = s.smass[k - 1];
        s.smass[k - 1] = s.smass[k - 1] + smelt1[k - 1];
        s.ssdn[k - 1] = mx(R(120.0), mn(s.ssdn[k - 1] * osm / s.smass[k - 1] + R(DENSITY_LIQ) * (R(1.0) - osm / s.smass[k - 1]), R(MAX_SSDN)));
        if (p.isoilm != 9) s.ssdn[k - 1] = mn(R(450.0), s.ssdn[k - 1]);
        s.sdepth[k - 1] = s.smass[k - 1] / s.ssdn[k - 1];
        sgamm = s.smass[k - 1] * R(CGSNOW);
        smelt1[k - 1] = R(0.0);
        smelt1[k] = R(0.0);
        if (s.tggsn[k - 1] > R(TFRZ)) {
          snowflx = (s.tggsn[k - 1] - R(TFRZ)) * sgamm;
          smelt1[k] = mn(snowflx / R(HLF), R(0.6) * s.smass[k - 1]);
          dtmlt[k - 1] = dtmlt[k - 1] + smelt1[k] * R(HLF) / sgamm;
          osm = s.smass[k - 1];
          s.smass[k - 1] = s.smass[k - 1] - smelt1[k];
          s.tggsn[k - 1] = s.tggsn[k - 1] - smelt1[k] * R(HLF) / sgamm;
          s.sdepth[k - 1] = s.smass[k - 1] / s.ssdn[k - 1];
        }
      }
    }
    if (s.snowd > R(0.0) && s.isflag > 0) {
      snowmlt = smelt1[1] + smelt1[2] + smelt1[3];
      s.snowd = s.snowd - snowmlt;
    }
    return snowmlt;
  }

};

}  // namespace cbmref
