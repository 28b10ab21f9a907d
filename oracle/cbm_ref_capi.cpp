// ORACLE / TEST INFRASTRUCTURE ONLY.
// C entry points of the CPU restatement, loaded by tests/ and by bench.py's
// CPU-baseline leg through ctypes.  Never linked by the product.
//
// Per-tile set-up follows the reference initialisation:
//   veg parameters  src/offline/cable_parameters.F90:3277-3345 (froot from
//                   rootbeta :3331-3343), dleaf cable_pft_params.F90:110,
//                   ejmax = 2 vcmax cable_parameters.F90:1543, meth = 1 :1262
//   soil parameters cable_parameters.F90:1511-1522, derived :2236-2245,
//                   zshh :1828-1831, zse :1241, cnsd from the in-source
//                   texture formula :2230
//   initial state   cable_parameters.F90:1188-1262 and :1607-1650,
//                   cable_initialise.F90:72-144, owetfac :2246-2254,
//                   tss = tgg(1) cable_serial.F90:439
#include <cstdint>
#include <cstring>
#include <vector>
#include <string>
#include "cbm_ref.hpp"
#include "forcing_ref.hpp"

using namespace cbmref;

namespace {

// ---------------------------------------------------------------- state map
struct Slot { const char* name; int width; };
const Slot kState[] = {
  {"wb", MS}, {"wbice", MS}, {"gammzz", MS}, {"tgg", MS}, {"tggsn", MSN}, {"ssdn", MSN}, {"smass", MSN},
  {"sdepth", MSN}, {"isflag", 1}, {"snowd", 1}, {"ssdnn", 1}, {"snage", 1}, {"pudsto", 1}, {"owetfac", 1},
  {"rtsoil", 1}, {"tss", 1}, {"wb_lake", 1}, {"wbtot1", 1}, {"wbtot2", 1}, {"cansto", 1}, {"cplant", 3},
  {"csoil", 2}, {"owb", 1}, {"ebal_tot", 1}, {"wbal_tot", 1}, {"first_call", 1}, {"ga", 1}, {"vlaiw", 1},
};
constexpr int kNState = sizeof(kState) / sizeof(kState[0]);
int state_slots() { int n = 0; for (auto& s : kState) n += s.width; return n; }

const char* kDiag[] = {
  "fe", "fh", "fev", "fhv", "fhs", "fns", "fnv", "ga", "tv", "tscrn", "qscrn", "rnet", "us", "cduv", "cdtq", "epot",
  "fes", "fevc", "dgdtg", "fevw", "fpn", "frday", "fgpp", "fnpp", "fnee", "fra", "frp", "frs", "trad",
  "albedo_vis", "albedo_nir", "transd", "precis", "through", "fwet", "wetfac", "potev", "runoff", "rnof1", "rnof2",
  "smelt", "ghflux", "sghflux", "drybal", "wetbal", "ebal", "wbal", "qssabs", "rniso", "vlaiw", "tvair", "qvair",
  "swnet", "lwnet", "wbtot", "gswx_sun", "gswx_shd", "fwsoil", "dryleaf_passes", "dryleaf_noconv", "evapfbl_err", "delwc", "cls", "frpw", "frpr",
};
constexpr int kNDiag = sizeof(kDiag) / sizeof(kDiag[0]);

template <class R, class R2>
void pack_state(const State<R, R2>& s, double* st, int mp, int t) {
  int j = 0;
  auto put = [&](double v) { st[(size_t)(j++) * mp + t] = v; };
  for (int k = 0; k < MS; ++k) put(s.wb[k]);
  for (int k = 0; k < MS; ++k) put(s.wbice[k]);
  for (int k = 0; k < MS; ++k) put(s.gammzz[k]);
  for (int k = 0; k < MS; ++k) put(s.tgg[k]);
  for (int k = 0; k < MSN; ++k) put(s.tggsn[k]);
  for (int k = 0; k < MSN; ++k) put(s.ssdn[k]);
  for (int k = 0; k < MSN; ++k) put(s.smass[k]);
  for (int k = 0; k < MSN; ++k) put(s.sdepth[k]);
  put(s.isflag); put(s.snowd); put(s.ssdnn); put(s.snage); put(s.pudsto); put(s.owetfac); put(s.rtsoil);
  put(s.tss); put(s.wb_lake); put(s.wbtot1); put(s.wbtot2); put(s.cansto);
  for (int k = 0; k < 3; ++k) put(s.cplant[k]);
  for (int k = 0; k < 2; ++k) put(s.csoil[k]);
  put(s.owb); put(s.ebal_tot); put(s.wbal_tot); put(s.first_soilsnow_call ? 1.0 : 0.0); put(s.ga);
  put(s.vlaiw);
}

template <class R, class R2>
void unpack_state(State<R, R2>& s, const double* st, int mp, int t) {
  int j = 0;
  auto get = [&]() { return st[(size_t)(j++) * mp + t]; };
  for (int k = 0; k < MS; ++k) s.wb[k] = R2(get());
  for (int k = 0; k < MS; ++k) s.wbice[k] = R2(get());
  for (int k = 0; k < MS; ++k) s.gammzz[k] = R2(get());
  for (int k = 0; k < MS; ++k) s.tgg[k] = R(get());
  for (int k = 0; k < MSN; ++k) s.tggsn[k] = R(get());
  for (int k = 0; k < MSN; ++k) s.ssdn[k] = R(get());
  for (int k = 0; k < MSN; ++k) s.smass[k] = R(get());
  for (int k = 0; k < MSN; ++k) s.sdepth[k] = R(get());
  s.isflag = (int)get(); s.snowd = R(get()); s.ssdnn = R(get()); s.snage = R(get()); s.pudsto = R(get());
  s.owetfac = R(get()); s.rtsoil = R(get()); s.tss = R(get()); s.wb_lake = R(get()); s.wbtot1 = R(get());
  s.wbtot2 = R(get()); s.cansto = R(get());
  for (int k = 0; k < 3; ++k) s.cplant[k] = R(get());
  for (int k = 0; k < 2; ++k) s.csoil[k] = R(get());
  s.owb = R2(get()); s.ebal_tot = R2(get()); s.wbal_tot = R2(get()); s.first_soilsnow_call = get() != 0.0;
  s.ga = R(get());
  s.vlaiw = R(get());
  s.pudsmx = 0; s.osnowd = s.snowd;
}

template <class R, class R2>
void pack_diag(const Diag<R, R2>& d, double* dg, int mp, int t) {
  const double v[kNDiag] = {
    d.fe, d.fh, d.fev, d.fhv, d.fhs, d.fns, d.fnv, d.ga, d.tv, d.tscrn, d.qscrn, d.rnet, d.us, d.cduv, d.cdtq, d.epot,
    (double)d.fes, (double)d.fevc, (double)d.dgdtg, d.fevw, d.fpn, d.frday, d.fgpp, d.fnpp, d.fnee, d.fra, d.frp, d.frs, d.trad,
    d.albedo[0], d.albedo[1], d.transd, d.precis, d.through, d.fwet, d.wetfac, d.potev, d.runoff, d.rnof1, d.rnof2,
    d.smelt, d.ghflux, d.sghflux, d.drybal, d.wetbal, d.ebal, d.wbal, d.qssabs, d.rniso, d.vlaiw, d.tvair, d.qvair,
    d.swnet, d.lwnet, (double)d.wbtot, d.gswx[0], d.gswx[1], d.fwsoil, (double)d.dryleaf_passes,
    (double)d.dryleaf_noconv, (double)d.evapfbl_err, d.delwc, d.cls, d.frpw, d.frpr,
  };
  for (int i = 0; i < kNDiag; ++i) dg[(size_t)i * mp + t] = v[i];
}

// ---------------------------------------------------------------- set-up
template <class R, class R2>
void make_params(Params<R, R2>& p, int iveg, int isoilm, double vlai, double lat, bool thermal_fix = false) {
  const PftTable& V = pft_table();
  const SoilTable& T = soil_table();
  const int v = iveg - 1, s = isoilm - 1;
  p.iveg = iveg; p.isoilm = isoilm;
  p.vlai = (iveg >= 14) ? R(0) : R(vlai);   // cable_serial.F90:575
  p.lat = R(lat);
  p.canst1 = R(V.canst1[v]);
  p.dleaf = std::sqrt(R(V.width[v]) * R(V.length[v]));
  p.vcmax = R(V.vcmax[v]);
  p.ejmax = R(2.0) * p.vcmax;
  p.frac4 = R(V.frac4[v]); p.hc = R(V.hc[v]); p.vbeta = R(V.vbeta[v]); p.rp20 = R(V.rp20[v]); p.rs20 = R(V.rs20[v]);
  p.shelrb = R(V.shelrb[v]); p.vegcf = R(V.vegcf[v]); p.extkn = R(V.extkn[v]); p.a1gs = R(V.a1gs[v]);
  p.d0gs = R(V.d0gs[v]); p.alpha = R(V.alpha[v]); p.convex = R(V.convex[v]); p.cfrd = R(V.cfrd[v]);
  p.gswmin = R(V.gswmin[v]); p.conkc0 = R(V.conkc0[v]); p.conko0 = R(V.conko0[v]); p.ekc = R(V.ekc[v]);
  p.eko = R(V.eko[v]); p.g0 = R(V.g0[v]); p.g1 = R(V.g1[v]); p.xfang = R(V.xfang[v]);
  p.refl[0] = R(V.refl1[v]); p.refl[1] = R(V.refl2[v]); p.refl[2] = R(0.01);
  p.taul[0] = R(V.taul1[v]); p.taul[1] = R(V.taul2[v]); p.taul[2] = R(0.01);
  p.meth = R(1);
  p.rw = R(V.rw[v]); p.tfcl = R(V.tfcl[v]); p.tvclst = R(V.tvclst[v]);
  p.clitt = R2(R(V.clitt[v]));
  for (int k = 0; k < 3; ++k) p.ratecp[k] = R(V.ratecp[k]);
  for (int k = 0; k < 2; ++k) p.ratecs[k] = R(V.ratecs[k]);
  for (int k = 0; k < MS; ++k) p.zse[k] = R(ZSE[k]);
  // froot from rootbeta (Jackson et al. 1996)
  {
    R2 rootbeta = R2(R(V.rootbeta[v]));
    R totdepth = 0;
    for (int is = 0; is < MS - 1; ++is) {
      totdepth = totdepth + p.zse[is] * R(100.0);
      p.froot[is] = R(mn(R2(1.0), R2(1.0) - std::pow(rootbeta, R2(totdepth))));
    }
    p.froot[MS - 1] = R(1.0) - p.froot[MS - 2];
    for (int is = MS - 2; is >= 1; --is) p.froot[is] = p.froot[is] - p.froot[is - 1];
  }
  p.bch = R(T.bch[s]); p.css = R(T.css[s]); p.hyds = R(T.hyds[s]); p.rhosoil = R(T.rhosoil[s]);
  p.sfc = R(T.sfc[s]); p.ssat = R(T.ssat[s]); p.sucs = R(-std::fabs(T.sucs[s])); p.swilt = R(T.swilt[s]);
  p.sand = R(T.sand[s]); p.clay = R(T.clay[s]); p.silt = R(T.silt[s]);
  p.cnsd = R2(p.sand * R(0.3) + p.clay * R(0.25) + p.silt * R(0.265));
  // soil_thermal_fix parameter set (cable_parameters.F90:2165-2227, r_2 with
  // default-REAL literals promoted): cnsd_vec from the bounded porosity and
  // the table bulk density; then rhosoil_vec / (1 - ssat), css from the
  // texture regression, and the scalar rhosoil, css, cnsd take the layer-3
  // (= every layer's) values
  p.ssat_vec = R2(p.ssat); p.sand_vec = R2(p.sand); p.watr = R2(0.01f);
  {
    const R2 sb = mn(R2(0.8f), mx(R2(0.1f), p.ssat_vec));
    const R2 rhov = R2(p.rhosoil);
    p.cnsd_vec = (R2(0.135f) * (R2(1.0) - sb) + R2(64.7f) / rhov) / (R2(1.0) - R2(0.947f) * (R2(1.0) - sb));
    if (thermal_fix) {
      p.rhosoil = R(rhov / (R2(1.0) - p.ssat_vec));
      p.css = R(mx(R2(910.6479f) * R2(p.silt) + R2(916.4438f) * R2(p.clay) + R2(740.7491f) * R2(p.sand), R2(800.0f)));
      p.cnsd = R2(R(p.cnsd_vec));
    }
  }
  p.hsbh = p.hyds * std::fabs(p.sucs) * p.bch;
  p.ibp2 = R(std::lround(p.bch) + 2);
  p.pwb_min = R2(std::pow(p.swilt / p.ssat, p.ibp2));
  p.i2bp3 = R(2 * std::lround(p.bch) + 3);
  p.albsoil[0] = R(T.albsoil_vis[s]); p.albsoil[1] = R(T.albsoil_nir[s]); p.albsoil[2] = 0;
  p.zshh[0] = R(0.5) * p.zse[0];
  p.zshh[MS] = R(0.5) * p.zse[MS - 1];
  for (int k = 1; k < MS; ++k) p.zshh[k] = R(0.5) * (p.zse[k - 1] + p.zse[k]);
  for (int k = 0; k < MS; ++k) {
    p.zse_vec[k] = R2(p.zse[k]); p.swilt_vec[k] = R2(p.swilt); p.sfc_vec[k] = R2(p.sfc);
  }
}

template <class R, class R2>
void make_state(State<R, R2>& s, const Params<R, R2>& p, int iveg, double snowd0, double tgg0, double wb0) {
  const PftTable& V = pft_table();
  const int v = iveg - 1;
  for (int k = 0; k < MS; ++k) {
    s.wb[k] = R2(R(wb0));
    s.tgg[k] = R(tgg0);
    s.wbice[k] = (s.tgg[k] < R(273.15)) ? s.wb[k] * R(0.8) : R2(0.0);
    s.gammzz[k] = 0;
  }
  s.snowd = R(snowd0);
  s.osnowd = 0;
  s.isflag = 0;
  s.snage = 0;
  if (s.snowd > R(0.0)) {
    s.ssdnn = R(120.0);
    for (int k = 0; k < MSN; ++k) { s.ssdn[k] = R(120.0); s.tggsn[k] = R(TFRZ); }
  } else {
    s.ssdnn = R(140.0);
    for (int k = 0; k < MSN; ++k) { s.ssdn[k] = R(140.0); s.tggsn[k] = R(273.1); }
  }
  for (int k = 0; k < MSN; ++k) { s.smass[k] = 0; s.sdepth[k] = 0; }
  s.pudsto = 0; s.pudsmx = 0; s.rtsoil = R(100.0); s.tss = s.tgg[0]; s.wb_lake = 0; s.wbtot1 = 0; s.wbtot2 = 0;
  s.cansto = 0;
  s.owetfac = mx(R(0.0), mn(R(1.0), (R(s.wb[0]) - p.swilt) / (p.sfc - p.swilt)));
  if (s.wbice[0] > 0.) {
    R tmp2 = R(s.wbice[0] / s.wb[0]);
    s.owetfac = s.owetfac * sq(R(1.0) - tmp2);
  }
  s.cplant[0] = R(V.cplant1[v]); s.cplant[1] = R(V.cplant2[v]); s.cplant[2] = R(V.cplant3[v]);
  s.csoil[0] = R(V.csoil1[v]); s.csoil[1] = R(V.csoil2[v]);
  s.owb = 0; s.ebal_tot = 0; s.wbal_tot = 0;
  s.first_soilsnow_call = true;
}

template <class R, class R2>
int run_impl(int mp, int nsteps, int ktau0, double dels, int switches, const int* iveg, const int* isoilm,
             const double* vlai, const double* lat, const float* forcing, const ForcingSpec* spec,
             const TileForcingParams* tfp, double* state, double* diag, int nthreads, const int* calls = nullptr) {
  const int nslots = state_slots();
  (void)nslots;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
  for (int t = 0; t < mp; ++t) {
    Params<R, R2> p;
    make_params(p, iveg[t], isoilm[t], vlai[t], lat[t], (switches & 2) != 0);
    State<R, R2> s;
    unpack_state(s, state, mp, t);
    CbmRef<R, R2> model;
    model.medlyn = (switches & 1) != 0;
    model.soil_thermal_fix = (switches & 2) != 0;
    model.litter = (switches & 4) != 0;
    model.l_rev_corr = (switches & 8) != 0;
    model.fwsoil_mode = (switches & 16) ? 1 : ((switches & 32) ? 2 : 0);
    model.potev_pm = (switches & 64) != 0;
    model.new_reduce_soilevp = (switches & 128) != 0;
    model.new_runoff_speed = (switches & 256) != 0;
    model.diag_soil_resp_off = (switches & 512) != 0;
    Diag<R, R2> d{};
    for (int n = 0; n < nsteps; ++n) {
      float fv[F_NFIELDS];
      if (forcing) {
        const float* fs = forcing + (size_t)n * F_NFIELDS * mp;
        for (int i = 0; i < F_NFIELDS; ++i) fv[i] = fs[(size_t)i * mp + t];
      } else {
        const int k = calls ? calls[4 * n] : ktau0 + n;
        forcing_at(*spec, tfp[t], (uint32_t)t, (uint32_t)(k - 1), fv);
      }
      Forcing<R> f;
      f.fsd[0] = R(fv[F_FSD1]); f.fsd[1] = R(fv[F_FSD2]); f.fld = R(fv[F_FLD]); f.precip = R(fv[F_PRECIP]);
      f.precip_sn = R(fv[F_PRECIP_SN]); f.tk = R(fv[F_TK]); f.pmb = R(fv[F_PMB]); f.ua = R(fv[F_UA]);
      f.qv = R(fv[F_QV]); f.ca = R(fv[F_CA]); f.coszen = R(fv[F_COSZEN]); f.doy = R(fv[F_DOY]); f.hod = R(fv[F_HOD]);
      if (calls) {
        const int* cl = calls + 4 * n;
        model.step(p, s, f, d, cl[0], R(dels), cl[1], cl[2] != 0, cl[3] != 0);
      } else {
        model.step(p, s, f, d, ktau0 + n, R(dels));
      }
    }
    pack_state(s, state, mp, t);
    if (diag) pack_diag(d, diag, mp, t);
  }
  return 0;
}

}  // namespace

extern "C" {

int cbmref_num_state_fields() { return kNState; }
const char* cbmref_state_field_name(int i) { return (i >= 0 && i < kNState) ? kState[i].name : nullptr; }
int cbmref_state_field_width(int i) { return (i >= 0 && i < kNState) ? kState[i].width : 0; }
int cbmref_state_slots() { return state_slots(); }
int cbmref_num_diag() { return kNDiag; }
const char* cbmref_diag_name(int i) { return (i >= 0 && i < kNDiag) ? kDiag[i] : nullptr; }
int cbmref_num_forcing_fields() { return F_NFIELDS; }

// Fills state[slot][tile] with the reference's cold-start initial state.
int cbmref_init(int mp, int precision, const int* iveg, const int* isoilm, const double* vlai, const double* lat,
                const double* snowd0, const double* tgg0, const double* wb0, double* state) {
  for (int t = 0; t < mp; ++t) {
    if (iveg[t] < 1 || iveg[t] > NPFT || isoilm[t] < 1 || isoilm[t] > NSOIL) return -1;
    if (precision == 0) {
      Params<double, double> p; make_params(p, iveg[t], isoilm[t], vlai[t], lat[t]);
      State<double, double> s; make_state(s, p, iveg[t], snowd0[t], tgg0[t], wb0[t]);
      pack_state(s, state, mp, t);
    } else {
      Params<float, double> p; make_params(p, iveg[t], isoilm[t], vlai[t], lat[t]);
      State<float, double> s; make_state(s, p, iveg[t], snowd0[t], tgg0[t], wb0[t]);
      pack_state(s, state, mp, t);
    }
  }
  return 0;
}

// Runs nsteps timesteps (ktau = ktau0 .. ktau0+nsteps-1).  forcing is
// [nsteps][13][mp] (float); when it is null the synthetic generator is used
// with (seed, doy0) and the per-tile forcing parameters.  diag receives the
// last step's diagnostics [ndiag][mp] (may be null).
// precision: 0 = <double,double> oracle, 1 = <float,double> reference mix.
// switches: bit 0 gs_switch='medlyn', bit 1 soil_thermal_fix, bit 2 litter,
// bit 3 l_rev_corr, bit 4 fwsoil_switch='non-linear extrapolation', bit 5
// fwsoil_switch='Lai and Ktaul 2000', bit 6 ssnow_potev='P-M', bit 7
// l_new_reduce_soilevp, bit 8 l_new_runoff_speed, bit 9 diag_soil_resp='OFF'.
int cbmref_run(int mp, int nsteps, int ktau0, double dels, int precision, int switches, const int* iveg,
               const int* isoilm, const double* vlai, const double* lat, const float* forcing, uint64_t seed,
               int doy0, const float* tf_lat, const float* tf_lonphase, const float* tf_tbase,
               const float* tf_swscale, double* state, double* diag, int nthreads) {
  ForcingSpec spec;
  spec.seed = seed; spec.doy0 = doy0; spec.dels = (float)dels;
  std::vector<TileForcingParams> tfp;
  if (!forcing) {
    tfp.resize(mp);
    for (int t = 0; t < mp; ++t) tfp[t] = {tf_lat[t], tf_lonphase[t], tf_tbase[t], tf_swscale[t]};
  }
  if (precision == 0)
    return run_impl<double, double>(mp, nsteps, ktau0, dels, switches, iveg, isoilm, vlai, lat, forcing, &spec,
                                    tfp.data(), state, diag, nthreads);
  return run_impl<float, double>(mp, nsteps, ktau0, dels, switches, iveg, isoilm, vlai, lat, forcing, &spec,
                                 tfp.data(), state, diag, nthreads);
}

// A sequence of ncalls cbm calls of the offline or the coupled kinds:
// calls[n] = {ktau, mode, final_cycle, lai_refresh} with mode 0 the offline
// cbm(), 1 cbm_expl, 2 cbm_impl (CbmRef::step).  forcing, if not null, is
// [ncalls][13][mp], one record per call; else the synthetic generator's
// record of step ktau.  Other arguments as for cbmref_run.
int cbmref_run_calls(int mp, int ncalls, const int* calls, double dels, int precision, int switches,
                     const int* iveg, const int* isoilm, const double* vlai, const double* lat, const float* forcing,
                     uint64_t seed, int doy0, const float* tf_lat, const float* tf_lonphase, const float* tf_tbase,
                     const float* tf_swscale, double* state, double* diag, int nthreads) {
  if (!calls || ncalls < 0) return -1;
  for (int n = 0; n < ncalls; ++n)
    if (calls[4 * n] < 1 || calls[4 * n + 1] < 0 || calls[4 * n + 1] > 2) return -1;
  ForcingSpec spec;
  spec.seed = seed; spec.doy0 = doy0; spec.dels = (float)dels;
  std::vector<TileForcingParams> tfp;
  if (!forcing) {
    tfp.resize(mp);
    for (int t = 0; t < mp; ++t) tfp[t] = {tf_lat[t], tf_lonphase[t], tf_tbase[t], tf_swscale[t]};
  }
  if (precision == 0)
    return run_impl<double, double>(mp, ncalls, 1, dels, switches, iveg, isoilm, vlai, lat, forcing, &spec,
                                    tfp.data(), state, diag, nthreads, calls);
  return run_impl<float, double>(mp, ncalls, 1, dels, switches, iveg, isoilm, vlai, lat, forcing, &spec,
                                 tfp.data(), state, diag, nthreads, calls);
}

// Synthetic forcing for tiles [0, mp) and steps [step0, step0+nsteps):
// out is [nsteps][13][mp].
int cbmref_forcing(int mp, int step0, int nsteps, uint64_t seed, int doy0, double dels, const float* tf_lat,
                   const float* tf_lonphase, const float* tf_tbase, const float* tf_swscale, float* out) {
  ForcingSpec spec;
  spec.seed = seed; spec.doy0 = doy0; spec.dels = (float)dels;
  for (int n = 0; n < nsteps; ++n)
    for (int t = 0; t < mp; ++t) {
      float fv[F_NFIELDS];
      TileForcingParams tp = {tf_lat[t], tf_lonphase[t], tf_tbase[t], tf_swscale[t]};
      forcing_at(spec, tp, (uint32_t)t, (uint32_t)(step0 + n), fv);
      for (int i = 0; i < F_NFIELDS; ++i) out[((size_t)n * F_NFIELDS + i) * mp + t] = fv[i];
    }
  return 0;
}

// Single-function unit checks used by the oracle self-tests.
double cbmref_psim(double z) { return CbmRef<double, double>::psim(z); }
double cbmref_psis(double z) { return CbmRef<double, double>::psis(z); }
double cbmref_qsat(double tc, double pmb) { return CbmRef<double, double>::qsatfjh(tc, pmb); }
double cbmref_spitter(int doy, double coszen, double fsd) { return CbmRef<double, double>::spitter(doy, coszen, fsd); }
void cbmref_trimb(const double* a, const double* b, const double* c, double* rhs, int n) {
  CbmRef<double, double>::trimb(a, b, c, rhs, n);
}
// photosynthesis for one leaf: returns net assimilation
double cbmref_photosynthesis(double csx, double cx1, double cx2, double gswmin, double rdx, double vcmxt3,
                             double vcmxt4, double vx3, double vx4, double gs_coeff, double fwsoil) {
  return CbmRef<double, double>::photosynthesis_leaf(csx, cx1, cx2, gswmin, rdx, vcmxt3, vcmxt4, vx3, vx4, gs_coeff,
                                                     fwsoil);
}
// table lookups, so tests can compare against the product's copy
double cbmref_pft_value(const char* name, int iveg) {
  const PftTable& V = pft_table();
  int v = iveg - 1;
  if (v < 0 || v >= NPFT) return NAN;
#define F(x) if (!std::strcmp(name, #x)) return V.x[v];
  F(a1gs) F(alpha) F(canst1) F(cfrd) F(conkc0) F(conko0) F(convex) F(cplant1) F(cplant2) F(cplant3) F(csoil1)
  F(csoil2) F(d0gs) F(ekc) F(eko) F(extkn) F(frac4) F(g0) F(g1) F(gswmin) F(hc) F(length) F(refl1) F(refl2)
  F(taul1) F(taul2) F(rootbeta) F(rp20) F(rs20) F(shelrb) F(vbeta) F(vcmax) F(vegcf) F(width) F(xfang) F(rw) F(tfcl)
  F(tvclst) F(clitt)
#undef F
  return NAN;
}
double cbmref_soil_value(const char* name, int isoilm) {
  const SoilTable& T = soil_table();
  int s = isoilm - 1;
  if (s < 0 || s >= NSOIL) return NAN;
#define F(x) if (!std::strcmp(name, #x)) return T.x[s];
  F(bch) F(clay) F(css) F(hyds) F(rhosoil) F(sand) F(sfc) F(silt) F(ssat) F(sucs) F(swilt) F(albsoil_vis) F(albsoil_nir)
#undef F
  return NAN;
}
// soil_thermal_fix parameter set of one soil type, for comparison with the
// product's tables: css, rhosoil, cnsd_vec and the saturated-conductivity
// factor Ktmp of total_soil_conductivity (cbl_conductivity.F90:36-43)
int cbmref_soil_thermal_fix(int isoilm, double* css, double* rhosoil, double* cnsd_vec, double* ktmp) {
  if (isoilm < 1 || isoilm > NSOIL) return -1;
  Params<double, double> p;
  make_params(p, 1, isoilm, 1.0, 0.0, true);
  *css = p.css; *rhosoil = p.rhosoil; *cnsd_vec = p.cnsd_vec;
  const double quartz = mx(0.0, mn(double(0.8f), p.sand_vec * double(0.92f)));
  const double Ko = quartz > double(0.2f) ? 2.0 : 3.0;
  *ktmp = std::pow(std::pow(double(7.7f), quartz) * std::pow(Ko, 1.0 - quartz), 1.0 - p.ssat_vec);
  return 0;
}
// derived per-tile parameters (froot etc.), for comparison with the product
int cbmref_params(int iveg, int isoilm, double* froot6, double* dleaf, double* pwb_min, double* hsbh) {
  Params<double, double> p;
  make_params(p, iveg, isoilm, 1.0, 0.0);
  for (int k = 0; k < MS; ++k) froot6[k] = p.froot[k];
  *dleaf = p.dleaf; *pwb_min = p.pwb_min; *hsbh = p.hsbh;
  return 0;
}

}  // extern "C"
