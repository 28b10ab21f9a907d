// Host-side construction of the parameter tables declared in tables.h.
#include "tables.h"

#include <algorithm>
#include <cmath>

namespace {
// pft_params.nml (indices 0..16 = PFT 1..17)
const double a1gs[] = {9,9,9,9,9,9,4,9,9,4,9,9,9,9,9,9,9};
const double alpha_[] = {.2,.2,.2,.2,.2,.2,.05,.2,.2,.05,.2,.2,.2,.2,.2,.2,.2};
const double cfrd[] = {.015,.015,.015,.015,.015,.015,.025,.015,.015,.025,.015,.015,.015,.015,.015,.015,.015};
const double convex[] = {.01,.01,.01,.01,.01,.01,.8,.01,.01,.8,.01,.01,.01,.01,.01,.01,.01};
const double cplant1[] = {200,300,200,300,159,250,250,250,150,150,250,1,.1,0,1,1,0};
const double cplant2[] = {10217,16833,5967,12000,5000,0,0,0,0,0,0,0,0,0,0,0,0};
const double cplant3[] = {876,1443,511,1029,500,500,500,500,607,607,500,1,.1,0,1,1,0};
const double csoil1[] = {184,303,107,216,100,275,275,275,149,149,275,1,.1,1,1,1,1};
const double csoil2[] = {367,606,214,432,250,314,314,314,300,300,314,1,.1,1,1,1,1};
const double frac4[] = {0,0,0,0,0,0,1,0,0,1,0,0,0,0,0,0,0};
const double g1[] = {2.346064,4.114762,2.346064,4.447321,4.694803,5.248500,1.616178,2.222156,5.789377,1.616178,
                     5.248500,5.248500,0.0,5.248500,5.248500,5.248500,5.248500};
const double gswmin[] = {.01,.01,.01,.01,.01,.01,.04,.01,.01,.04,.01,.01,.01,.01,.01,.01,.01};
const double hc[] = {17,35,15.5,20,.6,.567,.567,.567,.55,.55,.567,.2,6.017,.2,.2,.2,.2};
const double length_[] = {.055,.1,.04,.15,.1,.3,.3,.3,.3,.3,.3,.03,.242,.03,.03,.03,.03};
const double width_[] = {.001,.05,.001,.08,.005,.01,.01,.01,.01,.01,.01,.003,.015,.001,.001,.001,.001};
const double refl1[] = {.09,.09,.075,.09,.09,.11,.11,.075,.11,.11,.108,.055,.091,.238,.143,.143,.159};
const double refl2[] = {.3,.29,.3,.29,.3,.34,.34,.32,.34,.34,.343,.19,.31,.457,.275,.275,.305};
const double taul1[] = {.09,.09,.075,.09,.09,.11,.11,.075,.11,.11,.075,.023,.059,.039,.023,.023,.026};
const double taul2[] = {.3,.29,.3,.29,.3,.34,.34,.32,.34,.34,.146,.198,.163,.189,.113,.113,.113};
const double rootbeta[] = {.943,.962,.966,.961,.964,.943,.943,.943,.961,.961,.943,.975,.961,.961,.961,.961,.961};
const double rp20[] = {3,.6,3,2.2,1,1.5,2.8,2.5,1.5,1,1.5,1,1,1,1,1,1};
const double rs20[] = {1,1,1,1,1,1,1,1,1,1,1,0,1,0,0,0,0};
const double vbeta[] = {2,2,2,2,4,4,4,4,2,2,4,4,2,4,4,4,4};
const double vcmax[] = {.00004,.000055,.00004,.00006,.00004,.00006,.00001,.00004,.00008,.00008,.00006,.000017,
                        .000001,.000017,.000017,.000017,.000017};
const double vegcf[] = {9,14,9,8,5,7,7,5,7,1,7,1,1,1,1,1,1};
const double xfang[] = {.01,.1,.01,.25,.01,-.3,-.3,-.3,-.3,-.3,-.3,.1,0,0,0,0,0};
// cable_carbon.F90 CASE (17)
const double rw[] = {16,16,18,8.7,12.5,15.1,10.4,7.5,6.1,6.1,.001,5.8,.001,5.8,.001,9.0,.001};
const double tfcl[] = {.42,.248,.38,.345,.31,.73,2.4,.35,.997,.997,.95,.55,.95,.55,.95,2.4,.95};
const double tvclst[] = {235,283,268,278,278,235,278,278,278,278,278,278,278,278,268,278,278};
// litter carbon (t C / ha), pft_params.nml:9 (vegin%clitt)
const double clitt[] = {20,6,10,13,2,2,.3,.3,0,0,2,2,0,0,0,0,0};
// cable_soilparm.nml
const double bch[] = {4.2,7.1,11.4,5.15,10.4,10.4,7.12,5.83,7.1};
const double clay[] = {.09,.3,.67,.2,.42,.48,.27,.17,.3};
const double css[] = {850,850,850,850,850,850,850,1920,2100};
const double hyds[] = {.000166,.000004,.000001,.000021,.000002,.000001,.000006,.0008,.000001};
const double rhosoil[] = {1600,1600,1381,1373,1476,1521,1373,1537,917};
const double sand[] = {.83,.37,.16,.6,.52,.27,.58,.13,.37};
const double sfc[] = {.143,.301,.367,.218,.31,.37,.255,.45,.301};
const double silt[] = {.08,.33,.17,.2,.06,.25,.15,.7,.33};
const double ssat[] = {.398,.479,.482,.443,.426,.482,.42,.451,.479};
const double sucs[] = {-.106,-.591,-.405,-.348,-.153,-.49,-.299,-.356,-.153};
const double swilt[] = {.072,.216,.286,.135,.219,.283,.175,.395,.216};
const double alb_vis[] = {.16,.11,.10,.13,.12,.10,.12,.07,.60};
const double alb_nir[] = {.30,.22,.20,.26,.24,.20,.24,.14,.50};
const double zse[CG_MS] = {.022, .058, .154, .409, 1.085, 2.872};
}  // namespace

void cg_build_tables(CgPftTable* P, CgSoilTable* S) {
  for (int v = 0; v < CG_NPFT; ++v) {
    P->canst1[v] = 0.1f;
    P->dleaf[v] = std::sqrt((float)width_[v] * (float)length_[v]);
    P->vcmax[v] = (float)vcmax[v];
    P->ejmax[v] = 2.0f * P->vcmax[v];
    P->frac4[v] = (float)frac4[v];
    P->hc[v] = (float)hc[v];
    P->vbeta[v] = (float)vbeta[v];
    P->rp20[v] = (float)rp20[v];
    P->rs20[v] = (float)rs20[v];
    P->vegcf[v] = (float)vegcf[v];
    P->extkn[v] = 0.001f;
    P->a1gs[v] = (float)a1gs[v];
    P->d0gs[v] = 1500.0f;
    P->alpha[v] = (float)alpha_[v];
    P->convex[v] = (float)convex[v];
    P->cfrd[v] = (float)cfrd[v];
    P->gswmin[v] = (float)gswmin[v];
    P->conkc0[v] = 0.000302f;
    P->conko0[v] = 0.256f;
    P->ekc[v] = 59430.0f;
    P->eko[v] = 36000.0f;
    P->g0[v] = 0.0f;
    P->g1[v] = (float)g1[v];
    P->xfang[v] = (float)xfang[v];
    P->shelrb[v] = 2.0f;
    P->refl1[v] = (float)refl1[v];
    P->refl2[v] = (float)refl2[v];
    P->taul1[v] = (float)taul1[v];
    P->taul2[v] = (float)taul2[v];
    P->rw[v] = (float)rw[v];
    P->tfcl[v] = (float)tfcl[v];
    P->tvclst[v] = (float)tvclst[v];
    P->clitt[v] = (float)clitt[v];
    P->cplant0[0][v] = (float)cplant1[v];
    P->cplant0[1][v] = (float)cplant2[v];
    P->cplant0[2][v] = (float)cplant3[v];
    P->csoil0[0][v] = (float)csoil1[v];
    P->csoil0[1][v] = (float)csoil2[v];
    // root fraction per layer from rootbeta and cumulative depth (cm)
    float fr[CG_MS];
    double rb = (double)(float)rootbeta[v];
    float totdepth = 0.0f;
    for (int k = 0; k < CG_MS - 1; ++k) {
      totdepth += (float)zse[k] * 100.0f;
      double x = 1.0 - std::pow(rb, (double)totdepth);
      fr[k] = (float)(x < 1.0 ? x : 1.0);
    }
    fr[CG_MS - 1] = 1.0f - fr[CG_MS - 2];
    for (int k = CG_MS - 2; k >= 1; --k) fr[k] = fr[k] - fr[k - 1];
    for (int k = 0; k < CG_MS; ++k) P->froot[k][v] = fr[k];
  }
  P->ratecp[0] = 1.0f; P->ratecp[1] = 0.03f; P->ratecp[2] = 0.14f;
  P->ratecs[0] = 2.0f; P->ratecs[1] = 0.5f;

  for (int s = 0; s < CG_NSOIL; ++s) {
    S->bch[s] = (float)bch[s];
    S->css[s] = (float)css[s];
    S->hyds[s] = (float)hyds[s];
    S->rhosoil[s] = (float)rhosoil[s];
    S->sfc[s] = (float)sfc[s];
    S->ssat[s] = (float)ssat[s];
    S->sucs[s] = -std::fabs((float)sucs[s]);
    S->swilt[s] = (float)swilt[s];
    S->sand[s] = (float)sand[s];
    S->clay[s] = (float)clay[s];
    S->silt[s] = (float)silt[s];
    S->cnsd[s] = S->sand[s] * 0.3f + S->clay[s] * 0.25f + S->silt[s] * 0.265f;
    S->hsbh[s] = S->hyds[s] * std::fabs(S->sucs[s]) * S->bch[s];
    S->ibp2[s] = (float)(std::lround(S->bch[s]) + 2);
    S->i2bp3[s] = (float)(2 * std::lround(S->bch[s]) + 3);
    S->pwb_min[s] = std::pow(S->swilt[s] / S->ssat[s], S->ibp2[s]);
    S->albsoil_vis[s] = (float)alb_vis[s];
    S->albsoil_nir[s] = (float)alb_nir[s];
    // soil_thermal_fix inputs, in double with the reference's default-REAL
    // literals: the layer vectors hold the soil type's values
    {
      const double ssat_v = (double)S->ssat[s], sand_v = (double)S->sand[s];
      const double sb = std::min((double)0.8f, std::max((double)0.1f, ssat_v));
      S->cnsdv[s] = (float)(((double)0.135f * (1.0 - sb) + (double)64.7f / (double)S->rhosoil[s]) /
                            (1.0 - (double)0.947f * (1.0 - sb)));
      const double q = std::max(0.0, std::min((double)0.8f, sand_v * (double)0.92f));
      const double ko = q > (double)0.2f ? 2.0 : 3.0;
      S->ktmp[s] = (float)std::pow(std::pow((double)7.7f, q) * std::pow(ko, 1.0 - q), 1.0 - ssat_v);
    }
  }
  for (int k = 0; k < CG_MS; ++k) S->zse[k] = (float)zse[k];
  S->zshh[0] = 0.5f * S->zse[0];
  S->zshh[CG_MS] = 0.5f * S->zse[CG_MS - 1];
  for (int k = 1; k < CG_MS; ++k) S->zshh[k] = 0.5f * (S->zse[k - 1] + S->zse[k]);
}

void cg_apply_soil_thermal_fix(CgSoilTable* S) {
  for (int s = 0; s < CG_NSOIL; ++s) {
    const double ssat_v = (double)S->ssat[s];
    const double rho = (double)S->rhosoil[s] / (1.0 - ssat_v);
    const double cs = std::max((double)910.6479f * (double)S->silt[s] + (double)916.4438f * (double)S->clay[s] +
                                   (double)740.7491f * (double)S->sand[s],
                               (double)800.0f);
    S->rhosoil[s] = (float)rho;
    S->css[s] = (float)cs;
    S->cnsd[s] = S->cnsdv[s];
  }
}
