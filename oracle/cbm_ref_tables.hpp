// ORACLE / TEST INFRASTRUCTURE ONLY.
// Constants and per-PFT / per-soil parameter tables of the CPU restatement of
// CABLE's cbm() path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may use anything under oracle/.  The product (cable_gb300/)
// carries its own copy of these tables; a test checks the two agree.
//
// Parity status: pinned against physical invariants only.  The reference is
// Fortran and no Fortran compiler is available here, and the reference ships
// no golden vectors for this path (its unit tests cover netCDF I/O only).
//
// Sources (data transcribed, not code):
//   physical constants   src/params/cable_phys_constants_mod.F90
//   photosynthesis       src/params/cable_photo_constants_mod.F90
//   other constants      src/params/cable_other_constants_mod.F90
//   PFT table            src/offline/pft_params.nml:2-61
//   soil table           src/offline/cable_soilparm.nml:3-22
//   carbon tables        src/science/misc/cable_carbon.F90:129-140 (mvtype 17)
#pragma once

namespace cbmref {

constexpr int MS = 6;      // soil layers        (grid_constants_cbl.F90 nsl)
constexpr int MSN = 3;     // snow layers        (nsnl)
constexpr int NITER = 4;   // MO iterations      (niter)
constexpr int MAXITER = 20;// dryLeaf passes     (cable_photo_constants_mod.F90 maxiter)
constexpr int NPFT = 17;
constexpr int NSOIL = 9;

// cable_phys_constants_mod.F90
constexpr double TFRZ = 273.16, SBOLTZ = 5.67e-8, EMSOIL = 1.0, EMLEAF = 1.0;
constexpr double CAPP = 1004.64, HL = 2.5014e6, HLF = 0.334e6, HLS = 2.8350e6;
constexpr double DHEAT = 21.5e-6, GRAV = 9.8086, RGAS = 8.3143, RMAIR = 0.02897;
constexpr double RMH2O = 0.018016, CGSNOW = 2090.0, CSICE = 2.100e3, CSWAT = 4.218e3;
constexpr double DENSITY_LIQ = 1000.0, DENSITY_ICE = 921.0;
constexpr double TETENA = 6.106, TETENB = 17.27, TETENC = 237.3;
constexpr double VONK = 0.40, A33 = 1.25, CSW = 0.50, CTL = 0.40, APOL = 0.70;
constexpr double PRANDT = 0.71, CRD = 0.3, CSD = 0.003, CCD = 15.0, CCW_C = 2.0;
constexpr double USUHM = 0.3, ZETA0 = 0.0, ZETNEG = -15.0, ZETPOS = 1.0;
constexpr double ZDLIN = 1.0, UMIN = 0.1, SNOW_DEPTH_THRESH = 1.0;
// cable_photo_constants_mod.F90
constexpr double GAM0 = 28.0e-6, GAM1 = 0.0509, GAM2 = 0.0010, RGBWC = 1.32;
constexpr double RGSWC = 1.57, TREFK = 298.2;
// cable_other_constants_mod.F90
constexpr double GAUSS_W[3] = {0.308, 0.514, 0.178};
constexpr double RAD_THRESH = 0.001, LAI_THRESH = 0.001, COSZEN_TOLS = 1.0e-4;
constexpr double Z0SURF_MIN = 1.0e-7, WILT_LIMITFACTOR = 2.0;
// cable_maths_constants_mod.F90
constexpr double PI_C = 3.1415927, PI180 = 3.1415927 / 180.0;
// cable_common.F90:217-222
constexpr double MAX_GLACIER_SNOWD = 1100.0, SNOW_CCNSW = 2.0, MAX_SSDN = 750.0;
constexpr double MAX_SCONDS = 2.51, FROZEN_LIMIT = 0.85;
// cable_runtime_opts_mod.F90:14 (cable.nml:57)
constexpr double SNMIN = 1.0;
// surface types (cable_surface_types.F90)
constexpr int LAKES = 16, ICE_SURF = 17, ICE_SOIL = 9;

// ---------------------------------------------------------------- PFT table
// pft_params.nml, indices 0..16 = PFT 1..17
struct PftTable {
  double a1gs[NPFT], alpha[NPFT], canst1[NPFT], cfrd[NPFT], conkc0[NPFT], conko0[NPFT];
  double convex[NPFT], cplant1[NPFT], cplant2[NPFT], cplant3[NPFT], csoil1[NPFT], csoil2[NPFT];
  double d0gs[NPFT], ekc[NPFT], eko[NPFT], extkn[NPFT], frac4[NPFT], g0[NPFT], g1[NPFT];
  double gswmin[NPFT], hc[NPFT], length[NPFT], ratecp[3], ratecs[2];
  double refl1[NPFT], refl2[NPFT], taul1[NPFT], taul2[NPFT], rootbeta[NPFT];
  double rp20[NPFT], rs20[NPFT], shelrb[NPFT], vbeta[NPFT], vcmax[NPFT], vegcf[NPFT];
  double width[NPFT], xfang[NPFT];
  // cable_carbon.F90 CASE(17)
  double rw[NPFT], tfcl[NPFT], tvclst[NPFT];
  // litter carbon (t C / ha), pft_params.nml:9, used by the litter switch
  double clitt[NPFT];
};

inline const PftTable& pft_table() {
  static const PftTable t = {
    /*a1gs*/ {9,9,9,9,9,9,4,9,9,4,9,9,9,9,9,9,9},
    /*alpha*/ {.2,.2,.2,.2,.2,.2,.05,.2,.2,.05,.2,.2,.2,.2,.2,.2,.2},
    /*canst1*/ {.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1,.1},
    /*cfrd*/ {.015,.015,.015,.015,.015,.015,.025,.015,.015,.025,.015,.015,.015,.015,.015,.015,.015},
    /*conkc0*/ {.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302,.000302},
    /*conko0*/ {.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256,.256},
    /*convex*/ {.01,.01,.01,.01,.01,.01,.8,.01,.01,.8,.01,.01,.01,.01,.01,.01,.01},
    /*cplant1*/ {200,300,200,300,159,250,250,250,150,150,250,1,.1,0,1,1,0},
    /*cplant2*/ {10217,16833,5967,12000,5000,0,0,0,0,0,0,0,0,0,0,0,0},
    /*cplant3*/ {876,1443,511,1029,500,500,500,500,607,607,500,1,.1,0,1,1,0},
    /*csoil1*/ {184,303,107,216,100,275,275,275,149,149,275,1,.1,1,1,1,1},
    /*csoil2*/ {367,606,214,432,250,314,314,314,300,300,314,1,.1,1,1,1,1},
    /*d0gs*/ {1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500,1500},
    /*ekc*/ {59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430,59430},
    /*eko*/ {36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000,36000},
    /*extkn*/ {.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001,.001},
    /*frac4*/ {0,0,0,0,0,0,1,0,0,1,0,0,0,0,0,0,0},
    /*g0*/ {0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0},
    /*g1*/ {2.346064,4.114762,2.346064,4.447321,4.694803,5.248500,1.616178,2.222156,5.789377,1.616178,5.248500,5.248500,0.0,5.248500,5.248500,5.248500,5.248500},
    /*gswmin*/ {.01,.01,.01,.01,.01,.01,.04,.01,.01,.04,.01,.01,.01,.01,.01,.01,.01},
    /*hc*/ {17,35,15.5,20,.6,.567,.567,.567,.55,.55,.567,.2,6.017,.2,.2,.2,.2},
    /*length*/ {.055,.1,.04,.15,.1,.3,.3,.3,.3,.3,.3,.03,.242,.03,.03,.03,.03},
    /*ratecp*/ {1.0,0.03,0.14},
    /*ratecs*/ {2.0,0.5},
    /*refl1*/ {.09,.09,.075,.09,.09,.11,.11,.075,.11,.11,.108,.055,.091,.238,.143,.143,.159},
    /*refl2*/ {.3,.29,.3,.29,.3,.34,.34,.32,.34,.34,.343,.19,.31,.457,.275,.275,.305},
    /*taul1*/ {.09,.09,.075,.09,.09,.11,.11,.075,.11,.11,.075,.023,.059,.039,.023,.023,.026},
    /*taul2*/ {.3,.29,.3,.29,.3,.34,.34,.32,.34,.34,.146,.198,.163,.189,.113,.113,.113},
    /*rootbeta*/ {.943,.962,.966,.961,.964,.943,.943,.943,.961,.961,.943,.975,.961,.961,.961,.961,.961},
    /*rp20*/ {3,.6,3,2.2,1,1.5,2.8,2.5,1.5,1,1.5,1,1,1,1,1,1},
    /*rs20*/ {1,1,1,1,1,1,1,1,1,1,1,0,1,0,0,0,0},
    /*shelrb*/ {2,2,2,2,2,2,2,2,2,2,2,2,2,2,2,2,2},
    /*vbeta*/ {2,2,2,2,4,4,4,4,2,2,4,4,2,4,4,4,4},
    /*vcmax*/ {.00004,.000055,.00004,.00006,.00004,.00006,.00001,.00004,.00008,.00008,.00006,.000017,.000001,.000017,.000017,.000017,.000017},
    /*vegcf*/ {9,14,9,8,5,7,7,5,7,1,7,1,1,1,1,1,1},
    /*width*/ {.001,.05,.001,.08,.005,.01,.01,.01,.01,.01,.01,.003,.015,.001,.001,.001,.001},
    /*xfang*/ {.01,.1,.01,.25,.01,-.3,-.3,-.3,-.3,-.3,-.3,.1,0,0,0,0,0},
    /*rw*/ {16,16,18,8.7,12.5,15.1,10.4,7.5,6.1,6.1,.001,5.8,.001,5.8,.001,9.0,.001},
    /*tfcl*/ {.42,.248,.38,.345,.31,.73,2.4,.35,.997,.997,.95,.55,.95,.55,.95,2.4,.95},
    /*tvclst*/ {235,283,268,278,278,235,278,278,278,278,278,278,278,278,268,278,278},
    /*clitt*/ {20,6,10,13,2,2,.3,.3,0,0,2,2,0,0,0,0,0},
  };
  return t;
}

// ---------------------------------------------------------------- soil table
// cable_soilparm.nml, indices 0..8 = soil 1..9
struct SoilTable {
  double bch[NSOIL], clay[NSOIL], css[NSOIL], hyds[NSOIL], rhosoil[NSOIL], sand[NSOIL];
  double sfc[NSOIL], silt[NSOIL], ssat[NSOIL], sucs[NSOIL], swilt[NSOIL];
  // Soil albedo is not part of the reference tables (it comes from the gridded
  // soil file, which is not available); these VIS/NIR values are a stated
  // choice of this library, one pair per soil type.
  double albsoil_vis[NSOIL], albsoil_nir[NSOIL];
};

inline const SoilTable& soil_table() {
  static const SoilTable t = {
    /*bch*/ {4.2,7.1,11.4,5.15,10.4,10.4,7.12,5.83,7.1},
    /*clay*/ {.09,.3,.67,.2,.42,.48,.27,.17,.3},
    /*css*/ {850,850,850,850,850,850,850,1920,2100},
    /*hyds*/ {.000166,.000004,.000001,.000021,.000002,.000001,.000006,.0008,.000001},
    /*rhosoil*/ {1600,1600,1381,1373,1476,1521,1373,1537,917},
    /*sand*/ {.83,.37,.16,.6,.52,.27,.58,.13,.37},
    /*sfc*/ {.143,.301,.367,.218,.31,.37,.255,.45,.301},
    /*silt*/ {.08,.33,.17,.2,.06,.25,.15,.7,.33},
    /*ssat*/ {.398,.479,.482,.443,.426,.482,.42,.451,.479},
    /*sucs*/ {-.106,-.591,-.405,-.348,-.153,-.49,-.299,-.356,-.153},
    /*swilt*/ {.072,.216,.286,.135,.219,.283,.175,.395,.216},
    /*albsoil_vis*/ {.16,.11,.10,.13,.12,.10,.12,.07,.60},
    /*albsoil_nir*/ {.30,.22,.20,.26,.24,.20,.24,.14,.50},
  };
  return t;
}

// cable_define_types / cable_parameters.F90:1241 (ms = 6)
constexpr double ZSE[MS] = {.022, .058, .154, .409, 1.085, 2.872};

}  // namespace cbmref
