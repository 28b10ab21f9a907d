// Host runtime and C ABI (include/cablegpu.h) of the GB300 cbm() timestep.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cablegpu.h"
#include "phase_kernels.cuh"
#include "surrogate.cuh"
#include "surrogate_host.h"
#include "cgio.h"

// tile order 3: caller tiles per chunk (log2), sized so a chunk's forcing
// (13 rows) and outputs (8 rows) fit the L2 cache together
#ifndef CG_ORDER3_CHUNK_LOG2
#define CG_ORDER3_CHUNK_LOG2 18
#endif

using namespace cg;

namespace {

constexpr int kGraphSteps = 8;      // steps per captured CUDA graph
constexpr int kKernelsPerStep = 5;  // radiation, canopy, snow pack, soil heat, soil water
// The kernels index row r of a field as r * ld + t in 32-bit int: every
// multi-row block (the diagnostics, the hand-off records, the forcing) has
// at most 64 rows, and ld (mp rounded up to 256) stays at most
// CABLEGPU_MAX_TILES, so no offset reaches 2^31.
static_assert(CG_NDIAG <= 64 && CG_NA <= 64 && CG_NFORC <= 64 && CG_NOUT <= 64, "row blocks of at most 64 rows");
static_assert(CABLEGPU_MAX_TILES % 256 == 0 && 64LL * CABLEGPU_MAX_TILES <= 2147483647LL,
              "the largest context's row offsets fit 32 bits");

// ---------------------------------------------------------------- field registry
enum Storage { S_U8, S_F32, S_F64, S_DF };   // S_DF: double-FP32 pairs (hi rows, then lo rows)
struct FieldDef {
  const char* name;
  int nlayer;
  int dtype;   // external (host) type
  int kind;
  Storage st;  // device storage type
};

const char* kDiagNames[CG_NDIAG] = {
  "fe_d", "fh_d", "fev", "fhv", "fhs", "fns", "fnv", "ga_d", "tv_d", "tscrn", "qscrn", "rnet_d", "us", "cduv", "cdtq",
  "epot", "fes", "fevc", "dgdtg", "fevw", "fpn", "frday_d", "fgpp_d", "fnpp", "fnee", "fra", "frp", "frs", "trad_d",
  "albedo_vis", "albedo_nir", "transd", "precis", "through", "fwet", "wetfac", "potev", "runoff", "rnof1", "rnof2",
  "smelt", "ghflux", "sghflux", "drybal", "wetbal", "ebal", "wbal", "qssabs", "rniso", "vlaiw_d", "tvair", "qvair",
  "swnet", "lwnet", "wbtot", "gswx_sun", "gswx_shd", "fwsoil", "dryleaf_passes", "delwc", "cls", "frpw", "frpr",
};

std::vector<FieldDef> make_registry() {
  std::vector<FieldDef> f = {
    {"iveg", 1, CABLEGPU_I32, CABLEGPU_KIND_PARAM, S_U8},
    {"isoilm", 1, CABLEGPU_I32, CABLEGPU_KIND_PARAM, S_U8},
    {"vlai", 1, CABLEGPU_F32, CABLEGPU_KIND_PARAM, S_F32},
    {"lat", 1, CABLEGPU_F32, CABLEGPU_KIND_PARAM, S_F32},
    {"lonphase", 1, CABLEGPU_F32, CABLEGPU_KIND_PARAM, S_F32},
    {"tbase", 1, CABLEGPU_F32, CABLEGPU_KIND_PARAM, S_F32},
    {"swscale", 1, CABLEGPU_F32, CABLEGPU_KIND_PARAM, S_F32},
    // soil%albsoil(:,1), the VIS bare-soil albedo (read from the gridded soil
    // file by the reference); defaults to the soil type's table value
    {"albsoil", 1, CABLEGPU_F32, CABLEGPU_KIND_PARAM, S_F32},
    {"wb", CG_MS, CABLEGPU_F64, CABLEGPU_KIND_STATE, S_DF},
    {"wbice", CG_MS, CABLEGPU_F64, CABLEGPU_KIND_STATE, S_DF},
    {"gammzz1", 1, CABLEGPU_F64, CABLEGPU_KIND_STATE, S_F64},
    {"tgg", CG_MS, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"tggsn", 3, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"ssdn", 3, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"smass", 3, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"sdepth", 3, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"flags", 1, CABLEGPU_I32, CABLEGPU_KIND_STATE, S_U8},
    {"snowd", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"ssdnn", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"snage", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"pudsto", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"owetfac", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"rtsoil", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"tss", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"wb_lake", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"wbtot1", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"wbtot2", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"cansto", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"cplant", 3, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"csoil", 2, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"owb", 1, CABLEGPU_F64, CABLEGPU_KIND_STATE, S_F64},
    {"ebal_tot", 1, CABLEGPU_F64, CABLEGPU_KIND_STATE, S_F64},
    {"wbal_tot", 1, CABLEGPU_F64, CABLEGPU_KIND_STATE, S_F64},
    {"vlaiw", 1, CABLEGPU_F32, CABLEGPU_KIND_STATE, S_F32},
    {"out", CG_NOUT, CABLEGPU_F32, CABLEGPU_KIND_OUTPUT, S_F32},
    {"tile_status", 1, CABLEGPU_I32, CABLEGPU_KIND_OUTPUT, S_U8},
  };
  for (int i = 0; i < CG_NDIAG; ++i) f.push_back({kDiagNames[i], 1, CABLEGPU_F32, CABLEGPU_KIND_DIAG, S_F32});
  f.push_back({"forcing", CG_NFORC, CABLEGPU_F32, CABLEGPU_KIND_FORCING, S_F32});
  f.push_back({"forcing_in", CG_NFORC, CABLEGPU_F32, CABLEGPU_KIND_FORCING, S_F32});
  f.push_back({"work_a", CG_NA, CABLEGPU_F32, CABLEGPU_KIND_WORK, S_F32});
  f.push_back({"work_b", CG_NB_ALLOC, CABLEGPU_F32, CABLEGPU_KIND_WORK, S_F32});
  f.push_back({"work_c", CG_NC_ALLOC, CABLEGPU_F32, CABLEGPU_KIND_WORK, S_F32});
  return f;
}

const std::vector<FieldDef>& registry() {
  static const std::vector<FieldDef> r = make_registry();
  return r;
}

size_t storage_bytes(Storage s) { return s == S_U8 ? 1 : (s == S_F32 ? 4 : 8); }   // S_DF: 2 x 4 bytes

// ---------------------------------------------------------------- kernels
__global__ void advance_clock_kernel(int* clock) { clock[0] += 1; }

__global__ void explicit_trad_kernel(CgDev D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < D.mp) explicit_trad(D, t);
}

// The prognostic bank of the coupled implicit call (cbl_prognostic_bank.F90:
// 26-165): cable_store_prognostics saves these fields before each implicit
// cycle and cable_reinstate_prognostics puts them back after every cycle but
// the last (cable_implicit_main.F90:190-213).  Here the cycle runs on a
// copy instead: each banked field's [rows][ld] block is copied device to
// device (soil water and ice as their double-FP32 word pairs), the cycle's
// kernels read and write the copies, and the fields' own blocks, untouched,
// are the reinstated state.  isflag is bit 0 of flags, while bit 1
// (soil_snow's first call, the reference's SAVE counter) is not in the
// bank: the cycle's bit 1 is merged back (bank_flags_kernel).  Not banked,
// as in the reference, and so updated in place by the cycle: gammzz and the
// outputs (ga).  The coupled calls do not touch the balance totals (owb,
// ebal_tot, wbal_tot) or the lakes fix's wbtot1 / wbtot2 at all.
const char* const kBankFields[] = {"tgg", "wb", "wbice", "sdepth", "smass", "tggsn", "ssdn", "ssdnn", "snage",
                                   "snowd", "pudsto", "rtsoil", "owetfac", "wb_lake", "tss",
                                   "cansto" /* canopy%oldcansto of the next call */, "cplant", "csoil"};
__global__ void bank_flags_kernel(uint8_t* __restrict__ flags, const uint8_t* __restrict__ cycle, int mp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < mp) flags[t] = (uint8_t)((flags[t] & 1u) | (cycle[t] & 0xFEu));
}

// Cold start: the reference's initial state for a run without restart file.
__global__ void cold_start_kernel(CgDev D, const CgTables* __restrict__ T, const double* snowd0, const double* tgg0,
                                  const double* wb0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.mp) return;
  const int ld = D.ld;
  const int v = D.iveg[t] - 1, s = D.isoilm[t] - 1;
  const float swilt = T->soil.swilt[s], sfc = T->soil.sfc[s];
  const int o = D.tile_id[t];
  const float wbf = (float)wb0[o], tg = (float)tgg0[o], sn = (float)snowd0[o];
  const df32 ice0 = (tg < 273.15f) ? df_from_double((double)wbf * (double)0.8f) : df32{0.f, 0.f};
  for (int k = 0; k < CG_MS; ++k) {
    df_store(D.wb, CG_MS, ld, k, t, df32{wbf, 0.f});
    D.tgg[k * ld + t] = tg;
    df_store(D.wbice, CG_MS, ld, k, t, ice0);
  }
  const bool snow = sn > 0.0f;
  for (int k = 0; k < 3; ++k) {
    D.ssdn[k * ld + t] = snow ? 120.0f : 140.0f;
    D.tggsn[k * ld + t] = snow ? TFRZ : 273.1f;
    D.smass[k * ld + t] = 0.f;
    D.sdepth[k * ld + t] = 0.f;
  }
  D.snowd[t] = sn;
  D.ssdnn[t] = snow ? 120.0f : 140.0f;
  D.snage[t] = 0.f;
  D.flags[t] = 2;   // isflag 0, soil_snow first call pending
  D.gammzz1[t] = 0.0;
  D.pudsto[t] = 0.f; D.rtsoil[t] = 100.0f; D.tss[t] = tg; D.wb_lake[t] = 0.f; D.wbtot1[t] = 0.f; D.wbtot2[t] = 0.f;
  D.cansto[t] = 0.f;
  float ow = fmaxf(0.0f, fminf(1.0f, (wbf - swilt) / (sfc - swilt)));
  const double wbice1 = df_to_double(ice0);
  if (wbice1 > 0.) { float r = (float)(wbice1 / (double)wbf); ow = ow * (1.0f - r) * (1.0f - r); }
  D.owetfac[t] = ow;
  for (int k = 0; k < 3; ++k) D.cplant[k * ld + t] = T->pft.cplant0[k][v];
  for (int k = 0; k < 2; ++k) D.csoil[k * ld + t] = T->pft.csoil0[k][v];
  D.owb[t] = 0.0; D.ebal_tot[t] = 0.0; D.wbal_tot[t] = 0.0;
}

// Caller-order host arrays <-> device slot order.  dst/src are [nlayer][ld]
// on the device, stage is [nlayer][mp] in caller order.
template <typename TD, typename TS>
__global__ void scatter_in_kernel(TD* dst, const TS* stage, const int* order, int mp, int ld, int nlayer) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mp) return;
  const int o = order[s];
  for (int k = 0; k < nlayer; ++k) dst[(size_t)k * ld + s] = (TD)stage[(size_t)k * mp + o];
}
template <typename TD, typename TS>
__global__ void gather_out_kernel(TD* stage, const TS* src, const int* order, int mp, int ld, int nlayer) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mp) return;
  const int o = order[s];
  for (int k = 0; k < nlayer; ++k) stage[(size_t)k * mp + o] = (TD)src[(size_t)k * ld + s];
}
// double-FP32 fields: host FP64 <-> device (hi, lo) rows
__global__ void scatter_in_df_kernel(float* dst, const double* stage, const int* order, int mp, int ld, int nlayer) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mp) return;
  const int o = order[s];
  for (int k = 0; k < nlayer; ++k) df_store(dst, nlayer, ld, k, s, df_from_double(stage[(size_t)k * mp + o]));
}
__global__ void gather_out_df_kernel(double* stage, const float* src, const int* order, int mp, int ld, int nlayer) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= mp) return;
  const int o = order[s];
  for (int k = 0; k < nlayer; ++k) stage[(size_t)k * mp + o] = df_to_double(df_load(src, nlayer, ld, k, s));
}

}  // namespace

// ---------------------------------------------------------------- context
struct cablegpu_ctx {
  int device = 0;
  int mp = 0, ld = 0;
  cudaStream_t stream = nullptr;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  std::vector<void*> field_ptr;    // device pointer per registry entry
  CgTables* d_tables = nullptr;
  CgDev dev{};
  int* d_clock = nullptr;
  int* d_order = nullptr;          // device slot -> caller tile index
  char* d_stage = nullptr;         // staging buffer for field copies
  size_t stage_bytes = 0;
  int* h_clock = nullptr;          // pinned
  unsigned int* h_status = nullptr;
  bool host_forcing = false;
  CgForcingSpec forc{12345ull, 1, 1800.f};
  int medlyn = 0, diag = 0, capture_forcing = 0, thermal_fix = 0, litter = 0, rev_corr = 0;
  int switches = 0;                // the CABLEGPU_SW_* mask the fields above come from
  int solve64 = 1;                 // soil Thomas solves: 1 FP64 direct form (default), 0 FP32 on the change
  int canopy_pool = 0;             // canopy dryLeaf passes: 0 per lane (default), 1 block pool
  std::vector<int> h_iveg, h_isoilm;   // the tiles' plant and soil types, caller order
  int host_layout = 0;             // host buffers of step_host / forcing files: 0 caller order, 1 device order
  cudaGraphExec_t graph = nullptr;
  float graph_dels = -1.f;
  int graph_diag = -1, graph_switches = -1, graph_hostforc = -1, graph_capture = -1, graph_solve64 = -1;
  int graph_pool = -1;
  unsigned long long graph_seed = 0;
  int graph_doy0 = -1;
  long long launches = 0;
  // dryLeaf surrogate: training rows harvested from this context's own
  // steps, the network trained on them, and the in-loop switch
  float* d_harvest = nullptr;                // [harvest_cap][16]
  long long harvest_cap = 0;
  long long harvest_rows = 0;                // rows filled by the last harvest
  unsigned long long* d_harvest_n = nullptr;
  bool harvesting = false;
  float harvest_prob = 0.f;
  unsigned long long harvest_seed = 0;
  SurNet net;
  bool net_ready = false;
  int sur_enabled = 0;
  float sur_gate = 0.1f;
  unsigned long long* d_sur_stats = nullptr;  // [2]
  float* d_sur_dt = nullptr;                  // [ld] predicted leaf-temperature change
  void* d_bank = nullptr;                     // prognostic bank of the implicit coupled call (kBankFields)
  int graph_sur = -1;
  float graph_gate = -1.f;
  // threads per block of the five step kernels (radiation, canopy, snow
  // pack, soil heat, soil water) and the tile order the context was built with
  int block[5] = {128, 128, 128, 128, 128};
  int graph_block[5] = {0, 0, 0, 0, 0};
  int order = 0;
  // pipelined host I/O (cablegpu_step_host): one copy stream per direction
  // (an upload must not queue behind the previous step's download) and two
  // slots of device staging for the forcing in and the outputs out
  cudaStream_t cstream = nullptr, dstream = nullptr;
  float* d_fin[2] = {nullptr, nullptr};    // [CG_NFORC][mp] caller order
  float* d_fout[2] = {nullptr, nullptr};   // [CG_NOUT][mp] caller order
  cudaEvent_t ev_h2d[2] = {}, ev_used[2] = {}, ev_step[2] = {}, ev_d2h[2] = {};
  bool io_ready = false;
  const float* io_forcing = nullptr;          // staging slot the current step_host step reads
  float* io_out = nullptr;                    // staging slot it writes its outputs to (caller order)
  long long io_count = 0;
  std::string err;
};

namespace {

int fail(cablegpu_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
#define CG_CUDA(c, call)                                                                     \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return fail((c), CABLEGPU_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

void bind_device_view(cablegpu_ctx* c) {
  auto P = [&](const char* n) { return c->field_ptr[cablegpu_field_id(n)]; };
  CgDev& D = c->dev;
  D.mp = c->mp; D.ld = c->ld;
  D.tile_id = c->d_order;
  D.iveg = (const uint8_t*)P("iveg"); D.isoilm = (const uint8_t*)P("isoilm");
  D.vlai = (const float*)P("vlai"); D.lat = (const float*)P("lat"); D.lonphase = (const float*)P("lonphase");
  D.tbase = (const float*)P("tbase"); D.swscale = (const float*)P("swscale");
  D.albsoil = (const float*)P("albsoil");
  D.wb = (float*)P("wb"); D.wbice = (float*)P("wbice"); D.gammzz1 = (double*)P("gammzz1");
  D.tgg = (float*)P("tgg"); D.tggsn = (float*)P("tggsn"); D.ssdn = (float*)P("ssdn"); D.smass = (float*)P("smass");
  D.sdepth = (float*)P("sdepth"); D.flags = (uint8_t*)P("flags"); D.snowd = (float*)P("snowd");
  D.ssdnn = (float*)P("ssdnn"); D.snage = (float*)P("snage"); D.pudsto = (float*)P("pudsto");
  D.owetfac = (float*)P("owetfac"); D.rtsoil = (float*)P("rtsoil"); D.tss = (float*)P("tss");
  D.wb_lake = (float*)P("wb_lake"); D.wbtot1 = (float*)P("wbtot1"); D.wbtot2 = (float*)P("wbtot2");
  D.cansto = (float*)P("cansto"); D.cplant = (float*)P("cplant"); D.csoil = (float*)P("csoil");
  D.owb = (double*)P("owb"); D.ebal_tot = (double*)P("ebal_tot"); D.wbal_tot = (double*)P("wbal_tot");
  D.vlaiw = (float*)P("vlaiw");
  D.out = (float*)P("out");
  D.tile_status = (uint8_t*)P("tile_status");
  D.diag = c->diag ? (float*)P(kDiagNames[0]) : nullptr;
  D.forcing_in = c->host_forcing ? (const float*)P("forcing_in") : nullptr;
  D.forcing_caller_order = 0;
  if (c->io_forcing) {
    D.forcing_in = c->io_forcing;
    D.forcing_caller_order = c->host_layout == 0 ? 1 : 2;
  }
  D.out_caller = c->io_out;
  D.out_caller_order = c->host_layout == 0 ? 1 : 0;
  D.forcing_out = c->capture_forcing ? (float*)P("forcing") : nullptr;
  D.work_a = (float*)P("work_a");
  D.work_b = (float*)P("work_b");
  D.work_c = (float*)P("work_c");
  D.harvest = c->harvesting ? c->d_harvest : nullptr;
  D.harvest_n = c->d_harvest_n;
  D.harvest_cap = c->harvest_cap;
  D.harvest_prob = c->harvest_prob;
  D.harvest_seed = c->harvest_seed;
  D.sur_dt = c->sur_enabled ? c->d_sur_dt : nullptr;
  D.sur_gate = c->sur_gate;
  D.sur_strict = c->sur_enabled == 1 ? 1 : 0;
  D.sur_stats = c->sur_enabled ? c->d_sur_stats : nullptr;
}

// the surrogate network over all tiles, reading the radiation kernel's record
int launch_sur_net(cablegpu_ctx* c) {
  std::string e;
  if (sur_infer(c->net, c->dev.work_a, c->dev.iveg, c->dev.isoilm, c->d_tables, c->medlyn, c->mp, c->ld, c->d_sur_dt,
                c->dev.status, c->stream, e))
    return fail(c, CABLEGPU_ERR_CUDA, e);
  return CABLEGPU_OK;
}

int launch_step(cablegpu_ctx* c, const StepParams& p, const int* clock) {
  bind_device_view(c);
  const bool diag = c->diag != 0;
  const int* bk = c->block;
  launch_phase_a(diag, c->stream, c->dev, c->d_tables, p, clock, bk[0]);
  if (p.mode != 0) {
    // coupled calls: the plain canopy iteration (the surrogate start and the
    // training-row harvest are offline-driver features)
    launch_phase_b(diag, c->stream, c->dev, c->d_tables, p, clock, bk[1]);
  } else if (c->sur_enabled) {
    int rc = launch_sur_net(c);
    if (rc) return rc;
    ++c->launches;
    launch_phase_b_sur(diag, c->stream, c->dev, c->d_tables, p, clock, bk[1]);
  } else if (c->harvesting) {
    launch_phase_b_harvest(diag, c->stream, c->dev, c->d_tables, p, clock, bk[1]);
  } else {
    launch_phase_b(diag, c->stream, c->dev, c->d_tables, p, clock, bk[1]);
  }
  if (p.mode != 1) {
    launch_phase_c1(diag, c->stream, c->dev, c->d_tables, p, clock, bk[2]);
    launch_phase_c2(diag, c->stream, c->dev, c->d_tables, p, clock, bk[3]);
    launch_phase_c3(diag, c->stream, c->dev, c->d_tables, p, clock, bk[4]);
  } else {
    // the explicit coupled call stops after the canopy: its radiative temperature
    explicit_trad_kernel<<<(c->mp + 255) / 256, 256, 0, c->stream>>>(c->dev);
  }
  c->launches += p.mode == 1 ? 3 : kKernelsPerStep;
  CG_CUDA(c, cudaGetLastError());
  return CABLEGPU_OK;
}

StepParams make_params(cablegpu_ctx* c, int ktau, float dels) {
  StepParams p;
  p.ktau = ktau;
  p.dels = dels;
  p.medlyn = c->medlyn;
  p.thermal_fix = c->thermal_fix;
  p.litter = c->litter;
  p.rev_corr = c->rev_corr;
  p.fwsoil_mode = (c->switches & CABLEGPU_SW_FWSOIL_NONLINEAR) ? 1 : ((c->switches & CABLEGPU_SW_FWSOIL_LAI_KTAUL) ? 2 : 0);
  p.potev_pm = (c->switches & CABLEGPU_SW_POTEV_PM) ? 1 : 0;
  p.reduce_soilevp = (c->switches & CABLEGPU_SW_NEW_REDUCE_SOILEVP) ? 1 : 0;
  p.runoff_speed = (c->switches & CABLEGPU_SW_NEW_RUNOFF_SPEED) ? 1 : 0;
  p.soil_resp_off = (c->switches & CABLEGPU_SW_DIAG_SOIL_RESP_OFF) ? 1 : 0;
  p.forc = c->forc;
  p.forc.dels = dels;
  p.step_index = ktau - 1;
  p.mode = 0;
  p.final_cycle = 1;
  p.lai_refresh = 0;
  p.solve64 = c->solve64;
  p.canopy_pool = c->canopy_pool;
  return p;
}

int ensure_graph(cablegpu_ctx* c, float dels) {
  if (c->graph && c->graph_dels == dels && c->graph_diag == c->diag && c->graph_switches == c->switches &&
      c->graph_hostforc == (int)c->host_forcing && c->graph_capture == c->capture_forcing &&
      c->graph_seed == c->forc.seed && c->graph_doy0 == c->forc.doy0 && c->graph_sur == c->sur_enabled &&
      c->graph_gate == c->sur_gate && c->graph_solve64 == c->solve64 && c->graph_pool == c->canopy_pool &&
      std::equal(c->block, c->block + 5, c->graph_block))
    return CABLEGPU_OK;
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  StepParams p = make_params(c, 0, dels);
  cudaGraph_t g;
  CG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  long long before = c->launches;
  for (int i = 0; i < kGraphSteps; ++i) {
    int rc = launch_step(c, p, c->d_clock);
    if (rc) { cudaStreamEndCapture(c->stream, &g); return rc; }
    advance_clock_kernel<<<1, 1, 0, c->stream>>>(c->d_clock);
  }
  c->launches = before;   // captured launches are counted when replayed
  CG_CUDA(c, cudaStreamEndCapture(c->stream, &g));
  CG_CUDA(c, cudaGraphInstantiate(&c->graph, g, 0));
  cudaGraphDestroy(g);
  c->graph_dels = dels; c->graph_diag = c->diag; c->graph_switches = c->switches;
  c->graph_hostforc = (int)c->host_forcing; c->graph_capture = c->capture_forcing;
  c->graph_seed = c->forc.seed; c->graph_doy0 = c->forc.doy0;
  c->graph_sur = c->sur_enabled; c->graph_gate = c->sur_gate; c->graph_solve64 = c->solve64;
  c->graph_pool = c->canopy_pool;
  std::copy(c->block, c->block + 5, c->graph_block);
  return CABLEGPU_OK;
}

}  // namespace

extern "C" {

int cablegpu_num_fields(void) { return (int)registry().size(); }

int cablegpu_field_info(int id, const char** name, int* nlayer, int* dtype, int* kind) {
  if (id < 0 || id >= cablegpu_num_fields()) return CABLEGPU_ERR_ARG;
  const FieldDef& f = registry()[id];
  if (name) *name = f.name;
  if (nlayer) *nlayer = f.nlayer;
  if (dtype) *dtype = f.dtype;
  if (kind) *kind = f.kind;
  return CABLEGPU_OK;
}

int cablegpu_field_id(const char* name) {
  if (!name) return CABLEGPU_ERR_ARG;
  const auto& r = registry();
  for (size_t i = 0; i < r.size(); ++i)
    if (!std::strcmp(r[i].name, name)) return (int)i;
  return CABLEGPU_ERR_ARG;
}

int cablegpu_create(const cablegpu_tiles* tiles, int device, cablegpu_ctx** out) {
  if (!tiles || !out || tiles->mp <= 0 || tiles->mp > CABLEGPU_MAX_TILES || !tiles->iveg || !tiles->isoilm ||
      !tiles->vlai || !tiles->lat || tiles->order < -1 || tiles->order > 3)
    return CABLEGPU_ERR_ARG;
  for (int i = 0; i < tiles->mp; ++i)
    if (tiles->iveg[i] < 1 || tiles->iveg[i] > CG_NPFT || tiles->isoilm[i] < 1 || tiles->isoilm[i] > CG_NSOIL)
      return CABLEGPU_ERR_ARG;
  if (tiles->order == -1) {
    // autotuned: tile order and block sizes measured on a sample of these tiles
    int best_order = 0, blocks[5];
    float ms = 0.f;
    int rc = cablegpu_autotune(tiles, device, std::min(tiles->mp, 4 << 20), 8, &best_order, blocks, &ms);
    if (rc) return rc;
    cablegpu_tiles t = *tiles;
    t.order = best_order;
    rc = cablegpu_create(&t, device, out);
    if (rc) return rc;
    std::copy(blocks, blocks + 5, (*out)->block);
    return CABLEGPU_OK;
  }
  auto* c = new cablegpu_ctx();
  *out = c;
  c->device = device;
  c->order = tiles->order;
  c->mp = tiles->mp;
  c->ld = (tiles->mp + 255) / 256 * 256;
  CG_CUDA(c, cudaSetDevice(device));
  CG_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  // one arena, every field 256-byte aligned
  const auto& r = registry();
  std::vector<size_t> off(r.size());
  size_t bytes = 0;
  for (size_t i = 0; i < r.size(); ++i) {
    off[i] = bytes;
    bytes += ((size_t)r[i].nlayer * c->ld * storage_bytes(r[i].st) + 255) / 256 * 256;
  }
  c->arena_bytes = bytes;
  CG_CUDA(c, cudaMalloc(&c->arena, bytes));
  CG_CUDA(c, cudaMemsetAsync(c->arena, 0, bytes, c->stream));
  c->field_ptr.resize(r.size());
  for (size_t i = 0; i < r.size(); ++i) c->field_ptr[i] = c->arena + off[i];
  // tables
  CgTables h{};
  cg_build_tables(&h.pft, &h.soil);
  CG_CUDA(c, cudaMalloc(&c->d_tables, sizeof(CgTables)));
  CG_CUDA(c, cudaMemcpyAsync(c->d_tables, &h, sizeof(CgTables), cudaMemcpyHostToDevice, c->stream));
  upload_canopy_pft_table(h.pft, c->stream);
  prepare_phase_kernels();
  CG_CUDA(c, cudaGetLastError());
  // device tile order
  {
    std::vector<int> order(c->mp);
    for (int i = 0; i < c->mp; ++i) order[i] = i;
    if (tiles->order == 0 || tiles->order == 2 || tiles->order == 3) {
      // sort key, most significant first: plant type, soil type (order 0);
      // plant type, local solar hour, 5-degree latitude band, LAI (order 2),
      // so a warp's tiles share radiation and hence iteration counts; order 3
      // is order 2 applied within consecutive chunks of 2^CG_ORDER3_CHUNK_LOG2
      // caller tiles, so host-order forcing and outputs of a chunk stay
      // L2-resident while they are gathered into device order
      // (cablegpu_step_host)
      std::vector<std::pair<unsigned long long, int>> key(c->mp);
      for (int i = 0; i < c->mp; ++i) {
        unsigned long long k = (unsigned long long)(tiles->iveg[i] & 0xff) << 56;
        if (tiles->order == 3)
          k = (unsigned long long)(i >> CG_ORDER3_CHUNK_LOG2) << 51 | (unsigned long long)(tiles->iveg[i] & 0xff) << 43;
        if (tiles->order == 0) {
          k |= (unsigned long long)(tiles->isoilm[i] & 0xff) << 48;
        } else {
          const float ph = tiles->lonphase ? tiles->lonphase[i] : 0.f;
          const int hr = std::min(23, std::max(0, (int)ph));
          const int band = std::min(63, std::max(0, (int)((tiles->lat[i] + 90.f) / 5.f)));
          const int lai = std::min(255, std::max(0, (int)(tiles->vlai[i] * 32.f)));
          if (tiles->order == 2)
            k |= (unsigned long long)hr << 48 | (unsigned long long)band << 40 | (unsigned long long)lai << 32;
          else
            k |= (unsigned long long)hr << 38 | (unsigned long long)band << 32 | (unsigned long long)lai << 24;
        }
        key[i] = {k, i};
      }
      std::sort(key.begin(), key.end());
      for (int i = 0; i < c->mp; ++i) order[i] = key[i].second;
    }
    CG_CUDA(c, cudaMalloc(&c->d_order, sizeof(int) * c->mp));
    CG_CUDA(c, cudaMemcpy(c->d_order, order.data(), sizeof(int) * c->mp, cudaMemcpyHostToDevice));
    c->stage_bytes = (size_t)c->mp * 64;
    CG_CUDA(c, cudaMalloc(&c->d_stage, c->stage_bytes));
  }
  CG_CUDA(c, cudaMalloc(&c->d_clock, sizeof(int) * 4));
  CG_CUDA(c, cudaMallocHost(&c->h_clock, sizeof(int) * 4));
  CG_CUDA(c, cudaMallocHost(&c->h_status, sizeof(unsigned int)));
  c->dev.status = nullptr;
  CG_CUDA(c, cudaMalloc(&c->dev.status, sizeof(unsigned int)));
  CG_CUDA(c, cudaMemsetAsync(c->dev.status, 0, sizeof(unsigned int), c->stream));
  // tile description
  std::vector<float> lon(c->mp, 0.f), tb(c->mp, 288.f), sw(c->mp, 1.f), alb(c->mp);
  for (int i = 0; i < c->mp; ++i) alb[i] = h.soil.albsoil_vis[tiles->isoilm[i] - 1];
  c->h_iveg.assign(tiles->iveg, tiles->iveg + c->mp);
  c->h_isoilm.assign(tiles->isoilm, tiles->isoilm + c->mp);
  if (tiles->lonphase) std::memcpy(lon.data(), tiles->lonphase, sizeof(float) * c->mp);
  if (tiles->tbase) std::memcpy(tb.data(), tiles->tbase, sizeof(float) * c->mp);
  if (tiles->swscale) std::memcpy(sw.data(), tiles->swscale, sizeof(float) * c->mp);
  int rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("iveg"), tiles->iveg))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("isoilm"), tiles->isoilm))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("vlai"), tiles->vlai))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("lat"), tiles->lat))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("lonphase"), lon.data()))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("tbase"), tb.data()))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("swscale"), sw.data()))) return rc;
  if ((rc = cablegpu_set_field(c, cablegpu_field_id("albsoil"), alb.data()))) return rc;
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  return CABLEGPU_OK;
}

int cablegpu_destroy(cablegpu_ctx* c) {
  if (!c) return CABLEGPU_ERR_ARG;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  cudaFree(c->arena);
  cudaFree(c->d_tables);
  cudaFree(c->d_clock);
  cudaFree(c->d_order);
  cudaFree(c->d_stage);
  cudaFree(c->dev.status);
  if (c->d_harvest) cudaFree(c->d_harvest);
  if (c->d_harvest_n) cudaFree(c->d_harvest_n);
  if (c->d_sur_stats) cudaFree(c->d_sur_stats);
  if (c->io_ready) {
    cudaStreamSynchronize(c->cstream);
    cudaStreamSynchronize(c->dstream);
    for (int i = 0; i < 2; ++i) {
      cudaFree(c->d_fin[i]);
      cudaFree(c->d_fout[i]);
      cudaEventDestroy(c->ev_h2d[i]); cudaEventDestroy(c->ev_used[i]);
      cudaEventDestroy(c->ev_step[i]); cudaEventDestroy(c->ev_d2h[i]);
    }
    cudaStreamDestroy(c->cstream);
    cudaStreamDestroy(c->dstream);
  }
  if (c->d_sur_dt) cudaFree(c->d_sur_dt);
  if (c->d_bank) cudaFree(c->d_bank);
  sur_free(c->net);
  cudaFreeHost(c->h_clock);
  cudaFreeHost(c->h_status);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return CABLEGPU_OK;
}

int cablegpu_set_field(cablegpu_ctx* c, int id, const void* host) {
  if (!c || !host || id < 0 || id >= cablegpu_num_fields()) return fail(c, CABLEGPU_ERR_ARG, "set_field: bad argument");
  const FieldDef& f = registry()[id];
  const size_t n = (size_t)c->mp;
  const size_t hes = (f.dtype == CABLEGPU_F64) ? 8 : 4;   // host element size
  const size_t bytes = n * f.nlayer * hes;
  if (bytes > c->stage_bytes) return fail(c, CABLEGPU_ERR_ARG, "set_field: field too large");
  if (f.st == S_U8) {
    const int* h = (const int*)host;
    for (size_t i = 0; i < n * f.nlayer; ++i)
      if (h[i] < 0 || h[i] > 255) return fail(c, CABLEGPU_ERR_ARG, std::string("set_field: value out of range for ") + f.name);
  }
  CG_CUDA(c, cudaMemcpyAsync(c->d_stage, host, bytes, cudaMemcpyHostToDevice, c->stream));
  const int grid = (c->mp + 255) / 256;
  void* d = c->field_ptr[id];
  if (f.st == S_U8)
    scatter_in_kernel<uint8_t, int><<<grid, 256, 0, c->stream>>>((uint8_t*)d, (const int*)c->d_stage, c->d_order, c->mp, c->ld, f.nlayer);
  else if (f.st == S_F32)
    scatter_in_kernel<float, float><<<grid, 256, 0, c->stream>>>((float*)d, (const float*)c->d_stage, c->d_order, c->mp, c->ld, f.nlayer);
  else if (f.st == S_DF)
    scatter_in_df_kernel<<<grid, 256, 0, c->stream>>>((float*)d, (const double*)c->d_stage, c->d_order, c->mp, c->ld, f.nlayer);
  else
    scatter_in_kernel<double, double><<<grid, 256, 0, c->stream>>>((double*)d, (const double*)c->d_stage, c->d_order, c->mp, c->ld, f.nlayer);
  CG_CUDA(c, cudaGetLastError());
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  return CABLEGPU_OK;
}

namespace {
// Gathers one field into caller order in the staging buffer and queues its
// copy to host on the context's stream (no synchronisation).
int issue_get_field(cablegpu_ctx* c, int id, void* host) {
  if (!c || !host || id < 0 || id >= cablegpu_num_fields()) return fail(c, CABLEGPU_ERR_ARG, "get_field: bad argument");
  const FieldDef& f = registry()[id];
  if (f.kind == CABLEGPU_KIND_DIAG && !c->diag) return fail(c, CABLEGPU_ERR_STATE, "get_field: diagnostics are disabled");
  const size_t n = (size_t)c->mp;
  const size_t hes = (f.dtype == CABLEGPU_F64) ? 8 : 4;
  const size_t bytes = n * f.nlayer * hes;
  if (bytes > c->stage_bytes) return fail(c, CABLEGPU_ERR_ARG, "get_field: field too large");
  const int grid = (c->mp + 255) / 256;
  const void* d = c->field_ptr[id];
  if (f.st == S_U8)
    gather_out_kernel<int, uint8_t><<<grid, 256, 0, c->stream>>>((int*)c->d_stage, (const uint8_t*)d, c->d_order, c->mp, c->ld, f.nlayer);
  else if (f.st == S_F32)
    gather_out_kernel<float, float><<<grid, 256, 0, c->stream>>>((float*)c->d_stage, (const float*)d, c->d_order, c->mp, c->ld, f.nlayer);
  else if (f.st == S_DF)
    gather_out_df_kernel<<<grid, 256, 0, c->stream>>>((double*)c->d_stage, (const float*)d, c->d_order, c->mp, c->ld, f.nlayer);
  else
    gather_out_kernel<double, double><<<grid, 256, 0, c->stream>>>((double*)c->d_stage, (const double*)d, c->d_order, c->mp, c->ld, f.nlayer);
  CG_CUDA(c, cudaGetLastError());
  CG_CUDA(c, cudaMemcpyAsync(host, c->d_stage, bytes, cudaMemcpyDeviceToHost, c->stream));
  return CABLEGPU_OK;
}
}  // namespace

int cablegpu_get_field(cablegpu_ctx* c, int id, void* host) {
  const int rc = issue_get_field(c, id, host);
  if (rc) return rc;
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  return CABLEGPU_OK;
}

int cablegpu_get_fields(cablegpu_ctx* c, int n, const int* ids, void* const* host) {
  if (!c || n < 0 || (n > 0 && (!ids || !host))) return fail(c, CABLEGPU_ERR_ARG, "get_fields: bad argument");
  // the gathers reuse one staging buffer: each waits on the stream for the
  // copy before it, so the copies of all n fields go out back to back and
  // the caller waits once
  for (int i = 0; i < n; ++i) {
    const int rc = issue_get_field(c, ids[i], host[i]);
    if (rc) {
      cudaStreamSynchronize(c->stream);
      return rc;
    }
  }
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  return CABLEGPU_OK;
}

int cablegpu_field_device_ptr(cablegpu_ctx* c, int id, void** dptr, int* ld) {
  if (!c || !dptr || id < 0 || id >= cablegpu_num_fields()) return CABLEGPU_ERR_ARG;
  *dptr = c->field_ptr[id];
  if (ld) *ld = c->ld;
  return CABLEGPU_OK;
}

int cablegpu_cold_start(cablegpu_ctx* c, const double* snowd0, const double* tgg0, const double* wb0) {
  if (!c || !snowd0 || !tgg0 || !wb0) return fail(c, CABLEGPU_ERR_ARG, "cold_start: null argument");
  // the staging buffer belongs on the context's device, whichever device
  // the calling thread has current
  int prev = 0;
  CG_CUDA(c, cudaGetDevice(&prev));
  CG_CUDA(c, cudaSetDevice(c->device));
  const size_t n = (size_t)c->mp;
  double* tmp = nullptr;
  cudaError_t e = cudaMalloc(&tmp, 3 * n * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(tmp, snowd0, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + n, tgg0, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + 2 * n, wb0, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    bind_device_view(c);
    cold_start_kernel<<<(c->mp + 255) / 256, 256, 0, c->stream>>>(c->dev, c->d_tables, tmp, tmp + n, tmp + 2 * n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (tmp) {
    const cudaError_t ef = cudaFree(tmp);
    if (e == cudaSuccess) e = ef;
  }
  cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(c, CABLEGPU_ERR_CUDA, std::string("cold_start: ") + cudaGetErrorString(e));
  return CABLEGPU_OK;
}

int cablegpu_set_forcing(cablegpu_ctx* c, const float* host_forcing) {
  if (!c || !host_forcing) return fail(c, CABLEGPU_ERR_ARG, "set_forcing: null argument");
  c->host_forcing = true;
  return cablegpu_set_field(c, cablegpu_field_id("forcing_in"), host_forcing);
}

int cablegpu_set_synthetic_forcing(cablegpu_ctx* c, unsigned long long seed, int doy0) {
  if (!c || doy0 < 1 || doy0 > 365) return fail(c, CABLEGPU_ERR_ARG, "set_synthetic_forcing: bad argument");
  c->host_forcing = false;
  c->forc.seed = seed;
  c->forc.doy0 = doy0;
  return CABLEGPU_OK;
}

int cablegpu_set_canopy_schedule(cablegpu_ctx* c, int mode) {
  if (!c) return CABLEGPU_ERR_ARG;
  if (mode != CABLEGPU_CANOPY_POOL && mode != CABLEGPU_CANOPY_LANES)
    return fail(c, CABLEGPU_ERR_ARG, "set_canopy_schedule: unknown mode");
  c->canopy_pool = mode == CABLEGPU_CANOPY_POOL ? 1 : 0;
  return CABLEGPU_OK;
}

int cablegpu_set_soil_solve(cablegpu_ctx* c, int mode) {
  if (!c) return CABLEGPU_ERR_ARG;
  if (mode != CABLEGPU_SOLVE_FP64 && mode != CABLEGPU_SOLVE_FP32_CHANGE)
    return fail(c, CABLEGPU_ERR_ARG, "set_soil_solve: unknown mode");
  c->solve64 = mode == CABLEGPU_SOLVE_FP64 ? 1 : 0;
  return CABLEGPU_OK;
}

int cablegpu_set_options(cablegpu_ctx* c, int switches, int diag, int capture_forcing) {
  if (!c) return CABLEGPU_ERR_ARG;
  const int known = CABLEGPU_SW_MEDLYN | CABLEGPU_SW_SOIL_THERMAL_FIX | CABLEGPU_SW_LITTER | CABLEGPU_SW_L_REV_CORR |
                    CABLEGPU_SW_FWSOIL_NONLINEAR | CABLEGPU_SW_FWSOIL_LAI_KTAUL | CABLEGPU_SW_POTEV_PM |
                    CABLEGPU_SW_NEW_REDUCE_SOILEVP | CABLEGPU_SW_NEW_RUNOFF_SPEED | CABLEGPU_SW_DIAG_SOIL_RESP_OFF;
  if (switches & ~known) return fail(c, CABLEGPU_ERR_ARG, "set_options: unknown switch bit");
  if ((switches & CABLEGPU_SW_FWSOIL_NONLINEAR) && (switches & CABLEGPU_SW_FWSOIL_LAI_KTAUL))
    return fail(c, CABLEGPU_ERR_ARG, "set_options: two fwsoil_switch values");
  c->medlyn = (switches & CABLEGPU_SW_MEDLYN) ? 1 : 0;
  c->litter = (switches & CABLEGPU_SW_LITTER) ? 1 : 0;
  c->rev_corr = (switches & CABLEGPU_SW_L_REV_CORR) ? 1 : 0;
  const int fix = (switches & CABLEGPU_SW_SOIL_THERMAL_FIX) ? 1 : 0;
  if (fix != c->thermal_fix) {
    // the switch changes the soil heat capacity and dry conductivity
    // parameters: upload the matching tables, ordered after earlier steps
    CgTables h{};
    cg_build_tables(&h.pft, &h.soil);
    if (fix) cg_apply_soil_thermal_fix(&h.soil);
    CG_CUDA(c, cudaMemcpyAsync(c->d_tables, &h, sizeof(CgTables), cudaMemcpyHostToDevice, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->thermal_fix = fix;
  }
  c->switches = switches;
  c->diag = diag ? 1 : 0;
  c->capture_forcing = capture_forcing ? 1 : 0;
  return CABLEGPU_OK;
}

int cablegpu_step(cablegpu_ctx* c, int ktau, float dels) {
  if (!c || ktau < 1 || !(dels > 0.f)) return fail(c, CABLEGPU_ERR_ARG, "step: bad argument");
  return launch_step(c, make_params(c, ktau, dels), nullptr);
}

int cablegpu_step_explicit(cablegpu_ctx* c, int ktau, float dels, int lai_refresh) {
  if (!c || ktau < 1 || !(dels > 0.f)) return fail(c, CABLEGPU_ERR_ARG, "step_explicit: bad argument");
  StepParams p = make_params(c, ktau, dels);
  p.mode = 1;
  p.lai_refresh = lai_refresh ? 1 : 0;
  return launch_step(c, p, nullptr);
}

int cablegpu_step_implicit(cablegpu_ctx* c, int ktau, float dels, int cycleno, int numcycles) {
  if (!c || ktau < 1 || !(dels > 0.f) || numcycles < 1 || cycleno < 1 || cycleno > numcycles)
    return fail(c, CABLEGPU_ERR_ARG, "step_implicit: bad argument");
  StepParams p = make_params(c, ktau, dels);
  p.mode = 2;
  p.final_cycle = cycleno == numcycles ? 1 : 0;
  if (p.final_cycle) return launch_step(c, p, nullptr);
  // a cycle that is not the last runs on a copy of the banked fields
  const size_t ld = (size_t)c->ld;
  if (!c->d_bank) {
    size_t bytes = ld;   // flags
    for (const char* name : kBankFields) {
      const FieldDef& f = registry()[cablegpu_field_id(name)];
      bytes += storage_bytes(f.st) * (size_t)f.nlayer * ld;
    }
    CG_CUDA(c, cudaMalloc(&c->d_bank, bytes));
  }
  const int nbank = (int)(sizeof(kBankFields) / sizeof(kBankFields[0]));
  int ids[sizeof(kBankFields) / sizeof(kBankFields[0]) + 1];
  void* own[sizeof(kBankFields) / sizeof(kBankFields[0]) + 1];
  size_t off = 0;
  int nswapped = 0;
  cudaError_t ce = cudaSuccess;
  for (int i = 0; i <= nbank && ce == cudaSuccess; ++i) {
    ids[i] = cablegpu_field_id(i < nbank ? kBankFields[i] : "flags");
    const FieldDef& f = registry()[ids[i]];
    const size_t bytes = storage_bytes(f.st) * (size_t)f.nlayer * ld;
    own[i] = c->field_ptr[ids[i]];
    void* copy = (char*)c->d_bank + off;
    ce = cudaMemcpyAsync(copy, own[i], bytes, cudaMemcpyDeviceToDevice, c->stream);
    if (ce == cudaSuccess) { c->field_ptr[ids[i]] = copy; nswapped = i + 1; }
    off += bytes;
  }
  int rc = ce == cudaSuccess ? launch_step(c, p, nullptr) : CABLEGPU_OK;
  // the fields' own blocks again, whatever happened
  for (int i = 0; i < nswapped; ++i) c->field_ptr[ids[i]] = own[i];
  bind_device_view(c);
  CG_CUDA(c, ce);
  if (rc) return rc;
  bank_flags_kernel<<<(c->mp + 255) / 256, 256, 0, c->stream>>>((uint8_t*)own[nbank], (const uint8_t*)c->d_bank + off - ld,
                                                              c->mp);
  ++c->launches;
  CG_CUDA(c, cudaGetLastError());
  return CABLEGPU_OK;
}

int cablegpu_run(cablegpu_ctx* c, int ktau0, int nsteps, float dels) {
  if (!c || ktau0 < 1 || nsteps < 0 || !(dels > 0.f)) return fail(c, CABLEGPU_ERR_ARG, "run: bad argument");
  int done = 0;
  if (nsteps >= kGraphSteps) {
    int rc = ensure_graph(c, dels);
    if (rc) return rc;
    c->h_clock[0] = ktau0;
    CG_CUDA(c, cudaMemcpyAsync(c->d_clock, c->h_clock, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    while (nsteps - done >= kGraphSteps) {
      CG_CUDA(c, cudaGraphLaunch(c->graph, c->stream));
      // the five step kernels plus the one-thread clock kernel of each step
      c->launches += (kKernelsPerStep + 1 + (c->sur_enabled ? 1 : 0)) * kGraphSteps;
      done += kGraphSteps;
    }
    // the pinned clock buffer must not be rewritten before the copy ran
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  for (; done < nsteps; ++done) {
    int rc = launch_step(c, make_params(c, ktau0 + done, dels), nullptr);
    if (rc) return rc;
  }
  return CABLEGPU_OK;
}

int cablegpu_step_host(cablegpu_ctx* c, int ktau, float dels, const float* host_forcing, float* host_out) {
  if (!c || ktau < 1 || !(dels > 0.f) || !host_forcing || !host_out)
    return fail(c, CABLEGPU_ERR_ARG, "step_host: bad argument");
  if (!c->io_ready) {
    CG_CUDA(c, cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking));
    CG_CUDA(c, cudaStreamCreateWithFlags(&c->dstream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
      CG_CUDA(c, cudaMalloc(&c->d_fin[i], sizeof(float) * CG_NFORC * c->mp));
      CG_CUDA(c, cudaMalloc(&c->d_fout[i], sizeof(float) * CG_NOUT * c->mp));
      for (cudaEvent_t* e : {&c->ev_h2d[i], &c->ev_used[i], &c->ev_step[i], &c->ev_d2h[i]})
        CG_CUDA(c, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
      // slot free from the start
      CG_CUDA(c, cudaEventRecord(c->ev_used[i], c->stream));
      CG_CUDA(c, cudaEventRecord(c->ev_d2h[i], c->dstream));
    }
    c->io_ready = true;
  }
  const int slot = (int)(c->io_count & 1);
  const size_t fb = sizeof(float) * CG_NFORC * c->mp, ob = sizeof(float) * CG_NOUT * c->mp;
  // upload this step's forcing once the step two back has consumed the slot
  CG_CUDA(c, cudaStreamWaitEvent(c->cstream, c->ev_used[slot], 0));
  CG_CUDA(c, cudaMemcpyAsync(c->d_fin[slot], host_forcing, fb, cudaMemcpyHostToDevice, c->cstream));
  CG_CUDA(c, cudaEventRecord(c->ev_h2d[slot], c->cstream));
  // the step: the radiation kernel reads the forcing from the staging slot
  // and the canopy and soil-water kernels write the outputs to the output
  // slot, both in caller order, once the slot's previous download is done
  CG_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_h2d[slot], 0));
  CG_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_d2h[slot], 0));
  c->io_forcing = c->d_fin[slot];
  c->io_out = c->d_fout[slot];
  int rc = launch_step(c, make_params(c, ktau, dels), nullptr);
  c->io_forcing = nullptr;
  c->io_out = nullptr;
  if (rc) return rc;
  CG_CUDA(c, cudaEventRecord(c->ev_used[slot], c->stream));
  CG_CUDA(c, cudaEventRecord(c->ev_step[slot], c->stream));
  CG_CUDA(c, cudaStreamWaitEvent(c->dstream, c->ev_step[slot], 0));
  CG_CUDA(c, cudaMemcpyAsync(host_out, c->d_fout[slot], ob, cudaMemcpyDeviceToHost, c->dstream));
  CG_CUDA(c, cudaEventRecord(c->ev_d2h[slot], c->dstream));
  ++c->io_count;
  return CABLEGPU_OK;
}

}  // extern "C"

namespace {
// blocks handed out by cablegpu_host_alloc (cablegpu_host_free takes only these)
std::mutex g_host_mu;
std::vector<void*> g_host_blocks;
}  // namespace

extern "C" {

int cablegpu_host_alloc(size_t bytes, void** out) {
  if (!out || bytes == 0) return CABLEGPU_ERR_ARG;
  *out = nullptr;
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess || !p) return CABLEGPU_ERR_CUDA;
  std::memset(p, 0, bytes);
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    g_host_blocks.push_back(p);
  }
  *out = p;
  return CABLEGPU_OK;
}

int cablegpu_host_free(void* ptr) {
  if (!ptr) return CABLEGPU_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = std::find(g_host_blocks.begin(), g_host_blocks.end(), ptr);
    if (it == g_host_blocks.end()) return CABLEGPU_ERR_ARG;
    g_host_blocks.erase(it);
  }
  return cudaFreeHost(ptr) == cudaSuccess ? CABLEGPU_OK : CABLEGPU_ERR_CUDA;
}

int cablegpu_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return CABLEGPU_ERR_ARG;
  return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? CABLEGPU_OK : CABLEGPU_ERR_CUDA;
}

int cablegpu_host_unregister(void* ptr) {
  if (!ptr) return CABLEGPU_ERR_ARG;
  return cudaHostUnregister(ptr) == cudaSuccess ? CABLEGPU_OK : CABLEGPU_ERR_CUDA;
}

int cablegpu_set_host_layout(cablegpu_ctx* c, int layout) {
  if (!c || (layout != 0 && layout != 1)) return fail(c, CABLEGPU_ERR_ARG, "set_host_layout: layout must be 0 or 1");
  if (c->io_ready) CG_CUDA(c, cudaStreamSynchronize(c->stream));   // no step in flight changes layout
  c->host_layout = layout;
  return CABLEGPU_OK;
}

int cablegpu_tile_order(cablegpu_ctx* c, int* order_out) {
  if (!c || !order_out) return fail(c, CABLEGPU_ERR_ARG, "tile_order: null argument");
  CG_CUDA(c, cudaMemcpy(order_out, c->d_order, sizeof(int) * (size_t)c->mp, cudaMemcpyDeviceToHost));
  return CABLEGPU_OK;
}

int cablegpu_synchronize(cablegpu_ctx* c) {
  if (!c) return CABLEGPU_ERR_ARG;
  if (c->io_ready) {
    CG_CUDA(c, cudaStreamSynchronize(c->cstream));
    CG_CUDA(c, cudaStreamSynchronize(c->dstream));
  }
  CG_CUDA(c, cudaMemcpyAsync(c->h_status, c->dev.status, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*c->h_status) {
    const unsigned int st = *c->h_status;
    CG_CUDA(c, cudaMemsetAsync(c->dev.status, 0, sizeof(unsigned int), c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (st & 1u) return fail(c, CABLEGPU_ERR_NONFINITE, "a step produced a non-finite output flux");
    return fail(c, CABLEGPU_ERR_CUDA,
                "surrogate network: a tensor-core pass did not complete in time; the blocks affected used the "
                "plain dryLeaf iteration");
  }
  return CABLEGPU_OK;
}

int cablegpu_run_timed(cablegpu_ctx* c, int ktau0, int nsteps, float dels, float* ms_total) {
  if (!c || !ms_total) return CABLEGPU_ERR_ARG;
  if (nsteps >= kGraphSteps) { int rc = ensure_graph(c, dels); if (rc) return rc; }
  cudaEvent_t a, b;
  CG_CUDA(c, cudaEventCreate(&a));
  CG_CUDA(c, cudaEventCreate(&b));
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  CG_CUDA(c, cudaEventRecord(a, c->stream));
  int rc = cablegpu_run(c, ktau0, nsteps, dels);
  if (rc) return rc;
  CG_CUDA(c, cudaEventRecord(b, c->stream));
  CG_CUDA(c, cudaEventSynchronize(b));
  CG_CUDA(c, cudaEventElapsedTime(ms_total, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return CABLEGPU_OK;
}

int cablegpu_coupled_timed(cablegpu_ctx* c, int ktau0, int nsteps, float dels, int numcycles, float* ms_total) {
  if (!c || !ms_total || ktau0 < 1 || nsteps < 1 || numcycles < 1 || !(dels > 0.f))
    return fail(c, CABLEGPU_ERR_ARG, "coupled_timed: bad argument");
  cudaEvent_t a, b;
  CG_CUDA(c, cudaEventCreate(&a));
  CG_CUDA(c, cudaEventCreate(&b));
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  CG_CUDA(c, cudaEventRecord(a, c->stream));
  int rc = CABLEGPU_OK;
  for (int n = 0; n < nsteps && rc == CABLEGPU_OK; ++n) {
    rc = cablegpu_step_explicit(c, ktau0 + n, dels, 1);
    for (int cyc = 1; cyc <= numcycles && rc == CABLEGPU_OK; ++cyc)
      rc = cablegpu_step_implicit(c, ktau0 + n, dels, cyc, numcycles);
  }
  if (rc == CABLEGPU_OK) {
    CG_CUDA(c, cudaEventRecord(b, c->stream));
    CG_CUDA(c, cudaEventSynchronize(b));
    CG_CUDA(c, cudaEventElapsedTime(ms_total, a, b));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

int cablegpu_kernel_timed(cablegpu_ctx* c, int ktau0, int nsteps, float dels, float* ms_per_launch) {
  if (!c || !ms_per_launch || nsteps <= 0) return CABLEGPU_ERR_ARG;
  std::vector<cudaEvent_t> ev(2 * nsteps);
  for (auto& e : ev) CG_CUDA(c, cudaEventCreate(&e));
  for (int i = 0; i < nsteps; ++i) {
    CG_CUDA(c, cudaEventRecord(ev[2 * i], c->stream));
    int rc = launch_step(c, make_params(c, ktau0 + i, dels), nullptr);
    if (rc) return rc;
    CG_CUDA(c, cudaEventRecord(ev[2 * i + 1], c->stream));
  }
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  double tot = 0.0;
  for (int i = 0; i < nsteps; ++i) {
    float ms = 0.f;
    CG_CUDA(c, cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]));
    tot += ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  *ms_per_launch = (float)(tot / nsteps);
  return CABLEGPU_OK;
}

int cablegpu_harvest(cablegpu_ctx* c, int ktau0, int nsteps, float dels, float prob, unsigned long long seed,
                     long long capacity, long long* nrows) {
  if (!c || ktau0 < 1 || nsteps < 1 || !(dels > 0.f) || !(prob > 0.f) || prob > 1.f || capacity < 1)
    return fail(c, CABLEGPU_ERR_ARG, "harvest: bad argument");
  if (capacity > c->harvest_cap) {
    if (c->d_harvest) { CG_CUDA(c, cudaFree(c->d_harvest)); c->d_harvest = nullptr; c->harvest_cap = 0; }
    CG_CUDA(c, cudaMalloc(&c->d_harvest, (size_t)capacity * 16 * sizeof(float)));
    c->harvest_cap = capacity;
  }
  if (!c->d_harvest_n) CG_CUDA(c, cudaMalloc(&c->d_harvest_n, sizeof(unsigned long long)));
  CG_CUDA(c, cudaMemsetAsync(c->d_harvest_n, 0, sizeof(unsigned long long), c->stream));
  c->harvesting = true;
  c->harvest_prob = prob;
  c->harvest_seed = seed;
  int rc = CABLEGPU_OK;
  for (int n = 0; n < nsteps && !rc; ++n) rc = launch_step(c, make_params(c, ktau0 + n, dels), nullptr);
  c->harvesting = false;
  if (rc) return rc;
  unsigned long long h = 0;
  CG_CUDA(c, cudaMemcpyAsync(&h, c->d_harvest_n, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->harvest_rows = (long long)std::min<unsigned long long>(h, (unsigned long long)c->harvest_cap);
  if (nrows) *nrows = c->harvest_rows;
  return CABLEGPU_OK;
}

int cablegpu_harvest_rows(cablegpu_ctx* c, float* host, long long n) {
  if (!c || !host || n < 0 || n > c->harvest_rows) return fail(c, CABLEGPU_ERR_ARG, "harvest_rows: bad argument");
  CG_CUDA(c, cudaMemcpyAsync(host, c->d_harvest, (size_t)n * 16 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  return CABLEGPU_OK;
}

static int ensure_net(cablegpu_ctx* c) {
  if (c->net.params) return CABLEGPU_OK;
  std::string e;
  if (sur_alloc(c->net, e)) return fail(c, CABLEGPU_ERR_CUDA, e);
  CG_CUDA(c, cudaMalloc(&c->d_sur_stats, 2 * sizeof(unsigned long long)));
  CG_CUDA(c, cudaMemset(c->d_sur_stats, 0, 2 * sizeof(unsigned long long)));
  CG_CUDA(c, cudaMalloc(&c->d_sur_dt, (size_t)c->ld * sizeof(float)));
  return CABLEGPU_OK;
}

int cablegpu_surrogate_train(cablegpu_ctx* c, int epochs, int batch, float lr, float val_frac,
                             unsigned long long seed, float* losses) {
  if (!c || epochs < 1 || batch < 128 || !(lr > 0.f) || val_frac < 0.f || val_frac >= 1.f)
    return fail(c, CABLEGPU_ERR_ARG, "surrogate_train: bad argument");
  const long long nval = (long long)(val_frac * (double)c->harvest_rows);
  const long long ntrain = c->harvest_rows - nval;
  if (ntrain < 128) return fail(c, CABLEGPU_ERR_STATE, "surrogate_train: harvest fewer than 128 training rows first");
  int rc = ensure_net(c);
  if (rc) return rc;
  std::string e;
  rc = sur_fit(c->net, c->d_harvest, ntrain, nval, epochs, batch, lr, seed, true, losses, c->stream, e);
  if (rc) return fail(c, rc, e);
  c->net_ready = true;
  return CABLEGPU_OK;
}

int cablegpu_surrogate_weights(cablegpu_ctx* c, float* params, float* norm, int set) {
  if (!c || !params || !norm) return fail(c, CABLEGPU_ERR_ARG, "surrogate_weights: null argument");
  int rc = ensure_net(c);
  if (rc) return rc;
  const size_t pb = cg::sur::NPARAM * sizeof(float), nb = cg::sur::NNORM * sizeof(float);
  if (set) {
    CG_CUDA(c, cudaMemcpyAsync(c->net.params, params, pb, cudaMemcpyHostToDevice, c->stream));
    CG_CUDA(c, cudaMemcpyAsync(c->net.norm, norm, nb, cudaMemcpyHostToDevice, c->stream));
    std::string e;
    if (sur_pack(c->net, c->stream, e)) return fail(c, CABLEGPU_ERR_CUDA, e);
    c->net_ready = true;
  } else {
    if (!c->net_ready) return fail(c, CABLEGPU_ERR_STATE, "surrogate_weights: no trained network");
    CG_CUDA(c, cudaMemcpyAsync(params, c->net.params, pb, cudaMemcpyDeviceToHost, c->stream));
    CG_CUDA(c, cudaMemcpyAsync(norm, c->net.norm, nb, cudaMemcpyDeviceToHost, c->stream));
  }
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  return CABLEGPU_OK;
}

int cablegpu_set_surrogate(cablegpu_ctx* c, int mode, float gate_kelvin) {
  if (!c || mode < 0 || mode > 2 || !(gate_kelvin > 0.f) || gate_kelvin > 0.1f)
    return fail(c, CABLEGPU_ERR_ARG, "set_surrogate: mode 0..2, gate in (0, 0.1] K");
  if (mode && !c->net_ready) return fail(c, CABLEGPU_ERR_STATE, "set_surrogate: train or set the network first");
  c->sur_enabled = mode;
  c->sur_gate = gate_kelvin;
  return CABLEGPU_OK;
}

int cablegpu_surrogate_stats(cablegpu_ctx* c, long long* tried, long long* accepted, int reset) {
  if (!c || !tried || !accepted) return CABLEGPU_ERR_ARG;
  *tried = 0;
  *accepted = 0;
  if (!c->d_sur_stats) return CABLEGPU_OK;
  unsigned long long h[2];
  CG_CUDA(c, cudaMemcpyAsync(h, c->d_sur_stats, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if (reset) CG_CUDA(c, cudaMemsetAsync(c->d_sur_stats, 0, sizeof(h), c->stream));
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  *tried = (long long)h[0];
  *accepted = (long long)h[1];
  return CABLEGPU_OK;
}

int cablegpu_phase_timed(cablegpu_ctx* c, int ktau0, int nsteps, float dels, float* ms_per_phase) {
  if (!c || !ms_per_phase || nsteps <= 0) return CABLEGPU_ERR_ARG;
  // phases: radiation, canopy, snow pack, soil heat, soil water, surrogate network
  constexpr int K = kKernelsPerStep + 1;
  std::vector<cudaEvent_t> ev((K + 1) * nsteps);
  for (auto& e : ev) CG_CUDA(c, cudaEventCreate(&e));
  bind_device_view(c);
  const bool diag = c->diag != 0;
  const bool sur = c->sur_enabled != 0;
  for (int i = 0; i < nsteps; ++i) {
    const StepParams p = make_params(c, ktau0 + i, dels);
    cudaEvent_t* e = &ev[(K + 1) * i];
    CG_CUDA(c, cudaEventRecord(e[0], c->stream));
    launch_phase_a(diag, c->stream, c->dev, c->d_tables, p, nullptr, c->block[0]);
    CG_CUDA(c, cudaEventRecord(e[1], c->stream));
    if (sur) {
      int rc = launch_sur_net(c);
      if (rc) return rc;
    }
    CG_CUDA(c, cudaEventRecord(e[2], c->stream));
    if (sur) launch_phase_b_sur(diag, c->stream, c->dev, c->d_tables, p, nullptr, c->block[1]);
    else launch_phase_b(diag, c->stream, c->dev, c->d_tables, p, nullptr, c->block[1]);
    CG_CUDA(c, cudaEventRecord(e[3], c->stream));
    launch_phase_c1(diag, c->stream, c->dev, c->d_tables, p, nullptr, c->block[2]);
    CG_CUDA(c, cudaEventRecord(e[4], c->stream));
    launch_phase_c2(diag, c->stream, c->dev, c->d_tables, p, nullptr, c->block[3]);
    CG_CUDA(c, cudaEventRecord(e[5], c->stream));
    launch_phase_c3(diag, c->stream, c->dev, c->d_tables, p, nullptr, c->block[4]);
    CG_CUDA(c, cudaEventRecord(e[6], c->stream));
    CG_CUDA(c, cudaGetLastError());
    c->launches += kKernelsPerStep + (sur ? 1 : 0);
  }
  CG_CUDA(c, cudaStreamSynchronize(c->stream));
  // event intervals: [a][net][b][c1][c2][c3] -> output order a, b, c1, c2, c3, net
  const int order[K] = {0, 5, 1, 2, 3, 4};
  for (int k = 0; k < K; ++k) ms_per_phase[k] = 0.f;
  for (int i = 0; i < nsteps; ++i) {
    for (int k = 0; k < K; ++k) {
      float ms = 0.f;
      CG_CUDA(c, cudaEventElapsedTime(&ms, ev[(K + 1) * i + k], ev[(K + 1) * i + k + 1]));
      ms_per_phase[order[k]] += ms / nsteps;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return CABLEGPU_OK;
}

int cablegpu_set_blocks(cablegpu_ctx* c, const int* block5) {
  if (!c || !block5) return CABLEGPU_ERR_ARG;
  for (int k = 0; k < 5; ++k)
    if (block5[k] < 32 || block5[k] > 256 || block5[k] % 32) return fail(c, CABLEGPU_ERR_ARG, "set_blocks: 32..256, multiple of 32");
  std::copy(block5, block5 + 5, c->block);
  return CABLEGPU_OK;
}

int cablegpu_get_config(cablegpu_ctx* c, int* order, int* block5) {
  if (!c) return CABLEGPU_ERR_ARG;
  if (order) *order = c->order;
  if (block5) std::copy(c->block, c->block + 5, block5);
  return CABLEGPU_OK;
}

int cablegpu_tune_blocks(cablegpu_ctx* c, int ktau0, int nsteps, float dels, int* block5_out, float* ms_out) {
  if (!c || nsteps < 1 || nsteps > 64 || !(dels > 0.f)) return fail(c, CABLEGPU_ERR_ARG, "tune_blocks: 1..64 steps, dels > 0");
  CG_CUDA(c, cudaSetDevice(c->device));
  // every per-tile field lives in the arena: a copy of it taken before the
  // candidates' steps and put back after each leaves the context's state as
  // it was; the status word and the surrogate's counters are read back and
  // restored the same way
  char* snap = nullptr;
  CG_CUDA(c, cudaMalloc(&snap, c->arena_bytes));
  unsigned int status0 = 0;
  int rc = CABLEGPU_OK;
  auto cp = [&](void* dst, const void* src, size_t n, cudaMemcpyKind k) {
    if (rc) return;
    cudaError_t e = cudaMemcpyAsync(dst, src, n, k, c->stream);
    if (e != cudaSuccess) rc = fail(c, CABLEGPU_ERR_CUDA, std::string("tune_blocks: ") + cudaGetErrorString(e));
  };
  unsigned long long stats0[2] = {0ull, 0ull};
  cp(snap, c->arena, c->arena_bytes, cudaMemcpyDeviceToDevice);
  cp(&status0, c->dev.status, sizeof(unsigned int), cudaMemcpyDeviceToHost);
  if (c->d_sur_stats) cp(stats0, c->d_sur_stats, sizeof(stats0), cudaMemcpyDeviceToHost);
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = fail(c, CABLEGPU_ERR_CUDA, "tune_blocks: sync");
  const int cand_block[4] = {32, 64, 128, 256};
  int saved[5], pick[5];
  std::copy(c->block, c->block + 5, saved);
  std::copy(c->block, c->block + 5, pick);
  float per[5] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
  for (int b = 0; b < 4 && !rc; ++b) {
    std::fill(c->block, c->block + 5, cand_block[b]);
    float ms[6];
    rc = cablegpu_phase_timed(c, ktau0, nsteps, dels, ms);
    cp(c->arena, snap, c->arena_bytes, cudaMemcpyDeviceToDevice);
    for (int k = 0; k < 5 && !rc; ++k)
      if (ms[k] < per[k]) { per[k] = ms[k]; pick[k] = cand_block[b]; }
  }
  cp(c->dev.status, &status0, sizeof(unsigned int), cudaMemcpyHostToDevice);
  if (c->d_sur_stats) cp(c->d_sur_stats, stats0, sizeof(stats0), cudaMemcpyHostToDevice);
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = fail(c, CABLEGPU_ERR_CUDA, "tune_blocks: sync");
  cudaFree(snap);
  std::copy(rc ? saved : pick, (rc ? saved : pick) + 5, c->block);
  if (rc) return rc;
  if (block5_out) std::copy(pick, pick + 5, block5_out);
  if (ms_out) *ms_out = per[0] + per[1] + per[2] + per[3] + per[4];
  return CABLEGPU_OK;
}

int cablegpu_autotune(const cablegpu_tiles* tiles, int device, int sample_tiles, int nsteps, int* order_out,
                      int* block5_out, float* ms_out) {
  if (!tiles || tiles->mp <= 0 || sample_tiles < 1024 || nsteps < 1 || !order_out || !block5_out)
    return CABLEGPU_ERR_ARG;
  // an evenly strided sample of the tiles, cold-started without snow at
  // 285 K and 0.25 soil moisture, driven by the synthetic forcing
  const int n = std::min(sample_tiles, tiles->mp);
  std::vector<int> iveg(n), isoil(n);
  std::vector<float> vlai(n), lat(n), ph(n), tb(n), sw(n);
  for (int i = 0; i < n; ++i) {
    const int j = (int)((long long)i * tiles->mp / n);
    iveg[i] = tiles->iveg[j]; isoil[i] = tiles->isoilm[j]; vlai[i] = tiles->vlai[j]; lat[i] = tiles->lat[j];
    ph[i] = tiles->lonphase ? tiles->lonphase[j] : 0.f;
    tb[i] = tiles->tbase ? tiles->tbase[j] : 288.f;
    sw[i] = tiles->swscale ? tiles->swscale[j] : 1.f;
  }
  std::vector<double> sn(n, 0.0), tg(n, 285.0), wb(n, 0.25);
  // 32: a block releases its registers when its last warp finishes, so
  // one-warp blocks free a diverged warp's slot early (the canopy kernel)
  const int cand_block[4] = {32, 64, 128, 256};
  float best = 1e30f;
  for (int order = 0; order <= 3; ++order) {
    cablegpu_tiles t = {n, iveg.data(), isoil.data(), vlai.data(), lat.data(), ph.data(), tb.data(), sw.data(), order};
    cablegpu_ctx* c = nullptr;
    int rc = cablegpu_create(&t, device, &c);
    if (!rc) rc = cablegpu_cold_start(c, sn.data(), tg.data(), wb.data());
    if (!rc) rc = cablegpu_set_synthetic_forcing(c, 1234567ull, 1);
    if (!rc) rc = cablegpu_run(c, 1, 4, 1800.f);
    float per[5] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
    int pick[5] = {128, 128, 128, 128, 128};
    for (int b = 0; b < 4 && !rc; ++b) {
      int bb[5];
      std::fill(bb, bb + 5, cand_block[b]);
      rc = cablegpu_set_blocks(c, bb);
      float ms[6];
      if (!rc) rc = cablegpu_phase_timed(c, 5 + b * nsteps, nsteps, 1800.f, ms);
      for (int k = 0; k < 5 && !rc; ++k)
        if (ms[k] < per[k]) { per[k] = ms[k]; pick[k] = cand_block[b]; }
    }
    if (c) cablegpu_destroy(c);
    if (rc) return rc;
    const float tot = per[0] + per[1] + per[2] + per[3] + per[4];
    if (tot < best) {
      best = tot;
      *order_out = order;
      std::copy(pick, pick + 5, block5_out);
    }
  }
  if (ms_out) *ms_out = best;
  return CABLEGPU_OK;
}

long long cablegpu_launch_count(cablegpu_ctx* c) { return c ? c->launches : -1; }

// ---------------------------------------------------------------- files
namespace {

cgio::Entry file_entry(const char* name, uint32_t dtype, uint32_t width) {
  cgio::Entry e{};
  std::strncpy(e.name, name, sizeof(e.name) - 1);
  e.dtype = dtype;
  e.width = width;
  return e;
}

// the registry fields a restart file carries: tile description, state and
// the last step's outputs (the reference's restart holds ga and trad; ga is
// read again by ssnow_potev = 'P-M')
bool in_restart(const FieldDef& f) {
  return f.kind == CABLEGPU_KIND_PARAM || f.kind == CABLEGPU_KIND_STATE || f.kind == CABLEGPU_KIND_OUTPUT;
}
uint32_t file_dtype(const FieldDef& f) { return f.st == S_DF ? cgio::kDF32 : (uint32_t)f.dtype; }

}  // namespace

int cablegpu_restart_write(cablegpu_ctx* c, const char* path, int ktau) {
  if (!c || !path) return fail(c, CABLEGPU_ERR_ARG, "restart_write: null argument");
  const auto& reg = registry();
  std::vector<cgio::Entry> entries;
  std::vector<int> ids;
  for (int i = 0; i < (int)reg.size(); ++i)
    if (in_restart(reg[i])) { entries.push_back(file_entry(reg[i].name, file_dtype(reg[i]), reg[i].nlayer)); ids.push_back(i); }
  cgio::File f;
  if (cgio::create(f, path, CABLEGPU_FILE_RESTART, (uint64_t)c->mp, entries, 1, ktau, c->forc.doy0, c->forc.dels))
    return fail(c, CABLEGPU_ERR_IO, "restart_write: " + f.err);
  std::vector<char> host((size_t)c->mp * CG_MS * 8);
  int rc = CABLEGPU_OK;
  for (size_t j = 0; j < ids.size() && rc == CABLEGPU_OK; ++j) {
    const FieldDef& fd = reg[ids[j]];
    if (fd.st == S_DF) {
      // the exact word pairs: high rows then low rows, as stored
      const int grid = (c->mp + 255) / 256;
      gather_out_kernel<float, float><<<grid, 256, 0, c->stream>>>((float*)c->d_stage, (const float*)c->field_ptr[ids[j]],
                                                                   c->d_order, c->mp, c->ld, 2 * fd.nlayer);
      CG_CUDA(c, cudaGetLastError());
      CG_CUDA(c, cudaMemcpyAsync(host.data(), c->d_stage, (size_t)c->mp * 2 * fd.nlayer * sizeof(float),
                                 cudaMemcpyDeviceToHost, c->stream));
      CG_CUDA(c, cudaStreamSynchronize(c->stream));
    } else {
      rc = cablegpu_get_field(c, ids[j], host.data());
    }
    if (rc == CABLEGPU_OK && cgio::write_block(f, 0, (int)j, host.data()))
      rc = fail(c, CABLEGPU_ERR_IO, "restart_write: " + f.err);
  }
  cgio::close(f);
  return rc;
}

int cablegpu_restart_read(cablegpu_ctx* c, const char* path, int* ktau) {
  if (!c || !path) return fail(c, CABLEGPU_ERR_ARG, "restart_read: null argument");
  cgio::File f;
  if (cgio::open_read(f, path)) return fail(c, CABLEGPU_ERR_IO, "restart_read: " + f.err);
  struct Closer { cgio::File& f; ~Closer() { cgio::close(f); } } closer{f};
  if (f.h.kind != CABLEGPU_FILE_RESTART || f.h.nrecords != 1)
    return fail(c, CABLEGPU_ERR_IO, "restart_read: not a restart file");
  if (f.h.mp != (uint64_t)c->mp) return fail(c, CABLEGPU_ERR_ARG, "restart_read: the file's tile count differs");
  const auto& reg = registry();
  std::vector<char> host((size_t)c->mp * CG_MS * 8), mine((size_t)c->mp * 4);
  // the tiles must be the context's
  for (const char* name : {"iveg", "isoilm"}) {
    const int id = cablegpu_field_id(name), k = cgio::find(f, name);
    if (k < 0 || f.fields[k].dtype != cgio::kI32 || f.fields[k].width != 1)
      return fail(c, CABLEGPU_ERR_IO, std::string("restart_read: no valid field ") + name);
    if (cgio::read_block(f, 0, k, host.data())) return fail(c, CABLEGPU_ERR_IO, "restart_read: read failed");
    int rc = cablegpu_get_field(c, id, mine.data());
    if (rc) return rc;
    if (std::memcmp(host.data(), mine.data(), (size_t)c->mp * 4) != 0)
      return fail(c, CABLEGPU_ERR_ARG, std::string("restart_read: the file's ") + name + " differs from the context's");
  }
  for (int i = 0; i < (int)reg.size(); ++i) {
    const FieldDef& fd = reg[i];
    if (fd.kind != CABLEGPU_KIND_STATE && fd.kind != CABLEGPU_KIND_OUTPUT) continue;
    const int k = cgio::find(f, fd.name);
    if (k < 0) return fail(c, CABLEGPU_ERR_IO, std::string("restart_read: missing field ") + fd.name);
    if (f.fields[k].dtype != file_dtype(fd) || f.fields[k].width != (uint32_t)fd.nlayer)
      return fail(c, CABLEGPU_ERR_IO, std::string("restart_read: wrong type or width of ") + fd.name);
    if (cgio::read_block(f, 0, k, host.data())) return fail(c, CABLEGPU_ERR_IO, "restart_read: read failed");
    if (fd.st == S_DF) {
      const int grid = (c->mp + 255) / 256;
      CG_CUDA(c, cudaMemcpyAsync(c->d_stage, host.data(), (size_t)c->mp * 2 * fd.nlayer * sizeof(float),
                                 cudaMemcpyHostToDevice, c->stream));
      scatter_in_kernel<float, float><<<grid, 256, 0, c->stream>>>((float*)c->field_ptr[i], (const float*)c->d_stage,
                                                                   c->d_order, c->mp, c->ld, 2 * fd.nlayer);
      CG_CUDA(c, cudaGetLastError());
      CG_CUDA(c, cudaStreamSynchronize(c->stream));
    } else {
      int rc = cablegpu_set_field(c, i, host.data());
      if (rc) return rc;
    }
  }
  // the per-tile soil albedo, where the file carries it
  {
    const int k = cgio::find(f, "albsoil");
    if (k >= 0 && f.fields[k].dtype == cgio::kF32 && f.fields[k].width == 1) {
      if (cgio::read_block(f, 0, k, host.data())) return fail(c, CABLEGPU_ERR_IO, "restart_read: read failed");
      int rc = cablegpu_set_field(c, cablegpu_field_id("albsoil"), host.data());
      if (rc) return rc;
    }
  }
  if (ktau) *ktau = f.h.ktau;
  return CABLEGPU_OK;
}

int cablegpu_forcing_file_write(const char* path, int mp, int nsteps, int doy0, float dels, const float* forcing) {
  if (!path || mp < 1 || nsteps < 1 || !forcing || !(dels > 0.f)) return CABLEGPU_ERR_ARG;
  cgio::File f;
  if (cgio::create(f, path, CABLEGPU_FILE_FORCING, (uint64_t)mp, {file_entry("met", cgio::kF32, CG_NFORC)},
                   (uint32_t)nsteps, 1, doy0, dels))
    return CABLEGPU_ERR_IO;
  int rc = CABLEGPU_OK;
  for (int n = 0; n < nsteps && rc == CABLEGPU_OK; ++n)
    if (cgio::write_block(f, (uint32_t)n, 0, forcing + (size_t)n * CG_NFORC * mp)) rc = CABLEGPU_ERR_IO;
  cgio::close(f);
  return rc;
}

int cablegpu_file_info(const char* path, int* kind, long long* mp, int* nrecords, int* nfields, int* ktau, int* doy0,
                       float* dels) {
  cgio::File f;
  if (cgio::open_read(f, path)) { cgio::close(f); return CABLEGPU_ERR_IO; }
  if (kind) *kind = (int)f.h.kind;
  if (mp) *mp = (long long)f.h.mp;
  if (nrecords) *nrecords = (int)f.h.nrecords;
  if (nfields) *nfields = (int)f.h.nfields;
  if (ktau) *ktau = f.h.ktau;
  if (doy0) *doy0 = f.h.doy0;
  if (dels) *dels = f.h.dels;
  cgio::close(f);
  return CABLEGPU_OK;
}

int cablegpu_run_forcing_file(cablegpu_ctx* c, const char* forcing_path, int record0, int ktau0, int nsteps,
                              const char* output_path) {
  if (!c || !forcing_path || record0 < 0 || ktau0 < 1 || nsteps < 0)
    return fail(c, CABLEGPU_ERR_ARG, "run_forcing_file: bad argument");
  cgio::File in, out;
  if (cgio::open_read(in, forcing_path)) return fail(c, CABLEGPU_ERR_IO, "run_forcing_file: " + in.err);
  struct Closer { cgio::File& a; cgio::File& b; ~Closer() { cgio::close(a); cgio::close(b); } } closer{in, out};
  if (in.h.kind != CABLEGPU_FILE_FORCING || in.h.mp != (uint64_t)c->mp || in.fields.size() != 1 ||
      cgio::find(in, "met") != 0 || in.fields[0].dtype != cgio::kF32 || in.fields[0].width != CG_NFORC ||
      in.fields[0].offset != 0 || !(in.h.dels > 0.f))
    return fail(c, CABLEGPU_ERR_IO, "run_forcing_file: not a forcing file for this context's tiles");
  if ((long long)record0 + nsteps > (long long)in.h.nrecords)
    return fail(c, CABLEGPU_ERR_ARG, "run_forcing_file: the file holds fewer records than asked for");
  if (nsteps == 0) return CABLEGPU_OK;
  const float dels = in.h.dels;
  if (output_path &&
      cgio::create(out, output_path, CABLEGPU_FILE_OUTPUT, (uint64_t)c->mp, {file_entry("out", cgio::kF32, CG_NOUT)},
                   (uint32_t)nsteps, ktau0, in.h.doy0, dels))
    return fail(c, CABLEGPU_ERR_IO, "run_forcing_file: " + out.err);
  constexpr int NB = 3;   // host buffers in flight
  const size_t fbytes = sizeof(float) * CG_NFORC * (size_t)c->mp, obytes = sizeof(float) * CG_NOUT * (size_t)c->mp;
  float* fin[NB] = {};
  float* fout[NB] = {};
  cudaEvent_t ev_in[NB] = {}, ev_out[NB] = {};
  auto release = [&]() {
    for (int b = 0; b < NB; ++b) {
      if (fin[b]) cudaFreeHost(fin[b]);
      if (fout[b]) cudaFreeHost(fout[b]);
      if (ev_in[b]) cudaEventDestroy(ev_in[b]);
      if (ev_out[b]) cudaEventDestroy(ev_out[b]);
    }
  };
  for (int b = 0; b < NB; ++b) {
    if (cudaMallocHost(&fin[b], fbytes) != cudaSuccess || cudaMallocHost(&fout[b], obytes) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_in[b], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_out[b], cudaEventDisableTiming) != cudaSuccess) {
      release();
      return fail(c, CABLEGPU_ERR_CUDA, "run_forcing_file: cannot allocate pinned buffers");
    }
  }
  std::mutex m;
  std::condition_variable cv;
  int filled = 0, submitted = 0, written = 0;
  bool abort = false;
  std::string err;
  auto stop = [&](const std::string& why) {
    std::lock_guard<std::mutex> g(m);
    if (!abort) { abort = true; err = why; }
    cv.notify_all();
  };
  // reader: record n into buffer n % NB once the upload of step n - NB is done
  std::thread reader([&]() {
    cudaSetDevice(c->device);
    for (int n = 0; n < nsteps; ++n) {
      const int b = n % NB;
      if (n >= NB) {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return abort || submitted > n - NB; });
        if (abort) return;
        lk.unlock();
        if (cudaEventSynchronize(ev_in[b]) != cudaSuccess) { stop("run_forcing_file: upload failed"); return; }
      }
      if (cgio::read_record_prefix(in, (uint32_t)(record0 + n), fin[b], fbytes)) {
        stop("run_forcing_file: reading forcing record " + std::to_string(record0 + n) + " failed");
        return;
      }
      std::lock_guard<std::mutex> g(m);
      filled = n + 1;
      cv.notify_all();
    }
  });
  // writer: output of step n once its download is done
  std::thread writer([&]() {
    if (!output_path) return;
    cudaSetDevice(c->device);
    for (int n = 0; n < nsteps; ++n) {
      const int b = n % NB;
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return abort || submitted > n; });
        if (abort && submitted <= n) return;
      }
      if (cudaEventSynchronize(ev_out[b]) != cudaSuccess) { stop("run_forcing_file: download failed"); return; }
      if (cgio::write_block(out, (uint32_t)n, 0, fout[b])) { stop("run_forcing_file: " + out.err); return; }
      std::lock_guard<std::mutex> g(m);
      written = n + 1;
      cv.notify_all();
    }
  });
  int rc = CABLEGPU_OK;
  for (int n = 0; n < nsteps; ++n) {
    const int b = n % NB;
    {
      std::unique_lock<std::mutex> lk(m);
      cv.wait(lk, [&] { return abort || (filled > n && (!output_path || n < NB || written > n - NB)); });
      if (abort) break;
    }
    rc = cablegpu_step_host(c, ktau0 + n, dels, fin[b], fout[b]);
    if (rc == CABLEGPU_OK && (cudaEventRecord(ev_in[b], c->cstream) != cudaSuccess ||
                              cudaEventRecord(ev_out[b], c->dstream) != cudaSuccess))
      rc = fail(c, CABLEGPU_ERR_CUDA, "run_forcing_file: event record failed");
    if (rc) { stop("run_forcing_file: step failed"); break; }
    std::lock_guard<std::mutex> g(m);
    submitted = n + 1;
    cv.notify_all();
  }
  reader.join();
  writer.join();
  const int rs = cablegpu_synchronize(c);
  release();
  if (rc) return rc;
  if (abort) return fail(c, CABLEGPU_ERR_IO, err);
  return rs;
}

int cablegpu_param_table(int table, const char* name, float* out, int n) {
  if (!name || !out) return CABLEGPU_ERR_ARG;
  static CgTables tab;
  static bool built = false;
  if (!built) { cg_build_tables(&tab.pft, &tab.soil); built = true; }
  const float* src = nullptr;
  int len = 0;
  if (table == 0) {
    const CgPftTable& P = tab.pft;
#define CG_T(x) if (!std::strcmp(name, #x)) { src = P.x; len = CG_NPFT; }
    CG_T(canst1) CG_T(dleaf) CG_T(ejmax) CG_T(frac4) CG_T(hc) CG_T(vbeta) CG_T(rp20) CG_T(vegcf) CG_T(extkn)
    CG_T(a1gs) CG_T(d0gs) CG_T(alpha) CG_T(convex) CG_T(cfrd) CG_T(gswmin) CG_T(conkc0) CG_T(conko0) CG_T(ekc)
    CG_T(eko) CG_T(g0) CG_T(g1) CG_T(vcmax) CG_T(xfang) CG_T(shelrb) CG_T(refl1) CG_T(refl2) CG_T(taul1)
    CG_T(taul2) CG_T(rw) CG_T(tfcl) CG_T(tvclst) CG_T(clitt)
#undef CG_T
    if (!std::strcmp(name, "froot")) { src = &P.froot[0][0]; len = CG_MS * CG_NPFT; }
  } else if (table == 1 || table == 2) {
    static CgSoilTable fixed;
    static bool fixed_built = false;
    if (!fixed_built) { fixed = tab.soil; cg_apply_soil_thermal_fix(&fixed); fixed_built = true; }
    const CgSoilTable& S = table == 1 ? tab.soil : fixed;
#define CG_T(x) if (!std::strcmp(name, #x)) { src = S.x; len = CG_NSOIL; }
    CG_T(bch) CG_T(css) CG_T(hyds) CG_T(rhosoil) CG_T(sfc) CG_T(ssat) CG_T(sucs) CG_T(swilt) CG_T(cnsd) CG_T(hsbh)
    CG_T(ibp2) CG_T(i2bp3) CG_T(pwb_min) CG_T(albsoil_vis) CG_T(albsoil_nir) CG_T(sand) CG_T(clay) CG_T(silt)
    CG_T(cnsdv) CG_T(ktmp)
#undef CG_T
  }
  if (!src || n < len) return CABLEGPU_ERR_ARG;
  std::memcpy(out, src, sizeof(float) * len);
  return CABLEGPU_OK;
}

int cablegpu_check_tile_param(cablegpu_ctx* c, const char* name, const float* host) {
  if (!c || !name || !host) return fail(c, CABLEGPU_ERR_ARG, "check_tile_param: null argument");
  float tab[CG_MS * CG_NPFT];
  const int nl = std::strcmp(name, "froot") == 0 ? CG_MS : 1;
  bool per_pft = true;
  if (cablegpu_param_table(0, name, tab, CG_MS * CG_NPFT) != CABLEGPU_OK) {
    per_pft = false;
    // the soil table in effect: with soil_thermal_fix the parameter set-up
    // rewrites css, rhosoil and cnsd (cable_parameters.F90:2165-2227)
    if (cablegpu_param_table(c->thermal_fix ? 2 : 1, name, tab, CG_MS * CG_NPFT) != CABLEGPU_OK)
      return fail(c, CABLEGPU_ERR_ARG, std::string("check_tile_param: ") + name + " is not a table parameter");
  }
  const int ntypes = per_pft ? CG_NPFT : CG_NSOIL;
  const std::vector<int>& type = per_pft ? c->h_iveg : c->h_isoilm;
  for (int k = 0; k < nl; ++k) {
    for (int i = 0; i < c->mp; ++i) {
      const float want = tab[k * ntypes + type[i] - 1];
      const float got = host[(size_t)k * c->mp + i];
      if (!(std::fabs(got - want) <= 1e-6f * std::fabs(want))) {
        char msg[320];
        std::snprintf(msg, sizeof msg,
                      "check_tile_param: %s of tile %d%s is %.9g, the %s type %d table value is %.9g; the kernels "
                      "take this parameter from per-type tables", name, i + 1,
                      nl > 1 ? (", layer " + std::to_string(k + 1)).c_str() : "", (double)got,
                      per_pft ? "plant" : "soil", type[i], (double)want);
        return fail(c, CABLEGPU_ERR_ARG, msg);
      }
    }
  }
  return CABLEGPU_OK;
}

const char* cablegpu_last_error(cablegpu_ctx* c) { return c ? c->err.c_str() : "null context"; }

}  // extern "C"

// ---------------------------------------------------------------- cold start without allocation
// cablegpu_cold_start stages the three initial-state arrays in a buffer it
// cudaMallocs and cudaFrees per call.  Some callers cannot allow that: a host
// model that restarts ensemble members while other streams of the device are
// busy (cudaFree synchronises the whole device), one that runs with a
// reserved memory budget or a pool that owns every free byte, and one that
// re-initialises tiles in a region where allocation calls are forbidden
// (while another thread is capturing a CUDA graph in global mode).
// cablegpu_cold_start_noalloc stages the arrays in a fixed device array
// instead and calls no allocating API (no cudaMalloc/cudaFree, no library
// that allocates).
namespace {

constexpr int kNoAllocMaxTiles = CABLEGPU_NOALLOC_MAX_TILES;
constexpr int kNoAllocMaxDevices = 64;

// 3 x 65536 doubles = 1.5 MiB: snowd0, tgg0, wb0 of up to 65536 tiles.  The
// host-to-device copies overwrite every element the kernel reads before it
// runs, so nothing in it has to start at zero.
static __device__ __align__(256) double g_cold_start_scratch[3 * kNoAllocMaxTiles];

std::mutex g_scratch_mutex;
double* g_scratch_ptr[kNoAllocMaxDevices] = {};

// Address of the scratch array on the current device, resolved once per
// device (the first call may load the module's device code, so it belongs
// before any stream capture).
cudaError_t scratch_for_device(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_cold_start_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" int cablegpu_cold_start_noalloc(cablegpu_ctx* c, const double* snowd0, const double* tgg0,
                                           const double* wb0) {
  if (!c || !snowd0 || !tgg0 || !wb0) return fail(c, CABLEGPU_ERR_ARG, "cold_start_noalloc: null argument");
  if (c->mp > kNoAllocMaxTiles)
    return fail(c, CABLEGPU_ERR_ARG, "cold_start_noalloc: " + std::to_string(c->mp) + " tiles exceed the " +
                                         std::to_string(kNoAllocMaxTiles) +
                                         "-tile limit of its fixed scratch; use cablegpu_cold_start");
  if (c->device < 0 || c->device >= kNoAllocMaxDevices)
    return fail(c, CABLEGPU_ERR_ARG, "cold_start_noalloc: device index out of range");
  int prev = 0;
  CG_CUDA(c, cudaGetDevice(&prev));
  CG_CUDA(c, cudaSetDevice(c->device));
  double* tmp = nullptr;
  cudaError_t e = scratch_for_device(c->device, &tmp);
  int rc = CABLEGPU_OK;
  if (e != cudaSuccess) {
    rc = fail(c, CABLEGPU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  } else {
    const size_t n = (size_t)c->mp;
    e = cudaMemcpyAsync(tmp, snowd0, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + n, tgg0, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(tmp + 2 * n, wb0, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
      bind_device_view(c);
      cold_start_kernel<<<(c->mp + 255) / 256, 256, 0, c->stream>>>(c->dev, c->d_tables, tmp, tmp + n, tmp + 2 * n);
      e = cudaGetLastError();
    }
    // the scratch is shared by every context on the device: it is free again
    // only once the kernel has consumed it
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = fail(c, CABLEGPU_ERR_CUDA, std::string("cold_start_noalloc: ") + cudaGetErrorString(e));
  }
  cudaSetDevice(prev);
  return rc;
}
