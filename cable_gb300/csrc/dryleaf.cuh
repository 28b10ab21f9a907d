// The dryLeaf iteration of define_canopy (cbl_dryLeaf.F90:10-666) as a pass
// function and its two schedules on the GPU.
//
// A vegetated tile's dryLeaf call repeats one pass of the coupled leaf energy
// balance / photosynthesis / stomatal conductance fixed point until the leaf
// temperature moves by at most 0.1 K (at most MAXITER = 20 passes).  Tiles
// converge after different numbers of passes, and a converged tile is an
// exact no-op in the reference's later passes (the best-iterate store needs a
// strict improvement, damping and the body need |dT| > 0.1 K), so where a
// tile's passes run does not change its result.
//
//   lanes: each thread runs its own tile's passes; a warp issues while any of
//          its 32 tiles iterates, so the converged lanes idle.
//   pool:  the block's tiles park their pass inputs and state in shared-memory
//          slots; the block then runs rounds of single passes over a list of
//          the tiles still iterating, one tile per thread, so a thread whose
//          own tile converged runs another tile's pass.  After each round a
//          warp vote (__ballot_sync) marks the tiles that go on and one atomic
//          per warp appends them to the next round's list; one block barrier
//          per round.  A round costs a warp per 32 iterating tiles, instead
//          of a warp per 32 tiles for the slowest tile's passes.
#pragma once
#include "cbm_physics.cuh"

namespace cg {

// Inputs of one tile's dryLeaf call, fixed over its passes.
struct DlCtx {
  int v;                     // plant type - 1
  float tk, ca, cmolar, psyc, dsatdk, fwet, fwsoil;
  float scalex[2], fvlai[2], gradis[2], rniso[2], qcan_par[2];
  float dk_avail[CG_MS];     // water each layer can give to transpiration (mm)
  float tvair, dva, gbhu[2]; // this Monin-Obukhov iteration's canopy air and leaf boundary layer
  float conv;                // convergence test of the leaf temperature (K)
};
// State of one tile's dryLeaf call, updated by each pass.
struct DlState {
  float tlfx, dsx, csx[2], gswx[2], gbhf[2], psycst[2];
  float abs_deltlf, deltlfy, ecx;
  // best iterate (cbl_dryLeaf.F90:565-582): net radiation, sensible and
  // latent heat, leaf temperature, respiration and net assimilation of both
  // leaves, transpiration (mm) of its pass; transpiration of the latest pass
  float rny, hcy, ecy, tlfy, rdy_sum, an_y_sum, fe_mm_best, fe_mm_last;
  int k;                     // passes run in this call
};

// One pass of the dryLeaf iteration (cbl_dryLeaf.F90:239-590) for one
// vegetated tile: leaf boundary-layer conductance under free convection
// (:252-262), temperature responses of vcmax, jmax and the Michaelis-Menten
// constants (:265-301), electron transport and leaf respiration (:302-330),
// the stomatal coefficient (leuning or medlyn, :376-435), photosynthesis
// (:438-446), leaf-surface CO2, stomatal and total conductances
// (:449-470), canopy latent heat with the root-weighted transpiration
// extraction (:472-531), sensible heat, leaf temperature and leaf-surface
// VPD (:533-560), the best iterate (:565-582) and damping (:584-590).
// Returns whether the tile iterates again: its leaf temperature moved by
// more than c.conv and fewer than MAXITER passes have run.
__device__ __forceinline__ bool dl_pass(const DlCtx& c, DlState& s, const float (&froot)[CG_MS], int medlyn,
                                        float dels) {
  const int v = c.v;
  const int k = ++s.k;
  const float dleaf = ldk(c_pft.dleaf[v]);
  float gras = fmaxf(1.0e-6f, 1.595E8f * fabsf(s.tlfx - c.tvair) * (dleaf * dleaf * dleaf));
  float gr4 = sqrtf(sqrtf(gras));
  float gh[2], ghr[2];
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    s.gbhf[l] = fmaxf(1.e-6f, c.fvlai[l] * c.cmolar * 0.5f * DHEAT * gr4 / dleaf);
    gh[l] = 2.0f * (c.gbhu[l] + s.gbhf[l]);
    ghr[l] = c.gradis[l] + gh[l];
  }
  float vcmxt3[2], vcmxt4[2], vx3[2], vx4[2], gs_coeff[2], rdx[2];
  const float vcmax = ldk(c_pft.vcmax[v]), frac4 = ldk(c_pft.frac4[v]);
  const float tlfx = s.tlfx;
  float temp = xvcmxt3(tlfx) * vcmax * (1.0f - frac4);
  vcmxt3[0] = c.scalex[0] * temp; vcmxt3[1] = c.scalex[1] * temp;
  temp = xvcmxt4(tlfx - TFRZ) * vcmax * frac4;
  vcmxt4[0] = c.scalex[0] * temp; vcmxt4[1] = c.scalex[1] * temp;
  temp = xejmxt3(tlfx) * ldk(c_pft.ejmax[v]) * (1.0f - frac4);
  float ejmxt3[2] = {c.scalex[0] * temp, c.scalex[1] * temp};
  float tdiff = tlfx - TREFK;
  float arr = (1.0f - TREFK / tlfx) / (RGAS * TREFK);
  float conkct = ldk(c_pft.conkc0[v]) * expf(ldk(c_pft.ekc[v]) * arr);
  float conkot = ldk(c_pft.conko0[v]) * expf(ldk(c_pft.eko[v]) * arr);
  const float tlfxx = tlfx;
  float cx1 = conkct * (1.0f + 0.21f / conkot);
  float cx2 = 2.0f * GAM0 * __fmaf_rn(__fmaf_rn(GAM2, tdiff, GAM1), tdiff, 1.0f);
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    float par = c.qcan_par[l] * 4.6e-6f;
    const float alpha = ldk(c_pft.alpha[v]), convex = ldk(c_pft.convex[v]), cfrd = ldk(c_pft.cfrd[v]);
    vx3[l] = ej3x(par * (1.0f - frac4), alpha, convex, ejmxt3[l]);
    vx4[l] = ej4x(par * frac4, alpha, convex, vcmxt4[l]);
    rdx[l] = __fmaf_rn(cfrd, vcmxt3[l], cfrd * vcmxt4[l]);
  }
  const float gswmin_p = ldk(c_pft.gswmin[v]);
  float gswmin[2] = {fmaxf(1.e-6f, c.scalex[0] * gswmin_p), fmaxf(1.e-6f, c.scalex[1] * gswmin_p)};
  if (!medlyn) {
    float f = ldk(c_pft.a1gs[v]) / (1.0f + s.dsx / ldk(c_pft.d0gs[v]));
    gs_coeff[0] = (c.fwsoil / s.csx[0]) * f;
    gs_coeff[1] = (c.fwsoil / s.csx[1]) * f;
  } else {
    gswmin[0] = gswmin[1] = ldk(c_pft.g0[v]);
    float vpd = (s.dsx < 50.0f) ? 0.05f : s.dsx * 1e-3f;
    float num = (c.fwsoil <= 0.05f) ? c.fwsoil / 0.05f : 1.0f;
    float t2 = (ldk(c_pft.g1[v]) * c.fwsoil) * rsqrtf(vpd);
    gs_coeff[0] = (num + t2) / s.csx[0];
    gs_coeff[1] = (num + t2) / s.csx[1];
  }
  // photosynthesis: anx is zeroed and recomputed under the masks
  float anx[2] = {0.f, 0.f};
  if (c.fvlai[0] + c.fvlai[1] > LAI_THRESH) {
#pragma unroll
    for (int l = 0; l < 2; ++l)
      if (c.fvlai[l] > LAI_THRESH)
        anx[l] = photosynthesis_leaf(s.csx[l], cx1, cx2, gswmin[l], rdx[l], vcmxt3[l], vcmxt4[l], vx3[l], vx4[l],
                                     gs_coeff[l], c.fwsoil);
  }
#pragma unroll
  for (int l = 0; l < 2; ++l) {
    if (c.fvlai[l] > LAI_THRESH) {
      s.csx[l] = fmaxf(1.0e-4f, c.ca - RGBWC * anx[l] / (c.gbhu[l] + s.gbhf[l]));
      s.gswx[l] = fmaxf(1.e-3f, __fmaf_rn(gswmin[l], c.fwsoil, fmaxf(0.0f, RGSWC * gs_coeff[l] * anx[l])));
      float gw = 1.0f / (1.0f / s.gswx[l] + 1.0f / (1.075f * (c.gbhu[l] + s.gbhf[l])));
      gw = fmaxf(gw, 0.00001f);
      s.psycst[l] = c.psyc * (ghr[l] / gw);
    }
  }
  // Terms that combine a product of the call's fixed inputs with a
  // per-pass value are written with explicitly rounded operations: where a
  // pass runs (a per-lane loop, where the compiler hoists the fixed product,
  // or the pool, where it does not) must not change which products are
  // fused into multiply-adds, so both schedules compute identical results.
  const float cpr = CAPP * RMAIR;
  const float pc = __fmul_rn(cpr, __fsub_rn(c.tvair, c.tk)), pd = __fmul_rn(cpr, c.dva);
  float ecx = __fmaf_rn(c.dsatdk, __fmaf_rn(-pc, c.gradis[0], c.rniso[0]), __fmul_rn(pd, ghr[0])) /
                  (c.dsatdk + s.psycst[0]) +
              __fmaf_rn(c.dsatdk, __fmaf_rn(-pc, c.gradis[1], c.rniso[1]), __fmul_rn(pd, ghr[1])) /
                  (c.dsatdk + s.psycst[1]);
  float local_fevc = (1.0f - c.fwet) * ecx;
  if (local_fevc > 0.0f) {
    const float fe_mm = local_fevc * dels / HL;
    float ev[CG_MS];
    const float se = transp_extract(fe_mm, froot, c.dk_avail, ev);
    const float fevc = se * HL / dels;
    ecx = fevc / (1.0f - c.fwet);
    s.fe_mm_last = fe_mm;
  }
  const float sum_rad_rniso = c.rniso[0] + c.rniso[1];
  const float sum_rad_gradis = c.gradis[0] + c.gradis[1];
  float sgh = gh[0] + gh[1];
  const float hcx = __fmaf_rn(-pc, sum_rad_gradis, __fsub_rn(sum_rad_rniso, ecx)) * sgh / (ghr[0] + ghr[1]);
  s.tlfx = c.tvair + hcx / (cpr * sgh);
  const float rnx = __fmaf_rn(-(cpr * (s.tlfx - c.tk)), sum_rad_gradis, sum_rad_rniso);
  s.dsx = fmaxf(__fmaf_rn(c.dsatdk, s.tlfx - c.tvair, c.dva), 0.0f);
  const float deltlf = tlfxx - s.tlfx;
  s.abs_deltlf = fabsf(deltlf);
  s.ecx = ecx;
  // keep the best iterate (:565-582)
  if (s.abs_deltlf < fabsf(s.deltlfy) || k == 1) {
    if (s.abs_deltlf < fabsf(s.deltlfy)) s.deltlfy = deltlf;
    s.rny = rnx; s.hcy = hcx; s.ecy = ecx;
    s.rdy_sum = rdx[0] + rdx[1]; s.an_y_sum = anx[0] + anx[1];
    s.fe_mm_best = s.fe_mm_last;
    s.tlfy = s.tlfx;   // damping below is a no-op for k == 1
  }
  // damping once k > 5 (:584-590).  Written with explicitly rounded
  // operations: a*b + c*d leaves the compiler a choice of which product to
  // fuse, and that choice may differ between instantiations of the kernel,
  // which must give identical results.
  if (s.abs_deltlf > c.conv) {
    float fac = 0.5f * ((float)max(0, k - 5) / ((float)k - 4.9999f));
    s.tlfx = __fmaf_rn(fac, tlfxx, __fmul_rn(1.0f - fac, s.tlfx));
  }
  return s.abs_deltlf > c.conv && k < MAXITER;
}

// ---------------------------------------------------------------- the pool
// Shared-memory slot of one tile, [field][blockDim.x] floats (one bank per
// slot for consecutive slots), then two lists of blockDim.x uint16 slot
// indices and three round counters.
namespace dlp {
enum : int {
  TK, CA, CMOLAR, PSYC, DSATDK, FWET, FWSOIL, SCALEX, FVLAI = SCALEX + 2, GRADIS = FVLAI + 2, RNISO = GRADIS + 2,
  QCAN = RNISO + 2, DKAV = QCAN + 2,                        // fixed over the step
  TVAIR = DKAV + CG_MS, DVA, GBHU, CONV = GBHU + 2,       // fixed over one call
  TLFX, DSX, CSX, GSWX = CSX + 2, GBHF = GSWX + 2, PSYCST = GBHF + 2, ADL = PSYCST + 2, DLY, ECX, RNY, HCY, ECY,
  TLFY, RDY, ANY, FEB, FEL,                               // pass state
  KV,        // int bits: passes (0-7), plant type - 1 (8-15), surrogate flags (16-18)
  NF,        // fields of the plain and harvesting kernels
  // the surrogate kernel's entry state, for the strict mode's restart
  E_TLF = NF, E_DSX, E_CSX, E_GSWX = E_CSX + 2, E_GBHF = E_GSWX + 2, NF_SUR = E_GBHF + 2
};
constexpr int SUR_TRY = 1 << 16, SUR_ACC = 1 << 17, SUR_RESTART = 1 << 18;
__host__ __device__ constexpr int smem_bytes(int block, bool sur) {
  return (sur ? NF_SUR : NF) * 4 * block + 2 * 2 * block + 16;
}
}  // namespace dlp

template <bool kSur>
struct DlPool {
  float* sm;
  int B;
  __device__ float& f(int field, int slot) const { return sm[field * B + slot]; }
  __device__ int& kv(int slot) const { return reinterpret_cast<int*>(sm)[dlp::KV * B + slot]; }
  __device__ uint16_t* list(int which) const {
    return reinterpret_cast<uint16_t*>(sm + (kSur ? dlp::NF_SUR : dlp::NF) * B) + which * B;
  }
  __device__ int* cnt() const { return reinterpret_cast<int*>(list(2)); }

  __device__ void put_step(int slot, const DlCtx& c) const {
    using namespace dlp;
    f(TK, slot) = c.tk; f(CA, slot) = c.ca; f(CMOLAR, slot) = c.cmolar; f(PSYC, slot) = c.psyc;
    f(DSATDK, slot) = c.dsatdk; f(FWET, slot) = c.fwet; f(FWSOIL, slot) = c.fwsoil;
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      f(SCALEX + l, slot) = c.scalex[l]; f(FVLAI + l, slot) = c.fvlai[l]; f(GRADIS + l, slot) = c.gradis[l];
      f(RNISO + l, slot) = c.rniso[l]; f(QCAN + l, slot) = c.qcan_par[l];
    }
#pragma unroll
    for (int q = 0; q < CG_MS; ++q) f(DKAV + q, slot) = c.dk_avail[q];
  }
  __device__ void put_call(int slot, const DlCtx& c, const DlState& s, int flags) const {
    using namespace dlp;
    f(TVAIR, slot) = c.tvair; f(DVA, slot) = c.dva; f(GBHU, slot) = c.gbhu[0]; f(GBHU + 1, slot) = c.gbhu[1];
    f(CONV, slot) = c.conv;
    put_state(slot, s);
    kv(slot) = s.k | (c.v << 8) | flags;
  }
  __device__ void put_state(int slot, const DlState& s) const {
    using namespace dlp;
    f(TLFX, slot) = s.tlfx; f(DSX, slot) = s.dsx;
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      f(CSX + l, slot) = s.csx[l]; f(GSWX + l, slot) = s.gswx[l]; f(GBHF + l, slot) = s.gbhf[l];
      f(PSYCST + l, slot) = s.psycst[l];
    }
    f(ADL, slot) = s.abs_deltlf; f(DLY, slot) = s.deltlfy; f(ECX, slot) = s.ecx; f(RNY, slot) = s.rny;
    f(HCY, slot) = s.hcy; f(ECY, slot) = s.ecy; f(TLFY, slot) = s.tlfy; f(RDY, slot) = s.rdy_sum;
    f(ANY, slot) = s.an_y_sum; f(FEB, slot) = s.fe_mm_best; f(FEL, slot) = s.fe_mm_last;
  }
  __device__ void get_state(int slot, DlState& s) const {
    using namespace dlp;
    s.tlfx = f(TLFX, slot); s.dsx = f(DSX, slot);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      s.csx[l] = f(CSX + l, slot); s.gswx[l] = f(GSWX + l, slot); s.gbhf[l] = f(GBHF + l, slot);
      s.psycst[l] = f(PSYCST + l, slot);
    }
    s.abs_deltlf = f(ADL, slot); s.deltlfy = f(DLY, slot); s.ecx = f(ECX, slot); s.rny = f(RNY, slot);
    s.hcy = f(HCY, slot); s.ecy = f(ECY, slot); s.tlfy = f(TLFY, slot); s.rdy_sum = f(RDY, slot);
    s.an_y_sum = f(ANY, slot); s.fe_mm_best = f(FEB, slot); s.fe_mm_last = f(FEL, slot);
    s.k = kv(slot) & 0xff;
  }
  __device__ void get_ctx(int slot, DlCtx& c) const {
    using namespace dlp;
    c.v = (kv(slot) >> 8) & 0xff;
    c.tk = f(TK, slot); c.ca = f(CA, slot); c.cmolar = f(CMOLAR, slot); c.psyc = f(PSYC, slot);
    c.dsatdk = f(DSATDK, slot); c.fwet = f(FWET, slot); c.fwsoil = f(FWSOIL, slot);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      c.scalex[l] = f(SCALEX + l, slot); c.fvlai[l] = f(FVLAI + l, slot); c.gradis[l] = f(GRADIS + l, slot);
      c.rniso[l] = f(RNISO + l, slot); c.qcan_par[l] = f(QCAN + l, slot);
    }
#pragma unroll
    for (int q = 0; q < CG_MS; ++q) c.dk_avail[q] = f(DKAV + q, slot);
    c.tvair = f(TVAIR, slot); c.dva = f(DVA, slot); c.gbhu[0] = f(GBHU, slot); c.gbhu[1] = f(GBHU + 1, slot);
    c.conv = f(CONV, slot);
  }
  // the surrogate kernel: the state the plain iteration starts from
  __device__ void put_entry(int slot, const DlState& s) const {
    using namespace dlp;
    f(E_TLF, slot) = s.tlfx; f(E_DSX, slot) = s.dsx;
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      f(E_CSX + l, slot) = s.csx[l]; f(E_GSWX + l, slot) = s.gswx[l]; f(E_GBHF + l, slot) = s.gbhf[l];
    }
  }

  // One pass of the tile in `slot`; returns whether it iterates again.
  __device__ bool pass(int slot, int medlyn, float dels, int sur_strict) const {
    DlCtx c;
    DlState s;
    get_ctx(slot, c);
    get_state(slot, s);
    float fr[CG_MS];
#pragma unroll
    for (int q = 0; q < CG_MS; ++q) fr[q] = ldk(c_pft.froot[q][c.v]);
    bool more = dl_pass(c, s, fr, medlyn, dels);
    int bits = kv(slot) & ~0xff;
    if (kSur && (bits & dlp::SUR_TRY) && s.k == 1) {
      // the first pass started from the network's leaf temperature: it is
      // accepted when it moved the leaf temperature by at most the gate;
      // otherwise strict mode restarts the plain iteration from its usual
      // start (the surrogate kernel's per-lane schedule does the same)
      bits &= ~dlp::SUR_TRY;
      if (s.abs_deltlf <= c.conv) {
        bits |= dlp::SUR_ACC;
      } else if (sur_strict) {
        using namespace dlp;
        const float sum_rad_rniso = c.rniso[0] + c.rniso[1];
        s.tlfx = f(E_TLF, slot); s.dsx = f(E_DSX, slot);
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          s.csx[l] = f(E_CSX + l, slot); s.gswx[l] = f(E_GSWX + l, slot); s.gbhf[l] = f(E_GBHF + l, slot);
        }
        s.ecx = sum_rad_rniso; s.abs_deltlf = 999.0f; s.deltlfy = s.abs_deltlf;
        s.hcy = 0.f; s.fe_mm_last = 0.f; s.fe_mm_best = 0.f; s.rdy_sum = 0.f; s.an_y_sum = 0.f;
        s.k = 0;
        f(CONV, slot) = 0.1f;
        bits |= dlp::SUR_RESTART;
        more = true;
      }
    }
    put_state(slot, s);
    kv(slot) = s.k | bits;
    return more;
  }

  // One dryLeaf call of the whole block: every thread of the block calls it
  // (own = whether this thread's tile takes part, its pass inputs and state
  // already in slot threadIdx.x).  Before the call the caller has passed a
  // barrier after the previous call, written its slot, cleared the three
  // round counters (thread 0) and passed a second barrier.
  __device__ void run(bool own, int medlyn, float dels, int sur_strict) const {
    const int tid = threadIdx.x, lane = tid & 31;
    int* const C = cnt();
    // the initial list: this block's iterating tiles
    {
      const unsigned m = __ballot_sync(0xffffffffu, own);
      if (m) {
        int base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(&C[0], __popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        if (own) list(0)[base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)tid;
      }
    }
    __syncthreads();
    // round r: the list in buffer r & 1 with counter C[r % 3]; the tiles
    // that go on are appended to buffer (r + 1) & 1, counter C[(r + 1) % 3];
    // C[(r + 2) % 3], last read in round r - 1, is cleared for round r + 1
    for (int r = 0;; ++r) {
      const int n = C[r % 3];
      if (n == 0) break;
      bool keep = false;
      int slot = 0;
      if (tid < n) {
        slot = list(r & 1)[tid];
        keep = pass(slot, medlyn, dels, sur_strict);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (m) {
        int base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(&C[(r + 1) % 3], __popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        if (keep) list((r + 1) & 1)[base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)slot;
      }
      if (tid == 0) C[(r + 2) % 3] = 0;
      __syncthreads();
    }
  }
};

}  // namespace cg
