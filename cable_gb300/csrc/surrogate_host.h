// Host-side interface of the surrogate network's trainer (surrogate.cu),
// used by the context runtime (cablegpu.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

// Device workspace of one network: parameters, Adam moments, normalisation,
// packed BF16 operand image and the per-CTA partial-gradient buffer.
struct SurNet {
  float* params = nullptr;    // cg::sur::NPARAM
  float* m = nullptr;
  float* v = nullptr;
  float* norm = nullptr;      // cg::sur::NNORM
  uint8_t* packed = nullptr;  // cg::sur::PK_BYTES
  float* part = nullptr;      // [nblk][NPARAM]
  float* loss_part = nullptr;
  float* grad = nullptr;      // NPARAM
  unsigned int* err = nullptr;
  int nblk = 0;
  int adam_t = 0;
};

int sur_alloc(SurNet& n, std::string& err);
void sur_free(SurNet& n);
int sur_pack(SurNet& n, cudaStream_t st, std::string& err);
// Predicted first-iteration leaf-temperature change dt [mp] of every tile,
// its inputs formed from the radiation kernel's hand-off record work_a
// ([CG_NA][ld]) and the tile tables (stream-ordered, one kernel launch).
namespace cg { struct CgTables; }
int sur_infer(const SurNet& n, const float* work_a, const uint8_t* iveg, const uint8_t* isoilm,
              const cg::CgTables* tables, int medlyn, int mp, int ld, float* dt, unsigned int* status,
              cudaStream_t st, std::string& err);
// Trains on rows [0, ntrain) of d_rows, validating on [ntrain, ntrain+nval);
// losses: [epochs][2] (train, validation mean squared normalised error).
int sur_fit(SurNet& n, const float* d_rows, long long ntrain, long long nval, int epochs, int batch, float lr,
            unsigned long long seed, bool init, float* losses, cudaStream_t st, std::string& err);
