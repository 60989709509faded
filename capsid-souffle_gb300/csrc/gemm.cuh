// BF16 tensor-core GEMM for the surrogate network: C = A B^T with A [M][K] and B [N][K] both
// row-major BF16 (K contiguous, "K-major"), FP32 accumulation in tensor memory, and a fused
// epilogue (bias, SiLU or the SiLU derivative, FP32 / BF16 / transposed BF16 stores).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace souffle {

enum GemmAct : int { kActNone = 0, kActSilu = 1, kActSiluGrad = 2 };

struct GemmEpi {
  int M = 0, N = 0, K = 0;        // C is M x N, the contraction has length K
  const int* m_dyn = nullptr;     // optional device count: rows >= *m_dyn are skipped
  const float* bias = nullptr;    // [N], added first
  int act = kActNone;             // SiLU: z -> z sigma(z); SiluGrad: x -> x * SiLU'(zin)
  const float* zin = nullptr;     // SiluGrad: pre-activation [M][ldzin]
  int ldzin = 0;
  float* z_out = nullptr;         // Silu: pre-activation store [M][ldz]
  int ldz = 0;
  float* out_f32 = nullptr;       // [M][ldo]
  int ldo = 0;
  __nv_bfloat16* out_bf16 = nullptr;    // [M][ld_bf16]
  int ld_bf16 = 0;
  __nv_bfloat16* out_bf16_t = nullptr;  // transposed [N][ldt]
  int ldt = 0;
  unsigned int* err = nullptr;    // device flag word
  unsigned int err_bit = 1u;      // set in *err when a bounded wait ran out
};

// Device pointers to a network's normalisation of its training data (held by the network, so a
// trained network brings it to every handle it is attached to); *has is set once trained.
struct MlpNorm {
  float *x_mean, *x_istd, *t_mean, *t_std, *t_istd;
  bool* has;
};

// Launches on the stream; A/B base addresses 16-byte aligned, lda/ldb multiples of 8 elements.
cudaError_t gemm_bf16(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, const GemmEpi& e,
                      cudaStream_t stream);

}  // namespace souffle
