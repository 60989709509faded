// tcgen05 GEMM, persistent and warp-specialized: one CTA per SM (at most), each looping over
// 128 x BN output tiles (row tiles beyond *m_dyn are never visited), 384 threads (12 warps).
//   warp 0, lane 0  TMA producer: 128 x 64 A and BN x 64 B tiles (128-byte swizzle) into a
//                   4-stage shared-memory ring that runs across tile boundaries, one mbarrier per
//                   stage ("full"), freed by the MMA issuer ("empty")
//   warp 1, lane 0  MMA issuer: four K = 16 tcgen05.mma per stage into one of two FP32
//                   accumulators in tensor memory (tile i uses accumulator i % 2);
//                   tcgen05.commit frees the stage and, after a tile's last stage, signals the
//                   epilogue ("tmem full")
//   warps 4-11      epilogue: warp w reads accumulator lanes 32 (w % 4) .. + 31 (one output row
//                   per thread) and half (w - 4) / 4 of the columns, 32 at a time (two tcgen05.ld
//                   in flight, one wait), applies bias (staged in shared memory) / activation,
//                   stores each thread's 32 contiguous row elements as 16-byte vectors, and
//                   hands the accumulator back ("tmem empty"), so the next tile's MMAs overlap
//                   this tile's epilogue
// K tails and M/N edges are zero-filled by TMA (out-of-bounds box elements) and masked in the
// epilogue.  All waits are bounded (umma.cuh); a timeout sets err_bit in the error flag word and
// the role leaves its loop (the others then time out in turn).
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "gemm.cuh"
#include "umma.cuh"

namespace souffle {

constexpr int kBM = 128, kBK = 64, kEpiWarps = 8, kThreads = 32 * (4 + kEpiWarps);
constexpr int kStageCols = 32;   // epilogue chunk per warp
constexpr int kMaxBiasN = 512;   // bias staged in shared memory (N <= kMaxBiasN when bias is set)

template <int BN>
struct GemmTile {
  static constexpr int kA = kBM * kBK * 2;  // bytes of one A stage
  static constexpr int kB = BN * kBK * 2;
  static constexpr int kStage = kA + kB;
  // a tile's K = 256 in flight (deeper rings measured no faster)
  static constexpr int kStages = 4;
  // full[s], empty[s], tmem_full[2], tmem_empty[2], and one barrier the MMA issuer drains its own
  // MMAs on when it gives up early
  static constexpr int kBars = 2 * kStages + 5;
  static constexpr int kSmem = 1024 + kStages * kStage + kBars * 8 + 16;
  static constexpr int kTmemCols = 2 * BN;      // two accumulators
  static_assert(kStage % 1024 == 0, "stages stay on 1024-byte boundaries (128-byte swizzle atoms)");
  static_assert(BN % (2 * kStageCols) == 0, "each half of the columns is whole chunks");
  static_assert(kTmemCols == 128 || kTmemCols == 256, "tensor-memory allocations are powers of two");
};

// two floats rounded to BF16 (nearest even), low half = first
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// logistic function with the fast exponential and division (the BF16 outputs carry 8 bits)
__device__ __forceinline__ float sigmoid_fast(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

template <int BN, int ACT>
__global__ void __launch_bounds__(kThreads, 1)
    k_gemm_bf16(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, GemmEpi e) {
  using G = GemmTile<BN>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ float s_bias[kMaxBiasN];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  const uint32_t bars = base + G::kStages * G::kStage;
  const uint32_t full0 = bars, empty0 = bars + 8 * G::kStages;
  const uint32_t tfull0 = bars + 16 * G::kStages, tempty0 = tfull0 + 16, drain = tempty0 + 16;
  const uint32_t tmem_slot = bars + G::kBars * 8;
  volatile uint32_t* tmem_slot_ptr = reinterpret_cast<volatile uint32_t*>(smem_raw + (tmem_slot - raw));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_rows = e.m_dyn ? min(e.M, *e.m_dyn) : e.M;
  const int m_tiles = (m_rows + kBM - 1) / kBM;
  const int n_tiles = (e.N + BN - 1) / BN;
  const int tiles = m_tiles * n_tiles;
  if ((int)blockIdx.x >= tiles) return;  // uniform over the CTA, before any allocation
  const int nk = (e.K + kBK - 1) / kBK;

  if (warp == 0) {
    tmem_alloc(tmem_slot, G::kTmemCols);
    tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < G::kStages; s++) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, kEpiWarps);
    }
    mbar_init(drain, 1);
    mbar_fence_init();
  }
  if (threadIdx.x == 64) {
    tma_prefetch_map(&ta);
    tma_prefetch_map(&tb);
  }
  if (e.bias)
    for (int t = threadIdx.x; t < e.N; t += blockDim.x) s_bias[t] = e.bias[t];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;

  // tile t -> (row tile, column tile), column tiles of one row tile adjacent (A re-read from L2)
  if (warp == 0 && lane == 0) {
    // ---- producer: the stage ring runs on over all of this CTA's tiles (g counts k-steps)
    int g = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
      const int m0 = (t / n_tiles) * kBM, n0 = (t % n_tiles) * BN;
      for (int kt = 0; kt < nk; kt++, g++) {
        const int s = g % G::kStages;
        const uint32_t use = (uint32_t)(g / G::kStages);
        if (use > 0 && !mbar_wait(empty0 + 8 * s, (use - 1) & 1u)) {
          ok = false;
          break;
        }
        const uint32_t a_s = base + s * G::kStage;
        mbar_expect_tx(full0 + 8 * s, G::kStage);
        tma_load_2d(a_s, &ta, kt * kBK, m0, full0 + 8 * s);
        tma_load_2d(a_s + G::kA, &tb, kt * kBK, n0, full0 + 8 * s);
      }
    }
    // every copy started here has landed before the CTA can leave
    for (int q = (g > G::kStages ? g - G::kStages : 0); q < g; q++)
      if (!mbar_wait(full0 + 8 * (q % G::kStages), (uint32_t)(q / G::kStages) & 1u)) ok = false;
    if (!ok) atomicOr(e.err, e.err_bit);
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    constexpr uint32_t idesc = umma_idesc_bf16(kBM, BN);
    int g = 0, it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, it++) {
      const int b = it & 1;
      const uint32_t u = (uint32_t)(it >> 1);
      if (u > 0 && !mbar_wait(tempty0 + 8 * b, (u - 1) & 1u)) {  // the epilogue has drained it
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t acc = tmem + (uint32_t)(b * BN);
      for (int kt = 0; kt < nk; kt++, g++) {
        const int s = g % G::kStages;
        if (!mbar_wait(full0 + 8 * s, (uint32_t)(g / G::kStages) & 1u)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a_s = base + s * G::kStage;
        const uint64_t ad = sw128_kmajor_desc(a_s), bd = sw128_kmajor_desc(a_s + G::kA);
#pragma unroll
        for (int j = 0; j < kBK / 16; j++) umma_bf16(acc, ad + 2 * j, bd + 2 * j, idesc, (kt | j) != 0 ? 1u : 0u);
        umma_commit(empty0 + 8 * s);
      }
      umma_commit(tfull0 + 8 * b);  // after every MMA issued above has completed
    }
    if (!ok) {
      atomicOr(e.err, e.err_bit);
      // MMAs issued before the timeout may still be writing tensor memory: wait (bounded) for
      // them before the CTA releases it
      umma_commit(drain);
      mbar_wait(drain, 0);
    }
  } else if (warp >= 4) {
    // ---- epilogue
    const int quarter = warp & 3, half = (warp - 4) >> 2;
    // 16-byte vector stores/loads need 16-byte aligned rows
    const bool vec_bf16 = e.out_bf16 && (e.ld_bf16 % 8) == 0 && (reinterpret_cast<uintptr_t>(e.out_bf16) & 15) == 0;
    const bool vec_f32 = e.out_f32 && (e.ldo % 4) == 0 && (reinterpret_cast<uintptr_t>(e.out_f32) & 15) == 0;
    const bool vec_z = e.z_out && (e.ldz % 4) == 0 && (reinterpret_cast<uintptr_t>(e.z_out) & 15) == 0;
    const bool vec_zin = e.zin && (e.ldzin % 4) == 0 && (reinterpret_cast<uintptr_t>(e.zin) & 15) == 0;
    int it = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, it++) {
      const int b = it & 1;
      const int m0 = (t / n_tiles) * kBM, n0 = (t % n_tiles) * BN;
      if (!mbar_wait(tfull0 + 8 * b, (uint32_t)(it >> 1) & 1u)) {
        atomicOr(e.err, e.err_bit);
        break;
      }
      tc_fence_after();
      const int row = m0 + quarter * 32 + lane;
      const bool row_ok = row < m_rows;
      const uint32_t t_row = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * BN);
      for (int c = half * (BN / 2); c < (half + 1) * (BN / 2); c += kStageCols) {
        if (n0 + c >= e.N) break;  // uniform over the warp
        const int nv = min(kStageCols, e.N - (n0 + c));  // valid columns in this chunk
        float v[kStageCols];
        tmem_ld32(t_row + (uint32_t)c, v);
        float z[kStageCols];
#pragma unroll
        for (int i = 0; i < kStageCols; i++) z[i] = 0.f;
        if (ACT == kActSiluGrad && row_ok) {
          const float* zr = e.zin + (size_t)row * e.ldzin + n0 + c;
          if (nv == kStageCols && vec_zin) {
#pragma unroll
            for (int q = 0; q < kStageCols / 4; q++) {
              const float4 w4 = *reinterpret_cast<const float4*>(zr + 4 * q);
              z[4 * q] = w4.x; z[4 * q + 1] = w4.y; z[4 * q + 2] = w4.z; z[4 * q + 3] = w4.w;
            }
          } else {
#pragma unroll
            for (int i = 0; i < kStageCols; i++) z[i] = i < nv ? zr[i] : 0.f;
          }
        }
#pragma unroll
        for (int i = 0; i < kStageCols; i++) {
          float x = v[i] + (e.bias && i < nv ? s_bias[n0 + c + i] : 0.f);
          if (ACT == kActSilu) {
            z[i] = x;
            x = x * sigmoid_fast(x);
          } else if (ACT == kActSiluGrad) {
            const float sg = sigmoid_fast(z[i]);
            x *= sg * (1.0f + z[i] * (1.0f - sg));
          } else {
            z[i] = x;
          }
          v[i] = x;
        }
        if (row_ok) {
        if (e.out_bf16_t) {
#pragma unroll
          for (int i = 0; i < kStageCols; i++)
            if (i < nv) e.out_bf16_t[(size_t)(n0 + c + i) * e.ldt + row] = __float2bfloat16_rn(v[i]);
        }
        const bool fullc = nv == kStageCols;
        if (e.out_bf16) {
          __nv_bfloat16* o = e.out_bf16 + (size_t)row * e.ld_bf16 + n0 + c;
          if (fullc && vec_bf16) {
#pragma unroll
            for (int q = 0; q < kStageCols / 8; q++) {
              uint4 u4;
              u4.x = pack_bf16x2(v[8 * q], v[8 * q + 1]);
              u4.y = pack_bf16x2(v[8 * q + 2], v[8 * q + 3]);
              u4.z = pack_bf16x2(v[8 * q + 4], v[8 * q + 5]);
              u4.w = pack_bf16x2(v[8 * q + 6], v[8 * q + 7]);
              *reinterpret_cast<uint4*>(o + 8 * q) = u4;
            }
          } else {
#pragma unroll
            for (int i = 0; i < kStageCols; i++)
              if (i < nv) o[i] = __float2bfloat16_rn(v[i]);
          }
        }
        if (e.out_f32) {
          float* o = e.out_f32 + (size_t)row * e.ldo + n0 + c;
          if (fullc && vec_f32) {
#pragma unroll
            for (int q = 0; q < kStageCols / 4; q++)
              *reinterpret_cast<float4*>(o + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          } else {
#pragma unroll
            for (int i = 0; i < kStageCols; i++)
              if (i < nv) o[i] = v[i];
          }
        }
        if (ACT != kActSiluGrad && e.z_out) {
          float* o = e.z_out + (size_t)row * e.ldz + n0 + c;
          if (fullc && vec_z) {
#pragma unroll
            for (int q = 0; q < kStageCols / 4; q++)
              *reinterpret_cast<float4*>(o + 4 * q) = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
          } else {
#pragma unroll
            for (int i = 0; i < kStageCols; i++)
              if (i < nv) o[i] = z[i];
          }
        }
        }
        __syncwarp();
      }
      // this warp has read its part of the accumulator (tcgen05.ld waited above)
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty0 + 8 * b);
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, G::kTmemCols);
  }
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// [rows][cols] BF16 matrix with row stride ld elements; box = 64 columns x box_rows rows
bool make_map(CUtensorMap* m, const void* p, int rows, int cols, int ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(p), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int ACT>
cudaError_t launch(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, const GemmEpi& e, cudaStream_t st) {
  using G = GemmTile<BN>;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_gemm_bf16<BN, ACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::kSmem);
  });
  if (attr != cudaSuccess) return attr;
  CUtensorMap ta, tb;
  if (!make_map(&ta, A, e.M, e.K, lda, kBM) || !make_map(&tb, B, e.N, e.K, ldb, BN)) return cudaErrorInvalidValue;
  // persistent: at most one CTA per SM, each looping over tiles
  static int sms = 0;
  static std::once_flag once_sm;
  std::call_once(once_sm, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 0;
  });
  const long long tiles = (long long)((e.M + kBM - 1) / kBM) * ((e.N + BN - 1) / BN);
  const int gx = (int)std::min<long long>(tiles, sms > 0 ? sms : 148);
  dim3 grid(gx);
  k_gemm_bf16<BN, ACT><<<grid, kThreads, G::kSmem, st>>>(ta, tb, e);
  return cudaGetLastError();
}

template <int BN>
cudaError_t launch_act(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, const GemmEpi& e,
                       cudaStream_t st) {
  switch (e.act) {
    case kActSilu: return launch<BN, kActSilu>(A, lda, B, ldb, e, st);
    case kActSiluGrad: return launch<BN, kActSiluGrad>(A, lda, B, ldb, e, st);
    default: return launch<BN, kActNone>(A, lda, B, ldb, e, st);
  }
}

}  // namespace

cudaError_t gemm_bf16(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, const GemmEpi& e,
                      cudaStream_t stream) {
  if (e.M < 1 || e.N < 1 || e.K < 1 || !e.err || lda < e.K || ldb < e.K || lda % 8 || ldb % 8 ||
      (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15))
    return cudaErrorInvalidValue;
  if ((e.out_f32 && e.ldo < e.N) || (e.out_bf16 && e.ld_bf16 < e.N) || (e.out_bf16_t && e.ldt < e.M) ||
      (e.z_out && e.ldz < e.N) || (e.act == kActSiluGrad && (!e.zin || e.ldzin < e.N)) ||
      e.act < kActNone || e.act > kActSiluGrad)
    return cudaErrorInvalidValue;
  if (e.bias && e.N > kMaxBiasN) return cudaErrorInvalidValue;
  // 64-column tiles when 128-column tiles would leave SMs idle or pad more columns (the output
  // layer's 144 columns: 192 against 256); 128-column tiles otherwise (fewer re-reads of A)
  const long long mt = (e.M + kBM - 1) / kBM;
  const int n128 = (e.N + 127) / 128 * 128, n64 = (e.N + 63) / 64 * 64;
  const bool narrow = mt * (n128 / 128) < 152 || n64 < n128;
  return narrow ? launch_act<64>(A, lda, B, ldb, e, stream) : launch_act<128>(A, lda, B, ldb, e, stream);
}

}  // namespace souffle
