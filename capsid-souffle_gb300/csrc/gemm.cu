// tcgen05 GEMM: 128 x BN output tiles, 256 threads (8 warps) per CTA; at most one wave of CTAs,
// each looping over row tiles, so a large row capacity with few live rows (*m_dyn) costs little.
//   warp 0, lane 0  TMA producer: 128 x 64 A and BN x 64 B tiles (128-byte swizzle) into a
//                   4-stage shared-memory ring, one mbarrier per stage ("full")
//   warp 1, lane 0  MMA issuer: four K = 16 tcgen05.mma per stage into an FP32 accumulator in
//                   tensor memory; tcgen05.commit frees the stage ("empty") and, after the last
//                   stage, signals the epilogue ("accum")
//   warps 0-7       epilogue: warp w reads accumulator lanes 32 (w % 4) .. + 31 (one output row
//                   per thread) and half (w / 4) of the columns, 32 at a time (two tcgen05.ld in
//                   flight, one wait), applies bias / activation, and stores through shared
//                   memory so that global stores run along the rows
// The epilogue is the long part of a small GEMM (it is latency-bound per thread), so it gets all
// eight warps, the activation is a template parameter, and BN = 64 by default spreads a small M
// over more SMs.  K tails and M/N edges are zero-filled by TMA (out-of-bounds box elements) and
// masked in the epilogue.  All waits are bounded (umma.cuh); a timeout sets err_bit in the error
// flag word.
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "gemm.cuh"
#include "umma.cuh"

namespace souffle {

constexpr int kBM = 128, kBK = 64, kStages = 4, kThreads = 256;
constexpr int kStageCols = 32;                  // epilogue chunk per warp
constexpr int kStagePitch = kStageCols + 1;     // conflict-free rows and columns

template <int BN>
struct GemmTile {
  static constexpr int kA = kBM * kBK * 2;  // bytes of one A stage
  static constexpr int kB = BN * kBK * 2;
  static constexpr int kStage = kA + kB;
  static constexpr int kBars = 2 * kStages + 1;
  static constexpr int kSmem = 1024 + kStages * kStage + kBars * 8 + 16;
  static constexpr int kTmemCols = BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
  static constexpr int kEpiBytes = (kThreads / 32) * 2 * 32 * kStagePitch * 4;
  static_assert(kStage % 1024 == 0, "stages stay on 1024-byte boundaries (128-byte swizzle atoms)");
  static_assert(kEpiBytes <= kStages * kStage, "epilogue staging fits in the freed stages");
  static_assert(BN % (2 * kStageCols) == 0, "each half of the columns is whole chunks");
};

// logistic function with the fast exponential and division (the BF16 outputs carry 8 bits)
__device__ __forceinline__ float sigmoid_fast(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

template <int BN, int ACT>
__global__ void __launch_bounds__(kThreads, BN <= 64 ? 2 : 1)
    k_gemm_bf16(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, GemmEpi e) {
  using G = GemmTile<BN>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  const uint32_t bars = base + kStages * G::kStage;  // full[s], empty[s], accum
  const uint32_t tmem_slot = bars + G::kBars * 8;
  volatile uint32_t* tmem_slot_ptr = reinterpret_cast<volatile uint32_t*>(smem_raw + (tmem_slot - raw));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_rows = e.m_dyn ? min(e.M, *e.m_dyn) : e.M;
  const int m_tiles = (m_rows + kBM - 1) / kBM;
  const int n0 = blockIdx.y * BN;
  if ((int)blockIdx.x >= m_tiles) return;  // uniform over the CTA, before any allocation
  const int nk = (e.K + kBK - 1) / kBK;
  const uint32_t full0 = bars, empty0 = bars + 8 * kStages, accum = bars + 16 * kStages;
  __shared__ int s_fail;

  if (warp == 0) {
    tmem_alloc(tmem_slot, G::kTmemCols);
    tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accum, 1);
    mbar_fence_init();
    s_fail = 0;
  }
  if (threadIdx.x == 64) {
    tma_prefetch_map(&ta);
    tma_prefetch_map(&tb);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;

  // Row tiles blockIdx.x, blockIdx.x + gridDim.x, ... below the row count: the ring's stage and
  // phase follow the k-step count over all tiles so far (g), the accumulator's phase the tile
  // count (iter).  Each tile ends with a CTA barrier, after which the accumulator and the
  // stages (the epilogue's staging) are free for the next tile.
  int iter = 0;
  for (int mt = blockIdx.x; mt < m_tiles; mt += gridDim.x, iter++) {
  const int m0 = mt * kBM;
  const int g0 = iter * nk;
  bool ok = true;
  if (warp == 0 && lane == 0) {
    int issued = 0;
    for (int kt = 0; kt < nk; kt++) {
      const int g = g0 + kt;
      const int s = g % kStages;
      const uint32_t use = (uint32_t)(g / kStages);
      if (use > 0 && !mbar_wait(empty0 + 8 * s, (use - 1) & 1u)) {
        ok = false;
        break;
      }
      const uint32_t a_s = base + s * G::kStage;
      mbar_expect_tx(full0 + 8 * s, G::kStage);
      tma_load_2d(a_s, &ta, kt * kBK, m0, full0 + 8 * s);
      tma_load_2d(a_s + G::kA, &tb, kt * kBK, n0, full0 + 8 * s);
      issued = kt + 1;
    }
    // every copy this thread started has landed before the stages are reused or the CTA leaves
    for (int kt = (issued > kStages ? issued - kStages : 0); kt < issued; kt++) {
      const int g = g0 + kt;
      if (!mbar_wait(full0 + 8 * (g % kStages), (uint32_t)(g / kStages) & 1u)) ok = false;
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = umma_idesc_bf16(kBM, BN);
    for (int kt = 0; kt < nk; kt++) {
      const int g = g0 + kt;
      const int s = g % kStages;
      if (!mbar_wait(full0 + 8 * s, (uint32_t)(g / kStages) & 1u)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t a_s = base + s * G::kStage;
      const uint64_t ad = sw128_kmajor_desc(a_s), bd = sw128_kmajor_desc(a_s + G::kA);
#pragma unroll
      for (int j = 0; j < kBK / 16; j++) umma_bf16(tmem, ad + 2 * j, bd + 2 * j, idesc, (kt | j) != 0 ? 1u : 0u);
      umma_commit(empty0 + 8 * s);
    }
    umma_commit(accum);  // after every MMA issued above has completed
  }
  if (!ok) atomicOr(e.err, e.err_bit);
  __syncwarp();

  if (mbar_wait(accum, (uint32_t)iter & 1u)) {
    tc_fence_after();
    const int quarter = warp & 3, half = warp >> 2;
    const int row = m0 + quarter * 32 + lane;
    const uint32_t t_row = tmem + ((uint32_t)(quarter * 32) << 16);
    // Row-major outputs go through shared memory (the freed pipeline stages): each thread holds
    // one row, so storing straight from registers would touch 32 sectors per warp store.  A
    // 32 x 32 tile per warp is written by rows and stored with the lanes along the columns.
    // Transposed outputs are already coalesced from registers (consecutive lanes = rows).
    float* st_x = reinterpret_cast<float*>(smem_raw + (base - raw)) + warp * (2 * 32 * kStagePitch);
    float* st_z = st_x + 32 * kStagePitch;
    const bool rowmajor = e.out_f32 || e.out_bf16 || e.z_out;
    for (int c = half * (BN / 2); c < (half + 1) * (BN / 2); c += kStageCols) {
      if (n0 + c >= e.N) break;  // uniform over the warp
      float v[kStageCols];
      tmem_ld32(t_row + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < kStageCols; i++) {
        const int n = n0 + c + i;
        float x = v[i], z = 0.f;
        if (row < m_rows && n < e.N) {
          if (e.bias) x += e.bias[n];
          z = x;
          if (ACT == kActSilu) {
            x = x * sigmoid_fast(x);
          } else if (ACT == kActSiluGrad) {
            const float zi = e.zin[(size_t)row * e.ldzin + n];
            const float sg = sigmoid_fast(zi);
            x *= sg * (1.0f + zi * (1.0f - sg));
          }
          if (e.out_bf16_t && ok) e.out_bf16_t[(size_t)n * e.ldt + row] = __float2bfloat16_rn(x);
        }
        st_x[lane * kStagePitch + i] = x;
        if (e.z_out) st_z[lane * kStagePitch + i] = z;
      }
      __syncwarp();
      if (rowmajor && ok) {
        const int j = lane, n = n0 + c + lane;
        if (j < min(kStageCols, e.N - (n0 + c))) {
          for (int r = 0; r < 32; r++) {
            const int gr = m0 + quarter * 32 + r;
            if (gr >= m_rows) break;
            const float x = st_x[r * kStagePitch + j];
            if (e.out_f32) e.out_f32[(size_t)gr * e.ldo + n] = x;
            if (e.out_bf16) e.out_bf16[(size_t)gr * e.ld_bf16 + n] = __float2bfloat16_rn(x);
            if (e.z_out) e.z_out[(size_t)gr * e.ldz + n] = st_z[r * kStagePitch + j];
          }
        }
      }
      __syncwarp();
    }
  } else {
    atomicOr(e.err, e.err_bit);
    ok = false;
  }
  if (!ok) s_fail = 1;
  // the staging writes above precede the next tile's TMA writes into the same stages
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (s_fail) break;  // uniform: read after the barrier
  }
  if (warp == 0) {
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
  // at most one wave of CTAs; each loops over row tiles (rows beyond *m_dyn are never visited)
  static int max_ctas = 0;
  static std::once_flag once_occ;
  std::call_once(once_occ, [] {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_bf16<BN, ACT>, kThreads, G::kSmem) ==
            cudaSuccess)
      max_ctas = sms * std::max(1, per_sm);
  });
  const int tiles_m = (e.M + kBM - 1) / kBM, tiles_n = (e.N + BN - 1) / BN;
  const int gx = max_ctas > 0 ? std::min(tiles_m, std::max(1, max_ctas / tiles_n)) : tiles_m;
  dim3 grid(gx, tiles_n);
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
  // 64-column tiles keep small and medium problems spread over the SMs; very tall problems use
  // 128-column tiles (fewer re-reads of A)
  const long long tiles64 = (long long)((e.M + kBM - 1) / kBM) * ((e.N + 63) / 64);
  return (tiles64 > 8 * 152 && e.N > 64) ? launch_act<128>(A, lda, B, ldb, e, stream)
                                         : launch_act<64>(A, lda, B, ldb, e, stream);
}

}  // namespace souffle
