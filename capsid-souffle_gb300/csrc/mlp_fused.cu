// The surrogate network's whole forward pass (n_in <= 64 -> w -> w -> w -> out_pad, w = 128 or
// 256, SiLU on the hidden layers) in one persistent tcgen05 kernel: a 128-row tile's activations never leave
// the SM between layers.
//
// One CTA per SM (320 threads, 10 warps), looping over 128-row tiles.  Two tiles are in flight
// per CTA, in two slots; each slot owns a 128 x 256 BF16 activation buffer in shared memory
// (four 16 KB K-chunks in the 128-byte-swizzled K-major layout the MMA reads) and a 256-column
// FP32 accumulator in tensor memory (512 columns in all).  The units of work -- (slot, layer) --
// run in the order (0,L1) (1,L1) (0,L2) (1,L2) ... (1,L4), so the tensor cores work on one slot
// while the epilogue warps drain the other:
//   warp 0, lane 0  TMA producer: a tile's input rows (128 x 64 BF16) into chunk 0 of its slot's
//                   buffer once the slot's previous tile has finished its last layer, and the
//                   weights of every unit, 128 output rows x 64 K at a time, through a ring of
//                   16 KB stages (the weights are the same for every tile and stay in L2)
//   warp 1, lane 0  MMA issuer: per stage four K = 16 tcgen05.mma (M = 128, N = 128 or the
//                   output layer's remainder) from the slot's activation chunk and the stage into
//                   the slot's accumulator; tcgen05.commit frees the stage, and after a unit's
//                   last stage signals the epilogue ("acc full") and, after the output layer,
//                   frees the slot's buffer for the next input ("act free")
//   warps 2-9       epilogue: warp w reads accumulator lanes 32 (w % 4) .. + 31 (one row per
//                   thread) and half (w - 2) / 4 of the columns; hidden layers: + bias, SiLU,
//                   BF16, written straight into the slot's activation buffer (the next layer's A
//                   operand, same swizzle); output layer: + bias, FP32 rows to global memory.
//                   Then "epi done": the accumulator is drained and the buffer holds the next
//                   layer's input.
// SiLU(z) = z sigma(z) = h + h tanh(h), h = z / 2: one tanh.approx (a single MUFU operation,
// relative error below 2^-10) per element instead of an exponential and a division; the result
// is rounded to BF16 (2^-9) right after.  Every wait is bounded (umma.cuh); a timeout sets the
// caller's error bit and a shared abort flag that makes the other roles leave their loops.
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "gemm.cuh"
#include "umma.cuh"

namespace souffle {

namespace {

constexpr int kFRows = 128;                   // tile rows = MMA M
constexpr int kFK = 64;                       // K per chunk / stage (128 bytes of BF16)
constexpr int kFWidth = 256;                  // largest hidden width (buffers and bias slots are sized for it)
constexpr int kFChunk = kFRows * kFK * 2;     // 16 KB: one K-chunk of a tile, or one weight stage
constexpr int kFAct = kFWidth / kFK * kFChunk;  // 64 KB activation buffer per slot
constexpr int kFStages = 5;
constexpr int kFEpiWarps = 8;
constexpr int kFThreads = 32 * (2 + kFEpiWarps);
constexpr int kFMaxOut = 256;
constexpr int kFBias = 3 * kFWidth + kFMaxOut;  // hidden half-biases, then the output bias
// barriers: full[kFStages], empty[kFStages], x_full[2], acc_full[2], epi_done[2], act_free[2], drain
constexpr int kFBars = 2 * kFStages + 9;
constexpr int kFSmem = 1024 + 2 * kFAct + kFStages * kFChunk + kFBias * 4 + kFBars * 8 + 16;
static_assert(kFSmem <= 232448, "fits one CTA per SM");

struct FusedArgs {
  int m_cap;            // rows of the input / output buffers
  const int* m_dyn;     // live rows (device), or null = m_cap
  int n_in;             // <= 64
  int width;            // hidden width: 128 or 256
  int out_pad;          // output columns computed and stored (multiple of 16, <= 256)
  const float* bias[4];  // [256] x 3, [out_pad]
  float* y;             // [m_cap][ldy] FP32, or
  __nv_bfloat16* yb;    // [m_cap][ldy] BF16 (when set, instead of y)
  int ldy;
  unsigned int* err;
  unsigned int err_bit;
};

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack2_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// bounded wait that also gives up when another role has aborted
__device__ __forceinline__ bool fwait(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
  for (unsigned i = 0; i < kMaxPolls; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63u) == 63u && *abort_flag) return false;
  }
  *abort_flag = 1;
  return false;
}

// output columns of the layer: stage parts of up to 128 rows (the last may be narrower)
__device__ __forceinline__ int layer_n(int l, int out_pad, int width) { return l == 3 ? out_pad : width; }
__device__ __forceinline__ int layer_k_chunks(int l, int n_in, int width) {
  return l == 0 ? (n_in + kFK - 1) / kFK : width / kFK;
}

}  // namespace

__global__ void __launch_bounds__(kFThreads, 1)
    k_mlp_fused(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw0,
                const __grid_constant__ CUtensorMap tw1, const __grid_constant__ CUtensorMap tw2,
                const __grid_constant__ CUtensorMap tw3, FusedArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ int s_abort;
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  const uint32_t act0 = base;                               // slot buffers: act0 + s * kFAct
  const uint32_t ring = base + 2 * kFAct;                   // stage g: ring + g * kFChunk
  const uint32_t bias_s = ring + kFStages * kFChunk;        // float [kFBias]
  const uint32_t bars = bias_s + kFBias * 4;
  const uint32_t full0 = bars, empty0 = bars + 8 * kFStages;
  const uint32_t xfull0 = bars + 16 * kFStages, accfull0 = xfull0 + 16, epidone0 = accfull0 + 16,
                 actfree0 = epidone0 + 16, drain = actfree0 + 16;
  const uint32_t tmem_slot = drain + 8;
  float* s_bias = reinterpret_cast<float*>(smem_raw + (bias_s - raw));
  volatile uint32_t* tmem_slot_ptr = reinterpret_cast<volatile uint32_t*>(smem_raw + (tmem_slot - raw));
  volatile int* abort_flag = &s_abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_rows = a.m_dyn ? min(a.m_cap, *a.m_dyn) : a.m_cap;
  const int tiles = (m_rows + kFRows - 1) / kFRows;
  if ((int)blockIdx.x >= tiles) return;  // uniform over the CTA, before any allocation
  // this CTA's tiles: blockIdx.x + i gridDim.x, tile i in slot i % 2, pair i / 2
  const int my_tiles = (tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  const int pairs = (my_tiles + 1) / 2;

  if (warp == 1) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < kFStages; s++) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int s = 0; s < 2; s++) {
      mbar_init(xfull0 + 8 * s, 1);
      mbar_init(accfull0 + 8 * s, 1);
      mbar_init(epidone0 + 8 * s, kFEpiWarps);
      mbar_init(actfree0 + 8 * s, 1);
    }
    mbar_init(drain, 1);
    mbar_fence_init();
  }
  if (threadIdx.x == 32) {
    tma_prefetch_map(&tx);
    tma_prefetch_map(&tw0);
    tma_prefetch_map(&tw1);
    tma_prefetch_map(&tw2);
    tma_prefetch_map(&tw3);
  }
  // biases: half of each hidden bias (SiLU works on z / 2), the output bias as it is
  for (int t = threadIdx.x; t < kFBias; t += blockDim.x) {
    float v = 0.f;
    if (t < 3 * kFWidth) {
      if (t % kFWidth < a.width) v = 0.5f * a.bias[t / kFWidth][t % kFWidth];
    }
    else if (t - 3 * kFWidth < a.out_pad) v = a.bias[3][t - 3 * kFWidth];
    s_bias[t] = v;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;
  const CUtensorMap* wmap[4] = {&tw0, &tw1, &tw2, &tw3};

  if (warp == 0) {
    if (lane == 0) {
      // ---- producer
      int g = 0;          // weight stages issued
      int xs[2] = {0, 0};  // inputs loaded per slot
      bool ok = true;
      for (int p = 0; p < pairs && ok; p++) {
        for (int l = 0; l < 4 && ok; l++) {
          for (int s = 0; s < 2 && ok; s++) {
            const int i = 2 * p + s;
            if (i >= my_tiles) continue;
            if (l == 0) {
              // the slot's previous tile has finished its output layer (its MMAs read the buffer)
              if (xs[s] > 0 && !fwait(actfree0 + 8 * s, (uint32_t)(xs[s] - 1) & 1u, abort_flag)) {
                ok = false;
                break;
              }
              const int tile = (int)blockIdx.x + i * (int)gridDim.x;
              mbar_expect_tx(xfull0 + 8 * s, kFChunk);
              tma_load_2d(act0 + s * kFAct, &tx, 0, tile * kFRows, xfull0 + 8 * s);
              xs[s]++;
            }
            const int nk = layer_k_chunks(l, a.n_in, a.width), parts = (layer_n(l, a.out_pad, a.width) + 127) / 128;
            for (int kc = 0; kc < nk && ok; kc++) {
              for (int part = 0; part < parts; part++, g++) {
                const int st = g % kFStages;
                const uint32_t use = (uint32_t)(g / kFStages);
                if (use > 0 && !fwait(empty0 + 8 * st, (use - 1) & 1u, abort_flag)) {
                  ok = false;
                  break;
                }
                mbar_expect_tx(full0 + 8 * st, kFChunk);
                tma_load_2d(ring + st * kFChunk, wmap[l], kc * kFK, part * 128, full0 + 8 * st);
              }
            }
          }
        }
      }
      // every copy started here has landed before the CTA can leave
      for (int q = (g > kFStages ? g - kFStages : 0); q < g; q++)
        if (!mbar_wait(full0 + 8 * (q % kFStages), (uint32_t)(q / kFStages) & 1u)) ok = false;
      for (int s = 0; s < 2; s++)
        if (xs[s] > 0 && !mbar_wait(xfull0 + 8 * s, (uint32_t)(xs[s] - 1) & 1u)) ok = false;
      if (!ok) {
        *abort_flag = 1;
        atomicOr(a.err, a.err_bit);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer
      int g = 0;
      int units[2] = {0, 0};  // units issued per slot
      bool ok = true;
      for (int p = 0; p < pairs && ok; p++) {
        for (int l = 0; l < 4 && ok; l++) {
          for (int s = 0; s < 2 && ok; s++) {
            const int i = 2 * p + s;
            if (i >= my_tiles) continue;
            // the slot's previous unit has been drained by the epilogue (and, from the second
            // layer on, its output is this unit's input)
            if (units[s] > 0 && !fwait(epidone0 + 8 * s, (uint32_t)(units[s] - 1) & 1u, abort_flag)) {
              ok = false;
              break;
            }
            if (l == 0 && !fwait(xfull0 + 8 * s, (uint32_t)(i >> 1) & 1u, abort_flag)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const int n = layer_n(l, a.out_pad, a.width);
            const int nk = layer_k_chunks(l, a.n_in, a.width), parts = (n + 127) / 128;
            const uint32_t acc = tmem + (uint32_t)(s * kFWidth);
            const uint32_t abuf = act0 + s * kFAct;
            for (int kc = 0; kc < nk && ok; kc++) {
              for (int part = 0; part < parts; part++, g++) {
                const int st = g % kFStages;
                if (!fwait(full0 + 8 * st, (uint32_t)(g / kFStages) & 1u, abort_flag)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
                const int np_ = min(128, n - 128 * part);
                const uint32_t idesc = umma_idesc_bf16(kFRows, np_);
                const uint64_t ad = sw128_kmajor_desc(abuf + kc * kFChunk);
                const uint64_t bd = sw128_kmajor_desc(ring + st * kFChunk);
#pragma unroll
                for (int j = 0; j < kFK / 16; j++)
                  umma_bf16(acc + (uint32_t)(128 * part), ad + 2 * j, bd + 2 * j, idesc, (kc | j) != 0 ? 1u : 0u);
                umma_commit(empty0 + 8 * st);
              }
            }
            if (!ok) break;
            umma_commit(accfull0 + 8 * s);
            if (l == 3) umma_commit(actfree0 + 8 * s);
            units[s]++;
          }
        }
      }
      if (!ok) {
        atomicOr(a.err, a.err_bit);
        // MMAs issued before the failure may still be running: drain them (bounded) before the
        // tensor memory is released
        umma_commit(drain);
        mbar_wait(drain, 0);
      }
    }
  } else {
    // ---- epilogue
    const int q = warp & 3, half = (warp - 2) >> 2;
    const int r_local = q * 32 + lane;  // tile row = accumulator lane
    int units[2] = {0, 0};
    bool ok = true;
    for (int p = 0; p < pairs && ok; p++) {
      for (int l = 0; l < 4 && ok; l++) {
        for (int s = 0; s < 2 && ok; s++) {
          const int i = 2 * p + s;
          if (i >= my_tiles) continue;
          if (!fwait(accfull0 + 8 * s, (uint32_t)units[s] & 1u, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t t_row = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(s * kFWidth);
          if (l < 3) {
            // hidden layer: columns [half w/2, (half + 1) w/2) -> SiLU -> BF16 into the buffer
            const float* hb = s_bias + l * kFWidth;
            const uint32_t abuf = act0 + s * kFAct;
            const uint32_t rsw = (uint32_t)(r_local & 7);
#pragma unroll 1
            for (int c0 = half * (a.width >> 1); c0 < (half + 1) * (a.width >> 1); c0 += 32) {
              float v[32];
              tmem_ld32(t_row + (uint32_t)c0, v);
              uint32_t pk[16];
#pragma unroll
              for (int k = 0; k < 16; k++) {
                const float h0 = fmaf(v[2 * k], 0.5f, hb[c0 + 2 * k]);
                const float h1 = fmaf(v[2 * k + 1], 0.5f, hb[c0 + 2 * k + 1]);
                pk[k] = pack2_bf16(fmaf(h0, tanh_approx(h0), h0), fmaf(h1, tanh_approx(h1), h1));
              }
              // K-chunk c0 / 64, 16-byte units (c0 % 64) / 8 .. + 3, swizzled by the row
              const uint32_t rowaddr = abuf + (uint32_t)(c0 >> 6) * kFChunk + (uint32_t)r_local * 128u;
              const uint32_t u0 = (uint32_t)((c0 & 63) >> 3);
#pragma unroll
              for (int k = 0; k < 4; k++)
                st_shared_v4(rowaddr + (((u0 + k) ^ rsw) << 4), pk[4 * k], pk[4 * k + 1], pk[4 * k + 2], pk[4 * k + 3]);
            }
            fence_proxy_async_smem();
          } else {
            // output layer: columns [half n/2, (half + 1) n/2) + bias -> FP32 rows
            const int tile = (int)blockIdx.x + i * (int)gridDim.x;
            const int row = tile * kFRows + r_local;
            const bool row_ok = row < m_rows;
            const float* ob = s_bias + 3 * kFWidth;
            const int nh = a.out_pad >> 1;
            const int cb = half * nh, ce = cb + nh;
            float* yrow = a.y ? a.y + (size_t)row * a.ldy : nullptr;
            __nv_bfloat16* ybrow = a.yb ? a.yb + (size_t)row * a.ldy : nullptr;
            const bool vec = ((a.ldy & 3) == 0) && ((reinterpret_cast<uintptr_t>(a.y) & 15) == 0);
            const bool vecb = ((a.ldy & 7) == 0) && ((reinterpret_cast<uintptr_t>(a.yb) & 15) == 0);
            int c0 = cb;
#pragma unroll 1
            for (; c0 + 32 <= ce; c0 += 32) {
              float v[32];
              tmem_ld32(t_row + (uint32_t)c0, v);
              if (row_ok && ybrow) {  // BF16 rows: 16-byte stores of 8 values
                if (vecb && (c0 & 7) == 0) {
#pragma unroll
                  for (int k = 0; k < 4; k++)
                    *reinterpret_cast<uint4*>(ybrow + c0 + 8 * k) =
                        make_uint4(pack2_bf16(v[8 * k] + ob[c0 + 8 * k], v[8 * k + 1] + ob[c0 + 8 * k + 1]),
                                   pack2_bf16(v[8 * k + 2] + ob[c0 + 8 * k + 2], v[8 * k + 3] + ob[c0 + 8 * k + 3]),
                                   pack2_bf16(v[8 * k + 4] + ob[c0 + 8 * k + 4], v[8 * k + 5] + ob[c0 + 8 * k + 5]),
                                   pack2_bf16(v[8 * k + 6] + ob[c0 + 8 * k + 6], v[8 * k + 7] + ob[c0 + 8 * k + 7]));
                } else {
#pragma unroll
                  for (int k = 0; k < 32; k++) ybrow[c0 + k] = __float2bfloat16_rn(v[k] + ob[c0 + k]);
                }
              } else if (row_ok) {
                if (vec && (c0 & 3) == 0) {
#pragma unroll
                  for (int k = 0; k < 8; k++)
                    *reinterpret_cast<float4*>(yrow + c0 + 4 * k) =
                        make_float4(v[4 * k] + ob[c0 + 4 * k], v[4 * k + 1] + ob[c0 + 4 * k + 1],
                                    v[4 * k + 2] + ob[c0 + 4 * k + 2], v[4 * k + 3] + ob[c0 + 4 * k + 3]);
                } else {
#pragma unroll
                  for (int k = 0; k < 32; k++) yrow[c0 + k] = v[k] + ob[c0 + k];
                }
              }
            }
#pragma unroll 1
            for (; c0 < ce; c0 += 8) {
              float v[8];
              tmem_ld8(t_row + (uint32_t)c0, v);
              if (row_ok && ybrow) {
#pragma unroll
                for (int k = 0; k < 8; k++) ybrow[c0 + k] = __float2bfloat16_rn(v[k] + ob[c0 + k]);
              } else if (row_ok) {
#pragma unroll
                for (int k = 0; k < 8; k++) yrow[c0 + k] = v[k] + ob[c0 + k];
              }
            }
          }
          // this warp has read its part of the accumulator and written its part of the buffer
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(epidone0 + 8 * s);
          units[s]++;
        }
      }
    }
    if (!ok) atomicOr(a.err, a.err_bit);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 fused_encode_fn() {
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

// [rows][cols] BF16, row stride ld elements; box 64 columns x 128 rows, 128-byte swizzle
bool fused_map(CUtensorMap* m, const void* p, int rows, int cols, int ld) {
  auto fn = fused_encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kFK, (cuuint32_t)kFRows};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(p), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool mlp_fused_supported(int n_in, int width, int out_pad) {
  return n_in >= 8 && n_in <= kFK && n_in % 8 == 0 && (width == 128 || width == kFWidth) && out_pad >= 16 &&
         out_pad <= kFMaxOut && out_pad % 16 == 0;
}

cudaError_t mlp_forward_fused(const __nv_bfloat16* x, int ldx, int m_cap, const int* m_dyn, int n_in, int width,
                              const __nv_bfloat16* const w[4], const int ldw[4], int out_pad, const float* const bias[4],
                              float* y, int ldy, unsigned int* err, unsigned int err_bit, cudaStream_t st,
                              __nv_bfloat16* yb) {
  if (!mlp_fused_supported(n_in, width, out_pad) || m_cap < 1 || !x || !(y || yb) || !err || ldx < n_in || ldx % 8 ||
      ldy < out_pad || (reinterpret_cast<uintptr_t>(x) & 15) || ldw[0] < n_in || ldw[1] < width ||
      ldw[2] < width || ldw[3] < width)
    return cudaErrorInvalidValue;
  for (int l = 0; l < 4; l++)
    if (!w[l] || !bias[l] || ldw[l] % 8 || (reinterpret_cast<uintptr_t>(w[l]) & 15)) return cudaErrorInvalidValue;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kFSmem);
  });
  if (attr != cudaSuccess) return attr;
  CUtensorMap tx, tw[4];
  if (!fused_map(&tx, x, m_cap, n_in, ldx) || !fused_map(&tw[0], w[0], width, n_in, ldw[0]) ||
      !fused_map(&tw[1], w[1], width, width, ldw[1]) || !fused_map(&tw[2], w[2], width, width, ldw[2]) ||
      !fused_map(&tw[3], w[3], out_pad, width, ldw[3]))
    return cudaErrorInvalidValue;
  static int sms = 0;
  static std::once_flag once_sm;
  std::call_once(once_sm, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 0;
  });
  FusedArgs a;
  a.m_cap = m_cap;
  a.m_dyn = m_dyn;
  a.n_in = n_in;
  a.width = width;
  a.out_pad = out_pad;
  for (int l = 0; l < 4; l++) a.bias[l] = bias[l];
  a.y = yb ? nullptr : y;
  a.yb = yb;
  a.ldy = ldy;
  a.err = err;
  a.err_bit = err_bit;
  // one CTA per SM, each looping over tiles; CTAs beyond the live tiles leave at once
  const long long tiles = ((long long)m_cap + kFRows - 1) / kFRows;
  const int gx = (int)std::min<long long>(tiles, sms > 0 ? sms : 148);
  k_mlp_fused<<<gx, kFThreads, kFSmem, st>>>(tx, tw[0], tw[1], tw[2], tw[3], a);
  return cudaGetLastError();
}

}  // namespace souffle
