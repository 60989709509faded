// The surrogate network: n_in -> w -> w -> w -> n_out (w = 128 or 256) with SiLU, trained and evaluated with
// the tcgen05 GEMM (gemm.cu).  Parameters live as FP32 masters plus BF16 copies W [out][in] (the
// forward B operand) and W^T [in][out] (the backward B operand); activations are BF16, kept both
// row-major (next forward A operand) and transposed (A/B operands of the weight-gradient GEMMs,
// whose contraction runs over the batch).
//
// Forward, layer l:   z_l = a_{l-1} W_l^T + b_l,  a_l = SiLU(z_l)        (output layer: no SiLU)
// Backward:           dY = 2 (y - t) / (m n_out)
//                     dW_l = dZ_l^T a_{l-1},  db_l = column sums of dZ_l
//                     dZ_{l-1} = (dZ_l W_l) * SiLU'(z_{l-1})
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "devbuf.cuh"
#include "gemm.cuh"
#include "souffle_surrogate.h"

namespace souffle {
void record_error(const std::string& msg);
bool mlp_fused_supported(int n_in, int width, int out_pad);
cudaError_t mlp_forward_fused(const __nv_bfloat16* x, int ldx, int m_cap, const int* m_dyn, int n_in, int width,
                              const __nv_bfloat16* const w[4], const int ldw[4], int out_pad, const float* const bias[4],
                              float* y, int ldy, unsigned int* err, unsigned int err_bit, cudaStream_t st,
                              __nv_bfloat16* yb = nullptr);
}

using namespace souffle;

namespace {

constexpr int kLayers = 4;

souffle_status fail(souffle_status s, const std::string& msg) {
  record_error(msg);
  return s;
}

#define MLP_TRY(x)                                                                                   \
  do {                                                                                               \
    cudaError_t e_ = (x);                                                                            \
    if (e_ != cudaSuccess) return fail(SOUFFLE_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int round_up(int x, int m) { return (x + m - 1) / m * m; }

// x [m][n_in] FP32 -> a0 [m][ld] BF16 row-major and a0T [n_in][ldt] BF16
// (rows >= *m_dyn skipped when m_dyn is given; grid-stride over the rest)
__global__ void k_pack_input(const float* x, int m, int n_in, __nv_bfloat16* a0, int ld, __nv_bfloat16* a0t, int ldt,
                             const int* m_dyn = nullptr) {
  const int rows = m_dyn ? min(m, *m_dyn) : m;
  const long long n = (long long)rows * n_in;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / n_in), c = (int)(i - (long long)r * n_in);
    const __nv_bfloat16 v = __float2bfloat16_rn(x[i]);
    a0[(size_t)r * ld + c] = v;
    if (a0t) a0t[(size_t)c * ldt + r] = v;
  }
}

// dY = 2 (y - t) / (m n_out) as BF16 (row-major and transposed, zero beyond n_out), and per-block
// partial sums of (y - t)^2 in a fixed order.
__global__ void k_loss(const float* y, int ldy, const float* t, int m, int n_out, int n_pad, __nv_bfloat16* dy,
                       __nv_bfloat16* dyt, int ldt, float* partial) {
  __shared__ float red[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float sq = 0.0f;
  if (i < m * n_pad) {
    const int r = i / n_pad, c = i - r * n_pad;
    float g = 0.0f;
    if (c < n_out) {
      const float d = y[(size_t)r * ldy + c] - t[(size_t)r * n_out + c];
      sq = d * d;
      g = 2.0f * d / ((float)m * (float)n_out);
    }
    const __nv_bfloat16 gb = __float2bfloat16_rn(g);
    dy[(size_t)r * n_pad + c] = gb;
    dyt[(size_t)c * ldt + r] = gb;
  }
  red[threadIdx.x] = sq;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// row sums of a transposed BF16 gradient [n][ldt] over its first m columns: the bias gradient.
// One warp per row, fixed order.
__global__ void k_row_sums(const __nv_bfloat16* g, int n, int m, int ldt, float* out) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (row >= n) return;
  float s = 0.0f;
  for (int c = lane; c < m; c += 32) s += __bfloat162float(g[(size_t)row * ldt + c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[row] = s;
}

__global__ void k_sum(const float* p, int n, float* out) {
  __shared__ float red[256];
  float s = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Adam on one weight matrix [rows][cols] (rows >= valid_rows stay zero) and refresh of its BF16
// copy and BF16 transpose [cols][rows].
__global__ void k_adam_w(float* w, float* mo, float* ve, const float* g, int rows, int valid_rows, int cols, float lr,
                         float c1, float c2, __nv_bfloat16* wb, __nv_bfloat16* wbt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const int r = i / cols, c = i - r * cols;
  float p = w[i];
  if (r < valid_rows && lr > 0.0f) {
    const float gi = g[i];
    const float mi = 0.9f * mo[i] + 0.1f * gi;
    const float vi = 0.999f * ve[i] + 0.001f * gi * gi;
    mo[i] = mi;
    ve[i] = vi;
    p -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
    w[i] = p;
  }
  const __nv_bfloat16 b = __float2bfloat16_rn(p);
  wb[i] = b;
  wbt[(size_t)c * rows + r] = b;
}

__global__ void k_adam_b(float* b, float* mo, float* ve, const float* g, int n, float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = 0.9f * mo[i] + 0.1f * gi;
  const float vi = 0.999f * ve[i] + 0.001f * gi * gi;
  mo[i] = mi;
  ve[i] = vi;
  b[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

// y [m][ld] -> out [m][n_out]
__global__ void k_unpad(const float* y, int ld, int m, int n_out, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * n_out) return;
  const int r = i / n_out, c = i - r * n_out;
  out[i] = y[(size_t)r * ld + c];
}

int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

struct souffle_mlp {
  int n_in = 0, width = 0, n_out = 0, cap = 0, device = 0;
  int in[kLayers], out[kLayers], out_pad[kLayers];  // per layer; out_pad = rows stored (mult. of 16)
  int in_ld[kLayers];                               // row stride of the layer input (mult. of 8)
  cudaStream_t stream = nullptr;
  DevBuf<float> w[kLayers], b[kLayers], mw[kLayers], vw[kLayers], mb[kLayers], vb[kLayers];
  DevBuf<float> gw[kLayers], gb[kLayers];
  DevBuf<__nv_bfloat16> wb[kLayers], wbt[kLayers];
  DevBuf<__nv_bfloat16> act[kLayers], act_t[kLayers];  // a_0 .. a_3 and transposes
  DevBuf<float> z[kLayers];                            // z_1 .. z_3 (index l for layer l output)
  DevBuf<__nv_bfloat16> dz[kLayers + 1], dz_t[kLayers + 1];  // dZ_l for l = 1..4 (4 = dY)
  DevBuf<float> y, partial, loss;
  DevBuf<__nv_bfloat16> yb;  // BF16 copy of the output rows (fused forward for the surrogate)
  DevBuf<unsigned int> err;
  long long steps = 0;
  // the normalisation of the data the surrogate was trained on: per input feature mean and
  // 1/spread, per output mean, spread and 1/spread (set by souffle_surrogate_fit; travels with
  // the network to any handle it is attached to)
  DevBuf<float> x_mean, x_istd, t_mean, t_std, t_istd;
  bool has_norm = false;
};

namespace {

souffle_status check_gemm_err(souffle_mlp* h) {
  unsigned int e = 0;
  MLP_TRY(cudaMemcpyAsync(&e, h->err.p, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
  MLP_TRY(cudaStreamSynchronize(h->stream));
  if (e) {
    cudaMemsetAsync(h->err.p, 0, sizeof(unsigned int), h->stream);
    return fail(SOUFFLE_ERR_CUDA, "tensor-core GEMM: a bounded wait ran out");
  }
  return SOUFFLE_OK;
}

// forward over m rows of act[0] (rows >= *m_dyn skipped when given); keep = store z and
// transposed activations for the backward pass
cudaError_t forward_on(souffle_mlp* h, int m, bool keep, cudaStream_t st, const int* m_dyn, unsigned int* err,
                       unsigned int err_bit = 1u) {
  for (int l = 0; l < kLayers; l++) {
    GemmEpi e;
    e.M = m;
    e.m_dyn = m_dyn;
    e.N = (l == kLayers - 1) ? h->out_pad[l] : h->out[l];
    e.K = h->in[l];
    e.bias = h->b[l].p;
    e.err = err;
    e.err_bit = err_bit;
    if (l < kLayers - 1) {
      e.act = kActSilu;
      e.out_bf16 = h->act[l + 1].p;
      e.ld_bf16 = h->in_ld[l + 1];
      if (keep) {
        e.z_out = h->z[l + 1].p;
        e.ldz = h->out[l];
        e.out_bf16_t = h->act_t[l + 1].p;
        e.ldt = h->cap;
      }
    } else {
      e.out_f32 = h->y.p;
      e.ldo = h->out_pad[l];
    }
    const cudaError_t r = gemm_bf16(h->act[l].p, h->in_ld[l], h->wb[l].p, h->in_ld[l], e, st);
    if (r != cudaSuccess) return r;
  }
  return cudaSuccess;
}

souffle_status forward(souffle_mlp* h, int m, bool keep) {
  MLP_TRY(forward_on(h, m, keep, h->stream, nullptr, h->err.p));
  return SOUFFLE_OK;
}

// gradients into gw/gb for a batch whose forward (keep) has run; loss partials from k_loss
souffle_status backward(souffle_mlp* h, const float* t, int m) {
  const int L = kLayers - 1;
  const int np_out = h->out_pad[L];
  const int nb = blocks((long long)m * np_out, 256);
  MLP_TRY(h->partial.n < (size_t)nb ? cudaErrorInvalidValue : cudaSuccess);
  k_loss<<<nb, 256, 0, h->stream>>>(h->y.p, np_out, t, m, h->n_out, np_out, h->dz[L + 1].p, h->dz_t[L + 1].p, h->cap,
                                    h->partial.p);
  MLP_TRY(cudaGetLastError());
  k_sum<<<1, 256, 0, h->stream>>>(h->partial.p, nb, h->loss.p);
  for (int l = L; l >= 0; l--) {
    // dW_l [out_pad][in] = dZ_l^T a_{l-1}: A = dZ_l^T [out_pad][m], B = a_{l-1}^T [in][m], K = m
    const int rows = (l == L) ? np_out : h->out[l];
    GemmEpi e;
    e.M = rows;
    e.N = h->in[l];
    e.K = m;
    e.err = h->err.p;
    e.out_f32 = h->gw[l].p;
    e.ldo = h->in[l];
    MLP_TRY(gemm_bf16(h->dz_t[l + 1].p, h->cap, h->act_t[l].p, h->cap, e, h->stream));
    k_row_sums<<<blocks(rows, 8), 256, 0, h->stream>>>(h->dz_t[l + 1].p, rows, m, h->cap, h->gb[l].p);
    MLP_TRY(cudaGetLastError());
    if (l == 0) break;
    // dZ_{l} (input side of layer l) = (dZ_{l+1} W_l) * SiLU'(z_l): A = dZ [m][rows], B = W_l^T [in][rows]
    GemmEpi d;
    d.M = m;
    d.N = h->in[l];
    d.K = rows;
    d.err = h->err.p;
    d.act = kActSiluGrad;
    d.zin = h->z[l].p;
    d.ldzin = h->out[l - 1];
    d.out_bf16 = h->dz[l].p;
    d.ld_bf16 = h->in[l];
    d.out_bf16_t = h->dz_t[l].p;
    d.ldt = h->cap;
    MLP_TRY(gemm_bf16(h->dz[l + 1].p, rows, h->wbt[l].p, rows, d, h->stream));
  }
  return SOUFFLE_OK;
}

souffle_status pack_input(souffle_mlp* h, const float* x, int m, bool keep) {
  k_pack_input<<<blocks((long long)m * h->n_in, 256), 256, 0, h->stream>>>(
      x, m, h->n_in, h->act[0].p, h->in_ld[0], keep ? h->act_t[0].p : nullptr, h->cap);
  MLP_TRY(cudaGetLastError());
  return SOUFFLE_OK;
}

souffle_status refresh_bf16(souffle_mlp* h, float lr) {
  h->steps += lr > 0.0f ? 1 : 0;
  const float c1 = lr > 0.0f ? 1.0f / (1.0f - std::pow(0.9f, (float)h->steps)) : 0.0f;
  const float c2 = lr > 0.0f ? 1.0f / (1.0f - std::pow(0.999f, (float)h->steps)) : 0.0f;
  for (int l = 0; l < kLayers; l++) {
    const int rows = h->out_pad[l], cols = h->in[l];
    k_adam_w<<<blocks((long long)rows * cols, 256), 256, 0, h->stream>>>(
        h->w[l].p, h->mw[l].p, h->vw[l].p, h->gw[l].p, rows, h->out[l], cols, lr, c1, c2, h->wb[l].p, h->wbt[l].p);
    MLP_TRY(cudaGetLastError());
    if (lr > 0.0f) {
      k_adam_b<<<blocks(h->out[l], 256), 256, 0, h->stream>>>(h->b[l].p, h->mb[l].p, h->vb[l].p, h->gb[l].p, h->out[l],
                                                              lr, c1, c2);
      MLP_TRY(cudaGetLastError());
    }
  }
  return SOUFFLE_OK;
}

}  // namespace

namespace souffle {

constexpr unsigned int kErrSurrogateBit = 8u;  // the system's error word: surrogate network timeout

cudaError_t mlp_forward_packed_async(souffle_mlp* h, int m_cap, const int* m_dyn, unsigned int* err, cudaStream_t st,
                                     const float** y, int* ldy);

// For the surrogate inside a system handle: forward over m_cap rows of x on the caller's stream,
// rows >= *m_dyn skipped, output left in the network's buffer (*y, row stride *ldy).  Enqueues
// only, so it can be captured in a CUDA graph.
cudaError_t mlp_forward_async(souffle_mlp* h, const float* x, int m_cap, const int* m_dyn, unsigned int* err,
                              cudaStream_t st, const float** y, int* ldy) {
  if (m_cap < 1 || m_cap > h->cap) return cudaErrorInvalidValue;
  k_pack_input<<<std::min(blocks((long long)m_cap * h->n_in, 256), 152 * 8), 256, 0, st>>>(
      x, m_cap, h->n_in, h->act[0].p, h->in_ld[0], nullptr, h->cap, m_dyn);
  cudaError_t r = cudaGetLastError();
  if (r != cudaSuccess) return r;
  return mlp_forward_packed_async(h, m_cap, m_dyn, err, st, y, ldy);
}

// The fused forward over rows already in the BF16 input buffer, output rows in BF16 (*yb, row
// stride *ldy) -- the form the surrogate step reads; false when the shape has no fused forward.
bool mlp_forward_packed_bf16_async(souffle_mlp* h, int m_cap, const int* m_dyn, unsigned int* err, cudaStream_t st,
                                   const __nv_bfloat16** yb, int* ldy, cudaError_t* r) {
  const int L = kLayers - 1;
  if (m_cap < 1 || m_cap > h->cap || !mlp_fused_supported(h->n_in, h->width, h->out_pad[L])) return false;
  const __nv_bfloat16* w[4] = {h->wb[0].p, h->wb[1].p, h->wb[2].p, h->wb[3].p};
  const int ldw[4] = {h->in[0], h->in[1], h->in[2], h->in[3]};
  const float* b[4] = {h->b[0].p, h->b[1].p, h->b[2].p, h->b[3].p};
  *r = mlp_forward_fused(h->act[0].p, h->in_ld[0], m_cap, m_dyn, h->n_in, h->width, w, ldw, h->out_pad[L], b, nullptr,
                         h->out_pad[L], err, kErrSurrogateBit, st, h->yb.p);
  *yb = h->yb.p;
  *ldy = h->out_pad[L];
  return true;
}

// The network's BF16 input buffer [cap][*ld] (row-major), which mlp_forward_packed_async reads.
__nv_bfloat16* mlp_input_bf16(souffle_mlp* h, int* ld) {
  *ld = h->in_ld[0];
  return h->act[0].p;
}

// Forward over rows already in the BF16 input buffer: the fused one-kernel forward
// (mlp_fused.cu) where the shape allows it, else the per-layer GEMMs.  Enqueues only.
cudaError_t mlp_forward_packed_async(souffle_mlp* h, int m_cap, const int* m_dyn, unsigned int* err, cudaStream_t st,
                                     const float** y, int* ldy) {
  if (m_cap < 1 || m_cap > h->cap) return cudaErrorInvalidValue;
  const int L = kLayers - 1;
  cudaError_t r;
  if (mlp_fused_supported(h->n_in, h->width, h->out_pad[L])) {
    const __nv_bfloat16* w[4] = {h->wb[0].p, h->wb[1].p, h->wb[2].p, h->wb[3].p};
    const int ldw[4] = {h->in[0], h->in[1], h->in[2], h->in[3]};
    const float* b[4] = {h->b[0].p, h->b[1].p, h->b[2].p, h->b[3].p};
    r = mlp_forward_fused(h->act[0].p, h->in_ld[0], m_cap, m_dyn, h->n_in, h->width, w, ldw, h->out_pad[L], b, h->y.p,
                          h->out_pad[L], err, kErrSurrogateBit, st);
  } else {
    r = forward_on(h, m_cap, false, st, m_dyn, err, kErrSurrogateBit);
  }
  *y = h->y.p;
  *ldy = h->out_pad[L];
  return r;
}

MlpNorm mlp_norm(souffle_mlp* h) {
  return MlpNorm{h->x_mean.p, h->x_istd.p, h->t_mean.p, h->t_std.p, h->t_istd.p, &h->has_norm};
}

void mlp_dims(const souffle_mlp* h, int* n_in, int* n_out, int* cap) {
  *n_in = h->n_in;
  *n_out = h->n_out;
  *cap = h->cap;
}

}  // namespace souffle

extern "C" {

souffle_status souffle_mlp_create(int32_t n_in, int32_t width, int32_t n_out, int32_t max_batch, uint64_t seed,
                                  int32_t device, souffle_mlp** out) {
  if (!out) return fail(SOUFFLE_ERR_BAD_INPUT, "null output");
  *out = nullptr;
  if (n_in < 8 || n_in > 256 || n_in % 8 || (width != 128 && width != 256) || n_out < 1 || n_out > 256 || max_batch < 1 ||
      max_batch > (1 << 22))
    return fail(SOUFFLE_ERR_BAD_INPUT,
                "mlp shape: n_in a multiple of 8 up to 256, 1 <= n_out <= 256, width 128 or 256, 1 <= max_batch <= 2^22");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(SOUFFLE_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) return fail(SOUFFLE_ERR_BAD_INPUT, "bad device");
  MLP_TRY(cudaSetDevice(device));
  souffle_mlp* h = new souffle_mlp;
  h->n_in = n_in;
  h->width = width;
  h->n_out = n_out;
  h->cap = round_up(max_batch, 128);
  h->device = device;
  const int dims[kLayers + 1] = {n_in, width, width, width, n_out};
  for (int l = 0; l < kLayers; l++) {
    h->in[l] = dims[l];
    h->out[l] = dims[l + 1];
    h->out_pad[l] = round_up(dims[l + 1], 16);
    h->in_ld[l] = round_up(dims[l], 8);
  }
  auto cleanup = [&](souffle_status s) {
    delete h;
    return s;
  };
#define MLP_TRY_C(x)                                                                                  \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess) return cleanup(fail(SOUFFLE_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_))); \
  } while (0)
  MLP_TRY_C(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  std::mt19937_64 rng(seed);
  for (int l = 0; l < kLayers; l++) {
    const size_t nw = (size_t)h->out_pad[l] * h->in[l];
    std::vector<float> w(nw, 0.0f);
    const float lim = std::sqrt(3.0f / (float)h->in[l]);
    std::uniform_real_distribution<float> u(-lim, lim);
    for (int r = 0; r < h->out[l]; r++)
      for (int c = 0; c < h->in[l]; c++) w[(size_t)r * h->in[l] + c] = u(rng);
    for (auto* buf : {&h->w[l], &h->mw[l], &h->vw[l], &h->gw[l]}) {
      MLP_TRY_C(buf->alloc(nw));
      MLP_TRY_C(cudaMemset(buf->p, 0, nw * sizeof(float)));
    }
    MLP_TRY_C(cudaMemcpy(h->w[l].p, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice));
    for (auto* buf : {&h->b[l], &h->mb[l], &h->vb[l], &h->gb[l]}) {
      MLP_TRY_C(buf->alloc(h->out_pad[l]));
      MLP_TRY_C(cudaMemset(buf->p, 0, h->out_pad[l] * sizeof(float)));
    }
    MLP_TRY_C(h->wb[l].alloc(nw));
    MLP_TRY_C(h->wbt[l].alloc(nw));
    MLP_TRY_C(h->act[l].alloc((size_t)h->cap * h->in_ld[l]));
    MLP_TRY_C(h->act_t[l].alloc((size_t)h->in[l] * h->cap));
    MLP_TRY_C(cudaMemset(h->act[l].p, 0, (size_t)h->cap * h->in_ld[l] * 2));
    MLP_TRY_C(cudaMemset(h->act_t[l].p, 0, (size_t)h->in[l] * h->cap * 2));
    if (l > 0) MLP_TRY_C(h->z[l].alloc((size_t)h->cap * h->out[l - 1]));
  }
  for (int l = 1; l <= kLayers; l++) {
    const int cols = h->out_pad[l - 1];
    MLP_TRY_C(h->dz[l].alloc((size_t)h->cap * cols));
    MLP_TRY_C(h->dz_t[l].alloc((size_t)cols * h->cap));
    MLP_TRY_C(cudaMemset(h->dz_t[l].p, 0, (size_t)cols * h->cap * 2));
  }
  MLP_TRY_C(h->y.alloc((size_t)h->cap * h->out_pad[kLayers - 1]));
  MLP_TRY_C(h->yb.alloc((size_t)h->cap * h->out_pad[kLayers - 1]));
  for (auto* b : {&h->x_mean, &h->x_istd}) MLP_TRY_C(b->alloc(n_in));
  for (auto* b : {&h->t_mean, &h->t_std, &h->t_istd}) MLP_TRY_C(b->alloc(n_out));
  MLP_TRY_C(h->partial.alloc(blocks((long long)h->cap * h->out_pad[kLayers - 1], 256)));
  MLP_TRY_C(h->loss.alloc(1));
  MLP_TRY_C(h->err.alloc(1));
  MLP_TRY_C(cudaMemset(h->err.p, 0, sizeof(unsigned int)));
#undef MLP_TRY_C
  souffle_status s = refresh_bf16(h, 0.0f);
  if (s != SOUFFLE_OK) return cleanup(s);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return cleanup(fail(SOUFFLE_ERR_CUDA, "init"));
  *out = h;
  return SOUFFLE_OK;
}

void* souffle_mlp_stream(const souffle_mlp* h) { return h ? static_cast<void*>(h->stream) : nullptr; }

souffle_status souffle_mlp_destroy(souffle_mlp* h) {
  if (!h) return SOUFFLE_OK;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  cudaStream_t s = h->stream;
  delete h;
  if (s) cudaStreamDestroy(s);
  return SOUFFLE_OK;
}

int64_t souffle_mlp_param_count(const souffle_mlp* h) {
  if (!h) return 0;
  int64_t n = 0;
  for (int l = 0; l < kLayers; l++) n += (int64_t)h->out[l] * h->in[l] + h->out[l];
  return n;
}

souffle_status souffle_mlp_get_params(souffle_mlp* h, float* host_out, int64_t n) {
  if (!h || !host_out || n != souffle_mlp_param_count(h)) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(h->device));
  MLP_TRY(cudaStreamSynchronize(h->stream));
  float* p = host_out;
  for (int l = 0; l < kLayers; l++) {
    MLP_TRY(cudaMemcpy(p, h->w[l].p, sizeof(float) * h->out[l] * h->in[l], cudaMemcpyDeviceToHost));
    p += (size_t)h->out[l] * h->in[l];
    MLP_TRY(cudaMemcpy(p, h->b[l].p, sizeof(float) * h->out[l], cudaMemcpyDeviceToHost));
    p += h->out[l];
  }
  return SOUFFLE_OK;
}

souffle_status souffle_mlp_set_params(souffle_mlp* h, const float* host_in, int64_t n) {
  if (!h || !host_in || n != souffle_mlp_param_count(h)) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(h->device));
  MLP_TRY(cudaStreamSynchronize(h->stream));
  const float* p = host_in;
  for (int l = 0; l < kLayers; l++) {
    MLP_TRY(cudaMemcpy(h->w[l].p, p, sizeof(float) * h->out[l] * h->in[l], cudaMemcpyHostToDevice));
    p += (size_t)h->out[l] * h->in[l];
    MLP_TRY(cudaMemcpy(h->b[l].p, p, sizeof(float) * h->out[l], cudaMemcpyHostToDevice));
    p += h->out[l];
  }
  souffle_status s = refresh_bf16(h, 0.0f);
  if (s != SOUFFLE_OK) return s;
  MLP_TRY(cudaStreamSynchronize(h->stream));
  return SOUFFLE_OK;
}

souffle_status souffle_mlp_forward(souffle_mlp* h, const float* x_dev, int32_t m, float* y_dev) {
  if (!h || !x_dev || !y_dev || m < 1 || m > h->cap) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(h->device));
  souffle_status s = pack_input(h, x_dev, m, false);
  if (s != SOUFFLE_OK) return s;
  const float* y = nullptr;
  int ldy = 0;
  MLP_TRY(souffle::mlp_forward_packed_async(h, m, nullptr, h->err.p, h->stream, &y, &ldy));
  const int L = kLayers - 1;
  k_unpad<<<blocks((long long)m * h->n_out, 256), 256, 0, h->stream>>>(h->y.p, h->out_pad[L], m, h->n_out, y_dev);
  MLP_TRY(cudaGetLastError());
  return check_gemm_err(h);
}

souffle_status souffle_mlp_forward_layered(souffle_mlp* h, const float* x_dev, int32_t m, float* y_dev) {
  if (!h || !x_dev || !y_dev || m < 1 || m > h->cap) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(h->device));
  souffle_status s = pack_input(h, x_dev, m, false);
  if (s == SOUFFLE_OK) s = forward(h, m, false);
  if (s != SOUFFLE_OK) return s;
  const int L = kLayers - 1;
  k_unpad<<<blocks((long long)m * h->n_out, 256), 256, 0, h->stream>>>(h->y.p, h->out_pad[L], m, h->n_out, y_dev);
  MLP_TRY(cudaGetLastError());
  return check_gemm_err(h);
}

souffle_status souffle_mlp_profile_forward(souffle_mlp* h, int32_t m, int32_t iters, int32_t fused, double* us) {
  if (!h || !us || m < 1 || m > h->cap || iters < 1) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  const int L = kLayers - 1;
  if (fused && !mlp_fused_supported(h->n_in, h->width, h->out_pad[L]))
    return fail(SOUFFLE_ERR_BAD_INPUT, "network shape has no fused forward");
  MLP_TRY(cudaSetDevice(h->device));
  cudaEvent_t e0, e1;
  MLP_TRY(cudaEventCreate(&e0));
  MLP_TRY(cudaEventCreate(&e1));
  const __nv_bfloat16* w[4] = {h->wb[0].p, h->wb[1].p, h->wb[2].p, h->wb[3].p};
  const int ldw[4] = {h->in[0], h->in[1], h->in[2], h->in[3]};
  const float* b[4] = {h->b[0].p, h->b[1].p, h->b[2].p, h->b[3].p};
  auto run = [&]() {
    return fused ? mlp_forward_fused(h->act[0].p, h->in_ld[0], m, nullptr, h->n_in, h->width, w, ldw, h->out_pad[L], b, h->y.p,
                                     h->out_pad[L], h->err.p, 1u, h->stream)
                 : forward_on(h, m, false, h->stream, nullptr, h->err.p);
  };
  cudaError_t r = run();  // warm-up
  if (r == cudaSuccess) r = cudaEventRecord(e0, h->stream);
  for (int i = 0; i < iters && r == cudaSuccess; i++) r = run();
  if (r == cudaSuccess) r = cudaEventRecord(e1, h->stream);
  if (r == cudaSuccess) r = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MLP_TRY(r);
  *us = 1e3 * ms / iters;
  return check_gemm_err(h);
}

souffle_status souffle_mlp_gradients(souffle_mlp* h, const float* x_dev, const float* t_dev, int32_t m, float* loss,
                                     float* grad_host) {
  if (!h || !x_dev || !t_dev || !grad_host || m < 1 || m > h->cap) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(h->device));
  souffle_status s = pack_input(h, x_dev, m, true);
  if (s == SOUFFLE_OK) s = forward(h, m, true);
  if (s == SOUFFLE_OK) s = backward(h, t_dev, m);
  if (s != SOUFFLE_OK) return s;
  s = check_gemm_err(h);
  if (s != SOUFFLE_OK) return s;
  float* p = grad_host;
  for (int l = 0; l < kLayers; l++) {
    MLP_TRY(cudaMemcpy(p, h->gw[l].p, sizeof(float) * h->out[l] * h->in[l], cudaMemcpyDeviceToHost));
    p += (size_t)h->out[l] * h->in[l];
    MLP_TRY(cudaMemcpy(p, h->gb[l].p, sizeof(float) * h->out[l], cudaMemcpyDeviceToHost));
    p += h->out[l];
  }
  if (loss) {
    float sq = 0;
    MLP_TRY(cudaMemcpy(&sq, h->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    *loss = sq / ((float)m * (float)h->n_out);
  }
  return SOUFFLE_OK;
}

souffle_status souffle_mlp_train_step(souffle_mlp* h, const float* x_dev, const float* t_dev, int32_t m, float lr,
                                      float* loss) {
  if (!h || !x_dev || !t_dev || m < 1 || m > h->cap || !(lr > 0.0f)) return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(h->device));
  souffle_status s = pack_input(h, x_dev, m, true);
  if (s == SOUFFLE_OK) s = forward(h, m, true);
  if (s == SOUFFLE_OK) s = backward(h, t_dev, m);
  if (s == SOUFFLE_OK) s = refresh_bf16(h, lr);
  if (s != SOUFFLE_OK) return s;
  s = check_gemm_err(h);
  if (s != SOUFFLE_OK) return s;
  if (loss) {
    float sq = 0;
    MLP_TRY(cudaMemcpy(&sq, h->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    *loss = sq / ((float)m * (float)h->n_out);
  }
  return SOUFFLE_OK;
}

souffle_status souffle_gemm_bf16(const float* a_dev, const float* b_dev, int32_t m, int32_t n, int32_t k, float* c_dev,
                                 int32_t device) {
  if (!a_dev || !b_dev || !c_dev || m < 1 || n < 1 || k < 1 || (long long)m * k > (1ll << 28) ||
      (long long)n * k > (1ll << 28))
    return fail(SOUFFLE_ERR_BAD_INPUT, "bad argument");
  MLP_TRY(cudaSetDevice(device));
  const int ldk = round_up(k, 8);
  DevBuf<__nv_bfloat16> a, b;
  DevBuf<unsigned int> err;
  MLP_TRY(a.alloc((size_t)m * ldk));
  MLP_TRY(b.alloc((size_t)n * ldk));
  MLP_TRY(err.alloc(1));
  MLP_TRY(cudaMemset(err.p, 0, sizeof(unsigned int)));
  k_pack_input<<<blocks((long long)m * k, 256), 256>>>(a_dev, m, k, a.p, ldk, nullptr, 0);
  k_pack_input<<<blocks((long long)n * k, 256), 256>>>(b_dev, n, k, b.p, ldk, nullptr, 0);
  MLP_TRY(cudaGetLastError());
  GemmEpi e;
  e.M = m;
  e.N = n;
  e.K = k;
  e.err = err.p;
  e.out_f32 = c_dev;
  e.ldo = n;
  MLP_TRY(gemm_bf16(a.p, ldk, b.p, ldk, e, 0));
  unsigned int flag = 0;
  MLP_TRY(cudaMemcpy(&flag, err.p, sizeof(flag), cudaMemcpyDeviceToHost));
  if (flag) return fail(SOUFFLE_ERR_CUDA, "tensor-core GEMM: a bounded wait ran out");
  return SOUFFLE_OK;
}

}  // extern "C"
