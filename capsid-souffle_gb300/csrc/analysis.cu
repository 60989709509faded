// Post-run trajectory analysis on the GPU (include/souffle_analysis.h): pair correlation, oligomer
// mass spectrum and sub-oligomer sizes of one frame, the per-frame work of analyze_output
// (src/analysis.cpp:117-262).
//
// The reference grows each oligomer by testing every bead of every unassigned subunit against
// every bead of the oligomer (O(S^2 np^2) per frame, src/analysis.cpp:140-178) and the pair
// correlation over all pairs of beads (:117-131).  Here:
//   k_an_prep        FP32 copies of the positions, union-find roots reset, pcf beads listed
//   k_an_spheres     per subunit an anchor bead and the radius of the sphere about it that holds
//                    every bead (minimum image)
//   k_an_candidates  subunit pairs whose spheres come within the contact distance (all pairs, in
//                    FP32 with a margin); every separation rule used here is at least the minimum
//                    image separation, so no contact lies outside these pairs
//   k_an_contacts    one warp per candidate pair (and per subunit, for pairs inside it): every bead
//                    pair tested; a contact joins the two subunits, a contact between two so-type
//                    beads joins the two beads (lock-free union-find, larger root linked under
//                    smaller, so every component ends with its smallest index as root)
//   k_an_pcf         all pairs of pcf beads in 256 x 256 tiles, binned into warp-private shared
//                    histograms
//   k_an_finish/k_an_hist  roots, component sizes, the two size histograms
// Comparisons with the contact distance, the pcf cut-off and the bin edges are made in FP32 with
// an error bound; a pair inside the bound is decided by the FP64 evaluation the reference's
// formula gives (dx^2 + dy^2) + dz^2, correctly rounded square root and division), so counts are
// exact and independent of scheduling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "devbuf.cuh"
#include "souffle_analysis.h"

namespace souffle {
void record_error(const std::string& msg);  // souffle_gpu.cu: text for souffle_gpu_last_error()
}

namespace {

using souffle::DevBuf;

constexpr int kMaxBeadsPerSubunit = 256;
constexpr int kContactWarps = 8;           // warps per CTA in k_an_contacts
constexpr int kTile = 256;                 // tile edge of k_an_candidates and k_an_pcf
constexpr int kUnionIterLimit = 1 << 22;   // bound on retries of one union (never reached in practice)

// Counter slots.
enum { C_NPCF = 0, C_NCAND = 1, C_FP64 = 2, C_FLAGS = 3, C_COUNT = 4 };
enum { F_CAND_OVERFLOW = 1, F_SO_OVERFLOW = 2, F_UNION_LIMIT = 4, F_POS_RANGE = 8 };

struct AnParams {
  double L, half, dg, contact;
  float Lf, halff, inv_dgf, tolz, lo2, hi2, tol_r, tol_bin, sph_margin;
  int N, np, S, bins, pcf_type, so_type, image, cap;
};

__device__ __forceinline__ int type_of(float4 p) { return __float_as_int(p.w); }

// Separation of beads a and b in FP64, the reference's arithmetic: d = pa - pb, the image rule,
// (dx^2 + dy^2) + dz^2, correctly rounded sqrt.  No contraction into FMA.
__device__ __noinline__ double exact_sep(const double* __restrict__ pos, int a, int b, const AnParams P) {
  double d[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double x = __dsub_rn(pos[3 * a + c], pos[3 * b + c]);
    if (P.image == SOUFFLE_IMAGE_REFERENCE) {
      if (x > 0.0) x = __dsub_rn(x, P.L);
      else if (x < 0.0) x = __dadd_rn(x, P.L);
    } else {
      if (x > P.half) x = __dsub_rn(x, P.L);
      else if (x < -P.half) x = __dadd_rn(x, P.L);
    }
    d[c] = x;
  }
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
  return __dsqrt_rn(r2);
}

// FP32 squared separation; `unsure` is set when a coordinate difference is too close to zero for
// FP32 to tell whether the reference rule shifts it.
__device__ __forceinline__ float sep2_f(float4 p, float4 q, const AnParams& P, bool& unsure) {
  const float dx = fabsf(p.x - q.x), dy = fabsf(p.y - q.y), dz = fabsf(p.z - q.z);
  float gx, gy, gz;
  if (P.image == SOUFFLE_IMAGE_REFERENCE) {
    unsure |= (dx <= P.tolz) | (dy <= P.tolz) | (dz <= P.tolz);
    gx = P.Lf - dx;
    gy = P.Lf - dy;
    gz = P.Lf - dz;
  } else {
    gx = dx > P.halff ? P.Lf - dx : dx;
    gy = dy > P.halff ? P.Lf - dy : dy;
    gz = dz > P.halff ? P.Lf - dz : dz;
  }
  return gx * gx + gy * gy + gz * gz;
}

// Minimum-image separation squared in FP32 (sphere tests only).
__device__ __forceinline__ float min_image2_f(float4 p, float4 q, float L, float half) {
  float dx = fabsf(p.x - q.x), dy = fabsf(p.y - q.y), dz = fabsf(p.z - q.z);
  dx = dx > half ? L - dx : dx;
  dy = dy > half ? L - dy : dy;
  dz = dz > half ? L - dz : dz;
  return dx * dx + dy * dy + dz * dz;
}

// Union-find over `parent`, where parent[x] <= x always: roots are linked larger under smaller
// with a compare-and-swap, and path halving only ever points a node at one of its ancestors.
// Loads bypass L1 (__ldcg) so that another SM's links are seen.
__device__ __forceinline__ int uf_find(int* parent, int x) {
  int p = __ldcg(parent + x);
  while (p != x) {
    const int gp = __ldcg(parent + p);
    if (gp != p) __stcg(parent + x, gp);
    x = p;
    p = gp;
  }
  return x;
}

__device__ void uf_union(int* parent, int a, int b, unsigned int* flags) {
  for (int it = 0; it < kUnionIterLimit; it++) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a == b) return;
    if (a > b) {
      const int t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(parent + b, b, a) == b) return;
  }
  atomicOr(flags, F_UNION_LIMIT);
}

__global__ void k_an_prep(const double* __restrict__ pos, const int* __restrict__ types, const AnParams P,
                          float4* __restrict__ posf, int* __restrict__ parent_bead, int* __restrict__ size_bead,
                          int* __restrict__ parent_sub, int* __restrict__ size_sub, int* __restrict__ pcf_idx,
                          unsigned int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.N) {
    const int t = types[i];
    const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    // the FP32 error bounds and the sphere test assume coordinates inside the box (the MD writes
    // them wrapped into [-box/2, box/2]); far outside it, report instead of guessing
    if (!(fabs(x) <= 0.75 * P.L && fabs(y) <= 0.75 * P.L && fabs(z) <= 0.75 * P.L)) atomicOr(cnt + C_FLAGS, F_POS_RANGE);
    posf[i] = make_float4((float)x, (float)y, (float)z, __int_as_float(t));
    parent_bead[i] = i;
    size_bead[i] = 0;
    // warp-aggregated append of the pcf beads (their order does not matter: the histogram is a
    // sum over unordered pairs)
    const bool is_pcf = t == P.pcf_type;
    const unsigned am = __activemask();
    const unsigned m = __ballot_sync(am, is_pcf);
    if (m) {
      const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(cnt + C_NPCF, __popc(m));
      base = __shfl_sync(am, base, leader);
      if (is_pcf) pcf_idx[base + __popc(m & ((1u << lane) - 1))] = i;
    }
  }
  if (i < P.S) {
    parent_sub[i] = i;
    size_sub[i] = 0;
  }
}

// Warp per subunit: anchor = its first bead; radius = largest minimum-image distance from the
// anchor to a bead of the subunit, rounded up.
__global__ void k_an_spheres(const double* __restrict__ pos, const AnParams P, float4* __restrict__ sph) {
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= P.S) return;
  const long a0 = (long)s * P.np;
  const double ax = pos[3 * a0], ay = pos[3 * a0 + 1], az = pos[3 * a0 + 2];
  double r2 = 0;
  for (int b = lane; b < P.np; b += 32) {
    double d[3] = {pos[3 * (a0 + b)] - ax, pos[3 * (a0 + b) + 1] - ay, pos[3 * (a0 + b) + 2] - az};
    for (int c = 0; c < 3; c++) {
      if (d[c] > P.half) d[c] -= P.L;
      else if (d[c] < -P.half) d[c] += P.L;
    }
    r2 = fmax(r2, d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  }
  for (int o = 16; o; o >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xffffffffu, r2, o));
  if (lane == 0) sph[s] = make_float4((float)ax, (float)ay, (float)az, (float)sqrt(r2) * 1.0001f + P.sph_margin);
}

// All subunit pairs i < k in 256 x 256 tiles (grid-stride over tile pairs): a pair whose spheres
// come closer than the contact distance (plus the FP32 margin) is a candidate.
__global__ void __launch_bounds__(kTile) k_an_candidates(const float4* __restrict__ sph, const AnParams P,
                                                         int2* __restrict__ cand, unsigned int* __restrict__ cnt) {
  __shared__ float4 tile[kTile];
  const int T = (P.S + kTile - 1) / kTile;
  for (long t = blockIdx.x; t < (long)T * T; t += gridDim.x) {
    const int ti = (int)(t / T), tk = (int)(t % T);
    if (tk < ti) continue;
    __syncthreads();
    const int kk = tk * kTile + threadIdx.x;
    if (kk < P.S) tile[threadIdx.x] = sph[kk];
    __syncthreads();
    const int i = ti * kTile + threadIdx.x;
    if (i >= P.S) continue;
    const float4 si = sph[i];
    const int kend = min(kTile, P.S - tk * kTile);
    const int kbeg = tk == ti ? threadIdx.x + 1 : 0;
    for (int k = kbeg; k < kend; k++) {
      const float4 sk = tile[k];
      const float reach = si.w + sk.w + P.contact;
      if (min_image2_f(si, sk, P.Lf, P.halff) < reach * reach) {
        const unsigned slot = atomicAdd(cnt + C_NCAND, 1u);
        if (slot < (unsigned)P.cap) cand[slot] = make_int2(i, tk * kTile + k);
        else atomicOr(cnt + C_FLAGS, F_CAND_OVERFLOW);
      }
    }
  }
}

// Warp per work item: items [0, n_cand) are candidate subunit pairs, items [n_cand, n_cand + S)
// are single subunits (pairs of beads inside one subunit, which only matter for sub-oligomers).
__global__ void __launch_bounds__(kContactWarps * 32)
    k_an_contacts(const double* __restrict__ pos, const float4* __restrict__ posf, const int2* __restrict__ cand,
                  const AnParams P, int* parent_sub, int* parent_bead, unsigned int* __restrict__ cnt) {
  __shared__ float4 sb[kContactWarps][kMaxBeadsPerSubunit];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int n_cand = (int)min(__ldcg(cnt + C_NCAND), (unsigned)P.cap);
  const long items = (long)n_cand + P.S;
  unsigned fp64 = 0;
  for (long w = (long)blockIdx.x * kContactWarps + wid; w < items; w += (long)gridDim.x * kContactWarps) {
    int si, sk;
    const bool self = w >= n_cand;
    if (self) {
      si = sk = (int)(w - n_cand);
    } else {
      const int2 c = cand[w];
      si = c.x;
      sk = c.y;
    }
    const int bi = si * P.np, bk = sk * P.np;
    __syncwarp();
    for (int b = lane; b < P.np; b += 32) sb[wid][b] = posf[bk + b];
    __syncwarp();
    // self items only look for so-type contacts; pair items look for any contact until found
    bool joined = self;
    for (int a = 0; a < P.np; a++) {
      const float4 pa = posf[bi + a];
      const bool a_so = type_of(pa) == P.so_type;
      if (joined && !a_so) continue;
      bool hit_any = false;
      for (int b = self ? a + 1 + lane : lane; b < P.np; b += 32) {
        const float4 pb = sb[wid][b];
        const bool pair_so = a_so && type_of(pb) == P.so_type;
        if (joined && !pair_so) continue;
        bool unsure = false;
        const float r2 = sep2_f(pa, pb, P, unsure);
        bool hit;
        if (!unsure && r2 < P.lo2) hit = true;
        else if (!unsure && r2 >= P.hi2) hit = false;
        else {
          hit = exact_sep(pos, bi + a, bk + b, P) < P.contact;
          fp64++;
        }
        if (hit) {
          hit_any = true;
          if (pair_so) uf_union(parent_bead, bi + a, bk + b, cnt + C_FLAGS);
        }
      }
      if (!joined && __any_sync(0xffffffffu, hit_any)) {
        joined = true;
        if (lane == 0) uf_union(parent_sub, si, sk, cnt + C_FLAGS);
      }
    }
  }
  if (fp64) atomicAdd(cnt + C_FP64, fp64);
}

// All pairs of pcf beads, 256 x 256 tiles, warp-private histograms in shared memory.
__global__ void __launch_bounds__(kTile) k_an_pcf(const double* __restrict__ pos, const float4* __restrict__ posf,
                                                  const int* __restrict__ pcf_idx, const AnParams P,
                                                  unsigned long long* __restrict__ gr, unsigned int* __restrict__ cnt) {
  extern __shared__ unsigned int hist[];  // copies x bins
  __shared__ float4 tile[kTile];
  __shared__ int tidx[kTile];
  const int copies = P.bins <= 512 ? kTile / 32 : 1;
  unsigned int* h = hist + (copies > 1 ? (threadIdx.x >> 5) * P.bins : 0);
  for (int k = threadIdx.x; k < copies * P.bins; k += blockDim.x) hist[k] = 0;
  const int n = (int)__ldcg(cnt + C_NPCF);
  const int T = (n + kTile - 1) / kTile;
  unsigned fp64 = 0;
  for (long t = blockIdx.x; t < (long)T * T; t += gridDim.x) {
    const int ti = (int)(t / T), tk = (int)(t % T);
    if (tk < ti) continue;
    __syncthreads();
    const int kk = tk * kTile + threadIdx.x;
    if (kk < n) {
      tidx[threadIdx.x] = pcf_idx[kk];
      tile[threadIdx.x] = posf[tidx[threadIdx.x]];
    }
    __syncthreads();
    const int ii = ti * kTile + threadIdx.x;
    if (ii >= n) continue;
    const int gi = pcf_idx[ii];
    const float4 pi = posf[gi];
    const int kend = min(kTile, n - tk * kTile);
    for (int k = tk == ti ? threadIdx.x + 1 : 0; k < kend; k++) {
      bool unsure = false;
      const float r = sqrtf(sep2_f(pi, tile[k], P, unsure));
      int bin = -1;
      if (!unsure && r < P.halff - P.tol_r) {
        const float x = r * P.inv_dgf;
        const float f = floorf(x);
        if (x - f >= P.tol_bin && x - f <= 1.0f - P.tol_bin) bin = (int)f;
        else unsure = true;
      } else if (!unsure && r < P.halff + P.tol_r) {
        unsure = true;
      }
      if (unsure) {
        fp64++;
        const double rd = exact_sep(pos, gi, tidx[k], P);
        if (rd < P.half) {
          const double b = floor(__ddiv_rn(rd, P.dg));
          bin = b < (double)P.bins ? (int)b : -1;  // r/dg rounding up to bins: past the reference's histogram
        }
      }
      if (bin >= 0) atomicAdd(h + min(bin, P.bins - 1), 1u);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P.bins; k += blockDim.x) {
    unsigned long long s = 0;
    for (int c = 0; c < copies; c++) s += hist[c * P.bins + k];
    if (s) atomicAdd(gr + k, s);
  }
  if (fp64) atomicAdd(cnt + C_FP64, fp64);
}

// Roots and component sizes.
__global__ void k_an_finish(const float4* __restrict__ posf, const AnParams P, int* parent_sub, int* parent_bead,
                            int* __restrict__ size_sub, int* __restrict__ size_bead, int* __restrict__ labels) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.S) {
    const int r = uf_find(parent_sub, i);
    labels[i] = r;
    atomicAdd(size_sub + r, 1);
  }
  if (i < P.N && type_of(posf[i]) == P.so_type) atomicAdd(size_bead + uf_find(parent_bead, i), 1);
}

// Size histograms: oligomers of k + 1 subunits; sub-oligomers in bins of three beads.
__global__ void k_an_hist(const float4* __restrict__ posf, const AnParams P, const int* __restrict__ labels,
                          const int* __restrict__ size_sub, const int* __restrict__ parent_bead,
                          const int* __restrict__ size_bead, unsigned long long* __restrict__ olig,
                          unsigned long long* __restrict__ so, unsigned int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.S && labels[i] == i) atomicAdd(olig + size_sub[i] - 1, 1ull);
  if (i < P.N && type_of(posf[i]) == P.so_type && parent_bead[i] == i) {
    const int bin = (size_bead[i] - 1) / 3;
    if (bin < 2 * P.S) atomicAdd(so + bin, 1ull);
    else atomicOr(cnt + C_FLAGS, F_SO_OVERFLOW);
  }
}

int g_sm_count(int dev) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

}  // namespace

struct souffle_analysis {
  int dev = 0;
  int sms = 1;
  cudaStream_t st = nullptr;
  AnParams P{};
  DevBuf<double> pos;
  DevBuf<int> types;
  DevBuf<float4> posf, sph;
  DevBuf<int> pcf_idx, parent_sub, parent_bead, size_sub, size_bead, labels;
  DevBuf<int2> cand;
  DevBuf<unsigned int> cnt;
  DevBuf<unsigned long long> gr, olig, so;
  unsigned int* cnt_host = nullptr;  // pinned copy of the counters of the last enqueued frame
  bool have_types = false;
};

namespace {

souffle_status fail(souffle_status s, const std::string& msg) {
  souffle::record_error(msg);
  return s;
}

souffle_status cuda_fail(cudaError_t e, const char* what) {
  return fail(SOUFFLE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define AN_CHECK(call)                                    \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

souffle_status grow_candidates(souffle_analysis* h, long need) {
  const long cap = std::max<long>(2 * (long)h->P.cap, need + need / 4 + 1024);
  if (cap > (1L << 30)) return fail(SOUFFLE_ERR_NL_OVERFLOW, "analysis: more than 2^30 candidate subunit pairs");
  AN_CHECK(h->cand.alloc(cap));
  h->P.cap = (int)cap;
  return SOUFFLE_OK;
}

souffle_status enqueue(souffle_analysis* h, const double* pos, const int* types, unsigned long long* gr,
                       unsigned long long* olig, unsigned long long* so, int* labels) {
  const AnParams& P = h->P;
  cudaStream_t st = h->st;
  AN_CHECK(cudaMemsetAsync(h->cnt.p, 0, sizeof(unsigned int) * C_COUNT, st));
  AN_CHECK(cudaMemsetAsync(gr, 0, sizeof(unsigned long long) * P.bins, st));
  AN_CHECK(cudaMemsetAsync(olig, 0, sizeof(unsigned long long) * P.S, st));
  AN_CHECK(cudaMemsetAsync(so, 0, sizeof(unsigned long long) * 2 * P.S, st));
  const int nmax = std::max(P.N, P.S);
  k_an_prep<<<(nmax + 255) / 256, 256, 0, st>>>(pos, types, P, h->posf.p, h->parent_bead.p, h->size_bead.p,
                                                 h->parent_sub.p, h->size_sub.p, h->pcf_idx.p, h->cnt.p);
  k_an_spheres<<<(P.S + 7) / 8, 256, 0, st>>>(pos, P, h->sph.p);
  const long T = (P.S + kTile - 1) / kTile;
  const int gcand = (int)std::min<long>(T * T, 4L * h->sms);
  k_an_candidates<<<gcand, kTile, 0, st>>>(h->sph.p, P, h->cand.p, h->cnt.p);
  const long items_max = (long)P.cap + P.S;
  const int gcon = (int)std::min<long>((items_max + kContactWarps - 1) / kContactWarps, 8L * h->sms);
  k_an_contacts<<<gcon, kContactWarps * 32, 0, st>>>(pos, h->posf.p, h->cand.p, P, h->parent_sub.p,
                                                     h->parent_bead.p, h->cnt.p);
  const long Tp = (P.N + kTile - 1) / kTile;
  const int gpcf = (int)std::min<long>(Tp * Tp, 4L * h->sms);
  const int copies = P.bins <= 512 ? kTile / 32 : 1;
  k_an_pcf<<<gpcf, kTile, sizeof(unsigned int) * copies * P.bins, st>>>(pos, h->posf.p, h->pcf_idx.p, P, gr,
                                                                        h->cnt.p);
  k_an_finish<<<(nmax + 255) / 256, 256, 0, st>>>(h->posf.p, P, h->parent_sub.p, h->parent_bead.p,
                                                   h->size_sub.p, h->size_bead.p, labels);
  k_an_hist<<<(nmax + 255) / 256, 256, 0, st>>>(h->posf.p, P, labels, h->size_sub.p, h->parent_bead.p,
                                                 h->size_bead.p, olig, so, h->cnt.p);
  AN_CHECK(cudaGetLastError());
  AN_CHECK(cudaMemcpyAsync(h->cnt_host, h->cnt.p, sizeof(unsigned int) * C_COUNT, cudaMemcpyDeviceToHost, st));
  return SOUFFLE_OK;
}

// Status of the last enqueued frame (call after the stream has drained).
souffle_status frame_status(souffle_analysis* h) {
  const unsigned flags = h->cnt_host[C_FLAGS];
  if (flags & F_UNION_LIMIT) return fail(SOUFFLE_ERR_CUDA, "analysis: union-find retry limit reached");
  if (flags & F_POS_RANGE)
    return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: a coordinate lies more than 0.75 box from the origin");
  if (flags & F_SO_OVERFLOW)
    return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: a sub-oligomer has more than 6 x n_subunits beads");
  if (flags & F_CAND_OVERFLOW) return SOUFFLE_ERR_NL_OVERFLOW;
  return SOUFFLE_OK;
}

}  // namespace

extern "C" {

void souffle_analysis_default_options(souffle_analysis_options* opt) {
  if (!opt) return;
  opt->image = SOUFFLE_IMAGE_REFERENCE;
  opt->pcf_type = 5;
  opt->pcf_bins = 100;
  opt->so_type = 0;
  opt->contact = 2.0;
}

souffle_status souffle_analysis_create(int64_t n_beads, int32_t beads_per_subunit, double box,
                                       const souffle_analysis_options* opt, int32_t device,
                                       souffle_analysis** out) {
  if (!out) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: out is NULL");
  *out = nullptr;
  souffle_analysis_options o;
  souffle_analysis_default_options(&o);
  if (opt) o = *opt;
  if (beads_per_subunit < 1 || beads_per_subunit > kMaxBeadsPerSubunit || n_beads < beads_per_subunit ||
      n_beads % beads_per_subunit != 0 || n_beads > (1L << 30))
    return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: n_beads must be a positive multiple of beads_per_subunit "
                                       "(1..256), at most 2^30");
  if (!(box > 0) || !std::isfinite(box)) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: box must be positive");
  if (o.pcf_bins < 1 || o.pcf_bins > 4096) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: pcf_bins must be 1..4096");
  if (!(o.contact > 0) || !(o.contact < box / 2))
    return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: contact must be in (0, box / 2)");
  if (o.image != SOUFFLE_IMAGE_REFERENCE && o.image != SOUFFLE_IMAGE_MINIMUM)
    return fail(SOUFFLE_ERR_BAD_INPUT, "analysis: image must be SOUFFLE_IMAGE_REFERENCE or SOUFFLE_IMAGE_MINIMUM");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return fail(SOUFFLE_ERR_NO_DEVICE, "analysis: no such CUDA device");
  AN_CHECK(cudaSetDevice(device));
  auto* h = new souffle_analysis();
  h->dev = device;
  h->sms = g_sm_count(device);
  AnParams& P = h->P;
  P.N = (int)n_beads;
  P.np = beads_per_subunit;
  P.S = (int)(n_beads / beads_per_subunit);
  P.bins = o.pcf_bins;
  P.pcf_type = o.pcf_type;
  P.so_type = o.so_type;
  P.image = o.image;
  P.L = box;
  P.half = box / 2;
  P.dg = box / (2.0 * o.pcf_bins);
  P.contact = o.contact;
  P.Lf = (float)box;
  P.halff = (float)(box / 2);
  P.inv_dgf = (float)(1.0 / P.dg);
  // FP32 error bounds.  Each coordinate difference, and box - |difference|, carries at most
  // ~4 * 2^-24 * box of rounding (coordinates within about half a box of the origin); the
  // tolerances below are several times that, plus relative rounding of the squares, sums, square
  // root and the bin scaling.
  const double tol = 1e-6 * box;
  P.tolz = (float)(2 * tol);
  P.tol_r = (float)(4 * tol + 4e-6 * (box / 2));
  const double c = o.contact, tc = 4 * tol + 4e-6 * c;
  P.lo2 = (float)((c - tc) * (c - tc) * (1 - 4e-6));
  P.hi2 = (float)((c + tc) * (c + tc) * (1 + 4e-6));
  P.tol_bin = (float)(P.tol_r / P.dg + 4e-6 * (o.pcf_bins + 1));
  P.sph_margin = (float)(8 * tol + 1e-4);
  P.cap = std::max(4096, 32 * P.S);
  cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  const size_t N = (size_t)P.N, S = (size_t)P.S;
  if (e == cudaSuccess) e = h->pos.alloc(3 * N);
  if (e == cudaSuccess) e = h->types.alloc(N);
  if (e == cudaSuccess) e = h->posf.alloc(N);
  if (e == cudaSuccess) e = h->sph.alloc(S);
  if (e == cudaSuccess) e = h->pcf_idx.alloc(N);
  if (e == cudaSuccess) e = h->parent_sub.alloc(S);
  if (e == cudaSuccess) e = h->parent_bead.alloc(N);
  if (e == cudaSuccess) e = h->size_sub.alloc(S);
  if (e == cudaSuccess) e = h->size_bead.alloc(N);
  if (e == cudaSuccess) e = h->labels.alloc(S);
  if (e == cudaSuccess) e = h->cand.alloc(P.cap);
  if (e == cudaSuccess) e = h->cnt.alloc(C_COUNT);
  if (e == cudaSuccess) e = h->gr.alloc(P.bins);
  if (e == cudaSuccess) e = h->olig.alloc(S);
  if (e == cudaSuccess) e = h->so.alloc(2 * S);
  if (e == cudaSuccess) e = cudaMallocHost(&h->cnt_host, sizeof(unsigned int) * C_COUNT);
  if (e != cudaSuccess) {
    souffle_analysis_destroy(h);
    return cuda_fail(e, "analysis: allocation");
  }
  *out = h;
  return SOUFFLE_OK;
}

souffle_status souffle_analysis_destroy(souffle_analysis* h) {
  if (!h) return SOUFFLE_OK;
  cudaSetDevice(h->dev);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->cnt_host) cudaFreeHost(h->cnt_host);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return SOUFFLE_OK;
}

void* souffle_analysis_stream(souffle_analysis* h) { return h ? (void*)h->st : nullptr; }

souffle_status souffle_analysis_enqueue(souffle_analysis* h, const double* pos_dev, const int32_t* types_dev,
                                        int64_t* pcf_dev, int64_t* oligomers_dev, int64_t* so_bins_dev,
                                        int32_t* labels_dev) {
  if (!h || !pos_dev || !types_dev || !pcf_dev || !oligomers_dev || !so_bins_dev)
    return fail(SOUFFLE_ERR_BAD_INPUT, "analysis_enqueue: NULL argument");
  AN_CHECK(cudaSetDevice(h->dev));
  return enqueue(h, pos_dev, types_dev, reinterpret_cast<unsigned long long*>(pcf_dev),
                 reinterpret_cast<unsigned long long*>(oligomers_dev),
                 reinterpret_cast<unsigned long long*>(so_bins_dev), labels_dev ? labels_dev : h->labels.p);
}

souffle_status souffle_analysis_synchronize(souffle_analysis* h) {
  if (!h) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis_synchronize: NULL handle");
  AN_CHECK(cudaSetDevice(h->dev));
  AN_CHECK(cudaStreamSynchronize(h->st));
  const souffle_status s = frame_status(h);
  if (s == SOUFFLE_ERR_NL_OVERFLOW) {
    const souffle_status g = grow_candidates(h, h->cnt_host[C_NCAND]);
    if (g != SOUFFLE_OK) return g;
    return fail(SOUFFLE_ERR_NL_OVERFLOW, "analysis: candidate list overflowed; capacity grown, run the frame again");
  }
  return s;
}

souffle_status souffle_analysis_frames(souffle_analysis* h, int64_t n_frames, const double* pos,
                                       const int32_t* types, int64_t* pcf, int64_t* oligomers,
                                       int64_t* so_bins, int32_t* labels) {
  if (!h || n_frames < 0 || (n_frames > 0 && !pos)) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis_frames: bad argument");
  if (!types && !h->have_types) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis_frames: the first call needs types");
  AN_CHECK(cudaSetDevice(h->dev));
  const AnParams& P = h->P;
  const size_t N = (size_t)P.N, S = (size_t)P.S;
  for (int64_t f = 0; f < n_frames; f++) {
    AN_CHECK(cudaMemcpyAsync(h->pos.p, pos + 3 * N * f, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, h->st));
    if (types) {
      AN_CHECK(cudaMemcpyAsync(h->types.p, types + N * f, sizeof(int) * N, cudaMemcpyHostToDevice, h->st));
      h->have_types = true;
    }
    for (int attempt = 0;; attempt++) {
      souffle_status s = enqueue(h, h->pos.p, h->types.p, h->gr.p, h->olig.p, h->so.p, h->labels.p);
      if (s != SOUFFLE_OK) return s;
      AN_CHECK(cudaStreamSynchronize(h->st));
      s = frame_status(h);
      if (s == SOUFFLE_OK) break;
      if (s != SOUFFLE_ERR_NL_OVERFLOW || attempt > 8) return s;
      s = grow_candidates(h, h->cnt_host[C_NCAND]);
      if (s != SOUFFLE_OK) return s;
    }
    if (pcf) AN_CHECK(cudaMemcpyAsync(pcf + P.bins * f, h->gr.p, sizeof(int64_t) * P.bins, cudaMemcpyDeviceToHost, h->st));
    if (oligomers)
      AN_CHECK(cudaMemcpyAsync(oligomers + S * f, h->olig.p, sizeof(int64_t) * S, cudaMemcpyDeviceToHost, h->st));
    if (so_bins)
      AN_CHECK(cudaMemcpyAsync(so_bins + 2 * S * f, h->so.p, sizeof(int64_t) * 2 * S, cudaMemcpyDeviceToHost, h->st));
    if (labels)
      AN_CHECK(cudaMemcpyAsync(labels + S * f, h->labels.p, sizeof(int32_t) * S, cudaMemcpyDeviceToHost, h->st));
  }
  AN_CHECK(cudaStreamSynchronize(h->st));
  return SOUFFLE_OK;
}

souffle_status souffle_analysis_last_counts(souffle_analysis* h, int64_t* candidate_pairs, int64_t* fp64_pairs) {
  if (!h) return fail(SOUFFLE_ERR_BAD_INPUT, "analysis_last_counts: NULL handle");
  AN_CHECK(cudaSetDevice(h->dev));
  AN_CHECK(cudaStreamSynchronize(h->st));
  if (candidate_pairs) *candidate_pairs = h->cnt_host[C_NCAND];
  if (fp64_pairs) *fp64_pairs = h->cnt_host[C_FP64];
  return SOUFFLE_OK;
}

}  // extern "C"
