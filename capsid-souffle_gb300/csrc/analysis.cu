// Post-run trajectory analysis on the GPU (include/souffle_analysis.h): pair correlation, oligomer
// mass spectrum and sub-oligomer sizes of one frame, the per-frame work of analyze_output
// (src/analysis.cpp:117-262).
//
// The reference grows each oligomer by testing every bead of every unassigned subunit against
// every bead of the oligomer (O(S^2 np^2) per frame, src/analysis.cpp:140-178) and the pair
// correlation over all pairs of beads (:117-131).  Here:
//   k_an_prep        warp per subunit: FP32 copies of the positions, union-find roots reset, the
//                    subunit's bounding sphere about its first bead (minimum image), pcf beads
//                    listed, the output histograms cleared
//   k_an_candidates  subunit pairs whose spheres come within the contact distance (all pairs, a
//                    warp per folded pair of rows, FP32 with a margin); every separation rule used
//                    here is at least the minimum image separation, so no contact lies outside
//                    these pairs
//   k_an_contacts    one warp per candidate pair (and per subunit, for pairs inside it), both
//                    subunits staged in shared memory, each side cut to the beads within reach of
//                    the other's sphere: bead pairs 32 at a time until a contact joins the
//                    subunits, then the so-type pairs, each contact joining two beads (lock-free
//                    union-find, larger root linked under smaller, so every component ends with
//                    its smallest index as root)
//   k_an_pcf         all pairs of pcf beads in 128 x 128 tiles of the upper triangle, rejected
//                    on the squared separation first, binned into warp-private shared histograms
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
constexpr int kCandWarps = 8;              // warps per CTA in k_an_candidates (two rows each)
constexpr int kCandBuf = 2048;             // candidate hits gathered per CTA in shared memory
constexpr int kCandSeg = 256;              // values of k per block in k_an_candidates
constexpr int kPcfTile = 128;              // tile edge of k_an_pcf
constexpr int kPrivBins = 128;             // k_an_pcf: per-thread 16-bit histograms up to this many bins
constexpr int kPrivFlushTiles = 500;       // ... flushed after this many tiles (500 x 128 < 65536)
constexpr int kHistLocal = 256;            // k_an_hist: size bins counted in shared memory first
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
template <int IMAGE>
__device__ __forceinline__ float sep2_f_t(float4 p, float4 q, const AnParams& P, bool& unsure) {
  const float dx = fabsf(p.x - q.x), dy = fabsf(p.y - q.y), dz = fabsf(p.z - q.z);
  float gx, gy, gz;
  if (IMAGE == SOUFFLE_IMAGE_REFERENCE) {
    unsure |= fminf(fminf(dx, dy), dz) <= P.tolz;
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

__device__ __forceinline__ float sep2_f(float4 p, float4 q, const AnParams& P, bool& unsure) {
  return P.image == SOUFFLE_IMAGE_REFERENCE ? sep2_f_t<SOUFFLE_IMAGE_REFERENCE>(p, q, P, unsure)
                                            : sep2_f_t<SOUFFLE_IMAGE_MINIMUM>(p, q, P, unsure);
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

// Warp per subunit: FP32 copies of the positions, union-find roots reset, the subunit's bounding
// sphere (anchor = its first bead, radius = largest minimum-image distance from the anchor to a
// bead of the subunit, FP32 plus a margin that covers the FP32 rounding), pcf beads appended to
// their list.
__global__ void k_an_prep(const double* __restrict__ pos, const int* __restrict__ types, const AnParams P,
                          float4* __restrict__ posf, float4* __restrict__ sph, int* __restrict__ parent_bead,
                          int* __restrict__ size_bead, int* __restrict__ parent_sub, int* __restrict__ size_sub,
                          int* __restrict__ pcf_idx, unsigned long long* __restrict__ gr,
                          unsigned long long* __restrict__ olig, unsigned long long* __restrict__ so,
                          unsigned int* __restrict__ cnt) {
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= P.S) return;
  // the frame's output histograms start at zero (every later kernel runs after this one)
  if (lane == 0) {
    olig[s] = 0;
    so[2 * s] = 0;
    so[2 * s + 1] = 0;
  }
  for (int k = s + lane * P.S; k < P.bins; k += 32 * P.S) gr[k] = 0;
  const int b0 = s * P.np;
  float4 anchor = make_float4(0.f, 0.f, 0.f, 0.f);
  float r2max = 0.f;
  bool out_of_box = false;
  for (int base = 0; base < P.np; base += 32) {
    const int l = base + lane, i = b0 + l;
    const bool valid = l < P.np;
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    int t = 0;
    if (valid) {
      t = types[i];
      const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
      // the FP32 error bounds and the sphere test assume coordinates inside the box (the MD
      // writes them wrapped into [-box/2, box/2]); far outside it, report instead of guessing
      out_of_box |= !(fabs(x) <= 0.75 * P.L && fabs(y) <= 0.75 * P.L && fabs(z) <= 0.75 * P.L);
      f = make_float4((float)x, (float)y, (float)z, __int_as_float(t));
      posf[i] = f;
      parent_bead[i] = i;
      size_bead[i] = 0;
    }
    if (base == 0) {
      anchor.x = __shfl_sync(0xffffffffu, f.x, 0);
      anchor.y = __shfl_sync(0xffffffffu, f.y, 0);
      anchor.z = __shfl_sync(0xffffffffu, f.z, 0);
    }
    if (valid) r2max = fmaxf(r2max, min_image2_f(f, anchor, P.Lf, P.halff));
    // warp-aggregated append of the pcf beads (their order does not matter: the histogram is a
    // sum over unordered pairs)
    const bool is_pcf = valid && t == P.pcf_type;
    const unsigned m = __ballot_sync(0xffffffffu, is_pcf);
    if (m) {
      unsigned slot = 0;
      if (lane == 0) slot = atomicAdd(cnt + C_NPCF, __popc(m));
      slot = __shfl_sync(0xffffffffu, slot, 0);
      if (is_pcf) pcf_idx[slot + __popc(m & ((1u << lane) - 1))] = i;
    }
  }
  for (int o = 16; o; o >>= 1) r2max = fmaxf(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
  if (__any_sync(0xffffffffu, out_of_box) && lane == 0) atomicOr(cnt + C_FLAGS, F_POS_RANGE);
  if (lane == 0) {
    sph[s] = make_float4(anchor.x, anchor.y, anchor.z, sqrtf(r2max) * 1.0001f + P.sph_margin);
    parent_sub[s] = s;
    size_sub[s] = 0;
  }
}

// Subunit pairs i < k whose spheres come closer than the contact distance (plus the FP32 margin):
// the candidates.  Warp per pair of rows, folded (warp w takes rows w and S-1-w) so every warp has
// the same share of pairs; blockIdx.y selects a segment of kCandSeg values of k, staged in shared
// memory.  Hits are gathered in shared memory and reserved in the global list with one atomic per
// block.
__global__ void __launch_bounds__(kCandWarps * 32) k_an_candidates(const float4* __restrict__ sph, const AnParams P,
                                                                   int2* __restrict__ cand,
                                                                   unsigned int* __restrict__ cnt) {
  __shared__ float4 seg[kCandSeg];
  __shared__ int2 hits[kCandBuf];
  __shared__ unsigned n_hits, base;
  const int lane = threadIdx.x & 31;
  const int w = blockIdx.x * kCandWarps + (threadIdx.x >> 5);
  const int c0 = blockIdx.y * kCandSeg, c1 = min(P.S, c0 + kCandSeg);
  // rows of this block lie in [first, S - first); a segment at or below its smallest row has nothing
  const int first = blockIdx.x * kCandWarps;
  if (c1 <= first + 1) return;
  const bool active = w < (P.S + 1) / 2;  // warps past the fold have no rows
  const int row0 = w, row1 = P.S - 1 - w;
  const bool two = active && row1 > row0;
  if (threadIdx.x == 0) n_hits = 0;
  for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) seg[k - c0] = sph[k];
  __syncthreads();
  for (int r = 0; r < 2; r++) {
    if (!(r == 0 ? active : two)) continue;
    const int i = r == 0 ? row0 : row1;
    const float4 si = sph[i];
    for (int kb = max(c0, i + 1); kb < c1; kb += 128) {
      // four independent tests per lane, then the (rare) hits
      bool hit[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int k = kb + lane + 32 * j;
        hit[j] = false;
        if (k < c1) {
          const float4 sk = seg[k - c0];
          const float reach = si.w + sk.w + P.contact;
          hit[j] = min_image2_f(si, sk, P.Lf, P.halff) < reach * reach;
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        if (!hit[j]) continue;
        const int k = kb + lane + 32 * j;
        const unsigned slot = atomicAdd(&n_hits, 1u);
        if (slot < kCandBuf) {
          hits[slot] = make_int2(i, k);
        } else {  // a very dense block: straight to the global list
          const unsigned g = atomicAdd(cnt + C_NCAND, 1u);
          if (g < (unsigned)P.cap) cand[g] = make_int2(i, k);
          else atomicOr(cnt + C_FLAGS, F_CAND_OVERFLOW);
        }
      }
    }
  }
  __syncthreads();
  const unsigned nh = min(n_hits, (unsigned)kCandBuf);
  if (threadIdx.x == 0 && nh) base = atomicAdd(cnt + C_NCAND, nh);
  __syncthreads();
  for (unsigned h = threadIdx.x; h < nh; h += blockDim.x) {
    if (base + h < (unsigned)P.cap) cand[base + h] = hits[h];
    else atomicOr(cnt + C_FLAGS, F_CAND_OVERFLOW);
  }
}

// Local indices of the beads of a staged subunit that satisfy `keep`, ascending, into list;
// returns their number.  Whole warp.
template <class Keep>
__device__ __forceinline__ int warp_select(const float4* beads, int np, Keep keep, unsigned char* list) {
  const int lane = threadIdx.x & 31;
  int n = 0;
  for (int base = 0; base < np; base += 32) {
    const int l = base + lane;
    const bool k = l < np && keep(beads[l]);
    const unsigned m = __ballot_sync(0xffffffffu, k);
    if (k) list[n + __popc(m & ((1u << lane) - 1))] = (unsigned char)l;
    n += __popc(m);
  }
  __syncwarp();
  return n;
}

// Contact of bead a (global index ga) and bead b (global gb) from their FP32 copies; decided in
// FP64 where FP32 cannot tell.
__device__ __forceinline__ bool contact_test(const float4 pa, const float4 pb, const double* __restrict__ pos, int ga,
                                             int gb, const AnParams& P, unsigned& fp64) {
  bool unsure = false;
  const float r2 = sep2_f(pa, pb, P, unsure);
  if (!unsure && r2 < P.lo2) return true;
  if (!unsure && r2 >= P.hi2) return false;
  fp64++;
  return exact_sep(pos, ga, gb, P) < P.contact;
}

// Warp per work item: items [0, n_cand) are candidate subunit pairs, items [n_cand, n_cand + S)
// are single subunits (pairs of beads inside one subunit, which only matter for sub-oligomers).
// Both subunits are staged in shared memory.  For a pair item only beads within reach of the other
// subunit's sphere can touch it (every separation rule here is at least the minimum image), so
// each side is cut to those beads first; their pairs are scanned 32 at a time until a contact
// joins the subunits, then the so-type pairs among them are tested, each contact joining two
// beads.
__global__ void __launch_bounds__(kContactWarps * 32, 5)
    k_an_contacts(const double* __restrict__ pos, const float4* __restrict__ posf, const float4* __restrict__ sph,
                  const int2* __restrict__ cand, const AnParams P, int* parent_sub, int* parent_bead,
                  unsigned int* __restrict__ cnt) {
  extern __shared__ float4 stage[];  // [kContactWarps][2][np]
  __shared__ unsigned char sel[kContactWarps][4][kMaxBeadsPerSubunit];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, np = P.np;
  float4* A = stage + (size_t)wid * 2 * np;
  float4* B = A + np;
  unsigned char* la = sel[wid][0];
  unsigned char* lb = sel[wid][1];
  unsigned char* sa = sel[wid][2];
  unsigned char* sb = sel[wid][3];
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
    const int bi = si * np, bk = sk * np;
    __syncwarp();
    for (int b = lane; b < np; b += 32) {
      A[b] = posf[bi + b];
      if (!self) B[b] = posf[bk + b];
    }
    __syncwarp();
    if (self) {
      const int na = warp_select(A, np, [&](float4 p) { return type_of(p) == P.so_type; }, sa);
      for (int t = lane; t < na * na; t += 32) {
        const int x = sa[t / na], y = sa[t % na];
        if (y <= x) continue;
        if (contact_test(A[x], A[y], pos, bi + x, bi + y, P, fp64)) uf_union(parent_bead, bi + x, bi + y, cnt + C_FLAGS);
      }
      continue;
    }
    // beads of each side within reach of the other side's sphere
    const float4 ci = sph[si], ck = sph[sk];
    const float ri = ci.w + P.contact, rk = ck.w + P.contact;
    const int na = warp_select(A, np, [&](float4 p) { return min_image2_f(p, ck, P.Lf, P.halff) < rk * rk; }, la);
    const int nb = warp_select(B, np, [&](float4 p) { return min_image2_f(p, ci, P.Lf, P.halff) < ri * ri; }, lb);
    const int nab = na * nb;
    bool joined = false;
    if (nab > 0) {
      int x = lane / nb, y = lane % nb;  // pair t = x * nb + y, tracked as t advances by 32
      const int sx = 32 / nb, sy = 32 % nb;
      for (int base = 0; base < nab && !joined; base += 32) {
        bool hit = false;
        if (base + lane < nab) {
          const int a = la[x], b = lb[y];
          hit = contact_test(A[a], B[b], pos, bi + a, bk + b, P, fp64);
        }
        joined = __any_sync(0xffffffffu, hit);
        x += sx;
        y += sy;
        if (y >= nb) {
          y -= nb;
          x++;
        }
      }
    }
    if (!joined) continue;  // no contact: no so-type contact either
    if (lane == 0) uf_union(parent_sub, si, sk, cnt + C_FLAGS);
    const int ma = warp_select(A, np, [&](float4 p) {
      return type_of(p) == P.so_type && min_image2_f(p, ck, P.Lf, P.halff) < rk * rk; }, sa);
    const int mb = warp_select(B, np, [&](float4 p) {
      return type_of(p) == P.so_type && min_image2_f(p, ci, P.Lf, P.halff) < ri * ri; }, sb);
    for (int t = lane; t < ma * mb; t += 32) {
      const int a = sa[t / mb], b = sb[t % mb];
      if (contact_test(A[a], B[b], pos, bi + a, bk + b, P, fp64)) uf_union(parent_bead, bi + a, bk + b, cnt + C_FLAGS);
    }
  }
  if (fp64) atomicAdd(cnt + C_FP64, fp64);
}

// All pairs of pcf beads, kPcfTile x kPcfTile tiles over the upper triangle (grid-stride).  Pairs
// past the cut-off are rejected on the squared separation before any square root.  With at most
// kPrivBins bins every thread counts into its own 16-bit histogram column in shared memory (no
// atomics, no bank conflicts), flushed to the global histogram before a count could wrap; with
// more bins, warp-private 32-bit histograms with shared atomics.
template <int IMAGE>
__global__ void __launch_bounds__(kPcfTile) k_an_pcf(const double* __restrict__ pos, const float4* __restrict__ posf,
                                                     const int* __restrict__ pcf_idx, const AnParams P,
                                                     unsigned long long* __restrict__ gr, unsigned int* __restrict__ cnt) {
  extern __shared__ unsigned int hist[];
  __shared__ float4 tile[kPcfTile];
  __shared__ int tidx[kPcfTile];
  const bool priv = IMAGE == SOUFFLE_IMAGE_MINIMUM && P.bins <= kPrivBins;
  unsigned short* ph = reinterpret_cast<unsigned short*>(hist);  // [bins][kPcfTile] when priv
  const int copies = priv ? 0 : (P.bins <= 512 ? kPcfTile / 32 : 1);
  unsigned int* h = hist + (copies > 1 ? (threadIdx.x >> 5) * P.bins : 0);
  const int words = priv ? P.bins * kPcfTile / 2 : copies * P.bins;
  for (int k = threadIdx.x; k < words; k += blockDim.x) hist[k] = 0;
  // adds the shared counts to the global histogram and clears them (whole block)
  auto flush = [&]() {
    __syncthreads();
    if (priv) {  // warp per bin, lanes along the bin's row (conflict-free)
      const int lane = threadIdx.x & 31;
      for (int k = threadIdx.x >> 5; k < P.bins; k += kPcfTile / 32) {
        unsigned s = 0;
        for (int c = lane; c < kPcfTile; c += 32) {
          s += ph[k * kPcfTile + c];
          ph[k * kPcfTile + c] = 0;
        }
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s) atomicAdd(gr + k, (unsigned long long)s);
      }
    } else {
      for (int k = threadIdx.x; k < P.bins; k += blockDim.x) {
        unsigned long long s = 0;
        for (int c = 0; c < copies; c++) {
          s += hist[c * P.bins + k];
          hist[c * P.bins + k] = 0;
        }
        if (s) atomicAdd(gr + k, s);
      }
    }
  };
  const int n = (int)__ldcg(cnt + C_NPCF);
  const long T = (n + kPcfTile - 1) / kPcfTile;
  const long n_tiles = T * (T + 1) / 2;
  const float far2 = (P.halff + P.tol_r) * (P.halff + P.tol_r);
  unsigned fp64 = 0;
  int tiles_since_flush = 0;
  for (long t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    // upper-triangle index t -> (ti, tk), ti <= tk, row by row
    long ti = (long)((2 * T + 1 - sqrt((double)(2 * T + 1) * (2 * T + 1) - 8.0 * t)) / 2);
    while (ti > 0 && ti * T - ti * (ti - 1) / 2 > t) ti--;
    while ((ti + 1) * T - (ti + 1) * ti / 2 <= t) ti++;
    const long tk = ti + (t - (ti * T - ti * (ti - 1) / 2));
    if (priv && ++tiles_since_flush > kPrivFlushTiles) {  // each tile adds at most kPcfTile to a count
      flush();
      tiles_since_flush = 1;
    }
    __syncthreads();
    const long kk = tk * kPcfTile + threadIdx.x;
    if (kk < n) {
      tidx[threadIdx.x] = pcf_idx[kk];
      tile[threadIdx.x] = posf[tidx[threadIdx.x]];
    }
    __syncthreads();
    const long ii = ti * kPcfTile + threadIdx.x;
    if (ii >= n) continue;
    const int gi = pcf_idx[ii];
    const float4 pi = posf[gi];
    const int kend = (int)min((long)kPcfTile, n - tk * kPcfTile);
#pragma unroll 4
    for (int k = tk == ti ? threadIdx.x + 1 : 0; k < kend; k++) {
      bool unsure = false;
      const float r2 = sep2_f_t<IMAGE>(pi, tile[k], P, unsure);
      if (!unsure && r2 >= far2) continue;
      const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
      int bin = -1;
      if (!unsure && r < P.halff - P.tol_r) {
        const float x = r * P.inv_dgf;
        const float f = floorf(x);
        if (x - f >= P.tol_bin && x - f <= 1.0f - P.tol_bin) bin = (int)f;
        else unsure = true;
      } else {
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
      if (bin >= 0) {
        bin = min(bin, P.bins - 1);
        if (priv) ph[bin * kPcfTile + threadIdx.x] += 1;
        else atomicAdd(h + bin, 1u);
      }
    }
  }
  flush();
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
__global__ void __launch_bounds__(256) k_an_hist(const float4* __restrict__ posf, const AnParams P,
                                                 const int* __restrict__ labels, const int* __restrict__ size_sub,
                                                 const int* __restrict__ parent_bead, const int* __restrict__ size_bead,
                                                 unsigned long long* __restrict__ olig, unsigned long long* __restrict__ so,
                                                 unsigned int* __restrict__ cnt) {
  // most components are small: their bins are counted in shared memory first, so that thousands
  // of single subunits or beads do not queue on one global counter
  __shared__ unsigned lo[kHistLocal], ls[kHistLocal];
  for (int k = threadIdx.x; k < kHistLocal; k += blockDim.x) lo[k] = ls[k] = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.S && labels[i] == i) {
    const int bin = size_sub[i] - 1;
    if (bin < kHistLocal) atomicAdd(lo + bin, 1u);
    else atomicAdd(olig + bin, 1ull);
  }
  if (i < P.N && type_of(posf[i]) == P.so_type && parent_bead[i] == i) {
    const int bin = (size_bead[i] - 1) / 3;
    if (bin >= 2 * P.S) atomicOr(cnt + C_FLAGS, F_SO_OVERFLOW);
    else if (bin < kHistLocal) atomicAdd(ls + bin, 1u);
    else atomicAdd(so + bin, 1ull);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kHistLocal; k += blockDim.x) {
    if (lo[k]) atomicAdd(olig + k, (unsigned long long)lo[k]);
    if (ls[k]) atomicAdd(so + k, (unsigned long long)ls[k]);
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
  size_t contact_smem = 0;           // dynamic shared memory of k_an_contacts (two staged subunits per warp)
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
  const int nmax = std::max(P.N, P.S);
  k_an_prep<<<(P.S + 7) / 8, 256, 0, st>>>(pos, types, P, h->posf.p, h->sph.p, h->parent_bead.p, h->size_bead.p,
                                            h->parent_sub.p, h->size_sub.p, h->pcf_idx.p, gr, olig, so, h->cnt.p);
  const int cand_warps = (P.S + 1) / 2;
  const dim3 gcand((cand_warps + kCandWarps - 1) / kCandWarps, (P.S + kCandSeg - 1) / kCandSeg);
  k_an_candidates<<<gcand, kCandWarps * 32, 0, st>>>(h->sph.p, P, h->cand.p, h->cnt.p);
  const long items_max = (long)P.cap + P.S;
  const int gcon = (int)std::min<long>((items_max + kContactWarps - 1) / kContactWarps, 8L * h->sms);
  k_an_contacts<<<gcon, kContactWarps * 32, h->contact_smem, st>>>(pos, h->posf.p, h->sph.p, h->cand.p, P,
                                                                   h->parent_sub.p, h->parent_bead.p, h->cnt.p);
  const long Tp = (P.N + kPcfTile - 1) / kPcfTile;
  const int gpcf = (int)std::min<long>(Tp * (Tp + 1) / 2, 8L * h->sms);
  // the reference rule counts few pairs (those the long way round is short for), the minimum image
  // about half of all pairs: per-thread histograms only pay off for the latter
  const size_t pcf_smem = P.image == SOUFFLE_IMAGE_MINIMUM && P.bins <= kPrivBins
                              ? sizeof(unsigned short) * P.bins * kPcfTile
                              : sizeof(unsigned int) * (P.bins <= 512 ? kPcfTile / 32 : 1) * P.bins;
  if (P.image == SOUFFLE_IMAGE_REFERENCE)
    k_an_pcf<SOUFFLE_IMAGE_REFERENCE><<<gpcf, kPcfTile, pcf_smem, st>>>(pos, h->posf.p, h->pcf_idx.p, P, gr, h->cnt.p);
  else
    k_an_pcf<SOUFFLE_IMAGE_MINIMUM><<<gpcf, kPcfTile, pcf_smem, st>>>(pos, h->posf.p, h->pcf_idx.p, P, gr, h->cnt.p);
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
  h->contact_smem = sizeof(float4) * 2 * kContactWarps * (size_t)P.np;
  cudaError_t e = cudaFuncSetAttribute(k_an_contacts, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)h->contact_smem);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
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
