// Pair-list rebuild: counting-sort grid of subunit centres, candidate subunits, bead pairs.
//
// Reference: update_pairlist (src/functions.cpp:69-117), called per subunit from
// forceCalculation when step % B == 0 (src/forces.cpp:63-65, src/md.cpp:435-438).  The
// reference tests every subunit pair's centre beads against 1.5 x the list radius
// (|c_i - c_j|^2 < 2.25 r^2), then every bead pair of a passing subunit pair against r^2,
// appending neighbour ids in ascending order.  Here the O(S^2) centre scan becomes a
// counting-sort cell grid (cell edge >= 1.5 r, 27-cell stencil) that yields the same
// candidate set; candidates are sorted so lists come out in the reference's order.
//
// Decisions are exact: a float test on the rounded high words settles every pair farther than
// a safety margin from the cut-off, and the rest are decided in double from the exact 64-bit
// fixed-point differences, matching the reference up to long double vs double ties.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"

namespace souffle {


__device__ __forceinline__ int cell_coord(long long x, int ncell) {
  unsigned long long u = (unsigned long long)x + 0x8000000000000000ull;  // [0, 2^64) over [-L/2, L/2)
  return (int)__umul64hi(u, (unsigned long long)ncell);
}

__global__ void k_cells_count(CellArgs a) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n_sub_total) return;
  const SysParams& p = a.sys[a.sub_sys[s]];
  int c = s * a.np + p.center_local;
  int n = p.ncell;
  int cx = cell_coord(a.px[c], n), cy = cell_coord(a.py[c], n), cz = cell_coord(a.pz[c], n);
  int cell = p.cell0 + (cx * n + cy) * n + cz;
  a.sub_cell[s] = cell;
  a.sub_rank[s] = atomicAdd(&a.cell_count[cell], 1);
}

// Exclusive scan of cell counts, one CTA per system: a system's cells hold only its own
// subunits, which are contiguous, so its scan starts at the system's first subunit and the
// segments line up into one global cell_start array.  Each thread takes a run of kScanPer cells
// (their loads in flight together) and the runs' sums are scanned across the CTA.
constexpr int kScanPer = 8;
__global__ void __launch_bounds__(1024) k_cells_scan(CellArgs a) {
  __shared__ int warp_sums[32];
  __shared__ int carry;
  const SysParams& P = a.sys[blockIdx.x];
  const int c0 = P.cell0, nc = P.ncell * P.ncell * P.ncell;
  if (threadIdx.x == 0) carry = P.sub0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < nc; base += blockDim.x * kScanPer) {
    const int i0 = base + threadIdx.x * kScanPer;
    int v[kScanPer];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      v[k] = (i0 + k < nc) ? a.cell_count[c0 + i0 + k] : 0;
      sum += v[k];
    }
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int w = (lane < nw) ? warp_sums[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    int excl = x - sum + (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      if (i0 + k < nc) a.cell_start[c0 + i0 + k] = excl;
      excl += v[k];
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl;  // the pass's end: carry + all its counts
    __syncthreads();
  }
  // the end sentinel of the last system (other systems' ends are the next system's first start)
  if (threadIdx.x == 0 && c0 + nc == a.total_cells) a.cell_start[a.total_cells] = carry;
}

__global__ void k_cells_scatter(CellArgs a) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n_sub_total) return;
  a.cell_subs[a.cell_start[a.sub_cell[s]] + a.sub_rank[s]] = s;
}


// Margin (in length^2) within which the float test defers to the exact double test.
__device__ __forceinline__ float pair_margin(float nl2) { return 1e-4f * (1.0f + nl2); }

// One warp per subunit i: lane k scans stencil cell k (27 cells; with fewer than 3 cells per side
// every cell of the system is a neighbour and is scanned once), testing centre distances
// (src/functions.cpp:80-91): in float on the high words, and exactly in double from the 64-bit
// fixed-point differences when the float value lies within a safety margin of the cut-off.  Hits
// are compacted with a warp scan into shared memory and put in ascending order by rank.
// blockDim must be 128 (4 warps).
__global__ void __launch_bounds__(128) k_candidates(CandArgs a) {
  extern __shared__ int s_cand[];  // [4 warps][cap]
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= a.c.n_sub_total) return;  // uniform per warp
  int* buf = s_cand + wib * a.cap;
  const SysParams& p = a.c.sys[a.c.sub_sys[i]];
  const int np = a.c.np, cl = p.center_local;
  const int ci = i * np + cl;
  const long long xi = a.c.px[ci], yi = a.c.py[ci], zi = a.c.pz[ci];
  const int n = p.ncell;
  const int span = (n < 3) ? n : 3;
  const int ncells = span * span * span;
  int s0 = 0, s1 = 0;
  if (lane < ncells) {
    const int dx = lane / (span * span), dy = (lane / span) % span, dz = lane % span;
    const int cx = cell_coord(xi, n), cy = cell_coord(yi, n), cz = cell_coord(zi, n);
    const int gx = (n < 3) ? dx : (cx + dx - 1 + n) % n;
    const int gy = (n < 3) ? dy : (cy + dy - 1 + n) % n;
    const int gz = (n < 3) ? dz : (cz + dz - 1 + n) % n;
    const int cell = p.cell0 + (gx * n + gy) * n + gz;
    s0 = a.c.cell_start[cell];
    s1 = a.c.cell_start[cell + 1];
  }
  const int4 pci = a.pos32[ci];
  const float pre2f = (float)p.pre2, marg = pair_margin(pre2f);
  auto take = [&](int j) {
    if (j == i) return true;  // r2 = 0 for i == j (src/functions.cpp:90)
    const int cj = j * np + cl;
    const int4 pcj = a.pos32[cj];
    const float fx = hi_diff(pci.x, pcj.x, p.unit32), fy = hi_diff(pci.y, pcj.y, p.unit32),
                fz = hi_diff(pci.z, pcj.z, p.unit32);
    const float r2f = fx * fx + fy * fy + fz * fz;
    if (fabsf(r2f - pre2f) > marg) return r2f < pre2f;
    const double ddx = fixed_diff(xi, a.c.px[cj], p.fx_to_len);
    const double ddy = fixed_diff(yi, a.c.py[cj], p.fx_to_len);
    const double ddz = fixed_diff(zi, a.c.pz[cj], p.fx_to_len);
    return (ddx * ddx + ddy * ddy + ddz * ddz) < p.pre2;
  };
  int nh = 0;  // pass 1: count this lane's hits
  for (int k = s0; k < s1; k++) nh += take(a.c.cell_subs[k]) ? 1 : 0;
  // warp exclusive scan of hit counts
  int x = nh;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const int total = __shfl_sync(0xffffffffu, x, 31);
  int off = x - nh;  // pass 2: write at the lane's offset
  for (int k = s0; k < s1 && off < a.cap; k++) {
    const int j = a.c.cell_subs[k];
    if (take(j)) buf[off++] = j;
  }
  __syncwarp();
  const int cnt = total < a.cap ? total : a.cap;
  if (lane == 0 && total > a.cap) atomicOr(a.err, kErrCandOverflow);
  // rank sort (ids are distinct)
  int* out = a.cand + (size_t)i * a.cap;
  for (int k = lane; k < cnt; k += 32) {
    const int v = buf[k];
    int r = 0;
    for (int m = 0; m < cnt; m++) r += (buf[m] < v);
    out[r] = v;
  }
  if (lane == 0) a.cand_count[i] = cnt;
}



// One CTA per subunit i; thread t owns bead rows t, t + blockDim, ... (at most two: blockDim is
// np rounded up to whole warps, at most 128, so that a one-wave grid holds every subunit).
// Candidates are taken in ascending j, so each row's entries come out in ascending global id.
// Runs of ordinary candidates are staged together (a chunk): their high words load in one round,
// every (candidate, row) item computes its partner mask in parallel, and each row then appends
// the chunk's partners in order -- a handful of barriers per chunk instead of per candidate.
// Subunit i's own block (intra bits, each unordered pair once) and blocks with the stale-r2
// semantics of the system's subunit 0 take the per-block path, one candidate at a time.
__global__ void __launch_bounds__(128) k_pairs(PairArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int4* s32 = reinterpret_cast<int4*>(smem_raw);                   // [np] 16-byte entries first
  long long* sx = reinterpret_cast<long long*>(s32 + a.np);
  long long* sy = sx + a.np;
  long long* sz = sy + a.np;
  double* row_last = reinterpret_cast<double*>(sz + a.np);         // [np] quirk pass
  int* row_has = reinterpret_cast<int*>(row_last + a.np);          // [np]
  float* sq = reinterpret_cast<float*>(row_has + a.np);           // [np]
  unsigned int* s_imask = reinterpret_cast<unsigned int*>(sq + a.np);  // [np * words] intra bits

  const int i = blockIdx.x;
  const int sysid = a.sub_sys[i];
  const SysParams& p = a.sys[sysid];
  const int np = a.np;
  const int i_local = i - p.sub0;  // subunit index inside its system
  const float unit = p.unit32;
  const float nl2f = p.nl2_f;
  const float margin = pair_margin(nl2f);
  const int ncand = a.cand_count[i];
  const int* cand = a.cand + (size_t)i * a.cand_cap;

  for (int t = threadIdx.x; t < np; t += blockDim.x) sq[t] = a.q[t];

  // per-row state held in registers for up to 2 rows per thread (np <= 256, blockDim 128)
  int inter_n[2] = {0, 0};
  unsigned int* mask_rows = a.intra_mask + (size_t)i * np * a.words;
  for (int t = threadIdx.x; t < np * a.words; t += blockDim.x) mask_rows[t] = 0u;

  const int ci_global = i * np + p.center_local;
  const long long cxi = a.px[ci_global], cyi = a.py[ci_global], czi = a.pz[ci_global];

  // Exact shortcut by the triangle inequality, from candidate j's radius about its centre bead
  // (float on the high words, padded by eps far beyond their rounding): a row farther than
  // R_j + r_list from j's centre has no pair with j.  Cases touched by the stale-r2 quirk skip it.
  __shared__ float s_Rj;
  const float r_list = sqrtf(nl2f), eps = 1e-3f * (1.0f + r_list);
  for (int t = threadIdx.x; t < np * a.words; t += blockDim.x) s_imask[t] = 0u;

  const bool skip_far = a.cand_far && *a.far_ok;
  // chunk staging (after the per-block area, 16-byte aligned): the own rows' high words, the
  // chunk's candidates' high words, and a mask of partners per (candidate, row)
  const size_t blk_bytes = (size_t)np * (sizeof(int4) + 3 * sizeof(long long) + sizeof(double) + sizeof(int) +
                                         sizeof(float)) + sizeof(unsigned int) * (size_t)np * a.words;
  int4* s_own = reinterpret_cast<int4*>(smem_raw + ((blk_bytes + 15) & ~(size_t)15));
  int4* c32 = s_own + np;
  unsigned int* cmask = reinterpret_cast<unsigned int*>(c32 + (size_t)a.chunk * np);
  __shared__ int s_cj[kPairChunkMax];
  __shared__ float s_cR[kPairChunkMax];
  for (int t = threadIdx.x; t < np; t += blockDim.x) s_own[t] = a.pos32[(size_t)i * np + t];
  const bool cta_quirk = p.quirks && i_local == 0;  // every block of the system's subunit 0
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __shared__ int s_ctl[3];  // candidates consumed, chunk size, candidate for the per-block path (-1: none)
  int c = 0;
  while (c < ncand) {
    __syncthreads();  // the previous chunk's readers are done
    // Warp 0 looks at the next 32 candidates: far ones (left to the surrogate, or beyond every
    // cut-off) are skipped; the chunk takes up to a.chunk ordinary candidates before the first
    // one that needs the per-block path (subunit i itself, or a block with the stale-r2
    // semantics); with no ordinary candidate before it, that one goes to the per-block path.
    if (wid == 0) {
      const int cc = c + lane;
      const bool valid = cc < ncand;
      int j = -1;
      bool far = false;
      if (valid) {
        j = cand[cc];
        far = skip_far && a.cand_far[(size_t)i * a.cand_cap + cc];
      }
      const bool slow = valid && !far && (j == i || cta_quirk || (p.quirks && j == p.sub0));
      const unsigned int sb = __ballot_sync(0xffffffffu, slow);
      const unsigned int nb = __ballot_sync(0xffffffffu, valid && !far && !slow);
      const int fs = sb ? __ffs(sb) - 1 : 32;  // first slow lane
      const unsigned int take = fs < 32 ? nb & ((1u << fs) - 1u) : nb;
      const int rank = __popc(take & ((1u << lane) - 1u));
      const bool mine = ((take >> lane) & 1u) && rank < a.chunk;
      if (mine) s_cj[rank] = j;
      const int nk = min(__popc(take), a.chunk);
      int consumed, slow_j = -1;
      if (__popc(take) > a.chunk) {  // full chunk: up to and including its last candidate
        const unsigned int last = __ballot_sync(0xffffffffu, mine && rank == a.chunk - 1);
        consumed = __ffs(last);
      } else if (fs < 32) {
        consumed = nk > 0 ? fs : fs + 1;
        if (nk == 0) slow_j = __shfl_sync(0xffffffffu, j, fs);
      } else {
        consumed = min(32, ncand - c);
      }
      if (lane == 0) {
        s_ctl[0] = consumed;
        s_ctl[1] = nk;
        s_ctl[2] = slow_j;
      }
    }
    __syncthreads();
    const int nk = s_ctl[1];
    const int slow_j = s_ctl[2];
    c += s_ctl[0];
    if (nk > 0) {
      for (int t = threadIdx.x; t < nk * np; t += blockDim.x) {
        const int k = t / np;
        c32[t] = a.pos32[(size_t)s_cj[k] * np + (t - k * np)];
      }
      __syncthreads();
      // each candidate's radius about its centre bead, warp per candidate
      for (int k = wid; k < nk; k += nw) {
        const int4 pc = c32[k * np + p.center_local];
        float m = 0.0f;
        for (int t = lane; t < np; t += 32) {
          const int4 pt = c32[k * np + t];
          const float dx = hi_diff(pt.x, pc.x, unit), dy = hi_diff(pt.y, pc.y, unit), dz = hi_diff(pt.z, pc.z, unit);
          m = fmaxf(m, sqrtf(dx * dx + dy * dy + dz * dz));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) s_cR[k] = m;
      }
      __syncthreads();
      // partner masks of every (candidate, row) item: the same float test with its margin and
      // exact fallback, and the same reach shortcut, as the per-block path
      for (int t = threadIdx.x; t < nk * np; t += blockDim.x) {
        const int k = t / np, ii = t - k * np;
        unsigned int* mk = cmask + (size_t)t * a.words;
        const int4* cj32 = c32 + k * np;
        const int4 pi = s_own[ii];
        const int4 pc = cj32[p.center_local];
        const float reach = s_cR[k] + r_list + eps;
        const float ex = hi_diff(pi.x, pc.x, unit), ey = hi_diff(pi.y, pc.y, unit), ez = hi_diff(pi.z, pc.z, unit);
        const bool skip = ex * ex + ey * ey + ez * ez > reach * reach;
        const int gi = i * np + ii, jbase = s_cj[k] * np;
        for (int w0 = 0; w0 < np; w0 += 32) {
          unsigned int bits = 0;
          if (!skip) {
            const int w1 = min(np, w0 + 32);
            for (int jj = w0; jj < w1; jj++) {
              const int4 pj = cj32[jj];
              const float dx = hi_diff(pi.x, pj.x, unit), dy = hi_diff(pi.y, pj.y, unit), dz = hi_diff(pi.z, pj.z, unit);
              const float r2f = dx * dx + dy * dy + dz * dz;
              bool in;
              if (fabsf(r2f - nl2f) > margin) {
                in = r2f < nl2f;
              } else {
                const int gj = jbase + jj;
                const double ex = fixed_diff(a.px[gi], a.px[gj], p.fx_to_len);
                const double ey = fixed_diff(a.py[gi], a.py[gj], p.fx_to_len);
                const double ez = fixed_diff(a.pz[gi], a.pz[gj], p.fx_to_len);
                in = ex * ex + ey * ey + ez * ez < p.nl2;
              }
              if (in) bits |= 1u << (jj - w0);
            }
          }
          mk[w0 >> 5] = bits;
        }
      }
      __syncthreads();
      // ids in ascending global order: candidates in order, partners in bead order
      for (int r = 0, ii = threadIdx.x; ii < np; ii += blockDim.x, r++) {
        const int gi = i * np + ii;
        int n = inter_n[r];
        for (int k = 0; k < nk; k++) {
          const unsigned int* mk = cmask + (size_t)(k * np + ii) * a.words;
          const int jbase = s_cj[k] * np;
          for (int w = 0; w < a.words; w++) {
            unsigned int bits = mk[w];
            while (bits) {
              const int b = __ffs(bits) - 1;
              bits &= bits - 1;
              if (n < a.inter_cap) a.inter_ids[(size_t)gi * a.inter_cap + n] = jbase + (w << 5) + b;
              n++;
            }
          }
        }
        inter_n[r] = n;
      }
      continue;
    }
    if (slow_j < 0) continue;  // only far candidates in this window
    // per-block path for candidate slow_j
    const int j = slow_j;
    __syncthreads();
    if (threadIdx.x == 0) s_Rj = 0.0f;
    for (int t = threadIdx.x; t < np; t += blockDim.x) {
      int g = j * np + t;
      sx[t] = a.px[g];
      sy[t] = a.py[g];
      sz[t] = a.pz[g];
      s32[t] = a.pos32[g];
    }
    __syncthreads();
    const int j_local = j - p.sub0;
    const bool same = (j == i);
    // exact squared distance between bead gi and staged bead jj of subunit j
    auto d2_exact = [&](int gi, int jj) {
      const double ex = fixed_diff(a.px[gi], sx[jj], p.fx_to_len);
      const double ey = fixed_diff(a.py[gi], sy[jj], p.fx_to_len);
      const double ez = fixed_diff(a.pz[gi], sz[jj], p.fx_to_len);
      return ex * ex + ey * ey + ez * ez;
    };
    // r2 < r_list^2, decided in float unless within the margin of the cut-off
    auto inside = [&](int gi, int4 pi, int jj) {
      const int4 pj = s32[jj];
      const float dx = hi_diff(pi.x, pj.x, unit), dy = hi_diff(pi.y, pj.y, unit), dz = hi_diff(pi.z, pj.z, unit);
      const float r2f = dx * dx + dy * dy + dz * dz;
      if (fabsf(r2f - nl2f) > margin) return r2f < nl2f;
      return d2_exact(gi, jj) < p.nl2;
    };
    // The stale-r2 reuse of src/functions.cpp:97 can only trigger when subunit 0 of the system is
    // involved.  The test there compares a local index with a global id, so a distance is
    // recomputed unless (i is subunit 0 and ii is its centre) or (j is subunit 0 and jj is its
    // centre); otherwise the r2 of the most recently computed pair (row-major over the block) is
    // reused, starting from the centre-centre distance (or 0 when i == j).  Only two exact
    // distances per row are ever needed for that: the row's last computed pair (carried into
    // later rows) and the computed pair just before the stale column.
    const bool quirk = p.quirks && (i_local == 0 || j_local == 0);
    const int cl = p.center_local;
    if (!same && !quirk) {  // radius of candidate j about its centre bead
      const int4 pc = s32[cl];
      for (int t = threadIdx.x; t < np; t += blockDim.x) {
        const int4 pt = s32[t];
        const float dx = hi_diff(pt.x, pc.x, unit), dy = hi_diff(pt.y, pc.y, unit), dz = hi_diff(pt.z, pc.z, unit);
        atomicMax(reinterpret_cast<int*>(&s_Rj), __float_as_int(sqrtf(dx * dx + dy * dy + dz * dz)));
      }
      __syncthreads();
    }
    const float reach_j = s_Rj + r_list + eps;
    const bool i0 = quirk && (i_local == 0), j0 = quirk && (j_local == 0);
    double init_r2 = 0.0;
    if (quirk) {
      if (!same) {
        const int cj = j * np + cl;
        const double ex = fixed_diff(cxi, a.px[cj], p.fx_to_len), ey = fixed_diff(cyi, a.py[cj], p.fx_to_len),
                     ez = fixed_diff(czi, a.pz[cj], p.fx_to_len);
        init_r2 = ex * ex + ey * ey + ez * ez;
      }
      for (int ii = threadIdx.x; ii < np; ii += blockDim.x) {  // pass 1
        const int gi = i * np + ii;
        const bool qi = sq[ii] != 0.0f;
        double last = 0.0;
        int has = 0;
        if (!(i0 && ii == cl)) {
          for (int jj = np - 1; jj >= 0; jj--) {
            const bool cond = same ? (jj != ii && qi && sq[jj] != 0.0f) : true;
            if (cond && !(j0 && jj == cl)) {
              last = d2_exact(gi, jj);
              has = 1;
              break;
            }
          }
        }
        row_last[ii] = last;
        row_has[ii] = has;
      }
      __syncthreads();
    }
    for (int r = 0, ii = threadIdx.x; ii < np; ii += blockDim.x, r++) {
      const int gi = i * np + ii;
      const int4 pi = a.pos32[gi];
      const bool qi = sq[ii] != 0.0f;
      double carried = init_r2;
      if (quirk)
        for (int k = ii - 1; k >= 0; k--)
          if (row_has[k]) {
            carried = row_last[k];
            break;
          }
      if (same && !quirk) {
        // each unordered pair once: row ii takes partners ii + d (mod np), d = 1 .. (np - 1) / 2,
        // and d = np / 2 for ii < np / 2 when np is even (21 tests per row at np = 42).  The
        // decision is symmetric in (ii, jj) in both the float and the exact test, so both rows
        // get the bit the reference computes for each.
        if (!qi) continue;
        const int dmax = (np - 1) >> 1;
        const int dlast = ((np & 1) == 0 && ii < (np >> 1)) ? (np >> 1) : dmax;
        for (int dd = 1; dd <= dlast; dd++) {
          int jj = ii + dd;
          if (jj >= np) jj -= np;
          if (sq[jj] == 0.0f || !inside(gi, pi, jj)) continue;
          atomicOr(&s_imask[ii * a.words + (jj >> 5)], 1u << (jj & 31));
          atomicOr(&s_imask[jj * a.words + (ii >> 5)], 1u << (ii & 31));
        }
        continue;
      }
      if (!same && !quirk) {  // a row out of reach of subunit j has no pair with it
        const int4 pc = s32[cl];
        const float dx = hi_diff(pi.x, pc.x, unit), dy = hi_diff(pi.y, pc.y, unit), dz = hi_diff(pi.z, pc.z, unit);
        if (dx * dx + dy * dy + dz * dz > reach_j * reach_j) continue;
      }
      const bool row_stale = i0 && ii == cl;
      int prev_jj = -1;  // last computed pair of this row
      for (int w0 = 0; w0 < np; w0 += 32) {
        unsigned int bits = 0;  // the row's intra-subunit mask word, stored once
        const int w1 = min(np, w0 + 32);
        for (int jj = w0; jj < w1; jj++) {
          if (same && !(jj != ii && qi && sq[jj] != 0.0f)) continue;  // electrostatic only (:94-96)
          bool in;
          if (row_stale) {
            in = carried < p.nl2;
          } else if (j0 && jj == cl) {
            in = (prev_jj >= 0 ? d2_exact(gi, prev_jj) : carried) < p.nl2;
          } else {
            in = inside(gi, pi, jj);
            prev_jj = jj;
          }
          if (!in) continue;
          if (same) {
            bits |= 1u << (jj - w0);
          } else {
            int k = inter_n[r];
            if (k < a.inter_cap) a.inter_ids[(size_t)gi * a.inter_cap + k] = j * np + jj;
            inter_n[r] = k + 1;
          }
        }
        // the subunit's own block is the only one that sets intra bits (its candidate list holds
        // it once), so the word is written whole
        if (same) mask_rows[ii * a.words + (w0 >> 5)] = bits;
      }
    }
    if (same && !quirk) {  // the symmetric block's bits, complete once every row is done
      __syncthreads();
      for (int t = threadIdx.x; t < np * a.words; t += blockDim.x) mask_rows[t] = s_imask[t];
    }
  }
  __syncthreads();
  for (int r = 0, ii = threadIdx.x; ii < np; ii += blockDim.x, r++) {
    const int gi = i * np + ii;
    int n_inter = inter_n[r];
    if (n_inter > a.inter_cap) {
      atomicOr(a.err, kErrInterOverflow);
    }
    a.inter_count[gi] = n_inter < a.inter_cap ? n_inter : a.inter_cap;
    int n_intra = 0;
    for (int w = 0; w < a.words; w++) n_intra += __popc(mask_rows[ii * a.words + w]);
    a.ref_len[gi] = n_intra + n_inter;
  }
}

}  // namespace souffle

namespace souffle {
void launch_cells_count(const CellArgs& a, int grid, int block, cudaStream_t s) {
  k_cells_count<<<grid, block, 0, s>>>(a);
}
void launch_cells_scan(const CellArgs& a, cudaStream_t s) { k_cells_scan<<<a.n_sys, 1024, 0, s>>>(a); }
void launch_cells_scatter(const CellArgs& a, int grid, int block, cudaStream_t s) {
  k_cells_scatter<<<grid, block, 0, s>>>(a);
}
void launch_candidates(const CandArgs& a, int grid, int block, cudaStream_t s) {
  (void)grid;
  (void)block;
  const int warps_per_block = 4;
  const int g = (a.c.n_sub_total + warps_per_block - 1) / warps_per_block;
  k_candidates<<<g, 32 * warps_per_block, sizeof(int) * warps_per_block * a.cap, s>>>(a);
}
// About 8 KB of staging per CTA (8 candidates of 42 beads), so that a one-wave grid of 64-thread
// CTAs still fits the shared memory of an SM.
int pair_chunk(int np, int words) {
  const int per = np * (int)(sizeof(int4) + sizeof(unsigned int) * words);
  return std::max(1, std::min(kPairChunkMax, 8192 / per));
}
size_t pair_smem_bytes(int np, int words, int chunk) {
  const size_t blk = (size_t)np * (sizeof(int4) + 3 * sizeof(long long) + sizeof(double) + sizeof(int) + sizeof(float)) +
                     sizeof(unsigned int) * (size_t)np * words;
  return ((blk + 15) & ~(size_t)15) + sizeof(int4) * (size_t)np * (1 + chunk) +
         sizeof(unsigned int) * (size_t)chunk * np * words;
}
void launch_pairs(const PairArgs& a, int n_sub, size_t smem, cudaStream_t s) {
  const int block = std::min(128, 32 * ((a.np + 31) / 32));
  k_pairs<<<n_sub, block, smem, s>>>(a);
}
cudaError_t set_pairs_smem(size_t smem) {
  return cudaFuncSetAttribute(k_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
}  // namespace souffle
