// Energy block of run_simulation (src/md.cpp:553-605), evaluated in FP64.
//
//   k_energy_bonded   BEAD::update_stretching_energy (src/bead.cpp:9-14),
//                     EDGE::update_bending_energy (src/edge.cpp:51-67),
//                     BEAD::update_kinetic_energy (src/bead.h:129-131)
//   k_energy_pairs    update_LJ_ES_energies_simplified (src/energies.cpp:24-93): every pair
//                     j > i of the system (no pair list, no prefilter), energy credited to i;
//                     shifted Debye-Hueckel, WCA (+1 shift), and attractive LJ shifted at ecut
//                     with sbar^6 and epsilon = -E.
//   k_energy_bigbeads update_LJ_ES_energies_bigbeads (src/energies.cpp:96-137) when the system
//                     has encapsulation big beads
//   k_energy_totals   per-system sums in bead order (src/md.cpp:586-594).
// A float test on the high words skips pairs beyond every cut-off (a conservative margin, so the
// sums are those of all pairs); the rest use exact fixed-point differences in double.
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace souffle {


__device__ __forceinline__ void ddiff(const EnergyArgs& a, double fx, int i, int j, double& x,
                                      double& y, double& z) {
  x = fixed_diff(a.px[i], a.px[j], fx);
  y = fixed_diff(a.py[i], a.py[j], fx);
  z = fixed_diff(a.pz[i], a.pz[j], fx);
}

// Face area vector 1/2 (b1 - b0) x (b2 - b1) in double.
__device__ void face_area(const EnergyArgs& a, double fx, int base, int f, double A[3]) {
  const int* fb = a.tpl_i + a.L.o_face;
  int b0 = base + fb[3 * f], b1 = base + fb[3 * f + 1], b2 = base + fb[3 * f + 2];
  double u[3], v[3];
  ddiff(a, fx, b1, b0, u[0], u[1], u[2]);
  ddiff(a, fx, b2, b1, v[0], v[1], v[2]);
  A[0] = 0.5 * (u[1] * v[2] - u[2] * v[1]);
  A[1] = 0.5 * (u[2] * v[0] - u[0] * v[2]);
  A[2] = 0.5 * (u[0] * v[1] - u[1] * v[0]);
}

__global__ void k_energy_bonded(EnergyArgs a) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n) return;
  const TplLayout& L = a.L;
  const SysParams& P = a.sys[a.sysid];
  const SysState& S = a.state[a.sysid];
  const double fx = P.fx_to_len;
  const int g = a.n0 + t;
  const int np = L.np;
  const int l = g % np;
  const int base = g - l;
  const int* e_pack = a.tpl_i + L.o_edge;
  double se = 0.0;
  for (int k = 0; k < L.maxdeg; k++) {
    int e = a.tpl_i[L.o_bead_edges + l * L.maxdeg + k];
    if (e < 0) break;
    int pk = e_pack[e];
    double x, y, z;
    ddiff(a, fx, base + (pk & 0xffff), base + (pk >> 16), x, y, z);
    double len = sqrt(x * x + y * y + z * z);
    double d = a.len0[e] - len;
    se += 0.25 * P.ks_d * d * d;
  }
  // bending: kb/4 (1 - |n0 . n1|) per bending edge the bead belongs to, in edge order
  double be = 0.0;
  const int* bf = a.tpl_i + L.o_bendf;
  for (int k = 0; k < L.maxrole; k++) {
    int r = a.tpl_i[L.o_bead_roles + l * L.maxrole + k];
    if (r < 0) break;
    int kb_ = r >> 2;
    const double beta0 = (double)a.tpl_f[L.o_beta0 + kb_];
    if (beta0 != 0.0) {  // rest-angle option: kb/4 (1 - cos(beta - beta0)) per quad bead
      const int* bq = a.tpl_i + L.o_bend + 4 * kb_;
      double v1[3], v2[3], v3[3];
      ddiff(a, fx, base + bq[0], base + bq[2], v1[0], v1[1], v1[2]);
      ddiff(a, fx, base + bq[1], base + bq[0], v2[0], v2[1], v2[2]);
      ddiff(a, fx, base + bq[3], base + bq[1], v3[0], v3[1], v3[2]);
      const double m[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
      const double n[3] = {v2[1] * v3[2] - v2[2] * v3[1], v2[2] * v3[0] - v2[0] * v3[2], v2[0] * v3[1] - v2[1] * v3[0]};
      const double l2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
      const double beta = atan2(-l2 * (v1[0] * n[0] + v1[1] * n[1] + v1[2] * n[2]), -(m[0] * n[0] + m[1] * n[1] + m[2] * n[2]));
      be += P.kb_d * 0.25 * (1.0 - cos(beta - beta0));
      continue;
    }
    double A0[3], A1[3];
    face_area(a, fx, base, bf[2 * kb_], A0);
    face_area(a, fx, base, bf[2 * kb_ + 1], A1);
    double a0 = sqrt(A0[0] * A0[0] + A0[1] * A0[1] + A0[2] * A0[2]);
    double a1 = sqrt(A1[0] * A1[0] + A1[1] * A1[1] + A1[2] * A1[2]);
    double c = (A0[0] * A1[0] + A0[1] * A1[1] + A0[2] * A1[2]) / (a0 * a1);
    be += P.kb_d * 0.25 * (1.0 - fabs(c));
  }
  const double inv = 1.0 / kVelScale;
  const double vx = (double)(a.vx[g] - S.vcom_fx[0]) * inv, vy = (double)(a.vy[g] - S.vcom_fx[1]) * inv,
               vz = (double)(a.vz[g] - S.vcom_fx[2]) * inv;
  const double m = a.mass[l];
  a.se[t] = se;
  a.be[t] = be;
  a.ke[t] = 0.5 * m * (vx * vx + vy * vy + vz * vz);
}

// Per template bead pair (li, lj), the pair terms that do not depend on the distance, in the
// reference's expressions: the Yukawa size factor e^(kappa sbar) / ((1 + kappa s_i / 2)
// (1 + kappa s_j / 2)), sbar^6, the attractive LJ shift 4 eps ((sbar^6 / ecut^6)
// ((sbar^6 / ecut^6) - 1)), and whether (type_i, type_j) is a row of the directed LJ table.
__global__ void k_energy_tables(EnergyArgs a) {
  const int np = a.L.np;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= np * np) return;
  const int li = idx / np, lj = idx - li * np;
  const double kappa = a.kappa, ecut = a.ecut;
  const double ecut3 = ecut * ecut * ecut, ecut6 = ecut3 * ecut3;
  const double sgi = a.sigma[li], sgj = a.sigma[lj];
  const double shc = (sgi + sgj) / 2;
  const double s3 = shc * shc * shc, s6 = s3 * s3;
  a.pair_tab[idx] = exp(kappa * shc) / ((1 + kappa * sgi / 2) * (1 + kappa * sgj / 2));
  a.pair_tab[np * np + idx] = s6;
  a.pair_tab[2 * np * np + idx] = 4 * a.elj_att * ((s6 / ecut6) * ((s6 / ecut6) - 1));
  bool att = false;
  for (int m = 0; m < a.n_lj; m++)
    if (a.type[li] == a.lj_t[2 * m] && a.type[lj] == a.lj_t[2 * m + 1]) att = true;
  a.att_tab[idx] = att ? 1 : 0;
}

// The FP64 terms of one pair (i, j) within reach, credited to i (src/energies.cpp:40-89), with the
// distance-independent factors from k_energy_tables.  Out of line, so that none of its FP64
// work is scheduled into the pair loop's float test.
__device__ __noinline__ void pair_energy(const EnergyArgs& a, const SysParams& P, int gi, int gj, int lj_, int li,
                                         double qi, double sgi, bool elec, bool lj, double e_cut_el, double& ce,
                                         double& ne) {
  const double kappa = a.kappa, lb = a.lb, ecut = a.ecut, ecut_el = a.ecut_el;
  const int np = a.L.np, idx = li * np + lj_;
  const double qj = a.q[lj_];
  double x, y, z;
  ddiff(a, P.fx_to_len, gi, gj, x, y, z);
  const double r = sqrt(x * x + y * y + z * z);
  const double shc = (sgi + a.sigma[lj_]) / 2;
  const double ys = a.pair_tab[idx];
  if (elec && r < ecut_el && ecut_el != 0) {
    ce += ys * ((qi * qj * lb * exp(-kappa * r)) / r - ((qi * qj * lb * e_cut_el) / ecut_el));
  } else if (elec && ecut_el == 0) {
    ce += (qi * qj * lb * exp(-kappa * r) * ys) / r;
  }
  if (r >= ecut && r >= (1.12246205 * shc)) return;
  if (lj) {
    const double s6 = a.pair_tab[np * np + idx];
    const double r3 = r * r * r, r6 = r3 * r3;
    const double q6 = s6 / r6;
    const bool att = a.att_tab[idx] != 0;
    if (r < (1.12246205 * shc) && !att) {
      ne += (4 * q6 * (q6 - 1)) + 1;
    } else if (r < ecut && att) {
      ne += (4 * a.elj_att * q6 * (q6 - 1)) - a.pair_tab[2 * np * np + idx];
    }
  }
}

// One warp per bead i; lane L tests the partners j = i + 1 + L, i + 33 + L, ... of the whole
// system with integer and FP32 work only: the partner's template index is the .w of its position
// entry, "same subunit" is a range test on the index, "both charged" reads per-template flags in
// shared memory, then a float distance test with a conservative margin.  The few partners that
// pass go into a per-warp queue in shared memory (in lane order, by ballot), and the FP64 pair
// terms run 32 queued pairs at a time with every lane busy: GB300's FP64 unit is a small fraction
// of its FP32 rate, and with one call per passing lane most of it ran masked.  Each lane sums its
// queue slots in order; the warp then adds the lane sums in a fixed tree: deterministic.
constexpr int kEnergyWarps = 8;
__global__ void __launch_bounds__(32 * kEnergyWarps) k_energy_pairs(EnergyArgs a) {
  __shared__ unsigned char s_charged[kMaxNp];
  __shared__ int2 s_queue[kEnergyWarps][64];
  const SysParams& P = a.sys[a.sysid];
  const int np = a.L.np;
  for (int l = threadIdx.x; l < np; l += blockDim.x) s_charged[l] = a.q[l] != 0.0;  // np <= kMaxNp
  __syncthreads();
  const int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (t >= a.n) return;  // uniform over the warp
  int2* queue = s_queue[threadIdx.x >> 5];
  const int gi = a.n0 + t;
  const int li = gi % np, si = gi / np;
  const int sub_lo = si * np, sub_hi = sub_lo + np;  // global indices of i's subunit
  const int4 pi = a.pos32[gi];
  const double qi = a.q[li], sgi = a.sigma[li];
  const bool ci = qi != 0.0;
  const float unit = P.unit32;
  const double kappa = a.kappa, ecut = a.ecut, ecut_el = a.ecut_el;
  const double e_cut_el = exp(-kappa * ecut_el);  // the shift's exponential, the same for every pair
  const double rmax = fmax(fmax(ecut, ecut_el), 1.12246205 * a.sigma_max);
  const float rmax2 = (float)(rmax * rmax) * 1.001f + 1e-3f;
  // per-axis reach in high-word units (L / 2^32), rounded up with a margin: beyond it on any axis
  // the pair is out of reach without a conversion to floating point
  const int lim = (int)fmin(2147483647.0, ceil(rmax * 1.001 / (double)unit) + 4.0);
  const bool no_dh_cut = (ecut_el == 0.0);
  double ce = 0.0, ne = 0.0;
  int qn = 0;  // queued pairs (uniform over the warp)
  auto run_queue = [&](int count) {  // the first count queue slots, one per lane
    __syncwarp();
    if (lane < count) {
      const int2 e = queue[lane];
      pair_energy(a, P, gi, e.x, e.y & 0xffff, li, qi, sgi, (e.y >> 16) & 1, (e.y >> 17) & 1, e_cut_el, ce, ne);
    }
    __syncwarp();
  };
  const int n_iter = (a.n - (t + 1) + 31) / 32;  // uniform trip count
  for (int it = 0; it < n_iter; it++) {
    const int tj = t + 1 + it * 32 + lane;
    bool pass = false, lj = false, elec = false;
    int4 pj = make_int4(0, 0, 0, 0);
    if (tj < a.n) {
      const int gj = a.n0 + tj;
      pj = __ldg(&a.pos32[gj]);
      lj = gj < sub_lo || gj >= sub_hi;  // different subunits
      elec = ci && s_charged[pj.w];
      if (no_dh_cut && elec) {
        pass = true;
      } else if (elec || lj) {
        const int ix = (int)((unsigned int)pi.x - (unsigned int)pj.x), iy = (int)((unsigned int)pi.y - (unsigned int)pj.y),
                  iz = (int)((unsigned int)pi.z - (unsigned int)pj.z);
        // (abs of the most negative int stays negative and falls through to the float test)
        if (!(abs(ix) > lim || abs(iy) > lim || abs(iz) > lim)) {
          const float dx = (float)ix * unit, dy = (float)iy * unit, dz = (float)iz * unit;
          pass = !(dx * dx + dy * dy + dz * dz > rmax2);
        }
      }
    }
    const unsigned int m = __ballot_sync(0xffffffffu, pass);
    if (pass)
      queue[qn + __popc(m & ((1u << lane) - 1u))] =
          make_int2(a.n0 + tj, pj.w | (elec ? 1 << 16 : 0) | (lj ? 1 << 17 : 0));
    qn += __popc(m);
    if (qn >= 32) {
      run_queue(32);
      if (lane < qn - 32) queue[lane] = queue[32 + lane];
      qn -= 32;
    }
  }
  if (qn > 0) run_queue(qn);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ce += __shfl_xor_sync(0xffffffffu, ce, o);
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
  }
  if (lane == 0) {
    a.ne[t] = ne;
    a.ce[t] = ce;
  }
}

// ---- the pair pass on a cell grid ------------------------------------------------------------
// Pairs farther apart than every cut-off add exactly nothing to the reference's sums, so with a
// DH cut-off only pairs in neighbouring cells of a grid whose cells are at least that reach wide
// are visited: per bead i, the 27 cells around it in a fixed order and, in each, the beads j > i
// in ascending index order; the same float test and the same FP64 pair terms as the all-pairs
// pass.  Cells come from the high words of the fixed-point positions (box [-L/2, L/2) ->
// [0, 2^32)), cell = (u nc) >> 32, exact integer arithmetic.
__device__ __forceinline__ int ecell_axis(int hi, int nc) {
  const unsigned int u = (unsigned int)hi + 0x80000000u;
  return (int)(((unsigned long long)u * (unsigned int)nc) >> 32);
}

__global__ void k_ecell_count(EnergyArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n) return;
  const int4 p = a.pos32[a.n0 + t];
  const int nc = a.nc;
  const int c = (ecell_axis(p.z, nc) * nc + ecell_axis(p.y, nc)) * nc + ecell_axis(p.x, nc);
  a.bead_cell[t] = c;
  atomicAdd(&a.cell_count[c], 1);
}

// exclusive prefix sums of the cell counts, one CTA: each thread a contiguous run of cells
__global__ void __launch_bounds__(1024) k_ecell_scan(EnergyArgs a) {
  __shared__ int s_tot[1024];
  const int ncell = a.nc * a.nc * a.nc;
  const int per = (ncell + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per, b1 = min(ncell, b0 + per);
  int sum = 0;
  for (int c = b0; c < b1; c++) sum += a.cell_count[c];
  s_tot[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {  // inclusive scan of the run totals
    const int v = threadIdx.x >= o ? s_tot[threadIdx.x - o] : 0;
    __syncthreads();
    s_tot[threadIdx.x] += v;
    __syncthreads();
  }
  int off = s_tot[threadIdx.x] - sum;
  for (int c = b0; c < b1; c++) {
    a.cell_start[c] = off;
    off += a.cell_count[c];
  }
  if (threadIdx.x == blockDim.x - 1) a.cell_start[ncell] = s_tot[threadIdx.x];
}

__global__ void k_ecell_scatter(EnergyArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n) return;
  const int c = a.bead_cell[t];
  a.cell_beads[a.cell_start[c] + atomicAdd(&a.cell_fill[c], 1)] = t;
}

// each cell's beads in ascending order (insertion sort: a few beads per cell)
__global__ void k_ecell_sort(EnergyArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.nc * a.nc * a.nc) return;
  int* b = a.cell_beads + a.cell_start[c];
  const int m = a.cell_start[c + 1] - a.cell_start[c];
  for (int i = 1; i < m; i++) {
    const int v = b[i];
    int k = i - 1;
    while (k >= 0 && b[k] > v) {
      b[k + 1] = b[k];
      k--;
    }
    b[k + 1] = v;
  }
}

__global__ void __launch_bounds__(128) k_energy_pairs_cells(EnergyArgs a) {
  __shared__ unsigned char s_charged[kMaxNp];
  const SysParams& P = a.sys[a.sysid];
  const int np = a.L.np;
  for (int l = threadIdx.x; l < np; l += blockDim.x) s_charged[l] = a.q[l] != 0.0;  // np <= kMaxNp
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n) return;
  const int gi = a.n0 + t;
  const int li = gi % np, si = gi / np;
  const int sub_lo = si * np, sub_hi = sub_lo + np;
  const int4 pi = a.pos32[gi];
  const double qi = a.q[li], sgi = a.sigma[li];
  const bool ci = qi != 0.0;
  const float unit = P.unit32;
  const double kappa = a.kappa, ecut = a.ecut, ecut_el = a.ecut_el;
  const double e_cut_el = exp(-kappa * ecut_el);
  const double rmax = fmax(fmax(ecut, ecut_el), 1.12246205 * a.sigma_max);
  const float rmax2 = (float)(rmax * rmax) * 1.001f + 1e-3f;
  const int nc = a.nc;
  const int cx = ecell_axis(pi.x, nc), cy = ecell_axis(pi.y, nc), cz = ecell_axis(pi.z, nc);
  double ce = 0.0, ne = 0.0;
  for (int dz = -1; dz <= 1; dz++) {
    const int z = (cz + dz + nc) % nc;
    for (int dy = -1; dy <= 1; dy++) {
      const int y = (cy + dy + nc) % nc;
      for (int dx = -1; dx <= 1; dx++) {
        const int x = (cx + dx + nc) % nc;
        const int c = (z * nc + y) * nc + x;
        const int e = a.cell_start[c + 1];
        for (int k = a.cell_start[c]; k < e; k++) {
          const int tj = a.cell_beads[k];
          if (tj <= t) continue;
          const int gj = a.n0 + tj;
          const int4 pj = a.pos32[gj];
          const bool lj = gj < sub_lo || gj >= sub_hi;
          const bool elec = ci && s_charged[pj.w];
          if (!(elec || lj)) continue;
          const float ddx = hi_diff(pi.x, pj.x, unit), ddy = hi_diff(pi.y, pj.y, unit), ddz = hi_diff(pi.z, pj.z, unit);
          if (ddx * ddx + ddy * ddy + ddz * ddz > rmax2) continue;
          pair_energy(a, P, gi, gj, pj.w, li, qi, sgi, elec, lj, e_cut_el, ce, ne);
        }
      }
    }
  }
  a.ne[t] = ne;
  a.ce[t] = ce;
}

// Encapsulation big beads (update_LJ_ES_energies_bigbeads, src/energies.cpp:96-137): per
// subunit bead, the unshifted screened Coulomb energy with each big bead inside the DH cut-off
// (none without one) and the shifted WCA energy (+1) inside delta + 2^(1/6) shc, added to the
// bead's ne / ce (the reference credits them to the subunit bead and to the big bead) and kept
// apart for the big-bead totals.  Exact fixed-point differences in double.
__global__ void __launch_bounds__(128) k_energy_bigbeads(EnergyArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n) return;
  const SysParams& P = a.sys[a.sysid];
  const int gi = a.n0 + t, li = gi % a.L.np;
  const double qj = a.q[li], sgj = a.sigma[li];
  const double kappa = a.kappa, lb = a.lb, ecut_el = a.ecut_el;
  const double shc = P.bb_shc_d, sigb = P.bb_sigma_d;
  const double sigavg = (sigb + sgj) / 2;
  const double delta = sigavg - shc;
  const double shc6 = pow(shc, 6);
  const double ys = exp(kappa * sigavg) / ((1 + kappa * sigb / 2) * (1 + kappa * sgj / 2));
  double ce = 0.0, ne = 0.0;
  for (int k = 0; k < P.nbb; k++) {
    const int b = P.bb0 + k;
    const double x = fixed_diff(a.bb_fx[b], a.px[gi], P.fx_to_len);
    const double y = fixed_diff(a.bb_fx[a.bb_total + b], a.py[gi], P.fx_to_len);
    const double z = fixed_diff(a.bb_fx[2 * a.bb_total + b], a.pz[gi], P.fx_to_len);
    const double r = sqrt(x * x + y * y + z * z);
    const double r6 = pow(r - delta, 6);
    if (qj != 0 && r < ecut_el) ce += (P.bb_q * qj * lb * exp(-kappa * r) * ys) / r;
    if (r < delta + 1.12246205 * shc) ne += (4 * (shc6 / r6) * ((shc6 / r6) - 1)) + 1;
  }
  a.ne[t] += ne;
  a.ce[t] += ce;
  a.ne_bb[t] = ne;
  a.ce_bb[t] = ce;
}

// Big-bead energy totals (lj, electrostatic) in bead order with a fixed tree, one CTA.
__global__ void k_energy_bb_totals(EnergyArgs a) {
  __shared__ double red[2][512];
  double s0 = 0, s1 = 0;
  const int per = (a.n + blockDim.x - 1) / blockDim.x;
  const int beg = threadIdx.x * per, end = min(a.n, beg + per);
  for (int t = beg; t < end; t++) {
    s0 += a.ne_bb[t];
    s1 += a.ce_bb[t];
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.bb_totals[0] = red[0][0];
    a.bb_totals[1] = red[1][0];
  }
}

// Totals in bead order with a fixed tree: one CTA of 1024 threads per call.
__global__ void k_energy_totals(EnergyArgs a) {
  __shared__ double red[5][1024];
  double s[5] = {0, 0, 0, 0, 0};
  const int per = (a.n + blockDim.x - 1) / blockDim.x;
  const int beg = threadIdx.x * per, end = min(a.n, beg + per);
  for (int t = beg; t < end; t++) {
    s[0] += a.ke[t];
    s[1] += a.se[t];
    s[2] += a.be[t];
    s[3] += a.ne[t];
    s[4] += a.ce[t];
  }
  for (int k = 0; k < 5; k++) red[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 5; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 5; k++) a.totals[k] = red[k][0];
}

}  // namespace souffle

namespace souffle {
void launch_energies(const EnergyArgs& a, int n, cudaStream_t s) {
  const int g = (n + 127) / 128;
  k_energy_bonded<<<g, 128, 0, s>>>(a);
  k_energy_tables<<<(a.L.np * a.L.np + 127) / 128, 128, 0, s>>>(a);
  if (a.nc >= 3) {
    const int ncell = a.nc * a.nc * a.nc;
    cudaMemsetAsync(a.cell_count, 0, sizeof(int) * ncell, s);
    cudaMemsetAsync(a.cell_fill, 0, sizeof(int) * ncell, s);
    k_ecell_count<<<g, 128, 0, s>>>(a);
    k_ecell_scan<<<1, 1024, 0, s>>>(a);
    k_ecell_scatter<<<g, 128, 0, s>>>(a);
    k_ecell_sort<<<(ncell + 127) / 128, 128, 0, s>>>(a);
    k_energy_pairs_cells<<<g, 128, 0, s>>>(a);
  } else {  // no DH cut-off, or a box too small for a 3 x 3 x 3 grid: every pair j > i
    k_energy_pairs<<<(int)(((long long)n + kEnergyWarps - 1) / kEnergyWarps), 32 * kEnergyWarps, 0, s>>>(a);  // a warp per bead
  }
  if (a.bb_totals) {
    k_energy_bigbeads<<<g, 128, 0, s>>>(a);
    k_energy_bb_totals<<<1, 512, 0, s>>>(a);
  }
  k_energy_totals<<<1, 1024, 0, s>>>(a);
}
}  // namespace souffle
