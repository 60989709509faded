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
// A float test on the high words skips pairs beyond every cut-off; the rest use exact
// fixed-point differences in double.
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

// One thread per bead i, j > i over the whole system, tiles of j staged in shared memory.
__global__ void __launch_bounds__(128) k_energy_pairs(EnergyArgs a) {
  __shared__ int4 s_pos[128];
  const SysParams& P = a.sys[a.sysid];
  const int np = a.L.np;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // system-local i
  const bool active = t < a.n;
  const int gi = a.n0 + t;
  const int li = active ? gi % np : 0;
  const int si = active ? gi / np : 0;
  const int4 pi = active ? a.pos32[gi] : make_int4(0, 0, 0, 0);
  const double qi = a.q[li], sgi = a.sigma[li];
  const int ti = a.type[li];
  const float unit = P.unit32;
  const double kappa = a.kappa, lb = a.lb, ecut = a.ecut, ecut_el = a.ecut_el;
  const double ecut3 = ecut * ecut * ecut, ecut6 = ecut3 * ecut3;
  const double rmax = fmax(fmax(ecut, ecut_el), 1.12246205 * a.sigma_max);
  const float rmax2 = (float)(rmax * rmax) * 1.001f + 1e-3f;
  const bool no_dh_cut = (ecut_el == 0.0);
  double ce = 0.0, ne = 0.0;
  const int first_tile = (blockIdx.x * blockDim.x) & ~127;
  for (int base = first_tile; base < a.n; base += 128) {
    __syncthreads();
    if (base + (int)threadIdx.x < a.n) s_pos[threadIdx.x] = a.pos32[a.n0 + base + threadIdx.x];
    __syncthreads();
    if (!active) continue;
    const int jend = min(128, a.n - base);
    for (int k = 0; k < jend; k++) {
      const int tj = base + k;
      if (tj <= t) continue;
      const int gj = a.n0 + tj;
      const int lj_ = gj % np, sj = gj / np;
      const double qj = a.q[lj_];
      const bool elec = (qi != 0 && qj != 0);
      const bool lj = (si != sj);
      if (!(elec || lj)) continue;
      const int4 pj = s_pos[k];
      float dx = hi_diff(pi.x, pj.x, unit), dy = hi_diff(pi.y, pj.y, unit), dz = hi_diff(pi.z, pj.z, unit);
      float r2f = dx * dx + dy * dy + dz * dz;
      if (r2f > rmax2 && !(no_dh_cut && elec)) continue;
      double x, y, z;
      ddiff(a, P.fx_to_len, gi, gj, x, y, z);
      const double r = sqrt(x * x + y * y + z * z);
      const double sgj = a.sigma[lj_];
      const double shc = (sgi + sgj) / 2;
      const double ys = exp(kappa * shc) / ((1 + kappa * sgi / 2) * (1 + kappa * sgj / 2));
      if (elec && r < ecut_el && ecut_el != 0) {
        ce += ys * ((qi * qj * lb * exp(-kappa * r)) / r - ((qi * qj * lb * exp(-kappa * ecut_el)) / ecut_el));
      } else if (elec && ecut_el == 0) {
        ce += (qi * qj * lb * exp(-kappa * r) * ys) / r;
      }
      const double s3 = shc * shc * shc, s6 = s3 * s3;
      const double r3 = r * r * r, r6 = r3 * r3;
      if (r >= ecut && r >= (1.12246205 * shc)) continue;
      if (lj) {
        bool att = false;
        const int tj_ = a.type[lj_];
        for (int m = 0; m < a.n_lj; m++)
          if (ti == a.lj_t[2 * m] && tj_ == a.lj_t[2 * m + 1]) {
            att = true;
            break;
          }
        if (r < (1.12246205 * shc) && !att) {
          ne += (4 * (s6 / r6) * ((s6 / r6) - 1)) + 1;
        } else if (r < ecut && att) {
          ne += (4 * a.elj_att * (s6 / r6) * ((s6 / r6) - 1)) -
                (4 * a.elj_att * ((s6 / ecut6) * ((s6 / ecut6) - 1)));
        }
      }
    }
  }
  if (active) {
    a.ne[t] = ne;
    a.ce[t] = ce;
  }
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
  k_energy_pairs<<<g, 128, 0, s>>>(a);
  if (a.bb_totals) {
    k_energy_bigbeads<<<g, 128, 0, s>>>(a);
    k_energy_bb_totals<<<1, 512, 0, s>>>(a);
  }
  k_energy_totals<<<1, 1024, 0, s>>>(a);
}
}  // namespace souffle
