// Per-step force kernel and integrator kernels.
//
// k_forces reproduces forceCalculation (src/forces.cpp:13-171) for a run of subunits per CTA:
//   stretching   BEAD::update_stretching_force (src/bead.cpp:17-23) via EDGE::update_length
//                (src/edge.cpp:35-49)
//   bending      EDGE::update_bending_forces + get_gradS/get_grad0/get_grad1
//                (src/edge.cpp:69-188) over FACE::update_area_normal (src/face.cpp:11-17)
//   pair terms   the neighbour loop of src/forces.cpp:67-145: Debye-Hueckel for charged pairs,
//                then attractive LJ (directed table) or WCA for pairs in different subunits.
// Everything is evaluated in FP32 from exact integer coordinate differences; the per-bead
// partial sums (stretching, bending, intra-subunit DH, inter-subunit pairs) are combined in
// 64-bit fixed point, so the total is independent of summation order.  In MD mode the same
// kernel applies the second velocity half-kick (src/bead.h:113-117, src/md.cpp:450-455),
// reduces kinetic energy and momentum per CTA in a fixed order, and the last CTA of each
// system finishes the Nose-Hoover chain (src/md.cpp:456-460, src/functions.cpp:33-58) and the
// centre-of-mass velocity (src/md.cpp:505-514).
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace souffle {


__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 dvec(int4 a, int4 b, float unit) {
  return f3(hi_diff(a.x, b.x, unit), hi_diff(a.y, b.y, unit), hi_diff(a.z, b.z, unit));
}

// Forces in 64-bit fixed point: 2^32 units per force unit (range +-2^31, resolution 2.3e-10).
__device__ __forceinline__ long long fx64(float v) { return __float2ll_rn(v * 4294967296.0f); }

// Nose-Hoover chain link update, update_chain_xi (src/functions.cpp:33-58).
__device__ void chain_xi(double* xi, const double* q, const double* dof, const double* t, int j,
                         double dt, double ke) {
  if (q[j] == 0) return;
  if (j != 0) {
    xi[j] = xi[j] * exp(-0.5 * dt * xi[j + 1]) +
            0.5 * dt * (1.0 / q[j]) * (q[j - 1] * xi[j - 1] * xi[j - 1] - dof[j] * t[j]) *
                exp(-0.25 * dt * xi[j + 1]);
  } else {
    xi[j] = xi[j] * exp(-0.5 * dt * xi[j + 1]) +
            0.5 * dt * (1.0 / q[j]) * (2 * ke - dof[j] * t[j]) * exp(-0.25 * dt * xi[j + 1]);
  }
}

// Backward half at the start of a step (src/md.cpp:401-406), from (xi, eta) into (xi_b, eta_b).
__device__ void nhc_backward(SysState& s, double dt) {
  for (int j = 0; j < s.m; j++) {
    s.xi_b[j] = s.xi[j];
    s.eta_b[j] = s.eta[j];
  }
  for (int j = s.m - 1; j > -1; j--) chain_xi(s.xi_b, s.q, s.dof, s.t, j, dt, s.ke);
  for (int j = 0; j < s.m; j++)
    if (s.q[j] != 0) s.eta_b[j] = s.eta_b[j] + 0.5 * dt * s.xi_b[j];
  s.expfac = exp(-0.5 * dt * s.xi_b[0]);
}

// Forward half at the end of a step (src/md.cpp:457-460), from (xi_b, eta_b) into (xi, eta).
__device__ void nhc_forward(SysState& s, double dt) {
  for (int j = 0; j < s.m; j++) {
    s.xi[j] = s.xi_b[j];
    s.eta[j] = s.eta_b[j];
  }
  for (int j = 0; j < s.m; j++)
    if (s.q[j] != 0) s.eta[j] = s.eta[j] + 0.5 * dt * s.xi[j];
  for (int j = 0; j < s.m; j++) chain_xi(s.xi, s.q, s.dof, s.t, j, dt, s.ke);
}

__global__ void __launch_bounds__(128) k_forces(ForceArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TplLayout& L = a.L;
  const WorkItem w = a.work[blockIdx.x];
  const SysParams& P = a.sys[w.sys];
  const int np = L.np, ne = L.ne, nf = L.nf, nb = L.nbend;
  const int nbead = w.nsub * np;
  const int bead0 = w.sub_begin * np;  // global index of the first bead

  // shared-memory carve-up (16-byte aligned pieces first)
  float4* s_edge = reinterpret_cast<float4*>(smem);                 // [max_sub * ne]
  float4* s_face = s_edge + a.max_sub * ne;                         // [max_sub * nf]
  float4* s_bend = s_face + a.max_sub * nf;                         // [max_sub * nb * 4]
  int4* s_pos = reinterpret_cast<int4*>(s_bend + a.max_sub * nb * 4);  // [max_sub * np]
  double* s_red = reinterpret_cast<double*>(s_pos + a.max_sub * np);   // [4 * 32]
  float* s_tf = reinterpret_cast<float*>(s_red + 4 * 32);              // [n_float], n_float % 4 == 0
  int* s_ti = reinterpret_cast<int*>(s_tf + L.n_float);                // [n_int], n_int % 4 == 0
  float* s_w = reinterpret_cast<float*>(s_ti + L.n_int);               // [np]

  // template and tile staged with 16-byte loads (all pieces 16-byte aligned, sizes padded)
  {
    const int4* gi = reinterpret_cast<const int4*>(a.tpl_i);
    int4* si = reinterpret_cast<int4*>(s_ti);
    for (int t = threadIdx.x; t < (L.n_int >> 2); t += blockDim.x) si[t] = __ldg(gi + t);
    const float4* gf = reinterpret_cast<const float4*>(a.tpl_f);
    float4* sf = reinterpret_cast<float4*>(s_tf);
    for (int t = threadIdx.x; t < (L.n_float >> 2); t += blockDim.x) sf[t] = __ldg(gf + t);
  }
  for (int t = threadIdx.x; t < np; t += blockDim.x) s_w[t] = a.dh_w[w.sys * np + t];
  for (int t = threadIdx.x; t < nbead; t += blockDim.x) s_pos[t] = a.pos32[bead0 + t];
  __syncthreads();

  const float unit = P.unit32;
  const int* e_pack = s_ti + L.o_edge;
  const int* f_b = s_ti + L.o_face;
  const int* bq = s_ti + L.o_bend;
  const int* bf = s_ti + L.o_bendf;
  const float* len0 = s_tf + L.o_len0;

  // edges: length vector and stretching coefficient (len0 - l) ks / l
  for (int t = threadIdx.x; t < w.nsub * ne; t += blockDim.x) {
    const int s = t / ne, e = t - s * ne;
    const int pk = e_pack[e];
    const int4* sp = s_pos + s * np;
    float3 lv = dvec(sp[pk & 0xffff], sp[pk >> 16], unit);
    float l = sqrtf(dot3(lv, lv));
    float coef = (len0[e] - l) * P.ks / l;
    s_edge[t] = make_float4(lv.x, lv.y, lv.z, coef);
  }
  // faces: area vector 1/2 (b1 - b0) x (b2 - b1) and its magnitude
  for (int t = threadIdx.x; t < w.nsub * nf; t += blockDim.x) {
    const int s = t / nf, f = t - s * nf;
    const int4* sp = s_pos + s * np;
    int4 p0 = sp[f_b[3 * f]], p1 = sp[f_b[3 * f + 1]], p2 = sp[f_b[3 * f + 2]];
    float3 A = cross3(dvec(p1, p0, unit), dvec(p2, p1, unit)) * 0.5f;
    s_face[t] = make_float4(A.x, A.y, A.z, sqrtf(dot3(A, A)));
  }
  __syncthreads();
  // bending edges: the four bead contributions of EDGE::update_bending_forces.
  // The in-place normal flip (src/edge.cpp:78-81) makes S = 4 |A0 . A1| whatever the flip history.
  for (int t = threadIdx.x; t < w.nsub * nb; t += blockDim.x) {
    const int s = t / nb, k = t - s * nb;
    const int4* sp = s_pos + s * np;
    const int b0 = bq[4 * k], b1 = bq[4 * k + 1], r2 = bq[4 * k + 2], r3 = bq[4 * k + 3];
    const float4 F0 = s_face[s * nf + bf[2 * k]], F1 = s_face[s * nf + bf[2 * k + 1]];
    const float a0 = F0.w, a1 = F1.w;
    const float S = 4.0f * fabsf(F0.x * F1.x + F0.y * F1.y + F0.z * F1.z);
    const int4 P0 = sp[b0], P1 = sp[b1], P2 = sp[r2], P3 = sp[r3];
    const float3 d01 = dvec(P0, P1, unit), d02 = dvec(P0, P2, unit), d03 = dvec(P0, P3, unit);
    const float3 d12 = dvec(P1, P2, unit), d13 = dvec(P1, P3, unit);
    const float sa0 = S / a0, sa1 = S / a1, q0 = 0.25f / a0, q1 = 0.25f / a1;
    const float kk = P.kb / (a0 * a1 * 4.0f);
    float3 out[4];
    {  // role itsB[0]
      float3 d23 = d13, d32 = d13 * -1.0f, d20 = d01 * -1.0f, d21 = d12;
      float3 c1 = cross3(d20, d21), c2 = cross3(d20, d32);
      float3 gs = f3(d23.y * c1.z - d21.y * c2.z + d32.z * c1.y + d21.z * c2.y,
                     d32.x * c1.z + d21.x * c2.z + d23.z * c1.x - d21.z * c2.x,
                     d23.x * c1.y - d21.x * c2.y + d32.y * c1.x + d21.y * c2.x);
      float3 g0 = cross3(d12, cross3(d02, d01)) * (-q0);
      float3 g1 = cross3(d13, cross3(d03, d01)) * (-q1);
      out[0] = (gs - (g0 * sa0 + g1 * sa1)) * kk;
    }
    {  // role itsB[1]
      float3 d23 = d03, d32 = d03 * -1.0f, d20 = d01, d21 = d02;
      float3 c1 = cross3(d20, d21), c2 = cross3(d20, d32);
      float3 gs = f3(d23.y * c1.z - d21.y * c2.z + d32.z * c1.y + d21.z * c2.y,
                     d32.x * c1.z + d21.x * c2.z + d23.z * c1.x - d21.z * c2.x,
                     d23.x * c1.y - d21.x * c2.y + d32.y * c1.x + d21.y * c2.x);
      float3 g0 = cross3(d02, cross3(d12, d01)) * q0;
      float3 g1 = cross3(d03, cross3(d13, d01)) * q1;
      out[1] = (gs - (g0 * sa0 + g1 * sa1)) * kk;
    }
    {  // role across face 0: r1x = -r13 (the bead of face 1 off the edge)
      float3 gs = cross3(d01, cross3(d01, d13 * -1.0f));
      float3 g0 = cross3(d01, cross3(d02, d01)) * (-q0);
      out[2] = (gs - g0 * sa0) * kk;
    }
    {  // role across face 1: r1x = -r12
      float3 gs = cross3(d01, cross3(d01, d12 * -1.0f));
      float3 g1 = cross3(d01, cross3(d03, d01)) * (-q1);
      out[3] = (gs - g1 * sa1) * kk;
    }
    float4* o = s_bend + (size_t)(s * nb + k) * 4;
#pragma unroll
    for (int r = 0; r < 4; r++) o[r] = make_float4(out[r].x, out[r].y, out[r].z, 0.f);
  }
  __syncthreads();

  const int* bead_edges = s_ti + L.o_bead_edges;
  const int* bead_roles = s_ti + L.o_bead_roles;
  const int* species = s_ti + L.o_species;
  const float kappa = P.kappa;
  const float ecut_el2 = P.ecut_el2;
  const int words = L.words;
  const PairTable& pt = *a.pt;
  const SysState& st = a.state[w.sys];
  const double expfac = st.expfac;
  const double half_dt = 0.5 * P.dt;
  const double sq_e = sqrt(expfac);
  double ke_acc = 0.0, px_acc = 0.0, py_acc = 0.0, pz_acc = 0.0;

  for (int t = threadIdx.x; t < nbead; t += blockDim.x) {
    const int s = t / np, l = t - s * np;
    const int g = bead0 + t;
    const int4* sp = s_pos + s * np;
    const int4 pi = sp[l];
    // stretching, in the bead's edge order
    float3 fs = f3(0.f, 0.f, 0.f);
    for (int k = 0; k < L.maxdeg; k++) {
      int e = bead_edges[l * L.maxdeg + k];
      if (e < 0) break;
      float4 E = s_edge[s * ne + e];
      float c = ((e_pack[e] & 0xffff) == l) ? E.w : -E.w;
      fs = fs + f3(E.x, E.y, E.z) * c;
    }
    // bending, in template edge order
    float3 fb = f3(0.f, 0.f, 0.f);
    for (int k = 0; k < L.maxrole; k++) {
      int r = bead_roles[l * L.maxrole + k];
      if (r < 0) break;
      float4 B = s_bend[(size_t)s * nb * 4 + r];
      fb = fb + f3(B.x, B.y, B.z);
    }
    // intra-subunit pairs: Debye-Hueckel only (same subunit, src/forces.cpp:79-80)
    float3 fe = f3(0.f, 0.f, 0.f);
    const float wi = s_w[l];
    const unsigned int* mrow = a.intra_mask + ((size_t)(w.sub_begin + s) * np + l) * words;
    for (int wd = 0; wd < words; wd++) {
      unsigned int m = mrow[wd];
      while (m) {
        int jj = (wd << 5) + __ffs(m) - 1;
        m &= m - 1;
        float3 d = dvec(pi, sp[jj], unit);
        float r2 = dot3(d, d);
        if (r2 < ecut_el2) {
          float ir = rsqrtf(r2);
          float r = r2 * ir;
          float c = wi * s_w[jj] * __expf(-kappa * r) * (ir * ir) * (kappa + ir);
          fe = fe + d * c;
        }
      }
    }
    // inter-subunit pairs: DH + LJ/WCA
    float3 fp = f3(0.f, 0.f, 0.f);
    const int si = species[l];
    const int nint = a.inter_count[g];
    const int att_row = L.lj_att_bits[si];
    for (int k = 0; k < nint; k++) {
      const int j = a.inter_ids[(size_t)k * a.n_beads_total + g];
      const int4 pj = __ldg(&a.pos32[j]);
      const int lj = pj.w;
      float3 d = dvec(pi, pj, unit);
      float r2 = dot3(d, d);
      float c = 0.f;
      const float wj = s_w[lj];
      if (wi * wj != 0.f && r2 < ecut_el2) {
        float ir = rsqrtf(r2);
        float r = r2 * ir;
        c = wi * wj * __expf(-kappa * r) * (ir * ir) * (kappa + ir);
      }
      const int sj = species[lj];
      const int pidx = si * kMaxSpecies + sj;
      if (r2 < pt.cut2[pidx]) {
        const bool att = (att_row >> sj) & 1;
        const float eps = att ? (((L.type7_bits >> sj) & 1) ? 50.0f : P.elj_att) : 1.0f;
        const float ir2 = 1.0f / r2;
        const float s6 = pt.sig6[pidx] * ir2 * ir2 * ir2;
        c += 48.0f * eps * s6 * (s6 - 0.5f) * ir2;
      }
      fp = fp + d * c;
    }
    // combine in 64-bit fixed point
    long long Fx = fx64(fs.x) + fx64(fb.x) + fx64(fe.x) + fx64(fp.x);
    long long Fy = fx64(fs.y) + fx64(fb.y) + fx64(fe.y) + fx64(fp.y);
    long long Fz = fx64(fs.z) + fx64(fb.z) + fx64(fe.z) + fx64(fp.z);
    const double inv = 1.0 / kTwo32;
    double FX = (double)Fx * inv, FY = (double)Fy * inv, FZ = (double)Fz * inv;
    if (!(isfinite(FX) && isfinite(FY) && isfinite(FZ)) || !(isfinite(fs.x + fb.x + fe.x + fp.x)))
      atomicOr(a.err, kErrNonFinite);
    a.fx[g] = FX;
    a.fy[g] = FY;
    a.fz[g] = FZ;
    if (a.sfx) {
      a.sfx[g] = fs.x; a.sfy[g] = fs.y; a.sfz[g] = fs.z;
      a.bfx[g] = fb.x; a.bfy[g] = fb.y; a.bfz[g] = fb.z;
    }
    if (a.mode == 1) {
      const double c = half_dt * sq_e * a.inv_mass[l];
      double vx = a.vx[g] * expfac + FX * c;
      double vy = a.vy[g] * expfac + FY * c;
      double vz = a.vz[g] * expfac + FZ * c;
      a.vx[g] = vx;
      a.vy[g] = vy;
      a.vz[g] = vz;
      const double m = 1.0 / a.inv_mass[l];
      ke_acc += 0.5 * m * (vx * vx + vy * vy + vz * vz);
      px_acc += vx;
      py_acc += vy;
      pz_acc += vz;
    } else if (a.mode == 2) {
      double vx = a.vx[g], vy = a.vy[g], vz = a.vz[g];
      const double m = 1.0 / a.inv_mass[l];
      ke_acc += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    }
  }
  if (a.mode == 0) return;

  // deterministic CTA reduction: fixed shuffle tree, then warps in order
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ke_acc += __shfl_xor_sync(0xffffffffu, ke_acc, o);
    px_acc += __shfl_xor_sync(0xffffffffu, px_acc, o);
    py_acc += __shfl_xor_sync(0xffffffffu, py_acc, o);
    pz_acc += __shfl_xor_sync(0xffffffffu, pz_acc, o);
  }
  if (lane == 0) {
    s_red[wid * 4 + 0] = ke_acc;
    s_red[wid * 4 + 1] = px_acc;
    s_red[wid * 4 + 2] = py_acc;
    s_red[wid * 4 + 3] = pz_acc;
  }
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) {
    double k = 0, x = 0, y = 0, z = 0;
    for (int q = 0; q < nw; q++) {
      k += s_red[q * 4];
      x += s_red[q * 4 + 1];
      y += s_red[q * 4 + 2];
      z += s_red[q * 4 + 3];
    }
    double4* dst = reinterpret_cast<double4*>(a.partial) + w.slot;
    *dst = make_double4(k, x, y, z);
    __threadfence();
    const int2 sl = a.sys_slots[w.sys];
    unsigned int prev = atomicAdd(&a.state[w.sys].done, 1u);
    last = (prev == (unsigned int)sl.y - 1);
  }
  __syncthreads();
  if (!last) return;

  // Last CTA of this system: all its threads sum the slots (thread t takes slots t, t+blockDim,
  // ... in order, then the fixed shuffle tree and warps in order), so the totals are the same
  // on every run; then thread 0 applies the thermostat and COM updates.
  __threadfence();
  const int2 sl = a.sys_slots[w.sys];
  ke_acc = px_acc = py_acc = pz_acc = 0.0;
  for (int q = threadIdx.x; q < sl.y; q += blockDim.x) {
    const double2* src = reinterpret_cast<const double2*>(a.partial) + 2 * (size_t)(sl.x + q);
    const double2 v0 = __ldcg(src), v1 = __ldcg(src + 1);  // L2 (coherent), not L1
    ke_acc += v0.x;
    px_acc += v0.y;
    py_acc += v1.x;
    pz_acc += v1.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ke_acc += __shfl_xor_sync(0xffffffffu, ke_acc, o);
    px_acc += __shfl_xor_sync(0xffffffffu, px_acc, o);
    py_acc += __shfl_xor_sync(0xffffffffu, py_acc, o);
    pz_acc += __shfl_xor_sync(0xffffffffu, pz_acc, o);
  }
  __syncthreads();
  if (lane == 0) {
    s_red[wid * 4 + 0] = ke_acc;
    s_red[wid * 4 + 1] = px_acc;
    s_red[wid * 4 + 2] = py_acc;
    s_red[wid * 4 + 3] = pz_acc;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double k = 0, x = 0, y = 0, z = 0;
  for (int q = 0; q < nw; q++) {
    k += s_red[q * 4];
    x += s_red[q * 4 + 1];
    y += s_red[q * 4 + 2];
    z += s_red[q * 4 + 3];
  }
  SysState& S = a.state[w.sys];
  S.done = 0;
  S.ke = k;
  if (!isfinite(k)) atomicOr(a.err, kErrNonFinite);
  if (a.mode == 1) {
    nhc_forward(S, P.dt);
    const double inv_n = 1.0 / S.n_beads;
    S.vcom[0] = x * inv_n;
    S.vcom[1] = y * inv_n;
    S.vcom[2] = z * inv_n;
    S.vcom_mag = sqrt(S.vcom[0] * S.vcom[0] + S.vcom[1] * S.vcom[1] + S.vcom[2] * S.vcom[2]);
    S.steps += 1;
  } else {
    S.vcom[0] = S.vcom[1] = S.vcom[2] = 0.0;
  }
  nhc_backward(S, P.dt);
}


// First half-kick and drift with periodic wrap (src/md.cpp:409-414, src/bead.h:72-81,113-117),
// with the pending centre-of-mass velocity of the previous step subtracted first.
__global__ void __launch_bounds__(128) k_drift(DriftArgs a) {
  const WorkItem w = a.work[blockIdx.x];
  const SysParams& P = a.sys[w.sys];
  const SysState& S = a.state[w.sys];
  const double e = S.expfac;
  const double c0 = 0.5 * P.dt * sqrt(e);
  const double vcx = S.vcom[0], vcy = S.vcom[1], vcz = S.vcom[2];
  const double dt_over_L = P.dt / P.box;
  const int n = w.nsub * a.np;
  const int bead0 = w.sub_begin * a.np;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int g = bead0 + t;
    const int l = t % a.np;
    const double c = c0 * a.inv_mass[l];
    double vx = (a.vx[g] - vcx) * e + a.fx[g] * c;
    double vy = (a.vy[g] - vcy) * e + a.fy[g] * c;
    double vz = (a.vz[g] - vcz) * e + a.fz[g] * c;
    a.vx[g] = vx;
    a.vy[g] = vy;
    a.vz[g] = vz;
    long long X = (long long)((unsigned long long)a.px[g] + (unsigned long long)fixed_from_fraction(vx * dt_over_L));
    long long Y = (long long)((unsigned long long)a.py[g] + (unsigned long long)fixed_from_fraction(vy * dt_over_L));
    long long Z = (long long)((unsigned long long)a.pz[g] + (unsigned long long)fixed_from_fraction(vz * dt_over_L));
    a.px[g] = X;
    a.py[g] = Y;
    a.pz[g] = Z;
    a.pos32[g] = make_int4(hi_word(X), hi_word(Y), hi_word(Z), l);
  }
}


// Host state in: double positions to 64-bit fixed point, the float tile copy, velocities.
__global__ void k_state_in(StateArgs a) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n) return;
  const SysParams& P = a.sys[a.bead_sys[g]];
  const double invL = 1.0 / P.box;
  long long X = fixed_from_fraction(a.pos_in[3 * g] * invL);
  long long Y = fixed_from_fraction(a.pos_in[3 * g + 1] * invL);
  long long Z = fixed_from_fraction(a.pos_in[3 * g + 2] * invL);
  a.px[g] = X;
  a.py[g] = Y;
  a.pz[g] = Z;
  a.pos32[g] = make_int4(hi_word(X), hi_word(Y), hi_word(Z), g % a.np);
  if (a.vel_in) {
    a.vx[g] = a.vel_in[3 * g];
    a.vy[g] = a.vel_in[3 * g + 1];
    a.vz[g] = a.vel_in[3 * g + 2];
  } else {
    a.vx[g] = a.vy[g] = a.vz[g] = 0.0;
  }
}

// Device state out, with any pending COM velocity subtracted (what the reference holds after
// src/md.cpp:513-514).
__global__ void k_state_out(StateArgs a) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n) return;
  const int sy = a.bead_sys[g];
  const SysParams& P = a.sys[sy];
  const SysState& S = a.state[sy];
  if (a.pos_out) {
    a.pos_out[3 * g] = (double)a.px[g] * P.fx_to_len;
    a.pos_out[3 * g + 1] = (double)a.py[g] * P.fx_to_len;
    a.pos_out[3 * g + 2] = (double)a.pz[g] * P.fx_to_len;
  }
  if (a.vel_out) {
    a.vel_out[3 * g] = a.vx[g] - S.vcom[0];
    a.vel_out[3 * g + 1] = a.vy[g] - S.vcom[1];
    a.vel_out[3 * g + 2] = a.vz[g] - S.vcom[2];
  }
}

}  // namespace souffle

namespace souffle {
void launch_forces(const ForceArgs& a, int grid, int block, size_t smem, cudaStream_t s) {
  k_forces<<<grid, block, smem, s>>>(a);
}
void launch_drift(const DriftArgs& a, int grid, int block, cudaStream_t s) {
  k_drift<<<grid, block, 0, s>>>(a);
}
void launch_state_in(const StateArgs& a, int grid, int block, cudaStream_t s) {
  k_state_in<<<grid, block, 0, s>>>(a);
}
void launch_state_out(const StateArgs& a, int grid, int block, cudaStream_t s) {
  k_state_out<<<grid, block, 0, s>>>(a);
}
cudaError_t set_kernel_smem(size_t force_smem, size_t pair_smem) {
  cudaError_t e = cudaFuncSetAttribute(k_forces, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)force_smem);
  if (e != cudaSuccess) return e;
  return set_pairs_smem(pair_smem);
}
}  // namespace souffle
