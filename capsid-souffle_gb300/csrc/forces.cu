// Per-step force kernel and integrator kernels.
//
// k_forces reproduces forceCalculation (src/forces.cpp:13-171) for a run of subunits per CTA:
//   stretching   BEAD::update_stretching_force (src/bead.cpp:17-23) via EDGE::update_length
//                (src/edge.cpp:35-49)
//   bending      EDGE::update_bending_forces + get_gradS/get_grad0/get_grad1
//                (src/edge.cpp:69-188) over FACE::update_area_normal (src/face.cpp:11-17)
//   pair terms   the neighbour loop of src/forces.cpp:67-145: Debye-Hueckel for charged pairs,
//                then attractive LJ (directed table) or WCA for pairs in different subunits.
//   big beads    forceCalculation_bigbead (src/forces.cpp:174-236) when the system has
//                encapsulation big beads: added to the bead's total in the per-bead phase.
// Forces are evaluated in FP32 from exact integer coordinate differences.  Two threads share a
// bead (one takes stretching and the even intra/inter neighbours, the other bending and the odd
// ones); their partial sums are combined in 64-bit fixed point (2^-32 units), so the total does
// not depend on summation order.  In MD mode the kernel applies the second half-kick
// (src/bead.h:113-117, src/md.cpp:450-455) in integer arithmetic, reduces kinetic energy and
// momentum exactly (int64), and the last CTA of each system runs the Nose-Hoover chain
// (src/md.cpp:456-460, 401-406; src/functions.cpp:33-58) and the centre-of-mass velocity
// (src/md.cpp:505-514).  No FP64 instruction runs per bead: GB300's FP64 rate is a small
// fraction of its FP32 rate, so velocities, forces and positions are 64-bit fixed point and
// FP64 is used only for the per-system thermostat scalars.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"
#include "thermostat.cuh"

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

// int64 warp sum with a fixed xor tree (exact, so any order gives the same bits)
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// A bead's force component in 2^-32 fixed point kept as three 21-bit limbs in 32-bit words
// (v = l2 2^42 + l1 2^21 + l0, l0 and l1 in [0, 2^21), l2 signed), so that pair forces can be
// added with native 32-bit shared-memory atomics: the limb sums stay exact for up to 2^11 adds.
__device__ __forceinline__ void limbs_add(unsigned int* L, long long v) {
  atomicAdd(L, (unsigned int)(v & 0x1FFFFF));
  atomicAdd(L + 1, (unsigned int)((v >> 21) & 0x1FFFFF));
  atomicAdd(L + 2, (unsigned int)(int)(v >> 42));
}
__device__ __forceinline__ long long limbs_value(const unsigned int* L) {
  const unsigned long long hi = (unsigned long long)(long long)(int)L[2] << 42;
  return (long long)(hi + ((unsigned long long)L[1] << 21) + (unsigned long long)L[0]);
}

// Encapsulation big beads (forceCalculation_bigbead, src/forces.cpp:192-227) on one subunit bead
// at high words pi (DH weight wl, diameter sl): for each big bead (those flagged in mask, or all),
// r = big - subunit; screened Coulomb q_big q_j lb e^(-kappa r) / r^2 (kappa + 1/r) times the
// Yukawa size factor, and WCA with hard-core distance shc shifted by delta = (sigma_big +
// sigma_j)/2 - shc; the subunit bead takes minus their sum.  Out of line: it runs only for
// systems with big beads and keeps the force kernel's registers for the common path.
__device__ __noinline__ float3 bigbead_force(const ForceArgs& a, const SysParams& P, int4 pi, float wl, float sl,
                                             float unit, const unsigned int* mask) {
  const float kappa = P.kappa;
  const float delta = 0.5f * (P.bb_sigma + sl) - P.bb_shc;
  const float wc = delta + 1.12246205f * P.bb_shc;
  const float s3 = P.bb_shc * P.bb_shc * P.bb_shc, shc6 = s3 * s3;
  float3 fb = f3(0.f, 0.f, 0.f);
  for (int k = 0; k < P.nbb; k++) {
    if (mask) {  // next big bead within reach of the CTA
      const unsigned int m = mask[k >> 5] >> (k & 31);
      if (!m) {
        k |= 31;
        continue;
      }
      k += __ffs(m) - 1;
    }
    const float3 d = dvec(__ldg(&a.bb_pos32[P.bb0 + k]), pi, unit);
    const float r2 = dot3(d, d);
    const float r = sqrtf(r2);
    float c = 0.f;
    if (wl != 0.f && r2 < P.bb_dh_cut2) c = P.bb_w * wl * __expf(-kappa * r) / r2 * (kappa + 1.0f / r);
    if (r2 < wc * wc) {
      const float x = r - delta;
      const float x3 = x * x * x, s6 = shc6 / (x3 * x3);
      c += 48.0f * s6 * (s6 - 0.5f) / r / x;
    }
    fb = fb - d * c;
  }
  return fb;
}

constexpr int kBBWords = 8;   // per-subunit flags for up to 256 big beads (more: all visited)

// Flags the big beads within reach of each of the CTA's nsub subunits (bit k of mask[s * kBBWords
// ...]): a subunit's beads lie within R of its centre bead (R from the coordinates relative to
// the centre bead, s_rel), and a big bead farther than R + the reach of every big-bead pair term
// (bb_reach2, with a 1 % margin) acts on none of them.  A warp per subunit; all threads of the
// CTA call it.
__device__ __noinline__ void bigbead_mask(const ForceArgs& a, const SysParams& P, const int4* s_pos,
                                          const float4* s_rel, int nsub, int np, float unit, unsigned int* mask) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const float reach = sqrtf(P.bb_reach2);
  for (int s = wid; s < nsub; s += nw) {
    float r2 = 0.f;
    for (int l = lane; l < np; l += 32) {
      const float4 q = s_rel[s * np + l];
      r2 = fmaxf(r2, q.x * q.x + q.y * q.y + q.z * q.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, o));
    const float lim = sqrtf(r2) * 1.01f + reach;
    const int4 c = s_pos[s * np + P.center_local];
    for (int k = lane; k < P.nbb; k += 32) {
      const float3 d = dvec(__ldg(&a.bb_pos32[P.bb0 + k]), c, unit);
      if (dot3(d, d) < lim * lim) atomicOr(&mask[s * kBBWords + (k >> 5)], 1u << (k & 31));
    }
  }
}

// 5 CTAs of 256 threads per SM (<= 51 registers) so 3-subunit work items fit one wave of
// 152 x 5 CTAs at the 2000-subunit workload.
// kChain64: the tail runs the FP64 validation chain (souffle_options.chain_fp64) instead of the
// double-float one; a separate instantiation, so that the default kernel's code is untouched.
template <bool kChain64>
__global__ void __launch_bounds__(256, 5) k_forces(ForceArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TplLayout& L = a.L;
  const WorkItem w = a.work[blockIdx.x];
  const SysParams& P = a.sys[w.sys];
  const int np = L.np, ne = L.ne, nb = L.nbend;
  const int nbead = w.nsub * np;
  const int bead0 = w.sub_begin * np;  // global index of the first bead

  // shared-memory carve-up (16-byte aligned pieces first)
  float4* s_edge = reinterpret_cast<float4*>(smem);                 // [max_sub * ne]
  float4* s_bend = s_edge + a.max_sub * ne;                         // [max_sub * nb * 4]
  // (the tail of the system's last CTA reuses this first region for the system state)
  int4* s_pos = reinterpret_cast<int4*>(smem + force_tile_bytes(a.max_sub, ne, nb));  // [max_sub * np]
  float4* s_rel = reinterpret_cast<float4*>(s_pos + a.max_sub * np);   // [max_sub * np]
  long long* s_red = reinterpret_cast<long long*>(s_rel + a.max_sub * np);  // [4 * warps]
  unsigned int* s_F = reinterpret_cast<unsigned int*>(s_red + 4 * (blockDim.x >> 5));  // [force_slot_len(max_sub * np)]
  int* s_pref = reinterpret_cast<int*>(s_F + force_slot_len(a.max_sub * np));  // [force_pref_len(...)]
  float* tpl_f = reinterpret_cast<float*>(s_pref + force_pref_len(a.max_sub * np));  // [n_float], n_float % 4 == 0
  int* tpl_i = reinterpret_cast<int*>(tpl_f + L.n_float);                    // [n_int], n_int % 4 == 0
  float* s_w = reinterpret_cast<float*>(tpl_i + L.n_int);                    // [np]

  {  // the template tables, one copy per CTA
    const int4* gi = reinterpret_cast<const int4*>(a.tpl_i);
    int4* si = reinterpret_cast<int4*>(tpl_i);
    for (int t = threadIdx.x; t < (L.n_int >> 2); t += blockDim.x) si[t] = __ldg(gi + t);
    const float4* gf = reinterpret_cast<const float4*>(a.tpl_f);
    float4* sf = reinterpret_cast<float4*>(tpl_f);
    for (int t = threadIdx.x; t < (L.n_float >> 2); t += blockDim.x) sf[t] = __ldg(gf + t);
  }
  for (int t = threadIdx.x; t < np; t += blockDim.x) s_w[t] = a.dh_w[w.sys * np + t];
  const float unit = P.unit32;
  // the tile: exact high words for the bonded terms, and for the intra-subunit Debye-Hueckel
  // loop float coordinates relative to the subunit's centre bead (|r| within the subunit radius)
  // with the bead's DH weight in .w
  for (int t = threadIdx.x; t < nbead; t += blockDim.x) {
    const int4 p = a.pos32[bead0 + t];
    const int l = t % np;
    const int4 c = __ldg(&a.pos32[bead0 + (t - l) + P.center_local]);
    s_pos[t] = p;
    s_rel[t] = make_float4(hi_diff(p.x, c.x, unit), hi_diff(p.y, c.y, unit), hi_diff(p.z, c.z, unit),
                           __ldg(&a.dh_w[w.sys * np + l]));
  }
  for (int t = threadIdx.x; t < 9 * nbead; t += blockDim.x) s_F[t] = 0u;  // the beads' force limbs
  // big beads within reach of each of the CTA's subunits (s_bbm), flagged before phase 3
  __shared__ unsigned int s_bbm[16 * kBBWords];
  const bool bb_filter = P.nbb > 0 && P.nbb <= 32 * kBBWords && w.nsub <= 16;
  if (threadIdx.x < 16 * kBBWords) s_bbm[threadIdx.x] = 0u;
  // exclusive prefix sums of the beads' inter-subunit list lengths (s_pref[nbead] = total): each
  // thread a run of `per` beads, a warp scan, then the warp totals (s_red is free until the end)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int per = (nbead + blockDim.x - 1) / blockDim.x;
  int my_cnt = 0;
  for (int i = 0; i < per; i++) {
    const int b = threadIdx.x * per + i;
    if (b < nbead) my_cnt += __ldg(a.inter_count + bead0 + b);
  }
  int incl = my_cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  int* s_wtot = reinterpret_cast<int*>(s_red);
  if (lane == 31) s_wtot[wid] = incl;
  __syncthreads();
  {
    int off = incl - my_cnt;
    for (int q = 0; q < wid; q++) off += s_wtot[q];
    for (int i = 0; i < per; i++) {
      const int b = threadIdx.x * per + i;
      if (b < nbead) {
        s_pref[b] = off;
        off += __ldg(a.inter_count + bead0 + b);
      }
    }
    if (threadIdx.x == blockDim.x - 1) s_pref[nbead] = off;
  }

  const int* e_pack = tpl_i + L.o_edge;
  const int* f_b = tpl_i + L.o_face;
  const int* bq = tpl_i + L.o_bend;
  const int* bf = tpl_i + L.o_bendf;
  const float* len0 = tpl_f + L.o_len0;

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
  // bending edges: the four bead contributions of EDGE::update_bending_forces.
  // The in-place normal flip (src/edge.cpp:78-81) makes S = 4 |A0 . A1| whatever the flip history.
  for (int t = threadIdx.x; t < w.nsub * nb; t += blockDim.x) {
    const int s = t / nb, k = t - s * nb;
    const int4* sp = s_pos + s * np;
    const int b0 = bq[4 * k], b1 = bq[4 * k + 1], r2 = bq[4 * k + 2], r3 = bq[4 * k + 3];
    const float beta0 = tpl_f[L.o_beta0 + k];
    if (beta0 != 0.f) {
      // rest-angle option (no reference counterpart): E = kb (1 - cos(beta - beta0)) with beta
      // the signed bend angle of (across0, b0, b1, across1); -dE/dx = -kb sin(beta - beta0)
      // dbeta/dx, dbeta/dx the dihedral gradient (Blondel and Karplus 1996)
      const int4 Q0 = sp[b0], Q1 = sp[b1], Q2 = sp[r2], Q3 = sp[r3];
      const float3 v1 = dvec(Q0, Q2, unit), v2 = dvec(Q1, Q0, unit), v3 = dvec(Q3, Q1, unit);
      const float3 m = cross3(v1, v2), n = cross3(v2, v3);
      const float l2 = dot3(v2, v2), nv2 = sqrtf(l2);
      const float beta = atan2f(-nv2 * dot3(v1, n), -dot3(m, n));
      const float c = -P.kb * sinf(beta - beta0);
      const float3 ga0 = m * (-nv2 / dot3(m, m)), ga1 = n * (nv2 / dot3(n, n));
      const float p = dot3(v1, v2) / l2, q = dot3(v3, v2) / l2;
      const float3 gb0 = ga0 * (-(1.0f + p)) + ga1 * q, gb1 = ga0 * p - ga1 * (1.0f + q);
      float4* o = s_bend + (size_t)(s * nb + k) * 4;
      o[0] = make_float4(gb0.x * c, gb0.y * c, gb0.z * c, 0.f);
      o[1] = make_float4(gb1.x * c, gb1.y * c, gb1.z * c, 0.f);
      o[2] = make_float4(ga0.x * c, ga0.y * c, ga0.z * c, 0.f);
      o[3] = make_float4(ga1.x * c, ga1.y * c, ga1.z * c, 0.f);
      continue;
    }
    // the edge's two faces: area vector 1/2 (b1 - b0) x (b2 - b1) and its magnitude
    auto face = [&](int f) {
      const int4 p0 = sp[f_b[3 * f]], p1 = sp[f_b[3 * f + 1]], p2 = sp[f_b[3 * f + 2]];
      const float3 A = cross3(dvec(p1, p0, unit), dvec(p2, p1, unit)) * 0.5f;
      return make_float4(A.x, A.y, A.z, sqrtf(dot3(A, A)));
    };
    const float4 F0 = face(bf[2 * k]), F1 = face(bf[2 * k + 1]);
    const float a0 = F0.w, a1 = F1.w;
    const float S = 4.0f * fabsf(F0.x * F1.x + F0.y * F1.y + F0.z * F1.z);
    const int4 P0 = sp[b0], P1 = sp[b1], P2 = sp[r2], P3 = sp[r3];
    const float3 d01 = dvec(P0, P1, unit), d02 = dvec(P0, P2, unit), d03 = dvec(P0, P3, unit);
    const float3 d12 = dvec(P1, P2, unit), d13 = dvec(P1, P3, unit);
    const float sa0 = S / a0, sa1 = S / a1, q0 = 0.25f / a0, q1 = 0.25f / a1;
    const float kk = P.kb / (a0 * a1 * 4.0f);
    float4* o = s_bend + (size_t)(s * nb + k) * 4;
    {  // role itsB[0]
      float3 d23 = d13, d32 = d13 * -1.0f, d20 = d01 * -1.0f, d21 = d12;
      float3 c1 = cross3(d20, d21), c2 = cross3(d20, d32);
      float3 gs = f3(d23.y * c1.z - d21.y * c2.z + d32.z * c1.y + d21.z * c2.y,
                     d32.x * c1.z + d21.x * c2.z + d23.z * c1.x - d21.z * c2.x,
                     d23.x * c1.y - d21.x * c2.y + d32.y * c1.x + d21.y * c2.x);
      float3 g0 = cross3(d12, cross3(d02, d01)) * (-q0);
      float3 g1 = cross3(d13, cross3(d03, d01)) * (-q1);
      float3 r = (gs - (g0 * sa0 + g1 * sa1)) * kk;
      o[0] = make_float4(r.x, r.y, r.z, 0.f);
    }
    {  // role itsB[1]
      float3 d23 = d03, d32 = d03 * -1.0f, d20 = d01, d21 = d02;
      float3 c1 = cross3(d20, d21), c2 = cross3(d20, d32);
      float3 gs = f3(d23.y * c1.z - d21.y * c2.z + d32.z * c1.y + d21.z * c2.y,
                     d32.x * c1.z + d21.x * c2.z + d23.z * c1.x - d21.z * c2.x,
                     d23.x * c1.y - d21.x * c2.y + d32.y * c1.x + d21.y * c2.x);
      float3 g0 = cross3(d02, cross3(d12, d01)) * q0;
      float3 g1 = cross3(d03, cross3(d13, d01)) * q1;
      float3 r = (gs - (g0 * sa0 + g1 * sa1)) * kk;
      o[1] = make_float4(r.x, r.y, r.z, 0.f);
    }
    {  // role across face 0: r1x = -r13 (the bead of face 1 off the edge)
      float3 gs = cross3(d01, cross3(d01, d13 * -1.0f));
      float3 g0 = cross3(d01, cross3(d02, d01)) * (-q0);
      float3 r = (gs - g0 * sa0) * kk;
      o[2] = make_float4(r.x, r.y, r.z, 0.f);
    }
    {  // role across face 1: r1x = -r12
      float3 gs = cross3(d01, cross3(d01, d12 * -1.0f));
      float3 g1 = cross3(d01, cross3(d03, d01)) * (-q1);
      float3 r = (gs - g1 * sa1) * kk;
      o[3] = make_float4(r.x, r.y, r.z, 0.f);
    }
  }
  __syncthreads();

  const int* bead_edges = tpl_i + L.o_bead_edges;
  const int* bead_roles = tpl_i + L.o_bead_roles;
  const int* species = tpl_i + L.o_species;
  const float* s_mass = tpl_f + L.o_mass;
  const float kappa = P.kappa;
  const float ecut_el2 = P.ecut_el2;
  const int words = L.words;
  const PairTable& pt = *a.pt;
  const SysState& st = a.state[w.sys];
  const long long delta_fx = st.delta_fx;
  const long long* kick_c = a.kick_c + (size_t)w.sys * np;
  long long ke_acc = 0, px_acc = 0, py_acc = 0, pz_acc = 0;
  const int h = threadIdx.x & 1;
  const bool bd = P.brownian && a.mode == 1;  // Brownian MD step
  const unsigned int parity = h ? 0xAAAAAAAAu : 0x55555555u;
  const int half = blockDim.x >> 1;

  // Phase 1: bonded forces and intra-subunit Debye-Hueckel pairs, two threads per bead: thread
  // h = 0 the stretching terms, h = 1 the bending terms, and each its parity of the bead's
  // intra-subunit row.  The pair's sum is added to the bead's fixed-point limbs in s_F.
  // (uniform trip count so the pair shuffle always has both lanes)
  for (int base = 0; base < nbead; base += half) {
    const int t = base + (threadIdx.x >> 1);
    const bool act = t < nbead;
    long long Fx = 0, Fy = 0, Fz = 0;
    if (act) {
      const int s = t / np;
      const int l = t - s * np;
      const int g = bead0 + t;
      float3 fown = f3(0.f, 0.f, 0.f);
      if (h == 0) {  // stretching, in the bead's edge order
        for (int k = 0; k < L.maxdeg; k++) {
          int e = bead_edges[l * L.maxdeg + k];
          if (e < 0) break;
          float4 E = s_edge[s * ne + e];
          float c = ((e_pack[e] & 0xffff) == l) ? E.w : -E.w;
          fown = fown + f3(E.x, E.y, E.z) * c;
        }
        if (a.sfx) { a.sfx[g] = fown.x; a.sfy[g] = fown.y; a.sfz[g] = fown.z; }
      } else {  // bending, in template edge order
        for (int k = 0; k < L.maxrole; k++) {
          int r = bead_roles[l * L.maxrole + k];
          if (r < 0) break;
          float4 B = s_bend[(size_t)s * nb * 4 + r];
          fown = fown + f3(B.x, B.y, B.z);
        }
        if (a.bfx) { a.bfx[g] = fown.x; a.bfy[g] = fown.y; a.bfz[g] = fown.z; }
      }
      // intra-subunit pairs (Debye-Hueckel only: same subunit, src/forces.cpp:79-80), this
      // thread's parity of the row
      float3 fe = f3(0.f, 0.f, 0.f);
      const float4* sr = s_rel + s * np;
      const float4 ri = sr[l];
      const unsigned int* mrow = a.intra_mask + ((size_t)(w.sub_begin + s) * np + l) * words;
      for (int wd = 0; wd < words; wd++) {
        unsigned int m = __ldg(mrow + wd) & parity;
        // two pairs per iteration (independent chains for the scheduler), added in bit order
        while (m) {
          const int j1 = (wd << 5) + __ffs(m) - 1;
          m &= m - 1;
          const bool two = m != 0;
          const int j2 = two ? (wd << 5) + __ffs(m) - 1 : j1;
          m &= m - 1;
          const float4 rj1 = sr[j1], rj2 = sr[j2];
          const float3 d1 = f3(ri.x - rj1.x, ri.y - rj1.y, ri.z - rj1.z);
          const float3 d2 = f3(ri.x - rj2.x, ri.y - rj2.y, ri.z - rj2.z);
          const float r21 = dot3(d1, d1), r22 = dot3(d2, d2);
          const float ir1 = rsqrtf(r21), ir2 = rsqrtf(r22);
          const float c1 = ri.w * rj1.w * __expf(-kappa * (r21 * ir1)) * (ir1 * ir1) * (kappa + ir1);
          const float c2 = ri.w * rj2.w * __expf(-kappa * (r22 * ir2)) * (ir2 * ir2) * (kappa + ir2);
          if (r21 < ecut_el2) fe = fe + d1 * c1;
          if (two && r22 < ecut_el2) fe = fe + d2 * c2;
        }
      }
      float3 fs = f3(0.f, 0.f, 0.f);
      if (a.surr_f && h == 0) {  // far-field subunit pairs from the learned surrogate
        const float4 sv = a.surr_f[g];
        fs = f3(sv.x, sv.y, sv.z);
      }
      const float tx = fown.x + fe.x + fs.x, ty = fown.y + fe.y + fs.y, tz = fown.z + fe.z + fs.z;
      if (!(isfinite(tx) && isfinite(ty) && isfinite(tz)) ||
          fmaxf(fmaxf(fabsf(tx), fabsf(ty)), fabsf(tz)) > 1.0e9f)
        atomicOr(a.err, kErrNonFinite);
      Fx = f32_to_fx32(fown.x) + f32_to_fx32(fe.x) + f32_to_fx32(fs.x);
      Fy = f32_to_fx32(fown.y) + f32_to_fx32(fe.y) + f32_to_fx32(fs.y);
      Fz = f32_to_fx32(fown.z) + f32_to_fx32(fe.z) + f32_to_fx32(fs.z);
    }
    // the pair's total, exact in fixed point
    Fx += __shfl_xor_sync(0xffffffffu, Fx, 1);
    Fy += __shfl_xor_sync(0xffffffffu, Fy, 1);
    Fz += __shfl_xor_sync(0xffffffffu, Fz, 1);
    if (act && h == 0) {
      limbs_add(s_F + 9 * t, Fx);
      limbs_add(s_F + 9 * t + 3, Fy);
      limbs_add(s_F + 9 * t + 6, Fz);
    }
  }
  // (no barrier: phase 2 adds into the same zeroed limbs, in any order)

  // Phase 2: inter-subunit pairs (DH + LJ/WCA, src/forces.cpp:81-138).  The CTA's beads' lists
  // are one flat sequence (s_pref: exclusive prefix sums of their lengths) cut into equal
  // contiguous runs, one per thread, so a bead with a long list does not hold up its CTA.  A
  // thread walks its run bead by bead, sums the pair forces of each bead exactly in 2^-32 fixed
  // point in registers and adds the sum to the bead's limbs when it moves to the next bead
  // (order-independent, deterministic).
  {
    const int n_inter = s_pref[nbead];
    const int run = (n_inter + blockDim.x - 1) / blockDim.x;
    int p = threadIdx.x * run;
    const int pend = min(n_inter, p + run);
    if (p < pend) {
      int lo = 0, hi = nbead;  // s_pref[lo] <= p < s_pref[hi]: the run starts in bead lo
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_pref[mid] <= p) lo = mid;
        else hi = mid;
      }
      int b = lo, l = b % np, bend = s_pref[b + 1];
      int4 pi = s_pos[b];
      int si = species[l];
      float wi = s_w[l];
      // the row of bead b holds its pairs s_pref[b] .. s_pref[b + 1] - 1 of the flat sequence
      long long row = (long long)(bead0 + b) * a.inter_cap - s_pref[b];
      long long ax = 0, ay = 0, az = 0;
      for (; p < pend; p++) {
        if (p >= bend) {  // next bead with pairs: add this bead's sums to its limbs
          limbs_add(s_F + 9 * b, ax);
          limbs_add(s_F + 9 * b + 3, ay);
          limbs_add(s_F + 9 * b + 6, az);
          ax = ay = az = 0;
          do {
            b++;
            bend = s_pref[b + 1];
          } while (p >= bend);
          l = b % np;
          pi = s_pos[b];
          si = species[l];
          wi = s_w[l];
          row = (long long)(bead0 + b) * a.inter_cap - s_pref[b];
        }
        const int j = __ldg(a.inter_ids + (row + p));
        const int4 pj = __ldg(&a.pos32[j]);
        const int lj = pj.w;
        const float3 d = dvec(pi, pj, unit);
        const float r2 = dot3(d, d);
        float c = 0.f;
        const float wj = s_w[lj];
        if (wi * wj != 0.f && r2 < ecut_el2) {
          const float ir = rsqrtf(r2);
          const float r = r2 * ir;
          c = wi * wj * __expf(-kappa * r) * (ir * ir) * (kappa + ir);
        }
        const int sj = species[lj];
        const int pidx = si * kMaxSpecies + sj;
        if (r2 < pt.cut2[pidx]) {
          const bool att = (L.lj_att_bits[si] >> sj) & 1;
          const float eps = att ? (((L.type7_bits >> sj) & 1) ? 50.0f : P.elj_att) : 1.0f;
          const float ir2 = 1.0f / r2;
          const float s6 = pt.sig6[pidx] * ir2 * ir2 * ir2;
          c += 48.0f * eps * s6 * (s6 - 0.5f) * ir2;
        }
        const float3 f = d * c;
        if (!(isfinite(f.x) && isfinite(f.y) && isfinite(f.z)) ||
            fmaxf(fmaxf(fabsf(f.x), fabsf(f.y)), fabsf(f.z)) > 1.0e9f) {
          atomicOr(a.err, kErrNonFinite);
          continue;
        }
        ax += f32_to_fx32(f.x);
        ay += f32_to_fx32(f.y);
        az += f32_to_fx32(f.z);
      }
      limbs_add(s_F + 9 * b, ax);
      limbs_add(s_F + 9 * b + 3, ay);
      limbs_add(s_F + 9 * b + 6, az);
    }
  }
  if (bb_filter) bigbead_mask(a, P, s_pos, s_rel, w.nsub, np, unit, s_bbm);
  __syncthreads();

  // Phase 3: the bead's total force, the second half kick and the kinetic-energy and momentum
  // sums, one thread per bead
  for (int t = threadIdx.x; t < nbead; t += blockDim.x) {
    const int l = t % np, g = bead0 + t;
    long long Fx = limbs_value(s_F + 9 * t), Fy = limbs_value(s_F + 9 * t + 3), Fz = limbs_value(s_F + 9 * t + 6);
    if (P.nbb) {
      const float3 fb = bigbead_force(a, P, s_pos[t], s_w[l], tpl_f[L.o_sigma + l], unit,
                                      bb_filter ? s_bbm + (t / np) * kBBWords : nullptr);
      if (!(isfinite(fb.x) && isfinite(fb.y) && isfinite(fb.z)) ||
          fmaxf(fmaxf(fabsf(fb.x), fabsf(fb.y)), fabsf(fb.z)) > 1.0e9f)
        atomicOr(a.err, kErrNonFinite);
      Fx += f32_to_fx32(fb.x);
      Fy += f32_to_fx32(fb.y);
      Fz += f32_to_fx32(fb.z);
    }
    if (bd) {
      // Brownian: tforce + (fran - mean fran over the system) + fdrag (src/md.cpp:468-494,
      // src/bead.h:147-149)
      const long long N = a.n_beads_total;
      Fx += a.fran[g] - __double2ll_rn((double)st.fran_sum[0] * st.inv_n) + a.fdrag[g];
      Fy += a.fran[N + g] - __double2ll_rn((double)st.fran_sum[1] * st.inv_n) + a.fdrag[N + g];
      Fz += a.fran[2 * N + g] - __double2ll_rn((double)st.fran_sum[2] * st.inv_n) + a.fdrag[2 * N + g];
    }
    a.fx[g] = Fx;
    a.fy[g] = Fy;
    a.fz[g] = Fz;
    if (a.mode == 1 || a.mode == 2) {
      long long vx = a.vx[g], vy = a.vy[g], vz = a.vz[g];
      if (a.mode == 1) {  // v <- v exp(-dt xi/2) + F dt sqrt(expfac)/(2m)  (src/bead.h:113-117)
        const long long c = kick_c[l];
        vx = vx - mul_shr(vx, delta_fx, 62) + mul_shr(Fx, c, 56);
        vy = vy - mul_shr(vy, delta_fx, 62) + mul_shr(Fy, c, 56);
        vz = vz - mul_shr(vz, delta_fx, 62) + mul_shr(Fz, c, 56);
        a.vx[g] = vx;
        a.vy[g] = vy;
        a.vz[g] = vz;
        px_acc += vx;
        py_acc += vy;
        pz_acc += vz;
      }
      const float ux = vel_to_f32(vx), uy = vel_to_f32(vy), uz = vel_to_f32(vz);
      const float v2 = ux * ux + uy * uy + uz * uz;
      if (!(v2 < 1.0e12f)) atomicOr(a.err, kErrNonFinite);  // |v| beyond 1e6: a blown-up run
      ke_acc += f32_to_fx32(0.5f * s_mass[l] * v2);
    }
  }
  if (a.mode == 0) return;

  // exact CTA reduction in int64
  ke_acc = warp_sum_ll(ke_acc);
  px_acc = warp_sum_ll(px_acc);
  py_acc = warp_sum_ll(py_acc);
  pz_acc = warp_sum_ll(pz_acc);
  if (lane == 0) {
    s_red[wid * 4 + 0] = ke_acc;
    s_red[wid * 4 + 1] = px_acc;
    s_red[wid * 4 + 2] = py_acc;
    s_red[wid * 4 + 3] = pz_acc;
  }
  __syncthreads();
  __shared__ bool last;
  // the system's running sums (kinetic energy, momentum) for this launch: exact int64 adds,
  // order-independent; the last CTA reads them and clears them for the next launch
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(a.partial) + 4 * (size_t)w.sys;
  if (threadIdx.x == 0) {
    long long k = 0, x = 0, y = 0, z = 0;
    for (int q = 0; q < nw; q++) {
      k += s_red[q * 4];
      x += s_red[q * 4 + 1];
      y += s_red[q * 4 + 2];
      z += s_red[q * 4 + 3];
    }
    atomicAdd(acc + 0, (unsigned long long)k);
    atomicAdd(acc + 1, (unsigned long long)x);
    atomicAdd(acc + 2, (unsigned long long)y);
    atomicAdd(acc + 3, (unsigned long long)z);
    __threadfence();
    const int2 sl = a.sys_slots[w.sys];
    unsigned int prev = atomicAdd(&a.state[w.sys].done, 1u);
    last = (prev == (unsigned int)sl.y - 1);
  }
  __syncthreads();
  if (!last) return;

  // Last CTA of this system: the running sums and the system's state come into shared memory
  // (the tile area, free by now) in one round of loads; then warp 0 runs the thermostat chain
  // and warp 1 the centre-of-mass velocity.
  __threadfence();
  static_assert(sizeof(SysState) % 16 == 0, "SysState is copied as int4");
  constexpr int kStateVecs = (int)(sizeof(SysState) / 16);
  SysState& S = *reinterpret_cast<SysState*>(smem);
  dfloat* chain_scratch = reinterpret_cast<dfloat*>(smem + sizeof(SysState));  // 3 kMaxChain
  const int4* st_src = reinterpret_cast<const int4*>(a.state + w.sys);
  int4* st_dst = reinterpret_cast<int4*>(&S);
  long long sum = 0;
  if (threadIdx.x < 4) {
    sum = (long long)__ldcg(acc + threadIdx.x);  // L2 (coherent), not L1
    acc[threadIdx.x] = 0;
  }
  for (int q = threadIdx.x; q < kStateVecs; q += blockDim.x) st_dst[q] = __ldcg(st_src + q);
  if (threadIdx.x < 4) s_red[threadIdx.x] = sum;
  __syncthreads();
  const int vcom_warp = nw > 1 ? 1 : 0;
  if (wid == 0) {
    if (lane == 0) {
      S.done = 0;
      S.ke = df_from_fixed(s_red[0], 2.3283064365386963e-10f);  // 2^-32
      if (a.mode == 1) S.steps += 1;
      if (P.brownian && a.mode == 1) {  // this step's draws are used: next step's generator state
        S.fran_sum[0] = S.fran_sum[1] = S.fran_sum[2] = 0;
        S.lcg = lcg_mul(S.lcg, P.lcg_step);
      }
    }
    __syncwarp();
    if constexpr (kChain64) {  // FP64 validation variant, one thread
      if (lane == 0) {
        Chain64& c = a.chain64[w.sys];
        if (!chain64_tail(c, (double)s_red[0] * 2.3283064365386963e-10, a.mode == 1, S))  // KE: 2^-32 units
          atomicOr(a.err, kErrNonFinite);
      }
      __syncwarp();
    } else {
      if (a.mode == 1) nhc_forward_warp(S, lane, chain_scratch);
      if (!nhc_backward_warp(S, lane, chain_scratch + 2 * kMaxChain)) atomicOr(a.err, kErrNonFinite);
    }
  }
  if (wid == vcom_warp && lane == 0) {
    const long long x = s_red[1], y = s_red[2], z = s_red[3];
    if (a.mode == 1) {
      // mean velocity, removed from every bead before the next kick (src/md.cpp:505-514)
      const double vx = (double)x * S.inv_n, vy = (double)y * S.inv_n, vz = (double)z * S.inv_n;
      S.vcom_fx[0] = __double2ll_rn(vx);
      S.vcom_fx[1] = __double2ll_rn(vy);
      S.vcom_fx[2] = __double2ll_rn(vz);
      S.vcom_mag = sqrt(vx * vx + vy * vy + vz * vz) * (1.0 / kVelScale);
    } else {
      S.vcom_fx[0] = S.vcom_fx[1] = S.vcom_fx[2] = 0;
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kStateVecs; q += blockDim.x) reinterpret_cast<int4*>(a.state + w.sys)[q] = st_dst[q];
  // per-bead kick coefficients c0 / m, one template bead per thread
  long long* kc = a.kick_c + (size_t)w.sys * np;
  for (int l = threadIdx.x; l < np; l += blockDim.x) {
    long long c = 0;
    if (!nhc_kick_coefficient(S.kick_c0, a.inv_mass[l], c)) atomicOr(a.err, kErrNonFinite);
    kc[l] = c;
  }
}

// Half-kick and drift of one bead (src/md.cpp:409-414, src/bead.h:72-81,113-117), with the
// pending centre-of-mass velocity subtracted first; integer arithmetic only (x += v dt is an
// exact multiply into the fixed-point box).
__device__ __forceinline__ void drift_bead(int g, int l, long long c, long long delta_fx, long long vcx, long long vcy,
                                           long long vcz, long long dx_fx, const long long* fx, const long long* fy,
                                           const long long* fz, long long* vxp, long long* vyp, long long* vzp,
                                           long long* px, long long* py, long long* pz, int4* pos32) {
  long long vx = vxp[g] - vcx, vy = vyp[g] - vcy, vz = vzp[g] - vcz;
  vx = vx - mul_shr(vx, delta_fx, 62) + mul_shr(fx[g], c, 56);
  vy = vy - mul_shr(vy, delta_fx, 62) + mul_shr(fy[g], c, 56);
  vz = vz - mul_shr(vz, delta_fx, 62) + mul_shr(fz[g], c, 56);
  vxp[g] = vx;
  vyp[g] = vy;
  vzp[g] = vz;
  const long long X = (long long)((unsigned long long)px[g] + (unsigned long long)mul_shr(vx, dx_fx, 40));
  const long long Y = (long long)((unsigned long long)py[g] + (unsigned long long)mul_shr(vy, dx_fx, 40));
  const long long Z = (long long)((unsigned long long)pz[g] + (unsigned long long)mul_shr(vz, dx_fx, 40));
  px[g] = X;
  py[g] = Y;
  pz[g] = Z;
  pos32[g] = make_int4(hi_word(X), hi_word(Y), hi_word(Z), l);
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// First half-kick and drift with periodic wrap (src/md.cpp:409-414, src/bead.h:72-81,113-117),
// with the pending centre-of-mass velocity of the previous step subtracted first.  Integer
// arithmetic only: x += v dt is an exact multiply into the fixed-point box.
__global__ void __launch_bounds__(256) k_drift(DriftArgs a) {
  const WorkItem w = a.work[blockIdx.x];
  const SysParams& P = a.sys[w.sys];
  SysState& S = a.state[w.sys];
  const long long delta_fx = S.delta_fx;
  const long long vcx = S.vcom_fx[0], vcy = S.vcom_fx[1], vcz = S.vcom_fx[2];
  const long long dx_fx = P.drift_fx;
  const long long* kick_c = a.kick_c + (size_t)w.sys * a.np;
  const int n = w.nsub * a.np;
  const int bead0 = w.sub_begin * a.np;
  const int half = blockDim.x >> 1;
  if (P.brownian) {
    // Brownian step, first half (src/md.cpp:415-421): drag -m v / damp from the velocity after
    // the last centre-of-mass removal, half-kick with the stored total force, drift; then this
    // step's random forces (src/md.cpp:461-467): bead k of the system takes draws 6k+1 .. 6k+6
    // of the generator after the previous steps' draws (x, y, z: two draws each)
    const long long N = a.n_total;
    long long sx = 0, sy = 0, sz = 0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int g = bead0 + t, l = t % a.np;
      const long long dc = a.bd_drag[(size_t)w.sys * a.np + l];
      const long long vx = a.vx[g] - vcx, vy = a.vy[g] - vcy, vz = a.vz[g] - vcz;
      a.fdrag[g] = -mul_shr(vx, dc, 48);
      a.fdrag[N + g] = -mul_shr(vy, dc, 48);
      a.fdrag[2 * N + g] = -mul_shr(vz, dc, 48);
      drift_bead(g, l, kick_c[l], 0, vcx, vcy, vcz, dx_fx, a.fx, a.fy, a.fz, a.vx, a.vy, a.vz, a.px, a.py, a.pz,
                 a.pos32);
      unsigned int x = lcg_mul(S.lcg, a.lcg_table[g - P.bead0]);
      unsigned int d[6];
#pragma unroll
      for (int k = 0; k < 6; k++) d[k] = x = lcg_mul(x, 16807u);
      const double sc = a.bd_noise[(size_t)w.sys * a.np + l];
      const long long rx = __double2ll_rn(__dmul_rn(sc, lcg_uniform_half(d[0], d[1])) * 4294967296.0);
      const long long ry = __double2ll_rn(__dmul_rn(sc, lcg_uniform_half(d[2], d[3])) * 4294967296.0);
      const long long rz = __double2ll_rn(__dmul_rn(sc, lcg_uniform_half(d[4], d[5])) * 4294967296.0);
      a.fran[g] = rx;
      a.fran[N + g] = ry;
      a.fran[2 * N + g] = rz;
      sx += rx;
      sy += ry;
      sz += rz;
    }
    sx = warp_sum_ll(sx);
    sy = warp_sum_ll(sy);
    sz = warp_sum_ll(sz);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&S.fran_sum[0]), (unsigned long long)sx);
      atomicAdd(reinterpret_cast<unsigned long long*>(&S.fran_sum[1]), (unsigned long long)sy);
      atomicAdd(reinterpret_cast<unsigned long long*>(&S.fran_sum[2]), (unsigned long long)sz);
    }
    return;
  }
  if (a.inter_ids && n <= half && (int)threadIdx.x >= half) {
    // Idle half of the CTA: bring into L2 what k_forces of this work item reads next step, the
    // used part of each bead's inter-subunit row and the subunits' intra-pair masks (cold after
    // anything has evicted L2 since the last step).
    const int k0 = threadIdx.x - half;
    for (int t = k0; t < n; t += half) {
      const int g = bead0 + t;
      const int cnt = a.inter_count[g];
      const char* row = reinterpret_cast<const char*>(a.inter_ids + (size_t)g * a.inter_cap);
      for (int off = 0; off < cnt * 4; off += 128) prefetch_l2(row + off);
    }
    const char* mk = reinterpret_cast<const char*>(a.intra_mask + (size_t)bead0 * a.words);
    for (int off = k0 * 128; off < n * a.words * 4; off += half * 128) prefetch_l2(mk + off);
    return;
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int l = t % a.np;
    drift_bead(bead0 + t, l, kick_c[l], delta_fx, vcx, vcy, vcz, dx_fx, a.fx, a.fy, a.fz, a.vx, a.vy, a.vz, a.px, a.py,
               a.pz, a.pos32);
  }
}

// Host state in: double positions to 64-bit fixed point, the high-word copy, velocities to
// 2^-32 fixed point.
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
    a.vx[g] = __double2ll_rn(a.vel_in[3 * g] * kVelScale);
    a.vy[g] = __double2ll_rn(a.vel_in[3 * g + 1] * kVelScale);
    a.vz[g] = __double2ll_rn(a.vel_in[3 * g + 2] * kVelScale);
  } else {
    a.vx[g] = a.vy[g] = a.vz[g] = 0;
  }
}

// Device state out, with any pending COM velocity subtracted (what the reference holds after
// src/md.cpp:513-514); optionally the force in double.
__global__ void k_state_out(StateArgs a) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n) return;
  const int sy = a.bead_sys[g];
  const SysParams& P = a.sys[sy];
  const SysState& S = a.state[sy];
  const double inv = 1.0 / kTwo32;
  if (a.pos_out) {
    a.pos_out[3 * g] = (double)a.px[g] * P.fx_to_len;
    a.pos_out[3 * g + 1] = (double)a.py[g] * P.fx_to_len;
    a.pos_out[3 * g + 2] = (double)a.pz[g] * P.fx_to_len;
  }
  if (a.vel_out) {
    const double iv = 1.0 / kVelScale;
    a.vel_out[3 * g] = (double)(a.vx[g] - S.vcom_fx[0]) * iv;
    a.vel_out[3 * g + 1] = (double)(a.vy[g] - S.vcom_fx[1]) * iv;
    a.vel_out[3 * g + 2] = (double)(a.vz[g] - S.vcom_fx[2]) * iv;
  }
  if (a.force_out) {
    a.force_out[3 * g] = (double)a.fx_in[g] * inv;
    a.force_out[3 * g + 1] = (double)a.fy_in[g] * inv;
    a.force_out[3 * g + 2] = (double)a.fz_in[g] * inv;
  }
}

}  // namespace souffle

namespace souffle {
void launch_forces(const ForceArgs& a, int grid, int block, size_t smem, cudaStream_t s) {
  if (a.chain64)
    k_forces<true><<<grid, block, smem, s>>>(a);
  else
    k_forces<false><<<grid, block, smem, s>>>(a);
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
cudaError_t set_kernel_smem(size_t force_smem, int force_threads, size_t pair_smem) {
  cudaError_t e = cudaFuncSetAttribute(k_forces<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)force_smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_forces<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)force_smem);
  if (e != cudaSuccess) return e;
  // Ask for a shared-memory carveout that holds as many force CTAs as the registers allow (the
  // default may be smaller, which splits a one-wave grid into two waves).
  cudaFuncAttributes fa{};
  if ((e = cudaFuncGetAttributes(&fa, k_forces<false>)) != cudaSuccess) return e;
  int dev = 0, regs_sm = 0, smem_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
  const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
  const int ctas = regs_sm / (warp_regs * ((force_threads + 31) / 32));
  const size_t need = (size_t)ctas * (force_smem + fa.sharedSizeBytes + 1024);
  const int percent = (int)std::min<size_t>(100, (need * 100 + smem_sm - 1) / (size_t)smem_sm);
  if ((e = cudaFuncSetAttribute(k_forces<false>, cudaFuncAttributePreferredSharedMemoryCarveout, percent)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_forces<true>, cudaFuncAttributePreferredSharedMemoryCarveout, percent)) != cudaSuccess)
    return e;
  return set_pairs_smem(pair_smem);
}

cudaError_t force_wave_ctas(int threads, size_t smem, int* ctas) {
  int per_sm = 0, dev = 0, sms = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_forces<false>, threads, smem);
  if (e != cudaSuccess) return e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  *ctas = per_sm * sms;
  return cudaSuccess;
}
}  // namespace souffle
