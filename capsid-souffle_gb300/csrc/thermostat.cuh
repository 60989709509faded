// Nose-Hoover chain updates of one system in double-float arithmetic, run by the last CTA of
// each system after the kinetic energy of the step is known.
//
// Link update, update_chain_xi (src/functions.cpp:33-58):
//   xi_j <- xi_j e^{-dt xi_{j+1}/2} + dt/(2 Q_j) G_j e^{-dt xi_{j+1}/4}
//         = e4 (xi_j e4 + c_j G_j),  e4 = e^{-dt xi_{j+1}/4},  c_j = dt/(2 Q_j)
// with G_0 = 2 KE - dof_0 T and G_j = Q_{j-1} xi_{j-1}^2 - dof_j T.  Links with Q_j = 0 (the dummy
// end link) are never updated.
//
// Two forms with the same operations in the same order, so they give bitwise equal results:
// serial functions (host-callable; the CPU checks against FP64 use them) and warp functions for
// the device, where lane j evaluates link j's exponentials, G terms and eta updates at once and
// every lane then runs the short link recurrence from shared operands.
#pragma once
#include "souffle_dev.cuh"

namespace souffle {

__host__ __device__ inline bool nhc_active(const SysState& s, int j) { return s.c_q[j].hi != 0.0f; }

// G_j, with prev = xi_{j-1} (unused for j = 0)
__host__ __device__ inline dfloat nhc_g(const SysState& s, dfloat prev, int j) {
  if (j == 0) return df_add(dfloat{2.0f * s.ke.hi, 2.0f * s.ke.lo}, df_neg(s.c_dof_t[0]));
  return df_add(df_mul(s.c_q[j - 1], df_mul(prev, prev)), df_neg(s.c_dof_t[j]));
}

// e^{-dt xn / 4}; exactly 1 when xn is 0 (the dummy link's xi never moves from 0)
__host__ __device__ inline dfloat nhc_e4(const SysState& s, dfloat xn) {
  if (xn.hi == 0.0f && xn.lo == 0.0f) return dfloat{1.0f, 0.0f};
  return df_exp(df_mul(s.c_mqdt, xn));
}

__host__ __device__ inline dfloat nhc_link(dfloat x, dfloat e4, dfloat cg) {
  return df_mul(e4, df_add(df_mul(x, e4), cg));
}

__host__ __device__ inline dfloat nhc_eta(const SysState& s, dfloat eta, dfloat x) {
  return df_add(eta, df_mul(s.c_hdt, x));
}

// Kick factors of the next step from xi_0 after the backward half, h = -dt xi_0 / 4:
// sqrt(expfac) = e^h, 1 - expfac = -(e^h - 1)(e^h + 1), kick_c0 = dt e^h / 2.  Returns false when
// they leave the range the fixed-point kick can represent.
__host__ __device__ inline bool nhc_kick_factors(SysState& s, dfloat xb0) {
  const dfloat u = df_expm1(df_mul(s.c_mqdt, xb0));
  const dfloat one_minus = df_neg(df_mul(u, df_add(u, dfloat{2.0f, 0.0f})));
  s.kick_c0 = df_mul(s.c_hdt, df_add(u, dfloat{1.0f, 0.0f}));
  // |1 - expfac| < 1.9 keeps delta * 2^62 inside int64; NaN fails the comparison
  if (!(fabsf(one_minus.hi) < 1.9f) || !(fabsf(s.kick_c0.hi) < 1.0e6f)) return false;
  s.delta_fx = df_to_fixed(one_minus, 4611686018427387904.0f);  // 2^62
  return true;
}

// Forward half at the end of a step (src/md.cpp:457-460), from (xi_b, eta_b) into (xi, eta):
// links j = 0 .. M-1, each reading xi_{j+1} before it changes (so all exponentials come first)
// and G_j from the freshly updated xi_{j-1}.
// The forward link update e4 (xi_j e4 + c_j G_j) rearranged so that only one square, one product
// and one sum depend on the freshly updated xi_{j-1}: x_j = A_j + B_j xi_{j-1}^2 with
// A_j = e4 (xi_j e4 - c_j dof_j T_j) and B_j = e4 c_j Q_{j-1}; link 0 (G_0 = 2 KE - dof_0 T)
// depends on no other link and is A_0 itself.
__host__ __device__ inline void nhc_forward_terms(const SysState& s, int j, dfloat& A, dfloat& B) {
  const dfloat e4 = nhc_e4(s, s.xi_b[j + 1]);
  const dfloat p = df_mul(s.xi_b[j], e4);
  if (j == 0) {
    A = df_mul(e4, df_add(p, df_mul(s.c_hdt_inv_q[0], nhc_g(s, dfloat{0.0f, 0.0f}, 0))));
    B = dfloat{0.0f, 0.0f};
  } else {
    A = df_mul(e4, df_add(p, df_neg(df_mul(s.c_hdt_inv_q[j], s.c_dof_t[j]))));
    B = df_mul(df_mul(e4, s.c_hdt_inv_q[j]), s.c_q[j - 1]);
  }
}

__host__ __device__ inline dfloat nhc_forward_link(int j, dfloat A, dfloat B, dfloat prev) {
  return j == 0 ? A : df_add(A, df_mul(B, df_mul(prev, prev)));
}

__host__ __device__ inline void nhc_forward(SysState& s) {
  dfloat A[kMaxChain], B[kMaxChain];
  for (int j = 0; j < s.m; j++) {
    const bool on = nhc_active(s, j);
    s.eta[j] = on ? nhc_eta(s, s.eta_b[j], s.xi_b[j]) : s.eta_b[j];
    if (on) nhc_forward_terms(s, j, A[j], B[j]);
  }
  dfloat prev = {0.0f, 0.0f};
  for (int j = 0; j < s.m; j++) {
    dfloat x = s.xi_b[j];
    if (nhc_active(s, j)) x = nhc_forward_link(j, A[j], B[j], prev);
    s.xi[j] = x;
    prev = x;
  }
}

// Backward half at the start of a step (src/md.cpp:401-406), from (xi, eta) into (xi_b, eta_b):
// links j = M-1 .. 0, each reading the freshly updated xi_{j+1}; G_j reads xi_{j-1} before it
// changes, so all G_j come first.  Then the step's kick factors.
__host__ __device__ inline bool nhc_backward(SysState& s) {
  dfloat cg[kMaxChain];
  for (int j = 0; j < s.m; j++)
    if (nhc_active(s, j))
      cg[j] = df_mul(s.c_hdt_inv_q[j], nhc_g(s, j > 0 ? s.xi[j - 1] : dfloat{0.0f, 0.0f}, j));
  dfloat next = {0.0f, 0.0f};
  for (int j = s.m - 1; j > -1; j--) {
    dfloat x = s.xi[j];
    if (nhc_active(s, j)) x = nhc_link(x, nhc_e4(s, next), cg[j]);
    s.xi_b[j] = x;
    next = x;
  }
  for (int j = 0; j < s.m; j++) s.eta_b[j] = nhc_active(s, j) ? nhc_eta(s, s.eta[j], s.xi_b[j]) : s.eta[j];
  return nhc_kick_factors(s, s.xi_b[0]);
}

#ifdef __CUDACC__
// ---- the chain in FP64 on one thread (souffle_options.chain_fp64), a validation variant -----
// update_chain_xi (src/functions.cpp:33-58) and THERMOSTAT::update_eta (src/thermostat.h:35-40)
// in the reference's double arithmetic and link order.
__device__ inline void chain64_xi(Chain64& c, int j, double ke) {
  if (c.q[j] == 0) return;
  const double xn = j + 1 < kMaxChain ? c.xi[j + 1] : 0.0;
  const double g = j == 0 ? 2 * ke - c.dof[0] * c.t[0] : c.q[j - 1] * c.xi[j - 1] * c.xi[j - 1] - c.dof[j] * c.t[j];
  c.xi[j] = c.xi[j] * exp(-0.5 * c.dt * xn) + 0.5 * c.dt * (1.0 / c.q[j]) * g * exp(-0.25 * c.dt * xn);
}
__device__ inline void chain64_eta(Chain64& c) {
  for (int j = 0; j < c.m; j++)
    if (c.q[j] != 0) c.eta[j] = c.eta[j] + 0.5 * c.dt * c.xi[j];
}
// forward half at the end of a step (src/md.cpp:457-460); mirrors xi / eta for the energy output
__device__ inline void chain64_forward(Chain64& c, double ke, SysState& S) {
  chain64_eta(c);
  for (int j = 0; j < c.m; j++) chain64_xi(c, j, ke);
  for (int j = 0; j < c.m; j++) {
    S.xi[j] = df_from(c.xi[j]);
    S.eta[j] = df_from(c.eta[j]);
  }
}
// backward half at the start of the next step (src/md.cpp:401-406) and its kick factors:
// expfac = exp(-dt xi_0 / 2), 1 - expfac = -(e^h - 1)(e^h + 1) with h = -dt xi_0 / 4,
// kick_c0 = dt e^h / 2.  False when they leave the fixed-point kick's range.
__device__ inline bool chain64_backward(Chain64& c, double ke, SysState& S) {
  for (int j = c.m - 1; j > -1; j--) chain64_xi(c, j, ke);
  chain64_eta(c);
  for (int j = 0; j < c.m; j++) {
    S.xi_b[j] = df_from(c.xi[j]);
    S.eta_b[j] = df_from(c.eta[j]);
  }
  const double u = expm1(-0.25 * c.dt * c.xi[0]);
  const double one_minus = -u * (u + 2.0), kc0 = 0.5 * c.dt * (u + 1.0);
  if (!(fabs(one_minus) < 1.9) || !(fabs(kc0) < 1.0e6)) return false;
  S.delta_fx = __double2ll_rn(one_minus * 4611686018427387904.0);  // 2^62
  S.kick_c0 = df_from(kc0);
  return true;
}

// Both halves as the force kernel's tail runs them (forward only after an MD step); out of line so
// that the FP64 code does not weigh on the force kernel's registers.
static __device__ __noinline__ bool chain64_tail(Chain64& c, double ke, bool forward, SysState& S) {
  if (forward) chain64_forward(c, ke, S);
  return chain64_backward(c, ke, S);
}

static_assert(kMaxChain <= 32, "one lane per chain link");

// Forward half on one warp: lane j evaluates link j's exponential, A_j, B_j and eta_j at once;
// then every lane runs the link recurrence itself from those shared operands (no lane-to-lane
// hand-off in the dependent chain) and lane j stores xi_j.  scratch: 2 kMaxChain dfloats of
// shared memory.
__device__ inline void nhc_forward_warp(SysState& s, int lane, dfloat* scratch) {
  const int m = s.m;
  dfloat* As = scratch;
  dfloat* Bs = scratch + kMaxChain;
  if (lane < m) {
    const bool on = nhc_active(s, lane);
    s.eta[lane] = on ? nhc_eta(s, s.eta_b[lane], s.xi_b[lane]) : s.eta_b[lane];
    if (on) nhc_forward_terms(s, lane, As[lane], Bs[lane]);
  }
  __syncwarp();
  dfloat prev = {0.0f, 0.0f};
  for (int j = 0; j < m; j++) {
    dfloat x = s.xi_b[j];
    if (nhc_active(s, j)) x = nhc_forward_link(j, As[j], Bs[j], prev);
    if (lane == j) s.xi[j] = x;
    prev = x;
  }
  __syncwarp();
}

// Backward half on one warp: lane j evaluates c_j G_j (reads xi_{j-1} before it changes); then
// every lane runs the recurrence j = M-1 .. 0 and lane j stores xi_j; lane 0 sets the kick
// factors (its return value is the one that counts).  scratch: kMaxChain dfloats.
__device__ inline bool nhc_backward_warp(SysState& s, int lane, dfloat* scratch) {
  __syncwarp();  // xi / eta written by other lanes (the forward half) are visible from here on
  const int m = s.m;
  dfloat* cgs = scratch;
  if (lane < m && nhc_active(s, lane))
    cgs[lane] = df_mul(s.c_hdt_inv_q[lane], nhc_g(s, lane > 0 ? s.xi[lane - 1] : dfloat{0.0f, 0.0f}, lane));
  __syncwarp();
  dfloat next = {0.0f, 0.0f};
  for (int j = m - 1; j > -1; j--) {
    dfloat x = s.xi[j];
    if (nhc_active(s, j)) x = nhc_link(x, nhc_e4(s, next), cgs[j]);
    if (lane == j) s.xi_b[j] = x;
    next = x;
  }
  __syncwarp();
  if (lane < m) s.eta_b[lane] = nhc_active(s, lane) ? nhc_eta(s, s.eta[lane], s.xi_b[lane]) : s.eta[lane];
  return lane == 0 ? nhc_kick_factors(s, next) : true;
}
#endif

// Host side: chain constants of one system from its parameters (src/md.cpp:187-196).
inline void nhc_set_constants(SysState& s, double dt) {
  for (int j = 0; j < s.m; j++) {
    s.c_q[j] = df_from(s.q[j]);
    s.c_dof_t[j] = df_from(s.dof[j] * s.t[j]);
    s.c_hdt_inv_q[j] = s.q[j] != 0 ? df_from(0.5 * dt / s.q[j]) : dfloat{0.0f, 0.0f};
  }
  s.c_hdt = df_from(0.5 * dt);
  s.c_mqdt = df_from(-0.25 * dt);
}

// Per-bead kick coefficient c0 / m in 2^-64 units; false when it does not fit int64.
__host__ __device__ inline bool nhc_kick_coefficient(dfloat c0, dfloat inv_mass, long long& out) {
  const dfloat c = df_mul(c0, inv_mass);
  if (!(fabsf(c.hi) < 0.49f)) return false;  // < 2^63 - 2^40 in 2^-64 units, NaN excluded
  out = df_to_fixed(c, 18446744073709551616.0f);  // 2^64
  return true;
}

}  // namespace souffle
