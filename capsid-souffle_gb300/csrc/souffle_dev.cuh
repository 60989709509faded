// Device-side data layout shared by the kernels of the SOUFFLE force-and-integrate path.
//
// Layout in HBM (structure of arrays, systems concatenated):
//   pos_fx[3][N]   int64 fixed-point positions: coordinate = value * L / 2^64, so the periodic
//                  box maps onto the full int64 range and the minimum image of a difference is
//                  plain two's-complement wrap-around (the reference's single-shift image,
//                  src/functions.h:42-56, for any |d| < L/2).
//   pos32[N]       int4 {x>>32, y>>32, z>>32, meta}: the rounded high words read by the pair
//                  kernels with one 16-byte load; meta = template-local bead index.
//   vel[3][N]      int64 velocities in units of 2^-40.
//   force[3][N]    int64 total force in units of 2^-32 (an exact fixed-point sum).
//   intra_mask     per subunit, np rows of ceil(np/32) words: bit jj of row ii is set when the
//                  intra-subunit pair (ii, jj) is on bead ii's reference pair list.
//   inter_ids      [N][cap] row-major global ids of inter-subunit neighbours, ascending.
#pragma once
#include <cstdint>

#include "dfloat.cuh"

namespace souffle {

constexpr int kMaxNp = 256;        // beads per subunit
constexpr int kMaxChain = 16;      // Nose-Hoover chain links
constexpr int kMaxInterPerBead = 2047;  // inter-subunit pairs of one bead (force-kernel limb sums
                                        // hold 2^11 adds: these plus the bead's own terms)
constexpr int kMaxSpecies = 16;
constexpr double kTwo32 = 4294967296.0;

// Template tables, packed into one int buffer and one float buffer so a CTA can stage them into
// shared memory with two bulk copies.  Offsets are in elements.
struct TplLayout {
  int np, ne, nf, nbend;
  int words;          // 32-bit words per intra-mask row
  int maxdeg;         // max edges per bead
  int maxrole;        // max bending roles per bead
  // int buffer offsets
  int o_edge;         // [ne] packed (b0 | b1 << 16)
  int o_face;         // [nf*3]
  int o_bend;         // [nbend*4] b0, b1, across0, across1
  int o_bendf;        // [nbend*2] face0, face1
  int o_bead_edges;   // [np*maxdeg] edge index or -1
  int o_bead_roles;   // [np*maxrole] bend*4+role or -1
  int o_type;         // [np]
  int o_species;      // [np]
  int n_int;          // total ints
  // float buffer offsets
  int o_len0;         // [ne]
  int o_q;            // [np]
  int o_sigma;        // [np]
  int o_mass;         // [np]
  int o_beta0;        // [nbend] rest bend angle per bending edge (0 = no rest angle)
  int n_float;
  int nspecies;
  int lj_att_bits[kMaxSpecies];  // bit js of row is: (species is -> js) attractive
  int type7_bits;                // bit js: species js has type 7 (attractive epsilon 50)
};

// Per-system constants (one entry per replica).
struct SysParams {
  double box;          // L
  double fx_to_len;    // L / 2^64
  double len_to_fx;    // 2^64 / L (applied through split conversion)
  float unit32;        // L / 2^32: length of one unit of the high word
  float ks, kb;
  float kappa;
  float ecut2;         // LJ cut-off squared
  float ecut_el2;      // DH cut-off squared (+inf when the reference has no cut-off)
  float elj_att;
  float nl2_f;         // pair-list radius squared (float)
  double nl2;          // pair-list radius squared, exactly the reference's double
  double pre2;         // prefilter: 2.25 * nl2 (src/functions.cpp:91)
  int bead0, sub0, n_sub;   // first bead / subunit, subunit count
  int cell0, ncell;         // first cell, cells per dimension (subunit-centre grid)
  int quirks;               // reproduce src/functions.cpp:97
  int center_local;         // template-local centre bead (src/initialize.cpp:266-288)
  double dt;
  double ks_d, kb_d;        // double copies for the FP64 energy pass
  long long drift_fx;       // dt 2^32 / L in 2^-40 units: x_fixed += v_fixed * drift_fx >> 40
  int brownian;             // Brownian dynamics (src/md.cpp:415-431, 461-501) instead of the NHC
  unsigned int lcg_step;    // Brownian noise: 16807^(6 (n_beads + big beads)) mod (2^31 - 1), one step of draws
  // encapsulation big beads (src/forces.cpp:174-236): first index and count in the handle's
  // big-bead arrays; DH weight q e^(kappa sigma/2) / (1 + kappa sigma/2) sqrt(lb), diameter,
  // hard-core distance, DH cut-off squared (0 without a cut-off: the reference's test
  // r^2 < ecut_el^2 then never holds); double copies for the energy pass
  int bb0, nbb;
  float bb_w, bb_sigma, bb_shc, bb_dh_cut2;
  float bb_reach2;          // (1.01 max(DH cut-off, largest shifted WCA range))^2: beyond, no force
  double bb_q, bb_sigma_d, bb_shc_d;
};

// Thermostat chain and step scalars of one system, updated on the device.
// xi/eta is the chain after the forward half of the last step (what energy output reads);
// xi_b/eta_b is the chain after the backward half of the next step (what the next step
// integrates with).  Both halves only need particle_ke, so the backward half of step a+1 is
// applied right after the forward half of step a.  The chain is carried in double-float (hi + lo
// FP32 pairs, ~48-bit significand): its update is a serial dependency chain, and GB300's FP64
// latency would put several microseconds of it on every step.
struct __align__(16) SysState {
  int m;                 // chain length
  int n_beads;           // beads in this system
  double q[kMaxChain], t[kMaxChain], dof[kMaxChain];  // the chain's Q, T, dof (host copies)
  dfloat c_q[kMaxChain];          // Q_j                  (constants for the device update,
  dfloat c_dof_t[kMaxChain];      // dof_j T_j             set on the host at md_begin)
  dfloat c_hdt_inv_q[kMaxChain];  // dt / (2 Q_j), 0 for the massless dummy link
  dfloat c_hdt;                   // dt / 2
  dfloat c_mqdt;                  // -dt / 4
  double inv_n;                   // 1 / n_beads
  dfloat xi[kMaxChain], eta[kMaxChain];
  dfloat xi_b[kMaxChain], eta_b[kMaxChain];
  dfloat ke;             // particle_ke carried between steps (src/md.cpp:456)
  dfloat kick_c0;        // dt sqrt(expfac) / 2 of the next step (per-bead kick c = c0 / m)
  long long delta_fx;    // (1 - expfac) * 2^62 for the integer kicks, expfac = exp(-dt xi0 / 2)
  long long vcom_fx[3];  // mean velocity (2^-40 units) still to subtract from vel (0 once applied)
  double vcom_mag;       // |mean velocity| removed at the last step (src/md.cpp:623)
  unsigned int done;     // arrival counter for the last-block reduction
  unsigned int steps;    // MD steps completed since md_begin
  long long fran_sum[3]; // Brownian: sum of this step's random forces (2^-32 units)
  unsigned int lcg;      // Brownian: minstd_rand0 state before this step's draws
};

// The chain in FP64 (souffle_options.chain_fp64): the link variables and constants of one system
// in the reference's double arithmetic.  xi / eta are the current chain (after the backward half
// of the next step, between launches); SysState's double-float xi / eta and xi_b / eta_b mirror
// them for the energy output.
struct Chain64 {
  int m;
  double dt;
  double q[kMaxChain], t[kMaxChain], dof[kMaxChain];
  double xi[kMaxChain], eta[kMaxChain];
};

// Lengths of the force kernel's per-bead fixed-point force limbs (3 components x 3 32-bit limbs
// per bead, padded to keep 16-byte alignment) and of its prefix-sum array (nbead + 1 ints,
// padded to a multiple of 4).
__host__ __device__ inline int force_slot_len(int nbead_max) { return 9 * ((nbead_max + 3) & ~3); }
__host__ __device__ inline int force_pref_len(int nbead_max) { return (nbead_max + 4) & ~3; }

// Bytes of the force kernel's first shared-memory region: the bonded tile (edge and bending
// terms of max_sub subunits), and at least the system state plus the thermostat scratch
// (3 kMaxChain dfloats) that the tail of a system's last CTA keeps there.
__host__ __device__ inline size_t force_tile_bytes(int max_sub, int ne, int nb) {
  const size_t tile = 16 * (size_t)max_sub * (size_t)(ne + 4 * nb);
  const size_t tail = (sizeof(SysState) + 3 * kMaxChain * sizeof(dfloat) + 15) / 16 * 16;
  return tile > tail ? tile : tail;
}

// Work item: a run of subunits of one system handled by one CTA.
struct WorkItem {
  int sys, sub_begin, nsub, slot;
};

// Pair-species tables for the LJ/WCA branch of src/forces.cpp:112-138.
struct PairTable {
  float sig6[kMaxSpecies * kMaxSpecies];   // sigma_i^6 (attractive) or shc^6 (WCA)
  float cut2[kMaxSpecies * kMaxSpecies];   // ecut^2 (attractive) or (1.12246205 shc)^2
  float skip2[kMaxSpecies * kMaxSpecies];  // max(ecut^2, (1.12246205 shc)^2): beyond it no LJ
};

// Error flags raised by kernels and read by the host.
enum : unsigned int {
  kErrInterOverflow = 1u,
  kErrCandOverflow = 2u,
  kErrNonFinite = 4u,
  kErrSurrogate = 8u,  // a bounded wait of the surrogate network's tensor-core kernels ran out
};

__host__ __device__ inline long long fixed_from_fraction(double f) {
  // round(f * 2^64) modulo 2^64, for |f| < 2^20: split so no step overflows
  double a = f * kTwo32;
#ifdef __CUDA_ARCH__
  double ip = rint(a);
#else
  double ip = __builtin_rint(a);
#endif
  double rem = a - ip;  // exact, |rem| <= 0.5
#ifdef __CUDA_ARCH__
  long long lo = __double2ll_rn(rem * kTwo32);
#else
  long long lo = (long long)__builtin_llrint(rem * kTwo32);
#endif
  unsigned long long hi = (unsigned long long)(long long)ip;
  return (long long)((hi << 32) + (unsigned long long)lo);
}

__host__ __device__ inline int hi_word(long long x) {
  return (int)(unsigned int)(((unsigned long long)x + 0x80000000ull) >> 32);
}

__host__ __device__ inline double fixed_diff(long long a, long long b, double fx_to_len) {
  return (double)(long long)((unsigned long long)a - (unsigned long long)b) * fx_to_len;
}

__device__ inline float hi_diff(int a, int b, float unit) {
  return (float)(int)((unsigned int)a - (unsigned int)b) * unit;
}

// ---- 64-bit fixed point without FP64 instructions -------------------------------------------
// GB300 runs FP64 at a small fraction of its FP32 rate, so per-bead integration is done in
// integers: velocities and forces are int64 in units of 2^-32, positions int64 in units of
// L/2^64, and every product is an exact 64x64->128 multiply rounded to nearest.

// round(a * b / 2^s) for 0 < s < 64, exact (128-bit product, ties away from zero is not needed:
// adding 2^(s-1) rounds half up).
__device__ __forceinline__ long long mul_shr(long long a, long long b, int s) {
  unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
  long long hi = __mul64hi(a, b);
  const unsigned long long half = 1ull << (s - 1);
  const unsigned long long lo2 = lo + half;
  hi += (lo2 < lo) ? 1 : 0;
  return (long long)(((unsigned long long)hi << (64 - s)) | (lo2 >> s));
}

// round(v * 2^32) as int64 for |v| < 2^31, using only 32-bit conversions.
__device__ __forceinline__ long long f32_to_fx32(float v) {
  const float hi = floorf(v);
  const float frac = (v - hi) * 4294967296.0f;  // in [0, 2^32]
  const unsigned long long lo = (unsigned long long)__float2uint_rn(frac);
  return (long long)(((unsigned long long)(long long)__float2int_rz(hi) << 32) + lo);
}

// (e^x - 1) / x for the thermostat's small arguments (x = -dt xi / 4 or -dt xi / 2), by the
// Taylor series of e^x.  |x| <= 2^-9: terms through x^6/7! (truncation below x^7/8! < 2e-23
// relative); |x| <= 1/16: through x^10/11! (below x^11/12! < 4e-24).  The polynomials use
// Estrin's scheme, so the dependent chain is 3-4 multiply-adds deep instead of 7-11: on GB300 a
// dependent FP64 operation takes on the order of a hundred cycles, and these exponentials sit on
// the serial thermostat path that every MD step waits for.
__host__ __device__ inline double expm1_over_x_series(double x) {
  const double x2 = x * x;
  if (x >= -0.001953125 && x <= 0.001953125) {
    // 1 + x/2 + x^2/6 + x^3/24 + x^4/120 + x^5/720 + x^6/5040
    const double a = fma(x, 1.0 / 2.0, 1.0);
    const double b = fma(x, 1.0 / 24.0, 1.0 / 6.0);
    const double c = fma(x, 1.0 / 720.0, 1.0 / 120.0);
    const double x4 = x2 * x2;
    return fma(x4, fma(x2, 1.0 / 5040.0, c), fma(x2, b, a));
  }
  // 1 + x/2 + ... + x^10/11!
  const double a = fma(x, 1.0 / 2.0, 1.0);
  const double b = fma(x, 1.0 / 24.0, 1.0 / 6.0);
  const double c = fma(x, 1.0 / 720.0, 1.0 / 120.0);
  const double d = fma(x, 1.0 / 40320.0, 1.0 / 5040.0);
  const double e = fma(x, 1.0 / 3628800.0, 1.0 / 362880.0);
  const double x4 = x2 * x2;
  const double lo = fma(x2, b, a);
  const double hi = fma(x2, d, c);
  const double top = fma(x2, 1.0 / 39916800.0, e);
  return fma(x4, fma(x4, top, hi), lo);
}

// e^x for |x| <= 708: Cody-Waite reduction x = k ln2 + r with ln2 split into a 53-bit head and
// its tail (|r| <= ln2/2), e^r = 1 + r S(r) with S the series of (e^r - 1)/r through r^12/13!
// (truncation below r^13/14! < 1.3e-17), evaluated by Estrin's scheme, then an exact scaling by
// 2^k built from the exponent bits.  About 11 dependent FP64 operations.
// (e^r - 1)/r through r^12/13! by Estrin's scheme, for |r| <= ln2/2.
__host__ __device__ inline double expm1_over_r_s13(double r) {
  const double r2 = r * r, r4 = r2 * r2, r8 = r4 * r4;
  const double p01 = fma(r, 1.0 / 2.0, 1.0);
  const double p23 = fma(r, 1.0 / 24.0, 1.0 / 6.0);
  const double p45 = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  const double p67 = fma(r, 1.0 / 40320.0, 1.0 / 5040.0);
  const double p89 = fma(r, 1.0 / 3628800.0, 1.0 / 362880.0);
  const double pab = fma(r, 1.0 / 479001600.0, 1.0 / 39916800.0);
  return fma(r8, fma(r4, 1.0 / 6227020800.0, fma(r2, pab, p89)),
             fma(r4, fma(r2, p67, p45), fma(r2, p23, p01)));
}

__host__ __device__ inline double exp_reduced(double x) {
  if (!(x > -708.0 && x < 708.0)) return exp(x);  // overflow, underflow, NaN: the library
  const double k = rint(x * 1.4426950408889634074);
  const double r = fma(-k, 2.319046813846299558e-17, fma(-k, 0.69314718055994528623, x));
  const double er = fma(r, expm1_over_r_s13(r), 1.0);
  // 2^k for |k| <= 1022, split in two factors so k = +-1022 stays in range
  const long long ki = (long long)k;
  const long long k1 = ki / 2, k2 = ki - k1;
#ifdef __CUDA_ARCH__
  const double s1 = __longlong_as_double((k1 + 1023) << 52), s2 = __longlong_as_double((k2 + 1023) << 52);
#else
  double s1, s2;
  const long long b1 = (k1 + 1023) << 52, b2 = (k2 + 1023) << 52;
  __builtin_memcpy(&s1, &b1, 8);
  __builtin_memcpy(&s2, &b2, 8);
#endif
  return (er * s1) * s2;
}

__host__ __device__ inline double exp_small(double x) {
  if (!(x >= -0.0625 && x <= 0.0625)) return exp_reduced(x);
  return fma(x, expm1_over_x_series(x), 1.0);
}

// e^x - 1 without cancellation: x times a series up to |x| = ln2/2, beyond which e^x - 1 is
// at least 0.29 in magnitude and the subtraction loses under two bits.
__host__ __device__ inline double expm1_small(double x) {
  if (x >= -0.0625 && x <= 0.0625) return x * expm1_over_x_series(x);
  if (x >= -0.34657359027997264 && x <= 0.34657359027997264) return x * expm1_over_r_s13(x);
  return exp_reduced(x) - 1.0;
}

// ---- the reference's Brownian noise: std::default_random_engine = minstd_rand0 -------------
constexpr unsigned long long kLcgMod = 2147483647ull;  // 2^31 - 1
constexpr unsigned int kLcgSeed = 69521u;              // src/md.cpp:382

__host__ __device__ inline unsigned int lcg_mul(unsigned int x, unsigned int m) {
  return (unsigned int)(((unsigned long long)x * m) % kLcgMod);
}

// std::uniform_real_distribution<double>(-0.5, 0.5) on minstd_rand0 as libstdc++ evaluates it:
// generate_canonical<double, 53> takes two draws g1, g2 and returns
// ((g1 - 1) + (g2 - 1) r) / r^2 with r = 2^31 - 2, every operation rounded in double (r^2 is
// exact before its rounding), a result >= 1 replaced by the largest double below 1; then
// u * (0.5 - -0.5) + -0.5.
__host__ __device__ inline double lcg_uniform_half(unsigned int g1, unsigned int g2) {
  const double r = 2147483646.0;
#ifdef __CUDA_ARCH__
  const double sum = __dadd_rn((double)(g1 - 1u), __dmul_rn((double)(g2 - 1u), r));
  double u = __ddiv_rn(sum, __dmul_rn(r, r));
#else
  volatile double prod = (double)(g2 - 1u) * r;
  volatile double sum = (double)(g1 - 1u) + prod;
  volatile double r2 = r * r;
  double u = sum / r2;
#endif
  if (u >= 1.0) u = 0.99999999999999988898;  // nextafter(1, 0)
  return u - 0.5;
}

// Velocities are int64 in units of 2^-40 (resolution 9.1e-13, range +-8.4e6 in LJ units).
constexpr double kVelScale = 1099511627776.0;  // 2^40

// int64 velocity (2^-40 units) to float, using only 32-bit conversions.
__device__ __forceinline__ float vel_to_f32(long long x) {
  const int hi = (int)(x >> 32);
  const unsigned int lo = (unsigned int)x;
  return fmaf((float)lo, 9.094947017729282e-13f, (float)hi * 0.00390625f);
}

}  // namespace souffle
