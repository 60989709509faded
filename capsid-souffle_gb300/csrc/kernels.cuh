// Kernel argument blocks and launch wrappers of the SOUFFLE GPU path (definitions in
// pairlist.cu, forces.cu, energies.cu).
#pragma once
#include <cuda_runtime.h>

#include "souffle_dev.cuh"

namespace souffle {

struct CellArgs {
  const long long* px;
  const long long* py;
  const long long* pz;
  const SysParams* sys;
  const int* sub_sys;     // [S_total] system of each subunit
  int np, n_sub_total;
  int* cell_count;        // [total cells]
  int* cell_start;        // [total cells + 1]
  int* sub_rank;          // [S_total]
  int* sub_cell;          // [S_total]
  int* cell_subs;         // [S_total]
  int total_cells;
  int n_sys;
};

struct CandArgs {
  CellArgs c;
  const int4* pos32;  // [N] high words of the positions (float pre-test)
  int cap;
  int* cand;        // [S_total * cap] candidate subunits (global ids), ascending
  int* cand_count;  // [S_total]
  unsigned int* err;
};

struct PairArgs {
  const long long* px;
  const long long* py;
  const long long* pz;
  const int4* pos32;
  const SysParams* sys;
  const int* sub_sys;
  const float* q;       // [np] template charges (only q != 0 matters)
  int np, words, n_beads_total;
  const int* cand;
  const int* cand_count;
  int cand_cap;
  unsigned int* intra_mask;  // [S_total * np * words]
  int* inter_ids;            // [N][cap] row-major
  int* inter_count;          // [N]
  const unsigned char* cand_far = nullptr;  // [S_total * cand_cap]: nonzero = not in the pair list (1 left to the surrogate, 2 beyond every cut-off)
  const int* far_ok = nullptr;              // the far flags apply (no far-list overflow)
  int* ref_len;              // [N] reference list length (intra + inter)
  int inter_cap;
  int chunk;                 // candidates staged together (1 .. kPairChunkMax)
  unsigned int* err;
};

struct ForceArgs {
  TplLayout L;
  const int* tpl_i;
  const float* tpl_f;
  const SysParams* sys;
  SysState* state;
  const WorkItem* work;
  const int2* sys_slots;     // per system: first work item in system order, work-item (CTA) count
  const int4* pos32;
  const unsigned int* intra_mask;
  const int* inter_ids;      // [N][inter_cap] row-major, ascending
  const float4* surr_f = nullptr;  // [N] far-field forces from the surrogate, or null
  const long long* fdrag = nullptr;  // Brownian: [3][N] drag and random force of the step
  const long long* fran = nullptr;
  const int4* bb_pos32 = nullptr;  // encapsulation big beads: high words of their positions
  Chain64* chain64 = nullptr;      // [n_sys] the chain in FP64 (souffle_options.chain_fp64), or null
  const int* inter_count;
  int inter_cap;
  const float* dh_w;         // [n_sys * np] q * exp(kappa sigma/2)/(1 + kappa sigma/2) * sqrt(lb)
  const PairTable* pt;
  const dfloat* inv_mass;    // [np] 1 / m as double-float (kick coefficients)
  long long* kick_c;         // [n_sys * np] dt sqrt(expfac) / (2 m) * 2^62, written by the last CTA
  long long* fx; long long* fy; long long* fz;   // force, 2^-32 units
  long long* vx; long long* vy; long long* vz;   // velocity, 2^-32 units
  float* sfx; float* sfy; float* sfz;   // optional stretching force out
  float* bfx; float* bfy; float* bfz;   // optional bending force out
  long long* partial;        // [systems * 4] running KE and momentum sums (2^-32), zero between launches
  unsigned int* err;
  int n_beads_total;
  int max_sub;               // subunits per CTA (shared-memory sizing)
  int mode;                  // 0: forces only, 1: MD step (kick + reductions), 2: begin (KE only)
};

struct DriftArgs {
  const SysParams* sys;
  SysState* state;
  const WorkItem* work;
  const long long* kick_c;
  int np;
  const long long* fx; const long long* fy; const long long* fz;
  long long* vx; long long* vy; long long* vz;
  long long* px; long long* py; long long* pz;
  int4* pos32;
  // pair lists read by k_forces of the same work item, prefetched into L2 by the idle half of
  // the CTA (null: no prefetch)
  const int* inter_ids = nullptr;
  const int* inter_count = nullptr;
  int inter_cap = 0;
  const unsigned int* intra_mask = nullptr;
  int words = 0;
  // Brownian systems (src/md.cpp:415-431, 461-501): drag m/damp (2^40 units) and noise scale
  // sqrt(24 m / (damp dt)) per system and template bead, the minstd_rand0 skip-ahead table
  // 16807^(6k) mod (2^31 - 1) by system-local bead k, and the step's drag and noise (2^-32)
  const long long* bd_drag = nullptr;
  const double* bd_noise = nullptr;
  const unsigned int* lcg_table = nullptr;
  long long* fdrag = nullptr;  // [3][N]
  long long* fran = nullptr;   // [3][N]
  long long n_total = 0;
};

struct StateArgs {
  const SysParams* sys;
  SysState* state;
  const int* bead_sys;   // [N]
  int np, n;
  const double* pos_in;  // [N*3] xyz interleaved (device staging), may be null
  const double* vel_in;
  long long* px; long long* py; long long* pz;
  int4* pos32;
  long long* vx; long long* vy; long long* vz;
  double* pos_out;       // [N*3]
  double* vel_out;
  double* force_out;     // [N*3] optional
  const long long* fx_in; const long long* fy_in; const long long* fz_in;
};

struct EnergyArgs {
  TplLayout L;
  const int* tpl_i;
  const float* tpl_f;
  const SysParams* sys;
  const SysState* state;
  const long long* px; const long long* py; const long long* pz;
  const int4* pos32;
  const long long* vx; const long long* vy; const long long* vz;   // 2^-32 units
  const double* len0;      // [ne]
  const double* mass;      // [np]
  const double* q;         // [np]
  const double* sigma;     // [np]
  const int* type;         // [np]
  const int* lj_t;         // [2 * n_lj]
  int n_lj;
  double ecut;
  double elj_att;
  double lb, kappa, ecut_el;
  double sigma_max;        // largest bead diameter (pair pruning)
  int sysid;
  int n0, n;               // first bead of the system, beads in it
  double* se; double* be; double* ne; double* ce; double* ke;  // [n] (system-local)
  double* totals;          // [8] per call
  double* pair_tab;        // [3][np * np] per template bead pair (i, j): the Yukawa size factor,
                           // sbar^6, the attractive LJ shift at ecut (k_energy_tables)
  unsigned char* att_tab;  // [np * np] 1 = attractive by the directed LJ table
  // cell grid of the pair pass (nc cells per axis, nc >= 3; nc = 0: every pair j > i is visited)
  int nc;
  int* cell_count;         // [nc^3] (zeroed before the count)
  int* cell_start;         // [nc^3 + 1]
  int* cell_fill;          // [nc^3] (zeroed before the scatter)
  int* cell_beads;         // [n] system-local bead indices, ascending within each cell
  int* bead_cell;          // [n]
  // encapsulation big beads of the system: fixed-point positions [3][total], the big-bead parts
  // of ne and ce per subunit bead [n] and their sums ([2]: lj, electrostatic)
  const long long* bb_fx = nullptr;
  int bb_total = 0;
  double* ne_bb = nullptr; double* ce_bb = nullptr;
  double* bb_totals = nullptr;
};

void launch_cells_count(const CellArgs& a, int grid, int block, cudaStream_t s);
void launch_cells_scan(const CellArgs& a, cudaStream_t s);
void launch_cells_scatter(const CellArgs& a, int grid, int block, cudaStream_t s);
void launch_candidates(const CandArgs& a, int grid, int block, cudaStream_t s);
void launch_pairs(const PairArgs& a, int n_sub, size_t smem, cudaStream_t s);
// k_pairs' chunk of candidates staged together, and its dynamic shared memory
constexpr int kPairChunkMax = 32;
int pair_chunk(int np, int words);
size_t pair_smem_bytes(int np, int words, int chunk);
void launch_forces(const ForceArgs& a, int grid, int block, size_t smem, cudaStream_t s);
void launch_drift(const DriftArgs& a, int grid, int block, cudaStream_t s);
void launch_state_in(const StateArgs& a, int grid, int block, cudaStream_t s);
void launch_state_out(const StateArgs& a, int grid, int block, cudaStream_t s);
void launch_energies(const EnergyArgs& a, int n, cudaStream_t s);
cudaError_t set_kernel_smem(size_t force_smem, int force_threads, size_t pair_smem);
// force-kernel CTAs of the given shape resident on the device at once (one wave)
cudaError_t force_wave_ctas(int threads, size_t smem, int* ctas);
cudaError_t set_pairs_smem(size_t smem);

}  // namespace souffle
