// The handle behind include/souffle_gpu.h (private to the library): host template tables, device
// buffers and launch state of a batch of systems.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <vector>

#include "devbuf.cuh"
#include "kernels.cuh"
#include "souffle_dev.cuh"
#include "souffle_gpu.h"
#include "surrogate.cuh"

namespace souffle {

// Template tables derived on the host, following generate_lattice (src/initialize.cpp:317-401).
struct HostTemplate {
  int np = 0, ne = 0, nf = 0, n_lj = 0;
  std::vector<int> type, edge, edge_type, face, lj;
  std::vector<double> q, sigma, mass, len0;
  std::vector<int> edge_f0, edge_f1;   // faces of each edge, face order
  std::vector<int> bend_edge;          // bending edges in template order
  std::vector<int> bend;               // [nb*4] b0, b1, across0, across1
  std::vector<int> bendf;              // [nb*2]
  std::vector<int> species;            // per bead
  int nspecies = 0;
  std::vector<double> sp_sigma;
  std::vector<int> sp_type;
  int maxdeg = 1, maxrole = 1;
  std::vector<int> bead_edges, bead_roles;
  std::vector<double> beta0;           // [nb] rest bend angle (0: the reference's bending)
};

}  // namespace souffle

using namespace souffle;

struct souffle_gpu_system {
  HostTemplate tpl;
  TplLayout L{};
  std::vector<souffle_params> prm;
  std::vector<SysParams> sp;
  souffle_options opt{};
  int n_sys = 0;
  int64_t N = 0;
  int S = 0;
  int subs_per_cta = 1;
  int threads = 128;
  int total_cells = 0;
  std::vector<WorkItem> work;
  std::vector<int2> slots;
  int inter_cap = 96, cand_cap = 128;
  size_t force_smem = 0, pair_smem = 0;
  int pair_chunk = 1;
  cudaStream_t stream = nullptr;
  bool began = false, have_state = false;
  // device
  DevBuf<int> tpl_i;
  DevBuf<float> tpl_f;
  DevBuf<SysParams> d_sys;
  DevBuf<SysState> d_state;
  DevBuf<Chain64> chain64;  // souffle_options.chain_fp64: the chain in FP64
  DevBuf<WorkItem> d_work;
  DevBuf<int2> d_slots;
  DevBuf<int> d_sub_sys, d_bead_sys;
  DevBuf<long long> pos_fx;
  DevBuf<int4> pos32;
  DevBuf<long long> vel, force, partial, kick_c;   // 2^-32 fixed point
  DevBuf<float> sbforce;
  DevBuf<double> staging;
  DevBuf<unsigned int> intra_mask;
  DevBuf<int> inter_ids, inter_count, ref_len;
  DevBuf<int> cand, cand_count;
  DevBuf<int> cell_count, cell_start, sub_rank, sub_cell, cell_subs;
  DevBuf<float> dh_w;
  DevBuf<PairTable> pt;
  DevBuf<dfloat> inv_mass;
  DevBuf<double> mass_d, q_d, sigma_d, len0_d;
  DevBuf<int> type_d, lj_d;
  DevBuf<double> e_bead, e_tot, e_pair_tab;
  DevBuf<unsigned char> e_att_tab;
  DevBuf<int> e_cells;  // the energy pass's cell grid: count, start, fill (3 nc^3 + 1), beads, bead cells (2 n)
  DevBuf<unsigned int> err;
  unsigned int* err_host = nullptr;  // pinned landing word for the error flag's read-back
  // asynchronous snapshots (souffle_gpu_snapshot_enqueue / _wait): per slot a device copy of the
  // state in double, the error flag as it was behind the copy, and the event that marks it
  DevBuf<double> snap[2];
  unsigned int* snap_err = nullptr;  // pinned [2]
  cudaEvent_t snap_ev[2] = {nullptr, nullptr};
  bool snap_pending[2] = {false, false};
  // Brownian systems: per system and template bead drag (2^40 units) and noise scale, the
  // generator skip-ahead table, the step's drag and random forces
  bool any_brownian = false;
  DevBuf<long long> bd_drag, bd_fdrag, bd_fran;
  DevBuf<double> bd_noise;
  DevBuf<unsigned int> lcg_table;
  // encapsulation big beads: positions per system (host, [n][3] box coordinates, in system
  // order) and on the device as fixed point (high words as int4, full words [3][total])
  std::vector<std::vector<double>> bb_pos;
  DevBuf<int4> bb_pos32;
  DevBuf<long long> bb_fx;
  // graphs keyed by (2 window length + rebuild-first, mask of steps in the window that end with
  // a surrogate judgement)
  std::map<std::pair<int, unsigned long long>, cudaGraphExec_t> graphs;
  // learned far-field part (surrogate.cu); null until attached
  souffle::SurrogateCtx* sur = nullptr;
  ~souffle_gpu_system() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    souffle::surrogate_free(sur);
    if (err_host) cudaFreeHost(err_host);
    if (snap_err) cudaFreeHost(snap_err);
    for (auto& e : snap_ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace souffle {
// souffle_gpu.cu: candidate subunit search at the current positions (cell grid + candidates)
souffle_status rebuild_candidates(souffle_gpu_system* h);
// souffle_gpu.cu: waits for the stream and turns the device error flags into a status
souffle_status check_status(souffle_gpu_system* h);
}  // namespace souffle
