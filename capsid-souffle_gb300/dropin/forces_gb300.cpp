// Reference-side binding: a drop-in replacement for SOUFFLE's src/forces.cpp.
//
// Compile this file instead of src/forces.cpp, against the reference's own headers, and link
// libsouffle_gb300.so.  forceCalculation keeps the reference signature (src/forces.h:13-15) and
// the side effects run_simulation relies on (BEAD::tforce, ::sforce, ::bforce); the pair list,
// stretching, bending and pair forces run on the GPU through include/souffle_gpu.h.  The first
// call builds the device handle from subunit 0's beads, edges and faces (every subunit is a copy
// of one template, src/initialize.cpp:295-404).  Errors are fatal, as the reference treats a
// missing file (src/initialize.cpp:29-33): a message and exit(1).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bead.h"
#include "edge.h"
#include "face.h"
#include "forces.h"
#include "souffle_gpu.h"
#include "subunit.h"

using namespace std;

namespace {
souffle_gpu_system* g_handle = nullptr;
vector<double> g_pos, g_tf, g_sf, g_bf;

void die(souffle_status s, const char* what) {
  fprintf(stderr, "souffle_gb300: %s failed (%d): %s\n", what, (int)s, souffle_gpu_last_error());
  exit(1);
}

void create_handle(vector<SUBUNIT>& protein, vector<BEAD>& beads, double lb, double ecut, double ks,
                   double kb, const vector<vector<int> >& lj_a, double ecut_el, double kappa,
                   double elj_att, double NListCutoff) {
  const SUBUNIT& s0 = protein[0];
  const int np = (int)s0.itsB.size();
  const unsigned base = s0.itsB[0]->id;
  vector<int> type(np), eb, et, fb, lj;
  vector<double> q(np), sig(np), m(np), l0;
  for (int i = 0; i < np; i++) {
    type[i] = s0.itsB[i]->type;
    q[i] = s0.itsB[i]->q;
    sig[i] = s0.itsB[i]->sigma;
    m[i] = s0.itsB[i]->m;
  }
  for (EDGE* e : s0.itsE) {
    eb.push_back((int)(e->itsB[0]->id - base));
    eb.push_back((int)(e->itsB[1]->id - base));
    et.push_back(e->type);
    l0.push_back(e->len0);
  }
  for (FACE* f : s0.itsF)
    for (int k = 0; k < 3; k++) fb.push_back((int)(f->itsB[k]->id - base));
  for (size_t k = 0; k < lj_a[0].size(); k++) {
    lj.push_back(lj_a[1][k]);
    lj.push_back(lj_a[2][k]);
  }
  souffle_template t{np, (int)et.size(), (int)(fb.size() / 3), (int)(lj.size() / 2),
                     type.data(), q.data(), sig.data(), m.data(), eb.data(), et.data(), l0.data(),
                     fb.data(), lj.empty() ? nullptr : lj.data(), nullptr /* no rest dihedral */};
  souffle_params p{};
  p.n_subunits = (int)protein.size();
  p.box = (double)beads[0].bx.x;
  p.ks = ks;
  p.kb = kb;
  p.elj_att = elj_att;
  p.lb = lb;
  p.kappa = kappa;
  p.ecut = ecut;
  p.ecut_el = ecut_el;
  p.nlist_cutoff = NListCutoff;
  p.nlist_capacity = (int)beads[0].itsN.size();
  p.center_local = (int)(s0.centerBead->id - base);
  // forceCalculation receives no time step and the forces do not use one; the handle still
  // checks that dt / (2 m) fits its fixed-point kick, so give it the reference's default -t
  p.dt = 0.005;
  p.chain_length = 1;
  p.temperature = 1;
  p.build_freq = 1;
  souffle_status st = souffle_gpu_create(&t, &p, 1, nullptr, &g_handle);
  if (st != SOUFFLE_OK) die(st, "souffle_gpu_create");
  const size_t n = beads.size();
  g_pos.resize(3 * n);
  g_tf.resize(3 * n);
  g_sf.resize(3 * n);
  g_bf.resize(3 * n);
}
}  // namespace

void forceCalculation(vector<SUBUNIT>& protein, double lb, double ni, double qs, vector<BEAD>& subunit_bead,
                      double ecut, double ks, double kb, vector<vector<int> > lj_a, double ecut_el,
                      double kappa, double elj_att, bool updatePairlist, double NListCutoff) {
  (void)ni;
  (void)qs;
  if (!g_handle) {
    create_handle(protein, subunit_bead, lb, ecut, ks, kb, lj_a, ecut_el, kappa, elj_att, NListCutoff);
    updatePairlist = true;
  }
  const size_t n = subunit_bead.size();
  for (size_t i = 0; i < n; i++) {
    g_pos[3 * i] = (double)subunit_bead[i].pos.x;
    g_pos[3 * i + 1] = (double)subunit_bead[i].pos.y;
    g_pos[3 * i + 2] = (double)subunit_bead[i].pos.z;
  }
  souffle_status st = souffle_gpu_set_state(g_handle, g_pos.data(), nullptr);
  if (st != SOUFFLE_OK) die(st, "souffle_gpu_set_state");
  st = souffle_gpu_forces(g_handle, updatePairlist ? 1 : 0, g_tf.data(), g_sf.data(), g_bf.data());
  if (st != SOUFFLE_OK) die(st, "souffle_gpu_forces");
  for (size_t i = 0; i < n; i++) {
    subunit_bead[i].tforce = VECTOR3D(g_tf[3 * i], g_tf[3 * i + 1], g_tf[3 * i + 2]);
    subunit_bead[i].sforce = VECTOR3D(g_sf[3 * i], g_sf[3 * i + 1], g_sf[3 * i + 2]);
    subunit_bead[i].bforce = VECTOR3D(g_bf[3 * i], g_bf[3 * i + 1], g_bf[3 * i + 2]);
  }
}

// The encapsulation term (src/forces.cpp:174-236), called right after forceCalculation
// (src/md.cpp:242,444).  The big beads never move, so the first call hands them to the handle
// (souffle_gpu_set_big_beads: positions, diameter and charge of big_bead[0], hard-core distance)
// and re-evaluates the forces with them (same pair list); from then on forceCalculation's GPU
// forces already hold the big-bead terms and this call adds nothing.  The big beads' own
// eforce / ljforce / tforce, which run_simulation never reads, are not filled in.
void forceCalculation_bigbead(vector<BEAD>& big_bead, vector<BEAD>& subunit_bead, double ecut, double lb,
                              double ni, double qs, double ecut_el, double kappa, double shc) {
  (void)ecut; (void)lb; (void)ni; (void)qs; (void)ecut_el; (void)kappa;
  static bool big_set = false;
  if (big_set || big_bead.empty()) return;
  if (!g_handle) {
    fprintf(stderr, "souffle_gb300: forceCalculation_bigbead before forceCalculation\n");
    exit(1);
  }
  vector<double> bp(3 * big_bead.size());
  for (size_t i = 0; i < big_bead.size(); i++) {
    bp[3 * i] = (double)big_bead[i].pos.x;
    bp[3 * i + 1] = (double)big_bead[i].pos.y;
    bp[3 * i + 2] = (double)big_bead[i].pos.z;
  }
  souffle_status st = souffle_gpu_set_big_beads(g_handle, 0, (int32_t)big_bead.size(), bp.data(),
                                                big_bead[0].sigma, big_bead[0].q, shc);
  if (st != SOUFFLE_OK) die(st, "souffle_gpu_set_big_beads");
  big_set = true;
  st = souffle_gpu_forces(g_handle, 0, g_tf.data(), nullptr, nullptr);
  if (st != SOUFFLE_OK) die(st, "souffle_gpu_forces");
  for (size_t i = 0; i < subunit_bead.size(); i++)
    subunit_bead[i].tforce = VECTOR3D(g_tf[3 * i], g_tf[3 * i + 1], g_tf[3 * i + 2]);
}
