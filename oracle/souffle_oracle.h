/* Oracle test infrastructure -- NOT the product.
 *
 * A CPU restatement, in plain C, of SOUFFLE's force-and-integrate path
 * (softmaterialslab/capsid-souffle, src/): pair-list rebuild, stretching,
 * dihedral bending, Debye-Hueckel + LJ/WCA pair forces, energies, and the
 * velocity-Verlet / Nose-Hoover-chain MD loop.  Arithmetic follows the
 * reference's types (long double vectors, double scalars) so that on x86-64
 * it reproduces the compiled reference bit for bit; build with
 * -DORACLE_REAL=double for the FP64 variant.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker.
 */
#ifndef SOUFFLE_ORACLE_H
#define SOUFFLE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Template-replicated system, as built by generate_lattice
 * (src/initialize.cpp:295-404).  All template arrays use local indices. */
typedef struct oracle_desc {
  int n_sub;          /* number of subunits S */
  int np;             /* beads per subunit */
  int ne;             /* edges per subunit */
  int nf;             /* faces per subunit */
  int n_lj;           /* rows of the directed LJ-attraction table */
  const int* b_type;  /* [np] */
  const double* b_q;  /* [np] */
  const double* b_sigma; /* [np] */
  const double* b_mass;  /* [np] */
  const int* e_b;     /* [ne*2] */
  const int* e_type;  /* [ne] */
  const double* e_len0; /* [ne] */
  const int* f_b;     /* [nf*3] */
  const int* lj_t;    /* [n_lj*2] (type_i, type_j) */
  double box;         /* cubic box edge */
  double lb, kappa, ecut, ecut_el, elj_att, ks, kb, nlist_cutoff;
  int nlist_capacity; /* per-bead pair-list capacity (src/md.cpp:229-239) */
  int center_local;   /* template-local index of the subunit centre bead */
} oracle_desc;

typedef struct oracle_sys oracle_sys;

/* Centre bead of subunit 0 (src/initialize.cpp:266-288): returns local index. */
int oracle_center_bead(int np, const double* pos, double box);

/* Build derived topology.  Returns NULL on an inconsistent template (a bending
 * edge without two faces).  The descriptor arrays are copied. */
oracle_sys* oracle_create(const oracle_desc* d);
void oracle_destroy(oracle_sys* s);
void oracle_set_threads(int n);

/* Load a state (double in, held internally in the oracle's real type). */
void oracle_set_state(oracle_sys* s, const double* pos, const double* vel);
void oracle_get_state(const oracle_sys* s, double* pos, double* vel);

/* forceCalculation (src/forces.cpp:13-171).  rebuild != 0 runs update_pairlist
 * first.  Returns the number of pair-list overflows (0 when it fits). */
int oracle_forces(oracle_sys* s, int rebuild);
/* Per-bead results of the last oracle_forces: tforce, sforce, bforce [N*3]. */
void oracle_get_forces(const oracle_sys* s, double* tforce, double* sforce, double* bforce);
/* Pair lists: counts [N], ids [N*cap] (cap = nlist_capacity). */
void oracle_get_pairlist(const oracle_sys* s, int* counts, int* ids);

/* Energy block (src/md.cpp:553-594 with src/energies.cpp:13-93,
 * src/bead.cpp:9-14, src/edge.cpp:51-67): per-bead se, ke, be, ne, ce [N]. */
void oracle_energies(oracle_sys* s, double* se, double* ke, double* be, double* ne, double* ce);
double oracle_kinetic_energy(oracle_sys* s);

/* Encapsulation big beads (src/forces.cpp:174-236, src/energies.cpp:96-137): n static beads at
 * pos [n][3] of diameter sigma, charge q and hard-core distance shc.  oracle_forces adds their
 * forces to tforce and oracle_energies their energies to ne and ce; n = 0 removes them.
 * oracle_big_bead_energies: the big-bead sums of the last oracle_energies (src/md.cpp:606-614). */
void oracle_set_big_beads(oracle_sys* s, int n, const double* pos, double sigma, double charge, double shc);
void oracle_big_bead_energies(const oracle_sys* s, double* big_ne, double* big_ce);

/* Nose-Hoover chain (src/md.cpp:187-196). */
typedef struct oracle_nhc {
  int m;             /* chain length */
  double q[16], xi[16], eta[16], t[16];
  unsigned long dof[16];
} oracle_nhc;
void oracle_nhc_init(oracle_nhc* c, int chain_len, double q_mass, double temperature, int n_beads);

/* One MD step of src/md.cpp:400-514 (molecular dynamics branch) at loop index
 * a.  ke_io carries particle_ke between steps.  Writes |v_com| removed. */
int oracle_md_step(oracle_sys* s, oracle_nhc* c, unsigned a, double dt, int build_freq,
                   double* ke_io, double* vcom_mag);

/* Reference loop trip count for -T steps and -t dt (src/md.cpp:137,387). */
unsigned oracle_loop_end(double steps, double dt);

#ifdef __cplusplus
}
#endif
#endif
