/* souffle_gpu.h -- C ABI of the GB300 force-and-integrate path for SOUFFLE.
 *
 * One handle owns the device state of one or more independent systems
 * ("replicas") that share one capsomere template.  Every system is a
 * template-replicated set of subunits in its own cubic periodic box, exactly
 * the structure generate_lattice builds (src/initialize.cpp:295-404).  All
 * entry points return a souffle_status; none throws, none exits.  Array
 * arguments are plain host pointers in bead order (bead = subunit * np + l),
 * xyz interleaved, systems concatenated in creation order.
 *
 * Replaces (reference file:line in softmaterialslab/capsid-souffle):
 *   souffle_gpu_forces          forceCalculation          src/forces.cpp:13 (decl src/forces.h:13-15)
 *   souffle_gpu_get_pairlist    update_pairlist (result)  src/functions.cpp:69 (decl src/functions.h:31)
 *   souffle_gpu_energies        update_LJ_ES_energies_simplified + stretching/bending/kinetic
 *                               energies                  src/energies.cpp:24, src/bead.cpp:9,
 *                                                         src/edge.cpp:51, src/energies.cpp:13
 *   souffle_gpu_kinetic_energy  particle_kinetic_energy   src/energies.cpp:13 (decl src/energies.h:12)
 *   souffle_gpu_md_steps        the MD-loop body of run_simulation, molecular-dynamics branch
 *                               (NHC half steps, velocity Verlet, pair-list rebuild every B
 *                               steps, forces, COM-velocity removal)  src/md.cpp:400-514,
 *                               update_chain_xi src/functions.cpp:33, THERMOSTAT src/thermostat.h:35
 */
#ifndef SOUFFLE_GPU_H
#define SOUFFLE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum souffle_status {
  SOUFFLE_OK = 0,
  SOUFFLE_ERR_BAD_INPUT = 1,      /* invalid argument or inconsistent template */
  SOUFFLE_ERR_CUDA = 2,           /* a CUDA runtime call failed (see souffle_gpu_last_error) */
  SOUFFLE_ERR_NL_OVERFLOW = 3,    /* a pair-list or candidate capacity was exceeded */
  SOUFFLE_ERR_NONFINITE = 4,      /* a force, velocity or kinetic energy became NaN/Inf */
  SOUFFLE_ERR_NO_DEVICE = 5,      /* no CUDA device, or the library was built for another GPU */
  SOUFFLE_ERR_STATE = 6           /* call out of order (e.g. md_steps before set_state) */
} souffle_status;

/* One capsomere template: the contents of a reference infile
 * (src/initialize.cpp:47-128).  Indices are template-local. */
typedef struct souffle_template {
  int32_t np;                 /* beads per subunit (1..256) */
  int32_t ne;                 /* edges per subunit */
  int32_t nf;                 /* faces per subunit */
  int32_t n_lj;               /* rows of the directed LJ-attraction table */
  const int32_t* bead_type;   /* [np] */
  const double* bead_charge;  /* [np] */
  const double* bead_sigma;   /* [np] diameter in sigma units */
  const double* bead_mass;    /* [np] */
  const int32_t* edge_beads;  /* [2*ne] */
  const int32_t* edge_type;   /* [ne]  0 = spring only, != 0 = bending edge */
  const double* edge_len0;    /* [ne] */
  const int32_t* face_beads;  /* [3*nf] */
  const int32_t* lj_types;    /* [2*n_lj] (type of bead i, type of neighbour j) */
  /* Optional, no reference counterpart (the reference's bending has no rest angle,
   * src/edge.cpp:51-67): a rest shape [np][3].  When given, every bending edge relaxes to its
   * signed bend angle beta0 in that shape, E = kb (1 - cos(beta - beta0)); NULL (or a flat
   * shape) gives the reference's kb (1 - |n0 . n1|) exactly. */
  const double* bend_rest_pos;
} souffle_template;

/* Per-system parameters in reduced units, as run_simulation derives them
 * (src/md.cpp:135-196). */
typedef struct souffle_params {
  int32_t n_subunits;     /* -S */
  double box;             /* cubic box edge (src/md.cpp:159) */
  double ks, kb;          /* -s, -b */
  double elj_att;         /* -E */
  double lb;              /* Bjerrum length (src/md.cpp:165) */
  double kappa;           /* inverse screening length (src/md.cpp:169) */
  double ecut;            /* LJ cut-off (src/md.cpp:161) */
  double ecut_el;         /* Debye-Hueckel cut-off; 0 = none (src/md.cpp:171) */
  double nlist_cutoff;    /* pair-list radius (src/md.cpp:172-173) */
  int32_t nlist_capacity; /* reference pair-list capacity (src/md.cpp:231-232); lists longer
                             than this are reported by souffle_gpu_pairlist_stats */
  int32_t center_local;   /* template-local index of the subunit centre bead
                             (src/initialize.cpp:266-288) */
  double dt;              /* -t */
  int32_t chain_length;   /* -q */
  double nhc_mass;        /* -Q */
  double temperature;     /* reduced temperature T = K/298 (src/md.cpp:138) */
  int32_t build_freq;     /* -B: rebuild the pair list when step % B == 0 */
  int32_t brownian;       /* -D b: 1 = the reference's Brownian dynamics (src/md.cpp:415-431,
                             461-501), 0 = molecular dynamics with the Nose-Hoover chain */
  double damp;            /* -d: damping time of the Brownian integrator (drag m / damp) */
} souffle_params;

typedef struct souffle_options {
  int32_t inter_capacity; /* per-bead capacity of inter-subunit pair entries (0 = default 96) */
  int32_t cand_capacity;  /* per-subunit capacity of candidate subunits (0 = default 128) */
  int32_t compat_quirks;  /* 1 (default when 0 is not requested explicitly via -1): reproduce the
                             reference's stale-distance reuse for subunit 0's centre bead
                             (src/functions.cpp:97); -1 turns it off */
  int32_t device;         /* CUDA device ordinal */
  int32_t threads_per_cta;/* force-kernel block size, 64..256 in steps of 32 (0 = default 256;
                             souffle_gpu_autotune chooses it by measurement) */
  int32_t subunits_per_cta;/* subunits per force-kernel CTA (0 = default: up to 128 beads) */
  int32_t chain_fp64;     /* 1: run the Nose-Hoover chain in FP64 on one thread (the reference's
                             double arithmetic, src/functions.cpp:33-58), a validation variant of
                             the default double-float chain; slower by several microseconds per
                             step on GB300's FP64 latency.  0 = double-float (default) */
} souffle_options;

typedef struct souffle_energies {
  /* totals over the system's beads, the sums of src/md.cpp:586-605 */
  double kinetic, stretching, bending, lj, electrostatic;
  double thermo_pe, thermo_ke;  /* Nose-Hoover chain energies (src/thermostat.h:43-52) */
  double temperature;           /* 2 KE / (3 N) (src/md.cpp:622) */
  double vcom_magnitude;        /* |mean velocity| removed at the last step (src/md.cpp:623) */
  /* encapsulation: the big-bead pair parts of lj and electrostatic (already included in them),
     i.e. the sums over all big beads of src/md.cpp:606-614 (capenergy.out) */
  double bigbead_lj, bigbead_electrostatic;
} souffle_energies;

typedef struct souffle_pairlist_stats {
  double mean_length;     /* mean reference-list length (intra + inter entries) */
  int32_t max_length;     /* longest reference list */
  int32_t max_inter;      /* longest inter-subunit part */
  int32_t over_reference_capacity; /* beads whose list exceeds nlist_capacity */
} souffle_pairlist_stats;

typedef struct souffle_gpu_system souffle_gpu_system;

/* Create a handle for n_systems independent systems sharing one template.
 * opts may be NULL.  On success *out owns device memory until destroy. */
souffle_status souffle_gpu_create(const souffle_template* tpl, const souffle_params* params,
                                  int32_t n_systems, const souffle_options* opts,
                                  souffle_gpu_system** out);
souffle_status souffle_gpu_destroy(souffle_gpu_system* h);

/* Total beads / subunits over all systems. */
int64_t souffle_gpu_num_beads(const souffle_gpu_system* h);

/* Copy a state in (host, double) / out.  vel may be NULL on set (zero). */
souffle_status souffle_gpu_set_state(souffle_gpu_system* h, const double* pos, const double* vel);

/* Encapsulation big beads (-p; replaces forceCalculation_bigbead src/forces.cpp:174-236 and
 * update_LJ_ES_energies_bigbeads src/energies.cpp:96-137, as called at src/md.cpp:242,299,444,
 * 584): n static beads of diameter sigma and charge q (e) in one system, at pos [n][3] (box
 * coordinates, as generate_big_beads src/initialize.cpp:566-680 places or restarts them).
 * Every subunit bead feels each big bead through the screened Coulomb term (no shift; none at
 * all without a DH cut-off) and a WCA term shifted by delta = (sigma + sigma_j)/2 - shc with
 * hard-core distance shc; the reference never moves them.  Forces (souffle_gpu_forces, MD and
 * Brownian steps), energies and the Brownian noise sequence (three uniforms per big bead after
 * the subunit beads' draws, src/md.cpp:482-487) include them from the next call on; n = 0
 * removes them. */
souffle_status souffle_gpu_set_big_beads(souffle_gpu_system* h, int32_t system, int32_t n, const double* pos,
                                         double sigma, double charge, double shc);
souffle_status souffle_gpu_get_state(souffle_gpu_system* h, double* pos, double* vel);

/* forceCalculation: rebuild != 0 first rebuilds the pair lists (update_pairlist).
 * tforce/sforce/bforce (each N*3, may be NULL) receive total, stretching and bending
 * force per bead. */
souffle_status souffle_gpu_forces(souffle_gpu_system* h, int32_t rebuild, double* tforce,
                                  double* sforce, double* bforce);

/* The current pair lists in the reference's order (ascending neighbour id):
 * counts[N], ids[N*cap] padded with -1 (entries beyond cap are dropped and
 * counted in counts). */
souffle_status souffle_gpu_get_pairlist(souffle_gpu_system* h, int32_t cap, int32_t* counts,
                                        int32_t* ids);
souffle_status souffle_gpu_pairlist_stats(souffle_gpu_system* h, int32_t system,
                                          souffle_pairlist_stats* out);

/* Energy block of run_simulation (src/md.cpp:553-605) for one system.
 * Per-bead arrays (N_system each, may be NULL): se, be, ne (LJ), ce (DH), ke. */
souffle_status souffle_gpu_energies(souffle_gpu_system* h, int32_t system, souffle_energies* out,
                                    double* se, double* be, double* ne, double* ce, double* ke);

/* particle_kinetic_energy of one system (before COM removal semantics: the
 * current velocities as held). */
souffle_status souffle_gpu_kinetic_energy(souffle_gpu_system* h, int32_t system, double* ke);

/* Prepare the MD loop: initial forces with a pair-list rebuild (src/md.cpp:241),
 * particle_ke, thermostat chain set-up (src/md.cpp:187-196, 258). */
souffle_status souffle_gpu_md_begin(souffle_gpu_system* h);

/* Run MD-loop iterations a = first_step .. first_step + n_steps - 1 for every
 * system (src/md.cpp:387-514).  Uses CUDA graphs for whole rebuild windows. */
souffle_status souffle_gpu_md_steps(souffle_gpu_system* h, int64_t first_step, int32_t n_steps);

/* souffle_gpu_md_steps without the wait: queues the same iterations on the handle's stream and
 * returns.  Device-side errors of queued steps (pair-list overflow, non-finite forces) are
 * reported by the next souffle_gpu_md_steps or souffle_gpu_synchronize.  No reference
 * counterpart: lets a caller queue many windows, or time steps with events, without a host
 * round trip per call. */
souffle_status souffle_gpu_md_enqueue(souffle_gpu_system* h, int64_t first_step, int32_t n_steps);

/* Per-system scalars after the last step: particle_ke, xi[0], |v_com|. */
souffle_status souffle_gpu_md_scalars(souffle_gpu_system* h, int32_t system, double* ke,
                                      double* xi0, double* vcom);

/* Block until all queued GPU work of the handle has finished; reports the device-side errors
 * of queued steps like souffle_gpu_md_steps. */
souffle_status souffle_gpu_synchronize(souffle_gpu_system* h);

/* Asynchronous state read-back for writers that overlap file output with the next MD steps (the
 * restart and movie writers of src/md.cpp:526-546,647-678 read the state at the output step).
 * souffle_gpu_snapshot_enqueue queues, behind all work queued so far, what souffle_gpu_get_state
 * returns (positions; velocities with the pending centre-of-mass velocity removed) into slot 0 or
 * 1 and from there into pos / vel (N*3 each, may be NULL; page-locked memory from
 * souffle_gpu_host_alloc makes the copy truly asynchronous), and returns at once.  The host buffers
 * must stay untouched until souffle_gpu_snapshot_wait(h, slot) has returned; it blocks until the
 * copy has landed and reports the device-side errors of the work queued before it, as
 * souffle_gpu_synchronize does.  A slot takes one snapshot at a time.  No reference counterpart. */
souffle_status souffle_gpu_snapshot_enqueue(souffle_gpu_system* h, int32_t slot, double* pos, double* vel);
souffle_status souffle_gpu_snapshot_wait(souffle_gpu_system* h, int32_t slot);
/* Page-locked host memory for the snapshot buffers (NULL on failure); free with
 * souffle_gpu_host_free. */
void* souffle_gpu_host_alloc(int64_t bytes);
void souffle_gpu_host_free(void* p);

/* The CUDA stream (cudaStream_t) all work of the handle is queued on, so a caller can
 * order its own work or record events against it.  No reference counterpart. */
void* souffle_gpu_stream(souffle_gpu_system* h);

/* Per-kernel device times of MD steps a = first_step .. first_step + n_steps - 1, measured
 * with CUDA events between the launches on the handle's stream (launches are issued one by
 * one, not through a graph).  No reference counterpart: measurement support. */
typedef struct souffle_kernel_times {
  double drift_ms;    /* sum over steps: half-kick + drift kernel */
  double rebuild_ms;  /* sum over rebuild steps: cell grid, candidates, bead pairs */
  double forces_ms;   /* sum over steps: force + half-kick + thermostat kernel */
  int32_t steps, rebuilds;
} souffle_kernel_times;
souffle_status souffle_gpu_md_profile(souffle_gpu_system* h, int64_t first_step, int32_t n_steps,
                                      souffle_kernel_times* out);

/* Autotuner (no reference counterpart): times the force kernel (forces only, no state change) at
 * every candidate CTA shape -- subunits per CTA and threads per CTA -- over the handle's current
 * state, keeps the fastest, and reports it.  trials = timed launches per shape.  The chosen shape
 * can be passed back through souffle_options to skip the search next time. */
typedef struct souffle_tuning {
  int32_t subunits_per_cta, threads_per_cta;
  double forces_us;          /* mean force-kernel time of the chosen shape */
  double default_forces_us;  /* the same for the default shape */
  int32_t candidates;        /* shapes measured */
} souffle_tuning;
souffle_status souffle_gpu_autotune(souffle_gpu_system* h, int32_t trials, souffle_tuning* out);

/* Kinetic energy and velocity sum of a caller-owned device array, for callers that must not
 * allocate device memory after start-up (a loop that reserves all its GPU memory up front, or a
 * framework that owns the device heap).  No counterpart in the reference: it is the
 * particle_kinetic_energy reduction with its per-block scratch in a fixed array inside the
 * library (about 64 KB per GPU, held until exit) instead of a handle's buffers.
 *   vel    device pointer, n_beads x 3 doubles (xyz interleaved)
 *   mass   device pointer, n_beads doubles, or NULL for unit masses
 *   out    device pointer, 4 doubles: sum 1/2 m |v|^2, sum vx, sum vy, sum vz
 *   stream cudaStream_t (NULL = default stream); the call is asynchronous on it
 * At most 4,194,304 beads (SOUFFLE_ERR_BAD_INPUT beyond).  Nothing is allocated or freed.  The
 * first call on a device looks up the scratch address for that device and keeps it for the rest
 * of the process, so make it before any stream capture, and do not reset the device
 * (cudaDeviceReset) after it: the kept address would then be stale.  All calls share the scratch:
 * calls that overlap on the GPU race; order them on one stream.  The result is bitwise the same
 * on every call for the same input. */
souffle_status souffle_gpu_kinetic_energy_noalloc(const double* vel, const double* mass, int64_t n_beads,
                                                  double* out, void* stream);

/* Text of the last error on this thread. */
const char* souffle_gpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
