/*
 * Post-run analysis of a trajectory on the GPU: per frame the bead-pair correlation histogram,
 * the oligomer (cluster) mass spectrum and the sub-oligomer size histogram, the three per-frame
 * products of the reference's analyze_output (src/analysis.cpp:16-297).
 *
 * Definitions, as the reference's loops compute them:
 *   pcf         every pair i < j of beads of type pcf_type whose separation r is below box/2 adds
 *               one to bin floor(r / (box / (2 * pcf_bins)))             (src/analysis.cpp:117-136)
 *   oligomers   connected components of subunits, two subunits joined when any of their beads are
 *               closer than `contact`; oligomer_counts[k] = number of oligomers of k + 1 subunits
 *                                                                          (src/analysis.cpp:140-186)
 *   sub-oligomers  connected components of beads of type so_type, joined when closer than
 *               `contact`; so_bins[(size - 1) / 3] += 1 for each, 2 * n_subunits bins
 *                                                                          (src/analysis.cpp:189-245)
 * Separations follow dist() (src/functions.h:42-56) with the image rule chosen by `image`:
 *   SOUFFLE_IMAGE_REFERENCE  the analysis as shipped: its beads never get a half-box vector, so
 *                            every nonzero coordinate difference d becomes d - box (d > 0) or
 *                            d + box (d < 0) -- the long way round the periodic box;
 *   SOUFFLE_IMAGE_MINIMUM    the minimum image (one shift when |d| > box / 2), the evident intent.
 * Separations are evaluated in FP64 with a sum of squares (dx^2 + dy^2) + dz^2, a correctly
 * rounded square root and division; a pair whose comparison with a threshold cannot be told in
 * FP32 is decided in FP64.  Results are integers and do not depend on thread scheduling.
 *
 * Beads are ordered subunit by subunit (bead index = subunit * beads_per_subunit + local index),
 * positions are [n_beads][3] doubles as the trajectory prints them.  The reference infers
 * beads_per_subunit from the bead count (41, 43 or 78, src/analysis.cpp:81-83); here the caller
 * passes it.
 */
#ifndef SOUFFLE_ANALYSIS_H
#define SOUFFLE_ANALYSIS_H

#include <stdint.h>

#include "souffle_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { SOUFFLE_IMAGE_REFERENCE = 0, SOUFFLE_IMAGE_MINIMUM = 1 };

typedef struct souffle_analysis_options {
  int32_t image;     /* SOUFFLE_IMAGE_REFERENCE (default of the reference) or SOUFFLE_IMAGE_MINIMUM */
  int32_t pcf_type;  /* bead type of the pair correlation, 5 in the reference (src/analysis.cpp:67) */
  int32_t pcf_bins;  /* 1..4096; 100 in the reference (src/analysis.cpp:66) */
  int32_t so_type;   /* bead type of the sub-oligomers, 0 in the reference (src/analysis.cpp:192) */
  double contact;    /* contact distance, 2 in the reference (src/analysis.cpp:154,210) */
} souffle_analysis_options;

/* Fills the reference's settings (image rule as shipped, type 5, 100 bins, type 0, contact 2). */
void souffle_analysis_default_options(souffle_analysis_options* opt);

typedef struct souffle_analysis souffle_analysis;

/* One handle per trajectory shape: n_beads = n_subunits * beads_per_subunit, 1 <= beads_per_subunit
 * <= 256, box the periodic box length (twice the trajectory's upper box bound).  Device memory
 * for one frame and its work lists is allocated here; device = CUDA ordinal.  Replaces the set-up
 * block of analyze_output (src/analysis.cpp:79-95). */
souffle_status souffle_analysis_create(int64_t n_beads, int32_t beads_per_subunit, double box,
                                       const souffle_analysis_options* opt, int32_t device,
                                       souffle_analysis** out);
souffle_status souffle_analysis_destroy(souffle_analysis* h);

/* Analyses n_frames frames held in host memory, one after the other: the body of the frame loop of
 * analyze_output (src/analysis.cpp:117-262) for frames at or past the equilibrium step.
 *   pos        [n_frames][n_beads][3]
 *   types      [n_frames][n_beads], or NULL to use the types of the previous call's last frame
 *              (the first call must pass them)
 *   pcf        [n_frames][pcf_bins]            pair counts                      (may be NULL)
 *   oligomers  [n_frames][n_subunits]          oligomer_counts as defined above (may be NULL)
 *   so_bins    [n_frames][2 * n_subunits]      sub-oligomer histogram           (may be NULL)
 *   labels     [n_frames][n_subunits]          smallest subunit index of each subunit's oligomer
 *                                              (no counterpart in the reference; may be NULL)
 * Returns SOUFFLE_ERR_BAD_INPUT when a sub-oligomer is larger than 6 * n_subunits beads (the
 * reference writes past its histogram there, src/analysis.cpp:240). */
souffle_status souffle_analysis_frames(souffle_analysis* h, int64_t n_frames, const double* pos,
                                       const int32_t* types, int64_t* pcf, int64_t* oligomers,
                                       int64_t* so_bins, int32_t* labels);

/* One frame already in device memory (pos_dev [n_beads][3], types_dev [n_beads]), enqueued on
 * the handle's stream without waiting; results stay on the device (int64 pcf_dev [pcf_bins],
 * oligomers_dev [n_subunits], so_bins_dev [2 * n_subunits], int32 labels_dev [n_subunits] or NULL)
 * and are valid once souffle_analysis_synchronize returns OK.  A work-list overflow or an
 * oversized sub-oligomer is reported by that call. */
souffle_status souffle_analysis_enqueue(souffle_analysis* h, const double* pos_dev, const int32_t* types_dev,
                                        int64_t* pcf_dev, int64_t* oligomers_dev, int64_t* so_bins_dev,
                                        int32_t* labels_dev);
souffle_status souffle_analysis_synchronize(souffle_analysis* h);

/* The handle's CUDA stream (a cudaStream_t). */
void* souffle_analysis_stream(souffle_analysis* h);

/* Counters of the last frame: candidate subunit pairs tested bead by bead, bead pairs decided in
 * FP64 because FP32 could not tell them. */
souffle_status souffle_analysis_last_counts(souffle_analysis* h, int64_t* candidate_pairs, int64_t* fp64_pairs);

#ifdef __cplusplus
}
#endif

#endif /* SOUFFLE_ANALYSIS_H */
