// Post-run analysis of the driver (analysis_host.cpp).
#pragma once

namespace souffle_host {

struct AnalysisCli {
  int beads_per_subunit = 0;  // 0: the reference's rule (41, 43 or 78 from the bead count)
  int image = 0;              // SOUFFLE_IMAGE_REFERENCE or SOUFFLE_IMAGE_MINIMUM
};

// analyze_output (src/analysis.cpp:16-297) over outfiles/energy.out and outfiles/ovito.lammpstrj
// in the working directory.  Returns 0 on success (including "nothing to analyse"), 1 on error.
int analyze_output(const AnalysisCli& cli);

}  // namespace souffle_host
