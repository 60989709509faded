// Oracle test infrastructure.  Entry point for the reference's post-run analysis built from the
// unmodified SOUFFLE sources: calls analyze_output (src/analysis.cpp:16), which reads
// outfiles/energy.out and outfiles/ovito.lammpstrj in the working directory and writes
// outfiles/analysis.{ms,gr,so,rdat} and outfiles/info.gr.  It determines the subunit size from
// the bead count (41, 43 or 78 beads, src/analysis.cpp:81-83), so fixtures use 43-bead subunits.
// The globals the linked reference sources expect are defined here, as src/md.cpp:21-27 does.
#include "utility.h"

unsigned int lowerBound;
unsigned int upperBound;
unsigned int sizFVec;
unsigned int extraElements;
mpi::environment env;
mpi::communicator world;

int analyze_output(int, char**);

int main(int argc, char* argv[]) { return analyze_output(argc, argv); }
