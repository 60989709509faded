// Oracle test infrastructure.  Entry point for the reference MD driver built
// from the unmodified SOUFFLE sources: calls run_simulation (src/md.cpp:29)
// only.  The reference main (src/main.cpp:10-17) also calls analyze_output,
// which divides by zero for subunit sizes other than 41/43/78
// (src/analysis.cpp:81-85), so the checker skips it.
#include "md.h"

int main(int argc, char* argv[]) { return run_simulation(argc, argv); }
