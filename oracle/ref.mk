# Oracle test infrastructure: builds the reference SOUFFLE sources, unmodified
# and where they lie, against the stand-in headers in oracle/shim/, into
# oracle/_ref/ (git-ignored).  Two programs come out:
#   oracle/_ref/ref_run    run_simulation only (the reference MD driver)
#   oracle/_ref/ref_dump   forces, pair lists and energies for one state
#   oracle/_ref/ref_analyze  analyze_output only (the reference post-run analysis)
# Usage: make -f oracle/ref.mk REF=/path/to/capsid-souffle -j8
# The reference's own build (src/Makefile) needs mpicxx, Boost and GSL, none of
# which exist here, so this recipe compiles the same files with g++ instead,
# at the reference's optimisation flags (-O3 -fopenmp, src/Makefile:21).

REF ?= /root/reference
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(HERE)_ref
CXX ?= g++
CXXFLAGS ?= -O3 -fopenmp -std=c++17 -w
INC := -I$(HERE)shim -I$(REF)/src

LIBSRC := bead edge face subunit functions forces energies initialize analysis
LIBOBJ := $(addprefix $(OUT)/obj/,$(addsuffix .o,$(LIBSRC)))

all: $(OUT)/ref_run $(OUT)/ref_dump $(OUT)/ref_analyze

$(OUT)/obj/%.o: $(REF)/src/%.cpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/obj/md.o: $(REF)/src/md.cpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/ref_run: $(HERE)harness/ref_run_main.cpp $(LIBOBJ) $(OUT)/obj/md.o
	$(CXX) $(CXXFLAGS) $(INC) $^ -o $@

$(OUT)/ref_dump: $(HERE)harness/ref_dump_main.cpp $(LIBOBJ)
	$(CXX) $(CXXFLAGS) $(INC) $^ -o $@

$(OUT)/ref_analyze: $(HERE)harness/ref_analyze_main.cpp $(LIBOBJ)
	$(CXX) $(CXXFLAGS) $(INC) $^ -o $@

# Link-substitution check of the drop-in binding: the reference driver with src/forces.cpp
# replaced by capsid-souffle_gb300/dropin/forces_gb300.cpp, linked to libsouffle_gb300.so.
GB300 := $(HERE)../capsid-souffle_gb300
GB300LIB := $(GB300)/_build
DROPOBJ := $(filter-out $(OUT)/obj/forces.o,$(LIBOBJ))

$(OUT)/obj/forces_gb300.o: $(GB300)/dropin/forces_gb300.cpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) $(INC) -I$(HERE)../include -c $< -o $@

$(OUT)/ref_run_gb300: $(HERE)harness/ref_run_main.cpp $(DROPOBJ) $(OUT)/obj/md.o $(OUT)/obj/forces_gb300.o
	$(CXX) $(CXXFLAGS) $(INC) $^ -L$(GB300LIB) -lsouffle_gb300 -Wl,-rpath,$(abspath $(GB300LIB)) -o $@

dropin: $(OUT)/ref_run_gb300

clean:
	rm -rf $(OUT)

.PHONY: all clean dropin
