// Oracle test infrastructure.  Force / pair-list / energy dump built on the
// unmodified SOUFFLE sources (everything in src/ except md.cpp and main.cpp).
//
// It repeats the set-up half of run_simulation (src/md.cpp:132-241) for one
// state: generate_lattice reads infiles/<-f> and the newest
// outfiles/restart_*.out in the working directory, the unit and cut-off
// derivation follows src/md.cpp:135-173, the pair-list capacity
// src/md.cpp:229-239.  It then calls the reference's own forceCalculation
// (src/forces.cpp:13) with a pair-list rebuild and the reference energy
// routines in the order of src/md.cpp:553-594, and prints every result at
// full long-double precision:
//   P <name> <value>                      derived parameters
//   F <i> tforce(3) sforce(3) bforce(3)   per-bead forces
//   N <i> <n> <ids...>                    per-bead pair list (up to the -1)
//   E <i> se ke be ne ce                  per-bead energies
//   K <ke>                                particle_kinetic_energy
// With -p 1 (encapsulation) it also places the big beads with the reference's own
// generate_big_beads (src/initialize.cpp:566-680; restart: the newest outfiles/rb_*.out),
// adds forceCalculation_bigbead (src/forces.cpp:174-236) after forceCalculation and
// update_LJ_ES_energies_bigbeads (src/energies.cpp:96-137) after the pair energies, as
// src/md.cpp:242,299 do, and prints
//   BB <i> x y z                          big-bead positions as held
//   G <ne> <ce>                           big-bead energy sums (src/md.cpp:606-614)
// Option letters match the reference driver (src/md.cpp:53-90).
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bead.h"
#include "edge.h"
#include "energies.h"
#include "face.h"
#include "forces.h"
#include "functions.h"
#include "initialize.h"
#include "subunit.h"

unsigned int lowerBound;
unsigned int upperBound;
unsigned int sizFVec;
unsigned int extraElements;
mpi::environment env;
mpi::communicator world;

int main(int argc, char* argv[]) {
  std::string file_name = "41part_c";
  double capsomere_concentration = 200, salt_concentration = 500, number_capsomeres = 64;
  double ks = 50, kb = 20, ecut_c = 12, elj_att = 2, NListCutoff_c = 7.5;
  bool encapsulation = false;
  double radius_a = 3.0, charge_a = -78.0, shc = 3.5;
  int number_bigbeads = 1;
  for (int a = 1; a + 1 < argc; a += 2) {
    const char* k = argv[a];
    const char* v = argv[a + 1];
    if (!std::strcmp(k, "-f")) file_name = v;
    else if (!std::strcmp(k, "-C")) capsomere_concentration = atof(v);
    else if (!std::strcmp(k, "-c")) salt_concentration = atof(v);
    else if (!std::strcmp(k, "-S")) number_capsomeres = atof(v);
    else if (!std::strcmp(k, "-s")) ks = atof(v);
    else if (!std::strcmp(k, "-b")) kb = atof(v);
    else if (!std::strcmp(k, "-e")) ecut_c = atof(v);
    else if (!std::strcmp(k, "-E")) elj_att = atof(v);
    else if (!std::strcmp(k, "-L")) NListCutoff_c = atof(v);
    else if (!std::strcmp(k, "-p")) encapsulation = atoi(v) != 0;
    else if (!std::strcmp(k, "-a")) radius_a = atof(v);
    else if (!std::strcmp(k, "-G")) charge_a = atof(v);
    else if (!std::strcmp(k, "-m")) number_bigbeads = atoi(v);
    else if (!std::strcmp(k, "-H")) shc = atof(v);
    else {
      fprintf(stderr, "unknown option %s\n", k);
      return 2;
    }
  }

  std::vector<BEAD> subunit_bead;
  std::vector<EDGE> subunit_edge;
  std::vector<SUBUNIT> protein;
  std::vector<FACE> subunit_face;
  double bondlength, SIsigma, SImass;
  bool restartFile = true;
  int restartStep = 0;
  unsigned int cluster_size = 0;
  std::vector<std::vector<int> > lj_a = generate_lattice(
      capsomere_concentration, number_capsomeres, file_name, bondlength, SIsigma, SImass,
      subunit_bead, subunit_edge, protein, subunit_face, restartFile, restartStep, false,
      cluster_size);

  const double Avagadro = 6.022e23;
  const double Pi = 3.14159;
  const double qs = 1;
  double box_x = pow((number_capsomeres * 1000 /
                      (capsomere_concentration * pow(SIsigma, 3) * Avagadro)),
                     1.0 / 3.0);
  double ecut = 2.5 * (SIsigma / 1e-9);
  double lb = (0.701e-9) / SIsigma;
  double ni = salt_concentration * Avagadro * SIsigma * SIsigma * SIsigma;
  double kappa = sqrt(8 * Pi * ni * lb * qs * qs);
  double screen = 1 / kappa;
  double ecut_el = screen * ecut_c;
  double NListCutoff;
  if (ecut_el > ecut)
    NListCutoff = ecut_el + NListCutoff_c;
  else
    NListCutoff = ecut + NListCutoff_c;

  unsigned int rangeIons = protein.size();
  lowerBound = 0;
  upperBound = rangeIons - 1;
  sizFVec = rangeIons;

  unsigned int NListVectorSize =
      ceil((NListCutoff + 0.5) * (NListCutoff + 0.5) * (NListCutoff + 0.5));
  if (NListVectorSize > subunit_bead.size()) NListVectorSize = subunit_bead.size();
  for (unsigned int i = 0; i < subunit_bead.size(); i++) subunit_bead[i].itsN.assign(NListVectorSize, -1);

  forceCalculation(protein, lb, ni, qs, subunit_bead, ecut, ks, kb, lj_a, ecut_el, kappa, elj_att,
                   true, NListCutoff);
  std::vector<BEAD> big_beads;
  if (encapsulation) {
    VECTOR3D box_size = VECTOR3D(box_x, box_x, box_x);
    big_beads = generate_big_beads(number_bigbeads, 2 * radius_a, subunit_bead, box_size, 100.0, 3, charge_a,
                                   1000000, restartFile);
    forceCalculation_bigbead(big_beads, subunit_bead, ecut, lb, ni, qs, ecut_el, kappa, shc);
  }

  printf("P restart_step %d\n", restartStep);
  printf("P n_beads %zu\n", subunit_bead.size());
  printf("P n_subunits %zu\n", protein.size());
  printf("P box %La\n", (long double)box_x);
  printf("P sigma_si %La\n", (long double)SIsigma);
  printf("P mass_si %La\n", (long double)SImass);
  printf("P ecut %La\n", (long double)ecut);
  printf("P lb %La\n", (long double)lb);
  printf("P kappa %La\n", (long double)kappa);
  printf("P ecut_el %La\n", (long double)ecut_el);
  printf("P nlist_cutoff %La\n", (long double)NListCutoff);
  printf("P nlist_capacity %u\n", NListVectorSize);
  printf("P center_bead %u\n", protein[0].centerBead->id);
  printf("P long_double_mant_dig %d\n", (int)LDBL_MANT_DIG);

  for (size_t i = 0; i < subunit_bead.size(); i++) {
    const BEAD& b = subunit_bead[i];
    printf("F %zu %La %La %La %La %La %La %La %La %La\n", i,
           b.tforce.x, b.tforce.y, b.tforce.z, b.sforce.x, b.sforce.y, b.sforce.z, b.bforce.x,
           b.bforce.y, b.bforce.z);
  }
  for (size_t i = 0; i < subunit_bead.size(); i++) {
    const BEAD& b = subunit_bead[i];
    size_t n = 0;
    while (n < b.itsN.size() && b.itsN[n] != -1) n++;
    printf("N %zu %zu", i, n);
    for (size_t k = 0; k < n; k++) printf(" %d", b.itsN[k]);
    printf("\n");
  }

  // Energy block, in the order of src/md.cpp:553-583.
  dress_up(subunit_edge, subunit_face);
  for (size_t i = 0; i < protein.size(); i++)
    for (size_t ii = 0; ii < protein[i].itsB.size(); ii++) {
      protein[i].itsB[ii]->be = 0;
      protein[i].itsB[ii]->ne = 0;
      protein[i].itsB[ii]->ce = 0;
    }
  for (size_t i = 0; i < protein.size(); i++) {
    for (size_t ii = 0; ii < protein[i].itsB.size(); ii++) {
      protein[i].itsB[ii]->update_stretching_energy(ks);
      protein[i].itsB[ii]->update_kinetic_energy();
    }
    for (size_t kk = 0; kk < protein[i].itsE.size(); kk++)
      if (protein[i].itsE[kk]->type != 0) protein[i].itsE[kk]->update_bending_energy(kb);
  }
  update_LJ_ES_energies_simplified(subunit_bead, ecut, lj_a, elj_att, lb, ni, qs, ecut_el, kappa);
  if (encapsulation) {
    for (size_t i = 0; i < big_beads.size(); i++) {
      big_beads[i].be = 0;
      big_beads[i].ne = 0;
      big_beads[i].ce = 0;
    }
    update_LJ_ES_energies_bigbeads(big_beads, subunit_bead, ecut, lb, ni, qs, ecut_el, kappa, shc);
    double big_ne = 0, big_ce = 0;
    for (size_t i = 0; i < big_beads.size(); i++) {
      big_ne += big_beads[i].ne;
      big_ce += big_beads[i].ce;
      printf("BB %zu %La %La %La\n", i, (long double)big_beads[i].pos.x, (long double)big_beads[i].pos.y,
             (long double)big_beads[i].pos.z);
    }
    printf("G %La %La\n", (long double)big_ne, (long double)big_ce);
  }
  for (size_t i = 0; i < subunit_bead.size(); i++) {
    const BEAD& b = subunit_bead[i];
    printf("E %zu %La %La %La %La %La\n", i, (long double)b.se, (long double)b.ke,
           (long double)b.be, (long double)b.ne, (long double)b.ce);
  }
  long double ke = particle_kinetic_energy(subunit_bead);
  printf("K %La\n", ke);
  return 0;
}
