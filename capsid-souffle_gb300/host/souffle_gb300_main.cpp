// souffle_gb300: the SOUFFLE molecular-dynamics driver on the GB300 path.
//
// Same command line (letters and defaults of src/md.cpp:53-90), same inputs (infiles/<-f>,
// auto-restart from the newest outfiles/restart_*.out, src/initialize.cpp:166-214) and the same
// outfiles in the working directory:
//   outfiles/energy.out          header src/initialize.cpp:12-19, rows src/md.cpp:339-353,616-623
//   outfiles/ovito.lammpstrj     LAMMPS text dump, src/md.cpp:647-678
//   outfiles/restart_<a>.out     src/md.cpp:526-546 (12 significant digits)
//   outfiles/model.parameters.out  src/md.cpp:111-180,233-235
// The MD loop (src/md.cpp:387-688, molecular-dynamics branch) runs on the GPU through the C ABI
// in include/souffle_gpu.h; the host only steps between output points.  -D b runs the Brownian
// branch (src/md.cpp:400-470) on the same path; as in src/md.cpp:109-116 any -D other than 'm'
// selects Brownian dynamics.  Encapsulation (-p true) places -m static big beads (-a radius,
// -G charge, -H hard-core distance) as generate_big_beads does (src/initialize.cpp:566-680: the
// newest outfiles/rb_*.out on restart, else the C library's rand() after srand(0)) and writes
//   outfiles/capenergy.out       src/md.cpp:347-351,625-629 (created empty without -p)
//   outfiles/rb_<a>.out          src/md.cpp:537-545, beside each restart file
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dirent.h>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "analysis_host.h"
#include "text_out.h"
#include "souffle_analysis.h"
#include "souffle_gpu.h"

using namespace std;

namespace {

struct Options {
  char D = 'm';
  string f = "41part_c";
  double C = 200, c = 500, S = 64, s = 50, b = 20, T = 2500, t = 0.004, r = 1, d = 100, q = 5, Q = 10;
  double K = 298, e = 12;
  bool R = true, X = false, V = true;
  double E = 2;
  int B = 20;
  double L = 7.5;
  int M = 1000, W = 1000, w = 1000000, N = 4;
  bool p = false;
  double a = 3.0, G = -78.0;
  int m = 1;
  double H = 3.5;
  // not in the reference: what runs (r = MD then analysis, as src/main.cpp:15-16; o = analysis
  // only; n = MD only), beads per subunit for the analysis (0 = the reference's 41/43/78 rule),
  // and the analysis image rule (r = as the reference's analysis computes it, m = minimum image)
  char A = 'r';
  int Y = 0;
  char I = 'r';
};

bool parse_bool(const string& v) {
  if (v == "1" || v == "true" || v == "yes" || v == "on") return true;
  if (v == "0" || v == "false" || v == "no" || v == "off") return false;
  fprintf(stderr, "bad boolean value: %s\n", v.c_str());
  exit(2);
}

void usage() {
  printf("Usage:\nsouffle_gb300 <options>  (letters as the reference driver)\n"
         "  -D b|m  -f infile  -C uM  -c mM  -S subunits  -s ks  -b kb  -T steps  -t dt\n"
         "  -q chain  -Q mass  -K kelvin  -e ecut_c  -R bool  -E eps  -B rebuild  -L skin\n"
         "  -M movie  -W energy  -w restart  (-r -d -X -V -N -p -a -G -m -H accepted)\n"
         "  -A r|o|n  MD then analysis (default) | analysis only | MD only\n"
         "  -Y np     beads per subunit for the analysis (default: 41, 43 or 78 from the bead count)\n"
         "  -I r|m    analysis image rule: as the reference's analysis (default) | minimum image\n");
}

// Short options "-X value" or "-Xvalue" (src/md.cpp:53-90).
Options parse(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; i++) {
    string tok = argv[i];
    if (tok == "-h" || tok == "--help") {
      usage();
      exit(0);
    }
    if (tok.size() < 2 || tok[0] != '-') {
      fprintf(stderr, "unexpected argument %s\n", tok.c_str());
      exit(2);
    }
    char k = tok[1];
    string v;
    if (tok.size() > 2)
      v = tok.substr(2);
    else if (i + 1 < argc)
      v = argv[++i];
    else {
      fprintf(stderr, "option %s needs a value\n", tok.c_str());
      exit(2);
    }
    switch (k) {
      case 'D': o.D = v[0]; break;
      case 'f': o.f = v; break;
      case 'C': o.C = atof(v.c_str()); break;
      case 'c': o.c = atof(v.c_str()); break;
      case 'S': o.S = atof(v.c_str()); break;
      case 's': o.s = atof(v.c_str()); break;
      case 'b': o.b = atof(v.c_str()); break;
      case 'T': o.T = atof(v.c_str()); break;
      case 't': o.t = atof(v.c_str()); break;
      case 'r': o.r = atof(v.c_str()); break;
      case 'd': o.d = atof(v.c_str()); break;
      case 'q': o.q = atof(v.c_str()); break;
      case 'Q': o.Q = atof(v.c_str()); break;
      case 'K': o.K = atof(v.c_str()); break;
      case 'e': o.e = atof(v.c_str()); break;
      case 'R': o.R = parse_bool(v); break;
      case 'X': o.X = parse_bool(v); break;
      case 'V': o.V = parse_bool(v); break;
      case 'E': o.E = atof(v.c_str()); break;
      case 'B': o.B = atoi(v.c_str()); break;
      case 'L': o.L = atof(v.c_str()); break;
      case 'M': o.M = atoi(v.c_str()); break;
      case 'W': o.W = atoi(v.c_str()); break;
      case 'w': o.w = atoi(v.c_str()); break;
      case 'N': o.N = atoi(v.c_str()); break;
      case 'p': o.p = parse_bool(v); break;
      case 'a': o.a = atof(v.c_str()); break;
      case 'G': o.G = atof(v.c_str()); break;
      case 'm': o.m = atoi(v.c_str()); break;
      case 'H': o.H = atof(v.c_str()); break;
      case 'A': o.A = v[0]; break;
      case 'Y': o.Y = atoi(v.c_str()); break;
      case 'I': o.I = v[0]; break;
      default:
        fprintf(stderr, "unrecognised option -%c\n", k);
        exit(2);
    }
  }
  return o;
}

struct Infile {
  double bondlength = 0, mass_si = 0, sigma_si = 0;
  int np = 0, ne = 0, nf = 0, na = 0;
  vector<double> x, y, z, q, sigma, mass, len0;
  vector<int> type, eb, et, fb, lj;
};

// Token-counted infile layout of src/initialize.cpp:47-128.
bool read_infile(const string& path, Infile& in) {
  ifstream f(path.c_str());
  if (!f) return false;
  string d;
  f >> d >> d >> in.bondlength >> d >> d >> in.mass_si >> d >> d >> in.sigma_si;
  f >> d >> d >> d >> d >> d >> in.np;
  for (int k = 0; k < 8; k++) f >> d;
  for (int i = 0; i < in.np; i++) {
    double name, x, y, z, type, ch, rad, m;
    f >> name >> x >> y >> z >> type >> ch >> rad >> m;
    in.x.push_back(x);
    in.y.push_back(y);
    in.z.push_back(z);
    in.type.push_back((int)type);
    in.q.push_back(ch);
    in.sigma.push_back(rad);
    in.mass.push_back(m);
  }
  f >> d >> d >> d >> d >> d >> in.ne;
  for (int k = 0; k < 5; k++) f >> d;
  for (int i = 0; i < in.ne; i++) {
    double name, e1, e2, type, len;
    f >> name >> e1 >> e2 >> type >> len;
    in.eb.push_back((int)e1);
    in.eb.push_back((int)e2);
    in.et.push_back((int)type);
    in.len0.push_back(len);
  }
  f >> d >> d >> d >> d >> d >> in.nf;
  for (int k = 0; k < 6; k++) f >> d;
  for (int i = 0; i < in.nf; i++) {
    double name, t1, t2, t3, type, normal;
    f >> name >> t1 >> t2 >> t3 >> type >> normal;
    in.fb.push_back((int)t1);
    in.fb.push_back((int)t2);
    in.fb.push_back((int)t3);
  }
  f >> d >> d >> d >> d >> d >> d >> in.na;
  for (int k = 0; k < 5; k++) f >> d;
  for (int i = 0; i < in.na; i++) {
    double name, t1, t2, eps, sig;
    f >> name >> t1 >> t2 >> eps >> sig;
    in.lj.push_back((int)t1);
    in.lj.push_back((int)t2);
  }
  return !f.fail();
}

// Newest restart file: names containing "restart", shortest-then-lexicographic order
// (src/functions.cpp:262-311, src/initialize.cpp:166-191).
string newest_file(const string& dir, const char* key) {
  vector<string> names;
  if (DIR* dp = opendir(dir.c_str())) {
    while (dirent* e = readdir(dp)) {
      string n = e->d_name;
      if (n.find(key) != string::npos) names.push_back(n);
    }
    closedir(dp);
  }
  if (names.empty()) return "";
  sort(names.begin(), names.end(), [](const string& a, const string& b) {
    if (a.size() != b.size()) return a.size() < b.size();
    return a < b;
  });
  return names.back();
}

void check(souffle_status s, const char* what) {
  if (s != SOUFFLE_OK) {
    fprintf(stderr, "souffle_gb300: %s failed (%d): %s\n", what, (int)s, souffle_gpu_last_error());
    exit(1);
  }
}

void progress(double frac) {  // the bar of src/functions.cpp:24-30
  static const char* bar = "||||||||||||||||||||||||||||||||||||||||||||||||||||||||||||";
  int val = (int)(frac * 100), lpad = (int)(frac * 60), rpad = 60 - lpad;
  printf("\r%3d%% |%.*s%*s|", val, lpad, bar, rpad, "");
  fflush(stdout);
}

int run_simulation(const Options& o);

}  // namespace

int main(int argc, char** argv) {
  Options o = parse(argc, argv);
  if (o.A != 'r' && o.A != 'o' && o.A != 'n') {
    fprintf(stderr, "souffle_gb300: -A takes r, o or n\n");
    return 2;
  }
  if (o.A != 'o') {
    const int rc = run_simulation(o);
    if (rc != 0 || o.A == 'n') return rc;
  }
  souffle_host::AnalysisCli cli;
  cli.beads_per_subunit = o.Y;
  cli.image = o.I == 'm' ? SOUFFLE_IMAGE_MINIMUM : SOUFFLE_IMAGE_REFERENCE;
  return souffle_host::analyze_output(cli);
}

namespace {

int run_simulation(const Options& o) {
  ofstream traj("outfiles/energy.out", ios_base::app);
  ofstream encapdata("outfiles/capenergy.out", ios::out);
  ofstream ofile("outfiles/ovito.lammpstrj", ios_base::app);
  ofstream sysdata("outfiles/model.parameters.out", ios::out);
  if (!traj || !ofile || !sysdata) {
    cerr << "ERR: outfiles/ directory missing or not writable" << endl;
    return 1;
  }
  traj << "time" << setw(15) << "kinetic" << setw(15) << "stretching" << setw(15) << "bending" << setw(15)
       << "LJ" << setw(15) << "electrostatics" << setw(15) << "total" << setw(15) << "potential" << setw(15)
       << "temperature" << setw(20) << "thermo_potential" << setw(15) << "thermo_kinetic" << setw(15)
       << "system_velocity_magnitude" << endl;
  const bool brownian = o.D != 'm';  // src/md.cpp:31,109-116
  if (o.D == 'b') sysdata << "Running brownian dynamics." << endl;
  else if (o.D == 'm') sysdata << "Running molecular dynamics with Nose Hoover thermostat." << endl;

  Infile in;
  if (!read_infile("infiles/" + o.f, in)) {
    cerr << "ERR: FILE " << o.f << " NOT OPENED. Check directory and/or filename.";
    return 1;
  }
  const int S = (int)o.S, np = in.np;
  const long N = (long)S * np;
  const double Avagadro = 6.022e23, Boltzmann = 1.3806e-23, Pi = 3.14159;

  // state: restart file or cubic lattice (src/initialize.cpp:199-231)
  vector<double> pos(3 * N), vel(3 * N, 0.0);
  double box_x = pow((o.S * 1000 / (o.C * pow(in.sigma_si, 3) * Avagadro)), 1.0 / 3.0);
  int loopStart = 0;
  string rname = o.R ? newest_file("outfiles/", "restart") : "";
  bool restart = !rname.empty();
  if (restart) {
    cout << "Restarting from: " << rname << endl;
    ifstream rf(("outfiles/" + rname).c_str());
    if (!rf) {
      cerr << "ERR: RESTART FILE outfiles/restart.out NOT OPENED. Check directory and/or filename.";
      return 1;
    }
    string d;
    rf >> d >> d >> d >> d >> loopStart;
    for (long i = 0; i < N; i++) {
      rf >> d >> vel[3 * i] >> vel[3 * i + 1] >> vel[3 * i + 2] >> pos[3 * i] >> pos[3 * i + 1] >> pos[3 * i + 2];
      if (!rf) {
        cerr << "ERR: restart file " << rname << " has fewer than " << N << " beads" << endl;
        return 1;
      }
    }
  } else {
    cout << "No restart files found! Starting simulation from scratch." << endl;
    const unsigned nf = (unsigned)ceil(pow(double(S), 1.0 / 3.0));
    long k0 = 0;
    for (unsigned i = 0; i < nf; i++)
      for (unsigned j = 0; j < nf; j++)
        for (unsigned k = 0; k < nf; k++, k0++) {
          if (k0 >= S) continue;
          for (int l = 0; l < np; l++) {
            long g = k0 * np + l;
            pos[3 * g] = (double)i * box_x * (1 / (double)nf) + in.x[l];
            pos[3 * g + 1] = (double)j * box_x * (1 / (double)nf) + in.y[l];
            pos[3 * g + 2] = (double)k * box_x * (1 / (double)nf) + in.z[l];
          }
        }
  }
  // centre bead of subunit 0 (src/initialize.cpp:266-288)
  int center = 0;
  {
    double c[3] = {0, 0, 0};
    for (int l = 0; l < np; l++)
      for (int d = 0; d < 3; d++) c[d] += pos[3 * l + d];
    for (int d = 0; d < 3; d++) c[d] /= np;
    double best = 1000;
    for (int l = 0; l < np; l++) {
      double r2 = 0;
      for (int d = 0; d < 3; d++) {
        double r = pos[3 * l + d] - c[d];
        if (r > box_x / 2) r -= box_x;
        else if (r < -box_x / 2) r += box_x;
        r2 += r * r;
      }
      if (r2 < best) {
        best = r2;
        center = l;
      }
    }
  }

  // units (src/md.cpp:135-173)
  const double SIenergy = o.K * Boltzmann;
  const double SItime = sqrt(in.sigma_si * in.sigma_si * in.mass_si / SIenergy);
  const double totaltime = o.T * o.t;
  const double Tred = o.K / double(298);
  const double UnitEnergy = SIenergy * SItime * SItime / (in.mass_si * in.sigma_si * (1e-9));
  sysdata << "Simulation will run for " << totaltime * SItime / (1e-9) << " nanoseconds with a "
          << o.t * SItime / (1e-12) << " picosecond timestep." << endl;
  sysdata << "Capsomere concentration: " << o.C << " micromolar" << endl;
  sysdata << "Salt concentration: " << o.c << " millimolar" << endl;
  sysdata << "Stretching constant: " << o.s << " KbT" << "( " << (o.s * in.mass_si / (SItime * SItime)) << " N/m)" << endl;
  sysdata << "Bending constant: " << o.b << " KbT" << "( "
          << (o.b * in.mass_si * in.sigma_si * in.sigma_si / (SItime * SItime)) << " J)" << endl;
  sysdata << "Bondlength between beads is " << in.bondlength << " LJ reduced units, which is "
          << in.bondlength * in.sigma_si / (1e-9) << " nanometers." << endl;
  sysdata << "Mass of a bead is " << in.mass_si << " kg." << endl;
  sysdata << "Diameter of a bead is " << in.sigma_si / (1e-9) << " nanometers." << endl;
  sysdata << "Total number of subunits is " << o.S << endl;
  sysdata << "Temperature is " << o.K << " K" << " Which is " << Tred << " in reduced units" << endl;
  sysdata << "Attractive LJ paramerter is " << o.E << " Which is "
          << o.E * (SIenergy * Avagadro / (1000 * UnitEnergy)) << " kJ/mol." << endl;
  const double ecut = 2.5 * (in.sigma_si / 1e-9);
  const double lb = (0.701e-9) / in.sigma_si;
  const double ni = o.c * Avagadro * in.sigma_si * in.sigma_si * in.sigma_si;
  const double kappa = sqrt(8 * Pi * ni * lb * 1 * 1);
  const double screen = 1 / kappa;
  const double ecut_el = screen * o.e;
  const double NListCutoff = (ecut_el > ecut) ? ecut_el + o.L : ecut + o.L;
  sysdata << "Box length is " << box_x * in.sigma_si / (1e-9) << " nanometers." << endl;
  sysdata << "Screening length is " << screen << " nanometers." << endl;
  sysdata << "electrostatic cutoff is " << ecut_el * in.sigma_si / (1e-9) << " nanometers." << endl;
  sysdata << "Neighborlist cutoff is " << NListCutoff * in.sigma_si / (1e-9) << " nanometers." << endl;
  unsigned cap = (unsigned)ceil((NListCutoff + 0.5) * (NListCutoff + 0.5) * (NListCutoff + 0.5));
  if (cap > (unsigned)N) cap = (unsigned)N;
  sysdata << "Neighborlist has a maximum of " << cap << " neighbors per bead." << endl;

  if (!restart) {
    // rigid per-subunit velocities uniform in [-0.5, 0.5)^3, zero net momentum, scaled to T
    // (the structure of src/initialize.cpp:471-564, drawn from a fixed-seed std::mt19937)
    std::mt19937 eng(5489u);
    std::uniform_real_distribution<double> u(-0.5, 0.5);
    for (int i = 0; i < S; i++) {
      double vx = u(eng), vy = u(eng), vz = u(eng);
      for (int l = 0; l < np; l++) {
        long g = (long)i * np + l;
        vel[3 * g] = vx;
        vel[3 * g + 1] = vy;
        vel[3 * g + 2] = vz;
      }
    }
    double avg[3] = {0, 0, 0};
    for (long g = 0; g < N; g++)
      for (int d = 0; d < 3; d++) avg[d] += vel[3 * g + d];
    double ke = 0;
    for (long g = 0; g < N; g++) {
      double v2 = 0;
      for (int d = 0; d < 3; d++) {
        vel[3 * g + d] -= avg[d] / N;
        v2 += vel[3 * g + d] * vel[3 * g + d];
      }
      ke += 0.5 * in.mass[g % np] * v2;
    }
    const double sf = sqrt(Tred / (ke / (1.5 * N)));
    for (auto& v : vel) v *= sf;
  }

  // encapsulation big beads (generate_big_beads, src/initialize.cpp:566-680, called with
  // sigma = 2 a, mass 100, type 3, charge G and 1000000 attempts at src/md.cpp:185)
  const double big_sigma = 2 * o.a, big_mass = 100.0;
  vector<double> big_pos, big_vel;
  if (o.p) {
    const int nb = o.m;
    if (restart) {
      const string rb = newest_file("outfiles/", "rb");
      ifstream rf(("outfiles/" + rb).c_str());
      for (int i = 0; i < nb; i++) {
        double v[6];
        for (double& x : v) rf >> x;
        if (!rf || rb.empty()) {
          cerr << "ERR: big-bead restart file outfiles/" << rb << " has fewer than " << nb << " beads" << endl;
          return 1;
        }
        cout << v[0] << ", " << v[1] << ", " << v[2] << endl;
        big_vel.insert(big_vel.end(), v, v + 3);
        big_pos.insert(big_pos.end(), v + 3, v + 6);
      }
    } else {
      srand(0);
      const double R_squared = big_sigma * big_sigma;
      for (int i = 0; i < nb; i++) {
        bool placed = false;
        unsigned attempts = 0;
        while (!placed && attempts < 1000000u) {
          const double x = (static_cast<double>(rand()) / RAND_MAX - 0.5) * box_x;
          const double y = (static_cast<double>(rand()) / RAND_MAX - 0.5) * box_x;
          const double z = (static_cast<double>(rand()) / RAND_MAX - 0.5) * box_x;
          auto d2 = [&](double px, double py, double pz) {
            double dx = x - px, dy = y - py, dz = z - pz;
            dx -= box_x * floor(dx / box_x + 0.5);
            dy -= box_x * floor(dy / box_x + 0.5);
            dz -= box_x * floor(dz / box_x + 0.5);
            return dx * dx + dy * dy + dz * dz;
          };
          bool collision = false;
          for (long g = 0; g < N && !collision; g++) {
            const double min_dist = in.sigma[g % np] / 2 + big_sigma / 2;
            if (d2(pos[3 * g], pos[3 * g + 1], pos[3 * g + 2]) < min_dist * min_dist) collision = true;
          }
          for (size_t b = 0; b < big_pos.size() / 3 && !collision; b++)
            if (d2(big_pos[3 * b], big_pos[3 * b + 1], big_pos[3 * b + 2]) < R_squared) collision = true;
          if (!collision) {
            big_pos.insert(big_pos.end(), {x, y, z});
            big_vel.insert(big_vel.end(), {0.0, 0.0, 0.0});
            placed = true;
          }
          attempts++;
        }
        if (attempts >= 1000000u) {
          cerr << "Error: Failed to place big bead " << i + 1 << " after " << 1000000 << " attempts" << endl;
          exit(1);
        }
      }
    }
  }
  const int n_big = (int)(big_pos.size() / 3);
  // BEAD::update_kinetic_energy (src/bead.h:129-131) of the static big beads
  double big_ke = 0;
  for (int i = 0; i < n_big; i++) {
    const double v = sqrt(big_vel[3 * i] * big_vel[3 * i] + big_vel[3 * i + 1] * big_vel[3 * i + 1] +
                          big_vel[3 * i + 2] * big_vel[3 * i + 2]);
    big_ke += 0.5 * big_mass * v * v;
  }

  souffle_template t{np, in.ne, in.nf, in.na, in.type.data(), in.q.data(), in.sigma.data(), in.mass.data(),
                     in.eb.data(), in.et.data(), in.len0.data(), in.fb.data(), in.lj.empty() ? nullptr : in.lj.data(),
                     nullptr /* no rest dihedral: the reference's bending */};
  souffle_params p{};
  p.n_subunits = S;
  p.box = box_x;
  p.ks = o.s;
  p.kb = o.b;
  p.elj_att = o.E;
  p.lb = lb;
  p.kappa = kappa;
  p.ecut = ecut;
  p.ecut_el = ecut_el;
  p.nlist_cutoff = NListCutoff;
  p.nlist_capacity = (int)cap;
  p.center_local = center;
  p.dt = o.t;
  p.chain_length = (int)o.q;
  p.nhc_mass = o.Q;
  p.temperature = Tred;
  p.build_freq = o.B;
  p.brownian = brownian ? 1 : 0;
  p.damp = o.d;
  souffle_gpu_system* h = nullptr;
  check(souffle_gpu_create(&t, &p, 1, nullptr, &h), "souffle_gpu_create");
  // the reference wraps lattice positions only when they move; the fixed-point state wraps now
  check(souffle_gpu_set_state(h, pos.data(), vel.data()), "souffle_gpu_set_state");
  if (n_big > 0)
    check(souffle_gpu_set_big_beads(h, 0, n_big, big_pos.data(), big_sigma, o.G, o.H), "souffle_gpu_set_big_beads");
  check(souffle_gpu_md_begin(h), "souffle_gpu_md_begin");

  vector<double> be(N);
  auto energy_row = [&](long a, bool with_vcom) {
    souffle_energies e;
    check(souffle_gpu_energies(h, 0, &e, nullptr, be.data(), nullptr, nullptr, nullptr), "souffle_gpu_energies");
    const double tot = e.stretching + e.kinetic + e.lj + e.bending + e.electrostatic + e.thermo_pe + e.thermo_ke;
    traj << a << setw(15) << e.kinetic / N << setw(15) << e.stretching / N << setw(15) << e.bending / N
         << setw(15) << e.lj / N << setw(15) << e.electrostatic / N << setw(15) << tot / N << setw(15)
         << (e.bending + e.stretching + e.lj + e.electrostatic) / N << setw(15) << e.kinetic * 2 / (3 * N)
         << setw(15) << e.thermo_pe / N << setw(15) << e.thermo_ke / N;
    if (with_vcom) traj << setw(15) << e.vcom_magnitude;
    traj << endl;
    if (n_big > 0)  // src/md.cpp:347-351,625-629
      encapdata << a << setw(15) << big_ke / n_big << setw(15) << e.bigbead_lj / n_big << setw(15)
                << e.bigbead_electrostatic / n_big << setw(15)
                << (big_ke + e.bigbead_lj + e.bigbead_electrostatic) / n_big << setw(15)
                << big_ke * 2 / (3 * n_big) << endl;
  };
  energy_row(0, false);  // row 0 before the loop (src/md.cpp:339-346)

  ofstream rs;  // one stream object for every restart file, as src/md.cpp:104
  // Output pipeline: the state of an output step is read back asynchronously into one of two
  // page-locked buffers while the next window of steps is already queued behind it, and its
  // restart and movie files are written while the GPU runs that window.  Energy rows are computed
  // at their step (a blocking call) after the previous step's files are written; the movie's
  // per-bead bending energies are those of the last energy row, as in the reference.
  double* snap_pos[2] = {nullptr, nullptr};
  double* snap_vel[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; k++) {
    snap_pos[k] = static_cast<double*>(souffle_gpu_host_alloc((int64_t)sizeof(double) * 3 * N));
    snap_vel[k] = static_cast<double*>(souffle_gpu_host_alloc((int64_t)sizeof(double) * 3 * N));
    if (!snap_pos[k] || !snap_vel[k]) {
      cerr << "souffle_gb300: page-locked host buffers for the output could not be allocated" << endl;
      exit(1);
    }
  }
  struct Pending {
    bool active = false;
    long a = 0;
    int slot = 0;
  } pending;
  auto write_outputs = [&](long at, const double* P, const double* V) {
    if (at % o.w == 0) {
      rs.open(("outfiles/restart_" + to_string(at) + ".out").c_str(), ios::out);
      rs << "Velocities & Positions for " << at << endl;
      // the first velocity of a line takes the precision the previous line left (12; the
      // stream's earlier precision on the first line of the first file), as the reference's
      // reused stream does
      // (and each line leaves a width of 25 pending, which the next line's index takes)
      write_lines(rs, N, 12, 25, [&](std::ostream& os, long i) {
        os << i << "  " << V[3 * i] << setw(25) << setprecision(12) << V[3 * i + 1] << setw(25)
           << setprecision(12) << V[3 * i + 2] << setw(25) << setprecision(12) << P[3 * i] << setw(25)
           << setprecision(12) << P[3 * i + 1] << setw(25) << setprecision(12) << P[3 * i + 2] << setw(25)
           << setprecision(12);
        os.put('\n');
      });
      rs.close();
      if (o.p) {
        rs.open(("outfiles/rb_" + to_string(at) + ".out").c_str(), ios::out);
        for (int i = 0; i < n_big; i++)
          rs << big_vel[3 * i] << setw(25) << setprecision(12) << big_vel[3 * i + 1] << setw(25) << setprecision(12)
             << big_vel[3 * i + 2] << setw(25) << setprecision(12) << big_pos[3 * i] << setw(25) << setprecision(12)
             << big_pos[3 * i + 1] << setw(25) << setprecision(12) << big_pos[3 * i + 2] << setw(25)
             << setprecision(12) << endl;
        rs.close();
      }
    }
    if (at % o.M == 0) {
      ofile << "ITEM: TIMESTEP" << endl << at << endl << "ITEM: NUMBER OF ATOMS" << endl << N + n_big << endl
            << "ITEM: BOX BOUNDS" << endl << -box_x / 2 << setw(15) << box_x / 2 << endl << -box_x / 2
            << setw(15) << box_x / 2 << endl << -box_x / 2 << setw(15) << box_x / 2 << endl
            << "ITEM: ATOMS index type x y z b charge" << endl;
      write_lines(ofile, N, ofile.precision(), 0, [&](std::ostream& os, long g) {
        os << g + 1 << setw(15) << in.type[g % np] << setw(15) << P[3 * g] << setw(15) << P[3 * g + 1]
           << setw(15) << P[3 * g + 2] << setw(15) << be[g] << setw(15) << in.q[g % np];
        os.put('\n');
      });
      for (int bb = 0; bb < n_big; bb++)  // type 3, no bending energy (src/md.cpp:670-675)
        ofile << N + bb + 1 << setw(15) << 3 << setw(15) << big_pos[3 * bb] << setw(15) << big_pos[3 * bb + 1]
              << setw(15) << big_pos[3 * bb + 2] << setw(15) << 0 << setw(15) << o.G << endl;
    }
  };
  auto flush_pending = [&]() {
    if (!pending.active) return;
    check(souffle_gpu_snapshot_wait(h, pending.slot), "souffle_gpu_snapshot_wait");
    write_outputs(pending.a, snap_pos[pending.slot], snap_vel[pending.slot]);
    pending.active = false;
  };
  const double loop_end = (totaltime / o.t) + 1;  // src/md.cpp:387
  long a = loopStart;
  double pre = -1;
  int slot = 0;
  while (a < loop_end) {
    // advance to the next step that writes anything (inclusive)
    long next = a;
    while (next + 1 < loop_end && !(next % o.w == 0 || next % o.W == 0 || next % o.M == 0)) next++;
    check(souffle_gpu_md_enqueue(h, a, (int)(next - a + 1)), "souffle_gpu_md_enqueue");
    a = next;
    const bool state_out = a % o.w == 0 || a % o.M == 0;
    if (state_out) check(souffle_gpu_snapshot_enqueue(h, slot, snap_pos[slot], snap_vel[slot]), "souffle_gpu_snapshot_enqueue");
    flush_pending();  // the previous output step's files, while this window runs
    if (a % o.W == 0) energy_row(a, true);
    if (state_out) {
      pending.active = true;
      pending.a = a;
      pending.slot = slot;
      slot ^= 1;
    }
    double pct = roundf(a / (totaltime / o.t) * 100 * 10) / 10;
    if (pct != pre) {
      progress(pct / 100);
      pre = pct;
    }
    a++;
  }
  flush_pending();
  check(souffle_gpu_synchronize(h), "souffle_gpu_synchronize");
  for (int k = 0; k < 2; k++) {
    souffle_gpu_host_free(snap_pos[k]);
    souffle_gpu_host_free(snap_vel[k]);
  }
  printf("\n");
  souffle_gpu_destroy(h);
  return 0;
}

}  // namespace
