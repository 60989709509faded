// Post-run analysis of the souffle_gb300 driver: the reference's analyze_output
// (src/analysis.cpp:16-297) and compute_MD_trust_factor_R (src/functions.cpp:119-258), with the
// per-frame work (pair correlation, oligomers, sub-oligomers) on the GPU through
// include/souffle_analysis.h.
//
// Files, formats and the order of everything written follow the reference:
//   outfiles/analysis.rdat  sample size, standard deviations of total and kinetic energy, R
//   outfiles/analysis.gr    one row of pcf bin counts per analysed frame
//   outfiles/analysis.so    one row of sub-oligomer bins per analysed frame
//   outfiles/analysis.ms    the mass spectrum averaged over the analysed frames
//   outfiles/info.gr        subunit count, bin size and count, box, density, bead type
// Values go through std::ostream with the reference's manipulators, so the stream quirks come
// out the same: a setw(15) after the last value of a row pads the first value of the next row.
//
// energy.out is read the way the reference reads it: 11 header tokens, then groups of 11 tokens,
// a group skipped when column 1, 2, 5, 7 or 8 is not a number (an istringstream extraction that
// must consume the whole token).  The MD writes 12 columns after row 0, so the groups drift
// through the file; this is the reference's behaviour and is kept.
#include "analysis_host.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "souffle_analysis.h"

using namespace std;

namespace souffle_host {
namespace {

bool lexical_double(const string& tok, double& v) {
  istringstream in(tok);
  in >> v;
  if (in.fail()) return false;
  char extra;
  return !(in >> extra);
}

// Welford mean and sample variance (src/RunningStat.h:9-47).
struct Welford {
  int n = 0;
  double m = 0, s = 0;
  void push(double x) {
    n++;
    if (n == 1) {
      m = x;
      s = 0.0;
    } else {
      const double m1 = m + (x - m) / n;
      s = s + (x - m) * (x - m1);
      m = m1;
    }
  }
  double stdev() const { return sqrt(n > 1 ? s / (n - 1) : 0.0); }
};

// compute_MD_trust_factor_R: sets the equilibrium step and `done`, writes analysis.rdat.
double trust_factor(const string& directory, int& hiteqm, bool& done) {
  ifstream in((directory + "/energy.out").c_str());
  if (!in) {
    cout << "ERR: FILE " << directory + "/energy.out" << " NOT OPENED. Check directory and/or filename." << endl;
    return 0;
  }
  string dummy, c[11];
  for (int k = 0; k < 11; k++) in >> dummy;
  vector<double> ext, ke, pe, time;
  while (in >> c[0] >> c[1] >> c[2] >> c[3] >> c[4] >> c[5] >> c[6] >> c[7] >> c[8] >> c[9] >> c[10]) {
    double v1, v2, v7, v8, v5;
    if (!lexical_double(c[0], v1) || !lexical_double(c[1], v2) || !lexical_double(c[6], v7) ||
        !lexical_double(c[7], v8) || !lexical_double(c[4], v5)) {
      cout << "Caught a restart header! This will artificially inflate R value." << endl;
      continue;
    }
    time.push_back(v1);
    ext.push_back(v7);
    ke.push_back(v2);
    pe.push_back(v8);
  }
  const int nsec = 10;
  const int ss = (int)floor(pe.size() / nsec);
  cout << "Each energy section has " << ss << " points." << endl;
  vector<bool> flat(nsec);
  for (int i = 0; i < nsec; i++) {
    double xs = 0, ys = 0, xys = 0, xxs = 0;
    Welford w;
    for (int j = 0; j < ss; j++) {
      const double y = pe[i * ss + j];
      xs += j;
      ys += y;
      xys += j * y;
      xxs += j * j;
      w.push(y);
    }
    const double xm = xs / double(ss), ym = ys / double(ss);
    const double slope = (xys - double(ss) * xm * ym) / (xxs - double(ss) * xm * ym);
    flat[i] = w.stdev() < 0.02 && slope < 1e-4 && slope > -1e-4;
  }
  flat[nsec - 1] = true;
  int nflat = 0, idx = 0;
  for (int i = nsec - 1; i > -1; i--) {
    if (!flat[i]) break;
    nflat++;
    idx = i * ss;
  }
  if (time.empty()) {
    // the reference indexes an empty vector here
    cout << "ERR: no energy rows in " << directory + "/energy.out" << endl;
    return 0;
  }
  hiteqm = (int)time[idx];
  cout << "There are " << nflat << " ending consecutive flat sections" << endl;
  done = true;
  if (nflat > 1) {
    cout << 100.0 * double(nflat) / double(nsec) << "% of simulation is in equilibrium. Analyzing..." << endl;
    cout << "Equilibrium starts at timestep " << hiteqm << "." << endl;
  } else if (nflat == 1) {
    cout << "Simulation has not reached equilibrium! Analyzing last 10% anyway..." << endl;
  }
  auto sd = [](const vector<double>& v) {
    double m = 0;
    for (double x : v) m += x;
    m = m / v.size();
    double s = 0;
    for (double x : v) s += (x - m) * (x - m);
    return sqrt(s / v.size());
  };
  const double ext_sd = sd(ext), ke_sd = sd(ke);
  const double R = ext_sd / ke_sd;
  ofstream out((directory + "/analysis.rdat").c_str());
  out << "Sample size " << ext.size() << endl;
  out << "Standard Deviation: total energy, kinetic energy | R" << endl;
  out << ext_sd << setw(15) << ke_sd << setw(15) << R << endl;
  cout << endl << endl << "R is: " << R << endl << endl;
  return R;
}

// Whitespace tokenizer over a file read in large blocks.
class Tokens {
 public:
  explicit Tokens(const string& path) : f_(fopen(path.c_str(), "rb")), buf_(1 << 22) {}
  ~Tokens() {
    if (f_) fclose(f_);
  }
  bool ok() const { return f_ != nullptr; }
  // Next token into tok; false at end of file.
  bool next(string& tok) {
    tok.clear();
    for (;;) {
      if (pos_ == len_ && !fill()) return !tok.empty();
      const char ch = buf_[pos_];
      if (ch == ' ' || ch == '\n' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f') {
        pos_++;
        if (!tok.empty()) return true;
        continue;
      }
      tok.push_back(ch);
      pos_++;
    }
  }

 private:
  bool fill() {
    len_ = f_ ? fread(buf_.data(), 1, buf_.size(), f_) : 0;
    pos_ = 0;
    return len_ > 0;
  }
  FILE* f_;
  vector<char> buf_;
  size_t pos_ = 0, len_ = 0;
};

}  // namespace

int analyze_output(const AnalysisCli& cli) {
  const string directory = "outfiles";
  const string coords = directory + "/ovito.lammpstrj";
  Tokens crds(coords);
  if (!crds.ok()) {
    cerr << "ERR: FILE " << coords << " NOT OPENED. Check directory and/or filename.";
    return 1;
  }
  cout << endl;
  cout << "Mass spectrum file will be saved to " << directory + "/analysis.ms" << endl;
  cout << "Pair-correlation file will be saved to " << directory + "/analysis.gr" << endl;
  cout << "R value will be saved to " << directory + "/analysis.rdat" << endl;
  cout << "Sub-oligomer structural information will be saved to " << directory + "/analysis.so" << endl;
  ofstream msdata((directory + "/analysis.ms").c_str());
  ofstream sodata((directory + "/analysis.so").c_str());
  ofstream grdata((directory + "/analysis.gr").c_str());
  ofstream rdata((directory + "/analysis.rdat").c_str());
  ofstream grinfo((directory + "/info.gr").c_str());

  souffle_analysis_options opt;
  souffle_analysis_default_options(&opt);
  opt.image = cli.image;
  const int gr_size = opt.pcf_bins, bead_type = opt.pcf_type;

  int hiteqm = 0;
  bool done = false;
  trust_factor(directory, hiteqm, done);
  int status = 0;
  if (done) {
    string tok;
    long a = 0;
    int np = 0, S = 0, num_type = 0;
    long N = 0;
    double box_size = 0, delta_g = 0, rho = 0, box = 0;
    souffle_analysis* h = nullptr;
    vector<double> pos;
    vector<int32_t> types;
    vector<int64_t> pcf(gr_size), olig, so;
    vector<double> ms_histogram;
    long ms_frames = 0;
    bool skipped = false;
    while (crds.next(tok)) {  // "ITEM:"
      string t[6];
      crds.next(t[0]);
      crds.next(t[1]);
      const long timestep = atol(t[1].c_str());
      for (int k = 0; k < 4; k++) crds.next(t[k]);
      crds.next(tok);
      const long nb = atol(tok.c_str());
      for (int k = 0; k < 4; k++) crds.next(t[0]);
      crds.next(tok);
      box_size = strtod(tok.c_str(), nullptr);
      for (int k = 0; k < 13; k++) crds.next(t[0]);
      if (a == 0) {
        N = nb;
        if (cli.beads_per_subunit > 0) {
          np = cli.beads_per_subunit;
        } else {
          if (N % 41 == 0) np = 41;
          if (N % 43 == 0) np = 43;
          if (N % 78 == 0) np = 78;
        }
        if (np == 0 || N % np != 0) {
          cerr << "analysis: " << N << " beads are not a whole number of subunits of "
               << (np ? to_string(np) : string("41, 43 or 78")) << " beads; the reference stops here with a "
               << "division by zero (src/analysis.cpp:81-85).  Pass -Y <beads per subunit> to analyse; "
               << "skipped." << endl;
          skipped = true;
          break;
        }
        S = (int)(N / np);
        box = box_size * 2;
        delta_g = box / (2 * gr_size);
        pos.resize(3 * N);
        types.resize(N);
        olig.resize(S);
        so.resize(2 * S);
        ms_histogram.assign(S, 0.0);
        const souffle_status s = souffle_analysis_create(N, np, box, &opt, 0, &h);
        if (s != SOUFFLE_OK) {
          cerr << "analysis: souffle_analysis_create failed (" << (int)s << "): " << souffle_gpu_last_error() << endl;
          status = 1;
          break;
        }
      } else if (nb != N) {
        cerr << "analysis: frame " << a << " has " << nb << " beads, frame 0 had " << N << endl;
        status = 1;
        break;
      }
      bool short_file = false;
      for (long b = 0; b < N; b++) {
        string idx_tok, dummy;
        if (!crds.next(idx_tok)) {
          short_file = true;
          break;
        }
        crds.next(tok);
        types[b] = (int32_t)atol(tok.c_str());
        for (int c = 0; c < 3; c++) {
          crds.next(tok);
          pos[3 * b + c] = strtod(tok.c_str(), nullptr);
        }
        crds.next(dummy);
        crds.next(dummy);
        if (a == 0 && types[b] == bead_type) num_type++;
      }
      if (short_file) {
        cerr << "analysis: " << coords << " ends inside frame " << a << endl;
        status = 1;
        break;
      }
      if (a == 0) rho = num_type / (box * box * box);
      if (timestep >= hiteqm) {
        const souffle_status s =
            souffle_analysis_frames(h, 1, pos.data(), types.data(), pcf.data(), olig.data(), so.data(), nullptr);
        if (s != SOUFFLE_OK) {
          cerr << "analysis: souffle_analysis_frames failed (" << (int)s << "): " << souffle_gpu_last_error() << endl;
          status = 1;
          break;
        }
        for (int j = 0; j < gr_size; j++) grdata << (int)pcf[j] << setw(15);
        grdata << endl;
        for (int j = 0; j < S; j++) ms_histogram[j] += (int)olig[j] * (j + 1);
        ms_frames++;
        for (int j = 0; j < 2 * S; j++) sodata << (int)so[j] << setw(15);
        sodata << endl;
      }
      a++;
    }
    if (h) souffle_analysis_destroy(h);
    if (status == 0 && !skipped) {
      grinfo << "Number of Subunits: " << S << endl;
      grinfo << "PCF bin size: " << delta_g << endl;
      grinfo << "PCF bin number: " << gr_size << endl;
      grinfo << "Box size: " << box_size * 2 << " " << box_size * 2 << " " << box_size * 2 << endl;
      grinfo << "Number density: " << rho << endl;
      grinfo << "Bead Type: " << bead_type << endl;
      for (int j = 0; j < S; j++) ms_histogram[j] = ms_histogram[j] / (unsigned long)ms_frames;
      for (int j = 0; j < S; j++) msdata << ms_histogram[j] << setw(15);
      msdata << endl;
    }
  }
  if (!done) {
    grinfo.close();
    remove((directory + "/info.gr").c_str());
  }
  return status;
}

}  // namespace souffle_host
