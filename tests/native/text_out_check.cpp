// The driver's parallel text writer (capsid-souffle_gb300/host/text_out.h) against one sequential
// iostream pass, for the restart and movie line formats: byte equality, with the stream state
// (precision, pending field width) carried across files and frames as the driver's streams do.
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <vector>

#include "text_out.h"

using namespace std;

int main(int argc, char** argv) {
  const long N = argc > 1 ? atol(argv[1]) : 84000;
  mt19937_64 rng(5);
  uniform_real_distribution<double> U(-80, 80);
  vector<double> P(3 * N), V(3 * N), be(N);
  for (auto& x : P) x = U(rng);
  for (auto& x : V) x = U(rng) / 37.0;
  for (auto& x : be) x = U(rng) * 1e-3;
  vector<int> type(42, 1);
  vector<double> q(42, 0.5);
  ostringstream A, B;  // two restart files through one stream object
  for (int f = 0; f < 2; f++) {
    A << "Velocities & Positions for " << f << endl;
    for (long i = 0; i < N; i++)
      A << i << "  " << V[3 * i] << setw(25) << setprecision(12) << V[3 * i + 1] << setw(25) << setprecision(12)
        << V[3 * i + 2] << setw(25) << setprecision(12) << P[3 * i] << setw(25) << setprecision(12) << P[3 * i + 1]
        << setw(25) << setprecision(12) << P[3 * i + 2] << setw(25) << setprecision(12) << endl;
    B << "Velocities & Positions for " << f << endl;
    write_lines(B, N, 12, 25, [&](std::ostream& os, long i) {
      os << i << "  " << V[3 * i] << setw(25) << setprecision(12) << V[3 * i + 1] << setw(25) << setprecision(12)
         << V[3 * i + 2] << setw(25) << setprecision(12) << P[3 * i] << setw(25) << setprecision(12) << P[3 * i + 1]
         << setw(25) << setprecision(12) << P[3 * i + 2] << setw(25) << setprecision(12);
      os.put('\n');
    });
  }
  ostringstream C, D;  // two movie frames
  for (int f = 0; f < 2; f++) {
    C << "ITEM: TIMESTEP" << endl << f << endl << -80.5 / 2 << setw(15) << 80.5 / 2 << endl;
    for (long g = 0; g < N; g++)
      C << g + 1 << setw(15) << type[g % 42] << setw(15) << P[3 * g] << setw(15) << P[3 * g + 1] << setw(15)
        << P[3 * g + 2] << setw(15) << be[g] << setw(15) << q[g % 42] << endl;
    C << N + 1 << setw(15) << 3 << endl;
    D << "ITEM: TIMESTEP" << endl << f << endl << -80.5 / 2 << setw(15) << 80.5 / 2 << endl;
    write_lines(D, N, D.precision(), 0, [&](std::ostream& os, long g) {
      os << g + 1 << setw(15) << type[g % 42] << setw(15) << P[3 * g] << setw(15) << P[3 * g + 1] << setw(15)
         << P[3 * g + 2] << setw(15) << be[g] << setw(15) << q[g % 42];
      os.put('\n');
    });
    D << N + 1 << setw(15) << 3 << endl;
  }
  const bool r = A.str() == B.str(), m = C.str() == D.str();
  cout << "restart " << (r ? "identical" : "DIFFER") << ", movie " << (m ? "identical" : "DIFFER") << endl;
  return r && m ? 0 : 1;
}
