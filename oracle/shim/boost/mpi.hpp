// Oracle test infrastructure: a single-process stand-in for the few Boost.MPI
// names the SOUFFLE sources use (environment, communicator, all_gather).
// One rank, so all_gather is a local copy.  Used only to compile the reference
// sources as a CPU checker; nothing in the product links it.
#ifndef ORACLE_SHIM_BOOST_MPI_HPP
#define ORACLE_SHIM_BOOST_MPI_HPP
#include <vector>

namespace boost {
namespace mpi {

class environment {
 public:
  environment() {}
  environment(int&, char**&) {}
};

class communicator {
 public:
  int rank() const { return 0; }
  int size() const { return 1; }
};

template <class T>
void all_gather(const communicator&, const T* in, int n, std::vector<T>& out) {
  out.assign(in, in + n);
}

}  // namespace mpi
}  // namespace boost

#endif
