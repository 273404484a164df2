// Declaration-only stand-ins for the Boost.MPI names the reference's headers
// mention (a one-rank communicator whose calls do nothing), so that its
// element-level sources compile without MPI.  None of it runs in the element
// computations the oracle pin uses.  Test infrastructure (oracle/ref/Makefile).
#pragma once
#include <vector>
namespace boost {
namespace mpl {
struct true_ { static const bool value = true; };
struct false_ { static const bool value = false; };
}  // namespace mpl
namespace mpi {
template <class T> struct is_mpi_datatype : mpl::false_ {};
class status {};
class request {
 public:
  status wait() { return status(); }
  bool test() { return true; }
};
class communicator {
 public:
  int size() const { return 1; }
  int rank() const { return 0; }
  void barrier() const {}
  template <class T> request isend(int, int, const T&) const { return request(); }
  template <class T> request irecv(int, int, T&) const { return request(); }
  template <class T> void send(int, int, const T&) const {}
  template <class T> status recv(int, int, T&) const { return status(); }
};
template <class I> void wait_all(I, I) {}
}  // namespace mpi
}  // namespace boost
