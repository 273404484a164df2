// Stand-in for boost::array (a fixed-size array), used by the reference's
// staticVector; std::array provides the same interface.  Test infrastructure
// of the oracle pin (oracle/ref/Makefile).
#pragma once
#include <array>
#include <cstddef>
namespace boost { template <class T, std::size_t N> class array : public std::array<T, N> {}; }
