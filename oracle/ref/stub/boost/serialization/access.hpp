// Declaration-only stand-in for the one Boost.Serialization name the
// reference's dof types mention (friend class boost::serialization::access),
// so that its element-level sources compile without Boost.  Test
// infrastructure of the oracle pin (oracle/ref/Makefile); no behaviour.
#pragma once
namespace boost { namespace serialization { class access {}; } }
