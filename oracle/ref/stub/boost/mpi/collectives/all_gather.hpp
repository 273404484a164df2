// See ../../mpi.hpp: declaration-only stand-ins (oracle pin build).
#pragma once
#include "../../mpi.hpp"
