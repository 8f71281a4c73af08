// ORACLE (test infrastructure only): part of the project-owned Kokkos subset,
// whose declarations all live in Kokkos_Core.hpp.
#include "Kokkos_Core.hpp"
