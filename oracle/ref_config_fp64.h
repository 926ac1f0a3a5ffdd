/*
 * TEST INFRASTRUCTURE ONLY.  Force-included ahead of the reference's headers
 * when oracle/Makefile builds the FP64 reference harness: it claims the
 * include guard of src/config_static.h and states the same compile-time
 * configuration (FUSED_INTEGRATOR, FUSED_PAIRWISE, LANGEVIN, 3-vectors) with
 * the scalar type switched to double, as src/config_static.h:30-44 would with
 * `using real = double;`.  No reference source is copied or modified.
 */
#ifndef OPENRBC_CONFIG_STATIC_H_
#define OPENRBC_CONFIG_STATIC_H_

#include "math_vector.h"

namespace openrbc {
namespace config {
#define FUSED_INTEGRATOR
#define FUSED_PAIRWISE
#define LANGEVIN
using real = double;
using vect = vector<real, 3>;
const static std::size_t cacheline = 64;
}  // namespace config

namespace constant {
const static config::real zero = 0;
const static config::real half = 0.5;
const static config::real one = 1;
const static config::real onehalf = 1.5;
const static config::real two = 2;
const static config::real four = 4;
}  // namespace constant
}  // namespace openrbc

#endif
