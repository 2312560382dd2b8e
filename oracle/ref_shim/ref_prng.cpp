// Exposes the reference's own host MD5 generator (src/padenti/prng.hpp,
// md5Rand at prng.hpp:107-195), compiled from the reference source tree, to the
// oracle tests through a C symbol.  Test infrastructure only.
#include <padenti/prng.hpp>

extern "C" void ref_md5Rand(const unsigned int *seed, unsigned int *state) {
  md5Rand(seed, state);
}
