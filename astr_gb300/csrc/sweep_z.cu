// Line sweeps along z (direction 2); see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(2)
}  // namespace astr
