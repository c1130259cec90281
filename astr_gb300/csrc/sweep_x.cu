// Line sweeps along x (direction 0); see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(0)
}  // namespace astr
