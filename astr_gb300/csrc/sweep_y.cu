// Line sweeps along y (direction 1); see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(1)
}  // namespace astr
