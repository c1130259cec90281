// Line sweeps along y (direction 1) in float; see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(float, 1)
}  // namespace astr
