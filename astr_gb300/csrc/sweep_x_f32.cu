// Line sweeps along x (direction 0) in float; see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(float, 0)
}  // namespace astr
