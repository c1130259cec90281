// Line sweeps along z (direction 2) in float; see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(float, 2)
}  // namespace astr
