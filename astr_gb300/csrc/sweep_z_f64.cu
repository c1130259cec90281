// Line sweeps along z (direction 2) in double; see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(double, 2)
}  // namespace astr
