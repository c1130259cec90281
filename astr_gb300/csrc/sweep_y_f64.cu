// Line sweeps along y (direction 1) in double; see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(double, 1)
}  // namespace astr
