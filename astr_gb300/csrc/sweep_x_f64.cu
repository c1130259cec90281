// Line sweeps along x (direction 0) in double; see sweeps.cuh.
#include "sweeps.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS(double, 0)
}  // namespace astr
