// Tile-staged sweeps along x (direction 0) in float; see sweeps2.cuh.
#include "sweeps2.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS2(float, 0)
}  // namespace astr
