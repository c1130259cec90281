// Tile-staged sweeps along y (direction 1) in float; see sweeps2.cuh.
#include "sweeps2.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS2(float, 1)
}  // namespace astr
