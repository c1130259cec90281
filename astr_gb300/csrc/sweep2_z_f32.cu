// Tile-staged sweeps along z (direction 2) in float; see sweeps2.cuh.
#include "sweeps2.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS2(float, 2)
}  // namespace astr
