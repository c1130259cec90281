// Tile-staged sweeps along y (direction 1) in double; see sweeps2.cuh.
#include "sweeps2.cuh"

namespace astr {
ASTR_INSTANTIATE_SWEEPS2(double, 1)
}  // namespace astr
