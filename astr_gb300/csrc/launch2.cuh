// Host-side view of the tile-staged sweeps (definitions in sweeps2.cuh,
// instantiated per direction and precision in the sweep2_*.cu units).
#pragma once

#include "launch.cuh"

namespace astr {

// Everything a tiled-sweep launch needs besides the flags.
template <typename T>
struct V2Args {
  Geo g;
  DevT<T> d;
  DScheme<T> S;   // padded coefficient arrays (ks = 32 * CH)
  FTab<T> Tb;
  Phys ph;
  // uniform-chunk constants (FP64; cast per launch)
  double a1, a3, K[6], KD[5], gp[33], hp[33];
};

template <typename T, int DIR>
cudaError_t launch2_filter(const V2Args<T>& a, cudaStream_t st, int CH, int vsplit);
template <typename T, int DIR>
cudaError_t launch2_convgrad(const V2Args<T>& a, cudaStream_t st, int CH, CGFlags f, int vsplit);
template <typename T, int DIR>
cudaError_t launch2_visc(const V2Args<T>& a, cudaStream_t st, int CH, int vsplit);

#define ASTR_DECLARE_SWEEPS2(T, DIR)                                                              \
  extern template cudaError_t launch2_filter<T, DIR>(const V2Args<T>&, cudaStream_t, int, int);  \
  extern template cudaError_t launch2_convgrad<T, DIR>(const V2Args<T>&, cudaStream_t, int,       \
                                                       CGFlags, int);                            \
  extern template cudaError_t launch2_visc<T, DIR>(const V2Args<T>&, cudaStream_t, int, int);

ASTR_DECLARE_SWEEPS2(double, 0)
ASTR_DECLARE_SWEEPS2(double, 1)
ASTR_DECLARE_SWEEPS2(double, 2)
ASTR_DECLARE_SWEEPS2(float, 0)
ASTR_DECLARE_SWEEPS2(float, 1)
ASTR_DECLARE_SWEEPS2(float, 2)

}  // namespace astr
