// Host-side view of the line-sweep launchers (definitions in sweeps.cuh,
// instantiated per direction and precision in the sweep_*.cu units).
#pragma once

#include "astr_kernels.cuh"

namespace astr {

// lb: lines (warps) per block, at most X_LINES for the one-warp-per-line
// layout and YZ_LINES for the block layout.
template <int DIR, bool XB = false>
inline dim3 sweep_block(int lb) { return warp_lines<DIR, XB>() ? dim3(NCH, lb) : dim3(lb, NCH_B); }

template <int DIR, bool XB = false>
inline dim3 sweep_grid(const Geo& g, int lb) {
  if (warp_lines<DIR, XB>()) {
    long long nl = (long long)(g.jm + 1) * (g.km + 1);
    return dim3((unsigned)((nl + lb - 1) / lb), 1);
  }
  // lines: a = i (y, z sweeps) or j (x sweeps) across the block, b = the
  // remaining transverse index across blockIdx.y
  const int amax = DIR == 0 ? g.jm : g.im;
  const unsigned gx = (unsigned)((amax + lb) / lb);
  return dim3(gx, DIR == 1 ? g.km + 1 : (DIR == 0 ? g.km + 1 : g.jm + 1));
}

template <int DIR, bool XB, typename C>
inline int sweep_lb(const C& c) { return warp_lines<DIR, XB>() ? c.lbw : c.lbb[DIR]; }

template <typename T, int DIR>
cudaError_t launch_filter(const SweepCtx<T>& c, const DScheme<T>& S, const FTab<T>& Tb, int CH,
                          int do_q2f);
template <typename T, int DIR>
cudaError_t launch_convgrad(const SweepCtx<T>& c, const DScheme<T>& S, int CH, CGFlags f);
template <typename T, int DIR>
cudaError_t launch_visc(const SweepCtx<T>& c, const DScheme<T>& S, int CH, VFlags f);

#define ASTR_DECLARE_SWEEPS(T, DIR)                                                                \
  extern template cudaError_t launch_filter<T, DIR>(const SweepCtx<T>&, const DScheme<T>&,         \
                                                    const FTab<T>&, int, int);                    \
  extern template cudaError_t launch_convgrad<T, DIR>(const SweepCtx<T>&, const DScheme<T>&, int,  \
                                                      CGFlags);                                   \
  extern template cudaError_t launch_visc<T, DIR>(const SweepCtx<T>&, const DScheme<T>&, int, VFlags);

ASTR_DECLARE_SWEEPS(double, 0)
ASTR_DECLARE_SWEEPS(double, 1)
ASTR_DECLARE_SWEEPS(double, 2)
ASTR_DECLARE_SWEEPS(float, 0)
ASTR_DECLARE_SWEEPS(float, 1)
ASTR_DECLARE_SWEEPS(float, 2)

}  // namespace astr
