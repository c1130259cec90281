// Host-side view of the line-sweep launchers (definitions in sweeps.cuh,
// instantiated per direction in sweep_x.cu, sweep_y.cu, sweep_z.cu).
#pragma once

#include "astr_kernels.cuh"

namespace astr {

template <int DIR>
inline dim3 sweep_block() { return DIR == 0 ? dim3(NCH, X_LINES) : dim3(YZ_LINES, NCH); }

template <int DIR>
inline dim3 sweep_grid(const Geo& g) {
  if (DIR == 0) {
    long long nl = (long long)(g.jm + 1) * (g.km + 1);
    return dim3((unsigned)((nl + X_LINES - 1) / X_LINES), 1);
  }
  const unsigned gx = (unsigned)((g.im + YZ_LINES) / YZ_LINES);
  return dim3(gx, DIR == 1 ? g.km + 1 : g.jm + 1);
}

template <int DIR>
cudaError_t launch_filter(const SweepCtx& c, const DScheme& S, const FTab& T, int CH, int do_q2f);
template <int DIR>
cudaError_t launch_convgrad(const SweepCtx& c, const DScheme& S, int CH, CGFlags f);
template <int DIR>
cudaError_t launch_visc(const SweepCtx& c, const DScheme& S, int CH, VFlags f);

extern template cudaError_t launch_filter<0>(const SweepCtx&, const DScheme&, const FTab&, int, int);
extern template cudaError_t launch_filter<1>(const SweepCtx&, const DScheme&, const FTab&, int, int);
extern template cudaError_t launch_filter<2>(const SweepCtx&, const DScheme&, const FTab&, int, int);
extern template cudaError_t launch_convgrad<0>(const SweepCtx&, const DScheme&, int, CGFlags);
extern template cudaError_t launch_convgrad<1>(const SweepCtx&, const DScheme&, int, CGFlags);
extern template cudaError_t launch_convgrad<2>(const SweepCtx&, const DScheme&, int, CGFlags);
extern template cudaError_t launch_visc<0>(const SweepCtx&, const DScheme&, int, VFlags);
extern template cudaError_t launch_visc<1>(const SweepCtx&, const DScheme&, int, VFlags);
extern template cudaError_t launch_visc<2>(const SweepCtx&, const DScheme&, int, VFlags);

}  // namespace astr
