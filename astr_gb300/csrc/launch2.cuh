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

// One case of a batch (device memory): its geometry, fields, constants and
// padded schemes per direction.
template <typename T>
struct BCase {
  Geo g;
  DevT<T> d;
  Phys ph;
  FTab<T> Tb;
  DScheme<T> Sd[3], Sf[3];
  int vsplit;
};

// Stop control of batched steps.  Every step starts with a gate (one
// thread) that reads the host-mapped cancel word and the GPU's global timer
// against the deadline (ns, a device word set when the call starts; 0: none)
// and, when either says stop, sets the status word (bit 0 cancelled, bit 1
// deadline passed); otherwise it counts the step as started.  The items of
// the sweeps and point kernels read only the status word, so a step that
// passed its gate runs to its end and the cases stay at a step boundary.
struct BatchCtl {
  const volatile int* cancel;             // mapped host word; may be null
  const unsigned long long* deadline_ns;  // device word; 0 in it: no deadline
  int* status;
  int* started;                           // steps that passed their gate
};

#ifdef __CUDACC__
__device__ __forceinline__ int batch_stopped(const BatchCtl& c) { return *(volatile int*)c.status; }
#endif

// Lines per block of the tiled sweeps (FP32 storage / FP64).
#ifndef ASTR_V2_NL32
#define ASTR_V2_NL32 8
#endif
#ifndef ASTR_V2_NL64
#define ASTR_V2_NL64 4
#endif
template <typename T>
__host__ __device__ constexpr int v2_nl() { return sizeof(T) == 4 ? ASTR_V2_NL32 : ASTR_V2_NL64; }

// Blocks of a tiled sweep along dir (x: line groups of NL, y: the other
// transverse index), before the variable split.
inline void v2_blocks(const Geo& g, int dir, int NL, int& gx, int& gy) {
  const int amax = dir == 0 ? g.jm : g.im;
  gx = (amax + NL) / NL;
  gy = dir == 2 ? g.jm + 1 : g.km + 1;
}

template <typename T, int DIR>
cudaError_t launch2_filter(const V2Args<T>& a, cudaStream_t st, int CH, int vsplit);
template <typename T, int DIR>
cudaError_t launch2_convgrad(const V2Args<T>& a, cudaStream_t st, int CH, CGFlags f, int vsplit);
template <typename T, int DIR>
cudaError_t launch2_visc(const V2Args<T>& a, cudaStream_t st, int CH, int vsplit);
template <typename T, int DIR>
cudaError_t launch2_batch(int kind, int CH, const V2Args<T>& a, const BCase<T>* cases, const int4* items,
                          int nitems, BatchCtl ctl, int nsm, cudaStream_t st);

#define ASTR_DECLARE_SWEEPS2(T, DIR)                                                              \
  extern template cudaError_t launch2_filter<T, DIR>(const V2Args<T>&, cudaStream_t, int, int);  \
  extern template cudaError_t launch2_convgrad<T, DIR>(const V2Args<T>&, cudaStream_t, int,       \
                                                       CGFlags, int);                            \
  extern template cudaError_t launch2_visc<T, DIR>(const V2Args<T>&, cudaStream_t, int, int);     \
  extern template cudaError_t launch2_batch<T, DIR>(int, int, const V2Args<T>&, const BCase<T>*, \
                                                    const int4*, int, BatchCtl, int, cudaStream_t);

ASTR_DECLARE_SWEEPS2(double, 0)
ASTR_DECLARE_SWEEPS2(double, 1)
ASTR_DECLARE_SWEEPS2(double, 2)
ASTR_DECLARE_SWEEPS2(float, 0)
ASTR_DECLARE_SWEEPS2(float, 1)
ASTR_DECLARE_SWEEPS2(float, 2)

}  // namespace astr
