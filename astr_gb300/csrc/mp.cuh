// Compact MP convective scheme (conschm 543c, convrsdcmp,
// src/solver.F90:1271-1937) on the device, FP64.  Per direction:
//   k_mp_split   Steger-Warming split F+, F- at every node of the split
//                range (src/riemann.F90:23-160) into the fsw scratch;
//   k_mp_cflux   the compact upwind / downwind interface values of the ten
//                split components (src/flux.F90:125-256): chunked Thomas
//                solves, one block of lines x 32 chunks, as the filter;
//   k_mp_face    per interface: Roe eigenvectors (chardecomp,
//                src/solver.F90:1958-2162), projection of the five-point
//                stencils and the compact values, MP5 limiting
//                (src/flux.F90:363-496), back-projection -> Fh; with the
//                characteristic decomposition only on the interfaces the
//                sensor flags, listed by k_mp_face_split, which writes the
//                others;
//   k_mp_diff    qrhs = qrhs + Fh(i) - Fh(i-1), negated after the last
//                direction (rhscal's qrhs = -qrhs, src/solver.F90:242).
// The Ducros sensor (src/commcal.F90:196-353) runs before the directions
// when the characteristic decomposition is on.
#pragma once

#include "astr_kernels.cuh"

namespace astr {

// Device scratch and switches of the MP path.
struct MPDev {
  double* fsw;            // 10 halo arrays: F+ (5), F- (5) of the current direction
  double* fhc;            // 10 halo arrays: compact interface values, interface i at node i
  double* fh;             // 5 halo arrays: limited interface flux Fh(i) at node i
  double* ssf;            // halo array: shock-sensor function
  unsigned char* lshock;  // interior array
  int* flist;             // flagged interfaces of the current direction (box indices)
  int* fcount;            // their number
  int chard;              // lchardecomp: characteristic projection and sensor
  int npdc[3];
  double mach, rmach, bfac, shkcrt;  // rmach = 1/mach
};

struct MPSchemes {
  DScheme<double> uw[3], dw[3];
  int CH[3];
  int lbb[3];  // lines per block of the block layout, per direction
  int vsplit;  // 1: the ten variables of a line spread over gridDim.z blocks
};

// node range of the flux split (iss..iee), src/solver.F90:1318-1332
__host__ __device__ inline void mp_split_range(int npdc, int dim, int& a, int& b) {
  if (npdc == 1) { a = 0; b = dim + 5; }
  else if (npdc == 2) { a = -5; b = dim; }
  else if (npdc == 3) { a = -5; b = dim + 5; }
  else { a = 0; b = dim; }
}

// A box of nodes, x index fastest, for the point kernels of one direction.
struct Box {
  int i0, j0, k0, ni, nj, nk;
  __host__ __device__ long long count() const { return (long long)ni * nj * nk; }
};

cudaError_t launch_mp_sensor(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st,
                             int part);
template <int DIR>
cudaError_t launch_mp_split(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st);
template <int DIR>
cudaError_t launch_mp_cflux(const Geo& g, const MPDev& m, const MPSchemes& S, cudaStream_t st);
template <int DIR>
cudaError_t launch_mp_face(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st);
template <int DIR>
cudaError_t launch_mp_diff(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st,
                           int last);

}  // namespace astr
