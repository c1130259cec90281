// Device code of the GB300 (sm_103a) RHS hot path.
//
// One compact tridiagonal system per grid line.  A line is cut into 32
// chunks; each thread owns one chunk and runs the Thomas recurrences of the
// reference (src/commfunc.F90:790-813) locally in registers, assuming a zero
// carry at its chunk edge.  Because both recurrences are linear, the exact
// carries follow from one affine scan across the 32 chunks (warp shuffles
// when the chunks of a line share a warp, shared memory otherwise), after
// which every row is corrected by a precomputed carry weight:
//   forward   y_r = ytilde_r + G_r * y_{s-1},  G_r = prod_{m=s..r} (-ac3_m)
//   backward  x_r = xtilde_r + H_r * x_{e+1},  H_r = prod_{m=r..e} (-ac1_m)
// where s..e are the rows of the chunk.  The matrix factors ac1..ac3 are the
// reference's tridiagonal_thomas_proprocess (src/commfunc.F90:752-774).  The
// forward factor ac2 is folded into per-row right-hand-side coefficients
// (K7 = 7/9 ac2, K36 = 1/36 ac2 for the derivative; FK[m] = c10i(m) ac2 for
// the filter), so the forward step is one fused multiply-add.
//
// Precision: every kernel is a template on T, the type the sweeps store and
// compute in (double: the plain FP64 form; float: the FP32-storage form).
// The FP32-storage form keeps the conserved variables' RK3 base and master
// copy in FP64 (DevT::qsave, DevT::qm).
//
// Line orientation:
//   x-lines (DIR 0): a warp per line, lane = chunk; lines are contiguous.
//   y/z-lines (DIR 1,2): a block of 16 lines x 32 chunks; threadIdx.x walks
//   16 consecutive i so every row access is a coalesced segment.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace astr {

constexpr int HMD = 5;       // halo width (src/commvar.F90:184)
// Launch shape (lines per block, resident blocks per SM asked of the
// compiler), chosen by timing the 512^3 TGV step: several smaller blocks
// per SM overlap one block's loads with another's line solves.
#ifndef ASTR_YZ_LINES
#define ASTR_YZ_LINES 16
#endif
#ifndef ASTR_X_LINES
#define ASTR_X_LINES 4
#endif
#ifndef ASTR_MINB_YZ
#define ASTR_MINB_YZ 2
#endif
#ifndef ASTR_MINB_X
#define ASTR_MINB_X 6
#endif
#ifndef ASTR_NCH_B
#define ASTR_NCH_B 32
#endif
constexpr int NCH = 32;                // chunks per line, one-warp-per-line layout
constexpr int NCH_B = ASTR_NCH_B;      // chunks per line, block layouts (32 or 64)
static_assert(NCH_B == 32 || NCH_B == 64, "block layouts take 32 or 64 chunks per line");
constexpr int YZ_LINES = ASTR_YZ_LINES;  // lines per block for y/z sweeps
constexpr int X_LINES = ASTR_X_LINES;    // lines (warps) per block for x sweeps
constexpr int MINB_YZ = ASTR_MINB_YZ;    // resident blocks per SM asked of the compiler
constexpr int MINB_X = ASTR_MINB_X;

// One compact scheme (derivative or filter) of one direction, with the
// chunk carry weights for the chunk length used on that direction.
template <typename T>
struct DScheme {
  const T* ac1;
  const T* ac3;
  const T* G;
  const T* H;
  const T* ac2;  // forward factor (special rows)
  const T* K;    // folded interior coefficients: deriv 2 x n, filter 6 x n
  const T* KD;   // filter, correction form: 5 x n folded second-difference weights
  const T* A;    // off-diagonal coefficient of each row (a = c)
  int n;         // rows of the system
  int first;     // grid node of row 0
  int ntype;     // 3: periodic / inner block, 4: physical boundary at both ends
  int dim;       // im, jm or km
  int ks;        // row stride of K and KD: n, or 32 x CH in the padded arrays of the tiled sweeps
  // Chunks ulo..uhi lie where the Thomas factors have reached their steady
  // values exactly (bit for bit) and hold no boundary row: there the
  // factors and folded coefficients are these constants, and the carry
  // weights G, H are running products of -ac3, -ac1 in the host's order.
  int ulo, uhi;
  T u_ac1, u_ac3;
  T u_K[6];      // deriv: K7, K36; filter: the 6 folded c10i weights
  T u_KD[5];     // filter, correction form
};

// Filter right-hand-side tables (src/filter.F90:299-432).
template <typename T>
struct FTab {
  T c10[6], c8[5], c6[4];
  T cb[3][7];
  T ch[3][11];
};

struct Geo {
  int im, jm, km;
  long long NI, NJ, nh;  // halo-array strides and volume
  long long I, IJ, n0;   // interior strides and volume
  int per[3];            // periodic flags
  int lo[3], hi[3];      // is..ie, js..je, ks..ke
  int ndims;
};

template <typename T>
struct DevT {
  T* q;             // 5 halo arrays
  T* pr;            // 6 halo arrays: rho, u, v, w, p, T
  const T* xd;      // 3 halo arrays: dxi(1,1), dxi(2,2), dxi(3,3)
  const T* jac;     // halo array
  const double* jac64;   // halo array: J in FP64 (the RK3 base and update)
  const double* rjac64;  // halo array: 1/J in FP64
  T* qrhs;          // 5 interior arrays
  double* qsave;    // 5 interior arrays (RK3 base, FP64 in both forms)
  double* qm;       // 5 interior arrays: FP64 master of q (FP32 form only)
  T* grad;          // 12 interior arrays: dvel(n,m) at n+3m, dtmp(m) at 9+m
  T* sig;           // 6 interior arrays
  T* qf;            // 3 interior arrays
  double* part;     // statistics partial sums, 2 per warp
  int* flag;        // crash flag
  const double* chan;  // channel controller state (CHAN_*), null unless a channel
  const T* xg;      // general metrics: 9 halo arrays, dxi(d,m) at 3*d + m (0-based);
                    // null for diagonal metrics
};

// Channel controller state in device memory (FP64).
enum {
  CHAN_FORCE = 0,     // body force(1..3)
  CHAN_UBULK = 3,     // bulk velocity (1..3), src_chan
  CHAN_MASSFLUX = 6,  // massfluxchan of the last statcal
  CHAN_FBCX = 7,      // fbcxchan of the last statcal
  CHAN_TARGET = 8,    // target mass flux
  CHAN_N = 16
};

struct Phys {
  double const2, rconst6, hcc_scale;  // p/rho*const2 ; 1/const6 ; 1/(Pr*const5)
  double tempconst, tempconst1, rreynolds;
  double dt;
  double rk1, rk2, rk3;
  double rk3dt;   // rk3 * dt (the FP32-storage form's update)
  double rdx[3];  // mini-app reciprocal spacings
  // the same constants rounded to FP32 once, for the FP32 sweeps
  float f_const2, f_rconst6, f_hcc_scale, f_tempconst, f_tempconst1, f_rreynolds;
  float f_rdx[3];
  int mini;       // 1: mini-app ordering and scalings
};

// A physical constant in the sweep precision T.
template <typename T>
__device__ __forceinline__ T pc(double dv, float fv);
template <>
__device__ __forceinline__ double pc<double>(double dv, float) { return dv; }
template <>
__device__ __forceinline__ float pc<float>(double, float fv) { return fv; }

// Everything a sweep launch needs besides its scheme.
template <typename T>
struct SweepCtx {
  Geo g;
  DevT<T> d;
  Phys ph;
  cudaStream_t st;
  bool gen;    // general (non-diagonal) metrics
  int lbw;     // lines (warps) per block of the one-warp-per-line x layout
  int lbb[3];  // lines per block of the block layout, per direction
  int vsplit;  // 1: the variables of a line spread over gridDim.z blocks
};

__device__ __forceinline__ long long hidx(const Geo& g, int i, int j, int k) {
  return (long long)(i + HMD) + g.NI * ((long long)(j + HMD) + g.NJ * (long long)(k + HMD));
}
__device__ __forceinline__ long long zidx(const Geo& g, int i, int j, int k) {
  return (long long)i + g.I * (long long)j + g.IJ * (long long)k;
}
template <int DIR>
__device__ __forceinline__ long long hstride(const Geo& g) {
  return DIR == 0 ? 1 : (DIR == 1 ? g.NI : g.NI * g.NJ);
}
template <int DIR>
__device__ __forceinline__ long long zstride(const Geo& g) {
  return DIR == 0 ? 1 : (DIR == 1 ? g.I : g.IJ);
}
template <int DIR>
__device__ __forceinline__ void line_ijk(int a, int b, int l, int& i, int& j, int& k) {
  if (DIR == 0) { i = l; j = a; k = b; }
  else if (DIR == 1) { i = a; j = l; k = b; }
  else { i = a; j = b; k = l; }
}

// Line layout.  x sweeps with XB false hold one line per warp (lane = chunk,
// shuffle scans); every other sweep uses blocks of lines x 32 chunks with
// shared-memory scans (XB: the x filter, measured faster that way; the x
// derivative sweeps are faster one line per warp).  The lines (warps) per
// block are the launch's blockDim.x (blockDim.y), at most YZ_LINES
// (X_LINES): small grids launch fewer per block to occupy more SMs.
template <int DIR, bool XB = false>
constexpr bool warp_lines() { return DIR == 0 && !XB; }

// Thread -> (line, chunk) mapping.  Threads past the last line still take
// part in block-wide synchronisation (y/z); x-line warps past the end exit.
template <int DIR, bool XB = false>
struct LineMap {
  int a, b, c;
  bool active;
  __device__ __forceinline__ LineMap(const Geo& g) {
    if (warp_lines<DIR, XB>()) {
      c = threadIdx.x;
      const long long line = (long long)blockIdx.x * blockDim.y + threadIdx.y;
      const long long na = g.jm + 1, nl = na * (g.km + 1);
      active = line < nl;
      const long long L = active ? line : 0;
      a = (int)(L % na);
      b = (int)(L / na);
    } else {
      c = threadIdx.y;
      const int amax = DIR == 0 ? g.jm : g.im;
      const int ai = blockIdx.x * blockDim.x + threadIdx.x;
      active = ai <= amax;
      a = active ? ai : amax;
      b = blockIdx.y;
    }
  }
};

// ---------------------------------------------------------------------------
// Carry scans across the 32 chunks of a line.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T scan_fwd_warp(T M, T L, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const T Mo = __shfl_up_sync(0xffffffffu, M, off);
    const T Lo = __shfl_up_sync(0xffffffffu, L, off);
    if (lane >= off) {
      L = L + M * Lo;
      M = M * Mo;
    }
  }
  const T prev = __shfl_up_sync(0xffffffffu, L, 1);
  return lane == 0 ? T(0) : prev;
}

template <typename T>
__device__ __forceinline__ T scan_bwd_warp(T M, T L, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const T Mo = __shfl_down_sync(0xffffffffu, M, off);
    const T Lo = __shfl_down_sync(0xffffffffu, L, off);
    if (lane + off < 32) {
      L = L + M * Lo;
      M = M * Mo;
    }
  }
  const T next = __shfl_down_sync(0xffffffffu, L, 1);
  return lane == 31 ? T(0) : next;
}

constexpr int SM_PITCH = YZ_LINES + 1;
constexpr int SCAN_SMEM_WORDS = 2 * NCH_B * SM_PITCH;

// Block layouts: (M,L) of chunk c = threadIdx.y for line threadIdx.x.  Warp
// w scans line w; each lane takes NCH_B/32 consecutive chunks, composes them
// in scan order, joins the warp-wide affine scan, and writes each chunk's
// inclusive carry back.
template <bool FWD, typename T>
__device__ __forceinline__ T scan_block(T M, T L, T* sm) {
  T* sM = sm;
  T* sL = sm + NCH_B * SM_PITCH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  sM[ty * SM_PITCH + tx] = M;
  sL[ty * SM_PITCH + tx] = L;
  __syncthreads();
  const int nl = blockDim.x;  // lines in this block (at most YZ_LINES)
  const int tid = tx + nl * ty;
  const int w = tid >> 5, lane = tid & 31;
  if (w < nl) {
    constexpr int CPL = NCH_B / 32;
    T ml[CPL], ll[CPL];
#pragma unroll
    for (int e = 0; e < CPL; ++e) {
      ml[e] = sM[(lane * CPL + e) * SM_PITCH + w];
      ll[e] = sL[(lane * CPL + e) * SM_PITCH + w];
    }
    // the lane's chunks composed in scan order
    T m = FWD ? ml[0] : ml[CPL - 1];
    T l = FWD ? ll[0] : ll[CPL - 1];
#pragma unroll
    for (int k = 1; k < CPL; ++k) {
      const int e = FWD ? k : CPL - 1 - k;
      l = ll[e] + ml[e] * l;
      m = ml[e] * m;
    }
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const T Mo = FWD ? __shfl_up_sync(0xffffffffu, m, off) : __shfl_down_sync(0xffffffffu, m, off);
      const T Lo = FWD ? __shfl_up_sync(0xffffffffu, l, off) : __shfl_down_sync(0xffffffffu, l, off);
      const bool ok = FWD ? (lane >= off) : (lane + off < 32);
      if (ok) {
        l = l + m * Lo;
        m = m * Mo;
      }
    }
    if (CPL == 1) {
      sL[lane * SM_PITCH + w] = l;
    } else {
      // carry entering this lane's chunks, then each chunk's inclusive value
      const T prev = FWD ? __shfl_up_sync(0xffffffffu, l, 1) : __shfl_down_sync(0xffffffffu, l, 1);
      T carry = FWD ? (lane == 0 ? T(0) : prev) : (lane == 31 ? T(0) : prev);
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        const int e = FWD ? k : CPL - 1 - k;
        carry = ll[e] + ml[e] * carry;
        sL[(lane * CPL + e) * SM_PITCH + w] = carry;
      }
    }
  }
  __syncthreads();
  T r;
  if (FWD) r = ty == 0 ? T(0) : sL[(ty - 1) * SM_PITCH + tx];
  else r = ty == NCH_B - 1 ? T(0) : sL[(ty + 1) * SM_PITCH + tx];
  __syncthreads();
  return r;
}

// Whether task t (a variable of the sweep) is this block's: with gridDim.z
// > 1 the variables of a line are spread over the z blocks, one each (small
// grids, where one block per line group would leave SMs idle).  Tested
// inside the sweeps' constant-bound loops, so the unsplit kernels keep
// their register allocation.
__device__ __forceinline__ bool my_task(int t) { return gridDim.z == 1 || (int)blockIdx.z == t; }

// Is chunk c of a y/z sweep one of the scheme's uniform chunks?  (x sweeps
// hold a whole line in one warp, where a per-chunk branch would diverge.)
// Taken by the FP32 sweeps only: in the FP64 ones the second code path
// costs more in registers (64 per thread) than the loads it saves (3 %
// slower on the 512^3 step, 7 % faster in FP32).
template <int DIR, bool XB, typename T>
__device__ __forceinline__ bool uniform_chunk(const DScheme<T>& S, int c) {
  return sizeof(T) == 4 && !warp_lines<DIR, XB>() && c >= S.ulo && c <= S.uhi;
}

// In: y[t] = ac2-scaled right-hand side of row c*CH+t (row 0 unscaled).
// Out: y[t] = solution.
template <int CH, int DIR, bool XB, typename T>
__device__ __forceinline__ void chunk_solve(T (&y)[CH], const DScheme<T>& S, int c, T* sm,
                                            bool uni) {
  const int s = c * CH;
  T L = T(0), M = T(1);
  if (uni) {
    const T a3 = S.u_ac3;
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      if (t > 0) y[t] = y[t] - y[t - 1] * a3;
      M = M * (-a3);
    }
    L = y[CH - 1];
  } else {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int r = s + t;
      if (r < S.n) {
        if (t > 0) y[t] = y[t] - y[t - 1] * __ldg(S.ac3 + r);
        L = y[t];
        M = __ldg(S.G + r);
      }
    }
  }
  const T Yp = warp_lines<DIR, XB>() ? scan_fwd_warp(M, L, c) : scan_block<true>(M, L, sm);
  if (uni) {
    const T a3 = S.u_ac3;
    T gw = T(1);
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      gw = gw * (-a3);
      y[t] = y[t] + gw * Yp;
    }
  } else if (c > 0) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int r = s + t;
      if (r < S.n) y[t] = y[t] + __ldg(S.G + r) * Yp;
    }
  }
  T Lb = T(0), Mb = T(1);
  if (uni) {
    const T a1 = S.u_ac1;
#pragma unroll
    for (int t = CH - 2; t >= 0; --t) y[t] = y[t] - a1 * y[t + 1];
#pragma unroll
    for (int t = CH - 1; t >= 0; --t) Mb = Mb * (-a1);
    Lb = y[0];
  } else {
#pragma unroll
    for (int t = CH - 2; t >= 0; --t) {
      const int r = s + t;
      if (r < S.n - 1) y[t] = y[t] - __ldg(S.ac1 + r) * y[t + 1];
    }
    if (s < S.n) {
      Lb = y[0];
      Mb = __ldg(S.H + s);
    }
  }
  const T Xn = warp_lines<DIR, XB>() ? scan_bwd_warp(Mb, Lb, c) : scan_block<false>(Mb, Lb, sm);
  if (uni) {
    const T a1 = S.u_ac1;
    T hw = T(1);
#pragma unroll
    for (int t = CH - 1; t >= 0; --t) {
      hw = hw * (-a1);
      y[t] = y[t] + hw * Xn;
    }
  } else {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int r = s + t;
      if (r < S.n) y[t] = y[t] + __ldg(S.H + r) * Xn;
    }
  }
}

// Right-hand side of the compact first derivative (compact_fd_rhs,
// src/derivative.F90:210-306) for the rows of chunk c, scaled by ac2.
// f(node) is evaluated once per node into a window of radius 3.
template <int CH, typename T, class Fetch>
__device__ __forceinline__ void deriv_rhs(T (&y)[CH], const DScheme<T>& S, int c, const Fetch& f,
                                          bool uni) {
  const int s = c * CH;
  const int nb = S.first + s - 3;
  const int last = S.first + S.n - 1;
  T w[CH + 6];
#pragma unroll
  for (int t = 0; t < CH + 6; ++t) {
    const int nd = nb + t;
    w[t] = (nd >= S.first - 3 && nd <= last + 3) ? f(nd) : T(0);
  }
  if (uni) {
    const T k7 = S.u_K[0], k36 = S.u_K[1];
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const T* W = w + t + 3;
      y[t] = k7 * (W[1] - W[-1]) + k36 * (W[2] - W[-2]);
    }
    return;
  }
  const T* K7 = S.K;
  const T* K36 = S.K + S.n;
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    const T* W = w + t + 3;
    T d = T(0);
    if (r < S.n) {
      const bool special = S.ntype == 4 ? (r <= 1 || r >= S.n - 2) : (r == 0 || r == S.n - 1);
      if (!special) {
        d = __ldg(K7 + r) * (W[1] - W[-1]) + __ldg(K36 + r) * (W[2] - W[-2]);
      } else {
        if (S.ntype == 4) {
          if (r == 0) d = T(-2.5) * W[0] + T(2.0) * W[1] + T(0.5) * W[2];
          else if (r == S.n - 1) d = T(2.5) * W[0] - T(2.0) * W[-1] - T(0.5) * W[-2];
          else d = T(0.75) * (W[1] - W[-1]);
        } else {
          d = T(0.75) * (W[1] - W[-1]) - T(0.15) * (W[2] - W[-2]) + T(1.0 / 60.0) * (W[3] - W[-3]);
        }
        if (r > 0) d = d * __ldg(S.ac2 + r);
      }
    }
    y[t] = d;
  }
}

template <typename T, class Fetch>
__device__ __forceinline__ T filt_c8(const FTab<T>& Tb, const Fetch& f, int j) {
  const T v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
  const T v3 = f(j + 3) + f(j - 3), v4 = f(j + 4) + f(j - 4);
  return Tb.c8[0] * v0 + Tb.c8[1] * v1 + Tb.c8[2] * v2 + Tb.c8[3] * v3 + Tb.c8[4] * v4;
}
template <typename T, class Fetch>
__device__ __forceinline__ T filt_c6(const FTab<T>& Tb, const Fetch& f, int j) {
  const T v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
  const T v3 = f(j + 3) + f(j - 3);
  return Tb.c6[0] * v0 + Tb.c6[1] * v1 + Tb.c6[2] * v2 + Tb.c6[3] * v3;
}

// Boundary and end rows of the compact filter (compact_filter_rhs,
// src/filter.F90:176-269), scaled by ac2.  Out of line: only the first and
// last chunk of a line reach it.  v + base is node 0, hs the node stride.
// The row is evaluated on f - shift (shift = 0 is the reference's row).
template <typename T>
__device__ __noinline__ T filter_special_row(const DScheme<T>& S, const FTab<T>& Tb, int r,
                                             const T* v, long long base, long long hs, int per,
                                             T shift = T(0)) {
  const int dim = S.dim;
  auto f = [&](int node) -> T {
    int nd = node;
    if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
    return v[base + hs * nd] - shift;
  };
  const int last = S.first + S.n - 1;
  const int j = S.first + r;
  T d = T(0);
  if (S.ntype == 4) {
    if (r <= 2) {
      for (int m = 0; m <= 6; ++m) d = d + Tb.cb[r][m] * f(m);
    } else if (r >= S.n - 3) {
      const int kk = S.n - 1 - r;
      for (int m = 0; m <= 6; ++m) d = d + Tb.cb[kk][m] * f(last - m);
    } else if (r == 3 || r == S.n - 4) {
      d = filt_c6(Tb, f, j);
    } else {
      d = filt_c8(Tb, f, j);
    }
  } else {
    if (r <= 2) {
      for (int m = 0; m <= 10; ++m) d = d + Tb.ch[r][m] * f(S.first - 2 + m);
    } else {
      const int kk = S.n - 1 - r;
      for (int m = 0; m <= 10; ++m) d = d + Tb.ch[kk][m] * f(last + 2 - m);
    }
  }
  return r > 0 ? d * S.ac2[r] : d;
}

// The filter input of chunk c, loaded once: nodes first + c*CH - 5 ..
// first + c*CH + CH + 4 into w.  A periodic line wraps nodes below 0 and
// above dim onto the interior (as the reference's extended system reads
// them); only the end chunks need that, the others read straight through.
// Nodes no row of the chunk uses (rows past the system end) read as 0.
template <int CH, typename T>
__device__ __forceinline__ void filter_window(T (&w)[CH + 10], const DScheme<T>& S, int c,
                                              const T* v, long long base, long long hs,
                                              int per) {
  const int dim = S.dim;
  const int nb = S.first + c * CH - 5;
  if (nb >= 0 && nb + CH + 9 <= dim) {
    const T* p = v + base + hs * nb;
#pragma unroll
    for (int t = 0; t < CH + 10; ++t) w[t] = p[hs * t];
  } else {
#pragma unroll
    for (int t = 0; t < CH + 10; ++t) {
      int nd = nb + t;
      if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
      w[t] = (nd >= -HMD && nd <= dim + HMD) ? v[base + hs * nd] : T(0);
    }
  }
}

// Right-hand side of the compact filter (compact_filter_rhs,
// src/filter.F90:156-285) for the rows of chunk c, scaled by ac2, from the
// chunk's window w.  The interior stencil uses FK[m] = c10i(m) * ac2 with
// the centre weight doubled (the reference's f+f, exact).
template <int CH, typename T>
__device__ __forceinline__ void filter_rhs(T (&y)[CH], const T (&w)[CH + 10], const DScheme<T>& S,
                                           const FTab<T>& Tb, int c, const T* v, long long base,
                                           long long hs, int per, bool uni) {
  const int s = c * CH;
  const T* FK = S.K;
  const int n = S.n;
  if (uni) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const T* W = w + t + 5;
      y[t] = S.u_K[0] * W[0] + S.u_K[1] * (W[1] + W[-1]) + S.u_K[2] * (W[2] + W[-2]) +
             S.u_K[3] * (W[3] + W[-3]) + S.u_K[4] * (W[4] + W[-4]) + S.u_K[5] * (W[5] + W[-5]);
    }
    return;
  }
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    const T* W = w + t + 5;
    T d = T(0);
    if (r < n) {
      const bool special = S.ntype == 4 ? (r <= 4 || r >= n - 5) : (r <= 2 || r >= n - 3);
      if (special) {
        d = filter_special_row(S, Tb, r, v, base, hs, per);
      } else {
        d = __ldg(FK + r) * W[0] + __ldg(FK + n + r) * (W[1] + W[-1]) +
            __ldg(FK + 2 * n + r) * (W[2] + W[-2]) +
            __ldg(FK + 3 * n + r) * (W[3] + W[-3]) +
            __ldg(FK + 4 * n + r) * (W[4] + W[-4]) +
            __ldg(FK + 5 * n + r) * (W[5] + W[-5]);
      }
    }
    y[t] = d;
  }
}

// Correction form of the compact filter for the FP32 sweeps: the increment
// delta = A^{-1} (B - A) f.  B - A annihilates constants, so on interior rows
// (B - A) f is a sum of second differences f(j+k) + f(j-k) - 2 f(j), k = 1..5,
// with weights c10i(1) - alpha, c10i(2..5) (folded with ac2 in KD).  Their
// rounding scales with the variation of f, not its mean, which is what keeps
// the FP32 error of the filter small next to the field.  Every boundary and
// end row preserves constants as well (each B row sums to its A row: 1 + 2
// alpha, or 1 + beta on an end row), so those rows are evaluated on f - f(j)
// and the diagonal term drops out.
template <typename T>
__device__ __noinline__ T filter_special_delta(const DScheme<T>& S, const FTab<T>& Tb, int r,
                                               const T* v, long long base, long long hs,
                                               int per) {
  const int dim = S.dim;
  auto f = [&](int node) -> T {
    int nd = node;
    if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
    return v[base + hs * nd];
  };
  const int j = S.first + r;
  const T f0 = f(j);
  const T sc = r > 0 ? S.ac2[r] : T(1);
  const T d = filter_special_row(S, Tb, r, v, base, hs, per, f0);  // already * ac2
  const T a = S.A[r];
  T af = T(0);
  if (r > 0) af = af + a * (f(j - 1) - f0);
  if (r < S.n - 1) af = af + a * (f(j + 1) - f0);
  return d - af * sc;
}

template <int CH, typename T>
__device__ __forceinline__ void filter_rhs_delta(T (&y)[CH], const T (&w)[CH + 10],
                                                 const DScheme<T>& S, const FTab<T>& Tb, int c,
                                                 const T* v, long long base, long long hs,
                                                 int per, bool uni) {
  const int s = c * CH;
  const T* KD = S.KD;
  const int n = S.n;
  if (uni) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const T* W = w + t + 5;
      const T f0 = W[0];
      y[t] = S.u_KD[0] * ((W[1] - f0) + (W[-1] - f0)) + S.u_KD[1] * ((W[2] - f0) + (W[-2] - f0)) +
             S.u_KD[2] * ((W[3] - f0) + (W[-3] - f0)) + S.u_KD[3] * ((W[4] - f0) + (W[-4] - f0)) +
             S.u_KD[4] * ((W[5] - f0) + (W[-5] - f0));
    }
    return;
  }
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    const T* W = w + t + 5;
    T d = T(0);
    if (r < n) {
      const bool special = S.ntype == 4 ? (r <= 4 || r >= n - 5) : (r <= 2 || r >= n - 3);
      if (special) {
        d = filter_special_delta(S, Tb, r, v, base, hs, per);
      } else {
        const T f0 = W[0];
        d = __ldg(KD + r) * ((W[1] - f0) + (W[-1] - f0)) +
            __ldg(KD + n + r) * ((W[2] - f0) + (W[-2] - f0)) +
            __ldg(KD + 2 * n + r) * ((W[3] - f0) + (W[-3] - f0)) +
            __ldg(KD + 3 * n + r) * ((W[4] - f0) + (W[-4] - f0)) +
            __ldg(KD + 4 * n + r) * ((W[5] - f0) + (W[-5] - f0));
      }
    }
    y[t] = d;
  }
}

// q2fvar (src/fludyna.F90:545-634): conserved -> primitives at one point.
// The divisions by rho and const6 are multiplications by reciprocals.
template <typename T>
__device__ __forceinline__ void q2fvar_pt(const Phys& ph, T q1, T q2, T q3, T q4, T q5, T& ro,
                                          T& u, T& v, T& w, T& p, T& tt) {
  ro = q1;
  const T rr = T(1) / ro;
  u = q2 * rr;
  v = q3 * rr;
  w = q4 * rr;
  p = (q5 - T(0.5) * ro * (u * u + v * v + w * w)) * pc<T>(ph.rconst6, ph.f_rconst6);
  tt = p * rr * pc<T>(ph.const2, ph.f_const2);
}

template <typename T>
__device__ __forceinline__ void q2fvar_store(const Geo& g, const DevT<T>& d, const Phys& ph,
                                             long long p) {
  const long long nh = g.nh;
  T ro, u, v, w, pp, tt;
  q2fvar_pt<T>(ph, d.q[p], d.q[p + nh], d.q[p + 2 * nh], d.q[p + 3 * nh], d.q[p + 4 * nh], ro, u,
               v, w, pp, tt);
  d.pr[p] = ro;
  d.pr[p + nh] = u;
  d.pr[p + 2 * nh] = v;
  d.pr[p + 3 * nh] = w;
  d.pr[p + 4 * nh] = pp;
  d.pr[p + 5 * nh] = tt;
  if (!(ro > T(0))) atomicOr(d.flag, 1);
}

struct CGFlags {
  int conv, grad, first, last, sigma, stats, qsave;
};

struct VFlags {
  int last;  // fuse the RK3 update of all five variables
  int q2f;   // and recover the primitives (main ordering)
};

// Viscous stress and heat flux at one interior point (diffrsdcal6,
// src/solver.F90:2433-2545), miucal (src/fludyna.F90:791-820).
template <typename T>
__device__ __forceinline__ void sigma_point(const Geo& g, const DevT<T>& d, const Phys& ph,
                                            long long z, long long h) {
  const long long n0 = g.n0, nh = g.nh;
  const T* G = d.grad + z;
  const T tt = d.pr[h + 5 * nh];
  const T miu = tt * sqrt(tt) * pc<T>(ph.tempconst1, ph.f_tempconst1) /
                (tt + pc<T>(ph.tempconst, ph.f_tempconst)) * pc<T>(ph.rreynolds, ph.f_rreynolds);
  const T s11 = G[0];
  const T s12 = T(0.5) * (G[3 * n0] + G[1 * n0]);
  const T s13 = T(0.5) * (G[6 * n0] + G[2 * n0]);
  const T s22 = G[4 * n0];
  const T s23 = T(0.5) * (G[7 * n0] + G[5 * n0]);
  const T s33 = G[8 * n0];
  const T skk = T(1.0 / 3.0) * (s11 + s22 + s33);
  const T miu2 = T(2) * miu;
  const T hcc = miu * pc<T>(ph.hcc_scale, ph.f_hcc_scale);
  const T S1 = miu2 * (s11 - skk), S2 = miu2 * s12, S3 = miu2 * s13;
  const T S4 = miu2 * (s22 - skk), S5 = miu2 * s23, S6 = miu2 * (s33 - skk);
  const T u = d.pr[h + nh], v = d.pr[h + 2 * nh], w = d.pr[h + 3 * nh];
  T* Sg = d.sig + z;
  Sg[0] = S1; Sg[n0] = S2; Sg[2 * n0] = S3; Sg[3 * n0] = S4; Sg[4 * n0] = S5; Sg[5 * n0] = S6;
  T* Q = d.qf + z;
  Q[0] = hcc * G[9 * n0] + S1 * u + S2 * v + S3 * w;
  Q[n0] = hcc * G[10 * n0] + S2 * u + S4 * v + S5 * w;
  Q[2 * n0] = hcc * G[11 * n0] + S3 * u + S5 * v + S6 * w;
}

// The conserved value q at an interior point with FP64 accuracy: the FP64
// form reads it; the FP32-storage form reads its FP64 master, which every
// writer of interior q updates with the FP32 copy (RK3 update, filter
// increments, interface averaging, walls, upload).
__device__ __forceinline__ double q64(const DevT<double>& d, long long p, long long z, int m,
                                      long long nh, long long n0) {
  (void)z; (void)n0;
  return d.q[m * nh + p];
}
__device__ __forceinline__ double q64(const DevT<float>& d, long long p, long long z, int m,
                                      long long nh, long long n0) {
  (void)p; (void)nh;
  return d.qm[m * n0 + z];
}

// RK3 stage update (src/mainloop.F90:441-451) of variable m at one point.
// Main ordering: q = (rk1*qsave + rk2*q*J + rk3*dt*rhs)/J, the division a
// multiplication by the stored 1/J; mini-app ordering: no Jacobian.
// The updated value from its operands (qs: RK3 base, qv: current q, rhs:
// residual, J and 1/J; chan: the channel controller or null).
__device__ __forceinline__ double rk_value(const Phys& ph, const double* chan, int m, double qs,
                                           double qv, double rhs, double J, double rj) {
  if (chan) {
    // src_chan (src/solver.F90:335-346): body force and its work, times J
    const double* C = chan;
    const double f = m == 0 ? 0.0
                   : (m < 4 ? C[CHAN_FORCE + m - 1]
                            : C[CHAN_FORCE] * C[CHAN_UBULK] + C[CHAN_FORCE + 1] * C[CHAN_UBULK + 1] +
                                  C[CHAN_FORCE + 2] * C[CHAN_UBULK + 2]);
    rhs = rhs + f * J;
  }
  if (ph.mini) return ph.rk1 * qs + ph.rk2 * qv + ph.rk3 * rhs * ph.dt;
  return (ph.rk1 * qs + ph.rk2 * qv * J + ph.rk3 * rhs * ph.dt) * rj;
}

template <typename T>
__device__ __forceinline__ void rk_update(const Geo& g, const DevT<T>& d, const Phys& ph,
                                          long long p, long long z, int m, double rhs) {
  const long long nh = g.nh, n0 = g.n0;
  const double J = d.jac64[p], rj = d.rjac64[p];
  const double v = rk_value(ph, d.chan, m, d.qsave[m * n0 + z], q64(d, p, z, m, nh, n0), rhs, J, rj);
  d.q[m * nh + p] = (T)v;
  if (d.qm) d.qm[m * n0 + z] = v;
}

}  // namespace astr
