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
// reference's tridiagonal_thomas_proprocess (src/commfunc.F90:752-774).
//
// Line orientation:
//   x-lines (DIR 0): a warp per line, lane = chunk; lines are contiguous.
//   y/z-lines (DIR 1,2): a block of 16 lines x 32 chunks; threadIdx.x walks
//   16 consecutive i so every row access is a coalesced 128-byte segment.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace astr {

constexpr int HMD = 5;       // halo width (src/commvar.F90:184)
constexpr int NCH = 32;      // chunks per line
constexpr int YZ_LINES = 16; // lines per block for y/z sweeps
constexpr int X_LINES = 8;   // lines (warps) per block for x sweeps

constexpr double NUM1D3 = 1.0 / 3.0;
constexpr double NUM7D9 = 7.0 / 9.0;
constexpr double NUM1D36 = 1.0 / 36.0;
constexpr double NUM1D60 = 1.0 / 60.0;

// One compact scheme (derivative or filter) of one direction, with the
// chunk carry weights for the chunk length used on that direction.
struct DScheme {
  const double* ac1;
  const double* ac2;
  const double* ac3;
  const double* G;
  const double* H;
  int n;      // rows of the system
  int first;  // grid node of row 0
  int ntype;  // 3: periodic / inner block, 4: physical boundary at both ends
  int dim;    // im, jm or km
};

// Filter right-hand-side tables (src/filter.F90:299-432).
struct FTab {
  double c10[6], c8[5], c6[4];
  double cb[3][7];
  double ch[3][11];
};

struct Geo {
  int im, jm, km;
  long long NI, NJ, nh;  // halo-array strides and volume
  long long I, IJ, n0;   // interior strides and volume
  int per[3];            // periodic flags
  int lo[3], hi[3];      // is..ie, js..je, ks..ke
  int ndims;
};

struct Dev {
  double* q;        // 5 halo arrays
  double* pr;       // 6 halo arrays: rho, u, v, w, p, T
  const double* xd; // 3 halo arrays: dxi(1,1), dxi(2,2), dxi(3,3)
  const double* jac;// halo array
  double* qrhs;     // 5 interior arrays
  double* qsave;    // 5 interior arrays
  double* grad;     // 12 interior arrays: dvel(n,m) at n+3m, dtmp(m) at 9+m
  double* sig;      // 6 interior arrays
  double* qf;       // 3 interior arrays
  double* part;     // statistics partial sums, 2 per block
  int* flag;        // crash flag
};

struct Phys {
  double const2, const5, const6;
  double tempconst, tempconst1, reynolds, prandtl;
  double dt;
  double rk1, rk2, rk3;
  double dx[3];  // mini-app uniform spacings
  int mini;      // 1: mini-app ordering and scalings
};

// Everything a sweep launch needs besides its scheme.
struct SweepCtx {
  Geo g;
  Dev d;
  Phys ph;
  cudaStream_t st;
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

// Thread -> (line, chunk) mapping.  Returns false for threads past the last
// line; those threads still take part in block-wide synchronisation.
template <int DIR>
struct LineMap {
  int a, b, c;
  bool active;
  __device__ __forceinline__ LineMap(const Geo& g) {
    if (DIR == 0) {
      c = threadIdx.x;
      const long long line = (long long)blockIdx.x * X_LINES + threadIdx.y;
      const long long na = g.jm + 1, nl = na * (g.km + 1);
      active = line < nl;
      const long long L = active ? line : 0;
      a = (int)(L % na);
      b = (int)(L / na);
    } else {
      c = threadIdx.y;
      const int ai = blockIdx.x * YZ_LINES + threadIdx.x;
      active = ai <= g.im;
      a = active ? ai : g.im;
      b = blockIdx.y;
    }
  }
};

// ---------------------------------------------------------------------------
// Carry scans across the 32 chunks of a line.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double scan_fwd_warp(double M, double L, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double Mo = __shfl_up_sync(0xffffffffu, M, off);
    const double Lo = __shfl_up_sync(0xffffffffu, L, off);
    if (lane >= off) {
      L = L + M * Lo;
      M = M * Mo;
    }
  }
  const double prev = __shfl_up_sync(0xffffffffu, L, 1);
  return lane == 0 ? 0.0 : prev;
}

__device__ __forceinline__ double scan_bwd_warp(double M, double L, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double Mo = __shfl_down_sync(0xffffffffu, M, off);
    const double Lo = __shfl_down_sync(0xffffffffu, L, off);
    if (lane + off < 32) {
      L = L + M * Lo;
      M = M * Mo;
    }
  }
  const double next = __shfl_down_sync(0xffffffffu, L, 1);
  return lane == 31 ? 0.0 : next;
}

constexpr int SM_PITCH = YZ_LINES + 1;
constexpr int SCAN_SMEM_DOUBLES = 2 * NCH * SM_PITCH;

// y/z sweeps: (M,L) of chunk c = threadIdx.y for line threadIdx.x.
// Warp w scans line w with lane = chunk.
template <bool FWD>
__device__ __forceinline__ double scan_block(double M, double L, double* sm) {
  double* sM = sm;
  double* sL = sm + NCH * SM_PITCH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  sM[ty * SM_PITCH + tx] = M;
  sL[ty * SM_PITCH + tx] = L;
  __syncthreads();
  const int tid = tx + YZ_LINES * ty;
  const int w = tid >> 5, lane = tid & 31;
  if (w < YZ_LINES) {
    double m = sM[lane * SM_PITCH + w];
    double l = sL[lane * SM_PITCH + w];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double Mo = FWD ? __shfl_up_sync(0xffffffffu, m, off) : __shfl_down_sync(0xffffffffu, m, off);
      const double Lo = FWD ? __shfl_up_sync(0xffffffffu, l, off) : __shfl_down_sync(0xffffffffu, l, off);
      const bool ok = FWD ? (lane >= off) : (lane + off < 32);
      if (ok) {
        l = l + m * Lo;
        m = m * Mo;
      }
    }
    sL[lane * SM_PITCH + w] = l;
  }
  __syncthreads();
  double r;
  if (FWD) r = ty == 0 ? 0.0 : sL[(ty - 1) * SM_PITCH + tx];
  else r = ty == NCH - 1 ? 0.0 : sL[(ty + 1) * SM_PITCH + tx];
  __syncthreads();
  return r;
}

// In: y[t] = right-hand side of row c*CH+t.  Out: y[t] = solution.
template <int CH, int DIR>
__device__ __forceinline__ void chunk_solve(double (&y)[CH], const DScheme& S, int c, double* sm) {
  const int s = c * CH;
  double L = 0.0, M = 1.0;
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    if (r < S.n) {
      if (t == 0) {
        if (r != 0) y[0] = y[0] * __ldg(S.ac2 + r);
      } else {
        y[t] = y[t] * __ldg(S.ac2 + r) - y[t - 1] * __ldg(S.ac3 + r);
      }
      L = y[t];
      M = __ldg(S.G + r);
    }
  }
  const double Yp = (DIR == 0) ? scan_fwd_warp(M, L, c) : scan_block<true>(M, L, sm);
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    if (r < S.n) y[t] = y[t] + __ldg(S.G + r) * Yp;
  }
#pragma unroll
  for (int t = CH - 2; t >= 0; --t) {
    const int r = s + t;
    if (r < S.n - 1) y[t] = y[t] - __ldg(S.ac1 + r) * y[t + 1];
  }
  double Lb = 0.0, Mb = 1.0;
  if (s < S.n) {
    Lb = y[0];
    Mb = __ldg(S.H + s);
  }
  const double Xn = (DIR == 0) ? scan_bwd_warp(Mb, Lb, c) : scan_block<false>(Mb, Lb, sm);
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    if (r < S.n) y[t] = y[t] + __ldg(S.H + r) * Xn;
  }
}

// Right-hand side of the compact first derivative (compact_fd_rhs,
// src/derivative.F90:210-306) for the rows of chunk c.  f(node) is
// evaluated once per node into a window of radius 3.
template <int CH, class Fetch>
__device__ __forceinline__ void deriv_rhs(double (&y)[CH], const DScheme& S, int c, const Fetch& f) {
  const int s = c * CH;
  const int nb = S.first + s - 3;
  const int last = S.first + S.n - 1;
  double w[CH + 6];
#pragma unroll
  for (int t = 0; t < CH + 6; ++t) {
    const int nd = nb + t;
    w[t] = (nd >= S.first - 3 && nd <= last + 3) ? f(nd) : 0.0;
  }
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    const double* W = w + t + 3;
    double d;
    if (S.ntype == 4) {
      if (r == 0) d = -2.5 * W[0] + 2.0 * W[1] + 0.5 * W[2];
      else if (r == 1 || r == S.n - 2) d = 0.75 * (W[1] - W[-1]);
      else if (r == S.n - 1) d = 2.5 * W[0] - 2.0 * W[-1] - 0.5 * W[-2];
      else d = NUM7D9 * (W[1] - W[-1]) + NUM1D36 * (W[2] - W[-2]);
    } else {
      if (r == 0 || r == S.n - 1)
        d = 0.75 * (W[1] - W[-1]) - 0.15 * (W[2] - W[-2]) + NUM1D60 * (W[3] - W[-3]);
      else
        d = NUM7D9 * (W[1] - W[-1]) + NUM1D36 * (W[2] - W[-2]);
    }
    y[t] = (r < S.n) ? d : 0.0;
  }
}

template <class Fetch>
__device__ __forceinline__ double filt_c10(const FTab& T, const Fetch& f, int j) {
  const double v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
  const double v3 = f(j + 3) + f(j - 3), v4 = f(j + 4) + f(j - 4), v5 = f(j + 5) + f(j - 5);
  return T.c10[0] * v0 + T.c10[1] * v1 + T.c10[2] * v2 + T.c10[3] * v3 + T.c10[4] * v4 +
         T.c10[5] * v5;
}
template <class Fetch>
__device__ __forceinline__ double filt_c8(const FTab& T, const Fetch& f, int j) {
  const double v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
  const double v3 = f(j + 3) + f(j - 3), v4 = f(j + 4) + f(j - 4);
  return T.c8[0] * v0 + T.c8[1] * v1 + T.c8[2] * v2 + T.c8[3] * v3 + T.c8[4] * v4;
}
template <class Fetch>
__device__ __forceinline__ double filt_c6(const FTab& T, const Fetch& f, int j) {
  const double v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
  const double v3 = f(j + 3) + f(j - 3);
  return T.c6[0] * v0 + T.c6[1] * v1 + T.c6[2] * v2 + T.c6[3] * v3;
}

// Boundary and end rows of the compact filter (compact_filter_rhs,
// src/filter.F90:176-269).  Out of line: only the first and last chunk of a
// line reach it.  v + base is node 0 of the line, hs the node stride.
static __device__ __noinline__ double filter_special_row(const DScheme& S, const FTab& T, int r,
                                                  const double* v, long long base, long long hs,
                                                  int per) {
  const int dim = S.dim;
  auto f = [&](int node) -> double {
    int nd = node;
    if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
    return v[base + hs * nd];
  };
  const int last = S.first + S.n - 1;
  const int j = S.first + r;
  double d = 0.0;
  if (S.ntype == 4) {
    if (r <= 2) {
      for (int m = 0; m <= 6; ++m) d = d + T.cb[r][m] * f(m);
    } else if (r >= S.n - 3) {
      const int kk = S.n - 1 - r;
      for (int m = 0; m <= 6; ++m) d = d + T.cb[kk][m] * f(last - m);
    } else if (r == 3 || r == S.n - 4) {
      d = filt_c6(T, f, j);
    } else {
      d = filt_c8(T, f, j);
    }
  } else {
    if (r <= 2) {
      for (int m = 0; m <= 10; ++m) d = d + T.ch[r][m] * f(S.first - 2 + m);
    } else {
      const int kk = S.n - 1 - r;
      for (int m = 0; m <= 10; ++m) d = d + T.ch[kk][m] * f(last + 2 - m);
    }
  }
  return d;
}

// Right-hand side of the compact filter (compact_filter_rhs,
// src/filter.F90:156-285) for the rows of chunk c.
template <int CH>
__device__ __forceinline__ void filter_rhs(double (&y)[CH], const DScheme& S, const FTab& T, int c,
                                           const double* v, long long base, long long hs, int per) {
  const int s = c * CH;
  const int dim = S.dim;
  auto f = [&](int node) -> double {
    int nd = node;
    if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
    return v[base + hs * nd];
  };
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    double d = 0.0;
    if (r < S.n) {
      const bool special = S.ntype == 4 ? (r <= 4 || r >= S.n - 5) : (r <= 2 || r >= S.n - 3);
      if (special) d = filter_special_row(S, T, r, v, base, hs, per);
      else d = filt_c10(T, f, S.first + r);
    }
    y[t] = d;
  }
}

// q2fvar (src/fludyna.F90:545-634): conserved -> primitives at one point.
__device__ __forceinline__ void q2fvar_pt(const Phys& ph, double q1, double q2, double q3, double q4,
                                          double q5, double& ro, double& u, double& v, double& w,
                                          double& p, double& T) {
  ro = q1;
  u = q2 / ro;
  v = q3 / ro;
  w = q4 / ro;
  p = (q5 - 0.5 * ro * (u * u + v * v + w * w)) / ph.const6;
  T = p / ro * ph.const2;
}

__device__ __forceinline__ void q2fvar_store(const Geo& g, const Dev& d, const Phys& ph, long long p) {
  const long long nh = g.nh;
  double ro, u, v, w, pp, T;
  q2fvar_pt(ph, d.q[p], d.q[p + nh], d.q[p + 2 * nh], d.q[p + 3 * nh], d.q[p + 4 * nh], ro, u, v, w,
            pp, T);
  d.pr[p] = ro;
  d.pr[p + nh] = u;
  d.pr[p + 2 * nh] = v;
  d.pr[p + 3 * nh] = w;
  d.pr[p + 4 * nh] = pp;
  d.pr[p + 5 * nh] = T;
  if (!(ro > 0.0)) atomicOr(d.flag, 1);
}

struct CGFlags {
  int conv, grad, first, last, sigma, stats, qsave;
};

__device__ __forceinline__ void sigma_point(const Geo& g, const Dev& d, const Phys& ph, long long z,
                                            long long h) {
  const long long n0 = g.n0, nh = g.nh;
  const double* G = d.grad + z;
  const double T = d.pr[h + 5 * nh];
  // miucal (src/fludyna.F90:791-820) / reynolds
  const double miu = T * sqrt(T) * ph.tempconst1 / (T + ph.tempconst) / ph.reynolds;
  const double s11 = G[0];
  const double s12 = 0.5 * (G[3 * n0] + G[1 * n0]);
  const double s13 = 0.5 * (G[6 * n0] + G[2 * n0]);
  const double s22 = G[4 * n0];
  const double s23 = 0.5 * (G[7 * n0] + G[5 * n0]);
  const double s33 = G[8 * n0];
  const double skk = NUM1D3 * (s11 + s22 + s33);
  const double miu2 = 2.0 * miu;
  const double hcc = (miu / ph.prandtl) / ph.const5;
  const double S1 = miu2 * (s11 - skk), S2 = miu2 * s12, S3 = miu2 * s13;
  const double S4 = miu2 * (s22 - skk), S5 = miu2 * s23, S6 = miu2 * (s33 - skk);
  const double u = d.pr[h + nh], v = d.pr[h + 2 * nh], w = d.pr[h + 3 * nh];
  double* Sg = d.sig + z;
  Sg[0] = S1; Sg[n0] = S2; Sg[2 * n0] = S3; Sg[3 * n0] = S4; Sg[4 * n0] = S5; Sg[5 * n0] = S6;
  double* Q = d.qf + z;
  Q[0] = hcc * G[9 * n0] + S1 * u + S2 * v + S3 * w;
  Q[n0] = hcc * G[10 * n0] + S2 * u + S4 * v + S5 * w;
  Q[2 * n0] = hcc * G[11 * n0] + S3 * u + S5 * v + S6 * w;
}

struct VFlags {
  int last;  // fuse the RK3 update of all five variables
  int q2f;   // and recover the primitives (main ordering)
};

__device__ __forceinline__ double rk_combine(const Phys& ph, double qs, double qv, double J,
                                             double rhs) {
  if (ph.mini) return ph.rk1 * qs + ph.rk2 * qv + ph.rk3 * rhs * ph.dt;
  const double v = ph.rk1 * qs + ph.rk2 * qv * J + ph.rk3 * rhs * ph.dt;
  return v / J;
}

}  // namespace astr
