// Tile-staged line sweeps: the filter, convective + gradient and viscous
// sweeps of the main solver ordering with diagonal metrics, for lines of up
// to 17 rows per chunk (32 x 17 = 544 system rows).
//
// A block holds NL lines x 32 chunks.  For each task (one variable of the
// sweep) the block stages the task's input along its NL lines into a
// shared-memory tile with coalesced copies: consecutive threads take
// consecutive i for y and z lines and consecutive nodes of one line for x
// lines.  The chunked Thomas solve (astr_kernels.cuh) then reads each
// chunk's window from the tile.  The copies of task t+1 into the other tile
// are issued (cp.async, no registers held) before task t's right-hand side
// and solve, so the next task's data is in flight while the current one
// computes; the values the outputs combine with (the residual accumulated
// so far, the FP64 master) are read into registers before the solve for the
// same reason.
//
// Convective fluxes share three factors staged once per sweep:
//   A = J dxi u_d,  B = J dxi p,  C = p A,
// so the flux of variable n is q_n A (+ B for the momentum along the sweep,
// + C for the energy): one multiply-add per node (convrsdcal6,
// src/solver.F90:2200-2206).  The viscous fluxes are sigma (J dxi), with
// J dxi staged once (src/solver.F90:2623-2846).
//
// Chunks whose rows all carry the steady Thomas factors take every
// coefficient from kernel parameters (UCo: constant-bank operands of the
// unrolled row loops); the others read the coefficient arrays, padded to
// 32 x CH rows with rows that decouple (a = c = 0, zero right-hand side), so
// no row needs a bounds test in the recurrences.
//
// Outputs along y and z leave from registers (a warp writes NL consecutive
// i per row); along x they pass through the tile so that a warp writes
// consecutive nodes of its line.
#pragma once

#include "launch2.cuh"

namespace astr {

// Resident blocks per SM asked of the compiler (the lines per block,
// v2_nl, are in launch2.cuh).
#ifndef ASTR_V2_MINB
#define ASTR_V2_MINB 2
#endif
template <typename T>
constexpr int v2_nt() { return 32 * v2_nl<T>(); }
// The filter and viscous sweeps hold fewer tiles and fit more blocks per SM;
// timed on the 512^3 TGV (FP32 storage): the filter 8.6 (two blocks), 7.7
// (three), 7.2 ms (four) per launch; the viscous sweep 3.7, 3.4, 4.2 ms.
#ifndef ASTR_V2_MINB_F
#define ASTR_V2_MINB_F 4
#endif
#ifndef ASTR_V2_MINB_V
#define ASTR_V2_MINB_V 3
#endif
// Convective + gradient sweeps: one task tile instead of two (the next
// task's copies then start after the current task's outputs).
#ifndef ASTR_V2_CG_SINGLE
#define ASTR_V2_CG_SINGLE 0
#endif
constexpr bool V2_CG_SINGLE = ASTR_V2_CG_SINGLE != 0;
constexpr int V2_MINB = ASTR_V2_MINB;      // convective + gradient sweeps
constexpr int V2_MINB_F = ASTR_V2_MINB_F;  // filter
constexpr int V2_MINB_V = ASTR_V2_MINB_V;  // viscous sweeps
static_assert(ASTR_V2_NL32 == 4 || ASTR_V2_NL32 == 8 || ASTR_V2_NL32 == 16, "FP32 lines per block");
static_assert(ASTR_V2_NL64 == 4 || ASTR_V2_NL64 == 8 || ASTR_V2_NL64 == 16, "FP64 lines per block");

// Uniform-chunk constants of one scheme at chunk length CH.
template <typename T, int CH>
struct UCo {
  T a1, a3;
  T K[6];    // derivative: 7/9 ac2, 1/36 ac2; filter: the six folded c10i weights
  T KD[5];   // filter, increment form
  T gp[CH];  // forward carry weight of row t of a uniform chunk (G)
  T hp[CH];  // backward carry weight (H)
};

// Word of (line, row) in a tile: x tiles are line-major with pitch P (P =
// 32/NL mod 32 words in FP32, 16/NL mod 16 in FP64: a warp's (or, for 8-byte
// words, a half-warp's) NL lines x chunks then hit distinct banks, the chunk
// length being odd); y/z tiles are row-major over the NL lines.
template <int DIR, int NL>
__device__ __forceinline__ int tw(int line, int row, int P) {
  return DIR == 0 ? line * P + row : row * NL + line;
}

// The rows of a tile staged by this thread: y/z: line = threadIdx.x, rows
// threadIdx.y + 32 k; x: line = warp, rows lane + 32 k.
template <int DIR, int NL>
struct StageMap {
  int line, row0;
  __device__ __forceinline__ StageMap() {
    const int tid = threadIdx.x + NL * threadIdx.y;
    if (DIR == 0) { line = tid >> 5; row0 = tid & 31; }
    else { line = threadIdx.x; row0 = threadIdx.y; }
  }
};

// The block shape every tiled kernel assumes, NL lines x 32 chunks
// (v2_block on the host): a launch of any other shape returns at once
// instead of indexing its tiles out of range.
template <typename T>
__device__ __forceinline__ bool v2_shape_ok() {
  return blockDim.x == (unsigned)v2_nl<T>() && blockDim.y == 32 && blockDim.z == 1;
}

// Asynchronous global -> shared copy of one element (cp.async, completed
// by cp_async_wait_all); an invalid element is written as zero without a
// read (source size 0).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  const int nb = valid ? (int)sizeof(T) : 0;
  if (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(src), "r"(nb) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(src), "r"(nb) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// The block a sweep body works on: the launch's own block, or an item of
// a batch work list (nz > 1: the variables of a line spread over z blocks).
struct VB {
  int x, y, z, nz;
};
__device__ __forceinline__ VB vb_grid() {
  return VB{(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.z};
}

// Halo-array offset of node 0 of line l of block vb (or of the last line
// when l is past the end), and the interior-array offset of that node.
template <int DIR, int NL>
__device__ __forceinline__ bool v2_line(const Geo& g, const VB& vb, int l, int& hb, int& zb, int& la,
                                        int& lb) {
  const int amax = DIR == 0 ? g.jm : g.im;
  int a = vb.x * NL + l;
  const bool ok = a <= amax;
  if (!ok) a = amax;
  int i, j, k;
  line_ijk<DIR>(a, vb.y, 0, i, j, k);
  hb = (int)hidx(g, i, j, k);
  zb = (int)zidx(g, i, j, k);
  la = a;
  lb = vb.y;
  return ok;
}

template <int DIR>
__device__ __forceinline__ int v2_hs(const Geo& g) {
  return DIR == 0 ? 1 : (DIR == 1 ? (int)g.NI : (int)(g.NI * g.NJ));
}
template <int DIR>
__device__ __forceinline__ int v2_zs(const Geo& g) {
  return DIR == 0 ? 1 : (DIR == 1 ? (int)g.I : (int)g.IJ);
}

// Affine carry scan across the 32 chunks of each line of the block (as
// scan_block, astr_kernels.cuh), without the closing barrier: the forward
// and backward scans use separate halves of the scan memory, and every
// reuse of a half is separated from its last read by the other scan's
// barriers or the end-of-task barrier.
template <bool FWD, typename T>
__device__ __forceinline__ T scan2(T M, T L, T* sm) {
  T* sM = sm;
  T* sL = sm + 32 * SM_PITCH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  sM[ty * SM_PITCH + tx] = M;
  sL[ty * SM_PITCH + tx] = L;
  __syncthreads();
  const int nl = blockDim.x;
  const int tid = tx + nl * ty;
  const int w = tid >> 5, lane = tid & 31;
  if (w < nl) {
    T m = sM[lane * SM_PITCH + w];
    T l = sL[lane * SM_PITCH + w];
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
    sL[lane * SM_PITCH + w] = l;
  }
  __syncthreads();
  if (FWD) return ty == 0 ? T(0) : sL[(ty - 1) * SM_PITCH + tx];
  return ty == 31 ? T(0) : sL[(ty + 1) * SM_PITCH + tx];
}
constexpr int V2_SCAN_WORDS = 4 * 32 * SM_PITCH;  // two scans x (M, L)

// Chunked Thomas solve of chunk c (see astr_kernels.cuh), coefficients from
// U in uniform chunks and from the padded arrays elsewhere.
template <int CH, typename T>
__device__ __forceinline__ void solve2(T (&y)[CH], const DScheme<T>& S, const UCo<T, CH>& U, int c,
                                       T* sm, bool uni) {
  const int s = c * CH;
  T M;
  if (uni) {
#pragma unroll
    for (int t = 1; t < CH; ++t) y[t] = fma(-U.a3, y[t - 1], y[t]);
    M = U.gp[CH - 1];
  } else {
#pragma unroll
    for (int t = 1; t < CH; ++t) y[t] = y[t] - y[t - 1] * __ldg(S.ac3 + s + t);
    M = __ldg(S.G + s + CH - 1);
  }
  const T Yp = scan2<true>(M, y[CH - 1], sm);
  if (uni) {
#pragma unroll
    for (int t = 0; t < CH; ++t) y[t] = fma(U.gp[t], Yp, y[t]);
  } else if (c > 0) {
#pragma unroll
    for (int t = 0; t < CH; ++t) y[t] = fma(__ldg(S.G + s + t), Yp, y[t]);
  }
  T Mb;
  if (uni) {
#pragma unroll
    for (int t = CH - 2; t >= 0; --t) y[t] = fma(-U.a1, y[t + 1], y[t]);
    Mb = U.hp[0];
  } else {
#pragma unroll
    for (int t = CH - 2; t >= 0; --t) y[t] = y[t] - __ldg(S.ac1 + s + t) * y[t + 1];
    Mb = __ldg(S.H + s);
  }
  const T Xn = scan2<false>(Mb, y[0], sm + 2 * 32 * SM_PITCH);
  if (uni) {
#pragma unroll
    for (int t = 0; t < CH; ++t) y[t] = fma(U.hp[t], Xn, y[t]);
  } else {
#pragma unroll
    for (int t = 0; t < CH; ++t) y[t] = fma(__ldg(S.H + s + t), Xn, y[t]);
  }
}

// Right-hand side of the compact first derivative (compact_fd_rhs,
// src/derivative.F90:210-306) for the rows of chunk c, scaled by ac2, from
// a tile whose row rr holds node first - 3 + rr.
template <int DIR, int NL, int CH, typename T>
__device__ __forceinline__ void rhs_deriv2(T (&y)[CH], const T* tile, int P, int line,
                                           const DScheme<T>& S, const UCo<T, CH>& U, int c,
                                           bool uni) {
  constexpr int R = 3;
  T w[CH + 2 * R];
#pragma unroll
  for (int t = 0; t < CH + 2 * R; ++t) w[t] = tile[tw<DIR, NL>(line, c * CH + t, P)];
  if (uni) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const T* W = w + t + R;
      y[t] = U.K[0] * (W[1] - W[-1]) + U.K[1] * (W[2] - W[-2]);
    }
    return;
  }
  const int s = c * CH;
  const T* K7 = S.K;
  const T* K36 = S.K + S.ks;
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    const T* W = w + t + R;
    T dv = T(0);
    if (r < S.n) {
      const bool special = S.ntype == 4 ? (r <= 1 || r >= S.n - 2) : (r == 0 || r == S.n - 1);
      if (!special) {
        dv = __ldg(K7 + r) * (W[1] - W[-1]) + __ldg(K36 + r) * (W[2] - W[-2]);
      } else {
        if (S.ntype == 4) {
          if (r == 0) dv = T(-2.5) * W[0] + T(2.0) * W[1] + T(0.5) * W[2];
          else if (r == S.n - 1) dv = T(2.5) * W[0] - T(2.0) * W[-1] - T(0.5) * W[-2];
          else dv = T(0.75) * (W[1] - W[-1]);
        } else {
          dv = T(0.75) * (W[1] - W[-1]) - T(0.15) * (W[2] - W[-2]) + T(1.0 / 60.0) * (W[3] - W[-3]);
        }
        if (r > 0) dv = dv * __ldg(S.ac2 + r);
      }
    }
    y[t] = dv;
  }
}

// Boundary and end rows of the compact filter (compact_filter_rhs,
// src/filter.F90:176-269), scaled by ac2, read from the tile (row rr holds
// node first - 5 + rr, periodic nodes already wrapped).  FP64: the
// reference's row; FP32 storage: the increment form's row, evaluated on
// f - f(j) with the A row's off-diagonal terms subtracted (every filter row
// preserves constants, so the diagonal term drops out).
template <int DIR, int NL, typename T>
__device__ __noinline__ T filter_special_row2(const DScheme<T>& S, const FTab<T>& Tb, int r,
                                              const T* tile, int P, int line) {
  constexpr bool delta = sizeof(T) == 4;
  const int j = S.first + r;
  const T shift = delta ? tile[tw<DIR, NL>(line, r + 5, P)] : T(0);
  auto f = [&](int node) -> T { return tile[tw<DIR, NL>(line, node - S.first + 5, P)] - shift; };
  const int last = S.first + S.n - 1;
  T dv = T(0);
  if (S.ntype == 4) {
    if (r <= 2) {
      for (int m = 0; m <= 6; ++m) dv = dv + Tb.cb[r][m] * f(m);
    } else if (r >= S.n - 3) {
      const int kk = S.n - 1 - r;
      for (int m = 0; m <= 6; ++m) dv = dv + Tb.cb[kk][m] * f(last - m);
    } else if (r == 3 || r == S.n - 4) {
      const T v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
      const T v3 = f(j + 3) + f(j - 3);
      dv = Tb.c6[0] * v0 + Tb.c6[1] * v1 + Tb.c6[2] * v2 + Tb.c6[3] * v3;
    } else {
      const T v0 = f(j) + f(j), v1 = f(j + 1) + f(j - 1), v2 = f(j + 2) + f(j - 2);
      const T v3 = f(j + 3) + f(j - 3), v4 = f(j + 4) + f(j - 4);
      dv = Tb.c8[0] * v0 + Tb.c8[1] * v1 + Tb.c8[2] * v2 + Tb.c8[3] * v3 + Tb.c8[4] * v4;
    }
  } else {
    if (r <= 2) {
      for (int m = 0; m <= 10; ++m) dv = dv + Tb.ch[r][m] * f(S.first - 2 + m);
    } else {
      const int kk = S.n - 1 - r;
      for (int m = 0; m <= 10; ++m) dv = dv + Tb.ch[kk][m] * f(last + 2 - m);
    }
  }
  const T sc = r > 0 ? __ldg(S.ac2 + r) : T(1);
  if (!delta) return dv * sc;
  const T a = __ldg(S.A + r);
  T af = T(0);
  if (r > 0) af = af + a * f(j - 1);
  if (r < S.n - 1) af = af + a * f(j + 1);
  return dv * sc - af * sc;
}

// Right-hand side of the compact filter for chunk c: FP64 the reference's
// form A^{-1} B f; FP32 the increment form A^{-1} (B - A) f (second
// differences, see filter_rhs_delta).
template <int DIR, int NL, int CH, typename T>
__device__ __forceinline__ void rhs_filter2(T (&y)[CH], const T* tile, int P, int line,
                                            const DScheme<T>& S, const UCo<T, CH>& U,
                                            const FTab<T>& Tb, int c, bool uni) {
  constexpr int R = 5;
  constexpr bool delta = sizeof(T) == 4;
  T w[CH + 2 * R];
#pragma unroll
  for (int t = 0; t < CH + 2 * R; ++t) w[t] = tile[tw<DIR, NL>(line, c * CH + t, P)];
  if (uni) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const T* W = w + t + R;
      if (delta) {
        const T f0 = W[0];
        y[t] = U.KD[0] * ((W[1] - f0) + (W[-1] - f0)) + U.KD[1] * ((W[2] - f0) + (W[-2] - f0)) +
               U.KD[2] * ((W[3] - f0) + (W[-3] - f0)) + U.KD[3] * ((W[4] - f0) + (W[-4] - f0)) +
               U.KD[4] * ((W[5] - f0) + (W[-5] - f0));
      } else {
        y[t] = U.K[0] * W[0] + U.K[1] * (W[1] + W[-1]) + U.K[2] * (W[2] + W[-2]) +
               U.K[3] * (W[3] + W[-3]) + U.K[4] * (W[4] + W[-4]) + U.K[5] * (W[5] + W[-5]);
      }
    }
    return;
  }
  const int s = c * CH, n = S.n, ks = S.ks;
#pragma unroll
  for (int t = 0; t < CH; ++t) {
    const int r = s + t;
    const T* W = w + t + R;
    T dv = T(0);
    if (r < n) {
      const bool special = S.ntype == 4 ? (r <= 4 || r >= n - 5) : (r <= 2 || r >= n - 3);
      if (special) {
        dv = filter_special_row2<DIR, NL>(S, Tb, r, tile, P, line);
      } else if (delta) {
        const T f0 = W[0];
        const T* KD = S.KD;
        dv = __ldg(KD + r) * ((W[1] - f0) + (W[-1] - f0)) +
             __ldg(KD + ks + r) * ((W[2] - f0) + (W[-2] - f0)) +
             __ldg(KD + 2 * ks + r) * ((W[3] - f0) + (W[-3] - f0)) +
             __ldg(KD + 3 * ks + r) * ((W[4] - f0) + (W[-4] - f0)) +
             __ldg(KD + 4 * ks + r) * ((W[5] - f0) + (W[-5] - f0));
      } else {
        const T* FK = S.K;
        dv = __ldg(FK + r) * W[0] + __ldg(FK + ks + r) * (W[1] + W[-1]) +
             __ldg(FK + 2 * ks + r) * (W[2] + W[-2]) + __ldg(FK + 3 * ks + r) * (W[3] + W[-3]) +
             __ldg(FK + 4 * ks + r) * (W[4] + W[-4]) + __ldg(FK + 5 * ks + r) * (W[5] + W[-5]);
      }
    }
    y[t] = dv;
  }
}

// Shared memory of a tiled kernel with ntile tiles.
template <typename T, int DIR>
inline size_t v2_smem_bytes(int CH, int R, int P, int ntile) {
  const int NL = v2_nl<T>();
  const int nrt = 32 * CH + 2 * R;
  const size_t tw_ = DIR == 0 ? (size_t)NL * P : (size_t)nrt * NL;
  return (ntile * tw_ + V2_SCAN_WORDS) * sizeof(T);
}

// Pitch of an x tile: at least nrt words, 32/NL mod 32 (FP32) or 16/NL mod
// 16 (FP64).
template <typename T>
__host__ __device__ inline int v2_pitch(int CH, int R) {
  const int nrt = 32 * CH + 2 * R;
  const int m = sizeof(T) == 4 ? 32 : 16;
  const int want = (m / v2_nl<T>()) % m;
  int p = nrt;
  while (p % m != want) ++p;
  return p;
}

template <typename T, int CH>
inline UCo<T, CH> make_uco(const V2Args<T>& a) {
  UCo<T, CH> u;
  u.a1 = (T)a.a1; u.a3 = (T)a.a3;
  for (int m = 0; m < 6; ++m) u.K[m] = (T)a.K[m];
  for (int m = 0; m < 5; ++m) u.KD[m] = (T)a.KD[m];
  for (int t = 0; t < CH; ++t) { u.gp[t] = (T)a.gp[t]; u.hp[t] = (T)a.hp[t]; }
  return u;
}

// ---------------------------------------------------------------------------
// filterq (src/comsolver.F90:514-632): one direction, the five conserved
// variables in place.
// ---------------------------------------------------------------------------
template <typename T, int DIR, int CH>
__device__ __forceinline__ void filter_body(const Geo& g, const DevT<T>& d, const DScheme<T>& S,
                                            const UCo<T, CH>& U, const FTab<T>& Tb, int P, const VB vb,
                                            unsigned char* v2_smem) {
  constexpr int NL = v2_nl<T>(), R = 5, NRT = 32 * CH + 2 * R, E = (NRT + 31) / 32;
  constexpr bool delta = sizeof(T) == 4;
  const int TWd = DIR == 0 ? NL * P : NRT * NL;
  T* buf0 = reinterpret_cast<T*>(v2_smem);
  T* scan = buf0 + 2 * TWd;
  const int ol = threadIdx.x, c = threadIdx.y;
  const bool uni = c >= S.ulo && c <= S.uhi;
  const int hs = v2_hs<DIR>(g), zs = v2_zs<DIR>(g);
  const int dim = S.dim, first = S.first;
  const bool per = g.per[DIR] != 0;
  const int nh = (int)g.nh;
  StageMap<DIR, NL> sm_;
  int shb, szb, sa, sb;
  const bool sok = v2_line<DIR, NL>(g, vb, sm_.line, shb, szb, sa, sb);
  int ohb, ozb, oa, ob;
  const bool ook = v2_line<DIR, NL>(g, vb, ol, ohb, ozb, oa, ob);
  (void)sa; (void)sb; (void)oa; (void)ob;

  int t0 = 0, t1 = 5;
  if (vb.nz > 1) { t0 = vb.z; t1 = t0 + 1; }
  // task t's input (q, periodic nodes wrapped) into tile bf, asynchronously
  auto issue = [&](int t, T* bf) {
    const T* v = d.q + (size_t)t * nh + shb;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int row = sm_.row0 + 32 * k;
      int nd = first - R + row;
      if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
      const bool ok = sok && nd >= -HMD && nd <= dim + HMD;
      if (row < NRT) cp_async_elem(bf + tw<DIR, NL>(sm_.line, row, P), ok ? v + hs * nd : v, ok);
    }
    cp_async_commit();
  };
  const int lo_node = S.ntype == 4 ? 1 : 0, hi_node = S.ntype == 4 ? dim - 1 : dim;
  const int lane = (threadIdx.x + NL * threadIdx.y) & 31;
  // output slot k of this thread: y/z: row c*CH + k of its own line; x:
  // node lo_node + lane + 32 k of its staging line (after the tile pass)
  auto slot_node = [&](int k) -> int {
    if (DIR != 0) {
      const int r = c * CH + k, node = first + r;
      return (ook && r < S.n && node >= lo_node && node <= hi_node) ? node : -1;
    }
    const int node = lo_node + lane + 32 * k;
    return (sok && node <= hi_node) ? node : -1;
  };
  const int obh = DIR != 0 ? ohb : shb, obz = DIR != 0 ? ozb : szb;

  issue(t0, buf0);
  cp_async_wait_all();
  __syncthreads();
  int cur = 0;
#pragma unroll 1
  for (int t = t0; t < t1; ++t) {
    const bool more = t + 1 < t1;
    if (more) issue(t + 1, buf0 + (cur ^ 1) * TWd);
    T* bc = buf0 + cur * TWd;
    T y[CH];
    rhs_filter2<DIR, NL, CH>(y, bc, P, ol, S, U, Tb, c, uni);
    // FP32 storage: the FP64 master values the increments go to, read
    // before the solve so that they arrive while it runs
    double am[delta ? CH : 1];
    double* M = d.qm ? d.qm + (size_t)t * g.n0 + obz : nullptr;
    if (delta) {
#pragma unroll
      for (int k = 0; k < CH; ++k) {
        const int node = slot_node(k);
        am[delta ? k : 0] = (node >= 0 && M) ? M[zs * node] : 0.0;
      }
    }
    solve2<CH>(y, S, U, c, scan, uni);
    if (DIR == 0) {
      // x: through the tile, so that a warp writes consecutive nodes
#pragma unroll
      for (int k = 0; k < CH; ++k) bc[tw<DIR, NL>(ol, c * CH + k, P)] = y[k];
      __syncthreads();
    }
    T* v = d.q + (size_t)t * nh + obh;
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int node = slot_node(k);
      if (node >= 0) {
        const T val = DIR == 0 ? bc[tw<DIR, NL>(sm_.line, node - first, P)] : y[k];
        if (delta && M) {
          // FP32 storage: master += increment, q = (float) master
          const double nv = am[delta ? k : 0] + (double)val;
          M[zs * node] = nv;
          v[hs * node] = (T)nv;
        } else {
          v[hs * node] = val;
        }
      }
    }
    cp_async_wait_all();
    __syncthreads();
    cur ^= 1;
  }
}

// ---------------------------------------------------------------------------
// convrsdcal6 (src/solver.F90:2173-2341) and gradcal
// (src/comsolver.F90:244-497), one direction, diagonal metrics.
// ---------------------------------------------------------------------------
template <typename T, int DIR, int CH>
__device__ __forceinline__ void convgrad_body(const Geo& g, const DevT<T>& d, const DScheme<T>& S,
                                              const UCo<T, CH>& U, const CGFlags fl, int P, const VB vb,
                                              unsigned char* v2_smem) {
  constexpr int NL = v2_nl<T>(), R = 3, NRT = 32 * CH + 2 * R, E = (NRT + 31) / 32;
  const int TWd = DIR == 0 ? NL * P : NRT * NL;
  T* tA = reinterpret_cast<T*>(v2_smem);
  T* tB = tA + TWd;
  T* tC = tB + TWd;
  T* buf0 = tC + TWd;
  T* scan = buf0 + (V2_CG_SINGLE ? 1 : 2) * TWd;
  const int ol = threadIdx.x, c = threadIdx.y;
  const bool uni = c >= S.ulo && c <= S.uhi;
  const int hs = v2_hs<DIR>(g), zs = v2_zs<DIR>(g);
  const int dim = S.dim, first = S.first;
  const int nh = (int)g.nh;
  const size_t n0 = (size_t)g.n0;
  StageMap<DIR, NL> sm_;
  int shb, szb, sa, sb;
  const bool sok = v2_line<DIR, NL>(g, vb, sm_.line, shb, szb, sa, sb);
  int ohb, ozb, oa, ob;
  const bool ook = v2_line<DIR, NL>(g, vb, ol, ohb, ozb, oa, ob);
  const int lo = g.lo[DIR], hi = g.hi[DIR];
  constexpr int ta = DIR == 0 ? 1 : 0, tb = DIR == 2 ? 1 : 2;
  // convrsdcal6's transverse ranges, for the line a thread writes
  auto cl_of = [&](int a, int b) {
    return a >= g.lo[ta] && a <= g.hi[ta] && b >= g.lo[tb] && b <= g.hi[tb];
  };
  const T* xdd = d.xd + (size_t)DIR * nh;

  const int nconv = fl.conv ? 5 : 0;
  const int ntask = nconv + (fl.grad ? 4 : 0);
  int t0 = 0, t1 = ntask;
  if (vb.nz > 1) {
    t0 = vb.z;
    t1 = t0 + 1;
  }
  if (t0 >= ntask) return;  // whole block

  if (fl.conv && t0 < nconv) {
    // flux factors at every tile row: A = J dxi u_d, B = J dxi p, C = p A
    const T* ud = d.pr + (size_t)(1 + DIR) * nh;
    const T* pp = d.pr + (size_t)4 * nh;
    const T* jj = d.jac;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int row = sm_.row0 + 32 * k;
      const int nd = first - R + row;
      T A = T(0), B = T(0), C = T(0);
      if (sok && (k < E - 1 || row < NRT) && nd >= -HMD && nd <= dim + HMD) {
        const int p = shb + hs * nd;
        const T u = ud[p], pv = pp[p], x = xdd[p], J = jj[p];
        A = J * (x * u);
        B = J * (x * pv);
        C = pv * A;
      }
      if (k < E - 1 || row < NRT) {
        const int w = tw<DIR, NL>(sm_.line, row, P);
        tA[w] = A;
        tB[w] = B;
        tC[w] = C;
      }
    }
  }

  auto src_of = [&](int t) -> const T* {
    if (t < nconv) return d.q + (size_t)t * nh;
    const int n = t - nconv;
    return d.pr + (size_t)(n < 3 ? 1 + n : 5) * nh;
  };
  // task t's input (q_n or a primitive) into tile bf, asynchronously
  auto issue = [&](int t, T* bf) {
    const T* v = src_of(t) + shb;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int row = sm_.row0 + 32 * k;
      const int nd = first - R + row;
      const bool ok = sok && nd >= -HMD && nd <= dim + HMD;
      if (k < E - 1 || row < NRT) cp_async_elem(bf + tw<DIR, NL>(sm_.line, row, P), ok ? v + hs * nd : v, ok);
    }
    cp_async_commit();
  };
  // once the copies of task t have landed: the convective flux of variable
  // t from q_t and the staged factors (the thread's own elements)
  auto finish = [&](int t, T* bf) {
    cp_async_wait_all();
    if (t < nconv) {
#pragma unroll
      for (int k = 0; k < E; ++k) {
        const int row = sm_.row0 + 32 * k;
        if (k < E - 1 || row < NRT) {
          const int w = tw<DIR, NL>(sm_.line, row, P);
          const T v = bf[w];
          if (t == 1 + DIR) bf[w] = fma(v, tA[w], tB[w]);
          else if (t == 4) bf[w] = fma(v, tA[w], tC[w]);
          else bf[w] = v * tA[w];
        }
      }
    }
  };
  const int lane = (threadIdx.x + NL * threadIdx.y) & 31;
  auto slot_node = [&](int k) -> int {
    if (DIR != 0) {
      const int r = c * CH + k, node = first + r;
      return (ook && r < S.n && node >= 0 && node <= dim) ? node : -1;
    }
    const int node = lane + 32 * k;
    return (sok && node <= dim) ? node : -1;
  };
  const int obh = DIR != 0 ? ohb : shb, obz = DIR != 0 ? ozb : szb;
  const bool cl = DIR != 0 ? cl_of(oa, ob) : cl_of(sa, sb);

  issue(t0, buf0);
  finish(t0, buf0);
  __syncthreads();
  int cur = 0;
#pragma unroll 1
  for (int t = t0; t < t1; ++t) {
    const bool more = t + 1 < t1;
    if (more && !V2_CG_SINGLE) issue(t + 1, buf0 + (cur ^ 1) * TWd);
    T* bc = buf0 + cur * TWd;
    T y[CH];
    rhs_deriv2<DIR, NL, CH>(y, bc, P, ol, S, U, c, uni);
    // what the outputs combine with, read before the solve: the residual
    // accumulated so far (convective tasks) or the metric (gradients)
    const bool conv = t < nconv;
    const int gn = t - nconv;
    T* dst = conv ? d.qrhs + (size_t)t * n0 + obz
                  : d.grad + (size_t)(gn < 3 ? gn + 3 * DIR : 9 + DIR) * n0 + obz;
    T ar[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int node = slot_node(k);
      ar[k] = T(0);
      if (node >= 0) {
        if (!conv) ar[k] = xdd[obh + hs * node];
        else if (!fl.first) ar[k] = dst[zs * node];
      }
    }
    solve2<CH>(y, S, U, c, scan, uni);
    if (DIR == 0) {
#pragma unroll
      for (int k = 0; k < CH; ++k) bc[tw<DIR, NL>(ol, c * CH + k, P)] = y[k];
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int node = slot_node(k);
      if (node >= 0) {
        const T val = DIR == 0 ? bc[tw<DIR, NL>(sm_.line, node - first, P)] : y[k];
        if (conv) {
          const bool in = cl && node >= lo && node <= hi;
          const T add = in ? val : T(0);
          T v = fl.first ? add : ar[k] + add;
          if (fl.last) v = -v;
          dst[zs * node] = v;
        } else {
          dst[zs * node] = val * ar[k];
        }
      }
    }
    if (V2_CG_SINGLE) {
      if (DIR == 0) __syncthreads();  // the output pass has read the tile
      if (more) {
        issue(t + 1, buf0);
        finish(t + 1, buf0);
      }
    } else {
      if (more) finish(t + 1, buf0 + (cur ^ 1) * TWd);
      cur ^= 1;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// diffrsdcal6 sweeps (src/solver.F90:2619-2852), one direction; the RK3
// update after the last one runs as a point kernel.
// ---------------------------------------------------------------------------
template <typename T, int DIR, int CH>
__device__ __forceinline__ void visc_body(const Geo& g, const DevT<T>& d, const DScheme<T>& S,
                                          const UCo<T, CH>& U, int P, const VB vb,
                                          unsigned char* v2_smem) {
  constexpr int NL = v2_nl<T>(), R = 3, NRT = 32 * CH + 2 * R, E = (NRT + 31) / 32;
  const int TWd = DIR == 0 ? NL * P : NRT * NL;
  T* tF = reinterpret_cast<T*>(v2_smem);
  T* buf0 = tF + TWd;
  T* scan = buf0 + 2 * TWd;
  const int ol = threadIdx.x, c = threadIdx.y;
  const bool uni = c >= S.ulo && c <= S.uhi;
  const int hs = v2_hs<DIR>(g), zs = v2_zs<DIR>(g);
  const int dim = S.dim, first = S.first;
  const bool per = g.per[DIR] != 0;
  const int nh = (int)g.nh;
  const size_t n0 = (size_t)g.n0;
  StageMap<DIR, NL> sm_;
  int shb, szb, sa, sb;
  const bool sok = v2_line<DIR, NL>(g, vb, sm_.line, shb, szb, sa, sb);
  int ohb, ozb, oa, ob;
  const bool ook = v2_line<DIR, NL>(g, vb, ol, ohb, ozb, oa, ob);
  (void)sa; (void)sb; (void)oa; (void)ob; (void)ohb;
  const int lo = g.lo[DIR], hi = g.hi[DIR];

  int t0 = 0, t1 = 4;
  if (vb.nz > 1) { t0 = vb.z; t1 = t0 + 1; }
  {
    // J dxi at every tile row (the flux factor of the four variables)
    const T* xdd = d.xd + (size_t)DIR * nh;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int row = sm_.row0 + 32 * k;
      const int nd = first - R + row;
      T F = T(0);
      if (sok && (k < E - 1 || row < NRT) && nd >= -HMD && nd <= dim + HMD) {
        const int p = shb + hs * nd;
        F = xdd[p] * d.jac[p];
      }
      if (k < E - 1 || row < NRT) tF[tw<DIR, NL>(sm_.line, row, P)] = F;
    }
  }
  constexpr int s0 = DIR == 0 ? 0 : (DIR == 1 ? 1 : 2);
  constexpr int s1 = DIR == 0 ? 1 : (DIR == 1 ? 3 : 4);
  constexpr int s2 = DIR == 0 ? 2 : (DIR == 1 ? 4 : 5);
  // task t's input (a stress component or the heat flux, periodic nodes
  // wrapped) into tile bf, asynchronously
  auto issue = [&](int t, T* bf) {
    const int sc = t == 0 ? s0 : (t == 1 ? s1 : s2);
    const T* v = (t < 3 ? d.sig + (size_t)sc * n0 : d.qf + (size_t)DIR * n0) + szb;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int row = sm_.row0 + 32 * k;
      int nd = first - R + row;
      if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
      const bool ok = sok && nd >= 0 && nd <= dim;
      if (k < E - 1 || row < NRT) cp_async_elem(bf + tw<DIR, NL>(sm_.line, row, P), ok ? v + zs * nd : v, ok);
    }
    cp_async_commit();
  };
  // the flux: the staged input times J dxi (the thread's own elements)
  auto finish = [&](T* bf) {
    cp_async_wait_all();
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int row = sm_.row0 + 32 * k;
      if (k < E - 1 || row < NRT) {
        const int w = tw<DIR, NL>(sm_.line, row, P);
        bf[w] = bf[w] * tF[w];
      }
    }
  };
  const int lane = (threadIdx.x + NL * threadIdx.y) & 31;
  auto slot_node = [&](int k) -> int {
    if (DIR != 0) {
      const int r = c * CH + k, node = first + r;
      return (ook && r < S.n && node >= 0 && node <= dim) ? node : -1;
    }
    const int node = lane + 32 * k;
    return (sok && node <= dim) ? node : -1;
  };
  const int obz = DIR != 0 ? ozb : szb;

  issue(t0, buf0);
  finish(buf0);
  __syncthreads();
  int cur = 0;
#pragma unroll 1
  for (int t = t0; t < t1; ++t) {
    const bool more = t + 1 < t1;
    if (more) issue(t + 1, buf0 + (cur ^ 1) * TWd);
    T* bc = buf0 + cur * TWd;
    T y[CH];
    rhs_deriv2<DIR, NL, CH>(y, bc, P, ol, S, U, c, uni);
    // the residual the fluxes add to, read before the solve
    T* dst = d.qrhs + (size_t)(t + 1) * n0 + obz;
    T ar[CH];
    const int n0c = first + c * CH;
    const bool full = DIR != 0 && ook && n0c >= lo && c * CH + CH - 1 < S.n && n0c + CH - 1 <= hi;
    if (full) {
#pragma unroll
      for (int k = 0; k < CH; ++k) ar[k] = dst[zs * (n0c + k)];
    } else {
#pragma unroll
      for (int k = 0; k < CH; ++k) {
        const int node = slot_node(k);
        ar[k] = node >= 0 ? dst[zs * node] : T(0);
      }
    }
    solve2<CH>(y, S, U, c, scan, uni);
    if (DIR == 0) {
#pragma unroll
      for (int k = 0; k < CH; ++k) bc[tw<DIR, NL>(ol, c * CH + k, P)] = y[k];
      __syncthreads();
    }
    if (full) {
#pragma unroll
      for (int k = 0; k < CH; ++k) dst[zs * (n0c + k)] = ar[k] + y[k];
    } else {
#pragma unroll
      for (int k = 0; k < CH; ++k) {
        const int node = slot_node(k);
        if (node >= 0) {
          const T val = DIR == 0 ? bc[tw<DIR, NL>(sm_.line, node - first, P)] : y[k];
          const bool in = node >= lo && node <= hi;
          dst[zs * node] = ar[k] + (in ? val : T(0));
        }
      }
    }
    if (more) finish(buf0 + (cur ^ 1) * TWd);
    __syncthreads();
    cur ^= 1;
  }
}

// Copy of a descriptor into shared memory by the whole block (the bodies
// then read its fields from there, as the single-case kernels read theirs
// from the parameter bank, instead of holding them in registers).
template <typename X>
__device__ __forceinline__ void smem_copy(X* dst, const X* src) {
  static_assert(sizeof(X) % 4 == 0, "descriptor of whole words");
  const int nt = blockDim.x * blockDim.y, tid = threadIdx.x + blockDim.x * threadIdx.y;
  for (int i = tid; i < (int)(sizeof(X) / 4); i += nt) ((int*)dst)[i] = ((const int*)src)[i];
}

// ---------------------------------------------------------------------------
// Single-case kernels: the bodies on the launch's own blocks
// ---------------------------------------------------------------------------
// The filter's descriptors go through shared memory (thread 0 copies them
// from the parameter bank): read from there, its body holds fewer of their
// fields in registers and stops spilling at CH = 17 (ptxas).  The other
// sweeps spill less reading their descriptors from the parameter bank.
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(v2_nt<T>(), sizeof(T) == 4 ? V2_MINB_F : 2)
k2_filter(Geo g, DevT<T> d, DScheme<T> S, UCo<T, CH> U, FTab<T> Tb, int P) {
  extern __shared__ __align__(16) unsigned char v2_smem[];
  if (!v2_shape_ok<T>()) return;
  __shared__ Geo sg;
  __shared__ DevT<T> sd;
  __shared__ DScheme<T> sS;
  __shared__ FTab<T> sT;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    sg = g;
    sd = d;
    sS = S;
    sT = Tb;
  }
  __syncthreads();
  filter_body<T, DIR, CH>(sg, sd, sS, U, sT, P, vb_grid(), v2_smem);
}
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(v2_nt<T>(), V2_MINB)
k2_convgrad(Geo g, DevT<T> d, DScheme<T> S, UCo<T, CH> U, CGFlags fl, int P) {
  extern __shared__ __align__(16) unsigned char v2_smem[];
  if (!v2_shape_ok<T>()) return;
  convgrad_body<T, DIR, CH>(g, d, S, U, fl, P, vb_grid(), v2_smem);
}
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(v2_nt<T>(), sizeof(T) == 4 ? V2_MINB_V : 2)
k2_visc(Geo g, DevT<T> d, DScheme<T> S, UCo<T, CH> U, int P) {
  extern __shared__ __align__(16) unsigned char v2_smem[];
  if (!v2_shape_ok<T>()) return;
  visc_body<T, DIR, CH>(g, d, S, U, P, vb_grid(), v2_smem);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <int DIR>
inline dim3 v2_grid(const Geo& g, int NL, int nz) {
  int gx, gy;
  v2_blocks(g, DIR, NL, gx, gy);
  return dim3((unsigned)gx, (unsigned)gy, nz);
}

// Raise a kernel's dynamic shared-memory limit.  Each launcher calls it once
// per kernel instantiation (a function-local static: the size is fixed by
// the template arguments), never per launch: the call is not a stream
// operation, and made per launch it kept batches on separate streams from
// running concurrently.
template <typename T>
inline dim3 v2_block() {
  return dim3(v2_nl<T>(), 32);
}

template <class K>
inline cudaError_t v2_allow_smem(K kern, size_t bytes) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
#define ASTR_V2_CH_SWITCH(CHV, EXPR)                        \
  switch (CHV) {                                            \
    case 3: { constexpr int CHC = 3; EXPR; } break;         \
    case 5: { constexpr int CHC = 5; EXPR; } break;         \
    case 9: { constexpr int CHC = 9; EXPR; } break;         \
    case 17: { constexpr int CHC = 17; EXPR; } break;       \
    default: return cudaErrorInvalidValue;                  \
  }

template <typename T, int DIR, int CHC>
cudaError_t launch2_filter_ch(const V2Args<T>& a, cudaStream_t st, int vsplit) {
  const int P = v2_pitch<T>(CHC, 5);
  const size_t smem = v2_smem_bytes<T, DIR>(CHC, 5, P, 2);
  static const cudaError_t e = v2_allow_smem(k2_filter<T, DIR, CHC>, smem);
  if (e != cudaSuccess) return e;
  const dim3 gr = v2_grid<DIR>(a.g, v2_nl<T>(), vsplit ? 5 : 1);
  k2_filter<T, DIR, CHC><<<gr, v2_block<T>(), smem, st>>>(a.g, a.d, a.S, make_uco<T, CHC>(a),
                                                                  a.Tb, P);
  return cudaGetLastError();
}
template <typename T, int DIR, int CHC>
cudaError_t launch2_convgrad_ch(const V2Args<T>& a, cudaStream_t st, CGFlags f, int vsplit) {
  const int P = v2_pitch<T>(CHC, 3);
  const size_t smem = v2_smem_bytes<T, DIR>(CHC, 3, P, V2_CG_SINGLE ? 4 : 5);
  static const cudaError_t e = v2_allow_smem(k2_convgrad<T, DIR, CHC>, smem);
  if (e != cudaSuccess) return e;
  const int ntask = (f.conv ? 5 : 0) + (f.grad ? 4 : 0);
  const dim3 gr = v2_grid<DIR>(a.g, v2_nl<T>(), vsplit && ntask > 1 ? ntask : 1);
  k2_convgrad<T, DIR, CHC><<<gr, v2_block<T>(), smem, st>>>(a.g, a.d, a.S,
                                                                    make_uco<T, CHC>(a), f, P);
  return cudaGetLastError();
}
template <typename T, int DIR, int CHC>
cudaError_t launch2_visc_ch(const V2Args<T>& a, cudaStream_t st, int vsplit) {
  const int P = v2_pitch<T>(CHC, 3);
  const size_t smem = v2_smem_bytes<T, DIR>(CHC, 3, P, 3);
  static const cudaError_t e = v2_allow_smem(k2_visc<T, DIR, CHC>, smem);
  if (e != cudaSuccess) return e;
  const dim3 gr = v2_grid<DIR>(a.g, v2_nl<T>(), vsplit ? 4 : 1);
  k2_visc<T, DIR, CHC><<<gr, v2_block<T>(), smem, st>>>(a.g, a.d, a.S, make_uco<T, CHC>(a), P);
  return cudaGetLastError();
}

template <typename T, int DIR>
cudaError_t launch2_filter(const V2Args<T>& a, cudaStream_t st, int CH, int vsplit) {
  ASTR_V2_CH_SWITCH(CH, return (launch2_filter_ch<T, DIR, CHC>(a, st, vsplit)));
  return cudaSuccess;
}
template <typename T, int DIR>
cudaError_t launch2_convgrad(const V2Args<T>& a, cudaStream_t st, int CH, CGFlags f, int vsplit) {
  ASTR_V2_CH_SWITCH(CH, return (launch2_convgrad_ch<T, DIR, CHC>(a, st, f, vsplit)));
  return cudaSuccess;
}
template <typename T, int DIR>
cudaError_t launch2_visc(const V2Args<T>& a, cudaStream_t st, int CH, int vsplit) {
  ASTR_V2_CH_SWITCH(CH, return (launch2_visc_ch<T, DIR, CHC>(a, st, vsplit)));
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Batches: persistent kernels that take (case, block) items of many cases
// from a work list, every case with its own descriptor, so one launch runs a
// sweep of all the cases of a batch; the bodies are the single-case ones.
// The cases of one launch share the chunk length and the uniform-chunk
// constants (they depend on the scheme, not on the grid), which stay kernel
// parameters as in the single-case kernels.  Each item first reads the
// batch's status word (set by the step gates).
// ---------------------------------------------------------------------------
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(v2_nt<T>(), sizeof(T) == 4 ? V2_MINB_F : 2)
kb_filter(const BCase<T>* cases, const int4* items, int nitems, UCo<T, CH> U, BatchCtl ctl) {
  extern __shared__ __align__(16) unsigned char v2_smem[];
  if (!v2_shape_ok<T>()) return;
  __shared__ int stop;
  __shared__ Geo sg;
  __shared__ DevT<T> sd;
  __shared__ DScheme<T> sS;
  __shared__ FTab<T> sT;
  const int P = v2_pitch<T>(CH, 5);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];
    const BCase<T>* C = cases + w.x;
    if (threadIdx.x == 0 && threadIdx.y == 0) stop = batch_stopped(ctl);
    smem_copy(&sg, &C->g);
    smem_copy(&sd, &C->d);
    smem_copy(&sS, &C->Sf[DIR]);
    smem_copy(&sT, &C->Tb);
    __syncthreads();
    if (stop) break;
    filter_body<T, DIR, CH>(sg, sd, sS, U, sT, P, VB{w.y, w.z, w.w, C->vsplit ? 5 : 1}, v2_smem);
    __syncthreads();
  }
}
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(v2_nt<T>(), V2_MINB)
kb_convgrad(const BCase<T>* cases, const int4* items, int nitems, UCo<T, CH> U, BatchCtl ctl) {
  extern __shared__ __align__(16) unsigned char v2_smem[];
  if (!v2_shape_ok<T>()) return;
  __shared__ int stop;
  __shared__ Geo sg;
  __shared__ DevT<T> sd;
  __shared__ DScheme<T> sS;
  const int P = v2_pitch<T>(CH, 3);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];
    const BCase<T>* C = cases + w.x;
    if (threadIdx.x == 0 && threadIdx.y == 0) stop = batch_stopped(ctl);
    smem_copy(&sg, &C->g);
    smem_copy(&sd, &C->d);
    smem_copy(&sS, &C->Sd[DIR]);
    __syncthreads();
    if (stop) break;
    CGFlags f{};
    f.conv = 1;
    f.grad = 1;
    f.first = DIR == 0;
    f.last = DIR == sg.ndims - 1;
    convgrad_body<T, DIR, CH>(sg, sd, sS, U, f, P, VB{w.y, w.z, w.w, C->vsplit ? 9 : 1}, v2_smem);
    __syncthreads();
  }
}
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(v2_nt<T>(), sizeof(T) == 4 ? V2_MINB_V : 2)
kb_visc(const BCase<T>* cases, const int4* items, int nitems, UCo<T, CH> U, BatchCtl ctl) {
  extern __shared__ __align__(16) unsigned char v2_smem[];
  if (!v2_shape_ok<T>()) return;
  __shared__ int stop;
  __shared__ Geo sg;
  __shared__ DevT<T> sd;
  __shared__ DScheme<T> sS;
  const int P = v2_pitch<T>(CH, 3);
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];
    const BCase<T>* C = cases + w.x;
    if (threadIdx.x == 0 && threadIdx.y == 0) stop = batch_stopped(ctl);
    smem_copy(&sg, &C->g);
    smem_copy(&sd, &C->d);
    smem_copy(&sS, &C->Sd[DIR]);
    __syncthreads();
    if (stop) break;
    visc_body<T, DIR, CH>(sg, sd, sS, U, P, VB{w.y, w.z, w.w, C->vsplit ? 4 : 1}, v2_smem);
    __syncthreads();
  }
}

// kind: 0 filter, 1 convective + gradient, 2 viscous; a: the launch's
// uniform-chunk constants (its other fields are not used)
template <typename T, int DIR, int CHC>
cudaError_t launchb_ch(int kind, const V2Args<T>& a, const BCase<T>* cases, const int4* items, int nitems,
                       BatchCtl ctl, int nsm, cudaStream_t st) {
  const int R = kind == 0 ? 5 : 3;
  const int P = v2_pitch<T>(CHC, R);
  const int ntile = kind == 0 ? 2 : (kind == 1 ? (V2_CG_SINGLE ? 4 : 5) : 3);
  const size_t smem = v2_smem_bytes<T, DIR>(CHC, R, P, ntile);
  const int minb = kind == 0 ? (sizeof(T) == 4 ? V2_MINB_F : 2)
                             : (kind == 1 ? V2_MINB : (sizeof(T) == 4 ? V2_MINB_V : 2));
  const unsigned grid = (unsigned)std::min(nitems, nsm * minb);
  const dim3 bl = v2_block<T>();
  const UCo<T, CHC> U = make_uco<T, CHC>(a);
  if (kind == 0) {
    static const cudaError_t e = v2_allow_smem(kb_filter<T, DIR, CHC>, smem);
    if (e != cudaSuccess) return e;
    kb_filter<T, DIR, CHC><<<grid, bl, smem, st>>>(cases, items, nitems, U, ctl);
  } else if (kind == 1) {
    static const cudaError_t e = v2_allow_smem(kb_convgrad<T, DIR, CHC>, smem);
    if (e != cudaSuccess) return e;
    kb_convgrad<T, DIR, CHC><<<grid, bl, smem, st>>>(cases, items, nitems, U, ctl);
  } else {
    static const cudaError_t e = v2_allow_smem(kb_visc<T, DIR, CHC>, smem);
    if (e != cudaSuccess) return e;
    kb_visc<T, DIR, CHC><<<grid, bl, smem, st>>>(cases, items, nitems, U, ctl);
  }
  return cudaGetLastError();
}
template <typename T, int DIR>
cudaError_t launch2_batch(int kind, int CH, const V2Args<T>& a, const BCase<T>* cases, const int4* items,
                          int nitems, BatchCtl ctl, int nsm, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  ASTR_V2_CH_SWITCH(CH, return (launchb_ch<T, DIR, CHC>(kind, a, cases, items, nitems, ctl, nsm, st)));
  return cudaSuccess;
}

#define ASTR_INSTANTIATE_SWEEPS2(T, DIR)                                                          \
  template cudaError_t launch2_filter<T, DIR>(const V2Args<T>&, cudaStream_t, int, int);         \
  template cudaError_t launch2_convgrad<T, DIR>(const V2Args<T>&, cudaStream_t, int, CGFlags, int); \
  template cudaError_t launch2_visc<T, DIR>(const V2Args<T>&, cudaStream_t, int, int);          \
  template cudaError_t launch2_batch<T, DIR>(int, int, const V2Args<T>&, const BCase<T>*, const int4*, \
                                             int, BatchCtl, int, cudaStream_t);

}  // namespace astr
