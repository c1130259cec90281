// Line-sweep kernels (filter, convective + gradient, viscous) and their
// launchers.  Included once per sweep direction and precision by the
// sweep_*.cu translation units so they compile in parallel.
#pragma once

#include "launch.cuh"

namespace astr {

template <int DIR, bool XB = false>
constexpr int block_threads() { return warp_lines<DIR, XB>() ? NCH * X_LINES : NCH_B * YZ_LINES; }
template <int DIR, bool XB = false>
constexpr int min_blocks() { return warp_lines<DIR, XB>() ? MINB_X : MINB_YZ; }

// filterq (src/comsolver.F90:514-632): one direction, all five variables,
// in place.  do_q2f (mini-app ordering, last direction): recover the
// primitives of the filtered state.
template <typename T, int DIR, int CH>
__global__ void __launch_bounds__(block_threads<DIR, true>(), min_blocks<DIR, true>())
k_filter(Geo g, DevT<T> d, DScheme<T> S, FTab<T> Tb, Phys ph, int do_q2f) {
  __shared__ T sm[SCAN_SMEM_WORDS];
  LineMap<DIR, true> lm(g);
  const bool uni = uniform_chunk<DIR, true>(S, lm.c);
  if (warp_lines<DIR, true>() && !lm.active) return;  // whole warp: x-lines own a warp
  const long long hs = hstride<DIR>(g);
  int i0, j0, k0;
  line_ijk<DIR>(lm.a, lm.b, 0, i0, j0, k0);
  const long long base = hidx(g, i0, j0, k0);
  const long long bz = zidx(g, i0, j0, k0), zs = zstride<DIR>(g);
  const int dim = S.dim;
  const int per = g.per[DIR] ? 1 : 0;
#pragma unroll 1
  for (int n = 0; n < 5; ++n) {
    if (!my_task(n)) continue;
    T* v = d.q + n * g.nh;
    // FP64: the reference's form, x = A^{-1} B f.  FP32: the increment
    // form, x = f + A^{-1} (B - A) f (see filter_rhs_delta), with the
    // increment added to the FP64 master so that none of it is lost below
    // the FP32 spacing of f.
    constexpr bool delta = sizeof(T) == 4;
    T w[CH + 10];
    filter_window<CH>(w, S, lm.c, v, base, hs, per);
    T y[CH];
    if (delta) filter_rhs_delta<CH>(y, w, S, Tb, lm.c, v, base, hs, per, uni);
    else filter_rhs<CH>(y, w, S, Tb, lm.c, v, base, hs, per, uni);
    chunk_solve<CH, DIR, true>(y, S, lm.c, sm, uni);
    if (warp_lines<DIR, true>()) __syncwarp();
    if (lm.active) {
#pragma unroll
      for (int t = 0; t < CH; ++t) {
        const int r = lm.c * CH + t;
        const int node = S.first + r;
        const bool keep_end = S.ntype == 4 && (node == 0 || node == dim);
        if (r < S.n && node >= 0 && node <= dim && !keep_end) {
          if (delta && d.qm) {
            double* M = d.qm + n * g.n0 + bz + zs * node;
            const double nv = *M + (double)y[t];
            *M = nv;
            v[base + hs * node] = (T)nv;
          } else {
            v[base + hs * node] = delta ? w[t + 5] + y[t] : y[t];
          }
        }
      }
    }
  }
  if (do_q2f && lm.active) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int node = S.first + lm.c * CH + t;
      if (node >= 0 && node <= dim) q2fvar_store(g, d, ph, base + hs * node);
    }
  }
}

// convrsdcal6 (src/solver.F90:2173-2341) and gradcal
// (src/comsolver.F90:244-497), one direction, diagonal metrics.
// FP32 convective sweeps stage the two flux factors shared by the five
// conserved variables in dynamic shared memory, once per direction: main
// ordering A = J*(dxi*u_d), B = J*(dxi*p); mini-app A = u_d, B = p.  A line
// has rows -3 .. n+2 of them; y/z blocks store them node-major
// (row*YZ_LINES + line), x warps line-major (line*(n+6) + row), both
// conflict-free for the chunk-strided reads.
template <typename T>
constexpr bool stage_flux() { return sizeof(T) == 4; }


// GEN: general metrics.  The convective flux uses the whole metric row
// (U = dxi(d,1) u + dxi(d,2) v + dxi(d,3) w, pressure terms dxi(d,m) p, as
// src/solver.F90:2200-2206), and the gradients are stored as derivatives
// along the computational direction, contracted with the metrics by
// k_gradphys once all directions are done (gradcal's sum over d,
// src/comsolver.F90:244-497).  The last-direction stress and statistics are
// then computed by point kernels.
template <typename T, int DIR, int CH, bool GEN>
__global__ void __launch_bounds__(block_threads<DIR>(), min_blocks<DIR>())
k_convgrad(Geo g, DevT<T> d, DScheme<T> S, Phys ph, CGFlags fl) {
  __shared__ T sm[SCAN_SMEM_WORDS];
  extern __shared__ __align__(16) unsigned char conv_smem[];
  LineMap<DIR> lm(g);
  const bool uni = uniform_chunk<DIR, false>(S, lm.c);
  if (warp_lines<DIR>() && !lm.active) {  // whole warp: x-lines own a warp
    if (fl.stats && threadIdx.x == 0) {
      const long long wid = (long long)blockIdx.x * blockDim.y + threadIdx.y;
      d.part[2 * wid] = 0.0;
      d.part[2 * wid + 1] = 0.0;
    }
    return;
  }
  const long long hs = hstride<DIR>(g), zs = zstride<DIR>(g);
  int i0, j0, k0;
  line_ijk<DIR>(lm.a, lm.b, 0, i0, j0, k0);
  const long long bh = hidx(g, i0, j0, k0);
  const long long bz = zidx(g, i0, j0, k0);
  const int dim = S.dim;
  const long long nh = g.nh, n0 = g.n0;
  const int lo = g.lo[DIR], hi = g.hi[DIR];
  // transverse ranges of convrsdcal6 (js..je, ks..ke etc.)
  const int ta = DIR == 0 ? 1 : 0, tb = DIR == 2 ? 1 : 2;
  const bool cline = lm.a >= g.lo[ta] && lm.a <= g.hi[ta] && lm.b >= g.lo[tb] && lm.b <= g.hi[tb];
  const T rdx = pc<T>(ph.rdx[DIR], ph.f_rdx[DIR]);
  const T* xd = d.xd + DIR * nh;

  // tasks: the five convective fluxes (fl.conv), then the four gradients
  // (fl.grad); the RK3 base, stress and statistics only without a split
  const int nconv = fl.conv ? 5 : 0;
  if (fl.conv && (gridDim.z == 1 || (int)blockIdx.z < nconv)) {
    constexpr bool stg = stage_flux<T>() && !GEN;
    const int NL = warp_lines<DIR>() ? (int)blockDim.y : (int)blockDim.x;  // lines in the block
    T* fa = reinterpret_cast<T*>(conv_smem);
    const int np = S.n + 6;  // rows -3 .. n+2
    T* fb = fa + (size_t)np * NL;
    const int li = warp_lines<DIR>() ? (int)threadIdx.y : (int)threadIdx.x;
    auto sidx = [&](int rho) -> int {
      return warp_lines<DIR>() ? li * np + (rho + 3) : (rho + 3) * NL + li;
    };
    if (stg) {
      // this chunk's rows; chunk 0 adds rows -3..-1, the chunk of row n-1
      // adds rows n..n+2 (the windows of the end rows)
      const int s0 = lm.c * CH;
      const int r0 = lm.c == 0 ? -3 : s0;
      const int r1 = (s0 <= S.n - 1 && S.n - 1 < s0 + CH) ? S.n + 2 : min(s0 + CH, S.n) - 1;
      for (int rho = r0; rho <= r1; ++rho) {
        const long long p = bh + hs * (S.first + rho);
        const T pp = d.pr[p + 4 * nh];
        const T ud = d.pr[p + (1 + DIR) * nh];
        T A = ud, B = pp;
        if (!ph.mini) {
          const T x = xd[p];
          const T J = d.jac[p];
          A = J * (x * ud);
          B = J * (x * pp);
        }
        fa[sidx(rho)] = A;
        fb[sidx(rho)] = B;
      }
      if (warp_lines<DIR>()) __syncwarp();
      else __syncthreads();
    }
#pragma unroll 1
    for (int n = 0; n < 5; ++n) {
      if (!my_task(n)) continue;
      auto f = [&](int node) -> T {
        const long long p = bh + hs * node;
        const T qn = d.q[p + n * nh];
        if (GEN) {
          const T* X = d.xg + (3 * DIR) * nh + p;
          const T x0 = X[0], x1 = X[nh], x2 = X[2 * nh];
          const T uu = x0 * d.pr[p + nh] + x1 * d.pr[p + 2 * nh] + x2 * d.pr[p + 3 * nh];
          const T pp = d.pr[p + 4 * nh];
          const T J = d.jac[p];
          if (n == 0) return J * qn * uu;
          if (n == 4) return J * (qn + pp) * uu;
          return J * (qn * uu + (n == 1 ? x0 : (n == 2 ? x1 : x2)) * pp);
        }
        if (stg) {
          const int rho = node - S.first;
          const T A = fa[sidx(rho)], B = fb[sidx(rho)];
          if (ph.mini) {
            if (n == 4) return (qn + B) * A;
            if (n == 1 + DIR) return qn * A + B;
            return qn * A;
          }
          if (n == 4) return (qn + d.pr[p + 4 * nh]) * A;
          if (n == 1 + DIR) return qn * A + B;
          return qn * A;
        }
        const T pp = d.pr[p + 4 * nh];
        const T ud = d.pr[p + (1 + DIR) * nh];
        if (ph.mini) {
          const T uu = ud;
          if (n == 4) return (qn + pp) * uu;
          if (n == 1 + DIR) return qn * uu + pp;
          return qn * uu;
        }
        const T x = xd[p];
        const T J = d.jac[p];
        const T uu = x * ud;
        if (n == 0) return J * qn * uu;
        if (n == 4) return J * (qn + pp) * uu;
        if (n == 1 + DIR) return J * (qn * uu + x * pp);
        return J * (qn * uu);
      };
      T y[CH];
      deriv_rhs<CH>(y, S, lm.c, f, uni);
      chunk_solve<CH, DIR, false>(y, S, lm.c, sm, uni);
      if (lm.active) {
#pragma unroll
        for (int t = 0; t < CH; ++t) {
          const int node = S.first + lm.c * CH + t;
          if (node >= 0 && node <= dim) {
            T* R = d.qrhs + n * n0 + bz + zs * node;
            const bool in = cline && node >= lo && node <= hi;
            const T add = in ? (ph.mini ? y[t] * rdx : y[t]) : T(0);
            T val = fl.first ? add : (*R + add);
            if (fl.last) val = -val;
            *R = val;
          }
        }
      }
    }
  }
  if (fl.grad) {
#pragma unroll 1
    for (int n = 0; n < 4; ++n) {
      if (!my_task(n + nconv)) continue;
      const T* src = d.pr + (n < 3 ? 1 + n : 5) * nh;
      auto f = [&](int node) -> T { return src[bh + hs * node]; };
      T y[CH];
      deriv_rhs<CH>(y, S, lm.c, f, uni);
      chunk_solve<CH, DIR, false>(y, S, lm.c, sm, uni);
      const int comp = n < 3 ? n + 3 * DIR : 9 + DIR;
      if (lm.active) {
#pragma unroll
        for (int t = 0; t < CH; ++t) {
          const int node = S.first + lm.c * CH + t;
          if (node >= 0 && node <= dim) {
            const T gv = GEN ? y[t] : (ph.mini ? y[t] * rdx : y[t] * xd[bh + hs * node]);
            d.grad[comp * n0 + bz + zs * node] = gv;
          }
        }
      }
    }
  }
  if (fl.qsave && lm.active && blockIdx.z == 0) {
    // RK3 base at stage 1 (src/mainloop.F90:427-433): q*J (mini-app: q)
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int node = S.first + lm.c * CH + t;
      if (node >= 0 && node <= dim) {
        const long long p = bh + hs * node, z = bz + zs * node;
        const double J = d.jac64[p];
        for (int m = 0; m < 5; ++m) {
          const double qv = q64(d, p, z, m, nh, n0);
          d.qsave[m * n0 + z] = ph.mini ? qv : qv * J;
        }
      }
    }
  }
  if (fl.last && fl.sigma && lm.active && gridDim.z == 1) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int node = S.first + lm.c * CH + t;
      if (node >= 0 && node <= dim) sigma_point(g, d, ph, bz + zs * node, bh + hs * node);
    }
  }
  if (fl.stats) {
    double ke = 0.0, en = 0.0;
    if (lm.active) {
#pragma unroll
      for (int t = 0; t < CH; ++t) {
        const int node = S.first + lm.c * CH + t;
        int i, j, k;
        line_ijk<DIR>(lm.a, lm.b, node, i, j, k);
        const bool ink = g.ndims == 3 ? (k >= 1 && k <= g.km) : (k == 0);
        if (node >= 0 && node <= dim && i >= 1 && j >= 1 && ink) {
          const long long p = bh + hs * node, z = bz + zs * node;
          const double ro = d.pr[p], u = d.pr[p + nh], v = d.pr[p + 2 * nh], w = d.pr[p + 3 * nh];
          ke += ro * (u * u + v * v + w * w);
          const T* G = d.grad + z;
          const double o3 = (double)G[1 * n0] - (double)G[3 * n0];
          double om = o3 * o3;
          if (g.ndims == 3) {
            const double o1 = (double)G[5 * n0] - (double)G[7 * n0];
            const double o2 = (double)G[6 * n0] - (double)G[2 * n0];
            om = o1 * o1 + o2 * o2 + o3 * o3;
          }
          en += ro * om;
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      ke += __shfl_down_sync(0xffffffffu, ke, off);
      en += __shfl_down_sync(0xffffffffu, en, off);
    }
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    if ((tid & 31) == 0) {
      const long long wpb = (blockDim.x * blockDim.y) >> 5;
      const long long wid = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * wpb + (tid >> 5);
      d.part[2 * wid] = ke;
      d.part[2 * wid + 1] = en;
    }
  }
}

// diffrsdcal6 sweeps (src/solver.F90:2619-2852), one direction.  The last
// direction applies the RK3 update (and, main ordering, q2fvar).
// GEN: general metrics, fluxes J*(sigma . dxi(d,:)) and J*(qflux . dxi(d,:))
// (src/solver.F90:2627-2638).
template <typename T, int DIR, int CH, bool GEN>
__global__ void __launch_bounds__(block_threads<DIR>(), min_blocks<DIR>())
k_visc(Geo g, DevT<T> d, DScheme<T> S, Phys ph, VFlags fl) {
  __shared__ T sm[SCAN_SMEM_WORDS];
  LineMap<DIR> lm(g);
  const bool uni = uniform_chunk<DIR, false>(S, lm.c);
  if (warp_lines<DIR>() && !lm.active) return;  // whole warp: x-lines own a warp
  const long long hs = hstride<DIR>(g), zs = zstride<DIR>(g);
  int i0, j0, k0;
  line_ijk<DIR>(lm.a, lm.b, 0, i0, j0, k0);
  const long long bh = hidx(g, i0, j0, k0);
  const long long bz = zidx(g, i0, j0, k0);
  const int dim = S.dim;
  const long long nh = g.nh, n0 = g.n0;
  const int lo = g.lo[DIR], hi = g.hi[DIR];
  const bool per = g.per[DIR] != 0;
  const T rdx = pc<T>(ph.rdx[DIR], ph.f_rdx[DIR]);
  const T* xd = d.xd + DIR * nh;
  constexpr int s0 = DIR == 0 ? 0 : (DIR == 1 ? 1 : 2);
  constexpr int s1 = DIR == 0 ? 1 : (DIR == 1 ? 3 : 4);
  constexpr int s2 = DIR == 0 ? 2 : (DIR == 1 ? 4 : 5);
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    if (!my_task(n)) continue;
    const int sc = n == 0 ? s0 : (n == 1 ? s1 : s2);
    const T* src = n < 3 ? d.sig + sc * n0 : d.qf + DIR * n0;
    auto f = [&](int node) -> T {
      int nd = node;
      if (per) nd = nd < 0 ? nd + dim : (nd > dim ? nd - dim : nd);
      else if (nd < 0 || nd > dim) return T(0);
      if (GEN) {
        // sigma rows (1: s11 s12 s13, 2: s12 s22 s23, 3: s13 s23 s33) or qflux
        const long long zz = bz + zs * nd;
        const int c0 = n == 0 ? 0 : (n == 1 ? 1 : 2);
        const int c1 = n == 0 ? 1 : (n == 1 ? 3 : 4);
        const int c2 = n == 0 ? 2 : (n == 1 ? 4 : 5);
        const T* Sg = d.sig + zz;
        const T* Qf = d.qf + zz;
        const T a0 = n < 3 ? Sg[c0 * n0] : Qf[0];
        const T a1 = n < 3 ? Sg[c1 * n0] : Qf[n0];
        const T a2 = n < 3 ? Sg[c2 * n0] : Qf[2 * n0];
        const long long p = bh + hs * node;
        const T* X = d.xg + (3 * DIR) * nh + p;
        return (a0 * X[0] + a1 * X[nh] + a2 * X[2 * nh]) * d.jac[p];
      }
      const T sv = src[bz + zs * nd];
      if (ph.mini) return sv;
      const long long p = bh + hs * node;
      return (sv * xd[p]) * d.jac[p];
    };
    T y[CH];
    deriv_rhs<CH>(y, S, lm.c, f, uni);
    chunk_solve<CH, DIR, false>(y, S, lm.c, sm, uni);
    if (lm.active) {
#pragma unroll
      for (int t = 0; t < CH; ++t) {
        const int node = S.first + lm.c * CH + t;
        if (node >= 0 && node <= dim) {
          const long long z = bz + zs * node;
          T* R = d.qrhs + (n + 1) * n0 + z;
          const bool in = node >= lo && node <= hi;
          const T val = *R + (in ? (ph.mini ? y[t] * rdx : y[t]) : T(0));
          if (!fl.last) *R = val;
          else rk_update(g, d, ph, bh + hs * node, z, n + 1, (double)val);
        }
      }
    }
  }
  if (fl.last && lm.active) {
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int node = S.first + lm.c * CH + t;
      if (node >= 0 && node <= dim) {
        const long long z = bz + zs * node, p = bh + hs * node;
        rk_update(g, d, ph, p, z, 0, (double)d.qrhs[z]);
        if (fl.q2f) q2fvar_store(g, d, ph, p);
      }
    }
  }
}

#define ASTR_CH_SWITCH(CHV, EXPR)                           \
  switch (CHV) {                                            \
    case 3: { constexpr int CHC = 3; EXPR; } break;         \
    case 5: { constexpr int CHC = 5; EXPR; } break;         \
    case 9: { constexpr int CHC = 9; EXPR; } break;         \
    case 17: { constexpr int CHC = 17; EXPR; } break;       \
    case 33: { constexpr int CHC = 33; EXPR; } break;       \
    default: return cudaErrorInvalidValue;                  \
  }

template <typename T, int DIR>
cudaError_t launch_filter(const SweepCtx<T>& c, const DScheme<T>& S, const FTab<T>& Tb, int CH,
                          int do_q2f) {
  const int lb = sweep_lb<DIR, true>(c);
  dim3 gr = sweep_grid<DIR, true>(c.g, lb);
  const dim3 bl = sweep_block<DIR, true>(lb);
  gr.z = c.vsplit ? 5 : 1;
  ASTR_CH_SWITCH(CH, (k_filter<T, DIR, CHC><<<gr, bl, 0, c.st>>>(c.g, c.d, S, Tb, c.ph, do_q2f)));
  return cudaGetLastError();
}

template <typename T, int DIR, int CH, bool GEN>
cudaError_t launch_convgrad_gen(const SweepCtx<T>& c, const DScheme<T>& S, CGFlags f) {
  const int lb = sweep_lb<DIR, false>(c);
  dim3 gr = sweep_grid<DIR>(c.g, lb);
  const dim3 bl = sweep_block<DIR>(lb);
  const int ntask = (f.conv ? 5 : 0) + (f.grad ? 4 : 0);
  gr.z = c.vsplit && ntask > 1 ? ntask : 1;
  const size_t dyn = (stage_flux<T>() && !GEN && f.conv) ? 2 * (size_t)(S.n + 6) * lb * sizeof(T) : 0;
  static size_t attr_bytes = 48 * 1024;  // dynamic shared memory allowed so far (per instantiation)
  if (dyn > attr_bytes) {
    const cudaError_t ea = cudaFuncSetAttribute(k_convgrad<T, DIR, CH, GEN>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (ea != cudaSuccess) return ea;
    attr_bytes = dyn;
  }
  k_convgrad<T, DIR, CH, GEN><<<gr, bl, dyn, c.st>>>(c.g, c.d, S, c.ph, f);
  return cudaGetLastError();
}

template <typename T, int DIR, int CH>
cudaError_t launch_convgrad_ch(const SweepCtx<T>& c, const DScheme<T>& S, CGFlags f) {
  return c.gen ? launch_convgrad_gen<T, DIR, CH, true>(c, S, f)
               : launch_convgrad_gen<T, DIR, CH, false>(c, S, f);
}

// The same switch for a call that returns the launch status.
#define ASTR_CH_RETURN(CHV, ...)                                   \
  switch (CHV) {                                                   \
    case 3: { constexpr int CHC = 3; return __VA_ARGS__; }         \
    case 5: { constexpr int CHC = 5; return __VA_ARGS__; }         \
    case 9: { constexpr int CHC = 9; return __VA_ARGS__; }         \
    case 17: { constexpr int CHC = 17; return __VA_ARGS__; }       \
    case 33: { constexpr int CHC = 33; return __VA_ARGS__; }       \
    default: return cudaErrorInvalidValue;                         \
  }

template <typename T, int DIR>
cudaError_t launch_convgrad(const SweepCtx<T>& c, const DScheme<T>& S, int CH, CGFlags f) {
  ASTR_CH_RETURN(CH, launch_convgrad_ch<T, DIR, CHC>(c, S, f));
}

template <typename T, int DIR>
cudaError_t launch_visc(const SweepCtx<T>& c, const DScheme<T>& S, int CH, VFlags f) {
  const int lb = sweep_lb<DIR, false>(c);
  dim3 gr = sweep_grid<DIR>(c.g, lb);
  const dim3 bl = sweep_block<DIR>(lb);
  gr.z = c.vsplit ? 4 : 1;
  if (c.gen) {
    ASTR_CH_SWITCH(CH, (k_visc<T, DIR, CHC, true><<<gr, bl, 0, c.st>>>(c.g, c.d, S, c.ph, f)));
  } else {
    ASTR_CH_SWITCH(CH, (k_visc<T, DIR, CHC, false><<<gr, bl, 0, c.st>>>(c.g, c.d, S, c.ph, f)));
  }
  return cudaGetLastError();
}

#define ASTR_INSTANTIATE_SWEEPS(T, DIR)                                                          \
  template cudaError_t launch_filter<T, DIR>(const SweepCtx<T>&, const DScheme<T>&, const FTab<T>&, \
                                             int, int);                                         \
  template cudaError_t launch_convgrad<T, DIR>(const SweepCtx<T>&, const DScheme<T>&, int, CGFlags); \
  template cudaError_t launch_visc<T, DIR>(const SweepCtx<T>&, const DScheme<T>&, int, VFlags);

}  // namespace astr
