// GB300 (sm_103a) right-hand-side hot path of the ASTR compressible
// Navier-Stokes solver, behind the C ABI of include/astr_gpu.h.
//
// Per RK3 stage (main ordering, src/mainloop.F90:396-486) the context issues
//   filter  x, y, z        compact 10th-order filter of q, in place
//   qswap   i, j, k        periodic halos, node-0/im averaging, primitives on
//                          halos and boundary planes (src/parallel.F90:4848-5318)
//   conv+grad x, y, z      convective flux derivatives into qrhs and velocity /
//                          temperature gradients; the last direction negates
//                          qrhs, forms sigma and the heat flux (and, at stage 1,
//                          the statistics)
//   visc    x, y, z        viscous flux derivatives into qrhs; the last
//                          direction applies the RK3 update and recovers the
//                          primitives
// The mini-app ordering (miniapps/tgv_solver_3d/tgvsolver.F90:994-1082) runs
// the same kernels with its own halo fill, scalings and filter placement.
//
// Two precision forms share the kernels: plain FP64 (T = double), and FP32
// storage (T = float) with the RK3 base and a master copy of q in FP64.
#include "launch.cuh"
#include "launch2.cuh"
#include "mp.cuh"
#include "../../include/astr_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

using namespace astr;

namespace {

// ---------------------------------------------------------------------------
// Halo kernels
// ---------------------------------------------------------------------------
template <int DIR>
__device__ __forceinline__ bool face_line_at(const Geo& g, int a, int b, int& dim, long long& base,
                                             long long& hs, long long* zbase = nullptr,
                                             long long* zs = nullptr) {
  const int na = DIR == 0 ? g.jm : g.im;
  if (a > na) return false;
  dim = DIR == 0 ? g.im : (DIR == 1 ? g.jm : g.km);
  hs = hstride<DIR>(g);
  int i0, j0, k0;
  line_ijk<DIR>(a, b, 0, i0, j0, k0);
  base = hidx(g, i0, j0, k0);
  if (zbase) *zbase = zidx(g, i0, j0, k0);
  if (zs) *zs = zstride<DIR>(g);
  return true;
}
template <int DIR>
__device__ __forceinline__ bool face_line(const Geo& g, int& dim, long long& base, long long& hs,
                                          long long* zbase = nullptr, long long* zs = nullptr) {
  return face_line_at<DIR>(g, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y, dim, base, hs, zbase, zs);
}

// qswap single-rank periodic branch of one direction (src/parallel.F90:
// 4876-4920, 5018-5065, 5159-5206).
template <typename T, int DIR>
__device__ __forceinline__ void qswap_line(const Geo& g, const DevT<T>& d, const Phys& ph, int a, int b) {
  int dim;
  long long base, hs, zb, zs;
  if (!face_line_at<DIR>(g, a, b, dim, base, hs, &zb, &zs)) return;
  for (int n = 0; n < 5; ++n) {
    T* v = d.q + n * g.nh + base;
    if (dim == 0) {
      for (int l = -HMD; l <= HMD; ++l) v[hs * l] = v[0];
    } else {
      for (int h = 1; h <= HMD; ++h) v[-hs * h] = v[hs * (dim - h)];
      for (int h = 1; h <= HMD; ++h) v[hs * (dim + h)] = v[hs * h];
      if (d.qm) {
        // FP32-storage form: average the FP64 master (interior nodes 0 and
        // dim), so the FP32 copy never departs from it
        double* M = d.qm + n * g.n0 + zb;
        const double avg = 0.5 * (M[0] + M[zs * dim]);
        M[0] = avg;
        M[zs * dim] = avg;
        v[0] = (T)avg;
        v[hs * dim] = (T)avg;
      } else {
        const T avg = T(0.5) * (v[0] + v[hs * dim]);
        v[0] = avg;
        v[hs * dim] = avg;
      }
    }
  }
  for (int l = -HMD; l <= 0; ++l) q2fvar_store(g, d, ph, base + hs * l);
  for (int l = dim; l <= dim + HMD; ++l) q2fvar_store(g, d, ph, base + hs * l);
}
// dataswap of q along a periodic direction (the halo copy filterq makes
// before filtering that direction, src/comsolver.F90:530-575 with
// src/parallel.F90:4169-4303, single rank): the halo layers take the
// periodic images of the current interior; no averaging, no primitives.
template <typename T, int DIR>
__global__ void k_qhalo(Geo g, DevT<T> d) {
  int dim;
  long long base, hs;
  if (!face_line<DIR>(g, dim, base, hs)) return;
  for (int n = 0; n < 5; ++n) {
    T* v = d.q + n * g.nh + base;
    for (int h = 1; h <= HMD; ++h) v[-hs * h] = v[hs * (dim - h)];
    for (int h = 1; h <= HMD; ++h) v[hs * (dim + h)] = v[hs * h];
  }
}

template <typename T, int DIR>
__global__ void k_qswap(Geo g, DevT<T> d, Phys ph) {
  qswap_line<T, DIR>(g, d, ph, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// bchomo of the mini-app, one direction (tgvsolver.F90:271-369).
template <typename T, int DIR>
__global__ void k_bchomo(Geo g, DevT<T> d, Phys ph) {
  int dim;
  long long base, hs;
  if (!face_line<DIR>(g, dim, base, hs)) return;
  const long long nh = g.nh;
  const T c6 = T(1) / pc<T>(ph.rconst6, ph.f_rconst6);
  auto copy = [&](long long dst, long long src) {
    for (int m = 0; m < 6; ++m) d.pr[dst + m * nh] = d.pr[src + m * nh];
    const T ro = d.pr[dst], u = d.pr[dst + nh], v = d.pr[dst + 2 * nh], w = d.pr[dst + 3 * nh];
    d.q[dst] = ro;
    d.q[dst + nh] = ro * u;
    d.q[dst + 2 * nh] = ro * v;
    d.q[dst + 3 * nh] = ro * w;
    const T var1 = T(0.5) * (u * u + v * v + w * w);
    d.q[dst + 4 * nh] = d.pr[dst + 4 * nh] * c6 + ro * var1;
  };
  for (int h = 1; h <= HMD; ++h) copy(base - hs * h, base + hs * (dim - h));
  for (int h = 1; h <= HMD; ++h) copy(base + hs * (dim + h), base + hs * h);
}

// ---------------------------------------------------------------------------
// Pointwise kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool point_of(const Geo& g, long long idx, int& i, int& j, int& k) {
  if (idx >= g.n0) return false;
  i = (int)(idx % g.I);
  const long long r = idx / g.I;
  j = (int)(r % (g.jm + 1));
  k = (int)(r / (g.jm + 1));
  return true;
}

template <typename T>
__global__ void k_updatefvar(Geo g, DevT<T> d, Phys ph) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  q2fvar_store(g, d, ph, hidx(g, i, j, k));
}

template <typename T>
__global__ void k_sigma(Geo g, DevT<T> d, Phys ph) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  sigma_point(g, d, ph, idx, hidx(g, i, j, k));
}

// RK3 update of the five variables at one point (and q2fvar): every
// operand is read before anything is written, so the loads of the point
// are in flight together; the primitives come from the stored (storage
// precision) values, as q2fvar_store reads them.
template <typename T>
__device__ __forceinline__ void rk_point(const Geo& g, const DevT<T>& d, const Phys& ph, int q2f,
                                         long long idx) {
  int i, j, k;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k), nh = g.nh, n0 = g.n0;
  T rhs[5];
  double qs[5], qv[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    rhs[m] = d.qrhs[m * n0 + idx];
    qs[m] = d.qsave[m * n0 + idx];
    qv[m] = q64(d, p, idx, m, nh, n0);
  }
  const double J = d.jac64[p], rj = d.rjac64[p];
  T qn[5];
  // FP32 storage: the same update with fewer FP64 operations (the FP64
  // pipe bounds this kernel on GB300): rk2*J once per point, rk3*dt folded
  // on the host, the small term rk3*dt*rhs (rhs is stored in FP32) formed
  // in FP32, multiply-adds; the FP64 form keeps the reference's order
  const double c2J = ph.rk2 * J;
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    double v;
    if (sizeof(T) == 4 && !ph.mini && !d.chan)
      v = fma(ph.rk1, qs[m], fma(c2J, qv[m], (double)((float)ph.rk3dt * (float)rhs[m]))) * rj;
    else
      v = rk_value(ph, d.chan, m, qs[m], qv[m], (double)rhs[m], J, rj);
    qn[m] = (T)v;
    d.q[m * nh + p] = qn[m];
    if (d.qm) d.qm[m * n0 + idx] = v;
  }
  if (q2f) {
    T ro, u, v, w, pp, tt;
    q2fvar_pt<T>(ph, qn[0], qn[1], qn[2], qn[3], qn[4], ro, u, v, w, pp, tt);
    d.pr[p] = ro;
    d.pr[p + nh] = u;
    d.pr[p + 2 * nh] = v;
    d.pr[p + 3 * nh] = w;
    d.pr[p + 4 * nh] = pp;
    d.pr[p + 5 * nh] = tt;
    if (!(ro > T(0))) atomicOr(d.flag, 1);
  }
}
template <typename T>
__global__ void k_rkupdate(Geo g, DevT<T> d, Phys ph, int q2f) {
  rk_point(g, d, ph, q2f, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// RK3 base at stage 1 (src/mainloop.F90:427-433): q*J (mini-app: q), in
// FP64 from the FP64 state or master.
template <typename T>
__device__ __forceinline__ void qsave_point(const Geo& g, const DevT<T>& d, const Phys& ph, long long idx) {
  int i, j, k;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k);
  const double J = d.jac64[p];
  for (int m = 0; m < 5; ++m) {
    const double qv = q64(d, p, idx, m, g.nh, g.n0);
    d.qsave[m * g.n0 + idx] = ph.mini ? qv : qv * J;
  }
}
template <typename T>
__global__ void k_qsave(Geo g, DevT<T> d, Phys ph) {
  qsave_point(g, d, ph, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Shu-Osher RK3 coefficients of the three stages (src/mainloop.F90:350-366).
__constant__ double c_rk[3][3] = {{1.0, 0.0, 1.0}, {0.75, 0.25, 0.25}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};

// The point and face kernels of a batched step, persistent over a work list
// of (case, block) items: kind 0-2 qswap of direction kind (item: a block
// of 256 face lines, line index), 3 RK3 base, 4 stress and heat flux, 5 RK3
// update of stage `stage` with the primitives (item: KB_PPT x 256 points).
// Same bodies as the single-case kernels.
constexpr int KB_THREADS = 256;
constexpr int KB_PPT = 8;
constexpr int KB_PTS = KB_PPT * KB_THREADS;
template <typename T>
__global__ void __launch_bounds__(KB_THREADS)
kb_point(const BCase<T>* cases, const int4* items, int nitems, int kind, int stage, BatchCtl ctl) {
  __shared__ int stop;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];
    if (threadIdx.x == 0) stop = batch_stopped(ctl);
    __syncthreads();
    if (stop) break;
    const BCase<T>* C = cases + w.x;
    const Geo g = C->g;
    const DevT<T> d = C->d;
    Phys ph = C->ph;
    if (kind <= 2) {
      const int a = w.y * KB_THREADS + threadIdx.x;
      if (kind == 0) qswap_line<T, 0>(g, d, ph, a, w.z);
      else if (kind == 1) qswap_line<T, 1>(g, d, ph, a, w.z);
      else qswap_line<T, 2>(g, d, ph, a, w.z);
    } else {
      if (kind == 5) {
        ph.rk1 = c_rk[stage][0];
        ph.rk2 = c_rk[stage][1];
        ph.rk3 = c_rk[stage][2];
        ph.rk3dt = c_rk[stage][2] * ph.dt;
      }
      const long long base = (long long)w.y * KB_PTS + threadIdx.x;
#pragma unroll 1
      for (int r = 0; r < KB_PPT; ++r) {
        const long long idx = base + r * KB_THREADS;
        if (kind == 3) {
          qsave_point(g, d, ph, idx);
        } else if (kind == 4) {
          int i, j, k;
          if (point_of(g, idx, i, j, k)) sigma_point(g, d, ph, idx, hidx(g, i, j, k));
        } else {
          rk_point(g, d, ph, 1, idx);
        }
      }
    }
    __syncthreads();
  }
}

// Start of a batched call: the deadline (budget_ns after now on the GPU's
// global timer; 0: none), a clear status word and no steps started.
__global__ void k_batch_start(BatchCtl ctl, unsigned long long* deadline, unsigned long long budget_ns) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  *deadline = budget_ns ? t + budget_ns : 0ULL;
  *ctl.status = 0;
  *ctl.started = 0;
}

// Gate of one batched step: stop on the cancel word or a passed deadline,
// else count the step as started.
__global__ void k_batch_gate(BatchCtl ctl) {
  int s = *(volatile int*)ctl.status;
  if (!s) {
    if (ctl.cancel && *ctl.cancel) s |= 1;
    const unsigned long long dl = *ctl.deadline_ns;
    if (dl) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t > dl) s |= 2;
    }
    if (s) *ctl.status = s;
    else *ctl.started += 1;
  }
}

// Boundary routines of boucon (src/bc.F90:327-409) on face n (0-based:
// xmin, xmax, ymin, ymax, zmin, zmax), one thread per face node, in FP64
// from the stored fields; nondimensional, no species.  Each branch restates
// the face branch of its routine as the reference writes it, including
// where the faces differ:
//   41 noslip (6306-6712): u = 0, T = T_w, p extrapolated, rho = p/T*const2,
//      q with pressure;
//   42 noslip_adibatic (6728-7036, x and y faces): p and T extrapolated;
//   411 slipisotwall (7038-7229, y faces): slip up to xslip on ymin;
//   421 slipadibwall (7231-7430, y faces): p, T and u extrapolated;
//   21 outflow (3404-3617, xmax and ymax faces);
//   51 farfield (3008-3392, y and z faces);
//   50 zeroextrap (2356-2652): x faces extrapolate T, the others rho; q with
//      temperature on ymax only;
//   60 symmetry (2664-2996): x faces and zmax remove the velocity along the
//      metric row's unit vector, y faces and zmin zero the normal component;
//      q with temperature on the x faces, ymax and zmax;
//   11 inflow (1366-1562, xmin): v, w, T from the inflow arrays, p from the
//      incoming characteristic blended towards pinf, u from p; q with
//      temperature;
//   23 gcnscbc (8024-8254, xmax and ymax): LODI at node dim-1 relaxed
//      towards pinf (ymax inflow: towards the free stream), extrapolated
//      over 2 dx; q with pressure.
// extrapolate(v1, v2, 0) is (4 v1 - v2)/3 (extrapolate_2o,
// src/commfunc.F90:277-285).
__device__ __forceinline__ double bc_ex2(double v1, double v2) {
  return (1.0 / 3.0) * (4.0 * v1 - v2 - 2.0 * 0.0);
}

template <typename T>
__global__ void k_face_bc(Geo g, DevT<T> d, Phys ph, int n, int type, double tw, double const1,
                          double const6, double pinf, double adt, double mach,
                          const unsigned char* slip, const double* inflow, const double* gcd,
                          double gce) {
  const int dir = n / 2, side = n % 2;
  const int na = (dir == 0 ? g.jm : g.im) + 1;
  const int nb = (dir == 2 ? g.jm : g.km) + 1;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)na * nb) return;
  const int a = (int)(idx % na), b = (int)(idx / na);
  const int dim = dir == 0 ? g.im : (dir == 1 ? g.jm : g.km);
  auto node = [&](int l, int& i, int& j, int& k) {
    const int x = side ? dim - l : l;
    i = dir == 0 ? x : a;
    j = dir == 0 ? a : (dir == 1 ? x : b);
    k = dir == 2 ? x : b;
  };
  int i, j, k, i1, j1, k1, i2, j2, k2;
  node(0, i, j, k);
  node(1, i1, j1, k1);
  node(2, i2, j2, k2);
  const long long nh = g.nh;
  const long long p = hidx(g, i, j, k), p1 = hidx(g, i1, j1, k1), p2 = hidx(g, i2, j2, k2);
  const double c2 = ph.const2, c6 = const6;
  auto prim = [&](long long q, int m) { return (double)d.pr[q + m * nh]; };
  double ro, u, v, w, pe, te;
  bool tform = false;  // q with temperature (else with pressure)
  if (type == 41) {
    pe = (1.0 / 3.0) * (4.0 * prim(p1, 4) - prim(p2, 4));
    u = v = w = 0.0;
    te = tw;
    ro = pe / te * c2;
  } else if (type == 42) {
    pe = (1.0 / 3.0) * (4.0 * prim(p1, 4) - prim(p2, 4));
    te = (1.0 / 3.0) * (4.0 * prim(p1, 5) - prim(p2, 5));
    u = v = w = 0.0;
    ro = pe / te * c2;
  } else if (type == 411) {
    // slipisotwall (7038-7229, y faces): on ymin slip (u and T extrapolated,
    // v = 0) where x <= xslip, isothermal no-slip beyond (wall blowing 0);
    // ymax isothermal no-slip; p extrapolated
    pe = (1.0 / 3.0) * (4.0 * prim(p1, 4) - prim(p2, 4));
    if (n == 2 && slip[idx]) {
      u = (1.0 / 3.0) * (4.0 * prim(p1, 1) - prim(p2, 1));
      te = (1.0 / 3.0) * (4.0 * prim(p1, 5) - prim(p2, 5));
    } else {
      u = 0.0;
      te = tw;
    }
    v = w = 0.0;
    ro = pe / te * c2;
  } else if (type == 421) {
    // slipadibwall (7231-7430, y faces): p, T, u extrapolated; v = 0 on
    // ymin, extrapolated on ymax (as the reference writes it); w = 0
    pe = (1.0 / 3.0) * (4.0 * prim(p1, 4) - prim(p2, 4));
    te = (1.0 / 3.0) * (4.0 * prim(p1, 5) - prim(p2, 5));
    u = (1.0 / 3.0) * (4.0 * prim(p1, 1) - prim(p2, 1));
    v = n == 3 ? (1.0 / 3.0) * (4.0 * prim(p1, 2) - prim(p2, 2)) : 0.0;
    w = 0.0;
    ro = pe / te * c2;
  } else if (type == 23) {
    // gcnscbc xmax (8041-8148) / ymax (8150-8252), prs_t = pinf: gcd is
    // the face's x(dim-1) - x(dim-2) along the normal, gce the grid's
    // extent along it.  css, css2 and vnorm are INTEGER in the reference
    // (src/bc.F90:8035): truncated, mavg an integer division, and
    // lambda(5:numq) = vnorm leaves lambda(5) = vnorm.
    const int on = dir, ot = dir == 0 ? 1 : 0;
    const int css = (int)(sqrt(prim(p1, 5)) / mach);
    const int css2 = css * css;
    const int vnorm = (int)prim(p1, 1 + on);
    const double mavg = css != 0 ? (double)(vnorm / css) : 0.0;
    double lam[5] = {(double)(vnorm - css), (double)vnorm, (double)vnorm, (double)vnorm, (double)vnorm};
    for (int m = 0; m < 5; ++m) lam[m] = lam[m] + 1e-10;
    const double dx = gcd[idx];
    // every product and sum rounded on its own (no contracted multiply-
    // adds): the one-sided differences cancel, and the restatement the
    // parity tests hold this to rounds each operation
    auto M = [](double x, double y) { return __dmul_rn(x, y); };
    auto A = [](double x, double y) { return __dadd_rn(x, y); };
    auto S = [](double x, double y) { return __dsub_rn(x, y); };
    const double r1 = prim(p1, 0), t1 = prim(p1, 5), pr1 = prim(p1, 4), cs = (double)css;
    double dvel[3], dprs;
    for (int m = 0; m < 3; ++m) dvel[m] = -S(prim(p2, 1 + m), prim(p1, 1 + m)) / dx;
    dprs = -S(prim(p2, 4), pr1) / dx;
    const double drho = -S(prim(p2, 0), r1) / dx;
    double lodi[5];
    lodi[0] = M(lam[0], S(dprs, M(M(r1, cs), dvel[on])));
    lodi[1] = M(lam[1], S(M((double)css2, drho), dprs));
    lodi[2] = M(lam[2], dvel[ot]);
    lodi[3] = M(lam[3], dvel[2]);
    lodi[4] = M(lam[4], A(dprs, M(M(r1, cs), dvel[on])));
    const double m2 = S(1.0, M(mavg, mavg));
    if (dir == 0 || vnorm >= 0) {
      const double kamma = M(M(0.25, cs), m2) / gce;
      lodi[0] = M(kamma, S(pr1, pinf));
    } else {
      // the free stream: uinf = 1, vinf = winf = 0, tinf = 1
      const double eta = 0.25;
      lodi[0] = M(M(M(M(eta, r1), (double)css2), m2) / gce, S(prim(p1, 1 + on), 0.0));
      lodi[1] = M(M(M(eta, r1), (double)css2) / 1.4 / gce, S(t1, 1.0));
      lodi[2] = M(M(eta, cs) / gce, S(prim(p1, 1 + ot), 1.0));
      lodi[3] = M(M(eta, cs) / gce, S(prim(p1, 3), 0.0));
    }
    for (int m = 0; m < 5; ++m) lodi[m] = lodi[m] / lam[m];
    const double l05 = A(lodi[0], lodi[4]);
    const double dtmp = M(t1 / r1 / cs, A(-lodi[1], M(0.5 * (1.4 - 1.0), l05)));
    dprs = M(0.5, l05);
    dvel[on] = M(1.0 / M(M(2.0, r1), cs), S(lodi[4], lodi[0]));
    dvel[ot] = lodi[2];
    dvel[2] = lodi[3];
    const double dx2 = M(2.0, dx);  // rho follows from p and T
    te = A(t1, M(dx2, dtmp));
    pe = A(pr1, M(dx2, dprs));
    u = A(prim(p1, 1), M(dx2, dvel[0]));
    v = A(prim(p1, 2), M(dx2, dvel[1]));
    w = A(prim(p1, 3), M(dx2, dvel[2]));
    ro = pe / te * c2;
  } else if (type == 11) {
    // inflow xmin (1366-1562, its active subsonic branch): node (j, k) =
    // (a, b) of the face; inflow = vel_in(0:jm,0:km,1:3), tmp_in(0:jm,0:km),
    // tmp_prof(0:jm); rho_ref the first interior node; css the speed of
    // sound of the profile temperature; blend -> 1 as the inflow Mach
    // number passes 1
    const long long nf = (long long)(g.jm + 1) * (g.km + 1), fj = (long long)a + (long long)(g.jm + 1) * b;
    const double vin1 = inflow[fj], vin2 = inflow[fj + nf], vin3 = inflow[fj + 2 * nf];
    const double rho_ref = prim(p1, 0);
    const double css = sqrt(inflow[4 * nf + a]) / mach;
    const double pex = bc_ex2(prim(p1, 4), prim(p2, 4));
    const double ue = bc_ex2(prim(p1, 1), prim(p2, 1));
    const double malo = vin1 / css;
    const double blend = 0.5 * (tanh((malo - 1.0) * 6.0) + 1.0);
    pe = (0.5 * (pinf + pex) + 0.5 * rho_ref * css * (vin1 - ue)) * (1.0 - blend) + pinf * blend;
    u = vin1 + (pinf - pe) / rho_ref / css;
    v = vin2;
    w = vin3;
    te = inflow[3 * nf + fj];
    ro = pe / te * c2;
    tform = true;
  } else if (type == 21 && n == 1) {
    // outflow xmax (3427-3532): the i-1 node copied (its supersonic branch
    // is taken unconditionally); q in temperature form
    u = prim(p1, 1);
    v = prim(p1, 2);
    w = prim(p1, 3);
    pe = prim(p1, 4);
    te = prim(p1, 5);
    ro = pe / te * c2;
    tform = true;
  } else if (type == 21) {
    // outflow ymax (3534-3615): extrapolated where the face is supersonic,
    // else p relaxed towards pinf (adt = 0.25 deltat); T from p and rho
    const double css = sqrt(prim(p, 5)) / mach;
    const double vf = prim(p, 2);
    u = bc_ex2(prim(p1, 1), prim(p2, 1));
    v = bc_ex2(prim(p1, 2), prim(p2, 2));
    w = bc_ex2(prim(p1, 3), prim(p2, 3));
    if (vf >= css) {
      pe = bc_ex2(prim(p1, 4), prim(p2, 4));
      ro = bc_ex2(prim(p1, 0), prim(p2, 0));
    } else {
      pe = (prim(p, 4) + adt * pinf + prim(p, 0) * css * (v - vf)) / (1.0 + adt);
      ro = pe / bc_ex2(prim(p1, 5), prim(p2, 5)) * c2;
    }
    te = pe / ro * c2;
  } else if (type == 51 && n == 3) {
    // farfield ymax (3106-3233): its characteristic treatment is commented
    // out, so everything is extrapolated; q in temperature form
    u = bc_ex2(prim(p1, 1), prim(p2, 1));
    v = bc_ex2(prim(p1, 2), prim(p2, 2));
    w = bc_ex2(prim(p1, 3), prim(p2, 3));
    pe = bc_ex2(prim(p1, 4), prim(p2, 4));
    ro = bc_ex2(prim(p1, 0), prim(p2, 0));
    te = pe / ro * c2;
    tform = true;
  } else if (type == 51) {
    // farfield ymin (3024-3104), zmin (3235-3312), zmax (3314-3389):
    // free-stream inflow (Riemann invariants, isentropic rho) where the
    // normal velocity points inwards, else outflow at pinf; free stream
    // uinf = roinf = 1, vinf = winf = 0
    const int m = dir == 1 ? 2 : 3;
    const double css = sqrt(prim(p, 5)) / mach;
    const double ue = bc_ex2(prim(p1, 1), prim(p2, 1));
    const double ve = bc_ex2(prim(p1, 2), prim(p2, 2));
    const double we = bc_ex2(prim(p1, 3), prim(p2, 3));
    const double pex = bc_ex2(prim(p1, 4), prim(p2, 4));
    const double roe = bc_ex2(prim(p1, 0), prim(p2, 0));
    const double csse = bc_ex2(sqrt(prim(p1, 5)) / mach, sqrt(prim(p2, 5)) / mach);
    const double vn_e = dir == 1 ? ve : we;
    const double sgn = side ? -1.0 : 1.0;
    const double vnf = prim(p, m), rof = prim(p, 0);
    double vn;
    if (side ? vnf <= 0.0 : vnf >= 0.0) {
      vn = sgn * 0.5 * (pinf - pex) / (rof * css) + 0.5 * (0.0 + vn_e);
      pe = 0.5 * (pinf + pex) + sgn * 0.5 * rof * css * (0.0 - vn_e);
      ro = 1.0 * pow(pe / pinf, 1.0 / 1.4);
      u = 1.0;
      v = w = 0.0;
    } else {
      pe = pinf;
      ro = roe + (pe - pex) / csse / csse;
      vn = vn_e - sgn * (pex - pe) / roe / csse;
      u = ue;
      v = ve;
      w = we;
    }
    if (dir == 1) v = vn;
    else w = vn;
    te = pe / ro * c2;
  } else {
    u = bc_ex2(prim(p1, 1), prim(p2, 1));
    v = bc_ex2(prim(p1, 2), prim(p2, 2));
    w = bc_ex2(prim(p1, 3), prim(p2, 3));
    pe = bc_ex2(prim(p1, 4), prim(p2, 4));
    const bool rho_extrap = type == 50 ? dir != 0 : n == 5;
    if (rho_extrap) {
      ro = bc_ex2(prim(p1, 0), prim(p2, 0));
      te = pe / ro * c2;
    } else {
      te = bc_ex2(prim(p1, 5), prim(p2, 5));
      ro = pe / te * c2;
    }
    if (type == 50) {
      tform = n == 3;
    } else if (n <= 1 || n == 5) {
      // unit vector along the metric row (gridgeom's bnorm, src/geom.F90:700-830)
      double x0, x1, x2;
      if (d.xg) {
        x0 = (double)d.xg[(3 * dir + 0) * nh + p];
        x1 = (double)d.xg[(3 * dir + 1) * nh + p];
        x2 = (double)d.xg[(3 * dir + 2) * nh + p];
      } else {
        const double xv = (double)d.xd[dir * nh + p];
        x0 = dir == 0 ? xv : 0.0;
        x1 = dir == 1 ? xv : 0.0;
        x2 = dir == 2 ? xv : 0.0;
      }
      const double var1 = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
      const double n0 = x0 / var1, n1 = x1 / var1, n2 = x2 / var1;
      const double vne = u * n0 + v * n1 + w * n2;
      u = u - vne * n0;
      v = v - vne * n1;
      w = w - vne * n2;
      tform = true;
    } else {
      if (dir == 1) v = 0.0;
      else w = 0.0;
      tform = n == 3;
    }
  }
  const double var1 = 0.5 * (u * u + v * v + w * w);
  const double e = tform ? ro * (te * const1 + var1) : pe * c6 + ro * var1;
  d.pr[p] = (T)ro;
  d.pr[p + nh] = (T)u;
  d.pr[p + 2 * nh] = (T)v;
  d.pr[p + 3 * nh] = (T)w;
  d.pr[p + 4 * nh] = (T)pe;
  d.pr[p + 5 * nh] = (T)te;
  d.q[p] = (T)ro;
  d.q[p + nh] = (T)(ro * u);
  d.q[p + 2 * nh] = (T)(ro * v);
  d.q[p + 3 * nh] = (T)(ro * w);
  d.q[p + 4 * nh] = (T)e;
  if (d.qm) {
    const long long z = zidx(g, i, j, k), n0 = g.n0;
    d.qm[z] = ro;
    d.qm[z + n0] = ro * u;
    d.qm[z + 2 * n0] = ro * v;
    d.qm[z + 3 * n0] = ro * w;
    d.qm[z + 4 * n0] = e;
  }
}

// inflow_nscbc (src/bc.F90:2114-2344), bctype 12 on xmin with periodic y
// and z.  Three kernels: the domain-wide maximum of |u|^2/c^2 (gmachmax2);
// per face node (j, k) the residual the routine adds to qrhs at i = 0 --
// the LODI residual (the outgoing wave kept, the incoming waves relaxed
// towards the inflow arrays at the rate kin) and the face's tangential flux
// derivatives (ddfc '222e' with periodic ends: 0.5 (f(j+1) - f(j-1))) --
// in FP64 into B; and, after the convective sweeps (which leave qrhs at
// i = 0 zero: the face lies outside convrsdcal6's ranges), qrhs(0) -= B,
// the sign rhscal's negation gives the routine's additions.
__device__ __forceinline__ double nscbc_dxi(const Geo& g, const double* xg64, const void* xgv, const void* xdv,
                                            bool f32, int d, int m, long long p) {
  (void)g;
  (void)xg64;
  const long long nh = g.nh;
  if (xgv) return f32 ? (double)((const float*)xgv)[(3 * d + m) * nh + p] : ((const double*)xgv)[(3 * d + m) * nh + p];
  if (d != m) return 0.0;
  return f32 ? (double)((const float*)xdv)[d * nh + p] : ((const double*)xdv)[d * nh + p];
}

template <typename T>
__device__ __forceinline__ double nscbc_x(const Geo& g, const DevT<T>& d, int r, int m, long long p) {
  return nscbc_dxi(g, nullptr, (const void*)d.xg, (const void*)d.xd, sizeof(T) == 4, r, m, p);
}

// J (q u_r + dxi(r,:) p) at node p, every product and sum rounded on its own
template <typename T>
__device__ __forceinline__ void nscbc_flux(const Geo& g, const DevT<T>& d, int r, long long p, double* f) {
  const long long nh = g.nh;
  const double x1 = nscbc_x(g, d, r, 0, p), x2 = nscbc_x(g, d, r, 1, p), x3 = nscbc_x(g, d, r, 2, p);
  const double u = (double)d.pr[p + nh], v = (double)d.pr[p + 2 * nh], w = (double)d.pr[p + 3 * nh];
  const double pr = (double)d.pr[p + 4 * nh], J = d.jac64[p];
  const double uu = __dadd_rn(__dadd_rn(__dmul_rn(x1, u), __dmul_rn(x2, v)), __dmul_rn(x3, w));
  f[0] = __dmul_rn(__dmul_rn(J, (double)d.q[p]), uu);
  f[1] = __dmul_rn(J, __dadd_rn(__dmul_rn((double)d.q[p + nh], uu), __dmul_rn(x1, pr)));
  f[2] = __dmul_rn(J, __dadd_rn(__dmul_rn((double)d.q[p + 2 * nh], uu), __dmul_rn(x2, pr)));
  f[3] = __dmul_rn(J, __dadd_rn(__dmul_rn((double)d.q[p + 3 * nh], uu), __dmul_rn(x3, pr)));
  f[4] = __dmul_rn(__dmul_rn(J, __dadd_rn((double)d.q[p + 4 * nh], pr)), uu);
}

template <typename T>
__global__ void k_nscbc_gmach(Geo g, DevT<T> d, double mach, unsigned long long* out) {
  __shared__ double sh[256];
  double mx = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.n0;
       idx += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    point_of(g, idx, i, j, k);
    const long long p = hidx(g, i, j, k), nh = g.nh;
    const double u = (double)d.pr[p + nh], v = (double)d.pr[p + 2 * nh], w = (double)d.pr[p + 3 * nh];
    const double var1 = __dadd_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)), __dmul_rn(w, w));
    const double css = sqrt((double)d.pr[p + 5 * nh]) / mach;
    mx = fmax(mx, var1 / css / css);
  }
  sh[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  // non-negative doubles order as their bit patterns
  if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(sh[0]));
}

template <typename T>
__global__ void k_nscbc_inflow(Geo g, DevT<T> d, double mach, const double* inflow, double extent,
                               const unsigned long long* gmach, double* B) {
  const long long nf = (long long)(g.jm + 1) * (g.km + 1);
  const long long fj = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (fj >= nf) return;
  const int j = (int)(fj % (g.jm + 1)), k = (int)(fj / (g.jm + 1));
  auto M = [](double x, double y) { return __dmul_rn(x, y); };
  auto A = [](double x, double y) { return __dadd_rn(x, y); };
  auto S = [](double x, double y) { return __dsub_rn(x, y); };
  const long long nh = g.nh, p = hidx(g, 0, j, k), pa = hidx(g, 1, j, k);
  const double gm2 = __longlong_as_double((long long)*gmach);
  const double rho = (double)d.pr[p], u = (double)d.pr[p + nh], v = (double)d.pr[p + 2 * nh];
  const double w = (double)d.pr[p + 3 * nh], pr = (double)d.pr[p + 4 * nh], t = (double)d.pr[p + 5 * nh];
  const double J = d.jac64[p];
  double q[5];
  for (int m = 0; m < 5; ++m) q[m] = (double)d.q[p + m * nh];
  const double ddi[3] = {nscbc_x(g, d, 0, 0, p), nscbc_x(g, d, 0, 1, p), nscbc_x(g, d, 0, 2, p)};
  // pmatrix (src/bc.F90:5516-5611)
  const double c = sqrt(t) / mach;
  const double vr = 1.0 / sqrt(A(A(M(ddi[0], ddi[0]), M(ddi[1], ddi[1])), M(ddi[2], ddi[2])));
  const double nx = M(ddi[0], vr), ny = M(ddi[1], vr), nz = M(ddi[2], vr);
  const double phi = M(0.5 * (1.4 - 1.0), A(A(M(u, u), M(v, v)), M(w, w)));
  const double VV = A(A(M(nx, u), M(ny, v)), M(nz, w));
  const double a1 = 1.4 - 1.0, cc = M(c, c);
  const double a2 = 1.0 / M(M(sqrt(2.0), rho), c);
  const double a3 = rho / M(c, sqrt(2.0));
  const double a4 = A(phi, cc) / (1.4 - 1.0);
  const double a5 = S(1.0, phi / cc);
  const double a6 = phi / (1.4 - 1.0);
  const double n3[3] = {nx, ny, nz};
  double Pi[5][5], Pn[5][5];
  Pi[0][0] = S(M(nx, a5), S(M(nz, v), M(ny, w)) / rho);
  Pi[0][1] = M(M(nx, a1), u) / cc;
  Pi[0][2] = A(M(M(nx, a1), v) / cc, nz / rho);
  Pi[0][3] = S(M(M(nx, a1), w) / cc, ny / rho);
  Pi[1][0] = S(M(ny, a5), S(M(nx, w), M(nz, u)) / rho);
  Pi[1][1] = S(M(M(ny, a1), u) / cc, nz / rho);
  Pi[1][2] = M(M(ny, a1), v) / cc;
  Pi[1][3] = A(M(M(ny, a1), w) / cc, nx / rho);
  Pi[2][0] = S(M(nz, a5), S(M(ny, u), M(nx, v)) / rho);
  Pi[2][1] = A(M(M(nz, a1), u) / cc, ny / rho);
  Pi[2][2] = S(M(M(nz, a1), v) / cc, nx / rho);
  Pi[2][3] = M(M(nz, a1), w) / cc;
  for (int r = 0; r < 3; ++r) Pi[r][4] = -(M(n3[r], a1) / cc);
  Pi[3][0] = M(a2, S(phi, M(c, VV)));
  Pi[3][1] = -M(a2, S(M(a1, u), M(nx, c)));
  Pi[3][2] = -M(a2, S(M(a1, v), M(ny, c)));
  Pi[3][3] = -M(a2, S(M(a1, w), M(nz, c)));
  Pi[3][4] = M(a1, a2);
  Pi[4][0] = M(a2, A(phi, M(c, VV)));
  Pi[4][1] = -M(a2, A(M(a1, u), M(nx, c)));
  Pi[4][2] = -M(a2, A(M(a1, v), M(ny, c)));
  Pi[4][3] = -M(a2, A(M(a1, w), M(nz, c)));
  Pi[4][4] = M(a1, a2);
  Pn[0][0] = nx; Pn[0][1] = ny; Pn[0][2] = nz; Pn[0][3] = a3; Pn[0][4] = a3;
  Pn[1][0] = M(nx, u); Pn[1][1] = S(M(ny, u), M(nz, rho)); Pn[1][2] = A(M(nz, u), M(ny, rho));
  Pn[1][3] = M(a3, A(u, M(nx, c))); Pn[1][4] = M(a3, S(u, M(nx, c)));
  Pn[2][0] = A(M(nx, v), M(nz, rho)); Pn[2][1] = M(ny, v); Pn[2][2] = S(M(nz, v), M(nx, rho));
  Pn[2][3] = M(a3, A(v, M(ny, c))); Pn[2][4] = M(a3, S(v, M(ny, c)));
  Pn[3][0] = S(M(nx, w), M(ny, rho)); Pn[3][1] = A(M(ny, w), M(nx, rho)); Pn[3][2] = M(nz, w);
  Pn[3][3] = M(a3, A(w, M(nz, c))); Pn[3][4] = M(a3, S(w, M(nz, c)));
  Pn[4][0] = A(M(nx, a6), M(rho, S(M(nz, v), M(ny, w))));
  Pn[4][1] = A(M(ny, a6), M(rho, S(M(nx, w), M(nz, u))));
  Pn[4][2] = A(M(nz, a6), M(rho, S(M(ny, u), M(nx, v))));
  Pn[4][3] = M(a3, A(a4, M(c, VV))); Pn[4][4] = M(a3, S(a4, M(c, VV)));
  // normal flux difference, E/F/G at the node, metric derivatives
  double e0[5], e1[5];
  nscbc_flux(g, d, 0, p, e0);
  nscbc_flux(g, d, 0, pa, e1);
  const double E[5] = {q[1], A(M(q[1], u), pr), M(q[2], u), M(q[3], u), M(A(q[4], pr), u)};
  const double F[5] = {q[2], M(q[1], v), A(M(q[2], v), pr), M(q[3], v), M(A(q[4], pr), v)};
  const double G[5] = {q[3], M(q[1], w), M(q[2], w), A(M(q[3], w), pr), M(A(q[4], pr), w)};
  double jcbi[3];
  for (int m = 0; m < 3; ++m) jcbi[m] = A(-M(ddi[m], J), M(nscbc_x(g, d, 0, m, pa), d.jac64[pa]));
  double rest[5], l1[5], lodi[5];
  for (int n = 0; n < 5; ++n) {
    rest[n] = A(A(M(E[n], jcbi[0]), M(F[n], jcbi[1])), M(G[n], jcbi[2]));
    l1[n] = S(A(-e0[n], e1[n]), rest[n]);
  }
  for (int r = 0; r < 5; ++r) {
    double acc = 0.0;
    for (int m = 0; m < 5; ++m) acc = A(acc, M(Pi[r][m], l1[m]));
    lodi[r] = acc / J;
  }
  const double kin = M(M(0.25, S(1.0, gm2)), c) / extent;
  const long long fo = fj;
  const double ui = inflow[fo], vi = inflow[fo + nf], wi = inflow[fo + 2 * nf];
  const double pin = inflow[4 * nf + (g.jm + 1) + fo];
  const double x1 = M(ddi[0], vr), x2 = M(ddi[1], vr), x3 = M(ddi[2], vr);
  lodi[0] = 0.0;
  lodi[1] = M(M(kin, 0.5), S(M(x1, S(w, wi)), M(x3, S(u, ui))));
  lodi[2] = M(M(kin, 0.5), A(-M(x1, S(v, vi)), M(x2, S(u, ui))));
  lodi[3] = M(kin, A(A(A(M(x1, S(u, ui)), M(x2, S(v, vi))), M(x3, S(w, wi))), S(pr, pin) / rho / c));
  double b[5];
  for (int r = 0; r < 5; ++r) {
    double acc = 0.0;
    for (int m = 0; m < 5; ++m) acc = A(acc, M(Pn[r][m], lodi[m]));
    b[r] = A(0.0, A(M(acc, J), rest[r]));
  }
  // tangential derivatives of the face (y, and z in 3-D)
  double fp[5], fm[5];
  nscbc_flux(g, d, 1, hidx(g, 0, j + 1, k), fp);
  nscbc_flux(g, d, 1, hidx(g, 0, j - 1, k), fm);
  for (int n = 0; n < 5; ++n) b[n] = A(b[n], M(0.5, S(fp[n], fm[n])));
  if (g.ndims == 3) {
    nscbc_flux(g, d, 2, hidx(g, 0, j, k + 1), fp);
    nscbc_flux(g, d, 2, hidx(g, 0, j, k - 1), fm);
    for (int n = 0; n < 5; ++n) b[n] = A(b[n], M(0.5, S(fp[n], fm[n])));
  }
  for (int n = 0; n < 5; ++n) B[n * nf + fj] = b[n];
}

template <typename T>
__global__ void k_nscbc_apply(Geo g, DevT<T> d, const double* B) {
  const long long nf = (long long)(g.jm + 1) * (g.km + 1);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 5 * nf) return;
  const int n = (int)(t / nf);
  const long long fj = t % nf;
  const int j = (int)(fj % (g.jm + 1)), k = (int)(fj / (g.jm + 1));
  T* r = d.qrhs + (long long)n * g.n0 + zidx(g, 0, j, k);
  *r = (T)__dsub_rn((double)*r, B[t]);
}

// Channel volume sums, one thread per (i, k) column, i = 1..im, k = 1..km
// (k = 0 in 2-D), fixed order within a column and across the block:
// [0..3] trapezoid integrals over y of q(1..4) (src_chan,
// src/solver.F90:317-331; massfluxchan, src/statistic.F90:1437-1476);
// [4] the wall friction sum of fbcxchan (src/statistic.F90:1303-1367),
// miu(T) * du/dy at j = 0 minus at j = jm.  Block partials: 5 per block.
template <typename T>
__global__ void k_chan_sums(Geo g, DevT<T> d, Phys ph, const double* ycoord, double* part) {
  __shared__ double sh[5][256];
  const long long ncol = (long long)g.im * (g.ndims == 3 ? g.km : 1);
  const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (col < ncol) {
    const int i = 1 + (int)(col % g.im);
    const int k = g.ndims == 3 ? 1 + (int)(col / g.im) : 0;
    const long long nh = g.nh, n0 = g.n0;
    double prev[4];
    long long p = hidx(g, i, 0, k), z = zidx(g, i, 0, k);
    for (int m = 0; m < 4; ++m) prev[m] = q64(d, p, z, m, nh, n0);
    double yprev = ycoord[p];
    for (int j = 1; j <= g.jm; ++j) {
      p = hidx(g, i, j, k);
      z = zidx(g, i, j, k);
      const double yj = ycoord[p];
      const double dy = yj - yprev;
      yprev = yj;
      for (int m = 0; m < 4; ++m) {
        const double cur = q64(d, p, z, m, nh, n0);
        acc[m] = acc[m] + 0.5 * (prev[m] + cur) * dy;
        prev[m] = cur;
      }
    }
    for (int side = 0; side < 2; ++side) {
      const int j = side ? g.jm : 0;
      const double tt = (double)d.pr[hidx(g, i, j, k) + 5 * nh];
      const double miu = tt * sqrt(tt) * ph.tempconst1 / (tt + ph.tempconst) * ph.rreynolds;
      const double dudy = (double)d.grad[3 * n0 + zidx(g, i, j, k)];  // dvel(i,j,k,1,2)
      acc[4] = side ? acc[4] - miu * dudy : acc[4] + miu * dudy;
    }
  }
  for (int m = 0; m < 5; ++m) sh[m][threadIdx.x] = acc[m];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int m = 0; m < 5; ++m) sh[m][threadIdx.x] += sh[m][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 5) part[5 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// Channel controller, one thread: bulk velocity for src_chan every stage;
// at stage 1 from the second step on, statcal's mass flux, wall friction,
// target and the body force of chanfoce (src/statistic.F90:641-657,
// 1494-1533; uinf = ref_len = 1).
__global__ void k_chan_final(const double* part, int nblk, double* chan, double norm, double ly,
                             double dt, long long nstep, int statcal) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double sum[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < nblk; ++b)
    for (int m = 0; m < 5; ++m) sum[m] += part[5 * b + m];
  if (statcal) {
    const double fbcx = sum[4] / norm;
    const double massflux = sum[1] / norm;
    chan[CHAN_FBCX] = fbcx;
    chan[CHAN_MASSFLUX] = massflux;
    if (fabs(chan[CHAN_TARGET]) < 1e-16) {
      chan[CHAN_TARGET] = massflux;
      chan[CHAN_FORCE] = 0.0;
      chan[CHAN_FORCE + 1] = 0.0;
      chan[CHAN_FORCE + 2] = 0.0;
    }
    const double f = chan[CHAN_FORCE], tgt = chan[CHAN_TARGET];
    double fnew;
    if (nstep == 0) {
      fnew = fbcx / ly;
    } else {
      const double gn = ly * f - fbcx;
      const double qn1 = massflux + dt * gn;
      fnew = f - (2.0 * (qn1 - tgt) - 0.2 * (massflux - tgt)) / ly;
    }
    chan[CHAN_FORCE] = fnew;
  }
  chan[CHAN_UBULK] = sum[1] / sum[0];
  chan[CHAN_UBULK + 1] = sum[2] / sum[0];
  chan[CHAN_UBULK + 2] = sum[3] / sum[0];
}

// src_chan applied to qrhs itself (the per-routine rhscal entry point; the
// stage loop folds it into the RK3 update instead).
template <typename T>
__global__ void k_chan_src(Geo g, DevT<T> d) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const double J = d.jac64[hidx(g, i, j, k)];
  const double* C = d.chan;
  for (int m = 1; m < 5; ++m) {
    const double f = m < 4 ? C[CHAN_FORCE + m - 1]
                           : C[CHAN_FORCE] * C[CHAN_UBULK] + C[CHAN_FORCE + 1] * C[CHAN_UBULK + 1] +
                                 C[CHAN_FORCE + 2] * C[CHAN_UBULK + 2];
    T* R = d.qrhs + m * g.n0 + idx;
    *R = (T)((double)*R + f * J);
  }
}

// crashcheck (src/mainloop.F90:709-812) on every interior node: a node
// crashes when q1 >= 0 does not hold (negative or NaN density).  out[0]
// counts them, out[1] keeps the smallest interior linear index.
template <typename T>
__global__ void k_crashcheck(Geo g, DevT<T> d, unsigned long long* out) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const double q1 = q64(d, hidx(g, i, j, k), idx, 0, g.nh, g.n0);
  if (!(q1 >= 0.0)) {
    atomicAdd(out, 1ULL);
    atomicMin(out + 1, (unsigned long long)idx);
  }
}

// --- Crash control (lcracon): databakup, crinod, crashfix ----------------
// src/mainloop.F90:709-1198.  Snapshots hold the interior conserved state
// in FP64 (the FP32-storage form's master) plus the channel controller.
template <typename T>
__global__ void k_snap_save(Geo g, DevT<T> d, double* dst) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k);
  for (int m = 0; m < 5; ++m) dst[m * g.n0 + idx] = q64(d, p, idx, m, g.nh, g.n0);
}
template <typename T>
__global__ void k_snap_load(Geo g, DevT<T> d, const double* src) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k);
  for (int m = 0; m < 5; ++m) {
    const double v = src[m * g.n0 + idx];
    d.q[m * g.nh + p] = (T)v;
    if (d.qm) d.qm[m * g.n0 + idx] = v;
  }
}
// crashcheck's node test (q1 >= 0 fails: negative or NaN density) into the
// critical-node mask
template <typename T>
__global__ void k_crinod_mark(Geo g, DevT<T> d, unsigned char* crinod) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  if (!(q64(d, hidx(g, i, j, k), idx, 0, g.nh, g.n0) >= 0.0)) crinod[idx] = 1;
}
// crinod_expansion (src/mainloop.F90:985-1033): every critical node marks
// its 3x3x3 neighbourhood (interior nodes here; the reference's mask also
// spans two halo layers, which no computation reads)
__global__ void k_crinod_expand(Geo g, const unsigned char* in, unsigned char* out) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  unsigned char v = 0;
  for (int kk = -1; kk <= 1 && !v; ++kk)
    for (int jj = -1; jj <= 1 && !v; ++jj)
      for (int ii = -1; ii <= 1 && !v; ++ii) {
        const int a = i + ii, b = j + jj, e = k + kk;
        if (a < 0 || a > g.im || b < 0 || b > g.jm || e < 0 || e > g.km) continue;
        v = in[zidx(g, a, b, e)];
      }
  out[idx] = v;
}
// crashfix, pass 1 (src/mainloop.F90:1045-1198): nodes whose density,
// pressure or temperature is below its floor (or not a number) are flagged
// and marked critical; count[0] counts them.
template <typename T>
__global__ void k_crashfix_flag(Geo g, DevT<T> d, double eps_rho, double eps_prs, double eps_tmp,
                                unsigned char* flag, unsigned char* crinod, unsigned long long* count) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k);
  const double ro = d.pr[p], pp = d.pr[p + 4 * g.nh], tt = d.pr[p + 5 * g.nh];
  const bool bad = !(ro >= eps_rho && pp >= eps_prs && tt >= eps_tmp);
  flag[idx] = bad ? 1 : 0;
  if (bad) {
    crinod[idx] = 1;
    atomicAdd(count, 1ULL);
  }
}
// crashfix, pass 2: one block walks the interior in the reference's loop
// order (i fastest) and, node by node, replaces q at each flagged node by
// the mean of its 26 neighbours whose rho, p and T are non-negative
// (neighbours outside the domain in i or j skipped, as the reference's
// ig0/jg0 test does; k neighbours may be halo nodes), then recovers that
// node's primitives; later nodes see the earlier fixes, as in the serial
// loop.  Returns at once when pass 1 flagged nothing.
template <typename T>
__global__ void k_crashfix_apply(Geo g, DevT<T> d, Phys ph, const unsigned char* flag,
                                 unsigned long long* count) {
  if (count[0] == 0) return;
  __shared__ int any;
  const long long n0 = g.n0;
  for (long long base = 0; base < n0; base += blockDim.x) {
    const long long idx = base + threadIdx.x;
    const bool f = idx < n0 && flag[idx];
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    if (f) any = 1;
    __syncthreads();
    if (!any) continue;
    if (threadIdx.x == 0) {
      for (int t = 0; t < (int)blockDim.x && base + t < n0; ++t) {
        const long long z = base + t;
        if (!flag[z]) continue;
        const int i = (int)(z % g.I), j = (int)((z / g.I) % (g.jm + 1)), k = (int)(z / g.IJ);
        double qa[5] = {0, 0, 0, 0, 0};
        int norm = 0;
        // kk runs over -1..1 in 2-D as well: the reference reads the k halo
        // planes (copies of plane 0 as the last qswap left them)
        for (int kk = -1; kk <= 1; ++kk)
          for (int jj = -1; jj <= 1; ++jj)
            for (int ii = -1; ii <= 1; ++ii) {
              if (ii == 0 && jj == 0 && kk == 0) continue;
              const int a = i + ii, b = j + jj, e = k + kk;
              if (a < 0 || a > g.im || b < 0 || b > g.jm) continue;
              const long long pn = hidx(g, a, b, e);
              const double ro = d.pr[pn], pp = d.pr[pn + 4 * g.nh], tt = d.pr[pn + 5 * g.nh];
              if (ro >= 0.0 && pp >= 0.0 && tt >= 0.0) {
                const bool inner = e >= 0 && e <= g.km;
                for (int m = 0; m < 5; ++m)
                  qa[m] += inner ? q64(d, pn, zidx(g, a, b, e), m, g.nh, g.n0) : (double)d.q[m * g.nh + pn];
                ++norm;
              }
            }
        if (norm >= 1) {
          const long long p = hidx(g, i, j, k);
          for (int m = 0; m < 5; ++m) {
            const double v = qa[m] / (double)norm;
            d.q[m * g.nh + p] = (T)v;
            if (d.qm) d.qm[m * n0 + z] = v;
          }
          q2fvar_store(g, d, ph, p);
          atomicAdd(count + 1, 1ULL);
        }
      }
    }
    __syncthreads();
  }
}

// cflcal (src/commcal.F90:27-87), diagonal metrics: per direction the
// largest of 0 and dxi(d,d)*u_d + sqrt(T)/mach*|dxi(d,d)| over the interior
// nodes.  The maxima are non-negative, so their bit patterns order like the
// values and atomicMax on them is exact and order-independent.
template <typename T>
__global__ void k_cflcal(Geo g, DevT<T> d, double rmach, unsigned long long* out3) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m[3] = {0.0, 0.0, 0.0};
  if (point_of(g, idx, i, j, k)) {
    const long long p = hidx(g, i, j, k), nh = g.nh;
    const double css = sqrt((double)d.pr[p + 5 * nh]) * rmach;
    for (int dd = 0; dd < g.ndims; ++dd) {
      double ub, cs;
      if (d.xg) {  // general metrics: the whole row of dxi
        const double x0 = (double)d.xg[(3 * dd) * nh + p], x1 = (double)d.xg[(3 * dd + 1) * nh + p];
        const double x2 = (double)d.xg[(3 * dd + 2) * nh + p];
        ub = x0 * (double)d.pr[p + nh] + x1 * (double)d.pr[p + 2 * nh] + x2 * (double)d.pr[p + 3 * nh];
        cs = css * sqrt(x0 * x0 + x1 * x1 + x2 * x2);
      } else {
        const double x = (double)d.xd[p + dd * nh];
        ub = x * (double)d.pr[p + (1 + dd) * nh];
        cs = css * fabs(x);
      }
      m[dd] = fmax(0.0, fmax(ub, fmax(ub - cs, ub + cs)));
    }
  }
  for (int dd = 0; dd < 3; ++dd) {
    double v = m[dd];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
    if ((threadIdx.x & 31) == 0 && v > 0.0) atomicMax(out3 + dd, (unsigned long long)__double_as_longlong(v));
  }
}

// General metrics: the gradients the sweeps stored as derivatives along
// xi_d become physical ones, dvel(n,m) = sum_d d(u_n)/d(xi_d) dxi(d,m) and
// the same for T, summed over d = x, y(, z) in that order (gradcal,
// src/comsolver.F90:244-497).
template <typename T>
__global__ void k_gradphys(Geo g, DevT<T> d) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k), nh = g.nh, n0 = g.n0;
  T* G = d.grad + idx;
  T r[4][3];
  for (int v = 0; v < 4; ++v)
    for (int dd = 0; dd < 3; ++dd)
      r[v][dd] = dd < g.ndims ? G[(v < 3 ? v + 3 * dd : 9 + dd) * n0] : T(0);
  for (int v = 0; v < 4; ++v)
    for (int m = 0; m < 3; ++m) {
      T acc = r[v][0] * d.xg[(0 + m) * nh + p];
      acc = acc + r[v][1] * d.xg[(3 + m) * nh + p];
      if (g.ndims == 3) acc = acc + r[v][2] * d.xg[(6 + m) * nh + p];
      G[(v < 3 ? v + 3 * m : 9 + m) * n0] = acc;
    }
}

// kenergycal / enstophycal (src/statistic.F90:871-992) as a point kernel
// (general metrics), one partial pair per block, reduced by k_stats_final.
template <typename T>
__global__ void k_stats_pt(Geo g, DevT<T> d) {
  __shared__ double sk[256], se[256];
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0, en = 0.0;
  if (point_of(g, idx, i, j, k)) {
    const bool ink = g.ndims == 3 ? (k >= 1 && k <= g.km) : (k == 0);
    if (i >= 1 && j >= 1 && ink) {
      const long long p = hidx(g, i, j, k), nh = g.nh, n0 = g.n0;
      const double ro = d.pr[p], u = d.pr[p + nh], v = d.pr[p + 2 * nh], w = d.pr[p + 3 * nh];
      ke = ro * (u * u + v * v + w * w);
      const T* G = d.grad + idx;
      const double o3 = (double)G[1 * n0] - (double)G[3 * n0];
      double om = o3 * o3;
      if (g.ndims == 3) {
        const double o1 = (double)G[5 * n0] - (double)G[7 * n0];
        const double o2 = (double)G[6 * n0] - (double)G[2 * n0];
        om = o1 * o1 + o2 * o2 + o3 * o3;
      }
      en = ro * om;
    }
  }
  sk[threadIdx.x] = ke;
  se[threadIdx.x] = en;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if ((int)threadIdx.x < s2) {
      sk[threadIdx.x] += sk[threadIdx.x + s2];
      se[threadIdx.x] += se[threadIdx.x + s2];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    d.part[2 * blockIdx.x] = sk[0];
    d.part[2 * blockIdx.x + 1] = se[0];
  }
}

// Fixed-order reduction of the per-warp statistics partials.
__global__ void k_stats_final(const double* part, long long nw, double* out) {
  __shared__ double sk[1024], se[1024];
  double ke = 0.0, en = 0.0;
  for (long long w = threadIdx.x; w < nw; w += blockDim.x) {
    ke += part[2 * w];
    en += part[2 * w + 1];
  }
  sk[threadIdx.x] = ke;
  se[threadIdx.x] = en;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sk[threadIdx.x] += sk[threadIdx.x + s];
      se[threadIdx.x] += se[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sk[0];
    out[1] = se[0];
  }
}

// Precision conversions of whole arrays (upload / download of the FP32 form).
__global__ void k_to_float(const double* a, float* b, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __double2float_rn(a[i]);
}
__global__ void k_to_double(const float* a, double* b, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}
__global__ void k_reciprocal(const double* a, double* b, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i] != 0.0 ? 1.0 / a[i] : 0.0;
}
// interior of a halo-layout array <-> interior-layout array
__global__ void k_halo_to_interior(Geo g, const double* h, double* z) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  z[idx] = h[hidx(g, i, j, k)];
}
// h holds the FP32 copy widened to FP64; interior points take the FP64
// master plus the change the FP32 copy received since the last RK3 update.
__global__ void k_master_to_halo(Geo g, const double* z, double* h) {
  int i, j, k;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!point_of(g, idx, i, j, k)) return;
  const long long p = hidx(g, i, j, k);
  const double master = z[idx];
  const float inc = (float)h[p] - __double2float_rn(master);
  h[p] = master + (double)inc;
}

// FP64 FMA throughput probe: eight independent register-resident chains.
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Host-side scheme set-up (restates fd_scheme_initiate,
// src/derivative.F90:63-158; compact_filter_initiate, src/filter.F90:31-100;
// filter_coefficient_cal, src/filter.F90:299-432; tridiagonal_thomas_
// proprocess, src/commfunc.F90:752-774) plus the chunk carry weights and the
// ac2-folded interior coefficients.
// ---------------------------------------------------------------------------
const double H_NUM1D3 = 1.0 / 3.0;
const double H_NUM7D9 = 7.0 / 9.0;
const double H_NUM1D36 = 1.0 / 36.0;

struct HostFTab {
  double c10[6], c8[5], c6[4], cb[3][7], ch[3][11];
};

struct HostScheme {
  int first = 0, n = 0, ntype = 3, dim = 0;
  bool filter = false;
  std::vector<double> a, c, ac1, ac2, ac3, G, H, K, KD;
  int ulo = 1, uhi = 0;  // uniform chunks (empty range by default)
  double u_ac1 = 0.0, u_ac3 = 0.0, u_K[6] = {0, 0, 0, 0, 0, 0}, u_KD[5] = {0, 0, 0, 0, 0};

  // Chunks whose rows all carry the steady Thomas factors bit for bit and
  // no boundary row (derivative: row 0, n-1, and with walls 1, n-2; filter:
  // 3 end rows, 5 with walls).
  void find_uniform(int CH) {
    const int spec = filter ? (ntype == 4 ? 5 : 3) : (ntype == 4 ? 2 : 1);
    const int m = n / 2;
    if (m < spec || m > n - 1 - spec) return;
    auto same = [&](int r) {
      return ac1[r] == ac1[m] && ac2[r] == ac2[m] && ac3[r] == ac3[m] && a[r] == a[m] &&
             c[r] == c[m];
    };
    int rlo = m, rhi = m;
    while (rlo - 1 >= spec && same(rlo - 1)) --rlo;
    while (rhi + 1 <= n - 1 - spec && same(rhi + 1)) ++rhi;
    ulo = (rlo + CH - 1) / CH;
    uhi = (rhi + 1) / CH - 1;
    u_ac1 = ac1[m];
    u_ac3 = ac3[m];
    const int nk = filter ? 6 : 2;
    const size_t ks = K.size() / nk;  // row stride: n, or the padded row count
    for (int j = 0; j < nk; ++j) u_K[j] = K[(size_t)j * ks + m];
    if (filter)
      for (int j = 0; j < 5; ++j) u_KD[j] = KD[(size_t)j * ks + m];
  }
  // np: rows of the stored arrays (n, or 32 x CH for the tiled sweeps,
  // whose rows past n decouple: a = c = 0, so ac1 = ac3 = 0 there, the
  // carry weights vanish across them, and their coefficients are zero).
  void finish(int CH, const HostFTab& t, int np = 0) {
    if (np < n) np = n;
    a.resize(np, 0.0);
    c.resize(np, 0.0);
    ac1.assign(np, 0.0); ac2.assign(np, 0.0); ac3.assign(np, 0.0);
    ac1[0] = c[0];
    for (int i = 1; i < np; ++i) {
      ac1[i] = c[i] / (1.0 - a[i] * ac1[i - 1]);
      ac2[i] = 1.0 / (1.0 - a[i] * ac1[i - 1]);
      ac3[i] = a[i] / (1.0 - a[i] * ac1[i - 1]);
    }
    for (int i = n; i < np; ++i) ac2[i] = 0.0;
    G.assign(np, 0.0); H.assign(np, 0.0);
    for (int s = 0; s < np; s += CH) {
      const int e = std::min(s + CH, np) - 1;
      double p = 1.0;
      for (int r = s; r <= e; ++r) { p *= -ac3[r]; G[r] = p; }
      p = 1.0;
      for (int r = e; r >= s; --r) { p *= -ac1[r]; H[r] = p; }
    }
    // ac2-folded interior coefficients (row 0 is never an interior row)
    const size_t ks = (size_t)np;
    if (filter) {
      K.assign(6 * ks, 0.0);
      KD.assign(5 * ks, 0.0);
      for (int r = 0; r < n; ++r) {
        K[r] = 2.0 * t.c10[0] * ac2[r];
        for (int m = 1; m < 6; ++m) K[m * ks + r] = t.c10[m] * ac2[r];
        // second-difference weights of (B - A) f on interior rows
        KD[r] = (t.c10[1] - a[r]) * ac2[r];
        for (int m = 2; m < 6; ++m) KD[(m - 1) * ks + r] = t.c10[m] * ac2[r];
      }
    } else {
      K.assign(2 * ks, 0.0);
      for (int r = 0; r < n; ++r) {
        K[r] = H_NUM7D9 * ac2[r];
        K[ks + r] = H_NUM1D36 * ac2[r];
      }
    }
    find_uniform(CH);
  }
};

HostScheme make_deriv(int ntype, int dim, int CH, const HostFTab& t, int np = 0) {
  HostScheme s;
  int i0 = ntype == 4 ? 0 : -1, im = ntype == 4 ? dim : dim + 1;
  s.first = i0; s.n = im - i0 + 1; s.ntype = ntype; s.dim = dim;
  s.a.assign(s.n, H_NUM1D3); s.c.assign(s.n, H_NUM1D3);
  s.a[0] = s.c[0] = 0.0;
  s.a[s.n - 1] = s.c[s.n - 1] = 0.0;
  if (ntype == 4) {
    s.a[0] = s.c[0] = 2.0;
    s.a[1] = s.c[1] = 0.25;
    s.a[s.n - 1] = s.c[s.n - 1] = 2.0;
    s.a[s.n - 2] = s.c[s.n - 2] = 0.25;
  }
  s.finish(CH, t, np);
  return s;
}

HostScheme make_filter(int ntype, int dim, double alfa, int CH, const HostFTab& t, int np = 0) {
  HostScheme s;
  int i0 = ntype == 4 ? 0 : -3, im = ntype == 4 ? dim : dim + 3;
  double b = ntype == 4 ? 0.98 : 1.11;
  s.first = i0; s.n = im - i0 + 1; s.ntype = ntype; s.dim = dim; s.filter = true;
  s.a.assign(s.n, alfa); s.c.assign(s.n, alfa);
  s.a[0] = s.c[0] = b;
  s.a[s.n - 1] = s.c[s.n - 1] = b;
  s.finish(CH, t, np);
  return s;
}

// compact_flux_initiate, src/flux.F90:32-112 (scheme 543): rows -2..dim+1
// with explicit central end rows (periodic), or -1..dim with the
// third-order boundary rows (physical boundaries at both ends).
HostScheme make_flux(int ntype, int dim, int wind, double b, int CH, const HostFTab& t) {
  HostScheme s;
  const int i0 = ntype == 4 ? -1 : -2, imx = ntype == 4 ? dim : dim + 1;
  s.first = i0; s.n = imx - i0 + 1; s.ntype = ntype; s.dim = dim;
  const double lo = 0.5 - (1.0 / 6.0) * b, hi = (1.0 / 6.0) + (1.0 / 6.0) * b;
  s.a.assign(s.n, wind > 0 ? lo : hi);
  s.c.assign(s.n, wind > 0 ? hi : lo);
  s.a[0] = s.c[0] = 0.0;
  s.a[s.n - 1] = s.c[s.n - 1] = 0.0;
  if (ntype == 4) {
    s.a[0] = s.c[0] = 2.0;
    s.a[1] = s.c[1] = 0.25;
    s.a[s.n - 1] = s.c[s.n - 1] = 2.0;
    s.a[s.n - 2] = s.c[s.n - 2] = 0.25;
  }
  s.finish(CH, t);
  s.ulo = 1; s.uhi = 0;  // no uniform chunks (FP64 solves)
  return s;
}

HostFTab make_ftab(double alfa, double bh, double bb) {
  HostFTab t;
  std::memset(&t, 0, sizeof(t));
  t.c6[0] = (11.0 + 10.0 * alfa) / 32.0;
  t.c6[1] = (15.0 + 34.0 * alfa) / 64.0;
  t.c6[2] = (-3.0 + 6.0 * alfa) / 32.0;
  t.c6[3] = (1.0 - 2.0 * alfa) / 64.0;
  t.c8[0] = (93.0 + 70.0 * alfa) / 256.0;
  t.c8[1] = (7.0 + 18.0 * alfa) / 32.0;
  t.c8[2] = (-7.0 + 14.0 * alfa) / 64.0;
  t.c8[3] = (1.0 - 2.0 * alfa) / 32.0;
  t.c8[4] = (-1.0 + 2.0 * alfa) / 256.0;
  t.c10[0] = (193.0 + 126.0 * alfa) / 512.0;
  t.c10[1] = (105.0 + 302.0 * alfa) / 512.0;
  t.c10[2] = (-15.0 + 30.0 * alfa) / 128.0;
  t.c10[3] = (45.0 - 90.0 * alfa) / 1024.0;
  t.c10[4] = (-5.0 + 10.0 * alfa) / 512.0;
  t.c10[5] = (1.0 - 2.0 * alfa) / 1024.0;
  const double cb2[7] = {(-1.0 + 2.0 * alfa) / 64.0, (3.0 + 26.0 * alfa) / 32.0,
                         (49.0 + 30.0 * alfa) / 64.0, (5.0 + 6.0 * alfa) / 16.0,
                         (-15.0 + 30.0 * alfa) / 64.0, (3.0 - 6.0 * alfa) / 32.0,
                         (-1.0 + 2.0 * alfa) / 64.0};
  const double cb1[7] = {(1.0 + 62.0 * alfa) / 64.0, (29.0 + 6.0 * alfa) / 32.0,
                         (15.0 + 34.0 * alfa) / 64.0, (-5.0 + 10.0 * alfa) / 16.0,
                         (15.0 - 30.0 * alfa) / 64.0, (-3.0 + 6.0 * alfa) / 32.0,
                         (1.0 - 2.0 * alfa) / 64.0};
  const double cb0[7] = {(63.0 + 1.0 * bb) / 64.0, (3.0 + 29.0 * bb) / 32.0,
                         (-15.0 + 15.0 * bb) / 64.0, (5.0 - 5.0 * bb) / 16.0,
                         (-15.0 + 15.0 * bb) / 64.0, (3.0 - 3.0 * bb) / 32.0,
                         (-1.0 + 1.0 * bb) / 64.0};
  for (int m = 0; m < 7; ++m) { t.cb[0][m] = cb0[m]; t.cb[1][m] = cb1[m]; t.cb[2][m] = cb2[m]; }
  const double h0[11] = {(-1.0 + 1.0 * bh) / 1024.0, (5.0 - 5.0 * bh) / 512.0,
                         (979.0 + 45.0 * bh) / 1024.0, (15.0 + 113.0 * bh) / 128.0,
                         (-105.0 + 105.0 * bh) / 512.0, (63.0 - 63.0 * bh) / 256.0,
                         (-105.0 + 105.0 * bh) / 512.0, (15.0 - 15.0 * bh) / 128.0,
                         (-45.0 + 45.0 * bh) / 1024.0, (5.0 - 5.0 * bh) / 512.0,
                         (-1.0 + 1.0 * bh) / 1024.0};
  const double h1[11] = {(1.0 - 2.0 * alfa) / 1024.0, (-5.0 + 10.0 * alfa) / 512.0,
                         (45.0 + 934.0 * alfa) / 1024.0, (113.0 + 30.0 * alfa) / 128.0,
                         (105.0 + 302.0 * alfa) / 512.0, (-63.0 + 126.0 * alfa) / 256.0,
                         (105.0 - 210.0 * alfa) / 512.0, (-15.0 + 30.0 * alfa) / 128.0,
                         (45.0 - 90.0 * alfa) / 1024.0, (-5.0 + 10.0 * alfa) / 512.0,
                         (1.0 - 2.0 * alfa) / 1024.0};
  const double h2[11] = {(-1.0 + 2.0 * alfa) / 1024.0, (5.0 - 10.0 * alfa) / 512.0,
                         (-45.0 + 90.0 * alfa) / 1024.0, (15.0 + 98.0 * alfa) / 128.0,
                         (407.0 + 210.0 * alfa) / 512.0, (63.0 + 130.0 * alfa) / 256.0,
                         (-105.0 + 210.0 * alfa) / 512.0, (15.0 - 30.0 * alfa) / 128.0,
                         (-45.0 + 90.0 * alfa) / 1024.0, (5.0 - 10.0 * alfa) / 512.0,
                         (-1.0 + 2.0 * alfa) / 1024.0};
  for (int m = 0; m < 11; ++m) { t.ch[0][m] = h0[m]; t.ch[1][m] = h1[m]; t.ch[2][m] = h2[m]; }
  return t;
}

template <typename T>
FTab<T> cast_ftab(const HostFTab& h) {
  FTab<T> t;
  for (int m = 0; m < 6; ++m) t.c10[m] = (T)h.c10[m];
  for (int m = 0; m < 5; ++m) t.c8[m] = (T)h.c8[m];
  for (int m = 0; m < 4; ++m) t.c6[m] = (T)h.c6[m];
  for (int r = 0; r < 3; ++r) {
    for (int m = 0; m < 7; ++m) t.cb[r][m] = (T)h.cb[r][m];
    for (int m = 0; m < 11; ++m) t.ch[r][m] = (T)h.ch[r][m];
  }
  return t;
}

const int kCH[] = {3, 5, 9, 17, 33};

int pick_ch(int nmax, int nchunks) {
  for (int ch : kCH)
    if (nchunks * ch >= nmax) return ch;
  return -1;
}

thread_local std::string g_create_err;

}  // namespace

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
struct astr_batch;
static void batch_forget(astr_batch* b, astr_ctx* c);

struct astr_ctx {
  astr_dims dm;
  astr_params pm;
  Geo g;
  Phys ph;
  int prec = ASTR_FP64;
  DevT<double> d64;
  DevT<float> d32;
  FTab<double> ft64;
  FTab<float> ft32;
  DScheme<double> fd64[3], fl64[3];
  DScheme<float> fd32[3], fl32[3];
  int CH[3] = {0, 0, 0};   // chunk length of the derivative sweeps per direction
  int CHf[3] = {0, 0, 0};  // chunk length of the filter sweeps per direction
  double* stats_dev = nullptr;
  double* staging = nullptr;  // nh doubles (FP32 form: host <-> device conversions)
  double* staging2 = nullptr; // second buffer: copies overlap conversions
  cudaStream_t cst = nullptr; // copy stream of the host <-> device transfers
  cudaEvent_t ev_copy[2] = {nullptr, nullptr}, ev_use[2] = {nullptr, nullptr};
  cudaEvent_t ev_begin = nullptr;  // the copy stream waits for the context stream
  int xfer = 0;               // transfers issued through the double buffer
  double* jac64 = nullptr;
  double* rjac64 = nullptr;
  cudaStream_t st = nullptr;
  std::string err;
  long long launches = 0;
  bool metrics_set = false, state_set = false;
  double l0 = 1.0;
  // channel (flowtype 'channel')
  bool channel = false, grid_set = false;
  double* chan_dev = nullptr;   // CHAN_N doubles
  double* chan_part = nullptr;  // 5 per block of k_chan_sums
  int chan_nblk = 0;
  double* ycoord = nullptr;     // y coordinates, halo layout
  unsigned char* slip_mask = nullptr;  // 411 on ymin: node (i, k) at x <= xslip
  // 11 or 12 on xmin: vel_in(0:jm,0:km,1:3), tmp_in(0:jm,0:km),
  // tmp_prof(0:jm), prs_in(0:jm,0:km)
  double* inflow = nullptr;
  // 12 on xmin (inflow_nscbc): the residual it adds at i = 0 (5 arrays of
  // the face), the domain-wide Mach-number word, the grid's x extent, and
  // whether a boucon call has left B to be applied after the convection
  double* nscbc_b = nullptr;
  unsigned long long* nscbc_gm = nullptr;
  double nscbc_ext = 0.0;
  bool nscbc_pending = false;
  // 23 on xmax / ymax (index 0 / 1): the face's normal spacing
  // x(dim-1) - x(dim-2) per node and the grid's extent, from the grid
  double* gc_dx[2] = {nullptr, nullptr};
  double gc_ext[2] = {0.0, 0.0};
  double chan_ly = 0.0;         // ymax - ymin
  long long nstep = 0;          // completed time steps (statcal's nstep)
  bool rkfirst_called = false;  // rkfirst's firstcall flag
  // Execution plan of the last sweep direction: bit 0 computes the viscous
  // stress and heat flux in a separate point kernel instead of inside the
  // last convective sweep; bit 1 does the same for the RK3 update (and
  // primitive recovery) after the last viscous sweep.  Same arithmetic.
  // Timed on the 512^3 TGV: bit 0 saves 2 % (FP32 storage), bit 1 costs
  // 1 % (the FP64 master update is FP64-bound either way).
  int split_last = 1;
  // general (non-diagonal) metrics: dxi(d,m) at 3*d + m, allocated when the
  // first non-diagonal set arrives
  bool gen = false;
  void* xg = nullptr;
  // boundary routine and wall temperature of each face (boucon)
  int bct[6] = {0, 0, 0, 0, 0, 0};
  double btw[6] = {0, 0, 0, 0, 0, 0};
  bool has_bc = false;
  // lines per block: one-warp-per-line x layout (warps), block layout (per direction)
  int lbw = X_LINES;
  int lbb[3] = {YZ_LINES, YZ_LINES, YZ_LINES};
  // small grids: the variables of a line spread over blocks (gridDim.z) and
  // the stress, RK3 update and statistics run as point kernels
  bool vsplit = false;
  // tile-staged sweeps (sweeps2.cuh): main ordering, diagonal metrics;
  // padded schemes per direction and their uniform-chunk constants
  bool v2 = false;
  DScheme<double> v2d64[3], v2f64[3];
  DScheme<float> v2d32[3], v2f32[3];
  struct V2U {
    double a1 = 0, a3 = 0, K[6] = {0, 0, 0, 0, 0, 0}, KD[5] = {0, 0, 0, 0, 0}, gp[33] = {}, hp[33] = {};
  } v2ud[3], v2uf[3];
  // crash control (lcracon, src/mainloop.F90:709-1198)
  bool cracon = false, cc_started = false;
  double* snap[2] = {nullptr, nullptr};  // 5 interior FP64 arrays + CHAN_N each
  bool snap_valid[2] = {false, false};
  long long snap_nstep[2] = {0, 0};
  int snap_rec[2] = {0, 0};              // recover_counter of each snapshot
  int datpnt = -1;                       // -1: none yet ('o'), 0: 'a', 1: 'b'
  long long nxtbakup = 0, feqbakup = 5;
  unsigned char* crinod = nullptr;       // critical nodes (interior)
  unsigned char* crinod2 = nullptr;      // expansion scratch
  unsigned char* fixflag = nullptr;      // crashfix: flagged nodes of the pass
  unsigned long long* fixcount = nullptr;  // crashfix: [flagged, wiped] of the pass
  long long recoveries = 0, backups = 0, wiped = 0;
  // compact MP convective scheme (conschm 543c): scratch and schemes
  bool mp = false;
  MPDev mpd{};
  MPSchemes mps{};
  // the batch this case belongs to (astr_batch_add), or none
  astr_batch* batch = nullptr;
  // one RK3 step captured as a CUDA graph (asynchronous stepping)
  cudaGraphExec_t step_graph = nullptr;
  long long graph_kernels = 0;  // kernel launches in one captured step
  std::vector<void*> allocs;
  // profiling: event pairs per launch, by kernel class
  bool prof = false;
  std::vector<cudaEvent_t> ev;
  std::vector<int> ev_cls;
  size_t ev_used = 0;
};

namespace {

template <typename T> DevT<T>& dev(astr_ctx* c);
template <> DevT<double>& dev<double>(astr_ctx* c) { return c->d64; }
template <> DevT<float>& dev<float>(astr_ctx* c) { return c->d32; }
template <typename T> const FTab<T>& ftab(astr_ctx* c);
template <> const FTab<double>& ftab<double>(astr_ctx* c) { return c->ft64; }
template <> const FTab<float>& ftab<float>(astr_ctx* c) { return c->ft32; }
template <typename T> const DScheme<T>& sch_d(astr_ctx* c, int dir);
template <> const DScheme<double>& sch_d<double>(astr_ctx* c, int dir) { return c->fd64[dir]; }
template <> const DScheme<float>& sch_d<float>(astr_ctx* c, int dir) { return c->fd32[dir]; }
template <typename T> const DScheme<T>& sch_f(astr_ctx* c, int dir);
template <> const DScheme<double>& sch_f<double>(astr_ctx* c, int dir) { return c->fl64[dir]; }
template <> const DScheme<float>& sch_f<float>(astr_ctx* c, int dir) { return c->fl32[dir]; }

int fail(astr_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_err = msg;
  return code;
}

int cuda_check(astr_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ASTR_OK;
  return fail(c, e == cudaErrorMemoryAllocation ? ASTR_ERR_OOM : ASTR_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                 \
  do {                                                           \
    int _rc = cuda_check(c, (call), #call);                      \
    if (_rc != ASTR_OK) return _rc;                              \
  } while (0)

#define RC(x)                      \
  do {                             \
    int _r = (x);                  \
    if (_r != ASTR_OK) return _r;  \
  } while (0)

int after_launch(astr_ctx* c, const char* what) {
  ++c->launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(c, ASTR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return ASTR_OK;
}

enum { KC_FILTER = 0, KC_HALO, KC_CONVGRAD, KC_VISC, KC_POINT, KC_STATS, KC_MP, KC_N };

void prof_begin(astr_ctx* c, int cls) {
  if (!c->prof) return;
  if (c->ev_used + 2 > c->ev.size()) {
    for (int k = 0; k < 64; ++k) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      c->ev.push_back(e);
      c->ev_cls.push_back(0);
    }
  }
  c->ev_cls[c->ev_used] = cls;
  cudaEventRecord(c->ev[c->ev_used], c->st);
  c->ev_used += 1;
}

void prof_end(astr_ctx* c) {
  if (!c->prof) return;
  cudaEventRecord(c->ev[c->ev_used], c->st);
  c->ev_used += 1;
}

// Warps of the derivative sweep of direction DIR (one statistics partial
// sum each).
template <int DIR>
long long sweep_warps(const Geo& g, int lbw, const int* lbb) {
  const int lb = warp_lines<DIR>() ? lbw : lbb[DIR];
  const dim3 gr = sweep_grid<DIR>(g, lb), bl = sweep_block<DIR>(lb);
  return (long long)gr.x * gr.y * (bl.x * bl.y / 32);
}

template <typename T>
SweepCtx<T> sctx(astr_ctx* c) {
  return SweepCtx<T>{c->g, dev<T>(c), c->ph, c->st, c->gen, c->lbw, {c->lbb[0], c->lbb[1], c->lbb[2]},
                     c->vsplit ? 1 : 0};
}

int launch_result(astr_ctx* c, cudaError_t e, const char* what) {
  ++c->launches;
  if (e == cudaErrorInvalidValue)
    return fail(c, ASTR_ERR_UNSUPPORTED, std::string(what) + ": no chunk length for this line size");
  if (e != cudaSuccess) return fail(c, ASTR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return ASTR_OK;
}

template <typename T, int DIR>
int launch_filter(astr_ctx* c, int do_q2f) {
  prof_begin(c, KC_FILTER);
  const cudaError_t e = astr::launch_filter<T, DIR>(sctx<T>(c), sch_f<T>(c, DIR), ftab<T>(c),
                                                    c->CHf[DIR], do_q2f);
  prof_end(c);
  return launch_result(c, e, "k_filter");
}

template <typename T, int DIR>
int launch_convgrad(astr_ctx* c, CGFlags f) {
  prof_begin(c, (f.conv || f.grad) ? KC_CONVGRAD : KC_STATS);
  const cudaError_t e = astr::launch_convgrad<T, DIR>(sctx<T>(c), sch_d<T>(c, DIR), c->CH[DIR], f);
  prof_end(c);
  return launch_result(c, e, "k_convgrad");
}

template <typename T, int DIR>
int launch_visc(astr_ctx* c, VFlags f) {
  prof_begin(c, KC_VISC);
  const cudaError_t e = astr::launch_visc<T, DIR>(sctx<T>(c), sch_d<T>(c, DIR), c->CH[DIR], f);
  prof_end(c);
  return launch_result(c, e, "k_visc");
}

template <typename T, int DIR>
int launch_face(astr_ctx* c, bool mini) {
  const Geo& g = c->g;
  const int na = DIR == 0 ? g.jm : g.im;
  const int nb = DIR == 2 ? g.jm : g.km;
  dim3 bl(128), gr((na + 128) / 128, nb + 1);
  prof_begin(c, KC_HALO);
  if (mini) k_bchomo<T, DIR><<<gr, bl, 0, c->st>>>(c->g, dev<T>(c), c->ph);
  else k_qswap<T, DIR><<<gr, bl, 0, c->st>>>(c->g, dev<T>(c), c->ph);
  prof_end(c);
  return after_launch(c, mini ? "k_bchomo" : "k_qswap");
}

dim3 point_grid(long long n) { return dim3((unsigned)((n + 255) / 256)); }

template <typename T, int DIR>
int launch_qhalo(astr_ctx* c) {
  const Geo& g = c->g;
  const int na = DIR == 0 ? g.jm : g.im;
  const int nb = DIR == 2 ? g.jm : g.km;
  prof_begin(c, KC_HALO);
  k_qhalo<T, DIR><<<dim3((na + 128) / 128, nb + 1), 128, 0, c->st>>>(g, dev<T>(c));
  prof_end(c);
  return after_launch(c, "k_qhalo");
}

// The tiled sweeps run where the context built them and the metrics are
// diagonal (the compact MP path keeps the register-window sweeps).
bool use_v2(const astr_ctx* c) { return c->v2 && !c->gen && !c->mp; }

template <typename T> const DScheme<T>& v2_sd(astr_ctx* c, int dir);
template <> const DScheme<double>& v2_sd<double>(astr_ctx* c, int dir) { return c->v2d64[dir]; }
template <> const DScheme<float>& v2_sd<float>(astr_ctx* c, int dir) { return c->v2d32[dir]; }
template <typename T> const DScheme<T>& v2_sf(astr_ctx* c, int dir);
template <> const DScheme<double>& v2_sf<double>(astr_ctx* c, int dir) { return c->v2f64[dir]; }
template <> const DScheme<float>& v2_sf<float>(astr_ctx* c, int dir) { return c->v2f32[dir]; }

template <typename T>
V2Args<T> v2_args(astr_ctx* c, int dir, bool filter) {
  V2Args<T> a;
  a.g = c->g;
  a.d = dev<T>(c);
  a.S = filter ? v2_sf<T>(c, dir) : v2_sd<T>(c, dir);
  a.Tb = ftab<T>(c);
  a.ph = c->ph;
  const astr_ctx::V2U& u = filter ? c->v2uf[dir] : c->v2ud[dir];
  a.a1 = u.a1; a.a3 = u.a3;
  for (int m = 0; m < 6; ++m) a.K[m] = u.K[m];
  for (int m = 0; m < 5; ++m) a.KD[m] = u.KD[m];
  for (int t = 0; t < 33; ++t) { a.gp[t] = u.gp[t]; a.hp[t] = u.hp[t]; }
  return a;
}

template <typename T, int DIR>
int launch2_filter_c(astr_ctx* c) {
  prof_begin(c, KC_FILTER);
  const cudaError_t e = astr::launch2_filter<T, DIR>(v2_args<T>(c, DIR, true), c->st, c->CHf[DIR],
                                                     c->vsplit ? 1 : 0);
  prof_end(c);
  return launch_result(c, e, "k2_filter");
}
template <typename T, int DIR>
int launch2_convgrad_c(astr_ctx* c, CGFlags f) {
  prof_begin(c, KC_CONVGRAD);
  const cudaError_t e = astr::launch2_convgrad<T, DIR>(v2_args<T>(c, DIR, false), c->st, c->CH[DIR], f,
                                                       c->vsplit ? 1 : 0);
  prof_end(c);
  return launch_result(c, e, "k2_convgrad");
}
template <typename T, int DIR>
int launch2_visc_c(astr_ctx* c) {
  prof_begin(c, KC_VISC);
  const cudaError_t e = astr::launch2_visc<T, DIR>(v2_args<T>(c, DIR, false), c->st, c->CH[DIR],
                                                   c->vsplit ? 1 : 0);
  prof_end(c);
  return launch_result(c, e, "k2_visc");
}

template <typename T>
int run_filter(astr_ctx* c, bool q2f_last) {
  const int nd = c->g.ndims;
  // filterq refreshes the q halos of each periodic direction before
  // filtering it; the sweeps read wrapped interior nodes instead, so the
  // copy is made only where a routine reads those halos before the next
  // qswap: inflow_nscbc's tangential derivatives on the xmin face
  const bool halos = c->nscbc_b != nullptr;
  if (use_v2(c) && !q2f_last) {
    if (halos && c->g.per[0]) RC((launch_qhalo<T, 0>(c)));
    RC((launch2_filter_c<T, 0>(c)));
    if (halos && c->g.per[1]) RC((launch_qhalo<T, 1>(c)));
    RC((launch2_filter_c<T, 1>(c)));
    if (halos && nd == 3 && c->g.per[2]) RC((launch_qhalo<T, 2>(c)));
    if (nd == 3) RC((launch2_filter_c<T, 2>(c)));
    return ASTR_OK;
  }
  if (halos && c->g.per[0]) RC((launch_qhalo<T, 0>(c)));
  RC((launch_filter<T, 0>(c, 0)));
  if (halos && c->g.per[1]) RC((launch_qhalo<T, 1>(c)));
  RC((launch_filter<T, 1>(c, (q2f_last && nd == 2) ? 1 : 0)));
  if (halos && nd == 3 && c->g.per[2]) RC((launch_qhalo<T, 2>(c)));
  if (nd == 3) RC((launch_filter<T, 2>(c, q2f_last ? 1 : 0)));
  return ASTR_OK;
}

template <typename T>
int run_qswap(astr_ctx* c) {
  if (c->g.per[0]) RC((launch_face<T, 0>(c, false)));
  if (c->g.per[1]) RC((launch_face<T, 1>(c, false)));
  if (c->g.per[2]) RC((launch_face<T, 2>(c, false)));
  return ASTR_OK;
}

template <typename T>
int run_bchomo(astr_ctx* c) {
  RC((launch_face<T, 0>(c, true)));
  RC((launch_face<T, 1>(c, true)));
  if (c->g.ndims == 3) RC((launch_face<T, 2>(c, true)));
  return ASTR_OK;
}

template <typename T>
int run_convgrad(astr_ctx* c, bool conv, bool grad, bool sigma, bool stats, bool qsave) {
  const int nd = c->g.ndims;
  for (int dir = 0; dir < nd; ++dir) {
    CGFlags f;
    f.conv = conv; f.grad = grad;
    f.first = dir == 0;
    f.last = dir == nd - 1;
    f.sigma = sigma && f.last;
    f.stats = stats && f.last;
    f.qsave = qsave && dir == 0;
    if (use_v2(c) && (conv || grad) && !f.sigma && !f.stats && !f.qsave) {
      const int r2 = dir == 0 ? launch2_convgrad_c<T, 0>(c, f)
                              : (dir == 1 ? launch2_convgrad_c<T, 1>(c, f) : launch2_convgrad_c<T, 2>(c, f));
      RC(r2);
      continue;
    }
    int r = dir == 0 ? launch_convgrad<T, 0>(c, f)
                     : (dir == 1 ? launch_convgrad<T, 1>(c, f) : launch_convgrad<T, 2>(c, f));
    RC(r);
  }
  return ASTR_OK;
}

template <typename T>
int run_visc(astr_ctx* c, bool fuse_rk, bool q2f) {
  const int nd = c->g.ndims;
  for (int dir = 0; dir < nd; ++dir) {
    VFlags f;
    f.last = fuse_rk && dir == nd - 1;
    f.q2f = q2f;
    if (use_v2(c) && !f.last) {
      const int r2 = dir == 0 ? launch2_visc_c<T, 0>(c) : (dir == 1 ? launch2_visc_c<T, 1>(c) : launch2_visc_c<T, 2>(c));
      RC(r2);
      continue;
    }
    int r = dir == 0 ? launch_visc<T, 0>(c, f)
                     : (dir == 1 ? launch_visc<T, 1>(c, f) : launch_visc<T, 2>(c, f));
    RC(r);
  }
  return ASTR_OK;
}

int stats_finish(astr_ctx* c, double* out2) {
  const int last = c->g.ndims - 1;
  // partial sums: one per warp of the last convective sweep, or one per
  // block of the point statistics kernel (general metrics)
  const long long nw = (c->gen || c->vsplit || use_v2(c)) ? (long long)point_grid(c->g.n0).x
                              : (last == 2 ? sweep_warps<2>(c->g, c->lbw, c->lbb)
                                           : (last == 1 ? sweep_warps<1>(c->g, c->lbw, c->lbb)
                                                        : sweep_warps<0>(c->g, c->lbw, c->lbb)));
  prof_begin(c, KC_STATS);
  k_stats_final<<<1, 1024, 0, c->st>>>(c->d64.part, nw, c->stats_dev);
  prof_end(c);
  RC(after_launch(c, "k_stats_final"));
  double h[2];
  CK(cudaMemcpyAsync(h, c->stats_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const astr_dims& dm = c->dm;
  const double npts = c->g.ndims == 3 ? (double)dm.ia * dm.ja * dm.ka : (double)dm.ia * dm.ja;
  if (c->pm.order == ASTR_ORDER_MINIAPP) {
    out2[0] = 0.5 * h[0] / npts;
    out2[1] = 0.5 * h[1] / npts;
  } else {
    const double roinf = 1.0, uinf = 1.0;
    out2[0] = 0.5 * h[0] / npts / (roinf * uinf * uinf);
    out2[1] = 0.5 * h[1] / npts / (roinf * ((uinf / c->l0) * (uinf / c->l0)));
  }
  return ASTR_OK;
}

void set_stage(astr_ctx* c, int s) {
  static const double rk[3][3] = {{1.0, 0.0, 1.0}, {0.75, 0.25, 0.25}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
  c->ph.rk1 = rk[s][0];
  c->ph.rk2 = rk[s][1];
  c->ph.rk3 = rk[s][2];
  c->ph.rk3dt = rk[s][2] * c->ph.dt;
}

template <typename T>
int gradphys_pointwise(astr_ctx* c) {
  prof_begin(c, KC_POINT);
  k_gradphys<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c));
  prof_end(c);
  return after_launch(c, "k_gradphys");
}

template <typename T>
int stats_pointwise(astr_ctx* c) {
  prof_begin(c, KC_STATS);
  k_stats_pt<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c));
  prof_end(c);
  return after_launch(c, "k_stats_pt");
}

template <typename T>
int sigma_pointwise(astr_ctx* c) {
  prof_begin(c, KC_POINT);
  k_sigma<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c), c->ph);
  prof_end(c);
  return after_launch(c, "k_sigma");
}

template <typename T>
int qsave_pointwise(astr_ctx* c) {
  prof_begin(c, KC_POINT);
  k_qsave<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c), c->ph);
  prof_end(c);
  return after_launch(c, "k_qsave");
}

template <typename T>
int rk_pointwise(astr_ctx* c, int q2f) {
  prof_begin(c, KC_POINT);
  k_rkupdate<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c), c->ph, q2f);
  prof_end(c);
  return after_launch(c, "k_rkupdate");
}

constexpr int CHAN_THREADS = 256;

// boucon (src/bc.F90:327-409): the faces' boundary routines in face order.
template <typename T>
int run_boucon(astr_ctx* c) {
  const Geo& g = c->g;
  // refcal (src/solver.F90:102-128): const1 = 1/(gamma (gamma-1) M^2), const6 = 1/(gamma-1)
  const double gamma = 1.4, mach = c->pm.mach;
  const double const1 = 1.0 / (gamma * (gamma - 1.0) * (mach * mach));
  const double const6 = 1.0 / (gamma - 1.0);
  // pinf = roinf tinf / const2 (src/solver.F90:120); outflow's alpha = 0.25
  const double pinf = 1.0 / c->ph.const2, adt = 0.25 * c->pm.deltat;
  for (int n = 0; n < 2 * g.ndims; ++n) {
    const int type = c->bct[n];
    if (type == 12 && n == 0) {
      // inflow_nscbc: the state is read, the residual B kept for rhscal
      prof_begin(c, KC_HALO);
      CK(cudaMemsetAsync(c->nscbc_gm, 0, 8, c->st));
      k_nscbc_gmach<T><<<std::min<long long>((g.n0 + 255) / 256, 4096), 256, 0, c->st>>>(g, dev<T>(c), mach,
                                                                                      c->nscbc_gm);
      RC(after_launch(c, "k_nscbc_gmach"));
      const long long nf = (long long)(g.jm + 1) * (g.km + 1);
      k_nscbc_inflow<T><<<point_grid(nf), 256, 0, c->st>>>(g, dev<T>(c), mach, c->inflow, c->nscbc_ext,
                                                           c->nscbc_gm, c->nscbc_b);
      prof_end(c);
      RC(after_launch(c, "k_nscbc_inflow"));
      c->nscbc_pending = true;
      continue;
    }
    if (type != 41 && type != 42 && type != 50 && type != 60 && type != 421 && type != 21 &&
        type != 51 && type != 411 && type != 11 && type != 23)
      continue;
    const int dir = n / 2;
    const int gi = n == 3 ? 1 : 0;
    const long long cnt = (long long)((dir == 0 ? g.jm : g.im) + 1) * ((dir == 2 ? g.jm : g.km) + 1);
    prof_begin(c, KC_HALO);
    k_face_bc<T><<<point_grid(cnt), 256, 0, c->st>>>(g, dev<T>(c), c->ph, n, type, c->btw[n], const1,
                                                     const6, pinf, adt, mach, c->slip_mask, c->inflow,
                                                     c->gc_dx[gi], c->gc_ext[gi]);
    prof_end(c);
    RC(after_launch(c, "k_face_bc"));
  }
  return ASTR_OK;
}

// inflow_nscbc's residual into qrhs at i = 0, after the convective part and
// its negation (rhscal), so that qrhs(0) = -(B + the convective part)
template <typename T>
int nscbc_apply(astr_ctx* c) {
  const long long n = 5LL * (c->g.jm + 1) * (c->g.km + 1);
  prof_begin(c, KC_POINT);
  k_nscbc_apply<T><<<point_grid(n), 256, 0, c->st>>>(c->g, dev<T>(c), c->nscbc_b);
  prof_end(c);
  c->nscbc_pending = false;
  return after_launch(c, "k_nscbc_apply");
}

// Channel bulk sums and controller for one stage; statcal at stage 1 from
// the second step on (rkfirst, src/mainloop.F90:614-697).
template <typename T>
int run_chan(astr_ctx* c, bool stage1) {
  const bool statcal = stage1 && c->rkfirst_called;
  const double norm = c->g.ndims == 3 ? (double)c->dm.ia * (double)c->dm.ka : (double)c->dm.ia;
  prof_begin(c, KC_STATS);
  k_chan_sums<T><<<c->chan_nblk, CHAN_THREADS, 0, c->st>>>(c->g, dev<T>(c), c->ph, c->ycoord,
                                                          c->chan_part);
  prof_end(c);
  RC(after_launch(c, "k_chan_sums"));
  k_chan_final<<<1, 32, 0, c->st>>>(c->chan_part, c->chan_nblk, c->chan_dev, norm, c->chan_ly,
                                     c->pm.deltat, c->nstep, statcal ? 1 : 0);
  RC(after_launch(c, "k_chan_final"));
  if (stage1) c->rkfirst_called = true;
  return ASTR_OK;
}

// Compact MP convective residual (convrsdcmp, src/solver.F90:1271-1937),
// with the Ducros sensor first when the characteristic decomposition is on
// (rhscal, src/solver.F90:226-230) and rhscal's negation folded into the
// last direction.  qrhs starts from zero (time_integration_rk,
// src/mainloop.F90:408).
int run_mpconv(astr_ctx* c) {
  const Geo& g = c->g;
  const DevT<double>& d = c->d64;
  const MPDev& m = c->mpd;
  CK(cudaMemsetAsync(d.qrhs, 0, 5 * (size_t)g.n0 * sizeof(double), c->st));
  if (m.chard) {
    for (int part = 0; part < 3; ++part) {
      prof_begin(c, KC_MP);
      const cudaError_t e = launch_mp_sensor(g, d, m, c->st, part);
      prof_end(c);
      RC(launch_result(c, e, "k_mp_sensor"));
    }
  }
  const int nd = g.ndims;
  for (int dir = 0; dir < nd; ++dir) {
    cudaError_t e;
    prof_begin(c, KC_MP);
    e = dir == 0 ? launch_mp_split<0>(g, d, m, c->st)
                 : (dir == 1 ? launch_mp_split<1>(g, d, m, c->st) : launch_mp_split<2>(g, d, m, c->st));
    prof_end(c);
    RC(launch_result(c, e, "k_mp_split"));
    prof_begin(c, KC_MP);
    e = dir == 0 ? launch_mp_cflux<0>(g, m, c->mps, c->st)
                 : (dir == 1 ? launch_mp_cflux<1>(g, m, c->mps, c->st) : launch_mp_cflux<2>(g, m, c->mps, c->st));
    prof_end(c);
    RC(launch_result(c, e, "k_mp_cflux"));
    prof_begin(c, KC_MP);
    e = dir == 0 ? launch_mp_face<0>(g, d, m, c->st)
                 : (dir == 1 ? launch_mp_face<1>(g, d, m, c->st) : launch_mp_face<2>(g, d, m, c->st));
    prof_end(c);
    RC(launch_result(c, e, "k_mp_face"));
    if (m.chard) ++c->launches;  // k_mp_face_split before it
    const int last = dir == nd - 1;
    prof_begin(c, KC_MP);
    e = dir == 0 ? launch_mp_diff<0>(g, d, m, c->st, last)
                 : (dir == 1 ? launch_mp_diff<1>(g, d, m, c->st, last) : launch_mp_diff<2>(g, d, m, c->st, last));
    prof_end(c);
    RC(launch_result(c, e, "k_mp_diff"));
  }
  return ASTR_OK;
}

// crashfix after each stage's primitive recovery (lcracon,
// src/mainloop.F90:486): floors eps_rho = eps_tmp = 1e-5 and eps_prs =
// thermal(eps_rho, eps_tmp) = eps_rho eps_tmp / const2 (nondimensional).
template <typename T>
int run_crashfix(astr_ctx* c) {
  const double eps = 1e-5;
  CK(cudaMemsetAsync(c->fixcount, 0, sizeof(unsigned long long), c->st));
  prof_begin(c, KC_POINT);
  k_crashfix_flag<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c), eps, eps * eps / c->ph.const2,
                                                             eps, c->fixflag, c->crinod, c->fixcount);
  prof_end(c);
  RC(after_launch(c, "k_crashfix_flag"));
  k_crashfix_apply<T><<<1, 256, 0, c->st>>>(c->g, dev<T>(c), c->ph, c->fixflag, c->fixcount);
  return after_launch(c, "k_crashfix_apply");
}

template <typename T>
int one_step(astr_ctx* c, double* stats) {
  const bool mini = c->pm.order == ASTR_ORDER_MINIAPP;
  for (int s = 0; s < 3; ++s) {
    set_stage(c, s);
    const bool st1 = s == 0;
    if (mini) {
      RC(run_bchomo<T>(c));
      RC(run_convgrad<T>(c, true, true, c->pm.diffterm != 0, st1 && stats, st1));
      if (c->pm.diffterm) RC(run_visc<T>(c, true, false));
      else RC(rk_pointwise<T>(c, 0));
      RC(run_filter<T>(c, true));
    } else {
      const bool visc = c->pm.diffterm != 0;
      // the tiled sweeps leave the stress, the RK3 base and update and the
      // statistics to point kernels
      const bool v2 = use_v2(c);
      const bool split_sig = visc && ((c->split_last & 1) || c->gen || c->vsplit || v2);
      const bool split_rk = visc && ((c->split_last & 2) || c->vsplit || v2);
      const bool pt_stats = c->gen || c->vsplit || v2;  // statistics by the point kernel
      if (c->pm.lfilter) RC(run_filter<T>(c, false));
      if (c->has_bc) RC(run_boucon<T>(c));
      RC(run_qswap<T>(c));
      if (v2 && st1) RC(qsave_pointwise<T>(c));
      // compact MP: the sweeps give the gradients (and the RK3 base), the
      // convective residual comes from the MP kernels
      RC(run_convgrad<T>(c, !c->mp, true, visc && !split_sig, st1 && stats && !pt_stats, st1 && !v2));
      // general metrics: gradients contracted with the metrics; then the
      // statistics from them where the sweeps do not take them
      if (c->gen) RC(gradphys_pointwise<T>(c));
      if (pt_stats && st1 && stats) RC(stats_pointwise<T>(c));
      if (split_sig) RC(sigma_pointwise<T>(c));
      if (c->mp) RC(run_mpconv(c));
      if (c->nscbc_pending) RC(nscbc_apply<T>(c));
      if (c->channel) RC(run_chan<T>(c, st1));
      if (visc) RC(run_visc<T>(c, !split_rk, !split_rk));
      if (!visc || split_rk) RC(rk_pointwise<T>(c, 1));
      if (c->cracon) RC(run_crashfix<T>(c));
    }
    if (st1 && stats) RC(stats_finish(c, stats));
  }
  c->nstep += 1;
  return ASTR_OK;
}

int step(astr_ctx* c, double* stats) {
  return c->prec == ASTR_FP64 ? one_step<double>(c, stats) : one_step<float>(c, stats);
}

// --- host <-> device in the storage precision ---------------------------
size_t wsize(const astr_ctx* c) { return c->prec == ASTR_FP64 ? 8 : 4; }

// Host <-> device transfers.  The FP64 form copies straight between host
// arrays and fields on the context stream.  The FP32 form goes through two
// FP64 staging buffers: the copy stream moves array k into (or out of)
// buffer k%2 while the context stream converts the other one; events order
// each buffer's copy against its conversion.

// Start of a batch of transfers: the copy stream waits for every kernel
// already queued on the context stream.
int xfer_begin(astr_ctx* c) {
  CK(cudaEventRecord(c->ev_begin, c->st));
  CK(cudaStreamWaitEvent(c->cst, c->ev_begin, 0));
  return ASTR_OK;
}

// Upload: host FP64 array -> staging buffer, ready for conversion on c->st.
int xfer_in(astr_ctx* c, const double* src, size_t n, double** buf) {
  const int b = c->xfer++ & 1;
  *buf = b ? c->staging2 : c->staging;
  CK(cudaStreamWaitEvent(c->cst, c->ev_use[b], 0));
  CK(cudaMemcpyAsync(*buf, src, n * 8, cudaMemcpyHostToDevice, c->cst));
  CK(cudaEventRecord(c->ev_copy[b], c->cst));
  CK(cudaStreamWaitEvent(c->st, c->ev_copy[b], 0));
  return ASTR_OK;
}
// After the conversion kernels that read (upload) or wrote (download) buf.
int xfer_used(astr_ctx* c, const double* buf) {
  const int b = buf == c->staging2 ? 1 : 0;
  CK(cudaEventRecord(c->ev_use[b], c->st));
  return ASTR_OK;
}
// Download: the next free staging buffer for conversions on c->st.
int xfer_out_buf(astr_ctx* c, double** buf) {
  const int b = c->xfer++ & 1;
  *buf = b ? c->staging2 : c->staging;
  CK(cudaStreamWaitEvent(c->st, c->ev_copy[b], 0));  // its previous copy-out is done
  return ASTR_OK;
}
// Download: staging buffer (converted on c->st) -> host array on the copy stream.
int xfer_out(astr_ctx* c, double* dst, const double* buf, size_t n) {
  const int b = buf == c->staging2 ? 1 : 0;
  CK(cudaEventRecord(c->ev_use[b], c->st));
  CK(cudaStreamWaitEvent(c->cst, c->ev_use[b], 0));
  CK(cudaMemcpyAsync(dst, buf, n * 8, cudaMemcpyDeviceToHost, c->cst));
  CK(cudaEventRecord(c->ev_copy[b], c->cst));
  return ASTR_OK;
}
int xfer_sync(astr_ctx* c) {
  CK(cudaStreamSynchronize(c->cst));
  CK(cudaStreamSynchronize(c->st));
  return ASTR_OK;
}

int upload_array(astr_ctx* c, void* dst, const double* src, size_t n) {
  if (c->prec == ASTR_FP64) {
    CK(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyHostToDevice, c->st));
    return ASTR_OK;
  }
  double* buf = nullptr;
  RC(xfer_in(c, src, n, &buf));
  k_to_float<<<point_grid((long long)n), 256, 0, c->st>>>(buf, (float*)dst, (long long)n);
  RC(after_launch(c, "k_to_float"));
  return xfer_used(c, buf);
}

int download_array(astr_ctx* c, double* dst, const void* src, size_t n) {
  if (c->prec == ASTR_FP64) {
    CK(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToHost, c->st));
    return ASTR_OK;
  }
  double* buf = nullptr;
  RC(xfer_out_buf(c, &buf));
  k_to_double<<<point_grid((long long)n), 256, 0, c->st>>>((const float*)src, buf, (long long)n);
  RC(after_launch(c, "k_to_double"));
  return xfer_out(c, dst, buf, n);
}

template <typename T>
int rhscal_t(astr_ctx* c) {
  if (c->mp) RC(run_mpconv(c));
  else RC(run_convgrad<T>(c, true, false, false, false, false));
  if (c->nscbc_pending) RC(nscbc_apply<T>(c));
  if (c->pm.diffterm) {
    prof_begin(c, KC_POINT);
    k_sigma<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c), c->ph);
    prof_end(c);
    RC(after_launch(c, "k_sigma"));
    RC(run_visc<T>(c, false, false));
  }
  if (c->channel) {
    // src_chan with the current force (the force changes at statcal only)
    RC(run_chan<T>(c, false));
    k_chan_src<T><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, dev<T>(c));
    RC(after_launch(c, "k_chan_src"));
  }
  return ASTR_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

// The inflow arrays of bctypes 11 and 12 into HBM: vel_in(0:jm,0:km,1:3),
// tmp_in(0:jm,0:km), tmp_prof(0:jm), prs_in(0:jm,0:km); a NULL array takes
// freestreaminflow's values (src/bc.F90:7950-8003: uinf = 1, vinf = winf
// = 0, tinf = 1, prs_in = thermal(roinf, tinf) = pinf).
static int inflow_upload(astr_ctx* c, const double* vel_in, const double* tmp_in,
                         const double* tmp_prof, const double* prs_in) {
  const size_t nf = (size_t)(c->g.jm + 1) * (c->g.km + 1), nj = (size_t)c->g.jm + 1;
  const double pinf = 1.0 * 1.0 / c->ph.const2;
  std::vector<double> h(5 * nf + nj);
  for (size_t t = 0; t < 3 * nf; ++t) h[t] = vel_in ? vel_in[t] : (t < nf ? 1.0 : 0.0);
  for (size_t t = 0; t < nf; ++t) h[3 * nf + t] = tmp_in ? tmp_in[t] : 1.0;
  for (size_t t = 0; t < nj; ++t) h[4 * nf + t] = tmp_prof ? tmp_prof[t] : 1.0;
  for (size_t t = 0; t < nf; ++t) h[4 * nf + nj + t] = prs_in ? prs_in[t] : pinf;
  for (double v : h)
    if (!std::isfinite(v)) return fail(c, ASTR_ERR_ARG, "inflow arrays: a non-finite value");
  for (size_t t = 3 * nf; t < h.size(); ++t)
    if (!(h[t] > 0.0)) return fail(c, ASTR_ERR_ARG, "inflow temperatures and pressures must be > 0");
  CK(cudaMemcpyAsync(c->inflow, h.data(), h.size() * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return ASTR_OK;
}

size_t astr_gpu_footprint(const astr_dims* dims, const astr_params* params) {
  if (!dims) return 0;
  const size_t nh = (size_t)(dims->im + 2 * HMD + 1) * (dims->jm + 2 * HMD + 1) * (dims->km + 2 * HMD + 1);
  const size_t n0 = (size_t)(dims->im + 1) * (dims->jm + 1) * (dims->km + 1);
  const bool f32 = params && params->precision == ASTR_FP32_STORAGE;
  const size_t w = f32 ? 4 : 8;
  // q 5, primitives 6, metrics 4 (halo arrays, storage type); 1/J (FP64);
  // qrhs 5, gradients 12, sigma 6, heat flux 3 (interior, storage type);
  // qsave 5 (FP64); FP32 form: J, master q 5 and two staging arrays in FP64
  size_t b = w * (15 * nh + 26 * n0) + 8 * (nh + 5 * n0);
  if (f32) b += 8 * (3 * nh + 5 * n0);
  if (params && params->channel) b += 8 * nh;  // y coordinates
  // compact MP: split fluxes 10, compact interface values 10, interface
  // flux 5, sensor 1 (halo arrays, FP64), the shock flags (bytes) and the
  // list of flagged interfaces (at most nh ints)
  if (params && params->conschm == ASTR_CONSCHM_MP) b += 8 * 26 * nh + n0 + 4 * nh;
  if (params && (params->bctype[0] == 11 || params->bctype[0] == 12))  // inflow arrays (+ B)
    b += 8 * ((params->bctype[0] == 12 ? 10 : 5) * (size_t)(dims->jm + 1) * (dims->km + 1) +
              (size_t)(dims->jm + 1) + 1);
  return b;
}

int astr_gpu_create(const astr_dims* dims, const astr_params* params, astr_ctx** out) {
  astr_ctx* c = nullptr;
  if (!dims || !params || !out) return fail(nullptr, ASTR_ERR_ARG, "null argument");
  *out = nullptr;
  const int ndims = dims->ka > 0 ? 3 : 2;
  if (dims->im < 8 || dims->jm < 8 || (ndims == 3 && dims->km < 8) || (ndims == 2 && dims->km != 0))
    return fail(nullptr, ASTR_ERR_ARG, "grid too small (need im,jm(,km) >= 8; km == 0 for 2-D)");
  const int npdc[3] = {dims->npdci, dims->npdcj, dims->npdck};
  for (int i = 0; i < 3; ++i)
    if (npdc[i] != 3 && npdc[i] != 4) return fail(nullptr, ASTR_ERR_UNSUPPORTED, "npdc must be 3 or 4 on one rank");
  if (params->precision != ASTR_FP64 && params->precision != ASTR_FP32_STORAGE)
    return fail(nullptr, ASTR_ERR_ARG, "precision must be ASTR_FP64 or ASTR_FP32_STORAGE");
  if (params->order == ASTR_ORDER_MINIAPP && (npdc[0] != 3 || npdc[1] != 3 || (ndims == 3 && npdc[2] != 3)))
    return fail(nullptr, ASTR_ERR_ARG, "mini-app ordering is periodic only");
  if (ndims == 2 && npdc[2] != 3) return fail(nullptr, ASTR_ERR_ARG, "2-D cases need npdck = 3");
  if (params->channel && (npdc[1] != 4 || params->order != ASTR_ORDER_MAIN || !(params->twall > 0.0)))
    return fail(nullptr, ASTR_ERR_ARG, "a channel needs npdcj = 4, the main ordering and twall > 0");
  int bct[6];
  for (int n = 0; n < 6; ++n) {
    bct[n] = params->bctype[n];
    if (params->channel && (n == 2 || n == 3) && (bct[n] == 0 || bct[n] == 1)) bct[n] = 41;
    if (bct[n] == 0 || bct[n] == 1) continue;
    if (bct[n] != 41 && bct[n] != 42 && bct[n] != 50 && bct[n] != 60 && bct[n] != 421 &&
        bct[n] != 21 && bct[n] != 51 && bct[n] != 411 && bct[n] != 11 && bct[n] != 23 && bct[n] != 12)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED,
                  "bctype: 11, 12, 21, 23, 41, 42, 411, 421, 50, 51 and 60 are built (0/1: none)");
    if (bct[n] == 23 && n != 1 && n != 3)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "bctype 23 exists for the xmax and ymax faces only");
    if ((bct[n] == 11 || bct[n] == 12) && n != 0)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "bctypes 11 and 12 exist for the xmin face only");
    if (bct[n] == 12 && (npdc[1] != 3 || (ndims == 3 && npdc[2] != 3)))
      return fail(nullptr, ASTR_ERR_UNSUPPORTED,
                  "bctype 12 (inflow_nscbc) needs periodic y and z: its tangential derivatives (ddfc "
                  "'222e') have no closure for both ends physical on one rank");
    if (bct[n] == 51 && n < 2)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "bctype 51 exists for the y and z faces only");
    if (bct[n] == 21 && n != 1 && n != 3)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "bctype 21 exists for the xmax and ymax faces only");
    if (bct[n] == 42 && n >= 4)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "bctype 42 exists for the x and y faces only");
    if ((bct[n] == 421 || bct[n] == 411) && n / 2 != 1)
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "bctypes 411 and 421 exist for the y faces only");
    if (n / 2 >= ndims || npdc[n / 2] != 4)
      return fail(nullptr, ASTR_ERR_ARG, "a boundary routine needs npdc = 4 in its direction");
    const double tw = params->twall_face[n] != 0.0 ? params->twall_face[n] : params->twall;
    if ((bct[n] == 41 || bct[n] == 411) && !(tw > 0.0))
      return fail(nullptr, ASTR_ERR_ARG, "bctypes 41 and 411 need a wall temperature > 0");
  }
  if (params->conschm != ASTR_CONSCHM_CENTRAL && params->conschm != ASTR_CONSCHM_MP)
    return fail(nullptr, ASTR_ERR_ARG, "conschm must be ASTR_CONSCHM_CENTRAL or ASTR_CONSCHM_MP");
  if (params->conschm == ASTR_CONSCHM_MP &&
      (params->precision != ASTR_FP64 || params->order != ASTR_ORDER_MAIN))
    return fail(nullptr, ASTR_ERR_UNSUPPORTED, "the compact MP scheme runs in FP64 and the main ordering");

  c = new astr_ctx();
  c->dm = *dims;
  c->pm = *params;
  c->prec = params->precision;
  const int dimv[3] = {dims->im, dims->jm, dims->km};
  for (int d = 0; d < ndims; ++d) {
    // rows of the filter system (dim+7 periodic) and the derivative system
    // (dim+3); x derivative sweeps hold a line in one warp (32 chunks), the
    // filters and y/z sweeps in a block (NCH_B chunks)
    const int nf = npdc[d] == 4 ? dimv[d] + 1 : dimv[d] + 7;
    const int nd = npdc[d] == 4 ? dimv[d] + 1 : dimv[d] + 3;
    c->CHf[d] = pick_ch(nf, NCH_B);
    c->CH[d] = pick_ch(nd, d == 0 ? NCH : NCH_B);
    if (c->CH[d] < 0 || c->CHf[d] < 0 || nf > NCH * 33) {
      delete c;
      return fail(nullptr, ASTR_ERR_UNSUPPORTED, "line longer than 1049 nodes");
    }
  }
  Geo& g = c->g;
  g.im = dims->im; g.jm = dims->jm; g.km = dims->km;
  g.NI = g.im + 2 * HMD + 1; g.NJ = g.jm + 2 * HMD + 1;
  g.nh = g.NI * g.NJ * (long long)(g.km + 2 * HMD + 1);
  g.I = g.im + 1; g.IJ = g.I * (g.jm + 1); g.n0 = g.IJ * (g.km + 1);
  g.ndims = ndims;
  for (int d = 0; d < 3; ++d) {
    g.per[d] = npdc[d] == 3;
    g.lo[d] = npdc[d] == 4 ? 1 : 0;
    g.hi[d] = npdc[d] == 4 ? dimv[d] - 1 : dimv[d];
  }
  // refcal (src/solver.F90:102-128)
  const double gamma = 1.4, mach = params->mach;
  Phys& ph = c->ph;
  std::memset(&ph, 0, sizeof(ph));
  const double const2 = gamma * (mach * mach);
  const double const5 = (gamma - 1.0) * (mach * mach);
  const double const6 = 1.0 / (gamma - 1.0);
  ph.const2 = const2;
  ph.rconst6 = 1.0 / const6;
  ph.hcc_scale = 1.0 / (params->prandtl * const5);
  ph.tempconst = params->suth_const / params->ref_tem;
  ph.tempconst1 = 1.0 + ph.tempconst;
  ph.rreynolds = 1.0 / params->reynolds;
  ph.dt = params->deltat;
  ph.mini = params->order == ASTR_ORDER_MINIAPP;
  const double PI = 4.0 * std::atan(1.0);
  for (int d = 0; d < 3; ++d) ph.rdx[d] = dimv[d] > 0 ? 1.0 / (2.0 * PI / (double)dimv[d]) : 1.0;
  ph.f_const2 = (float)ph.const2; ph.f_rconst6 = (float)ph.rconst6;
  ph.f_hcc_scale = (float)ph.hcc_scale; ph.f_tempconst = (float)ph.tempconst;
  ph.f_tempconst1 = (float)ph.tempconst1; ph.f_rreynolds = (float)ph.rreynolds;
  for (int d = 0; d < 3; ++d) ph.f_rdx[d] = (float)ph.rdx[d];
  const HostFTab hft = make_ftab(params->alfa_filter, params->beter_halo, params->beter_bound);
  c->ft64 = cast_ftab<double>(hft);
  c->ft32 = cast_ftab<float>(hft);

  cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->cst, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_begin, cudaEventDisableTiming);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaEventCreateWithFlags(&c->ev_copy[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_use[b], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    std::string m = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    astr_gpu_destroy(c);  // the streams and events created before the failure
    return fail(nullptr, ASTR_ERR_CUDA, m);
  }
  bool ok = true;
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) { ok = false; return nullptr; }
    c->allocs.push_back(p);
    return p;
  };
  const bool f32 = c->prec == ASTR_FP32_STORAGE;
  const size_t nh = (size_t)g.nh, n0 = (size_t)g.n0, w = wsize(c);
  void* q = alloc(5 * nh * w);
  void* pr = alloc(6 * nh * w);
  void* xd = alloc(3 * nh * w);
  void* jac = alloc(nh * w);
  void* qrhs = alloc(5 * n0 * w);
  void* grad = alloc(12 * n0 * w);
  void* sig = alloc(6 * n0 * w);
  void* qf = alloc(3 * n0 * w);
  double* qsave = (double*)alloc(5 * n0 * 8);
  double* qm = f32 ? (double*)alloc(5 * n0 * 8) : nullptr;
  c->staging = f32 ? (double*)alloc(nh * 8) : nullptr;
  c->staging2 = f32 ? (double*)alloc(nh * 8) : nullptr;
  c->jac64 = f32 ? (double*)alloc(nh * 8) : (double*)jac;
  c->rjac64 = (double*)alloc(nh * 8);
  // lines per block: the largest that still gives every SM blocks (the
  // one-warp-per-line x layout wants MINB_X blocks per SM, the block layout
  // two); small grids launch fewer lines per block.  FP64 form only: its
  // sweeps are FP64-bound and gain from the SMs (vortex 512^2: 224 -> 280
  // Mpts*stages/s); the FP32-storage sweeps are load-latency bound and lose
  // a little with the narrower rows of 4-line blocks (443 -> 435).
  {
    const bool adapt = !std::getenv("ASTR_FIXED_BLOCKS") && c->prec == ASTR_FP64;
    const long long nsm = 152;
    const long long xl = (long long)(g.jm + 1) * (g.km + 1);
    c->lbw = X_LINES;
    while (adapt && c->lbw > 1 && (xl + c->lbw - 1) / c->lbw < MINB_X * nsm) c->lbw /= 2;
    for (int d = 0; d < 3; ++d) {
      const long long na = (d == 0 ? g.jm : g.im) + 1, nb = (d == 2 ? g.jm : g.km) + 1;
      c->lbb[d] = YZ_LINES;
      while (adapt && c->lbb[d] > 4 && ((na + c->lbb[d] - 1) / c->lbb[d]) * nb < 2 * nsm) c->lbb[d] /= 2;
    }
    // launch-shape override for tuning: "warps,x,y,z" (powers of two within the maxima)
    if (const char* e = std::getenv("ASTR_LINES_PER_BLOCK")) {
      int v[4];
      if (std::sscanf(e, "%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3]) == 4) {
        auto ok = [](int x, int mx) { return x >= 1 && x <= mx && (x & (x - 1)) == 0; };
        if (ok(v[0], X_LINES)) c->lbw = v[0];
        for (int d = 0; d < 3; ++d)
          if (ok(v[1 + d], YZ_LINES)) c->lbb[d] = v[1 + d];
      }
    }
  }
  {
    // fewer y-line blocks than SMs: spread the variables of a line over
    // blocks (mini-app ordering excluded: its last filter direction
    // recovers the primitives of all variables)
    const long long yblocks = ((g.im + 1 + c->lbb[1] - 1) / c->lbb[1]) * (long long)(g.km + 1);
    c->vsplit = yblocks < 152 && params->order == ASTR_ORDER_MAIN;
    if (const char* e = std::getenv("ASTR_VAR_SPLIT"))
      c->vsplit = std::atoi(e) != 0 && params->order == ASTR_ORDER_MAIN;
  }
  long long nw = std::max(sweep_warps<0>(g, c->lbw, c->lbb),
                          std::max(sweep_warps<1>(g, c->lbw, c->lbb), sweep_warps<2>(g, c->lbw, c->lbb)));
  nw = std::max(nw, (long long)((g.n0 + 255) / 256));  // point statistics blocks
  double* part = (double*)alloc(2 * nw * 8);
  int* flag = (int*)alloc(64);
  c->stats_dev = (double*)alloc(64);
  c->channel = params->channel != 0;
  for (int n = 0; n < 6; ++n) {
    c->bct[n] = bct[n];
    c->btw[n] = params->twall_face[n] != 0.0 ? params->twall_face[n] : params->twall;
    if (bct[n] != 0 && bct[n] != 1) c->has_bc = true;
  }
  if (const char* e = std::getenv("ASTR_SPLIT_LAST")) c->split_last = std::atoi(e) & 3;
  if (c->channel) {
    const long long ncol = (long long)g.im * (ndims == 3 ? g.km : 1);
    c->chan_nblk = (int)((ncol + CHAN_THREADS - 1) / CHAN_THREADS);
    c->chan_dev = (double*)alloc(CHAN_N * 8);
    c->chan_part = (double*)alloc(5 * (size_t)c->chan_nblk * 8);
    c->ycoord = (double*)alloc(nh * 8);
  }
  if (bct[2] == 411) c->slip_mask = (unsigned char*)alloc((size_t)(g.im + 1) * (g.km + 1));
  const size_t n_face0 = (size_t)(g.jm + 1) * (g.km + 1);
  const size_t n_inflow = 5 * n_face0 + (size_t)(g.jm + 1);
  if (bct[0] == 11 || bct[0] == 12) c->inflow = (double*)alloc(n_inflow * 8);
  if (bct[0] == 12) {
    c->nscbc_b = (double*)alloc(5 * n_face0 * 8);
    c->nscbc_gm = (unsigned long long*)alloc(8);
  }
  if (bct[1] == 23) c->gc_dx[0] = (double*)alloc((size_t)(g.jm + 1) * (g.km + 1) * 8);
  if (bct[3] == 23) c->gc_dx[1] = (double*)alloc((size_t)(g.im + 1) * (g.km + 1) * 8);
  // schemes: per direction derivative + filter, in both precisions
  std::vector<HostScheme> hs;
  for (int dd = 0; dd < 3; ++dd) {
    const int CHd = dd < ndims ? c->CH[dd] : 3, CHf = dd < ndims ? c->CHf[dd] : 3;
    hs.push_back(make_deriv(npdc[dd], std::max(dimv[dd], 1), CHd, hft));
    hs.push_back(make_filter(npdc[dd], std::max(dimv[dd], 1), params->alfa_filter, CHf, hft));
  }
  size_t tot = 0;
  for (auto& s : hs) tot += 6 * (size_t)s.n + s.K.size() + s.KD.size();
  double* coef64 = (double*)alloc(tot * 8);
  float* coef32 = (float*)alloc(tot * 4);
  if (!ok) {
    astr_gpu_destroy(c);
    return fail(nullptr, ASTR_ERR_OOM, "device allocation failed");
  }
  std::vector<double> hbuf(tot);
  std::vector<float> fbuf(tot);
  size_t off = 0;
  for (int idx = 0; idx < 6; ++idx) {
    HostScheme& s = hs[idx];
    const size_t n = s.n, nk = s.K.size(), nkd = s.KD.size();
    const std::vector<double>* arr[6] = {&s.ac1, &s.ac3, &s.G, &s.H, &s.ac2, &s.a};
    for (int a = 0; a < 6; ++a) std::memcpy(&hbuf[off + a * n], arr[a]->data(), n * 8);
    std::memcpy(&hbuf[off + 6 * n], s.K.data(), nk * 8);
    if (nkd) std::memcpy(&hbuf[off + 6 * n + nk], s.KD.data(), nkd * 8);
    const size_t len = 6 * n + nk + nkd;
    for (size_t i = 0; i < len; ++i) fbuf[off + i] = (float)hbuf[off + i];
    DScheme<double> d8;
    DScheme<float> d4;
    d8.ac1 = coef64 + off; d8.ac3 = coef64 + off + n; d8.G = coef64 + off + 2 * n;
    d8.H = coef64 + off + 3 * n; d8.ac2 = coef64 + off + 4 * n; d8.A = coef64 + off + 5 * n;
    d8.K = coef64 + off + 6 * n; d8.KD = nkd ? coef64 + off + 6 * n + nk : nullptr;
    d4.ac1 = coef32 + off; d4.ac3 = coef32 + off + n; d4.G = coef32 + off + 2 * n;
    d4.H = coef32 + off + 3 * n; d4.ac2 = coef32 + off + 4 * n; d4.A = coef32 + off + 5 * n;
    d4.K = coef32 + off + 6 * n; d4.KD = nkd ? coef32 + off + 6 * n + nk : nullptr;
    d8.n = d4.n = s.n; d8.first = d4.first = s.first; d8.ntype = d4.ntype = s.ntype;
    d8.ks = d4.ks = s.n;
    d8.dim = d4.dim = s.dim;
    d8.ulo = d4.ulo = s.ulo; d8.uhi = d4.uhi = s.uhi;
    d8.u_ac1 = s.u_ac1; d8.u_ac3 = s.u_ac3;
    d4.u_ac1 = (float)s.u_ac1; d4.u_ac3 = (float)s.u_ac3;
    for (int j = 0; j < 6; ++j) { d8.u_K[j] = s.u_K[j]; d4.u_K[j] = (float)s.u_K[j]; }
    for (int j = 0; j < 5; ++j) { d8.u_KD[j] = s.u_KD[j]; d4.u_KD[j] = (float)s.u_KD[j]; }
    if (idx % 2 == 0) { c->fd64[idx / 2] = d8; c->fd32[idx / 2] = d4; }
    else { c->fl64[idx / 2] = d8; c->fl32[idx / 2] = d4; }
    off += len;
  }
  e = cudaMemcpy(coef64, hbuf.data(), tot * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(coef32, fbuf.data(), tot * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(q, 0, 5 * nh * w);
  if (e == cudaSuccess) e = cudaMemset(pr, 0, 6 * nh * w);
  if (e == cudaSuccess) e = cudaMemset(qrhs, 0, 5 * n0 * w);
  if (e == cudaSuccess) e = cudaMemset(grad, 0, 12 * n0 * w);
  if (e == cudaSuccess) e = cudaMemset(flag, 0, 64);
  if (e == cudaSuccess && c->channel) e = cudaMemset(c->chan_dev, 0, CHAN_N * 8);
  if (e != cudaSuccess) {
    std::string m = std::string("initialisation: ") + cudaGetErrorString(e);
    astr_gpu_destroy(c);
    return fail(nullptr, ASTR_ERR_CUDA, m);
  }
  auto fill = [&](auto& D, auto* tag) {
    using TT = std::remove_pointer_t<decltype(tag)>;
    D.q = (TT*)q; D.pr = (TT*)pr; D.xd = (const TT*)xd; D.jac = (const TT*)jac;
    D.jac64 = c->jac64; D.rjac64 = c->rjac64;
    D.qrhs = (TT*)qrhs; D.qsave = qsave; D.qm = qm; D.grad = (TT*)grad; D.sig = (TT*)sig;
    D.qf = (TT*)qf; D.part = part; D.flag = flag; D.chan = c->chan_dev; D.xg = nullptr;
  };
  fill(c->d64, (double*)nullptr);
  fill(c->d32, (float*)nullptr);
  {
    // Tile-staged sweeps: main ordering, lines of at most 32 x 17 rows, every
    // halo array addressable with 32-bit offsets (small grids spread the
    // variables of a line over blocks as the register-window sweeps do).
    // ASTR_V2=0 keeps the register-window sweeps.
    bool el = params->order == ASTR_ORDER_MAIN && g.nh < (1LL << 31) / 6;
    for (int d = 0; d < ndims; ++d) el = el && c->CH[d] <= 17 && c->CHf[d] <= 17;
    // FP64 form: the register-window sweeps, whose occupancy keeps the FP64
    // pipe busier (ASTR_V2=2 selects the tiled sweeps there too)
    int v2mode = 1;
    if (const char* ev = std::getenv("ASTR_V2")) v2mode = std::atoi(ev);
    el = el && v2mode != 0 && (c->prec == ASTR_FP32_STORAGE || v2mode == 2);
    if (el) {
      std::vector<HostScheme> ps;
      for (int dd = 0; dd < ndims; ++dd) {
        ps.push_back(make_deriv(npdc[dd], dimv[dd], c->CH[dd], hft, 32 * c->CH[dd]));
        ps.push_back(make_filter(npdc[dd], dimv[dd], params->alfa_filter, c->CHf[dd], hft,
                                 32 * c->CHf[dd]));
      }
      size_t ptot = 0;
      for (auto& q : ps) ptot += 6 * q.a.size() + q.K.size() + q.KD.size();
      double* p64 = (double*)alloc(ptot * 8);
      float* p32 = (float*)alloc(ptot * 4);
      if (!ok) {
        astr_gpu_destroy(c);
        return fail(nullptr, ASTR_ERR_OOM, "device allocation failed");
      }
      std::vector<double> hb(ptot);
      std::vector<float> fb2(ptot);
      size_t po = 0;
      for (size_t idx = 0; idx < ps.size(); ++idx) {
        const HostScheme& q = ps[idx];
        const size_t np = q.a.size(), nk = q.K.size(), nkd = q.KD.size();
        const std::vector<double>* arr[6] = {&q.ac1, &q.ac3, &q.G, &q.H, &q.ac2, &q.a};
        for (int a = 0; a < 6; ++a) std::memcpy(&hb[po + a * np], arr[a]->data(), np * 8);
        std::memcpy(&hb[po + 6 * np], q.K.data(), nk * 8);
        if (nkd) std::memcpy(&hb[po + 6 * np + nk], q.KD.data(), nkd * 8);
        const size_t len = 6 * np + nk + nkd;
        for (size_t i = 0; i < len; ++i) fb2[po + i] = (float)hb[po + i];
        DScheme<double> d8{};
        DScheme<float> d4{};
        d8.ac1 = p64 + po; d8.ac3 = p64 + po + np; d8.G = p64 + po + 2 * np;
        d8.H = p64 + po + 3 * np; d8.ac2 = p64 + po + 4 * np; d8.A = p64 + po + 5 * np;
        d8.K = p64 + po + 6 * np; d8.KD = nkd ? p64 + po + 6 * np + nk : nullptr;
        d4.ac1 = p32 + po; d4.ac3 = p32 + po + np; d4.G = p32 + po + 2 * np;
        d4.H = p32 + po + 3 * np; d4.ac2 = p32 + po + 4 * np; d4.A = p32 + po + 5 * np;
        d4.K = p32 + po + 6 * np; d4.KD = nkd ? p32 + po + 6 * np + nk : nullptr;
        d8.n = d4.n = q.n; d8.first = d4.first = q.first; d8.ntype = d4.ntype = q.ntype;
        d8.dim = d4.dim = q.dim; d8.ks = d4.ks = (int)np;
        d8.ulo = d4.ulo = q.ulo; d8.uhi = d4.uhi = q.uhi;
        astr_ctx::V2U u;
        const int CHs = (int)(np / 32);
        if (q.ulo <= q.uhi) {
          u.a1 = q.u_ac1; u.a3 = q.u_ac3;
          for (int m = 0; m < 6; ++m) u.K[m] = q.u_K[m];
          for (int m = 0; m < 5; ++m) u.KD[m] = q.u_KD[m];
          for (int t = 0; t < CHs; ++t) {
            u.gp[t] = q.G[(size_t)q.ulo * CHs + t];
            u.hp[t] = q.H[(size_t)q.ulo * CHs + t];
          }
        }
        const int dd = (int)idx / 2;
        if (idx % 2 == 0) { c->v2d64[dd] = d8; c->v2d32[dd] = d4; c->v2ud[dd] = u; }
        else { c->v2f64[dd] = d8; c->v2f32[dd] = d4; c->v2uf[dd] = u; }
        po += len;
      }
      e = cudaMemcpy(p64, hb.data(), ptot * 8, cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(p32, fb2.data(), ptot * 4, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        std::string m = std::string("initialisation: ") + cudaGetErrorString(e);
        astr_gpu_destroy(c);
        return fail(nullptr, ASTR_ERR_CUDA, m);
      }
      c->v2 = true;
    }
  }
  if (params->conschm == ASTR_CONSCHM_MP) {
    // compact MP: scratch, and the upwind / downwind interface schemes of
    // each direction (compact_flux_initiate, src/flux.F90:32-112)
    MPDev& m = c->mpd;
    m.fsw = (double*)alloc(10 * nh * 8);
    m.fhc = (double*)alloc(10 * nh * 8);
    m.fh = (double*)alloc(5 * nh * 8);
    m.ssf = (double*)alloc(nh * 8);
    m.lshock = (unsigned char*)alloc(n0);
    long long nif = 0;  // interfaces of the largest direction box
    for (int d = 0; d < ndims; ++d) {
      long long c1 = dimv[d] + 2;
      for (int t = 0; t < ndims; ++t)
        if (t != d) c1 *= dimv[t] + 1;
      nif = std::max(nif, c1);
    }
    m.flist = (int*)alloc((size_t)nif * sizeof(int));
    m.fcount = (int*)alloc(64);
    m.chard = params->lchardecomp != 0;
    for (int d = 0; d < 3; ++d) m.npdc[d] = npdc[d];
    m.mach = params->mach;
    m.rmach = 1.0 / params->mach;
    m.bfac = params->bfacmpld;
    m.shkcrt = params->shkcrt;
    std::vector<HostScheme> fs;
    for (int d = 0; d < 3; ++d) {
      const int dim = std::max(dimv[d], 1);
      const int rows = npdc[d] == 4 ? dim + 2 : dim + 4;
      c->mps.CH[d] = d < ndims ? pick_ch(rows, NCH_B) : 3;
      c->mps.lbb[d] = c->lbb[d];
      c->mps.vsplit = c->vsplit ? 1 : 0;
      if (c->mps.CH[d] < 0) ok = false;
      fs.push_back(make_flux(npdc[d], dim, +1, params->bfacmpld, std::max(c->mps.CH[d], 3), hft));
      fs.push_back(make_flux(npdc[d], dim, -1, params->bfacmpld, std::max(c->mps.CH[d], 3), hft));
    }
    size_t ftot = 0;
    for (auto& f : fs) ftot += 5 * (size_t)f.n;
    double* fcoef = ok ? (double*)alloc(ftot * 8) : nullptr;
    if (!ok) {
      astr_gpu_destroy(c);
      return fail(nullptr, ASTR_ERR_OOM, "device allocation failed (compact MP scratch or line length)");
    }
    std::vector<double> fb(ftot);
    size_t fo = 0;
    for (int idx = 0; idx < 6; ++idx) {
      const HostScheme& f = fs[idx];
      const size_t n = f.n;
      const std::vector<double>* arr[5] = {&f.ac1, &f.ac3, &f.G, &f.H, &f.ac2};
      for (int a = 0; a < 5; ++a) std::memcpy(&fb[fo + a * n], arr[a]->data(), n * 8);
      DScheme<double> d8{};
      d8.ac1 = fcoef + fo; d8.ac3 = fcoef + fo + n; d8.G = fcoef + fo + 2 * n;
      d8.H = fcoef + fo + 3 * n; d8.ac2 = fcoef + fo + 4 * n;
      d8.n = f.n; d8.first = f.first; d8.ntype = f.ntype; d8.dim = f.dim; d8.ks = f.n;
      d8.ulo = 1; d8.uhi = 0;
      if (idx % 2 == 0) c->mps.uw[idx / 2] = d8;
      else c->mps.dw[idx / 2] = d8;
      fo += 5 * n;
    }
    e = cudaMemcpy(fcoef, fb.data(), ftot * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m.fsw, 0, 10 * nh * 8);
    if (e == cudaSuccess) e = cudaMemset(m.fhc, 0, 10 * nh * 8);
    if (e == cudaSuccess) e = cudaMemset(m.fh, 0, 5 * nh * 8);
    if (e == cudaSuccess) e = cudaMemset(m.ssf, 0, nh * 8);
    if (e == cudaSuccess) e = cudaMemset(m.lshock, 0, n0);
    if (e != cudaSuccess) {
      std::string msg = std::string("compact MP initialisation: ") + cudaGetErrorString(e);
      astr_gpu_destroy(c);
      return fail(nullptr, ASTR_ERR_CUDA, msg);
    }
    c->mp = true;
  }
  if (c->inflow) {
    const int rc = inflow_upload(c, nullptr, nullptr, nullptr, nullptr);
    if (rc != ASTR_OK) {
      std::string msg = c->err;
      astr_gpu_destroy(c);
      return fail(nullptr, rc, msg);
    }
  }
  *out = c;
  return ASTR_OK;
}

void astr_gpu_destroy(astr_ctx* c) {
  if (!c) return;
  if (c->batch) batch_forget(c->batch, c);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
  if (c->cst) cudaStreamSynchronize(c->cst);
  for (int b = 0; b < 2; ++b) {
    if (c->ev_copy[b]) cudaEventDestroy(c->ev_copy[b]);
    if (c->ev_use[b]) cudaEventDestroy(c->ev_use[b]);
  }
  if (c->ev_begin) cudaEventDestroy(c->ev_begin);
  for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
  for (void* p : c->allocs) cudaFree(p);
  if (c->st) cudaStreamDestroy(c->st);
  if (c->cst) cudaStreamDestroy(c->cst);
  delete c;
}

static int metrics_common(astr_ctx* c, const double* const src[3], const double* jacob) {
  const size_t nh = (size_t)c->g.nh, w = wsize(c);
  char* xd = (char*)c->d64.xd;
  RC(xfer_begin(c));
  for (int dd = 0; dd < 3; ++dd) RC(upload_array(c, xd + dd * nh * w, src[dd], nh));
  RC(upload_array(c, (void*)c->d64.jac, jacob, nh));
  RC(xfer_sync(c));
  if (c->prec == ASTR_FP32_STORAGE)
    CK(cudaMemcpyAsync(c->jac64, jacob, nh * 8, cudaMemcpyHostToDevice, c->st));
  k_reciprocal<<<point_grid((long long)nh), 256, 0, c->st>>>(c->jac64, c->rjac64, (long long)nh);
  RC(after_launch(c, "k_reciprocal"));
  CK(cudaStreamSynchronize(c->st));
  c->metrics_set = true;
  return ASTR_OK;
}

int astr_gpu_set_metrics(astr_ctx* c, const double* dxi, const double* jacob) {
  if (!c || !dxi || !jacob) return fail(c, ASTR_ERR_ARG, "null argument");
  const size_t nh = (size_t)c->g.nh;
  // Diagonal metrics (every off-diagonal exactly zero) take the rectilinear
  // kernels; anything else the general-metric ones.
  bool diag = true;
  for (int m = 0; m < 3 && diag; ++m)
    for (int dd = 0; dd < 3 && diag; ++dd) {
      if (m == dd) continue;
      const double* p = dxi + (size_t)(dd + 3 * m) * nh;
      for (size_t i = 0; i < nh; ++i)
        if (p[i] != 0.0) { diag = false; break; }
    }
  if (!diag && c->pm.order == ASTR_ORDER_MINIAPP)
    return fail(c, ASTR_ERR_ARG, "the mini-app ordering takes no metrics");
  if (c->step_graph) {  // a captured step holds the old metric mode
    CK(cudaStreamSynchronize(c->st));
    cudaGraphExecDestroy(c->step_graph);
    c->step_graph = nullptr;
  }
  const double* const src[3] = {dxi, dxi + 4 * nh, dxi + 8 * nh};
  RC(metrics_common(c, src, jacob));
  if (diag) {
    c->gen = false;
    c->d64.xg = nullptr;
    c->d32.xg = nullptr;
    return ASTR_OK;
  }
  const size_t w = wsize(c);
  if (!c->xg) {
    void* p = nullptr;
    CK(cudaMalloc(&p, 9 * nh * w));
    c->allocs.push_back(p);
    c->xg = p;
  }
  RC(xfer_begin(c));
  for (int dd = 0; dd < 3; ++dd)
    for (int m = 0; m < 3; ++m)
      RC(upload_array(c, (char*)c->xg + (size_t)(3 * dd + m) * nh * w, dxi + (size_t)(dd + 3 * m) * nh, nh));
  RC(xfer_sync(c));
  c->d64.xg = (const double*)c->xg;
  c->d32.xg = (const float*)c->xg;
  c->gen = true;
  return ASTR_OK;
}

int astr_gpu_set_grid(astr_ctx* c, const double* x) {
  if (!c || !x) return fail(c, ASTR_ERR_ARG, "null argument");
  if (!c->channel && !c->slip_mask && !c->gc_dx[0] && !c->gc_dx[1] && !c->nscbc_b) return ASTR_OK;
  const size_t nh = (size_t)c->g.nh;
  const long long NI = c->g.NI, NJ = c->g.NJ;
  auto h = [&](int i, int j, int k) {
    return (size_t)((i + HMD) + NI * ((j + HMD) + NJ * (long long)(k + HMD)));
  };
  std::vector<unsigned char> mask;
  if (c->slip_mask) {
    // slipisotwall's test x(i,0,k,1) <= xslip (src/bc.F90:7132), node (i, k)
    // at i + (im+1) k, the face kernel's thread order on a y face
    const int im = c->g.im, km = c->g.km;
    mask.resize((size_t)(im + 1) * (km + 1));
    for (int k = 0; k <= km; ++k)
      for (int i = 0; i <= im; ++i)
        mask[(size_t)i + (size_t)(im + 1) * k] = x[h(i, 0, k)] <= c->pm.xslip ? 1 : 0;
    CK(cudaMemcpyAsync(c->slip_mask, mask.data(), mask.size(), cudaMemcpyHostToDevice, c->st));
  }
  if (c->nscbc_b) {
    // inflow_nscbc's xmax - xmin (gridgeom, src/geom.F90:684-696)
    double lo = 1e300, hi = -1e300;
    for (int k = 0; k <= c->g.km; ++k)
      for (int j = 0; j <= c->g.jm; ++j)
        for (int i = 0; i <= c->g.im; ++i) {
          lo = std::min(lo, x[h(i, j, k)]);
          hi = std::max(hi, x[h(i, j, k)]);
        }
    c->nscbc_ext = hi - lo;
  }
  for (int f = 0; f < 2; ++f) {
    // gcnscbc's spacing x(dim-1) - x(dim-2) along the face normal at every
    // face node (the face kernel's order: j + (jm+1) k on xmax, i + (im+1) k
    // on ymax) and the grid's extent along it (xmax - xmin, ymax - ymin)
    if (!c->gc_dx[f]) continue;
    const int im = c->g.im, jm = c->g.jm, km = c->g.km;
    const double* xc = x + (size_t)f * nh;
    double lo = 1e300, hi = -1e300;
    for (int k = 0; k <= km; ++k)
      for (int j = 0; j <= jm; ++j)
        for (int i = 0; i <= im; ++i) {
          lo = std::min(lo, xc[h(i, j, k)]);
          hi = std::max(hi, xc[h(i, j, k)]);
        }
    c->gc_ext[f] = hi - lo;
    const int na = f == 0 ? jm : im;
    std::vector<double> dxv((size_t)(na + 1) * (km + 1));
    for (int k = 0; k <= km; ++k)
      for (int a = 0; a <= na; ++a)
        dxv[(size_t)a + (size_t)(na + 1) * k] =
            f == 0 ? xc[h(im - 1, a, k)] - xc[h(im - 2, a, k)] : xc[h(a, jm - 1, k)] - xc[h(a, jm - 2, k)];
    CK(cudaMemcpyAsync(c->gc_dx[f], dxv.data(), dxv.size() * 8, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  if (c->channel) {
    const double* y = x + nh;  // x(..,2)
    CK(cudaMemcpyAsync(c->ycoord, y, nh * 8, cudaMemcpyHostToDevice, c->st));
    c->chan_ly = y[h(0, c->g.jm, 0)] - y[h(0, 0, 0)];
  }
  CK(cudaStreamSynchronize(c->st));
  c->grid_set = true;
  return ASTR_OK;
}

int astr_gpu_set_inflow(astr_ctx* c, const double* vel_in, const double* tmp_in, const double* tmp_prof,
                        const double* prs_in) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  if (!c->inflow) return fail(c, ASTR_ERR_STATE, "no inflow face (bctype 11 or 12 on xmin)");
  return inflow_upload(c, vel_in, tmp_in, tmp_prof, prs_in);
}

int astr_gpu_channel_state(astr_ctx* c, double* out) {
  if (!c || !out) return fail(c, ASTR_ERR_ARG, "null argument");
  if (!c->channel) return fail(c, ASTR_ERR_STATE, "not a channel context");
  double h[CHAN_N];
  CK(cudaMemcpyAsync(h, c->chan_dev, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  out[0] = h[CHAN_FORCE];
  out[1] = h[CHAN_MASSFLUX];
  out[2] = h[CHAN_TARGET];
  out[3] = h[CHAN_FBCX];
  out[4] = (double)c->nstep;
  return ASTR_OK;
}

static int ready(astr_ctx* c);

int astr_gpu_crashcheck(astr_ctx* c, long long* ncrash, int* ijk) {
  RC(ready(c));
  if (!ncrash) return fail(c, ASTR_ERR_ARG, "null argument");
  unsigned long long* dv = (unsigned long long*)c->stats_dev;  // 64 B scratch
  const unsigned long long init[2] = {0ULL, ~0ULL};
  CK(cudaMemcpyAsync(dv, init, sizeof(init), cudaMemcpyHostToDevice, c->st));
  if (c->prec == ASTR_FP64)
    k_crashcheck<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, dv);
  else
    k_crashcheck<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, dv);
  RC(after_launch(c, "k_crashcheck"));
  unsigned long long h[2];
  CK(cudaMemcpyAsync(h, dv, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *ncrash = (long long)h[0];
  if (ijk) {
    ijk[0] = ijk[1] = ijk[2] = -1;
    if (h[0]) {
      const long long z = (long long)h[1];
      ijk[0] = (int)(z % c->g.I);
      ijk[1] = (int)((z / c->g.I) % (c->g.jm + 1));
      ijk[2] = (int)(z / c->g.IJ);
    }
  }
  return ASTR_OK;
}

int astr_gpu_cflcal(astr_ctx* c, double deltat, double* cfl, double* delta3) {
  RC(ready(c));
  if (!cfl) return fail(c, ASTR_ERR_ARG, "null argument");
  unsigned long long* dv = (unsigned long long*)c->stats_dev;
  CK(cudaMemsetAsync(dv, 0, 3 * sizeof(unsigned long long), c->st));
  const double rmach = 1.0 / c->pm.mach;
  if (c->prec == ASTR_FP64)
    k_cflcal<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, rmach, dv);
  else
    k_cflcal<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, rmach, dv);
  RC(after_launch(c, "k_cflcal"));
  unsigned long long h[3];
  CK(cudaMemcpyAsync(h, dv, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  double dl[3];
  for (int dd = 0; dd < 3; ++dd) std::memcpy(&dl[dd], &h[dd], 8);
  *cfl = deltat * (dl[0] + dl[1] + dl[2]);
  if (delta3)
    for (int dd = 0; dd < 3; ++dd) delta3[dd] = dl[dd];
  return ASTR_OK;
}

int astr_gpu_boucon(astr_ctx* c) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  if (!c->has_bc) return ASTR_OK;
  return c->prec == ASTR_FP64 ? run_boucon<double>(c) : run_boucon<float>(c);
}

int astr_gpu_set_metrics_diag(astr_ctx* c, const double* x11, const double* x22, const double* x33,
                              const double* jacob) {
  if (!c || !x11 || !x22 || !x33 || !jacob) return fail(c, ASTR_ERR_ARG, "null argument");
  if (c->step_graph) {
    CK(cudaStreamSynchronize(c->st));
    cudaGraphExecDestroy(c->step_graph);
    c->step_graph = nullptr;
  }
  c->gen = false;
  c->d64.xg = nullptr;
  c->d32.xg = nullptr;
  const double* const src[3] = {x11, x22, x33};
  return metrics_common(c, src, jacob);
}

int astr_gpu_upload_state(astr_ctx* c, const double* q, const double* rho, const double* vel,
                          const double* prs, const double* tmp) {
  if (!c || !q || !rho || !vel || !prs || !tmp) return fail(c, ASTR_ERR_ARG, "null argument");
  const size_t nh = (size_t)c->g.nh, w = wsize(c);
  char* dq = (char*)c->d64.q;
  char* dp = (char*)c->d64.pr;
  RC(xfer_begin(c));
  for (int m = 0; m < 5; ++m) {
    if (c->prec == ASTR_FP64) {
      RC(upload_array(c, dq + m * nh * w, q + m * nh, nh));
    } else {
      double* buf = nullptr;
      RC(xfer_in(c, q + m * nh, nh, &buf));
      k_to_float<<<point_grid((long long)nh), 256, 0, c->st>>>(buf, (float*)(dq + m * nh * w),
                                                                 (long long)nh);
      RC(after_launch(c, "k_to_float"));
      // the FP64 master takes the uploaded interior values directly
      k_halo_to_interior<<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, buf, c->d32.qm + m * c->g.n0);
      RC(after_launch(c, "k_halo_to_interior"));
      RC(xfer_used(c, buf));
    }
  }
  RC(upload_array(c, dp, rho, nh));
  for (int m = 0; m < 3; ++m) RC(upload_array(c, dp + (1 + m) * nh * w, vel + m * nh, nh));
  RC(upload_array(c, dp + 4 * nh * w, prs, nh));
  RC(upload_array(c, dp + 5 * nh * w, tmp, nh));
  RC(xfer_sync(c));
  c->state_set = true;
  return ASTR_OK;
}

int astr_gpu_upload_q(astr_ctx* c, const double* q) {
  if (!c || !q) return fail(c, ASTR_ERR_ARG, "null argument");
  const size_t nh = (size_t)c->g.nh, w = wsize(c);
  char* dq = (char*)c->d64.q;
  RC(xfer_begin(c));
  for (int m = 0; m < 5; ++m) {
    if (c->prec == ASTR_FP64) {
      RC(upload_array(c, dq + m * nh * w, q + m * nh, nh));
    } else {
      double* buf = nullptr;
      RC(xfer_in(c, q + m * nh, nh, &buf));
      k_to_float<<<point_grid((long long)nh), 256, 0, c->st>>>(buf, (float*)(dq + m * nh * w),
                                                                 (long long)nh);
      RC(after_launch(c, "k_to_float"));
      k_halo_to_interior<<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, buf, c->d32.qm + m * c->g.n0);
      RC(after_launch(c, "k_halo_to_interior"));
      RC(xfer_used(c, buf));
    }
  }
  // primitives of the interior nodes from q (updatefvar); halo primitives are
  // rebuilt by qswap at the start of each stage (periodic directions) or
  // keep what the last full upload put there (physical ends)
  if (c->prec == ASTR_FP64)
    k_updatefvar<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, c->ph);
  else
    k_updatefvar<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, c->ph);
  RC(after_launch(c, "k_updatefvar"));
  RC(xfer_sync(c));
  c->state_set = true;
  return ASTR_OK;
}

int astr_gpu_download_state(astr_ctx* c, double* q, double* rho, double* vel, double* prs, double* tmp) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  const size_t nh = (size_t)c->g.nh, w = wsize(c);
  const char* dq = (const char*)c->d64.q;
  const char* dp = (const char*)c->d64.pr;
  RC(xfer_begin(c));
  if (q) {
    for (int m = 0; m < 5; ++m) {
      if (c->prec == ASTR_FP64) {
        RC(download_array(c, q + m * nh, dq + m * nh * w, nh));
      } else {
        // halos from the FP32 copy, interior from the FP64 master
        double* buf = nullptr;
        RC(xfer_out_buf(c, &buf));
        k_to_double<<<point_grid((long long)nh), 256, 0, c->st>>>((const float*)(dq + m * nh * w),
                                                                   buf, (long long)nh);
        RC(after_launch(c, "k_to_double"));
        k_master_to_halo<<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32.qm + m * c->g.n0, buf);
        RC(after_launch(c, "k_master_to_halo"));
        RC(xfer_out(c, q + m * nh, buf, nh));
      }
    }
  }
  if (rho) RC(download_array(c, rho, dp, nh));
  if (vel)
    for (int m = 0; m < 3; ++m) RC(download_array(c, vel + m * nh, dp + (1 + m) * nh * w, nh));
  if (prs) RC(download_array(c, prs, dp + 4 * nh * w, nh));
  if (tmp) RC(download_array(c, tmp, dp + 5 * nh * w, nh));
  return xfer_sync(c);
}

int astr_gpu_download_rhs(astr_ctx* c, double* qrhs, double* dvel, double* dtmp) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  const size_t n0 = (size_t)c->g.n0, w = wsize(c);
  RC(xfer_begin(c));
  if (qrhs)
    for (int m = 0; m < 5; ++m) RC(download_array(c, qrhs + m * n0, (char*)c->d64.qrhs + m * n0 * w, n0));
  if (dvel)
    for (int m = 0; m < 9; ++m) RC(download_array(c, dvel + m * n0, (char*)c->d64.grad + m * n0 * w, n0));
  if (dtmp)
    for (int m = 0; m < 3; ++m)
      RC(download_array(c, dtmp + m * n0, (char*)c->d64.grad + (9 + m) * n0 * w, n0));
  return xfer_sync(c);
}

static int ready(astr_ctx* c) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  if (!c->metrics_set && c->pm.order == ASTR_ORDER_MAIN)
    return fail(c, ASTR_ERR_STATE, "metrics not set (astr_gpu_set_metrics)");
  if (!c->state_set) return fail(c, ASTR_ERR_STATE, "state not uploaded (astr_gpu_upload_state)");
  if ((c->channel || c->slip_mask || c->gc_dx[0] || c->gc_dx[1] || c->nscbc_b) && !c->grid_set)
    return fail(c, ASTR_ERR_STATE, "grid not set (astr_gpu_set_grid): a channel or bctype 411, 23 or 12");
  return ASTR_OK;
}

// databakup (src/mainloop.F90:824-972), device side: backup copies the
// interior conserved state and the channel controller into the snapshot
// datpnt points at and moves datpnt to the other one; recovery restores the
// snapshot datpnt points at (the older of two), moves datpnt, recovers the
// primitives (updatefvar) and, from the second recovery from the same
// snapshot on, expands the critical nodes (crinod_expansion).  With a
// single snapshot taken, datpnt points at the empty one, which the
// reference would read unallocated; the one snapshot taken is used.
static int databakup(astr_ctx* c, int recovery) {
  const size_t n0 = (size_t)c->g.n0;
  const size_t bytes = 5 * n0 * sizeof(double);
  if (!recovery) {
    const int slot = c->datpnt < 0 ? 0 : c->datpnt;
    if (c->prec == ASTR_FP64)
      k_snap_save<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, c->snap[slot]);
    else
      k_snap_save<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, c->snap[slot]);
    RC(after_launch(c, "k_snap_save"));
    if (c->chan_dev)
      CK(cudaMemcpyAsync(c->snap[slot] + 5 * n0, c->chan_dev, CHAN_N * sizeof(double),
                         cudaMemcpyDeviceToDevice, c->st));
    c->snap_valid[slot] = true;
    c->snap_nstep[slot] = c->nstep;
    c->snap_rec[slot] = 0;
    c->datpnt = 1 - slot;
    c->backups += 1;
    return ASTR_OK;
  }
  if (c->datpnt < 0 || (!c->snap_valid[0] && !c->snap_valid[1]))
    return fail(c, ASTR_ERR_NONFINITE, "crash with no backup data available (databakup)");
  int slot = c->datpnt;
  if (!c->snap_valid[slot]) slot = 1 - slot;
  if (c->prec == ASTR_FP64)
    k_snap_load<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, c->snap[slot]);
  else
    k_snap_load<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, c->snap[slot]);
  RC(after_launch(c, "k_snap_load"));
  if (c->chan_dev)
    CK(cudaMemcpyAsync(c->chan_dev, c->snap[slot] + 5 * n0, CHAN_N * sizeof(double),
                       cudaMemcpyDeviceToDevice, c->st));
  (void)bytes;
  c->nstep = c->snap_nstep[slot];
  c->snap_rec[slot] += 1;
  c->datpnt = 1 - slot;
  c->recoveries += 1;
  if (c->prec == ASTR_FP64)
    k_updatefvar<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, c->ph);
  else
    k_updatefvar<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, c->ph);
  RC(after_launch(c, "k_updatefvar"));
  if (c->snap_rec[slot] > 1) {
    k_crinod_expand<<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->crinod, c->crinod2);
    RC(after_launch(c, "k_crinod_expand"));
    std::swap(c->crinod, c->crinod2);
  }
  CK(cudaMemsetAsync(c->d64.flag, 0, sizeof(int), c->st));
  return ASTR_OK;
}

// crashcheck before a step (src/mainloop.F90:709-812, called at the top of
// steploop's loop, 103-110) with lcracon: a crashed state (q1 >= 0 fails at
// some node) is marked critical and rolled back; otherwise the state is
// backed up when nstep reaches nxtbakup, whose interval then doubles up to
// 500 steps.  Returns 1 in *recovered when it rolled back.
static int crash_control_step(astr_ctx* c, int* recovered) {
  *recovered = 0;
  if (!c->cc_started) {
    c->nxtbakup = c->nstep + c->feqbakup;  // steploop's set-up (src/mainloop.F90:90)
    c->cc_started = true;
  }
  long long ncrash = 0;
  RC(astr_gpu_crashcheck(c, &ncrash, nullptr));
  if (ncrash > 0) {
    if (c->prec == ASTR_FP64)
      k_crinod_mark<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, c->crinod);
    else
      k_crinod_mark<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, c->crinod);
    RC(after_launch(c, "k_crinod_mark"));
    RC(databakup(c, 1));
    *recovered = 1;
  } else if (c->nstep == c->nxtbakup) {
    RC(databakup(c, 0));
    c->nxtbakup = c->nstep + c->feqbakup;
    c->feqbakup = std::min<long long>(500, 2 * c->feqbakup);
  }
  return ASTR_OK;
}

int astr_gpu_rk3_step(astr_ctx* c, int nsteps, double* hist, astr_status* status) {
  RC(ready(c));
  if (nsteps < 0) return fail(c, ASTR_ERR_ARG, "nsteps < 0");
  if (c->cracon) {
    // crash control: crashcheck / databakup before every step, crashfix
    // after every stage; a rollback is reported in status->crash
    int any = 0;
    for (int s = 0; s < nsteps; ++s) {
      int rec = 0;
      RC(crash_control_step(c, &rec));
      any |= rec;
      RC(step(c, hist ? hist + 2 * s : nullptr));
    }
    if (status) {
      status->crash = any;
      status->kenergy = hist && nsteps > 0 ? hist[2 * (nsteps - 1)] : 0.0;
      status->enstrophy = hist && nsteps > 0 ? hist[2 * (nsteps - 1) + 1] : 0.0;
    }
    return ASTR_OK;
  }
  for (int s = 0; s < nsteps; ++s) RC(step(c, hist ? hist + 2 * s : nullptr));
  if (status) {
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, c->d64.flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    status->crash = flag;
    status->kenergy = hist && nsteps > 0 ? hist[2 * (nsteps - 1)] : 0.0;
    status->enstrophy = hist && nsteps > 0 ? hist[2 * (nsteps - 1) + 1] : 0.0;
    if (flag) return fail(c, ASTR_ERR_NONFINITE, "crash check: rho <= 0 or non-finite state");
  }
  return ASTR_OK;
}

int astr_gpu_filterq(astr_ctx* c) {
  RC(ready(c));
  return c->prec == ASTR_FP64 ? run_filter<double>(c, false) : run_filter<float>(c, false);
}

int astr_gpu_qswap(astr_ctx* c) {
  RC(ready(c));
  const bool mini = c->pm.order == ASTR_ORDER_MINIAPP;
  if (c->prec == ASTR_FP64) return mini ? run_bchomo<double>(c) : run_qswap<double>(c);
  return mini ? run_bchomo<float>(c) : run_qswap<float>(c);
}

int astr_gpu_gradcal(astr_ctx* c) {
  RC(ready(c));
  if (c->prec == ASTR_FP64) {
    RC(run_convgrad<double>(c, false, true, false, false, false));
    return c->gen ? gradphys_pointwise<double>(c) : ASTR_OK;
  }
  RC(run_convgrad<float>(c, false, true, false, false, false));
  return c->gen ? gradphys_pointwise<float>(c) : ASTR_OK;
}

int astr_gpu_rhscal(astr_ctx* c) {
  RC(ready(c));
  return c->prec == ASTR_FP64 ? rhscal_t<double>(c) : rhscal_t<float>(c);
}

int astr_gpu_updatefvar(astr_ctx* c) {
  RC(ready(c));
  if (c->prec == ASTR_FP64)
    k_updatefvar<double><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d64, c->ph);
  else
    k_updatefvar<float><<<point_grid(c->g.n0), 256, 0, c->st>>>(c->g, c->d32, c->ph);
  return after_launch(c, "k_updatefvar");
}

int astr_gpu_set_crash_control(astr_ctx* c, int on) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  if (on && c->pm.order != ASTR_ORDER_MAIN)
    return fail(c, ASTR_ERR_UNSUPPORTED, "crash control belongs to the main solver ordering");
  if (on && !c->snap[0]) {
    const size_t n0 = (size_t)c->g.n0;
    auto alloc = [&](size_t bytes) -> void* {
      void* p = nullptr;
      if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
      c->allocs.push_back(p);
      return p;
    };
    c->snap[0] = (double*)alloc((5 * n0 + CHAN_N) * sizeof(double));
    c->snap[1] = (double*)alloc((5 * n0 + CHAN_N) * sizeof(double));
    c->crinod = (unsigned char*)alloc(n0);
    c->crinod2 = (unsigned char*)alloc(n0);
    c->fixflag = (unsigned char*)alloc(n0);
    c->fixcount = (unsigned long long*)alloc(2 * sizeof(unsigned long long));
    if (!c->snap[0] || !c->snap[1] || !c->crinod || !c->crinod2 || !c->fixflag || !c->fixcount)
      return fail(c, ASTR_ERR_OOM, "crash control: device allocation failed");
    CK(cudaMemset(c->crinod, 0, n0));
    CK(cudaMemset(c->fixcount, 0, 2 * sizeof(unsigned long long)));
  }
  c->cracon = on != 0;
  return ASTR_OK;
}

int astr_gpu_databakup(astr_ctx* c, int mode, long long* nstep) {
  RC(ready(c));
  if (!c->snap[0]) return fail(c, ASTR_ERR_STATE, "crash control not enabled (astr_gpu_set_crash_control)");
  if (mode != 0 && mode != 1) return fail(c, ASTR_ERR_ARG, "mode: 0 backup, 1 recovery");
  RC(databakup(c, mode));
  CK(cudaStreamSynchronize(c->st));
  if (nstep) *nstep = c->nstep;
  return ASTR_OK;
}

int astr_gpu_crashfix(astr_ctx* c, long long* wiped) {
  RC(ready(c));
  if (!c->snap[0]) return fail(c, ASTR_ERR_STATE, "crash control not enabled (astr_gpu_set_crash_control)");
  unsigned long long before[2];
  CK(cudaMemcpyAsync(before, c->fixcount, sizeof(before), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  RC(c->prec == ASTR_FP64 ? run_crashfix<double>(c) : run_crashfix<float>(c));
  unsigned long long after[2];
  CK(cudaMemcpyAsync(after, c->fixcount, sizeof(after), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (wiped) *wiped = (long long)(after[1] - before[1]);
  return ASTR_OK;
}

int astr_gpu_crash_report(astr_ctx* c, long long* out6) {
  if (!c || !out6) return fail(c, ASTR_ERR_ARG, "null argument");
  for (int m = 0; m < 6; ++m) out6[m] = 0;
  out6[0] = c->recoveries;
  out6[1] = c->backups;
  out6[4] = c->nstep;
  out6[5] = c->cracon ? c->nxtbakup : -1;
  if (c->snap[0]) {
    unsigned long long cnt[2];
    CK(cudaMemcpyAsync(cnt, c->fixcount, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
    std::vector<unsigned char> m((size_t)c->g.n0);
    CK(cudaMemcpyAsync(m.data(), c->crinod, m.size(), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    out6[2] = (long long)cnt[1];
    long long n = 0;
    for (unsigned char v : m) n += v ? 1 : 0;
    out6[3] = n;
  }
  return ASTR_OK;
}

int astr_gpu_reduce_stats(astr_ctx* c, double* ke, double* en) {
  RC(ready(c));
  // statistics over the current primitives and gradients: the point
  // kernel where the step takes them from it (general metrics, variables
  // split over blocks, tiled sweeps), else the last conv/grad direction with only the
  // statistics enabled (stats_finish reads the matching partial sums)
  int r;
  if (c->gen || c->vsplit || use_v2(c)) {
    r = c->prec == ASTR_FP64 ? stats_pointwise<double>(c) : stats_pointwise<float>(c);
  } else {
    CGFlags f{0, 0, 0, 0, 0, 1, 0};
    const int last = c->g.ndims - 1;
    if (c->prec == ASTR_FP64) r = last == 2 ? launch_convgrad<double, 2>(c, f) : launch_convgrad<double, 1>(c, f);
    else r = last == 2 ? launch_convgrad<float, 2>(c, f) : launch_convgrad<float, 1>(c, f);
  }
  RC(r);
  double o[2];
  RC(stats_finish(c, o));
  if (ke) *ke = o[0];
  if (en) *en = o[1];
  return ASTR_OK;
}

int astr_gpu_synchronize(astr_ctx* c) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->st));
  return ASTR_OK;
}

int astr_gpu_last_error(astr_ctx* c, char* buf, int len) {
  const std::string& m = c ? c->err : g_create_err;
  if (buf && len > 0) {
    std::strncpy(buf, m.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)m.size();
}

long long astr_gpu_launch_count(astr_ctx* c) { return c ? c->launches : 0; }

void* astr_gpu_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void astr_gpu_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int astr_gpu_timed_steps(astr_ctx* c, int nsteps, double* elapsed_ms) {
  RC(ready(c));
  if (nsteps < 0 || !elapsed_ms) return fail(c, ASTR_ERR_ARG, "bad argument");
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, c->st));
  int rc = ASTR_OK;
  for (int s = 0; s < nsteps && rc == ASTR_OK; ++s) rc = step(c, nullptr);
  CK(cudaEventRecord(e1, c->st));
  CK(cudaEventSynchronize(e1));
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *elapsed_ms = ms;
  return rc;
}

int astr_gpu_step_async(astr_ctx* c, int nsteps) {
  RC(ready(c));
  if (nsteps < 0) return fail(c, ASTR_ERR_ARG, "nsteps < 0");
  if (c->channel)
    return fail(c, ASTR_ERR_UNSUPPORTED, "a channel step depends on host counters; use astr_gpu_rk3_step");
  if (c->prof) return fail(c, ASTR_ERR_STATE, "profiling is on");
  if (c->cracon)
    return fail(c, ASTR_ERR_UNSUPPORTED, "crash control decides on the host before each step; use astr_gpu_rk3_step");
  if (nsteps == 0) return ASTR_OK;
  if (!c->step_graph) {
    // capture one step (no statistics, no host synchronisation inside)
    cudaGraph_t graph = nullptr;
    const long long l0 = c->launches;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    const int rc = step(c, nullptr);
    const cudaError_t e = cudaStreamEndCapture(c->st, &graph);
    c->nstep -= 1;  // the captured step has not run
    if (rc != ASTR_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CK(e);
    const cudaError_t ei = cudaGraphInstantiate(&c->step_graph, graph, 0);
    cudaGraphDestroy(graph);
    CK(ei);
    c->graph_kernels = c->launches - l0;
    c->launches = l0;
  }
  for (int s = 0; s < nsteps; ++s) {
    CK(cudaGraphLaunch(c->step_graph, c->st));
    c->launches += c->graph_kernels;
    c->nstep += 1;
  }
  return ASTR_OK;
}

int astr_gpu_poll(astr_ctx* c) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  const cudaError_t e = cudaStreamQuery(c->st);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return fail(c, ASTR_ERR_CUDA, std::string("astr_gpu_poll: ") + cudaGetErrorString(e));
}

int astr_gpu_set_profiling(astr_ctx* c, int on) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->st));
  c->prof = on != 0;
  c->ev_used = 0;
  return ASTR_OK;
}

int astr_gpu_kernel_times(astr_ctx* c, double* ms, long long* launches, int nclass) {
  if (!c) return fail(c, ASTR_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->st));
  std::vector<double> acc(KC_N, 0.0);
  std::vector<long long> cnt(KC_N, 0);
  for (size_t i = 0; i + 1 < c->ev_used; i += 2) {
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, c->ev[i], c->ev[i + 1]));
    acc[c->ev_cls[i]] += t;
    cnt[c->ev_cls[i]] += 1;
  }
  for (int k = 0; k < nclass && k < KC_N; ++k) {
    if (ms) ms[k] = acc[k];
    if (launches) launches[k] = cnt[k];
  }
  c->ev_used = 0;
  return KC_N;
}

int astr_gpu_measure_fp64_peak(double* tflops) {
  if (!tflops) return ASTR_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ASTR_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  const int blocks = sms * 8, threads = 256, iters = 8000;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return ASTR_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_fp64_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return ASTR_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return ASTR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches of cases (continuous batching; no counterpart in the reference)
// ---------------------------------------------------------------------------
// A batch steps many independent cases with one launch per phase of an RK3
// stage: each persistent kernel walks a work list of (case, block) items
// drawn from every case of the batch.  A case runs exactly the kernels, in
// the order and with the arithmetic, that its own context issues for a step
// on the tiled sweeps, so it advances bit for bit as it would alone.
struct astr_batch {
  int prec = ASTR_FP64;
  int nsm = 152;
  double share = 1.0;  // fraction of the GPU's resident blocks a launch takes
  std::vector<astr_ctx*> cases;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_desc = nullptr;  // the descriptors of the last call copied
  cudaEvent_t ev_done = nullptr;  // end of the last call
  cudaEvent_t ev_in = nullptr;    // joins a case's stream into the batch stream
  void* dcases = nullptr;         // BCase<T>[cases]
  void* hcases = nullptr;         // page-locked staging of the descriptors
  size_t desc_cap = 0;            // bytes of both
  int4* ditems = nullptr;
  size_t items_cap = 0;
  // One launch of a step: op (filter, convective + gradient, viscous
  // sweeps; qswap, RK3 base, stress, RK3 update point kernels), its
  // direction and chunk length, and its items.
  struct Phase {
    int op, dir, CH;
    int rep;      // a case whose uniform-chunk constants the launch takes
    size_t off;
    int n;
    bool stage0;  // first stage only
  };
  std::vector<Phase> phases;
  bool dirty = true;
  int* dctl = nullptr;                  // device: status, steps started
  unsigned long long* ddeadline = nullptr;
  int* hword = nullptr;                 // mapped page-locked: cancel, status, started
  int* hword_dev = nullptr;             // its device address
  bool pending = false;
  int result = ASTR_OK, result_steps = 0;
  long long launches = 0;
  std::string err;
};

namespace {

enum { BOP_FILTER = 0, BOP_CONVGRAD = 1, BOP_VISC = 2, BOP_QSWAP, BOP_QSAVE, BOP_SIGMA, BOP_RK };

int bfail(astr_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

#define BCK(call)                                                                          \
  do {                                                                                     \
    const cudaError_t _e = (call);                                                         \
    if (_e != cudaSuccess)                                                                 \
      return bfail(b, _e == cudaErrorMemoryAllocation ? ASTR_ERR_OOM : ASTR_ERR_CUDA,       \
                   std::string(#call) + ": " + cudaGetErrorString(_e));                   \
  } while (0)

// Why a context cannot join a batch (empty: it can).
std::string batch_refusal(const astr_ctx* c, int prec) {
  if (c->prec != prec) return "the case's precision differs from the batch's";
  if (c->pm.order != ASTR_ORDER_MAIN) return "batches run the main ordering only";
  if (!use_v2(c))
    return "the case does not run the tiled sweeps (general metrics, the MP scheme, FP64 without "
           "ASTR_V2=2, or a line outside the tiled chunk lengths)";
  if (c->channel) return "a channel step depends on host counters";
  if (c->has_bc) return "batches run periodic cases only (boundary routines set)";
  if (c->cracon) return "crash control decides on the host before each step";
  if (c->prof) return "profiling is on";
  if (!c->metrics_set || !c->state_set) return "metrics or state not set";
  return std::string();
}

// The work lists of one step, every phase's items of all cases in a row.
template <typename T>
void batch_plan(astr_batch* b, std::vector<int4>& items) {
  items.clear();
  b->phases.clear();
  const int NL = v2_nl<T>();
  const int nc = (int)b->cases.size();
  auto push = [&](int op, int dir, int CH, int rep, bool stage0, size_t off) {
    const int n = (int)(items.size() - off);
    if (n > 0) b->phases.push_back(astr_batch::Phase{op, dir, CH, rep, off, n, stage0});
  };
  // sweeps of one op and direction, one launch per chunk length and set of
  // uniform-chunk constants (cases of one scheme share them)
  auto sweep = [&](int op, int dir) {
    auto takes = [&](const astr_ctx* c) {
      return dir < c->g.ndims && (op != BOP_FILTER || c->pm.lfilter) && (op != BOP_VISC || c->pm.diffterm);
    };
    auto same = [&](const astr_ctx* a, const astr_ctx* c) {
      const bool f = op == BOP_FILTER;
      if ((f ? a->CHf[dir] : a->CH[dir]) != (f ? c->CHf[dir] : c->CH[dir])) return false;
      const astr_ctx::V2U& ua = f ? a->v2uf[dir] : a->v2ud[dir];
      const astr_ctx::V2U& uc = f ? c->v2uf[dir] : c->v2ud[dir];
      return std::memcmp(&ua, &uc, sizeof(ua)) == 0;
    };
    std::vector<int> reps;
    for (int i = 0; i < nc; ++i) {
      if (!takes(b->cases[i])) continue;
      bool found = false;
      for (int r : reps) found = found || same(b->cases[r], b->cases[i]);
      if (!found) reps.push_back(i);
    }
    for (int r : reps) {
      const size_t off = items.size();
      const int ch = op == BOP_FILTER ? b->cases[r]->CHf[dir] : b->cases[r]->CH[dir];
      for (int i = 0; i < nc; ++i) {
        const astr_ctx* c = b->cases[i];
        if (!takes(c) || !same(b->cases[r], c)) continue;
        int gx, gy;
        v2_blocks(c->g, dir, NL, gx, gy);
        const int nz = !c->vsplit ? 1 : (op == BOP_FILTER ? 5 : (op == BOP_CONVGRAD ? 9 : 4));
        for (int z = 0; z < nz; ++z)
          for (int y = 0; y < gy; ++y)
            for (int x = 0; x < gx; ++x) items.push_back(make_int4(i, x, y, z));
      }
      push(op, dir, ch, r, false, off);
    }
  };
  auto points = [&](int op, bool stage0) {
    const size_t off = items.size();
    for (int i = 0; i < nc; ++i) {
      const astr_ctx* c = b->cases[i];
      if (op == BOP_SIGMA && !c->pm.diffterm) continue;
      const long long nb = (c->g.n0 + KB_PTS - 1) / KB_PTS;
      for (long long x = 0; x < nb; ++x) items.push_back(make_int4(i, (int)x, 0, 0));
    }
    push(op, 0, 0, 0, stage0, off);
  };
  for (int dir = 0; dir < 3; ++dir) sweep(BOP_FILTER, dir);
  for (int dir = 0; dir < 3; ++dir) {
    const size_t off = items.size();
    for (int i = 0; i < nc; ++i) {
      const astr_ctx* c = b->cases[i];
      if (!c->g.per[dir]) continue;
      const Geo& g = c->g;
      const int na = dir == 0 ? g.jm : g.im, nb = dir == 2 ? g.jm : g.km;
      const int nx = (na + KB_THREADS) / KB_THREADS;
      for (int y = 0; y <= nb; ++y)
        for (int x = 0; x < nx; ++x) items.push_back(make_int4(i, x, y, 0));
    }
    push(BOP_QSWAP, dir, 0, 0, false, off);
  }
  points(BOP_QSAVE, true);
  for (int dir = 0; dir < 3; ++dir) sweep(BOP_CONVGRAD, dir);
  points(BOP_SIGMA, false);
  for (int dir = 0; dir < 3; ++dir) sweep(BOP_VISC, dir);
  points(BOP_RK, false);
}

template <typename T>
void batch_desc(astr_ctx* c, BCase<T>& o) {
  std::memset((void*)&o, 0, sizeof(o));
  o.g = c->g;
  o.d = dev<T>(c);
  o.ph = c->ph;
  o.Tb = ftab<T>(c);
  for (int dir = 0; dir < 3; ++dir) {
    o.Sd[dir] = v2_sd<T>(c, dir);
    o.Sf[dir] = v2_sf<T>(c, dir);
  }
  o.vsplit = c->vsplit ? 1 : 0;
}

template <typename T>
int batch_launch(astr_batch* b, const astr_batch::Phase& p, int stage, const BatchCtl& ctl) {
  const BCase<T>* cs = (const BCase<T>*)b->dcases;
  const int4* it = b->ditems + p.off;
  cudaError_t e = cudaSuccess;
  if (p.op <= BOP_VISC) {
    const V2Args<T> a = v2_args<T>(b->cases[p.rep], p.dir, p.op == BOP_FILTER);
    const int nsm = std::max(1, (int)(b->nsm * b->share + 0.5));
    e = p.dir == 0 ? astr::launch2_batch<T, 0>(p.op, p.CH, a, cs, it, p.n, ctl, nsm, b->st)
                   : (p.dir == 1 ? astr::launch2_batch<T, 1>(p.op, p.CH, a, cs, it, p.n, ctl, nsm, b->st)
                                 : astr::launch2_batch<T, 2>(p.op, p.CH, a, cs, it, p.n, ctl, nsm, b->st));
  } else {
    const int kind = p.op == BOP_QSWAP ? p.dir : (p.op == BOP_QSAVE ? 3 : (p.op == BOP_SIGMA ? 4 : 5));
    const unsigned grid = (unsigned)std::min(p.n, std::max(1, (int)(b->nsm * b->share * 8 + 0.5)));
    kb_point<T><<<grid, KB_THREADS, 0, b->st>>>(cs, it, p.n, kind, stage, ctl);
    e = cudaGetLastError();
  }
  ++b->launches;
  if (e != cudaSuccess) return bfail(b, ASTR_ERR_CUDA, std::string("batched launch: ") + cudaGetErrorString(e));
  return ASTR_OK;
}

template <typename T>
int batch_enqueue(astr_batch* b, int nsteps, double budget_ms) {
  const size_t nc = b->cases.size();
  if (b->dirty) {
    std::vector<int4> items;
    batch_plan<T>(b, items);
    BCK(cudaStreamSynchronize(b->st));
    if (items.size() > b->items_cap) {
      if (b->ditems) BCK(cudaFree(b->ditems));
      b->ditems = nullptr;
      b->items_cap = 0;
      BCK(cudaMalloc(&b->ditems, items.size() * sizeof(int4)));
      b->items_cap = items.size();
    }
    if (!items.empty())
      BCK(cudaMemcpy(b->ditems, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    const size_t bytes = std::max<size_t>(nc, 1) * sizeof(BCase<T>);
    if (bytes > b->desc_cap) {
      if (b->dcases) BCK(cudaFree(b->dcases));
      if (b->hcases) BCK(cudaFreeHost(b->hcases));
      b->dcases = b->hcases = nullptr;
      b->desc_cap = 0;
      BCK(cudaMalloc(&b->dcases, bytes));
      BCK(cudaMallocHost(&b->hcases, bytes));
      b->desc_cap = bytes;
    }
    b->dirty = false;
  }
  // descriptors (time step, constants) as the contexts hold them now
  BCK(cudaEventSynchronize(b->ev_desc));
  BCase<T>* h = (BCase<T>*)b->hcases;
  for (size_t i = 0; i < nc; ++i) batch_desc<T>(b->cases[i], h[i]);
  BCK(cudaMemcpyAsync(b->dcases, b->hcases, nc * sizeof(BCase<T>), cudaMemcpyHostToDevice, b->st));
  BCK(cudaEventRecord(b->ev_desc, b->st));
  // after the work already queued on every case
  for (astr_ctx* c : b->cases) {
    BCK(cudaEventRecord(b->ev_in, c->st));
    BCK(cudaStreamWaitEvent(b->st, b->ev_in, 0));
  }
  ((volatile int*)b->hword)[0] = 0;
  BatchCtl ctl{b->hword_dev, b->ddeadline, b->dctl, b->dctl + 1};
  const unsigned long long budget = budget_ms > 0 ? (unsigned long long)(budget_ms * 1e6) : 0ULL;
  k_batch_start<<<1, 1, 0, b->st>>>(ctl, b->ddeadline, budget < 1 && budget_ms > 0 ? 1ULL : budget);
  BCK(cudaGetLastError());
  ++b->launches;
  for (int s = 0; s < nsteps; ++s) {
    k_batch_gate<<<1, 1, 0, b->st>>>(ctl);
    BCK(cudaGetLastError());
    ++b->launches;
    for (int stage = 0; stage < 3; ++stage)
      for (const astr_batch::Phase& p : b->phases)
        if (!p.stage0 || stage == 0) RC(batch_launch<T>(b, p, stage, ctl));
  }
  BCK(cudaMemcpyAsync(b->hword + 1, b->dctl, 2 * sizeof(int), cudaMemcpyDeviceToHost, b->st));
  BCK(cudaEventRecord(b->ev_done, b->st));
  // later work on each case waits for the batch
  for (astr_ctx* c : b->cases) BCK(cudaStreamWaitEvent(c->st, b->ev_done, 0));
  b->pending = true;
  return ASTR_OK;
}

// The call's outcome, once its work has finished.
void batch_finish(astr_batch* b) {
  const int status = ((volatile int*)b->hword)[1];
  const int started = ((volatile int*)b->hword)[2];
  for (astr_ctx* c : b->cases) c->nstep += started;
  b->result_steps = started;
  b->result = (status & 1) ? ASTR_ERR_CANCELLED : ((status & 2) ? ASTR_ERR_TIMEOUT : ASTR_OK);
  if (b->result == ASTR_ERR_CANCELLED) b->err = "cancelled";
  if (b->result == ASTR_ERR_TIMEOUT) b->err = "deadline passed";
  b->pending = false;
}

}  // namespace

static void batch_forget(astr_batch* b, astr_ctx* c) {
  if (b->pending) {
    cudaEventSynchronize(b->ev_done);
    batch_finish(b);
  }
  auto it = std::find(b->cases.begin(), b->cases.end(), c);
  if (it != b->cases.end()) b->cases.erase(it);
  c->batch = nullptr;
  b->dirty = true;
}

extern "C" {

int astr_batch_create(int precision, astr_batch** out) {
  if (!out) return ASTR_ERR_ARG;
  *out = nullptr;
  if (precision != ASTR_FP64 && precision != ASTR_FP32_STORAGE) return ASTR_ERR_ARG;
  astr_batch* b = new astr_batch();
  b->prec = precision;
  int dev = 0;
  auto bad = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    g_create_err = std::string("astr_batch_create: ") + cudaGetErrorString(e);
    astr_batch_destroy(b);
    return true;
  };
  if (bad(cudaGetDevice(&dev))) return ASTR_ERR_CUDA;
  if (bad(cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev))) return ASTR_ERR_CUDA;
  if (bad(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking))) return ASTR_ERR_CUDA;
  if (bad(cudaEventCreateWithFlags(&b->ev_desc, cudaEventDisableTiming))) return ASTR_ERR_CUDA;
  if (bad(cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming))) return ASTR_ERR_CUDA;
  if (bad(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming))) return ASTR_ERR_CUDA;
  if (bad(cudaMalloc(&b->dctl, 2 * sizeof(int)))) return ASTR_ERR_OOM;
  if (bad(cudaMalloc(&b->ddeadline, sizeof(unsigned long long)))) return ASTR_ERR_OOM;
  if (bad(cudaHostAlloc(&b->hword, 4 * sizeof(int), cudaHostAllocMapped))) return ASTR_ERR_OOM;
  std::memset(b->hword, 0, 4 * sizeof(int));
  if (bad(cudaHostGetDevicePointer((void**)&b->hword_dev, b->hword, 0))) return ASTR_ERR_CUDA;
  *out = b;
  return ASTR_OK;
}

void astr_batch_destroy(astr_batch* b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  for (astr_ctx* c : b->cases) c->batch = nullptr;
  if (b->ev_desc) cudaEventDestroy(b->ev_desc);
  if (b->ev_done) cudaEventDestroy(b->ev_done);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->dcases) cudaFree(b->dcases);
  if (b->hcases) cudaFreeHost(b->hcases);
  if (b->ditems) cudaFree(b->ditems);
  if (b->dctl) cudaFree(b->dctl);
  if (b->ddeadline) cudaFree(b->ddeadline);
  if (b->hword) cudaFreeHost(b->hword);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

int astr_batch_add(astr_batch* b, astr_ctx* c) {
  if (!b) return ASTR_ERR_ARG;
  if (!c) return bfail(b, ASTR_ERR_ARG, "null context");
  const std::string why = batch_refusal(c, b->prec);
  if (!why.empty()) return bfail(b, ASTR_ERR_UNSUPPORTED, why);
  if (c->batch) return bfail(b, ASTR_ERR_STATE, "the case is already in a batch");
  if (b->pending) return bfail(b, ASTR_ERR_STATE, "a batched call is in flight (astr_batch_wait)");
  b->cases.push_back(c);
  c->batch = b;
  b->dirty = true;
  return ASTR_OK;
}

int astr_batch_remove(astr_batch* b, astr_ctx* c) {
  if (!b) return ASTR_ERR_ARG;
  if (!c || c->batch != b) return bfail(b, ASTR_ERR_ARG, "the case is not in this batch");
  if (b->pending) return bfail(b, ASTR_ERR_STATE, "a batched call is in flight (astr_batch_wait)");
  batch_forget(b, c);
  return ASTR_OK;
}

int astr_batch_size(astr_batch* b) { return b ? (int)b->cases.size() : ASTR_ERR_ARG; }

int astr_batch_set_share(astr_batch* b, double share) {
  if (!b) return ASTR_ERR_ARG;
  if (!(share > 0.0 && share <= 1.0)) return bfail(b, ASTR_ERR_ARG, "share outside (0, 1]");
  b->share = share;
  return ASTR_OK;
}

int astr_batch_step_async(astr_batch* b, int nsteps, double budget_ms) {
  if (!b) return ASTR_ERR_ARG;
  if (nsteps < 0) return bfail(b, ASTR_ERR_ARG, "nsteps < 0");
  if (b->pending) return bfail(b, ASTR_ERR_STATE, "a batched call is in flight (astr_batch_wait)");
  for (astr_ctx* c : b->cases) {
    const std::string why = batch_refusal(c, b->prec);
    if (!why.empty()) return bfail(b, ASTR_ERR_UNSUPPORTED, why);
  }
  return b->prec == ASTR_FP64 ? batch_enqueue<double>(b, nsteps, budget_ms)
                              : batch_enqueue<float>(b, nsteps, budget_ms);
}

int astr_batch_poll(astr_batch* b) {
  if (!b) return ASTR_ERR_ARG;
  if (!b->pending) return 1;
  const cudaError_t e = cudaEventQuery(b->ev_done);
  if (e == cudaErrorNotReady) return 0;
  if (e != cudaSuccess) return bfail(b, ASTR_ERR_CUDA, std::string("astr_batch_poll: ") + cudaGetErrorString(e));
  batch_finish(b);
  return 1;
}

int astr_batch_wait(astr_batch* b, int* steps_done) {
  if (!b) return ASTR_ERR_ARG;
  if (b->pending) {
    BCK(cudaEventSynchronize(b->ev_done));
    batch_finish(b);
  }
  if (steps_done) *steps_done = b->result_steps;
  return b->result;
}

int astr_batch_cancel(astr_batch* b) {
  if (!b) return ASTR_ERR_ARG;
  ((volatile int*)b->hword)[0] = 1;
  return ASTR_OK;
}

int astr_batch_step(astr_batch* b, int nsteps, double budget_ms, int* steps_done) {
  RC(astr_batch_step_async(b, nsteps, budget_ms));
  return astr_batch_wait(b, steps_done);
}

int astr_batch_last_error(astr_batch* b, char* buf, int len) {
  const std::string& m = b ? b->err : g_create_err;
  if (buf && len > 0) {
    std::strncpy(buf, m.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)m.size();
}

long long astr_batch_launch_count(astr_batch* b) { return b ? b->launches : 0; }

}  // extern "C"
