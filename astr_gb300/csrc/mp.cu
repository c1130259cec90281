// Compact MP convective scheme on the device: kernels and launchers (see
// mp.cuh).  FP64 throughout, as the reference.
#include "mp.cuh"
#include "launch.cuh"

namespace astr {
namespace {

constexpr double GAM = 1.4;                       // ideal gas, no species
constexpr double N37D60 = 37.0 / 60.0, N2D15 = 2.0 / 15.0, N1D60 = 1.0 / 60.0;  // src/constdef.F90

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// The limiter's comparisons, minima and maxima run on the integer pipe (the
// FP64 pipe is the bound of these kernels): for doubles that are not NaN,
// x > 0 is bits(x) > 0, x < 0 is bits(-x) > 0, magnitudes order as
// bits & ~sign, and the order of two values is the order of their sortable
// keys (negative values with the magnitude bits flipped).  Results are
// bit-identical to the floating-point forms (a zero may come out as -0.0
// where those give +0.0, which no later sum can tell apart).
constexpr long long SIGN = (long long)0x8000000000000000ULL;
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double dval(long long b) { return __longlong_as_double(b); }
__device__ __forceinline__ long long dkey(double x) {
  const long long b = dbits(x);
  return b >= 0 ? b : b ^ 0x7fffffffffffffffLL;
}
__device__ __forceinline__ double dmin(double a, double b) { return dkey(a) <= dkey(b) ? a : b; }
__device__ __forceinline__ double dmax(double a, double b) { return dkey(a) >= dkey(b) ? a : b; }

// minmod2, minmod4: src/commfunc.F90:699-738
__device__ __forceinline__ double minmod2(double a, double b) {
  const long long ia = dbits(a), ib = dbits(b);
  if (ia > 0 && ib > 0) return ia <= ib ? a : b;
  const long long na = ia ^ SIGN, nb = ib ^ SIGN;
  if (na > 0 && nb > 0) return na <= nb ? a : b;
  return 0.0;
}
__device__ __forceinline__ double minmod4(double a, double b, double c, double d) {
  const long long ia = dbits(a), ib = dbits(b), ic = dbits(c), id = dbits(d);
  if (ia > 0 && ib > 0 && ic > 0 && id > 0) return dval(min(min(ia, ib), min(ic, id)));
  const long long na = ia ^ SIGN, nb = ib ^ SIGN, nc = ic ^ SIGN, nd = id ^ SIGN;
  if (na > 0 && nb > 0 && nc > 0 && nd > 0) return dval(min(min(na, nb), min(nc, nd)) ^ SIGN);
  return 0.0;
}

// MP5 with the compact value as the linear one (src/flux.F90:434-496;
// Suresh & Huynh, JCP 136, 1997), in two parts: the test whether the
// linear value needs limiting uses the three centre points only; the
// limiter itself needs all five.
__device__ __forceinline__ bool mp5_needs(double u1, double u2, double u3, double ulinear) {
  const double uMP = u2 + minmod2(u3 - u2, 4.0 * (u2 - u1));
  const double var1 = (ulinear - u2) * (ulinear - uMP);
  return dbits(var1) >= dbits(1.e-10);  // var1 >= 1e-10
}
__device__ __forceinline__ double mp5_limit(double u0, double u1, double u2, double u3, double u4,
                                            double ulinear) {
  const double dm1 = u0 - 2.0 * u1 + u2;
  const double d0 = u1 - 2.0 * u2 + u3;
  const double d1 = u2 - 2.0 * u3 + u4;
  const double dhm1 = minmod4(4.0 * dm1 - d0, 4.0 * d0 - dm1, dm1, d0);
  const double dh0 = minmod4(4.0 * d0 - d1, 4.0 * d1 - d0, d0, d1);
  const double uUL = u2 + 4.0 * (u2 - u1);
  const double uAV = 0.5 * (u2 + u3);
  const double uMD = uAV - 0.5 * dh0;
  const double uLC = u2 + 0.5 * (u2 - u1) + 1.333333333333333 * dhm1;
  const double uMIN = dmax(dmin(dmin(u2, u3), uMD), dmin(dmin(u2, uUL), uLC));
  const double uMAX = dmin(dmax(dmax(u2, u3), uMD), dmax(dmax(u2, uUL), uLC));
  return ulinear + minmod2(uMIN - ulinear, uMAX - ulinear);
}

// mplimiter (src/flux.F90:363-379) on a five-point stencil fetched by
// point index (0..4): the two outer points are fetched only when MP5
// limits.  shock false: MP5 returns the linear value.
template <class Fetch>
__device__ __forceinline__ double mplimiter(const Fetch& u, double fl, bool shock, int inode, int dim,
                                            int ntype) {
  if ((ntype == 1 && (inode == 0 || inode == 1)) || (ntype == 2 && (inode == dim - 1 || inode == dim - 2)))
    return fl;
  if (!shock) return fl;
  const double u1 = u(1), u2 = u(2), u3 = u(3);
  if (!mp5_needs(u1, u2, u3, fl)) return fl;
  return mp5_limit(u(0), u1, u2, u3, u(4), fl);
}

__device__ __forceinline__ void metric_row(const Geo& g, const DevT<double>& d, int DIR, long long p,
                                           double& x0, double& x1, double& x2) {
  if (d.xg) {
    x0 = d.xg[(3 * DIR + 0) * g.nh + p];
    x1 = d.xg[(3 * DIR + 1) * g.nh + p];
    x2 = d.xg[(3 * DIR + 2) * g.nh + p];
  } else {
    const double v = d.xd[DIR * g.nh + p];
    x0 = DIR == 0 ? v : 0.0;
    x1 = DIR == 1 ? v : 0.0;
    x2 = DIR == 2 ? v : 0.0;
  }
}

__device__ __forceinline__ bool box_node(const Box& b, long long t, int& i, int& j, int& k) {
  if (t >= b.count()) return false;
  i = b.i0 + (int)(t % b.ni);
  const long long r = t / b.ni;
  j = b.j0 + (int)(r % b.nj);
  k = b.k0 + (int)(r / b.nj);
  return true;
}

template <int DIR>
__device__ __forceinline__ int along(int i, int j, int k) { return DIR == 0 ? i : (DIR == 1 ? j : k); }

// ---------------------------------------------------------------------------
// Ducros sensor, src/commcal.F90:196-353
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mp_ssf(Geo g, DevT<double> d, MPDev m) {
  int i, j, k;
  const Box b{0, 0, 0, g.im + 1, g.jm + 1, g.km + 1};
  if (!box_node(b, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
  const long long z = zidx(g, i, j, k), n0 = g.n0;
  const double* G = d.grad + z;
  auto dv = [&](int n, int mm) { return G[((n - 1) + 3 * (mm - 1)) * n0]; };
  const double dsum = dv(1, 1) + dv(2, 2) + dv(3, 3);
  const double div2 = dsum * dsum;
  const double vx = dv(3, 2) - dv(2, 3), vy = dv(1, 3) - dv(3, 1), vz = dv(2, 1) - dv(1, 2);
  const double vort = vx * vx + vy * vy + vz * vz;
  int ip1 = i + 1, im1 = i - 1, jp1 = j + 1, jm1 = j - 1, kp1 = k + 1, km1 = k - 1;
  if (m.npdc[0] == 1 && im1 < 0) im1 = 0;
  if (m.npdc[1] == 1 && jm1 < 0) jm1 = 0;
  if (m.npdc[2] == 1 && km1 < 0) km1 = 0;
  if (m.npdc[0] == 2 && ip1 > g.im) ip1 = g.im;
  if (m.npdc[1] == 2 && jp1 > g.jm) jp1 = g.jm;
  if (m.npdc[2] == 2 && kp1 > g.km) kp1 = g.km;
  const double* P = d.pr + 4 * g.nh;
  const double p0 = P[hidx(g, i, j, k)];
  auto dp = [&](double pm, double pp) { return fabs(pp - 2.0 * p0 + pm) / (pp + 2.0 * p0 + pm); };
  const double dpdi = dp(P[hidx(g, im1, j, k)], P[hidx(g, ip1, j, k)]);
  const double dpdj = dp(P[hidx(g, i, jm1, k)], P[hidx(g, i, jp1, k)]);
  // 2-D: the k halo planes are copies of plane 0, so the k difference is 0
  const double dpdk = g.ndims == 3 ? dp(P[hidx(g, i, j, km1)], P[hidx(g, i, j, kp1)]) : 0.0;
  m.ssf[hidx(g, i, j, k)] = div2 / (div2 + vort + 1.e-30) * fmax(fmax(dpdi, dpdj), dpdk);
}

// dataswap(ssf) on one rank (src/parallel.F90:3499-…): the periodic copies
// of the homogeneous directions (2-D: the k planes are not needed, the
// lshock k-window is skipped).
__global__ void __launch_bounds__(256) k_mp_ssf_halo(Geo g, MPDev m) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nx = g.per[0] ? 10LL * (g.jm + 1) * (g.km + 1) : 0;
  const long long ny = g.per[1] ? 10LL * (g.im + 1) * (g.km + 1) : 0;
  const long long nz = (g.per[2] && g.ndims == 3) ? 10LL * (g.im + 1) * (g.jm + 1) : 0;
  double* s = m.ssf;
  if (t < nx) {
    const int h = (int)(t % 10);
    const long long r = t / 10;
    const int j = (int)(r % (g.jm + 1)), k = (int)(r / (g.jm + 1));
    if (h < 5) s[hidx(g, -1 - h, j, k)] = s[hidx(g, g.im - 1 - h, j, k)];
    else s[hidx(g, g.im + h - 4, j, k)] = s[hidx(g, h - 4, j, k)];
    return;
  }
  t -= nx;
  if (t < ny) {
    const int h = (int)(t % 10);
    const long long r = t / 10;
    const int i = (int)(r % (g.im + 1)), k = (int)(r / (g.im + 1));
    if (h < 5) s[hidx(g, i, -1 - h, k)] = s[hidx(g, i, g.jm - 1 - h, k)];
    else s[hidx(g, i, g.jm + h - 4, k)] = s[hidx(g, i, h - 4, k)];
    return;
  }
  t -= ny;
  if (t < nz) {
    const int h = (int)(t % 10);
    const long long r = t / 10;
    const int i = (int)(r % (g.im + 1)), j = (int)(r / (g.im + 1));
    if (h < 5) s[hidx(g, i, j, -1 - h)] = s[hidx(g, i, j, g.km - 1 - h)];
    else s[hidx(g, i, j, g.km + h - 4)] = s[hidx(g, i, j, h - 4)];
  }
}

__global__ void __launch_bounds__(256) k_mp_lshock(Geo g, MPDev m) {
  int i, j, k;
  const Box b{0, 0, 0, g.im + 1, g.jm + 1, g.km + 1};
  if (!box_node(b, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
  const double* s = m.ssf;
  double mx = 0.0;
  for (int o = -4; o <= 5; ++o) {
    int ii = i + o;
    if (m.npdc[0] == 1 && ii < 0) ii = 0;
    if (m.npdc[0] == 2 && ii > g.im) ii = g.im;
    mx = fmax(mx, s[hidx(g, ii, j, k)]);
  }
  for (int o = -4; o <= 5; ++o) {
    int jj = j + o;
    if (m.npdc[1] == 1 && jj < 0) jj = 0;
    if (m.npdc[1] == 2 && jj > g.jm) jj = g.jm;
    mx = fmax(mx, s[hidx(g, i, jj, k)]);
  }
  if (g.ndims == 3) {
    for (int o = -4; o <= 5; ++o) {
      int kk = k + o;
      if (m.npdc[2] == 1 && kk < 0) kk = 0;
      if (m.npdc[2] == 2 && kk > g.km) kk = g.km;
      mx = fmax(mx, s[hidx(g, i, j, kk)]);
    }
  }
  m.lshock[zidx(g, i, j, k)] = mx > m.shkcrt ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Steger-Warming split, src/riemann.F90:23-160 (nondimensional, sos =
// sqrt(T)/M, src/fludyna.F90:832-859)
// ---------------------------------------------------------------------------
template <int DIR>
__global__ void __launch_bounds__(256) k_mp_split(Geo g, DevT<double> d, MPDev m, Box b) {
  int i, j, k;
  if (!box_node(b, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
  const long long nh = g.nh, p = hidx(g, i, j, k);
  const double rho = d.pr[p], u = d.pr[nh + p], v = d.pr[2 * nh + p], w = d.pr[3 * nh + p];
  const double prs = d.pr[4 * nh + p], tmp = d.pr[5 * nh + p];
  const double q0 = d.q[p], q1 = d.q[nh + p], q2 = d.q[2 * nh + p], q3 = d.q[3 * nh + p], q4 = d.q[4 * nh + p];
  double x0, x1, x2;
  metric_row(g, d, DIR, p, x0, x1, x2);
  const double J = d.jac[p];
  double* F = m.fsw + p;
  // The divisions of the reference that only scale by constants or by
  // var0 are multiplications here (sos uses 1/M, csa = css |grad xi|, the
  // energy term 1/(gamma-1)), and the sonic test compares uu with csa
  // instead of uu/csa with 1: rounding-level differences.
  const double eps = 0.04;
  const double uu = x0 * u + x1 * v + x2 * w;
  const double sg = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
  const double var0 = 1.0 / sg;
  const double g0 = x0 * var0, g1 = x1 * var0, g2 = x2 * var0;
  const double gm2 = 0.5 / GAM;
  const double css = sqrt(tmp) * m.rmach;
  const double csa = css * sg;
  const bool sup = uu >= csa, sdn = uu <= -csa;
  if (sup || sdn) {
    const int on = sup ? 0 : 5, off = sup ? 5 : 0;
    F[(on + 0) * nh] = J * q0 * uu;
    F[(on + 1) * nh] = J * (q1 * uu + x0 * prs);
    F[(on + 2) * nh] = J * (q2 * uu + x1 * prs);
    F[(on + 3) * nh] = J * (q3 * uu + x2 * prs);
    F[(on + 4) * nh] = J * (q4 + prs) * uu;
    for (int n = 0; n < 5; ++n) F[(off + n) * nh] = 0.0;
    return;
  }
  const double lmda[3] = {uu, uu + csa, uu - csa};
  double lp[3], lm[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    lp[n] = 0.5 * (lmda[n] + sqrt(lmda[n] * lmda[n] + eps * eps));
    lm[n] = lmda[n] - lp[n];
  }
  const double fhi = 0.5 * (GAM - 1.0) * (u * u + v * v + w * w);
  const double jro = J * rho;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const double* L = s == 0 ? lp : lm;
    const double var1 = L[0];
    const double var2 = L[1] - L[2];
    const double var3 = 2.0 * L[0] - L[1] - L[2];
    const double var4 = var1 - var3 * gm2;
    double* Fs = F + 5 * s * nh;
    Fs[0] = jro * var4;
    Fs[nh] = jro * (var4 * u + var2 * css * g0 * gm2);
    Fs[2 * nh] = jro * (var4 * v + var2 * css * g1 * gm2);
    Fs[3 * nh] = jro * (var4 * w + var2 * css * g2 * gm2);
    Fs[4 * nh] = J * (var1 * q4 + rho * (var2 * uu * var0 * css * gm2 -
                                         var3 * (fhi + css * css) * gm2 * (1.0 / (GAM - 1.0))));
  }
}

// ---------------------------------------------------------------------------
// Compact upwind / downwind interface values, src/flux.F90:125-256: the ten
// split components of a line, one after the other, on the chunked Thomas
// solve of the block layout (lines across threadIdx.x, chunks across
// threadIdx.y).  Rows first..last = -2..dim+1 (periodic) or -1..dim
// (physical boundaries); interface i is stored at node i.
// ---------------------------------------------------------------------------
// Interior-row weights of the compact upwind right-hand side (bfacmpld folded in).
struct UpwindWeights {
  double x, y, z, w;
};

template <int DIR, int CH>
__global__ void __launch_bounds__(YZ_LINES * NCH_B, 1)
k_mp_cflux(Geo g, MPDev m, DScheme<double> SU, DScheme<double> SD, UpwindWeights wt) {
  __shared__ double sm[SCAN_SMEM_WORDS];
  LineMap<DIR, true> lm(g);
  const long long hs = hstride<DIR>(g), nh = g.nh;
  int i0, j0, k0;
  line_ijk<DIR>(lm.a, lm.b, 0, i0, j0, k0);
  const long long base = hidx(g, i0, j0, k0);
  constexpr int ta = DIR == 0 ? 1 : 0, tb = DIR == 2 ? 1 : 2;
  const bool cline = lm.active && lm.a >= g.lo[ta] && lm.a <= g.hi[ta] && lm.b >= g.lo[tb] &&
                     lm.b <= g.hi[tb];
  const int dim = SU.dim;
  int iss, iee;
  mp_split_range(m.npdc[DIR], dim, iss, iee);
#pragma unroll 1
  for (int v = 0; v < 10; ++v) {
    if (!my_task(v)) continue;
    const DScheme<double>& S = v < 5 ? SU : SD;
    const bool up = v < 5;
    const double* f = m.fsw + v * nh + base;
    const int s = lm.c * CH;
    const int nb = S.first + s - 2;
    double w[CH + 5];
#pragma unroll
    for (int t = 0; t < CH + 5; ++t) {
      const int nd = nb + t;
      w[t] = (nd >= iss && nd <= iee) ? __ldg(f + hs * nd) : 0.0;
    }
    double y[CH];
#pragma unroll
    for (int t = 0; t < CH; ++t) {
      const int r = s + t;
      const double* W = w + t + 2;  // W[o] = f(node + o)
      double dv = 0.0;
      if (r < S.n) {
        const bool wall = S.ntype == 4;
        if (wall && r == 0) dv = 2.5 * W[1] + 0.5 * W[2];
        else if (wall && r == 1) dv = 0.75 * W[0] + 0.75 * W[1];
        else if (wall && r == S.n - 2) dv = 0.75 * W[1] + 0.75 * W[0];
        else if (wall && r == S.n - 1) dv = 2.5 * W[0] + 0.5 * W[-1];
        else if (!wall && (r == 0 || r == S.n - 1)) {
          const double v1 = W[0] + W[1], v2 = W[-1] + W[2], v3 = W[-2] + W[3];
          dv = N37D60 * v1 - N2D15 * v2 + N1D60 * v3;
        } else if (up) {
          dv = wt.x * W[-1] + wt.y * W[0] + wt.z * W[1] + wt.w * W[2];
        } else {
          dv = wt.x * W[2] + wt.y * W[1] + wt.z * W[0] + wt.w * W[-1];
        }
        if (r > 0) dv = dv * __ldg(S.ac2 + r);
      }
      y[t] = dv;
    }
    chunk_solve<CH, DIR, true>(y, S, lm.c, sm, false);
    if (cline) {
      double* o = m.fhc + v * nh + base;
#pragma unroll
      for (int t = 0; t < CH; ++t) {
        const int r = s + t;
        const int node = S.first + r;
        if (r < S.n && node >= -1 && node <= dim) o[hs * node] = y[t];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Interface flux, src/solver.F90:1363-1497 (and the j, k copies): one
// thread per interface i (between nodes i and i+1) of a line.
// ---------------------------------------------------------------------------
// The sensor flag of interface f (between nodes f and f+1) of the line
// through (i, j, k).
template <int DIR>
__device__ __forceinline__ bool iface_shock(const Geo& g, const MPDev& m, int i, int j, int k, int f,
                                            int dim) {
  const long long zs = zstride<DIR>(g);
  const long long zb = zidx(g, i, j, k) - zs * f;
  auto ls = [&](int l) { return m.lshock[zb + zs * l] != 0; };
  if (f < 0) return ls(f + 1);
  if (f + 1 > dim) return ls(f);
  return ls(f) || ls(f + 1);
}

// Characteristic form, every interface: where the sensor is off at both
// nodes MP5 returns the linear value for every characteristic field, so the
// reference forms R L (fhcp + fhcm) with R L = I; the sum is written here
// (a rounding-level difference, eps * cond(R)).  Flagged interfaces are
// listed (warp-aggregated append) for k_mp_face, which then runs densely
// over them.
template <int DIR>
__global__ void __launch_bounds__(256) k_mp_face_split(Geo g, MPDev m, Box b) {
  int i, j, k;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = box_node(b, t, i, j, k);
  bool flagged = false;
  if (in) {
    const int f = along<DIR>(i, j, k);
    const int dim = DIR == 0 ? g.im : (DIR == 1 ? g.jm : g.km);
    flagged = iface_shock<DIR>(g, m, i, j, k, f, dim);
    if (!flagged) {
      const long long nh = g.nh, p = hidx(g, i, j, k);
      const double* HC = m.fhc + p;
#pragma unroll
      for (int r = 0; r < 5; ++r) m.fh[r * nh + p] = HC[r * nh] + HC[(5 + r) * nh];
    }
  }
  const unsigned mask = __ballot_sync(0xffffffffu, flagged);
  if (mask == 0u) return;
  const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(m.fcount, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (flagged) m.flist[base + __popc(mask & ((1u << lane) - 1u))] = (int)t;
}

// Interface flux with the limiter: every interface of the box (no
// characteristic decomposition: the MP5 test runs everywhere), or the
// listed ones (characteristic form: the flagged interfaces).
template <int DIR>
__global__ void __launch_bounds__(128) k_mp_face(Geo g, DevT<double> d, MPDev m, Box b, int listed) {
  int i, j, k;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (listed) {
    if (t >= *m.fcount) return;
    t = m.flist[t];
  }
  if (!box_node(b, t, i, j, k)) return;
  const int f = along<DIR>(i, j, k);  // interface index
  const long long nh = g.nh, hs = hstride<DIR>(g);
  const long long p = hidx(g, i, j, k);
  const long long base = p - hs * f;
  const int dim = DIR == 0 ? g.im : (DIR == 1 ? g.jm : g.km);
  const int npdc = m.npdc[DIR];
  int iss, iee;
  mp_split_range(npdc, dim, iss, iee);
  // stencil nodes, iwind6 (src/solver.F90:1236-1257)
  int wp[5], wm[5];
#pragma unroll
  for (int n = 0; n < 5; ++n) {
    wp[n] = clampi(f + n - 2, iss, iee);
    wm[n] = clampi(f + 3 - n, iss, iee);
  }
  // without the characteristic decomposition there is no sensor and MP5
  // limits everywhere; with it, only flagged interfaces reach this kernel
  const bool lsh = true;
  const double* FP = m.fsw + base;
  const double* FM = m.fsw + 5 * nh + base;
  const double* HC = m.fhc + p;
  double* out = m.fh + p;
  if (!m.chard) {
#pragma unroll 1
    for (int c = 0; c < 5; ++c) {
      const double* a = FP + c * nh;
      const double* z = FM + c * nh;
      auto up = [&](int n) { return __ldg(a + hs * wp[n]); };
      auto dn = [&](int n) { return __ldg(z + hs * wm[n]); };
      const double v1 = mplimiter(up, HC[c * nh], lsh, f, dim, npdc);
      const double v2 = mplimiter(dn, HC[(5 + c) * nh], lsh, f, dim, npdc);
      out[c * nh] = v1 + v2;
    }
    return;
  }
  // chardecomp, src/solver.F90:1958-2162, between nodes f and f+1
  const long long pr_ = p + hs;
  const double* P = d.pr;
  const double ro_l = P[p], ro_r = P[pr_];
  const double ul[3] = {P[nh + p], P[2 * nh + p], P[3 * nh + p]};
  const double ur[3] = {P[nh + pr_], P[2 * nh + pr_], P[3 * nh + pr_]};
  const double E_l = d.q[4 * nh + p], E_r = d.q[4 * nh + pr_];
  const double p_l = P[4 * nh + p], p_r = P[4 * nh + pr_];
  double xl0, xl1, xl2, xr0, xr1, xr2;
  metric_row(g, d, DIR, p, xl0, xl1, xl2);
  metric_row(g, d, DIR, pr_, xr0, xr1, xr2);
  const double WRoe = sqrt(ro_l) / (sqrt(ro_l) + sqrt(ro_r));
  const double WRoe1 = 1.0 - WRoe;
  const double u1 = WRoe * ul[0] + WRoe1 * ur[0];
  const double u2 = WRoe * ul[1] + WRoe1 * ur[1];
  const double u3 = WRoe * ul[2] + WRoe1 * ur[2];
  const double KRoe = 0.5 * (u1 * u1 + u2 * u2 + u3 * u3);
  const double HRoe = WRoe * ((E_l + p_l) / ro_l) + WRoe1 * ((E_r + p_r) / ro_r);
  const double Css = sqrt((GAM - 1.0) * (HRoe - KRoe));
  const double rcs = 1.0 / Css;
  const double var1 = 0.5 * (xl0 + xr0), var2 = 0.5 * (xl1 + xr1), var3 = 0.5 * (xl2 + xr2);
  const double var4 = 1.0 / sqrt(var1 * var1 + var2 * var2 + var3 * var3);
  const double g1 = var1 * var4, g2 = var2 * var4, g3 = var3 * var4;
  const double ugp = u1 * g1 + u2 * g2 + u3 * g3;
  const double b1 = (GAM - 1.0) / (Css * Css);
  const double b2 = 1.0 + 2.0 * b1 * KRoe - b1 * HRoe;
  const int br = fabs(var1) > 1.e-12 ? 0 : (fabs(var2) > 1.e-12 ? 1 : 2);
  const double rgp = 1.0 / (br == 0 ? g1 : (br == 1 ? g2 : g3));
  double Fh[5];
#pragma unroll 1
  for (int c = 0; c < 5; ++c) {
    // LEV(c+1, :) and REV(:, c+1)
    double L[5], R[5];
    if (c == 0) {
      L[0] = 0.5 * (b2 + ugp * rcs); L[1] = -0.5 * (b1 * u1 + g1 * rcs);
      L[2] = -0.5 * (b1 * u2 + g2 * rcs); L[3] = -0.5 * (b1 * u3 + g3 * rcs); L[4] = 0.5 * b1;
      R[0] = 1.0; R[1] = u1 - Css * g1; R[2] = u2 - Css * g2; R[3] = u3 - Css * g3; R[4] = HRoe - ugp * Css;
    } else if (c == 1) {
      L[0] = 1.0 - b2; L[1] = b1 * u1; L[2] = b1 * u2; L[3] = b1 * u3; L[4] = -b1;
      R[0] = 1.0; R[1] = u1; R[2] = u2; R[3] = u3; R[4] = HRoe - 1.0 / b1;
    } else if (c == 4) {
      L[0] = 0.5 * (b2 - ugp * rcs); L[1] = -0.5 * (b1 * u1 - g1 * rcs);
      L[2] = -0.5 * (b1 * u2 - g2 * rcs); L[3] = -0.5 * (b1 * u3 - g3 * rcs); L[4] = 0.5 * b1;
      R[0] = 1.0; R[1] = u1 + Css * g1; R[2] = u2 + Css * g2; R[3] = u3 + Css * g3; R[4] = HRoe + ugp * Css;
    } else if (br == 0) {
      if (c == 2) {
        L[0] = (ugp * g2 - u2) * rgp; L[1] = -g2; L[2] = (1.0 - g2 * g2) * rgp; L[3] = -g2 * g3 * rgp; L[4] = 0.0;
        R[0] = 0.0; R[1] = -g2; R[2] = g1; R[3] = 0.0; R[4] = u2 * g1 - u1 * g2;
      } else {
        L[0] = (ugp * g3 - u3) * rgp; L[1] = -g3; L[2] = -g2 * g3 * rgp; L[3] = (1.0 - g3 * g3) * rgp; L[4] = 0.0;
        R[0] = 0.0; R[1] = -g3; R[2] = 0.0; R[3] = g1; R[4] = u3 * g1 - u1 * g3;
      }
    } else if (br == 1) {
      if (c == 2) {
        L[0] = (ugp * g1 - u1) * rgp; L[1] = (1.0 - g1 * g1) * rgp; L[2] = -g1; L[3] = -g1 * g3 * rgp; L[4] = 0.0;
        R[0] = 0.0; R[1] = g2; R[2] = -g1; R[3] = 0.0; R[4] = u1 * g2 - u2 * g1;
      } else {
        L[0] = (ugp * g3 - u3) * rgp; L[1] = -g1 * g3 * rgp; L[2] = -g3; L[3] = (1.0 - g3 * g3) * rgp; L[4] = 0.0;
        R[0] = 0.0; R[1] = 0.0; R[2] = -g3; R[3] = g2; R[4] = u3 * g2 - u2 * g3;
      }
    } else {
      if (c == 2) {
        L[0] = (ugp * g1 - u1) * rgp; L[1] = (1.0 - g1 * g1) * rgp; L[2] = -g1 * g2 * rgp; L[3] = -g1; L[4] = 0.0;
        R[0] = 0.0; R[1] = g3; R[2] = 0.0; R[3] = -g1; R[4] = u1 * g3 - u3 * g1;
      } else {
        L[0] = (ugp * g2 - u2) * rgp; L[1] = -g1 * g2 * rgp; L[2] = (1.0 - g2 * g2) * rgp; L[3] = -g2; L[4] = 0.0;
        R[0] = 0.0; R[1] = 0.0; R[2] = g3; R[3] = -g2; R[4] = u2 * g3 - u3 * g2;
      }
    }
    // projections onto field c of the compact values and, where the
    // limiter may act, of the stencil points
    auto proj = [&](const double* a) {
      return L[0] * __ldg(a) + L[1] * __ldg(a + nh) + L[2] * __ldg(a + 2 * nh) +
             L[3] * __ldg(a + 3 * nh) + L[4] * __ldg(a + 4 * nh);
    };
    auto up = [&](int n) { return proj(FP + hs * wp[n]); };
    auto dn = [&](int n) { return proj(FM + hs * wm[n]); };
    const double hp = L[0] * HC[0] + L[1] * HC[nh] + L[2] * HC[2 * nh] + L[3] * HC[3 * nh] + L[4] * HC[4 * nh];
    const double hm = L[0] * HC[5 * nh] + L[1] * HC[6 * nh] + L[2] * HC[7 * nh] + L[3] * HC[8 * nh] +
                      L[4] * HC[9 * nh];
    const double Fc = mplimiter(up, hp, lsh, f, dim, npdc) + mplimiter(dn, hm, lsh, f, dim, npdc);
#pragma unroll
    for (int r = 0; r < 5; ++r) Fh[r] = c == 0 ? R[r] * Fc : Fh[r] + R[r] * Fc;
  }
#pragma unroll
  for (int r = 0; r < 5; ++r) out[r * nh] = Fh[r];
}

// qrhs(l) = qrhs(l) + Fh(l) - Fh(l-1); after the last direction rhscal's
// negation (src/solver.F90:1500-1504 and the j, k copies; 242).
template <int DIR>
__global__ void __launch_bounds__(256) k_mp_diff(Geo g, DevT<double> d, MPDev m, Box b, int last) {
  int i, j, k;
  if (!box_node(b, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
  const long long nh = g.nh, n0 = g.n0, hs = hstride<DIR>(g);
  const long long p = hidx(g, i, j, k), z = zidx(g, i, j, k);
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    double* R = d.qrhs + r * n0 + z;
    const double* F = m.fh + r * nh + p;
    double v = *R + F[0] - F[-hs];
    *R = last ? -v : v;
  }
}

dim3 grid_of(long long n, int threads) { return dim3((unsigned)((n + threads - 1) / threads)); }

// The node box of one direction: a0..a1 along DIR, is..ie across.
template <int DIR>
Box dir_box(const Geo& g, int a0, int a1) {
  Box b;
  b.i0 = DIR == 0 ? a0 : g.lo[0];
  b.ni = DIR == 0 ? a1 - a0 + 1 : g.hi[0] - g.lo[0] + 1;
  b.j0 = DIR == 1 ? a0 : g.lo[1];
  b.nj = DIR == 1 ? a1 - a0 + 1 : g.hi[1] - g.lo[1] + 1;
  b.k0 = DIR == 2 ? a0 : g.lo[2];
  b.nk = DIR == 2 ? a1 - a0 + 1 : g.hi[2] - g.lo[2] + 1;
  return b;
}

template <int DIR>
int dim_of(const Geo& g) { return DIR == 0 ? g.im : (DIR == 1 ? g.jm : g.km); }

}  // namespace

cudaError_t launch_mp_sensor(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st,
                             int part) {
  if (part == 0) {
    k_mp_ssf<<<grid_of(g.n0, 256), 256, 0, st>>>(g, d, m);
  } else if (part == 1) {
    const long long n = 10LL * ((g.jm + 1) * (long long)(g.km + 1) + (g.im + 1) * (long long)(g.km + 1) +
                                (g.im + 1) * (long long)(g.jm + 1));
    k_mp_ssf_halo<<<grid_of(n, 256), 256, 0, st>>>(g, m);
  } else {
    k_mp_lshock<<<grid_of(g.n0, 256), 256, 0, st>>>(g, m);
  }
  return cudaGetLastError();
}

template <int DIR>
cudaError_t launch_mp_split(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st) {
  int a0, a1;
  mp_split_range(m.npdc[DIR], dim_of<DIR>(g), a0, a1);
  const Box b = dir_box<DIR>(g, a0, a1);
  k_mp_split<DIR><<<grid_of(b.count(), 256), 256, 0, st>>>(g, d, m, b);
  return cudaGetLastError();
}

template <int DIR>
cudaError_t launch_mp_cflux(const Geo& g, const MPDev& m, const MPSchemes& S, cudaStream_t st) {
  const int lb = S.lbb[DIR];
  dim3 gr = sweep_grid<DIR, true>(g, lb);
  const dim3 bl = sweep_block<DIR, true>(lb);
  gr.z = S.vsplit ? 10 : 1;
  // compact upwind RHS weights, src/flux.F90:243-253
  const double b = m.bfac;
  const UpwindWeights wt{1.0 / 18.0 - 1.0 / 36.0 * b, 19.0 / 18.0 - 9.0 / 36.0 * b,
                         5.0 / 9.0 + 9.0 / 36.0 * b, 1.0 / 36.0 * b};
  switch (S.CH[DIR]) {
    case 3: k_mp_cflux<DIR, 3><<<gr, bl, 0, st>>>(g, m, S.uw[DIR], S.dw[DIR], wt); break;
    case 5: k_mp_cflux<DIR, 5><<<gr, bl, 0, st>>>(g, m, S.uw[DIR], S.dw[DIR], wt); break;
    case 9: k_mp_cflux<DIR, 9><<<gr, bl, 0, st>>>(g, m, S.uw[DIR], S.dw[DIR], wt); break;
    case 17: k_mp_cflux<DIR, 17><<<gr, bl, 0, st>>>(g, m, S.uw[DIR], S.dw[DIR], wt); break;
    case 33: k_mp_cflux<DIR, 33><<<gr, bl, 0, st>>>(g, m, S.uw[DIR], S.dw[DIR], wt); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int DIR>
cudaError_t launch_mp_face(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st) {
  const Box b = dir_box<DIR>(g, g.lo[DIR] - 1, g.hi[DIR]);
  if (!m.chard) {
    k_mp_face<DIR><<<grid_of(b.count(), 128), 128, 0, st>>>(g, d, m, b, 0);
    return cudaGetLastError();
  }
  cudaError_t e = cudaMemsetAsync(m.fcount, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_mp_face_split<DIR><<<grid_of(b.count(), 256), 256, 0, st>>>(g, m, b);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // sized for every interface; threads past the listed count return at once
  k_mp_face<DIR><<<grid_of(b.count(), 128), 128, 0, st>>>(g, d, m, b, 1);
  return cudaGetLastError();
}

template <int DIR>
cudaError_t launch_mp_diff(const Geo& g, const DevT<double>& d, const MPDev& m, cudaStream_t st,
                           int last) {
  const Box b = dir_box<DIR>(g, g.lo[DIR], g.hi[DIR]);
  k_mp_diff<DIR><<<grid_of(b.count(), 256), 256, 0, st>>>(g, d, m, b, last);
  return cudaGetLastError();
}

#define ASTR_INSTANTIATE_MP(DIR)                                                                  \
  template cudaError_t launch_mp_split<DIR>(const Geo&, const DevT<double>&, const MPDev&,         \
                                            cudaStream_t);                                        \
  template cudaError_t launch_mp_cflux<DIR>(const Geo&, const MPDev&, const MPSchemes&,            \
                                            cudaStream_t);                                        \
  template cudaError_t launch_mp_face<DIR>(const Geo&, const DevT<double>&, const MPDev&,          \
                                           cudaStream_t);                                         \
  template cudaError_t launch_mp_diff<DIR>(const Geo&, const DevT<double>&, const MPDev&,          \
                                           cudaStream_t, int);
ASTR_INSTANTIATE_MP(0)
ASTR_INSTANTIATE_MP(1)
ASTR_INSTANTIATE_MP(2)

}  // namespace astr
