// ORACLE — test infrastructure only (see astr_oracle.h).
//
// CPU FP64 restatement of the ASTR right-hand-side hot path.  Every routine
// below names the reference routine it restates (file:line, paths relative to
// the ASTR source tree).  Operation order inside each expression follows the
// Fortran left-to-right evaluation of the reference so that, built with
// -ffp-contract=off, the arithmetic is the reference's own.
#include "astr_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const int HM = 5;                 // halo width, src/commvar.F90:184
const double PI = 4.0 * std::atan(1.0);   // src/constdef.F90:12
const double NUM1D3 = 1.0 / 3.0, NUM2D3 = 2.0 / 3.0;
const double NUM7D9 = 7.0 / 9.0, NUM1D36 = 1.0 / 36.0, NUM1D60 = 1.0 / 60.0;

// compact_scheme (src/commtype.F90:13-23) with the Thomas factors of
// tridiagonal_thomas_proprocess (src/commfunc.F90:752-774).
struct Scheme {
  int first = 0, last = 0, dim = 0, ntype = 3;
  std::vector<double> a, c, ac1, ac2, ac3;  // index node-first
  int n() const { return last - first + 1; }
  void alloc() {
    int m = n();
    a.assign(m, 0.0); c.assign(m, 0.0);
    ac1.assign(m, 0.0); ac2.assign(m, 0.0); ac3.assign(m, 0.0);
  }
  // src/commfunc.F90:752-774
  void preprocess() {
    int m = n();
    ac1[0] = c[0];
    for (int i = 1; i < m; ++i) {
      ac1[i] = c[i] / (1.0 - a[i] * ac1[i - 1]);
      ac2[i] = 1.0 / (1.0 - a[i] * ac1[i - 1]);
      ac3[i] = a[i] / (1.0 - a[i] * ac1[i - 1]);
    }
  }
  // src/commfunc.F90:790-813 (d is overwritten, x returned in x)
  void solve(double* d, double* x) const {
    int m = n();
    for (int i = 1; i < m; ++i) d[i] = d[i] * ac2[i] - d[i - 1] * ac3[i];
    x[m - 1] = d[m - 1];
    for (int i = m - 2; i >= 0; --i) x[i] = d[i] - ac1[i] * x[i + 1];
  }
};

struct FilterTables {  // src/filter.F90:299-432
  double c2i[2], c4i[3], c6i[4], c8i[5], c10i[6];
  double cb[5][9];   // coefb(0:4,0:8)
  double ch[5][11];  // coefh(0:4,0:10)
};

}  // namespace

struct orc_ctx {
  orc_config cfg;
  int im, jm, km, ndims;
  long NI, NJ, NK, nh, n0;
  int is, ie, js, je, ks, ke;
  double const1, const2, const3, const4, const5, const6, const7;
  double tempconst, tempconst1, pinf, roinf, uinf, tinf;
  double dxm, dym, dzm;  // mini-app uniform spacings
  Scheme fd[3], flt[3];
  Scheme fuw[3], fdw[3];  // compact upwind / downwind interface-flux schemes
  FilterTables ft;
  // halo arrays
  std::vector<double> q, rho, vel, prs, tmp, x, dxi, jacob, sigma, qflux;
  // interior arrays
  std::vector<double> qrhs, qsave, dvel, dtmp;
  std::vector<double> ssf;              // shock-sensor function (halo array)
  std::vector<unsigned char> lshock;    // lshock(0:im,0:jm,0:km)
  // inflow (bctypes 11 and 12 on xmin): vel_in(0:jm,0:km,1:3),
  // tmp_in(0:jm,0:km), tmp_prof(0:jm), prs_in(0:jm,0:km) (alloinflow,
  // src/bc.F90:69-83; freestreaminflow's values, src/bc.F90:7950-8003,
  // until the host sets a profile)
  std::vector<double> vel_in, tmp_in, tmp_prof, prs_in;
  bool sson = false;                    // allocated(lshock)
  double force[3] = {0, 0, 0};
  double massflux_target = 0.0;
  double massflux = 0.0, fbcx = 0.0;  // last statcal values (channel)
  long nstep = 0;                     // completed time steps
  bool rkfirst_called = false;        // rkfirst's firstcall flag

  inline long h(int i, int j, int k) const {
    return (long)(i + HM) + NI * ((long)(j + HM) + NJ * (long)(k + HM));
  }
  inline long z(int i, int j, int k) const {
    return (long)i + (long)(im + 1) * ((long)j + (long)(jm + 1) * (long)k);
  }
  int dimof(int d) const { return d == 0 ? im : (d == 1 ? jm : km); }
  int npdc(int d) const { return d == 0 ? cfg.npdci : (d == 1 ? cfg.npdcj : cfg.npdck); }
  bool homo(int d) const { return npdc(d) == 3; }
  // stride (in elements) of a halo array along direction d
  long hstride(int d) const { return d == 0 ? 1 : (d == 1 ? NI : NI * NJ); }
  long zstride(int d) const {
    return d == 0 ? 1 : (d == 1 ? (long)(im + 1) : (long)(im + 1) * (jm + 1));
  }
};

namespace {

// ---------------------------------------------------------------------------
// Scheme set-up
// ---------------------------------------------------------------------------

// fd_scheme_initiate, src/derivative.F90:63-158 (scheme '643c')
void fd_scheme_initiate(Scheme& s, int ntype, int dim) {
  int i0 = 0, imx = 0;
  switch (ntype) {
    case 1: i0 = 0; imx = dim + 1; break;
    case 2: i0 = -1; imx = dim; break;
    case 3: i0 = -1; imx = dim + 1; break;
    default: i0 = 0; imx = dim; break;
  }
  s.first = i0; s.last = imx; s.dim = dim; s.ntype = ntype;
  s.alloc();
  for (int i = 0; i < s.n(); ++i) { s.a[i] = NUM1D3; s.c[i] = NUM1D3; }
  s.a[0] = 0.0; s.c[0] = 0.0;
  s.a[imx - i0] = 0.0; s.c[imx - i0] = 0.0;
  if (ntype == 1 || ntype == 4) {
    s.a[0] = 2.0; s.c[0] = 2.0;
    s.a[1] = 0.25; s.c[1] = 0.25;
  }
  if (ntype == 2 || ntype == 4) {
    s.a[imx - i0] = 2.0; s.c[imx - i0] = 2.0;
    s.a[imx - 1 - i0] = 0.25; s.c[imx - 1 - i0] = 0.25;
  }
  s.preprocess();
}

// compact_filter_initiate, src/filter.F90:31-100
void compact_filter_initiate(Scheme& s, int ntype, int dim, double alfa) {
  int i0 = 0, imx = 0;
  double b0 = 0, bm = 0;
  switch (ntype) {
    case 1: i0 = 0; imx = dim + 3; b0 = 0.98; bm = 1.11; break;
    case 2: i0 = -3; imx = dim; b0 = 1.11; bm = 0.98; break;
    case 3: i0 = -3; imx = dim + 3; b0 = 1.11; bm = 1.11; break;
    default: i0 = 0; imx = dim; b0 = 0.98; bm = 0.98; break;
  }
  s.first = i0; s.last = imx; s.dim = dim; s.ntype = ntype;
  s.alloc();
  for (int i = 0; i < s.n(); ++i) { s.a[i] = alfa; s.c[i] = alfa; }
  s.a[0] = b0; s.c[0] = b0;
  s.a[imx - i0] = bm; s.c[imx - i0] = bm;
  s.preprocess();
}

// filter_coefficient_cal, src/filter.F90:299-432
void filter_coefficient_cal(FilterTables& t, double alfa, double bh, double bb) {
  t.c2i[0] = (1.0 + 2.0 * alfa) / 4.0;
  t.c2i[1] = (1.0 + 2.0 * alfa) / 4.0;
  t.c4i[0] = (5.0 + 6.0 * alfa) / 16.0;
  t.c4i[1] = (1.0 + 2.0 * alfa) / 4.0;
  t.c4i[2] = (-1.0 + 2.0 * alfa) / 16.0;
  t.c6i[0] = (11.0 + 10.0 * alfa) / 32.0;
  t.c6i[1] = (15.0 + 34.0 * alfa) / 64.0;
  t.c6i[2] = (-3.0 + 6.0 * alfa) / 32.0;
  t.c6i[3] = (1.0 - 2.0 * alfa) / 64.0;
  t.c8i[0] = (93.0 + 70.0 * alfa) / 256.0;
  t.c8i[1] = (7.0 + 18.0 * alfa) / 32.0;
  t.c8i[2] = (-7.0 + 14.0 * alfa) / 64.0;
  t.c8i[3] = (1.0 - 2.0 * alfa) / 32.0;
  t.c8i[4] = (-1.0 + 2.0 * alfa) / 256.0;
  t.c10i[0] = (193.0 + 126.0 * alfa) / 512.0;
  t.c10i[1] = (105.0 + 302.0 * alfa) / 512.0;
  t.c10i[2] = (-15.0 + 30.0 * alfa) / 128.0;
  t.c10i[3] = (45.0 - 90.0 * alfa) / 1024.0;
  t.c10i[4] = (-5.0 + 10.0 * alfa) / 512.0;
  t.c10i[5] = (1.0 - 2.0 * alfa) / 1024.0;
  std::memset(t.cb, 0, sizeof(t.cb));
  t.cb[3][0] = (1.0 - 2.0 * alfa) / 256.0;
  t.cb[3][1] = (-1.0 + 2.0 * alfa) / 32.0;
  t.cb[3][2] = (7.0 + 50.0 * alfa) / 64.0;
  t.cb[3][3] = (25.0 + 14.0 * alfa) / 32.0;
  t.cb[3][4] = (35.0 + 58.0 * alfa) / 128.0;
  t.cb[3][5] = (-7.0 + 14.0 * alfa) / 32.0;
  t.cb[3][6] = (7.0 - 14.0 * alfa) / 64.0;
  t.cb[3][7] = (-1.0 + 2.0 * alfa) / 32.0;
  t.cb[3][8] = (1.0 - 2.0 * alfa) / 256.0;
  t.cb[2][0] = (-1.0 + 2.0 * alfa) / 64.0;
  t.cb[2][1] = (3.0 + 26.0 * alfa) / 32.0;
  t.cb[2][2] = (49.0 + 30.0 * alfa) / 64.0;
  t.cb[2][3] = (5.0 + 6.0 * alfa) / 16.0;
  t.cb[2][4] = (-15.0 + 30.0 * alfa) / 64.0;
  t.cb[2][5] = (3.0 - 6.0 * alfa) / 32.0;
  t.cb[2][6] = (-1.0 + 2.0 * alfa) / 64.0;
  t.cb[1][0] = (1.0 + 62.0 * alfa) / 64.0;
  t.cb[1][1] = (29.0 + 6.0 * alfa) / 32.0;
  t.cb[1][2] = (15.0 + 34.0 * alfa) / 64.0;
  t.cb[1][3] = (-5.0 + 10.0 * alfa) / 16.0;
  t.cb[1][4] = (15.0 - 30.0 * alfa) / 64.0;
  t.cb[1][5] = (-3.0 + 6.0 * alfa) / 32.0;
  t.cb[1][6] = (1.0 - 2.0 * alfa) / 64.0;
  t.cb[0][0] = (63.0 + 1.0 * bb) / 64.0;
  t.cb[0][1] = (3.0 + 29.0 * bb) / 32.0;
  t.cb[0][2] = (-15.0 + 15.0 * bb) / 64.0;
  t.cb[0][3] = (5.0 - 5.0 * bb) / 16.0;
  t.cb[0][4] = (-15.0 + 15.0 * bb) / 64.0;
  t.cb[0][5] = (3.0 - 3.0 * bb) / 32.0;
  t.cb[0][6] = (-1.0 + 1.0 * bb) / 64.0;
  std::memset(t.ch, 0, sizeof(t.ch));
  t.ch[0][0] = (-1.0 + 1.0 * bh) / 1024.0;
  t.ch[0][1] = (5.0 - 5.0 * bh) / 512.0;
  t.ch[0][2] = (979.0 + 45.0 * bh) / 1024.0;
  t.ch[0][3] = (15.0 + 113.0 * bh) / 128.0;
  t.ch[0][4] = (-105.0 + 105.0 * bh) / 512.0;
  t.ch[0][5] = (63.0 - 63.0 * bh) / 256.0;
  t.ch[0][6] = (-105.0 + 105.0 * bh) / 512.0;
  t.ch[0][7] = (15.0 - 15.0 * bh) / 128.0;
  t.ch[0][8] = (-45.0 + 45.0 * bh) / 1024.0;
  t.ch[0][9] = (5.0 - 5.0 * bh) / 512.0;
  t.ch[0][10] = (-1.0 + 1.0 * bh) / 1024.0;
  t.ch[1][0] = (1.0 - 2.0 * alfa) / 1024.0;
  t.ch[1][1] = (-5.0 + 10.0 * alfa) / 512.0;
  t.ch[1][2] = (45.0 + 934.0 * alfa) / 1024.0;
  t.ch[1][3] = (113.0 + 30.0 * alfa) / 128.0;
  t.ch[1][4] = (105.0 + 302.0 * alfa) / 512.0;
  t.ch[1][5] = (-63.0 + 126.0 * alfa) / 256.0;
  t.ch[1][6] = (105.0 - 210.0 * alfa) / 512.0;
  t.ch[1][7] = (-15.0 + 30.0 * alfa) / 128.0;
  t.ch[1][8] = (45.0 - 90.0 * alfa) / 1024.0;
  t.ch[1][9] = (-5.0 + 10.0 * alfa) / 512.0;
  t.ch[1][10] = (1.0 - 2.0 * alfa) / 1024.0;
  t.ch[2][0] = (-1.0 + 2.0 * alfa) / 1024.0;
  t.ch[2][1] = (5.0 - 10.0 * alfa) / 512.0;
  t.ch[2][2] = (-45.0 + 90.0 * alfa) / 1024.0;
  t.ch[2][3] = (15.0 + 98.0 * alfa) / 128.0;
  t.ch[2][4] = (407.0 + 210.0 * alfa) / 512.0;
  t.ch[2][5] = (63.0 + 130.0 * alfa) / 256.0;
  t.ch[2][6] = (-105.0 + 210.0 * alfa) / 512.0;
  t.ch[2][7] = (15.0 - 30.0 * alfa) / 128.0;
  t.ch[2][8] = (-45.0 + 90.0 * alfa) / 1024.0;
  t.ch[2][9] = (5.0 - 10.0 * alfa) / 512.0;
  t.ch[2][10] = (-1.0 + 2.0 * alfa) / 1024.0;
}

// ---------------------------------------------------------------------------
// Line kernels.  f points at node 0 of a contiguous line with valid entries
// f[-HM .. dim+HM].
// ---------------------------------------------------------------------------

// compact_fd_rhs, src/derivative.F90:210-306 ; df_compact 171-198
void df_compact(const Scheme& s, const double* f, double* df, double* d, double* xx) {
  const int i0 = s.first, imx = s.last, nt = s.ntype;
  auto D = [&](int j) -> double& { return d[j - i0]; };
  int is_, ie_;
  if (nt == 1 || nt == 4) {
    is_ = i0 + 2;
    int j = i0 + 1;
    double v1 = f[j + 1] - f[j - 1];
    D(j) = 0.75 * v1;
    j = i0;
    D(j) = -2.5 * f[j] + 2.0 * f[j + 1] + 0.5 * f[j + 2];
  } else {
    is_ = i0 + 1;
    int j = i0;
    double v1 = f[j + 1] - f[j - 1], v2 = f[j + 2] - f[j - 2], v3 = f[j + 3] - f[j - 3];
    D(j) = 0.75 * v1 - 0.15 * v2 + NUM1D60 * v3;
  }
  if (nt == 2 || nt == 4) {
    ie_ = imx - 2;
    int j = imx - 1;
    double v1 = f[j + 1] - f[j - 1];
    D(j) = 0.75 * v1;
    j = imx;
    D(j) = 2.5 * f[j] - 2.0 * f[j - 1] - 0.5 * f[j - 2];
  } else {
    ie_ = imx - 1;
    int j = imx;
    double v1 = f[j + 1] - f[j - 1], v2 = f[j + 2] - f[j - 2], v3 = f[j + 3] - f[j - 3];
    D(j) = 0.75 * v1 - 0.15 * v2 + NUM1D60 * v3;
  }
  for (int j = is_; j <= ie_; ++j) {
    double v1 = f[j + 1] - f[j - 1], v2 = f[j + 2] - f[j - 2];
    D(j) = NUM7D9 * v1 + NUM1D36 * v2;
  }
  s.solve(d, xx);
  for (int j = 0; j <= s.dim; ++j) df[j] = xx[j - i0];
}

// compact_filter_rhs, src/filter.F90:156-285 ; compact_filter 112-144
void compact_filter(const Scheme& s, const FilterTables& t, const double* f, double* ff,
                    double* d, double* xx) {
  const int i0 = s.first, imx = s.last, nt = s.ntype;
  auto D = [&](int j) -> double& { return d[j - i0]; };
  int is_, ie_;
  if (nt == 1 || nt == 4) {
    is_ = i0 + 5;
    for (int k = i0; k <= i0 + 2; ++k) {
      double v0 = 0.0;
      for (int j = 0; j <= 6; ++j) v0 = v0 + t.cb[k - i0][j] * f[i0 + j];
      D(k) = v0;
    }
    int j = i0 + 3;
    double v0 = f[j] + f[j], v1 = f[j + 1] + f[j - 1], v2 = f[j + 2] + f[j - 2], v3 = f[j + 3] + f[j - 3];
    D(j) = t.c6i[0] * v0 + t.c6i[1] * v1 + t.c6i[2] * v2 + t.c6i[3] * v3;
    j = i0 + 4;
    v0 = f[j] + f[j]; v1 = f[j + 1] + f[j - 1]; v2 = f[j + 2] + f[j - 2]; v3 = f[j + 3] + f[j - 3];
    double v4 = f[j + 4] + f[j - 4];
    D(j) = t.c8i[0] * v0 + t.c8i[1] * v1 + t.c8i[2] * v2 + t.c8i[3] * v3 + t.c8i[4] * v4;
  } else {
    is_ = i0 + 3;
    for (int k = i0; k <= i0 + 2; ++k) {
      double v0 = 0.0;
      for (int j = 0; j <= 10; ++j) v0 = v0 + t.ch[k - i0][j] * f[i0 - 2 + j];
      D(k) = v0;
    }
  }
  if (nt == 2 || nt == 4) {
    ie_ = imx - 5;
    for (int k = imx - 2; k <= imx; ++k) {
      double v0 = 0.0;
      for (int j = 0; j <= 6; ++j) v0 = v0 + t.cb[imx - k][j] * f[imx - j];
      D(k) = v0;
    }
    int j = imx - 3;
    double v0 = f[j] + f[j], v1 = f[j + 1] + f[j - 1], v2 = f[j + 2] + f[j - 2], v3 = f[j + 3] + f[j - 3];
    D(j) = t.c6i[0] * v0 + t.c6i[1] * v1 + t.c6i[2] * v2 + t.c6i[3] * v3;
    j = imx - 4;
    v0 = f[j] + f[j]; v1 = f[j + 1] + f[j - 1]; v2 = f[j + 2] + f[j - 2]; v3 = f[j + 3] + f[j - 3];
    double v4 = f[j + 4] + f[j - 4];
    D(j) = t.c8i[0] * v0 + t.c8i[1] * v1 + t.c8i[2] * v2 + t.c8i[3] * v3 + t.c8i[4] * v4;
  } else {
    ie_ = imx - 3;
    for (int k = imx - 2; k <= imx; ++k) {
      double v0 = 0.0;
      for (int j = 0; j <= 10; ++j) v0 = v0 + t.ch[imx - k][j] * f[imx + 2 - j];
      D(k) = v0;
    }
  }
  for (int j = is_; j <= ie_; ++j) {
    double v0 = f[j] + f[j], v1 = f[j + 1] + f[j - 1], v2 = f[j + 2] + f[j - 2];
    double v3 = f[j + 3] + f[j - 3], v4 = f[j + 4] + f[j - 4], v5 = f[j + 5] + f[j - 5];
    D(j) = t.c10i[0] * v0 + t.c10i[1] * v1 + t.c10i[2] * v2 + t.c10i[3] * v3 +
           t.c10i[4] * v4 + t.c10i[5] * v5;
  }
  s.solve(d, xx);
  for (int j = 0; j <= s.dim; ++j) ff[j] = xx[j - i0];
  if (nt == 1 || nt == 4) ff[0] = f[0];
  if (nt == 2 || nt == 4) ff[s.dim] = f[s.dim];
}

// Per-thread scratch for one line.
struct LineBuf {
  std::vector<double> fb, ob, d, xx;
  explicit LineBuf(int dim) : fb(dim + 2 * HM + 1), ob(dim + 1), d(dim + 16), xx(dim + 16) {}
  double* f() { return fb.data() + HM; }
};

inline int nthreads_env() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Iterate the lines of direction d over a rectangle of the two transverse
// indices.  fn(a, b) gets the two transverse indices in (i,j,k) order with
// the line index removed.
template <typename Fn>
void for_lines(const orc_ctx& c, int d, int a0, int a1, int b0, int b1, Fn fn) {
  (void)c; (void)d;
  long na = a1 - a0 + 1, nb = b1 - b0 + 1;
  if (na <= 0 || nb <= 0) return;
#pragma omp parallel
  {
    fn(-1, -1);  // per-thread init hook (allocates scratch)
#pragma omp for collapse(2) schedule(static)
    for (long b = 0; b < nb; ++b)
      for (long a = 0; a < na; ++a) fn((int)(a0 + a), (int)(b0 + b));
  }
}

// position of the (line index l, transverse a, b) node, halo layout
inline long hpos(const orc_ctx& c, int d, int l, int a, int b) {
  if (d == 0) return c.h(l, a, b);
  if (d == 1) return c.h(a, l, b);
  return c.h(a, b, l);
}
inline long zpos(const orc_ctx& c, int d, int l, int a, int b) {
  if (d == 0) return c.z(l, a, b);
  if (d == 1) return c.z(a, l, b);
  return c.z(a, b, l);
}
// transverse ranges (interior) for direction d
inline void trans_range(const orc_ctx& c, int d, int& a1, int& b1) {
  if (d == 0) { a1 = c.jm; b1 = c.km; }
  else if (d == 1) { a1 = c.im; b1 = c.km; }
  else { a1 = c.im; b1 = c.jm; }
}

// ---------------------------------------------------------------------------
// Halo swaps, single rank (src/parallel.F90)
// ---------------------------------------------------------------------------

// array4d_sendrecv single-rank branches, src/parallel.F90:4169-4174,
// 4229-4238, 4294-4303: periodic copy of nvar components of a halo array.
void dataswap(orc_ctx& c, double* var, int nvar, int dir) {
  const int im = c.im, jm = c.jm, km = c.km;
  if ((dir == 1 || dir == 0) && c.homo(0)) {
#pragma omp parallel for collapse(2)
    for (int n = 0; n < nvar; ++n)
      for (int k = 0; k <= km; ++k) {
        double* v = var + (long)n * c.nh;
        for (int j = 0; j <= jm; ++j) {
          for (int i = -HM; i <= -1; ++i) v[c.h(i, j, k)] = v[c.h(im + i, j, k)];
          for (int i = im + 1; i <= im + HM; ++i) v[c.h(i, j, k)] = v[c.h(i - im, j, k)];
        }
      }
  }
  if ((dir == 2 || dir == 0) && c.homo(1)) {
#pragma omp parallel for collapse(2)
    for (int n = 0; n < nvar; ++n)
      for (int k = 0; k <= km; ++k) {
        double* v = var + (long)n * c.nh;
        if (c.cfg.ja == 0) {
          for (int j = -HM; j <= HM; ++j)
            for (int i = 0; i <= im; ++i) v[c.h(i, j, k)] = v[c.h(i, 0, k)];
        } else {
          for (int j = -HM; j <= -1; ++j)
            for (int i = 0; i <= im; ++i) v[c.h(i, j, k)] = v[c.h(i, jm + j, k)];
          for (int j = jm + 1; j <= jm + HM; ++j)
            for (int i = 0; i <= im; ++i) v[c.h(i, j, k)] = v[c.h(i, j - jm, k)];
        }
      }
  }
  if ((dir == 3 || dir == 0) && c.homo(2)) {
#pragma omp parallel for
    for (int n = 0; n < nvar; ++n) {
      double* v = var + (long)n * c.nh;
      if (c.cfg.ka == 0) {
        for (int k = -HM; k <= HM; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) v[c.h(i, j, k)] = v[c.h(i, j, 0)];
      } else {
        for (int k = -HM; k <= -1; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) v[c.h(i, j, k)] = v[c.h(i, j, km + k)];
        for (int k = km + 1; k <= km + HM; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) v[c.h(i, j, k)] = v[c.h(i, j, k - km)];
      }
    }
  }
}

// q2fvar_3da (src/fludyna.F90:545-634, nondimensional, no species) at one node
inline void q2fvar_node(orc_ctx& c, long p) {
  const long nh = c.nh;
  double ro = c.q[p];
  c.rho[p] = ro;
  double u = c.q[p + nh] / ro, v = c.q[p + 2 * nh] / ro, w = c.q[p + 3 * nh] / ro;
  c.vel[p] = u; c.vel[p + nh] = v; c.vel[p + 2 * nh] = w;
  double pr = (c.q[p + 4 * nh] - 0.5 * ro * (u * u + v * v + w * w)) / c.const6;
  c.prs[p] = pr;
  c.tmp[p] = pr / ro * c.const2;  // thermal_3d(pressure,density)
}

void q2fvar_box(orc_ctx& c, int i0, int i1, int j0, int j1, int k0, int k1) {
#pragma omp parallel for collapse(2)
  for (int k = k0; k <= k1; ++k)
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) q2fvar_node(c, c.h(i, j, k));
}

// mini-app fvar2q with pressure (miniapps/tgv_solver_3d/tgvsolver.F90:48-71)
inline void fvar2q_prs_node(orc_ctx& c, long p) {
  const long nh = c.nh;
  double ro = c.rho[p], u = c.vel[p], v = c.vel[p + nh], w = c.vel[p + 2 * nh];
  c.q[p] = ro;
  c.q[p + nh] = ro * u;
  c.q[p + 2 * nh] = ro * v;
  c.q[p + 3 * nh] = ro * w;
  double var1 = 0.5 * (u * u + v * v + w * w);
  c.q[p + 4 * nh] = c.prs[p] * c.const6 + ro * var1;
}


// ---------------------------------------------------------------------------
// Compact MP convective scheme (conschm 543c)
// ---------------------------------------------------------------------------
const double GAMMA = 1.4;  // src/commvar.F90 (ideal gas, no species)
const double NUM1D6 = 1.0 / 6.0, NUM1D18 = 1.0 / 18.0, NUM19D18 = 19.0 / 18.0;
const double NUM5D9 = 5.0 / 9.0, NUM9D36 = 9.0 / 36.0, NUM2D15 = 2.0 / 15.0;
const double NUM37D60 = 37.0 / 60.0;  // src/constdef.F90:15-26

// compact_flux_initiate, src/flux.F90:32-112 (scheme 543)
void compact_flux_initiate(Scheme& s, int ntype, int dim, int wind, double b) {
  int i0 = -2, imx = dim + 1;
  switch (ntype) {
    case 1: i0 = -1; imx = dim + 1; break;
    case 2: i0 = -2; imx = dim; break;
    case 3: i0 = -2; imx = dim + 1; break;
    default: i0 = -1; imx = dim; break;
  }
  s.first = i0; s.last = imx; s.dim = dim; s.ntype = ntype;
  s.alloc();
  const double lo = 0.5 - NUM1D6 * b, hi = NUM1D6 + NUM1D6 * b;
  for (int i = 0; i < s.n(); ++i) {
    s.a[i] = wind > 0 ? lo : hi;
    s.c[i] = wind > 0 ? hi : lo;
  }
  s.a[0] = 0.0; s.c[0] = 0.0;
  s.a[imx - i0] = 0.0; s.c[imx - i0] = 0.0;
  if (ntype == 1 || ntype == 4) {
    s.a[0] = 2.0; s.c[0] = 2.0;
    s.a[1] = 0.25; s.c[1] = 0.25;
  }
  if (ntype == 2 || ntype == 4) {
    s.a[imx - i0] = 2.0; s.c[imx - i0] = 2.0;
    s.a[imx - 1 - i0] = 0.25; s.c[imx - 1 - i0] = 0.25;
  }
  s.preprocess();
}

// compact_flux_rhs, src/flux.F90:163-256 ; flux_compact 125-150.
// f points at node 0 (valid -HM..dim+HM); fh receives interfaces -1..dim.
void flux_compact(const Scheme& s, int wind, double b, const double* f, double* fh, double* d,
                  double* xx) {
  const int i0 = s.first, imx = s.last, nt = s.ntype;
  auto D = [&](int j) -> double& { return d[j - i0]; };
  int is_ = i0 + 1, ie_ = imx - 1;
  if (nt == 1 || nt == 4) {
    int j = i0;
    D(j) = 2.5 * f[j + 1] + 0.5 * f[j + 2];
    j = i0 + 1;
    D(j) = 0.75 * f[j] + 0.75 * f[j + 1];
    is_ = i0 + 2;
  } else {
    int j = i0;
    double v1 = f[j] + f[j + 1], v2 = f[j - 1] + f[j + 2], v3 = f[j - 2] + f[j + 3];
    D(j) = NUM37D60 * v1 - NUM2D15 * v2 + NUM1D60 * v3;
  }
  if (nt == 2 || nt == 4) {
    int j = imx - 1;
    D(j) = 0.75 * f[j + 1] + 0.75 * f[j];
    j = imx;
    D(j) = 2.5 * f[j] + 0.5 * f[j - 1];
    ie_ = imx - 2;
  } else {
    int j = imx;
    double v1 = f[j] + f[j + 1], v2 = f[j - 1] + f[j + 2], v3 = f[j - 2] + f[j + 3];
    D(j) = NUM37D60 * v1 - NUM2D15 * v2 + NUM1D60 * v3;
  }
  const double w0 = NUM1D18 - NUM1D36 * b, w1 = NUM19D18 - NUM9D36 * b;
  const double w2 = NUM5D9 + NUM9D36 * b, w3 = NUM1D36 * b;
  if (wind > 0) {
    for (int j = is_; j <= ie_; ++j) D(j) = w0 * f[j - 1] + w1 * f[j] + w2 * f[j + 1] + w3 * f[j + 2];
  } else {
    for (int j = is_; j <= ie_; ++j) D(j) = w0 * f[j + 2] + w1 * f[j + 1] + w2 * f[j] + w3 * f[j - 1];
  }
  s.solve(d, xx);
  for (int j = -1; j <= s.dim; ++j) fh[j + 1] = xx[j - i0];
}

// flux_steger_warming, src/riemann.F90:23-160 (nondimensional, no species)
void steger_warming(double mach, double rho, const double* vel, double prs, double tmp,
                    const double* q, const double* dxi, double jac, double* fp, double* fm) {
  const double eps = 0.04;
  const double uu = dxi[0] * vel[0] + dxi[1] * vel[1] + dxi[2] * vel[2];
  const double var0 = 1.0 / std::sqrt(dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2]);
  const double gpd[3] = {dxi[0] * var0, dxi[1] * var0, dxi[2] * var0};
  const double gm2 = 0.5 / GAMMA;
  const double css = std::sqrt(tmp) / mach;  // sos, src/fludyna.F90:832-859
  const double csa = css / var0;
  const double lmach = uu / csa;
  if (lmach >= 1.0) {
    fp[0] = jac * q[0] * uu;
    fp[1] = jac * (q[1] * uu + dxi[0] * prs);
    fp[2] = jac * (q[2] * uu + dxi[1] * prs);
    fp[3] = jac * (q[3] * uu + dxi[2] * prs);
    fp[4] = jac * (q[4] + prs) * uu;
    for (int n = 0; n < 5; ++n) fm[n] = 0.0;
    return;
  }
  if (lmach <= -1.0) {
    for (int n = 0; n < 5; ++n) fp[n] = 0.0;
    fm[0] = jac * q[0] * uu;
    fm[1] = jac * (q[1] * uu + dxi[0] * prs);
    fm[2] = jac * (q[2] * uu + dxi[1] * prs);
    fm[3] = jac * (q[3] * uu + dxi[2] * prs);
    fm[4] = jac * (q[4] + prs) * uu;
    return;
  }
  const double lmda[3] = {uu, uu + csa, uu - csa};  // lmda(1)=lmda(2)=lmda(3), (4), (5)
  double lp[3], lm[3];
  for (int n = 0; n < 3; ++n) {
    lp[n] = 0.5 * (lmda[n] + std::sqrt(lmda[n] * lmda[n] + eps * eps));
    lm[n] = lmda[n] - lp[n];
  }
  const double fhi = 0.5 * (GAMMA - 1.0) * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
  const double jro = jac * rho;
  for (int s = 0; s < 2; ++s) {
    const double* L = s == 0 ? lp : lm;
    double* F = s == 0 ? fp : fm;
    const double var1 = L[0];
    const double var2 = L[1] - L[2];
    const double var3 = 2.0 * L[0] - L[1] - L[2];
    const double var4 = var1 - var3 * gm2;
    F[0] = jro * var4;
    F[1] = jro * (var4 * vel[0] + var2 * css * gpd[0] * gm2);
    F[2] = jro * (var4 * vel[1] + var2 * css * gpd[1] * gm2);
    F[3] = jro * (var4 * vel[2] + var2 * css * gpd[2] * gm2);
    F[4] = jac * (var1 * q[4] + rho * (var2 * uu * var0 * css * gm2 -
                                       var3 * (fhi + css * css) * gm2 / (GAMMA - 1.0)));
  }
}

// chardecomp, src/solver.F90:1958-2162 (no species).  st = {T, rho, p, E,
// u, v, w, dxi1, dxi2, dxi3}.  R, L column-major 5x5: R[(m-1)+5(n-1)] = REV(m,n).
void chardecomp(const double* stl, const double* str, double* R, double* L) {
  auto rv = [&](int m, int n) -> double& { return R[(m - 1) + 5 * (n - 1)]; };
  auto lv = [&](int m, int n) -> double& { return L[(m - 1) + 5 * (n - 1)]; };
  const double ro_l = stl[1], p_l = stl[2], E_l = stl[3];
  const double ro_r = str[1], p_r = str[2], E_r = str[3];
  const double* vl = stl + 4;
  const double* vr = str + 4;
  const double rero = 1.e-12;
  const double WRoe = std::sqrt(ro_l) / (std::sqrt(ro_l) + std::sqrt(ro_r));
  const double WRoe1 = 1.0 - WRoe;
  const double u1 = WRoe * vl[0] + WRoe1 * vr[0];
  const double u2 = WRoe * vl[1] + WRoe1 * vr[1];
  const double u3 = WRoe * vl[2] + WRoe1 * vr[2];
  const double KRoe = 0.5 * (u1 * u1 + u2 * u2 + u3 * u3);
  const double HL = (E_l + p_l) / ro_l;
  const double HR = (E_r + p_r) / ro_r;
  const double HRoe = WRoe * HL + WRoe1 * HR;
  const double Css = std::sqrt((GAMMA - 1.0) * (HRoe - KRoe));
  const double rcs = 1.0 / Css;
  const double var1 = 0.5 * (stl[7] + str[7]);
  const double var2 = 0.5 * (stl[8] + str[8]);
  const double var3 = 0.5 * (stl[9] + str[9]);
  const double var4 = 1.0 / std::sqrt(var1 * var1 + var2 * var2 + var3 * var3);
  const double g1 = var1 * var4, g2 = var2 * var4, g3 = var3 * var4;
  const double ugp = u1 * g1 + u2 * g2 + u3 * g3;
  const double b1 = (GAMMA - 1.0) / (Css * Css);
  const double b2 = 1.0 + 2.0 * b1 * KRoe - b1 * HRoe;
  lv(1, 1) = 0.5 * (b2 + ugp * rcs);
  lv(1, 2) = -0.5 * (b1 * u1 + g1 * rcs);
  lv(1, 3) = -0.5 * (b1 * u2 + g2 * rcs);
  lv(1, 4) = -0.5 * (b1 * u3 + g3 * rcs);
  lv(1, 5) = 0.5 * b1;
  rv(1, 1) = 1.0;
  rv(2, 1) = u1 - Css * g1;
  rv(3, 1) = u2 - Css * g2;
  rv(4, 1) = u3 - Css * g3;
  rv(5, 1) = HRoe - ugp * Css;
  lv(2, 1) = 1.0 - b2;
  lv(2, 2) = b1 * u1;
  lv(2, 3) = b1 * u2;
  lv(2, 4) = b1 * u3;
  lv(2, 5) = -b1;
  rv(1, 2) = 1.0;
  rv(2, 2) = u1;
  rv(3, 2) = u2;
  rv(4, 2) = u3;
  rv(5, 2) = HRoe - 1.0 / b1;
  if (std::fabs(var1) > rero) {
    const double rgp = 1.0 / g1;
    lv(3, 1) = (ugp * g2 - u2) * rgp;
    lv(3, 2) = -g2;
    lv(3, 3) = (1.0 - g2 * g2) * rgp;
    lv(3, 4) = -g2 * g3 * rgp;
    lv(3, 5) = 0.0;
    lv(4, 1) = (ugp * g3 - u3) * rgp;
    lv(4, 2) = -g3;
    lv(4, 3) = -g2 * g3 * rgp;
    lv(4, 4) = (1.0 - g3 * g3) * rgp;
    lv(4, 5) = 0.0;
    rv(1, 3) = 0.0; rv(2, 3) = -g2; rv(3, 3) = g1; rv(4, 3) = 0.0; rv(5, 3) = u2 * g1 - u1 * g2;
    rv(1, 4) = 0.0; rv(2, 4) = -g3; rv(3, 4) = 0.0; rv(4, 4) = g1; rv(5, 4) = u3 * g1 - u1 * g3;
  } else if (std::fabs(var2) > rero) {
    const double rgp = 1.0 / g2;
    lv(3, 1) = (ugp * g1 - u1) * rgp;
    lv(3, 2) = (1.0 - g1 * g1) * rgp;
    lv(3, 3) = -g1;
    lv(3, 4) = -g1 * g3 * rgp;
    lv(3, 5) = 0.0;
    lv(4, 1) = (ugp * g3 - u3) * rgp;
    lv(4, 2) = -g1 * g3 * rgp;
    lv(4, 3) = -g3;
    lv(4, 4) = (1.0 - g3 * g3) * rgp;
    lv(4, 5) = 0.0;
    rv(1, 3) = 0.0; rv(2, 3) = g2; rv(3, 3) = -g1; rv(4, 3) = 0.0; rv(5, 3) = u1 * g2 - u2 * g1;
    rv(1, 4) = 0.0; rv(2, 4) = 0.0; rv(3, 4) = -g3; rv(4, 4) = g2; rv(5, 4) = u3 * g2 - u2 * g3;
  } else {
    // the reference stops when all three components are below rero
    const double rgp = 1.0 / g3;
    lv(3, 1) = (ugp * g1 - u1) * rgp;
    lv(3, 2) = (1.0 - g1 * g1) * rgp;
    lv(3, 3) = -g1 * g2 * rgp;
    lv(3, 4) = -g1;
    lv(3, 5) = 0.0;
    lv(4, 1) = (ugp * g2 - u2) * rgp;
    lv(4, 2) = -g1 * g2 * rgp;
    lv(4, 3) = (1.0 - g2 * g2) * rgp;
    lv(4, 4) = -g2;
    lv(4, 5) = 0.0;
    rv(1, 3) = 0.0; rv(2, 3) = g3; rv(3, 3) = 0.0; rv(4, 3) = -g1; rv(5, 3) = u1 * g3 - u3 * g1;
    rv(1, 4) = 0.0; rv(2, 4) = 0.0; rv(3, 4) = g3; rv(4, 4) = -g2; rv(5, 4) = u2 * g3 - u3 * g2;
  }
  lv(5, 1) = 0.5 * (b2 - ugp * rcs);
  lv(5, 2) = -0.5 * (b1 * u1 - g1 * rcs);
  lv(5, 3) = -0.5 * (b1 * u2 - g2 * rcs);
  lv(5, 4) = -0.5 * (b1 * u3 - g3 * rcs);
  lv(5, 5) = 0.5 * b1;
  rv(1, 5) = 1.0;
  rv(2, 5) = u1 + Css * g1;
  rv(3, 5) = u2 + Css * g2;
  rv(4, 5) = u3 + Css * g3;
  rv(5, 5) = HRoe + ugp * Css;
}

// minmod2, minmod4: src/commfunc.F90:699-738
inline double minmod2(double a, double b) {
  if (a > 0.0 && b > 0.0) return std::min(std::fabs(a), std::fabs(b));
  if (a < 0.0 && b < 0.0) return -1.0 * std::min(std::fabs(a), std::fabs(b));
  return 0.0;
}
inline double minmod4(double a, double b, double c, double d) {
  if (a > 0.0 && b > 0.0 && c > 0.0 && d > 0.0)
    return std::min(std::min(std::fabs(a), std::fabs(b)), std::min(std::fabs(c), std::fabs(d)));
  if (a < 0.0 && b < 0.0 && c < 0.0 && d < 0.0)
    return -1.0 * std::min(std::min(std::fabs(a), std::fabs(b)), std::min(std::fabs(c), std::fabs(d)));
  return 0.0;
}

// MP5 with a supplied linear value, src/flux.F90:434-496 (Suresh & Huynh 1997)
double mp5(const double* u, double ulinear, bool lskt) {
  const double u1 = u[0], u2 = u[1], u3 = u[2], u4 = u[3], u5 = u[4];
  double var1 = u4 - u3;
  double var2 = 4.0 * (u3 - u2);
  const double uMP = u3 + minmod2(var1, var2);
  var1 = (ulinear - u3) * (ulinear - uMP);
  if (lskt && var1 >= 1.e-10) {
    const double dm1 = u1 - 2.0 * u2 + u3;
    const double d0 = u2 - 2.0 * u3 + u4;
    const double d1 = u3 - 2.0 * u4 + u5;
    const double dhm1 = minmod4(4.0 * dm1 - d0, 4.0 * d0 - dm1, dm1, d0);
    const double dh0 = minmod4(4.0 * d0 - d1, 4.0 * d1 - d0, d0, d1);
    const double uUL = u3 + 4.0 * (u3 - u2);
    const double uAV = 0.5 * (u3 + u4);
    const double uMD = uAV - 0.5 * dh0;
    const double uLC = u3 + 0.5 * (u3 - u2) + 1.333333333333333 * dhm1;
    const double uMIN = std::max(std::min(std::min(u3, u4), uMD), std::min(std::min(u3, uUL), uLC));
    const double uMAX = std::min(std::max(std::max(u3, u4), uMD), std::max(std::max(u3, uUL), uLC));
    return ulinear + minmod2(uMIN - ulinear, uMAX - ulinear);
  }
  return ulinear;
}

// mplimiter, src/flux.F90:363-379
inline double mplimiter(const double* f, double fl, bool shock, int inode, int dim, int ntype) {
  if ((ntype == 1 && inode == 0) || (ntype == 2 && inode == dim - 1) || (ntype == 1 && inode == 1) ||
      (ntype == 2 && inode == dim - 2))
    return fl;
  return mp5(f, fl, shock);
}

// iwind6, src/solver.F90:1236-1257
inline int iwind6(int i, int n, int imin, int imax, int dir) {
  int w = dir > 0 ? i + n - 3 : i + 4 - n;
  if (w < imin) w = imin;
  if (w > imax) w = imax;
  return w;
}

// node range of the flux split (iss..iee), src/solver.F90:1318-1332
inline void split_range(int npdc, int dim, int& a, int& b) {
  if (npdc == 1) { a = 0; b = dim + HM; }
  else if (npdc == 2) { a = -HM; b = dim; }
  else if (npdc == 3) { a = -HM; b = dim + HM; }
  else { a = 0; b = dim; }
}

}  // namespace

// ---------------------------------------------------------------------------
// Public API
// ---------------------------------------------------------------------------
extern "C" {

orc_ctx* orc_create(const orc_config* cfg) {
  orc_ctx* c = new orc_ctx();
  c->cfg = *cfg;
  c->im = cfg->im; c->jm = cfg->jm; c->km = cfg->km;
  c->ndims = (cfg->ka > 0) ? 3 : 2;
  c->NI = c->im + 2 * HM + 1; c->NJ = c->jm + 2 * HM + 1; c->NK = c->km + 2 * HM + 1;
  c->nh = c->NI * c->NJ * c->NK;
  c->n0 = (long)(c->im + 1) * (c->jm + 1) * (c->km + 1);
  // is..ke: periodic -> 0..dim (src/parallel.F90:1042-1046); a direction
  // with a physical boundary at both ends on one rank is not assigned there;
  // the wall-rank convention of the multi-rank branches (1080-1089) is used.
  c->is = 0; c->ie = c->im; c->js = 0; c->je = c->jm; c->ks = 0; c->ke = c->km;
  if (cfg->npdci == 4) { c->is = 1; c->ie = c->im - 1; }
  if (cfg->npdcj == 4) { c->js = 1; c->je = c->jm - 1; }
  if (cfg->npdck == 4) { c->ks = 1; c->ke = c->km - 1; }
  // refcal, src/solver.F90:102-128 (nondimensional)
  const double gamma = 1.4, mach = cfg->mach, pr = cfg->prandtl, re = cfg->reynolds;
  c->const1 = 1.0 / (gamma * (gamma - 1.0) * (mach * mach));
  c->const2 = gamma * (mach * mach);
  c->const3 = (gamma - 1.0) / 3.0 * pr * (mach * mach);
  c->const4 = (gamma - 1.0) * (mach * mach) * re * pr;
  c->const5 = (gamma - 1.0) * (mach * mach);
  c->const6 = 1.0 / (gamma - 1.0);
  c->const7 = (gamma - 1.0) * (mach * mach) * re * pr;
  c->roinf = 1.0; c->uinf = 1.0; c->tinf = 1.0;
  c->pinf = c->roinf * c->tinf / c->const2;
  c->tempconst = cfg->suth_const / cfg->ref_tem;
  c->tempconst1 = 1.0 + c->tempconst;
  c->dxm = 2.0 * PI / (double)c->im;
  c->dym = 2.0 * PI / (double)c->jm;
  c->dzm = (c->km > 0) ? 2.0 * PI / (double)c->km : 1.0;
  // solvrinit, src/comsolver.F90:47-146
  fd_scheme_initiate(c->fd[0], cfg->npdci, c->im);
  fd_scheme_initiate(c->fd[1], cfg->npdcj, c->jm);
  fd_scheme_initiate(c->fd[2], cfg->npdck, c->km);
  filter_coefficient_cal(c->ft, cfg->alfa_filter, cfg->beter_halo, cfg->beter_bound);
  compact_filter_initiate(c->flt[0], cfg->npdci, c->im, cfg->alfa_filter);
  compact_filter_initiate(c->flt[1], cfg->npdcj, c->jm, cfg->alfa_filter);
  compact_filter_initiate(c->flt[2], cfg->npdck, c->km, cfg->alfa_filter);
  if (cfg->conschm_mp) {
    const int np[3] = {cfg->npdci, cfg->npdcj, cfg->npdck};
    const int dm[3] = {c->im, c->jm, c->km};
    for (int d = 0; d < 3; ++d) {
      compact_flux_initiate(c->fuw[d], np[d], dm[d], +1, cfg->bfacmpld);
      compact_flux_initiate(c->fdw[d], np[d], dm[d], -1, cfg->bfacmpld);
    }
  }
  // commarray allocation (src/commarray.F90:56-108)
  c->q.assign(5 * c->nh, 0.0);
  c->rho.assign(c->nh, 0.0); c->prs.assign(c->nh, 0.0); c->tmp.assign(c->nh, 0.0);
  c->vel.assign(3 * c->nh, 0.0);
  c->x.assign(3 * c->nh, 0.0);
  c->dxi.assign(9 * c->nh, 0.0);
  c->jacob.assign(c->nh, 1.0);
  c->sigma.assign(6 * c->nh, 0.0);
  c->qflux.assign(3 * c->nh, 0.0);
  c->qrhs.assign(5 * c->n0, 0.0);
  c->qsave.assign(5 * c->n0, 0.0);
  c->dvel.assign(9 * c->n0, 0.0);
  c->dtmp.assign(3 * c->n0, 0.0);
  // the sensor's work array: halos of directions without a periodic copy
  // are never written by the reference (it reads them as allocated); here
  // they hold zero
  c->ssf.assign(c->nh, 0.0);
  c->lshock.assign(c->n0, 0);
  const size_t nf = (size_t)(c->jm + 1) * (c->km + 1);
  c->vel_in.assign(3 * nf, 0.0);
  for (size_t t = 0; t < nf; ++t) c->vel_in[t] = c->uinf;  // (uinf, vinf = 0, winf = 0)
  c->tmp_in.assign(nf, c->tinf);
  c->tmp_prof.assign((size_t)c->jm + 1, c->tinf);
  c->prs_in.assign(nf, c->roinf * c->tinf / c->const2);  // thermal(density, temperature)
  return c;
}

void orc_destroy(orc_ctx* c) { delete c; }

double* orc_field(orc_ctx* c, const char* name) {
  std::string s(name);
  if (s == "q") return c->q.data();
  if (s == "rho") return c->rho.data();
  if (s == "vel") return c->vel.data();
  if (s == "prs") return c->prs.data();
  if (s == "tmp") return c->tmp.data();
  if (s == "x") return c->x.data();
  if (s == "vel_in") return c->vel_in.data();
  if (s == "tmp_in") return c->tmp_in.data();
  if (s == "tmp_prof") return c->tmp_prof.data();
  if (s == "prs_in") return c->prs_in.data();
  if (s == "dxi") return c->dxi.data();
  if (s == "jacob") return c->jacob.data();
  if (s == "sigma") return c->sigma.data();
  if (s == "qflux") return c->qflux.data();
  if (s == "ssf") return c->ssf.data();
  if (s == "qrhs") return c->qrhs.data();
  if (s == "qsave") return c->qsave.data();
  if (s == "dvel") return c->dvel.data();
  if (s == "dtmp") return c->dtmp.data();
  return nullptr;
}

int orc_scheme(orc_ctx* c, int dir, int kind, int* first, double* out, int cap) {
  const Scheme& s = kind == 0 ? c->fd[dir] : c->flt[dir];
  int n = s.n();
  *first = s.first;
  if (cap < 5 * n) return -n;
  for (int i = 0; i < n; ++i) {
    out[i] = s.a[i]; out[n + i] = s.c[i];
    out[2 * n + i] = s.ac1[i]; out[3 * n + i] = s.ac2[i]; out[4 * n + i] = s.ac3[i];
  }
  return n;
}

void orc_filter_tables(orc_ctx* c, double* c10, double* c8, double* c6, double* cb, double* ch) {
  for (int i = 0; i < 6; ++i) c10[i] = c->ft.c10i[i];
  for (int i = 0; i < 5; ++i) c8[i] = c->ft.c8i[i];
  for (int i = 0; i < 4; ++i) c6[i] = c->ft.c6i[i];
  for (int j = 0; j < 9; ++j)
    for (int r = 0; r < 5; ++r) cb[r + 5 * j] = c->ft.cb[r][j];
  for (int j = 0; j < 11; ++j)
    for (int r = 0; r < 5; ++r) ch[r + 5 * j] = c->ft.ch[r][j];
}

void orc_constants(orc_ctx* c, double* o) {
  o[0] = c->const1; o[1] = c->const2; o[2] = c->const3; o[3] = c->const4;
  o[4] = c->const5; o[5] = c->const6; o[6] = c->const7; o[7] = c->tempconst;
  o[8] = c->tempconst1;
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_threads(void) { return nthreads_env(); }

// gridcube, src/gridgeneration.F90:233-267 (single rank: ig0=jg0=kg0=0)
void orc_gridcube(orc_ctx* c, double lx, double ly, double lz) {
  const orc_config& g = c->cfg;
  for (int k = 0; k <= c->km; ++k)
    for (int j = 0; j <= c->jm; ++j)
      for (int i = 0; i <= c->im; ++i) {
        long p = c->h(i, j, k);
        c->x[p] = lx / (double)g.ia * (double)i;
        c->x[p + c->nh] = (g.ja == 0) ? ly : ly / (double)g.ja * (double)j;
        c->x[p + 2 * c->nh] = (g.ka == 0) ? 0.0 : lz / (double)g.ka * (double)k;
      }
}

// gridsendrecv single-rank branches, src/parallel.F90:2861-2866, 2930-2960,
// 3010-3030
static void gridsendrecv(orc_ctx* c) {
  const int im = c->im, jm = c->jm, km = c->km;
  const long nh = c->nh;
  double* x = c->x.data();
  if (c->cfg.ia > 0) {
    for (int m = 0; m < 3; ++m)
      for (int k = 0; k <= km; ++k)
        for (int j = 0; j <= jm; ++j)
          for (int n = 1; n <= HM; ++n) {
            double* v = x + m * nh;
            v[c->h(im + n, j, k)] = v[c->h(im, j, k)] + (v[c->h(n, j, k)] - v[c->h(0, j, k)]);
            v[c->h(-n, j, k)] = v[c->h(0, j, k)] - (v[c->h(im, j, k)] - v[c->h(im - n, j, k)]);
          }
  }
  if (c->cfg.ja == 0) {
    for (int k = 0; k <= km; ++k)
      for (int j = -HM; j <= HM; ++j)
        for (int i = 0; i <= im; ++i) {
          x[c->h(i, j, k)] = x[c->h(i, 0, k)];
          x[c->h(i, j, k) + nh] = x[c->h(i, 0, k) + nh] + (double)j;
          x[c->h(i, j, k) + 2 * nh] = x[c->h(i, 0, k) + 2 * nh];
        }
  } else {
    for (int m = 0; m < 3; ++m)
      for (int k = 0; k <= km; ++k)
        for (int n = 1; n <= HM; ++n)
          for (int i = 0; i <= im; ++i) {
            double* v = x + m * nh;
            v[c->h(i, jm + n, k)] = v[c->h(i, jm, k)] + (v[c->h(i, n, k)] - v[c->h(i, 0, k)]);
            v[c->h(i, -n, k)] = v[c->h(i, 0, k)] - (v[c->h(i, jm, k)] - v[c->h(i, jm - n, k)]);
          }
  }
  if (c->cfg.ka == 0) {
    for (int k = -HM; k <= HM; ++k)
      for (int j = 0; j <= jm; ++j)
        for (int i = 0; i <= im; ++i) {
          x[c->h(i, j, k)] = x[c->h(i, j, 0)];
          x[c->h(i, j, k) + nh] = x[c->h(i, j, 0) + nh];
          x[c->h(i, j, k) + 2 * nh] = x[c->h(i, j, 0) + 2 * nh] + (double)k;
        }
  } else {
    for (int m = 0; m < 3; ++m)
      for (int n = 1; n <= HM; ++n)
        for (int j = 0; j <= jm; ++j)
          for (int i = 0; i <= im; ++i) {
            double* v = x + m * nh;
            v[c->h(i, j, km + n)] = v[c->h(i, j, km)] + (v[c->h(i, j, n)] - v[c->h(i, j, 0)]);
            v[c->h(i, j, -n)] = v[c->h(i, j, 0)] - (v[c->h(i, j, km)] - v[c->h(i, j, km - n)]);
          }
  }
}

// derivative of a halo-array line (direction d, transverse a,b) via the
// context's compact scheme; out receives 0..dim.
static void line_deriv(orc_ctx* c, int d, const double* var, int a, int b, LineBuf& lb, double* out) {
  const int dim = c->dimof(d);
  const long st = c->hstride(d);
  const long p0 = hpos(*c, d, 0, a, b);
  double* f = lb.f();
  for (int l = -HM; l <= dim + HM; ++l) f[l] = var[p0 + st * l];
  df_compact(c->fd[d], f, out, lb.d.data(), lb.xx.data());
}

// gridgeom, src/geom.F90:99-930 (the parts that produce dxi and jacob)
void orc_gridgeom(orc_ctx* c) {
  const int im = c->im, jm = c->jm, km = c->km;
  const long nh = c->nh;
  gridsendrecv(c);
  std::vector<double> dx(9 * nh, 0.0);  // dx(:,:,:,m,d) -> comp m + 3*d
  auto DX = [&](int m, int d) { return dx.data() + (long)(m + 3 * d) * nh; };
  const double* x = c->x.data();
  for (int d = 0; d < 3; ++d) {
    int a1, b1;
    trans_range(*c, d, a1, b1);
    const int dim = c->dimof(d);
    const long st = c->hstride(d);
    for_lines(*c, d, 0, a1, 0, b1, [&](int a, int b) {
      thread_local LineBuf* lb = nullptr;
      thread_local std::vector<double>* ob = nullptr;
      if (a < 0) {
        delete lb; delete ob;
        lb = new LineBuf(std::max(im, std::max(jm, km)));
        ob = new std::vector<double>(std::max(im, std::max(jm, km)) + 1);
        return;
      }
      for (int m = 0; m < 3; ++m) {
        line_deriv(c, d, x + m * nh, a, b, *lb, ob->data());
        long p0 = hpos(*c, d, 0, a, b);
        for (int l = 0; l <= dim; ++l) DX(m, d)[p0 + st * l] = (*ob)[l];
      }
    });
  }
  for (int n = 0; n < 9; ++n) dataswap(*c, dx.data() + n * nh, 1, 0);
  // Jacobian, src/geom.F90:350-385
  double* J = c->jacob.data();
  for (int k = 0; k <= km; ++k)
    for (int j = 0; j <= jm; ++j)
      for (int i = 0; i <= im; ++i) {
        long p = c->h(i, j, k);
        auto X = [&](int m, int d) { return DX(m - 1, d - 1)[p]; };
        if (c->ndims == 3)
          J[p] = X(1, 1) * X(2, 2) * X(3, 3) + X(1, 2) * X(2, 3) * X(3, 1) +
                 X(1, 3) * X(2, 1) * X(3, 2) - X(1, 3) * X(2, 2) * X(3, 1) -
                 X(1, 2) * X(2, 1) * X(3, 3) - X(1, 1) * X(2, 3) * X(3, 2);
        else
          J[p] = X(1, 1) * X(2, 2) - X(1, 2) * X(2, 1);
      }
  dataswap(*c, J, 1, 0);
  // dxi, src/geom.F90:395-664 ; dxi(:,:,:,d,m) -> comp d + 3*m
  std::fill(c->dxi.begin(), c->dxi.end(), 0.0);
  auto DXI = [&](int d, int m) { return c->dxi.data() + (long)((d - 1) + 3 * (m - 1)) * nh; };
  auto DXh = [&](int m, int d) { return DX(m - 1, d - 1); };
  auto Xc = [&](int m) { return x + (long)(m - 1) * nh; };
  if (c->ndims == 3) {
    struct Term { int dd, mm; int am, ad, bm; int cm, cd, dm; };
    // phi = 0.5*(dx(am,ad)*x(bm) - dx(cm,cd)*x(dm)), added to dxi(dd,mm)
    const Term tx[6] = {{2, 1, 2, 3, 3, 3, 3, 2}, {2, 2, 3, 3, 1, 1, 3, 3}, {2, 3, 1, 3, 2, 2, 3, 1},
                        {3, 1, 3, 2, 2, 2, 2, 3}, {3, 2, 1, 2, 3, 3, 2, 1}, {3, 3, 2, 2, 1, 1, 2, 2}};
    const Term ty[6] = {{1, 1, 3, 3, 2, 2, 3, 3}, {1, 2, 1, 3, 3, 3, 3, 1}, {1, 3, 2, 3, 1, 1, 3, 2},
                        {3, 1, 2, 1, 3, 3, 1, 2}, {3, 2, 3, 1, 1, 1, 1, 3}, {3, 3, 1, 1, 2, 2, 1, 1}};
    const Term tz[6] = {{1, 1, 2, 2, 3, 3, 2, 2}, {1, 2, 3, 2, 1, 1, 2, 3}, {1, 3, 1, 2, 2, 2, 2, 1},
                        {2, 1, 3, 1, 2, 2, 1, 3}, {2, 2, 1, 1, 3, 3, 1, 1}, {2, 3, 2, 1, 1, 1, 1, 2}};
    const Term* tabs[3] = {tx, ty, tz};
    for (int d = 0; d < 3; ++d) {
      int a1, b1;
      trans_range(*c, d, a1, b1);
      const int dim = c->dimof(d);
      const long st = c->hstride(d);
      for_lines(*c, d, 0, a1, 0, b1, [&](int a, int b) {
        thread_local LineBuf* lb = nullptr;
        thread_local std::vector<double>* ob = nullptr;
        if (a < 0) {
          delete lb; delete ob;
          lb = new LineBuf(std::max(im, std::max(jm, km)));
          ob = new std::vector<double>(std::max(im, std::max(jm, km)) + 1);
          return;
        }
        long p0 = hpos(*c, d, 0, a, b);
        double* f = lb->f();
        for (int t = 0; t < 6; ++t) {
          const Term& T = tabs[d][t];
          for (int l = -HM; l <= dim + HM; ++l) {
            long p = p0 + st * l;
            f[l] = 0.5 * (DXh(T.am, T.ad)[p] * Xc(T.bm)[p] - DXh(T.cm, T.cd)[p] * Xc(T.dm)[p]);
          }
          df_compact(c->fd[d], f, ob->data(), lb->d.data(), lb->xx.data());
          double* o = DXI(T.dd, T.mm);
          for (int l = 0; l <= dim; ++l) o[p0 + st * l] = o[p0 + st * l] + (*ob)[l];
        }
      });
    }
  } else {
    for (int k = 0; k <= km; ++k)
      for (int j = 0; j <= jm; ++j)
        for (int i = 0; i <= im; ++i) {
          long p = c->h(i, j, k);
          DXI(1, 1)[p] = DXh(2, 2)[p];
          DXI(1, 2)[p] = -DXh(1, 2)[p];
          DXI(2, 1)[p] = -DXh(2, 1)[p];
          DXI(2, 2)[p] = DXh(1, 1)[p];
        }
  }
  for (int n = 0; n < 9; ++n) dataswap(*c, c->dxi.data() + n * nh, 1, 0);
  for (int m = 1; m <= 3; ++m)
    for (int d = 1; d <= 3; ++d)
      for (int k = 0; k <= km; ++k)
        for (int j = 0; j <= jm; ++j)
          for (int i = 0; i <= im; ++i) {
            long p = c->h(i, j, k);
            DXI(d, m)[p] = DXI(d, m)[p] / J[p];
          }
  for (int n = 0; n < 9; ++n) dataswap(*c, c->dxi.data() + n * nh, 1, 0);
}

// tgvini + updateq (src/initialisation.F90:621-691 ; src/fludyna.F90:254-300)
// or mini-app flowfield_init (miniapps/tgv_solver_3d/tgvsolver.F90:172-234).
void orc_init_tgv(orc_ctx* c) {
  const long nh = c->nh;
  if (c->cfg.mode == ORC_MODE_MINIAPP) {
    const double pinf = 1.0 / c->const2;
    for (int k = 0; k <= c->km; ++k)
      for (int j = 0; j <= c->jm; ++j)
        for (int i = 0; i <= c->im; ++i) {
          long p = c->h(i, j, k);
          double x1 = 2.0 * PI / (double)c->im * (double)i;
          double x2 = 2.0 * PI / (double)c->jm * (double)j;
          double x3 = 2.0 * PI / (double)c->km * (double)k;
          c->rho[p] = 1.0;
          c->vel[p] = std::sin(x1) * std::cos(x2) * std::cos(x3);
          c->vel[p + nh] = -std::cos(x1) * std::sin(x2) * std::cos(x3);
          c->vel[p + 2 * nh] = 0.0;
          c->prs[p] = pinf + 1.0 / 16.0 * (std::cos(2.0 * x1) + std::cos(2.0 * x2)) *
                                 (std::cos(2.0 * x3) + 2.0);
          c->tmp[p] = c->prs[p] / c->rho[p] * c->const2;
          fvar2q_prs_node(*c, p);
        }
    return;
  }
  const double l0 = 1.0;
  const double* x = c->x.data();
  for (int k = 0; k <= c->km; ++k)
    for (int j = 0; j <= c->jm; ++j)
      for (int i = 0; i <= c->im; ++i) {
        long p = c->h(i, j, k);
        double X = x[p], Y = x[p + nh], Z = x[p + 2 * nh];
        c->rho[p] = c->roinf;
        c->vel[p] = c->uinf * std::sin(X / l0) * std::cos(Y / l0) * std::cos(Z / l0);
        c->vel[p + nh] = -(c->uinf * std::cos(X / l0) * std::sin(Y / l0) * std::cos(Z / l0));
        c->vel[p + 2 * nh] = 0.0;
        c->prs[p] = c->pinf + c->rho[p] / 16.0 * (c->uinf * c->uinf) *
                                  (std::cos(2.0 * X / l0) + std::cos(2.0 * Y / l0)) *
                                  (std::cos(2.0 * Z / l0) + 2.0);
        c->tmp[p] = c->prs[p] / c->rho[p] * c->const2;
      }
  orc_updateq(c);
}

// updateq -> fvar2q_3da with temperature (src/fludyna.F90:254-300, 480-533)
void orc_updateq(orc_ctx* c) {
  const long nh = c->nh;
  for (int k = 0; k <= c->km; ++k)
    for (int j = 0; j <= c->jm; ++j)
      for (int i = 0; i <= c->im; ++i) {
        long p = c->h(i, j, k);
        double ro = c->rho[p], u = c->vel[p], v = c->vel[p + nh], w = c->vel[p + 2 * nh];
        c->q[p] = ro;
        c->q[p + nh] = ro * u;
        c->q[p + 2 * nh] = ro * v;
        c->q[p + 3 * nh] = ro * w;
        c->q[p + 4 * nh] = ro * (c->tmp[p] * c->const1 + 0.5 * (u * u + v * v + w * w));
      }
}

// ---------------------------------------------------------------------------
// Hot path
// ---------------------------------------------------------------------------

// filterq, src/comsolver.F90:514-632 (mini-app: tgvsolver.F90:791-883).
void orc_filterq(orc_ctx* c) {
  const long nh = c->nh;
  for (int d = 0; d < c->ndims; ++d) {
    dataswap(*c, c->q.data(), 5, d + 1);
    int a1, b1;
    trans_range(*c, d, a1, b1);
    const int dim = c->dimof(d);
    const long st = c->hstride(d);
    const int mx = std::max(c->im, std::max(c->jm, c->km));
    for_lines(*c, d, 0, a1, 0, b1, [&](int a, int b) {
      thread_local LineBuf* lb = nullptr;
      if (a < 0) { delete lb; lb = new LineBuf(mx); return; }
      long p0 = hpos(*c, d, 0, a, b);
      double* f = lb->f();
      std::vector<double>& out = lb->ob;
      // filter all variables of the line first, then write back
      // (q(0:dim,..,:) = fph), as the reference does
      thread_local std::vector<double> res;
      res.resize(5 * (dim + 1));
      for (int n = 0; n < 5; ++n) {
        const double* v = c->q.data() + n * nh;
        for (int l = -HM; l <= dim + HM; ++l) f[l] = v[p0 + st * l];
        compact_filter(c->flt[d], c->ft, f, out.data(), lb->d.data(), lb->xx.data());
        for (int l = 0; l <= dim; ++l) res[n * (dim + 1) + l] = out[l];
      }
      for (int n = 0; n < 5; ++n) {
        double* v = c->q.data() + n * nh;
        for (int l = 0; l <= dim; ++l) v[p0 + st * l] = res[n * (dim + 1) + l];
      }
    });
  }
}

// qswap single-rank periodic branches, src/parallel.F90:4876-4920,
// 5018-5065, 5159-5206.  Non-periodic directions on one rank exchange
// nothing (MPI_PROC_NULL neighbours).
void orc_qswap(orc_ctx* c) {
  const int im = c->im, jm = c->jm, km = c->km;
  const long nh = c->nh;
  double* q = c->q.data();
  if (c->homo(0)) {
    for (int n = 0; n < 5; ++n)
      for (int k = 0; k <= km; ++k)
        for (int j = 0; j <= jm; ++j) {
          double* v = q + n * nh;
          for (int i = -HM; i <= -1; ++i) v[c->h(i, j, k)] = v[c->h(im + i, j, k)];
          for (int i = im + 1; i <= im + HM; ++i) v[c->h(i, j, k)] = v[c->h(i - im, j, k)];
          v[c->h(0, j, k)] = 0.5 * (v[c->h(0, j, k)] + v[c->h(im, j, k)]);
          v[c->h(im, j, k)] = v[c->h(0, j, k)];
        }
    q2fvar_box(*c, im, im + HM, 0, jm, 0, km);
    q2fvar_box(*c, -HM, 0, 0, jm, 0, km);
  }
  if (c->homo(1)) {
    for (int n = 0; n < 5; ++n)
      for (int k = 0; k <= km; ++k) {
        double* v = q + n * nh;
        if (jm == 0) {
          for (int j = -HM; j <= HM; ++j)
            for (int i = 0; i <= im; ++i) v[c->h(i, j, k)] = v[c->h(i, 0, k)];
        } else {
          for (int j = -HM; j <= -1; ++j)
            for (int i = 0; i <= im; ++i) v[c->h(i, j, k)] = v[c->h(i, jm + j, k)];
          for (int j = jm + 1; j <= jm + HM; ++j)
            for (int i = 0; i <= im; ++i) v[c->h(i, j, k)] = v[c->h(i, j - jm, k)];
          for (int i = 0; i <= im; ++i) {
            v[c->h(i, 0, k)] = 0.5 * (v[c->h(i, 0, k)] + v[c->h(i, jm, k)]);
            v[c->h(i, jm, k)] = v[c->h(i, 0, k)];
          }
        }
      }
    q2fvar_box(*c, 0, im, -HM, 0, 0, km);
    q2fvar_box(*c, 0, im, jm, jm + HM, 0, km);
  }
  if (c->homo(2)) {
    for (int n = 0; n < 5; ++n) {
      double* v = q + n * nh;
      if (c->cfg.ka == 0) {
        for (int k = -HM; k <= HM; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) v[c->h(i, j, k)] = v[c->h(i, j, 0)];
      } else {
        for (int k = -HM; k <= -1; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) v[c->h(i, j, k)] = v[c->h(i, j, km + k)];
        for (int k = km + 1; k <= km + HM; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) v[c->h(i, j, k)] = v[c->h(i, j, k - km)];
        for (int j = 0; j <= jm; ++j)
          for (int i = 0; i <= im; ++i) {
            v[c->h(i, j, 0)] = 0.5 * (v[c->h(i, j, 0)] + v[c->h(i, j, km)]);
            v[c->h(i, j, km)] = v[c->h(i, j, 0)];
          }
      }
    }
    q2fvar_box(*c, 0, im, 0, jm, -HM, 0);
    q2fvar_box(*c, 0, im, 0, jm, km, km + HM);
  }
}

// Boundary routines of boucon (src/bc.F90:327-409), single rank, no
// species, nondimensional.  Face n (0-based: xmin, xmax, ymin, ymax, zmin,
// zmax), applied in face order (faces share their edge nodes; the later
// face's values stay).  Each restates the face branch of its routine as the
// reference writes it, including where the faces differ.
namespace {

// extrapolate(v1, v2, dv=0): extrapolate_2o, src/commfunc.F90:277-285
inline double ex2(double v1, double v2) { return NUM1D3 * (4.0 * v1 - v2 - 2.0 * 0.0); }

// fvar2q_sca with temperature (src/fludyna.F90:312-370)
inline void fvar2q_tmp_node(orc_ctx& c, long p) {
  const long nh = c.nh;
  double ro = c.rho[p], u = c.vel[p], v = c.vel[p + nh], w = c.vel[p + 2 * nh];
  c.q[p] = ro;
  c.q[p + nh] = ro * u;
  c.q[p + 2 * nh] = ro * v;
  c.q[p + 3 * nh] = ro * w;
  double var1 = 0.5 * (u * u + v * v + w * w);
  c.q[p + 4 * nh] = ro * (c.tmp[p] * c.const1 + var1);
}

int face_bctype(const orc_ctx& c, int n) {
  int t = c.cfg.bctype[n];
  if (c.cfg.channel && (n == 2 || n == 3) && (t == 0 || t == 1)) t = 41;
  return t;
}

double face_twall(const orc_ctx& c, int n) {
  return c.cfg.twall6[n] != 0.0 ? c.cfg.twall6[n] : c.cfg.twall;
}

// unit vector along the metric row d at node p (gridgeom's bnorm,
// src/geom.F90:700-830; its sign does not enter the symmetry condition)
inline void bnorm(const orc_ctx& c, int d, long p, double* nv) {
  const double* X = c.dxi.data() + p;
  const long nh = c.nh;
  double a = X[(d + 0) * nh], b = X[(d + 3) * nh], e = X[(d + 6) * nh];
  double var1 = std::sqrt(a * a + b * b + e * e);
  nv[0] = a / var1; nv[1] = b / var1; nv[2] = e / var1;
}

// Extent of the grid along direction d (xmax - xmin, ymax - ymin, ...:
// gridgeom's maxval / minval over the interior nodes, src/geom.F90:684-696).
double grid_extent(const orc_ctx& c, int d) {
  double lo = 1e300, hi = -1e300;
  for (int k = 0; k <= c.km; ++k)
    for (int j = 0; j <= c.jm; ++j)
      for (int i = 0; i <= c.im; ++i) {
        const double v = c.x[c.h(i, j, k) + d * c.nh];
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
  return hi - lo;
}

void face_node(orc_ctx& c, int n, int type, double tw, int i, int j, int k, double extent) {
  const int d = n / 2, side = n % 2;
  const int dim = c.dimof(d);
  const long nh = c.nh;
  auto at = [&](int l) {
    int ii = i, jj = j, kk = k;
    const int node = side ? dim - l : l;
    if (d == 0) ii = node; else if (d == 1) jj = node; else kk = node;
    return c.h(ii, jj, kk);
  };
  const long p = at(0), p1 = at(1), p2 = at(2);
  double* R = c.rho.data(); double* P = c.prs.data(); double* T = c.tmp.data();
  double* V = c.vel.data();
  if (type == 41) {  // noslip, src/bc.F90:6306-6712 (all faces)
    const double pe = NUM1D3 * (4.0 * P[p1] - P[p2]);
    V[p] = 0.0; V[p + nh] = 0.0; V[p + 2 * nh] = 0.0;
    P[p] = pe;
    T[p] = tw;
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_prs_node(c, p);
  } else if (type == 42) {  // noslip_adibatic, src/bc.F90:6728-7036 (x, y faces)
    const double pe = NUM1D3 * (4.0 * P[p1] - P[p2]);
    const double te = NUM1D3 * (4.0 * T[p1] - T[p2]);
    V[p] = 0.0; V[p + nh] = 0.0; V[p + 2 * nh] = 0.0;
    P[p] = pe;
    T[p] = te;
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_prs_node(c, p);
  } else if (type == 411) {  // slipisotwall, src/bc.F90:7038-7229 (y faces)
    // ymin: slip (u and T extrapolated, v = 0) up to x = xslip, isothermal
    // no-slip beyond (the wall-blowing velocity is 0 without its input
    // file); ymax: isothermal no-slip
    const double pe = NUM1D3 * (4.0 * P[p1] - P[p2]);
    if (n == 2 && c.x[p] <= c.cfg.xslip) {
      const double ue = NUM1D3 * (4.0 * V[p1] - V[p2]);
      const double te = NUM1D3 * (4.0 * T[p1] - T[p2]);
      V[p] = ue; V[p + nh] = 0.0;
      T[p] = te;
    } else {
      V[p] = 0.0; V[p + nh] = 0.0;
      T[p] = tw;
    }
    V[p + 2 * nh] = 0.0;
    P[p] = pe;
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_prs_node(c, p);
  } else if (type == 421) {  // slipadibwall, src/bc.F90:7231-7430 (y faces)
    const double pe = NUM1D3 * (4.0 * P[p1] - P[p2]);
    const double te = NUM1D3 * (4.0 * T[p1] - T[p2]);
    const double ue = NUM1D3 * (4.0 * V[p1] - V[p2]);
    // ymin: v = 0; ymax: v extrapolated too (as the reference writes it)
    const double ve = n == 3 ? NUM1D3 * (4.0 * V[p1 + nh] - V[p2 + nh]) : 0.0;
    V[p] = ue; V[p + nh] = ve; V[p + 2 * nh] = 0.0;
    T[p] = te;
    P[p] = pe;
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_prs_node(c, p);
  } else if (type == 21 && n == 1) {  // outflow xmax, src/bc.F90:3427-3532
    // the first-order copy of the i-1 node (the supersonic branch is taken
    // unconditionally); rho from p and T, q in temperature form
    V[p] = V[p1]; V[p + nh] = V[p1 + nh]; V[p + 2 * nh] = V[p1 + 2 * nh];
    P[p] = P[p1];
    T[p] = T[p1];
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_tmp_node(c, p);
  } else if (type == 21) {  // outflow ymax, src/bc.F90:3534-3615
    const double css = std::sqrt(T[p]) / c.cfg.mach;  // sos of the face node
    const double ub = V[p + nh];
    const double ue = ex2(V[p1], V[p2]), ve = ex2(V[p1 + nh], V[p2 + nh]);
    const double we = ex2(V[p1 + 2 * nh], V[p2 + 2 * nh]);
    const double pe = ex2(P[p1], P[p2]), te = ex2(T[p1], T[p2]), roe = ex2(R[p1], R[p2]);
    if (ub >= css) {  // supersonic: everything extrapolated
      P[p] = pe;
      R[p] = roe;
    } else {  // subsonic: relaxation of p towards pinf (alpha = 0.25)
      const double adt = 0.25 * c.cfg.deltat;
      P[p] = (P[p] + adt * c.pinf + R[p] * css * (ve - V[p + nh])) / (1.0 + adt);
      T[p] = te;
      R[p] = P[p] / T[p] * c.const2;
    }
    V[p] = ue; V[p + nh] = ve; V[p + 2 * nh] = we;
    T[p] = P[p] / R[p] * c.const2;  // nondimensional: T from p and rho
    fvar2q_prs_node(c, p);
  } else if (type == 51 && n == 3) {  // farfield ymax, src/bc.F90:3106-3233
    // the characteristic treatment there is commented out: all extrapolated,
    // T from p and rho, q in temperature form
    const double ue = ex2(V[p1], V[p2]), ve = ex2(V[p1 + nh], V[p2 + nh]);
    const double we = ex2(V[p1 + 2 * nh], V[p2 + 2 * nh]);
    P[p] = ex2(P[p1], P[p2]);
    R[p] = ex2(R[p1], R[p2]);
    V[p] = ue; V[p + nh] = ve; V[p + 2 * nh] = we;
    T[p] = P[p] / R[p] * c.const2;
    fvar2q_tmp_node(c, p);
  } else if (type == 51) {  // farfield ymin 3024-3104, zmin 3235-3312, zmax 3314-3389
    // inflow where the normal velocity points into the domain (Riemann
    // invariants against the free stream, isentropic rho), else outflow at
    // pinf; the normal component is v on ymin and w on the z faces
    const long m = (d == 1 ? 1 : 2) * nh;  // offset of the normal velocity
    const double css = std::sqrt(T[p]) / c.cfg.mach;
    const double ue = ex2(V[p1], V[p2]), ve = ex2(V[p1 + nh], V[p2 + nh]);
    const double we = ex2(V[p1 + 2 * nh], V[p2 + 2 * nh]);
    const double pe = ex2(P[p1], P[p2]), roe = ex2(R[p1], R[p2]);
    const double csse = ex2(std::sqrt(T[p1]) / c.cfg.mach, std::sqrt(T[p2]) / c.cfg.mach);
    const double vn_e = d == 1 ? ve : we;
    const double vinf = 0.0, winf = 0.0;  // refcal, nondimensional (src/solver.F90:114-118)
    const double vn_inf = d == 1 ? vinf : winf;
    const double sgn = side ? -1.0 : 1.0;  // zmax faces the other way
    const bool inflow = side ? V[p + m] <= 0.0 : V[p + m] >= 0.0;
    if (inflow) {
      const double vn = sgn * 0.5 * (c.pinf - pe) / (R[p] * css) + 0.5 * (vn_inf + vn_e);
      const double pb = 0.5 * (c.pinf + pe) + sgn * 0.5 * R[p] * css * (vn_inf - vn_e);
      V[p] = c.uinf;
      V[p + nh] = d == 1 ? vn : vinf;
      V[p + 2 * nh] = d == 1 ? winf : vn;
      P[p] = pb;
      R[p] = c.roinf * std::pow(P[p] / c.pinf, 1.0 / GAMMA);
    } else {
      P[p] = c.pinf;
      R[p] = roe + (P[p] - pe) / csse / csse;
      const double vn = vn_e - sgn * (pe - P[p]) / roe / csse;
      V[p] = ue;
      V[p + nh] = d == 1 ? vn : ve;
      V[p + 2 * nh] = d == 1 ? we : vn;
    }
    T[p] = P[p] / R[p] * c.const2;
    fvar2q_prs_node(c, p);
  } else if (type == 23) {  // gcnscbc xmax 8041-8148, ymax 8150-8252 (prs_t = pinf)
    // LODI at node dim-1 with one-sided differences, the outgoing wave
    // relaxed towards pinf (ymax: and, where the normal velocity is
    // negative, the incoming waves towards the free stream), projected
    // back and extrapolated over 2 dx.  css, css2 and vnorm are INTEGER in
    // the reference's declarations (src/bc.F90:8035): sos and the velocity
    // are truncated, mavg = vnorm/css is an integer division, and
    // lambda(5:numq) = vnorm leaves lambda(5) = vnorm with numq = 5.
    const long vn_off = d * nh;                       // normal velocity component
    const long t1_off = (d == 0 ? 1 : 0) * nh;        // the other in-plane one
    const int css = (int)(std::sqrt(T[p1]) / c.cfg.mach);
    const int css2 = css * css;
    const int vnorm = (int)V[p1 + vn_off];
    // (css = 0, sos below 1, would divide by zero in the reference; 0 here)
    const double mavg = css != 0 ? (double)(vnorm / css) : 0.0;
    double lambda[5] = {(double)(vnorm - css), (double)vnorm, (double)vnorm, (double)vnorm,
                        (double)vnorm};
    for (int m = 0; m < 5; ++m) lambda[m] = lambda[m] + 1e-10;
    const double* X = c.x.data() + d * nh;
    const double dx = X[p1] - X[p2];
    auto dr = [&](double v0, double v1) { return -(-v0 + v1) / dx; };  // -deriv(v0, v1)/dx
    double dvel[3] = {dr(V[p1], V[p2]), dr(V[p1 + nh], V[p2 + nh]), dr(V[p1 + 2 * nh], V[p2 + 2 * nh])};
    double dprs = dr(P[p1], P[p2]), drho = dr(R[p1], R[p2]), dtmp;
    const int dn = d, dt1 = d == 0 ? 1 : 0;
    double lodi[5];
    lodi[0] = lambda[0] * (dprs - R[p1] * css * dvel[dn]);
    lodi[1] = lambda[1] * (css2 * drho - dprs);
    lodi[2] = lambda[2] * dvel[dt1];
    lodi[3] = lambda[3] * dvel[2];
    lodi[4] = lambda[4] * (dprs + R[p1] * css * dvel[dn]);
    if (d == 0 || vnorm >= 0) {
      const double sigma = 0.25;
      const double kamma = sigma * css * (1.0 - mavg * mavg) / extent;
      lodi[0] = kamma * (P[p1] - c.pinf);
    } else {
      const double eta = 0.25, vinf = 0.0, winf = 0.0;
      lodi[0] = eta * R[p1] * css2 * (1.0 - mavg * mavg) / extent * (V[p1 + vn_off] - vinf);
      lodi[1] = eta * R[p1] * css2 / GAMMA / extent * (T[p1] - c.tinf);
      lodi[2] = eta * css / extent * (V[p1 + t1_off] - c.uinf);
      lodi[3] = eta * css / extent * (V[p1 + 2 * nh] - winf);
    }
    for (int m = 0; m < 5; ++m) lodi[m] = lodi[m] / lambda[m];
    drho = 1.0 / (double)(css * css) * (lodi[1] + 0.5 * (lodi[0] + lodi[4]));
    dtmp = T[p1] / R[p1] / css * (-lodi[1] + 0.5 * (GAMMA - 1.0) * (lodi[0] + lodi[4]));
    dprs = 0.5 * (lodi[0] + lodi[4]);
    dvel[dn] = 1.0 / (2.0 * R[p1] * css) * (lodi[4] - lodi[0]);
    dvel[dt1] = lodi[2];
    dvel[2] = lodi[3];
    T[p] = T[p1] + 2.0 * dx * dtmp;
    R[p] = R[p1] + 2.0 * dx * drho;
    P[p] = P[p1] + 2.0 * dx * dprs;
    for (int m = 0; m < 3; ++m) V[p + m * nh] = V[p1 + m * nh] + 2.0 * dx * dvel[m];
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_prs_node(c, p);
  } else if (type == 11) {  // inflow xmin, src/bc.F90:1366-1562 (its active, subsonic branch)
    // v, w and T from the inflow arrays; p from the incoming characteristic
    // against pinf blended towards pinf by the local inflow Mach number
    // (the speed of sound of the profile temperature); u from p; rho from
    // p and T; q in temperature form.  rho_ref is the first interior node.
    const size_t fj = (size_t)j + (size_t)(c.jm + 1) * (size_t)k;
    const size_t nf = (size_t)(c.jm + 1) * (c.km + 1);
    const double vin1 = c.vel_in[fj], vin2 = c.vel_in[fj + nf], vin3 = c.vel_in[fj + 2 * nf];
    const double rho_ref = R[p1];
    const double css = std::sqrt(c.tmp_prof[j]) / c.cfg.mach;
    V[p + nh] = vin2;
    V[p + 2 * nh] = vin3;
    T[p] = c.tmp_in[fj];
    const double pe = ex2(P[p1], P[p2]);
    const double ue = ex2(V[p1], V[p2]);
    const double pwave_in = c.pinf;
    const double malo = vin1 / css;
    const double blend = 0.5 * (std::tanh((malo - 1.0) * 6.0) + 1.0);
    P[p] = (0.5 * (pwave_in + pe) + 0.5 * rho_ref * css * (vin1 - ue)) * (1.0 - blend) + pwave_in * blend;
    V[p] = vin1 + (c.pinf - P[p]) / rho_ref / css;
    R[p] = P[p] / T[p] * c.const2;
    fvar2q_tmp_node(c, p);
  } else if (type == 50) {  // zeroextrap, src/bc.F90:2356-2652
    const double ue = ex2(V[p1], V[p2]), ve = ex2(V[p1 + nh], V[p2 + nh]);
    const double we = ex2(V[p1 + 2 * nh], V[p2 + 2 * nh]);
    const double pe = ex2(P[p1], P[p2]);
    if (d == 0) {
      const double te = ex2(T[p1], T[p2]);
      P[p] = pe;
      T[p] = te;
      V[p] = ue; V[p + nh] = ve; V[p + 2 * nh] = we;
      R[p] = P[p] / T[p] * c.const2;
      fvar2q_prs_node(c, p);
    } else {
      const double roe = ex2(R[p1], R[p2]);
      P[p] = pe;
      R[p] = roe;
      V[p] = ue; V[p + nh] = ve; V[p + 2 * nh] = we;
      T[p] = P[p] / R[p] * c.const2;
      if (n == 3) fvar2q_tmp_node(c, p);
      else fvar2q_prs_node(c, p);
    }
  } else if (type == 60) {  // symmetry, src/bc.F90:2664-2996
    const double ue = ex2(V[p1], V[p2]), ve = ex2(V[p1 + nh], V[p2 + nh]);
    const double we = ex2(V[p1 + 2 * nh], V[p2 + 2 * nh]);
    const double pe = ex2(P[p1], P[p2]);
    if (n <= 1) {  // x faces: tangential projection, temperature form
      const double te = ex2(T[p1], T[p2]);
      double nv[3];
      bnorm(c, 0, p, nv);
      double vec[3] = {ue, ve, we};
      const double vne = vec[0] * nv[0] + vec[1] * nv[1] + vec[2] * nv[2];
      for (int m = 0; m < 3; ++m) vec[m] = vec[m] - vne * nv[m];
      P[p] = pe;
      T[p] = te;
      V[p] = vec[0]; V[p + nh] = vec[1]; V[p + 2 * nh] = vec[2];
      R[p] = P[p] / T[p] * c.const2;
      fvar2q_tmp_node(c, p);
    } else if (n <= 4) {  // y faces and zmin: the normal component set to 0
      const double te = ex2(T[p1], T[p2]);
      V[p] = ue; V[p + nh] = ve; V[p + 2 * nh] = we;
      V[p + (d == 1 ? 1 : 2) * nh] = 0.0;
      P[p] = pe;
      T[p] = te;
      R[p] = P[p] / T[p] * c.const2;
      if (n == 3) fvar2q_tmp_node(c, p);
      else fvar2q_prs_node(c, p);
    } else {  // zmax: density extrapolated, tangential projection
      const double roe = ex2(R[p1], R[p2]);
      P[p] = pe;
      R[p] = roe;
      double nv[3];
      bnorm(c, 2, p, nv);
      double vec[3] = {ue, ve, we};
      const double vne = vec[0] * nv[0] + vec[1] * nv[1] + vec[2] * nv[2];
      for (int m = 0; m < 3; ++m) vec[m] = vec[m] - vne * nv[m];
      V[p] = vec[0]; V[p + nh] = vec[1]; V[p + 2 * nh] = vec[2];
      T[p] = P[p] / R[p] * c.const2;
      fvar2q_tmp_node(c, p);
    }
  }
}

// pmatrix (src/bc.F90:5516-5611): the characteristic matrix of the face
// whose metric row is ddi (inv false) or its inverse (inv true).
void pmatrix(double rho, double u, double v, double w, double t, const double ddi[3], bool inv,
             double mach, double P[5][5]) {
  const double c = std::sqrt(t) / mach;  // sos, nondimensional
  const double var1 = 1.0 / std::sqrt(ddi[0] * ddi[0] + ddi[1] * ddi[1] + ddi[2] * ddi[2]);
  const double nx = ddi[0] * var1, ny = ddi[1] * var1, nz = ddi[2] * var1;
  const double phi = 0.5 * (GAMMA - 1.0) * (u * u + v * v + w * w);
  const double VV = nx * u + ny * v + nz * w;
  const double a1 = GAMMA - 1.0;
  const double a2 = 1.0 / (std::sqrt(2.0) * rho * c);
  const double a3 = rho / (c * std::sqrt(2.0));
  const double a4 = (phi + c * c) / (GAMMA - 1.0);
  const double a5 = 1.0 - phi / (c * c);
  const double a6 = phi / (GAMMA - 1.0);
  if (inv) {
    const double n3[3] = {nx, ny, nz};
    P[0][0] = nx * a5 - (nz * v - ny * w) / rho;
    P[0][1] = nx * a1 * u / (c * c);
    P[0][2] = nx * a1 * v / (c * c) + nz / rho;
    P[0][3] = nx * a1 * w / (c * c) - ny / rho;
    P[1][0] = ny * a5 - (nx * w - nz * u) / rho;
    P[1][1] = ny * a1 * u / (c * c) - nz / rho;
    P[1][2] = ny * a1 * v / (c * c);
    P[1][3] = ny * a1 * w / (c * c) + nx / rho;
    P[2][0] = nz * a5 - (ny * u - nx * v) / rho;
    P[2][1] = nz * a1 * u / (c * c) + ny / rho;
    P[2][2] = nz * a1 * v / (c * c) - nx / rho;
    P[2][3] = nz * a1 * w / (c * c);
    for (int r = 0; r < 3; ++r) P[r][4] = -(n3[r] * a1 / (c * c));
    P[3][0] = a2 * (phi - c * VV);
    P[3][1] = -(a2 * (a1 * u - nx * c));
    P[3][2] = -(a2 * (a1 * v - ny * c));
    P[3][3] = -(a2 * (a1 * w - nz * c));
    P[3][4] = a1 * a2;
    P[4][0] = a2 * (phi + c * VV);
    P[4][1] = -(a2 * (a1 * u + nx * c));
    P[4][2] = -(a2 * (a1 * v + ny * c));
    P[4][3] = -(a2 * (a1 * w + nz * c));
    P[4][4] = a1 * a2;
  } else {
    P[0][0] = nx; P[0][1] = ny; P[0][2] = nz; P[0][3] = a3; P[0][4] = a3;
    P[1][0] = nx * u; P[1][1] = ny * u - nz * rho; P[1][2] = nz * u + ny * rho;
    P[1][3] = a3 * (u + nx * c); P[1][4] = a3 * (u - nx * c);
    P[2][0] = nx * v + nz * rho; P[2][1] = ny * v; P[2][2] = nz * v - nx * rho;
    P[2][3] = a3 * (v + ny * c); P[2][4] = a3 * (v - ny * c);
    P[3][0] = nx * w - ny * rho; P[3][1] = ny * w + nx * rho; P[3][2] = nz * w;
    P[3][3] = a3 * (w + nz * c); P[3][4] = a3 * (w - nz * c);
    P[4][0] = nx * a6 + rho * (nz * v - ny * w); P[4][1] = ny * a6 + rho * (nx * w - nz * u);
    P[4][2] = nz * a6 + rho * (ny * u - nx * v);
    P[4][3] = a3 * (a4 + c * VV); P[4][4] = a3 * (a4 - c * VV);
  }
}

// The inviscid flux of node p through the metric row d (the Ecs / fcs of
// inflow_nscbc): J (q u_d + dxi(d,:) p) with u_d = dxi(d,:) . u; dxi(d,m)
// is array d + 3 m of the Fortran dxi(..,1:3,1:3).
void row_flux(const orc_ctx& c, long p, int d, double* f) {
  const long nh = c.nh;
  const double* X = c.dxi.data() + p;
  const double x1 = X[(d + 0) * nh], x2 = X[(d + 3) * nh], x3 = X[(d + 6) * nh];
  const double* V = c.vel.data() + p;
  const double uu = x1 * V[0] + x2 * V[nh] + x3 * V[2 * nh];
  const double J = c.jacob[p], pr = c.prs[p];
  const double* Q = c.q.data() + p;
  f[0] = J * Q[0] * uu;
  f[1] = J * (Q[nh] * uu + x1 * pr);
  f[2] = J * (Q[2 * nh] * uu + x2 * pr);
  f[3] = J * (Q[3 * nh] * uu + x3 * pr);
  f[4] = J * (Q[4 * nh] + pr) * uu;
}

// inflow_nscbc (src/bc.F90:2114-2344) on xmin: adds to qrhs at i = 0 the
// characteristic residual (LODI: the incoming waves relaxed towards the
// inflow arrays at rate kin, the outgoing one kept) and the tangential
// flux derivatives of the face (ddfc '222e' with periodic y and z,
// diff2ec ntype 3: 0.5 (f(j+1) - f(j-1)), halo values included).
void inflow_nscbc(orc_ctx& c) {
  const long nh = c.nh, n0 = c.n0;
  const int im = c.im, jm = c.jm, km = c.km;
  const double mach = c.cfg.mach;
  double gm2 = 0.0;
  for (int k = 0; k <= km; ++k)
    for (int j = 0; j <= jm; ++j)
      for (int i = 0; i <= im; ++i) {
        const long p = c.h(i, j, k);
        const double u = c.vel[p], v = c.vel[p + nh], w = c.vel[p + 2 * nh];
        const double var1 = u * u + v * v + w * w;
        const double css = std::sqrt(c.tmp[p]) / mach;
        gm2 = std::max(gm2, var1 / css / css);
      }
  const double extent = grid_extent(c, 0);
  const size_t nf = (size_t)(jm + 1) * (km + 1);
  for (int k = 0; k <= km; ++k)
    for (int j = 0; j <= jm; ++j) {
      const long p = c.h(0, j, k), pa = c.h(1, j, k);
      const size_t fj = (size_t)j + (size_t)(jm + 1) * k;
      const double rho = c.rho[p], u = c.vel[p], v = c.vel[p + nh], w = c.vel[p + 2 * nh];
      const double t = c.tmp[p], pr = c.prs[p], J = c.jacob[p];
      const double* Q = c.q.data() + p;
      const double ddi[3] = {c.dxi[p], c.dxi[p + 3 * nh], c.dxi[p + 6 * nh]};  // dxi(i,j,k,1,:)
      double pnor[5][5], pinv[5][5];
      pmatrix(rho, u, v, w, t, ddi, false, mach, pnor);
      pmatrix(rho, u, v, w, t, ddi, true, mach, pinv);
      double e0[5], e1[5], dE[5];
      row_flux(c, p, 0, e0);
      row_flux(c, pa, 0, e1);
      for (int n = 0; n < 5; ++n) dE[n] = -e0[n] + e1[n];  // deriv(Ecs(0), Ecs(1))
      const double E[5] = {Q[nh], Q[nh] * u + pr, Q[2 * nh] * u, Q[3 * nh] * u, (Q[4 * nh] + pr) * u};
      const double F[5] = {Q[2 * nh], Q[nh] * v, Q[2 * nh] * v + pr, Q[3 * nh] * v, (Q[4 * nh] + pr) * v};
      const double G[5] = {Q[3 * nh], Q[nh] * w, Q[2 * nh] * w, Q[3 * nh] * w + pr, (Q[4 * nh] + pr) * w};
      double jcbi[3];
      for (int m = 0; m < 3; ++m)
        jcbi[m] = -(c.dxi[p + 3 * m * nh] * J) + c.dxi[pa + 3 * m * nh] * c.jacob[pa];
      double rest[5], l1[5], lodi[5];
      for (int n = 0; n < 5; ++n) {
        rest[n] = E[n] * jcbi[0] + F[n] * jcbi[1] + G[n] * jcbi[2];
        l1[n] = dE[n] - rest[n];
      }
      for (int r = 0; r < 5; ++r) {
        double acc = 0.0;
        for (int m = 0; m < 5; ++m) acc = acc + pinv[r][m] * l1[m];
        lodi[r] = acc / J;
      }
      const double css = std::sqrt(t) / mach;
      const double kin = 0.25 * (1.0 - gm2) * css / extent;
      const double var1 = 1.0 / std::sqrt(ddi[0] * ddi[0] + ddi[1] * ddi[1] + ddi[2] * ddi[2]);
      const size_t nfv = nf;
      const double ui = c.vel_in[fj], vi = c.vel_in[fj + nfv], wi = c.vel_in[fj + 2 * nfv];
      lodi[0] = 0.0;
      lodi[1] = kin * 0.5 * (ddi[0] * var1 * (w - wi) - ddi[2] * var1 * (u - ui));
      lodi[2] = kin * 0.5 * (-(ddi[0] * var1 * (v - vi)) + ddi[1] * var1 * (u - ui));
      lodi[3] = kin * (ddi[0] * var1 * (u - ui) + ddi[1] * var1 * (v - vi) + ddi[2] * var1 * (w - wi) +
                       (pr - c.prs_in[fj]) / rho / css);
      for (int r = 0; r < 5; ++r) {
        double acc = 0.0;
        for (int m = 0; m < 5; ++m) acc = acc + pnor[r][m] * lodi[m];
        const double add = acc * J + rest[r];
        c.qrhs[c.z(0, j, k) + r * n0] += add;
      }
    }
  // tangential derivatives on the face: y for k = ks..ke, z for j = js..je
  for (int k = c.ks; k <= c.ke; ++k)
    for (int j = c.js; j <= c.je; ++j) {
      double fp[5], fm[5];
      row_flux(c, c.h(0, j + 1, k), 1, fp);
      row_flux(c, c.h(0, j - 1, k), 1, fm);
      for (int n = 0; n < 5; ++n) c.qrhs[c.z(0, j, k) + n * n0] += 0.5 * (fp[n] - fm[n]);
    }
  if (c.ndims == 3)
    for (int j = c.js; j <= c.je; ++j)
      for (int k = c.ks; k <= c.ke; ++k) {
        double fp[5], fm[5];
        row_flux(c, c.h(0, j, k + 1), 2, fp);
        row_flux(c, c.h(0, j, k - 1), 2, fm);
        for (int n = 0; n < 5; ++n) c.qrhs[c.z(0, j, k) + n * n0] += 0.5 * (fp[n] - fm[n]);
      }
}

}  // namespace

void orc_boucon(orc_ctx* c) {
  for (int n = 0; n < 2 * c->ndims; ++n) {
    const int type = face_bctype(*c, n);
    if (type == 12 && n == 0 && c->npdc(0) == 4) {
      inflow_nscbc(*c);
      continue;
    }
    if (type != 41 && type != 42 && type != 50 && type != 60 && type != 421 && type != 21 &&
        type != 51 && type != 411 && type != 11 && type != 23)
      continue;
    const int d = n / 2;
    if (c->npdc(d) != 4 || ((type == 421 || type == 411) && d != 1) ||
        ((type == 21 || type == 23) && n != 1 && n != 3) || (type == 51 && d == 0) ||
        (type == 11 && n != 0))
      continue;
    const double tw = face_twall(*c, n);
    const double extent = type == 23 ? grid_extent(*c, d) : 0.0;
    const int a1 = d == 0 ? c->jm : c->im, b1 = d == 2 ? c->jm : c->km;
    for (int b = 0; b <= b1; ++b)
      for (int a = 0; a <= a1; ++a) {
        const int i = d == 0 ? 0 : a, j = d == 0 ? a : (d == 1 ? 0 : b), k = d == 2 ? 0 : b;
        face_node(*c, n, type, tw, i, j, k, extent);
      }
  }
}

namespace {

// Trapezoid sums over y of 0.5*(f(j-1)+f(j))*dy, i = 1..im, j = 1..jm,
// k = 1..km (k = 0 in 2-D): the bulk integrals of src_chan and
// massfluxchan (src/solver.F90:295-353, src/statistic.F90:1437-1476).
double ytrapezoid(const orc_ctx& c, int m) {
  const int k1 = c.ndims == 3 ? 1 : 0, k2 = c.ndims == 3 ? c.km : 0;
  const long nh = c.nh;
  double s = 0.0;
  for (int k = k1; k <= k2; ++k)
    for (int j = 1; j <= c.jm; ++j)
      for (int i = 1; i <= c.im; ++i) {
        const double dy = c.x[c.h(i, j, k) + nh] - c.x[c.h(i, j - 1, k) + nh];
        s = s + 0.5 * (c.q[c.h(i, j - 1, k) + m * nh] + c.q[c.h(i, j, k) + m * nh]) * dy;
      }
  return s;
}

// src_chan, src/solver.F90:295-353: body force and its work.
void src_chan(orc_ctx& c) {
  double robulk = ytrapezoid(c, 0);
  double u1 = ytrapezoid(c, 1) / robulk;
  double u2 = ytrapezoid(c, 2) / robulk;
  double u3 = ytrapezoid(c, 3) / robulk;
  const long n0 = c.n0;
  for (int k = 0; k <= c.km; ++k)
    for (int j = 0; j <= c.jm; ++j)
      for (int i = 0; i <= c.im; ++i) {
        const long z = c.z(i, j, k);
        const double J = c.jacob[c.h(i, j, k)];
        c.qrhs[z + 1 * n0] = c.qrhs[z + 1 * n0] + c.force[0] * J;
        c.qrhs[z + 2 * n0] = c.qrhs[z + 2 * n0] + c.force[1] * J;
        c.qrhs[z + 3 * n0] = c.qrhs[z + 3 * n0] + c.force[2] * J;
        c.qrhs[z + 4 * n0] =
            c.qrhs[z + 4 * n0] + (c.force[0] * u1 + c.force[1] * u2 + c.force[2] * u3) * J;
      }
}

// statcal for flowtype 'channel' (src/statistic.F90:641-657): wall friction
// fbcxchan (1303-1367), mass flux massfluxchan (1437-1476), the target set
// on the first call, and the body force from chanfoce (1494-1533).
void chan_statcal(orc_ctx& c) {
  const int k1 = c.ndims == 3 ? 1 : 0, k2 = c.ndims == 3 ? c.km : 0;
  const double norm = c.ndims == 3 ? (double)c.cfg.ia * (double)c.cfg.ka : (double)c.cfg.ia;
  const long n0 = c.n0;
  double fb = 0.0;
  for (int side = 0; side < 2; ++side) {
    const int j = side == 0 ? 0 : c.jm;
    for (int k = k1; k <= k2; ++k)
      for (int i = 1; i <= c.im; ++i) {
        const double T = c.tmp[c.h(i, j, k)];
        const double miu = T * std::sqrt(T) * c.tempconst1 / (T + c.tempconst) / c.cfg.reynolds;
        const double dudy = c.dvel[c.z(i, j, k) + 3 * n0];  // dvel(i,j,k,1,2)
        fb = side == 0 ? fb + miu * dudy : fb - miu * dudy;
      }
  }
  c.fbcx = fb / norm;
  c.massflux = ytrapezoid(c, 1) / norm;
  if (std::fabs(c.massflux_target) < 1e-16) {
    c.massflux_target = c.massflux;
    c.force[0] = c.force[1] = c.force[2] = 0.0;
  }
  const double ly = c.x[c.h(0, c.jm, 0) + c.nh] - c.x[c.h(0, 0, 0) + c.nh];
  const double f = c.force[0];
  double fnew;
  if (c.nstep == 0) {
    fnew = c.fbcx / ly;
  } else {
    const double gn = ly * f - c.fbcx;
    const double qn1 = c.massflux + c.cfg.deltat * gn;
    const double ref_len = 1.0;  // nondimensional reference length, src/solver.F90:126
    fnew = f - (2.0 * (qn1 - c.massflux_target) - 0.2 * (c.massflux - c.massflux_target)) / ly *
                   (c.uinf / ref_len);
  }
  c.force[0] = fnew;
}

}  // namespace

void orc_chan_state(orc_ctx* c, double* out) {
  out[0] = c->force[0];
  out[1] = c->massflux;
  out[2] = c->massflux_target;
  out[3] = c->fbcx;
  out[4] = (double)c->nstep;
}

// gradcal, src/comsolver.F90:244-497 (main) ; tgvsolver.F90:450-537 (mini-app)
void orc_gradcal(orc_ctx* c) {
  const long nh = c->nh, n0 = c->n0;
  const bool mini = c->cfg.mode == ORC_MODE_MINIAPP;
  if (!mini) {
    std::fill(c->dvel.begin(), c->dvel.end(), 0.0);
    std::fill(c->dtmp.begin(), c->dtmp.end(), 0.0);
  }
  const int mx = std::max(c->im, std::max(c->jm, c->km));
  for (int d = 0; d < c->ndims; ++d) {
    int a1, b1;
    trans_range(*c, d, a1, b1);
    const int dim = c->dimof(d);
    const long sz = c->zstride(d);
    const double hdx = d == 0 ? c->dxm : (d == 1 ? c->dym : c->dzm);
    for_lines(*c, d, 0, a1, 0, b1, [&](int a, int b) {
      thread_local LineBuf* lb = nullptr;
      thread_local std::vector<double> df;
      if (a < 0) { delete lb; lb = new LineBuf(mx); df.resize(4 * (mx + 1)); return; }
      const double* src[4] = {c->vel.data(), c->vel.data() + nh, c->vel.data() + 2 * nh, c->tmp.data()};
      for (int n = 0; n < 4; ++n) line_deriv(c, d, src[n], a, b, *lb, df.data() + n * (dim + 1));
      long z0 = zpos(*c, d, 0, a, b);
      long h0 = hpos(*c, d, 0, a, b);
      const long hs = c->hstride(d);
      for (int l = 0; l <= dim; ++l) {
        long zp = z0 + sz * l, hp = h0 + hs * l;
        if (mini) {
          for (int n = 0; n < 3; ++n) c->dvel[zp + (n + 3 * d) * n0] = df[n * (dim + 1) + l] / hdx;
          c->dtmp[zp + d * n0] = df[3 * (dim + 1) + l] / hdx;
        } else {
          for (int n = 0; n < 3; ++n)
            for (int m = 0; m < 3; ++m) {
              double& g = c->dvel[zp + (n + 3 * m) * n0];
              g = g + df[n * (dim + 1) + l] * c->dxi[hp + (d + 3 * m) * nh];
            }
          for (int m = 0; m < 3; ++m) {
            double& g = c->dtmp[zp + m * n0];
            g = g + df[3 * (dim + 1) + l] * c->dxi[hp + (d + 3 * m) * nh];
          }
        }
      }
    });
  }
}

// convrsdcal6, src/solver.F90:2173-2341 (main) ; convection,
// tgvsolver.F90:539-633 (mini-app)
void orc_convrsdcal6(orc_ctx* c) {
  const long nh = c->nh, n0 = c->n0;
  const bool mini = c->cfg.mode == ORC_MODE_MINIAPP;
  const int mx = std::max(c->im, std::max(c->jm, c->km));
  for (int d = 0; d < c->ndims; ++d) {
    const int dim = c->dimof(d);
    const long hs = c->hstride(d), sz = c->zstride(d);
    int a0, a1, b0, b1, l0, l1;
    if (mini) {
      a0 = 0; b0 = 0; trans_range(*c, d, a1, b1); l0 = 0; l1 = dim;
    } else if (d == 0) { a0 = c->js; a1 = c->je; b0 = c->ks; b1 = c->ke; l0 = c->is; l1 = c->ie; }
    else if (d == 1) { a0 = c->is; a1 = c->ie; b0 = c->ks; b1 = c->ke; l0 = c->js; l1 = c->je; }
    else { a0 = c->is; a1 = c->ie; b0 = c->js; b1 = c->je; l0 = c->ks; l1 = c->ke; }
    const double hdx = d == 0 ? c->dxm : (d == 1 ? c->dym : c->dzm);
    for_lines(*c, d, a0, a1, b0, b1, [&](int a, int b) {
      thread_local LineBuf* lb = nullptr;
      thread_local std::vector<double> fcs, dfc;
      if (a < 0) {
        delete lb; lb = new LineBuf(mx);
        fcs.resize(5 * (mx + 2 * HM + 1)); dfc.resize(5 * (mx + 1));
        return;
      }
      const long h0 = hpos(*c, d, 0, a, b);
      const int L = dim + 2 * HM + 1;
      const double* q = c->q.data();
      const double* J = c->jacob.data();
      for (int l = -HM; l <= dim + HM; ++l) {
        long p = h0 + hs * l;
        double* F = fcs.data() + (l + HM);
        double q1 = q[p], q2 = q[p + nh], q3 = q[p + 2 * nh], q4 = q[p + 3 * nh], q5 = q[p + 4 * nh];
        double pr = c->prs[p];
        if (mini) {
          double uu = c->vel[p + d * nh];
          F[0] = q1 * uu;
          F[L] = q2 * uu;
          F[2 * L] = q3 * uu;
          F[3 * L] = q4 * uu;
          F[(1 + d) * L] = F[(1 + d) * L] + pr;
          F[4 * L] = (q5 + pr) * uu;
        } else {
          const double* X = c->dxi.data() + p;
          double x1 = X[(d + 0) * nh], x2 = X[(d + 3) * nh], x3 = X[(d + 6) * nh];
          double uu = x1 * c->vel[p] + x2 * c->vel[p + nh] + x3 * c->vel[p + 2 * nh];
          double jj = J[p];
          F[0] = jj * q1 * uu;
          F[L] = jj * (q2 * uu + x1 * pr);
          F[2 * L] = jj * (q3 * uu + x2 * pr);
          F[3 * L] = jj * (q4 * uu + x3 * pr);
          F[4 * L] = jj * (q5 + pr) * uu;
        }
      }
      for (int n = 0; n < 5; ++n)
        df_compact(c->fd[d], fcs.data() + n * L + HM, dfc.data() + n * (dim + 1), lb->d.data(),
                   lb->xx.data());
      const long z0 = zpos(*c, d, 0, a, b);
      for (int n = 0; n < 5; ++n)
        for (int l = l0; l <= l1; ++l) {
          double& r = c->qrhs[z0 + sz * l + n * n0];
          if (mini) r = r + dfc[n * (dim + 1) + l] / hdx;
          else r = r + dfc[n * (dim + 1) + l];
        }
    });
  }
}

// diffrsdcal6, src/solver.F90:2354-2873 (turbmode none, no species) ;
// diffusion, tgvsolver.F90:635-789 (mini-app)
void orc_diffrsdcal6(orc_ctx* c) {
  const long nh = c->nh, n0 = c->n0;
  const bool mini = c->cfg.mode == ORC_MODE_MINIAPP;
  std::fill(c->sigma.begin(), c->sigma.end(), 0.0);
  std::fill(c->qflux.begin(), c->qflux.end(), 0.0);
  const double re = c->cfg.reynolds, pr = c->cfg.prandtl;
#pragma omp parallel for collapse(2)
  for (int k = 0; k <= c->km; ++k)
    for (int j = 0; j <= c->jm; ++j)
      for (int i = 0; i <= c->im; ++i) {
        long p = c->h(i, j, k), zp = c->z(i, j, k);
        double T = c->tmp[p];
        // miucal, src/fludyna.F90:791-820
        double miu = T * std::sqrt(T) * c->tempconst1 / (T + c->tempconst) / re;
        auto dv = [&](int n, int m) { return c->dvel[zp + ((n - 1) + 3 * (m - 1)) * n0]; };
        double s11 = dv(1, 1);
        double s12 = 0.5 * (dv(1, 2) + dv(2, 1));
        double s13 = 0.5 * (dv(1, 3) + dv(3, 1));
        double s22 = dv(2, 2);
        double s23 = 0.5 * (dv(2, 3) + dv(3, 2));
        double s33 = dv(3, 3);
        double skk = NUM1D3 * (s11 + s22 + s33);
        double miu2 = 2.0 * miu;
        double hcc = (miu / pr) / c->const5;
        double* S = c->sigma.data() + p;
        S[0] = miu2 * (s11 - skk);
        S[nh] = miu2 * s12;
        S[2 * nh] = miu2 * s13;
        S[3 * nh] = miu2 * (s22 - skk);
        S[4 * nh] = miu2 * s23;
        S[5 * nh] = miu2 * (s33 - skk);
        double u = c->vel[p], v = c->vel[p + nh], w = c->vel[p + 2 * nh];
        double* Q = c->qflux.data() + p;
        const double* dT = c->dtmp.data() + zp;
        Q[0] = hcc * dT[0] + S[0] * u + S[nh] * v + S[2 * nh] * w;
        Q[nh] = hcc * dT[n0] + S[nh] * u + S[3 * nh] * v + S[4 * nh] * w;
        Q[2 * nh] = hcc * dT[2 * n0] + S[2 * nh] * u + S[4 * nh] * v + S[5 * nh] * w;
      }
  dataswap(*c, c->sigma.data(), 6, 0);
  dataswap(*c, c->qflux.data(), 3, 0);
  // sigma components needed per direction: (1,2,3) (2,4,5) (3,5,6)
  const int sidx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  const int mx = std::max(c->im, std::max(c->jm, c->km));
  for (int d = 0; d < c->ndims; ++d) {
    const int dim = c->dimof(d);
    const long hs = c->hstride(d), sz = c->zstride(d);
    int a1, b1;
    trans_range(*c, d, a1, b1);
    int l0, l1;
    if (mini) { l0 = 0; l1 = dim; }
    else if (d == 0) { l0 = c->is; l1 = c->ie; }
    else if (d == 1) { l0 = c->js; l1 = c->je; }
    else { l0 = c->ks; l1 = c->ke; }
    const double hdx = d == 0 ? c->dxm : (d == 1 ? c->dym : c->dzm);
    for_lines(*c, d, 0, a1, 0, b1, [&](int a, int b) {
      thread_local LineBuf* lb = nullptr;
      thread_local std::vector<double> ff, df;
      if (a < 0) {
        delete lb; lb = new LineBuf(mx);
        ff.resize(4 * (mx + 2 * HM + 1)); df.resize(4 * (mx + 1));
        return;
      }
      const long h0 = hpos(*c, d, 0, a, b);
      const int L = dim + 2 * HM + 1;
      const double* S = c->sigma.data();
      const double* Q = c->qflux.data();
      for (int l = -HM; l <= dim + HM; ++l) {
        long p = h0 + hs * l;
        double* F = ff.data() + (l + HM);
        if (mini) {
          F[0] = S[p + sidx[d][0] * nh];
          F[L] = S[p + sidx[d][1] * nh];
          F[2 * L] = S[p + sidx[d][2] * nh];
          F[3 * L] = Q[p + d * nh];
        } else {
          const double* X = c->dxi.data() + p;
          double x1 = X[(d + 0) * nh], x2 = X[(d + 3) * nh], x3 = X[(d + 6) * nh];
          double jj = c->jacob[p];
          F[0] = (S[p] * x1 + S[p + nh] * x2 + S[p + 2 * nh] * x3) * jj;
          F[L] = (S[p + nh] * x1 + S[p + 3 * nh] * x2 + S[p + 4 * nh] * x3) * jj;
          F[2 * L] = (S[p + 2 * nh] * x1 + S[p + 4 * nh] * x2 + S[p + 5 * nh] * x3) * jj;
          F[3 * L] = (Q[p] * x1 + Q[p + nh] * x2 + Q[p + 2 * nh] * x3) * jj;
        }
      }
      for (int n = 0; n < 4; ++n)
        df_compact(c->fd[d], ff.data() + n * L + HM, df.data() + n * (dim + 1), lb->d.data(),
                   lb->xx.data());
      const long z0 = zpos(*c, d, 0, a, b);
      for (int n = 0; n < 4; ++n)
        for (int l = l0; l <= l1; ++l) {
          double& r = c->qrhs[z0 + sz * l + (n + 1) * n0];
          if (mini) r = r + df[n * (dim + 1) + l] / hdx;
          else r = r + df[n * (dim + 1) + l];
        }
    });
  }
}


// ducrossensor, src/commcal.F90:196-353
void orc_ducrossensor(orc_ctx* c) {
  const int im = c->im, jm = c->jm, km = c->km;
  const long n0 = c->n0;
  const int npi = c->cfg.npdci, npj = c->cfg.npdcj, npk = c->cfg.npdck;
#pragma omp parallel for collapse(2)
  for (int k = 0; k <= km; ++k)
    for (int j = 0; j <= jm; ++j)
      for (int i = 0; i <= im; ++i) {
        const long zp = c->z(i, j, k);
        auto dv = [&](int n, int m) { return c->dvel[zp + ((n - 1) + 3 * (m - 1)) * n0]; };
        const double dsum = dv(1, 1) + dv(2, 2) + dv(3, 3);
        const double div2 = dsum * dsum;
        const double vortx = dv(3, 2) - dv(2, 3);
        const double vorty = dv(1, 3) - dv(3, 1);
        const double vortz = dv(2, 1) - dv(1, 2);
        const double vort = vortx * vortx + vorty * vorty + vortz * vortz;
        int ip1 = i + 1, im1 = i - 1, jp1 = j + 1, jm1 = j - 1, kp1 = k + 1, km1 = k - 1;
        if (npi == 1 && im1 < 0) im1 = 0;
        if (npj == 1 && jm1 < 0) jm1 = 0;
        if (npk == 1 && km1 < 0) km1 = 0;
        if (npi == 2 && ip1 > im) ip1 = im;
        if (npj == 2 && jp1 > jm) jp1 = jm;
        if (npk == 2 && kp1 > km) kp1 = km;
        const double* P = c->prs.data();
        const double p0 = P[c->h(i, j, k)];
        auto dp = [&](double pm, double pp) {
          return std::fabs(pp - 2.0 * p0 + pm) / (pp + 2.0 * p0 + pm);
        };
        const double dpdi = dp(P[c->h(im1, j, k)], P[c->h(ip1, j, k)]);
        const double dpdj = dp(P[c->h(i, jm1, k)], P[c->h(i, jp1, k)]);
        const double dpdk = dp(P[c->h(i, j, km1)], P[c->h(i, j, kp1)]);
        c->ssf[c->h(i, j, k)] = div2 / (div2 + vort + 1.e-30) * std::max(std::max(dpdi, dpdj), dpdk);
      }
  dataswap(*c, c->ssf.data(), 1, 0);
#pragma omp parallel for collapse(2)
  for (int k = 0; k <= km; ++k)
    for (int j = 0; j <= jm; ++j)
      for (int i = 0; i <= im; ++i) {
        double mx = 0.0;
        for (int i1 = -HM + 1; i1 <= HM; ++i1) {
          int ii = i + i1;
          if (npi == 1 && ii < 0) ii = 0;
          if (npi == 2 && ii > im) ii = im;
          mx = std::max(mx, c->ssf[c->h(ii, j, k)]);
        }
        for (int j1 = -HM + 1; j1 <= HM; ++j1) {
          int jj = j + j1;
          if (npj == 1 && jj < 0) jj = 0;
          if (npj == 2 && jj > jm) jj = jm;
          mx = std::max(mx, c->ssf[c->h(i, jj, k)]);
        }
        for (int k1 = -HM + 1; k1 <= HM; ++k1) {
          int kk = k + k1;
          if (npk == 1 && kk < 0) kk = 0;
          if (npk == 2 && kk > km) kk = km;
          mx = std::max(mx, c->ssf[c->h(i, j, kk)]);
        }
        c->lshock[c->z(i, j, k)] = mx > c->cfg.shkcrt ? 1 : 0;
      }
  c->sson = true;
}

int orc_lshock(orc_ctx* c, unsigned char* out) {
  if (!c->sson) return 0;
  std::memcpy(out, c->lshock.data(), c->lshock.size());
  return 1;
}

// convrsdcmp, src/solver.F90:1271-1937 (no species, crinod all false: the
// reference sets it only in crash recovery, src/mainloop.F90:81, 738)
void orc_convrsdcmp(orc_ctx* c) {
  const long nh = c->nh, n0 = c->n0;
  const int mx = std::max(c->im, std::max(c->jm, c->km));
  const bool chard = c->cfg.lchardecomp != 0;
  const double mach = c->cfg.mach, bf = c->cfg.bfacmpld;
  for (int d = 0; d < c->ndims; ++d) {
    const int dim = c->dimof(d), npdc = c->npdc(d);
    const long hs = c->hstride(d), sz = c->zstride(d);
    int a0, a1, b0, b1, l0, l1;
    if (d == 0) { a0 = c->js; a1 = c->je; b0 = c->ks; b1 = c->ke; l0 = c->is; l1 = c->ie; }
    else if (d == 1) { a0 = c->is; a1 = c->ie; b0 = c->ks; b1 = c->ke; l0 = c->js; l1 = c->je; }
    else { a0 = c->is; a1 = c->ie; b0 = c->js; b1 = c->je; l0 = c->ks; l1 = c->ke; }
    int iss, iee;
    split_range(npdc, dim, iss, iee);
    for_lines(*c, d, a0, a1, b0, b1, [&](int a, int b) {
      thread_local std::vector<double> fsw, fhc, Fh, dd, xx;
      const int L = mx + 2 * HM + 1;
      if (a < 0) {
        fsw.assign(10 * L, 0.0); fhc.assign(10 * (mx + 2), 0.0); Fh.assign(5 * (mx + 2), 0.0);
        dd.assign(mx + 16, 0.0); xx.assign(mx + 16, 0.0);
        return;
      }
      const long h0 = hpos(*c, d, 0, a, b), z0 = zpos(*c, d, 0, a, b);
      auto FP = [&](int n, int l) -> double& { return fsw[n * L + l + HM]; };
      auto FM = [&](int n, int l) -> double& { return fsw[(5 + n) * L + l + HM]; };
      for (int l = iss; l <= iee; ++l) {
        const long p = h0 + hs * l;
        const double vel[3] = {c->vel[p], c->vel[p + nh], c->vel[p + 2 * nh]};
        const double q[5] = {c->q[p], c->q[p + nh], c->q[p + 2 * nh], c->q[p + 3 * nh], c->q[p + 4 * nh]};
        const double xr[3] = {c->dxi[p + (d + 0) * nh], c->dxi[p + (d + 3) * nh], c->dxi[p + (d + 6) * nh]};
        double fp[5], fm[5];
        steger_warming(mach, c->rho[p], vel, c->prs[p], c->tmp[p], q, xr, c->jacob[p], fp, fm);
        for (int n = 0; n < 5; ++n) { FP(n, l) = fp[n]; FM(n, l) = fm[n]; }
      }
      for (int n = 0; n < 5; ++n) {
        flux_compact(c->fuw[d], +1, bf, &FP(n, 0), fhc.data() + n * (mx + 2), dd.data(), xx.data());
        flux_compact(c->fdw[d], -1, bf, &FM(n, 0), fhc.data() + (5 + n) * (mx + 2), dd.data(), xx.data());
      }
      auto HCP = [&](int n, int i) { return fhc[n * (mx + 2) + i + 1]; };
      auto HCM = [&](int n, int i) { return fhc[(5 + n) * (mx + 2) + i + 1]; };
      auto state = [&](int l, double* st) {
        const long p = h0 + hs * l;
        st[0] = c->tmp[p]; st[1] = c->rho[p]; st[2] = c->prs[p]; st[3] = c->q[p + 4 * nh];
        st[4] = c->vel[p]; st[5] = c->vel[p + nh]; st[6] = c->vel[p + 2 * nh];
        st[7] = c->dxi[p + (d + 0) * nh]; st[8] = c->dxi[p + (d + 3) * nh]; st[9] = c->dxi[p + (d + 6) * nh];
      };
      auto lsh_at = [&](int l) { return c->lshock[z0 + sz * l] != 0; };
      for (int i = l0 - 1; i <= l1; ++i) {
        double R[25], Lv[25], flcp[5][5], flcm[5][5], fhcpc[5], fhcmc[5];
        if (chard) {
          double sl[10], sr[10];
          state(i, sl);
          state(i + 1, sr);
          chardecomp(sl, sr, R, Lv);
          auto lev = [&](int m, int k) { return Lv[m + 5 * k]; };
          for (int m = 0; m < 5; ++m) {
            for (int n = 1; n <= 5; ++n) {
              int w = iwind6(i, n, iss, iee, +1);
              flcp[m][n - 1] = lev(m, 0) * FP(0, w) + lev(m, 1) * FP(1, w) + lev(m, 2) * FP(2, w) +
                               lev(m, 3) * FP(3, w) + lev(m, 4) * FP(4, w);
              w = iwind6(i, n, iss, iee, -1);
              flcm[m][n - 1] = lev(m, 0) * FM(0, w) + lev(m, 1) * FM(1, w) + lev(m, 2) * FM(2, w) +
                               lev(m, 3) * FM(3, w) + lev(m, 4) * FM(4, w);
            }
            fhcpc[m] = lev(m, 0) * HCP(0, i) + lev(m, 1) * HCP(1, i) + lev(m, 2) * HCP(2, i) +
                       lev(m, 3) * HCP(3, i) + lev(m, 4) * HCP(4, i);
            fhcmc[m] = lev(m, 0) * HCM(0, i) + lev(m, 1) * HCM(1, i) + lev(m, 2) * HCM(2, i) +
                       lev(m, 3) * HCM(3, i) + lev(m, 4) * HCM(4, i);
          }
        } else {
          for (int n = 1; n <= 5; ++n) {
            const int wp = iwind6(i, n, iss, iee, +1), wm = iwind6(i, n, iss, iee, -1);
            for (int m = 0; m < 5; ++m) { flcp[m][n - 1] = FP(m, wp); flcm[m][n - 1] = FM(m, wm); }
          }
          for (int m = 0; m < 5; ++m) { fhcpc[m] = HCP(m, i); fhcmc[m] = HCM(m, i); }
        }
        bool lsh = true;
        if (c->sson) {
          if (i < 0) lsh = lsh_at(i + 1);
          else if (i + 1 > dim) lsh = lsh_at(i);
          else lsh = lsh_at(i) || lsh_at(i + 1);
        }
        double Fhc[5];
        for (int m = 0; m < 5; ++m) {
          const double v1 = mplimiter(flcp[m], fhcpc[m], lsh, i, dim, npdc);
          const double v2 = mplimiter(flcm[m], fhcmc[m], lsh, i, dim, npdc);
          Fhc[m] = v1 + v2;
        }
        for (int m = 0; m < 5; ++m) {
          double v = Fhc[m];
          if (chard)
            v = R[m] * Fhc[0] + R[m + 5] * Fhc[1] + R[m + 10] * Fhc[2] + R[m + 15] * Fhc[3] +
                R[m + 20] * Fhc[4];
          Fh[m * (mx + 2) + i + 1] = v;
        }
      }
      for (int l = l0; l <= l1; ++l)
        for (int m = 0; m < 5; ++m) {
          double& r = c->qrhs[z0 + sz * l + m * n0];
          r = r + Fh[m * (mx + 2) + l + 1] - Fh[m * (mx + 2) + l];
        }
    });
  }
}

void orc_line_flux(orc_ctx* c, int dir, int wind, const double* f, double* fh) {
  const int dim = c->dimof(dir);
  std::vector<double> d(dim + 16), xx(dim + 16);
  const Scheme& s = wind > 0 ? c->fuw[dir] : c->fdw[dir];
  flux_compact(s, wind, c->cfg.bfacmpld, f + HM, fh, d.data(), xx.data());
}

double orc_mp5(const double* u5, double ul, int discont) { return mp5(u5, ul, discont != 0); }

void orc_steger_warming(orc_ctx* c, const double* prim, const double* q5, const double* dxi3,
                        double jac, double* fp, double* fm) {
  steger_warming(c->cfg.mach, prim[0], prim + 1, prim[4], prim[5], q5, dxi3, jac, fp, fm);
}

void orc_chardecomp(const double* stl, const double* str, double* rev, double* lev) {
  chardecomp(stl, str, rev, lev);
}

// rhscal, src/solver.F90:185-282 (main) ; tgvsolver.F90:962-992 (mini-app)
void orc_rhscal(orc_ctx* c) {
  if (c->cfg.conschm_mp && c->cfg.mode == ORC_MODE_MAIN) {
    if (c->cfg.lchardecomp) orc_ducrossensor(c);
    orc_convrsdcmp(c);
  } else {
    orc_convrsdcal6(c);
  }
  for (auto& r : c->qrhs) r = -r;
  if (c->cfg.diffterm) orc_diffrsdcal6(c);
  if (c->cfg.channel) src_chan(*c);
}

// updatefvar -> q2fvar_3da on 0:im (src/fludyna.F90:191-242)
void orc_updatefvar(orc_ctx* c) { q2fvar_box(*c, 0, c->im, 0, c->jm, 0, c->km); }

// bchomo, tgvsolver.F90:271-369
void orc_bchomo(orc_ctx* c) {
  const int im = c->im, jm = c->jm, km = c->km;
  const long nh = c->nh;
  auto copy = [&](long dst, long src) {
    c->rho[dst] = c->rho[src];
    for (int n = 0; n < 3; ++n) c->vel[dst + n * nh] = c->vel[src + n * nh];
    c->tmp[dst] = c->tmp[src];
    c->prs[dst] = c->prs[src];
    fvar2q_prs_node(*c, dst);
  };
  for (int k = 0; k <= km; ++k)
    for (int j = 0; j <= jm; ++j) {
      for (int i = -HM; i <= -1; ++i) copy(c->h(i, j, k), c->h(im + i, j, k));
      for (int i = im + 1; i <= im + HM; ++i) copy(c->h(i, j, k), c->h(i - im, j, k));
    }
  for (int k = 0; k <= km; ++k)
    for (int i = 0; i <= im; ++i) {
      for (int j = -HM; j <= -1; ++j) copy(c->h(i, j, k), c->h(i, jm + j, k));
      for (int j = jm + 1; j <= jm + HM; ++j) copy(c->h(i, j, k), c->h(i, j - jm, k));
    }
  for (int j = 0; j <= jm; ++j)
    for (int i = 0; i <= im; ++i) {
      for (int k = -HM; k <= -1; ++k) copy(c->h(i, j, k), c->h(i, j, km + k));
      for (int k = km + 1; k <= km + HM; ++k) copy(c->h(i, j, k), c->h(i, j, k - km));
    }
}

// kenergycal / enstophycal, src/statistic.F90:871-992 ;
// mini-app stacal, tgvsolver.F90:893-942
double orc_kenergy(orc_ctx* c) {
  const long nh = c->nh;
  double s = 0.0;
  const int k0 = c->ndims == 3 ? 1 : 0, k1 = c->ndims == 3 ? c->km : 0;
  for (int k = k0; k <= k1; ++k)
    for (int j = 1; j <= c->jm; ++j)
      for (int i = 1; i <= c->im; ++i) {
        long p = c->h(i, j, k);
        double u = c->vel[p], v = c->vel[p + nh], w = c->vel[p + 2 * nh];
        double var1 = u * u + v * v + w * w;
        s = s + c->rho[p] * var1;
      }
  double npts = c->ndims == 3 ? (double)c->cfg.ia * c->cfg.ja * c->cfg.ka
                              : (double)c->cfg.ia * c->cfg.ja;
  if (c->cfg.mode == ORC_MODE_MINIAPP) return 0.5 * s / npts;
  return 0.5 * s / npts / (c->roinf * c->uinf * c->uinf);
}

double orc_enstrophy(orc_ctx* c) {
  const long n0 = c->n0;
  double s = 0.0;
  const int k0 = c->ndims == 3 ? 1 : 0, k1 = c->ndims == 3 ? c->km : 0;
  for (int k = k0; k <= k1; ++k)
    for (int j = 1; j <= c->jm; ++j)
      for (int i = 1; i <= c->im; ++i) {
        long zp = c->z(i, j, k);
        auto dv = [&](int n, int m) { return c->dvel[zp + ((n - 1) + 3 * (m - 1)) * n0]; };
        double o1 = dv(3, 2) - dv(2, 3), o2 = dv(1, 3) - dv(3, 1), o3 = dv(2, 1) - dv(1, 2);
        double om = c->ndims == 3 ? o1 * o1 + o2 * o2 + o3 * o3 : o3 * o3;
        s = s + c->rho[c->h(i, j, k)] * om;
      }
  double npts = c->ndims == 3 ? (double)c->cfg.ia * c->cfg.ja * c->cfg.ka
                              : (double)c->cfg.ia * c->cfg.ja;
  if (c->cfg.mode == ORC_MODE_MINIAPP) return 0.5 * s / npts;
  double xmax = c->x[c->h(c->im, 0, 0)];
  double l0 = xmax / (2.0 * PI);
  return 0.5 * s / npts / (c->roinf * ((c->uinf / l0) * (c->uinf / l0)));
}

// One RK3 step.  Main ordering: time_integration_rk, src/mainloop.F90:396-486.
// Mini-app ordering: rk3, tgvsolver.F90:994-1082.
void orc_rk3_step(orc_ctx* c, double* stats) {
  static const double rk[3][3] = {{1.0, 0.0, 1.0}, {0.75, 0.25, 0.25}, {NUM1D3, NUM2D3, NUM2D3}};
  const long nh = c->nh, n0 = c->n0;
  const int im = c->im, jm = c->jm, km = c->km;
  const double dt = c->cfg.deltat;
  const bool mini = c->cfg.mode == ORC_MODE_MINIAPP;
  for (int s = 0; s < 3; ++s) {
    if (mini) {
      orc_bchomo(c);
      std::fill(c->qrhs.begin(), c->qrhs.end(), 0.0);
      orc_gradcal(c);
      orc_rhscal(c);
      if (s == 0) {
        if (stats) { stats[0] = orc_kenergy(c); stats[1] = orc_enstrophy(c); }
        for (int n = 0; n < 5; ++n)
          for (int k = 0; k <= km; ++k)
            for (int j = 0; j <= jm; ++j)
              for (int i = 0; i <= im; ++i)
                c->qsave[c->z(i, j, k) + n * n0] = c->q[c->h(i, j, k) + n * nh];
      }
#pragma omp parallel for collapse(2)
      for (int n = 0; n < 5; ++n)
        for (int k = 0; k <= km; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) {
              long p = c->h(i, j, k) + n * nh, zp = c->z(i, j, k) + n * n0;
              c->q[p] = rk[s][0] * c->qsave[zp] + rk[s][1] * c->q[p] + rk[s][2] * c->qrhs[zp] * dt;
            }
      orc_filterq(c);
      orc_updatefvar(c);
    } else {
      if (c->cfg.lfilter) orc_filterq(c);
      std::fill(c->qrhs.begin(), c->qrhs.end(), 0.0);
      orc_boucon(c);
      orc_qswap(c);
      orc_gradcal(c);
      if (s == 0) {
        for (int n = 0; n < 5; ++n)
          for (int k = 0; k <= km; ++k)
            for (int j = 0; j <= jm; ++j)
              for (int i = 0; i <= im; ++i) {
                long p = c->h(i, j, k);
                c->qsave[c->z(i, j, k) + n * n0] = c->q[p + n * nh] * c->jacob[p];
              }
        if (stats) { stats[0] = orc_kenergy(c); stats[1] = orc_enstrophy(c); }
        // rkfirst (src/mainloop.F90:614-697): statcal from the second call on
        if (c->cfg.channel && c->rkfirst_called) chan_statcal(*c);
        c->rkfirst_called = true;
      }
      orc_rhscal(c);
#pragma omp parallel for collapse(2)
      for (int n = 0; n < 5; ++n)
        for (int k = 0; k <= km; ++k)
          for (int j = 0; j <= jm; ++j)
            for (int i = 0; i <= im; ++i) {
              long p = c->h(i, j, k), zp = c->z(i, j, k) + n * n0;
              double J = c->jacob[p];
              double v = rk[s][0] * c->qsave[zp] + rk[s][1] * c->q[p + n * nh] * J +
                         rk[s][2] * c->qrhs[zp] * dt;
              c->q[p + n * nh] = v / J;
            }
      orc_updatefvar(c);
    }
  }
  c->nstep = c->nstep + 1;
}

void orc_rk3_steps(orc_ctx* c, int nsteps, double* stats) {
  for (int s = 0; s < nsteps; ++s) orc_rk3_step(c, stats ? stats + 2 * s : nullptr);
}

void orc_line_derivative(orc_ctx* c, int dir, const double* f, double* df) {
  LineBuf lb(c->dimof(dir));
  df_compact(c->fd[dir], f + HM, df, lb.d.data(), lb.xx.data());
}

void orc_line_filter(orc_ctx* c, int dir, const double* f, double* ff) {
  LineBuf lb(c->dimof(dir));
  compact_filter(c->flt[dir], c->ft, f + HM, ff, lb.d.data(), lb.xx.data());
}

}  // extern "C"
