// smac_adjoint.cu -- discrete adjoint of the converged pseudo-time iteration.
//
// The reference has no sensitivities; this file adds them on top of its steady equations.
// At a fixed point of the iteration (dq = 0) the state q and the far-field vortex strength
// clift satisfy
//
//   F(q, clift; x, y, alpha) = 0      and      clift = Cl(q; x, y, alpha),
//
// where F is the assembled right-hand side s (conup + viscterms + blanking + bcmain,
// ref/step.f:268-519, ref/conup.f, ref/visc.f:50-160, ref/bc.f:1080-1869) on every row except
// the wake cut, and on the wake cut
//
//   F(jt,1) = (q(jt,2) + q(jb,2)) / 2 - q(jt,1),
//
// the condition bcimpds (ref/bc.f:566-595) imposes once dq = 0.  A perimeter point that no
// bcmain.dat region covers keeps its value (its row of the implicit operator is the identity
// and s = 0 there), so its equation is q = const.  The far field uses the previous iteration's
// lift (ref/bc.f:1364-1374, ref/smac2d.f:1825), which becomes the clift equation.
//
// For an objective J (Cl or Cd of iterout, ref/smac2d.f:1737-1745) the adjoint lambda solves
//
//   A^T lambda = -dJ/dq,     A = dF/dq + (dF/dclift) (dCl/dq)^T,
//
// and the gradient for a design variable b (a grid motion dx/db, dy/db and a change of alpha) is
//
//   dJ/db = J_b + lambda . F_b + (lambda . dF/dclift) Cl_b.
//
// dF/dq is assembled exactly, by forward-mode differentiation with dual numbers: F at a point
// depends on q on the 9-point cross of radius 2 (third-order fluxes) and, on the wake cut only,
// on the partner point across the cut (handled separately).  Colouring points by
// (j + 5k) mod 13 gives the nine cross offsets nine different colours, so 13 x 3 seeded
// evaluations recover every 3x3 block.  The transposed system is solved by restarted GMRES,
// right-preconditioned by stationary steps of the transposed iteration whose inner solve is
// zebra line relaxation of the transposed implicit operator (FP32 by default; FP64 lines or
// its LU-SGS sweeps as options).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "smac_common.cuh"
#include "smac_kernels.cuh"
#include "smac_adjoint.cuh"

namespace smac {

// ------------------------------------------------------------------------------------------
// dual numbers (value, one directional derivative)
struct Dual {
  double v, d;
  __device__ __forceinline__ Dual() : v(0.0), d(0.0) {}
  __device__ __forceinline__ Dual(double x) : v(x), d(0.0) {}
  __device__ __forceinline__ Dual(double x, double dx) : v(x), d(dx) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
__device__ __forceinline__ Dual operator/(double a, Dual b) {
  double q = a / b.v;
  return Dual(q, -q * b.d / b.v);
}
__device__ __forceinline__ Dual dsqrt(Dual a) {
  double r = sqrt(a.v);
  return Dual(r, a.d / (2.0 * r));
}
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ Dual dabs(Dual a) { return a.v < 0.0 ? Dual(-a.v, -a.d) : a; }
__device__ __forceinline__ double dabs(double a) { return fabs(a); }
__device__ __forceinline__ double dval(double a) { return a; }
__device__ __forceinline__ double dval(Dual a) { return a.v; }

// su = vfp*udp - vfm*udm of viscterms.  Reference arithmetic: the four factors and the
// result are REAL*4 (ref/visc.f:68); the derivative is that of the exact expression.
__device__ __forceinline__ double visc_diff(double vfp, double udp, double vfm, double udm, bool f64) {
  if (f64) return vfp * udp - vfm * udm;
  float a = (float)vfp, b = (float)udp, c = (float)vfm, e = (float)udm;
  return (double)__fsub_rn(__fmul_rn(a, b), __fmul_rn(c, e));
}
__device__ __forceinline__ Dual visc_diff(Dual vfp, Dual udp, Dual vfm, Dual udm, bool f64) {
  double v = visc_diff(vfp.v, udp.v, vfm.v, udm.v, f64);
  return Dual(v, vfp.d * udp.v + vfp.v * udp.d - vfm.d * udm.v - vfm.v * udm.d);
}

// ------------------------------------------------------------------------------------------
// accessors: q and the geometry as T, with the derivative seeds of each use
struct QPlain {  // q, no derivative
  const double* q;
  size_t N;
  int jmax;
  template <class T>
  __device__ __forceinline__ T get(int j, int k, int n) const { return T(q[ix(j, k, jmax) + N * n]); }
};
struct QSeed {  // q with a unit seed on component comp of the points of one colour
  const double* q;
  size_t N;
  int jmax, color, comp;
  template <class T>
  __device__ __forceinline__ T get(int j, int k, int n) const;
};
template <>
__device__ __forceinline__ Dual QSeed::get<Dual>(int j, int k, int n) const {
  double s = (n == comp && (j + 5 * k) % 13 == color) ? 1.0 : 0.0;
  return Dual(q[ix(j, k, jmax) + N * n], s);
}
struct GeoPlain {
  const double *rtxy, *dj, *x, *y;
  size_t N;
  template <class T>
  __device__ __forceinline__ T rt(size_t id, int c) const { return T(rtxy[id + N * c]); }
  template <class T>
  __device__ __forceinline__ T jac(size_t id) const { return T(dj[id]); }
  template <class T>
  __device__ __forceinline__ T gx(size_t id) const { return T(x[id]); }
  template <class T>
  __device__ __forceinline__ T gy(size_t id) const { return T(y[id]); }
};
struct GeoDir {  // geometry with the derivative of a grid motion
  const double *rtxy, *dj, *x, *y;
  const double *drtxy, *ddj, *dx, *dy;
  size_t N;
  template <class T>
  __device__ __forceinline__ T rt(size_t id, int c) const { return T(rtxy[id + N * c], drtxy[id + N * c]); }
  template <class T>
  __device__ __forceinline__ T jac(size_t id) const { return T(dj[id], ddj[id]); }
  template <class T>
  __device__ __forceinline__ T gx(size_t id) const { return T(x[id], dx[id]); }
  template <class T>
  __device__ __forceinline__ T gy(size_t id) const { return T(y[id], dy[id]); }
};

// ------------------------------------------------------------------------------------------
// the steady equations at one point

// split Jacobians of a face, ref/conup.f:127-185 (entry (row r, col c) at [r + 3c])
template <class T>
__device__ __forceinline__ void face_split_t(T rt, T rx, T ry, T q2, T q3, double beta, T* ap, T* am) {
  T cvel = rx * q2 + ry * q3;
  T t = cvel + 0.5 * rt;
  T cc = dsqrt(t * t + beta * (rx * rx + ry * ry));
  T eig = cvel + rt;
  T eig1 = 0.5 * (eig + dabs(eig));
  T eig2 = cvel + rt * 0.5 + cc;
  T x21 = -(ry * eig1 / (cc * cc - 0.25 * rt * rt));
  T x31 = rx * eig1 / (cc * cc - 0.25 * rt * rt);
  T x12 = 0.5 * eig2 / cc;
  T x22 = 0.5 * eig2 * (q2 * eig2 + beta * rx) / (beta * cc * (cc - 0.5 * rt));
  T x32 = 0.5 * eig2 * (q3 * eig2 + beta * ry) / (beta * cc * (cc - 0.5 * rt));
  T xi11 = ry * q2 - rx * q3;
  T xi12 = -(q3 * (cvel + rt)) - ry * beta;
  T xi13 = q2 * (cvel + rt) + rx * beta;
  T xi21 = cc - cvel - 0.5 * rt;
  T xi22 = rx * beta;
  T xi23 = ry * beta;
  ap[0] = x12 * xi21;
  ap[1] = x21 * xi11 + x22 * xi21;
  ap[2] = x31 * xi11 + x32 * xi21;
  ap[3] = x12 * xi22;
  ap[4] = x21 * xi12 + x22 * xi22;
  ap[5] = x31 * xi12 + x32 * xi22;
  ap[6] = x12 * xi23;
  ap[7] = x21 * xi13 + x22 * xi23;
  ap[8] = x31 * xi13 + x32 * xi23;
  am[0] = -ap[0];
  am[1] = -ap[1] + rx;
  am[2] = -ap[2] + ry;
  am[3] = -ap[3] + rx * beta;
  am[4] = -ap[4] + rt + 2. * rx * q2 + ry * q3;
  am[5] = -ap[5] + rx * q3;
  am[6] = -ap[6] + ry * beta;
  am[7] = -ap[7] + ry * q2;
  am[8] = -ap[8] + rt + rx * q2 + 2. * ry * q3;
}

struct LineAt {  // position pos of line `line` in direction d (0: j varies, 1: k varies)
  int d, line, jmax;
  __device__ __forceinline__ int j(int pos) const { return d == 0 ? pos : line; }
  __device__ __forceinline__ int k(int pos) const { return d == 0 ? line : pos; }
  __device__ __forceinline__ size_t id(int pos) const { return d == 0 ? ix(pos, line, jmax) : ix(line, pos, jmax); }
};

// flux differences A+ dq, A- dq of face f (between f and f+1); f = n-1 is not a face
template <class T, class QA, class GA>
__device__ __forceinline__ void face_df(const LineAt& L, int n, int f, const QA& qa, const GA& ga, double beta,
                                        T* dfp, T* dfm) {
  if (f < 0 || f > n - 2) {
    for (int r = 0; r < 3; ++r) { dfp[r] = T(0.0); dfm[r] = T(0.0); }
    return;
  }
  const int d = L.d;
  size_t i0 = L.id(f), i1 = L.id(f + 1);
  T rt = 0.5 * (ga.template rt<T>(i1, 0 + d) + ga.template rt<T>(i0, 0 + d));
  T rx = 0.5 * (ga.template rt<T>(i1, 2 + d) + ga.template rt<T>(i0, 2 + d));
  T ry = 0.5 * (ga.template rt<T>(i1, 4 + d) + ga.template rt<T>(i0, 4 + d));
  T a1 = qa.template get<T>(L.j(f), L.k(f), 0), a2 = qa.template get<T>(L.j(f), L.k(f), 1),
    a3 = qa.template get<T>(L.j(f), L.k(f), 2);
  T b1 = qa.template get<T>(L.j(f + 1), L.k(f + 1), 0), b2 = qa.template get<T>(L.j(f + 1), L.k(f + 1), 1),
    b3 = qa.template get<T>(L.j(f + 1), L.k(f + 1), 2);
  T q2 = 0.5 * (b2 + a2);
  T q3 = 0.5 * (b3 + a3);
  T ap[9], am[9];
  face_split_t<T>(rt, rx, ry, q2, q3, beta, ap, am);
  T dq1 = b1 - a1, dq2 = b2 - a2, dq3 = b3 - a3;
  for (int r = 0; r < 3; ++r) {
    dfp[r] = ap[r] * dq1 + ap[r + 3] * dq2 + ap[r + 6] * dq3;
    dfm[r] = am[r] * dq1 + am[r + 3] * dq2 + am[r + 6] * dq3;
  }
}

// physical flux at a point (ref/flux.f:185-200)
template <class T, class QA, class GA>
__device__ __forceinline__ void point_fv(const LineAt& L, int p, const QA& qa, const GA& ga, double beta, T* F) {
  const int d = L.d;
  size_t id = L.id(p);
  T r1 = ga.template rt<T>(id, 0 + d), r2 = ga.template rt<T>(id, 2 + d), r3 = ga.template rt<T>(id, 4 + d);
  T q1 = qa.template get<T>(L.j(p), L.k(p), 0), q2 = qa.template get<T>(L.j(p), L.k(p), 1),
    q3 = qa.template get<T>(L.j(p), L.k(p), 2);
  T cvel = r1 + r2 * q2 + r3 * q3;
  F[0] = r1 * q1 + beta * (cvel - r1);
  F[1] = q2 * cvel + r2 * q1;
  F[2] = q3 * cvel + r3 * q1;
}

// third-order numerical flux at face f (ref/flux.f:213-256) from the flux differences of faces
// f-1, f, f+1 (dfp[0..2], dfm[0..2]; face f+1 is zero when it is the non-face n-1, and face f-1
// is replaced by face f at the start of the line, as the reference's index clamps do)
template <class T>
__device__ __forceinline__ void face_flux(int n, int f, const T (*dfp)[3], const T (*dfm)[3], const T* F0, const T* F1,
                                          double cdis, T* out) {
  int fm = f - 1 > 0 ? f - 1 : 0;
  int fp = f + 1 < n - 1 ? f + 1 : n - 1;
  int fpp = f + 2 < n - 1 ? f + 2 : n - 1;
  double cp = (double)(fpp - fp);
  double cm = (double)(f - fm);
  const double r6 = FLIT(1.0f / 6.0f);
  const int im = (fm == f) ? 1 : 0;
  for (int m = 0; m < 3; ++m) {
    T fmv = (dfp[1][m] + dfm[1][m] - dfp[2][m] - dfm[2][m]) * r6;
    T fpv = (dfp[im][m] + dfm[im][m] - dfp[1][m] - dfm[1][m]) * r6;
    T f3 = (dfp[im][m] - dfp[1][m] + dfm[1][m] - dfm[2][m]) * r6;
    out[m] = 0.5 * (F1[m] + F0[m]) + cdis * (cp * cm * f3 + cm * (1. - cp) * fpv + cp * (1. - cm) * fmv);
  }
}

// f(p) - f(p-1) of one direction at interior position p of a line
template <class T, class QA, class GA>
__device__ __forceinline__ void line_resid(const LineAt& L, int n, int p, const QA& qa, const GA& ga, double beta,
                                           double cdis, T* out) {
  T dfp[4][3], dfm[4][3];  // faces p-2 .. p+1
  for (int i = 0; i < 4; ++i) face_df<T>(L, n, p - 2 + i, qa, ga, beta, dfp[i], dfm[i]);
  T fv0[3], fv1[3], fv2[3];  // points p-1, p, p+1
  point_fv<T>(L, p - 1, qa, ga, beta, fv0);
  point_fv<T>(L, p, qa, ga, beta, fv1);
  point_fv<T>(L, p + 1, qa, ga, beta, fv2);
  T flm[3], flp[3];
  face_flux<T>(n, p - 1, dfp, dfm, fv0, fv1, cdis, flm);
  face_flux<T>(n, p, dfp + 1, dfm + 1, fv1, fv2, cdis, flp);
  for (int m = 0; m < 3; ++m) out[m] = flp[m] - flm[m];
}

struct AdjPoint {
  int jmax, kmax;
  size_t N;
  double beta, cdis, vnu, pout, pi;
  int ivis, visc64;
};

// point kinds
constexpr int kRowInterior = 0, kRowBC = 1, kRowWake = 2, kRowFrozen = 3;

__device__ __forceinline__ bool on_wake(const BCTable* bc, int j, int k) {
  if (k != 0) return false;
  for (int r = 0; r < bc->nwake; ++r)
    if (j >= bc->jt_b[r] && j <= bc->jt_e[r]) return true;
  return false;
}

// F at (j,k) for the non-wake rows; returns the row kind (wake rows: F untouched)
template <class T, class QA, class GA>
__device__ int point_F(const AdjPoint& P, const BCTable* bc, int j, int k, const QA& qa, const GA& ga, T uinf,
                       T vinf, T clift, T* F) {
  const int jmax = P.jmax, kmax = P.kmax;
  const double beta = P.beta;
  const size_t id = ix(j, k, jmax);
  const bool perim = j == 0 || j == jmax - 1 || k == 0 || k == kmax - 1;
  if (!perim) {
    T sj[3], sk[3];
    LineAt Lj{0, k, jmax}, Lk{1, j, jmax};
    line_resid<T>(Lj, jmax, j, qa, ga, beta, P.cdis, sj);
    line_resid<T>(Lk, kmax, k, qa, ga, beta, P.cdis, sk);
    for (int m = 0; m < 3; ++m) F[m] = -sj[m];
    for (int m = 0; m < 3; ++m) F[m] = F[m] - sk[m];
    if (P.ivis) {
      const double vnu = P.vnu;
      for (int vd = 0; vd < 2; ++vd) {
        int jm = vd == 0 ? j - 1 : j, km = vd == 0 ? k : k - 1;
        int jp = vd == 0 ? j + 1 : j, kp = vd == 0 ? k : k + 1;
        size_t im = ix(jm, km, jmax), ip = ix(jp, kp, jmax);
        T djvm = 0.5 * (ga.template jac<T>(im) * vnu + ga.template jac<T>(id) * vnu);
        T djvp = 0.5 * (ga.template jac<T>(id) * vnu + ga.template jac<T>(ip) * vnu);
        T rxm = 0.5 * (ga.template rt<T>(im, 2 + vd) + ga.template rt<T>(id, 2 + vd));
        T rym = 0.5 * (ga.template rt<T>(im, 4 + vd) + ga.template rt<T>(id, 4 + vd));
        T rxp = 0.5 * (ga.template rt<T>(id, 2 + vd) + ga.template rt<T>(ip, 2 + vd));
        T ryp = 0.5 * (ga.template rt<T>(id, 4 + vd) + ga.template rt<T>(ip, 4 + vd));
        T vfm = djvm * (rxm * rxm + rym * rym);
        T vfp = djvp * (rxp * rxp + ryp * ryp);
        T u0 = qa.template get<T>(j, k, 1), um = qa.template get<T>(jm, km, 1), up = qa.template get<T>(jp, kp, 1);
        T v0 = qa.template get<T>(j, k, 2), vm = qa.template get<T>(jm, km, 2), vp = qa.template get<T>(jp, kp, 2);
        F[1] = F[1] + visc_diff(vfp, up - u0, vfm, u0 - um, P.visc64 != 0);
        F[2] = F[2] + visc_diff(vfp, vp - v0, vfm, v0 - vm, P.visc64 != 0);
      }
    }
    return kRowInterior;
  }
  if (on_wake(bc, j, k)) return kRowWake;
  // boundary rows: blanked to zero, then the bcmain.dat regions in file order (ref/bc.f:60-224)
  for (int m = 0; m < 3; ++m) F[m] = T(0.0);
  bool covered = false;
  for (int r = 0; r < bc->nreg; ++r) {
    const BCRegion& R = bc->reg[r];
    if (j < R.jb || j > R.je || k < R.kb || k > R.ke) continue;
    int dir = R.jkbc;
    bool lo = dir == 1 ? (j == 0) : (k == 0);
    int jn = dir == 1 ? (lo ? j + 1 : j - 1) : j, kn = dir == 1 ? k : (lo ? k + 1 : k - 1);
    if (R.ibcval == 0) {
      // bcnoslj / bcnoslk (ref/bc.f:1093-1104, 1147-1158)
      int jf = dir == 1 ? j + 1 : j, kf = dir == 1 ? k : k + 1;
      F[0] = qa.template get<T>(jf, kf, 0) - qa.template get<T>(j, k, 0);
      F[1] = -qa.template get<T>(j, k, 1);
      F[2] = -qa.template get<T>(j, k, 2);
      covered = true;
    } else if (R.ibcval == 25) {
      // bccgridj / bccgridk (ref/bc.f:1202-1276, 1351-1431)
      T dx = ga.template gx<T>(id) - 0.25;
      T dy = ga.template gy<T>(id);
      T ucirc = clift * dy / (4. * P.pi * (dx * dx + dy * dy));
      T vcirc = -(clift * dx / (4. * P.pi * (dx * dx + dy * dy)));
      T q1 = qa.template get<T>(j, k, 0), q2 = qa.template get<T>(j, k, 1), q3 = qa.template get<T>(j, k, 2);
      F[1] = uinf + ucirc - q2;
      F[2] = vinf + vcirc - q3;
      int jk = dir - 1;
      T r2 = ga.template rt<T>(id, 2 + jk), r3 = ga.template rt<T>(id, 4 + jk);
      T qq = r2 * q2 + r3 * q3;
      T cc = dsqrt(qq * qq + beta * (r2 * r2 + r3 * r3));
      T n1 = qa.template get<T>(jn, kn, 0), n2 = qa.template get<T>(jn, kn, 1), n3 = qa.template get<T>(jn, kn, 2);
      if (lo) {
        T b0 = r2 * r2 + r3 * r3, b3 = r2 * (qq - cc), b6 = r3 * (qq - cc);
        F[0] = -b0 * (n1 - q1) - b3 * (n2 - q2) - b6 * (n3 - q3);
      } else {
        T b0 = -(r2 * r2 + r3 * r3), b3 = -(r2 * (qq + cc)), b6 = -(r3 * (qq + cc));
        F[0] = b0 * (q1 - n1) + b3 * (q2 - n2) + b6 * (q3 - n3);
      }
      covered = true;
    } else if (R.ibcval == 31) {
      // bcoutj / bcoutk (ref/bc.f:1622-1669, 1813-1858)
      F[1] = qa.template get<T>(jn, kn, 1) - qa.template get<T>(j, k, 1);
      F[2] = qa.template get<T>(jn, kn, 2) - qa.template get<T>(j, k, 2);
      F[0] = P.pout - qa.template get<T>(j, k, 0);
      covered = true;
    }
  }
  if (covered) return kRowBC;
  // q = const: F = q_now - q (zero at the state, derivative -I)
  for (int m = 0; m < 3; ++m) {
    T qm = qa.template get<T>(j, k, m);
    F[m] = dval(qm) - qm;
  }
  return kRowFrozen;
}

// ------------------------------------------------------------------------------------------
// kernels
struct AdjArgs {
  AdjPoint P;
  const BCTable* bc;
  const double *q, *rtxy, *dj, *x, *y;
  double uinf, vinf, clift;
};

// F (values) at every point; wake rows from the averaging condition
__global__ void k_adj_residual(AdjArgs a, double* __restrict__ F) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= a.P.jmax || k >= a.P.kmax) return;
  const size_t N = a.P.N;
  QPlain qa{a.q, N, a.P.jmax};
  GeoPlain ga{a.rtxy, a.dj, a.x, a.y, N};
  double f[3];
  int kind = point_F<double>(a.P, a.bc, j, k, qa, ga, a.uinf, a.vinf, a.clift, f);
  size_t id = ix(j, k, a.P.jmax);
  if (kind == kRowWake) return;  // k_adj_wake_residual
  for (int m = 0; m < 3; ++m) F[id + N * m] = f[m];
}

__global__ void k_adj_wake_residual(const BCTable* __restrict__ bc, const double* __restrict__ q, int jmax, size_t N,
                                    double* __restrict__ F) {
  for (int r = 0; r < bc->nwake; ++r)
    for (int jt = bc->jt_b[r], i = 0; jt <= bc->jt_e[r]; ++jt, ++i) {
      int jb = bc->jb_b[r] - i;
      for (int n = 0; n < 3; ++n)
        F[ix(jt, 0, jmax) + N * n] =
            0.5 * (q[ix(jt, 1, jmax) + N * n] + q[ix(jb, 1, jmax) + N * n]) - q[ix(jt, 0, jmax) + N * n];
    }
}

// offsets of the nine blocks of a row: centre, j-1, j+1, j-2, j+2, k-1, k+1, k-2, k+2
__constant__ int c_offj[kAdjSlots] = {0, -1, 1, -2, 2, 0, 0, 0, 0};
__constant__ int c_offk[kAdjSlots] = {0, 0, 0, 0, 0, -1, 1, -2, 2};

// one colour and one component: the columns of that colour of every row's blocks
__global__ void k_adj_jac_color(AdjArgs a, int color, int comp, double* __restrict__ jac) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  const int jmax = a.P.jmax, kmax = a.P.kmax;
  if (j >= jmax || k >= kmax) return;
  const size_t N = a.P.N;
  QSeed qa{a.q, N, jmax, color, comp};
  GeoPlain ga{a.rtxy, a.dj, a.x, a.y, N};
  Dual f[3];
  int kind = point_F<Dual>(a.P, a.bc, j, k, qa, ga, Dual(a.uinf), Dual(a.vinf), Dual(a.clift), f);
  if (kind == kRowWake) return;  // rows stay zero (jac is cleared before the colours)
  size_t id = ix(j, k, jmax);
  for (int s = 0; s < kAdjSlots; ++s) {
    int jj = j + c_offj[s], kk = k + c_offk[s];
    if (jj < 0 || jj >= jmax || kk < 0 || kk >= kmax) continue;
    if ((jj + 5 * kk) % 13 != color) continue;
    for (int r = 0; r < 3; ++r) jac[id + N * (size_t)(s * 9 + r + 3 * comp)] = f[r].d;
    break;
  }
}

// dF/dclift
__global__ void k_adj_dclift(AdjArgs a, double* __restrict__ fc) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= a.P.jmax || k >= a.P.kmax) return;
  const size_t N = a.P.N;
  QPlain qa{a.q, N, a.P.jmax};
  GeoPlain ga{a.rtxy, a.dj, a.x, a.y, N};
  Dual f[3];
  int kind = point_F<Dual>(a.P, a.bc, j, k, qa, ga, Dual(a.uinf), Dual(a.vinf), Dual(a.clift, 1.0), f);
  size_t id = ix(j, k, a.P.jmax);
  for (int m = 0; m < 3; ++m) fc[id + N * m] = kind == kRowWake ? 0.0 : f[m].d;
}

// F_b for a grid motion (drtxy, ddj, dx, dy) and a change of the free stream (duinf, dvinf)
__global__ void k_adj_design(AdjArgs a, const double* __restrict__ drtxy, const double* __restrict__ ddj,
                             const double* __restrict__ dx, const double* __restrict__ dy, double duinf,
                             double dvinf, double* __restrict__ fb) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= a.P.jmax || k >= a.P.kmax) return;
  const size_t N = a.P.N;
  QPlain qa{a.q, N, a.P.jmax};
  GeoDir ga{a.rtxy, a.dj, a.x, a.y, drtxy, ddj, dx, dy, N};
  Dual f[3];
  int kind = point_F<Dual>(a.P, a.bc, j, k, qa, ga, Dual(a.uinf, duinf), Dual(a.vinf, dvinf), Dual(a.clift), f);
  size_t id = ix(j, k, a.P.jmax);
  for (int m = 0; m < 3; ++m) fb[id + N * m] = kind == kRowWake ? 0.0 : f[m].d;
}

// derivative of the metric (ref/metric.f:49-278) along a grid motion (dx, dy)
__global__ void k_adj_metric_dir(const double* __restrict__ x, const double* __restrict__ y,
                                 const double* __restrict__ dx, const double* __restrict__ dy, int jmax, int kmax,
                                 double* __restrict__ drtxy, double* __restrict__ ddj) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t N = (size_t)jmax * kmax;
  auto X = [&](int a, int b) { size_t i = ix(a, b, jmax); return Dual(x[i], dx[i]); };
  auto Y = [&](int a, int b) { size_t i = ix(a, b, jmax); return Dual(y[i], dy[i]); };
  Dual xj, yj, xk, yk;
  if (j == 0) {
    xj = 0.5 * (-X(j + 2, k) + 4. * X(j + 1, k) - 3. * X(j, k));
    yj = 0.5 * (-Y(j + 2, k) + 4. * Y(j + 1, k) - 3. * Y(j, k));
  } else if (j == jmax - 1) {
    xj = 0.5 * (3. * X(j, k) - 4. * X(j - 1, k) + X(j - 2, k));
    yj = 0.5 * (3. * Y(j, k) - 4. * Y(j - 1, k) + Y(j - 2, k));
  } else {
    xj = 0.5 * (X(j + 1, k) - X(j - 1, k));
    yj = 0.5 * (Y(j + 1, k) - Y(j - 1, k));
  }
  if (k == 0) {
    xk = 0.5 * (-X(j, k + 2) + 4. * X(j, k + 1) - 3. * X(j, k));
    yk = 0.5 * (-Y(j, k + 2) + 4. * Y(j, k + 1) - 3. * Y(j, k));
  } else if (k == kmax - 1) {
    xk = 0.5 * (3. * X(j, k) - 4. * X(j, k - 1) + X(j, k - 2));
    yk = 0.5 * (3. * Y(j, k) - 4. * Y(j, k - 1) + Y(j, k - 2));
  } else {
    xk = 0.5 * (X(j, k + 1) - X(j, k - 1));
    yk = 0.5 * (Y(j, k + 1) - Y(j, k - 1));
  }
  size_t id = ix(j, k, jmax);
  Dual rdj = xj * yk - xk * yj;
  ddj[id] = (1. / rdj).d;
  drtxy[id + N * 0] = 0.0;
  drtxy[id + N * 1] = 0.0;
  drtxy[id + N * 2] = yk.d;
  drtxy[id + N * 4] = -xk.d;
  drtxy[id + N * 3] = -yj.d;
  drtxy[id + N * 5] = xj.d;
}

// ------------------------------------------------------------------------------------------
// forces (ref/fm.f:156-324, ref/smac2d.f:1737-1745): Cd and Cl are linear in q; their
// gradients in q come from the two faces next to each wall point.
struct ForceGeo {
  int jmax;
  size_t N;
  double vnu;
  int ivis;
};

// face i of wall w (between positions i and i+1): the x and y force contributions
// (pressure faces enter fxp, fyp with a minus sign; viscous faces fxs, fys with a plus sign)
template <class T, class QA, class GA>
__device__ __forceinline__ void wall_face(const ForceGeo& G, const BCTable* bc, int w, int i, const QA& qa,
                                          const GA& ga, T& fx, T& fy) {
  int dir = bc->wjk[w] == 1 ? 1 : 2;
  int at = dir == 2 ? bc->wk1[w] : bc->wj1[w];
  int d = dir == 2 ? 1 : 0;
  auto pj = [&](int pos, int off) { return dir == 2 ? pos : at + off; };
  auto pk = [&](int pos, int off) { return dir == 2 ? at + off : pos; };
  size_t i0 = ix(pj(i, 0), pk(i, 0), G.jmax), i1 = ix(pj(i + 1, 0), pk(i + 1, 0), G.jmax);
  T pave = 0.5 * (qa.template get<T>(pj(i + 1, 0), pk(i + 1, 0), 0) + qa.template get<T>(pj(i, 0), pk(i, 0), 0));
  T da1 = 0.5 * (ga.template rt<T>(i1, 2 + d) + ga.template rt<T>(i0, 2 + d));
  T da2 = 0.5 * (ga.template rt<T>(i1, 4 + d) + ga.template rt<T>(i0, 4 + d));
  fx = -(pave * da1);
  fy = -(pave * da2);
  if (!G.ivis) return;
  T t11[2], t22[2], t12[2];
  for (int e = 0; e < 2; ++e) {
    int pos = i + e;
    size_t id = ix(pj(pos, 0), pk(pos, 0), G.jmax);
    T ueta = 0.5 * (-(3. * qa.template get<T>(pj(pos, 0), pk(pos, 0), 1)) +
                    4. * qa.template get<T>(pj(pos, 1), pk(pos, 1), 1) - qa.template get<T>(pj(pos, 2), pk(pos, 2), 1));
    T veta = 0.5 * (-(3. * qa.template get<T>(pj(pos, 0), pk(pos, 0), 2)) +
                    4. * qa.template get<T>(pj(pos, 1), pk(pos, 1), 2) - qa.template get<T>(pj(pos, 2), pk(pos, 2), 2));
    T r2 = ga.template rt<T>(id, 2 + d), r3 = ga.template rt<T>(id, 4 + d);
    T djv = ga.template jac<T>(id);
    t11[e] = 2. * G.vnu * r2 * djv * ueta;
    t22[e] = 2. * G.vnu * r3 * djv * veta;
    t12[e] = G.vnu * (r3 * ueta + r2 * veta) * djv;
  }
  T t11a = 0.5 * (t11[1] + t11[0]), t22a = 0.5 * (t22[1] + t22[0]), t12a = 0.5 * (t12[1] + t12[0]);
  fx = fx + (t11a * da1 + t12a * da2);
  fy = fy + (t12a * da1 + t22a * da2);
}

struct QPoint {  // q with a unit seed on one point and component
  const double* q;
  size_t N;
  int jmax, sj, sk, sn;
  template <class T>
  __device__ __forceinline__ T get(int j, int k, int n) const;
};
template <>
__device__ __forceinline__ Dual QPoint::get<Dual>(int j, int k, int n) const {
  return Dual(q[ix(j, k, jmax) + N * n], (j == sj && k == sk && n == sn) ? 1.0 : 0.0);
}

// dCl/dq and dCd/dq: one thread per (wall point, normal offset 0..2, component)
__global__ void k_adj_force_grad(ForceGeo G, const BCTable* __restrict__ bc, int w, const double* __restrict__ q,
                                 GeoPlain ga, double ca, double sa, double* __restrict__ gcl,
                                 double* __restrict__ gcd) {
  int dir = bc->wjk[w] == 1 ? 1 : 2;
  int at = dir == 2 ? bc->wk1[w] : bc->wj1[w];
  int b = dir == 2 ? bc->wj1[w] : bc->wk1[w];
  int e = dir == 2 ? bc->wj2[w] : bc->wk2[w];
  int npts = e - b + 1;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * 9) return;
  int pos = b + t / 9, off = (t % 9) / 3, n = t % 3;
  int sj = dir == 2 ? pos : at + off, sk = dir == 2 ? at + off : pos;
  QPoint qa{q, G.N, G.jmax, sj, sk, n};
  Dual fx(0.0), fy(0.0);
  for (int f = pos - 1; f <= pos; ++f) {
    if (f < b || f > e - 1) continue;
    Dual ax, ay;
    wall_face<Dual>(G, bc, w, f, qa, ga, ax, ay);
    fx = fx + ax;
    fy = fy + ay;
  }
  size_t id = ix(sj, sk, G.jmax) + G.N * n;
  gcd[id] = 2. * fx.d * ca + 2. * fy.d * sa;
  gcl[id] = 2. * fy.d * ca - 2. * fx.d * sa;
}

// Cl, Cd and their derivatives along a grid motion and a change of alpha (dca, dsa): one
// block, faces strided over the threads, a fixed-order tree sum
template <class GA>
__global__ void k_adj_force_dir(ForceGeo G, const BCTable* __restrict__ bc, const double* __restrict__ q, GA ga,
                                double ca, double dca, double sa, double dsa, double* __restrict__ out) {
  __shared__ double red[4][256];
  QPlain qa{q, G.N, G.jmax};
  Dual fx(0.0), fy(0.0);
  for (int w = 0; w < bc->nwall; ++w) {
    int dir = bc->wjk[w] == 1 ? 1 : 2;
    int b = dir == 2 ? bc->wj1[w] : bc->wk1[w];
    int e = dir == 2 ? bc->wj2[w] : bc->wk2[w];
    for (int f = b + threadIdx.x; f <= e - 1; f += blockDim.x) {
      Dual ax, ay;
      wall_face<Dual>(G, bc, w, f, qa, ga, ax, ay);
      fx = fx + ax;
      fy = fy + ay;
    }
  }
  red[0][threadIdx.x] = fx.v; red[1][threadIdx.x] = fx.d;
  red[2][threadIdx.x] = fy.v; red[3][threadIdx.x] = fy.d;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    Dual Fx(red[0][0], red[1][0]), Fy(red[2][0], red[3][0]);
    Dual C(ca, dca), S(sa, dsa);
    Dual cd = 2. * Fx * C + 2. * Fy * S;
    Dual cl = 2. * Fy * C - 2. * Fx * S;
    out[0] = cl.v; out[1] = cl.d; out[2] = cd.v; out[3] = cd.d;
  }
}

// ------------------------------------------------------------------------------------------
// the operator A and its transpose, and vector kernels

// y = dF/dq v (wake rows zero here)
__global__ void k_adj_jv(const double* __restrict__ jac, int jmax, int kmax, const double* __restrict__ v,
                         double* __restrict__ y) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t N = (size_t)jmax * kmax, id = ix(j, k, jmax);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int s = 0; s < kAdjSlots; ++s) {
    int jj = j + c_offj[s], kk = k + c_offk[s];
    if (jj < 0 || jj >= jmax || kk < 0 || kk >= kmax) continue;
    size_t ic = ix(jj, kk, jmax);
    double v0 = v[ic], v1 = v[ic + N], v2 = v[ic + 2 * N];
    for (int r = 0; r < 3; ++r) {
      const double* B = jac + id + N * (size_t)(s * 9 + r);
      acc[r] += B[0] * v0 + B[3 * N] * v1 + B[6 * N] * v2;
    }
  }
  for (int r = 0; r < 3; ++r) y[id + N * r] = acc[r];
}

// y = dF/dq^T w (wake rows contribute nothing here): column (j,k) gathers from the rows
// (j,k) - offset of each slot
__global__ void k_adj_jtv(const double* __restrict__ jac, int jmax, int kmax, const double* __restrict__ w,
                          double* __restrict__ y) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t N = (size_t)jmax * kmax, id = ix(j, k, jmax);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int s = 0; s < kAdjSlots; ++s) {
    int jr = j - c_offj[s], kr = k - c_offk[s];
    if (jr < 0 || jr >= jmax || kr < 0 || kr >= kmax) continue;
    size_t ir = ix(jr, kr, jmax);
    double w0 = w[ir], w1 = w[ir + N], w2 = w[ir + 2 * N];
    for (int c = 0; c < 3; ++c) {
      const double* B = jac + ir + N * (size_t)(s * 9 + 3 * c);
      acc[c] += B[0] * w0 + B[N] * w1 + B[2 * N] * w2;
    }
  }
  for (int c = 0; c < 3; ++c) y[id + N * c] = acc[c];
}

// wake-cut rows, one thread per wake point jt (and component).  Forward:
// y(jt,1) = (v(jt,2) + v(jb,2))/2 - v(jt,1).  Transposed: the rows (jt,1) and (jb,1) are the
// only ones that reach column (jt,2) (the two wake segments pair up as mirrors, so jb's partner
// is jt), so the thread of jt adds -w(jt,1) to column (jt,1) and (w(jt,1) + w(jb,1))/2 to
// column (jt,2): no two threads write the same entry.
__global__ void k_adj_wake(const BCTable* __restrict__ bc, int jmax, size_t N, int transpose,
                           const double* __restrict__ v, double* __restrict__ y) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = t % 3;
  t /= 3;
  for (int r = 0; r < bc->nwake; ++r) {
    const int len = bc->jt_e[r] - bc->jt_b[r] + 1;
    if (t >= len) { t -= len; continue; }
    const int jt = bc->jt_b[r] + t, jb = bc->jb_b[r] - t;
    const size_t t0 = ix(jt, 0, jmax) + N * n, t1 = ix(jt, 1, jmax) + N * n;
    const size_t b0 = ix(jb, 0, jmax) + N * n, b1 = ix(jb, 1, jmax) + N * n;
    if (!transpose) {
      y[t0] = 0.5 * (v[t1] + v[b1]) - v[t0];
    } else {
      y[t0] -= v[t0];
      y[t1] += 0.5 * v[t0] + 0.5 * v[b0];
    }
    return;
  }
}

// deterministic dot products: partial sums per block, then one fixed-order tree
constexpr int kDotBlocks = 304, kDotThreads = 256;

__global__ void __launch_bounds__(kDotThreads) k_adj_mdot_partial(const double* __restrict__ V, size_t ldv,
                                                                  const double* __restrict__ w, size_t n,
                                                                  double* __restrict__ part) {
  __shared__ double red[kDotThreads];
  const double* a = V + ldv * blockIdx.y;
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)kDotThreads + threadIdx.x; i < n; i += (size_t)kDotBlocks * kDotThreads)
    acc += a[i] * w[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kDotThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)blockIdx.y * kDotBlocks + blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(512) k_adj_mdot_final(const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double red[512];
  const double* p = part + (size_t)blockIdx.x * kDotBlocks;
  red[threadIdx.x] = threadIdx.x < kDotBlocks ? p[threadIdx.x] : 0.0;
  __syncthreads();
  for (int s = 256; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// w -= sum_i h[i] V_i  (h on the device)
__global__ void k_adj_gs_sub(const double* __restrict__ V, size_t ldv, int nv, const double* __restrict__ h,
                             double* __restrict__ w, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = w[i];
  for (int c = 0; c < nv; ++c) acc -= h[c] * V[ldv * c + i];
  w[i] = acc;
}

// y += sum_i c[i] V_i (c on the device)
__global__ void k_adj_combine(const double* __restrict__ V, size_t ldv, int nv, const double* __restrict__ c,
                              double* __restrict__ y, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = y[i];
  for (int m = 0; m < nv; ++m) acc += c[m] * V[ldv * m + i];
  y[i] = acc;
}

// y = a x + b y with a and b on the host, or a = *ad (device) when ad != null
__global__ void k_adj_axpby(double a, const double* __restrict__ ad, const double* __restrict__ x, double b,
                            double* __restrict__ y, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double aa = ad ? *ad : a;
  y[i] = aa * x[i] + b * y[i];
}

__global__ void k_adj_to_f32(const double* __restrict__ x, float* __restrict__ y, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}

// transposed implicit operator for the preconditioner (line relaxation or LU-SGS sweeps of
// P^T), whose blocks at (j,k) are btc^T, bjp(j-1,k)^T (lower j), bjm(j+1,k)^T (upper j), bkp(j,k-1)^T,
// bkm(j,k+1)^T
// The pseudo-time term of interior points, I / (dj dtau) (ref/step.f:419-437), is replaced by
// I / (dj dtau_p) of the preconditioner's own step.
__global__ void k_adj_transpose_lhs(const double* __restrict__ btc, const double* __restrict__ bjm,
                                    const double* __restrict__ bjp, const double* __restrict__ bkm,
                                    const double* __restrict__ bkp, const double* __restrict__ dj, double dtau,
                                    double dtau_p, int jmax, int kmax, double* __restrict__ tbtc,
                                    double* __restrict__ tbjm, double* __restrict__ tbjp, double* __restrict__ tbkm,
                                    double* __restrict__ tbkp) {
  int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t N = (size_t)jmax * kmax, id = ix(j, k, jmax);
  const bool interior = j > 0 && j < jmax - 1 && k > 0 && k < kmax - 1;
  const double shift = interior ? 1. / (dj[id] * dtau_p) - 1. / (dj[id] * dtau) : 0.0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      size_t e = N * (size_t)(r + 3 * c), et = N * (size_t)(c + 3 * r);
      tbtc[id + e] = btc[id + et] + (r == c ? shift : 0.0);
      tbjm[id + e] = j > 0 ? bjp[ix(j - 1, k, jmax) + et] : 0.0;
      tbjp[id + e] = j < jmax - 1 ? bjm[ix(j + 1, k, jmax) + et] : 0.0;
      tbkm[id + e] = k > 0 ? bkp[ix(j, k - 1, jmax) + et] : 0.0;
      tbkp[id + e] = k < kmax - 1 ? bkm[ix(j, k + 1, jmax) + et] : 0.0;
    }
}

// ------------------------------------------------------------------------------------------
// host side
#define ADJ_CK(x)                                                                   \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess) {                                                        \
      snprintf(err, sizeof err, "%s: %s", #x, cudaGetErrorString(e_));               \
      return SMAC_ERR_CUDA;                                                         \
    }                                                                               \
  } while (0)

struct AdjointImpl {
  AdjointCtx C;
  size_t N, n3;
  AdjointOptions opt;
  int m = 0;  // GMRES restart length of the allocated Krylov basis
  double *jac = nullptr, *fc = nullptr, *gq[2] = {nullptr, nullptr};
  double *tb = nullptr, *tprm = nullptr, *fj = nullptr, *fk = nullptr;  // P^T; its j and k line factors
  double *V = nullptr, *Z = nullptr, *w = nullptr, *tmp = nullptr, *lam[2] = {nullptr, nullptr};
  double *pr = nullptr, *rr = nullptr, *dz = nullptr, *zw = nullptr;
  F32Ops o32{};                 // FP32 copy of P^T and its line factors (SMAC_ADJ_PREC_LINES_F32)
  double *part = nullptr, *dsc = nullptr;
  double *drtxy = nullptr, *ddj = nullptr, *ddx = nullptr, *ddy = nullptr, *fb = nullptr;
  bool prepared = false, solved[2] = {false, false};
  double cl = 0.0, cd = 0.0;
  char err[256];
  std::vector<void*> allocs;

  // dsc: [0, kAdjMaxRestart + 2) dot products of the Gram-Schmidt passes, then 8 scalars
  static constexpr size_t tail() { return (size_t)kAdjMaxRestart + 2; }
  dim3 grid2() const { return dim3((unsigned)((C.jmax + 127) / 128), (unsigned)C.kmax); }
  unsigned blocks1(size_t n) const { return (unsigned)((n + 255) / 256); }

  AdjArgs args() const {
    AdjArgs a;
    a.P.jmax = C.jmax; a.P.kmax = C.kmax; a.P.N = N;
    a.P.beta = C.beta; a.P.cdis = C.cdis; a.P.vnu = C.vnu; a.P.pout = C.pout; a.P.pi = C.pi;
    a.P.ivis = C.ivis; a.P.visc64 = C.visc64;
    a.bc = C.d_bc;
    a.q = C.q; a.rtxy = C.rtxy; a.dj = C.dj; a.x = C.x; a.y = C.y;
    a.uinf = C.ca; a.vinf = C.sa; a.clift = C.clift;
    return a;
  }
  ForceGeo fgeo() const { return ForceGeo{C.jmax, N, C.vnu, C.ivis}; }
  unsigned wake_blocks() const {
    int pts = 0;
    for (int r = 0; r < C.bc->nwake; ++r) pts += C.bc->jt_e[r] - C.bc->jt_b[r] + 1;
    return (unsigned)((3 * pts + 127) / 128 > 0 ? (3 * pts + 127) / 128 : 1);
  }

  int alloc(double** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(double));
    if (e != cudaSuccess) {
      snprintf(err, sizeof err, "cudaMalloc of %zu bytes: %s", n * sizeof(double), cudaGetErrorString(e));
      return SMAC_ERR_NOMEM;
    }
    allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, n * sizeof(double), C.st) == cudaSuccess ? SMAC_OK : SMAC_ERR_CUDA;
  }

  int allocf(float** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(float));
    if (e != cudaSuccess) {
      snprintf(err, sizeof err, "cudaMalloc of %zu bytes: %s", n * sizeof(float), cudaGetErrorString(e));
      return SMAC_ERR_NOMEM;
    }
    allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, n * sizeof(float), C.st) == cudaSuccess ? SMAC_OK : SMAC_ERR_CUDA;
  }

  int init(const AdjointCtx& c) {
    C = c;
    N = (size_t)C.jmax * C.kmax;
    n3 = 3 * N;
    int rc;
    if ((rc = alloc(&jac, (size_t)kAdjSlots * 9 * N))) return rc;
    if ((rc = alloc(&fc, n3))) return rc;
    if ((rc = alloc(&gq[0], n3)) || (rc = alloc(&gq[1], n3))) return rc;
    if ((rc = alloc(&tb, 45 * N)) || (rc = alloc(&tprm, 9 * N))) return rc;
    if ((rc = alloc(&fj, 18 * N)) || (rc = alloc(&fk, 18 * N))) return rc;
    if ((rc = alloc(&Z, n3)) || (rc = alloc(&w, n3)) || (rc = alloc(&tmp, n3))) return rc;
    if ((rc = alloc(&lam[0], n3)) || (rc = alloc(&lam[1], n3))) return rc;
    if ((rc = alloc(&pr, n3)) || (rc = alloc(&rr, n3)) || (rc = alloc(&dz, n3)) || (rc = alloc(&zw, n3))) return rc;
    if ((rc = alloc(&part, (size_t)kDotBlocks * (kAdjMaxRestart + 2)))) return rc;
    if ((rc = alloc(&dsc, (size_t)2 * (kAdjMaxRestart + 2) + 16))) return rc;
    if ((rc = alloc(&drtxy, 6 * N)) || (rc = alloc(&ddj, N)) || (rc = alloc(&ddx, N)) || (rc = alloc(&ddy, N)))
      return rc;
    if ((rc = alloc(&fb, n3))) return rc;
    float** fs[] = {&o32.btc_j, &o32.btc_k, &o32.bjm, &o32.bjp_f, &o32.bjp_o, &o32.bkm, &o32.bkp, &o32.bkp_o};
    for (float** f : fs)
      if ((rc = allocf(f, 9 * N))) return rc;
    if ((rc = allocf(&o32.s, n3)) || (rc = allocf(&o32.dq, n3)) || (rc = allocf(&o32.work, n3))) return rc;
    return SMAC_OK;
  }

  // the Krylov basis for the restart length of the options
  int ensure_basis() {
    if (V && m == opt.restart) return SMAC_OK;
    if (V) {
      for (auto it = allocs.begin(); it != allocs.end(); ++it)
        if (*it == (void*)V) { allocs.erase(it); break; }
      cudaFree(V);
      V = nullptr;
    }
    m = opt.restart;
    return alloc(&V, (size_t)(m + 1) * n3);
  }

  void release() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
  }

  // dots of nv vectors V_0.. (stride ldv) with x, into dsc[0..nv-1] (device)
  void mdot(const double* Vs, size_t ldv, int nv, const double* x, double* out) {
    k_adj_mdot_partial<<<dim3(kDotBlocks, nv), kDotThreads, 0, C.st>>>(Vs, ldv, x, n3, part);
    k_adj_mdot_final<<<nv, 512, 0, C.st>>>(part, out);
  }
  double dot_host(const double* a, const double* b) {
    mdot(a, 0, 1, b, dsc);
    double h = 0.0;
    cudaMemcpyAsync(&h, dsc, sizeof(double), cudaMemcpyDeviceToHost, C.st);
    cudaStreamSynchronize(C.st);
    return h;
  }

  // y = A v or A^T v
  void apply(int transpose, const double* v, double* y) {
    if (!transpose) {
      k_adj_jv<<<grid2(), 128, 0, C.st>>>(jac, C.jmax, C.kmax, v, y);
      k_adj_wake<<<wake_blocks(), 128, 0, C.st>>>(C.d_bc, C.jmax, N, 0, v, y);
      // + fc (gcl . v)
      mdot(gq[0], 0, 1, v, dsc + tail() + 4);
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(0.0, dsc + tail() + 4, fc, 1.0, y, n3);
    } else {
      k_adj_jtv<<<grid2(), 128, 0, C.st>>>(jac, C.jmax, C.kmax, v, y);
      k_adj_wake<<<wake_blocks(), 128, 0, C.st>>>(C.d_bc, C.jmax, N, 1, v, y);
      // + gcl (fc . w)
      mdot(fc, 0, 1, v, dsc + tail() + 4);
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(0.0, dsc + tail() + 4, gq[0], 1.0, y, n3);
    }
  }

  // z = -M v, M an approximate inverse of P^T (P ~ -dF/dq, the implicit operator): the LU-SGS
  // sweeps of P^T, or zebra line relaxation of P^T (block-tridiagonal solves along transposed
  // j lines, then k lines)
  void m_apply(const double* v, double* z) {
    if (opt.preconditioner == SMAC_ADJ_PREC_LUSGS) {
      cudaMemcpyAsync(pr, v, n3 * sizeof(double), cudaMemcpyDeviceToDevice, C.st);
      launch_lusgs3(C.jmax, C.kmax, tb, tb + 9 * N, tb + 18 * N, tb + 27 * N, tb + 36 * N, tprm, pr, z, C.st);
    } else if (opt.preconditioner == SMAC_ADJ_PREC_LINES_F32) {
      k_adj_to_f32<<<blocks1(n3), 256, 0, C.st>>>(v, o32.s, n3);
      launch_fill_f32(o32.dq, 0.f, n3, C.st);
      ZebraArgs<float, float> a;
      a.jmax = C.jmax; a.kmax = C.kmax; a.N = N; a.s = o32.s; a.dq = o32.dq; a.work = o32.work; a.underr = 1.f;
      a.btc = o32.btc_j; a.am = o32.bjm; a.cp = o32.bjp_f; a.om = o32.bkm; a.op = o32.bkp_o;
      for (int i = 0; i < opt.sweeps; ++i) {
        launch_zebra(0, a, i & 1, C.st, C.lpw[0]);
        launch_zebra(0, a, 1 - (i & 1), C.st, C.lpw[0]);
      }
      a.btc = o32.btc_k; a.am = o32.bkm; a.cp = o32.bkp; a.om = o32.bjm; a.op = o32.bjp_o;
      for (int i = 0; i < opt.sweeps; ++i) {
        launch_zebra(1, a, i & 1, C.st, C.lpw[1]);
        launch_zebra(1, a, 1 - (i & 1), C.st, C.lpw[1]);
      }
      launch_dq_to_f64(o32.dq, z, n3, C.st);
    } else {
      launch_fill(z, 0.0, n3, C.st);
      ZebraArgs<double, double> a;
      a.jmax = C.jmax; a.kmax = C.kmax; a.N = N; a.s = v; a.dq = z; a.work = zw; a.underr = 1.0;
      a.btc = fj; a.am = tb + 9 * N; a.cp = fj + 9 * N; a.om = tb + 27 * N; a.op = tb + 36 * N;
      for (int i = 0; i < opt.sweeps; ++i) {
        launch_zebra(0, a, i & 1, C.st, C.lpw[0]);
        launch_zebra(0, a, 1 - (i & 1), C.st, C.lpw[0]);
      }
      a.btc = fk; a.am = tb + 27 * N; a.cp = fk + 9 * N; a.om = tb + 9 * N; a.op = tb + 18 * N;
      for (int i = 0; i < opt.sweeps; ++i) {
        launch_zebra(1, a, i & 1, C.st, C.lpw[1]);
        launch_zebra(1, a, 1 - (i & 1), C.st, C.lpw[1]);
      }
    }
    k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(0.0, nullptr, z, -1.0, z, n3);
  }

  // z = K v: opt.inner steps of the stationary iteration z += -M (v - A^T z) from z = 0
  void precond(const double* v, double* z) {
    m_apply(v, z);
    for (int i = 1; i < opt.inner; ++i) {
      apply(1, z, rr);
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(1.0, nullptr, v, -1.0, rr, n3);
      m_apply(rr, dz);
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(1.0, nullptr, dz, 1.0, z, n3);
    }
  }

  int prepare() {
    AdjArgs a = args();
    const dim3 g = grid2();
    ADJ_CK(cudaMemsetAsync(jac, 0, (size_t)kAdjSlots * 9 * N * sizeof(double), C.st));
    for (int color = 0; color < 13; ++color)
      for (int comp = 0; comp < 3; ++comp) k_adj_jac_color<<<g, 128, 0, C.st>>>(a, color, comp, jac);
    k_adj_dclift<<<g, 128, 0, C.st>>>(a, fc);
    // force gradients and values
    ADJ_CK(cudaMemsetAsync(gq[0], 0, n3 * sizeof(double), C.st));
    ADJ_CK(cudaMemsetAsync(gq[1], 0, n3 * sizeof(double), C.st));
    GeoPlain ga{C.rtxy, C.dj, C.x, C.y, N};
    for (int wl = 0; wl < C.bc->nwall; ++wl) {
      const int dir = C.bc->wjk[wl] == 1 ? 1 : 2;
      const int npts = dir == 2 ? C.bc->wj2[wl] - C.bc->wj1[wl] + 1 : C.bc->wk2[wl] - C.bc->wk1[wl] + 1;
      k_adj_force_grad<<<(npts * 9 + 127) / 128, 128, 0, C.st>>>(fgeo(), C.d_bc, wl, C.q, ga, C.ca, C.sa, gq[0],
                                                                gq[1]);
    }
    k_adj_force_dir<GeoPlain><<<1, 256, 0, C.st>>>(fgeo(), C.d_bc, C.q, ga, C.ca, 0.0, C.sa, 0.0, dsc);
    double h[4];
    ADJ_CK(cudaMemcpyAsync(h, dsc, sizeof h, cudaMemcpyDeviceToHost, C.st));
    // transposed implicit operator (the blocks were assembled at this state by the caller)
    const double dtp = opt.dtau > 0.0 ? opt.dtau : 40.0 * C.dtau;
    k_adj_transpose_lhs<<<g, 128, 0, C.st>>>(C.btc, C.bjm, C.bjp, C.bkm, C.bkp, C.dj, C.dtau, dtp, C.jmax, C.kmax,
                                            tb, tb + 9 * N, tb + 18 * N, tb + 27 * N, tb + 36 * N);
    // block-tridiagonal factors of the transposed j and k lines (centre block and upper block,
    // factored in place on copies)
    ADJ_CK(cudaMemcpyAsync(fj, tb, 9 * N * sizeof(double), cudaMemcpyDeviceToDevice, C.st));
    ADJ_CK(cudaMemcpyAsync(fj + 9 * N, tb + 18 * N, 9 * N * sizeof(double), cudaMemcpyDeviceToDevice, C.st));
    ADJ_CK(cudaMemcpyAsync(fk, tb, 9 * N * sizeof(double), cudaMemcpyDeviceToDevice, C.st));
    ADJ_CK(cudaMemcpyAsync(fk + 9 * N, tb + 36 * N, 9 * N * sizeof(double), cudaMemcpyDeviceToDevice, C.st));
    launch_btlu(0, tb + 9 * N, fj, fj + 9 * N, C.jmax, C.kmax, C.st, false);
    launch_btlu(1, tb + 27 * N, fk, fk + 9 * N, C.jmax, C.kmax, C.st, false);
    // the same in FP32 (the rhs plane of the conversion is scratch here)
    launch_to_f32(tb, tb + 9 * N, tb + 18 * N, tb + 27 * N, tb + 36 * N, fc, o32, N, C.st);
    launch_btlu_f32(0, o32.bjm, o32.btc_j, o32.bjp_f, C.jmax, C.kmax, C.st);
    launch_btlu_f32(1, o32.bkm, o32.btc_k, o32.bkp, C.jmax, C.kmax, C.st);
    ADJ_CK(cudaStreamSynchronize(C.st));
    ADJ_CK(cudaGetLastError());
    cl = h[0];
    cd = h[2];
    prepared = true;
    solved[0] = solved[1] = false;
    return SMAC_OK;
  }

  // restarted GMRES, right-preconditioned, on A^T lambda = -dJ/dq
  int solve(int obj, double rtol, int max_iter, int* iters, double* rel) {
    if (!prepared) { snprintf(err, sizeof err, "adjoint: prepare first"); return SMAC_ERR_ARG; }
    int rc = ensure_basis();
    if (rc) return rc;
    double* b = w;  // -dJ/dq
    k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(-1.0, nullptr, gq[obj], 0.0, b, n3);
    double* x = lam[obj];
    ADJ_CK(cudaMemsetAsync(x, 0, n3 * sizeof(double), C.st));
    const double bnorm = sqrt(dot_host(b, b));
    if (!(bnorm > 0.0)) {
      snprintf(err, sizeof err, "adjoint: zero objective gradient");
      return SMAC_ERR_ARG;
    }
    // r0 = b (x = 0), kept in V_0 before normalisation
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hcol(m + 1), y(m);
    int it = 0;
    double res = bnorm;
    double* r = V;
    cudaMemcpyAsync(r, b, n3 * sizeof(double), cudaMemcpyDeviceToDevice, C.st);
    while (it < max_iter) {
      double beta = sqrt(dot_host(r, r));
      res = beta;
      if (beta / bnorm <= rtol) break;
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(1.0 / beta, nullptr, r, 0.0, V, n3);
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int jdone = 0;
      for (int j = 0; j < m && it < max_iter; ++j, ++it) {
        double* vj = V + (size_t)j * n3;
        double* vn = V + (size_t)(j + 1) * n3;
        precond(vj, Z);
        apply(1, Z, vn);
        // classical Gram-Schmidt, twice
        for (int pass = 0; pass < 2; ++pass) {
          mdot(V, n3, j + 1, vn, dsc);
          k_adj_gs_sub<<<blocks1(n3), 256, 0, C.st>>>(V, n3, j + 1, dsc, vn, n3);
          double hh[kAdjMaxRestart + 1];
          ADJ_CK(cudaMemcpyAsync(hh, dsc, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, C.st));
          ADJ_CK(cudaStreamSynchronize(C.st));
          for (int i = 0; i <= j; ++i) hcol[i] = (pass == 0 ? 0.0 : hcol[i]) + hh[i];
        }
        double hn = sqrt(dot_host(vn, vn));
        hcol[j + 1] = hn;
        if (hn > 0.0) k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(1.0 / hn, nullptr, vn, 0.0, vn, n3);
        // Givens rotations
        for (int i = 0; i < j; ++i) {
          double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
          hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
          hcol[i] = t;
        }
        double den = sqrt(hcol[j] * hcol[j] + hcol[j + 1] * hcol[j + 1]);
        cs[j] = den > 0.0 ? hcol[j] / den : 1.0;
        sn[j] = den > 0.0 ? hcol[j + 1] / den : 0.0;
        hcol[j] = den;
        hcol[j + 1] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hcol[i];
        jdone = j + 1;
        res = fabs(g[j + 1]);
        if (res / bnorm <= rtol || hn == 0.0) { ++it; break; }
      }
      // y = R^-1 g, x += K (V y)
      for (int i = jdone - 1; i >= 0; --i) {
        double s = g[i];
        for (int l = i + 1; l < jdone; ++l) s -= H[(size_t)i * m + l] * y[l];
        y[i] = s / H[(size_t)i * m + i];
      }
      ADJ_CK(cudaMemcpyAsync(dsc, y.data(), sizeof(double) * jdone, cudaMemcpyHostToDevice, C.st));
      ADJ_CK(cudaMemsetAsync(tmp, 0, n3 * sizeof(double), C.st));
      k_adj_combine<<<blocks1(n3), 256, 0, C.st>>>(V, n3, jdone, dsc, tmp, n3);
      ADJ_CK(cudaStreamSynchronize(C.st));
      precond(tmp, Z);
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(1.0, nullptr, Z, 1.0, x, n3);
      // true residual r = b - A^T x
      apply(1, x, r);
      k_adj_axpby<<<blocks1(n3), 256, 0, C.st>>>(1.0, nullptr, b, -1.0, r, n3);
      res = sqrt(dot_host(r, r));
      if (res / bnorm <= rtol) break;
    }
    ADJ_CK(cudaStreamSynchronize(C.st));
    ADJ_CK(cudaGetLastError());
    if (iters) *iters = it;
    if (rel) *rel = res / bnorm;
    solved[obj] = true;
    return SMAC_OK;
  }

  // dJ/db for design variables given as grid motions (host arrays ndv x N) and alpha changes
  int gradient(int obj, int ndv, const double* dxdb, const double* dydb, const double* dalpha, double* grad) {
    if (!solved[obj]) { snprintf(err, sizeof err, "adjoint: solve this objective first"); return SMAC_ERR_ARG; }
    AdjArgs a = args();
    const dim3 g = grid2();
    const double rad = C.pi / 180.;
    double fcl = dot_host(fc, lam[obj]);  // lambda . dF/dclift
    for (int i = 0; i < ndv; ++i) {
      if (dxdb) ADJ_CK(cudaMemcpyAsync(ddx, dxdb + (size_t)i * N, N * sizeof(double), cudaMemcpyHostToDevice, C.st));
      else ADJ_CK(cudaMemsetAsync(ddx, 0, N * sizeof(double), C.st));
      if (dydb) ADJ_CK(cudaMemcpyAsync(ddy, dydb + (size_t)i * N, N * sizeof(double), cudaMemcpyHostToDevice, C.st));
      else ADJ_CK(cudaMemsetAsync(ddy, 0, N * sizeof(double), C.st));
      double da = dalpha ? dalpha[i] : 0.0;
      // d(cos(alpha pi/180)), d(sin(alpha pi/180)) per unit of the design variable
      double dca = -C.sa * rad * da, dsa = C.ca * rad * da;
      k_adj_metric_dir<<<g, 128, 0, C.st>>>(C.x, C.y, ddx, ddy, C.jmax, C.kmax, drtxy, ddj);
      k_adj_design<<<g, 128, 0, C.st>>>(a, drtxy, ddj, ddx, ddy, dca, dsa, fb);
      GeoDir gd{C.rtxy, C.dj, C.x, C.y, drtxy, ddj, ddx, ddy, N};
      k_adj_force_dir<GeoDir><<<1, 256, 0, C.st>>>(fgeo(), C.d_bc, C.q, gd, C.ca, dca, C.sa, dsa, dsc + tail());
      double h[4];
      ADJ_CK(cudaMemcpyAsync(h, dsc + tail(), sizeof h, cudaMemcpyDeviceToHost, C.st));
      double lfb = dot_host(lam[obj], fb);  // synchronises
      double jb = obj == 0 ? h[1] : h[3], clb = h[1];
      grad[i] = jb + lfb + fcl * clb;
    }
    ADJ_CK(cudaGetLastError());
    return SMAC_OK;
  }

  int residual(double* F_host) {
    AdjArgs a = args();
    k_adj_residual<<<grid2(), 128, 0, C.st>>>(a, tmp);
    k_adj_wake_residual<<<1, 1, 0, C.st>>>(C.d_bc, C.q, C.jmax, N, tmp);
    ADJ_CK(cudaMemcpyAsync(F_host, tmp, n3 * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    ADJ_CK(cudaStreamSynchronize(C.st));
    ADJ_CK(cudaGetLastError());
    return SMAC_OK;
  }

  int jacvec(int transpose, const double* v_host, double* y_host) {
    if (!prepared) { snprintf(err, sizeof err, "adjoint: prepare first"); return SMAC_ERR_ARG; }
    ADJ_CK(cudaMemcpyAsync(Z, v_host, n3 * sizeof(double), cudaMemcpyHostToDevice, C.st));
    apply(transpose, Z, tmp);
    ADJ_CK(cudaMemcpyAsync(y_host, tmp, n3 * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    ADJ_CK(cudaStreamSynchronize(C.st));
    ADJ_CK(cudaGetLastError());
    return SMAC_OK;
  }

  int get(int what, double* host) {
    const double* src = nullptr;
    size_t n = n3;
    if (what == SMAC_ADJ_LAMBDA_CL) src = lam[0];
    else if (what == SMAC_ADJ_LAMBDA_CD) src = lam[1];
    else if (what == SMAC_ADJ_DCL_DQ) src = gq[0];
    else if (what == SMAC_ADJ_DCD_DQ) src = gq[1];
    else if (what == SMAC_ADJ_DF_DCLIFT) src = fc;
    else if (what == SMAC_ADJ_JACOBIAN) { src = jac; n = (size_t)kAdjSlots * 9 * N; }
    if (!src) { snprintf(err, sizeof err, "adjoint: unknown field %d", what); return SMAC_ERR_ARG; }
    ADJ_CK(cudaMemcpyAsync(host, src, n * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    ADJ_CK(cudaStreamSynchronize(C.st));
    return SMAC_OK;
  }
};

AdjointImpl* adjoint_new(const AdjointCtx& c, const AdjointOptions& o, int* rc, char* msg, size_t msglen) {
  AdjointImpl* A = new AdjointImpl();
  A->opt = o;
  *rc = A->init(c);
  if (*rc) {
    snprintf(msg, msglen, "%s", A->err);
    A->release();
    delete A;
    return nullptr;
  }
  return A;
}
void adjoint_free(AdjointImpl* A) {
  if (!A) return;
  A->release();
  delete A;
}
void adjoint_update(AdjointImpl* A, const AdjointCtx& c, const AdjointOptions& o) {
  A->C = c;
  A->opt = o;
}
const char* adjoint_error(AdjointImpl* A) { return A->err; }
int adjoint_prepare(AdjointImpl* A) { return A->prepare(); }
int adjoint_solve(AdjointImpl* A, int obj, double rtol, int max_iter, int* iters, double* rel) {
  return A->solve(obj, rtol, max_iter, iters, rel);
}
int adjoint_gradient(AdjointImpl* A, int obj, int ndv, const double* dx, const double* dy, const double* da,
                     double* grad) {
  return A->gradient(obj, ndv, dx, dy, da, grad);
}
int adjoint_residual(AdjointImpl* A, double* F) { return A->residual(F); }
int adjoint_jacvec(AdjointImpl* A, int transpose, const double* v, double* y) { return A->jacvec(transpose, v, y); }
int adjoint_get(AdjointImpl* A, int what, double* host) { return A->get(what, host); }
void adjoint_forces(AdjointImpl* A, double* cl, double* cd) {
  *cl = A->cl;
  *cd = A->cd;
}

}  // namespace smac
