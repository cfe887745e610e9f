// smac_assemble.cu -- residual and implicit-operator assembly of the pseudo-time iteration.
//
// FP64 kernels that evaluate, operation for operation, what the reference computes in
//   metric            ref/metric.f:49-278
//   conup + fluxj3/k3 ref/conup.f:49-478, ref/flux.f:160-372
//   viscterms         ref/visc.f:50-160 (REAL*4 scratch kept: vf, udif, vdif are float)
//   blank + identity  ref/step.f:386-437
//   bcmain + BCs      ref/bc.f:60-224, 1080-1869
//   resid             ref/step.f:613-756 (isamax first-index rule, ref/blas.f:48-83)
//   SA model          ref/tursa.f:66-1372 (vortsa, curvature, tsafill, tsaibt, tsabc, tsaupd)
//   update            ref/step.f:804-809
//   force / fmk       ref/geom.f:135-213, ref/fm.f:156-324, ref/smac2d.f:1706-1825
//
// Work decomposition: the convective terms run as two line-tiled passes (j lines, then k
// lines) whose CTAs stage the face Jacobians A+/A-, the flux differences and the physical
// fluxes of a tile in shared memory; every face is evaluated once.  The k pass also adds the
// viscous terms and the pseudo-time identity, so an interior point's blocks and residual are
// written in two passes.  Boundary points (all blanked by the reference) are written by the
// BC kernel, which applies the bcmain.dat regions in file order.
#include <math.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

namespace smac {

// ------------------------------------------------------------------------------------------
// metric (ref/metric.f:49-278)
__global__ void k_metric(const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ rtxy,
                         double* __restrict__ dj, int jmax, int kmax) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t N = (size_t)jmax * kmax;
#define X(a, b) x[ix(a, b, jmax)]
#define Y(a, b) y[ix(a, b, jmax)]
  double xj, yj, xk, yk;
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
#undef X
#undef Y
  size_t id = ix(j, k, jmax);
  double rdj = xj * yk - xk * yj;
  dj[id] = 1. / rdj;
  rtxy[id + N * 0] = 0.0;   // (1,1) d xi / d tau
  rtxy[id + N * 1] = 0.0;   // (2,1) d eta / d tau
  rtxy[id + N * 2] = yk;    // (1,2)
  rtxy[id + N * 4] = -xk;   // (1,3)
  rtxy[id + N * 3] = -yj;   // (2,2)
  rtxy[id + N * 5] = xj;    // (2,3)
}

// ic (ref/geom.f:88-131): free stream, then no-slip on the walls
__global__ void k_ic(double* __restrict__ q, size_t N, double ca, double sa) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  q[i] = 1.0;
  q[i + N] = ca;
  q[i + 2 * N] = sa;
}

__global__ void k_ic_walls(double* __restrict__ q, const BCTable* __restrict__ bc, int jmax, int kmax) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t N = (size_t)jmax * kmax;
  for (int w = 0; w < bc->nwall; ++w)
    if (j >= bc->wj1[w] && j <= bc->wj2[w] && k >= bc->wk1[w] && k <= bc->wk2[w]) {
      q[ix(j, k, jmax) + N] = 0.0;
      q[ix(j, k, jmax) + 2 * N] = 0.0;
    }
}

// ------------------------------------------------------------------------------------------
// convective terms: conup (ref/conup.f:49-478) with the third-order fluxes of fluxj3/fluxk3
// (ref/flux.f:160-372).  DIR 0: lines of varying j at fixed k; DIR 1: lines of varying k at
// fixed j.  A CTA handles W lines x TP output points.
template <int DIR>
struct LineGeom {
  int n, nlines;  // line length, number of lines
  int jmax;
  size_t N;
  __device__ __forceinline__ size_t at(int line, int pos) const {
    return DIR == 0 ? ix(pos, line, jmax) : ix(line, pos, jmax);
  }
};

// per-face record in shared memory
struct FaceRec {
  double ap[9], am[9], dfp[3], dfm[3];
};

__device__ __forceinline__ void face_split(double rt, double rx, double ry, double q2, double q3, double beta,
                                           double* ap, double* am) {
  // ref/conup.f:127-185, entry (row r, col c) at [r + 3c]
  double cvel = rx * q2 + ry * q3;
  double t = cvel + 0.5 * rt;
  double cc = sqrt(t * t + beta * (rx * rx + ry * ry));
  double eig = cvel + rt;
  double eig1 = 0.5 * (eig + fabs(eig));
  double eig2 = cvel + rt * 0.5 + cc;
  double x21 = -(ry * eig1 / (cc * cc - 0.25 * rt * rt));
  double x31 = rx * eig1 / (cc * cc - 0.25 * rt * rt);
  double x12 = 0.5 * eig2 / cc;
  double x22 = 0.5 * eig2 * (q2 * eig2 + beta * rx) / (beta * cc * (cc - 0.5 * rt));
  double x32 = 0.5 * eig2 * (q3 * eig2 + beta * ry) / (beta * cc * (cc - 0.5 * rt));
  double xi11 = ry * q2 - rx * q3;
  double xi12 = -(q3 * (cvel + rt)) - ry * beta;
  double xi13 = q2 * (cvel + rt) + rx * beta;
  double xi21 = cc - cvel - 0.5 * rt;
  double xi22 = rx * beta;
  double xi23 = ry * beta;
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

// the point matrix "at" of ref/conup.f:89-105 for metric direction d (0 xi, 1 eta)
__device__ __forceinline__ void point_at(const double* __restrict__ rtxy, const double* __restrict__ q, size_t id,
                                         size_t N, int d, double beta, double* at) {
  double r1 = rtxy[id + N * (0 + d)], r2 = rtxy[id + N * (2 + d)], r3 = rtxy[id + N * (4 + d)];
  double q2 = q[id + N], q3 = q[id + 2 * N];
  double cvel = r1 + r2 * q2 + r3 * q3;
  at[0] = r1;
  at[1] = r2;
  at[2] = r3;
  at[3] = r2 * beta;
  at[4] = r2 * q2 + cvel;
  at[5] = r2 * q3;
  at[6] = r3 * beta;
  at[7] = r3 * q2;
  at[8] = r3 * q3 + cvel;
}

template <int DIR, int W, int TP>
__global__ void __launch_bounds__(256) k_conup(AssembleArgs a) {
  constexpr int NF = TP + 3;  // faces p0-2 .. p0+TP
  constexpr int NV = TP + 2;  // fv at points p0-1 .. p0+TP
  constexpr int NFL = TP + 1; // fluxes at faces p0-1 .. p0+TP-1
  extern __shared__ double smem[];
  FaceRec* fr = reinterpret_cast<FaceRec*>(smem);                  // [W][NF]
  double* fv = smem + (size_t)W * NF * (sizeof(FaceRec) / 8);       // [W][NV][3]
  double* fl = fv + (size_t)W * NV * 3;                              // [W][NFL][3]

  const int jmax = a.jmax, kmax = a.kmax;
  const size_t N = a.N;
  const int n = DIR == 0 ? jmax : kmax;
  const int nlines = DIR == 0 ? kmax : jmax;
  const int d = DIR;  // metric row used by this direction
  const double beta = a.beta, cdis = a.cdis;
  const int line0 = 1 + blockIdx.y * W;  // interior lines only
  const int p0 = 1 + blockIdx.x * TP;    // interior output points p0 .. p0+TP-1
  auto gid = [&](int line, int pos) -> size_t { return DIR == 0 ? ix(pos, line, jmax) : ix(line, pos, jmax); };

  // 1. faces: split Jacobians and flux differences
  for (int it = threadIdx.x; it < W * NF; it += blockDim.x) {
    int w, fi;
    if (DIR == 0) { w = it / NF; fi = it % NF; } else { w = it % W; fi = it / W; }
    int line = line0 + w;
    int f = p0 - 2 + fi;
    FaceRec& R = fr[w * NF + fi];
    if (line > nlines - 2 || f < 0 || f > n - 2) {
      for (int e = 0; e < 3; ++e) { R.dfp[e] = 0.0; R.dfm[e] = 0.0; }
      continue;
    }
    size_t i0 = gid(line, f), i1 = gid(line, f + 1);
    double rt = 0.5 * (a.rtxy[i1 + N * (0 + d)] + a.rtxy[i0 + N * (0 + d)]);
    double rx = 0.5 * (a.rtxy[i1 + N * (2 + d)] + a.rtxy[i0 + N * (2 + d)]);
    double ry = 0.5 * (a.rtxy[i1 + N * (4 + d)] + a.rtxy[i0 + N * (4 + d)]);
    double q2 = 0.5 * (a.q[i1 + N] + a.q[i0 + N]);
    double q3 = 0.5 * (a.q[i1 + 2 * N] + a.q[i0 + 2 * N]);
    face_split(rt, rx, ry, q2, q3, beta, R.ap, R.am);
    double dq1 = a.q[i1] - a.q[i0];
    double dq2 = a.q[i1 + N] - a.q[i0 + N];
    double dq3 = a.q[i1 + 2 * N] - a.q[i0 + 2 * N];
    for (int r = 0; r < 3; ++r) {
      R.dfp[r] = R.ap[r] * dq1 + R.ap[r + 3] * dq2 + R.ap[r + 6] * dq3;
      R.dfm[r] = R.am[r] * dq1 + R.am[r + 3] * dq2 + R.am[r + 6] * dq3;
    }
  }
  // physical fluxes at points
  for (int it = threadIdx.x; it < W * NV; it += blockDim.x) {
    int w, vi;
    if (DIR == 0) { w = it / NV; vi = it % NV; } else { w = it % W; vi = it / W; }
    int line = line0 + w;
    int p = p0 - 1 + vi;
    double* F = fv + (w * NV + vi) * 3;
    if (line > nlines - 2 || p < 0 || p > n - 1) continue;
    size_t id = gid(line, p);
    double r1 = a.rtxy[id + N * (0 + d)], r2 = a.rtxy[id + N * (2 + d)], r3 = a.rtxy[id + N * (4 + d)];
    double q1 = a.q[id], q2 = a.q[id + N], q3 = a.q[id + 2 * N];
    double cvel = r1 + r2 * q2 + r3 * q3;
    F[0] = r1 * q1 + beta * (cvel - r1);
    F[1] = q2 * cvel + r2 * q1;
    F[2] = q3 * cvel + r3 * q1;
  }
  __syncthreads();
  // 2. numerical fluxes at faces p0-1 .. p0+TP-1 (ref/flux.f:213-256)
  const double r6 = FLIT(1.0f / 6.0f);
  for (int it = threadIdx.x; it < W * NFL; it += blockDim.x) {
    int w, li;
    if (DIR == 0) { w = it / NFL; li = it % NFL; } else { w = it % W; li = it / W; }
    int line = line0 + w;
    int f = p0 - 1 + li;
    if (line > nlines - 2 || f < 0 || f > n - 2) continue;
    int fm = f - 1 > 0 ? f - 1 : 0;
    int fp = f + 1 < n - 1 ? f + 1 : n - 1;   // n-1 is not a face: its differences are zero
    int fpp = f + 2 < n - 1 ? f + 2 : n - 1;
    double cp = (double)(fpp - fp);
    double cm = (double)(f - fm);
    const FaceRec& Rm = fr[w * NF + (fm - (p0 - 2))];
    const FaceRec& R0 = fr[w * NF + (f - (p0 - 2))];
    const FaceRec& Rp = fr[w * NF + (fp - (p0 - 2))];
    const double* F0 = fv + (w * NV + (f - (p0 - 1))) * 3;
    const double* F1 = fv + (w * NV + (f + 1 - (p0 - 1))) * 3;
    double* out = fl + (w * NFL + li) * 3;
    for (int m = 0; m < 3; ++m) {
      double fmv = (R0.dfp[m] + R0.dfm[m] - Rp.dfp[m] - Rp.dfm[m]) * r6;
      double fpv = (Rm.dfp[m] + Rm.dfm[m] - R0.dfp[m] - R0.dfm[m]) * r6;
      double f3 = (Rm.dfp[m] - R0.dfp[m] + R0.dfm[m] - Rp.dfm[m]) * r6;
      out[m] = 0.5 * (F1[m] + F0[m]) + cdis * (cp * cm * f3 + cm * (1. - cp) * fpv + cp * (1. - cm) * fmv);
    }
  }
  __syncthreads();
  // 3. point outputs
  for (int it = threadIdx.x; it < W * TP; it += blockDim.x) {
    int w, pi;
    if (DIR == 0) { w = it / TP; pi = it % TP; } else { w = it % W; pi = it / W; }
    int line = line0 + w;
    int p = p0 + pi;
    if (line > nlines - 2 || p > n - 2) continue;
    size_t id = gid(line, p);
    double atm[9], atp[9];
    point_at(a.rtxy, a.q, gid(line, p - 1), N, d, beta, atm);
    point_at(a.rtxy, a.q, gid(line, p + 1), N, d, beta, atp);
    const FaceRec& Fm = fr[w * NF + (p - 1 - (p0 - 2))];  // face p-1/2
    const FaceRec& Fp = fr[w * NF + (p - (p0 - 2))];      // face p+1/2
    const double* flm = fl + (w * NFL + (p - 1 - (p0 - 1))) * 3;
    const double* flp = fl + (w * NFL + (p - (p0 - 1))) * 3;
    double* Bm = DIR == 0 ? a.bjm : a.bkm;
    double* Bp = DIR == 0 ? a.bjp : a.bkp;
    double bt[9];
    for (int e = 0; e < 9; ++e) {
      Bm[id + N * e] = 0.5 * (-atm[e] - Fm.ap[e] + Fm.am[e]);
      Bp[id + N * e] = 0.5 * (atp[e] - Fp.ap[e] + Fp.am[e]);
      double c = 0.5 * (Fp.ap[e] + Fm.ap[e] - Fp.am[e] - Fm.am[e]);
      if (DIR == 0) bt[e] = c;
      else bt[e] = a.btc[id + N * e] + c;
    }
    double sv[3];
    for (int m = 0; m < 3; ++m) {
      if (DIR == 0) sv[m] = -(flp[m] - flm[m]);
      else sv[m] = a.s[id + N * m] - (flp[m] - flm[m]);
    }
    if (DIR == 1) {
      const int j = line, k = p;
      if (a.ivis) {
        // viscous terms, j then k direction (ref/visc.f:94-140)
        const double vnu = a.vnu;
        double bjm22 = a.bjm[id + N * 4], bjm33 = a.bjm[id + N * 8];
        double bjp22 = a.bjp[id + N * 4], bjp33 = a.bjp[id + N * 8];
        double bkm22 = Bm[id + N * 4], bkm33 = Bm[id + N * 8];
        double bkp22 = Bp[id + N * 4], bkp33 = Bp[id + N * 8];
        for (int vd = 0; vd < 2; ++vd) {
          size_t im = vd == 0 ? ix(j - 1, k, jmax) : ix(j, k - 1, jmax);
          size_t ip = vd == 0 ? ix(j + 1, k, jmax) : ix(j, k + 1, jmax);
          // faces (m, id) and (id, p)
          double djvm = 0.5 * (a.dj[im] * vnu + a.dj[id] * vnu);
          double djvp = 0.5 * (a.dj[id] * vnu + a.dj[ip] * vnu);
          double rxm = 0.5 * (a.rtxy[im + N * (2 + vd)] + a.rtxy[id + N * (2 + vd)]);
          double rym = 0.5 * (a.rtxy[im + N * (4 + vd)] + a.rtxy[id + N * (4 + vd)]);
          double rxp = 0.5 * (a.rtxy[id + N * (2 + vd)] + a.rtxy[ip + N * (2 + vd)]);
          double ryp = 0.5 * (a.rtxy[id + N * (4 + vd)] + a.rtxy[ip + N * (4 + vd)]);
          float vfm = (float)(djvm * (rxm * rxm + rym * rym));
          float vfp = (float)(djvp * (rxp * rxp + ryp * ryp));
          float udm = (float)(a.q[id + N] - a.q[im + N]);
          float udp = (float)(a.q[ip + N] - a.q[id + N]);
          float vdm = (float)(a.q[id + 2 * N] - a.q[im + 2 * N]);
          float vdp = (float)(a.q[ip + 2 * N] - a.q[id + 2 * N]);
          double vm = (double)vfm, vp = (double)vfp;
          if (vd == 0) {
            bjm22 = bjm22 - vm; bjm33 = bjm33 - vm;
            bjp22 = bjp22 - vp; bjp33 = bjp33 - vp;
          } else {
            bkm22 = bkm22 - vm; bkm33 = bkm33 - vm;
            bkp22 = bkp22 - vp; bkp33 = bkp33 - vp;
          }
          bt[4] = bt[4] + vm + vp;
          bt[8] = bt[8] + vm + vp;
          if (a.visc64) {
            // FP64 viscous fluxes (labelled deviation: smooth in q and the grid)
            double wm = djvm * (rxm * rxm + rym * rym), wp = djvp * (rxp * rxp + ryp * ryp);
            double su = wp * (a.q[ip + N] - a.q[id + N]) - wm * (a.q[id + N] - a.q[im + N]);
            double sw = wp * (a.q[ip + 2 * N] - a.q[id + 2 * N]) - wm * (a.q[id + 2 * N] - a.q[im + 2 * N]);
            sv[1] = sv[1] + su;
            sv[2] = sv[2] + sw;
          } else {
            float su = __fsub_rn(__fmul_rn(vfp, udp), __fmul_rn(vfm, udm));
            float sw = __fsub_rn(__fmul_rn(vfp, vdp), __fmul_rn(vfm, vdm));
            sv[1] = sv[1] + (double)su;
            sv[2] = sv[2] + (double)sw;
          }
        }
        a.bjm[id + N * 4] = bjm22; a.bjm[id + N * 8] = bjm33;
        a.bjp[id + N * 4] = bjp22; a.bjp[id + N * 8] = bjp33;
        Bm[id + N * 4] = bkm22; Bm[id + N * 8] = bkm33;
        Bp[id + N * 4] = bkp22; Bp[id + N * 8] = bkp33;
      }
      // pseudo-time identity for interior points (ref/step.f:419-437, fib = 1)
      double fib = 1.0;
      double rdjdtau = fib / (a.dj[id] * a.dtau) + 1. - fib;
      bt[0] = bt[0] + rdjdtau;
      bt[4] = bt[4] + rdjdtau;
      bt[8] = bt[8] + rdjdtau;
    }
    for (int e = 0; e < 9; ++e) a.btc[id + N * e] = bt[e];
    for (int m = 0; m < 3; ++m) a.s[id + N * m] = sv[m];
  }
}

// the tile shapes of each direction (W lines x TP points, threads per CTA); entry 0 is the
// default, the others are the autotuner's choices.  The shape changes only which CTA computes
// a point, not how: every shape gives the same bits.
struct ConupShape { int W, TP, threads; };
static const ConupShape kConupShapes[2][kConupNumShapes] = {
    {{kConupW0, kConupTP0, 128}, {2, 64, 128}, {1, 256, 256}, {4, 32, 128}},
    {{kConupW1, kConupTP1, 256}, {16, 16, 256}, {8, 32, 256}, {4, 32, 128}}};

static size_t conup_smem_of(int W, int TP) {
  return sizeof(double) * ((size_t)W * (TP + 3) * (sizeof(FaceRec) / 8) + (size_t)W * (TP + 2) * 3 +
                           (size_t)W * (TP + 1) * 3);
}

template <int DIR, int W, int TP>
static void conup_one(const AssembleArgs& a, int threads, cudaStream_t st) {
  static bool attr = false;
  const size_t smem = conup_smem_of(W, TP);
  if (!attr) {
    cudaFuncSetAttribute(k_conup<DIR, W, TP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  const int n = DIR == 0 ? a.jmax : a.kmax, nl = DIR == 0 ? a.kmax : a.jmax;
  dim3 g((n - 2 + TP - 1) / TP, (nl - 2 + W - 1) / W);
  ++g_kernel_launches;
  k_conup<DIR, W, TP><<<g, threads, smem, st>>>(a);
}

void launch_conup_dir(const AssembleArgs& a, int dir, int shape, cudaStream_t st) {
  if (shape < 0 || shape >= kConupNumShapes) shape = 0;
  const int t = kConupShapes[dir][shape].threads;
  if (dir == 0) {
    switch (shape) {
      case 1: conup_one<0, 2, 64>(a, t, st); break;
      case 2: conup_one<0, 1, 256>(a, t, st); break;
      case 3: conup_one<0, 4, 32>(a, t, st); break;
      default: conup_one<0, kConupW0, kConupTP0>(a, t, st);
    }
  } else {
    switch (shape) {
      case 1: conup_one<1, 16, 16>(a, t, st); break;
      case 2: conup_one<1, 8, 32>(a, t, st); break;
      case 3: conup_one<1, 4, 32>(a, t, st); break;
      default: conup_one<1, kConupW1, kConupTP1>(a, t, st);
    }
  }
}

void launch_conup(const AssembleArgs& a, cudaStream_t st, int shape_j, int shape_k) {
  launch_conup_dir(a, 0, shape_j, st);
  launch_conup_dir(a, 1, shape_k, st);
}

// ------------------------------------------------------------------------------------------
// boundary points: blanked to zero with a unit diagonal (ref/step.f:386-437, fib = 0), then the
// bcmain.dat regions in file order (ref/bc.f:60-224)
__global__ void k_bc(AssembleArgs a, const BCTable* __restrict__ bc, const DevScalars* __restrict__ sc) {
  const int jmax = a.jmax, kmax = a.kmax;
  const size_t N = a.N;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int nper = 2 * jmax + 2 * (kmax - 2);
  if (t >= nper) return;
  int j, k;
  if (t < jmax) { j = t; k = 0; }
  else if (t < 2 * jmax) { j = t - jmax; k = kmax - 1; }
  else if (t < 2 * jmax + kmax - 2) { j = 0; k = 1 + (t - 2 * jmax); }
  else { j = jmax - 1; k = 1 + (t - 2 * jmax - (kmax - 2)); }
  size_t id = ix(j, k, jmax);
  double bt[9], bjm[9], bjp[9], bkm[9], bkp[9], s[3];
  for (int e = 0; e < 9; ++e) { bt[e] = 0.0; bjm[e] = 0.0; bjp[e] = 0.0; bkm[e] = 0.0; bkp[e] = 0.0; }
  for (int m = 0; m < 3; ++m) s[m] = 0.0;
  bt[0] = 1.0; bt[4] = 1.0; bt[8] = 1.0;
  const double* q = a.q;
  const double beta = a.beta, pi = a.pi, clift = sc->clift;
  for (int r = 0; r < bc->nreg; ++r) {
    const BCRegion& R = bc->reg[r];
    if (j < R.jb || j > R.je || k < R.kb || k > R.ke) continue;
    int dir = R.jkbc;  // 1: j const (line along k), 2: k const
    bool lo = dir == 1 ? (j == 0) : (k == 0);
    size_t inb = dir == 1 ? ix(lo ? j + 1 : j - 1, k, jmax) : ix(j, lo ? k + 1 : k - 1, jmax);
    double* Bp = dir == 1 ? bjp : bkp;
    double* Bm = dir == 1 ? bjm : bkm;
    if (R.ibcval == 0) {
      // bcnoslj / bcnoslk, flow at +1 (ref/bc.f:1093-1104, 1147-1158)
      size_t ip = dir == 1 ? ix(j + 1, k, jmax) : ix(j, k + 1, jmax);
      bt[0] = 1.0; bt[4] = 1.0; bt[8] = 1.0;
      Bp[0] = -1.0;
      s[0] = q[ip] - q[id];
      s[1] = -q[id + N];
      s[2] = -q[id + 2 * N];
    } else if (R.ibcval == 25) {
      // bccgridj / bccgridk (ref/bc.f:1202-1276, 1351-1431)
      double uinf = a.uinf, vinf = a.vinf;
      double dx = a.x[id] - 0.25;
      double dy = a.y[id];
      double ucirc = clift * dy / (4. * pi * (dx * dx + dy * dy));
      double vcirc = -(clift * dx / (4. * pi * (dx * dx + dy * dy)));
      bt[4] = 1.0;
      bt[8] = 1.0;
      s[1] = uinf + ucirc - q[id + N];
      s[2] = vinf + vcirc - q[id + 2 * N];
      int jk = dir - 1;  // metric row
      double r2 = a.rtxy[id + N * (2 + jk)], r3 = a.rtxy[id + N * (4 + jk)];
      double qq = r2 * q[id + N] + r3 * q[id + 2 * N];
      double cc = sqrt(qq * qq + beta * (r2 * r2 + r3 * r3));
      if (lo) {
        Bp[0] = r2 * r2 + r3 * r3;
        Bp[3] = r2 * (qq - cc);
        Bp[6] = r3 * (qq - cc);
        bt[0] = -Bp[0]; bt[3] = -Bp[3]; bt[6] = -Bp[6];
        double dq1 = q[inb] - q[id], dq2 = q[inb + N] - q[id + N], dq3 = q[inb + 2 * N] - q[id + 2 * N];
        s[0] = -Bp[0] * dq1 - Bp[3] * dq2 - Bp[6] * dq3;
      } else {
        Bm[0] = -(r2 * r2 + r3 * r3);
        Bm[3] = -(r2 * (qq + cc));
        Bm[6] = -(r3 * (qq + cc));
        bt[0] = -Bm[0]; bt[3] = -Bm[3]; bt[6] = -Bm[6];
        double dq1 = q[id] - q[inb], dq2 = q[id + N] - q[inb + N], dq3 = q[id + 2 * N] - q[inb + 2 * N];
        s[0] = Bm[0] * dq1 + Bm[3] * dq2 + Bm[6] * dq3;
      }
    } else if (R.ibcval == 31) {
      // bcoutj / bcoutk: velocity extrapolated, static pressure pout (ref/bc.f:1622-1669, 1813-1858)
      bt[4] = 1.0;
      bt[8] = 1.0;
      if (lo) { Bp[4] = -1.0; Bp[8] = -1.0; }
      else { Bm[4] = -1.0; Bm[8] = -1.0; }
      s[1] = q[inb + N] - q[id + N];
      s[2] = q[inb + 2 * N] - q[id + 2 * N];
      bt[0] = 1.0;
      s[0] = a.pout - q[id];
    }
  }
  for (int e = 0; e < 9; ++e) {
    a.btc[id + N * e] = bt[e];
    a.bjm[id + N * e] = bjm[e];
    a.bjp[id + N * e] = bjp[e];
    a.bkm[id + N * e] = bkm[e];
    a.bkp[id + N * e] = bkp[e];
  }
  for (int m = 0; m < 3; ++m) a.s[id + N * m] = s[m];
}

void launch_bc(const AssembleArgs& a, const BCTable* bc, const DevScalars* sc, cudaStream_t st) {
  int nper = 2 * a.jmax + 2 * (a.kmax - 2);
  ++g_kernel_launches;
  k_bc<<<(nper + 127) / 128, 128, 0, st>>>(a, bc, sc);
}

// ------------------------------------------------------------------------------------------
// resid (ref/step.f:613-756): resmax = max |s*dj| with the first-index rule over the flat
// (j, k, n) order; divmax from equation 1; plus the L2 norm of s (ref/step.f:513-519).
struct MaxRec {
  double v;      // |value|
  long long i;   // flat index
};
__device__ __forceinline__ MaxRec better(MaxRec a, MaxRec b) {
  if (b.v > a.v) return b;
  if (b.v == a.v && b.i < a.i) return b;
  return a;
}

__global__ void k_resid_partial(const double* __restrict__ s, const double* __restrict__ dj, size_t N,
                                MaxRec* __restrict__ pmax, MaxRec* __restrict__ pdiv, double* __restrict__ psum) {
  MaxRec bm{-1.0, 0x7fffffffffffffffLL}, bd{-1.0, 0x7fffffffffffffffLL};
  double sum = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
    double d = dj[i];
    for (int n = 0; n < 3; ++n) {
      double sv = s[i + N * n];
      double v = sv * d;
      MaxRec c{fabs(v), (long long)(i + N * n)};
      bm = better(bm, c);
      if (n == 0) bd = better(bd, c);
      sum += sv * sv;
    }
  }
  __shared__ MaxRec sm[256], sd[256];
  __shared__ double ss[256];
  sm[threadIdx.x] = bm; sd[threadIdx.x] = bd; ss[threadIdx.x] = sum;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sm[threadIdx.x] = better(sm[threadIdx.x], sm[threadIdx.x + o]);
      sd[threadIdx.x] = better(sd[threadIdx.x], sd[threadIdx.x + o]);
      ss[threadIdx.x] += ss[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    pmax[blockIdx.x] = sm[0];
    pdiv[blockIdx.x] = sd[0];
    psum[blockIdx.x] = ss[0];
  }
}

__global__ void k_resid_final(const double* __restrict__ s, const double* __restrict__ dj, int jmax, size_t N,
                              const MaxRec* __restrict__ pmax, const MaxRec* __restrict__ pdiv,
                              const double* __restrict__ psum, int nparts, double beta, DevScalars* __restrict__ sc) {
  __shared__ MaxRec sm[256], sd[256];
  __shared__ double ss[256];
  MaxRec bm{-1.0, 0x7fffffffffffffffLL}, bd{-1.0, 0x7fffffffffffffffLL};
  double sum = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    bm = better(bm, pmax[i]);
    bd = better(bd, pdiv[i]);
    sum += psum[i];
  }
  sm[threadIdx.x] = bm; sd[threadIdx.x] = bd; ss[threadIdx.x] = sum;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sm[threadIdx.x] = better(sm[threadIdx.x], sm[threadIdx.x + o]);
      sd[threadIdx.x] = better(sd[threadIdx.x], sd[threadIdx.x + o]);
      ss[threadIdx.x] += ss[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    long long im = sm[0].i;
    int n = (int)(im / (long long)N);
    long long p = im - (long long)n * (long long)N;
    sc->neq = n + 1;
    sc->kres = (int)(p / jmax) + 1;
    sc->jres = (int)(p % jmax) + 1;
    double v = s[im] * dj[p];
    sc->resmax = fabs(v);
    if (sc->nt == 1) {
      sc->resmax0 = sc->resmax;
      if (sc->resmax0 < 1.) sc->resmax0 = 1.0;
    }
    long long id = sd[0].i;
    sc->divmax = fabs(s[id] * dj[id] / beta);
    sc->rhsnorm = sqrt(ss[0]);
    if (!isfinite(sc->resmax) || !isfinite(sc->rhsnorm)) sc->status = SMAC_ERR_NONFINITE;
  }
}

void launch_resid(const double* s, const double* dj, int jmax, size_t N, void* scratch, double beta,
                  DevScalars* sc, cudaStream_t st) {
  const int parts = kResidParts;
  MaxRec* pmax = reinterpret_cast<MaxRec*>(scratch);
  MaxRec* pdiv = pmax + parts;
  double* psum = reinterpret_cast<double*>(pdiv + parts);
  ++g_kernel_launches;
  k_resid_partial<<<parts, 256, 0, st>>>(s, dj, N, pmax, pdiv, psum);
  ++g_kernel_launches;
  k_resid_final<<<1, 256, 0, st>>>(s, dj, jmax, N, pmax, pdiv, psum, parts, beta, sc);
}

size_t resid_scratch_bytes() { return (size_t)kResidParts * (2 * sizeof(MaxRec) + sizeof(double)); }

// ------------------------------------------------------------------------------------------
// update (ref/step.f:804-809)
__global__ void k_update(double* __restrict__ q, const double* __restrict__ dq, size_t n3) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n3) q[i] = q[i] + dq[i];
}

// iteration prologue: counter and per-iteration reductions
__global__ void k_iter_begin(DevScalars* sc) {
  sc->nt = sc->nt + 1;
  sc->turres = 0.0;
  sc->wait_status = 0;
}

// ------------------------------------------------------------------------------------------
// forces (ref/smac2d.f:1706-1825, ref/geom.f:135-213, ref/fm.f:156-324).  The wall stresses and
// every face's contributions (with the reference's expressions) are evaluated in parallel; one
// thread only adds them up in the reference's order, so that Cl, which feeds the next
// iteration's far-field vortex, is bit-reproducible.  Per wall point kForceRec doubles: the
// stresses t11, t22, t12 at the point, then the face (point, point+1) terms fx, fy, the
// pressure moment, gx, gy, xave*gy, yave*gx.
__global__ void k_force_terms(ForceArgs f, const BCTable* __restrict__ bc, double* __restrict__ terms, int w) {
  const int jmax = f.jmax;
  const size_t N = f.N;
  int dir = bc->wjk[w] == 1 ? 1 : 2;  // 1: j const wall (line along k)
  int at = dir == 2 ? bc->wk1[w] : bc->wj1[w];
  int b = dir == 2 ? bc->wj1[w] : bc->wk1[w];
  int e = dir == 2 ? bc->wj2[w] : bc->wk2[w];
  int d = dir == 2 ? 1 : 0;  // metric row normal to the wall
  int npts = e - b + 1;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  auto gid = [&](int pos) -> size_t { return dir == 2 ? ix(pos, at, jmax) : ix(at, pos, jmax); };
  auto gin = [&](int pos, int off) -> size_t { return dir == 2 ? ix(pos, at + off, jmax) : ix(at + off, pos, jmax); };
  int pos = b + i;
  size_t id = gid(pos);
  // wall stresses at the point
  double ueta = 0.5 * (-(3. * f.q[id + N]) + 4. * f.q[gin(pos, 1) + N] - f.q[gin(pos, 2) + N]);
  double veta = 0.5 * (-(3. * f.q[id + 2 * N]) + 4. * f.q[gin(pos, 1) + 2 * N] - f.q[gin(pos, 2) + 2 * N]);
  double r2 = f.rtxy[id + N * (2 + d)], r3 = f.rtxy[id + N * (4 + d)];
  double* T = terms + (size_t)kForceRec * i;
  T[0] = 2. * f.vnu * r2 * f.dj[id] * ueta;          // t11
  T[1] = 2. * f.vnu * r3 * f.dj[id] * veta;          // t22
  T[2] = f.vnu * (r3 * ueta + r2 * veta) * f.dj[id]; // t12
}

// face terms of wall w with the reference's expressions (ref/fm.f:156-324)
__global__ void k_force_faces(ForceArgs f, const BCTable* __restrict__ bc, double* __restrict__ terms, int w) {
  const int jmax = f.jmax;
  const size_t N = f.N;
  const double x0 = 0.25, y0 = 0.0;
  int dir = bc->wjk[w] == 1 ? 1 : 2;
  int at = dir == 2 ? bc->wk1[w] : bc->wj1[w];
  int b = dir == 2 ? bc->wj1[w] : bc->wk1[w];
  int e = dir == 2 ? bc->wj2[w] : bc->wk2[w];
  int d = dir == 2 ? 1 : 0;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= e - b) return;
  auto gid = [&](int pos) -> size_t { return dir == 2 ? ix(pos, at, jmax) : ix(at, pos, jmax); };
  int pos = b + i;
  size_t i0 = gid(pos), i1 = gid(pos + 1);
  double* S = terms + (size_t)kForceRec * i + 3;
  double pave = 0.5 * (f.q[i1] + f.q[i0]);
  double da1 = 0.5 * (f.rtxy[i1 + N * (2 + d)] + f.rtxy[i0 + N * (2 + d)]);
  double da2 = 0.5 * (f.rtxy[i1 + N * (4 + d)] + f.rtxy[i0 + N * (4 + d)]);
  double xave = 0.5 * (f.x[i1] + f.x[i0]) - x0;
  double yave = 0.5 * (f.y[i1] + f.y[i0]) - y0;
  double fx = pave * da1;
  double fy = pave * da2;
  S[0] = fx;
  S[1] = fy;
  S[2] = xave * fy - yave * fx;
  if (f.ivis) {
    const double* T0 = terms + (size_t)kForceRec * i;
    const double* T1 = T0 + kForceRec;
    double t11ave = 0.5 * (T1[0] + T0[0]);
    double t22ave = 0.5 * (T1[1] + T0[1]);
    double t12ave = 0.5 * (T1[2] + T0[2]);
    double t21ave = t12ave;
    double gx = t11ave * da1 + t12ave * da2;
    double gy = t21ave * da1 + t22ave * da2;
    S[3] = gx;
    S[4] = gy;
    S[5] = xave * gy;
    S[6] = yave * gx;
  }
}

__global__ void k_force_sum(ForceArgs f, const BCTable* __restrict__ bc, double* __restrict__ terms,
                            DevScalars* __restrict__ sc) {
  // The three running sums are independent chains of dependent FP64 adds (one FP64 instruction
  // per warp every 64 cycles): each is carried by lane 0 of its own warp, in the reference's
  // order (walls in order, pressure faces, then viscous faces).
  __shared__ double res[5];
  const int chain = threadIdx.x >> 5;  // 0: x forces, 1: y forces, 2: moment
  if ((threadIdx.x & 31) == 0 && chain < 3) {
    double p = 0.0, v = 0.0, mom = 0.0;
    for (int w = 0; w < bc->nwall; ++w) {
      int dir = bc->wjk[w] == 1 ? 1 : 2;
      int b = dir == 2 ? bc->wj1[w] : bc->wk1[w];
      int e = dir == 2 ? bc->wj2[w] : bc->wk2[w];
      const double* T = terms + (size_t)kForceRec * f.term_off[w];
      const int nseg = e - b;
      p = 0.0;
      v = 0.0;
      if (chain < 2) {
        for (int i = 0; i < nseg; ++i) p = p - T[(size_t)kForceRec * i + 3 + chain];
        if (f.ivis)
          for (int i = 0; i < nseg; ++i) v = v + T[(size_t)kForceRec * i + 6 + chain];
      } else {
        for (int i = 0; i < nseg; ++i) mom = mom - T[(size_t)kForceRec * i + 5];
        if (f.ivis)
          for (int i = 0; i < nseg; ++i) {
            const double* S = T + (size_t)kForceRec * i + 3;
            mom = mom + S[5] - S[6];
          }
      }
    }
    // forces of the last wall (the reference zeroes them per wall), moments of all walls
    if (chain < 2) { res[chain] = p; res[2 + chain] = v; }
    else res[4] = mom;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double chord = 1.0;
    double fxp = res[0], fyp = res[1], fxs = res[2], fys = res[3], fmom = res[4];
    double ca = f.ca, sa = f.sa;
    sc->cd = (2. * (fxp + fxs) * ca + 2. * (fyp + fys) * sa) / chord;
    sc->cl = (2. * (fyp + fys) * ca - 2. * (fxp + fxs) * sa) / chord;
    sc->cm = -(2. * fmom / (chord * chord));
    sc->cdp = (2. * fxp * ca + 2. * fyp * sa) / chord;
    sc->clp = (2. * fyp * ca - 2. * fxp * sa) / chord;
    sc->clift = sc->cl;
  }
}

// the same integrals as k_force_sum, accumulated by a fixed tree (deterministic, not the
// reference's sequential order)
__global__ void __launch_bounds__(1024) k_force_tree(ForceArgs f, const BCTable* __restrict__ bc,
                                                     const double* __restrict__ terms, DevScalars* __restrict__ sc) {
  const int jmax = f.jmax;
  const size_t N = f.N;
  const double x0 = 0.25, y0 = 0.0, chord = 1.0;
  __shared__ double red[5][1024];
  double acc[5] = {0, 0, 0, 0, 0};  // fxp, fyp, fxs, fys, fmom
  double fxp = 0, fyp = 0, fxs = 0, fys = 0, fmom = 0;
  for (int w = 0; w < bc->nwall; ++w) {
    int at = bc->wk1[w], b = bc->wj1[w], e = bc->wj2[w];
    const double* T = terms + (size_t)kForceRec * f.term_off[w];
    for (int k = 0; k < 5; ++k) acc[k] = 0.0;
    for (int pos = b + (int)threadIdx.x; pos <= e - 1; pos += blockDim.x) {
      size_t i0 = ix(pos, at, jmax), i1 = ix(pos + 1, at, jmax);
      double pave = 0.5 * (f.q[i1] + f.q[i0]);
      double da1 = 0.5 * (f.rtxy[i1 + N * 3] + f.rtxy[i0 + N * 3]);
      double da2 = 0.5 * (f.rtxy[i1 + N * 5] + f.rtxy[i0 + N * 5]);
      double xave = 0.5 * (f.x[i1] + f.x[i0]) - x0;
      double yave = 0.5 * (f.y[i1] + f.y[i0]) - y0;
      double fx = pave * da1, fy = pave * da2;
      acc[0] -= fx;
      acc[1] -= fy;
      acc[4] -= (xave * fy - yave * fx);
      if (f.ivis) {
        const double* T0 = T + (size_t)kForceRec * (pos - b);
        const double* T1 = T0 + kForceRec;
        double t11 = 0.5 * (T1[0] + T0[0]), t22 = 0.5 * (T1[1] + T0[1]), t12 = 0.5 * (T1[2] + T0[2]);
        double gx = t11 * da1 + t12 * da2, gy = t12 * da1 + t22 * da2;
        acc[2] += gx;
        acc[3] += gy;
        acc[4] += xave * gy - yave * gx;
      }
    }
    for (int k = 0; k < 5; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o)
        for (int k = 0; k < 5; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
      __syncthreads();
    }
    // forces of the last wall, moments of all walls (the reference's accumulation)
    fxp = red[0][0]; fyp = red[1][0]; fxs = red[2][0]; fys = red[3][0]; fmom += red[4][0];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double ca = f.ca, sa = f.sa;
    sc->cd = (2. * (fxp + fxs) * ca + 2. * (fyp + fys) * sa) / chord;
    sc->cl = (2. * (fyp + fys) * ca - 2. * (fxp + fxs) * sa) / chord;
    sc->cm = -(2. * fmom / (chord * chord));
    sc->cdp = (2. * fxp * ca + 2. * fyp * sa) / chord;
    sc->clp = (2. * fyp * ca - 2. * fxp * sa) / chord;
    sc->clift = sc->cl;
  }
}

void launch_forces_parallel(const ForceArgs& f, const BCTable* bc_dev, const BCTable& bc_host, double* terms,
                            DevScalars* sc, cudaStream_t st) {
  for (int w = 0; w < bc_host.nwall; ++w) {
    int npts = bc_host.wj2[w] - bc_host.wj1[w] + 1;
    ++g_kernel_launches;
    k_force_terms<<<(npts + 127) / 128, 128, 0, st>>>(f, bc_dev, terms + (size_t)kForceRec * f.term_off[w], w);
  }
  ++g_kernel_launches;
  k_force_tree<<<1, 1024, 0, st>>>(f, bc_dev, terms, sc);
}

void launch_forces(const ForceArgs& f, const BCTable* bc_dev, const BCTable& bc_host, double* terms,
                   DevScalars* sc, cudaStream_t st) {
  for (int w = 0; w < bc_host.nwall; ++w) {
    int npts = bc_host.wjk[w] == 1 ? bc_host.wk2[w] - bc_host.wk1[w] + 1 : bc_host.wj2[w] - bc_host.wj1[w] + 1;
    ++g_kernel_launches;
    k_force_terms<<<(npts + 127) / 128, 128, 0, st>>>(f, bc_dev, terms + (size_t)kForceRec * f.term_off[w], w);
  }
  for (int w = 0; w < bc_host.nwall; ++w) {
    int npts = bc_host.wjk[w] == 1 ? bc_host.wk2[w] - bc_host.wk1[w] + 1 : bc_host.wj2[w] - bc_host.wj1[w] + 1;
    if (npts < 2) continue;
    ++g_kernel_launches;
    k_force_faces<<<(npts - 1 + 127) / 128, 128, 0, st>>>(f, bc_dev, terms + (size_t)kForceRec * f.term_off[w], w);
  }
  ++g_kernel_launches;
  k_force_sum<<<1, 96, 0, st>>>(f, bc_dev, terms, sc);
}

// ------------------------------------------------------------------------------------------
// Spalart-Allmaras model (ref/tursa.f)

// wall distance (dfunsa, ref/tursa.f:351-433): exact min over the wall points
// The minimum over the wall points is taken on the squared distances and the square root once
// at the end: IEEE sqrt is correctly rounded and monotone, so the result is the reference's
// running minimum of the distances bit for bit, without a square root per pair.  The wall
// coordinates are staged through shared memory in tiles.
constexpr int kDfunTile = 256;
__global__ void __launch_bounds__(kDfunTile) k_dfunsa(const double* __restrict__ x, const double* __restrict__ y,
                                                      size_t N, const double* __restrict__ wx,
                                                      const double* __restrict__ wy, int nw,
                                                      double* __restrict__ smin) {
  __shared__ double swx[kDfunTile], swy[kDfunTile];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const bool live = i < N;
  const double xi = live ? x[i] : 0.0, yi = live ? y[i] : 0.0;
  double m2 = INFINITY;
  for (int p0 = 0; p0 < nw; p0 += kDfunTile) {
    const int cnt = nw - p0 < kDfunTile ? nw - p0 : kDfunTile;
    if ((int)threadIdx.x < cnt) { swx[threadIdx.x] = wx[p0 + threadIdx.x]; swy[threadIdx.x] = wy[p0 + threadIdx.x]; }
    __syncthreads();
    for (int t = 0; t < cnt; ++t) {
      double dxx = xi - swx[t], dyy = yi - swy[t];
      double d2 = dxx * dxx + dyy * dyy;
      m2 = d2 < m2 ? d2 : m2;
    }
    __syncthreads();
  }
  if (live) smin[i] = fminf90(FLIT(1.e6), sqrt(m2));
}

// tsaic (ref/tursa.f:1263-1323)
__global__ void k_tsaic(double* __restrict__ anut, const double* __restrict__ smin, int jmax, int kmax,
                        const BCTable* __restrict__ bc, double anutinf) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  size_t id = ix(j, k, jmax);
  double v = anutinf + 10.0 * exp(-10. * smin[id]);
  for (int w = 0; w < bc->nwall; ++w)
    if (j >= bc->wj1[w] && j <= bc->wj2[w] && k >= bc->wk1[w] && k <= bc->wk2[w]) v = 0.0;
  anut[id] = v;
}

// velocity differences of vortsa / curvature (ref/tursa.f:959-1012, 1044-1098)
__device__ __forceinline__ void sa_diffs(const double* __restrict__ q, int j, int k, int jmax, int kmax, size_t N,
                                         double& uj, double& vj, double& uk, double& vk) {
  const double* u = q + N;
  const double* v = q + 2 * N;
#define U(a, b) u[ix(a, b, jmax)]
#define V(a, b) v[ix(a, b, jmax)]
  if (j == 0) {
    uj = 0.5 * (-U(j + 2, k) + 4. * U(j + 1, k) - 3. * U(j, k));
    vj = 0.5 * (-V(j + 2, k) + 4. * V(j + 1, k) - 3. * V(j, k));
  } else if (j == jmax - 1) {
    uj = 0.5 * (3. * U(j, k) - 4. * U(j - 1, k) + U(j - 2, k));
    vj = 0.5 * (3. * V(j, k) - 4. * V(j - 1, k) + V(j - 2, k));
  } else {
    uj = 0.5 * (U(j + 1, k) - U(j - 1, k));
    vj = 0.5 * (V(j + 1, k) - V(j - 1, k));
  }
  if (k == 0) {
    uk = 0.5 * (-U(j, k + 2) + 4. * U(j, k + 1) - 3. * U(j, k));
    vk = 0.5 * (-V(j, k + 2) + 4. * V(j, k + 1) - 3. * V(j, k));
  } else if (k == kmax - 1) {
    uk = 0.5 * (3. * U(j, k) - 4. * U(j, k - 1) + U(j, k - 2));
    vk = 0.5 * (3. * V(j, k) - 4. * V(j, k - 1) + V(j, k - 2));
  } else {
    uk = 0.5 * (U(j, k + 1) - U(j, k - 1));
    vk = 0.5 * (V(j, k + 1) - V(j, k - 1));
  }
#undef U
#undef V
}

// point part of vortsa (|omega|) and of curvature (strain terms), all points
__global__ void k_sa_grad(SAArgs a) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  const int jmax = a.jmax, kmax = a.kmax;
  if (j >= jmax || k >= kmax) return;
  const size_t N = a.N;
  size_t id = ix(j, k, jmax);
  double uj, vj, uk, vk;
  sa_diffs(a.q, j, k, jmax, kmax, N, uj, vj, uk, vk);
  double djk = a.dj[id];
  double r12 = a.rtxy[id + N * 2], r22 = a.rtxy[id + N * 3], r13 = a.rtxy[id + N * 4], r23 = a.rtxy[id + N * 5];
  a.vort[id] = fabs(djk * (r12 * vj + r22 * vk - r13 * uj - r23 * uk));
  double ux = djk * (r12 * uj + r22 * uk);
  double vx = djk * (r12 * vj + r22 * vk);
  double uy = djk * (r13 * uj + r23 * uk);
  double vy = djk * (r13 * vj + r23 * vk);
  double rs = sqrt(2. * (p2(ux) + vx * uy + p2(vy)) + p2(uy) + p2(vx));
  if (vx - uy != 0.) rs = rs / fabs(vx - uy);
  a.crs[id] = rs;
  a.cs11[id] = (ux - vy) / 2;
  a.cs12[id] = (uy + vx) / 2;
  double fr = 2 * (vx - uy);
  double denom = (2. * (p2(ux) + vx * uy + p2(vy)) + p2(uy) + p2(vx)) * (p2(ux) + p2(vx) + p2(uy) + p2(vy));
  if (denom != 0.) fr = fr / denom;
  a.fr1[id] = fr;
}

// tsafill (loops 101 of curvature, 180, 190, 220, 230, 235, 260) + tsaibt, all points
__global__ void k_sa_fill(SAArgs a, const DevScalars* __restrict__ sc) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  const int jmax = a.jmax, kmax = a.kmax;
  if (j >= jmax || k >= kmax) return;
  const size_t N = a.N;
  size_t id = ix(j, k, jmax);
  if (j == 0 || j == jmax - 1 || k == 0 || k == kmax - 1) {
    // tsaibt with fib = 0
    a.sjm[id] = 0.0; a.sjp[id] = 0.0; a.skm[id] = 0.0; a.skp[id] = 0.0;
    a.stc[id] = 1.0; a.sf[id] = 0.0;
    return;
  }
  const double* q = a.q;
  const double* anut = a.anut;
  const double* dj = a.dj;
  const double* rt = a.rtxy;
  const double vnu = a.vnu;
  const double cb2 = a.cb2, sigma = a.sigma;
  // curvature loop 101 (ref/tursa.f:1128-1141)
  double fr1;
  {
    int km = k - 1, kp = k + 1;
    double dk = (double)(kp - km);
    double uu = (rt[id + N * 3] * q[id + N] + rt[id + N * 5] * q[id + 2 * N]) * dj[id];
    double vv = (rt[id + N * 2] * q[id + N] + rt[id + N * 4] * q[id + 2 * N]) * dj[id];
    double ds11dt = uu * (a.cs11[ix(j, kp, jmax)] - a.cs11[ix(j, km, jmax)]) / dk +
                    vv * (a.cs11[ix(j + 1, k, jmax)] - a.cs11[ix(j - 1, k, jmax)]) / 2;
    double ds12dt = uu * (a.cs12[ix(j, kp, jmax)] - a.cs12[ix(j, km, jmax)]) / dk +
                    vv * (a.cs12[ix(j + 1, k, jmax)] - a.cs12[ix(j - 1, k, jmax)]) / 2;
    double rtilde = (a.cs11[id] * ds12dt - a.cs12[id] * ds11dt) * a.fr1[id];
    double rs = a.crs[id];
    fr1 = (1 + a.cr1) * 2 * rs / (1 + rs) * (1 - a.cr3 * atan(a.cr2 * rtilde)) - a.cr1;
  }
  double an = anut[id];
  double djk = dj[id];
  double diff, conv, sjm, sjp, skm, skp, stc;
  // eta-eta viscous terms (loop 180)
  {
    size_t ip = ix(j, k + 1, jmax), im = ix(j, k - 1, jmax);
    double xy3p = .5 * (rt[id + N * 3] * djk + rt[ip + N * 3] * dj[ip]);
    double xy4p = .5 * (rt[id + N * 5] * djk + rt[ip + N * 5] * dj[ip]);
    double ttp = (xy3p * rt[id + N * 3] * djk + xy4p * rt[id + N * 5] * djk);
    double xy3m = .5 * (rt[id + N * 3] * djk + rt[im + N * 3] * dj[im]);
    double xy4m = .5 * (rt[id + N * 5] * djk + rt[im + N * 5] * dj[im]);
    double ttm = (xy3m * rt[id + N * 3] * djk + xy4m * rt[id + N * 5] * djk);
    double anp = anut[ip], anm = anut[im];
    double coef = -(cb2 * vnu * (1. + an) / sigma);
    diff = coef * (ttp * (anp - an) - ttm * (an - anm));
    skm = -(coef * ttm);
    skp = -(coef * ttp);
    stc = coef * (ttm + ttp);
    coef = vnu * (1. + cb2) / sigma;
    double vnup = 1.0 + 0.5 * (anp + an);
    double vnum = 1.0 + 0.5 * (anm + an);
    ttp = ttp * vnup;
    ttm = ttm * vnum;
    diff = diff + coef * (ttp * (anp - an) - ttm * (an - anm));
    skm = skm - coef * ttm;
    skp = skp - coef * ttp;
    stc = stc + coef * (ttm + ttp);
    // eta advection (loop 190)
    double uu = (rt[id + N * 3] * q[id + N] + rt[id + N * 5] * q[id + 2 * N]) * djk;
    double sgnu = copysign(1.0, uu);
    double app = .5 * (1. + sgnu);
    double apm = .5 * (1. - sgnu);
    conv = uu * (app * (an - anm) + apm * (anp - an));
    skm = skm - uu * app;
    stc = stc + uu * (app - apm);
    skp = skp + uu * apm;
  }
  // xi-xi viscous terms (loop 220) and xi advection (loop 230)
  {
    size_t ip = ix(j + 1, k, jmax), im = ix(j - 1, k, jmax);
    double xy1p = .5 * (rt[id + N * 2] * djk + rt[ip + N * 2] * dj[ip]);
    double xy2p = .5 * (rt[id + N * 4] * djk + rt[ip + N * 4] * dj[ip]);
    double ttp = (xy1p * rt[id + N * 2] * djk + xy2p * rt[id + N * 4] * djk);
    double xy1m = .5 * (rt[id + N * 2] * djk + rt[im + N * 2] * dj[im]);
    double xy2m = .5 * (rt[id + N * 4] * djk + rt[im + N * 4] * dj[im]);
    double ttm = (xy1m * rt[id + N * 2] * djk + xy2m * rt[id + N * 4] * djk);
    double anp = anut[ip], anm = anut[im];
    double coef = -(cb2 * vnu * (1. + an) / sigma);
    diff = diff + coef * (ttp * (anp - an) - ttm * (an - anm));
    sjm = -(coef * ttm);
    sjp = -(coef * ttp);
    stc = coef * (ttm + ttp) + stc;
    coef = vnu * (1. + cb2) / sigma;
    double vnup = 1.0 + 0.5 * (anp + an);
    double vnum = 1.0 + 0.5 * (anm + an);
    ttp = ttp * vnup;
    ttm = ttm * vnum;
    diff = diff + coef * (ttp * (anp - an) - ttm * (an - anm));
    sjm = sjm - coef * ttm;
    sjp = sjp - coef * ttp;
    stc = stc + coef * (ttm + ttp);
    double uu = (rt[id + N * 2] * q[id + N] + rt[id + N * 4] * q[id + 2 * N]) * djk;
    double sgnu = copysign(1.0, uu);
    double app = .5 * (1. + sgnu);
    double apm = .5 * (1. - sgnu);
    conv = conv + uu * (app * (an - anm) + apm * (anp - an));
    sjm = sjm - uu * app;
    stc = stc + uu * (app - apm);
    sjp = sjp + uu * apm;
  }
  double sf = -conv + diff;
  // production and destruction (loop 260)
  {
    const double ak = a.akarman, cb1 = a.cb1, cw1 = a.cw1, cw2 = a.cw2, cv1 = a.cv1, cv2 = a.cv2, ct4 = a.ct4;
    const double cw3r6 = a.cw3r6, ct3tmp = a.ct3tmp;
    const double ten = 10.0, epss = FLIT(1.e-12), epss2 = FLIT(0.00001), epss3 = FLIT(1.e-20);
    const double sixth = FLIT(1.0f / 6.0f);
    double fib = 1;
    double smin = (sc->nt == 1 || a.wall_fixed) ? a.smin[id] : 0.0;
    double sminlim = fmaxf90(smin, epss);
    double rkd2 = 1. / p2(ak * sminlim);
    double ss = a.vort[id];
    double chi = fmaxf90(an, epss2);
    double fv1 = p3(chi) / (p3(chi) + p3(cv1));
    double fv2 = 1 / p3(1. + chi / cv2);
    double fv3 = (1 + chi * fv1) / chi * (1 - fv2);
    double ft2 = ct3tmp * exp(-(ct4 * p2(chi)));
    double sst = fv3 * ss + vnu * chi * fv2 * rkd2;
    sst = fmaxf90(sst, epss3);
    double rr = fminf90(ten, vnu * an * rkd2 / sst);
    double gg = rr + cw2 * (p6(rr) - rr);
    double gg6 = p6(gg);
    double fg = (1. + cw3r6) / (gg6 + cw3r6);
    double fwdg = pow(fg, sixth);
    double fw = gg * fwdg;
    double pp = cb1 * sst * (1. - ft2);
    double dd = vnu * (cw1 * fw - cb1 * ft2 / p2(ak)) * an / p2(sminlim);
    double ft2p = -(2. * ct4 * ct3tmp * chi * exp(-(ct4 * p2(chi))));
    double fv1p = 3. * p2(chi) * p3(cv1) / p2(p3(chi) + p3(cv1));
    double fv2p = -(3 / cv2 / p4(1. + chi / cv2));
    double fv3p = ((fv1 + chi * fv1p) * (1 - fv2) - (1 + chi * fv1) * ((1 - fv2) / chi + fv2p)) / chi;
    double sstp = fv3p * ss + vnu * (chi * fv2p + fv2) * rkd2;
    double rrp = vnu * rkd2 * (sst - chi * sstp) / p2(sst);
    double ggp = rrp * (1. + cw2 * (6. * p5(rr) - 1.));
    double fwp = ggp * fwdg * (1. - gg6 / (gg6 + cw3r6));
    double ppp = cb1 * (sstp - ft2p * sst - ft2 * sstp);
    double ddp = vnu * (cw1 * fw - cb1 * ft2 / p2(ak) + (cw1 * fwp - cb1 * ft2p / p2(ak)) * chi) / p2(sminlim);
    double prod = fib * pp * an * fr1;
    double dest = fib * dd * an;
    sf = sf + prod - dest;
    double zero = 0.;
    double addpp = fmaxf90(dd - pp, zero);
    double addpppp = fmaxf90(ddp - ppp, zero);
    stc = stc + fib * addpp;
    stc = stc + fib * addpppp * an;
  }
  // tsaibt with fib = 1 (ref/tursa.f:1353-1367)
  {
    double fib = 1;
    a.sjm[id] = fib * sjm;
    a.sjp[id] = fib * sjp;
    a.skm[id] = fib * skm;
    a.skp[id] = fib * skp;
    a.stc[id] = fib * (stc + a.rterm) + (1. - fib);
    a.sf[id] = fib * sf;
  }
}

// tsabc (ref/tursa.f:1173-1259): outflow rows extrapolate the SA variable
__global__ void k_sa_bc(SAArgs a, const BCTable* __restrict__ bc) {
  const int jmax = a.jmax, kmax = a.kmax;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int nper = 2 * jmax + 2 * (kmax - 2);
  if (t >= nper) return;
  int j, k;
  if (t < jmax) { j = t; k = 0; }
  else if (t < 2 * jmax) { j = t - jmax; k = kmax - 1; }
  else if (t < 2 * jmax + kmax - 2) { j = 0; k = 1 + (t - 2 * jmax); }
  else { j = jmax - 1; k = 1 + (t - 2 * jmax - (kmax - 2)); }
  size_t id = ix(j, k, jmax);
  const double* an = a.anut;
  for (int r = 0; r < bc->nreg; ++r) {
    const BCRegion& R = bc->reg[r];
    int ib = R.ibcval;
    if (!(ib == 30 || ib == 31 || ib == 32 || ib == 33 || ib == 40)) continue;
    if (j < R.jb || j > R.je || k < R.kb || k > R.ke) continue;
    if (R.jkbc == 1 && R.jb == 0) {
      a.stc[id] = 1.0; a.sjp[id] = -1.0; a.sf[id] = an[ix(j + 1, k, jmax)] - an[id];
    } else if (R.jkbc == 1 && R.jb == jmax - 1) {
      a.stc[id] = 1.0; a.sjm[id] = -1.0; a.sf[id] = an[ix(j - 1, k, jmax)] - an[id];
    } else if (R.jkbc == 2 && R.kb == 0) {
      a.stc[id] = 1.0; a.skp[id] = -1.0; a.sf[id] = an[ix(j, k + 1, jmax)] - an[id];
    } else if (R.jkbc == 2 && R.kb == kmax - 1) {
      a.stc[id] = 1.0; a.skm[id] = -1.0; a.sf[id] = an[ix(j, k - 1, jmax)] - an[id];
    }
  }
}

// tsaupd (ref/tursa.f:314-347) and the eddy viscosity (ref/tursa.f:287-292)
__global__ void k_sa_update(double* __restrict__ anut, const double* __restrict__ ds, double* __restrict__ vnut,
                            size_t N, double cv1, double vnu, DevScalars* __restrict__ sc) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double dsm = 0.0;
  if (i < N) {
    double a = fmaxf90(0.0, anut[i] + ds[i]);
    anut[i] = a;
    dsm = fmaxf90(ds[i], 0.0);
    double chi = a;
    double fv1 = p3(chi) / (p3(chi) + p3(cv1));
    vnut[i] = fv1 * a * vnu;
  }
  // max over non-negative doubles == max over their bit patterns
  unsigned long long b = (unsigned long long)__double_as_longlong(dsm);
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long ob = __shfl_down_sync(0xffffffffu, b, o);
    b = ob > b ? ob : b;
  }
  if ((threadIdx.x & 31) == 0 && b) atomicMax(reinterpret_cast<unsigned long long*>(&sc->turres), b);
}

void launch_sa_assembly(const SAArgs& a, const BCTable* bc, const DevScalars* sc, cudaStream_t st) {
  dim3 g((a.jmax + 127) / 128, a.kmax);
  ++g_kernel_launches;
  k_sa_grad<<<g, 128, 0, st>>>(a);
  ++g_kernel_launches;
  k_sa_fill<<<g, 128, 0, st>>>(a, sc);
  int nper = 2 * a.jmax + 2 * (a.kmax - 2);
  ++g_kernel_launches;
  k_sa_bc<<<(nper + 127) / 128, 128, 0, st>>>(a, bc);
}

void launch_sa_update(double* anut, const double* ds, double* vnut, size_t N, double cv1, double vnu,
                      DevScalars* sc, cudaStream_t st) {
  ++g_kernel_launches;
  k_sa_update<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(anut, ds, vnut, N, cv1, vnu, sc);
}

void launch_metric(const double* x, const double* y, double* rtxy, double* dj, int jmax, int kmax,
                   cudaStream_t st) {
  dim3 g((jmax + 127) / 128, kmax);
  ++g_kernel_launches;
  k_metric<<<g, 128, 0, st>>>(x, y, rtxy, dj, jmax, kmax);
}

void launch_ic(double* q, int jmax, int kmax, double ca, double sa, const BCTable* bc, cudaStream_t st) {
  size_t N = (size_t)jmax * kmax;
  ++g_kernel_launches;
  k_ic<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(q, N, ca, sa);
  dim3 g((jmax + 127) / 128, kmax);
  ++g_kernel_launches;
  k_ic_walls<<<g, 128, 0, st>>>(q, bc, jmax, kmax);
}

void launch_dfunsa(const double* x, const double* y, size_t N, const double* wx, const double* wy, int nw,
                   double* smin, cudaStream_t st) {
  ++g_kernel_launches;
  k_dfunsa<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(x, y, N, wx, wy, nw, smin);
}

void launch_tsaic(double* anut, const double* smin, int jmax, int kmax, const BCTable* bc, double anutinf,
                  cudaStream_t st) {
  dim3 g((jmax + 127) / 128, kmax);
  ++g_kernel_launches;
  k_tsaic<<<g, 128, 0, st>>>(anut, smin, jmax, kmax, bc, anutinf);
}

void launch_update(double* q, const double* dq, size_t N, cudaStream_t st) {
  size_t n3 = 3 * N;
  ++g_kernel_launches;
  k_update<<<(unsigned)((n3 + 255) / 256), 256, 0, st>>>(q, dq, n3);
}

void launch_iter_begin(DevScalars* sc, cudaStream_t st) {
  ++g_kernel_launches;
  k_iter_begin<<<1, 1, 0, st>>>(sc);
}

}  // namespace smac
