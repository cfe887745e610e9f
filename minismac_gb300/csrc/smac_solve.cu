// smac_solve.cu -- implicit solvers of the pseudo-time iteration.
//
//   btlu3j/k, btund3j/k   ref/btlu3.f:52-1055  block tridiagonal LU of every line, and its undo
//   ljsweep / lksweep     ref/lrelax.f:225-561 Gauss-Seidel line relaxation in the reference's
//                                              line order, with under-relaxation
//   bcimpds               ref/bc.f:566-595     wake-cut injection (single subgrid)
//   turswpj/k + scatri    ref/lreltur.f:164-359 scalar SA line relaxation
//   lusgs / ilusol3/1     ref/lusgs.f, ref/ilusol.f  ILU(0) forward / backward substitution
//
// Every kernel keeps the reference's per-point operation order (the library is built with
// -fmad=false).  The natural-order ILU sweeps run as j+k hyperplanes: the two wrap-around
// terms of ref/ilusol.f:185-233 and 415-436 multiply blocks that the boundary blanking sets to
// zero, so the hyperplane order reproduces the natural order.
#include <cooperative_groups.h>
#include <math.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

namespace cg = cooperative_groups;

namespace smac {

__global__ void k_fill(double* p, double v, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_fill_f32(float* p, float v, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

void launch_fill_f32(float* p, float v, size_t n, cudaStream_t st) {
  if (n == 0) return;
  ++g_kernel_launches;
  k_fill_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, v, n);
}

void launch_fill(double* p, double v, size_t n, cudaStream_t st) {
  if (n == 0) return;
  ++g_kernel_launches;
  k_fill<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, v, n);
}

// ------------------------------------------------------------------------------------------
// 3x3 block helpers, entry (r, c) at [r + 3c]
__device__ __forceinline__ void blu(double* b) {  // ref/btlu3.f:148-155
  b[0] = 1. / b[0];
  b[3] = b[3] * b[0];
  b[6] = b[6] * b[0];
  b[4] = 1. / (b[4] - b[1] * b[3]);
  b[7] = (b[7] - b[1] * b[6]) * b[4];
  b[5] = b[5] - b[2] * b[3];
  b[8] = 1. / (b[8] - b[2] * b[6] - b[7] * b[5]);
}

__device__ __forceinline__ void bsolvec(const double* b, double* c) {  // ref/btlu3.f:157-179
  for (int m = 0; m < 3; ++m) {
    double d1 = b[0] * c[0 + 3 * m];
    double d2 = b[4] * (c[1 + 3 * m] - b[1] * d1);
    double d3 = b[8] * (c[2 + 3 * m] - b[2] * d1 - b[5] * d2);
    c[2 + 3 * m] = d3;
    c[1 + 3 * m] = d2 - b[7] * c[2 + 3 * m];
    c[0 + 3 * m] = d1 - b[6] * c[2 + 3 * m] - b[3] * c[1 + 3 * m];
  }
}

__device__ __forceinline__ void load9(const double* p, size_t id, size_t N, double* v) {
  for (int e = 0; e < 9; ++e) v[e] = p[id + N * e];
}
__device__ __forceinline__ void store9(double* p, size_t id, size_t N, const double* v) {
  for (int e = 0; e < 9; ++e) p[id + N * e] = v[e];
}

// factorisation of every line of one direction (btlu3j dir 0 / btlu3k dir 1, ref/btlu3.f:52-398).
// Three lanes per line.  GB300 issues one FP64 instruction per warp
// every 64 cycles however many lanes are active, so the walk is bound by FP64 instructions per
// warp: lane m of a line owns column m of the blocks (the Schur update of column m needs only
// column m of the previous c, and column m of c = B'^-1 C is solved on its own); the three
// columns of B are exchanged by shuffles and the 3x3 LU is done redundantly by the three lanes.
// Every entry sees the operations of btlu3 in the same order, so the factors are identical.
constexpr int kBtluLinesPerWarp = 10;

// FMA = true contracts the products into fused multiply-adds (the partitioned and zebra solves,
// whose results are compared with a tolerance); FMA = false keeps btlu3's operations exactly.
__device__ __forceinline__ void blu_fma(double* b) {
  b[0] = 1. / b[0];
  b[3] = b[3] * b[0];
  b[6] = b[6] * b[0];
  b[4] = 1. / __fma_rn(-b[1], b[3], b[4]);
  b[7] = __fma_rn(-b[1], b[6], b[7]) * b[4];
  b[5] = __fma_rn(-b[2], b[3], b[5]);
  b[8] = 1. / __fma_rn(-b[7], b[5], __fma_rn(-b[2], b[6], b[8]));
}

template <int DIR, bool FMA>
__global__ void __launch_bounds__(32) k_btlu_lanes(const double* __restrict__ a, double* __restrict__ b,
                                                   double* __restrict__ c, int jmax, int kmax) {
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const int lane = threadIdx.x;
  const int slot = lane / 3, m = lane - 3 * (lane / 3);
  const int l0 = blockIdx.x * kBtluLinesPerWarp + slot;
  const bool act = lane < 3 * kBtluLinesPerWarp && l0 < nl;
  const int l = act ? l0 : 0;  // idle lanes read line 0 and store nothing
  const int src = 3 * (lane < 3 * kBtluLinesPerWarp ? slot : 0);
  const size_t N = (size_t)jmax * kmax;
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  double cprev[3] = {0.0, 0.0, 0.0};  // column m of the previous point's c
  double Bn[3], An[9], Cn[3];
  {
    size_t id = P(0);
    for (int r = 0; r < 3; ++r) { Bn[r] = b[id + N * (r + 3 * m)]; Cn[r] = c[id + N * (r + 3 * m)]; }
    for (int e = 0; e < 9; ++e) An[e] = 0.0;
  }
  for (int i = 0; i < n; ++i) {
    const size_t id = P(i);
    double Bc[3], A[9], Cc[3];
    for (int r = 0; r < 3; ++r) { Bc[r] = Bn[r]; Cc[r] = Cn[r]; }
    for (int e = 0; e < 9; ++e) A[e] = An[e];
    if (i + 1 < n) {
      size_t in = P(i + 1);
      for (int r = 0; r < 3; ++r) Bn[r] = b[in + N * (r + 3 * m)];
      for (int e = 0; e < 9; ++e) An[e] = a[in + N * e];
      if (i + 1 < n - 1)
        for (int r = 0; r < 3; ++r) Cn[r] = c[in + N * (r + 3 * m)];
    }
    if (i > 0)
      for (int r = 0; r < 3; ++r) {
        if (FMA) Bc[r] = __fma_rn(-A[r + 6], cprev[2], __fma_rn(-A[r + 3], cprev[1], __fma_rn(-A[r], cprev[0], Bc[r])));
        else Bc[r] = Bc[r] - A[r + 0] * cprev[0] - A[r + 3] * cprev[1] - A[r + 6] * cprev[2];
      }
    double B[9];
    for (int mm = 0; mm < 3; ++mm)
      for (int r = 0; r < 3; ++r) B[r + 3 * mm] = __shfl_sync(0xffffffffu, Bc[r], src + mm);
    if (FMA) blu_fma(B);
    else blu(B);
    if (act)
      for (int r = 0; r < 3; ++r) b[id + N * (r + 3 * m)] = m == 0 ? B[r] : (m == 1 ? B[r + 3] : B[r + 6]);
    if (i < n - 1) {
      // column m of bsolvec (ref/btlu3.f:157-179)
      double d1 = B[0] * Cc[0];
      if (FMA) {
        double d2 = B[4] * __fma_rn(-B[1], d1, Cc[1]);
        double d3 = B[8] * __fma_rn(-B[5], d2, __fma_rn(-B[2], d1, Cc[2]));
        Cc[2] = d3;
        Cc[1] = __fma_rn(-B[7], d3, d2);
        Cc[0] = __fma_rn(-B[3], Cc[1], __fma_rn(-B[6], d3, d1));
      } else {
        double d2 = B[4] * (Cc[1] - B[1] * d1);
        double d3 = B[8] * (Cc[2] - B[2] * d1 - B[5] * d2);
        Cc[2] = d3;
        Cc[1] = d2 - B[7] * Cc[2];
        Cc[0] = d1 - B[6] * Cc[2] - B[3] * Cc[1];
      }
      if (act)
        for (int r = 0; r < 3; ++r) c[id + N * (r + 3 * m)] = Cc[r];
      for (int r = 0; r < 3; ++r) cprev[r] = Cc[r];
    }
  }
}

void launch_btlu(int dir, const double* a, double* b, double* c, int jmax, int kmax, cudaStream_t st, bool exact) {
  int nl = dir == 0 ? kmax : jmax;
  int nb = (nl + kBtluLinesPerWarp - 1) / kBtluLinesPerWarp;
  ++g_kernel_launches;
  if (exact) {
    if (dir == 0) k_btlu_lanes<0, false><<<nb, 32, 0, st>>>(a, b, c, jmax, kmax);
    else k_btlu_lanes<1, false><<<nb, 32, 0, st>>>(a, b, c, jmax, kmax);
  } else {
    if (dir == 0) k_btlu_lanes<0, true><<<nb, 32, 0, st>>>(a, b, c, jmax, kmax);
    else k_btlu_lanes<1, true><<<nb, 32, 0, st>>>(a, b, c, jmax, kmax);
  }
}

// undo (btund3j dir 0 / btund3k dir 1): point-wise given the factored state
template <int DIR>
__global__ void k_btund(const double* __restrict__ a, double* __restrict__ b, const double* __restrict__ c,
                        double* __restrict__ c_out, int jmax, int kmax) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (j >= jmax || k >= kmax) return;
  const size_t N = (size_t)jmax * kmax;
  const int n = DIR == 0 ? jmax : kmax;
  const int p = DIR == 0 ? j : k;
  size_t id = ix(j, k, jmax);
  double B[9];
  load9(b, id, N, B);
  // LU product (ref/btlu3.f:645-658)
  B[8] = 1. / B[8] + B[2] * B[6] + B[5] * B[7];
  B[5] = B[5] + B[2] * B[3];
  B[4] = 1. / B[4];
  B[7] = B[7] * B[4] + B[1] * B[6];
  B[4] = B[4] + B[1] * B[3];
  B[0] = 1. / B[0];
  B[6] = B[6] * B[0];
  B[3] = B[3] * B[0];
  if (c_out) {
    double C[9];
    load9(c, id, N, C);
    if (p <= n - 2) {
      double Cn[9];
      for (int m = 0; m < 3; ++m)
        for (int r = 0; r < 3; ++r)
          Cn[r + 3 * m] = B[r + 0] * C[0 + 3 * m] + B[r + 3] * C[1 + 3 * m] + B[r + 6] * C[2 + 3 * m];
      store9(c_out, id, N, Cn);
    } else {
      store9(c_out, id, N, C);
    }
  }
  if (p >= 1) {
    size_t ip = DIR == 0 ? ix(j - 1, k, jmax) : ix(j, k - 1, jmax);
    double A[9], Cp[9];
    load9(a, id, N, A);
    load9(c, ip, N, Cp);
    for (int m = 0; m < 3; ++m)
      for (int r = 0; r < 3; ++r)
        B[r + 3 * m] = B[r + 3 * m] + A[r + 0] * Cp[0 + 3 * m] + A[r + 3] * Cp[1 + 3 * m] + A[r + 6] * Cp[2 + 3 * m];
  }
  store9(b, id, N, B);
}

void launch_btund(int dir, const double* a, double* b, const double* c, double* c_out, int jmax, int kmax,
                  cudaStream_t st) {
  dim3 g((jmax + 127) / 128, kmax);
  if (dir == 0) { ++g_kernel_launches; k_btund<0><<<g, 128, 0, st>>>(a, b, c, c_out, jmax, kmax); }
  else { ++g_kernel_launches; k_btund<1><<<g, 128, 0, st>>>(a, b, c, c_out, jmax, kmax); }
}

// ------------------------------------------------------------------------------------------
// Gauss-Seidel line sweep, reference order, sequential recurrence per line (one CTA walks all
// lines; the right-hand sides and the relaxation update are formed in parallel)
template <int DIR>
__global__ void k_gs_sweep_exact(SweepArgs a, int nsw) {
  extern __shared__ double rhs[];  // [3][n]
  const int jmax = a.jmax, kmax = a.kmax;
  const size_t N = a.N;
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const double half = 0.5;
  int lb, le, li;
  if ((nsw / 2) * 2 == nsw) { lb = nl - 1; le = 0; li = -1; }
  else { lb = 0; le = nl - 1; li = 1; }
  for (int l = lb;; l += li) {
    int lm = l - 1 > 0 ? l - 1 : 0;
    int lp = l + 1 < nl - 1 ? l + 1 : nl - 1;
    double swm = half + copysign(half, (double)(l - 1 - lm));
    double swp = half + copysign(half, (double)(lp - l - 1));
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
      size_t im = DIR == 0 ? ix(i, lm, jmax) : ix(lm, i, jmax);
      size_t ip = DIR == 0 ? ix(i, lp, jmax) : ix(lp, i, jmax);
      double d1 = a.dq[im], d2 = a.dq[im + N], d3 = a.dq[im + 2 * N];
      double e1 = a.dq[ip], e2 = a.dq[ip + N], e3 = a.dq[ip + 2 * N];
      for (int r = 0; r < 3; ++r)
        rhs[r * n + i] = a.s[id + N * r] -
                         (a.om[id + N * (r + 0)] * d1 + a.om[id + N * (r + 3)] * d2 + a.om[id + N * (r + 6)] * d3) *
                             swm -
                         (a.op[id + N * (r + 0)] * e1 + a.op[id + N * (r + 3)] * e2 + a.op[id + N * (r + 6)] * e3) *
                             swp;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double r0[3] = {0, 0, 0};
      for (int i = 0; i < n; ++i) {
        size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
        double x1 = rhs[i], x2 = rhs[n + i], x3 = rhs[2 * n + i];
        if (i > 0) {
          const double* A = a.am;
          double y1 = x1 - A[id] * r0[0] - A[id + 3 * N] * r0[1] - A[id + 6 * N] * r0[2];
          double y2 = x2 - A[id + N] * r0[0] - A[id + 4 * N] * r0[1] - A[id + 7 * N] * r0[2];
          double y3 = x3 - A[id + 2 * N] * r0[0] - A[id + 5 * N] * r0[1] - A[id + 8 * N] * r0[2];
          x1 = y1; x2 = y2; x3 = y3;
        }
        const double* B = a.btc;
        double d1 = B[id] * x1;
        double d2 = B[id + 4 * N] * (x2 - B[id + N] * d1);
        double d3 = B[id + 8 * N] * (x3 - B[id + 2 * N] * d1 - B[id + 5 * N] * d2);
        x3 = d3;
        x2 = d2 - B[id + 7 * N] * x3;
        x1 = d1 - B[id + 6 * N] * x3 - B[id + 3 * N] * x2;
        rhs[i] = x1; rhs[n + i] = x2; rhs[2 * n + i] = x3;
        r0[0] = x1; r0[1] = x2; r0[2] = x3;
      }
      for (int i = n - 2; i >= 0; --i) {
        size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
        const double* C = a.cp;
        double x1 = rhs[i], x2 = rhs[n + i], x3 = rhs[2 * n + i];
        double n1 = rhs[i + 1], n2 = rhs[n + i + 1], n3 = rhs[2 * n + i + 1];
        rhs[i] = x1 - C[id] * n1 - C[id + 3 * N] * n2 - C[id + 6 * N] * n3;
        rhs[n + i] = x2 - C[id + N] * n1 - C[id + 4 * N] * n2 - C[id + 7 * N] * n3;
        rhs[2 * n + i] = x3 - C[id + 2 * N] * n1 - C[id + 5 * N] * n2 - C[id + 8 * N] * n3;
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
      for (int r = 0; r < 3; ++r) {
        double d = a.dq[id + N * r];
        a.dq[id + N * r] = d + a.underr * (rhs[r * n + i] - d);
      }
    }
    __syncthreads();
    if (l == le) break;
  }
}

void launch_gs_sweep(int dir, int nsw, const SweepArgs& a, int exact, cudaStream_t st) {
  (void)exact;
  int n = dir == 0 ? a.jmax : a.kmax;
  size_t sm = sizeof(double) * 3 * (size_t)n;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gs_sweep_exact<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(k_gs_sweep_exact<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  if (dir == 0) { ++g_kernel_launches; k_gs_sweep_exact<0><<<1, 256, sm, st>>>(a, nsw); }
  else { ++g_kernel_launches; k_gs_sweep_exact<1><<<1, 256, sm, st>>>(a, nsw); }
}

// ------------------------------------------------------------------------------------------
// bcimpds, single subgrid (ref/bc.f:566-595): wake-cut rows k = 1 from the average of both
// sides at k = 2; the injected value also replaces the right-hand side
// kmaj = 0: ds and rhs in the reference layout; kmaj = kmax: ds and rhs k-major ((j,k) at
// k + kmax*j), the state s always in the reference layout
__global__ void k_bcimpds(const BCTable* __restrict__ bc, int neqs, int jmax, int kmaj, size_t N,
                          const double* __restrict__ s, double* __restrict__ ds, double* __restrict__ rhs) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  auto dx = [&](int j, int k) -> size_t { return kmaj ? (size_t)k + (size_t)kmaj * j : ix(j, k, jmax); };
  for (int r = 0; r < bc->nwake; ++r) {
    int len = bc->jt_e[r] - bc->jt_b[r] + 1;
    if (t >= len * neqs) { t -= len * neqs; continue; }
    int off = t / neqs, neq = t % neqs;
    int jt = bc->jt_b[r] + off;
    int jb = bc->jb_b[r] - off;
    size_t n0 = N * neq;
    double snew = 0.5 * (s[ix(jt, 1, jmax) + n0] + s[ix(jb, 1, jmax) + n0]);
    double dsnew = 0.5 * (ds[dx(jt, 1) + n0] + ds[dx(jb, 1) + n0]);
    double v = snew + dsnew - s[ix(jt, 0, jmax) + n0];
    ds[dx(jt, 0) + n0] = v;
    rhs[dx(jt, 0) + n0] = v;
    return;
  }
}

void launch_bcimpds(const BCTable* bc, int neqs, int jmax, size_t N, const double* s, double* ds, double* rhs,
                    cudaStream_t st, int kmajor_kmax) {
  int maxn = 2 * jmax * neqs;
  ++g_kernel_launches;
  k_bcimpds<<<(maxn + 127) / 128, 128, 0, st>>>(bc, neqs, jmax, kmajor_kmax, N, s, ds, rhs);
}

// ------------------------------------------------------------------------------------------
// scalar SA line relaxation (turswpj dir 0 / turswpk dir 1), reference order: lines 1..max,
// then line 1 again; scatri per line
template <int DIR>
__global__ void k_sa_sweep_exact(ScalarSweepArgs a) {
  extern __shared__ double sh[];
  const int jmax = a.jmax, kmax = a.kmax;
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  double* ff = sh;
  double* cc = sh + n;
  const double* am = DIR == 0 ? a.sjm : a.skm;  // in-line
  const double* ap = DIR == 0 ? a.sjp : a.skp;
  const double* om = DIR == 0 ? a.skm : a.sjm;  // off-line
  const double* op = DIR == 0 ? a.skp : a.sjp;
  for (int step = 0; step <= nl; ++step) {
    int l = step < nl ? step : 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
      size_t im = DIR == 0 ? ix(i, l - 1, jmax) : ix(l - 1, i, jmax);
      size_t ip = DIR == 0 ? ix(i, l + 1, jmax) : ix(l + 1, i, jmax);
      double f;
      if (l == 0) f = a.rhs[id] - op[id] * a.ds[ip];
      else if (l == nl - 1) f = a.rhs[id] - om[id] * a.ds[im];
      else f = a.rhs[id] - om[id] * a.ds[im] - op[id] * a.ds[ip];
      ff[i] = f;
      cc[i] = ap[id];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
      size_t i0 = P(0);
      ff[0] = ff[0] / a.stc[i0];
      cc[0] = cc[0] / a.stc[i0];
      for (int i = 1; i <= n - 2; ++i) {
        size_t id = P(i);
        double z = 1. / (a.stc[id] - am[id] * cc[i - 1]);
        cc[i] = cc[i] * z;
        ff[i] = (ff[i] - am[id] * ff[i - 1]) * z;
      }
      {
        size_t id = P(n - 1);
        ff[n - 1] = (ff[n - 1] - am[id] * ff[n - 2]) / (a.stc[id] - am[id] * cc[n - 2]);
      }
      for (int i = n - 2; i >= 0; --i) ff[i] = ff[i] - cc[i] * ff[i + 1];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
      a.ds[id] = ff[i];
    }
    __syncthreads();
  }
}

void launch_sa_sweep(int dir, const ScalarSweepArgs& a, int exact, cudaStream_t st) {
  (void)exact;
  int n = dir == 0 ? a.jmax : a.kmax;
  size_t sm = sizeof(double) * 2 * (size_t)n;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_sa_sweep_exact<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_sa_sweep_exact<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  if (dir == 0) { ++g_kernel_launches; k_sa_sweep_exact<0><<<1, 256, sm, st>>>(a); }
  else { ++g_kernel_launches; k_sa_sweep_exact<1><<<1, 256, sm, st>>>(a); }
}

// ------------------------------------------------------------------------------------------
// LU-SGS: lusini3 (ref/lusgs.f:185-214)
__global__ void k_lusini3(const double* __restrict__ btc, double* __restrict__ bprm, size_t N) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  double T[9], P[9];
  load9(btc, i, N, T);
  P[0] = 1. / T[0];
  P[3] = T[3] * P[0];
  P[6] = T[6] * P[0];
  P[1] = T[1];
  P[4] = 1. / (T[4] - P[1] * P[3]);
  P[7] = (T[7] - P[1] * P[6]) * P[4];
  P[2] = T[2];
  P[5] = T[5] - P[2] * P[3];
  P[8] = 1. / (T[8] - P[2] * P[6] - P[5] * P[7]);
  store9(bprm, i, N, P);
}

__device__ __forceinline__ void lu_apply(const double* __restrict__ bp, size_t id, size_t N, double r1, double r2,
                                         double r3, double& o1, double& o2, double& o3) {
  double z1 = r1 * bp[id];
  double z2 = (r2 - bp[id + N] * z1) * bp[id + 4 * N];
  double z3 = (r3 - bp[id + 2 * N] * z1 - bp[id + 5 * N] * z2) * bp[id + 8 * N];
  o3 = z3;
  o2 = z2 - bp[id + 7 * N] * o3;
  o1 = z1 - bp[id + 6 * N] * o3 - bp[id + 3 * N] * o2;
}

// forward substitution at one point (ref/ilusol.f:80-287)
__device__ __forceinline__ void ilu3_fwd_point(int j, int k, int jmax, size_t N, const double* __restrict__ bp,
                                               const double* __restrict__ bjm, const double* __restrict__ bkm,
                                               double* __restrict__ r) {
  size_t id = ix(j, k, jmax);
  double rr[3];
  if (k == 0 && j == 0) {
    rr[0] = r[id]; rr[1] = r[id + N]; rr[2] = r[id + 2 * N];
  } else if (k == 0) {
    size_t iw = ix(j - 1, k, jmax);
    for (int n = 0; n < 3; ++n)
      rr[n] = r[id + N * n] - bjm[id + N * (n + 0)] * r[iw] - bjm[id + N * (n + 3)] * r[iw + N] -
              bjm[id + N * (n + 6)] * r[iw + 2 * N];
  } else {
    size_t iw = j == 0 ? ix(jmax - 1, k - 1, jmax) : ix(j - 1, k, jmax);
    size_t is = ix(j, k - 1, jmax);
    for (int n = 0; n < 3; ++n)
      rr[n] = r[id + N * n] - bjm[id + N * (n + 0)] * r[iw] - bjm[id + N * (n + 3)] * r[iw + N] -
              bjm[id + N * (n + 6)] * r[iw + 2 * N] - bkm[id + N * (n + 0)] * r[is] -
              bkm[id + N * (n + 3)] * r[is + N] - bkm[id + N * (n + 6)] * r[is + 2 * N];
  }
  double o1, o2, o3;
  lu_apply(bp, id, N, rr[0], rr[1], rr[2], o1, o2, o3);
  r[id] = o1; r[id + N] = o2; r[id + 2 * N] = o3;
}

// multiply by the diagonal block rebuilt from its LU form (ref/ilusol.f:307-341)
__global__ void k_ilu3_dmul(const double* __restrict__ bt, double* __restrict__ r, size_t N) {
  size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= N) return;
  double b11 = 1. / bt[id];
  double b12 = bt[id + 3 * N] * b11;
  double b13 = bt[id + 6 * N] * b11;
  double b21 = bt[id + N];
  double b22 = 1. / bt[id + 4 * N] + bt[id + N] * bt[id + 3 * N];
  double b23 = bt[id + 7 * N] / bt[id + 4 * N] + bt[id + N] * bt[id + 6 * N];
  double b31 = bt[id + 2 * N];
  double b32 = bt[id + 5 * N] + bt[id + 2 * N] * bt[id + 3 * N];
  double b33 = 1. / bt[id + 8 * N] + bt[id + 2 * N] * bt[id + 6 * N] + bt[id + 5 * N] * bt[id + 7 * N];
  double r1 = r[id], r2 = r[id + N], r3 = r[id + 2 * N];
  double s1 = b11 * r1 + b12 * r2 + b13 * r3;
  double s2 = b21 * r1 + b22 * r2 + b23 * r3;
  double s3 = b31 * r1 + b32 * r2 + b33 * r3;
  r[id] = s1; r[id + N] = s2; r[id + 2 * N] = s3;
}

// backward substitution at one point (ref/ilusol.f:349-469)
__device__ __forceinline__ void ilu3_bwd_point(int j, int k, int jmax, int kmax, size_t N,
                                               const double* __restrict__ bp, const double* __restrict__ bjp,
                                               const double* __restrict__ bkp, const double* __restrict__ r,
                                               double* __restrict__ dq) {
  size_t id = ix(j, k, jmax);
  double rr[3];
  if (k == kmax - 1 && j == jmax - 1) {
    rr[0] = r[id]; rr[1] = r[id + N]; rr[2] = r[id + 2 * N];
  } else if (k == kmax - 1) {
    size_t ie = ix(j + 1, k, jmax);
    for (int n = 0; n < 3; ++n)
      rr[n] = r[id + N * n] - bjp[id + N * (n + 0)] * dq[ie] - bjp[id + N * (n + 3)] * dq[ie + N] -
              bjp[id + N * (n + 6)] * dq[ie + 2 * N];
  } else {
    size_t in = ix(j, k + 1, jmax);
    for (int n = 0; n < 3; ++n) {
      size_t ie = j == jmax - 1 ? (n == 2 ? ix(0, kmax - 1, jmax) : ix(jmax - 1, kmax - 1, jmax)) : ix(j + 1, k, jmax);
      rr[n] = r[id + N * n] - bkp[id + N * (n + 0)] * dq[in] - bkp[id + N * (n + 3)] * dq[in + N] -
              bkp[id + N * (n + 6)] * dq[in + 2 * N] - bjp[id + N * (n + 0)] * dq[ie] -
              bjp[id + N * (n + 3)] * dq[ie + N] - bjp[id + N * (n + 6)] * dq[ie + 2 * N];
    }
  }
  double o1, o2, o3;
  lu_apply(bp, id, N, rr[0], rr[1], rr[2], o1, o2, o3);
  dq[id] = o1; dq[id + N] = o2; dq[id + 2 * N] = o3;
}

// scalar ILU(0) for the SA equation (lusini1 + ilusol1, ref/lusgs.f:218-236, ref/ilusol.f:486-591)
__global__ void k_lusini1(const double* __restrict__ stc, double* __restrict__ bprm, size_t N) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < N) bprm[i] = 1. / stc[i];
}

__device__ __forceinline__ void ilu1_fwd_point(int j, int k, int jmax, const double* __restrict__ bt,
                                               const double* __restrict__ bjm, const double* __restrict__ bkm,
                                               double* __restrict__ r) {
  size_t id = ix(j, k, jmax);
  if (k == 0 && j == 0) r[id] = r[id] * bt[id];
  else if (k == 0) r[id] = bt[id] * (r[id] - bjm[id] * r[ix(j - 1, 0, jmax)]);
  else if (j == 0) r[id] = bt[id] * (r[id] - bjm[id] * r[ix(jmax - 1, k - 1, jmax)] - bkm[id] * r[ix(j, k - 1, jmax)]);
  else r[id] = bt[id] * (r[id] - bjm[id] * r[ix(j - 1, k, jmax)] - bkm[id] * r[ix(j, k - 1, jmax)]);
}

__global__ void k_ilu1_div(const double* __restrict__ bt, double* __restrict__ r, size_t N) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < N) r[i] = r[i] / bt[i];
}

__device__ __forceinline__ void ilu1_bwd_point(int j, int k, int jmax, int kmax, const double* __restrict__ bt,
                                               const double* __restrict__ bjp, const double* __restrict__ bkp,
                                               const double* __restrict__ r, double* __restrict__ dq) {
  size_t id = ix(j, k, jmax);
  if (k == kmax - 1 && j == jmax - 1) dq[id] = r[id] * bt[id];
  else if (k == kmax - 1) dq[id] = bt[id] * (r[id] - bjp[id] * dq[ix(j + 1, k, jmax)]);
  else if (j == jmax - 1)
    dq[id] = bt[id] * (r[id] - bkp[id] * dq[ix(j, k + 1, jmax)] - bjp[id] * dq[ix(0, k + 1, jmax)]);
  else dq[id] = bt[id] * (r[id] - bkp[id] * dq[ix(j, k + 1, jmax)] - bjp[id] * dq[ix(j + 1, k, jmax)]);
}

// Hyperplane sweeps: the points of one diagonal j + k = d depend only on the previous diagonal
// (forward: (j-1,k) and (j,k-1); backward: (j+1,k) and (j,k+1)), so one cluster of kIluCL CTAs
// walks the diagonals in order, a thread per point of the diagonal, with a cluster barrier
// (release/acquire at cluster scope) between diagonals.  The per-point arithmetic is the
// reference's; the two wrap-around terms of the flattened natural order multiply blocks that the
// boundary blanking zeroes, so the diagonal order reproduces the natural order bit for bit.
constexpr int kIluCL = 8, kIluNT = 256;

template <int FWD, int NEQ>
__global__ void __cluster_dims__(kIluCL, 1, 1) __launch_bounds__(kIluNT)
    k_ilu_diag(int jmax, int kmax, size_t N, const double* __restrict__ bt, const double* __restrict__ b1,
               const double* __restrict__ b2, double* __restrict__ r, double* __restrict__ dq) {
  cg::cluster_group cluster = cg::this_cluster();
  const int t = (int)cluster.block_rank() * kIluNT + threadIdx.x;
  const int nd = jmax + kmax - 1;
  for (int dd = 0; dd < nd; ++dd) {
    const int d = FWD ? dd : nd - 1 - dd;
    const int kb = d - (jmax - 1) > 0 ? d - (jmax - 1) : 0;
    const int ke = d < kmax - 1 ? d : kmax - 1;
    for (int k = kb + t; k <= ke; k += kIluCL * kIluNT) {
      const int j = d - k;
      if (NEQ == 3) {
        if (FWD) ilu3_fwd_point(j, k, jmax, N, bt, b1, b2, r);
        else ilu3_bwd_point(j, k, jmax, kmax, N, bt, b1, b2, r, dq);
      } else {
        if (FWD) ilu1_fwd_point(j, k, jmax, bt, b1, b2, r);
        else ilu1_bwd_point(j, k, jmax, kmax, bt, b1, b2, r, dq);
      }
    }
    cluster.sync();
  }
}

// The same sweeps with one row k per thread triple (block ILU) or per thread (scalar ILU), for
// grids of at most kIluRows rows: the row's previous point (j -+ 1, k) stays in registers, only
// the neighbour row's value crosses threads; in the block sweeps lane r of a triple evaluates
// row r of the point's right-hand side (the reference's expression, term by term) and the three
// lanes then apply the factored diagonal block; the next diagonal's fixed operands are loaded
// before the barrier.
constexpr int kIluRows = kIluCL * (kIluNT / 32) * 10;

template <int FWD, int CL, int NT>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NT)
    k_ilu3_rows(int jmax, int kmax, size_t N, const double* __restrict__ bp, const double* __restrict__ bA,
                const double* __restrict__ bB, double* __restrict__ r, double* __restrict__ dq) {
  // FWD: bA = bjm, bB = bkm, r rewritten in place; backward: bA = bjp, bB = bkp, dq written.
  // The neighbour row's outputs of the previous diagonal ((j, k-1) forward, (j, k+1) backward)
  // come by shuffle from the next triple of the warp, through shared memory from the
  // neighbouring warp, or through distributed shared memory from the neighbouring CTA (written
  // before the cluster barrier), not back through L2.
  constexpr int NW = NT / 32;
  __shared__ double edge[2][NW][3];  // [parity][warp]: the warp's edge row, for the neighbouring warp
  __shared__ double edge_in[2][3];   // [parity]: the neighbouring CTA's edge row
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int slot = lane / 3, rr = lane - 3 * (lane / 3);
  const int base = 3 * (slot < 10 ? slot : 9);
  const int k = (rank * NW + w) * 10 + slot;
  const bool row = slot < 10 && k < kmax;
  const int nd = jmax + kmax - 1;
  if (threadIdx.x < 6) edge_in[threadIdx.x / 3][threadIdx.x % 3] = 0.0;
  cluster.sync();  // before any neighbour writes into edge_in
  double xp[3] = {0.0, 0.0, 0.0};   // this row's previous point: (j-1,k) forward, (j+1,k) backward
  double nbr[3] = {0.0, 0.0, 0.0};  // the neighbour row's point on the previous diagonal
  // fixed operands of this lane's point on the current diagonal
  auto load_fixed = [&](int d, double& rv, double* a3, double* b3, double* P) {
    const int j = d - k;
    if (!(row && j >= 0 && j < jmax)) return;
    const size_t id = ix(j, k, jmax);
    rv = r[id + N * rr];
    for (int c = 0; c < 3; ++c) { a3[c] = bA[id + N * (rr + 3 * c)]; b3[c] = bB[id + N * (rr + 3 * c)]; }
    for (int e = 0; e < 9; ++e) P[e] = bp[id + N * e];
  };
  double rv = 0.0, a3[3] = {0.0, 0.0, 0.0}, b3[3] = {0.0, 0.0, 0.0}, P[9];
  for (int e = 0; e < 9; ++e) P[e] = 0.0;
  load_fixed(FWD ? 0 : nd - 1, rv, a3, b3, P);
  for (int dd = 0; dd < nd; ++dd) {
    const int par = dd & 1;
    const int d = FWD ? dd : nd - 1 - dd;
    const int j = d - k;
    const bool act = row && j >= 0 && j < jmax;
    double cr = rv, ca[3] = {a3[0], a3[1], a3[2]}, cb[3] = {b3[0], b3[1], b3[2]}, CP[9];
    for (int e = 0; e < 9; ++e) CP[e] = P[e];
    if (dd + 1 < nd) load_fixed(FWD ? d + 1 : d - 1, rv, a3, b3, P);
    double v = 0.0;
    if (act) {
      if (FWD) {
        // ref/ilusol.f:80-287 (ilu3_fwd_point)
        if (k == 0 && j == 0) {
          v = cr;
        } else if (k == 0) {
          v = cr - ca[0] * xp[0] - ca[1] * xp[1] - ca[2] * xp[2];
        } else {
          double wv[3];
          if (j == 0) {
            const size_t iw = ix(jmax - 1, k - 1, jmax);
            wv[0] = r[iw]; wv[1] = r[iw + N]; wv[2] = r[iw + 2 * N];
          } else {
            wv[0] = xp[0]; wv[1] = xp[1]; wv[2] = xp[2];
          }
          v = cr - ca[0] * wv[0] - ca[1] * wv[1] - ca[2] * wv[2] - cb[0] * nbr[0] - cb[1] * nbr[1] - cb[2] * nbr[2];
        }
      } else {
        // ref/ilusol.f:349-469 (ilu3_bwd_point)
        if (k == kmax - 1 && j == jmax - 1) {
          v = cr;
        } else if (k == kmax - 1) {
          v = cr - ca[0] * xp[0] - ca[1] * xp[1] - ca[2] * xp[2];
        } else {
          double ev[3];
          if (j == jmax - 1) {
            const size_t ie = rr == 2 ? ix(0, kmax - 1, jmax) : ix(jmax - 1, kmax - 1, jmax);
            ev[0] = dq[ie]; ev[1] = dq[ie + N]; ev[2] = dq[ie + 2 * N];
          } else {
            ev[0] = xp[0]; ev[1] = xp[1]; ev[2] = xp[2];
          }
          v = cr - cb[0] * nbr[0] - cb[1] * nbr[1] - cb[2] * nbr[2] - ca[0] * ev[0] - ca[1] * ev[1] - ca[2] * ev[2];
        }
      }
    }
    double rv3[3];
    rv3[0] = __shfl_sync(0xffffffffu, v, base);
    rv3[1] = __shfl_sync(0xffffffffu, v, base + 1);
    rv3[2] = __shfl_sync(0xffffffffu, v, base + 2);
    if (act) {
      // lu_apply with the factored diagonal block (ref/lusgs.f:185-214 factors, ilusol solve)
      double z1 = rv3[0] * CP[0];
      double z2 = (rv3[1] - CP[1] * z1) * CP[4];
      double z3 = (rv3[2] - CP[2] * z1 - CP[5] * z2) * CP[8];
      double o3 = z3;
      double o2 = z2 - CP[7] * o3;
      double o1 = z1 - CP[6] * o3 - CP[3] * o2;
      xp[0] = o1; xp[1] = o2; xp[2] = o3;
      const size_t id = ix(j, k, jmax);
      const double mine = rr == 0 ? o1 : (rr == 1 ? o2 : o3);
      if (FWD) r[id + N * rr] = mine;
      else dq[id + N * rr] = mine;
    }
    // this row's point goes to its neighbour row for the next diagonal (a row is active there
    // exactly when its neighbour was active here, so xp is fresh whenever it is used)
    const int src = FWD ? (slot >= 1 && slot < 10 ? base - 3 : lane) : (slot <= 8 ? base + 3 : lane);
    const double t0 = __shfl_sync(0xffffffffu, xp[0], src);
    const double t1 = __shfl_sync(0xffffffffu, xp[1], src);
    const double t2 = __shfl_sync(0xffffffffu, xp[2], src);
    if (lane == (FWD ? 27 : 0)) {  // the warp's edge row: slot 9 forward, slot 0 backward
      edge[par][w][0] = xp[0]; edge[par][w][1] = xp[1]; edge[par][w][2] = xp[2];
      const bool cta_edge = FWD ? (w == NW - 1 && rank + 1 < CL) : (w == 0 && rank > 0);
      if (cta_edge) {
        double* rem = cluster.map_shared_rank(&edge_in[par][0], (unsigned)(FWD ? rank + 1 : rank - 1));
        rem[0] = xp[0]; rem[1] = xp[1]; rem[2] = xp[2];
      }
    }
    cluster.sync();
    if (FWD ? slot != 0 : slot != 9) {
      nbr[0] = t0; nbr[1] = t1; nbr[2] = t2;
    } else {
      const int wn = FWD ? w - 1 : w + 1;
      const double* e = (wn >= 0 && wn < NW) ? edge[par][wn] : edge_in[par];
      nbr[0] = e[0]; nbr[1] = e[1]; nbr[2] = e[2];
    }
  }
}

template <int FWD>
__global__ void __cluster_dims__(kIluCL, 1, 1) __launch_bounds__(kIluNT)
    k_ilu1_rows(int jmax, int kmax, const double* __restrict__ bt, const double* __restrict__ bA,
                const double* __restrict__ bB, double* __restrict__ r, double* __restrict__ dq) {
  cg::cluster_group cluster = cg::this_cluster();
  const int k = (int)cluster.block_rank() * kIluNT + threadIdx.x;
  const bool row = k < kmax;
  const int nd = jmax + kmax - 1;
  double xp = 0.0;
  for (int dd = 0; dd < nd; ++dd) {
    const int d = FWD ? dd : nd - 1 - dd;
    const int j = d - k;
    if (row && j >= 0 && j < jmax) {
      const size_t id = ix(j, k, jmax);
      double o;
      if (FWD) {  // ref/ilusol.f:486-540 (ilu1_fwd_point)
        if (k == 0 && j == 0) o = r[id] * bt[id];
        else if (k == 0) o = bt[id] * (r[id] - bA[id] * xp);
        else if (j == 0) o = bt[id] * (r[id] - bA[id] * r[ix(jmax - 1, k - 1, jmax)] - bB[id] * r[ix(j, k - 1, jmax)]);
        else o = bt[id] * (r[id] - bA[id] * xp - bB[id] * r[ix(j, k - 1, jmax)]);
        r[id] = o;
      } else {  // ref/ilusol.f:545-591 (ilu1_bwd_point)
        if (k == kmax - 1 && j == jmax - 1) o = r[id] * bt[id];
        else if (k == kmax - 1) o = bt[id] * (r[id] - bA[id] * xp);
        else if (j == jmax - 1) o = bt[id] * (r[id] - bB[id] * dq[ix(j, k + 1, jmax)] - bA[id] * dq[ix(0, k + 1, jmax)]);
        else o = bt[id] * (r[id] - bB[id] * dq[ix(j, k + 1, jmax)] - bA[id] * xp);
        dq[id] = o;
      }
      xp = o;
    }
    cluster.sync();
  }
}

// The block sweeps spread the rows over 16 CTAs of four warps (a non-portable cluster size)
// where the device can place such a cluster, else over 8 CTAs of eight warps: each warp issues
// its ~27 FP64 instructions per diagonal, and GB300 issues one FP64 warp instruction per
// sub-partition every 64 cycles, so fewer warps per SM shorten every diagonal (1921x481
// LU-SGS iteration 24.0 -> 18.3 ms).
static bool ilu_wide() {
  static int wide = -1;
  if (wide < 0) {
    wide = 0;
    if (cudaFuncSetAttribute(k_ilu3_rows<1, 16, 128>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaFuncSetAttribute(k_ilu3_rows<0, 16, 128>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(16, 1, 1);
      cfg.blockDim = dim3(128, 1, 1);
      cudaLaunchAttribute at;
      at.id = cudaLaunchAttributeClusterDimension;
      at.val.clusterDim.x = 16; at.val.clusterDim.y = 1; at.val.clusterDim.z = 1;
      cfg.attrs = &at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, k_ilu3_rows<1, 16, 128>, &cfg) == cudaSuccess &&
          nclusters >= 1)
        wide = 1;
    }
    cudaGetLastError();
  }
  return wide == 1;
}

void ilu_setup() { (void)ilu_wide(); }

template <int FWD>
static void launch_ilu3_rows(int jmax, int kmax, size_t N, const double* bp, const double* bA, const double* bB,
                             double* r, double* dq, cudaStream_t st) {
  if (ilu_wide()) k_ilu3_rows<FWD, 16, 128><<<16, 128, 0, st>>>(jmax, kmax, N, bp, bA, bB, r, dq);
  else k_ilu3_rows<FWD, 8, 256><<<8, 256, 0, st>>>(jmax, kmax, N, bp, bA, bB, r, dq);
}

template <int NEQ>
static void ilu_sweeps(int jmax, int kmax, const double* bt, const double* bm1, const double* bm2, const double* bp1,
                       const double* bp2, double* r, double* dq, cudaStream_t st) {
  const size_t N = (size_t)jmax * kmax;
  const bool rows = NEQ == 3 ? kmax <= kIluRows : kmax <= kIluCL * kIluNT;
  ++g_kernel_launches;
  if (rows && NEQ == 3) launch_ilu3_rows<1>(jmax, kmax, N, bt, bm1, bm2, r, dq, st);
  else if (rows) k_ilu1_rows<1><<<kIluCL, kIluNT, 0, st>>>(jmax, kmax, bt, bm1, bm2, r, dq);
  else k_ilu_diag<1, NEQ><<<kIluCL, kIluNT, 0, st>>>(jmax, kmax, N, bt, bm1, bm2, r, dq);
  if (NEQ == 3) {
    ++g_kernel_launches;
    k_ilu3_dmul<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(bt, r, N);
  } else {
    ++g_kernel_launches;
    k_ilu1_div<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(bt, r, N);
  }
  ++g_kernel_launches;
  if (rows && NEQ == 3) launch_ilu3_rows<0>(jmax, kmax, N, bt, bp1, bp2, r, dq, st);
  else if (rows) k_ilu1_rows<0><<<kIluCL, kIluNT, 0, st>>>(jmax, kmax, bt, bp1, bp2, r, dq);
  else k_ilu_diag<0, NEQ><<<kIluCL, kIluNT, 0, st>>>(jmax, kmax, N, bt, bp1, bp2, r, dq);
}

void launch_lusgs3(int jmax, int kmax, const double* btc, const double* bjm, const double* bjp, const double* bkm,
                   const double* bkp, double* bprm, double* rhs, double* dq, cudaStream_t st) {
  size_t N = (size_t)jmax * kmax;
  ++g_kernel_launches;
  k_lusini3<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(btc, bprm, N);
  ilu_sweeps<3>(jmax, kmax, bprm, bjm, bkm, bjp, bkp, rhs, dq, st);
}

void launch_lusgs1(int jmax, int kmax, const double* stc, const double* sjm, const double* sjp, const double* skm,
                   const double* skp, double* bprm, double* rhs, double* ds, cudaStream_t st) {
  size_t N = (size_t)jmax * kmax;
  ++g_kernel_launches;
  k_lusini1<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(stc, bprm, N);
  ilu_sweeps<1>(jmax, kmax, bprm, sjm, skm, sjp, skp, rhs, ds, st);
}

}  // namespace smac
