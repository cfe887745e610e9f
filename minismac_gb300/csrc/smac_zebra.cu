// smac_zebra.cu -- throughput forms of the implicit solve: zebra (two-colour) line relaxation
// in FP64 or FP32, and the FP32 copy of the implicit operator for mixed-precision defect
// correction.
//
// The reference relaxes the lines of a sweep one after the other (ref/lrelax.f:225-561).  The
// zebra order relaxes all even lines at once, then all odd lines with the new even values; it
// has the same fixed point (s = 0) and a different iteration history.  Each line is solved by
// one warp: the 32 lanes own consecutive segments, run the block-tridiagonal recurrences of
// their segment with a zero carry-in, combine the segment (transfer, value) pairs with a
// Kogge-Stone scan composed on the fly, and re-run the segment from the true carry-in.
//
// Mixed precision: the FP64 residual s is what the iteration drives to zero; the implicit
// operator (blocks, factorisation, line solves) only has to approximate its Jacobian, so it is
// kept in FP32 (half the bytes, 58x the FP64 issue rate on GB300).  q += dq stays in FP64.
#include <math.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

namespace smac {

// ------------------------------------------------------------------------------ FP32 operator
// btc -> two copies (one factored along j, one along k); bjp and bkp -> a copy to factor and the
// original (the other direction's sweeps read it while this one is factored)
__global__ void k_to_f32(const double* __restrict__ btc, const double* __restrict__ bjm,
                         const double* __restrict__ bjp, const double* __restrict__ bkm,
                         const double* __restrict__ bkp, const double* __restrict__ s, F32Ops o, size_t N) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int e = 0; e < 9; ++e) {
    size_t k = i + N * e;
    float b = (float)btc[k];
    o.btc_j[k] = b;
    o.btc_k[k] = b;
    o.bjm[k] = (float)bjm[k];
    float p = (float)bjp[k];
    o.bjp_f[k] = p;
    o.bjp_o[k] = p;
    o.bkm[k] = (float)bkm[k];
    float kp = (float)bkp[k];
    o.bkp[k] = kp;
    o.bkp_o[k] = kp;
  }
  for (int q = 0; q < 3; ++q) o.s[i + N * q] = (float)s[i + N * q];
}

// ------------------------------------------------------------------------------ factorisation
template <typename T>
__device__ __forceinline__ void blu_t(T* b) {
  b[0] = T(1) / b[0];
  b[3] = b[3] * b[0];
  b[6] = b[6] * b[0];
  b[4] = T(1) / (b[4] - b[1] * b[3]);
  b[7] = (b[7] - b[1] * b[6]) * b[4];
  b[5] = b[5] - b[2] * b[3];
  b[8] = T(1) / (b[8] - b[2] * b[6] - b[7] * b[5]);
}
template <typename T>
__device__ __forceinline__ void lu_t(const T* B, T& x1, T& x2, T& x3) {
  T d1 = B[0] * x1;
  T d2 = B[4] * (x2 - B[1] * d1);
  T d3 = B[8] * (x3 - B[2] * d1 - B[5] * d2);
  x3 = d3;
  x2 = d2 - B[7] * x3;
  x1 = d1 - B[6] * x3 - B[3] * x2;
}

// ------------------------------------------------------------------------------ zebra sweep
template <typename T>
__device__ __forceinline__ void mm_t(const T* A, const T* B, T* C) {
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) C[r + 3 * c] = A[r] * B[3 * c] + A[r + 3] * B[1 + 3 * c] + A[r + 6] * B[2 + 3 * c];
}

// LPW lines of the given colour per warp, G = 32 / LPW lanes per line (the autotuner picks LPW
// per direction and grid).  W: working precision of the operator and of dq.
template <int DIR, typename W, typename S, int LPW>
__global__ void __launch_bounds__(128) k_zebra(ZebraArgs<W, S> a, int color) {
  constexpr int G = 32 / LPW;
  constexpr int LEV = G == 32 ? 5 : G == 16 ? 4 : G == 8 ? 3 : 2;
  const int jmax = a.jmax, kmax = a.kmax;
  const size_t N = a.N;
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const int wlane = threadIdx.x & 31;
  const int lane = wlane % G;  // lane within the line's group
  const int line_idx = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * LPW + wlane / G;
  const int l_want = 2 * line_idx + color;
  if (2 * (((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * LPW) + color >= nl) return;  // whole warp
  const bool live = l_want < nl;  // groups past the last line run the shuffles and store nothing
  const int l = live ? l_want : color;
  const int L = (n + G - 1) / G;
  const int beg = lane * L;
  const int cnt = (live && beg < n) ? min(n, beg + L) - beg : 0;
  const int lm = l - 1 > 0 ? l - 1 : 0;
  const int lp = l + 1 < nl - 1 ? l + 1 : nl - 1;
  const W half = W(0.5);
  const W swm = half + copysign(half, (W)(l - 1 - lm));
  const W swp = half + copysign(half, (W)(lp - l - 1));
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  auto PM = [&](int i) -> size_t { return DIR == 0 ? ix(i, lm, jmax) : ix(lm, i, jmax); };
  auto PP = [&](int i) -> size_t { return DIR == 0 ? ix(i, lp, jmax) : ix(lp, i, jmax); };
  W* rb = a.work;  // right-hand sides, then forward values
  // pass 1: right-hand sides, local forward recurrence, segment transfer
  W y[3] = {W(0), W(0), W(0)};
  W F[9];
  for (int e = 0; e < 9; ++e) F[e] = W(0);
  F[0] = F[4] = F[8] = W(1);
  for (int t = 0; t < cnt; ++t) {
    int i = beg + t;
    size_t id = P(i), im = PM(i), ip = PP(i);
    W d1 = a.dq[im], d2 = a.dq[im + N], d3 = a.dq[im + 2 * N];
    W e1 = a.dq[ip], e2 = a.dq[ip + N], e3 = a.dq[ip + 2 * N];
    W r[3];
    for (int q = 0; q < 3; ++q) {
      r[q] = (W)a.s[id + N * q] -
             (a.om[id + N * q] * d1 + a.om[id + N * (q + 3)] * d2 + a.om[id + N * (q + 6)] * d3) * swm -
             (a.op[id + N * q] * e1 + a.op[id + N * (q + 3)] * e2 + a.op[id + N * (q + 6)] * e3) * swp;
      rb[id + N * q] = r[q];
    }
    W B[9], A[9];
    for (int e = 0; e < 9; ++e) B[e] = a.btc[id + N * e];
    W x1 = r[0], x2 = r[1], x3 = r[2];
    if (i > 0) {
      for (int e = 0; e < 9; ++e) A[e] = a.am[id + N * e];
      if (t > 0) {
        x1 = x1 - A[0] * y[0] - A[3] * y[1] - A[6] * y[2];
        x2 = x2 - A[1] * y[0] - A[4] * y[1] - A[7] * y[2];
        x3 = x3 - A[2] * y[0] - A[5] * y[1] - A[8] * y[2];
      }
      // M = -B'^-1 A ; F = M F
      W M[9], T9[9];
      for (int col = 0; col < 3; ++col) {
        W m1 = A[3 * col], m2 = A[1 + 3 * col], m3 = A[2 + 3 * col];
        lu_t(B, m1, m2, m3);
        M[3 * col] = -m1; M[1 + 3 * col] = -m2; M[2 + 3 * col] = -m3;
      }
      mm_t(M, F, T9);
      for (int e = 0; e < 9; ++e) F[e] = T9[e];
    } else {
      for (int e = 0; e < 9; ++e) F[e] = W(0);
    }
    lu_t(B, x1, x2, x3);
    y[0] = x1; y[1] = x2; y[2] = x3;
  }
  if (cnt == 0) { for (int e = 0; e < 9; ++e) F[e] = W(0); }
  // forward scan over the lanes, (transfer, value) composed on the fly
  for (int d = 0; d < LEV; ++d) {
    const int o = 1 << d;
    W vn[3], Fn[9];
    for (int q = 0; q < 3; ++q) vn[q] = __shfl_up_sync(0xffffffffu, y[q], o, G);
    for (int e = 0; e < 9; ++e) Fn[e] = __shfl_up_sync(0xffffffffu, F[e], o, G);
    if (lane >= o) {
      for (int q = 0; q < 3; ++q) y[q] = y[q] + (F[q] * vn[0] + F[q + 3] * vn[1] + F[q + 6] * vn[2]);
      W T9[9];
      mm_t(F, Fn, T9);
      for (int e = 0; e < 9; ++e) F[e] = T9[e];
    }
  }
  W yin[3];
  for (int q = 0; q < 3; ++q) {
    yin[q] = __shfl_up_sync(0xffffffffu, y[q], 1, G);
    if (lane == 0) yin[q] = W(0);
  }
  // pass 2: forward recurrence from the true carry-in; y stored over the right-hand sides
  for (int q = 0; q < 3; ++q) y[q] = yin[q];
  for (int t = 0; t < cnt; ++t) {
    int i = beg + t;
    size_t id = P(i);
    W x1 = rb[id], x2 = rb[id + N], x3 = rb[id + 2 * N];
    if (i > 0) {
      const W* A = a.am;
      W z1 = x1 - A[id] * y[0] - A[id + 3 * N] * y[1] - A[id + 6 * N] * y[2];
      W z2 = x2 - A[id + N] * y[0] - A[id + 4 * N] * y[1] - A[id + 7 * N] * y[2];
      W z3 = x3 - A[id + 2 * N] * y[0] - A[id + 5 * N] * y[1] - A[id + 8 * N] * y[2];
      x1 = z1; x2 = z2; x3 = z3;
    }
    W B[9];
    for (int e = 0; e < 9; ++e) B[e] = a.btc[id + N * e];
    lu_t(B, x1, x2, x3);
    y[0] = x1; y[1] = x2; y[2] = x3;
    rb[id] = x1; rb[id + N] = x2; rb[id + 2 * N] = x3;
  }
  // pass 3: local backward recurrence, segment transfer H_b ... H_e (H_i = -c_i, H_{n-1} = 0)
  W x[3] = {W(0), W(0), W(0)};
  W Gm[9];
  for (int e = 0; e < 9; ++e) Gm[e] = W(0);
  Gm[0] = Gm[4] = Gm[8] = W(1);
  for (int t = cnt - 1; t >= 0; --t) {
    int i = beg + t;
    size_t id = P(i);
    W x1 = rb[id], x2 = rb[id + N], x3 = rb[id + 2 * N];
    if (i < n - 1) {
      W C[9];
      for (int e = 0; e < 9; ++e) C[e] = a.cp[id + N * e];
      if (t < cnt - 1) {
        x1 = x1 - C[0] * x[0] - C[3] * x[1] - C[6] * x[2];
        x2 = x2 - C[1] * x[0] - C[4] * x[1] - C[7] * x[2];
        x3 = x3 - C[2] * x[0] - C[5] * x[1] - C[8] * x[2];
      }
      W H[9], T9[9];
      for (int e = 0; e < 9; ++e) H[e] = -C[e];
      mm_t(H, Gm, T9);
      for (int e = 0; e < 9; ++e) Gm[e] = T9[e];
    } else {
      for (int e = 0; e < 9; ++e) Gm[e] = W(0);
    }
    x[0] = x1; x[1] = x2; x[2] = x3;
  }
  if (cnt == 0) { for (int e = 0; e < 9; ++e) Gm[e] = W(0); }
  for (int d = 0; d < LEV; ++d) {
    const int o = 1 << d;
    W vn[3], Gn[9];
    for (int q = 0; q < 3; ++q) vn[q] = __shfl_down_sync(0xffffffffu, x[q], o, G);
    for (int e = 0; e < 9; ++e) Gn[e] = __shfl_down_sync(0xffffffffu, Gm[e], o, G);
    if (lane + o <= G - 1) {
      for (int q = 0; q < 3; ++q) x[q] = x[q] + (Gm[q] * vn[0] + Gm[q + 3] * vn[1] + Gm[q + 6] * vn[2]);
      W T9[9];
      mm_t(Gm, Gn, T9);
      for (int e = 0; e < 9; ++e) Gm[e] = T9[e];
    }
  }
  W xin[3];
  for (int q = 0; q < 3; ++q) {
    xin[q] = __shfl_down_sync(0xffffffffu, x[q], 1, G);
    if (lane == G - 1) xin[q] = W(0);
  }
  // pass 4: backward recurrence from the true carry-in and the relaxation update
  for (int q = 0; q < 3; ++q) x[q] = xin[q];
  for (int t = cnt - 1; t >= 0; --t) {
    int i = beg + t;
    size_t id = P(i);
    W x1 = rb[id], x2 = rb[id + N], x3 = rb[id + 2 * N];
    if (i < n - 1) {
      const W* C = a.cp;
      x1 = x1 - C[id] * x[0] - C[id + 3 * N] * x[1] - C[id + 6 * N] * x[2];
      x2 = x2 - C[id + N] * x[0] - C[id + 4 * N] * x[1] - C[id + 7 * N] * x[2];
      x3 = x3 - C[id + 2 * N] * x[0] - C[id + 5 * N] * x[1] - C[id + 8 * N] * x[2];
    }
    x[0] = x1; x[1] = x2; x[2] = x3;
    for (int q = 0; q < 3; ++q) {
      W o = a.dq[id + N * q];
      a.dq[id + N * q] = o + a.underr * (x[q] - o);
    }
  }
}

// The same line solve with WPL warps per line (one CTA per line, 32 WPL segments): for long
// lines a warp per line leaves each lane a chain of n/32 dependent points whose operands miss
// in L1; WPL warps shorten the chains WPL times and put WPL times the warps on the SMs.  The
// segment scans run inside each warp as above; the warps' aggregates are combined through
// shared memory (at most three compositions per warp).
// line l of a's grid, by the whole CTA (32 WPL threads)
template <int DIR, typename W, typename S, int WPL>
__device__ __forceinline__ void zebra_wide_line(const ZebraArgs<W, S>& a, int l) {
  __shared__ W sF[WPL][9], sy[WPL][3], sG[WPL][9], sx[WPL][3];
  const int jmax = a.jmax, kmax = a.kmax;
  const size_t N = a.N;
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const int lane = threadIdx.x, wl = lane & 31, wi = lane >> 5;
  const int L = (n + 32 * WPL - 1) / (32 * WPL);
  const int beg = lane * L;
  const int cnt = beg < n ? min(n, beg + L) - beg : 0;
  const int lm = l - 1 > 0 ? l - 1 : 0;
  const int lp = l + 1 < nl - 1 ? l + 1 : nl - 1;
  const W half = W(0.5);
  const W swm = half + copysign(half, (W)(l - 1 - lm));
  const W swp = half + copysign(half, (W)(lp - l - 1));
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  auto PM = [&](int i) -> size_t { return DIR == 0 ? ix(i, lm, jmax) : ix(lm, i, jmax); };
  auto PP = [&](int i) -> size_t { return DIR == 0 ? ix(i, lp, jmax) : ix(lp, i, jmax); };
  W* rb = a.work;
  // pass 1: right-hand sides, local forward recurrence from a zero carry, segment transfer
  W y[3] = {W(0), W(0), W(0)};
  W F[9];
  for (int e = 0; e < 9; ++e) F[e] = W(0);
  F[0] = F[4] = F[8] = W(1);
  for (int t = 0; t < cnt; ++t) {
    int i = beg + t;
    size_t id = P(i), im = PM(i), ip = PP(i);
    W d1 = a.dq[im], d2 = a.dq[im + N], d3 = a.dq[im + 2 * N];
    W e1 = a.dq[ip], e2 = a.dq[ip + N], e3 = a.dq[ip + 2 * N];
    W r[3];
    for (int q = 0; q < 3; ++q) {
      r[q] = (W)a.s[id + N * q] -
             (a.om[id + N * q] * d1 + a.om[id + N * (q + 3)] * d2 + a.om[id + N * (q + 6)] * d3) * swm -
             (a.op[id + N * q] * e1 + a.op[id + N * (q + 3)] * e2 + a.op[id + N * (q + 6)] * e3) * swp;
      rb[id + N * q] = r[q];
    }
    W B[9], A[9];
    for (int e = 0; e < 9; ++e) B[e] = a.btc[id + N * e];
    W x1 = r[0], x2 = r[1], x3 = r[2];
    if (i > 0) {
      for (int e = 0; e < 9; ++e) A[e] = a.am[id + N * e];
      if (t > 0) {
        x1 = x1 - A[0] * y[0] - A[3] * y[1] - A[6] * y[2];
        x2 = x2 - A[1] * y[0] - A[4] * y[1] - A[7] * y[2];
        x3 = x3 - A[2] * y[0] - A[5] * y[1] - A[8] * y[2];
      }
      W M[9], T9[9];
      for (int col = 0; col < 3; ++col) {
        W m1 = A[3 * col], m2 = A[1 + 3 * col], m3 = A[2 + 3 * col];
        lu_t(B, m1, m2, m3);
        M[3 * col] = -m1; M[1 + 3 * col] = -m2; M[2 + 3 * col] = -m3;
      }
      mm_t(M, F, T9);
      for (int e = 0; e < 9; ++e) F[e] = T9[e];
    } else {
      for (int e = 0; e < 9; ++e) F[e] = W(0);
    }
    lu_t(B, x1, x2, x3);
    y[0] = x1; y[1] = x2; y[2] = x3;
  }
  if (cnt == 0) { for (int e = 0; e < 9; ++e) F[e] = W(0); }
  // forward scan inside the warp
  for (int d = 0; d < 5; ++d) {
    const int o = 1 << d;
    W vn[3], Fn[9];
    for (int q = 0; q < 3; ++q) vn[q] = __shfl_up_sync(0xffffffffu, y[q], o);
    for (int e = 0; e < 9; ++e) Fn[e] = __shfl_up_sync(0xffffffffu, F[e], o);
    if (wl >= o) {
      for (int q = 0; q < 3; ++q) y[q] = y[q] + (F[q] * vn[0] + F[q + 3] * vn[1] + F[q + 6] * vn[2]);
      W T9[9];
      mm_t(F, Fn, T9);
      for (int e = 0; e < 9; ++e) F[e] = T9[e];
    }
  }
  // carry into this warp: the warps before it, folded in order
  if (wl == 31) {
    for (int e = 0; e < 9; ++e) sF[wi][e] = F[e];
    for (int q = 0; q < 3; ++q) sy[wi][q] = y[q];
  }
  __syncthreads();
  W cw[3] = {W(0), W(0), W(0)};
  for (int v = 0; v < wi; ++v) {
    W c0 = sy[v][0] + sF[v][0] * cw[0] + sF[v][3] * cw[1] + sF[v][6] * cw[2];
    W c1 = sy[v][1] + sF[v][1] * cw[0] + sF[v][4] * cw[1] + sF[v][7] * cw[2];
    W c2 = sy[v][2] + sF[v][2] * cw[0] + sF[v][5] * cw[1] + sF[v][8] * cw[2];
    cw[0] = c0; cw[1] = c1; cw[2] = c2;
  }
  W yin[3];
  {
    W yp[3], Fp[9];
    for (int q = 0; q < 3; ++q) yp[q] = __shfl_up_sync(0xffffffffu, y[q], 1);
    for (int e = 0; e < 9; ++e) Fp[e] = __shfl_up_sync(0xffffffffu, F[e], 1);
    for (int q = 0; q < 3; ++q)
      yin[q] = wl == 0 ? cw[q] : yp[q] + (Fp[q] * cw[0] + Fp[q + 3] * cw[1] + Fp[q + 6] * cw[2]);
  }
  // pass 2: forward recurrence from the true carry-in; y stored over the right-hand sides
  for (int q = 0; q < 3; ++q) y[q] = yin[q];
  for (int t = 0; t < cnt; ++t) {
    int i = beg + t;
    size_t id = P(i);
    W x1 = rb[id], x2 = rb[id + N], x3 = rb[id + 2 * N];
    if (i > 0) {
      const W* A = a.am;
      W z1 = x1 - A[id] * y[0] - A[id + 3 * N] * y[1] - A[id + 6 * N] * y[2];
      W z2 = x2 - A[id + N] * y[0] - A[id + 4 * N] * y[1] - A[id + 7 * N] * y[2];
      W z3 = x3 - A[id + 2 * N] * y[0] - A[id + 5 * N] * y[1] - A[id + 8 * N] * y[2];
      x1 = z1; x2 = z2; x3 = z3;
    }
    W B[9];
    for (int e = 0; e < 9; ++e) B[e] = a.btc[id + N * e];
    lu_t(B, x1, x2, x3);
    y[0] = x1; y[1] = x2; y[2] = x3;
    rb[id] = x1; rb[id + N] = x2; rb[id + 2 * N] = x3;
  }
  // pass 3: local backward recurrence from a zero carry, segment transfer
  W x[3] = {W(0), W(0), W(0)};
  W Gm[9];
  for (int e = 0; e < 9; ++e) Gm[e] = W(0);
  Gm[0] = Gm[4] = Gm[8] = W(1);
  for (int t = cnt - 1; t >= 0; --t) {
    int i = beg + t;
    size_t id = P(i);
    W x1 = rb[id], x2 = rb[id + N], x3 = rb[id + 2 * N];
    if (i < n - 1) {
      W C[9];
      for (int e = 0; e < 9; ++e) C[e] = a.cp[id + N * e];
      if (t < cnt - 1) {
        x1 = x1 - C[0] * x[0] - C[3] * x[1] - C[6] * x[2];
        x2 = x2 - C[1] * x[0] - C[4] * x[1] - C[7] * x[2];
        x3 = x3 - C[2] * x[0] - C[5] * x[1] - C[8] * x[2];
      }
      W H[9], T9[9];
      for (int e = 0; e < 9; ++e) H[e] = -C[e];
      mm_t(H, Gm, T9);
      for (int e = 0; e < 9; ++e) Gm[e] = T9[e];
    } else {
      for (int e = 0; e < 9; ++e) Gm[e] = W(0);
    }
    x[0] = x1; x[1] = x2; x[2] = x3;
  }
  if (cnt == 0) { for (int e = 0; e < 9; ++e) Gm[e] = W(0); }
  // backward scan inside the warp
  for (int d = 0; d < 5; ++d) {
    const int o = 1 << d;
    W vn[3], Gn[9];
    for (int q = 0; q < 3; ++q) vn[q] = __shfl_down_sync(0xffffffffu, x[q], o);
    for (int e = 0; e < 9; ++e) Gn[e] = __shfl_down_sync(0xffffffffu, Gm[e], o);
    if (wl + o <= 31) {
      for (int q = 0; q < 3; ++q) x[q] = x[q] + (Gm[q] * vn[0] + Gm[q + 3] * vn[1] + Gm[q + 6] * vn[2]);
      W T9[9];
      mm_t(Gm, Gn, T9);
      for (int e = 0; e < 9; ++e) Gm[e] = T9[e];
    }
  }
  // carry into this warp from the right: the warps after it, folded from the last
  if (wl == 0) {
    for (int e = 0; e < 9; ++e) sG[wi][e] = Gm[e];
    for (int q = 0; q < 3; ++q) sx[wi][q] = x[q];
  }
  __syncthreads();
  W cb[3] = {W(0), W(0), W(0)};
  for (int v = WPL - 1; v > wi; --v) {
    W c0 = sx[v][0] + sG[v][0] * cb[0] + sG[v][3] * cb[1] + sG[v][6] * cb[2];
    W c1 = sx[v][1] + sG[v][1] * cb[0] + sG[v][4] * cb[1] + sG[v][7] * cb[2];
    W c2 = sx[v][2] + sG[v][2] * cb[0] + sG[v][5] * cb[1] + sG[v][8] * cb[2];
    cb[0] = c0; cb[1] = c1; cb[2] = c2;
  }
  W xin[3];
  {
    W xn[3], Gn[9];
    for (int q = 0; q < 3; ++q) xn[q] = __shfl_down_sync(0xffffffffu, x[q], 1);
    for (int e = 0; e < 9; ++e) Gn[e] = __shfl_down_sync(0xffffffffu, Gm[e], 1);
    for (int q = 0; q < 3; ++q)
      xin[q] = wl == 31 ? cb[q] : xn[q] + (Gn[q] * cb[0] + Gn[q + 3] * cb[1] + Gn[q + 6] * cb[2]);
  }
  // pass 4: backward recurrence from the true carry-in and the relaxation update
  for (int q = 0; q < 3; ++q) x[q] = xin[q];
  for (int t = cnt - 1; t >= 0; --t) {
    int i = beg + t;
    size_t id = P(i);
    W x1 = rb[id], x2 = rb[id + N], x3 = rb[id + 2 * N];
    if (i < n - 1) {
      const W* C = a.cp;
      x1 = x1 - C[id] * x[0] - C[id + 3 * N] * x[1] - C[id + 6 * N] * x[2];
      x2 = x2 - C[id + N] * x[0] - C[id + 4 * N] * x[1] - C[id + 7 * N] * x[2];
      x3 = x3 - C[id + 2 * N] * x[0] - C[id + 5 * N] * x[1] - C[id + 8 * N] * x[2];
    }
    x[0] = x1; x[1] = x2; x[2] = x3;
    for (int q = 0; q < 3; ++q) {
      W o = a.dq[id + N * q];
      a.dq[id + N * q] = o + a.underr * (x[q] - o);
    }
  }
}

template <int DIR, typename W, typename S, int WPL>
__global__ void __launch_bounds__(32 * WPL) k_zebra_wide(ZebraArgs<W, S> a, int color) {
  const int nl = DIR == 0 ? a.kmax : a.jmax;
  const int l = 2 * blockIdx.x + color;
  if (l >= nl) return;  // the whole CTA
  zebra_wide_line<DIR, W, S, WPL>(a, l);
}

// The lines of one colour of every case of a batch in one launch: CTA b solves line
// 2 (b - start[c]) + color of case c, start[c] <= b < start[c+1] (a prefix of the cases' line
// counts), with the case's operator, right-hand side and dq.
template <int DIR, int WPL>
__global__ void __launch_bounds__(32 * WPL) k_zebra_packed(const ZebraArgs<float, float>* __restrict__ args,
                                                           const int* __restrict__ start, int ncases, int color) {
  const int b = blockIdx.x;
  int lo = 0, hi = ncases - 1;  // the case whose range holds b
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  const ZebraArgs<float, float> a = args[lo];
  const int nl = DIR == 0 ? a.kmax : a.jmax;
  const int l = 2 * (b - start[lo]) + color;
  if (l >= nl) return;
  zebra_wide_line<DIR, float, float, WPL>(a, l);
}

void launch_zebra_packed(int dir, const ZebraArgs<float, float>* args, const int* start, int ncases, int nblocks,
                         int color, int wpl, cudaStream_t st) {
  if (nblocks <= 0) return;
  ++g_kernel_launches;
  if (dir == 0 && wpl == 4) k_zebra_packed<0, 4><<<nblocks, 128, 0, st>>>(args, start, ncases, color);
  else if (dir == 0) k_zebra_packed<0, 2><<<nblocks, 64, 0, st>>>(args, start, ncases, color);
  else if (wpl == 4) k_zebra_packed<1, 4><<<nblocks, 128, 0, st>>>(args, start, ncases, color);
  else k_zebra_packed<1, 2><<<nblocks, 64, 0, st>>>(args, start, ncases, color);
}

template <typename W, typename S>
void launch_zebra(int dir, const ZebraArgs<W, S>& a, int color, cudaStream_t st, int lpw) {
  int nl = dir == 0 ? a.kmax : a.jmax;
  int lines = (nl - color + 1) / 2;
  if (lines <= 0) return;
  if (lpw == -2 || lpw == -4) {  // warps per line
    ++g_kernel_launches;
    if (dir == 0 && lpw == -2) k_zebra_wide<0, W, S, 2><<<lines, 64, 0, st>>>(a, color);
    else if (dir == 0) k_zebra_wide<0, W, S, 4><<<lines, 128, 0, st>>>(a, color);
    else if (lpw == -2) k_zebra_wide<1, W, S, 2><<<lines, 64, 0, st>>>(a, color);
    else k_zebra_wide<1, W, S, 4><<<lines, 128, 0, st>>>(a, color);
    return;
  }
  if (lpw != 2 && lpw != 4) lpw = 1;
  int warps = (lines + lpw - 1) / lpw;
  int blocks = (warps + 3) / 4;
  ++g_kernel_launches;
  if (dir == 0) {
    if (lpw == 1) k_zebra<0, W, S, 1><<<blocks, 128, 0, st>>>(a, color);
    else if (lpw == 2) k_zebra<0, W, S, 2><<<blocks, 128, 0, st>>>(a, color);
    else k_zebra<0, W, S, 4><<<blocks, 128, 0, st>>>(a, color);
  } else {
    if (lpw == 1) k_zebra<1, W, S, 1><<<blocks, 128, 0, st>>>(a, color);
    else if (lpw == 2) k_zebra<1, W, S, 2><<<blocks, 128, 0, st>>>(a, color);
    else k_zebra<1, W, S, 4><<<blocks, 128, 0, st>>>(a, color);
  }
}

template void launch_zebra<double, double>(int, const ZebraArgs<double, double>&, int, cudaStream_t, int);
template void launch_zebra<float, float>(int, const ZebraArgs<float, float>&, int, cudaStream_t, int);

void launch_to_f32(const double* btc, const double* bjm, const double* bjp, const double* bkm, const double* bkp,
                   const double* s, const F32Ops& o, size_t N, cudaStream_t st) {
  ++g_kernel_launches;
  k_to_f32<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(btc, bjm, bjp, bkm, bkp, s, o, N);
}

// FP32 factorisation with three lanes per line (lane m: column m of the blocks), as the FP64
// k_btlu_lanes: three times the lines in flight of a thread-per-line walk and a third of the
// loads per lane, which is what bounds this memory-latency-bound walk.
constexpr int kLinesPerWarpF32 = 10;

template <int DIR>
__global__ void __launch_bounds__(32) k_btlu_lanes_f32(const float* __restrict__ a, float* __restrict__ b,
                                                       float* __restrict__ c, int jmax, int kmax) {
  // The step along the line is a short FP32 chain; the operands of each point come from L2
  // (written by the assembly just before), so they are loaded kPF points ahead into a register
  // ring (the ring index is a compile-time constant of the unrolled inner loop).
  constexpr int kPF = 3;
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const int lane = threadIdx.x;
  const int slot = lane / 3, m = lane - 3 * (lane / 3);
  const int l0 = blockIdx.x * kLinesPerWarpF32 + slot;
  const bool act = lane < 3 * kLinesPerWarpF32 && l0 < nl;
  const int l = act ? l0 : 0;
  const int src = 3 * (lane < 3 * kLinesPerWarpF32 ? slot : 0);
  const size_t N = (size_t)jmax * kmax;
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  float cprev[3] = {0.f, 0.f, 0.f};
  float Bq[kPF][3], Aq[kPF][9], Cq[kPF][3];
  auto load = [&](int i, float* Bn, float* An, float* Cn) {
    if (i >= n) return;
    size_t in = P(i);
    for (int r = 0; r < 3; ++r) Bn[r] = b[in + N * (r + 3 * m)];
    for (int e = 0; e < 9; ++e) An[e] = i > 0 ? a[in + N * e] : 0.f;
    for (int r = 0; r < 3; ++r) Cn[r] = c[in + N * (r + 3 * m)];
  };
#pragma unroll
  for (int q = 0; q < kPF; ++q) load(q, Bq[q], Aq[q], Cq[q]);
  for (int i0 = 0; i0 < n; i0 += kPF) {
#pragma unroll
    for (int q = 0; q < kPF; ++q) {
      const int i = i0 + q;
      if (i >= n) break;
      const size_t id = P(i);
      float Bc[3], A[9], Cc[3];
      for (int r = 0; r < 3; ++r) { Bc[r] = Bq[q][r]; Cc[r] = Cq[q][r]; }
      for (int e = 0; e < 9; ++e) A[e] = Aq[q][e];
      load(i + kPF, Bq[q], Aq[q], Cq[q]);
      if (i > 0)
        for (int r = 0; r < 3; ++r) Bc[r] = Bc[r] - A[r + 0] * cprev[0] - A[r + 3] * cprev[1] - A[r + 6] * cprev[2];
      float B[9];
      for (int mm = 0; mm < 3; ++mm)
        for (int r = 0; r < 3; ++r) B[r + 3 * mm] = __shfl_sync(0xffffffffu, Bc[r], src + mm);
      blu_t(B);
      if (act)
        for (int r = 0; r < 3; ++r) b[id + N * (r + 3 * m)] = m == 0 ? B[r] : (m == 1 ? B[r + 3] : B[r + 6]);
      if (i < n - 1) {
        float x1 = Cc[0], x2 = Cc[1], x3 = Cc[2];
        lu_t(B, x1, x2, x3);
        Cc[0] = x1; Cc[1] = x2; Cc[2] = x3;
        if (act)
          for (int r = 0; r < 3; ++r) c[id + N * (r + 3 * m)] = Cc[r];
        for (int r = 0; r < 3; ++r) cprev[r] = Cc[r];
      }
    }
  }
}

void launch_btlu_f32(int dir, const float* a, float* b, float* c, int jmax, int kmax, cudaStream_t st) {
  int nl = dir == 0 ? kmax : jmax;
  int nb = (nl + kLinesPerWarpF32 - 1) / kLinesPerWarpF32;
  ++g_kernel_launches;
  if (dir == 0) k_btlu_lanes_f32<0><<<nb, 32, 0, st>>>(a, b, c, jmax, kmax);
  else k_btlu_lanes_f32<1><<<nb, 32, 0, st>>>(a, b, c, jmax, kmax);
}

// FP32 wake-cut injection on the FP32 dq and right-hand side (bcimpds, ref/bc.f:566-595)
__global__ void k_bcimpds_f32(const BCTable* __restrict__ bc, int jmax, size_t N, const double* __restrict__ q,
                              float* __restrict__ dq, float* __restrict__ rhs) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  for (int r = 0; r < bc->nwake; ++r) {
    int len = bc->jt_e[r] - bc->jt_b[r] + 1;
    if (t >= len * 3) { t -= len * 3; continue; }
    int off = t / 3, neq = t % 3;
    int jt = bc->jt_b[r] + off;
    int jb = bc->jb_b[r] - off;
    size_t n0 = N * neq;
    double snew = 0.5 * (q[ix(jt, 1, jmax) + n0] + q[ix(jb, 1, jmax) + n0]);
    double dsnew = 0.5 * ((double)dq[ix(jt, 1, jmax) + n0] + (double)dq[ix(jb, 1, jmax) + n0]);
    float v = (float)(snew + dsnew - q[ix(jt, 0, jmax) + n0]);
    dq[ix(jt, 0, jmax) + n0] = v;
    rhs[ix(jt, 0, jmax) + n0] = v;
    return;
  }
}

void launch_bcimpds_f32(const BCTable* bc, int jmax, size_t N, const double* q, float* dq, float* rhs,
                        cudaStream_t st) {
  ++g_kernel_launches;
  k_bcimpds_f32<<<(2 * jmax * 3 + 127) / 128, 128, 0, st>>>(bc, jmax, N, q, dq, rhs);
}

// the wake-cut injection of one case of a batch, elements t0, t0 + stride, ...
__device__ __forceinline__ void bcimp_case(const BcimpArgs& a, int t0, int stride) {
  for (int t = t0; t < 2 * a.jmax * 3; t += stride) {
    int u = t;
    for (int r = 0; r < a.bc->nwake; ++r) {
      int len = a.bc->jt_e[r] - a.bc->jt_b[r] + 1;
      if (u >= len * 3) { u -= len * 3; continue; }
      int off = u / 3, neq = u % 3;
      int jt = a.bc->jt_b[r] + off;
      int jb = a.bc->jb_b[r] - off;
      size_t n0 = a.N * neq;
      double snew = 0.5 * (a.q[ix(jt, 1, a.jmax) + n0] + a.q[ix(jb, 1, a.jmax) + n0]);
      double dsnew = 0.5 * ((double)a.dq[ix(jt, 1, a.jmax) + n0] + (double)a.dq[ix(jb, 1, a.jmax) + n0]);
      float v = (float)(snew + dsnew - a.q[ix(jt, 0, a.jmax) + n0]);
      a.dq[ix(jt, 0, a.jmax) + n0] = v;
      a.rhs[ix(jt, 0, a.jmax) + n0] = v;
      break;
    }
  }
}

// the same for every case of a batch: blockIdx.y is the case
__global__ void k_bcimpds_f32_packed(const BcimpArgs* __restrict__ args) {
  const BcimpArgs a = args[blockIdx.y];
  bcimp_case(a, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

void launch_bcimpds_f32_packed(const BcimpArgs* args, int ncases, int max_jmax, cudaStream_t st) {
  ++g_kernel_launches;
  k_bcimpds_f32_packed<<<dim3((unsigned)((2 * max_jmax * 3 + 127) / 128), (unsigned)ncases), 128, 0, st>>>(args);
}

// ------------------------------------------------------------------------------ line work queue
// The line sweeps of one FP32-operator zebra iteration of every case of a batch (every sweep
// colour of both directions and the wake-cut injections) in one persistent launch.  The work is
// a queue of items (one line to sweep, one case's wake-cut injection) cut into phases; a phase
// belongs to one case and may start when the previous phase of that case is complete.  CTAs
// take items in queue order from a counter, wait for the item's phase dependency, do the item
// and count it done.  Every phase comes after its dependency in the queue, so an item is only
// ever waited for by items taken after it, and the item with the lowest index not done has
// nothing left to wait for: the queue empties for any number of resident CTAs.  Waits are
// bounded; one that runs out records SMAC_ERR_TIMEOUT in *status, after which no CTA waits any
// more and the launch finishes.
constexpr unsigned long long kQueueWaitNs = 1000000000ull;

__device__ __forceinline__ unsigned long long queue_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// one thread: until `target` items of phase ph are done (ph < 0: nothing to wait for)
__device__ __noinline__ void queue_wait(const QueueArgs& q, int ph, int target) {
  if (ph < 0) return;
  if (ld_acquire(q.done + ph) >= target) return;
  const unsigned long long t0 = queue_ns();
  for (;;) {
    if (ld_acquire(q.done + ph) >= target) return;
    if (ld_relaxed(q.status) != 0) return;  // a wait ran out: finish without waiting
    if (queue_ns() - t0 > kQueueWaitNs) {
      atomicCAS(q.status, 0, SMAC_ERR_TIMEOUT);
      return;
    }
    __nanosleep(200);
  }
}

template <int WPL>
__global__ void __launch_bounds__(32 * WPL) k_lines_queue(QueueArgs q) {
  __shared__ int s_item, s_ph;
  for (;;) {
    if (threadIdx.x == 0) {
      const int item = atomicAdd(q.head, 1);
      int ph = -1;
      if (item < q.nitems) {
        int lo = 0, hi = q.nphases - 1;  // the phase holding the item
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (q.phases[mid].first <= item) lo = mid;
          else hi = mid - 1;
        }
        ph = lo;
        // a host-requested stall (tests of the bounded waits): the first item also waits for
        // one item more than its own phase will ever count
        if (item == 0 && ld_relaxed(q.stall) != 0 && atomicExch(q.stall, 0) != 0)
          queue_wait(q, ph, q.phases[ph].nitems + 1);
        const int dep = q.phases[ph].dep;
        if (dep >= 0) queue_wait(q, dep, q.phases[dep].nitems);
      }
      s_item = item;
      s_ph = ph;
    }
    __syncthreads();
    const int item = s_item, ph = s_ph;
    if (item >= q.nitems) return;
    const QPhase P = q.phases[ph];
    if (P.type == kQSweep) {
      const ZebraArgs<float, float> a = q.zargs[P.dir * q.ncases + P.cas];
      const int l = 2 * (item - P.first) + P.color;
      if (P.dir == 0) zebra_wide_line<0, float, float, WPL>(a, l);
      else zebra_wide_line<1, float, float, WPL>(a, l);
    } else {
      bcimp_case(q.bcim[P.cas], threadIdx.x, blockDim.x);
    }
    __syncthreads();  // every thread's stores are made before the item is counted
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(q.done + ph, 1);
    }
  }
}

int lines_queue_blocks(int wpl) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  cudaError_t e = wpl == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lines_queue<4>, 128, 0)
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lines_queue<2>, 64, 0);
  if (e != cudaSuccess) return 0;
  return sms * per_sm;
}

void launch_lines_queue(const QueueArgs& q, int wpl, int nblocks, cudaStream_t st) {
  if (nblocks <= 0) return;
  ++g_kernel_launches;
  if (wpl == 4) k_lines_queue<4><<<nblocks, 128, 0, st>>>(q);
  else k_lines_queue<2><<<nblocks, 64, 0, st>>>(q);
}

// the FP32 correction widened for the FP64 update q += dq
__global__ void k_dq_to_f64(const float* __restrict__ dq, double* __restrict__ dq64, size_t n3) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n3) dq64[i] = (double)dq[i];
}

void launch_dq_to_f64(const float* dq, double* dq64, size_t n3, cudaStream_t st) {
  ++g_kernel_launches;
  k_dq_to_f64<<<(unsigned)((n3 + 255) / 256), 256, 0, st>>>(dq, dq64, n3);
}

// ------------------------------------------------------------------------------ SA, zebra order
// scalar line solves, one warp per line of the colour (scatri arithmetic per point)
template <int DIR>
__global__ void __launch_bounds__(128) k_sa_zebra(SAZebraArgs a, int color) {
  const int jmax = a.jmax, kmax = a.kmax;
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const int lane = threadIdx.x & 31;
  const int l = 2 * ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) + color;
  if (l >= nl) return;
  const int L = (n + 31) / 32;
  const int beg = lane * L;
  const int cnt = beg < n ? min(n, beg + L) - beg : 0;
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  double* fb = a.work;
  double f = 0.0, phi = 1.0;
  for (int t = 0; t < cnt; ++t) {
    int i = beg + t;
    size_t id = P(i);
    size_t im = DIR == 0 ? ix(i, l - 1, jmax) : ix(l - 1, i, jmax);
    size_t ip = DIR == 0 ? ix(i, l + 1, jmax) : ix(l + 1, i, jmax);
    double v;
    if (l == 0) v = a.rhs[id] - a.op[id] * a.ds[ip];
    else if (l == nl - 1) v = a.rhs[id] - a.om[id] * a.ds[im];
    else v = a.rhs[id] - a.om[id] * a.ds[im] - a.op[id] * a.ds[ip];
    fb[id] = v;
    double pv = a.piv[id];
    double m;
    if (i == 0) { v = v / pv; m = 0.0; }
    else if (i == n - 1) { v = (v - a.am[id] * (t > 0 ? f : 0.0)) / pv; m = -(a.am[id] / pv); }
    else { v = (v - a.am[id] * (t > 0 ? f : 0.0)) * pv; m = -(a.am[id] * pv); }
    f = v;
    phi = t == 0 ? m : m * phi;
  }
  double vv = cnt ? f : 0.0, pp = cnt ? phi : 0.0;
  for (int d = 0; d < 5; ++d) {
    const int o = 1 << d;
    double vn = __shfl_up_sync(0xffffffffu, vv, o), pn = __shfl_up_sync(0xffffffffu, pp, o);
    if (lane >= o) { vv = vv + pp * vn; pp = pp * pn; }
  }
  double yin = __shfl_up_sync(0xffffffffu, vv, 1);
  if (lane == 0) yin = 0.0;
  f = yin;
  for (int t = 0; t < cnt; ++t) {
    int i = beg + t;
    size_t id = P(i);
    double pv = a.piv[id];
    double ff = fb[id];
    double v;
    if (i == 0) v = ff / pv;
    else if (i == n - 1) v = (ff - a.am[id] * f) / pv;
    else v = (ff - a.am[id] * f) * pv;
    f = v;
    fb[id] = v;
  }
  double un = 0.0, ps = 1.0;
  for (int t = cnt - 1; t >= 0; --t) {
    int i = beg + t;
    size_t id = P(i);
    double h = i == n - 1 ? 0.0 : -a.cf[id];
    double v = fb[id];
    if (t < cnt - 1) v = v - a.cf[id] * un;
    un = v;
    ps = (t == cnt - 1) ? h : h * ps;
  }
  double uu = cnt ? un : 0.0, qq = cnt ? ps : 0.0;
  for (int d = 0; d < 5; ++d) {
    const int o = 1 << d;
    double vn = __shfl_down_sync(0xffffffffu, uu, o), qn = __shfl_down_sync(0xffffffffu, qq, o);
    if (lane + o <= 31) { uu = uu + qq * vn; qq = qq * qn; }
  }
  double xin = __shfl_down_sync(0xffffffffu, uu, 1);
  if (lane == 31) xin = 0.0;
  double xn = xin;
  for (int t = cnt - 1; t >= 0; --t) {
    int i = beg + t;
    size_t id = P(i);
    double v = fb[id];
    if (i < n - 1) v = v - a.cf[id] * xn;
    xn = v;
    a.ds[id] = v;
  }
}

void launch_sa_zebra(int dir, const SAZebraArgs& a, int color, cudaStream_t st) {
  int nl = dir == 0 ? a.kmax : a.jmax;
  int lines = (nl - color + 1) / 2;
  if (lines <= 0) return;
  ++g_kernel_launches;
  if (dir == 0) k_sa_zebra<0><<<(lines + 3) / 4, 128, 0, st>>>(a, color);
  else k_sa_zebra<1><<<(lines + 3) / 4, 128, 0, st>>>(a, color);
}

}  // namespace smac
