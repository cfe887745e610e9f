// smac_lines.cu -- partitioned block-tridiagonal line solves for the Gauss-Seidel sweeps.
//
// The reference relaxes its lines one after the other (ljsweep / lksweep, ref/lrelax.f:225-561):
// line l's right-hand side needs the updated dq of line l-1 (or l+1), so the lines of a sweep
// form a chain.  That order is kept.  What runs in parallel is the solve of ONE line: a
// thread-block cluster of kCL CTAs splits the line into segments of L points, one per thread.
//
// With the blocks already factored (btlu3j/k: diagonal B' in LU form, super-diagonal
// c = B'^-1 C), a line solve is two affine recurrences:
//   forward   y_i = B'_i^-1 (r_i - a_i y_{i-1}) = B'_i^-1 r_i + M_i y_{i-1},  M_i = -B'_i^-1 a_i
//   backward  x_i = y_i - c_i x_{i+1}                                  H_i = -c_i
// Each thread runs its segment with a zero carry-in, the segments' end values are combined by
// a Kogge-Stone scan (within warps by shuffles, across the cluster's warps in CTA 0's shared
// memory through distributed shared memory), and each thread re-runs its segment from the
// correct carry-in.  The per-point arithmetic of the re-run is the reference's; only the
// carries at segment boundaries come from the scan.  The scan's transfer operators (products of
// M and H over segments and over the scan windows) depend only on the factored blocks, so a
// preparation kernel computes them once per factorisation, in parallel over all lines; the
// sweeps then only apply 3x3 matrix-vector products in the scan.
#include <cooperative_groups.h>
#include <cuda_pipeline.h>
#include <math.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

namespace cg = cooperative_groups;

namespace smac {

// ----------------------------------------------------------------------------------- 3x3 algebra
struct M3 {
  double v[9];  // (r, c) at [r + 3c]
};
// GB300 issues one FP64 instruction per warp every 64 cycles whatever the number of active lanes,
// so these solves are bound by FP64 instructions per warp: the partitioned path uses fused
// multiply-adds throughout (its results agree with the reference's to rounding, not bit for bit;
// the bit-identical path is the sequential sweep in smac_solve.cu).
__device__ __forceinline__ void mm(const double* A, const double* B, double* C) {  // C = A B
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r)
      C[r + 3 * c] = __fma_rn(A[r + 6], B[2 + 3 * c], __fma_rn(A[r + 3], B[1 + 3 * c], A[r] * B[3 * c]));
}
__device__ __forceinline__ void mv_acc(const double* A, const double* x, double* y) {  // y += A x
  for (int r = 0; r < 3; ++r) y[r] = __fma_rn(A[r + 6], x[2], __fma_rn(A[r + 3], x[1], __fma_rn(A[r], x[0], y[r])));
}
__device__ __forceinline__ void mv_sub(const double* A, const double* x, double* y) {  // y -= A x
  for (int r = 0; r < 3; ++r) y[r] = __fma_rn(-A[r + 6], x[2], __fma_rn(-A[r + 3], x[1], __fma_rn(-A[r], x[0], y[r])));
}
// solve with a factored diagonal block (LU, reciprocal diagonal), the reference's elimination order
__device__ __forceinline__ void lu_solve(const double* B, double& x1, double& x2, double& x3) {
  double d1 = B[0] * x1;
  double d2 = B[4] * __fma_rn(-B[1], d1, x2);
  double d3 = B[8] * __fma_rn(-B[5], d2, __fma_rn(-B[2], d1, x3));
  x3 = d3;
  x2 = __fma_rn(-B[7], x3, d2);
  x1 = __fma_rn(-B[3], x2, __fma_rn(-B[6], x3, d1));
}

__device__ __forceinline__ void pf_l2(const double* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__device__ __forceinline__ void ld9(const double* __restrict__ p, size_t id, size_t N, double* v) {
  for (int e = 0; e < 9; ++e) v[e] = p[id + N * e];
}

// operator storage of one direction: per line, kOpsPerSeg 3x3 operators per segment and
// kOpsPerWarp per warp, entry-major so that a warp's loads are coalesced
constexpr int kLevels = 5;                    // warp scan levels (32 = 2^5)
constexpr int kOpsPerSeg = 2 * (kLevels + 1); // fwd G^(0..5), bwd G^(0..5)
constexpr int kOpsPerWarp = 2 * kLevels;      // fwd KW^(0..4), bwd KW^(0..4)
constexpr int kCL = 8;                        // CTAs per cluster
constexpr int kNT = 128;                      // threads per CTA
constexpr int kMaxSeg = kCL * kNT;            // 1024 segments
constexpr int kMaxWarps = kMaxSeg / 32;       // 32 warps

struct LinePlan {
  int n, nl;     // line length, number of lines
  int L, ps;     // segment length, segments per line
  int pst;       // segment stride (ps rounded up to 32)
  int nw;        // warps with segments (pst / 32)
};

LinePlan line_plan(int dir, int jmax, int kmax) {
  LinePlan p;
  p.n = dir == 0 ? jmax : kmax;
  p.nl = dir == 0 ? kmax : jmax;
  p.L = (p.n + kMaxSeg - 1) / kMaxSeg;
  p.ps = (p.n + p.L - 1) / p.L;
  p.pst = ((p.ps + 31) / 32) * 32;
  p.nw = p.pst / 32;
  return p;
}

size_t line_ops_doubles(int dir, int jmax, int kmax) {
  LinePlan p = line_plan(dir, jmax, kmax);
  return (size_t)p.nl * ((size_t)kOpsPerSeg * 9 * p.pst + (size_t)kOpsPerWarp * 9 * kMaxWarps);
}

__device__ __forceinline__ double* seg_op(double* ops, const LinePlan& P, int line, int which) {
  size_t per_line = (size_t)kOpsPerSeg * 9 * P.pst + (size_t)kOpsPerWarp * 9 * kMaxWarps;
  return ops + per_line * line + (size_t)which * 9 * P.pst;  // entry e of segment s at [e*pst + s]
}
__device__ __forceinline__ double* warp_op(double* ops, const LinePlan& P, int line, int which) {
  size_t per_line = (size_t)kOpsPerSeg * 9 * P.pst + (size_t)kOpsPerWarp * 9 * kMaxWarps;
  return ops + per_line * line + (size_t)kOpsPerSeg * 9 * P.pst + (size_t)which * 9 * kMaxWarps;
}

// ----------------------------------------------------------------------------------- preparation
// One CTA per line, one thread per segment (blockDim = pst).  Computes, for the forward scan,
// G^(d)_s = product of the transfers of the last min(2^d, lane+1) segments ending at s (d = 0..5;
// d = 5 is the prefix from the warp's first segment), and for the backward scan the mirrored
// suffix products; then the same across the warps of the line.
template <int DIR>
__global__ void __launch_bounds__(1024) k_line_prep(LinePlan P, int jmax, size_t N, const double* __restrict__ b,
                                                    const double* __restrict__ a, const double* __restrict__ c,
                                                    double* __restrict__ ops) {
  const int line = blockIdx.x;
  const int s = threadIdx.x;
  const int lane = s & 31, w = s >> 5;
  __shared__ double sT[2][kMaxWarps][9];  // warp transfer products, fwd / bwd
  double F[9], Bw[9];
  const bool valid = s < P.ps;
  if (valid) {
    int b0 = s * P.L;
    int e0 = min(P.n, b0 + P.L) - 1;
    // forward transfer of the segment: F = M_e ... M_b, M_i = -B'^-1 a_i (M_0 = 0)
    for (int i = b0; i <= e0; ++i) {
      size_t id = DIR == 0 ? ix(i, line, jmax) : ix(line, i, jmax);
      double Bf[9], Mi[9];
      ld9(b, id, N, Bf);
      if (i == 0) {
        for (int e = 0; e < 9; ++e) Mi[e] = 0.0;
      } else {
        ld9(a, id, N, Mi);
        for (int col = 0; col < 3; ++col) {
          double x1 = Mi[3 * col], x2 = Mi[1 + 3 * col], x3 = Mi[2 + 3 * col];
          lu_solve(Bf, x1, x2, x3);
          Mi[3 * col] = -x1; Mi[1 + 3 * col] = -x2; Mi[2 + 3 * col] = -x3;
        }
      }
      if (i == b0) {
        for (int e = 0; e < 9; ++e) F[e] = Mi[e];
      } else {
        double T[9];
        mm(Mi, F, T);
        for (int e = 0; e < 9; ++e) F[e] = T[e];
      }
    }
    // backward transfer: Bw = H_b ... H_e, H_i = -c_i (H_{n-1} = 0)
    for (int i = e0; i >= b0; --i) {
      size_t id = DIR == 0 ? ix(i, line, jmax) : ix(line, i, jmax);
      double Hi[9];
      if (i == P.n - 1) {
        for (int e = 0; e < 9; ++e) Hi[e] = 0.0;
      } else {
        ld9(c, id, N, Hi);
        for (int e = 0; e < 9; ++e) Hi[e] = -Hi[e];
      }
      if (i == e0) {
        for (int e = 0; e < 9; ++e) Bw[e] = Hi[e];
      } else {
        double T[9];
        mm(Hi, Bw, T);
        for (int e = 0; e < 9; ++e) Bw[e] = T[e];
      }
    }
  } else {
    for (int e = 0; e < 9; ++e) { F[e] = 0.0; Bw[e] = 0.0; }
  }
  // warp Kogge-Stone compositions
  for (int d = 0; d <= kLevels; ++d) {
    double* of = seg_op(ops, P, line, d);
    double* ob = seg_op(ops, P, line, kLevels + 1 + d);
    if (s < P.pst)
      for (int e = 0; e < 9; ++e) { of[(size_t)e * P.pst + s] = F[e]; ob[(size_t)e * P.pst + s] = Bw[e]; }
    if (d == kLevels) break;
    const int o = 1 << d;
    double Fn[9], Bn[9];
    for (int e = 0; e < 9; ++e) {
      Fn[e] = __shfl_up_sync(0xffffffffu, F[e], o);
      Bn[e] = __shfl_down_sync(0xffffffffu, Bw[e], o);
    }
    double T[9];
    if (lane >= o) { mm(F, Fn, T); for (int e = 0; e < 9; ++e) F[e] = T[e]; }
    if (lane + o <= 31) { mm(Bw, Bn, T); for (int e = 0; e < 9; ++e) Bw[e] = T[e]; }
  }
  // warp transfers: forward = prefix at lane 31, backward = suffix at lane 0
  if (lane == 31) for (int e = 0; e < 9; ++e) sT[0][w][e] = F[e];
  if (lane == 0) for (int e = 0; e < 9; ++e) sT[1][w][e] = Bw[e];
  __syncthreads();
  if (w == 0) {
    double G[9], H[9];
    for (int e = 0; e < 9; ++e) {
      G[e] = lane < P.nw ? sT[0][lane][e] : 0.0;
      H[e] = lane < P.nw ? sT[1][lane][e] : 0.0;
    }
    for (int d = 0; d < kLevels; ++d) {
      double* of = warp_op(ops, P, line, d);
      double* ob = warp_op(ops, P, line, kLevels + d);
      for (int e = 0; e < 9; ++e) { of[(size_t)e * kMaxWarps + lane] = G[e]; ob[(size_t)e * kMaxWarps + lane] = H[e]; }
      const int o = 1 << d;
      double Gn[9], Hn[9];
      for (int e = 0; e < 9; ++e) {
        Gn[e] = __shfl_up_sync(0xffffffffu, G[e], o);
        Hn[e] = __shfl_down_sync(0xffffffffu, H[e], o);
      }
      double T[9];
      if (lane >= o) { mm(G, Gn, T); for (int e = 0; e < 9; ++e) G[e] = T[e]; }
      if (lane + o <= 31) { mm(H, Hn, T); for (int e = 0; e < 9; ++e) H[e] = T[e]; }
    }
  }
}

// ----------------------------------------------------------------------------------- sweep
// Shared memory of the sweep kernel: the thread's scan operators for the current line (staged
// with cp.async at the start of the line), warp 0's cross-warp operators, the warp aggregates
// (double-buffered by line parity so that a CTA that runs ahead cannot overwrite values that
// another CTA still reads) and the carries.
struct SweepSmem {
  double ops[kOpsPerSeg * 9][kNT];
  double kw[kOpsPerWarp * 9][32];
  double agg[2][2][kMaxWarps / kCL][3];  // [parity][fwd/bwd][warp of this CTA][component]
  double carry[2][kNT / 32][3];          // [fwd/bwd][warp of this CTA]
};

template <int DIR, int LMAX>
__global__ void __cluster_dims__(kCL, 1, 1) __launch_bounds__(kNT, 1)
    k_gs_sweep_part(SweepArgs a, int nsw, LinePlan P, const double* __restrict__ ops) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SweepSmem& S = *reinterpret_cast<SweepSmem*>(smem_raw);
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const int tid = threadIdx.x;
  const int s = rank * kNT + tid;          // segment
  const int lane = tid & 31;
  const int w = s >> 5;                    // warp index in the cluster
  const int wl = tid >> 5;                 // warp index in this CTA
  constexpr int WPC = kNT / 32;            // warps per CTA

  const int jmax = a.jmax;
  const size_t N = a.N;
  const int n = P.n, nl = P.nl;
  const int L = P.L;
  const bool valid = s < P.ps;
  const bool active_warp = w < P.nw;
  const int beg = s * L;
  // cross-warp scan levels: ceil(log2(warps with segments))
  const int wlev = P.nw > 1 ? 32 - __clz(P.nw - 1) : 0;
  const int cnt = valid ? min(n, beg + L) - beg : 0;
  const double half = 0.5;
  int lb, le, li;
  if ((nsw / 2) * 2 == nsw) { lb = nl - 1; le = 0; li = -1; }
  else { lb = 0; le = nl - 1; li = 1; }

  double dnew[LMAX][3];  // dq of the line relaxed just before (same points, same thread)
#pragma unroll
  for (int t = 0; t < LMAX; ++t) dnew[t][0] = dnew[t][1] = dnew[t][2] = 0.0;
  // staging of scan operators for line `line`: rows [k0, k1) of this thread's segment operators,
  // and (warp 0) of the cross-warp operators
  const size_t per_line = (size_t)kOpsPerSeg * 9 * P.pst + (size_t)kOpsPerWarp * 9 * kMaxWarps;
  auto stage_seg = [&](int line, int k0, int k1) {
    if (!active_warp) return;
    const double* base = ops + per_line * line;
#pragma unroll 2
    for (int k = k0; k < k1; ++k) __pipeline_memcpy_async(&S.ops[k][tid], base + (size_t)k * P.pst + s, 8);
  };
  auto stage_warp = [&](int line, int k0, int k1) {
    if (wl != 0) return;
    const double* base = ops + per_line * line + (size_t)kOpsPerSeg * 9 * P.pst;
#pragma unroll 2
    for (int k = k0; k < k1; ++k) __pipeline_memcpy_async(&S.kw[k][lane], base + (size_t)k * kMaxWarps + lane, 8);
  };
  constexpr int kSegHalf = (kLevels + 1) * 9;  // forward rows [0, kSegHalf), backward after
  constexpr int kWarpHalf = kLevels * 9;
  stage_seg(lb, 0, kOpsPerSeg * 9);
  stage_warp(lb, 0, kOpsPerWarp * 9);
  __pipeline_commit();
  int par = 0;
  for (int l = lb;; l += li, par ^= 1) {
    const int lm = l - 1 > 0 ? l - 1 : 0;
    const int lp = l + 1 < nl - 1 ? l + 1 : nl - 1;
    const double swm = half + copysign(half, (double)(l - 1 - lm));
    const double swp = half + copysign(half, (double)(lp - l - 1));
    const bool first = (l == lb);
    double r[LMAX][3], y[LMAX][3], dold[LMAX][3];
    // right-hand sides and the local forward pass (zero carry-in)
    double yp[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      if (t < cnt) {
        int i = beg + t;
        size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
        size_t im = DIR == 0 ? ix(i, lm, jmax) : ix(lm, i, jmax);
        size_t ip = DIR == 0 ? ix(i, lp, jmax) : ix(lp, i, jmax);
        double d1, d2, d3, e1, e2, e3;
        // the neighbour relaxed just before this line is in registers; the other one was
        // written by the previous sweep
        if (li > 0 && !first) { d1 = dnew[t][0]; d2 = dnew[t][1]; d3 = dnew[t][2]; }
        else { d1 = a.dq[im]; d2 = a.dq[im + N]; d3 = a.dq[im + 2 * N]; }
        if (li < 0 && !first) { e1 = dnew[t][0]; e2 = dnew[t][1]; e3 = dnew[t][2]; }
        else { e1 = a.dq[ip]; e2 = a.dq[ip + N]; e3 = a.dq[ip + 2 * N]; }
        dold[t][0] = a.dq[id]; dold[t][1] = a.dq[id + N]; dold[t][2] = a.dq[id + 2 * N];
        // the selectors swm, swp are exactly 0 or 1: a zero selector drops the neighbour
        if (swm == 0.0) d1 = d2 = d3 = 0.0;
        if (swp == 0.0) e1 = e2 = e3 = 0.0;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          double v = a.s[id + N * q];
          v = __fma_rn(-a.om[id + N * (q + 0)], d1, v);
          v = __fma_rn(-a.om[id + N * (q + 3)], d2, v);
          v = __fma_rn(-a.om[id + N * (q + 6)], d3, v);
          v = __fma_rn(-a.op[id + N * (q + 0)], e1, v);
          v = __fma_rn(-a.op[id + N * (q + 3)], e2, v);
          r[t][q] = __fma_rn(-a.op[id + N * (q + 6)], e3, v);
        }
        double x1 = r[t][0], x2 = r[t][1], x3 = r[t][2];
        if (t > 0) {
          const double* A = a.am;
          x1 = __fma_rn(-A[id + 6 * N], yp[2], __fma_rn(-A[id + 3 * N], yp[1], __fma_rn(-A[id], yp[0], x1)));
          x2 = __fma_rn(-A[id + 7 * N], yp[2], __fma_rn(-A[id + 4 * N], yp[1], __fma_rn(-A[id + N], yp[0], x2)));
          x3 = __fma_rn(-A[id + 8 * N], yp[2], __fma_rn(-A[id + 5 * N], yp[1], __fma_rn(-A[id + 2 * N], yp[0], x3)));
        }
        double Bf[9];
        ld9(a.btc, id, N, Bf);
        lu_solve(Bf, x1, x2, x3);
        y[t][0] = x1; y[t][1] = x2; y[t][2] = x3;
        yp[0] = x1; yp[1] = x2; yp[2] = x3;
      }
    }
    // this line's scan operators: staged while the previous line was solved (each thread copies
    // and reads only its own column, so the waits need no barrier).  The forward half is here
    // now; the backward half, staged last, is waited for before the backward scan.
    __pipeline_wait_prior(1);
    const bool more = l != le;
    const int lnext = l + li;
    // the next line's operands into L2 while this line is solved (all of them are fixed during
    // the sweep except the dq of this line, which the next line takes from registers)
    if (more) {
      const int lfar = min(max(lnext + li, 0), nl - 1);
#pragma unroll
      for (int t = 0; t < LMAX; ++t) {
        if (t < cnt) {
          int i = beg + t;
          size_t id = DIR == 0 ? ix(i, lnext, jmax) : ix(lnext, i, jmax);
          size_t ifar = DIR == 0 ? ix(i, lfar, jmax) : ix(lfar, i, jmax);
#pragma unroll
          for (int e = 0; e < 9; ++e) {
            pf_l2(a.om + id + N * e); pf_l2(a.op + id + N * e); pf_l2(a.am + id + N * e);
            pf_l2(a.btc + id + N * e); pf_l2(a.cp + id + N * e);
          }
#pragma unroll
          for (int q = 0; q < 3; ++q) { pf_l2(a.s + id + N * q); pf_l2(a.dq + id + N * q); pf_l2(a.dq + ifar + N * q); }
        }
      }
    }
    // forward scan of the segment end values inside the warp
    double v[3] = {yp[0], yp[1], yp[2]};
    if (!valid) v[0] = v[1] = v[2] = 0.0;
#pragma unroll
    for (int d = 0; d < kLevels; ++d) {
      const int o = 1 << d;
      double vn[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) vn[q] = __shfl_up_sync(0xffffffffu, v[q], o);
      if (lane >= o && active_warp) {
        double K[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) K[e] = S.ops[d * 9 + e][tid];
        mv_acc(K, vn, v);
      }
    }
    if (lane == 31)
#pragma unroll
      for (int q = 0; q < 3; ++q) S.agg[par][0][wl][q] = v[q];
    cluster.sync();
    // every CTA scans across all the cluster's warps (lane = warp) and keeps its own carries
    if (wl == 0) {
      double z[3];
      {
        const double* src = cluster.map_shared_rank(&S.agg[par][0][0][0], (unsigned)(lane / WPC));
#pragma unroll
        for (int q = 0; q < 3; ++q) z[q] = lane < P.nw ? src[(lane % WPC) * 3 + q] : 0.0;
      }
      for (int d = 0; d < wlev; ++d) {
        const int o = 1 << d;
        double zn[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) zn[q] = __shfl_up_sync(0xffffffffu, z[q], o);
        if (lane >= o && lane < P.nw) {
          double K[9];
#pragma unroll
          for (int e = 0; e < 9; ++e) K[e] = S.kw[d * 9 + e][lane];
          mv_acc(K, zn, z);
        }
      }
      if (more) { stage_warp(lnext, 0, kWarpHalf); __pipeline_commit(); }
      // carry into warp lane = Z of warp lane-1
      double zc[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        zc[q] = __shfl_up_sync(0xffffffffu, z[q], 1);
        if (lane == 0) zc[q] = 0.0;
      }
      int mine = lane - (int)rank * WPC;
      if (mine >= 0 && mine < WPC)
#pragma unroll
        for (int q = 0; q < 3; ++q) S.carry[0][mine][q] = zc[q];
    }
    __syncthreads();
    double cin[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) cin[q] = active_warp ? S.carry[0][wl][q] : 0.0;
    double Y[3] = {v[0], v[1], v[2]};
    if (valid) {
      double K[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) K[e] = S.ops[kLevels * 9 + e][tid];
      mv_acc(K, cin, Y);
    }
    if (more) { stage_seg(lnext, 0, kSegHalf); __pipeline_commit(); }
    double yin[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      yin[q] = __shfl_up_sync(0xffffffffu, Y[q], 1);
      if (lane == 0) yin[q] = cin[q];
    }
    // forward pass again from the true carry-in (the reference's per-point arithmetic); a
    // one-point segment takes the scanned value directly
    if (LMAX == 1) {
      if (valid) { y[0][0] = Y[0]; y[0][1] = Y[1]; y[0][2] = Y[2]; }
    } else if (valid && beg > 0) {
      yp[0] = yin[0]; yp[1] = yin[1]; yp[2] = yin[2];
#pragma unroll
      for (int t = 0; t < LMAX; ++t) {
        if (t < cnt) {
          int i = beg + t;
          size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
          const double* A = a.am;
          double x1 = __fma_rn(-A[id + 6 * N], yp[2], __fma_rn(-A[id + 3 * N], yp[1], __fma_rn(-A[id], yp[0], r[t][0])));
          double x2 = __fma_rn(-A[id + 7 * N], yp[2], __fma_rn(-A[id + 4 * N], yp[1], __fma_rn(-A[id + N], yp[0], r[t][1])));
          double x3 = __fma_rn(-A[id + 8 * N], yp[2], __fma_rn(-A[id + 5 * N], yp[1], __fma_rn(-A[id + 2 * N], yp[0], r[t][2])));
          double Bf[9];
          ld9(a.btc, id, N, Bf);
          lu_solve(Bf, x1, x2, x3);
          y[t][0] = x1; y[t][1] = x2; y[t][2] = x3;
          yp[0] = x1; yp[1] = x2; yp[2] = x3;
        }
      }
    }
    __pipeline_wait_prior(0);
    // local backward pass (zero carry-in from the right): u = segment start value
    double Cl[LMAX][9];
    double u[3] = {0.0, 0.0, 0.0};
    {
      double xn[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        if (t < cnt) {
          int i = beg + t;
          size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
          if (i < n - 1) ld9(a.cp, id, N, Cl[t]);
          else for (int e = 0; e < 9; ++e) Cl[t][e] = 0.0;
          double x1 = y[t][0], x2 = y[t][1], x3 = y[t][2];
          if (t < cnt - 1) {
            double xv[3] = {x1, x2, x3};
            mv_sub(Cl[t], xn, xv);
            x1 = xv[0]; x2 = xv[1]; x3 = xv[2];
          }
          xn[0] = x1; xn[1] = x2; xn[2] = x3;
        }
      }
      u[0] = xn[0]; u[1] = xn[1]; u[2] = xn[2];
      if (!valid) u[0] = u[1] = u[2] = 0.0;
    }
#pragma unroll
    for (int d = 0; d < kLevels; ++d) {
      const int o = 1 << d;
      double un[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) un[q] = __shfl_down_sync(0xffffffffu, u[q], o);
      if (lane + o <= 31 && active_warp) {
        double K[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) K[e] = S.ops[(kLevels + 1 + d) * 9 + e][tid];
        mv_acc(K, un, u);
      }
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 3; ++q) S.agg[par][1][wl][q] = u[q];
    cluster.sync();
    if (wl == 0) {
      double z[3];
      {
        const double* src = cluster.map_shared_rank(&S.agg[par][1][0][0], (unsigned)(lane / WPC));
#pragma unroll
        for (int q = 0; q < 3; ++q) z[q] = lane < P.nw ? src[(lane % WPC) * 3 + q] : 0.0;
      }
      for (int d = 0; d < wlev; ++d) {
        const int o = 1 << d;
        double zn[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) zn[q] = __shfl_down_sync(0xffffffffu, z[q], o);
        if (lane + o < P.nw) {
          double K[9];
#pragma unroll
          for (int e = 0; e < 9; ++e) K[e] = S.kw[(kLevels + d) * 9 + e][lane];
          mv_acc(K, zn, z);
        }
      }
      if (more) { stage_warp(lnext, kWarpHalf, kOpsPerWarp * 9); __pipeline_commit(); }
      double zc[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        zc[q] = __shfl_down_sync(0xffffffffu, z[q], 1);
        if (lane == 31 || lane + 1 >= P.nw) zc[q] = 0.0;
      }
      int mine = lane - (int)rank * WPC;
      if (mine >= 0 && mine < WPC)
#pragma unroll
        for (int q = 0; q < 3; ++q) S.carry[1][mine][q] = zc[q];
    }
    __syncthreads();
    double bin[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) bin[q] = active_warp ? S.carry[1][wl][q] : 0.0;
    double X[3] = {u[0], u[1], u[2]};
    if (valid) {
      double K[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) K[e] = S.ops[(2 * kLevels + 1) * 9 + e][tid];
      mv_acc(K, bin, X);
    }
    if (more) { stage_seg(lnext, kSegHalf, kOpsPerSeg * 9); __pipeline_commit(); }
    double xin[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      xin[q] = __shfl_down_sync(0xffffffffu, X[q], 1);
      if (lane == 31) xin[q] = bin[q];
    }
    // backward pass from the true carry-in, then the relaxation update
    if (LMAX == 1 && valid) {
      size_t id = DIR == 0 ? ix(beg, l, jmax) : ix(l, beg, jmax);
      double x1 = X[0], x2 = X[1], x3 = X[2];
      double n1 = __fma_rn(a.underr, x1 - dold[0][0], dold[0][0]);
      double n2 = __fma_rn(a.underr, x2 - dold[0][1], dold[0][1]);
      double n3 = __fma_rn(a.underr, x3 - dold[0][2], dold[0][2]);
      a.dq[id] = n1; a.dq[id + N] = n2; a.dq[id + 2 * N] = n3;
      dnew[0][0] = n1; dnew[0][1] = n2; dnew[0][2] = n3;
    } else if (valid) {
      const bool last = beg + cnt == n;
      double xn[3] = {xin[0], xin[1], xin[2]};
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        if (t < cnt) {
          int i = beg + t;
          size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
          double x1 = y[t][0], x2 = y[t][1], x3 = y[t][2];
          if (!(last && t == cnt - 1)) {
            double xv[3] = {x1, x2, x3};
            mv_sub(Cl[t], xn, xv);
            x1 = xv[0]; x2 = xv[1]; x3 = xv[2];
          }
          xn[0] = x1; xn[1] = x2; xn[2] = x3;
          double n1 = __fma_rn(a.underr, x1 - dold[t][0], dold[t][0]);
          double n2 = __fma_rn(a.underr, x2 - dold[t][1], dold[t][1]);
          double n3 = __fma_rn(a.underr, x3 - dold[t][2], dold[t][2]);
          a.dq[id] = n1; a.dq[id + N] = n2; a.dq[id + 2 * N] = n3;
          dnew[t][0] = n1; dnew[t][1] = n2; dnew[t][2] = n3;
        }
      }
    }
    if (l == le) break;
  }
  // no CTA may leave while another still reads its aggregates
  cluster.sync();
}

void launch_line_prep(int dir, int jmax, int kmax, const double* b, const double* a, const double* c, double* ops,
                      cudaStream_t st) {
  LinePlan P = line_plan(dir, jmax, kmax);
  size_t N = (size_t)jmax * kmax;
  ++g_kernel_launches;
  if (dir == 0) k_line_prep<0><<<P.nl, P.pst, 0, st>>>(P, jmax, N, b, a, c, ops);
  else k_line_prep<1><<<P.nl, P.pst, 0, st>>>(P, jmax, N, b, a, c, ops);
}

template <int DIR, int LMAX>
static void launch_part(const SweepArgs& a, int nsw, const LinePlan& P, const double* ops, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gs_sweep_part<DIR, LMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(SweepSmem));
    attr = true;
  }
  ++g_kernel_launches;
  k_gs_sweep_part<DIR, LMAX><<<kCL, kNT, sizeof(SweepSmem), st>>>(a, nsw, P, ops);
}

// ----------------------------------------------------------------------------------- layouts
// The k-lines of the sweep are strided by jmax in the reference layout, so a line's loads touch
// one sector per point.  Before the k-sweeps their operands are transposed to k-major planes
// (element (j,k) at k + kmax*j), where a k-line is contiguous and the j-line kernel solves it.
__global__ void k_transpose(const double* __restrict__ in, double* __restrict__ out, int rows, int cols, size_t N) {
  // in: plane of rows x cols with the row index fastest; out: cols x rows, col index fastest
  __shared__ double tile[32][33];
  const size_t plane = blockIdx.z;
  in += plane * N;
  out += plane * N;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    int r = r0 + threadIdx.x, c = c0 + dy;
    if (r < rows && c < cols) tile[dy][threadIdx.x] = in[(size_t)r + (size_t)rows * c];
  }
  __syncthreads();
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    int c = c0 + threadIdx.x, r = r0 + dy;
    if (r < rows && c < cols) out[(size_t)c + (size_t)cols * r] = tile[threadIdx.x][dy];
  }
}

void launch_transpose(const double* in, double* out, int rows, int cols, size_t N, int planes, cudaStream_t st) {
  dim3 grid((rows + 31) / 32, (cols + 31) / 32, planes);
  ++g_kernel_launches;
  k_transpose<<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols, N);
}

int launch_gs_sweep_part(int dir, int nsw, const SweepArgs& a, const double* ops, cudaStream_t st) {
  LinePlan P = line_plan(dir, a.jmax, a.kmax);
  if (P.L > 8) return 1;
  int lm = P.L <= 1 ? 1 : P.L <= 2 ? 2 : P.L <= 4 ? 4 : 8;
  if (dir == 0) {
    if (lm == 1) launch_part<0, 1>(a, nsw, P, ops, st);
    else if (lm == 2) launch_part<0, 2>(a, nsw, P, ops, st);
    else if (lm == 4) launch_part<0, 4>(a, nsw, P, ops, st);
    else launch_part<0, 8>(a, nsw, P, ops, st);
  } else {
    if (lm == 1) launch_part<1, 1>(a, nsw, P, ops, st);
    else if (lm == 2) launch_part<1, 2>(a, nsw, P, ops, st);
    else if (lm == 4) launch_part<1, 4>(a, nsw, P, ops, st);
    else launch_part<1, 8>(a, nsw, P, ops, st);
  }
  return 0;
}

}  // namespace smac

namespace smac {

// ==================================================================================================
// Scalar SA line relaxation (turswpj / turswpk with scatri, ref/lreltur.f:164-359), partitioned
// like the block sweeps.  scatri's coefficient recurrence (c' and the pivots) does not depend on
// the right-hand side, so it is computed once per line in parallel over lines; the sweep kernel
// then runs the right-hand-side recurrences with segment scans whose scalar transfers are
// composed on the fly.

// pivots per line: piv[0] = b_0 and piv[n-1] = b - a c' (the reference divides by them), piv[i]
// = 1 / (b_i - a_i c'_{i-1}) inside (the reference multiplies by it); cf = c'
// A thread walks its line; the operands of the point kSaPF steps ahead are loaded into a
// register ring (the loads of neighbouring threads fall on different cache lines, so each step
// would otherwise wait for its own).
constexpr int kSaPF = 8;
template <int DIR>
__global__ void k_sa_factor(const double* __restrict__ am, const double* __restrict__ bt,
                            const double* __restrict__ cp, double* __restrict__ piv, double* __restrict__ cf,
                            int jmax, int kmax) {
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nl) return;
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  size_t i0 = P(0);
  double b0 = bt[i0];
  piv[i0] = b0;
  double cprev = cp[i0] / b0;
  cf[i0] = cprev;
  double ra[kSaPF], rb[kSaPF], rc[kSaPF];
#pragma unroll
  for (int q = 0; q < kSaPF; ++q) {
    const int i = 1 + q;
    if (i <= n - 2) { size_t id = P(i); ra[q] = am[id]; rb[q] = bt[id]; rc[q] = cp[id]; }
  }
  for (int i0b = 1; i0b <= n - 2; i0b += kSaPF) {
#pragma unroll
    for (int q = 0; q < kSaPF; ++q) {
      const int i = i0b + q;
      if (i > n - 2) break;
      const double a = ra[q], b = rb[q], c = rc[q];
      const int inext = i + kSaPF;
      if (inext <= n - 2) { size_t idn = P(inext); ra[q] = am[idn]; rb[q] = bt[idn]; rc[q] = cp[idn]; }
      size_t id = P(i);
      double z = 1. / (b - a * cprev);
      cprev = c * z;
      cf[id] = cprev;
      piv[id] = z;
    }
  }
  size_t ie = P(n - 1);
  piv[ie] = bt[ie] - am[ie] * cprev;
  cf[ie] = 0.0;
}

// The same pivots with a warp per line, for the throughput forms (zebra order, FP32 operator).
// c'_i = c_i / (b_i - a_i c'_{i-1}) is a Moebius map of c'_{i-1}: with homogeneous coordinates
// it is the 2x2 matrix M_i = [[0, c_i], [-a_i, b_i]] (a_0 taken as 0, so that M_0 gives
// c'_0 = c_0 / b_0 whatever it is applied to).  Lane s composes the matrices of its segment
// (rescaled by powers of two, which round nothing, so that long products neither overflow nor
// underflow), a warp scan composes the segments, c'_{beg-1} is the ratio of the second column of
// the product of the segments before, and each lane reruns its segment with the one-thread
// kernel's arithmetic from there.  The map is a contraction where the lines are diagonally
// dominant, so the pivots agree with the sequential ones to rounding.
__device__ __forceinline__ void mob_scale(double* T) {  // T *= 2^-e, 2^e ~ the largest |entry|
  double m = fmax(fmax(fabs(T[0]), fabs(T[1])), fmax(fabs(T[2]), fabs(T[3])));
  if (m > 0.0 && isfinite(m)) {
    int e;
    frexp(m, &e);
    const double s = ldexp(1.0, -e);
    T[0] *= s; T[1] *= s; T[2] *= s; T[3] *= s;
  }
}
// C = A B for 2x2 matrices stored [00, 01, 10, 11]
__device__ __forceinline__ void mob_mul(const double* A, const double* B, double* C) {
  C[0] = fma(A[0], B[0], A[1] * B[2]);
  C[1] = fma(A[0], B[1], A[1] * B[3]);
  C[2] = fma(A[2], B[0], A[3] * B[2]);
  C[3] = fma(A[2], B[1], A[3] * B[3]);
}
template <int DIR>
__global__ void __launch_bounds__(128) k_sa_factor_warp(const double* __restrict__ am, const double* __restrict__ bt,
                                                        const double* __restrict__ cp, double* __restrict__ piv,
                                                        double* __restrict__ cf, int jmax, int kmax) {
  const int n = DIR == 0 ? jmax : kmax;
  const int nl = DIR == 0 ? kmax : jmax;
  const int lane = threadIdx.x & 31;
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (l >= nl) return;  // warp-uniform
  auto P = [&](int i) -> size_t { return DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax); };
  const int L = (n + 31) / 32;
  const int beg = lane * L;
  const int end = min(n - 1, beg + L);  // the chain covers points 0..n-2
  // the segment's product of M_i, i = beg .. end-1 (identity for an empty segment)
  double T[4] = {1.0, 0.0, 0.0, 1.0};
  for (int i = beg; i < end; ++i) {
    const size_t id = P(i);
    const double a = i == 0 ? 0.0 : am[id], b = bt[id], c = cp[id];
    const double M[4] = {0.0, c, -a, b};
    double X[4];
    mob_mul(M, T, X);
    T[0] = X[0]; T[1] = X[1]; T[2] = X[2]; T[3] = X[3];
    if (((i - beg) & 3) == 3) mob_scale(T);
  }
  mob_scale(T);
  // inclusive scan: lane s holds the product of the segments 0..s (later segments on the left)
#pragma unroll
  for (int d = 0; d < 5; ++d) {
    const int o = 1 << d;
    double U[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) U[e] = __shfl_up_sync(0xffffffffu, T[e], o);
    if (lane >= o) {
      double X[4];
      mob_mul(T, U, X);
      T[0] = X[0]; T[1] = X[1]; T[2] = X[2]; T[3] = X[3];
      mob_scale(T);
    }
  }
  const double p01 = __shfl_up_sync(0xffffffffu, T[1], 1), p11 = __shfl_up_sync(0xffffffffu, T[3], 1);
  if (beg >= n) return;
  // rerun the segment with the sequential arithmetic from c'_{beg-1}
  double cprev = lane == 0 ? 0.0 : p01 / p11;
  for (int i = beg; i < min(n, beg + L); ++i) {
    const size_t id = P(i);
    if (i == 0) {
      const double b0 = bt[id];
      piv[id] = b0;
      cprev = cp[id] / b0;
      cf[id] = cprev;
    } else if (i == n - 1) {
      piv[id] = bt[id] - am[id] * cprev;
      cf[id] = 0.0;
    } else {
      const double z = 1. / (bt[id] - am[id] * cprev);
      cprev = cp[id] * z;
      cf[id] = cprev;
      piv[id] = z;
    }
  }
}

void launch_sa_factor_warp(int dir, const ScalarSweepArgs& s, double* piv, double* cf, cudaStream_t st) {
  const int nl = dir == 0 ? s.kmax : s.jmax;
  const double* am = dir == 0 ? s.sjm : s.skm;
  const double* cp = dir == 0 ? s.sjp : s.skp;
  ++g_kernel_launches;
  const unsigned blocks = (unsigned)((nl + 3) / 4);
  if (dir == 0) k_sa_factor_warp<0><<<blocks, 128, 0, st>>>(am, s.stc, cp, piv, cf, s.jmax, s.kmax);
  else k_sa_factor_warp<1><<<blocks, 128, 0, st>>>(am, s.stc, cp, piv, cf, s.jmax, s.kmax);
}

struct SASweepArgs {
  int jmax, kmax;
  size_t N;
  const double *am, *om, *op, *rhs, *piv, *cf;
  double* ds;
};

template <int DIR, int LMAX>
__global__ void __cluster_dims__(kCL, 1, 1) __launch_bounds__(kNT)
    k_sa_sweep_part(SASweepArgs a, LinePlan P) {
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const int s = rank * kNT + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int w = s >> 5;
  __shared__ double sh_v[kMaxWarps], sh_p[kMaxWarps], sh_u[kMaxWarps], sh_q[kMaxWarps];
  double* v0 = cluster.map_shared_rank(&sh_v[0], 0);
  double* p0 = cluster.map_shared_rank(&sh_p[0], 0);
  double* u0 = cluster.map_shared_rank(&sh_u[0], 0);
  double* q0 = cluster.map_shared_rank(&sh_q[0], 0);
  const int jmax = a.jmax;
  const int n = P.n, nl = P.nl, L = P.L;
  const bool valid = s < P.ps;
  const int beg = s * L;
  const int cnt = valid ? min(n, beg + L) - beg : 0;

  for (int step = 0; step <= nl; ++step) {
    const int l = step < nl ? step : 0;  // lines 1..max, then line 1 again
    double ff[LMAX], f[LMAX];
    double fprev = 0.0, phi = 1.0;
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      if (t < cnt) {
        int i = beg + t;
        size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
        size_t im = DIR == 0 ? ix(i, l - 1, jmax) : ix(l - 1, i, jmax);
        size_t ip = DIR == 0 ? ix(i, l + 1, jmax) : ix(l + 1, i, jmax);
        double v;
        if (l == 0) v = a.rhs[id] - a.op[id] * a.ds[ip];
        else if (l == nl - 1) v = a.rhs[id] - a.om[id] * a.ds[im];
        else v = a.rhs[id] - a.om[id] * a.ds[im] - a.op[id] * a.ds[ip];
        ff[t] = v;
        double pv = a.piv[id];
        double m;
        if (i == 0) { v = v / pv; m = 0.0; }
        else if (i == n - 1) { v = (v - a.am[id] * (t > 0 ? fprev : 0.0)) / pv; m = -(a.am[id] / pv); }
        else { v = (v - a.am[id] * (t > 0 ? fprev : 0.0)) * pv; m = -(a.am[id] * pv); }
        f[t] = v;
        fprev = v;
        phi = t == 0 ? m : m * phi;
      }
    }
    // forward scan, (transfer, value) pairs composed on the fly
    double vv = valid ? fprev : 0.0, pp = valid ? phi : 0.0;
#pragma unroll
    for (int d = 0; d < kLevels; ++d) {
      const int o = 1 << d;
      double vn = __shfl_up_sync(0xffffffffu, vv, o);
      double pn = __shfl_up_sync(0xffffffffu, pp, o);
      if (lane >= o) { vv = vv + pp * vn; pp = pp * pn; }
    }
    if (lane == 31 && w < P.nw) { v0[w] = vv; p0[w] = pp; }
    cluster.sync();
    if (rank == 0 && threadIdx.x < 32) {
      double z = lane < P.nw ? sh_v[lane] : 0.0, g = lane < P.nw ? sh_p[lane] : 0.0;
#pragma unroll
      for (int d = 0; d < kLevels; ++d) {
        const int o = 1 << d;
        double zn = __shfl_up_sync(0xffffffffu, z, o);
        double gn = __shfl_up_sync(0xffffffffu, g, o);
        if (lane >= o) { z = z + g * zn; g = g * gn; }
      }
      if (lane < P.nw) sh_v[lane] = z;
    }
    cluster.sync();
    double cin = (w > 0 && w <= P.nw) ? v0[w - 1] : 0.0;
    double Y = vv + pp * cin;
    double yin = __shfl_up_sync(0xffffffffu, Y, 1);
    if (lane == 0) yin = cin;
    if (valid && beg > 0) {
      fprev = yin;
#pragma unroll
      for (int t = 0; t < LMAX; ++t) {
        if (t < cnt) {
          int i = beg + t;
          size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
          double pv = a.piv[id];
          double v = (i == n - 1) ? (ff[t] - a.am[id] * fprev) / pv : (ff[t] - a.am[id] * fprev) * pv;
          f[t] = v;
          fprev = v;
        }
      }
    }
    // backward: f_i = f_i - c'_i f_{i+1}
    double un = 0.0, ps = 1.0;
#pragma unroll
    for (int t = LMAX - 1; t >= 0; --t) {
      if (t < cnt) {
        int i = beg + t;
        size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
        double h = i == n - 1 ? 0.0 : -a.cf[id];
        double v = f[t];
        if (t < cnt - 1) v = v - a.cf[id] * un;
        un = v;
        ps = (t == cnt - 1) ? h : h * ps;
      }
    }
    double uu = valid ? un : 0.0, qq = valid ? ps : 0.0;
#pragma unroll
    for (int d = 0; d < kLevels; ++d) {
      const int o = 1 << d;
      double vn = __shfl_down_sync(0xffffffffu, uu, o);
      double qn = __shfl_down_sync(0xffffffffu, qq, o);
      if (lane + o <= 31) { uu = uu + qq * vn; qq = qq * qn; }
    }
    if (lane == 0 && w < P.nw) { u0[w] = uu; q0[w] = qq; }
    cluster.sync();
    if (rank == 0 && threadIdx.x < 32) {
      double z = lane < P.nw ? sh_u[lane] : 0.0, g = lane < P.nw ? sh_q[lane] : 0.0;
#pragma unroll
      for (int d = 0; d < kLevels; ++d) {
        const int o = 1 << d;
        double zn = __shfl_down_sync(0xffffffffu, z, o);
        double gn = __shfl_down_sync(0xffffffffu, g, o);
        if (lane + o <= 31) { z = z + g * zn; g = g * gn; }
      }
      if (lane < P.nw) sh_u[lane] = z;
    }
    cluster.sync();
    double bin = (w + 1 < P.nw) ? u0[w + 1] : 0.0;
    double X = uu + qq * bin;
    double xin = __shfl_down_sync(0xffffffffu, X, 1);
    if (lane == 31) xin = bin;
    if (valid) {
      bool last = beg + cnt == n;
      double xn = xin;
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        if (t < cnt) {
          int i = beg + t;
          size_t id = DIR == 0 ? ix(i, l, jmax) : ix(l, i, jmax);
          double v = f[t];
          if (!(last && t == cnt - 1)) v = v - a.cf[id] * xn;
          xn = v;
          a.ds[id] = v;
        }
      }
    }
    __threadfence();
    cluster.sync();
  }
}

template <int DIR, int LMAX>
static void launch_sa_part(const SASweepArgs& a, const LinePlan& P, cudaStream_t st) {
  ++g_kernel_launches;
  k_sa_sweep_part<DIR, LMAX><<<kCL, kNT, 0, st>>>(a, P);
}

void launch_sa_factor(int dir, const ScalarSweepArgs& s, double* piv, double* cf, cudaStream_t st) {
  LinePlan P = line_plan(dir, s.jmax, s.kmax);
  const double* am = dir == 0 ? s.sjm : s.skm;
  const double* cp = dir == 0 ? s.sjp : s.skp;
  ++g_kernel_launches;
  if (dir == 0) k_sa_factor<0><<<(P.nl + 31) / 32, 32, 0, st>>>(am, s.stc, cp, piv, cf, s.jmax, s.kmax);
  else k_sa_factor<1><<<(P.nl + 31) / 32, 32, 0, st>>>(am, s.stc, cp, piv, cf, s.jmax, s.kmax);
}

// one SA sweep, partitioned: factor the lines, then sweep
int launch_sa_sweep_part(int dir, const ScalarSweepArgs& s, double* piv, double* cf, cudaStream_t st) {
  LinePlan P = line_plan(dir, s.jmax, s.kmax);
  if (P.L > 8) return 1;
  const double* am = dir == 0 ? s.sjm : s.skm;
  const double* cp = dir == 0 ? s.sjp : s.skp;
  ++g_kernel_launches;
  if (dir == 0) k_sa_factor<0><<<(P.nl + 63) / 64, 64, 0, st>>>(am, s.stc, cp, piv, cf, s.jmax, s.kmax);
  else k_sa_factor<1><<<(P.nl + 63) / 64, 64, 0, st>>>(am, s.stc, cp, piv, cf, s.jmax, s.kmax);
  SASweepArgs a;
  a.jmax = s.jmax; a.kmax = s.kmax; a.N = s.N;
  a.am = am;
  a.om = dir == 0 ? s.skm : s.sjm;
  a.op = dir == 0 ? s.skp : s.sjp;
  a.rhs = s.rhs; a.piv = piv; a.cf = cf; a.ds = s.ds;
  int lm = P.L <= 1 ? 1 : P.L <= 2 ? 2 : P.L <= 4 ? 4 : 8;
  if (dir == 0) {
    if (lm == 1) launch_sa_part<0, 1>(a, P, st);
    else if (lm == 2) launch_sa_part<0, 2>(a, P, st);
    else if (lm == 4) launch_sa_part<0, 4>(a, P, st);
    else launch_sa_part<0, 8>(a, P, st);
  } else {
    if (lm == 1) launch_sa_part<1, 1>(a, P, st);
    else if (lm == 2) launch_sa_part<1, 2>(a, P, st);
    else if (lm == 4) launch_sa_part<1, 4>(a, P, st);
    else launch_sa_part<1, 8>(a, P, st);
  }
  return 0;
}

}  // namespace smac
