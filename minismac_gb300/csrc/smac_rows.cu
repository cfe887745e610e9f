// smac_rows.cu -- reference-order line sweeps with three lanes per segment.
//
// The lines of a sweep are relaxed one after the other (ljsweep / lksweep, ref/lrelax.f:225-561);
// one line is solved by a cluster of kRCL CTAs.  As in smac_lines.cu the line is split into
// segments whose forward (y_i = B'^-1 r_i + M_i y_{i-1}) and backward (x_i = y_i - c_i x_{i+1})
// recurrences are combined by Kogge-Stone scans over precomputed transfer operators.  What is
// different is the mapping to GB300's FP64 issue limit (one FP64 instruction per warp every 64
// cycles, whatever the active lanes): a segment is owned by three lanes, lane r computing row r
// of every 3x3 product and the 3-vectors being re-assembled by shuffles, so the products of the
// scans cost three fused multiply-adds per lane instead of nine.  A warp holds ten segments
// (30 lanes), a CTA eight warps, the cluster eight CTAs (640 segments), and the scan is
// hierarchical: inside the warp (shuffles), across the warps of a CTA (shared memory, one warp),
// across the CTAs (each CTA pushes its aggregate into every CTA's shared memory before the
// cluster barrier; two cluster barriers per line).
// Each lane keeps only the rows of the operators it applies.  With one-point segments the next
// line's operands wait in registers; a line one point longer than a multiple of the segments
// takes its first point out of the scan (row_plan).  The arithmetic is contracted to fused
// multiply-adds: results agree with the reference's to rounding, not bit for bit.
#include <cooperative_groups.h>
#include <cuda_pipeline.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

namespace cg = cooperative_groups;

namespace smac {

namespace {

constexpr int kRCL = 8;                    // CTAs per cluster
constexpr int kRW = 8;                     // warps per CTA
constexpr int kRNT = 32 * kRW;             // threads per CTA
constexpr int kSPW = 10;                   // segments per warp (three lanes each)
constexpr int kSPC = kSPW * kRW;           // segments per CTA
constexpr int kRMaxSeg = kSPC * kRCL;      // segments per line
constexpr int kSegLev = 4;                 // scan levels inside a warp (10 slots); level 4: prefix
constexpr int kWLev = 3;                   // levels across the warps of a CTA; level 3: prefix
constexpr int kCLev = 3;                   // levels across the CTAs
// operator rows per lane (3 doubles per 3x3 operator)
constexpr int kSegOps = 2 * (kSegLev + 1); // forward windows 0..3 + prefix, backward the same
constexpr int kWOps = 2 * (kWLev + 1);     // forward windows 0..2 + shifted prefix, backward the same
constexpr int kCOps = 2 * kCLev;           // forward windows 0..2, backward windows 0..2
constexpr size_t kSegBlock = (size_t)3 * kSegOps * kRCL * kRNT;
constexpr size_t kWBlock = (size_t)kRCL * 3 * kWOps * 32;
constexpr size_t kCBlock = (size_t)3 * kCOps * 32;
constexpr size_t kScanBlocks = kSegBlock + kWBlock + kCBlock;
// then per point of a segment (t = 0..L-1) the rows of B'^-1 and of M = -B'^-1 a, then (lines
// with a head point) the head block: for lane r of the first triple the rows r of B'^-1 at
// point 0, of K = M_1 B'^-1_0, of c_0 and of D = c_0 c_1, entry e of row r at [3 e + r]
constexpr size_t kHeadBlock = 36;
__host__ __device__ constexpr size_t per_line(int L, int H) {
  return kScanBlocks + (size_t)L * 6 * kRCL * kRNT + (size_t)H * kHeadBlock;
}

struct RowPlan {
  int n, nl;  // line length, number of lines
  int L, S;   // points per segment, segments
  int H;      // 1: the line's first point is taken out of the scan (the head point)
};

// A line one point longer than a multiple of the cluster's segments (1921 = 3 x 640 + 1) would
// need one more point in every segment; instead its first point is folded into the first
// segment's carry-free start (y_1 = z_1 + M_1 B'^-1_0 r_0) and solved last from the first
// segment's second point (x_0 = y_0 - c_0 y_1 + c_0 c_1 x_2), beside that segment's own chain.
RowPlan row_plan(int n, int nl) {
  RowPlan p;
  p.n = n;
  p.nl = nl;
  p.L = (n + kRMaxSeg - 1) / kRMaxSeg;
  p.H = 0;
  const int L1 = (n - 1 + kRMaxSeg - 1) / kRMaxSeg;
  if (L1 >= 2 && L1 <= 4 && L1 < p.L) { p.L = L1; p.H = 1; }
  p.S = (n - p.H + p.L - 1) / p.L;
  return p;
}

__device__ __forceinline__ void mm3(const double* A, const double* B, double* C) {  // C = A B
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r)
      C[r + 3 * c] = __fma_rn(A[r + 6], B[2 + 3 * c], __fma_rn(A[r + 3], B[1 + 3 * c], A[r] * B[3 * c]));
}
__device__ __forceinline__ void lu3(const double* B, double* x) {  // factored diagonal block
  double d1 = B[0] * x[0];
  double d2 = B[4] * __fma_rn(-B[1], d1, x[1]);
  double d3 = B[8] * __fma_rn(-B[5], d2, __fma_rn(-B[2], d1, x[2]));
  x[2] = d3;
  x[1] = __fma_rn(-B[7], d3, d2);
  x[0] = __fma_rn(-B[3], x[1], __fma_rn(-B[6], d3, d1));
}
// the three components of the vector whose row `r` each lane of a triple holds
__device__ __forceinline__ void pf_l2(const double* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
__device__ __forceinline__ void gather3(double mine, int base, double* v) {
  v[0] = __shfl_sync(0xffffffffu, mine, base);
  v[1] = __shfl_sync(0xffffffffu, mine, base + 1);
  v[2] = __shfl_sync(0xffffffffu, mine, base + 2);
}
// component r of a 3-vector held in registers (a select, not an indexed load)
__device__ __forceinline__ double sel3(const double* v, int r) { return r == 0 ? v[0] : (r == 1 ? v[1] : v[2]); }

}  // namespace

size_t line_ops_rows_doubles(int n, int nl) {
  const RowPlan P = row_plan(n, nl);
  return (size_t)nl * per_line(P.L, P.H);
}
bool rows_supported(int n) { return (n + kRMaxSeg - 1) / kRMaxSeg <= 8; }

// -------------------------------------------------------------------------------- preparation
// One CTA per line, one thread per segment.  Writes, for lane (3 slot + r) of the thread that
// owns segment s, row r of: the forward windows G^(d)_s (product of the transfers of the last
// min(2^d, slot+1) segments of the warp ending at s, d = 0..3) and the warp prefix G^(4)_s; the
// backward windows and suffix mirrored; for the CTA scan (lane 3w + r) the windows over warps
// and the prefix of the warps before w (suffix after w backward); for the cluster scan (lane
// 3c + r) the windows over CTAs.
__global__ void __launch_bounds__(kRMaxSeg) k_line_prep_rows(int n, int nl, int L, int S, int head, int jmax, size_t N,
                                                            const double* __restrict__ b, const double* __restrict__ a,
                                                            const double* __restrict__ c, double* __restrict__ ops) {
  extern __shared__ double sm[];
  double* shF = sm;                  // [kRMaxSeg][9]
  double* shB = sm + kRMaxSeg * 9;   // [kRMaxSeg][9]
  const int line = blockIdx.x;
  const int s = threadIdx.x;
  const bool valid = s < S;
  double* lops = ops + per_line(L, head) * (size_t)line;
  auto pid = [&](int i) -> size_t { return ix(i, line, jmax); };  // lines contiguous (j-lines or k-major copies)
  double F[9], Bw[9];
  for (int e = 0; e < 9; ++e) { F[e] = 0.0; Bw[e] = 0.0; }
  if (valid) {
    const int b0 = head + s * L, e0 = min(n, b0 + L) - 1;
    const int gw0 = s / kSPW, slot0 = s - kSPW * gw0, cta0 = gw0 / kRW, w0 = gw0 - kRW * cta0;
    double* pt = lops + kScanBlocks;
    for (int i = b0; i <= e0; ++i) {
      size_t id = pid(i);
      double Bf[9], M[9], Bi[9];
      for (int e = 0; e < 9; ++e) Bf[e] = b[id + N * e];
      for (int col = 0; col < 3; ++col) {  // explicit inverse of the factored diagonal block
        double x[3] = {col == 0 ? 1.0 : 0.0, col == 1 ? 1.0 : 0.0, col == 2 ? 1.0 : 0.0};
        lu3(Bf, x);
        Bi[3 * col] = x[0]; Bi[1 + 3 * col] = x[1]; Bi[2 + 3 * col] = x[2];
      }
      if (i == 0) {
        for (int e = 0; e < 9; ++e) M[e] = 0.0;
      } else {
        for (int e = 0; e < 9; ++e) M[e] = a[id + N * e];
        for (int col = 0; col < 3; ++col) {
          double x[3] = {M[3 * col], M[1 + 3 * col], M[2 + 3 * col]};
          lu3(Bf, x);
          M[3 * col] = -x[0]; M[1 + 3 * col] = -x[1]; M[2 + 3 * col] = -x[2];
        }
      }
      const int t = i - b0;
      for (int r = 0; r < 3; ++r)
        for (int col = 0; col < 3; ++col) {
          const size_t lanecol = (size_t)cta0 * kRNT + w0 * 32 + 3 * slot0 + r;
          pt[(size_t)(t * 6 + col) * kRCL * kRNT + lanecol] = Bi[r + 3 * col];
          pt[(size_t)(t * 6 + 3 + col) * kRCL * kRNT + lanecol] = M[r + 3 * col];
        }
      if (i == b0) { for (int e = 0; e < 9; ++e) F[e] = M[e]; }
      else { double T[9]; mm3(M, F, T); for (int e = 0; e < 9; ++e) F[e] = T[e]; }
      if (head && i == 1) {  // the head block (the first segment starts at point 1)
        double Bh[9], B0i[9], K[9], C0[9], C1[9], D[9];
        const size_t i0 = pid(0);
        for (int e = 0; e < 9; ++e) Bh[e] = b[i0 + N * e];
        for (int col = 0; col < 3; ++col) {
          double x[3] = {col == 0 ? 1.0 : 0.0, col == 1 ? 1.0 : 0.0, col == 2 ? 1.0 : 0.0};
          lu3(Bh, x);
          B0i[3 * col] = x[0]; B0i[1 + 3 * col] = x[1]; B0i[2 + 3 * col] = x[2];
        }
        mm3(M, B0i, K);
        for (int e = 0; e < 9; ++e) { C0[e] = c[i0 + N * e]; C1[e] = n > 2 ? c[id + N * e] : 0.0; }
        mm3(C0, C1, D);
        double* hb = lops + kScanBlocks + (size_t)L * 6 * kRCL * kRNT;
        for (int r = 0; r < 3; ++r)
          for (int col = 0; col < 3; ++col) {
            hb[3 * col + r] = B0i[r + 3 * col];
            hb[3 * (3 + col) + r] = K[r + 3 * col];
            hb[3 * (6 + col) + r] = C0[r + 3 * col];
            hb[3 * (9 + col) + r] = D[r + 3 * col];
          }
      }
    }
    for (int i = e0; i >= b0; --i) {
      size_t id = pid(i);
      double H[9];
      if (i == n - 1) { for (int e = 0; e < 9; ++e) H[e] = 0.0; }
      else { for (int e = 0; e < 9; ++e) H[e] = -c[id + N * e]; }
      if (i == e0) { for (int e = 0; e < 9; ++e) Bw[e] = H[e]; }
      else { double T[9]; mm3(H, Bw, T); for (int e = 0; e < 9; ++e) Bw[e] = T[e]; }
    }
  }
  const int gw = s / kSPW, slot = s - kSPW * gw;          // warp group and slot of the segment
  const int cta = gw / kRW, w = gw - kRW * cta;
  const int lastslot = min(kSPW - 1, S - 1 - kSPW * gw);  // last valid slot of the group
  auto put_seg = [&](int op, const double* X) {           // rows of X for the three lanes of s
    if (!valid) return;
    for (int r = 0; r < 3; ++r)
      for (int col = 0; col < 3; ++col)
        lops[((size_t)(op * 3 + col) * kRCL + cta) * kRNT + w * 32 + 3 * slot + r] = X[r + 3 * col];
  };
  // windows inside the warp group
  for (int d = 0; d <= kSegLev; ++d) {
    put_seg(d, F);
    put_seg(kSegLev + 1 + d, Bw);
    if (d == kSegLev) break;
    const int o = 1 << d;
    for (int e = 0; e < 9; ++e) { shF[s * 9 + e] = F[e]; shB[s * 9 + e] = Bw[e]; }
    __syncthreads();
    double T[9];
    if (valid && slot - o >= 0) { mm3(F, &shF[(s - o) * 9], T); for (int e = 0; e < 9; ++e) F[e] = T[e]; }
    if (valid && slot + o <= lastslot) { mm3(Bw, &shB[(s + o) * 9], T); for (int e = 0; e < 9; ++e) Bw[e] = T[e]; }
    __syncthreads();
  }
  // warp transfers: forward = prefix at the last slot, backward = suffix at slot 0
  __syncthreads();
  const int ngw = (S + kSPW - 1) / kSPW;  // warp groups with segments
  if (valid && slot == lastslot) for (int e = 0; e < 9; ++e) shF[gw * 9 + e] = F[e];
  __syncthreads();
  if (valid && slot == 0) for (int e = 0; e < 9; ++e) shB[gw * 9 + e] = Bw[e];
  __syncthreads();
  // CTA scan operators: thread t < kRCL * kRW handles warp group t
  const int ncta = (ngw + kRW - 1) / kRW;
  double WF[9], WB[9];
  const int tg = s;                                   // warp group of this thread (if < 64)
  const bool gvalid = tg < ngw;
  const int gc = tg / kRW, gwi = tg - kRW * gc;
  const int glast = min(kRW - 1, ngw - 1 - kRW * gc);  // last valid warp of the CTA
  for (int e = 0; e < 9; ++e) { WF[e] = gvalid ? shF[tg * 9 + e] : 0.0; WB[e] = gvalid ? shB[tg * 9 + e] : 0.0; }
  __syncthreads();
  auto put_w = [&](int op, const double* X, int wi) {  // rows for the lanes 3 wi + r of CTA gc
    for (int r = 0; r < 3; ++r)
      for (int col = 0; col < 3; ++col)
        lops[kSegBlock + ((size_t)gc * 3 * kWOps + op * 3 + col) * 32 + 3 * wi + r] = X[r + 3 * col];
  };
  double shiftF[9], shiftB[9];
  for (int d = 0; d <= kWLev; ++d) {
    if (d < kWLev && gvalid) { put_w(d, WF, gwi); put_w(kWLev + 1 + d, WB, gwi); }
    if (d == kWLev) break;
    const int o = 1 << d;
    if (tg < kRCL * kRW) for (int e = 0; e < 9; ++e) { shF[tg * 9 + e] = WF[e]; shB[tg * 9 + e] = WB[e]; }
    __syncthreads();
    double T[9];
    if (gvalid && gwi - o >= 0) { mm3(WF, &shF[(tg - o) * 9], T); for (int e = 0; e < 9; ++e) WF[e] = T[e]; }
    if (gvalid && gwi + o <= glast) { mm3(WB, &shB[(tg + o) * 9], T); for (int e = 0; e < 9; ++e) WB[e] = T[e]; }
    __syncthreads();
  }
  // WF: product of the transfers of warps 0..gwi of the CTA; WB: of warps gwi..glast.  The
  // carry into warp w uses the prefix of warps 0..w-1 (held by lane 3w + r) and the suffix of
  // warps w+1..glast.
  if (tg < kRCL * kRW) for (int e = 0; e < 9; ++e) { shF[tg * 9 + e] = WF[e]; shB[tg * 9 + e] = WB[e]; }
  __syncthreads();
  if (gvalid) {
    for (int e = 0; e < 9; ++e) {
      shiftF[e] = gwi > 0 ? shF[(tg - 1) * 9 + e] : 0.0;
      shiftB[e] = gwi < glast ? shB[(tg + 1) * 9 + e] : 0.0;
    }
    put_w(kWLev, shiftF, gwi);
    put_w(2 * kWLev + 1, shiftB, gwi);
  }
  __syncthreads();
  // CTA transfers: forward = prefix at the last warp, backward = suffix at warp 0
  if (gvalid && gwi == glast) for (int e = 0; e < 9; ++e) shF[(kRCL * kRW + gc) * 9 + e] = WF[e];
  if (gvalid && gwi == 0) for (int e = 0; e < 9; ++e) shB[(kRCL * kRW + gc) * 9 + e] = WB[e];
  __syncthreads();
  // cluster scan operators: thread t < kRCL handles CTA t
  if (s < kRCL) {
    const bool cv = s < ncta;
    double CF[9], CB[9];
    for (int e = 0; e < 9; ++e) {
      CF[e] = cv ? shF[(kRCL * kRW + s) * 9 + e] : 0.0;
      CB[e] = cv ? shB[(kRCL * kRW + s) * 9 + e] : 0.0;
    }
    double* shF2 = sm + 2 * kRMaxSeg * 9;  // [kRCL][9] scratch, written by these 8 threads only
    double* shB2 = shF2 + kRCL * 9;
    for (int d = 0; d < kCLev; ++d) {
      for (int r = 0; r < 3; ++r)
        for (int col = 0; col < 3; ++col) {
          lops[kSegBlock + kWBlock + (size_t)(d * 3 + col) * 32 + 3 * s + r] = CF[r + 3 * col];
          lops[kSegBlock + kWBlock + (size_t)((kCLev + d) * 3 + col) * 32 + 3 * s + r] = CB[r + 3 * col];
        }
      const int o = 1 << d;
      for (int e = 0; e < 9; ++e) { shF2[s * 9 + e] = CF[e]; shB2[s * 9 + e] = CB[e]; }
      __syncwarp(0xffu);
      double T[9];
      if (cv && s - o >= 0) { mm3(CF, &shF2[(s - o) * 9], T); for (int e = 0; e < 9; ++e) CF[e] = T[e]; }
      if (cv && s + o <= ncta - 1) { mm3(CB, &shB2[(s + o) * 9], T); for (int e = 0; e < 9; ++e) CB[e] = T[e]; }
      __syncwarp(0xffu);
    }
  }
}


// -------------------------------------------------------------------------------------- sweep
struct RowSmem {
  double seg[2][3 * kSegOps][kRNT];   // this thread's operator rows, double-buffered by line
  double wop[2][3 * kWOps][32];       // CTA-scan operator rows (warp 0)
  double cop[2][3 * kCOps][32];       // cluster-scan operator rows (warp 0)
  double aggw[2][kRW][3];             // warp aggregates [fwd/bwd]
  double aggc[2][2][kRCL][3];         // every CTA's aggregate, pushed by its owner [parity][fwd/bwd][cta]
  double carry[2][kRW][3];            // carries into the warps [fwd/bwd]
};

namespace {
// one operator row (3 doubles at stride `stride` starting at p)
__device__ __forceinline__ void ldrow(const double* p, int stride, double* k) {
  k[0] = p[0];
  k[1] = p[stride];
  k[2] = p[2 * stride];
}
// vector held by the triple `off` lanes away (each lane of a triple holds the whole vector)
__device__ __forceinline__ void shfl_vec(const double* v, int src, double* out) {
  out[0] = __shfl_sync(0xffffffffu, v[0], src);
  out[1] = __shfl_sync(0xffffffffu, v[1], src);
  out[2] = __shfl_sync(0xffffffffu, v[2], src);
}
}  // namespace

template <int LMAX>
__global__ void __cluster_dims__(kRCL, 1, 1) __launch_bounds__(kRNT, 1)
    k_gs_sweep_rows(SweepArgs a, int nsw, RowPlan P, const double* __restrict__ ops) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RowSmem& S = *reinterpret_cast<RowSmem*>(smem_raw);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int w = tid >> 5, lane = tid & 31;
  const int slot = lane / 3, r = lane - 3 * (lane / 3);  // lanes 30, 31: slot 10 (idle)
  const int base = 3 * min(slot, kSPW - 1);               // first lane of this triple
  const int gw = rank * kRW + w;
  const int seg = gw * kSPW + slot;
  const bool valid = slot < kSPW && seg < P.S;
  const int ngw = (P.S + kSPW - 1) / kSPW;
  const int ncta = (ngw + kRW - 1) / kRW;
  const int lastslot = min(kSPW - 1, P.S - 1 - kSPW * gw);
  const int nwc = max(0, min(kRW, ngw - kRW * rank));
  const int sw = lane / 3;  // warp 0: warp (CTA scan) or CTA (cluster scan) index of the triple
  const bool wv = w == 0 && lane < 3 * kRW && sw < nwc;    // CTA-scan triple with a warp
  const bool cv = w == 0 && lane < 3 * kRCL && sw < ncta;  // cluster-scan triple with a CTA
  const int up = lane >= 3 ? lane - 3 : lane, dn = lane + 3 <= 31 ? lane + 3 : lane;
  const int jmax = a.jmax;
  const size_t N = a.N;
  const int n = P.n, nl = P.nl, L = P.L;
  const int H = (LMAX >= 2 && LMAX <= 4) ? P.H : 0;  // the plan gives head points only to L = 2..4
  const int beg = H + seg * L;
  // the warp that holds the head point (warp-uniform) and the head point's triple
  const bool hw = H && rank == 0 && w == 0;
  const bool hd = hw && slot == 0;
  const int cnt = valid ? min(n, beg + L) - beg : 0;
  int lb, le, li;
  if ((nsw / 2) * 2 == nsw) { lb = nl - 1; le = 0; li = -1; }
  else { lb = 0; le = nl - 1; li = 1; }

  // every thread copies (and later reads) only its own operator column, so no barrier guards
  // the staging; the next line's operators are staged while this line is solved
  auto stage = [&](int line, int buf) {
    const double* lo = ops + per_line(L, H) * (size_t)line;
    if (valid) {  // threads without a segment never read operators
#pragma unroll 5
      for (int k = 0; k < 3 * kSegOps; ++k)
        __pipeline_memcpy_async(&S.seg[buf][k][tid], lo + ((size_t)k * kRCL + rank) * kRNT + tid, 8);
    }
    // the scan operators that warp 0 applies are copied by warps 1 and 2 (they wait for their
    // copies at the next line's start, before the barrier that precedes warp 0's first use)
    if (w == 1 && nwc > 0) {
      const double* wo = lo + kSegBlock + (size_t)rank * 3 * kWOps * 32;
#pragma unroll 4
      for (int k = 0; k < 3 * kWOps; ++k) __pipeline_memcpy_async(&S.wop[buf][k][lane], wo + (size_t)k * 32 + lane, 8);
    } else if (w == 2 && nwc > 0) {
      const double* co = lo + kSegBlock + kWBlock;
#pragma unroll 3
      for (int k = 0; k < 3 * kCOps; ++k) __pipeline_memcpy_async(&S.cop[buf][k][lane], co + (size_t)k * 32 + lane, 8);
    }
    __pipeline_commit();
  };
  stage(lb, 0);

  double dnew[LMAX][3];
#pragma unroll
  for (int t = 0; t < LMAX; ++t) dnew[t][0] = dnew[t][1] = dnew[t][2] = 0.0;
  // one-point segments: the next line's operands (s, row r of the two off-line blocks, old dq
  // of the point and of the far neighbour line, row r of B'^-1 and M) are loaded into registers
  // while this line is solved, so that a line starts without waiting on memory
  double nx_s = 0.0, nx_dold = 0.0, nx_om[3], nx_op[3], nx_far[3], nx_b[3], nx_m[3];
  double dnew_h[3] = {0.0, 0.0, 0.0};  // the head point's new dq
#pragma unroll
  for (int e = 0; e < 3; ++e) nx_om[e] = nx_op[e] = nx_far[e] = nx_b[e] = nx_m[e] = 0.0;
  int par = 0;
  for (int l = lb;; l += li, par ^= 1) {
    const int buf = par;
    __pipeline_wait_prior(0);
    if (l != le) {
      stage(l + li, buf ^ 1);
      // longer segments: the next line's operands into L2 (each lane of a triple its third of
      // them; one-point segments load theirs into registers below)
      if (LMAX > 1) {
        const int ln = l + li, lf = min(max(ln + li, 0), nl - 1);
        const double* ptn = ops + per_line(L, H) * (size_t)ln + kScanBlocks + (size_t)rank * kRNT + tid;
#pragma unroll
        for (int t = 0; t < LMAX; ++t) {
          if (t < cnt) {
            const size_t id = ix(beg + t, ln, jmax), ifar = ix(beg + t, lf, jmax);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              const size_t e = N * (r + 3 * q);
              pf_l2(a.om + id + e); pf_l2(a.op + id + e); pf_l2(a.cp + id + e);
            }
            pf_l2(a.s + id + N * r); pf_l2(a.dq + id + N * r); pf_l2(a.dq + ifar + N * r);
#pragma unroll
            for (int k = 0; k < 6; ++k) pf_l2(ptn + (size_t)(t * 6 + k) * kRCL * kRNT);
          }
        }
      }
    }
    const int lm = l - 1 > 0 ? l - 1 : 0;
    const int lp = l + 1 < nl - 1 ? l + 1 : nl - 1;
    const bool usem = l - 1 - lm >= 0;  // the reference's 0/1 selectors of the neighbour lines
    const bool usep = lp - l - 1 >= 0;
    const bool first = l == lb;
    const double* sg = &S.seg[buf][0][tid];
    // ---- right-hand sides (row r): independent of one another, all points first
    double rr[LMAX][3], y[LMAX][3], dold[LMAX];
    // rows r of the upper blocks, used by the backward passes, loaded with the right-hand sides
    // (a load after the forward scan's barriers would wait for memory in the middle of the line)
    double Cl[LMAX][3];
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      Cl[t][0] = Cl[t][1] = Cl[t][2] = 0.0;
      if (LMAX > 1 && t < cnt && beg + t < n - 1) {
        const size_t id = ix(beg + t, l, jmax);
        Cl[t][0] = a.cp[id + N * r];
        Cl[t][1] = a.cp[id + N * (r + 3)];
        Cl[t][2] = a.cp[id + N * (r + 6)];
      }
    }
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      double mine = 0.0;
      dold[t] = 0.0;
      if (t < cnt) {
        const int i = beg + t;
        const size_t id = ix(i, l, jmax);
        const size_t im = ix(i, lm, jmax), ip = ix(i, lp, jmax);
        double dm[3], dp[3], omr[3], opr[3], v;
        if (LMAX == 1 && !first) {  // operands loaded during the previous line
          const double* dnw = dnew[t];
          const double* dm_src = li > 0 ? dnw : nx_far;
          const double* dp_src = li > 0 ? nx_far : dnw;
#pragma unroll
          for (int e = 0; e < 3; ++e) { dm[e] = dm_src[e]; dp[e] = dp_src[e]; omr[e] = nx_om[e]; opr[e] = nx_op[e]; }
          dold[t] = nx_dold;
          v = nx_s;
        } else {
          if (li > 0 && !first) { dm[0] = dnew[t][0]; dm[1] = dnew[t][1]; dm[2] = dnew[t][2]; }
          else { dm[0] = a.dq[im]; dm[1] = a.dq[im + N]; dm[2] = a.dq[im + 2 * N]; }
          if (li < 0 && !first) { dp[0] = dnew[t][0]; dp[1] = dnew[t][1]; dp[2] = dnew[t][2]; }
          else { dp[0] = a.dq[ip]; dp[1] = a.dq[ip + N]; dp[2] = a.dq[ip + 2 * N]; }
#pragma unroll
          for (int e = 0; e < 3; ++e) { omr[e] = a.om[id + N * (r + 3 * e)]; opr[e] = a.op[id + N * (r + 3 * e)]; }
          dold[t] = a.dq[id + N * r];
          v = a.s[id + N * r];
        }
        if (!usem) dm[0] = dm[1] = dm[2] = 0.0;
        if (!usep) dp[0] = dp[1] = dp[2] = 0.0;
        v = __fma_rn(-omr[0], dm[0], v);
        v = __fma_rn(-omr[1], dm[1], v);
        v = __fma_rn(-omr[2], dm[2], v);
        v = __fma_rn(-opr[0], dp[0], v);
        v = __fma_rn(-opr[1], dp[1], v);
        mine = __fma_rn(-opr[2], dp[2], v);
      }
      gather3(mine, base, rr[t]);
    }
    // ---- the head point: r_0, y_0 = z_0 = B'^-1_0 r_0, and K r_0 (K = M_1 B'^-1_0), which
    // starts the first segment from y_0 with no carry
    double h_op[12], h_y0[3] = {0.0, 0.0, 0.0}, h_dold = 0.0, h_fold = 0.0;
#pragma unroll
    for (int e = 0; e < 12; ++e) h_op[e] = 0.0;
    if (hw) {
      double mine = 0.0;
      if (hd) {
        const double* hb = ops + per_line(L, 1) * (size_t)l + kScanBlocks + (size_t)L * 6 * kRCL * kRNT;
#pragma unroll
        for (int e = 0; e < 12; ++e) h_op[e] = hb[3 * e + r];
        const size_t id = ix(0, l, jmax), im = ix(0, lm, jmax), ip = ix(0, lp, jmax);
        double dm[3], dp[3];
        if (li > 0 && !first) { dm[0] = dnew_h[0]; dm[1] = dnew_h[1]; dm[2] = dnew_h[2]; }
        else { dm[0] = a.dq[im]; dm[1] = a.dq[im + N]; dm[2] = a.dq[im + 2 * N]; }
        if (li < 0 && !first) { dp[0] = dnew_h[0]; dp[1] = dnew_h[1]; dp[2] = dnew_h[2]; }
        else { dp[0] = a.dq[ip]; dp[1] = a.dq[ip + N]; dp[2] = a.dq[ip + 2 * N]; }
        if (!usem) dm[0] = dm[1] = dm[2] = 0.0;
        if (!usep) dp[0] = dp[1] = dp[2] = 0.0;
        h_dold = a.dq[id + N * r];
        double v = a.s[id + N * r];
        v = __fma_rn(-a.om[id + N * r], dm[0], v);
        v = __fma_rn(-a.om[id + N * (r + 3)], dm[1], v);
        v = __fma_rn(-a.om[id + N * (r + 6)], dm[2], v);
        v = __fma_rn(-a.op[id + N * r], dp[0], v);
        v = __fma_rn(-a.op[id + N * (r + 3)], dp[1], v);
        mine = __fma_rn(-a.op[id + N * (r + 6)], dp[2], v);
      }
      double rh[3];
      gather3(mine, 0, rh);
      double y0r = 0.0;
      if (hd) {
        y0r = __fma_rn(h_op[2], rh[2], __fma_rn(h_op[1], rh[1], h_op[0] * rh[0]));
        h_fold = __fma_rn(h_op[5], rh[2], __fma_rn(h_op[4], rh[1], h_op[3] * rh[0]));
      }
      gather3(y0r, 0, h_y0);
    }
    // ---- local forward pass from a zero carry: y_t = z_t + M_t y_{t-1}, z_t = B'_t^-1 r_t (row r
    // of each, from the precomputed rows; the z_t do not depend on one another)
    const double* pt = ops + per_line(L, H) * (size_t)l + kScanBlocks + (size_t)rank * kRNT + tid;
    double zt[LMAX], Mr[LMAX][3];
    double yp[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      zt[t] = 0.0;
      Mr[t][0] = Mr[t][1] = Mr[t][2] = 0.0;
      if (t < cnt) {
        double b0, b1, b2;
        if (LMAX == 1 && !first) {
          b0 = nx_b[0]; b1 = nx_b[1]; b2 = nx_b[2];
          Mr[t][0] = nx_m[0]; Mr[t][1] = nx_m[1]; Mr[t][2] = nx_m[2];
        } else {
          const double* q = pt + (size_t)(t * 6) * kRCL * kRNT;
          b0 = q[0]; b1 = q[(size_t)kRCL * kRNT]; b2 = q[(size_t)2 * kRCL * kRNT];
          Mr[t][0] = q[(size_t)3 * kRCL * kRNT]; Mr[t][1] = q[(size_t)4 * kRCL * kRNT]; Mr[t][2] = q[(size_t)5 * kRCL * kRNT];
        }
        zt[t] = __fma_rn(b2, rr[t][2], __fma_rn(b1, rr[t][1], b0 * rr[t][0]));
        if (t == 0 && hd) zt[0] = zt[0] + h_fold;
      }
    }
    // this line's operands are consumed: load the next line's (all are fixed during the sweep
    // except this line's dq, which the next line takes from registers; the far neighbour line
    // is not reached before the next line).  Longer segments hide the latency behind their chain.
    if (LMAX == 1 && cnt > 0 && l != le) {
      const int ln = l + li, lf = min(max(ln + li, 0), nl - 1);
      const size_t id = ix(beg, ln, jmax), ifar = ix(beg, lf, jmax);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const size_t e = N * (r + 3 * q);
        nx_om[q] = a.om[id + e];
        nx_op[q] = a.op[id + e];
        nx_far[q] = a.dq[ifar + N * q];
      }
      nx_s = a.s[id + N * r];
      nx_dold = a.dq[id + N * r];
      const double* ptn = ops + per_line(L, H) * (size_t)ln + kScanBlocks + (size_t)rank * kRNT + tid;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        nx_b[k] = ptn[(size_t)k * kRCL * kRNT];
        nx_m[k] = ptn[(size_t)(3 + k) * kRCL * kRNT];
      }
    }
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      double yr = zt[t];
      if (t > 0 && t < cnt) yr = __fma_rn(Mr[t][2], yp[2], __fma_rn(Mr[t][1], yp[1], __fma_rn(Mr[t][0], yp[0], yr)));
      double x[3];
      gather3(yr, base, x);
      if (t < cnt) { yp[0] = x[0]; yp[1] = x[1]; yp[2] = x[2]; }
      y[t][0] = x[0]; y[t][1] = x[1]; y[t][2] = x[2];
    }
    // ---- forward scan of the segment end values inside the warp
    double v[3] = {yp[0], yp[1], yp[2]};
    if (!valid) v[0] = v[1] = v[2] = 0.0;
#pragma unroll
    for (int d = 0; d < kSegLev; ++d) {
      const int o = 1 << d;
      double vn[3];
      shfl_vec(v, lane - 3 * o >= 0 ? lane - 3 * o : lane, vn);
      double nr = sel3(v, r);
      if (valid && slot >= o) {
        double k[3];
        ldrow(sg + (size_t)(d * 3) * kRNT, kRNT, k);
        nr = __fma_rn(k[2], vn[2], __fma_rn(k[1], vn[1], __fma_rn(k[0], vn[0], nr)));
      }
      gather3(nr, base, v);
    }
    if (valid && slot == lastslot) S.aggw[0][w][r] = sel3(v, r);
    __syncthreads();
    double z[3] = {0.0, 0.0, 0.0};
    if (w == 0) {  // CTA scan over the warps
      if (wv) { z[0] = S.aggw[0][sw][0]; z[1] = S.aggw[0][sw][1]; z[2] = S.aggw[0][sw][2]; }
      const int zb = 3 * min(sw, kSPW - 1);
#pragma unroll
      for (int d = 0; d < kWLev; ++d) {
        const int o = 1 << d;
        double zn[3];
        shfl_vec(z, lane - 3 * o >= 0 ? lane - 3 * o : lane, zn);
        double nz = sel3(z, r);
        if (wv && sw >= o) {
          double k[3];
          ldrow(&S.wop[buf][d * 3][lane], 32, k);
          nz = __fma_rn(k[2], zn[2], __fma_rn(k[1], zn[1], __fma_rn(k[0], zn[0], nz)));
        }
        gather3(nz, zb, z);
      }
      if (wv && sw == nwc - 1) {  // push this CTA's aggregate into every CTA of the cluster
        const double val = sel3(z, r);
#pragma unroll
        for (int dst = 0; dst < kRCL; ++dst) *cluster.map_shared_rank(&S.aggc[par][0][rank][r], (unsigned)dst) = val;
      }
    }
    cluster.sync();
    if (w == 0) {  // scan over the CTAs, then the carries into this CTA's warps
      double yc[3] = {0.0, 0.0, 0.0};
      if (cv) { yc[0] = S.aggc[par][0][sw][0]; yc[1] = S.aggc[par][0][sw][1]; yc[2] = S.aggc[par][0][sw][2]; }
      const int cb = 3 * min(sw, kSPW - 1);
#pragma unroll
      for (int d = 0; d < kCLev; ++d) {
        const int o = 1 << d;
        double yn[3];
        shfl_vec(yc, lane - 3 * o >= 0 ? lane - 3 * o : lane, yn);
        double ny = sel3(yc, r);
        if (cv && sw >= o) {
          double k[3];
          ldrow(&S.cop[buf][d * 3][lane], 32, k);
          ny = __fma_rn(k[2], yn[2], __fma_rn(k[1], yn[1], __fma_rn(k[0], yn[0], ny)));
        }
        gather3(ny, cb, yc);
      }
      double cinC[3];  // every lane of a triple holds the vector: take it from lane 3 (rank - 1)
      cinC[0] = __shfl_sync(0xffffffffu, yc[0], rank > 0 ? 3 * (rank - 1) : 0);
      cinC[1] = __shfl_sync(0xffffffffu, yc[1], rank > 0 ? 3 * (rank - 1) : 0);
      cinC[2] = __shfl_sync(0xffffffffu, yc[2], rank > 0 ? 3 * (rank - 1) : 0);
      if (rank == 0) cinC[0] = cinC[1] = cinC[2] = 0.0;
      double zp[3];
      shfl_vec(z, up, zp);  // CTA-local prefix of the warp before
      double ncw = sel3(cinC, r);
      if (wv && sw > 0) {
        double k[3];
        ldrow(&S.wop[buf][kWLev * 3][lane], 32, k);
        ncw = sel3(zp, r) + __fma_rn(k[2], cinC[2], __fma_rn(k[1], cinC[1], k[0] * cinC[0]));
      }
      if (wv) S.carry[0][sw][r] = ncw;
    }
    __syncthreads();
    double cin[3] = {0.0, 0.0, 0.0};
    if (w < nwc) { cin[0] = S.carry[0][w][0]; cin[1] = S.carry[0][w][1]; cin[2] = S.carry[0][w][2]; }
    // segment end values with the carry, and the carry into each segment
    double Yr = sel3(v, r);
    if (valid) {
      double k[3];
      ldrow(sg + (size_t)(kSegLev * 3) * kRNT, kRNT, k);
      Yr = __fma_rn(k[2], cin[2], __fma_rn(k[1], cin[1], __fma_rn(k[0], cin[0], Yr)));
    }
    double Y[3];
    gather3(Yr, base, Y);
    double yin[3];
    shfl_vec(Y, up, yin);
    if (slot == 0) { yin[0] = cin[0]; yin[1] = cin[1]; yin[2] = cin[2]; }
    // forward pass again from the true carry-in (one-point segments take the scanned value)
    if (LMAX == 1) {
      y[0][0] = Y[0]; y[0][1] = Y[1]; y[0][2] = Y[2];
    } else {
      double q[3] = {yin[0], yin[1], yin[2]};
#pragma unroll
      for (int t = 0; t < LMAX; ++t) {
        // M of a line's first point is zero, so the carry drops out there
        double yr = __fma_rn(Mr[t][2], q[2], __fma_rn(Mr[t][1], q[1], __fma_rn(Mr[t][0], q[0], zt[t])));
        double x[3];
        gather3(yr, base, x);
        if (t < cnt) {
          q[0] = x[0]; q[1] = x[1]; q[2] = x[2];
          y[t][0] = x[0]; y[t][1] = x[1]; y[t][2] = x[2];
        }
      }
    }
    // the head point's backward value is y_0 - c_0 y_1 + D x_2 (D = c_0 c_1): the first part now
    double h_w0 = 0.0, h_x0r = 0.0;
    if (hd)
      h_w0 = __fma_rn(-h_op[8], y[0][2], __fma_rn(-h_op[7], y[0][1], __fma_rn(-h_op[6], y[0][0], sel3(h_y0, r))));
    // ---- local backward pass from a zero carry: u = segment start value
    double u[3] = {0.0, 0.0, 0.0};
    {
      double xn[3] = {0.0, 0.0, 0.0};
      bool have = false;
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        double xr = sel3(y[t], r);
        if (t < cnt) {
          if (have) xr = __fma_rn(-Cl[t][2], xn[2], __fma_rn(-Cl[t][1], xn[1], __fma_rn(-Cl[t][0], xn[0], xr)));
        }
        double x[3];
        gather3(xr, base, x);
        if (t < cnt) { xn[0] = x[0]; xn[1] = x[1]; xn[2] = x[2]; have = true; }
      }
      u[0] = xn[0]; u[1] = xn[1]; u[2] = xn[2];
      if (!valid) u[0] = u[1] = u[2] = 0.0;
    }
#pragma unroll
    for (int d = 0; d < kSegLev; ++d) {
      const int o = 1 << d;
      double un[3];
      shfl_vec(u, lane + 3 * o <= 31 ? lane + 3 * o : lane, un);
      double nu = sel3(u, r);
      if (valid && slot + o <= lastslot) {
        double k[3];
        ldrow(sg + (size_t)((kSegLev + 1 + d) * 3) * kRNT, kRNT, k);
        nu = __fma_rn(k[2], un[2], __fma_rn(k[1], un[1], __fma_rn(k[0], un[0], nu)));
      }
      gather3(nu, base, u);
    }
    if (valid && slot == 0) S.aggw[1][w][r] = sel3(u, r);
    __syncthreads();
    if (w == 0) {  // CTA suffix scan over the warps
      z[0] = z[1] = z[2] = 0.0;
      if (wv) { z[0] = S.aggw[1][sw][0]; z[1] = S.aggw[1][sw][1]; z[2] = S.aggw[1][sw][2]; }
      const int zb = 3 * min(sw, kSPW - 1);
#pragma unroll
      for (int d = 0; d < kWLev; ++d) {
        const int o = 1 << d;
        double zn[3];
        shfl_vec(z, lane + 3 * o <= 31 ? lane + 3 * o : lane, zn);
        double nz = sel3(z, r);
        if (wv && sw + o <= nwc - 1) {
          double k[3];
          ldrow(&S.wop[buf][(kWLev + 1 + d) * 3][lane], 32, k);
          nz = __fma_rn(k[2], zn[2], __fma_rn(k[1], zn[1], __fma_rn(k[0], zn[0], nz)));
        }
        gather3(nz, zb, z);
      }
      if (wv && sw == 0) {
        const double val = sel3(z, r);
#pragma unroll
        for (int dst = 0; dst < kRCL; ++dst) *cluster.map_shared_rank(&S.aggc[par][1][rank][r], (unsigned)dst) = val;
      }
    }
    cluster.sync();
    if (w == 0) {
      double yc[3] = {0.0, 0.0, 0.0};
      if (cv) { yc[0] = S.aggc[par][1][sw][0]; yc[1] = S.aggc[par][1][sw][1]; yc[2] = S.aggc[par][1][sw][2]; }
      const int cb = 3 * min(sw, kSPW - 1);
#pragma unroll
      for (int d = 0; d < kCLev; ++d) {
        const int o = 1 << d;
        double yn[3];
        shfl_vec(yc, lane + 3 * o <= 31 ? lane + 3 * o : lane, yn);
        double ny = sel3(yc, r);
        if (cv && sw + o <= ncta - 1) {
          double k[3];
          ldrow(&S.cop[buf][(kCLev + d) * 3][lane], 32, k);
          ny = __fma_rn(k[2], yn[2], __fma_rn(k[1], yn[1], __fma_rn(k[0], yn[0], ny)));
        }
        gather3(ny, cb, yc);
      }
      double cinC[3];
      const int from = rank + 1 < ncta ? 3 * (rank + 1) : 0;
      cinC[0] = __shfl_sync(0xffffffffu, yc[0], from);
      cinC[1] = __shfl_sync(0xffffffffu, yc[1], from);
      cinC[2] = __shfl_sync(0xffffffffu, yc[2], from);
      if (rank + 1 >= ncta) cinC[0] = cinC[1] = cinC[2] = 0.0;
      double zq[3];
      shfl_vec(z, dn, zq);  // CTA-local suffix of the warp after
      double ncw = sel3(cinC, r);
      if (wv && sw < nwc - 1) {
        double k[3];
        ldrow(&S.wop[buf][(2 * kWLev + 1) * 3][lane], 32, k);
        ncw = sel3(zq, r) + __fma_rn(k[2], cinC[2], __fma_rn(k[1], cinC[1], k[0] * cinC[0]));
      }
      if (wv) S.carry[1][sw][r] = ncw;
    }
    __syncthreads();
    double bin[3] = {0.0, 0.0, 0.0};
    if (w < nwc) { bin[0] = S.carry[1][w][0]; bin[1] = S.carry[1][w][1]; bin[2] = S.carry[1][w][2]; }
    double Xr = sel3(u, r);
    if (valid) {
      double k[3];
      ldrow(sg + (size_t)((2 * kSegLev + 1) * 3) * kRNT, kRNT, k);
      Xr = __fma_rn(k[2], bin[2], __fma_rn(k[1], bin[1], __fma_rn(k[0], bin[0], Xr)));
    }
    double X[3];
    gather3(Xr, base, X);
    double xin[3];
    shfl_vec(X, dn, xin);
    if (slot == lastslot || !valid) { xin[0] = bin[0]; xin[1] = bin[1]; xin[2] = bin[2]; }
    // ---- backward pass from the true carry-in, then the relaxation update (row r)
    {
      double xn[3] = {xin[0], xin[1], xin[2]};
      const bool last_seg = beg + cnt == n;
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        double xr;
        if (LMAX == 1) {
          xr = sel3(X, r);
        } else {
          xr = sel3(y[t], r);
          if (t < cnt && !(last_seg && t == cnt - 1))
            xr = __fma_rn(-Cl[t][2], xn[2], __fma_rn(-Cl[t][1], xn[1], __fma_rn(-Cl[t][0], xn[0], xr)));
          if (t == 0 && hd) h_x0r = __fma_rn(h_op[11], xn[2], __fma_rn(h_op[10], xn[1], __fma_rn(h_op[9], xn[0], h_w0)));
        }
        double x[3];
        gather3(xr, base, x);
        double nr = 0.0;
        if (t < cnt) {
          xn[0] = x[0]; xn[1] = x[1]; xn[2] = x[2];
          nr = __fma_rn(a.underr, sel3(x, r) - dold[t], dold[t]);
          a.dq[ix(beg + t, l, jmax) + N * r] = nr;
        }
        double dn3[3];
        gather3(nr, base, dn3);
        dnew[t][0] = dn3[0]; dnew[t][1] = dn3[1]; dnew[t][2] = dn3[2];
      }
    }
    if (hw) {  // the head point's update
      double x0[3];
      gather3(h_x0r, 0, x0);
      double nr = 0.0;
      if (hd) {
        nr = __fma_rn(a.underr, sel3(x0, r) - h_dold, h_dold);
        a.dq[ix(0, l, jmax) + N * r] = nr;
      }
      gather3(nr, 0, dnew_h);
    }
    if (l == le) break;
  }
  // no CTA may leave while another still reads its aggregates
  cluster.sync();
}

void launch_line_prep_rows(int n, int nl, int jmax, size_t N, const double* b, const double* a, const double* c,
                           double* ops, cudaStream_t st) {
  RowPlan P = row_plan(n, nl);
  const int smem = (2 * kRMaxSeg * 9 + 2 * kRCL * 9) * (int)sizeof(double);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_line_prep_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  ++g_kernel_launches;
  k_line_prep_rows<<<nl, kRMaxSeg, smem, st>>>(n, nl, P.L, P.S, P.H, jmax, N, b, a, c, ops);
}

template <int LMAX>
static void launch_rows(const SweepArgs& a, int nsw, const RowPlan& P, const double* ops, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gs_sweep_rows<LMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RowSmem));
    attr = true;
  }
  ++g_kernel_launches;
  k_gs_sweep_rows<LMAX><<<kRCL, kRNT, sizeof(RowSmem), st>>>(a, nsw, P, ops);
}

// lines of length a.jmax, a.kmax of them, contiguous (j-lines, or k-lines on k-major copies)
int launch_gs_sweep_rows(int nsw, const SweepArgs& a, const double* ops, cudaStream_t st) {
  RowPlan P = row_plan(a.jmax, a.kmax);
  if (P.L > 8) return 1;
  if (P.L <= 1) launch_rows<1>(a, nsw, P, ops, st);
  else if (P.L <= 2) launch_rows<2>(a, nsw, P, ops, st);
  else if (P.L <= 3) launch_rows<3>(a, nsw, P, ops, st);
  else if (P.L <= 4) launch_rows<4>(a, nsw, P, ops, st);
  else launch_rows<8>(a, nsw, P, ops, st);
  return 0;
}

}  // namespace smac
