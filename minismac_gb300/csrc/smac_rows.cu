// smac_rows.cu -- reference-order line sweeps with three lanes per segment.
//
// The lines of a sweep are relaxed one after the other (ljsweep / lksweep, ref/lrelax.f:225-561);
// one line is solved by a cluster of kRCL CTAs.  As in smac_lines.cu the line is split into
// segments whose forward (y_i = B'^-1 r_i + M_i y_{i-1}) and backward (x_i = y_i - c_i x_{i+1})
// recurrences are combined over precomputed transfer operators.  The mapping follows GB300's
// FP64 issue limit: a sub-partition issues one FP64 warp instruction every 64 cycles whatever
// the active lanes (152 cycles when two warps share it), so
//   - a segment is owned by three lanes, lane r computing row r of every 3x3 product: three
//     fused multiply-adds per lane and product instead of nine;
//   - a CTA has four warps, one per sub-partition, and a line spreads over a 16-CTA cluster
//     (640 segments of ten per warp);
//   - inside a warp the segments are combined by a Kogge-Stone scan (four levels of three
//     shuffles and three FMAs);
//   - across warps there is no scan: every warp forms its own carry directly, as the sum of its
//     CTA's earlier warps' aggregates and of the earlier CTAs' aggregates, each through a
//     precomputed product of transfers (two terms per lane triple, then a reduction over the
//     warp's triples).  A CTA's aggregate is the sum of its warps' terms, pushed into every CTA
//     of the cluster before one cluster barrier per direction.
// Everything that depends only on the factored blocks (the scan windows, the carry products,
// the rows of B'^-1 and M of every point) is computed once per factorisation for all lines
// (k_line_prep_rows) and laid out per line and CTA as one contiguous block, which one thread
// copies into shared memory with a bulk asynchronous copy (TMA) while the line before it is
// solved.  The waits for those copies are bounded: a wait that runs out records an error status
// that the host reports (SMAC_ERR_TIMEOUT); the kernel then finishes its lines without waiting
// and leaves no copy in flight.  A line one point longer than a multiple of the segments takes
// its first point out of the scan (row_plan).  The arithmetic is contracted to fused
// multiply-adds: results agree with the reference's to rounding, not bit for bit.
#include <cooperative_groups.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

namespace cg = cooperative_groups;

namespace smac {

namespace {

constexpr int kRCL = 16;                    // CTAs per cluster (a non-portable cluster size)
constexpr int kRW = 4;                      // warps per CTA: one per sub-partition
constexpr int kRNT = 32 * kRW;              // threads per CTA
constexpr int kSPW = 10;                    // segments per warp (three lanes each)
constexpr int kSPC = kSPW * kRW;            // segments per CTA
constexpr int kRMaxSeg = kSPC * kRCL;       // segments per line
constexpr int kRWarps = kRW * kRCL;         // warps per line
constexpr int kSegLev = 4;                  // scan levels inside a warp (10 slots); level 4: prefix
constexpr int kSegOps = 2 * (kSegLev + 1);  // forward windows 0..3 + prefix, backward the same
constexpr int kSlots = 2 * kSPW;            // carry terms of a warp: two per lane triple
static_assert(kRCL + kRW - 1 <= kSlots, "a warp's carry terms must fit two per triple");
// Rows (kRNT doubles each, element = thread of the CTA) of one CTA's block of one line.  A lane
// holds row r of every 3x3 operator it applies, column col in row (base + col).
constexpr int kRowSeg = 0;                  // scan operator op (0..9): rows 3 op + col
constexpr int kRowCarF = 3 * kSegOps;       // forward carry terms h = 0, 1 (slots t, t + 10): 3 h + col
constexpr int kRowCarB = kRowCarF + 6;      // backward carry terms
constexpr int kRowAggF = kRowCarB + 6;      // the warp's term of its CTA's forward aggregate
constexpr int kRowAggB = kRowAggF + 3;      // backward
constexpr int kRowPt = kRowAggB + 3;        // per point t of the segment: rows of B'^-1 (3), of M (3)
__host__ __device__ constexpr int block_rows(int L) { return kRowPt + 6 * L; }
__host__ __device__ constexpr size_t block_doubles(int L) { return (size_t)block_rows(L) * kRNT; }
// after the kRCL blocks of a line (lines with a head point): for lane r of the first triple the
// rows r of B'^-1 at point 0, of K = M_1 B'^-1_0, of c_0 and of D = c_0 c_1 (entry e at 3 e + r)
constexpr size_t kHeadBlock = 36;
__host__ __device__ constexpr size_t per_line(int L, int H) {
  return (size_t)kRCL * block_doubles(L) + (size_t)H * kHeadBlock;
}
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // bounded waits: one second

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

__host__ __device__ __forceinline__ void mm3(const double* A, const double* B, double* C) {  // C = A B
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r)
      C[r + 3 * c] = fma(A[r + 6], B[2 + 3 * c], fma(A[r + 3], B[1 + 3 * c], A[r] * B[3 * c]));
}
__device__ __forceinline__ void eye3(double* A) {
  for (int e = 0; e < 9; ++e) A[e] = (e % 4 == 0) ? 1.0 : 0.0;
}
__device__ __forceinline__ void lu3(const double* B, double* x) {  // factored diagonal block
  double d1 = B[0] * x[0];
  double d2 = B[4] * __fma_rn(-B[1], d1, x[1]);
  double d3 = B[8] * __fma_rn(-B[5], d2, __fma_rn(-B[2], d1, x[2]));
  x[2] = d3;
  x[1] = __fma_rn(-B[7], d3, d2);
  x[0] = __fma_rn(-B[3], x[1], __fma_rn(-B[6], d3, d1));
}
__device__ __forceinline__ void pf_l2(const double* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
// the three components of the vector whose row `r` each lane of a triple holds
__device__ __forceinline__ void gather3(double mine, int base, double* v) {
  v[0] = __shfl_sync(0xffffffffu, mine, base);
  v[1] = __shfl_sync(0xffffffffu, mine, base + 1);
  v[2] = __shfl_sync(0xffffffffu, mine, base + 2);
}
// component r of a 3-vector held in registers (a select, not an indexed load)
__device__ __forceinline__ double sel3(const double* v, int r) { return r == 0 ? v[0] : (r == 1 ? v[1] : v[2]); }
// row r of an operator (three doubles kRNT apart in a block) times a 3-vector, added to acc
__device__ __forceinline__ double rowmv(const double* k, const double* v, double acc) {
  return __fma_rn(k[2 * kRNT], v[2], __fma_rn(k[kRNT], v[1], __fma_rn(k[0], v[0], acc)));
}

// --- mbarrier and bulk-copy primitives (inline PTX)
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(void* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try(void* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for the phase of `bar` with parity `parity` to complete; false after kWaitLimitNs
__device__ __noinline__ bool mbar_wait(void* bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  do {
    if (mbar_try(bar, parity)) return true;
  } while (global_ns() - t0 < kWaitLimitNs);
  return false;
}
// one thread: `bytes` (a multiple of 16, both addresses 16-byte aligned) from global memory
// into this CTA's shared memory, completion counted on `bar`
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, void* bar) {
  constexpr uint32_t kChunk = 32768;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  for (uint32_t off = 0; off < bytes; off += kChunk) {
    const uint32_t nb = bytes - off < kChunk ? bytes - off : kChunk;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(static_cast<char*>(dst) + off)),
        "l"(static_cast<const char*>(src) + off), "r"(nb), "r"(smem_addr(bar))
        : "memory");
  }
}

}  // namespace

size_t line_ops_rows_doubles(int n, int nl) {
  const RowPlan P = row_plan(n, nl);
  return (size_t)nl * per_line(P.L, P.H);
}

template <int LMAX>
__global__ void __launch_bounds__(kRNT, 1)
    k_gs_sweep_rows(SweepArgs a, int nsw, RowPlan P, const double* __restrict__ ops, int* __restrict__ wait_status,
                    int stall);

// Whether a 16-CTA cluster of this kernel (one CTA per SM, shared memory of the largest block)
// can be placed on this device.
static bool rows_cluster_ok() {
  static int ok = -1;
  if (ok < 0) {
    ok = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kRCL, 1, 1);
    cfg.blockDim = dim3(kRNT, 1, 1);
    cfg.dynamicSmemBytes = 2 * block_doubles(8) * sizeof(double) + 4096;
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = kRCL; at.val.clusterDim.y = 1; at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaFuncSetAttribute(k_gs_sweep_rows<8>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
        cudaFuncSetAttribute(k_gs_sweep_rows<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)cfg.dynamicSmemBytes) == cudaSuccess &&
        cudaOccupancyMaxActiveClusters(&ncl, k_gs_sweep_rows<8>, &cfg) == cudaSuccess && ncl >= 1)
      ok = 1;
    cudaGetLastError();
  }
  return ok == 1;
}

bool rows_supported(int n) { return (n + kRMaxSeg - 1) / kRMaxSeg <= 8 && rows_cluster_ok(); }

// -------------------------------------------------------------------------------- preparation
// One CTA per line, one thread per segment.  Writes the line's kRCL blocks: for the three lanes
// of each segment's triple the rows of its points' B'^-1 and M, of its scan windows (forward:
// the products of the transfers of the last min(2^d, slot+1) segments of the warp ending at it,
// d = 0..3, and the warp prefix; backward mirrored), and for every warp its carry products:
//   forward, slot c' < kRCL:          K_w Psi_f(c; c')  (c' < c), slot kRCL + w': Phi_f(w; w')  (w' < w)
//   backward, slot c' < kRCL:         Kb_w Psi_b(c; c') (c' > c), slot kRCL + w' - 1: Phi_b(w; w') (w' > w)
// with W_g / V_g the forward / backward transfer of warp g (the product of its segments'),
// T_c = W_{4c+3}..W_{4c} and G_c = V_{4c}..V_{4c+3} the CTAs', Psi_f(c; c') = T_{c-1}..T_{c'+1},
// Psi_b(c; c') = G_{c+1}..G_{c'-1}, K_w = W_{g-1}..W_{4c}, Kb_w = V_{g+1}..V_{4c+3},
// Phi_f(w; w') = W_{g-1}..W_{4c+w'+1}, Phi_b(w; w') = V_{g+1}..V_{4c+w'-1} (empty products are
// the identity), and the warp's term of its CTA's aggregates: W_{4c+3}..W_{g+1} forward,
// V_{4c}..V_{g-1} backward.  Warps and CTAs without segments have identity transfers.
__global__ void __launch_bounds__(kRMaxSeg) k_line_prep_rows(int n, int nl, int L, int S, int head, int jmax, size_t N,
                                                            const double* __restrict__ b, const double* __restrict__ a,
                                                            const double* __restrict__ c, double* __restrict__ ops) {
  extern __shared__ double sm[];
  double* shF = sm;                     // [kRMaxSeg][9]
  double* shB = shF + kRMaxSeg * 9;     // [kRMaxSeg][9]
  double* wF = shB + kRMaxSeg * 9;      // [kRWarps][9] W_g
  double* wB = wF + kRWarps * 9;        // [kRWarps][9] V_g
  double* cF = wB + kRWarps * 9;        // [kRCL][9] T_c
  double* cB = cF + kRCL * 9;           // [kRCL][9] G_c
  double* psF = cB + kRCL * 9;          // [kRCL][kRCL][9] Psi_f(c; c')
  double* psB = psF + kRCL * kRCL * 9;  // [kRCL][kRCL][9] Psi_b(c; c')
  const int line = blockIdx.x;
  const int s = threadIdx.x;
  const bool valid = s < S;
  double* lops = ops + per_line(L, head) * (size_t)line;
  auto pid = [&](int i) -> size_t { return ix(i, line, jmax); };  // lines contiguous (j-lines or k-major copies)
  const int gw = s / kSPW, slot = s - kSPW * gw;  // warp of the segment (along the line) and slot
  const int cta = gw / kRW, w = gw - kRW * cta;
  // rows of X for the three lanes of triple t of warp ww of CTA cc, starting at block row row0
  auto put = [&](int cc, int ww, int t, int row0, const double* X) {
    double* blk = lops + (size_t)cc * block_doubles(L);
    for (int r = 0; r < 3; ++r)
      for (int col = 0; col < 3; ++col) blk[(size_t)(row0 + col) * kRNT + ww * 32 + 3 * t + r] = X[r + 3 * col];
  };
  double F[9], Bw[9];
  eye3(F);
  eye3(Bw);
  if (valid) {
    const int b0 = head + s * L, e0 = min(n, b0 + L) - 1;
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
      put(cta, w, slot, kRowPt + 6 * t, Bi);
      put(cta, w, slot, kRowPt + 6 * t + 3, M);
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
        double* hb = lops + (size_t)kRCL * block_doubles(L);
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
  const int lastslot = min(kSPW - 1, S - 1 - kSPW * gw);  // last valid slot of the warp
  // windows inside the warp (Kogge-Stone), level kSegLev = the warp prefix / suffix
  for (int d = 0; d <= kSegLev; ++d) {
    if (valid) {
      put(cta, w, slot, 3 * d, F);
      put(cta, w, slot, 3 * (kSegLev + 1 + d), Bw);
    }
    if (d == kSegLev) break;
    const int o = 1 << d;
    for (int e = 0; e < 9; ++e) { shF[s * 9 + e] = F[e]; shB[s * 9 + e] = Bw[e]; }
    __syncthreads();
    double T[9];
    if (valid && slot - o >= 0) { mm3(F, &shF[(s - o) * 9], T); for (int e = 0; e < 9; ++e) F[e] = T[e]; }
    if (valid && slot + o <= lastslot) { mm3(Bw, &shB[(s + o) * 9], T); for (int e = 0; e < 9; ++e) Bw[e] = T[e]; }
    __syncthreads();
  }
  // warp transfers: forward = prefix at the last valid slot, backward = suffix at slot 0
  if (s < kRWarps) { eye3(&wF[s * 9]); eye3(&wB[s * 9]); }
  __syncthreads();
  if (valid && slot == lastslot) for (int e = 0; e < 9; ++e) wF[gw * 9 + e] = F[e];
  if (valid && slot == 0) for (int e = 0; e < 9; ++e) wB[gw * 9 + e] = Bw[e];
  __syncthreads();
  // CTA transfers T_c = W_{4c+3}..W_{4c}, G_c = V_{4c}..V_{4c+3}
  if (s < kRCL) {
    double T[9], U[9], X[9];
    for (int e = 0; e < 9; ++e) { T[e] = wF[(kRW * s) * 9 + e]; U[e] = wB[(kRW * s + kRW - 1) * 9 + e]; }
    for (int k = 1; k < kRW; ++k) {
      mm3(&wF[(kRW * s + k) * 9], T, X); for (int e = 0; e < 9; ++e) T[e] = X[e];
      mm3(&wB[(kRW * s + kRW - 1 - k) * 9], U, X); for (int e = 0; e < 9; ++e) U[e] = X[e];
    }
    for (int e = 0; e < 9; ++e) { cF[s * 9 + e] = T[e]; cB[s * 9 + e] = U[e]; }
  }
  __syncthreads();
  // Psi_f(c; c') = T_{c-1}..T_{c'+1} for c' < c, Psi_b(c; c') = G_{c+1}..G_{c'-1} for c' > c
  if (s < kRCL) {
    const int cc = s;
    double P[9], X[9];
    eye3(P);
    for (int cp = cc - 1; cp >= 0; --cp) {  // P = Psi_f(cc; cp)
      for (int e = 0; e < 9; ++e) psF[(cc * kRCL + cp) * 9 + e] = P[e];
      mm3(P, &cF[cp * 9], X); for (int e = 0; e < 9; ++e) P[e] = X[e];
    }
    eye3(P);
    for (int cp = cc + 1; cp < kRCL; ++cp) {  // P = Psi_b(cc; cp)
      for (int e = 0; e < 9; ++e) psB[(cc * kRCL + cp) * 9 + e] = P[e];
      mm3(P, &cB[cp * 9], X); for (int e = 0; e < 9; ++e) P[e] = X[e];
    }
  }
  __syncthreads();
  // carry products: thread s handles warp g = s / kSPW, triple t = s % kSPW, slots t and t + kSPW
  {
    const int g = gw, t = slot, cc = cta, ww = w;
    // K_w = W_{g-1}..W_{4c} and Kb_w = V_{g+1}..V_{4c+3}
    double K[9], Kb[9], X[9];
    eye3(K);
    for (int k = kRW * cc; k < g; ++k) { mm3(&wF[k * 9], K, X); for (int e = 0; e < 9; ++e) K[e] = X[e]; }
    eye3(Kb);
    for (int k = kRW * cc + kRW - 1; k > g; --k) { mm3(&wB[k * 9], Kb, X); for (int e = 0; e < 9; ++e) Kb[e] = X[e]; }
    for (int h = 0; h < 2; ++h) {
      const int sl = t + kSPW * h;
      double Of[9], Ob[9];
      for (int e = 0; e < 9; ++e) { Of[e] = 0.0; Ob[e] = 0.0; }
      if (sl < kRCL) {
        const int cp = sl;
        if (cp < cc) mm3(K, &psF[(cc * kRCL + cp) * 9], Of);
        if (cp > cc) mm3(Kb, &psB[(cc * kRCL + cp) * 9], Ob);
      } else if (sl < kRCL + kRW - 1) {
        const int wf = sl - kRCL;      // forward: earlier warp w' = wf < ww
        if (wf < ww) {
          eye3(Of);
          for (int k = kRW * cc + wf + 1; k < g; ++k) { mm3(&wF[k * 9], Of, X); for (int e = 0; e < 9; ++e) Of[e] = X[e]; }
        }
        const int wb = sl - kRCL + 1;  // backward: later warp w' = wb > ww
        if (wb > ww) {
          eye3(Ob);
          for (int k = kRW * cc + wb - 1; k > g; --k) { mm3(&wB[k * 9], Ob, X); for (int e = 0; e < 9; ++e) Ob[e] = X[e]; }
        }
      }
      put(cc, ww, t, kRowCarF + 3 * h, Of);
      put(cc, ww, t, kRowCarB + 3 * h, Ob);
    }
    // the warp's term of its CTA's aggregate: W_{4c+3}..W_{g+1} forward, V_{4c}..V_{g-1} backward
    double Af[9], Ab[9];
    eye3(Af);
    for (int k = g + 1; k < kRW * cc + kRW; ++k) { mm3(&wF[k * 9], Af, X); for (int e = 0; e < 9; ++e) Af[e] = X[e]; }
    eye3(Ab);
    for (int k = g - 1; k >= kRW * cc; --k) { mm3(&wB[k * 9], Ab, X); for (int e = 0; e < 9; ++e) Ab[e] = X[e]; }
    put(cc, ww, t, kRowAggF, Af);
    put(cc, ww, t, kRowAggB, Ab);
  }
}

// -------------------------------------------------------------------------------------- sweep
template <int LMAX>
struct RowSmem {
  double blk[2][block_rows(LMAX)][kRNT];  // this CTA's block of the line, double-buffered by line
  double aggw[2][kRW][3];                 // raw warp aggregates [fwd/bwd][warp]
  double aggt[2][kRW][3];                 // the warps' terms of the CTA aggregate
  double aggc[2][2][kRCL][3];             // every CTA's aggregate, pushed by its owner [parity][fwd/bwd][cta]
  unsigned long long mbar[2];             // completion of the bulk copy into blk[buf]
  unsigned long long mstall;              // a barrier nothing completes (test of the bounded wait)
};

template <int LMAX>
__global__ void __launch_bounds__(kRNT, 1)
    k_gs_sweep_rows(SweepArgs a, int nsw, RowPlan P, const double* __restrict__ ops, int* __restrict__ wait_status,
                    int stall) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  RowSmem<LMAX>& S = *reinterpret_cast<RowSmem<LMAX>*>(smem_raw);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int w = tid >> 5, lane = tid & 31;
  const int slot = lane / 3, r = lane - 3 * (lane / 3);  // lanes 30, 31: slot 10 (idle)
  const bool tl = slot < kSPW;                            // lane of a triple
  const int base = 3 * min(slot, kSPW - 1);               // first lane of this triple
  const int gw = rank * kRW + w;                          // warp along the line
  const int seg = gw * kSPW + slot;
  const bool valid = tl && seg < P.S;
  const int ngw = (P.S + kSPW - 1) / kSPW;                // warps with segments
  const int ncta = (ngw + kRW - 1) / kRW;                 // CTAs with segments
  const bool wvalid = gw < ngw;
  const bool cvalid = rank < ncta;
  const int lastslot = wvalid ? min(kSPW - 1, P.S - 1 - kSPW * gw) : 0;
  const int jmax = a.jmax;
  const size_t N = a.N;
  const int n = P.n, nl = P.nl, L = P.L;
  const int H = (LMAX >= 2 && LMAX <= 4) ? P.H : 0;  // the plan gives head points only to L = 2..4
  const int beg = H + seg * L;
  // the warp that holds the head point (warp-uniform) and the head point's triple
  const bool hw = H && rank == 0 && w == 0;
  const bool hd = hw && slot == 0;
  const int cnt = valid ? min(n, beg + L) - beg : 0;
  const uint32_t bbytes = (uint32_t)(block_doubles(L) * sizeof(double));
  int lb, le, li;
  if ((nsw / 2) * 2 == nsw) { lb = nl - 1; le = 0; li = -1; }
  else { lb = 0; le = nl - 1; li = 1; }
  auto block_src = [&](int line) { return ops + per_line(L, H) * (size_t)line + (size_t)rank * block_doubles(L); };

  if (tid == 0) {
    mbar_init(&S.mbar[0], 1);
    mbar_init(&S.mbar[1], 1);
    mbar_init(&S.mstall, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t ph[2] = {0u, 0u};  // parity of the next phase of each buffer's barrier
  // thread 0: a bulk copy into blk[b] not yet waited for, and the parity of its completion
  bool pending[2] = {false, false};
  uint32_t pend_ph[2] = {0u, 0u};
  if (tid == 0 && cvalid) { bulk_load(&S.blk[0][0][0], block_src(lb), bbytes, &S.mbar[0]); pending[0] = true; }
  bool failed = false;
  // every CTA runs before any CTA writes into another's shared memory
  cluster.sync();

  double dnew[LMAX][3];
#pragma unroll
  for (int t = 0; t < LMAX; ++t) dnew[t][0] = dnew[t][1] = dnew[t][2] = 0.0;
  // one-point segments: the next line's operands (s, row r of the two off-line blocks, old dq
  // of the point and of the far neighbour line) are loaded into registers while this line is
  // solved, so that a line starts without waiting on memory
  double nx_s = 0.0, nx_dold = 0.0, nx_om[3], nx_op[3], nx_far[3];
  double dnew_h[3] = {0.0, 0.0, 0.0};  // the head point's new dq
#pragma unroll
  for (int e = 0; e < 3; ++e) nx_om[e] = nx_op[e] = nx_far[e] = 0.0;
  int par = 0;
  for (int l = lb;; l += li, par ^= 1) {
    const int buf = par;
    if (cvalid) {
      if (!failed && !mbar_wait(&S.mbar[buf], ph[buf])) {
        failed = true;
        atomicExch(wait_status, SMAC_ERR_TIMEOUT);
      }
      if (tid == 0 && !failed) pending[buf] = false;
      ph[buf] ^= 1u;
    }
    if (stall && rank == 0 && l == lb && !failed && !mbar_wait(&S.mstall, 0u)) {
      failed = true;
      atomicExch(wait_status, SMAC_ERR_TIMEOUT);
    }
    // longer segments: the next line's operands into L2 (each lane of a triple its third of them;
    // one-point segments load theirs into registers below)
    if (LMAX > 1 && l != le) {
      const int ln = l + li, lf = min(max(ln + li, 0), nl - 1);
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
        }
      }
    }
    const int lm = l - 1 > 0 ? l - 1 : 0;
    const int lp = l + 1 < nl - 1 ? l + 1 : nl - 1;
    const bool usem = l - 1 - lm >= 0;  // the reference's 0/1 selectors of the neighbour lines
    const bool usep = lp - l - 1 >= 0;
    const bool first = l == lb;
    const double* bk = &S.blk[buf][0][tid];  // this lane's column of the block
    // ---- right-hand sides (row r): independent of one another, all points first
    double rr[LMAX][3], y[LMAX][3], dold[LMAX];
#pragma unroll
    for (int t = 0; t < LMAX; ++t) y[t][0] = y[t][1] = y[t][2] = 0.0;
    // rows r of the upper blocks, used by the backward passes, loaded with the right-hand sides
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
        const double* hb = ops + per_line(L, 1) * (size_t)l + (size_t)kRCL * block_doubles(L);
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
    // of each, from the block's point rows; the z_t do not depend on one another)
    double zt[LMAX];
#pragma unroll
    for (int t = 0; t < LMAX; ++t) {
      zt[t] = 0.0;
      if (t < cnt) {
        zt[t] = __fma_rn(bk[(kRowPt + 6 * t + 2) * kRNT], rr[t][2],
                         __fma_rn(bk[(kRowPt + 6 * t + 1) * kRNT], rr[t][1], bk[(kRowPt + 6 * t) * kRNT] * rr[t][0]));
        if (t == 0 && hd) zt[0] = zt[0] + h_fold;
      }
    }
    // this line's field operands are consumed: load the next line's (all are fixed during the
    // sweep except this line's dq, which the next line takes from registers; the far neighbour
    // line is not reached before the next line)
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
    }
    double yr_end = 0.0;  // row r of the segment's end value from a zero carry
    {
      double yp[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int t = 0; t < LMAX; ++t) {
        double yr = zt[t];
        if (t > 0 && t < cnt) yr = rowmv(bk + (kRowPt + 6 * t + 3) * kRNT, yp, yr);
        if (LMAX > 1) {
          double x[3];
          gather3(yr, base, x);
          if (t < cnt) { yp[0] = x[0]; yp[1] = x[1]; yp[2] = x[2]; yr_end = yr; }
        } else {
          yr_end = yr;
        }
      }
    }
    // ---- forward scan of the segment end values inside the warp (three shuffles a level: the
    // other triple's components come straight from its three lanes)
    double vr = valid ? yr_end : 0.0;
#pragma unroll
    for (int d = 0; d < kSegLev; ++d) {
      const int o = 1 << d;
      const int src = slot >= o && tl ? base - 3 * o : base;
      double vn[3];
      gather3(vr, src, vn);
      if (valid && slot >= o) vr = rowmv(bk + (3 * d) * kRNT, vn, vr);
    }
    // the warp aggregate (end value of its last segment) and its term of the CTA aggregate
    {
      double av[3];
      gather3(vr, 3 * lastslot, av);
      if (lane < 3) {
        double ar = 0.0, tr = 0.0;
        if (wvalid) {
          ar = sel3(av, r);
          tr = rowmv(bk + kRowAggF * kRNT, av, 0.0);
        }
        S.aggw[0][w][r] = ar;
        S.aggt[0][w][r] = tr;
      }
    }
    __syncthreads();
    // the next line's block: every thread is past its last read of the other buffer
    if (tid == 0 && cvalid && l != le && !failed) {
      bulk_load(&S.blk[buf ^ 1][0][0], block_src(l + li), bbytes, &S.mbar[buf ^ 1]);
      pending[buf ^ 1] = true;
      pend_ph[buf ^ 1] = ph[buf ^ 1];
    }
    if (w == 0 && lane < 3) {  // this CTA's forward aggregate into every CTA of the cluster
      double A = 0.0;
#pragma unroll
      for (int k = 0; k < kRW; ++k) A += S.aggt[0][k][r];
#pragma unroll
      for (int dst = 0; dst < kRCL; ++dst) *cluster.map_shared_rank(&S.aggc[par][0][rank][r], (unsigned)dst) = A;
    }
    // carry into this warp: the terms of the CTA's earlier warps now, the earlier CTAs' after
    // the barrier (row r, two terms per triple)
    double part = 0.0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int sl = slot + kSPW * h;
      if (tl && wvalid && sl >= kRCL && sl < kRCL + kRW - 1 && sl - kRCL < w) {
        const double* av = S.aggw[0][sl - kRCL];
        double v3[3] = {av[0], av[1], av[2]};
        part = rowmv(bk + (kRowCarF + 3 * h) * kRNT, v3, part);
      }
    }
    cluster.sync();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int sl = slot + kSPW * h;
      if (tl && wvalid && sl < kRCL && sl < rank) {
        const double* av = S.aggc[par][0][sl];
        double v3[3] = {av[0], av[1], av[2]};
        part = rowmv(bk + (kRowCarF + 3 * h) * kRNT, v3, part);
      }
    }
#pragma unroll
    for (int o = 1; o < kSPW; o <<= 1) {  // sum over the warp's triples
      const double other = __shfl_down_sync(0xffffffffu, part, 3 * o);
      if (tl && slot + o < kSPW) part += other;
    }
    double cin[3];
    gather3(part, 0, cin);
    // segment end values with the carry, and the carry into each segment
    double Yr = vr;
    if (valid) Yr = rowmv(bk + (3 * kSegLev) * kRNT, cin, Yr);
    double yin[3];
    gather3(Yr, slot >= 1 && tl ? base - 3 : base, yin);
    if (slot == 0) { yin[0] = cin[0]; yin[1] = cin[1]; yin[2] = cin[2]; }
    // forward pass again from the true carry-in (one-point segments take the scanned value)
    if (LMAX > 1) {
      double q[3] = {yin[0], yin[1], yin[2]};
#pragma unroll
      for (int t = 0; t < LMAX; ++t) {
        // M of a line's first point is zero, so the carry drops out there
        double yr = rowmv(bk + (kRowPt + 6 * t + 3) * kRNT, q, zt[t]);
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
    // ---- local backward pass from a zero carry: ur = row r of the segment's start value
    double ur = 0.0;
    {
      double xn[3] = {0.0, 0.0, 0.0};
      bool have = false;
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        double xr = LMAX == 1 ? Yr : sel3(y[t], r);
        if (t < cnt) {
          if (have) xr = __fma_rn(-Cl[t][2], xn[2], __fma_rn(-Cl[t][1], xn[1], __fma_rn(-Cl[t][0], xn[0], xr)));
        }
        if (LMAX > 1) {
          double x[3];
          gather3(xr, base, x);
          if (t < cnt) { xn[0] = x[0]; xn[1] = x[1]; xn[2] = x[2]; have = true; ur = xr; }
        } else {
          ur = xr;
        }
      }
      if (!valid) ur = 0.0;
    }
#pragma unroll
    for (int d = 0; d < kSegLev; ++d) {
      const int o = 1 << d;
      const int src = slot + o <= lastslot && tl ? base + 3 * o : base;
      double un[3];
      gather3(ur, src, un);
      if (valid && slot + o <= lastslot) ur = rowmv(bk + (3 * (kSegLev + 1 + d)) * kRNT, un, ur);
    }
    {
      double bv[3];
      gather3(ur, 0, bv);
      if (lane < 3) {
        double br = 0.0, tr = 0.0;
        if (wvalid) {
          br = sel3(bv, r);
          tr = rowmv(bk + kRowAggB * kRNT, bv, 0.0);
        }
        S.aggw[1][w][r] = br;
        S.aggt[1][w][r] = tr;
      }
    }
    __syncthreads();
    // this CTA's backward aggregate into every CTA of the cluster, by the last warp: it has no
    // later warps in the CTA, so no terms to add before the barrier, while warp 0 has three
    if (w == kRW - 1 && lane < 3) {
      double B = 0.0;
#pragma unroll
      for (int k = 0; k < kRW; ++k) B += S.aggt[1][k][r];
#pragma unroll
      for (int dst = 0; dst < kRCL; ++dst) *cluster.map_shared_rank(&S.aggc[par][1][rank][r], (unsigned)dst) = B;
    }
    part = 0.0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int sl = slot + kSPW * h;
      if (tl && wvalid && sl >= kRCL && sl < kRCL + kRW - 1 && sl - kRCL + 1 > w) {
        const double* bv = S.aggw[1][sl - kRCL + 1];
        double v3[3] = {bv[0], bv[1], bv[2]};
        part = rowmv(bk + (kRowCarB + 3 * h) * kRNT, v3, part);
      }
    }
    cluster.sync();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int sl = slot + kSPW * h;
      if (tl && wvalid && sl < kRCL && sl > rank) {
        const double* bv = S.aggc[par][1][sl];
        double v3[3] = {bv[0], bv[1], bv[2]};
        part = rowmv(bk + (kRowCarB + 3 * h) * kRNT, v3, part);
      }
    }
#pragma unroll
    for (int o = 1; o < kSPW; o <<= 1) {
      const double other = __shfl_down_sync(0xffffffffu, part, 3 * o);
      if (tl && slot + o < kSPW) part += other;
    }
    double bin[3];
    gather3(part, 0, bin);
    double Xr = ur;
    if (valid) Xr = rowmv(bk + (3 * (2 * kSegLev + 1)) * kRNT, bin, Xr);
    double xin[3];
    gather3(Xr, slot + 1 <= lastslot && tl ? base + 3 : base, xin);
    if (slot >= lastslot || !valid) { xin[0] = bin[0]; xin[1] = bin[1]; xin[2] = bin[2]; }
    // ---- backward pass from the true carry-in, then the relaxation update (row r)
    {
      double xn[3] = {xin[0], xin[1], xin[2]};
      const bool last_seg = beg + cnt == n;
#pragma unroll
      for (int t = LMAX - 1; t >= 0; --t) {
        double xr;
        if (LMAX == 1) {
          xr = Xr;
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
          nr = __fma_rn(a.underr, xr - dold[t], dold[t]);
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
  // a wait that ran out: wait (again bounded) for this CTA's own copies still in flight
  if (tid == 0) {
    for (int bb = 0; bb < 2; ++bb)
      if (pending[bb] && !mbar_wait(&S.mbar[bb], pend_ph[bb])) atomicExch(wait_status, SMAC_ERR_TIMEOUT);
  }
  // no CTA may leave while another still writes into its shared memory
  cluster.sync();
}

void launch_line_prep_rows(int n, int nl, int jmax, size_t N, const double* b, const double* a, const double* c,
                           double* ops, cudaStream_t st) {
  RowPlan P = row_plan(n, nl);
  const int smem = (2 * kRMaxSeg * 9 + 2 * kRWarps * 9 + 2 * kRCL * 9 + 2 * kRCL * kRCL * 9) * (int)sizeof(double);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_line_prep_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  ++g_kernel_launches;
  k_line_prep_rows<<<nl, kRMaxSeg, smem, st>>>(n, nl, P.L, P.S, P.H, jmax, N, b, a, c, ops);
}

template <int LMAX>
static void launch_rows(const SweepArgs& a, int nsw, const RowPlan& P, const double* ops, int* wait_status, int stall,
                        cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gs_sweep_rows<LMAX>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(k_gs_sweep_rows<LMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(RowSmem<LMAX>));
    attr = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kRCL, 1, 1);
  cfg.blockDim = dim3(kRNT, 1, 1);
  cfg.dynamicSmemBytes = sizeof(RowSmem<LMAX>);
  cfg.stream = st;
  cudaLaunchAttribute at;
  at.id = cudaLaunchAttributeClusterDimension;
  at.val.clusterDim.x = kRCL; at.val.clusterDim.y = 1; at.val.clusterDim.z = 1;
  cfg.attrs = &at;
  cfg.numAttrs = 1;
  ++g_kernel_launches;
  cudaLaunchKernelEx(&cfg, k_gs_sweep_rows<LMAX>, a, nsw, P, ops, wait_status, stall);
}

// lines of length a.jmax, a.kmax of them, contiguous (j-lines, or k-lines on k-major copies)
int launch_gs_sweep_rows(int nsw, const SweepArgs& a, const double* ops, int* wait_status, int stall,
                         cudaStream_t st) {
  RowPlan P = row_plan(a.jmax, a.kmax);
  if (P.L > 8) return 1;
  if (P.L <= 1) launch_rows<1>(a, nsw, P, ops, wait_status, stall, st);
  else if (P.L <= 2) launch_rows<2>(a, nsw, P, ops, wait_status, stall, st);
  else if (P.L <= 3) launch_rows<3>(a, nsw, P, ops, wait_status, stall, st);
  else if (P.L <= 4) launch_rows<4>(a, nsw, P, ops, wait_status, stall, st);
  else launch_rows<8>(a, nsw, P, ops, wait_status, stall, st);
  return 0;
}

}  // namespace smac
