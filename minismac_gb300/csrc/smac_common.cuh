// smac_common.cuh -- shared device-side types and helpers of the GB300 pseudo-time iteration.
//
// Layout: every field is stored exactly as the reference's Fortran arrays, column-major with
// j fastest: point (j,k) (0-based here) at j + jmax*k; component n of a vector field at
// + N*n; entry (row r, col c) of a 3x3 block field at + N*(r + 3*c).  One plane per component
// keeps every point-wise kernel fully coalesced.
//
// Arithmetic: the library is compiled with -fmad=false so that the FP64 kernels evaluate the
// reference's expressions operation by operation (no fused multiply-add contraction).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/smac_gb300.h"

#define FLIT(x) ((double)(float)(x))  // a Fortran REAL*4 literal promoted to REAL*8

namespace smac {

constexpr int kMaxWallPts = 1 << 16;

struct BCRegion {
  int ibcval, jkbc;  // jkbc: 1 = j constant, 2 = k constant
  int jb, je, kb, ke;  // 0-based inclusive
};

// Preprocessed bcmain.dat (single zone), see ref/rbc.f:347-398, 926-989, 1160-1345.
struct BCTable {
  int nreg;
  BCRegion reg[SMAC_MAX_BC];
  int nwall;
  int wjk[SMAC_MAX_BC], wj1[SMAC_MAX_BC], wj2[SMAC_MAX_BC], wk1[SMAC_MAX_BC], wk2[SMAC_MAX_BC];
  int nwake;  // 0 or 2 wake-cut pairs
  int jt_b[2], jt_e[2], jb_b[2];  // target range (ascending) and base start (descending), 0-based
};

// Scalars that live on the device across iterations (ref COMMON /airfr/ /rmssr/ /rmssi/).
struct DevScalars {
  double clift, resmax0, resmax, divmax, turres, rhsnorm;
  double cd, cl, cm, cdp, clp;
  double rhs_partial_pad;
  int nt, jres, kres, neq, status;
  int wait_status;  // SMAC_ERR_TIMEOUT when a bounded device wait of this iteration ran out
  int pad[2];
};

struct Dims {
  int jmax, kmax;
  size_t N;
};

__host__ __device__ __forceinline__ size_t ix(int j, int k, int jmax) { return (size_t)j + (size_t)jmax * (size_t)k; }

// gfortran -O2 expansion of integer powers
__device__ __forceinline__ double p2(double x) { return x * x; }
__device__ __forceinline__ double p3(double x) { return (x * x) * x; }
__device__ __forceinline__ double p4(double x) { double t = x * x; return t * t; }
__device__ __forceinline__ double p5(double x) { double t2 = x * x; double t3 = t2 * x; return t3 * t2; }
__device__ __forceinline__ double p6(double x) { double t3 = (x * x) * x; return t3 * t3; }
__device__ __forceinline__ double fmaxf90(double a, double b) { return (a >= b) ? a : b; }
__device__ __forceinline__ double fminf90(double a, double b) { return (a < b) ? a : b; }

}  // namespace smac
