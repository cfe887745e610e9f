// smac_adjoint.cuh -- host interface of the discrete adjoint (smac_adjoint.cu).
#pragma once
#include "smac_common.cuh"

namespace smac {

constexpr int kAdjSlots = 9;
constexpr int kAdjMaxRestart = 200;

struct AdjointOptions {
  int preconditioner;  // SMAC_ADJ_PREC_*
  double dtau;         // pseudo-time step of the preconditioner's operator (<= 0: the iteration's)
  int inner;           // stationary steps per preconditioner application
  int sweeps;          // zebra sweeps per line direction
  int restart;         // GMRES restart length
};  // blocks of a Jacobian row: centre, j-1, j+1, j-2, j+2, k-1, k+1, k-2, k+2

// what the adjoint reads from a context: the converged state, its geometry and the implicit
// operator assembled at that state
struct AdjointCtx {
  int jmax, kmax;
  double beta, cdis, vnu, pout, pi, ca, sa, clift, dtau;
  int ivis, visc64;
  const double *q, *rtxy, *dj, *x, *y;
  const double *btc, *bjm, *bjp, *bkm, *bkp;
  const BCTable* d_bc;  // device copy
  const BCTable* bc;    // host copy
  int lpw[2];           // zebra line shapes of the context (lines per warp; negative: warps per line)
  cudaStream_t st;
};

struct AdjointImpl;
AdjointImpl* adjoint_new(const AdjointCtx& c, const AdjointOptions& o, int* rc, char* msg, size_t msglen);
void adjoint_free(AdjointImpl* A);
void adjoint_update(AdjointImpl* A, const AdjointCtx& c, const AdjointOptions& o);
const char* adjoint_error(AdjointImpl* A);
int adjoint_prepare(AdjointImpl* A);
int adjoint_solve(AdjointImpl* A, int obj, double rtol, int max_iter, int* iters, double* rel);
int adjoint_gradient(AdjointImpl* A, int obj, int ndv, const double* dx, const double* dy, const double* da,
                     double* grad);
int adjoint_residual(AdjointImpl* A, double* F);
int adjoint_jacvec(AdjointImpl* A, int transpose, const double* v, double* y);
int adjoint_get(AdjointImpl* A, int what, double* host);
void adjoint_forces(AdjointImpl* A, double* cl, double* cd);

}  // namespace smac
