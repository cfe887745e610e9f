/*
 * smac_gb300.h -- C ABI of the GB300 pseudo-time iteration of miniSMAC2D.
 *
 * One opaque context holds one structured C-grid subgrid resident in GPU
 * memory (grid, metrics, q, the SA variable, the five 3x3 block arrays and
 * all line-solver scratch).  The entry points mirror the reference solver's
 * own interfaces so that a Fortran ISO_C_BINDING shim (or ctypes / any FFI)
 * can replace them one for one:
 *
 *   smac_step     <- subroutine step   (ref/step.f:53-609), followed by the
 *                    force integration of iterout (ref/smac2d.f:1706-1825)
 *   smac_lrelax   <- subroutine lrelax (ref/lrelax.f:51-221)
 *   smac_lreltur  <- subroutine lreltur(ref/lreltur.f:52-160)
 *   smac_lusgs    <- subroutine lusgs  (ref/lusgs.f:51-181)
 *
 * Arrays crossing the boundary use the reference's Fortran layout: REAL*8,
 * column-major, j fastest, e.g. q(jmax,kmax,3) and b(jmax,kmax,3,3) with
 * b(j,k,row,col).  Dimensions are plain ints.  Every call returns an int
 * status (SMAC_OK == 0); the reference has no status codes and stops the
 * program instead (e.g. ref/step.f:557-560, ref/bc.f:202-208).
 *
 * The COMMON blocks that carry the reference's run parameters
 * (ref/include/common.f:45-89: /timm/ /visc/ /impli/ /implr/ /iparmi/
 * /iparmr/ /airfr/ /mass/) become the explicit smac_params struct; the
 * boundary-condition tables read from bcmain.dat (/bcsurf/ /bcwake/) become
 * smac_bcspec; the residual outputs of /rmssi/ /rmssr/ and the forces of
 * iterout become smac_iter_out.
 */
#ifndef SMAC_GB300_H
#define SMAC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SMAC_MAX_BC 64

/* status codes */
#define SMAC_OK 0
#define SMAC_ERR_ARG 1        /* bad argument (sizes, null pointer, parameter out of range) */
#define SMAC_ERR_BC 2         /* boundary-condition table not usable */
#define SMAC_ERR_NONFINITE 3  /* residual or solution not finite */
#define SMAC_ERR_CUDA 4       /* CUDA runtime error */
#define SMAC_ERR_UNSUPPORTED 5
#define SMAC_ERR_NOMEM 6
#define SMAC_ERR_TIMEOUT 7     /* a device-side wait ran out of time (about a second): that iteration's
                                 results are undefined; the context stays usable */

/* smac_params.precision */
#define SMAC_PREC_FP64 0      /* everything in FP64 (parity path) */
#define SMAC_PREC_MIXED 1     /* FP32 implicit operator + line solves inside FP64 defect correction */

/* smac_params.order */
#define SMAC_ORDER_REFERENCE 0  /* the reference's sequential Gauss-Seidel line order */
#define SMAC_ORDER_MULTICOLOR 1 /* red/black (zebra) line order: same fixed point, different history */

/* smac_params.line_solver */
#define SMAC_LINES_PARTITIONED 0 /* segments of a line in parallel + scan across segments */
#define SMAC_LINES_SEQUENTIAL 1  /* one thread walks the line: the reference's exact arithmetic */

/* smac_params.wall_distance */
#define SMAC_WALLDIST_REFERENCE 0 /* as the reference: wall distance only on the first SA call */
#define SMAC_WALLDIST_FIXED 1     /* labelled deviation: keep the wall distance on every call */

typedef struct smac_params {
  /* namelist &input (ref/initia.f:85-89) */
  double alpha;    /* angle of attack, degrees */
  double beta;     /* artificial compressibility */
  double dt;       /* SA time step (1e12: steady) */
  double dtau;     /* pseudo-time step */
  double reynum;   /* Reynolds number; vnu = 1/reynum */
  double underr;   /* line-relaxation under-relaxation factor */
  /* hard-coded defaults (ref/initia.f:104-108, 418-437) */
  double pin, pout; /* pout: outflow static pressure */
  double cdis;      /* flux dissipation coefficient (1.0) */
  double anut_inf;  /* <= 0: the reference's SA free-stream value 0.001 (a REAL*4 literal);
                       > 0: labelled deviation, e.g. 3.0 for nu~ = 3 nu */
  int impsch;       /* 1: line relaxation, 2: LU-SGS */
  int ivis, iturb;  /* viscous / SA switches */
  int njsp, nksp;   /* mean-flow j / k sweeps (2, 2) */
  int ntjsp, ntksp; /* SA j / k sweeps (2, 0) */
  int nbcimp;       /* implicit BC injection frequency (1) */
  int iflxo;        /* flux order: only 3 is reachable in the reference */
  int itrans;       /* transition switch: only 0 (see DESIGN) */
  int wall_distance;/* SMAC_WALLDIST_* */
  int precision;    /* SMAC_PREC_* (GPU only; the oracle is FP64) */
  int order;        /* SMAC_ORDER_* (GPU only) */
  int line_solver;  /* SMAC_LINES_* (GPU only): how one line of a Gauss-Seidel sweep is solved */
  int visc_fp64;    /* 0: viscous fluxes formed in REAL*4 scratch as the reference (ref/visc.f:68);
                       1: labelled deviation, formed in FP64, so that the residual is smooth in q
                       and the grid (finite-difference checks of the adjoint) */
  int reserved[2];
} smac_params;

/* bcmain.dat rows: ibcval zone jbeg jend kbeg kend, with the reference's
   negative index convention (-1 -> max, -2 -> max-1, ref/rbc.f:387-398). */
typedef struct smac_bcspec {
  int nbc;
  int ibcval[SMAC_MAX_BC];
  int nzbc[SMAC_MAX_BC];
  int jbcb[SMAC_MAX_BC];
  int jbce[SMAC_MAX_BC];
  int kbcb[SMAC_MAX_BC];
  int kbce[SMAC_MAX_BC];
} smac_bcspec;

/* one pseudo-time iteration's scalars: /rmssi/ /rmssr/ of resid (ref/step.f:613-756)
   and the coefficients of iterout (ref/smac2d.f:1737-1745, 1830-1947) */
typedef struct smac_iter_out {
  int nt;          /* iteration counter (1-based) */
  int jres, kres;  /* location of resmax (1-based, first maximum) */
  int neq_res;     /* equation of resmax (1..3) */
  double resmax;   /* max |s*dj| over all points and equations */
  double resmax0;  /* resmax of iteration 1, at least 1.0 */
  double rmax;     /* resmax / resmax0 */
  double divmax;   /* max |s1*dj| / beta */
  double turres;   /* max SA update */
  double rhsnorm;  /* L2 norm of s before the solve (ref/step.f:513-519) */
  double cd, cl, cm, cdp, clp;
} smac_iter_out;

typedef struct smac_ctx smac_ctx;

/* Reference defaults (ref/initia.f, inizone; ref/smac2d.in flow values). */
void smac_params_default(smac_params* p);

/* Create a context on the current CUDA device: uploads x,y (jmax*kmax each,
   j fastest), preprocesses the BC table, computes metrics (ref/metric.f:49-278)
   and the initial condition (ref/geom.f:88-131).  Replaces the setup half of
   solve (ref/smac2d.f:1238-1332). */
int smac_ctx_create(const smac_params* p, int jmax, int kmax, const double* x,
                    const double* y, const smac_bcspec* bc, smac_ctx** out);
int smac_ctx_destroy(smac_ctx* ctx);

/* One pseudo-time iteration (ref/step.f:53-609) plus the force integration
   and residual bookkeeping of iterout (ref/smac2d.f:1706-1947): state stays
   on the device; out receives the scalars. */
int smac_step(smac_ctx* ctx, smac_iter_out* out);

/* The first half of a step only: SA model, residual, implicit operator, boundary
   conditions and resid (ref/step.f:104-519), without the solve and the update.
   For stage-by-stage checks; the next smac_step starts a new iteration. */
int smac_assemble(smac_ctx* ctx, smac_iter_out* out);

/* Run n iterations; hist (may be NULL) receives n records.  Stops early only
   on a non-finite residual (status SMAC_ERR_NONFINITE). */
int smac_run(smac_ctx* ctx, int n, smac_iter_out* hist);

/* Copy state between host and device.  Fields below; sizes are jmax*kmax*ncomp doubles. */
#define SMAC_FIELD_Q 0      /* q(jmax,kmax,3)        */
#define SMAC_FIELD_ANUT 1   /* turvar(:,:,1)         */
#define SMAC_FIELD_VNUT 2   /* vnut                  */
#define SMAC_FIELD_S 3      /* s(jmax,kmax,3)        */
#define SMAC_FIELD_DQ 4     /* dq(jmax,kmax,3)       */
#define SMAC_FIELD_RTXY 5   /* rtxy(jmax,kmax,2,3)   */
#define SMAC_FIELD_DJ 6     /* dj                    */
#define SMAC_FIELD_BTC 7    /* btc(jmax,kmax,3,3)    */
#define SMAC_FIELD_BJM 8
#define SMAC_FIELD_BJP 9
#define SMAC_FIELD_BKM 10
#define SMAC_FIELD_BKP 11
#define SMAC_FIELD_SMIN 12  /* wall distance (first SA call) */
int smac_get_field(smac_ctx* ctx, int field, double* host);
int smac_set_field(smac_ctx* ctx, int field, const double* host);
/* Host copies of the state most callers want: q (3N), turvar (N), vnut (N); any may be NULL.
   An iteration whose residual is not finite leaves a flag that makes it and every later
   iteration return SMAC_ERR_NONFINITE; smac_set_state with a q clears it. */
int smac_get_state(smac_ctx* ctx, double* q, double* turvar, double* vnut);
int smac_set_state(smac_ctx* ctx, const double* q, const double* turvar);
/* The far-field vortex strength the next iteration uses (COMMON /airfr/ clift: the lift of the
   previous iteration, 0 before the first, ref/initia.f:329, ref/bc.f:1364-1374).  For restarts
   from a saved state. */
int smac_get_clift(smac_ctx* ctx, double* clift);
int smac_set_clift(smac_ctx* ctx, double clift);

/* Stage-level drop-ins with the reference's argument lists.  They run on the
   device on the caller's host arrays (copied in and out): */
/* lrelax(jmax,kmax,q,dq,s,btc,bjm,bjp,bkm,bkp): dq out; s modified on the
   wake-cut rows by the implicit BC injection; btc,bjm,bjp,bkm,bkp restored. */
int smac_lrelax(smac_ctx* ctx, int jmax, int kmax, const double* q, double* dq, double* s,
                double* btc, double* bjm, double* bjp, double* bkm, double* bkp);
/* lreltur(jmax,kmax,turvar,ds,rhs,sjm,sjp,skm,skp,stc,nodeidp1) */
int smac_lreltur(smac_ctx* ctx, int jmax, int kmax, const double* turvar, double* ds,
                 double* rhs, const double* sjm, const double* sjp, const double* skm,
                 const double* skp, const double* stc);
/* lusgs(jmax,kmax,neqs,q,dq,rhs,btc,bjm,bjp,bkm,bkp,scr1), neqs 1 or 3: dq
   out; rhs overwritten (as the reference's ilusol does); scr1 receives the
   factored diagonal blocks bprm. */
int smac_lusgs(smac_ctx* ctx, int jmax, int kmax, int neqs, const double* q, double* dq,
               double* rhs, const double* btc, const double* bjm, const double* bjp,
               const double* bkm, const double* bkp, double* scr1);

/* Timing helpers for measurement: device time (ms) of the last smac_run, and
   the number of kernel launches one iteration issues. */
double smac_last_run_ms(smac_ctx* ctx);
int smac_launches_per_iter(smac_ctx* ctx);

/* Stages of one iteration, timed by smac_profile_iteration (device ms each). */
#define SMAC_STAGE_SA 0        /* turvis/tursa: SA assembly, SA solve, update */
#define SMAC_STAGE_ASSEMBLE 1  /* conup + viscterms + blanking + identity + bcmain */
#define SMAC_STAGE_RESID 2     /* resid + L2 norm */
#define SMAC_STAGE_FACTOR_J 3  /* btlu3j (impsch 1) or the whole LU-SGS solve (impsch 2) */
#define SMAC_STAGE_SWEEP_J 4   /* j line sweeps + bcimpds */
#define SMAC_STAGE_UNDO_J 5    /* btund3j */
#define SMAC_STAGE_FACTOR_K 6  /* btlu3k */
#define SMAC_STAGE_SWEEP_K 7   /* k line sweeps + bcimpds */
#define SMAC_STAGE_UPDATE 8    /* update + force integration */
#define SMAC_NSTAGES 9
/* Run one iteration with an event at every stage boundary; stage_ms[SMAC_NSTAGES]. */
int smac_profile_iteration(smac_ctx* ctx, double* stage_ms);

/* Autotuner of the throughput forms (zebra order, FP32 operator): picks the shape of
   the line solves per line direction, 1, 2 or 4 lines per warp or (negative values)
   2 or 4 warps per line, by timing the choices on this context's grid; runs once at
   context creation (unless the environment sets SMAC_NO_AUTOTUNE) and again here only
   if it has not run.  lines_per_warp[2] receives the choice for j and k lines (may be
   NULL).  The environment variable SMAC_ZEBRA_SHAPE="j,k" (each 1, 2, 4, -2 or -4) fixes the
   shapes instead of timing them, for comparisons between shapes.  At the same time, for
   every form, it picks the tile shape of the assembly kernels (lines x points per CTA) per
   direction among four, by timing them on this grid; every tile shape gives the same bits.
   SMAC_CONUP_SHAPE="j,k" (each 0..3, 0 = the default tile) fixes them instead.  No reference
   counterpart. */
int smac_autotune(smac_ctx* ctx, int* lines_per_warp);
/* The assembly tile shapes in use, j and k direction (0..3), into tiles[2]. */
int smac_assembly_tiles(smac_ctx* ctx, int* tiles);

/* Batches: many independent cases (each its own context: grid, airfoil, flow, form)
   advanced together, one CUDA graph launch per pseudo-time iteration of all cases
   (one branch per case, run concurrently).  No reference counterpart: the reference
   runs one case per process.  The contexts stay owned by the caller and must outlive
   the batch; a context may belong to one batch at a time.  smac_batch_run advances
   every case n iterations; hist (may be NULL) receives ncases x n records, case-major.
   Before its first run (and after smac_batch_options) a batch picks one assembly tile shape
   per direction for all its cases by timing their assembly kernels launched together (unless
   SMAC_CONUP_SHAPE fixes them); the cases keep that shape.
   smac_batch_last_run_ms: device time of the last smac_batch_run. */
typedef struct smac_batch smac_batch;
int smac_batch_create(int ncases, smac_ctx* const* cases, smac_batch** batch);
int smac_batch_run(smac_batch* batch, int n, smac_iter_out* hist);
/* Batch layout (before the first smac_batch_run, or to rebuild the graph): SMAC_BATCH_GRAPH
   [default] = each case's iteration as its own branch of the graph; SMAC_BATCH_PACKED_LINES =
   the line solves of all cases packed into one launch per sweep colour, a CTA of
   warps_per_line (2 or 4) warps per line, between the cases' own work before and after their
   sweeps (every case must be the FP32-operator zebra form with the same sweep counts;
   otherwise SMAC_ERR_UNSUPPORTED); SMAC_BATCH_QUEUE_LINES = the line sweeps of an iteration
   of all cases (every sweep colour of both directions and the wake-cut injections) in one
   persistent launch that takes its items (a line, or a case's wake-cut injection) from one
   work queue, largest cases first, between the cases' own work before and after their sweeps;
   an item waits only for the previous phase of its own case, with a bounded wait (about a
   second) whose running out makes smac_batch_run return SMAC_ERR_TIMEOUT (same requirements
   as SMAC_BATCH_PACKED_LINES; bit-identical to it). */
#define SMAC_BATCH_GRAPH 0
#define SMAC_BATCH_PACKED_LINES 1
#define SMAC_BATCH_QUEUE_LINES 2
int smac_batch_options(smac_batch* batch, int layout, int warps_per_line);
double smac_batch_last_run_ms(smac_batch* batch);
int smac_batch_destroy(smac_batch* batch);

/* Discrete adjoint of the converged iteration.  No reference counterpart: the reference
   computes no sensitivities.  At a fixed point (dq = 0) the state satisfies the steady
   equations F(q, clift) = 0: F is the assembled right-hand side s of step (ref/step.f:268-519)
   on every row but the wake cut, where F(jt,1) = (q(jt,2) + q(jb,2))/2 - q(jt,1) (what bcimpds,
   ref/bc.f:566-595, imposes), and the far field's vortex strength is the lift itself
   (clift = Cl, ref/smac2d.f:1825).  For J = Cl or Cd the adjoint lambda solves
       A^T lambda = -dJ/dq,   A = dF/dq + (dF/dclift) (dCl/dq)^T,
   and dJ/db = J_b + lambda . F_b + (lambda . dF/dclift) Cl_b for a design variable b.
   Sequence: converge the state (smac_run), smac_adjoint_prepare (linearises at the current
   state: exact dF/dq on the 9-point cross stencil by forward-mode differentiation, the force
   gradients, the transposed implicit operator), smac_adjoint_solve per objective (restarted
   GMRES on A^T, preconditioned by transposed line relaxation of the implicit operator),
   then smac_adjoint_gradient for any number of design variables. */
#define SMAC_OBJ_CL 0
#define SMAC_OBJ_CD 1
int smac_adjoint_prepare(smac_ctx* ctx);
/* Preconditioner of the transposed solve (set before smac_adjoint_prepare; defaults in
   brackets): zebra block-tridiagonal line relaxation of the transposed implicit operator with
   that operator rounded to FP32 [SMAC_ADJ_PREC_LINES_F32] or in FP64 (SMAC_ADJ_PREC_LINES),
   `sweeps` red/black sweeps per line direction [1]; or its LU-SGS sweeps (SMAC_ADJ_PREC_LUSGS).
   dtau = pseudo-time step of that operator [<= 0: 40 x the iteration's dtau]; inner =
   stationary steps of the transposed iteration per preconditioner application [16]; restart =
   GMRES restart length, 1..200 [100]. */
#define SMAC_ADJ_PREC_LUSGS 0
#define SMAC_ADJ_PREC_LINES 1
#define SMAC_ADJ_PREC_LINES_F32 2  /* the line relaxation with the operator rounded to FP32 */
int smac_adjoint_options(smac_ctx* ctx, int preconditioner, double dtau, int inner, int sweeps, int restart);
/* rtol: relative residual of the adjoint system; max_iter: GMRES iterations.
   iters, rel_resid may be NULL. */
int smac_adjoint_solve(smac_ctx* ctx, int objective, double rtol, int max_iter, int* iters, double* rel_resid);
/* ndv design variables, each a grid motion (dxdb, dydb: ndv x jmax*kmax host arrays, j fastest;
   NULL = no motion) and a change of the angle of attack in degrees per unit of the variable
   (dalpha: ndv values; NULL = none).  grad: ndv values of dJ/db for the objective of the last
   smac_adjoint_solve with that objective. */
int smac_adjoint_gradient(smac_ctx* ctx, int objective, int ndv, const double* dxdb, const double* dydb,
                          const double* dalpha, double* grad);
/* F(q, clift) at the current state (3*jmax*kmax doubles, host) */
int smac_adjoint_residual(smac_ctx* ctx, double* F);
/* y = A v (transpose 0) or A^T v (transpose 1), host arrays of 3*jmax*kmax doubles */
int smac_adjoint_jacvec(smac_ctx* ctx, int transpose, const double* v, double* y);
/* copies of the adjoint's fields (host; 3*jmax*kmax doubles, the Jacobian 81*jmax*kmax:
   block s (centre, j-1, j+1, j-2, j+2, k-1, k+1, k-2, k+2) entry (row r, col c) of point p at
   p + N*(9s + r + 3c)) */
#define SMAC_ADJ_LAMBDA_CL 0
#define SMAC_ADJ_LAMBDA_CD 1
#define SMAC_ADJ_DCL_DQ 2
#define SMAC_ADJ_DCD_DQ 3
#define SMAC_ADJ_DF_DCLIFT 4
#define SMAC_ADJ_JACOBIAN 5
int smac_adjoint_get(smac_ctx* ctx, int field, double* host);
/* Cl and Cd of the state the adjoint was prepared at */
int smac_adjoint_forces(smac_ctx* ctx, double* cl, double* cd);

/* Last error message of this thread (static storage). */
const char* smac_last_error(void);

/* Residual norms without any device allocation.  This entry point has no
   counterpart in the reference: it exists for callers that cannot call
   cudaMalloc, such as a Fortran host that owns every device array itself
   (CUDA Fortran or OpenACC data regions) and may not let a library allocate
   behind it, or a host loop running under a fixed device-memory budget.
   From s(jmax,kmax,3) and dj(jmax,kmax) already in device memory it computes
   the residual scalars of one pseudo-time iteration and writes them to the
   host struct out: resmax = max |s*dj| over all points and equations, with
   the first point in j-fastest order winning ties, its location jres, kres,
   neq_res, divmax = max |s(:,:,1)*dj| / beta, and rhsnorm, the L2 norm of s.
   With first_iteration != 0 the call also reports resmax0 = max(resmax, 1)
   and rmax = resmax / resmax0 (nt = 1); with first_iteration == 0 it keeps no
   resmax0 between calls, so resmax0, rmax and nt come back as 0 and the
   caller divides resmax by the resmax0 of its own first call.
   Limits: jmax and kmax between 5 and 8100; larger grids are rejected with
   SMAC_ERR_ARG.  Scratch: a fixed 16 KiB file-scope device array that every
   GPU loading the library keeps until the process exits; all calls share it,
   so calls that overlap on the GPU race.  The first call on each device looks
   the array's address up (cudaGetSymbolAddress) with that device current.
   Every call copies through host memory and waits for stream, so no call may
   be made while stream (or, for a NULL stream, the legacy stream) is being
   captured into a graph: such a call returns SMAC_ERR_UNSUPPORTED without
   touching the stream.  stream may be NULL (the legacy default stream); the
   call returns after the result is on the host.
   Errors: smac_noalloc_last_error(). */
int smac_resid_noalloc(const double* s_dev, const double* dj_dev, int jmax, int kmax, double beta,
                       int first_iteration, void* stream, smac_iter_out* out);
const char* smac_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
