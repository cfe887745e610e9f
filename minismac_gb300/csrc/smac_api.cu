// smac_api.cu -- the C ABI (include/smac_gb300.h): context, setup and the per-iteration
// launch sequence of the pseudo-time step.
//
// One context = one subgrid resident in HBM.  An iteration is a fixed sequence of kernel
// launches on the context's stream with no host synchronisation: the scalars that the
// reference keeps in COMMON (clift, resmax0, nt, ...) live in device memory, so the sequence
// can be replayed from a captured CUDA graph.
#include <math.h>
#include <stddef.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "smac_adjoint.cuh"
#include "smac_common.cuh"
#include "smac_kernels.cuh"

using namespace smac;

long long smac::g_kernel_launches = 0;

// optional stage timing (smac_profile_iteration): an event at every stage boundary, in order
struct StageTimer {
  cudaEvent_t ev[64];
  int stage[64];
  int n;
  bool on;
};
static thread_local StageTimer* g_timer = nullptr;

static void mark(cudaStream_t st, int stage) {
  if (!g_timer || !g_timer->on || g_timer->n >= 64) return;
  cudaEventRecord(g_timer->ev[g_timer->n], st);
  g_timer->stage[g_timer->n] = stage;
  g_timer->n++;
}

static thread_local char g_err[512];

static void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

#define CK(x)                                                                          \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) {                                                           \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));         \
      return SMAC_ERR_CUDA;                                                            \
    }                                                                                  \
  } while (0)

struct smac_ctx {
  smac_params p;
  int jmax, kmax;
  size_t N;
  BCTable bc;
  BCTable* d_bc;
  double vnu, pi, ca, sa, rterm, anutinf, cv1;
  cudaStream_t st;
  cudaStream_t st_sa;          // the SA model runs here, beside the mean-flow solve
  cudaEvent_t ev_fork, ev_join;
  cudaStream_t st_fk;          // FP32 k-line factorisation beside the j-line factorisation and sweeps
  cudaEvent_t ev_fk_fork, ev_fk_join;
  // fields (Fortran layout)
  double *x, *y, *rtxy, *dj, *q, *dq, *s, *anut, *vnut, *smin;
  double *btc, *bjm, *bjp, *bkm, *bkp, *bjp_r, *scr9, *bprm;
  double* kmaj;               // k-major copies of the k-sweep operands (partitioned lines)
  bool rows;                  // partitioned lines with three lanes per segment (smac_rows.cu)
  double *sjm, *sjp, *skm, *skp, *stc, *sf, *ds, *sa_piv, *sa_cf;
  double *vort, *crs, *cs11, *cs12, *fr1;
  double *wall_xy;
  double *line_ops;
  double *line_ops_k, *kfac; // k-line operators and unfactored k blocks, prepared beside the j sweeps
  double *zwork, *sa_work;   // zebra scratch (FP64 line forward values, SA line values)
  F32Ops f32;                // FP32 operator of the mixed-precision form
  bool throughput;           // zebra order and/or FP32 operator
  int zlpw[2];               // zebra lines per warp, j and k lines (autotuned; 0 = 1)
  int conup[2];              // assembly tile shapes, j and k direction (autotuned; 0 = default)
  bool tuned;
  int nwall_pts;
  void* resid_scr;
  double* force_terms;
  int force_off[SMAC_MAX_BC];
  DevScalars* sc;
  DevScalars* hist;
  int hist_cap;
  std::vector<void*> allocs;
  cudaEvent_t ev0, ev1;
  float last_ms;
  int launches;
  // one iteration captured as a CUDA graph (replayed by smac_run)
  cudaGraphExec_t graph;
  bool graph_tried;
  // discrete adjoint (smac_adjoint.cu), created by the first adjoint call
  AdjointImpl* adj;
  AdjointOptions adj_opt;
  bool adj_opt_set;
  // a launch sequence that could not be issued as asked (e.g. an SA line longer than the
  // partitioned sweep supports); reported by the entry point that issued it
  int launch_err;
  // test of the bounded device waits: SMAC_TEST_STALL_WAIT set at creation makes the first line
  // of the first reference-order sweep of the next smac_step wait on a barrier that nothing
  // completes, so that the wait runs out and the step returns SMAC_ERR_TIMEOUT
  int stall_armed, stall_now;
  bool sa_pending;           // an iteration's SA model still to be forked (reference order: beside the j sweeps)
  // the throughput forms' SA line pivots: a warp per line (default) or, with
  // SMAC_SA_FACTOR_SEQUENTIAL set at creation, one thread per line (for comparisons)
  bool sa_factor_seq;
};

// device address of the iteration's wait status (DevScalars::wait_status)
static int* wait_status_ptr(smac_ctx* c) {
  return reinterpret_cast<int*>(reinterpret_cast<char*>(c->sc) + offsetof(DevScalars, wait_status));
}

// Report (and clear) a launch-sequence failure recorded while an iteration was issued.
static int take_launch_err(smac_ctx* c) {
  int rc = c->launch_err;
  if (rc) {
    c->launch_err = SMAC_OK;
    set_err("the SA line sweep does not support lines of this length (%dx%d)", c->jmax, c->kmax);
  }
  return rc;
}

static int autotune(smac_ctx* c);

extern "C" const char* smac_last_error(void) { return g_err; }

extern "C" void smac_params_default(smac_params* p) {
  memset(p, 0, sizeof *p);
  p->alpha = 10.0; p->beta = 5.0; p->dt = 1.0e12; p->dtau = 0.1; p->reynum = 1.5e6; p->underr = 0.01;
  p->pin = 1.5; p->pout = 1.0; p->cdis = 1.0; p->anut_inf = 0.0;
  p->impsch = 1; p->ivis = 1; p->iturb = 1;
  p->njsp = 2; p->nksp = 2; p->ntjsp = 2; p->ntksp = 0; p->nbcimp = 1;
  p->iflxo = 3; p->itrans = 0;
  p->wall_distance = SMAC_WALLDIST_REFERENCE; p->precision = SMAC_PREC_FP64; p->order = SMAC_ORDER_REFERENCE;
  p->line_solver = SMAC_LINES_PARTITIONED;
}

// bcmain.dat preprocessing, single zone (ref/rbc.f:347-398, 926-989, 1160-1345)
static int bc_prepare(const smac_bcspec* in, int jmax, int kmax, BCTable* bc) {
  memset(bc, 0, sizeof *bc);
  if (in->nbc < 1 || in->nbc > SMAC_MAX_BC) { set_err("BC table: %d rows", in->nbc); return SMAC_ERR_BC; }
  bc->nreg = in->nbc;
  for (int r = 0; r < in->nbc; ++r) {
    int v[4] = {in->jbcb[r], in->jbce[r], in->kbcb[r], in->kbce[r]};
    int mx[4] = {jmax, jmax, kmax, kmax};
    for (int i = 0; i < 4; ++i) {
      if (v[i] == -1) v[i] = mx[i];
      else if (v[i] == -2) v[i] = mx[i] - 1;
      if (v[i] < 1 || v[i] > mx[i]) { set_err("BC row %d: index out of range", r + 1); return SMAC_ERR_BC; }
    }
    if (in->nzbc[r] != 1) { set_err("BC row %d: zone %d (one subgrid only)", r + 1, in->nzbc[r]); return SMAC_ERR_BC; }
    BCRegion& R = bc->reg[r];
    R.ibcval = in->ibcval[r];
    R.jb = v[0] - 1; R.je = v[1] - 1; R.kb = v[2] - 1; R.ke = v[3] - 1;
    if (R.jb == R.je) R.jkbc = 1;
    else if (R.kb == R.ke) R.jkbc = 2;
    else { set_err("BC row %d is not a surface", r + 1); return SMAC_ERR_BC; }
    if (R.jb > R.je || R.kb > R.ke) { set_err("BC row %d: reversed range", r + 1); return SMAC_ERR_BC; }
    int ib = R.ibcval;
    if (ib != 0 && ib != 25 && ib != 31 && ib != 60) {
      set_err("BC row %d: ibcval %d is not one the reference dispatches", r + 1, ib);
      return SMAC_ERR_BC;
    }
    bool on_edge = R.jkbc == 1 ? (R.jb == 0 || R.jb == jmax - 1) : (R.kb == 0 || R.kb == kmax - 1);
    if ((ib == 25 || ib == 31) && !on_edge) { set_err("BC row %d must lie on the grid edge", r + 1); return SMAC_ERR_BC; }
    if (ib == 0) {
      if (R.jkbc != 2 || R.kb != 0) { set_err("BC row %d: walls must be k = 1 surfaces", r + 1); return SMAC_ERR_BC; }
      int w = bc->nwall++;
      bc->wjk[w] = R.jkbc; bc->wj1[w] = R.jb; bc->wj2[w] = R.je; bc->wk1[w] = R.kb; bc->wk2[w] = R.ke;
    }
  }
  int ws[SMAC_MAX_BC], nws = 0;
  for (int r = 0; r < bc->nreg; ++r)
    if (bc->reg[r].ibcval == 60) ws[nws++] = r;
  if (nws == 2) {
    const BCRegion& A = bc->reg[ws[0]];
    const BCRegion& B = bc->reg[ws[1]];
    if (A.jkbc != 2 || B.jkbc != 2 || A.kb != 0 || B.kb != 0 || (A.je - A.jb) != (B.je - B.jb)) {
      set_err("wake cut: two equal k = 1 surfaces expected");
      return SMAC_ERR_BC;
    }
    bc->jt_b[0] = A.jb; bc->jt_e[0] = A.je; bc->jb_b[0] = B.je;
    bc->jt_b[1] = B.jb; bc->jt_e[1] = B.je; bc->jb_b[1] = A.je;
    bc->nwake = 2;
  } else if (nws != 0) {
    set_err("wake cut: %d surfaces (0 or 2 supported)", nws);
    return SMAC_ERR_BC;
  }
  return SMAC_OK;
}

template <typename T>
static int dalloc(smac_ctx* c, T** p, size_t n) {
  void* v = nullptr;
  cudaError_t e = cudaMalloc(&v, n * sizeof(T) + 256);
  if (e != cudaSuccess) { set_err("cudaMalloc(%zu): %s", n * sizeof(T), cudaGetErrorString(e)); return SMAC_ERR_NOMEM; }
  // zeroed on the context's stream: its work runs on non-blocking streams, which would not wait
  // for a memset on the legacy default stream
  e = cudaMemsetAsync(v, 0, n * sizeof(T) + 256, c->st);
  if (e != cudaSuccess) { cudaFree(v); set_err("cudaMemsetAsync: %s", cudaGetErrorString(e)); return SMAC_ERR_CUDA; }
  c->allocs.push_back(v);
  *p = (T*)v;
  return SMAC_OK;
}

extern "C" int smac_ctx_destroy(smac_ctx* c) {
  if (!c) return SMAC_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->st_sa) cudaStreamSynchronize(c->st_sa);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  adjoint_free(c->adj);
  for (void* v : c->allocs) cudaFree(v);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->st) cudaStreamDestroy(c->st);
  if (c->st_sa) cudaStreamDestroy(c->st_sa);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->st_fk) cudaStreamSynchronize(c->st_fk);
  if (c->st_fk) cudaStreamDestroy(c->st_fk);
  if (c->ev_fk_fork) cudaEventDestroy(c->ev_fk_fork);
  if (c->ev_fk_join) cudaEventDestroy(c->ev_fk_join);
  delete c;
  return SMAC_OK;
}

static int validate(const smac_params* p, int jmax, int kmax) {
  if (jmax < 5 || kmax < 5 || jmax > 8100 || kmax > 8100) { set_err("grid %dx%d outside 5..8100", jmax, kmax); return SMAC_ERR_ARG; }
  if (p->impsch != 1 && p->impsch != 2) { set_err("impsch must be 1 or 2"); return SMAC_ERR_ARG; }
  if (p->iflxo != 3) { set_err("iflxo must be 3 (the only order the reference reaches)"); return SMAC_ERR_UNSUPPORTED; }
  if (p->itrans != 0) { set_err("itrans must be 0"); return SMAC_ERR_UNSUPPORTED; }
  if (p->nbcimp < 1 || p->njsp < 0 || p->nksp < 0 || p->ntjsp < 0 || p->ntksp < 0) { set_err("sweep counts"); return SMAC_ERR_ARG; }
  if (!(p->beta > 0) || !(p->dtau > 0) || !(p->reynum > 0) || !(p->dt > 0)) { set_err("beta, dtau, reynum, dt must be > 0"); return SMAC_ERR_ARG; }
  if (p->precision != SMAC_PREC_FP64 && p->precision != SMAC_PREC_MIXED) { set_err("precision mode %d unknown", p->precision); return SMAC_ERR_ARG; }
  if (p->order != SMAC_ORDER_REFERENCE && p->order != SMAC_ORDER_MULTICOLOR) { set_err("order mode %d unknown", p->order); return SMAC_ERR_ARG; }
  if (p->precision == SMAC_PREC_MIXED && p->impsch != 1) { set_err("the FP32 operator is implemented for line relaxation (impsch 1)"); return SMAC_ERR_UNSUPPORTED; }
  if (p->order == SMAC_ORDER_MULTICOLOR && p->impsch != 1) { set_err("the zebra order applies to line relaxation (impsch 1)"); return SMAC_ERR_UNSUPPORTED; }
  if (p->line_solver != SMAC_LINES_PARTITIONED && p->line_solver != SMAC_LINES_SEQUENTIAL) { set_err("line_solver %d unknown", p->line_solver); return SMAC_ERR_ARG; }
  return SMAC_OK;
}

extern "C" int smac_ctx_create(const smac_params* p, int jmax, int kmax, const double* x, const double* y,
                               const smac_bcspec* bcs, smac_ctx** out) {
  g_err[0] = 0;
  if (!p || !x || !y || !bcs || !out) { set_err("null argument"); return SMAC_ERR_ARG; }
  *out = nullptr;
  int rc = validate(p, jmax, kmax);
  if (rc) return rc;
  smac_ctx* c = new smac_ctx();
  memset(c->force_off, 0, sizeof c->force_off);
  c->p = *p;
  c->jmax = jmax; c->kmax = kmax; c->N = (size_t)jmax * kmax;
  rc = bc_prepare(bcs, jmax, kmax, &c->bc);
  if (rc) { delete c; return rc; }
  ilu_setup();
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) { set_err("no CUDA device"); delete c; return SMAC_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) { set_err("stream"); delete c; return SMAC_ERR_CUDA; }
  cudaEventCreate(&c->ev0);
  if (cudaStreamCreateWithFlags(&c->st_sa, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->st_fk, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fk_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fk_join, cudaEventDisableTiming) != cudaSuccess) {
    set_err("stream"); smac_ctx_destroy(c); return SMAC_ERR_CUDA;
  }
  cudaEventCreate(&c->ev1);
  const size_t N = c->N;
#define AL(ptr, n) do { if ((rc = dalloc(c, &c->ptr, (n)))) { smac_ctx_destroy(c); return rc; } } while (0)
  AL(x, N); AL(y, N); AL(rtxy, 6 * N); AL(dj, N); AL(q, 3 * N); AL(dq, 3 * N); AL(s, 3 * N);
  AL(anut, N); AL(vnut, N); AL(smin, N);
  AL(btc, 9 * N); AL(bjm, 9 * N); AL(bjp, 9 * N); AL(bkm, 9 * N); AL(bkp, 9 * N); AL(bjp_r, 9 * N);
  AL(scr9, 9 * N); AL(bprm, 9 * N);
  AL(sjm, N); AL(sjp, N); AL(skm, N); AL(skp, N); AL(stc, N); AL(sf, N); AL(ds, N);
  AL(sa_piv, N); AL(sa_cf, N);
  AL(vort, N); AL(crs, N); AL(cs11, N); AL(cs12, N); AL(fr1, N);
  AL(sc, 1); AL(d_bc, 1);
  c->throughput = p->order == SMAC_ORDER_MULTICOLOR || p->precision == SMAC_PREC_MIXED;
  memset(&c->f32, 0, sizeof c->f32);
  if (c->throughput) {
    AL(sa_work, N);
    if (p->precision == SMAC_PREC_MIXED) {
      float** fs[] = {&c->f32.btc_j, &c->f32.btc_k, &c->f32.bjm, &c->f32.bjp_f, &c->f32.bjp_o, &c->f32.bkm, &c->f32.bkp,
                      &c->f32.bkp_o};
      for (float** f : fs) if ((rc = dalloc(c, f, 9 * N))) { smac_ctx_destroy(c); return rc; }
      float** fv[] = {&c->f32.s, &c->f32.dq, &c->f32.work};
      for (float** f : fv) if ((rc = dalloc(c, f, 3 * N))) { smac_ctx_destroy(c); return rc; }
    } else {
      AL(zwork, 3 * N);
    }
  }
  if (p->impsch == 1 && p->line_solver == SMAC_LINES_PARTITIONED && !c->throughput) {
    size_t nops = line_ops_doubles(0, jmax, kmax);
    size_t nk = line_ops_doubles(1, jmax, kmax);
    // three lanes per segment up to 5,120-point lines; longer lines (the reference caps them at
    // 8,100) use one lane per segment (smac_lines.cu)
    c->rows = rows_supported(jmax) && rows_supported(kmax);
    if (c->rows) {
      size_t rj = line_ops_rows_doubles(jmax, kmax), rk = line_ops_rows_doubles(kmax, jmax);
      nops = rj > nops ? rj : nops;
      nk = rk > nk ? rk : nk;
    }
    AL(line_ops, nops > nk ? nops : nk);
    AL(kmaj, 51 * N);  // btc, bkm, bkp, bjm, bjp (9 planes each), s, dq (3 each)
    if (c->rows) {
      AL(line_ops_k, line_ops_rows_doubles(kmax, jmax));
      AL(kfac, 18 * N);
    }
  }
  c->hist_cap = 0;
  c->hist = nullptr;
  {
    void* v = nullptr;
    if ((rc = dalloc(c, (char**)&v, resid_scratch_bytes()))) { smac_ctx_destroy(c); return rc; }
    c->resid_scr = v;
  }
  // wall points for the wall distance and the force terms
  int nwp = 0;
  for (int w = 0; w < c->bc.nwall; ++w) {
    c->force_off[w] = nwp;
    nwp += c->bc.wj2[w] - c->bc.wj1[w] + 1;
  }
  c->nwall_pts = nwp;
  AL(wall_xy, 2 * (size_t)(nwp > 0 ? nwp : 1));
  AL(force_terms, kForceRec * ((size_t)(nwp > 0 ? nwp : 1) + 1));
#undef AL
  CK(cudaMemcpyAsync(c->x, x, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->y, y, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->d_bc, &c->bc, sizeof(BCTable), cudaMemcpyHostToDevice, c->st));
  {
    std::vector<double> wxy(2 * (size_t)(nwp > 0 ? nwp : 1));
    int i = 0;
    for (int w = 0; w < c->bc.nwall; ++w)
      for (int j = c->bc.wj1[w]; j <= c->bc.wj2[w]; ++j, ++i) {
        wxy[i] = x[ix(j, c->bc.wk1[w], jmax)];
        wxy[nwp + i] = y[ix(j, c->bc.wk1[w], jmax)];
      }
    CK(cudaMemcpyAsync(c->wall_xy, wxy.data(), wxy.size() * 8, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  // constants computed once on the host (same libm as a host reference build)
  c->vnu = 1.0 / p->reynum;
  c->pi = 4.0 * atan(1.0);
  c->ca = cos(p->alpha * c->pi / 180.);
  c->sa = sin(p->alpha * c->pi / 180.);
  c->rterm = 1. / p->dt;
  c->anutinf = p->anut_inf > 0 ? p->anut_inf : FLIT(0.001);
  c->cv1 = FLIT(7.1);
  // setup: metric, initial condition, wall distance and SA initial state
  launch_metric(c->x, c->y, c->rtxy, c->dj, jmax, kmax, c->st);
  launch_ic(c->q, jmax, kmax, c->ca, c->sa, c->d_bc, c->st);
  if (nwp > 0) launch_dfunsa(c->x, c->y, N, c->wall_xy, c->wall_xy + nwp, nwp, c->smin, c->st);
  else launch_fill(c->smin, FLIT(1.e6), N, c->st);
  launch_tsaic(c->anut, c->smin, jmax, kmax, c->d_bc, c->anutinf, c->st);
  CK(cudaMemsetAsync(c->sc, 0, sizeof(DevScalars), c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  if (!getenv("SMAC_NO_AUTOTUNE") && (rc = autotune(c)) != SMAC_OK) { smac_ctx_destroy(c); return rc; }
  c->stall_armed = getenv("SMAC_TEST_STALL_WAIT") != nullptr;
  c->sa_factor_seq = getenv("SMAC_SA_FACTOR_SEQUENTIAL") != nullptr;
  *out = c;
  return SMAC_OK;
}

// ------------------------------------------------------------------------------------------
static AssembleArgs assemble_args(smac_ctx* c) {
  AssembleArgs a;
  a.jmax = c->jmax; a.kmax = c->kmax; a.N = c->N;
  a.q = c->q; a.rtxy = c->rtxy; a.dj = c->dj; a.x = c->x; a.y = c->y;
  a.s = c->s; a.btc = c->btc; a.bjm = c->bjm; a.bjp = c->bjp; a.bkm = c->bkm; a.bkp = c->bkp;
  a.beta = c->p.beta; a.cdis = c->p.cdis; a.vnu = c->vnu; a.dtau = c->p.dtau; a.pout = c->p.pout;
  a.uinf = c->ca; a.vinf = c->sa; a.pi = c->pi; a.ivis = c->p.ivis; a.visc64 = c->p.visc_fp64 != 0;
  return a;
}

static SAArgs sa_args(smac_ctx* c) {
  SAArgs a;
  a.jmax = c->jmax; a.kmax = c->kmax; a.N = c->N;
  a.q = c->q; a.rtxy = c->rtxy; a.dj = c->dj; a.anut = c->anut; a.smin = c->smin;
  a.vort = c->vort; a.crs = c->crs; a.cs11 = c->cs11; a.cs12 = c->cs12; a.fr1 = c->fr1;
  a.sjm = c->sjm; a.sjp = c->sjp; a.skm = c->skm; a.skp = c->skp; a.stc = c->stc; a.sf = c->sf;
  // SA constants (ref/tursa.f:468-491), single-precision literals promoted
  a.vnu = c->vnu;
  a.akarman = FLIT(0.41); a.cb1 = FLIT(0.1355); a.cb2 = FLIT(0.622);
  a.sigma = 2.0 / 3.0;
  a.cw1 = a.cb1 / (a.akarman * a.akarman) + (1. + a.cb2) / a.sigma;
  a.cw2 = FLIT(0.3);
  double cw3 = 2.0;
  double t3 = (cw3 * cw3) * cw3;
  a.cw3r6 = t3 * t3;
  a.cv1 = FLIT(7.1); a.cv2 = 5.0;
  a.ct3tmp = 0.0;  // itrans = 0
  a.ct4 = 0.5; a.cr1 = 1; a.cr2 = 12; a.cr3 = 1;
  a.rterm = c->rterm;
  a.wall_fixed = c->p.wall_distance == SMAC_WALLDIST_FIXED;
  return a;
}

// SA model: tursa (ref/tursa.f:66-310); tsaic and dfunsa ran at context creation
static void sa_model(smac_ctx* c, cudaStream_t st) {
  SAArgs a = sa_args(c);
  launch_sa_assembly(a, c->d_bc, c->sc, st);
  const int exact = c->p.line_solver == SMAC_LINES_SEQUENTIAL;
  if (c->p.impsch == 1 && c->throughput) {
    // lreltur in zebra order: the lines of one colour at once, same sweep counts
    launch_fill(c->ds, 0.0, c->N, st);
    ScalarSweepArgs s;
    s.jmax = c->jmax; s.kmax = c->kmax; s.N = c->N;
    s.sjm = c->sjm; s.sjp = c->sjp; s.skm = c->skm; s.skp = c->skp; s.stc = c->stc; s.rhs = c->sf; s.ds = c->ds;
    int nsmax = c->p.ntjsp > c->p.ntksp ? c->p.ntjsp : c->p.ntksp;
    // scatri's pivots depend on the coefficients only: once per direction and iteration
    // (the two directions share the pivot scratch, so the k direction refactors when used)
    bool have[2] = {false, false};
    for (int njk = 1; njk <= nsmax; ++njk) {
      for (int dir = 0; dir < 2; ++dir) {
        if ((dir == 0 ? c->p.ntjsp : c->p.ntksp) < njk) continue;
        bool both = c->p.ntjsp > 0 && c->p.ntksp > 0;
        if (!have[dir] || both) {
          if (c->sa_factor_seq) launch_sa_factor(dir, s, c->sa_piv, c->sa_cf, st);
          else launch_sa_factor_warp(dir, s, c->sa_piv, c->sa_cf, st);
        }
        have[dir] = true;
        SAZebraArgs z;
        z.jmax = c->jmax; z.kmax = c->kmax; z.N = c->N;
        z.am = dir == 0 ? c->sjm : c->skm;
        z.om = dir == 0 ? c->skm : c->sjm;
        z.op = dir == 0 ? c->skp : c->sjp;
        z.rhs = c->sf; z.piv = c->sa_piv; z.cf = c->sa_cf; z.ds = c->ds; z.work = c->sa_work;
        int c0 = (njk & 1) ? 0 : 1;
        launch_sa_zebra(dir, z, c0, st);
        launch_sa_zebra(dir, z, 1 - c0, st);
        launch_bcimpds(c->d_bc, 1, c->jmax, c->N, c->anut, c->ds, c->sf, st);
      }
    }
  } else if (c->p.impsch == 1) {
    // lreltur (ref/lreltur.f:83-149)
    launch_fill(c->ds, 0.0, c->N, st);
    ScalarSweepArgs s;
    s.jmax = c->jmax; s.kmax = c->kmax; s.N = c->N;
    s.sjm = c->sjm; s.sjp = c->sjp; s.skm = c->skm; s.skp = c->skp; s.stc = c->stc; s.rhs = c->sf; s.ds = c->ds;
    int nsmax = c->p.ntjsp > c->p.ntksp ? c->p.ntjsp : c->p.ntksp;
    for (int njk = 1; njk <= nsmax; ++njk) {
      if (c->p.ntjsp >= njk) {
        if (exact) launch_sa_sweep(0, s, exact, st);
        else if (launch_sa_sweep_part(0, s, c->sa_piv, c->sa_cf, st)) c->launch_err = SMAC_ERR_UNSUPPORTED;
        launch_bcimpds(c->d_bc, 1, c->jmax, c->N, c->anut, c->ds, c->sf, st);
      }
      if (c->p.ntksp >= njk) {
        if (exact) launch_sa_sweep(1, s, exact, st);
        else if (launch_sa_sweep_part(1, s, c->sa_piv, c->sa_cf, st)) c->launch_err = SMAC_ERR_UNSUPPORTED;
        launch_bcimpds(c->d_bc, 1, c->jmax, c->N, c->anut, c->ds, c->sf, st);
      }
    }
  } else {
    // the scalar ILU keeps its diagonal in the SA pivot array, so that it can run beside the
    // mean-flow LU-SGS, which owns bprm
    launch_lusgs1(c->jmax, c->kmax, c->stc, c->sjm, c->sjp, c->skm, c->skp, c->sa_piv, c->sf, c->ds, st);
    launch_bcimpds(c->d_bc, 1, c->jmax, c->N, c->anut, c->ds, c->sf, st);
  }
  launch_sa_update(c->anut, c->ds, c->vnut, c->N, c->cv1, c->vnu, c->sc, st);
}

// lrelax (ref/lrelax.f:51-221) on the context's arrays.  restore_k: also undo the k
// factorisation (needed only when the caller reads the blocks back).
static void fork_sa(smac_ctx* c);

static void lrelax(smac_ctx* c, bool restore_k) {
  const int jmax = c->jmax, kmax = c->kmax;
  const int exact = c->p.line_solver == SMAC_LINES_SEQUENTIAL || c->line_ops == nullptr;
  launch_fill(c->dq, 0.0, 3 * c->N, c->st);
  SweepArgs a;
  a.jmax = jmax; a.kmax = kmax; a.N = c->N; a.s = c->s; a.dq = c->dq; a.underr = c->p.underr;
  const double* bjp_now = c->bjp;
  // In an iteration of the partitioned solve the k direction's factorisation and line operators
  // need only the assembled blocks: they are prepared on a forked stream, from copies of the
  // unfactored blocks, while the j lines are factored and swept (the stage API keeps the
  // reference's factor / undo / factor sequence, and so does stage timing).
  const size_t NN = c->N;
  double* tkm = c->kmaj;  // k-major operands: btc, bkm, bkp, bjm, bjp, s, dq
  const bool fork_k = !exact && c->rows && !restore_k && !g_timer && c->p.njsp > 0 && c->p.nksp > 0;
  if (fork_k) {
    double *kb = c->kfac, *kc = c->kfac + 9 * NN;
    cudaMemcpyAsync(kb, c->btc, 9 * NN * 8, cudaMemcpyDeviceToDevice, c->st);
    cudaMemcpyAsync(kc, c->bkp, 9 * NN * 8, cudaMemcpyDeviceToDevice, c->st);
    cudaMemcpyAsync(c->bjp_r, c->bjp, 9 * NN * 8, cudaMemcpyDeviceToDevice, c->st);  // for the k sweeps
    cudaEventRecord(c->ev_fk_fork, c->st);
    cudaStreamWaitEvent(c->st_fk, c->ev_fk_fork, 0);
    launch_btlu(1, c->bkm, kb, kc, jmax, kmax, c->st_fk, false);
    launch_transpose(kb, tkm, jmax, kmax, NN, 9, c->st_fk);
    launch_transpose(c->bkm, tkm + 9 * NN, jmax, kmax, NN, 9, c->st_fk);
    launch_transpose(kc, tkm + 18 * NN, jmax, kmax, NN, 9, c->st_fk);
    launch_line_prep_rows(kmax, jmax, kmax, NN, tkm, tkm + 9 * NN, tkm + 18 * NN, c->line_ops_k, c->st_fk);
    cudaEventRecord(c->ev_fk_join, c->st_fk);
  }
  mark(c->st, SMAC_STAGE_FACTOR_J);
  if (c->p.njsp > 0) {
    launch_btlu(0, c->bjm, c->btc, c->bjp, jmax, kmax, c->st, exact);
    if (!exact && c->rows) launch_line_prep_rows(jmax, kmax, jmax, c->N, c->btc, c->bjm, c->bjp, c->line_ops, c->st);
    else if (!exact) launch_line_prep(0, jmax, kmax, c->btc, c->bjm, c->bjp, c->line_ops, c->st);
    // the SA model beside the j sweeps, which leave most SMs idle (beside the j factorisation it
    // shares the sub-partitions of its FP64-issue-bound chains)
    if (c->sa_pending) {
      fork_sa(c);
      c->sa_pending = false;
    }
    mark(c->st, SMAC_STAGE_SWEEP_J);
    a.btc = c->btc; a.am = c->bjm; a.cp = c->bjp; a.om = c->bkm; a.op = c->bkp;
    for (int nj = 1; nj <= c->p.njsp; ++nj) {
      if (exact) launch_gs_sweep(0, nj, a, exact, c->st);
      else if (c->rows) {
        launch_gs_sweep_rows(nj, a, c->line_ops, wait_status_ptr(c), c->stall_now, c->st);
        c->stall_now = 0;
      }
      else launch_gs_sweep_part(0, nj, a, c->line_ops, c->st);
      if ((nj / c->p.nbcimp) * c->p.nbcimp == nj) launch_bcimpds(c->d_bc, 3, jmax, c->N, c->q, c->dq, c->s, c->st);
    }
    // undo: btc restored in place, bjp restored into bjp_r (the forked k preparation copied
    // the unfactored blocks instead)
    mark(c->st, SMAC_STAGE_UNDO_J);
    if (!fork_k) launch_btund(0, c->bjm, c->btc, c->bjp, c->bjp_r, jmax, kmax, c->st);
    bjp_now = c->bjp_r;
  }
  mark(c->st, SMAC_STAGE_FACTOR_K);
  if (c->p.nksp > 0) {
    if (!fork_k) launch_btlu(1, c->bkm, c->btc, c->bkp, jmax, kmax, c->st, exact);
    if (!exact && !c->rows) launch_line_prep(1, jmax, kmax, c->btc, c->bkm, c->bkp, c->line_ops, c->st);
    mark(c->st, SMAC_STAGE_SWEEP_K);
    a.btc = c->btc; a.am = c->bkm; a.cp = c->bkp; a.om = c->bjm; a.op = bjp_now;
    if (exact) {
      for (int nk = 1; nk <= c->p.nksp; ++nk) {
        launch_gs_sweep(1, nk, a, exact, c->st);
        if ((nk / c->p.nbcimp) * c->p.nbcimp == nk) launch_bcimpds(c->d_bc, 3, jmax, c->N, c->q, c->dq, c->s, c->st);
      }
    } else {
      // k-lines solved as contiguous lines of k-major copies: (j,k) at k + kmax*j
      const size_t N = c->N;
      double* t = c->kmaj;
      double *tb = t, *ta = t + 9 * N, *tc = t + 18 * N, *tom = t + 27 * N, *top = t + 36 * N;
      double *ts = t + 45 * N, *tdq = t + 48 * N;
      if (!fork_k) {
        launch_transpose(c->btc, tb, jmax, kmax, N, 9, c->st);
        launch_transpose(c->bkm, ta, jmax, kmax, N, 9, c->st);
        launch_transpose(c->bkp, tc, jmax, kmax, N, 9, c->st);
      }
      launch_transpose(c->bjm, tom, jmax, kmax, N, 9, c->st);
      launch_transpose(bjp_now, top, jmax, kmax, N, 9, c->st);
      launch_transpose(c->s, ts, jmax, kmax, N, 3, c->st);
      launch_transpose(c->dq, tdq, jmax, kmax, N, 3, c->st);
      SweepArgs at = a;
      at.jmax = kmax; at.kmax = jmax;
      at.btc = tb; at.am = ta; at.cp = tc; at.om = tom; at.op = top; at.s = ts; at.dq = tdq;
      const double* kops = fork_k ? c->line_ops_k : c->line_ops;
      if (fork_k) cudaStreamWaitEvent(c->st, c->ev_fk_join, 0);
      else if (c->rows) launch_line_prep_rows(kmax, jmax, kmax, N, tb, ta, tc, c->line_ops, c->st);
      for (int nk = 1; nk <= c->p.nksp; ++nk) {
        if (c->rows) launch_gs_sweep_rows(nk, at, kops, wait_status_ptr(c), c->stall_now, c->st);
        else launch_gs_sweep_part(0, nk, at, c->line_ops, c->st);
        if ((nk / c->p.nbcimp) * c->p.nbcimp == nk) launch_bcimpds(c->d_bc, 3, jmax, N, c->q, tdq, ts, c->st, kmax);
      }
      launch_transpose(tdq, c->dq, kmax, jmax, N, 3, c->st);
      launch_transpose(ts, c->s, kmax, jmax, N, 3, c->st);
    }
    if (restore_k) {
      launch_btund(1, c->bkm, c->btc, c->bkp, c->scr9, jmax, kmax, c->st);
      cudaMemcpyAsync(c->bkp, c->scr9, 9 * c->N * 8, cudaMemcpyDeviceToDevice, c->st);
    }
  }
  if (restore_k && bjp_now != c->bjp) cudaMemcpyAsync(c->bjp, c->bjp_r, 9 * c->N * 8, cudaMemcpyDeviceToDevice, c->st);
}

// Autotuner of the zebra line solves: lines per warp (1, 2 or 4; a line then has 32, 16 or 8
// lanes) per direction, picked by timing each choice on this grid with the operator the
// iteration uses.  The timed launches write scratch copies of dq and of the line work array,
// so the iteration's state is untouched.  Line solves do no data-dependent branching, so the
// contents of the operator do not change the timing.
template <typename W, typename S>
static int tune_dir(smac_ctx* c, int dir, ZebraArgs<W, S> z, cudaEvent_t e0, cudaEvent_t e1) {
  const int cand[5] = {1, 2, 4, -2, -4};  // lines per warp; negative: warps per line
  float best = 1e30f;
  int pick = 1;
  for (int lpw : cand) {
    launch_zebra(dir, z, 0, c->st, lpw);
    cudaEventRecord(e0, c->st);
    for (int r = 0; r < 3; ++r) {
      launch_zebra(dir, z, 0, c->st, lpw);
      launch_zebra(dir, z, 1, c->st, lpw);
    }
    cudaEventRecord(e1, c->st);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < 0.97f * best) { best = ms; pick = lpw; }
  }
  return pick;
}

// Autotuner of the assembly (conup) tiles: per direction, the tile shape (lines x points per
// CTA, threads) that assembles this grid fastest.  Every shape computes each point the same
// way, so the choice changes no result.  The timed launches write the operator and residual
// arrays, which every assembly rewrites before they are read.
static void tune_conup(smac_ctx* c, cudaEvent_t e0, cudaEvent_t e1) {
  c->conup[0] = c->conup[1] = 0;
  if (const char* f = getenv("SMAC_CONUP_SHAPE")) {  // fixed shapes "j,k" (tests)
    int sj = 0, sk = 0;
    if (sscanf(f, "%d,%d", &sj, &sk) == 2) {
      c->conup[0] = sj >= 0 && sj < kConupNumShapes ? sj : 0;
      c->conup[1] = sk >= 0 && sk < kConupNumShapes ? sk : 0;
    }
    return;
  }
  const AssembleArgs a = assemble_args(c);
  for (int dir = 0; dir < 2; ++dir) {
    float best = 1e30f;
    for (int shape = 0; shape < kConupNumShapes; ++shape) {
      launch_conup_dir(a, dir, shape, c->st);
      cudaEventRecord(e0, c->st);
      for (int r = 0; r < 3; ++r) launch_conup_dir(a, dir, shape, c->st);
      cudaEventRecord(e1, c->st);
      if (cudaEventSynchronize(e1) != cudaSuccess) return;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < 0.97f * best) { best = ms; c->conup[dir] = shape; }
    }
  }
}

static int autotune(smac_ctx* c) {
  if (c->tuned) return SMAC_OK;
  c->tuned = true;
  c->zlpw[0] = c->zlpw[1] = 1;
  {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    tune_conup(c, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (cudaGetLastError() != cudaSuccess) return SMAC_ERR_CUDA;
  }
  if (!c->throughput || c->p.impsch != 1) return SMAC_OK;
  // fixed shapes instead of timing ("j,k", e.g. "-4,1"): for tests that compare the shapes
  if (const char* f = getenv("SMAC_ZEBRA_SHAPE")) {
    int sj = 1, sk = 1;
    if (sscanf(f, "%d,%d", &sj, &sk) == 2) {
      auto ok = [](int v) { return v == 1 || v == 2 || v == 4 || v == -2 || v == -4; };
      c->zlpw[0] = ok(sj) ? sj : 1;
      c->zlpw[1] = ok(sk) ? sk : 1;
      return SMAC_OK;
    }
  }
  const size_t N = c->N;
  const bool f32 = c->p.precision == SMAC_PREC_MIXED;
  const size_t wb = f32 ? sizeof(float) : sizeof(double);
  void *dq = nullptr, *work = nullptr;
  if (cudaMalloc(&dq, 3 * N * wb) != cudaSuccess || cudaMalloc(&work, 3 * N * wb) != cudaSuccess) {
    cudaFree(dq);
    cudaGetLastError();
    return SMAC_OK;  // keep one line per warp
  }
  cudaMemsetAsync(dq, 0, 3 * N * wb, c->st);
  cudaMemsetAsync(work, 0, 3 * N * wb, c->st);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (f32) {
    F32Ops& o = c->f32;
    ZebraArgs<float, float> z;
    z.jmax = c->jmax; z.kmax = c->kmax; z.N = N; z.s = o.s; z.dq = (float*)dq; z.work = (float*)work;
    z.underr = (float)c->p.underr;
    z.btc = o.btc_j; z.am = o.bjm; z.cp = o.bjp_f; z.om = o.bkm; z.op = o.bkp_o;
    c->zlpw[0] = tune_dir(c, 0, z, e0, e1);
    z.btc = o.btc_k; z.am = o.bkm; z.cp = o.bkp; z.om = o.bjm; z.op = o.bjp_o;
    c->zlpw[1] = tune_dir(c, 1, z, e0, e1);
  } else {
    ZebraArgs<double, double> z;
    z.jmax = c->jmax; z.kmax = c->kmax; z.N = N; z.s = c->s; z.dq = (double*)dq; z.work = (double*)work;
    z.underr = c->p.underr;
    z.btc = c->btc; z.am = c->bjm; z.cp = c->bjp; z.om = c->bkm; z.op = c->bkp;
    c->zlpw[0] = tune_dir(c, 0, z, e0, e1);
    z.btc = c->btc; z.am = c->bkm; z.cp = c->bkp; z.om = c->bjm; z.op = c->bjp;
    c->zlpw[1] = tune_dir(c, 1, z, e0, e1);
  }
  cudaStreamSynchronize(c->st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dq);
  cudaFree(work);
  return cudaGetLastError() == cudaSuccess ? SMAC_OK : SMAC_ERR_CUDA;
}

extern "C" int smac_autotune(smac_ctx* c, int* lines_per_warp) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  int rc = autotune(c);
  if (lines_per_warp) {
    lines_per_warp[0] = c->zlpw[0] ? c->zlpw[0] : 1;
    lines_per_warp[1] = c->zlpw[1] ? c->zlpw[1] : 1;
  }
  return rc;
}

extern "C" int smac_assembly_tiles(smac_ctx* c, int* tiles) {
  if (!c || !tiles) { set_err("null argument"); return SMAC_ERR_ARG; }
  tiles[0] = c->conup[0];
  tiles[1] = c->conup[1];
  return SMAC_OK;
}

// lrelax in zebra order (FP64) or with the FP32 operator (mixed precision)
static void lrelax_zebra(smac_ctx* c) {
  const int jmax = c->jmax, kmax = c->kmax;
  const size_t N = c->N;
  if (c->p.precision == SMAC_PREC_MIXED) {
    F32Ops& o = c->f32;
    launch_to_f32(c->btc, c->bjm, c->bjp, c->bkm, c->bkp, c->s, o, N, c->st);
    launch_fill_f32(o.dq, 0.f, 3 * N, c->st);
    // the k-line factorisation does not depend on the j sweeps (they read the unfactored copy
    // bkp_o): it runs on its own stream beside them, except under stage timing
    const bool fork_k = c->p.nksp > 0 && !g_timer;
    if (fork_k) {
      cudaEventRecord(c->ev_fk_fork, c->st);
      cudaStreamWaitEvent(c->st_fk, c->ev_fk_fork, 0);
      launch_btlu_f32(1, o.bkm, o.btc_k, o.bkp, jmax, kmax, c->st_fk);
      cudaEventRecord(c->ev_fk_join, c->st_fk);
    }
    mark(c->st, SMAC_STAGE_FACTOR_J);
    ZebraArgs<float, float> z;
    z.jmax = jmax; z.kmax = kmax; z.N = N; z.s = o.s; z.dq = o.dq; z.work = o.work; z.underr = (float)c->p.underr;
    if (c->p.njsp > 0) {
      launch_btlu_f32(0, o.bjm, o.btc_j, o.bjp_f, jmax, kmax, c->st);
      mark(c->st, SMAC_STAGE_SWEEP_J);
      z.btc = o.btc_j; z.am = o.bjm; z.cp = o.bjp_f; z.om = o.bkm; z.op = o.bkp_o;
      for (int nj = 1; nj <= c->p.njsp; ++nj) {
        int c0 = (nj & 1) ? 0 : 1;
        launch_zebra(0, z, c0, c->st, c->zlpw[0]);
        launch_zebra(0, z, 1 - c0, c->st, c->zlpw[0]);
        if ((nj / c->p.nbcimp) * c->p.nbcimp == nj) launch_bcimpds_f32(c->d_bc, jmax, N, c->q, o.dq, o.s, c->st);
      }
    }
    mark(c->st, SMAC_STAGE_FACTOR_K);
    if (c->p.nksp > 0) {
      if (fork_k) cudaStreamWaitEvent(c->st, c->ev_fk_join, 0);
      else launch_btlu_f32(1, o.bkm, o.btc_k, o.bkp, jmax, kmax, c->st);
      mark(c->st, SMAC_STAGE_SWEEP_K);
      z.btc = o.btc_k; z.am = o.bkm; z.cp = o.bkp; z.om = o.bjm; z.op = o.bjp_o;
      for (int nk = 1; nk <= c->p.nksp; ++nk) {
        int c0 = (nk & 1) ? 0 : 1;
        launch_zebra(1, z, c0, c->st, c->zlpw[1]);
        launch_zebra(1, z, 1 - c0, c->st, c->zlpw[1]);
        if ((nk / c->p.nbcimp) * c->p.nbcimp == nk) launch_bcimpds_f32(c->d_bc, jmax, N, c->q, o.dq, o.s, c->st);
      }
    }
    launch_dq_to_f64(o.dq, c->dq, 3 * N, c->st);
    return;
  }
  launch_fill(c->dq, 0.0, 3 * N, c->st);
  ZebraArgs<double, double> z;
  z.jmax = jmax; z.kmax = kmax; z.N = N; z.s = c->s; z.dq = c->dq; z.work = c->zwork; z.underr = c->p.underr;
  const double* bjp_now = c->bjp;
  mark(c->st, SMAC_STAGE_FACTOR_J);
  if (c->p.njsp > 0) {
    launch_btlu(0, c->bjm, c->btc, c->bjp, jmax, kmax, c->st, false);
    mark(c->st, SMAC_STAGE_SWEEP_J);
    z.btc = c->btc; z.am = c->bjm; z.cp = c->bjp; z.om = c->bkm; z.op = c->bkp;
    for (int nj = 1; nj <= c->p.njsp; ++nj) {
      int c0 = (nj & 1) ? 0 : 1;
      launch_zebra(0, z, c0, c->st, c->zlpw[0]);
      launch_zebra(0, z, 1 - c0, c->st, c->zlpw[0]);
      if ((nj / c->p.nbcimp) * c->p.nbcimp == nj) launch_bcimpds(c->d_bc, 3, jmax, N, c->q, c->dq, c->s, c->st);
    }
    mark(c->st, SMAC_STAGE_UNDO_J);
    launch_btund(0, c->bjm, c->btc, c->bjp, c->bjp_r, jmax, kmax, c->st);
    bjp_now = c->bjp_r;
  }
  mark(c->st, SMAC_STAGE_FACTOR_K);
  if (c->p.nksp > 0) {
    launch_btlu(1, c->bkm, c->btc, c->bkp, jmax, kmax, c->st, false);
    mark(c->st, SMAC_STAGE_SWEEP_K);
    z.btc = c->btc; z.am = c->bkm; z.cp = c->bkp; z.om = c->bjm; z.op = bjp_now;
    for (int nk = 1; nk <= c->p.nksp; ++nk) {
      int c0 = (nk & 1) ? 0 : 1;
      launch_zebra(1, z, c0, c->st, c->zlpw[1]);
      launch_zebra(1, z, 1 - c0, c->st, c->zlpw[1]);
      if ((nk / c->p.nbcimp) * c->p.nbcimp == nk) launch_bcimpds(c->d_bc, 3, jmax, N, c->q, c->dq, c->s, c->st);
    }
  }
}

// The SA model (tursa) reads q and writes only its own arrays and sc->turres: it does not feed
// the mean flow (viscterms uses the laminar viscosity), so it can run beside the mean-flow
// assembly and line solves and must only finish before the update writes q.  concurrent_sa
// forks it onto the second stream; stage timing and the stage API keep it in line.
static bool sa_forks(smac_ctx* c, bool concurrent_sa) {
  return concurrent_sa && c->p.ivis == 1 && c->p.iturb == 1 && !g_timer;
}

static void fork_sa(smac_ctx* c) {
  cudaEventRecord(c->ev_fork, c->st);
  cudaStreamWaitEvent(c->st_sa, c->ev_fork, 0);
  sa_model(c, c->st_sa);
  cudaEventRecord(c->ev_join, c->st_sa);
}

// The forked SA model runs where it takes no FP64 issue slots from the mean flow's critical
// path.  In the reference-order form with line relaxation it starts with the j-line sweeps
// (lrelax), which hold 16 SMs and leave the others idle; started with the iteration it shared
// sub-partitions with the j factorisation, whose chains are bound by FP64 issue (1.4 ms per
// iteration at 1921x481).  With LU-SGS it starts with the iteration.  In the throughput forms
// it starts after the mean-flow assembly: both assemblies are FP64-bound, while the FP32
// factorisation and zebra sweeps that follow leave most SMs' FP64 units idle.
static void assemble(smac_ctx* c, bool concurrent_sa = false) {
  mark(c->st, SMAC_STAGE_SA);
  launch_iter_begin(c->sc, c->st);
  const bool fork = sa_forks(c, concurrent_sa);
  c->sa_pending = fork && !c->throughput && c->p.impsch == 1;
  if (fork && !c->throughput && !c->sa_pending) fork_sa(c);
  else if (!fork && c->p.ivis == 1 && c->p.iturb == 1) sa_model(c, c->st);
  mark(c->st, SMAC_STAGE_ASSEMBLE);
  AssembleArgs a = assemble_args(c);
  launch_conup(a, c->st, c->conup[0], c->conup[1]);
  launch_bc(a, c->d_bc, c->sc, c->st);
  mark(c->st, SMAC_STAGE_RESID);
  launch_resid(c->s, c->dj, c->jmax, c->N, c->resid_scr, c->p.beta, c->sc, c->st);
  if (fork && c->throughput) fork_sa(c);
}

static void forces(smac_ctx* c) {
  ForceArgs f;
  f.jmax = c->jmax; f.N = c->N; f.q = c->q; f.rtxy = c->rtxy; f.dj = c->dj; f.x = c->x; f.y = c->y;
  f.vnu = c->vnu; f.ca = c->ca; f.sa = c->sa; f.ivis = c->p.ivis;
  memcpy(f.term_off, c->force_off, sizeof f.term_off);
  if (c->throughput) launch_forces_parallel(f, c->d_bc, c->bc, c->force_terms, c->sc, c->st);
  else launch_forces(f, c->d_bc, c->bc, c->force_terms, c->sc, c->st);
}

static void iteration(smac_ctx* c) {
  const bool fork = sa_forks(c, true);
  assemble(c, true);
  if (c->p.impsch == 1 && c->throughput) lrelax_zebra(c);
  else if (c->p.impsch == 1) lrelax(c, false);
  else {
    mark(c->st, SMAC_STAGE_FACTOR_J);
    launch_lusgs3(c->jmax, c->kmax, c->btc, c->bjm, c->bjp, c->bkm, c->bkp, c->bprm, c->s, c->dq, c->st);
    launch_bcimpds(c->d_bc, 3, c->jmax, c->N, c->q, c->dq, c->s, c->st);
  }
  if (c->sa_pending) {  // not started by the line sweeps
    fork_sa(c);
    c->sa_pending = false;
  }
  mark(c->st, SMAC_STAGE_UPDATE);
  if (fork) cudaStreamWaitEvent(c->st, c->ev_join, 0);
  launch_update(c->q, c->dq, c->N, c->st);
  forces(c);
  mark(c->st, SMAC_NSTAGES);
}

static void fill_out(const DevScalars& d, smac_iter_out* o) {
  o->nt = d.nt; o->jres = d.jres; o->kres = d.kres; o->neq_res = d.neq;
  o->resmax = d.resmax; o->resmax0 = d.resmax0;
  double r0 = d.resmax0 == 0.0 ? 1.0 : d.resmax0;
  o->rmax = d.resmax / r0;
  o->divmax = d.divmax; o->turres = d.turres; o->rhsnorm = d.rhsnorm;
  o->cd = d.cd; o->cl = d.cl; o->cm = d.cm; o->cdp = d.cdp; o->clp = d.clp;
}

__global__ void k_record(const DevScalars* sc, DevScalars* hist, int slot) { hist[slot] = *sc; }

extern "C" int smac_step(smac_ctx* c, smac_iter_out* out) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  c->stall_now = c->stall_armed;
  c->stall_armed = 0;
  iteration(c);
  c->stall_now = 0;
  DevScalars d;
  CK(cudaMemcpyAsync(&d, c->sc, sizeof d, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  if (int rc = take_launch_err(c)) return rc;
  if (out) fill_out(d, out);
  if (d.wait_status) { set_err("a device wait ran out of time at iteration %d", d.nt); return d.wait_status; }
  if (d.status) { set_err("non-finite residual at iteration %d", d.nt); return d.status; }
  return SMAC_OK;
}

extern "C" int smac_assemble(smac_ctx* c, smac_iter_out* out) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  assemble(c);
  DevScalars d;
  CK(cudaMemcpyAsync(&d, c->sc, sizeof d, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  if (int rc = take_launch_err(c)) return rc;
  if (out) { memset(out, 0, sizeof *out); fill_out(d, out); }
  return d.status;
}

// Capture one iteration (the launch sequence never depends on host state once the context
// exists: scalars such as nt and clift live on the device).  Returns false if capture is not
// possible, in which case the iteration is launched directly.
static bool ensure_graph(smac_ctx* c) {
  if (c->graph) return true;
  if (c->graph_tried) return false;
  c->graph_tried = true;
  if (getenv("SMAC_NO_GRAPH")) return false;
  cudaGraph_t g;
  if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); return false; }
  iteration(c);
  if (cudaStreamEndCapture(c->st, &g) != cudaSuccess) { cudaGetLastError(); return false; }
  cudaGraphExec_t ge;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  c->graph = ge;
  return true;
}

extern "C" int smac_run(smac_ctx* c, int n, smac_iter_out* hist) {
  if (!c || n < 0) { set_err("bad arguments"); return SMAC_ERR_ARG; }
  if (n == 0) return SMAC_OK;
  if (n > c->hist_cap) {
    if (c->hist) {
      for (auto it = c->allocs.begin(); it != c->allocs.end(); ++it)
        if (*it == (void*)c->hist) { c->allocs.erase(it); break; }
      cudaFree(c->hist);
    }
    int rc = dalloc(c, &c->hist, (size_t)n);
    if (rc) return rc;
    c->hist_cap = n;
  }
  const bool use_graph = ensure_graph(c);
  if (int rc = take_launch_err(c)) return rc;
  CK(cudaEventRecord(c->ev0, c->st));
  for (int i = 0; i < n; ++i) {
    if (use_graph) CK(cudaGraphLaunch(c->graph, c->st));
    else iteration(c);
    ++g_kernel_launches;
    k_record<<<1, 1, 0, c->st>>>(c->sc, c->hist, i);
  }
  CK(cudaEventRecord(c->ev1, c->st));
  if (int rc = take_launch_err(c)) { cudaStreamSynchronize(c->st); return rc; }
  std::vector<DevScalars> h(n);
  CK(cudaMemcpyAsync(h.data(), c->hist, sizeof(DevScalars) * n, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
  for (int i = 0; i < n; ++i) {
    if (hist) fill_out(h[i], hist + i);
    if (h[i].wait_status) { set_err("a device wait ran out of time at iteration %d", h[i].nt); return h[i].wait_status; }
    if (h[i].status) { set_err("non-finite residual at iteration %d", h[i].nt); return h[i].status; }
  }
  return SMAC_OK;
}

extern "C" double smac_last_run_ms(smac_ctx* c) { return c ? (double)c->last_ms : 0.0; }

// ------------------------------------------------------------------------------------- batches
// Many independent cases (own grid, airfoil and flow), one CUDA graph per pseudo-time
// iteration of all of them: every case's launch sequence is captured on its own stream, forked
// from and joined to the batch's stream, so the graph holds one branch per case and one launch
// runs all of them concurrently; small grids that leave most SMs idle on their own fill the GPU
// together.  Each case keeps its own autotuned line solver.  The history of each case is
// appended on the device by a counter, so the graph needs no per-iteration argument.
struct smac_batch {
  std::vector<smac_ctx*> cases;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_fork = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> ev_done;
  cudaGraphExec_t graph = nullptr;
  DevScalars* hist = nullptr;  // [case][cap]
  int* count = nullptr;        // [case]
  int cap = 0;
  float last_ms = 0.f;
  // packed line solves (SMAC_BATCH_PACKED_LINES)
  bool packed = false;
  int wpl = 2;
  ZebraArgs<float, float>* d_zargs = nullptr;  // [2][case]: j lines, then k lines
  int* d_start = nullptr;                      // [4][case + 1]: (direction, colour) CTA prefixes
  BcimpArgs* d_bcim = nullptr;                 // [case]
  int nblocks[4] = {0, 0, 0, 0};
  int max_jmax = 0;
  std::vector<cudaEvent_t> ev_pre;             // [case]: work before the line sweeps done
  cudaEvent_t ev_sweeps = nullptr;
  // line work queue (SMAC_BATCH_QUEUE_LINES)
  bool queue = false;
  QPhase* d_phases = nullptr;
  int* d_qint = nullptr;                       // status, stall, head, done[nphases]
  int nphases = 0, nitems = 0, qblocks = 0;
  bool stall_armed = false;                    // SMAC_TEST_STALL_WAIT at creation
};

__global__ void k_record_next(const DevScalars* sc, DevScalars* hist, int* count, int cap) {
  int slot = *count;
  if (slot < cap) hist[slot] = *sc;
  *count = slot + 1;
}

static int batch_alloc(smac_batch* b, int cap) {
  if (cap <= b->cap) return SMAC_OK;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  cudaFree(b->hist);
  b->hist = nullptr;
  if (cudaMalloc(&b->hist, sizeof(DevScalars) * (size_t)cap * b->cases.size()) != cudaSuccess) {
    cudaGetLastError();
    b->cap = 0;
    set_err("batch history of %d iterations x %zu cases", cap, b->cases.size());
    return SMAC_ERR_NOMEM;
  }
  b->cap = cap;
  return SMAC_OK;
}

// An FP32-operator zebra iteration around its line sweeps (the packed batch runs the sweeps of
// all cases together): the same launches, in the same order, as iteration() and lrelax_zebra().
static void iteration_pre_sweeps(smac_ctx* c) {
  assemble(c, true);
  const int jmax = c->jmax, kmax = c->kmax;
  const size_t N = c->N;
  F32Ops& o = c->f32;
  launch_to_f32(c->btc, c->bjm, c->bjp, c->bkm, c->bkp, c->s, o, N, c->st);
  launch_fill_f32(o.dq, 0.f, 3 * N, c->st);
  cudaEventRecord(c->ev_fk_fork, c->st);
  cudaStreamWaitEvent(c->st_fk, c->ev_fk_fork, 0);
  launch_btlu_f32(1, o.bkm, o.btc_k, o.bkp, jmax, kmax, c->st_fk);
  cudaEventRecord(c->ev_fk_join, c->st_fk);
  launch_btlu_f32(0, o.bjm, o.btc_j, o.bjp_f, jmax, kmax, c->st);
}

static void iteration_post_sweeps(smac_ctx* c) {
  launch_dq_to_f64(c->f32.dq, c->dq, 3 * c->N, c->st);
  if (sa_forks(c, true)) cudaStreamWaitEvent(c->st, c->ev_join, 0);
  launch_update(c->q, c->dq, c->N, c->st);
  forces(c);
}

static bool packable(const smac_batch* b, const char** why) {
  const smac_ctx* c0 = b->cases[0];
  for (const smac_ctx* c : b->cases) {
    if (!c->throughput || c->p.precision != SMAC_PREC_MIXED || c->p.impsch != 1) {
      *why = "every case must be the FP32-operator zebra form with line relaxation";
      return false;
    }
    if (c->p.njsp != c0->p.njsp || c->p.nksp != c0->p.nksp || c->p.nbcimp != c0->p.nbcimp || c->p.njsp < 1 ||
        c->p.nksp < 1) {
      *why = "every case needs the same (non-zero) sweep counts";
      return false;
    }
  }
  return true;
}

// device tables of the packed line solves
static int batch_pack_tables(smac_batch* b) {
  const int nc = (int)b->cases.size();
  std::vector<ZebraArgs<float, float>> za(2 * (size_t)nc);
  std::vector<int> start(4 * (size_t)(nc + 1), 0);
  std::vector<BcimpArgs> bi(nc);
  b->max_jmax = 0;
  for (int i = 0; i < nc; ++i) {
    smac_ctx* c = b->cases[i];
    F32Ops& o = c->f32;
    for (int d = 0; d < 2; ++d) {
      ZebraArgs<float, float>& z = za[(size_t)d * nc + i];
      z.jmax = c->jmax; z.kmax = c->kmax; z.N = c->N; z.s = o.s; z.dq = o.dq; z.work = o.work;
      z.underr = (float)c->p.underr;
      if (d == 0) { z.btc = o.btc_j; z.am = o.bjm; z.cp = o.bjp_f; z.om = o.bkm; z.op = o.bkp_o; }
      else { z.btc = o.btc_k; z.am = o.bkm; z.cp = o.bkp; z.om = o.bjm; z.op = o.bjp_o; }
      const int nl = d == 0 ? c->kmax : c->jmax;
      for (int col = 0; col < 2; ++col) {
        int* st = &start[(size_t)(2 * d + col) * (nc + 1)];
        st[i + 1] = st[i] + (nl - col + 1) / 2;
      }
    }
    bi[i].bc = c->d_bc; bi[i].jmax = c->jmax; bi[i].N = c->N; bi[i].q = c->q; bi[i].dq = o.dq; bi[i].rhs = o.s;
    if (c->jmax > b->max_jmax) b->max_jmax = c->jmax;
  }
  for (int k = 0; k < 4; ++k) b->nblocks[k] = start[(size_t)k * (nc + 1) + nc];
  if (!b->d_zargs) {
    CK(cudaMalloc(&b->d_zargs, sizeof(ZebraArgs<float, float>) * za.size()));
    CK(cudaMalloc(&b->d_start, sizeof(int) * start.size()));
    CK(cudaMalloc(&b->d_bcim, sizeof(BcimpArgs) * bi.size()));
  }
  // on the batch's stream (non-blocking: a copy on the legacy stream would not be ordered before
  // its launches); the host vectors are staged before each call returns
  CK(cudaMemcpyAsync(b->d_zargs, za.data(), sizeof(ZebraArgs<float, float>) * za.size(), cudaMemcpyHostToDevice, b->st));
  CK(cudaMemcpyAsync(b->d_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, b->st));
  CK(cudaMemcpyAsync(b->d_bcim, bi.data(), sizeof(BcimpArgs) * bi.size(), cudaMemcpyHostToDevice, b->st));
  CK(cudaStreamSynchronize(b->st));
  return SMAC_OK;
}

// one graph per iteration of all cases with the line solves packed: every case's work before
// its sweeps (a branch per case), one launch per sweep colour for the lines of all cases with
// the wake-cut injections of all cases after each sweep, then every case's work after its sweeps
static int batch_capture_packed(smac_batch* b) {
  int rc = batch_pack_tables(b);
  if (rc) return rc;
  const int nc = (int)b->cases.size();
  const smac_ctx* c0 = b->cases[0];
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(b->ev_fork, b->st);
  for (int i = 0; i < nc; ++i) {
    smac_ctx* c = b->cases[i];
    cudaStreamWaitEvent(c->st, b->ev_fork, 0);
    iteration_pre_sweeps(c);
    cudaEventRecord(b->ev_pre[i], c->st);
    cudaStreamWaitEvent(b->st, b->ev_pre[i], 0);
  }
  const int* st0 = b->d_start;
  for (int nj = 1; nj <= c0->p.njsp; ++nj) {
    const int col = (nj & 1) ? 0 : 1;
    launch_zebra_packed(0, b->d_zargs, st0 + (size_t)col * (nc + 1), nc, b->nblocks[col], col, b->wpl, b->st);
    launch_zebra_packed(0, b->d_zargs, st0 + (size_t)(1 - col) * (nc + 1), nc, b->nblocks[1 - col], 1 - col, b->wpl,
                        b->st);
    if ((nj / c0->p.nbcimp) * c0->p.nbcimp == nj) launch_bcimpds_f32_packed(b->d_bcim, nc, b->max_jmax, b->st);
  }
  for (int i = 0; i < nc; ++i) cudaStreamWaitEvent(b->st, b->cases[i]->ev_fk_join, 0);
  for (int nk = 1; nk <= c0->p.nksp; ++nk) {
    const int col = (nk & 1) ? 0 : 1;
    launch_zebra_packed(1, b->d_zargs + nc, st0 + (size_t)(2 + col) * (nc + 1), nc, b->nblocks[2 + col], col, b->wpl,
                        b->st);
    launch_zebra_packed(1, b->d_zargs + nc, st0 + (size_t)(3 - col) * (nc + 1), nc, b->nblocks[3 - col], 1 - col,
                        b->wpl, b->st);
    if ((nk / c0->p.nbcimp) * c0->p.nbcimp == nk) launch_bcimpds_f32_packed(b->d_bcim, nc, b->max_jmax, b->st);
  }
  cudaEventRecord(b->ev_sweeps, b->st);
  for (int i = 0; i < nc; ++i) {
    smac_ctx* c = b->cases[i];
    cudaStreamWaitEvent(c->st, b->ev_sweeps, 0);
    iteration_post_sweeps(c);
    ++g_kernel_launches;
    k_record_next<<<1, 1, 0, c->st>>>(c->sc, b->hist + (size_t)i * b->cap, b->count + i, b->cap);
    cudaEventRecord(b->ev_done[i], c->st);
    cudaStreamWaitEvent(b->st, b->ev_done[i], 0);
  }
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  if (e != cudaSuccess) { set_err("batch capture: %s", cudaGetErrorString(e)); cudaGetLastError(); return SMAC_ERR_CUDA; }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { set_err("batch graph: %s", cudaGetErrorString(e)); cudaGetLastError(); return SMAC_ERR_CUDA; }
  return SMAC_OK;
}

// the phases of the line sweep queue: every sweep colour and wake-cut injection in the order of
// one iteration, each phase of every case before the next; within a phase the cases come
// largest first (their lines are the longest)
static int batch_queue_tables(smac_batch* b) {
  int rc = batch_pack_tables(b);
  if (rc) return rc;
  const int nc = (int)b->cases.size();
  const smac_ctx* c0 = b->cases[0];
  std::vector<int> order(nc);
  for (int i = 0; i < nc; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->cases[x]->N > b->cases[y]->N; });
  std::vector<QPhase> ph;
  int nitems = 0;
  auto add = [&](int type, int cas, int dir, int color, int n, int dep) {
    QPhase p;
    p.type = type; p.cas = cas; p.dir = dir; p.color = color; p.first = nitems; p.nitems = n; p.dep = dep;
    ph.push_back(p);
    nitems += n;
    return (int)ph.size() - 1;
  };
  std::vector<int> last(nc, -1);
  for (int nj = 1; nj <= c0->p.njsp; ++nj) {
    const int col = (nj & 1) ? 0 : 1;
    for (int cc : {col, 1 - col})
      for (int i : order) last[i] = add(kQSweep, i, 0, cc, (b->cases[i]->kmax - cc + 1) / 2, last[i]);
    if ((nj / c0->p.nbcimp) * c0->p.nbcimp == nj)
      for (int i : order) last[i] = add(kQBcimp, i, 0, 0, 1, last[i]);
  }
  for (int nk = 1; nk <= c0->p.nksp; ++nk) {
    const int col = (nk & 1) ? 0 : 1;
    for (int cc : {col, 1 - col})
      for (int i : order) last[i] = add(kQSweep, i, 1, cc, (b->cases[i]->jmax - cc + 1) / 2, last[i]);
    if ((nk / c0->p.nbcimp) * c0->p.nbcimp == nk)
      for (int i : order) last[i] = add(kQBcimp, i, 1, 0, 1, last[i]);
  }
  const int blocks = lines_queue_blocks(b->wpl);
  if (blocks <= 0) { set_err("line sweep queue: no resident CTAs (%s)", cudaGetErrorString(cudaGetLastError())); return SMAC_ERR_CUDA; }
  if ((int)ph.size() != b->nphases) {
    cudaFree(b->d_phases);
    cudaFree(b->d_qint);
    b->d_phases = nullptr;
    b->d_qint = nullptr;
    CK(cudaMalloc(&b->d_phases, sizeof(QPhase) * ph.size()));
    CK(cudaMalloc(&b->d_qint, sizeof(int) * (3 + ph.size())));
    CK(cudaMemsetAsync(b->d_qint, 0, sizeof(int) * (3 + ph.size()), b->st));
  }
  CK(cudaMemcpyAsync(b->d_phases, ph.data(), sizeof(QPhase) * ph.size(), cudaMemcpyHostToDevice, b->st));
  CK(cudaStreamSynchronize(b->st));
  b->nphases = (int)ph.size();
  b->nitems = nitems;
  b->qblocks = std::min(blocks, nitems);
  return SMAC_OK;
}

// one graph per iteration of all cases with the line sweeps in one persistent launch: every
// case's work before its sweeps (a branch per case, factorisations included), the queue, every
// case's work after its sweeps
static int batch_capture_queue(smac_batch* b) {
  int rc = batch_queue_tables(b);
  if (rc) return rc;
  const int nc = (int)b->cases.size();
  QueueArgs qa;
  qa.phases = b->d_phases; qa.nphases = b->nphases; qa.nitems = b->nitems; qa.ncases = nc;
  qa.zargs = b->d_zargs; qa.bcim = b->d_bcim;
  qa.status = b->d_qint; qa.stall = b->d_qint + 1; qa.head = b->d_qint + 2; qa.done = b->d_qint + 3;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(b->ev_fork, b->st);
  for (int i = 0; i < nc; ++i) {
    smac_ctx* c = b->cases[i];
    cudaStreamWaitEvent(c->st, b->ev_fork, 0);
    iteration_pre_sweeps(c);
    cudaEventRecord(b->ev_pre[i], c->st);
    cudaStreamWaitEvent(b->st, b->ev_pre[i], 0);
    cudaStreamWaitEvent(b->st, c->ev_fk_join, 0);
  }
  cudaMemsetAsync(qa.head, 0, sizeof(int) * (1 + (size_t)b->nphases), b->st);
  launch_lines_queue(qa, b->wpl, b->qblocks, b->st);
  cudaEventRecord(b->ev_sweeps, b->st);
  for (int i = 0; i < nc; ++i) {
    smac_ctx* c = b->cases[i];
    cudaStreamWaitEvent(c->st, b->ev_sweeps, 0);
    iteration_post_sweeps(c);
    ++g_kernel_launches;
    k_record_next<<<1, 1, 0, c->st>>>(c->sc, b->hist + (size_t)i * b->cap, b->count + i, b->cap);
    cudaEventRecord(b->ev_done[i], c->st);
    cudaStreamWaitEvent(b->st, b->ev_done[i], 0);
  }
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  if (e != cudaSuccess) { set_err("batch capture: %s", cudaGetErrorString(e)); cudaGetLastError(); return SMAC_ERR_CUDA; }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { set_err("batch graph: %s", cudaGetErrorString(e)); cudaGetLastError(); return SMAC_ERR_CUDA; }
  return SMAC_OK;
}

// The assembly tile shapes of a batch: the default shape for every case.  A shape that is
// fastest for one grid on an otherwise idle GPU (the contexts' own autotuner) was measured to
// be slower when every SM is shared with other cases: 64 cases, 31.3 ms per iteration with the
// default shapes, 48.6 ms with each case's own choice and 34.9 ms with the shape that assembles
// all cases fastest when nothing else runs.
static int batch_default_tiles(smac_batch* b) {
  if (getenv("SMAC_CONUP_SHAPE")) return SMAC_OK;  // fixed by the environment (tests)
  for (smac_ctx* c : b->cases) c->conup[0] = c->conup[1] = 0;
  return SMAC_OK;
}

static int batch_capture(smac_batch* b) {
  int rc = batch_default_tiles(b);
  if (rc) return rc;
  if (b->queue) return batch_capture_queue(b);
  if (b->packed) return batch_capture_packed(b);
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(b->ev_fork, b->st);
  for (size_t i = 0; i < b->cases.size(); ++i) {
    smac_ctx* c = b->cases[i];
    cudaStreamWaitEvent(c->st, b->ev_fork, 0);
    iteration(c);
    ++g_kernel_launches;
    k_record_next<<<1, 1, 0, c->st>>>(c->sc, b->hist + (size_t)i * b->cap, b->count + i, b->cap);
    cudaEventRecord(b->ev_done[i], c->st);
    cudaStreamWaitEvent(b->st, b->ev_done[i], 0);
  }
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  if (e != cudaSuccess) { set_err("batch capture: %s", cudaGetErrorString(e)); cudaGetLastError(); return SMAC_ERR_CUDA; }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { set_err("batch graph: %s", cudaGetErrorString(e)); cudaGetLastError(); return SMAC_ERR_CUDA; }
  return SMAC_OK;
}

extern "C" int smac_batch_destroy(smac_batch* b) {
  if (!b) return SMAC_OK;
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->hist);
  cudaFree(b->count);
  cudaFree(b->d_zargs);
  cudaFree(b->d_start);
  cudaFree(b->d_bcim);
  cudaFree(b->d_phases);
  cudaFree(b->d_qint);
  for (cudaEvent_t e : b->ev_done) cudaEventDestroy(e);
  for (cudaEvent_t e : b->ev_pre) if (e) cudaEventDestroy(e);
  if (b->ev_sweeps) cudaEventDestroy(b->ev_sweeps);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return SMAC_OK;
}

extern "C" int smac_batch_create(int ncases, smac_ctx* const* cases, smac_batch** out) {
  if (!out || ncases < 1 || !cases) { set_err("bad arguments"); return SMAC_ERR_ARG; }
  *out = nullptr;
  smac_batch* b = new smac_batch();
  for (int i = 0; i < ncases; ++i) {
    if (!cases[i]) { set_err("case %d is null", i); delete b; return SMAC_ERR_ARG; }
    for (int k = 0; k < i; ++k)
      if (cases[k] == cases[i]) { set_err("case %d appears twice", i); delete b; return SMAC_ERR_ARG; }
    b->cases.push_back(cases[i]);
  }
  b->ev_done.resize(ncases, nullptr);
  b->ev_pre.resize(ncases, nullptr);
  b->stall_armed = getenv("SMAC_TEST_STALL_WAIT") != nullptr;
  bool ok = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_sweeps, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreate(&b->ev0) == cudaSuccess && cudaEventCreate(&b->ev1) == cudaSuccess &&
            cudaMalloc(&b->count, sizeof(int) * (size_t)ncases) == cudaSuccess;
  for (int i = 0; ok && i < ncases; ++i)
    ok = cudaEventCreateWithFlags(&b->ev_done[i], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->ev_pre[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) { set_err("batch streams/events: %s", cudaGetErrorString(cudaGetLastError())); smac_batch_destroy(b); return SMAC_ERR_CUDA; }
  *out = b;
  return SMAC_OK;
}

extern "C" int smac_batch_options(smac_batch* b, int layout, int warps_per_line) {
  if (!b) { set_err("null batch"); return SMAC_ERR_ARG; }
  if (layout != SMAC_BATCH_GRAPH && layout != SMAC_BATCH_PACKED_LINES && layout != SMAC_BATCH_QUEUE_LINES) {
    set_err("batch layout %d unknown", layout);
    return SMAC_ERR_ARG;
  }
  if (warps_per_line != 2 && warps_per_line != 4) { set_err("warps per line must be 2 or 4"); return SMAC_ERR_ARG; }
  const char* why = nullptr;
  if (layout != SMAC_BATCH_GRAPH && !packable(b, &why)) {
    set_err("%s: %s", layout == SMAC_BATCH_QUEUE_LINES ? "line sweep queue" : "packed lines", why);
    return SMAC_ERR_UNSUPPORTED;
  }
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  b->packed = layout == SMAC_BATCH_PACKED_LINES;
  b->queue = layout == SMAC_BATCH_QUEUE_LINES;
  b->wpl = warps_per_line;
  return SMAC_OK;
}

extern "C" int smac_batch_run(smac_batch* b, int n, smac_iter_out* hist) {
  if (!b || n < 0) { set_err("bad arguments"); return SMAC_ERR_ARG; }
  if (n == 0) return SMAC_OK;
  int rc = batch_alloc(b, n);
  if (rc) return rc;
  // the cases' own pending work comes first
  for (smac_ctx* c : b->cases) CK(cudaStreamSynchronize(c->st));
  if (!b->graph && (rc = batch_capture(b)) != SMAC_OK) return rc;
  for (smac_ctx* c : b->cases)
    if ((rc = take_launch_err(c)) != SMAC_OK) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
      return rc;
    }
  const size_t nc = b->cases.size();
  CK(cudaMemsetAsync(b->count, 0, sizeof(int) * nc, b->st));
  if (b->queue) {
    // the queue's wait status, and the stall a test asked for (any nonzero word)
    CK(cudaMemsetAsync(b->d_qint, 0, sizeof(int), b->st));
    if (b->stall_armed) CK(cudaMemsetAsync(b->d_qint + 1, 1, sizeof(int), b->st));
    b->stall_armed = false;
  }
  CK(cudaEventRecord(b->ev0, b->st));
  for (int i = 0; i < n; ++i) CK(cudaGraphLaunch(b->graph, b->st));
  CK(cudaEventRecord(b->ev1, b->st));
  std::vector<DevScalars> h((size_t)b->cap * nc);
  CK(cudaMemcpyAsync(h.data(), b->hist, sizeof(DevScalars) * h.size(), cudaMemcpyDeviceToHost, b->st));
  int qstatus = 0;
  if (b->queue) CK(cudaMemcpyAsync(&qstatus, b->d_qint, sizeof(int), cudaMemcpyDeviceToHost, b->st));
  CK(cudaStreamSynchronize(b->st));
  CK(cudaGetLastError());
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  int status = SMAC_OK;
  if (qstatus) {
    set_err("a wait of the line sweep queue ran out of time");
    status = qstatus;
  }
  for (size_t k = 0; k < nc; ++k)
    for (int i = 0; i < n; ++i) {
      const DevScalars& d = h[k * b->cap + i];
      if (hist) fill_out(d, hist + k * n + i);
      if (d.wait_status && status == SMAC_OK) { set_err("case %zu: a device wait ran out of time at iteration %d", k, d.nt); status = d.wait_status; }
      if (d.status && status == SMAC_OK) { set_err("case %zu: non-finite residual at iteration %d", k, d.nt); status = d.status; }
    }
  return status;
}

extern "C" double smac_batch_last_run_ms(smac_batch* b) { return b ? (double)b->last_ms : 0.0; }

extern "C" int smac_launches_per_iter(smac_ctx* c) {
  if (!c) return 0;
  if (c->launches == 0) {
    // count the launches of one iteration without running it: capture it into a graph
    // that is discarded
    cudaGraph_t g;
    long long before = g_kernel_launches;
    if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      iteration(c);
      if (cudaStreamEndCapture(c->st, &g) == cudaSuccess) cudaGraphDestroy(g);
    }
    c->launches = (int)(g_kernel_launches - before);
    cudaGetLastError();
  }
  return c->launches;
}

extern "C" int smac_profile_iteration(smac_ctx* c, double* stage_ms) {
  if (!c || !stage_ms) { set_err("null argument"); return SMAC_ERR_ARG; }
  StageTimer t;
  for (int i = 0; i < 64; ++i) CK(cudaEventCreate(&t.ev[i]));
  t.on = true;
  t.n = 0;
  CK(cudaStreamSynchronize(c->st));
  g_timer = &t;
  iteration(c);
  g_timer = nullptr;
  CK(cudaStreamSynchronize(c->st));
  if (int rc = take_launch_err(c)) {
    for (int i = 0; i < 64; ++i) cudaEventDestroy(t.ev[i]);
    return rc;
  }
  for (int i = 0; i < SMAC_NSTAGES; ++i) stage_ms[i] = 0.0;
  // each recorded boundary starts a stage that lasts until the next recorded boundary
  for (int i = 0; i + 1 < t.n; ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t.ev[i], t.ev[i + 1]);
    if (t.stage[i] >= 0 && t.stage[i] < SMAC_NSTAGES) stage_ms[t.stage[i]] += (double)ms;
  }
  for (int i = 0; i < 64; ++i) cudaEventDestroy(t.ev[i]);
  CK(cudaGetLastError());
  return SMAC_OK;
}

static double* field_ptr(smac_ctx* c, int f, size_t* n) {
  size_t N = c->N;
  switch (f) {
    case SMAC_FIELD_Q: *n = 3 * N; return c->q;
    case SMAC_FIELD_ANUT: *n = N; return c->anut;
    case SMAC_FIELD_VNUT: *n = N; return c->vnut;
    case SMAC_FIELD_S: *n = 3 * N; return c->s;
    case SMAC_FIELD_DQ: *n = 3 * N; return c->dq;
    case SMAC_FIELD_RTXY: *n = 6 * N; return c->rtxy;
    case SMAC_FIELD_DJ: *n = N; return c->dj;
    case SMAC_FIELD_BTC: *n = 9 * N; return c->btc;
    case SMAC_FIELD_BJM: *n = 9 * N; return c->bjm;
    case SMAC_FIELD_BJP: *n = 9 * N; return c->bjp;
    case SMAC_FIELD_BKM: *n = 9 * N; return c->bkm;
    case SMAC_FIELD_BKP: *n = 9 * N; return c->bkp;
    case SMAC_FIELD_SMIN: *n = N; return c->smin;
    default: return nullptr;
  }
}

extern "C" int smac_get_field(smac_ctx* c, int f, double* host) {
  if (!c || !host) { set_err("null argument"); return SMAC_ERR_ARG; }
  size_t n;
  double* p = field_ptr(c, f, &n);
  if (!p) { set_err("unknown field %d", f); return SMAC_ERR_ARG; }
  CK(cudaMemcpyAsync(host, p, n * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMAC_OK;
}

extern "C" int smac_set_field(smac_ctx* c, int f, const double* host) {
  if (!c || !host) { set_err("null argument"); return SMAC_ERR_ARG; }
  size_t n;
  double* p = field_ptr(c, f, &n);
  if (!p) { set_err("unknown field %d", f); return SMAC_ERR_ARG; }
  CK(cudaMemcpyAsync(p, host, n * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMAC_OK;
}

extern "C" int smac_get_state(smac_ctx* c, double* q, double* turvar, double* vnut) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  if (q) CK(cudaMemcpyAsync(q, c->q, 3 * c->N * 8, cudaMemcpyDeviceToHost, c->st));
  if (turvar) CK(cudaMemcpyAsync(turvar, c->anut, c->N * 8, cudaMemcpyDeviceToHost, c->st));
  if (vnut) CK(cudaMemcpyAsync(vnut, c->vnut, c->N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMAC_OK;
}

extern "C" int smac_set_state(smac_ctx* c, const double* q, const double* turvar) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  if (q) {
    CK(cudaMemcpyAsync(c->q, q, 3 * c->N * 8, cudaMemcpyHostToDevice, c->st));
    // the non-finite flag belonged to the state this one replaces
    CK(cudaMemsetAsync(&c->sc->status, 0, sizeof(int), c->st));
  }
  if (turvar) CK(cudaMemcpyAsync(c->anut, turvar, c->N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMAC_OK;
}

extern "C" int smac_get_clift(smac_ctx* c, double* clift) {
  if (!c || !clift) { set_err("null argument"); return SMAC_ERR_ARG; }
  CK(cudaStreamSynchronize(c->st));
  CK(cudaMemcpyAsync(clift, &c->sc->clift, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMAC_OK;
}

extern "C" int smac_set_clift(smac_ctx* c, double clift) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  CK(cudaStreamSynchronize(c->st));
  CK(cudaMemcpyAsync(&c->sc->clift, &clift, sizeof(double), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SMAC_OK;
}

// ------------------------------------------------------------------------------------------
// stage-level drop-ins: the caller's arrays are loaded into the context's buffers
static int check_dims(smac_ctx* c, int jmax, int kmax) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  if (jmax != c->jmax || kmax != c->kmax) { set_err("dimensions %dx%d differ from the context's %dx%d", jmax, kmax, c->jmax, c->kmax); return SMAC_ERR_ARG; }
  return SMAC_OK;
}

extern "C" int smac_lrelax(smac_ctx* c, int jmax, int kmax, const double* q, double* dq, double* s, double* btc,
                           double* bjm, double* bjp, double* bkm, double* bkp) {
  int rc = check_dims(c, jmax, kmax);
  if (rc) return rc;
  if (!q || !dq || !s || !btc || !bjm || !bjp || !bkm || !bkp) { set_err("null array"); return SMAC_ERR_ARG; }
  const size_t N = c->N;
  CK(cudaMemcpyAsync(c->q, q, 3 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->s, s, 3 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->btc, btc, 9 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->bjm, bjm, 9 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->bjp, bjp, 9 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->bkm, bkm, 9 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->bkp, bkp, 9 * N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(wait_status_ptr(c), 0, sizeof(int), c->st));
  lrelax(c, true);
  int ws = 0;
  CK(cudaMemcpyAsync(&ws, wait_status_ptr(c), sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(dq, c->dq, 3 * N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(s, c->s, 3 * N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(btc, c->btc, 9 * N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(bjp, c->bjp, 9 * N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(bkp, c->bkp, 9 * N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  if (ws) { set_err("a device wait ran out of time"); return ws; }
  return SMAC_OK;
}

extern "C" int smac_lreltur(smac_ctx* c, int jmax, int kmax, const double* turvar, double* ds, double* rhs,
                            const double* sjm, const double* sjp, const double* skm, const double* skp,
                            const double* stc) {
  int rc = check_dims(c, jmax, kmax);
  if (rc) return rc;
  if (!turvar || !ds || !rhs || !sjm || !sjp || !skm || !skp || !stc) { set_err("null array"); return SMAC_ERR_ARG; }
  const size_t N = c->N;
  CK(cudaMemcpyAsync(c->anut, turvar, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->sf, rhs, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->sjm, sjm, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->sjp, sjp, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->skm, skm, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->skp, skp, N * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->stc, stc, N * 8, cudaMemcpyHostToDevice, c->st));
  launch_fill(c->ds, 0.0, N, c->st);
  ScalarSweepArgs s;
  s.jmax = jmax; s.kmax = kmax; s.N = N;
  s.sjm = c->sjm; s.sjp = c->sjp; s.skm = c->skm; s.skp = c->skp; s.stc = c->stc; s.rhs = c->sf; s.ds = c->ds;
  const int exact = c->p.line_solver == SMAC_LINES_SEQUENTIAL;
  int nsmax = c->p.ntjsp > c->p.ntksp ? c->p.ntjsp : c->p.ntksp;
  for (int njk = 1; njk <= nsmax; ++njk) {
    if (c->p.ntjsp >= njk) {
      if (exact) launch_sa_sweep(0, s, exact, c->st);
      else if (launch_sa_sweep_part(0, s, c->sa_piv, c->sa_cf, c->st)) c->launch_err = SMAC_ERR_UNSUPPORTED;
      launch_bcimpds(c->d_bc, 1, jmax, N, c->anut, c->ds, c->sf, c->st);
    }
    if (c->p.ntksp >= njk) {
      if (exact) launch_sa_sweep(1, s, exact, c->st);
      else if (launch_sa_sweep_part(1, s, c->sa_piv, c->sa_cf, c->st)) c->launch_err = SMAC_ERR_UNSUPPORTED;
      launch_bcimpds(c->d_bc, 1, jmax, N, c->anut, c->ds, c->sf, c->st);
    }
  }
  CK(cudaMemcpyAsync(ds, c->ds, N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(rhs, c->sf, N * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  return take_launch_err(c);
}

extern "C" int smac_lusgs(smac_ctx* c, int jmax, int kmax, int neqs, const double* q, double* dq, double* rhs,
                          const double* btc, const double* bjm, const double* bjp, const double* bkm,
                          const double* bkp, double* scr1) {
  int rc = check_dims(c, jmax, kmax);
  if (rc) return rc;
  if (neqs != 1 && neqs != 3) { set_err("neqs must be 1 or 3"); return SMAC_ERR_ARG; }
  if (!q || !dq || !rhs || !btc || !bjm || !bjp || !bkm || !bkp) { set_err("null array"); return SMAC_ERR_ARG; }
  const size_t N = c->N;
  const size_t nb = (size_t)neqs * neqs * N, nv = (size_t)neqs * N;
  double* dq_d = neqs == 3 ? c->dq : c->ds;
  double* q_d = neqs == 3 ? c->q : c->anut;
  double* r_d = neqs == 3 ? c->s : c->sf;
  double *b0 = neqs == 3 ? c->btc : c->stc, *b1 = neqs == 3 ? c->bjm : c->sjm, *b2 = neqs == 3 ? c->bjp : c->sjp;
  double *b3 = neqs == 3 ? c->bkm : c->skm, *b4 = neqs == 3 ? c->bkp : c->skp;
  CK(cudaMemcpyAsync(q_d, q, nv * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(r_d, rhs, nv * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(b0, btc, nb * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(b1, bjm, nb * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(b2, bjp, nb * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(b3, bkm, nb * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(b4, bkp, nb * 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(dq_d, dq, nv * 8, cudaMemcpyHostToDevice, c->st));
  if (neqs == 3) launch_lusgs3(jmax, kmax, b0, b1, b2, b3, b4, c->bprm, r_d, dq_d, c->st);
  else launch_lusgs1(jmax, kmax, b0, b1, b2, b3, b4, c->bprm, r_d, dq_d, c->st);
  launch_bcimpds(c->d_bc, neqs, jmax, N, q_d, dq_d, r_d, c->st);
  CK(cudaMemcpyAsync(dq, dq_d, nv * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(rhs, r_d, nv * 8, cudaMemcpyDeviceToHost, c->st));
  if (scr1) CK(cudaMemcpyAsync(scr1, c->bprm, nb * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaGetLastError());
  return SMAC_OK;
}

// ------------------------------------------------------------------------------------------
// discrete adjoint (smac_adjoint.cu)
static int adj_ensure(smac_ctx* c) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  CK(cudaStreamSynchronize(c->st));
  CK(cudaStreamSynchronize(c->st_sa));
  DevScalars h;
  CK(cudaMemcpy(&h, c->sc, sizeof h, cudaMemcpyDeviceToHost));
  AdjointCtx v;
  v.jmax = c->jmax; v.kmax = c->kmax;
  v.beta = c->p.beta; v.cdis = c->p.cdis; v.vnu = c->vnu; v.pout = c->p.pout; v.pi = c->pi;
  v.ca = c->ca; v.sa = c->sa; v.clift = h.clift; v.dtau = c->p.dtau;
  v.ivis = c->p.ivis; v.visc64 = c->p.visc_fp64 != 0;
  v.q = c->q; v.rtxy = c->rtxy; v.dj = c->dj; v.x = c->x; v.y = c->y;
  v.btc = c->btc; v.bjm = c->bjm; v.bjp = c->bjp; v.bkm = c->bkm; v.bkp = c->bkp;
  v.d_bc = c->d_bc; v.bc = &c->bc; v.st = c->st;
  v.lpw[0] = c->zlpw[0] ? c->zlpw[0] : 1; v.lpw[1] = c->zlpw[1] ? c->zlpw[1] : 1;
  if (!c->adj_opt_set) {
    c->adj_opt = AdjointOptions{SMAC_ADJ_PREC_LINES_F32, 0.0, 16, 1, 100};
    c->adj_opt_set = true;
  }
  if (!c->adj) {
    int rc = SMAC_OK;
    char msg[256];
    c->adj = adjoint_new(v, c->adj_opt, &rc, msg, sizeof msg);
    if (!c->adj) { set_err("%s", msg); return rc; }
  } else {
    adjoint_update(c->adj, v, c->adj_opt);
  }
  return SMAC_OK;
}

static int adj_rc(smac_ctx* c, int rc) {
  if (rc) set_err("%s", adjoint_error(c->adj));
  return rc;
}

extern "C" int smac_adjoint_prepare(smac_ctx* c) {
  int rc = adj_ensure(c);
  if (rc) return rc;
  // the implicit operator at this state: its blocks give the preconditioner
  AssembleArgs a = assemble_args(c);
  launch_conup(a, c->st, c->conup[0], c->conup[1]);
  launch_bc(a, c->d_bc, c->sc, c->st);
  return adj_rc(c, adjoint_prepare(c->adj));
}

extern "C" int smac_adjoint_options(smac_ctx* c, int preconditioner, double dtau, int inner, int sweeps,
                                    int restart) {
  if (!c) { set_err("null context"); return SMAC_ERR_ARG; }
  if (preconditioner != SMAC_ADJ_PREC_LUSGS && preconditioner != SMAC_ADJ_PREC_LINES && preconditioner != SMAC_ADJ_PREC_LINES_F32) { set_err("preconditioner %d unknown", preconditioner); return SMAC_ERR_ARG; }
  if (inner < 1 || sweeps < 1 || restart < 1 || restart > kAdjMaxRestart) { set_err("inner, sweeps >= 1; restart 1..%d", kAdjMaxRestart); return SMAC_ERR_ARG; }
  c->adj_opt = AdjointOptions{preconditioner, dtau, inner, sweeps, restart};
  c->adj_opt_set = true;
  return SMAC_OK;
}

extern "C" int smac_adjoint_solve(smac_ctx* c, int objective, double rtol, int max_iter, int* iters,
                                  double* rel_resid) {
  if (!c || !c->adj) { set_err("smac_adjoint_prepare first"); return SMAC_ERR_ARG; }
  if (objective != SMAC_OBJ_CL && objective != SMAC_OBJ_CD) { set_err("objective %d unknown", objective); return SMAC_ERR_ARG; }
  if (!(rtol > 0.0) || max_iter < 1) { set_err("rtol > 0 and max_iter >= 1"); return SMAC_ERR_ARG; }
  return adj_rc(c, adjoint_solve(c->adj, objective, rtol, max_iter, iters, rel_resid));
}

extern "C" int smac_adjoint_gradient(smac_ctx* c, int objective, int ndv, const double* dxdb, const double* dydb,
                                     const double* dalpha, double* grad) {
  if (!c || !c->adj) { set_err("smac_adjoint_prepare first"); return SMAC_ERR_ARG; }
  if (objective != SMAC_OBJ_CL && objective != SMAC_OBJ_CD) { set_err("objective %d unknown", objective); return SMAC_ERR_ARG; }
  if (ndv < 0 || (ndv > 0 && !grad)) { set_err("ndv < 0 or grad NULL"); return SMAC_ERR_ARG; }
  return adj_rc(c, adjoint_gradient(c->adj, objective, ndv, dxdb, dydb, dalpha, grad));
}

extern "C" int smac_adjoint_residual(smac_ctx* c, double* F) {
  if (!F) { set_err("F is NULL"); return SMAC_ERR_ARG; }
  int rc = adj_ensure(c);
  if (rc) return rc;
  return adj_rc(c, adjoint_residual(c->adj, F));
}

extern "C" int smac_adjoint_jacvec(smac_ctx* c, int transpose, const double* v, double* y) {
  if (!c || !c->adj) { set_err("smac_adjoint_prepare first"); return SMAC_ERR_ARG; }
  if (!v || !y) { set_err("null vector"); return SMAC_ERR_ARG; }
  return adj_rc(c, adjoint_jacvec(c->adj, transpose != 0, v, y));
}

extern "C" int smac_adjoint_get(smac_ctx* c, int field, double* host) {
  if (!c || !c->adj) { set_err("smac_adjoint_prepare first"); return SMAC_ERR_ARG; }
  if (!host) { set_err("null buffer"); return SMAC_ERR_ARG; }
  return adj_rc(c, adjoint_get(c->adj, field, host));
}

extern "C" int smac_adjoint_forces(smac_ctx* c, double* cl, double* cd) {
  if (!c || !c->adj) { set_err("smac_adjoint_prepare first"); return SMAC_ERR_ARG; }
  adjoint_forces(c->adj, cl, cd);
  return SMAC_OK;
}
