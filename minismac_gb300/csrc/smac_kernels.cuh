// smac_kernels.cuh -- launch interfaces of the assembly and solver kernels.
#pragma once
#include "smac_common.cuh"

namespace smac {

// kernels launched by this library (host-side count, for the launch budget of an iteration)
extern long long g_kernel_launches;

// conup line tiles: W lines x TP points per CTA
constexpr int kConupW0 = 1, kConupTP0 = 128;   // j lines
constexpr int kConupW1 = 8, kConupTP1 = 16;    // k lines (8 consecutive j columns)
constexpr int kConupNumShapes = 4;              // tile shapes per direction the autotuner times
constexpr int kForceRec = 16;                   // doubles per wall point in the force scratch
constexpr int kResidParts = 304;               // 2 x 152 SMs

struct AssembleArgs {
  int jmax, kmax;
  size_t N;
  const double *q, *rtxy, *dj, *x, *y;
  double *s, *btc, *bjm, *bjp, *bkm, *bkp;
  double beta, cdis, vnu, dtau, pout, uinf, vinf, pi;
  int ivis, visc64;
};

struct SAArgs {
  int jmax, kmax;
  size_t N;
  const double *q, *rtxy, *dj, *anut, *smin;
  double *vort, *crs, *cs11, *cs12, *fr1;
  double *sjm, *sjp, *skm, *skp, *stc, *sf;
  double vnu, cb1, cb2, sigma, akarman, cw1, cw2, cw3r6, cv1, cv2, ct3tmp, ct4, cr1, cr2, cr3, rterm;
  int wall_fixed;
};

struct ForceArgs {
  int jmax;
  size_t N;
  const double *q, *rtxy, *dj, *x, *y;
  double vnu, ca, sa;
  int ivis;
  int term_off[SMAC_MAX_BC];
};

// assembly (smac_assemble.cu)
void launch_metric(const double* x, const double* y, double* rtxy, double* dj, int jmax, int kmax, cudaStream_t st);
void launch_ic(double* q, int jmax, int kmax, double ca, double sa, const BCTable* bc, cudaStream_t st);
void launch_dfunsa(const double* x, const double* y, size_t N, const double* wx, const double* wy, int nw,
                   double* smin, cudaStream_t st);
void launch_tsaic(double* anut, const double* smin, int jmax, int kmax, const BCTable* bc, double anutinf,
                  cudaStream_t st);
// both directions with tile shapes shape_j, shape_k (0 .. kConupNumShapes - 1; 0 = default)
void launch_conup(const AssembleArgs& a, cudaStream_t st, int shape_j = 0, int shape_k = 0);
void launch_conup_dir(const AssembleArgs& a, int dir, int shape, cudaStream_t st);
void launch_bc(const AssembleArgs& a, const BCTable* bc, const DevScalars* sc, cudaStream_t st);
void launch_resid(const double* s, const double* dj, int jmax, size_t N, void* scratch, double beta,
                  DevScalars* sc, cudaStream_t st);
size_t resid_scratch_bytes();
void launch_update(double* q, const double* dq, size_t N, cudaStream_t st);
void launch_iter_begin(DevScalars* sc, cudaStream_t st);
void launch_forces(const ForceArgs& f, const BCTable* bc_dev, const BCTable& bc_host, double* terms,
                   DevScalars* sc, cudaStream_t st);
void launch_sa_assembly(const SAArgs& a, const BCTable* bc, const DevScalars* sc, cudaStream_t st);
void launch_sa_update(double* anut, const double* ds, double* vnut, size_t N, double cv1, double vnu,
                      DevScalars* sc, cudaStream_t st);

// implicit solvers (smac_solve.cu)
struct BlockLines {
  int jmax, kmax;
  size_t N;
  double* btc;          // diagonal blocks (factored in place)
  const double* bjm;    // j sub-diagonal
  double* bjp;          // j super-diagonal (factored in place)
  const double* bkm;
  double* bkp;
};

// block tridiagonal factorisation of all lines of one direction (btlu3j/btlu3k)
void launch_btlu(int dir, const double* a, double* b, double* c, int jmax, int kmax, cudaStream_t st,
                 bool exact = true);
// undo of the factorisation (btund3j/btund3k): b restored in place, c restored into c_out
void launch_btund(int dir, const double* a, double* b, const double* c, double* c_out, int jmax, int kmax,
                  cudaStream_t st);

struct SweepArgs {
  int jmax, kmax;
  size_t N;
  const double *s, *btc, *am, *cp;   // factored diagonal, in-line sub / (factored) super diagonal
  const double *om, *op;             // off-line blocks (previous / next line)
  double* dq;
  double underr;
};
// one Gauss-Seidel line sweep in the reference order (ljsweep / lksweep)
void launch_gs_sweep(int dir, int nsw, const SweepArgs& a, int exact, cudaStream_t st);
// partitioned line solves (smac_lines.cu): transfer operators of every line after a
// factorisation, then a cluster-parallel sweep in the reference's line order
size_t line_ops_doubles(int dir, int jmax, int kmax);
void launch_line_prep(int dir, int jmax, int kmax, const double* b, const double* a, const double* c, double* ops,
                      cudaStream_t st);
int launch_gs_sweep_part(int dir, int nsw, const SweepArgs& a, const double* ops, cudaStream_t st);
size_t line_ops_rows_doubles(int n, int nl);
bool rows_supported(int n);
void launch_line_prep_rows(int n, int nl, int jmax, size_t N, const double* b, const double* a, const double* c,
                           double* ops, cudaStream_t st);
// wait_status: set to SMAC_ERR_TIMEOUT if a bounded wait for an operator block runs out; stall != 0
// makes the first line wait on a barrier that nothing completes (a test of that bound)
int launch_gs_sweep_rows(int nsw, const SweepArgs& a, const double* ops, int* wait_status, int stall,
                         cudaStream_t st);
void launch_bcimpds(const BCTable* bc, int neqs, int jmax, size_t N, const double* s, double* ds, double* rhs,
                    cudaStream_t st,
                    int kmajor_kmax = 0);
void launch_transpose(const double* in, double* out, int rows, int cols, size_t N, int planes, cudaStream_t st);

struct ScalarSweepArgs {
  int jmax, kmax;
  size_t N;
  const double *sjm, *sjp, *skm, *skp, *stc, *rhs;
  double* ds;
};
void launch_sa_sweep(int dir, const ScalarSweepArgs& a, int exact, cudaStream_t st);
// partitioned SA sweep (smac_lines.cu); piv, cf: N-sized scratch for the line pivots and c'
int launch_sa_sweep_part(int dir, const ScalarSweepArgs& a, double* piv, double* cf, cudaStream_t st);

// LU-SGS (lusgs / lusini3 / ilusol3 / lusini1 / ilusol1)
// picks the cluster shape of the LU-SGS sweeps (call outside stream capture, before the first sweep)
void ilu_setup();
void launch_lusgs3(int jmax, int kmax, const double* btc, const double* bjm, const double* bjp, const double* bkm,
                   const double* bkp, double* bprm, double* rhs, double* dq, cudaStream_t st);
void launch_lusgs1(int jmax, int kmax, const double* stc, const double* sjm, const double* sjp, const double* skm,
                   const double* skp, double* bprm, double* rhs, double* ds, cudaStream_t st);

void launch_fill(double* p, double v, size_t n, cudaStream_t st);
void launch_fill_f32(float* p, float v, size_t n, cudaStream_t st);

// throughput forms (smac_zebra.cu)
struct F32Ops {
  float *btc_j, *btc_k, *bjm, *bjp_f, *bjp_o, *bkm, *bkp, *bkp_o;  // 9N each (_f factored, _o original)
  float *s, *dq, *work;                                   // 3N each
};
template <typename W, typename S>
struct ZebraArgs {
  int jmax, kmax;
  size_t N;
  const W *btc, *am, *cp, *om, *op;
  const S* s;
  W* dq;
  W* work;
  W underr;
};
template <typename W, typename S>
void launch_zebra(int dir, const ZebraArgs<W, S>& a, int color, cudaStream_t st, int lines_per_warp = 1);
// the FP32 zebra lines of one colour of every case of a batch in one launch (one CTA of `wpl`
// warps per line; start: prefix of the cases' CTA counts, ncases + 1 entries)
void launch_zebra_packed(int dir, const ZebraArgs<float, float>* args, const int* start, int ncases, int nblocks,
                         int color, int wpl, cudaStream_t st);
struct BcimpArgs {  // one case of the packed FP32 wake-cut injection
  const BCTable* bc;
  int jmax;
  size_t N;
  const double* q;
  float *dq, *rhs;
};
void launch_bcimpds_f32_packed(const BcimpArgs* args, int ncases, int max_jmax, cudaStream_t st);
// the line sweeps of a batch iteration as one queue in one persistent launch (smac_zebra.cu)
enum QItemType { kQSweep = 0, kQBcimp = 1 };
struct QPhase {     // the items first .. first + nitems - 1 of one case
  int type, cas, dir, color;
  int first, nitems;
  int dep;          // the phase that must be complete before any item of this one (-1: none)
};
struct QueueArgs {
  const QPhase* phases;
  int nphases, nitems, ncases;
  const ZebraArgs<float, float>* zargs; // [direction][case]
  const BcimpArgs* bcim;                // [case]
  int* head;    // next item; zero at launch
  int* done;    // [phase] items done; zero at launch
  int* status;  // SMAC_ERR_TIMEOUT when a wait ran out
  int* stall;   // nonzero: the first item's wait is made to run out (tests)
};
int lines_queue_blocks(int wpl);
void launch_lines_queue(const QueueArgs& q, int wpl, int nblocks, cudaStream_t st);
void launch_to_f32(const double* btc, const double* bjm, const double* bjp, const double* bkm, const double* bkp,
                   const double* s, const F32Ops& o, size_t N, cudaStream_t st);
void launch_btlu_f32(int dir, const float* a, float* b, float* c, int jmax, int kmax, cudaStream_t st);
void launch_bcimpds_f32(const BCTable* bc, int jmax, size_t N, const double* q, float* dq, float* rhs,
                        cudaStream_t st);
void launch_dq_to_f64(const float* dq, double* dq64, size_t n3, cudaStream_t st);
struct SAZebraArgs {
  int jmax, kmax;
  size_t N;
  const double *am, *om, *op, *rhs, *piv, *cf;
  double *ds, *work;
};
void launch_sa_zebra(int dir, const SAZebraArgs& a, int color, cudaStream_t st);
// SA line pivots (scatri coefficient recurrence) of every line of one direction
void launch_sa_factor(int dir, const ScalarSweepArgs& s, double* piv, double* cf, cudaStream_t st);
// the same pivots with a warp per line (segment products of the pivot recurrence, scanned)
void launch_sa_factor_warp(int dir, const ScalarSweepArgs& s, double* piv, double* cf, cudaStream_t st);
// deterministic parallel force integration (tree reduction) for the throughput forms
void launch_forces_parallel(const ForceArgs& f, const BCTable* bc_dev, const BCTable& bc_host, double* terms,
                            DevScalars* sc, cudaStream_t st);

}  // namespace smac
