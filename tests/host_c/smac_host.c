/*
 * smac_host.c -- a C host of the GB300 library, written against include/smac_gb300.h only.
 *
 * It makes the calls the Fortran ISO_C_BINDING module of the integration notes makes from the
 * reference's solve loop (ref/smac2d.f:1238-1431): fill the run parameters from their
 * defaults (smac_params_default), create the context from the grid and the bcmain.dat rows
 * (smac_ctx_create), take nsteps pseudo-time iterations (smac_step, the call that replaces
 * `call step(...)` at ref/smac2d.f:1395), read the state back (smac_get_state) and destroy the
 * context.  The struct layouts it uses are the header's, so a layout mismatch between the
 * header and the library shows up here as wrong results.
 *
 * Input (binary, native byte order): int32 jmax, kmax, nbc, nsteps; float64 alpha, beta,
 * reynum; int32 rows[nbc][6] (ibcval zone jbeg jend kbeg kend); float64 x[jmax*kmax],
 * y[jmax*kmax] (j fastest).
 * Output: one text line per iteration "nt cl cd resmax rhsnorm" (%.17e) on stdout, and
 * q[3*jmax*kmax], turvar[jmax*kmax], vnut[jmax*kmax] (float64) into the output file.
 *
 * Usage: smac_host INPUT OUTPUT      exit status 0 on success.
 */
#include <stdio.h>
#include <stdlib.h>

#include "smac_gb300.h"

static int read_exact(FILE* f, void* p, size_t size, size_t n) { return fread(p, size, n, f) == n; }

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s INPUT OUTPUT\n", argv[0]);
    return 2;
  }
  FILE* in = fopen(argv[1], "rb");
  if (!in) { perror(argv[1]); return 2; }
  int hdr[4];
  double flow[3];
  if (!read_exact(in, hdr, sizeof(int), 4) || !read_exact(in, flow, sizeof(double), 3)) {
    fprintf(stderr, "short input header\n");
    return 2;
  }
  const int jmax = hdr[0], kmax = hdr[1], nbc = hdr[2], nsteps = hdr[3];
  if (jmax < 5 || kmax < 5 || nbc < 1 || nbc > SMAC_MAX_BC || nsteps < 1) {
    fprintf(stderr, "bad sizes %d %d %d %d\n", jmax, kmax, nbc, nsteps);
    return 2;
  }
  smac_bcspec bc;
  bc.nbc = nbc;
  for (int r = 0; r < nbc; ++r) {
    int row[6];
    if (!read_exact(in, row, sizeof(int), 6)) { fprintf(stderr, "short BC rows\n"); return 2; }
    bc.ibcval[r] = row[0]; bc.nzbc[r] = row[1]; bc.jbcb[r] = row[2];
    bc.jbce[r] = row[3]; bc.kbcb[r] = row[4]; bc.kbce[r] = row[5];
  }
  const size_t N = (size_t)jmax * (size_t)kmax;
  double* x = malloc(N * sizeof(double));
  double* y = malloc(N * sizeof(double));
  double* q = malloc(3 * N * sizeof(double));
  double* turvar = malloc(N * sizeof(double));
  double* vnut = malloc(N * sizeof(double));
  if (!x || !y || !q || !turvar || !vnut) { fprintf(stderr, "out of host memory\n"); return 2; }
  if (!read_exact(in, x, sizeof(double), N) || !read_exact(in, y, sizeof(double), N)) {
    fprintf(stderr, "short grid\n");
    return 2;
  }
  fclose(in);

  smac_params p;
  smac_params_default(&p);
  p.alpha = flow[0];
  p.beta = flow[1];
  p.reynum = flow[2];
  smac_ctx* ctx = NULL;
  int rc = smac_ctx_create(&p, jmax, kmax, x, y, &bc, &ctx);
  if (rc != SMAC_OK) { fprintf(stderr, "smac_ctx_create: %d %s\n", rc, smac_last_error()); return 1; }
  for (int it = 0; it < nsteps; ++it) {
    smac_iter_out o;
    rc = smac_step(ctx, &o);
    if (rc != SMAC_OK) { fprintf(stderr, "smac_step: %d %s\n", rc, smac_last_error()); return 1; }
    printf("%d %.17e %.17e %.17e %.17e\n", o.nt, o.cl, o.cd, o.resmax, o.rhsnorm);
  }
  rc = smac_get_state(ctx, q, turvar, vnut);
  if (rc != SMAC_OK) { fprintf(stderr, "smac_get_state: %d %s\n", rc, smac_last_error()); return 1; }
  rc = smac_ctx_destroy(ctx);
  if (rc != SMAC_OK) { fprintf(stderr, "smac_ctx_destroy: %d %s\n", rc, smac_last_error()); return 1; }
  FILE* out = fopen(argv[2], "wb");
  if (!out) { perror(argv[2]); return 2; }
  int ok = fwrite(q, sizeof(double), 3 * N, out) == 3 * N && fwrite(turvar, sizeof(double), N, out) == N &&
           fwrite(vnut, sizeof(double), N, out) == N;
  fclose(out);
  free(x); free(y); free(q); free(turvar); free(vnut);
  return ok ? 0 : 2;
}
