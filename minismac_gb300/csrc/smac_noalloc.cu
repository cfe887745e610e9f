// smac_noalloc.cu -- residual norms without any device allocation.
//
// Some callers cannot call cudaMalloc: a Fortran host that owns every device array itself
// (CUDA Fortran or OpenACC data regions) and is not allowed to let a library allocate behind
// it, or a host loop that runs under a fixed device-memory budget.  For them this file offers
// the residual scalars of one pseudo-time iteration (the largest |s*dj| with its location,
// divmax and the L2 norm of s) on caller-owned device arrays, with its scratch in a fixed
// file-scope device array instead of a context allocation.  The entry point has no
// counterpart in the reference.
//
// The scratch array is 16 KiB; every GPU that loads the library holds it until the process
// exits.  All calls share it and it keeps the last call's contents, so calls that overlap on
// the GPU (issued to different streams without ordering) race on it.  The partial records are
// fully rewritten by every call; the record that carries the result is initialised by each
// call before use.
#include <stdio.h>
#include <string.h>

#include "smac_common.cuh"
#include "smac_kernels.cuh"

using namespace smac;

namespace {

constexpr size_t kNoAllocScratchBytes = 16384;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_resid_scratch[kNoAllocScratchBytes];

// device address of g_resid_scratch per device, looked up once with that device current
static void* g_scratch_addr[kMaxDevices];
static thread_local char g_noalloc_err[256];

int scratch_for_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "no usable current CUDA device: %s", cudaGetErrorString(e));
    return SMAC_ERR_CUDA;
  }
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_resid_scratch);
    if (e != cudaSuccess || !ptr) {
      snprintf(g_noalloc_err, sizeof g_noalloc_err, "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return SMAC_ERR_CUDA;
    }
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return SMAC_OK;
}

}  // namespace

extern "C" const char* smac_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int smac_resid_noalloc(const double* s_dev, const double* dj_dev, int jmax, int kmax, double beta,
                                  int first_iteration, void* stream, smac_iter_out* out) {
  g_noalloc_err[0] = 0;
  if (!s_dev || !dj_dev || !out) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "null argument");
    return SMAC_ERR_ARG;
  }
  if (jmax < 5 || kmax < 5 || jmax > 8100 || kmax > 8100) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err,
             "grid %dx%d outside the supported 5..8100 per direction", jmax, kmax);
    return SMAC_ERR_ARG;
  }
  if (!(beta > 0)) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "beta must be > 0");
    return SMAC_ERR_ARG;
  }
  const size_t parts_bytes = resid_scratch_bytes();
  const size_t sc_off = (parts_bytes + 255) / 256 * 256;
  if (sc_off + sizeof(DevScalars) > kNoAllocScratchBytes) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "scratch of %zu bytes too small", kNoAllocScratchBytes);
    return SMAC_ERR_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  // every call copies through pageable host memory and waits for the stream: neither may be
  // captured into a graph, so a call on a capturing stream is refused before it touches it
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(st, &cap);
  if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    if (ce != cudaSuccess) cudaGetLastError();  // the query's own error is reported here, not left pending
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "stream is being captured (or its capture state is unknown: %s)",
             cudaGetErrorString(ce));
    return SMAC_ERR_UNSUPPORTED;
  }
  void* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  DevScalars* sc = reinterpret_cast<DevScalars*>(static_cast<unsigned char*>(base) + sc_off);
  DevScalars init;
  memset(&init, 0, sizeof init);
  init.nt = first_iteration ? 1 : 2;
  cudaError_t e = cudaMemcpyAsync(sc, &init, sizeof init, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "copy to scratch: %s", cudaGetErrorString(e));
    return SMAC_ERR_CUDA;
  }
  const size_t N = (size_t)jmax * kmax;
  launch_resid(s_dev, dj_dev, jmax, N, base, beta, sc, st);
  // a launch that failed is reported here, before anything reads the scratch it did not write
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "resid launch: %s", cudaGetErrorString(e));
    return SMAC_ERR_CUDA;
  }
  DevScalars d;
  e = cudaMemcpyAsync(&d, sc, sizeof d, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // execution errors of the kernels
  if (e != cudaSuccess) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "resid: %s", cudaGetErrorString(e));
    return SMAC_ERR_CUDA;
  }
  memset(out, 0, sizeof *out);
  out->nt = first_iteration ? 1 : 0;
  out->jres = d.jres;
  out->kres = d.kres;
  out->neq_res = d.neq;
  out->resmax = d.resmax;
  out->resmax0 = first_iteration ? d.resmax0 : 0.0;
  out->rmax = first_iteration ? d.resmax / d.resmax0 : 0.0;
  out->divmax = d.divmax;
  out->rhsnorm = d.rhsnorm;
  return d.status;
}
