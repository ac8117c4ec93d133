// noalloc.cu -- build_tree's root cube without any device allocation.
//
// fmmgen_root_box_noalloc computes the same root cube as fmmgen_tree_build
// (mean of the positions accumulated in particle order, half-width 1.001 times
// the largest |x - mean|; example/tree.cpp:139-187) with the same kernels, but
// its scratch -- the chunk sums, prefix values and chunk maps of the exact
// sequential sum, and the per-axis maxima -- lives in one file-scope device
// array instead of memory from cudaMalloc.  It is for callers that cannot
// allocate device memory at the point where they need the root cube: code
// running while another allocator (for example a framework's caching
// allocator) already holds the GPU's free memory, so a cudaMalloc would fail,
// and latency-bound callers that cannot afford cudaMalloc's implicit device
// synchronisation.
//
// The array is sized for at most FMMGEN_NOALLOC_MAX_N particles.  CUDA loads
// a library's device code lazily by default (CUDA_MODULE_LOADING=LAZY): the
// array, and the kernels this function launches, are placed on a device when
// the first call on that device looks the array up and launches them, and they
// stay there until the process exits (or the context is destroyed).  So the
// first call on each device needs the array's ~11 MiB and the kernels' code to
// be free on it: make that first call (a tiny input will do) before another
// allocator takes the GPU's free memory, and before any stream capture; later
// calls allocate nothing.  The looked-up address is cached per device for the
// life of the process: do not call this function again on a device after
// cudaDeviceReset.  All calls share the array and it keeps the last call's
// contents; what must start at zero (the maxima) is cleared by each call on
// its own stream.  Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array and give wrong results.
#include <algorithm>
#include <mutex>
#include "../../include/fmmgen_gb300.h"
#include "internal.h"

size_t fmm_seqsum_scratch(long N);
int fmm_seqsum3(const double *pos, long N, double *out, void *scratch, cudaStream_t st);
__global__ void k_root_absmax(const double *__restrict__ pos, long N, const double *sums, unsigned long long *mx);
__global__ void k_root_final(const double *sums, const unsigned long long *mx, long N, double *root, double *lev,
                             float2 *levf);

// layout: sums [0,24) | maxima [24,48) | level table [64,416) | FP32 level table [512,688) | sequential-sum scratch [1024,...)
#define NOALLOC_BYTES (11u << 20)  // 11 MiB: 1024 + fmm_seqsum_scratch(16,777,216) = 11,011,328 bytes
static __device__ __align__(256) unsigned char g_rootbox_scratch[NOALLOC_BYTES];

namespace {
std::mutex g_mu;
void *g_addr[64] = {};  // device address of g_rootbox_scratch, per device

// Looks the array's device address up once per device, with that device current.
int scratch_address(void **out) {
  int dev = 0;
  FMM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return FMM_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    FMM_CUDA_TRY(cudaGetSymbolAddress(&p, g_rootbox_scratch));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return FMM_OK;
}
}  // namespace

extern "C" int fmmgen_root_box_noalloc(const double *pos, long N, double *root4, void *stream) {
  if (!pos || !root4 || N < 1) {
    fmm_set_error_text("fmmgen_root_box_noalloc: pos and root4 must be device pointers and N >= 1");
    return FMM_ERR_ARG;
  }
  if (N > FMMGEN_NOALLOC_MAX_N || 1024 + fmm_seqsum_scratch(N) > NOALLOC_BYTES) {
    fmm_set_error_text("fmmgen_root_box_noalloc: N exceeds FMMGEN_NOALLOC_MAX_N (16777216) particles");
    return FMM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  void *base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  unsigned char *b = (unsigned char *)base;
  double *sums = (double *)b;
  unsigned long long *mx = (unsigned long long *)(b + 24);
  double *lev = (double *)(b + 64);
  float2 *levf = (float2 *)(b + 512);
  void *ss = b + 1024;
  // the maxima are combined with atomicMax and must start at zero
  FMM_CUDA_TRY(cudaMemsetAsync(mx, 0, 3 * sizeof(unsigned long long), st));
  rc = fmm_seqsum3(pos, N, sums, ss, st);
  if (rc) return rc;
  unsigned nbm = std::min<unsigned>(fmm_blocks(N, 256), 152 * 8);
  fmm_note_launch(), k_root_absmax<<<nbm, 256, 0, st>>>(pos, N, sums, mx);
  fmm_note_launch(), k_root_final<<<1, 1, 0, st>>>(sums, mx, N, root4, lev, levf);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
