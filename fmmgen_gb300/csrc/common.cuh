// common.cuh -- shared device/host helpers for the GB300 octree FMM library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#define FMM_PMAX 12          // highest expansion order the device code supports
#define FMM_NTMAX 455        // Nterms(12)
#define FMM_MAXLEVEL 21      // 3 bits per level in a 64-bit key
#define FMM_WARPS 4          // warps per block of the warp-per-cell kernels

// Multi-index layout of fmmgen (fmmgen/utils.py:26-35, 65-118): monomials ordered
// by total degree, then nx descending, then ny descending.
__host__ __device__ __forceinline__ int fmm_nterms(int p) {
  return p < 0 ? 0 : (p + 1) * (p + 2) * (p + 3) / 6;
}
__host__ __device__ __forceinline__ int fmm_idx3(int nx, int ny, int nz) {
  int d = nx + ny + nz, j = d - nx;
  return fmm_nterms(d - 1) + j * (j + 1) / 2 + (j - ny);
}
// row length rounded up to a multiple of 4 elements (16-byte rows for FP32 float4 access)
__host__ __device__ __forceinline__ int fmm_stride4(int n) { return (n + 3) / 4 * 4; }
struct MI { unsigned char x, y, z, d; };
__host__ __device__ __forceinline__ MI fmm_decode(int i) {
  int d = 0;
  while (fmm_nterms(d) <= i) d++;
  int r = i - fmm_nterms(d - 1);
  int j = 0;
  while ((j + 1) * (j + 2) / 2 <= r) j++;
  int ny = j - (r - j * (j + 1) / 2);
  int nx = d - j;
  MI m;
  m.x = (unsigned char)nx; m.y = (unsigned char)ny; m.z = (unsigned char)(d - nx - ny); m.d = (unsigned char)d;
  return m;
}

// Error flags raised by kernels (OR-ed into a device word the host reads).
#define FMM_EFLAG_DEPTH 1u     // a cell at FMM_MAXLEVEL still holds >= ncrit particles
#define FMM_EFLAG_RANGE 2u     // an M2L offset outside the class table's range
#define FMM_EFLAG_BOUNDS 4u    // an index check failed (never expected)
#define FMM_EFLAG_KEYS 8u      // the particle keys need more levels (the build recomputes them)
#define FMM_KEYLEVELS 10       // levels of digits in the first keys of a build

// Quadrupole sources (source order 2): S holds the degree-2 multipole
// coefficients (xx, xy, xz, yy, yz, zz) and a source at offset r = target -
// source contributes phi = sum_m S_m d^m (1/r) and E = -grad phi (the P2P of
// fmmgen/generator.py:257-288 for source_order 2, with the exact field).  With
// A the symmetric matrix of S (A_ii = S_ii, A_ij = S_ij / 2) and t = trace:
//   phi = (3 r.A.r - t r^2) / r^5,  E = 15 (r.A.r) r / r^7 - 3 (t r + 2 A r) / r^5.
template <typename T>
__host__ __device__ __forceinline__ void quadrupole_p2p(T x, T y, T z, const T *s, T &phi, T &ex, T &ey, T &ez) {
  const T r2 = x * x + y * y + z * z;
  const T rinv = T(1) / sqrt(r2), ri2 = rinv * rinv;
  const T r5 = ri2 * ri2 * rinv, r7 = r5 * ri2;
  const T h = T(0.5);
  const T ax = s[0] * x + h * (s[1] * y + s[2] * z);
  const T ay = h * (s[1] * x + s[4] * z) + s[3] * y;
  const T az = h * (s[2] * x + s[4] * y) + s[5] * z;
  const T rar = x * ax + y * ay + z * az, tr = s[0] + s[3] + s[5];
  phi += (T(3) * rar - tr * r2) * r5;
  const T c = T(15) * rar * r7, t3 = T(3) * r5;
  ex += c * x - t3 * (tr * x + T(2) * ax);
  ey += c * y - t3 * (tr * y + T(2) * ay);
  ez += c * z - t3 * (tr * z + T(2) * az);
}

// Status codes of the C ABI (mirrored in include/fmmgen_gb300.h).
#define FMM_OK 0
#define FMM_ERR_ARG 1
#define FMM_ERR_CUDA 2
#define FMM_ERR_DEPTH 3
#define FMM_ERR_RANGE 4
#define FMM_ERR_STATE 5

#define FMM_CUDA_TRY(expr)                                  \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) { fmm_set_cuda_error(_e, #expr, __FILE__, __LINE__); return FMM_ERR_CUDA; } \
  } while (0)

void fmm_set_cuda_error(cudaError_t e, const char *what, const char *file, int line);
void fmm_set_error_text(const char *msg);
// Counts kernel launches made by this library (every launch site calls it).
void fmm_note_launch();
long long fmm_launches();            // kernels launched so far
void fmm_add_launches(long long n);  // correction: kernels recorded in (not launched by) a graph capture, or replayed

__device__ __forceinline__ unsigned fmm_lane() { return threadIdx.x & 31u; }

template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t cap = 0;  // elements
};
// Grow-only device buffer (contents are not preserved on growth).
template <typename T> int fmm_reserve(DevBuf<T> &b, size_t n) {
  if (n <= b.cap && b.p) return FMM_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr; b.cap = 0;
  size_t want = n < 16 ? 16 : n + n / 8;
  FMM_CUDA_TRY(cudaMalloc((void **)&b.p, want * sizeof(T)));
  b.cap = want;
  return FMM_OK;
}
template <typename T> void fmm_release(DevBuf<T> &b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr; b.cap = 0;
}

static inline unsigned fmm_blocks(size_t n, unsigned bs) {
  size_t b = (n + bs - 1) / bs;
  return (unsigned)(b == 0 ? 1 : b);
}
