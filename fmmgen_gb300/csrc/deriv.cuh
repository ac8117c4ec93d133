// deriv.cuh -- warp-cooperative derivatives of 1/R.
//
// D[idx(n)] = d^n (1/R) at (x, y, z), |n| <= p, the quantity fmmgen's
// Phi_derivatives / generate_derivs differentiate symbolically
// (fmmgen/expansions.py:108-141, fmmgen/generator.py:82-93).  Evaluated with
// the Hermite-type recurrence for g(R^2) = (R^2)^(-1/2):
//   R^(m)_0     = (-1)^m (2m-1)!! / R^(2m+1)
//   R^(m)_{n+e} = x_e R^(m+1)_n + n_e R^(m+1)_{n-e},      D_n = R^(0)_n
// One level m at a time, all monomials of that level in parallel across lanes.
#pragma once
#include "common.cuh"
#include "mi_table.cuh"

// Buffers D and tmp (each >= Nterms(p) elements) must be warp-private shared
// memory; sbase needs p+1 elements.  Result ends in D.
template <typename T>
__device__ void warp_derivs(T x, T y, T z, int p, T *D, T *tmp, T *sbase) {
  const int lane = threadIdx.x & 31;
  T r2 = x * x + y * y + z * z;
  T rinv = T(1) / sqrt(r2);
  T rinv2 = rinv * rinv;
  if (lane <= p) {
    T b = rinv;
    for (int i = 1; i <= lane; i++) b = -T(2 * i - 1) * rinv2 * b;
    sbase[lane] = b;
  }
  __syncwarp();
  // level m = p lives in the buffer that ends up being read at level p-1;
  // choose the start buffer so the final level (m = 0) lands in D.
  T *A = (p & 1) ? tmp : D;
  T *B = (p & 1) ? D : tmp;
  // after processing levels p-1..0 we swap p times: final = A if p even.
  if (lane == 0) A[0] = sbase[p];
  __syncwarp();
  for (int m = p - 1; m >= 0; m--) {
    int cnt = fmm_nterms(p - m);
    T base = sbase[m];
    for (int i = lane; i < cnt; i += 32) {
      int nx = c_mi[i][0], ny = c_mi[i][1], nz = c_mi[i][2];
      T v;
      if (i == 0) v = base;
      else if (nx > 0) {
        v = x * A[fmm_idx3(nx - 1, ny, nz)];
        if (nx > 1) v += T(nx - 1) * A[fmm_idx3(nx - 2, ny, nz)];
      } else if (ny > 0) {
        v = y * A[fmm_idx3(nx, ny - 1, nz)];
        if (ny > 1) v += T(ny - 1) * A[fmm_idx3(nx, ny - 2, nz)];
      } else {
        v = z * A[fmm_idx3(nx, ny, nz - 1)];
        if (nz > 1) v += T(nz - 1) * A[fmm_idx3(nx, ny, nz - 2)];
      }
      B[i] = v;
    }
    __syncwarp();
    T *t = A; A = B; B = t;
  }
  // A == D here by the parity choice above
}

// D[idx(n)] = d^n (1/|y|) at y, |n| <= q, in one thread, degree by degree:
//   |n| |y|^2 D_n = -(2|n| - 1) sum_a n_a y_a D_(n - e_a) - (|n| - 1) sum_a n_a (n_a - 1) D_(n - 2 e_a)
template <typename T>
__device__ __forceinline__ void thread_derivs(T yx, T yy, T yz, int q, T *D) {
  const T ir2 = T(1) / (yx * yx + yy * yy + yz * yz);
  D[0] = sqrt(ir2);
  int i = 1;
  for (int d = 1; d <= q; d++) {
    const T rd = T(1) / T(d), a1 = -T(2 * d - 1) * ir2 * rd, a2 = -T(d - 1) * ir2 * rd;
    for (int nx = d; nx >= 0; nx--)
      for (int ny = d - nx; ny >= 0; ny--, i++) {
        const int nz = d - nx - ny;
        T s1 = 0, s2 = 0;
        if (nx) {
          s1 += T(nx) * yx * D[fmm_idx3(nx - 1, ny, nz)];
          if (nx > 1) s2 += T(nx * (nx - 1)) * D[fmm_idx3(nx - 2, ny, nz)];
        }
        if (ny) {
          s1 += T(ny) * yy * D[fmm_idx3(nx, ny - 1, nz)];
          if (ny > 1) s2 += T(ny * (ny - 1)) * D[fmm_idx3(nx, ny - 2, nz)];
        }
        if (nz) {
          s1 += T(nz) * yz * D[fmm_idx3(nx, ny, nz - 1)];
          if (nz > 1) s2 += T(nz * (nz - 1)) * D[fmm_idx3(nx, ny, nz - 2)];
        }
        D[i] = a1 * s1 + a2 * s2;
      }
  }
}
