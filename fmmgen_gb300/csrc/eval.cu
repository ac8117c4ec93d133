// eval.cu -- the FMM evaluation pass on the device octree
// (Tree::compute_field_fmm, example/tree.cpp:243-271).
//
// Expansions are kept scaled by the cell half-width s so that both FP64 and
// FP32 see O(1) numbers at any cell size:
//   M~_n = M_n / s^|n|            L^_n = s^(|n|+1) L_n
// which turns the operators into
//   P2M  M~_n  = sum_p q ((c - x)/s)^n / n!                      (dipole: sum_j S_j/s (..)^(n-e_j)/(n-e_j)!)
//   M2M  M~p_n = sum_k M~c_{n-k} 2^-|n-k| (d/s_p)^k / k!          d = parent - child
//   M2L  L^A_n = sum_m 2^((lA-lB)|m|) D_{n+m}(d/s_A) M~B_m        d = A - B
//   L2L  L^c_n = 2^-(|n|+1) sum_k (d/s_p)^k / k! L^p_{n+k}          d = child - parent
//   L2P  phi   = (1/s) sum_n L^_n (r/s)^n / n!,  E = -grad phi      r = particle - cell
// (fmmgen/expansions.py:22-207 with D homogeneous of degree -|k|-1).  The
// displacement conventions are those of example/calculate.cpp:149-151, 182-184,
// 201-203, 227-229, 243-245.
#include <algorithm>
#include <type_traits>
#include "internal.h"
#include "mi_table.cuh"
#include "m2l_gen.cuh"
#include "deriv.cuh"

#define TRY(x) do { int _rc = (x); if (_rc) return _rc; } while (0)

// ---------------------------------------------------------------------------
// warp contraction engine (plans.cu)
// ---------------------------------------------------------------------------
// Four tasks per round: their words and operands are loaded before the first
// is applied, so the dependent task-word -> shared-memory loads of a round
// overlap (a lane's tasks are one contiguous range; pad words end it).
template <typename T>
__device__ __forceinline__ void engine_run(const Plan &P, const T *A, const T *B, T *slots, int lane) {
  constexpr uint32_t PAD = 0xffffffffu;
  T acc = T(0);
  // the next round's task words are requested while this round is applied
  uint32_t wn[4];
#pragma unroll
  for (int u = 0; u < 4; u++) wn[u] = u < P.iters ? __ldg(&P.task[u * 32 + lane]) : PAD;
  for (int it = 0; it < P.iters; it += 4) {
    uint32_t w[4];
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      w[u] = wn[u];
      wn[u] = it + 4 + u < P.iters ? __ldg(&P.task[(it + 4 + u) * 32 + lane]) : PAD;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const uint32_t x = w[u] == PAD ? 0u : w[u];
      a[u] = A[x & 1023u];
      b[u] = B[(x >> 10) & 1023u];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (w[u] == PAD) return;
      acc += a[u] * b[u];
      if (w[u] >> 31) {
        slots[(w[u] >> 20) & 2047u] += acc;
        acc = T(0);
      }
    }
  }
}
template <typename T> __device__ __forceinline__ T engine_out(const Plan &P, const T *slots, int n) {
  T s = T(0);
  for (int k = __ldg(&P.out_seg[n]); k < __ldg(&P.out_seg[n + 1]); k++) s += slots[k];
  return s;
}

// 2^e built from the exponent bits (|e| well inside the normal range here);
// avoids FP64 ldexp, which runs on GB300's narrow FP64 pipe.
template <typename T> __device__ __forceinline__ T exp2i(int e);
template <> __device__ __forceinline__ float exp2i<float>(int e) { return __int_as_float((e + 127) << 23); }
template <> __device__ __forceinline__ double exp2i<double>(int e) {
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// 1/q for the factorials, in each precision (no divisions in the loops)
static __constant__ float c_rcpf[FMM_PMAX + 1] = {0.f, 1.f, 1.f / 2, 1.f / 3, 1.f / 4, 1.f / 5, 1.f / 6,
                                                  1.f / 7, 1.f / 8, 1.f / 9, 1.f / 10, 1.f / 11, 1.f / 12};
static __constant__ double c_rcpd[FMM_PMAX + 1] = {0., 1., 1. / 2, 1. / 3, 1. / 4, 1. / 5, 1. / 6,
                                                   1. / 7, 1. / 8, 1. / 9, 1. / 10, 1. / 11, 1. / 12};
template <typename T> __device__ __forceinline__ T rcp_int(int q);
template <> __device__ __forceinline__ float rcp_int<float>(int q) { return c_rcpf[q]; }
template <> __device__ __forceinline__ double rcp_int<double>(int q) { return c_rcpd[q]; }

// ---------------------------------------------------------------------------
// P2M (example/calculate.cpp:135-161)
// ---------------------------------------------------------------------------
#define NPL ((FMM_NTMAX + 31) / 32)
template <typename T>
__global__ void __launch_bounds__(32 * FMM_WARPS) k_p2m(const int *leaf_cells, int nleaves, const int *pstart,
                                                        const int *pcount, const unsigned char *clevel,
                                                        const double *cx, const double *cy, const double *cz,
                                                        const double *px, const double *py, const double *pz,
                                                        const uint32_t *perm, const double *S, int so, int order,
                                                        const double *cr, T *M, int mstr) {
  __shared__ T tb[FMM_WARPS][3][32][FMM_PMAX + 1];
  __shared__ T sq[FMM_WARPS][32][6];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int leaf = blockIdx.x * FMM_WARPS + w;
  if (leaf >= nleaves) return;
  const int c = leaf_cells[leaf];
  const int off = fmm_nterms(so - 1), msize = fmm_nterms(order) - off;
  const double s = cr[c];
  const double inv_s = s > 0 ? 1.0 / s : 0.0;  // a zero-width root (coincident points) has no far field
  const double ccx = cx[c], ccy = cy[c], ccz = cz[c];
  const int p0 = pstart[c], np = pcount[c];
  T acc[NPL];
#pragma unroll
  for (int k = 0; k < NPL; k++) acc[k] = T(0);
  for (int base = 0; base < np; base += 32) {
    int j = base + lane;
    if (j < np) {
      int i = p0 + j;
      T ux = (T)((ccx - px[i]) * inv_s), uy = (T)((ccy - py[i]) * inv_s), uz = (T)((ccz - pz[i]) * inv_s);
      T a = 1, b = 1, d = 1;
      tb[w][0][lane][0] = a; tb[w][1][lane][0] = b; tb[w][2][lane][0] = d;
      for (int k = 1; k <= order; k++) {
        const T rk = rcp_int<T>(k);
        a = a * ux * rk; b = b * uy * rk; d = d * uz * rk;
        tb[w][0][lane][k] = a; tb[w][1][lane][k] = b; tb[w][2][lane][k] = d;
      }
      uint32_t o = perm[i];
      if (so == 0) {
        sq[w][lane][0] = (T)S[o];
      } else if (so == 1) {
        sq[w][lane][0] = (T)(S[3 * (size_t)o] * inv_s);
        sq[w][lane][1] = (T)(S[3 * (size_t)o + 1] * inv_s);
        sq[w][lane][2] = (T)(S[3 * (size_t)o + 2] * inv_s);
      } else {  // quadrupole: the degree-2 coefficients, scaled by 1 / s^2
        for (int k = 0; k < 6; k++) sq[w][lane][k] = (T)(S[6 * (size_t)o + k] * inv_s * inv_s);
      }
    }
    __syncwarp();
    int cnt = min(32, np - base);
#pragma unroll
    for (int k = 0; k < NPL; k++) {
      int i = lane + 32 * k;
      if (i < msize) {
        int nx = c_mi[i + off][0], ny = c_mi[i + off][1], nz = c_mi[i + off][2];
        T sum = acc[k];
        if (so == 0) {
          for (int jj = 0; jj < cnt; jj++)
            sum += sq[w][jj][0] * tb[w][0][jj][nx] * tb[w][1][jj][ny] * tb[w][2][jj][nz];
        } else if (so == 1) {
          for (int jj = 0; jj < cnt; jj++) {
            if (nx) sum += sq[w][jj][0] * tb[w][0][jj][nx - 1] * tb[w][1][jj][ny] * tb[w][2][jj][nz];
            if (ny) sum += sq[w][jj][1] * tb[w][0][jj][nx] * tb[w][1][jj][ny - 1] * tb[w][2][jj][nz];
            if (nz) sum += sq[w][jj][2] * tb[w][0][jj][nx] * tb[w][1][jj][ny] * tb[w][2][jj][nz - 1];
          }
        } else {
          // M~_n += sum_{|k| = 2, k <= n} S~_k u^(n-k) / (n-k)!, k in the layout
          // order xx xy xz yy yz zz
          for (int jj = 0; jj < cnt; jj++)
#pragma unroll
            for (int kk = 0; kk < 6; kk++) {
              const int kx = c_mi[4 + kk][0], ky = c_mi[4 + kk][1], kz = c_mi[4 + kk][2];
              if (nx >= kx && ny >= ky && nz >= kz)
                sum += sq[w][jj][kk] * tb[w][0][jj][nx - kx] * tb[w][1][jj][ny - ky] * tb[w][2][jj][nz - kz];
            }
        }
        acc[k] = sum;
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int k = 0; k < NPL; k++) {
    int i = lane + 32 * k;
    if (i < msize) M[(size_t)c * mstr + i] = acc[k];
  }
}

// shift monomials mon[idx(k)] = v^k / k! for |k| <= pmax (warp-parallel, in T)
template <typename T>
__device__ __forceinline__ void warp_monomials(double vx, double vy, double vz, int pmax, T *mon, int lane) {
  int cnt = fmm_nterms(pmax);
  const T x = (T)vx, y = (T)vy, z = (T)vz;
  for (int i = lane; i < cnt; i += 32) {
    int kx = c_mi[i][0], ky = c_mi[i][1], kz = c_mi[i][2];
    T a = 1, b = 1, d = 1;
    for (int q = 1; q <= kx; q++) a = a * x * rcp_int<T>(q);
    for (int q = 1; q <= ky; q++) b = b * y * rcp_int<T>(q);
    for (int q = 1; q <= kz; q++) d = d * z * rcp_int<T>(q);
    mon[i] = a * b * d;
  }
}

// ---------------------------------------------------------------------------
// M2M for all parents of one level (example/calculate.cpp:163-187)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(32 * FMM_WARPS) k_m2m(Plan P, int lo, int hi, int so, int order,
                                                        const unsigned char *child_mask, const int *child_first,
                                                        const unsigned char *clevel, const double *cx,
                                                        const double *cy, const double *cz, const double *cr,
                                                        T *M, int mstr) {
  __shared__ T sA[FMM_WARPS][FMM_NTMAX], sB[FMM_WARPS][FMM_NTMAX], sS[FMM_WARPS][FMM_NTMAX + 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = lo + blockIdx.x * FMM_WARPS + w;
  if (c >= hi) return;
  unsigned mask = child_mask[c];
  if (!mask) return;
  const int off = fmm_nterms(so - 1), msize = fmm_nterms(order) - off;
  const double inv_s = 1.0 / cr[c];
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = T(0);
  int ch = child_first[c];
  int nch = __popc(mask);
  for (int q = 0; q < nch; q++, ch++) {
    __syncwarp();
    warp_monomials<T>((cx[c] - cx[ch]) * inv_s, (cy[c] - cy[ch]) * inv_s, (cz[c] - cz[ch]) * inv_s, order - so,
                      sA[w], lane);
    for (int j = lane; j < msize; j += 32) sB[w][j] = M[(size_t)ch * mstr + j] * exp2i<T>(-(int)c_mi[j + off][3]);
    __syncwarp();
    engine_run<T>(P, sA[w], sB[w], sS[w], lane);
  }
  __syncwarp();
  for (int n = lane; n < msize; n += 32) M[(size_t)c * mstr + n] = engine_out<T>(P, sS[w], n);
}

// ---------------------------------------------------------------------------
// M2L, one warp per target cell (example/calculate.cpp:190-206)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(32 * FMM_WARPS) k_m2l(Plan P, int ncells, int so, int order, const int *off_,
                                                        const int *src, const int *cls, const T *clsD,
                                                        const unsigned char *clevel, const T *M, T *L, int mstr,
                                                        int lstr, int dstr) {
  __shared__ T sA[FMM_WARPS][FMM_NTMAX], sB[FMM_WARPS][FMM_NTMAX], sS[FMM_WARPS][FMM_NTMAX + 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int A = blockIdx.x * FMM_WARPS + w;
  if (A >= ncells) return;
  const int moff = fmm_nterms(so - 1), msize = fmm_nterms(order) - moff, lsize = fmm_nterms(order - so);
  const int nt = fmm_nterms(order);
  const int k0 = off_[A], k1 = off_[A + 1];
  if (k0 == k1) {
    for (int n = lane; n < lsize; n += 32) L[(size_t)A * lstr + n] = T(0);
    return;
  }
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = T(0);
  const int la = clevel[A];
  for (int k = k0; k < k1; k++) {
    const int B = src[k];
    const T *D = clsD + (size_t)cls[k] * dstr;
    const int dl = la - (int)clevel[B];  // rho = s_B / s_A = 2^(lA - lB)
    __syncwarp();
    for (int i = lane; i < nt; i += 32) sA[w][i] = D[i];
    for (int j = lane; j < msize; j += 32) sB[w][j] = M[(size_t)B * mstr + j] * exp2i<T>(dl * (int)c_mi[j + moff][3]);
    __syncwarp();
    engine_run<T>(P, sA[w], sB[w], sS[w], lane);
  }
  __syncwarp();
  for (int n = lane; n < lsize; n += 32) L[(size_t)A * lstr + n] = engine_out<T>(P, sS[w], n);
}

// ---------------------------------------------------------------------------
// M2L with a per-pair order (learned order selection, learn.cu): pair k of
// target A is applied at order q_k <= order, i.e. only the terms with
// |n| + |m| <= q_k of the order-`order` contraction -- the leading blocks of D,
// M and L in the degree-major layout, so the order-q_k plan runs on the same
// rows.  One launch per order q: every warp of it runs the one order-q plan
// (whose task words then stay in L1), takes its target's pairs of order q and
// accumulates them in its slots, and adds the sums to L once; L is zeroed
// before the first launch.  One warp per target.
// ---------------------------------------------------------------------------
#define M2LV_R ((FMM_NTMAX + 31) / 32)
template <typename T>
__global__ void __launch_bounds__(32 * FMM_WARPS) k_m2l_var(Plan P, int q, int ncells, int so, int order,
                                                            const int *off_, const int *src, const int *cls,
                                                            const unsigned char *ord, const T *clsD,
                                                            const unsigned char *clevel, const T *M, T *L, int mstr,
                                                            int lstr, int dstr) {
  __shared__ T sA[FMM_WARPS][FMM_NTMAX], sB[FMM_WARPS][FMM_NTMAX], sS[FMM_WARPS][FMM_NTMAX + 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int A = blockIdx.x * FMM_WARPS + w;
  if (A >= ncells) return;
  const int moff = fmm_nterms(so - 1), nt = fmm_nterms(q), ms = nt - moff, ls = fmm_nterms(q - so);
  const int la = clevel[A];
  const int k0 = off_[A], k1 = off_[A + 1];
  // the next pair of order q: 32 orders at a time, one ballot each (warp-uniform)
  int cbase = k0 - 32;
  unsigned hits = 0;
  auto next = [&]() -> int {
    while (!hits) {
      cbase += 32;
      if (cbase >= k1) return -1;
      const int kk = cbase + lane;
      hits = __ballot_sync(0xffffffffu, kk < k1 && min(max((int)ord[kk], so + 1), order) == q);
    }
    const int b = __ffs(hits) - 1;
    hits &= hits - 1;
    return cbase + b;
  };
  int kn = next();
  if (kn < 0) return;
  // the operands of the next pair are loaded into registers while the engine
  // runs on the current one
  T dr[M2LV_R], mr[M2LV_R];
  int dln = 0;
  auto fetch = [&](int k) {
    const int B = src[k];
    const T *D = clsD + (size_t)cls[k] * dstr;
    dln = la - (int)clevel[B];
#pragma unroll
    for (int r = 0; r < M2LV_R; r++) {
      const int i = lane + 32 * r;
      dr[r] = i < nt ? D[i] : T(0);
      mr[r] = i < ms ? M[(size_t)B * mstr + i] : T(0);
    }
  };
  fetch(kn);
  for (int s = lane; s < P.nseg; s += 32) sS[w][s] = T(0);
  while (kn >= 0) {
    const int dl = dln;
    __syncwarp();
#pragma unroll
    for (int r = 0; r < M2LV_R; r++) {
      const int i = lane + 32 * r;
      if (i < nt) sA[w][i] = dr[r];
      if (i < ms) sB[w][i] = mr[r] * exp2i<T>(dl * (int)c_mi[i + moff][3]);
    }
    __syncwarp();
    kn = next();
    if (kn >= 0) fetch(kn);
    engine_run<T>(P, sA[w], sB[w], sS[w], lane);
  }
  __syncwarp();
  for (int n = lane; n < ls; n += 32) L[(size_t)A * lstr + n] += engine_out<T>(P, sS[w], n);
}

// ---------------------------------------------------------------------------
// FP32 M2L with NP (2 or 4) source cells per engine pass.  A and B hold the NP
// pairs' operands side by side, so one task word drives NP/2 packed FMAs
// (fma.rn.f32x2): the task-word load and index decoding, which bound the
// engine's issue rate, are shared by NP multiply-adds.  All lanes of the
// accumulator go to the same output slot.  With `ord` set only the pairs of
// order q are taken and the sums are added to L (one launch per order); with
// `ord` null every pair is taken at order q and L is written.  Missing pairs of
// a target's last group run beside zeros.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ float hsum2(unsigned long long v) {
  return __uint_as_float((unsigned)v) + __uint_as_float((unsigned)(v >> 32));
}
template <int NP> struct PackF;
template <> struct PackF<2> {
  using V = unsigned long long;
  static constexpr int WARPS = 4;
  struct Acc {
    unsigned long long a = 0ull;
    __device__ __forceinline__ void fma(V x, V y) { a = ffma2(x, y, a); }
    __device__ __forceinline__ float take() { const float r = hsum2(a); a = 0ull; return r; }
  };
};
template <> struct PackF<4> {
  using V = ulonglong2;
  static constexpr int WARPS = 2;  // 16.5 KB of operands and slots per warp
  struct Acc {
    unsigned long long a = 0ull, b = 0ull;
    __device__ __forceinline__ void fma(V x, V y) { a = ffma2(x.x, y.x, a); b = ffma2(x.y, y.y, b); }
    __device__ __forceinline__ float take() {
      const float r = hsum2(a) + hsum2(b);
      a = b = 0ull;
      return r;
    }
  };
};
template <int NP>
__device__ __forceinline__ void engine_run_pk(const Plan &P, const float *A, const float *B, float *slots, int lane) {
  using V = typename PackF<NP>::V;
  constexpr uint32_t PAD = 0xffffffffu;
  const V *A2 = reinterpret_cast<const V *>(A);
  const V *B2 = reinterpret_cast<const V *>(B);
  typename PackF<NP>::Acc acc;
  // the next round's task words are requested while this round's operands are
  // read and applied (they come from L2 when the plan does not fit in L1)
  uint32_t wn[4];
#pragma unroll
  for (int u = 0; u < 4; u++) wn[u] = u < P.iters ? __ldg(&P.task[u * 32 + lane]) : PAD;
  for (int it = 0; it < P.iters; it += 4) {
    uint32_t w[4];
    V a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      w[u] = wn[u];
      wn[u] = it + 4 + u < P.iters ? __ldg(&P.task[(it + 4 + u) * 32 + lane]) : PAD;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const uint32_t x = w[u] == PAD ? 0u : w[u];
      a[u] = A2[x & 1023u];
      b[u] = B2[(x >> 10) & 1023u];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (w[u] == PAD) return;
      acc.fma(a[u], b[u]);
      if (w[u] >> 31) slots[(w[u] >> 20) & 2047u] += acc.take();
    }
  }
}
template <int NP>
__global__ void __launch_bounds__(32 * PackF<NP>::WARPS) k_m2l_pk(Plan P, int q, int ncells, int so, int order,
                                                                 const int *off_, const int *src, const int *cls,
                                                                 const unsigned char *ord, const float *clsD,
                                                                 const unsigned char *clevel, const float *M,
                                                                 float *L, int mstr, int lstr, int dstr) {
  constexpr int W = PackF<NP>::WARPS;
  __shared__ __align__(16) float sA[W][FMM_NTMAX * NP], sB[W][FMM_NTMAX * NP];
  __shared__ float sS[W][FMM_NTMAX + 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int A = blockIdx.x * W + w;
  if (A >= ncells) return;
  const int moff = fmm_nterms(so - 1), nt = fmm_nterms(q), ms = nt - moff, ls = fmm_nterms(q - so);
  const int la = clevel[A];
  const int k0 = off_[A], k1 = off_[A + 1];
  int cbase = k0 - 32;
  unsigned hits = 0;
  auto next = [&]() -> int {
    while (!hits) {
      cbase += 32;
      if (cbase >= k1) return -1;
      const int kk = cbase + lane;
      hits = __ballot_sync(0xffffffffu, kk < k1 && (!ord || min(max((int)ord[kk], so + 1), order) == q));
    }
    const int b = __ffs(hits) - 1;
    hits &= hits - 1;
    return cbase + b;
  };
  int kc = next();
  if (kc < 0) {
    if (!ord)
      for (int n = lane; n < ls; n += 32) L[(size_t)A * lstr + n] = 0.f;
    return;
  }
  for (int s = lane; s < P.nseg; s += 32) sS[w][s] = 0.f;
  while (kc >= 0) {
    const float *Dp[NP];
    const float *Mp[NP];
    int dl[NP];
    float z[NP];
    int ks[NP];
    ks[0] = kc;
#pragma unroll
    for (int u = 1; u < NP; u++) ks[u] = next();  // -1 once the pairs run out, and after
#pragma unroll
    for (int u = 0; u < NP; u++) {
      const bool have = ks[u] >= 0;
      const int kk = have ? ks[u] : kc;  // a missing pair reads the first one's rows, scaled by zero
      const int B = src[kk];
      Dp[u] = clsD + (size_t)cls[kk] * dstr;
      Mp[u] = M + (size_t)B * mstr;
      dl[u] = la - (int)clevel[B];
      z[u] = have ? 1.f : 0.f;
    }
    __syncwarp();
    for (int i = lane; i < nt; i += 32) {
      float v[NP];
#pragma unroll
      for (int u = 0; u < NP; u++) v[u] = Dp[u][i];
#pragma unroll
      for (int u = 0; u < NP; u++) sA[w][i * NP + u] = v[u];
    }
    for (int j = lane; j < ms; j += 32) {
      const int dg = (int)c_mi[j + moff][3];
      float v[NP];
#pragma unroll
      for (int u = 0; u < NP; u++) v[u] = z[u] * Mp[u][j] * exp2i<float>(dl[u] * dg);
#pragma unroll
      for (int u = 0; u < NP; u++) sB[w][j * NP + u] = v[u];
    }
    __syncwarp();
    engine_run_pk<NP>(P, sA[w], sB[w], sS[w], lane);
    kc = z[NP - 1] != 0.f ? next() : -1;
  }
  __syncwarp();
  for (int n = lane; n < ls; n += 32) {
    const float v = engine_out<float>(P, sS[w], n);
    if (ord) L[(size_t)A * lstr + n] += v;
    else L[(size_t)A * lstr + n] = v;
  }
}
// Two pairs per pass: four measured slower (the 16.5 KB per warp halves the
// warps an SM holds; learned 8e6 step 747 -> 762 ms).
#define M2L_PACK 2

// ---------------------------------------------------------------------------
// L2L for all cells of one level (example/calculate.cpp:219-234)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(32 * FMM_WARPS) k_l2l(Plan P, int lo, int hi, int so, int order,
                                                        const int *parent, const unsigned char *clevel,
                                                        const double *cx, const double *cy, const double *cz,
                                                        const double *cr, T *L, int lstr) {
  __shared__ T sA[FMM_WARPS][FMM_NTMAX], sB[FMM_WARPS][FMM_NTMAX], sS[FMM_WARPS][FMM_NTMAX + 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = lo + blockIdx.x * FMM_WARPS + w;
  if (c >= hi) return;
  const int p = parent[c];
  const int lsize = fmm_nterms(order - so);
  const double inv_s = 1.0 / cr[p];
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = T(0);
  warp_monomials<T>((cx[c] - cx[p]) * inv_s, (cy[c] - cy[p]) * inv_s, (cz[c] - cz[p]) * inv_s, order - so, sA[w],
                    lane);
  for (int j = lane; j < lsize; j += 32) sB[w][j] = L[(size_t)p * lstr + j];
  __syncwarp();
  engine_run<T>(P, sA[w], sB[w], sS[w], lane);
  __syncwarp();
  for (int n = lane; n < lsize; n += 32)
    L[(size_t)c * lstr + n] += engine_out<T>(P, sS[w], n) * exp2i<T>(-((int)c_mi[n][3] + 1));
}

// ---------------------------------------------------------------------------
// L2P, one warp per leaf, one lane per particle (example/calculate.cpp:236-250)
// ---------------------------------------------------------------------------
#define L2P_WARPS 2
template <typename T>
__global__ void __launch_bounds__(32 * L2P_WARPS) k_l2p(const int *leaf_cells, int nleaves, const int *pstart,
                                                        const int *pcount, const unsigned char *clevel,
                                                        const double *cx, const double *cy, const double *cz,
                                                        const double *px, const double *py, const double *pz,
                                                        int so, int order, const double *cr, const T *L,
                                                        double *Ffar, int lstr) {
  __shared__ T sL[L2P_WARPS][FMM_NTMAX];
  __shared__ T tb[L2P_WARPS][3][FMM_PMAX + 1][33];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int leaf = blockIdx.x * L2P_WARPS + w;
  if (leaf >= nleaves) return;
  const int c = leaf_cells[leaf];
  const int pl = order - so, lsize = fmm_nterms(pl);
  const double s = cr[c], inv_s = s > 0 ? 1.0 / s : 0.0;
  for (int j = lane; j < lsize; j += 32) sL[w][j] = s > 0 ? L[(size_t)c * lstr + j] : T(0);
  __syncwarp();
  const int p0 = pstart[c], np = pcount[c];
  for (int base = 0; base < np; base += 32) {
    int i = p0 + base + lane;
    bool ok = base + lane < np;
    if (ok) {
      T ux = (T)((px[i] - cx[c]) * inv_s), uy = (T)((py[i] - cy[c]) * inv_s), uz = (T)((pz[i] - cz[c]) * inv_s);
      T a = 1, b = 1, d = 1;
      tb[w][0][0][lane] = a; tb[w][1][0][lane] = b; tb[w][2][0][lane] = d;
      for (int k = 1; k <= pl; k++) {
        const T rk = rcp_int<T>(k);
        a = a * ux * rk; b = b * uy * rk; d = d * uz * rk;
        tb[w][0][k][lane] = a; tb[w][1][k][lane] = b; tb[w][2][k][lane] = d;
      }
      T phi = 0, ex = 0, ey = 0, ez = 0;
      for (int n = 0; n < lsize; n++) {
        int nx = c_mi[n][0], ny = c_mi[n][1], nz = c_mi[n][2];
        T l = sL[w][n];
        T yz = tb[w][1][ny][lane] * tb[w][2][nz][lane];
        phi += l * tb[w][0][nx][lane] * yz;
        if (nx) ex += l * tb[w][0][nx - 1][lane] * yz;
        if (ny) ey += l * tb[w][0][nx][lane] * tb[w][1][ny - 1][lane] * tb[w][2][nz][lane];
        if (nz) ez += l * tb[w][0][nx][lane] * tb[w][1][ny][lane] * tb[w][2][nz - 1][lane];
      }
      double is2 = inv_s * inv_s;
      Ffar[4 * (size_t)i] = (double)phi * inv_s;
      Ffar[4 * (size_t)i + 1] = -(double)ex * is2;
      Ffar[4 * (size_t)i + 2] = -(double)ey * is2;
      Ffar[4 * (size_t)i + 3] = -(double)ez * is2;
    }
  }
}

// P2P and the FP32 staging live in p2p.cu
int fmm_p2p_launch(DevTree *t, bool mixed, const double *S, cudaStream_t st, bool narrow = false);
int fmm_stage_particles(DevTree *t, const double *S, cudaStream_t st);

// F[caller index][outsize] = near + far, in FP64
__global__ void k_finalize(const double *Fnear, const double *Ffar, const uint32_t *perm, long N, int potential,
                           int field, double *F) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  int outsize = (potential ? 1 : 0) + (field ? 3 : 0);
  size_t o = (size_t)perm[i] * outsize;
  const double *a = Fnear + 4 * (size_t)i, *b = Ffar + 4 * (size_t)i;
  int k = 0;
  if (potential) F[o + k++] = a[0] + b[0];
  if (field) {
    F[o + k] = a[1] + b[1];
    F[o + k + 1] = a[2] + b[2];
    F[o + k + 2] = a[3] + b[3];
  }
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
// phase boundary i; while a graph is being recorded the record becomes a node
// of the graph, so the replayed pass keeps its phase times
static int rec(DevTree *t, int i, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FMM_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusActive)
    FMM_CUDA_TRY(cudaEventRecordWithFlags(t->ev[6 + i], st, cudaEventRecordExternal));
  else
    FMM_CUDA_TRY(cudaEventRecord(t->ev[6 + i], st));
  return FMM_OK;
}

int fmm_mark_kernel(DevTree *t, int which, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FMM_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusActive)
    FMM_CUDA_TRY(cudaEventRecordWithFlags(t->ev_mk[which], st, cudaEventRecordExternal));
  else
    FMM_CUDA_TRY(cudaEventRecord(t->ev_mk[which], st));
  return FMM_OK;
}

template <typename T>
static int m2l_phase(DevTree *t, const PlanSet *ps, const T *M, T *L, bool mixed, int impl, int mstr, int lstr,
                     int dstr, cudaStream_t st);

template <typename T>
static int m2l_p2p(DevTree *t, const PlanSet *ps, const double *S, const T *M, T *L, bool mixed, int impl, int mstr,
                   int lstr, int dstr, cudaStream_t st);

template <typename T>
static int run_pass(DevTree *t, const PlanSet *ps, const double *S, T *M, T *L, bool mixed, int impl, int mstr,
                    int lstr, int dstr, cudaStream_t st) {
  const int p = t->order, so = t->so;
  const double *cr = t->cr.p;  // per-cell half-widths
  const int nl = t->nleaves, nc = t->ncells;
  // P2M
  fmm_note_launch(), k_p2m<T><<<fmm_blocks(nl, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
      t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, t->px.p, t->py.p,
      t->pz.p, t->perm.p, S, so, p, cr, M, mstr);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 1, st));
  // M2M, deepest parents first (mixed pass: the eight fixed child-shift
  // operators, shift.cu; FP64: the contraction engine)
  for (int l = t->nlevels - 2; l >= 0; l--) {
    int lo = t->level_off[l], hi = t->level_off[l + 1];
    if (mixed)
      TRY(fmm_m2m_tab(t, lo, hi, (float *)(void *)M, mstr, st));
    else
      fmm_note_launch(), k_m2m<T><<<fmm_blocks(hi - lo, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
          ps->m2m, lo, hi, so, p, t->child_mask.p, t->child_first.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, cr, M,
          mstr);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 2, st));
  // with an order model, P2P runs first: the predicted orders read its near field
  t->p2p_first = t->ord_mode == 2;
  if (t->p2p_first) {
    TRY(fmm_p2p_launch(t, mixed, S, st));
    TRY(rec(t, 3, st));
  }
  if (t->p2p_first) {
    TRY(m2l_phase<T>(t, ps, M, L, mixed, impl, mstr, lstr, dstr, st));
    TRY(rec(t, 4, st));
  } else {
    TRY(m2l_p2p<T>(t, ps, S, M, L, mixed, impl, mstr, lstr, dstr, st));
  }
  // L2L, top-down (as M2M: fixed child-shift operators in the mixed pass)
  for (int l = 1; l < t->nlevels; l++) {
    int lo = t->level_off[l], hi = t->level_off[l + 1];
    if (mixed)
      TRY(fmm_l2l_tab(t, lo, hi, (float *)(void *)L, lstr, st));
    else
      fmm_note_launch(), k_l2l<T><<<fmm_blocks(hi - lo, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
          ps->l2l, lo, hi, so, p, t->parent.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, cr, L, lstr);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 5, st));
  // L2P
  fmm_note_launch(), k_l2p<T><<<fmm_blocks(nl, L2P_WARPS), 32 * L2P_WARPS, 0, st>>>(
      t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, t->px.p, t->py.p,
      t->pz.p, so, p, cr, L, t->Ffar.p, lstr);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 6, st));
  return FMM_OK;
}

// M2L implementation of a pass: per-pair orders when set; else (mixed pass)
// the tuned choice or, by default, tensor cores where the order allows
// (p <= 9, precision "mixed": with source rows boxed from level grids when
// every level is complete, else gathered row by row), else the generated
// CUDA-core kernels where this order has them (register-resident, p <= 8;
// then the target-major kernels of every order up to 12), else the warp
// contraction engine; FP64: the engine.
enum { M2L_TC = 0, M2L_GEN = 1, M2L_ENGINE = 2, M2L_TCG = 3, M2L_CM = 4, M2L_TP = 5 };
static inline bool is_tc(int impl) { return impl == M2L_TC || impl == M2L_TCG; }
bool fmm_m2l_gen_supported(int p, int so) {
  m2l_reg_kernel kg[4];
  int kt[4];
  return m2l_reg_kernels(p, so, kg, kt) > 0;
}
static int m2l_impl(const DevTree *t, int precision) {
  if (precision == 0) return M2L_ENGINE;
  const bool tc_ok = fmm_m2l_tc_supported(t->order, t->so), gen_ok = fmm_m2l_gen_supported(t->order, t->so);
  int impl = t->tune.impl;
  if (impl < 0) impl = precision == 1 ? M2L_TCG : M2L_GEN;
  if (is_tc(impl) && (!tc_ok || t->nclasses > 262144)) impl = M2L_GEN;  // class bitmap of the tile schedule
  if (impl == M2L_CM && (!fmm_m2l_cm_supported(t->order, t->so) || t->nclasses > 262144)) impl = M2L_GEN;
  if (impl == M2L_TP && !fmm_m2l_cm_supported(t->order, t->so)) impl = M2L_GEN;
  if (impl == M2L_GEN && !gen_ok) impl = fmm_m2l_cm_supported(t->order, t->so) ? M2L_TP : M2L_ENGINE;
  return impl;
}

static int side_stream(DevTree *t) {
  if (t->s_hi) return FMM_OK;
  int lo = 0, hi = 0;
  FMM_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  FMM_CUDA_TRY(cudaStreamCreateWithPriority(&t->s_hi, cudaStreamNonBlocking, hi));
  FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_fork, cudaEventDisableTiming));
  FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_join, cudaEventDisableTiming));
  return FMM_OK;
}

// M2L, then P2P (phase records 3 and 4).  With the overlap switch and the
// tensor-core M2L, the M2L runs on a highest-priority side stream -- its
// persistent CTAs take one SM each first -- and the P2P blocks run beside it
// in the registers and shared memory the M2L CTA leaves free (one 4-warp block
// per SM), so the P2P's FP32 work fills issue slots of the latency-bound MMA
// pipeline; record 3 marks the M2L's end, record 4 the join.
template <typename T>
static int m2l_p2p(DevTree *t, const PlanSet *ps, const double *S, const T *M, T *L, bool mixed, int impl, int mstr,
                   int lstr, int dstr, cudaStream_t st) {
  if (!(t->tune.overlap && mixed && is_tc(impl) && t->nm2l > 0)) {
    TRY(m2l_phase<T>(t, ps, M, L, mixed, impl, mstr, lstr, dstr, st));
    TRY(rec(t, 3, st));
    TRY(fmm_p2p_launch(t, mixed, S, st));
    return rec(t, 4, st);
  }
  TRY(side_stream(t));
  FMM_CUDA_TRY(cudaEventRecord(t->ev_fork, st));
  FMM_CUDA_TRY(cudaStreamWaitEvent(t->s_hi, t->ev_fork, 0));
  TRY(m2l_phase<T>(t, ps, M, L, mixed, impl, mstr, lstr, dstr, t->s_hi));
  TRY(rec(t, 3, t->s_hi));
  FMM_CUDA_TRY(cudaEventRecord(t->ev_join, t->s_hi));
  TRY(fmm_p2p_launch(t, mixed, S, st, t->tune.overlap == 2));
  FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_join, 0));
  return rec(t, 4, st);
}

template <typename T>
static int m2l_phase(DevTree *t, const PlanSet *ps, const T *M, T *L, bool mixed, int impl, int mstr, int lstr,
                     int dstr, cudaStream_t st) {
  const int p = t->order, so = t->so, nc = t->ncells;
  t->tc_ran = 0;
  // every M2L but the tensor cores' reads the target lists
  if (t->ord_mode != 0 || !(mixed && (is_tc(impl) || impl == M2L_CM))) TRY(fmm_m2l_csr(t, st));
  // a tuned choice pins the per-pair-order kernels: 2 the engine, 4 class-major, else target-major
  const int timpl = t->tune.impl;
  if (t->ord_mode != 0) {
    // per-pair orders: predicted now from this pass's multipoles, or given
    if (t->ord_mode == 2) TRY(fmm_learned_orders(t, st));
    else if (t->ord_serial != t->build_serial) {
      fmm_set_error_text("per-pair M2L orders were set for an earlier build");
      return FMM_ERR_STATE;
    }
    if constexpr (std::is_same<T, float>::value) {
      // mixed: the generated kernels, each lane truncating at its pair's order
      const int rc = timpl == M2L_ENGINE ? FMM_ERR_STATE
                     : timpl == M2L_CM   ? fmm_m2l_cm(t, M, mstr, L, lstr, t->m2l_ord.p, st)
                                         : fmm_m2l_tp(t, M, mstr, L, lstr, t->m2l_ord.p, st);
      if (rc != FMM_ERR_STATE) return rc;
    }
    FMM_CUDA_TRY(cudaMemsetAsync(L, 0, sizeof(T) * (size_t)nc * lstr, st));
    TRY(fmm_mark_kernel(t, 0, st));
    for (int q = so + 1; q <= p; q++) {
      const PlanSet *pq = fmm_get_plans(q, so);
      if (!pq) return FMM_ERR_CUDA;
      if constexpr (std::is_same<T, float>::value)
        fmm_note_launch(), k_m2l_pk<M2L_PACK><<<fmm_blocks(nc, PackF<M2L_PACK>::WARPS), 32 * PackF<M2L_PACK>::WARPS, 0, st>>>(
            pq->m2l, q, nc, so, p, t->m2l_off.p, t->m2l_src.p, t->m2l_cls.p, t->m2l_ord.p, (const float *)t->cls_Df.p,
            t->clevel.p, M, L, mstr, lstr, dstr);
      else
        fmm_note_launch(), k_m2l_var<T><<<fmm_blocks(nc, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
            pq->m2l, q, nc, so, p, t->m2l_off.p, t->m2l_src.p, t->m2l_cls.p, t->m2l_ord.p,
            mixed ? (const T *)(const void *)t->cls_Df.p : (const T *)(const void *)t->cls_D.p, t->clevel.p, M, L,
            mstr, lstr, dstr);
    }
    TRY(fmm_mark_kernel(t, 1, st));
  } else if (mixed && is_tc(impl)) {
    TRY(fmm_m2l_tc(t, (const float *)(const void *)M, mstr, (float *)(void *)L, lstr, st, impl == M2L_TCG));
  } else if (mixed && impl == M2L_CM) {
    TRY(fmm_m2l_cm(t, (const float *)(const void *)M, mstr, (float *)(void *)L, lstr, nullptr, st));
  } else if (mixed && impl == M2L_TP) {
    TRY(fmm_m2l_tp(t, (const float *)(const void *)M, mstr, (float *)(void *)L, lstr, nullptr, st));
  } else if (mixed && impl == M2L_GEN) {
    m2l_reg_kernel kg[4];
    int kthreads[4];
    const int ng = m2l_reg_kernels(p, so, kg, kthreads);
    TRY(fmm_mark_kernel(t, 0, st));
    for (int g = 0; g < ng; g++)
      fmm_note_launch(), kg[g]<<<(nc + kthreads[g] - 1) / kthreads[g], kthreads[g], 0, st>>>(
          t->nm2l > 0 ? t->m2l_order.p : nullptr, nc, t->m2l_off.p, t->m2l_src.p, t->m2l_cls.p,
          (const float *)t->cls_Df.p, t->clevel.p,
          (const float *)(const void *)M, (float *)(void *)L);
    TRY(fmm_mark_kernel(t, 1, st));
  } else if constexpr (std::is_same<T, float>::value) {
    TRY(fmm_mark_kernel(t, 0, st));
    fmm_note_launch(), k_m2l_pk<M2L_PACK><<<fmm_blocks(nc, PackF<M2L_PACK>::WARPS), 32 * PackF<M2L_PACK>::WARPS, 0, st>>>(
        ps->m2l, p, nc, so, p, t->m2l_off.p, t->m2l_src.p, t->m2l_cls.p, nullptr, (const float *)t->cls_Df.p,
        t->clevel.p, M, L, mstr, lstr, dstr);
    TRY(fmm_mark_kernel(t, 1, st));
  } else {
    TRY(fmm_mark_kernel(t, 0, st));
    fmm_note_launch(), k_m2l<T><<<fmm_blocks(nc, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
        ps->m2l, nc, so, p, t->m2l_off.p, t->m2l_src.p, t->m2l_cls.p,
        mixed ? (const T *)(const void *)t->cls_Df.p : (const T *)(const void *)t->cls_D.p, t->clevel.p, M, L, mstr,
        lstr, dstr);
    TRY(fmm_mark_kernel(t, 1, st));
  }
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

static int evaluate_pass(DevTree *t, const double *S, double *F, int potential, int field, int precision,
                         cudaStream_t st);

void fmm_graph_release(DevTree *t) {
  if (t->gexec) cudaGraphExecDestroy(t->gexec);
  if (t->graph) cudaGraphDestroy(t->graph);
  t->gexec = nullptr;
  t->graph = nullptr;
  t->gkey = DevTree::GraphKey();
}

// Tree::compute_field_fmm (example/tree.cpp:243-271).  With the graph mode on,
// the first pass after a build (or after a change of S, F or the switches)
// runs normally -- reserving every buffer -- and is then recorded as a CUDA
// graph on a private stream; later passes replay that graph on `st`, one launch.
int fmm_tree_evaluate(DevTree *t, const double *S, double *F, int potential, int field, int precision,
                      cudaStream_t st) {
  if (!t || t->ncells == 0) return FMM_ERR_STATE;
  if (!S || !F || (!potential && !field) || precision < 0 || precision > 2) return FMM_ERR_ARG;
  if (!t->graph_on) return evaluate_pass(t, S, F, potential, field, precision, st);
  const DevTree::GraphKey key{S, F, potential, field, precision, t->build_serial};
  const DevTree::GraphKey &k = t->gkey;
  if (t->gexec && k.S == key.S && k.F == key.F && k.potential == key.potential && k.field == key.field &&
      k.precision == key.precision && k.serial == key.serial) {
    FMM_CUDA_TRY(cudaGraphLaunch(t->gexec, st));
    fmm_add_launches(t->glaunches);
    return FMM_OK;
  }
  TRY(evaluate_pass(t, S, F, potential, field, precision, st));
  fmm_graph_release(t);
  if (!t->gstream) FMM_CUDA_TRY(cudaStreamCreateWithFlags(&t->gstream, cudaStreamNonBlocking));
  const long long n0 = fmm_launches();
  FMM_CUDA_TRY(cudaStreamBeginCapture(t->gstream, cudaStreamCaptureModeRelaxed));
  const int rc = evaluate_pass(t, S, F, potential, field, precision, t->gstream);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(t->gstream, &g);
  t->glaunches = fmm_launches() - n0;
  fmm_add_launches(-t->glaunches);  // recorded, not launched
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) {
    fmm_set_cuda_error(ce, "graph capture", __FILE__, __LINE__);
    return FMM_ERR_CUDA;
  }
  t->graph = g;
  FMM_CUDA_TRY(cudaGraphInstantiate(&t->gexec, t->graph, 0));
  t->gkey = key;
  return FMM_OK;
}

static int evaluate_pass(DevTree *t, const double *S, double *F, int potential, int field, int precision,
                         cudaStream_t st) {
  const PlanSet *ps = fmm_get_plans(t->order, t->so);
  if (!ps) return FMM_ERR_CUDA;
  const bool mixed = precision != 0;
  const int impl = m2l_impl(t, precision);
  t->last_prec = mixed ? 1 : 0;
  t->pass_potential = potential != 0;
  if (t->grouping_built != t->tune.grouping) TRY(fmm_m2l_cell_order(t, t->tune.grouping, st));
  const int p = t->order, so = t->so;
  const size_t msize = fmm_nterms(p) - fmm_nterms(so - 1), lsize = fmm_nterms(p - so);
  const size_t nc = t->ncells;
  TRY(fmm_reserve(t->Fnear, 4 * (size_t)t->N));
  TRY(fmm_reserve(t->Ffar, 4 * (size_t)t->N));
  TRY(rec(t, 0, st));
  if (mixed) {
    // FP32 rows padded to 16 bytes for the float4 loads of the M2L kernels
    const int mstr = fmm_stride4((int)msize), lstr = fmm_stride4((int)lsize), dstr = fmm_stride4(fmm_nterms(p));
    TRY(fmm_reserve(t->Mf, nc * mstr));
    TRY(fmm_reserve(t->Lf, nc * lstr));
    TRY(fmm_reserve(t->phi4, t->N)); TRY(fmm_reserve(t->plo4, t->N));
    TRY(fmm_reserve(t->sdip, t->so == 1 ? t->N : 1));
    TRY(fmm_stage_particles(t, S, st));
    TRY(run_pass<float>(t, ps, S, t->Mf.p, t->Lf.p, true, impl, mstr, lstr, dstr, st));
  } else {
    TRY(fmm_reserve(t->M, nc * msize));
    TRY(fmm_reserve(t->L, nc * lsize));
    TRY(run_pass<double>(t, ps, S, t->M.p, t->L.p, false, impl, (int)msize, (int)lsize, fmm_nterms(p), st));
  }
  fmm_note_launch(), k_finalize<<<fmm_blocks(t->N, 256), 256, 0, st>>>(t->Fnear.p, t->Ffar.p, t->perm.p, t->N, potential, field, F);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 7, st));
  return FMM_OK;
}

// ---------------------------------------------------------------------------
// build + evaluate in one call
// ---------------------------------------------------------------------------
// The multipoles need nothing of the interaction lists, so as soon as the
// cells exist a second stream stages the particles and runs P2M and M2M
// (near_start, beside the walk and the class build).  The M2L follows the classes on the
// highest-priority stream -- its persistent CTAs take the SMs first -- and the
// P2P starts beside it on the caller's stream (in the blocks the tuning
// chose), as in the overlapped pass; L2L, L2P and the final sum follow.  Phase
// records follow the streams: "M2L" spans the end of M2M to the end of M2L
// (the class build included), "P2P" the near field's tail after it.
// Stage the particles and run P2M and M2M on the near-field stream as soon as
// the cells exist: the walk that builds the interaction lists runs beside them.
struct NearStart {
  const PlanSet *ps;
  const double *S;
  bool mixed;
  cudaStream_t st;
};
template <typename T>
static int near_start(DevTree *t, void *arg) {
  const NearStart &a = *(const NearStart *)arg;
  const int p = t->order, so = t->so, nl = t->nleaves;
  const double *cr = t->cr.p;
  const size_t msize = fmm_nterms(p) - fmm_nterms(so - 1), lsize = fmm_nterms(p - so), nc = t->ncells;
  const int mstr = a.mixed ? fmm_stride4((int)msize) : (int)msize;
  TRY(fmm_reserve(t->Fnear, 4 * (size_t)t->N));
  TRY(fmm_reserve(t->Ffar, 4 * (size_t)t->N));
  T *M;
  if (a.mixed) {
    TRY(fmm_reserve(t->Mf, nc * mstr));
    TRY(fmm_reserve(t->Lf, nc * fmm_stride4((int)lsize)));
    TRY(fmm_reserve(t->phi4, t->N)); TRY(fmm_reserve(t->plo4, t->N));
    TRY(fmm_reserve(t->sdip, t->so == 1 ? t->N : 1));
    M = (T *)(void *)t->Mf.p;
  } else {
    TRY(fmm_reserve(t->M, nc * msize));
    TRY(fmm_reserve(t->L, nc * lsize));
    M = (T *)(void *)t->M.p;
  }
  cudaStream_t sn = t->s_near;
  FMM_CUDA_TRY(cudaEventRecord(t->ev_fork, a.st));
  FMM_CUDA_TRY(cudaStreamWaitEvent(sn, t->ev_fork, 0));
  TRY(rec(t, 0, sn));
  if (a.mixed) TRY(fmm_stage_particles(t, a.S, sn));
  FMM_CUDA_TRY(cudaEventRecord(t->ev_s, sn));
  fmm_note_launch(), k_p2m<T><<<fmm_blocks(nl, FMM_WARPS), 32 * FMM_WARPS, 0, sn>>>(
      t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, t->px.p, t->py.p,
      t->pz.p, t->perm.p, a.S, so, p, cr, M, mstr);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 1, sn));
  for (int l = t->nlevels - 2; l >= 0; l--) {
    int lo = t->level_off[l], hi = t->level_off[l + 1];
    if (a.mixed)
      TRY(fmm_m2m_tab(t, lo, hi, (float *)(void *)M, mstr, sn));
    else
      fmm_note_launch(), k_m2m<T><<<fmm_blocks(hi - lo, FMM_WARPS), 32 * FMM_WARPS, 0, sn>>>(
          a.ps->m2m, lo, hi, so, p, t->child_mask.p, t->child_first.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, cr,
          M, mstr);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 2, sn));
  FMM_CUDA_TRY(cudaEventRecord(t->ev_m, sn));
  return FMM_OK;
}

template <typename T>
static int fused_pass(DevTree *t, const PlanSet *ps, const double *S, T *M, T *L, bool mixed, int precision,
                      int mstr, int lstr, int dstr, cudaStream_t st) {
  const int p = t->order, so = t->so, nl = t->nleaves;
  const double *cr = t->cr.p;
  FMM_CUDA_TRY(cudaEventRecord(t->ev_l, st));  // the interaction lists are built
  // the classes (the host waits on this stream only), then the M2L
  FMM_CUDA_TRY(cudaStreamWaitEvent(t->s_hi, t->ev_l, 0));
  TRY(fmm_tree_finish_build(t, t->s_hi));
  const int impl = m2l_impl(t, precision);
  t->p2p_first = false;
  FMM_CUDA_TRY(cudaEventRecord(t->ev_c, t->s_hi));
  FMM_CUDA_TRY(cudaStreamWaitEvent(t->s_hi, t->ev_m, 0));
  const bool learned = t->ord_mode == 2;
  if (learned) {  // the orders read the near field: P2P first
    FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_c, 0));
    FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_s, 0));  // the staged particles
    TRY(fmm_p2p_launch(t, mixed, S, st));
    FMM_CUDA_TRY(cudaEventRecord(t->ev_p, st));
    FMM_CUDA_TRY(cudaStreamWaitEvent(t->s_hi, t->ev_p, 0));
  }
  TRY(m2l_phase<T>(t, ps, M, L, mixed, impl, mstr, lstr, dstr, t->s_hi));
  TRY(rec(t, 3, t->s_hi));
  FMM_CUDA_TRY(cudaEventRecord(t->ev_join, t->s_hi));
  if (!learned) {  // launched after the M2L, beside it; behind the tensor-core M2L without the overlap
                   // switch (its CTA leaves room for one P2P block per SM: side by side gains nothing there)
    FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_c, 0));
    FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_s, 0));
    if (!t->tune.overlap && mixed && is_tc(impl)) FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_join, 0));
    TRY(fmm_p2p_launch(t, mixed, S, st, mixed && is_tc(impl) && t->tune.overlap == 2));
  }
  FMM_CUDA_TRY(cudaStreamWaitEvent(st, t->ev_join, 0));
  TRY(rec(t, 4, st));
  for (int l = 1; l < t->nlevels; l++) {
    int lo = t->level_off[l], hi = t->level_off[l + 1];
    if (mixed)
      TRY(fmm_l2l_tab(t, lo, hi, (float *)(void *)L, lstr, st));
    else
      fmm_note_launch(), k_l2l<T><<<fmm_blocks(hi - lo, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
          ps->l2l, lo, hi, so, p, t->parent.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, cr, L, lstr);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 5, st));
  fmm_note_launch(), k_l2p<T><<<fmm_blocks(nl, L2P_WARPS), 32 * L2P_WARPS, 0, st>>>(
      t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, t->px.p, t->py.p,
      t->pz.p, so, p, cr, L, t->Ffar.p, lstr);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 6, st));
  return FMM_OK;
}

int fmm_tree_build_evaluate(DevTree *t, const double *pos, long N, long ncrit, int order, double theta, int so,
                            const long *sys_off, int nsys, const double *S, double *F, int potential, int field,
                            int precision, cudaStream_t st) {
  if (!S || !F || (!potential && !field) || precision < 0 || precision > 2) return FMM_ERR_ARG;
  fmm_graph_release(t);  // a recorded pass belongs to the previous build
  TRY(side_stream(t));
  if (!t->s_near) {
    // the multipoles are on the M2L's critical path: highest priority too
    int lo = 0, hi = 0;
    FMM_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    FMM_CUDA_TRY(cudaStreamCreateWithPriority(&t->s_near, cudaStreamNonBlocking, hi));
    FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_m, cudaEventDisableTiming));
    FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_c, cudaEventDisableTiming));
    FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_p, cudaEventDisableTiming));
    FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_s, cudaEventDisableTiming));
    FMM_CUDA_TRY(cudaEventCreateWithFlags(&t->ev_l, cudaEventDisableTiming));
  }
  if (so < 0 || so > 2 || order < so + 1 || order > FMM_PMAX) return FMM_ERR_ARG;
  const PlanSet *ps = fmm_get_plans(order, so);
  if (!ps) return FMM_ERR_CUDA;
  const bool mixed = precision != 0;
  // the tree, with the multipoles started beside its walk
  NearStart ns{ps, S, mixed, st};
  int rc = fmm_tree_build(t, pos, N, ncrit, order, theta, so, st, sys_off, nsys, true,
                          mixed ? near_start<float> : near_start<double>, &ns);
  if (rc) {
    if (t->s_near) cudaStreamSynchronize(t->s_near);
    return rc;
  }
  t->last_prec = mixed ? 1 : 0;
  t->pass_potential = potential != 0;
  const int p = t->order;
  const size_t msize = fmm_nterms(p) - fmm_nterms(so - 1), lsize = fmm_nterms(p - so);
  if (mixed) {
    const int mstr = fmm_stride4((int)msize), lstr = fmm_stride4((int)lsize), dstr = fmm_stride4(fmm_nterms(p));
    rc = fused_pass<float>(t, ps, S, t->Mf.p, t->Lf.p, true, precision, mstr, lstr, dstr, st);
  } else {
    rc = fused_pass<double>(t, ps, S, t->M.p, t->L.p, false, precision, (int)msize, (int)lsize, fmm_nterms(p), st);
  }
  if (rc == FMM_OK && t->eflags) {  // the build's own error, after the near-field stream is done
    FMM_CUDA_TRY(cudaStreamSynchronize(t->s_near));
    return (t->eflags & FMM_EFLAG_DEPTH) ? FMM_ERR_DEPTH : FMM_ERR_RANGE;
  }
  if (rc) {
    cudaStreamSynchronize(t->s_near);
    return rc;
  }
  fmm_note_launch(), k_finalize<<<fmm_blocks(t->N, 256), 256, 0, st>>>(t->Fnear.p, t->Ffar.p, t->perm.p, t->N,
                                                                        potential, field, F);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 7, st));
  return FMM_OK;
}

// The M2L and P2P phases alone on the multipoles and staged particles of the
// last pass (same precision class): the autotuner's timed unit.
int fmm_m2l_p2p_only(DevTree *t, const double *S, int precision, cudaStream_t st) {
  if (t->last_prec < 0 || (precision != 0) != (t->last_prec != 0) || t->ord_mode != 0) return FMM_ERR_STATE;
  const PlanSet *ps = fmm_get_plans(t->order, t->so);
  if (!ps) return FMM_ERR_CUDA;
  if (t->grouping_built != t->tune.grouping) TRY(fmm_m2l_cell_order(t, t->tune.grouping, st));
  const int p = t->order, so = t->so;
  const int msize = fmm_nterms(p) - fmm_nterms(so - 1), lsize = fmm_nterms(p - so);
  const int impl = m2l_impl(t, precision);
  if (precision != 0)
    return m2l_p2p<float>(t, ps, S, t->Mf.p, t->Lf.p, true, impl, fmm_stride4(msize), fmm_stride4(lsize),
                          fmm_stride4(fmm_nterms(p)), st);
  return m2l_p2p<double>(t, ps, S, t->M.p, t->L.p, false, impl, msize, lsize, fmm_nterms(p), st);
}

// ---------------------------------------------------------------------------
// Barnes-Hut (Tree::compute_field_bh, example/tree.cpp:273-293)
// ---------------------------------------------------------------------------
// One thread per particle (sorted order), FP64: evaluate_M2P_and_P2P
// (example/calculate.cpp:266-314) from the particle's root with an explicit
// stack.  A child c of an open cell is opened when r_c > theta |x_i - c_c|,
// else its multipole acts through M2P -- the potential of fmmgen's M2P
// (fmmgen/generator.py:174-206) and its exact gradient as the field,
//   phi = (1/s) sum_m D_m(y) M~_m,  E = -(1/s^2) sum_m D_(m+e)(y) M~_m,  y = (x_i - c_c) / s,
// in the scaled multipoles M~ = M / s^|m| -- and a leaf's particles through
// P2P.  NTQ holds the derivatives to order p + 1.
#define BH_THREADS 128
#define BH_STACK (8 * 22)
template <int NTQ>
__global__ void __launch_bounds__(BH_THREADS) k_bh64(long N, int nsys, const long *sys_off, const double *px,
                                                     const double *py, const double *pz, const uint32_t *perm,
                                                     const double *S, int so, int p, double theta,
                                                     const double *cx, const double *cy, const double *cz,
                                                     const double *cr, const int *child_first,
                                                     const unsigned char *child_mask, const int *pstart,
                                                     const int *pcount, const double *M, int msize, int potential,
                                                     int field, double *F, uint32_t *eflag) {
  const long i = blockIdx.x * (long)BH_THREADS + threadIdx.x;
  if (i >= N) return;
  int root = 0;
  if (nsys > 1) {  // the system holding sorted particle i: sys_off[s] <= i < sys_off[s + 1]
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sys_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    root = lo;
  }
  const double xi = px[i], yi = py[i], zi = pz[i];
  const int moff = fmm_nterms(so - 1);
  double phi = 0, ex = 0, ey = 0, ez = 0;
  double D[NTQ];
  int stack[BH_STACK];
  int sp = 0;
  stack[sp++] = root;
  while (sp > 0) {
    const int c0 = stack[--sp];
    const unsigned mask = child_mask[c0];
    if (mask) {
      int c = child_first[c0];
      for (int o = 0; o < 8; o++) {
        if (!((mask >> o) & 1u)) continue;
        const double dx = xi - cx[c], dy = yi - cy[c], dz = zi - cz[c];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double s = cr[c];
        if (s > theta * r) {
          if (sp < BH_STACK) stack[sp++] = c;
          else atomicOr(eflag, 1u);  // deeper than the stack: reported, not walked
        } else {
          const double is = 1.0 / s;
          thread_derivs(dx * is, dy * is, dz * is, p + 1, D);
          const double *Mc = M + (size_t)c * msize;
          double v = 0, gx = 0, gy = 0, gz = 0;
          int j = moff;  // multipole terms in the degree-major layout
          for (int d = so; d <= p; d++)
            for (int mx = d; mx >= 0; mx--)
              for (int my = d - mx; my >= 0; my--, j++) {
                const int mz = d - mx - my;
                const double w = Mc[j - moff];
                v += D[j] * w;
                gx += D[fmm_idx3(mx + 1, my, mz)] * w;
                gy += D[fmm_idx3(mx, my + 1, mz)] * w;
                gz += D[fmm_idx3(mx, my, mz + 1)] * w;
              }
          phi += v * is;
          const double is2 = is * is;
          ex -= gx * is2;
          ey -= gy * is2;
          ez -= gz * is2;
        }
        c++;
      }
    } else {
      const int j0 = pstart[c0], j1 = j0 + pcount[c0];
      for (int j = j0; j < j1; j++) {
        if (j == i) continue;
        const double dx = xi - px[j], dy = yi - py[j], dz = zi - pz[j];
        const uint32_t oj = perm[j];
        if (so == 2) {
          quadrupole_p2p<double>(dx, dy, dz, S + 6 * (size_t)oj, phi, ex, ey, ez);
          continue;
        }
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double rinv = 1.0 / sqrt(r2), r3 = rinv * rinv * rinv;
        if (so == 0) {
          const double q = S[oj];
          phi += q * rinv;
          ex += q * r3 * dx;
          ey += q * r3 * dy;
          ez += q * r3 * dz;
        } else {
          const double sx = S[3 * (size_t)oj], sy = S[3 * (size_t)oj + 1], sz = S[3 * (size_t)oj + 2];
          const double sr = sx * dx + sy * dy + sz * dz;
          const double r5 = 3.0 * sr * r3 * rinv * rinv;
          phi -= sr * r3;
          ex += sx * r3 - r5 * dx;
          ey += sy * r3 - r5 * dy;
          ez += sz * r3 - r5 * dz;
        }
      }
    }
  }
  const int outsize = (potential ? 1 : 0) + (field ? 3 : 0);
  double *f = F + (size_t)perm[i] * outsize;
  int k = 0;
  if (potential) f[k++] = phi;
  if (field) {
    f[k] = ex;
    f[k + 1] = ey;
    f[k + 2] = ez;
  }
}

// Tree::compute_field_bh (example/tree.cpp:273-293): FP64 P2M and M2M, then
// the walk of every particle.
int fmm_tree_evaluate_bh(DevTree *t, const double *S, double *F, int potential, int field, cudaStream_t st) {
  if (!t || t->ncells == 0) return FMM_ERR_STATE;
  if (!S || !F || (!potential && !field)) return FMM_ERR_ARG;
  const PlanSet *ps = fmm_get_plans(t->order, t->so);
  if (!ps) return FMM_ERR_CUDA;
  const int p = t->order, so = t->so;
  const int msize = fmm_nterms(p) - fmm_nterms(so - 1);
  const double *cr = t->cr.p;
  TRY(fmm_reserve(t->M, (size_t)t->ncells * msize));
  TRY(fmm_reserve(t->d_eflags, 1));
  FMM_CUDA_TRY(cudaMemsetAsync(t->d_eflags.p, 0, sizeof(uint32_t), st));
  fmm_note_launch(), k_p2m<double><<<fmm_blocks(t->nleaves, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
      t->leaf_cells.p, t->nleaves, t->pstart.p, t->pcount.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, t->px.p,
      t->py.p, t->pz.p, t->perm.p, S, so, p, cr, t->M.p, msize);
  for (int l = t->nlevels - 2; l >= 0; l--) {
    int lo = t->level_off[l], hi = t->level_off[l + 1];
    fmm_note_launch(), k_m2m<double><<<fmm_blocks(hi - lo, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(
        ps->m2m, lo, hi, so, p, t->child_mask.p, t->child_first.p, t->clevel.p, t->cx.p, t->cy.p, t->cz.p, cr,
        t->M.p, msize);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  const unsigned nb = (unsigned)((t->N + BH_THREADS - 1) / BH_THREADS);
#define BH_ARGS                                                                                              \
  t->N, t->nsys, t->nsys > 1 ? t->sys_off.p : nullptr, t->px.p, t->py.p, t->pz.p, t->perm.p, S, so, p,       \
      t->theta, t->cx.p, t->cy.p, t->cz.p, cr, t->child_first.p, t->child_mask.p, t->pstart.p, t->pcount.p, \
      t->M.p, msize, potential, field, F, t->d_eflags.p
  const int q = p + 1;
  if (q <= 4) fmm_note_launch(), k_bh64<35><<<nb, BH_THREADS, 0, st>>>(BH_ARGS);
  else if (q <= 6) fmm_note_launch(), k_bh64<84><<<nb, BH_THREADS, 0, st>>>(BH_ARGS);
  else if (q <= 9) fmm_note_launch(), k_bh64<220><<<nb, BH_THREADS, 0, st>>>(BH_ARGS);
  else fmm_note_launch(), k_bh64<560><<<nb, BH_THREADS, 0, st>>>(BH_ARGS);
#undef BH_ARGS
  FMM_CUDA_TRY(cudaGetLastError());
  uint32_t fl = 0;
  FMM_CUDA_TRY(cudaMemcpyAsync(&fl, t->d_eflags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaStreamSynchronize(st));
  if (fl) {
    fmm_set_error_text("Barnes-Hut walk deeper than its stack");
    return FMM_ERR_DEPTH;
  }
  t->last_prec = 0;  // the FP64 multipoles of this pass are in t->M
  return FMM_OK;
}

// Per-phase times of the last evaluate (needs the stream to have completed).
void fmm_eval_times(DevTree *t) {
  float ms;
  for (int i = 0; i < 8; i++) {
    const int a = i < 7 ? 6 + i : 6, b = i < 7 ? 7 + i : 13;
    if (cudaEventElapsedTime(&ms, t->ev[a], t->ev[b]) != cudaSuccess) {
      ms = -1.f;          // not recorded
      cudaGetLastError();  // and leave no error behind for the next call
    }
    t->phase_ms[i] = ms;
  }
  if (t->p2p_first) std::swap(t->phase_ms[2], t->phase_ms[3]);  // the pass ran P2P, then M2L
  for (int k = 0; k < 2; k++) {
    if (cudaEventElapsedTime(&ms, t->ev_mk[2 * k], t->ev_mk[2 * k + 1]) != cudaSuccess) {
      ms = -1.f;
      cudaGetLastError();
    }
    t->kernel_ms[k] = ms;
  }
}

// ---------------------------------------------------------------------------
// direct O(N^2) sum in FP64 (example/calculate.cpp:252-264)
// ---------------------------------------------------------------------------
#define DIR_BS 128
__global__ void __launch_bounds__(DIR_BS) k_direct(const double *pos, const double *S, long N, const long *targets,
                                                   long nt, int so, int potential, int field, double *F) {
  __shared__ double sx[DIR_BS], sy[DIR_BS], sz[DIR_BS], sq[DIR_BS][6];
  long t = blockIdx.x * (long)DIR_BS + threadIdx.x;
  long i = t < nt ? (targets ? targets[t] : t) : -1;
  double xi = 0, yi = 0, zi = 0;
  if (i >= 0) { xi = pos[3 * i]; yi = pos[3 * i + 1]; zi = pos[3 * i + 2]; }
  double phi = 0, ex = 0, ey = 0, ez = 0;
  for (long b = 0; b < N; b += DIR_BS) {
    __syncthreads();
    long j = b + threadIdx.x;
    if (j < N) {
      sx[threadIdx.x] = pos[3 * j]; sy[threadIdx.x] = pos[3 * j + 1]; sz[threadIdx.x] = pos[3 * j + 2];
      if (so == 0) sq[threadIdx.x][0] = S[j];
      else if (so == 1) { sq[threadIdx.x][0] = S[3 * j]; sq[threadIdx.x][1] = S[3 * j + 1]; sq[threadIdx.x][2] = S[3 * j + 2]; }
      else for (int k = 0; k < 6; k++) sq[threadIdx.x][k] = S[6 * j + k];
    }
    __syncthreads();
    int cnt = (int)min((long)DIR_BS, N - b);
    if (i < 0) continue;
    for (int jj = 0; jj < cnt; jj++) {
      if (b + jj == i) continue;
      double dx = xi - sx[jj], dy = yi - sy[jj], dz = zi - sz[jj];
      if (so == 2) {
        quadrupole_p2p<double>(dx, dy, dz, sq[jj], phi, ex, ey, ez);
        continue;
      }
      double R = sqrt(dx * dx + dy * dy + dz * dz);
      double rinv = 1.0 / R;
      double r3 = rinv * rinv * rinv;
      if (so == 0) {
        double q = sq[jj][0];
        phi += q * rinv;
        ex += q * dx * r3; ey += q * dy * r3; ez += q * dz * r3;
      } else {
        double a = sq[jj][0], bb = sq[jj][1], c = sq[jj][2];
        double sr = a * dx + bb * dy + c * dz;
        double r5 = r3 * rinv * rinv;
        phi -= sr * r3;
        ex += a * r3 - 3.0 * sr * dx * r5; ey += bb * r3 - 3.0 * sr * dy * r5; ez += c * r3 - 3.0 * sr * dz * r5;
      }
    }
  }
  if (i >= 0) {
    int outsize = (potential ? 1 : 0) + (field ? 3 : 0);
    size_t o = (size_t)t * outsize;
    int k = 0;
    if (potential) F[o + k++] = phi;
    if (field) { F[o + k] = ex; F[o + k + 1] = ey; F[o + k + 2] = ez; }
  }
}

int fmm_direct(const double *pos, const double *S, long N, const long *targets, long ntargets, int so,
               int potential, int field, double *F, cudaStream_t st) {
  if (!pos || !S || !F || N < 1 || (!potential && !field) || so < 0 || so > 2) return FMM_ERR_ARG;
  long nt = targets ? ntargets : N;
  if (nt < 1) return FMM_OK;
  fmm_note_launch(), k_direct<<<fmm_blocks(nt, DIR_BS), DIR_BS, 0, st>>>(pos, S, N, targets, nt, so, potential, field, F);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
