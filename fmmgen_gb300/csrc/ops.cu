// ops.cu -- batched device versions of fmmgen's generated operators.
//
// Each entry applies one operator to n independent (displacement, input,
// output) triples with the generated code's "+=" semantics and unscaled
// coefficients, in FP64 (or FP32 through the _f32 entries).  They replace n calls of P2M_p / M2M_p / M2L_p /
// L2L_p / L2P_p / P2P from fmmgen/writer.py:142-264 (signatures
// fmmgen/printers.py:296-313), one warp per application.
#include "internal.h"
#include "deriv.cuh"

template <typename T>
__device__ __forceinline__ void engine_run_op(const Plan &P, const T *A, const T *B, T *slots, int lane) {
  T acc = T(0);
  for (int it = 0; it < P.iters; ++it) {
    uint32_t w = __ldg(&P.task[it * 32 + lane]);
    if (w == 0xffffffffu) break;
    acc += A[w & 1023u] * B[(w >> 10) & 1023u];
    if (w >> 31) {
      slots[(w >> 20) & 2047u] += acc;
      acc = T(0);
    }
  }
}
template <typename T> __device__ __forceinline__ T engine_out_op(const Plan &P, const T *slots, int n) {
  T s = 0;
  for (int k = __ldg(&P.out_seg[n]); k < __ldg(&P.out_seg[n + 1]); k++) s += slots[k];
  return s;
}

// mon[idx(k)] = x^k / k!, |k| <= pmax
template <typename T>
__device__ __forceinline__ void op_monomials(T vx, T vy, T vz, int pmax, T *mon, int lane) {
  int cnt = fmm_nterms(pmax);
  for (int i = lane; i < cnt; i += 32) {
    int kx = c_mi[i][0], ky = c_mi[i][1], kz = c_mi[i][2];
    T a = 1, b = 1, d = 1;
    for (int q = 1; q <= kx; q++) a = a * vx / T(q);
    for (int q = 1; q <= ky; q++) b = b * vy / T(q);
    for (int q = 1; q <= kz; q++) d = d * vz / T(q);
    mon[i] = a * b * d;
  }
}

#define OPW 4

// P2M_p: M[n] += (-1)^|n| q x^n/n!  (fmmgen/expansions.py:22-39)
template <typename T>
__global__ void k_op_p2m(int n, const T *d, const T *q, T *M, int order, int so) {
  __shared__ T mon[OPW][FMM_NTMAX];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  op_monomials(-d[3 * i], -d[3 * i + 1], -d[3 * i + 2], order, mon[w], lane);
  __syncwarp();
  int off = fmm_nterms(so - 1), ms = fmm_nterms(order) - off;
  for (int j = lane; j < ms; j += 32) M[(size_t)i * ms + j] += q[i] * mon[w][j + off];
}

// M2M_p (fmmgen/expansions.py:42-78) and L2L_p (fmmgen/expansions.py:175-194)
template <typename T>
__global__ void k_op_shift(Plan P, int n, const T *d, const T *in, T *out, int order, int so,
                           int insize, int outsize, int pmax) {
  __shared__ T sA[OPW][FMM_NTMAX], sB[OPW][FMM_NTMAX], sS[OPW][FMM_NTMAX + 32];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  op_monomials(d[3 * i], d[3 * i + 1], d[3 * i + 2], pmax, sA[w], lane);
  for (int j = lane; j < insize; j += 32) sB[w][j] = in[(size_t)i * insize + j];
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = 0;
  __syncwarp();
  engine_run_op<T>(P, sA[w], sB[w], sS[w], lane);
  __syncwarp();
  for (int j = lane; j < outsize; j += 32) out[(size_t)i * outsize + j] += engine_out_op(P, sS[w], j);
}

// M2L_p (fmmgen/expansions.py:144-172): derivatives at d, then the contraction
template <typename T>
__global__ void k_op_m2l(Plan P, int n, const T *d, const T *M, T *L, int order, int so) {
  // sT is the recurrence's scratch, then holds the source multipole
  __shared__ T sD[OPW][FMM_NTMAX], sT[OPW][FMM_NTMAX], sS[OPW][FMM_NTMAX + 32];
  __shared__ T sb[OPW][FMM_PMAX + 1];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  warp_derivs<T>(d[3 * i], d[3 * i + 1], d[3 * i + 2], order, sD[w], sT[w], sb[w]);
  T *sB = sT[w];
  int ms = fmm_nterms(order) - fmm_nterms(so - 1), ls = fmm_nterms(order - so);
  for (int j = lane; j < ms; j += 32) sB[j] = M[(size_t)i * ms + j];
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = 0;
  __syncwarp();
  engine_run_op<T>(P, sD[w], sB, sS[w], lane);
  __syncwarp();
  for (int j = lane; j < ls; j += 32) L[(size_t)i * ls + j] += engine_out_op(P, sS[w], j);
}

// L2P_p (fmmgen/expansions.py:197-207)
template <typename T>
__global__ void k_op_l2p(int n, const T *d, const T *L, T *F, int order, int so, int potential,
                         int field) {
  __shared__ T mon[OPW][FMM_NTMAX];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  int pl = order - so, ls = fmm_nterms(pl);
  op_monomials(d[3 * i], d[3 * i + 1], d[3 * i + 2], pl, mon[w], lane);
  __syncwarp();
  T phi = 0, ex = 0, ey = 0, ez = 0;
  const T *Li = L + (size_t)i * ls;
  for (int j = lane; j < ls; j += 32) {
    int nx = c_mi[j][0], ny = c_mi[j][1], nz = c_mi[j][2];
    T l = Li[j];
    phi += l * mon[w][j];
    if (nx) ex -= l * mon[w][fmm_idx3(nx - 1, ny, nz)];
    if (ny) ey -= l * mon[w][fmm_idx3(nx, ny - 1, nz)];
    if (nz) ez -= l * mon[w][fmm_idx3(nx, ny, nz - 1)];
  }
  for (int o = 16; o; o >>= 1) {
    phi += __shfl_xor_sync(0xffffffffu, phi, o);
    ex += __shfl_xor_sync(0xffffffffu, ex, o);
    ey += __shfl_xor_sync(0xffffffffu, ey, o);
    ez += __shfl_xor_sync(0xffffffffu, ez, o);
  }
  if (lane == 0) {
    int os = (potential ? 1 : 0) + (field ? 3 : 0);
    T *Fi = F + (size_t)i * os;
    int k = 0;
    if (potential) Fi[k++] += phi;
    if (field) { Fi[k] += ex; Fi[k + 1] += ey; Fi[k + 2] += ez; }
  }
}

// P2P (Coulomb form of example/operators.cpp:54-66; dipole and quadrupole
// fields restated as the gradients of the generated potentials)
template <typename T>
__global__ void k_op_p2p(int n, const T *d, const T *S, T *F, int so, int potential, int field) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T x = d[3 * i], y = d[3 * i + 1], z = d[3 * i + 2];
  T R = sqrt(x * x + y * y + z * z);
  T phi = 0, ex = 0, ey = 0, ez = 0;
  if (so == 2) {
    quadrupole_p2p<T>(x, y, z, S + 6 * (size_t)i, phi, ex, ey, ez);
  } else if (so == 0) {
    T q = S[i];
    T r3 = T(1) / (R * R * R);
    phi = q / R;
    ex = q * x * r3; ey = q * y * r3; ez = q * z * r3;
  } else {
    const T *s = S + 3 * (size_t)i;
    T rinv = T(1) / R, r3 = rinv * rinv * rinv, r5 = r3 * rinv * rinv;
    T sr = s[0] * x + s[1] * y + s[2] * z;
    phi = -sr * r3;
    ex = s[0] * r3 - T(3) * sr * x * r5; ey = s[1] * r3 - T(3) * sr * y * r5; ez = s[2] * r3 - T(3) * sr * z * r5;
  }
  int os = (potential ? 1 : 0) + (field ? 3 : 0);
  T *Fi = F + (size_t)i * os;
  int k = 0;
  if (potential) Fi[k++] += phi;
  if (field) { Fi[k] += ex; Fi[k + 1] += ey; Fi[k + 2] += ez; }
}

// op: 0 P2M, 1 M2M, 2 M2L, 3 L2L, 4 L2P, 5 P2P
// M2P_p (fmmgen/generator.py:174-206), one thread per application: the
// potential V = sum_m D_m(d) M_m of fmmgen's M2P and its exact gradient
// E = -sum_m D_(m+e)(d) M_m (the generated field is not that gradient);
// d = particle - cell.  NTQ holds the derivatives to order + 1.
template <typename T, int NTQ>
__global__ void k_op_m2p(int n, const T *d, const T *M, T *F, int order, int so, int potential,
                         int field) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T D[NTQ];
  thread_derivs(d[3 * i], d[3 * i + 1], d[3 * i + 2], order + 1, D);
  const int moff = fmm_nterms(so - 1), ms = fmm_nterms(order) - moff;
  const T *Mi = M + (size_t)i * ms;
  T v = 0, gx = 0, gy = 0, gz = 0;
  int j = moff;
  for (int dg = so; dg <= order; dg++)
    for (int mx = dg; mx >= 0; mx--)
      for (int my = dg - mx; my >= 0; my--, j++) {
        const int mz = dg - mx - my;
        const T w = Mi[j - moff];
        v += D[j] * w;
        gx += D[fmm_idx3(mx + 1, my, mz)] * w;
        gy += D[fmm_idx3(mx, my + 1, mz)] * w;
        gz += D[fmm_idx3(mx, my, mz + 1)] * w;
      }
  const int os = (potential ? 1 : 0) + (field ? 3 : 0);
  T *Fi = F + (size_t)i * os;
  int k = 0;
  if (potential) Fi[k++] += v;
  if (field) {
    Fi[k] -= gx;
    Fi[k + 1] -= gy;
    Fi[k + 2] -= gz;
  }
}

template <typename T>
static int op_batch(int op, int n, const T *d, const T *in, T *out, int order, int so, int potential, int field,
                    cudaStream_t st) {
  if (n < 0 || so < 0 || so > 2 || !d || !in || !out) return FMM_ERR_ARG;
  if (op != 5 && (order < 0 || order > FMM_PMAX || order < so)) return FMM_ERR_ARG;
  if ((op == 4 || op == 5 || op == 6) && !potential && !field) return FMM_ERR_ARG;
  if (n == 0) return FMM_OK;
  unsigned nb = fmm_blocks(n, OPW);
  int ms = fmm_nterms(order) - fmm_nterms(so - 1), ls = fmm_nterms(order - so);
  const PlanSet *ps = nullptr;
  if (op >= 1 && op <= 3) {
    ps = fmm_get_plans(order, so);
    if (!ps) return FMM_ERR_CUDA;
  }
  switch (op) {
    case 0: fmm_note_launch(), k_op_p2m<T><<<nb, 32 * OPW, 0, st>>>(n, d, in, out, order, so); break;
    case 1: fmm_note_launch(), k_op_shift<T><<<nb, 32 * OPW, 0, st>>>(ps->m2m, n, d, in, out, order, so, ms, ms, order - so); break;
    case 2: fmm_note_launch(), k_op_m2l<T><<<nb, 32 * OPW, 0, st>>>(ps->m2l, n, d, in, out, order, so); break;
    case 3: fmm_note_launch(), k_op_shift<T><<<nb, 32 * OPW, 0, st>>>(ps->l2l, n, d, in, out, order, so, ls, ls, order - so); break;
    case 4: fmm_note_launch(), k_op_l2p<T><<<nb, 32 * OPW, 0, st>>>(n, d, in, out, order, so, potential, field); break;
    case 5: fmm_note_launch(), k_op_p2p<T><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, so, potential, field); break;
    case 6:
      if (order + 1 <= 6) fmm_note_launch(), k_op_m2p<T, 84><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, order, so, potential, field);
      else if (order + 1 <= 9) fmm_note_launch(), k_op_m2p<T, 220><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, order, so, potential, field);
      else fmm_note_launch(), k_op_m2p<T, 560><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, order, so, potential, field);
      break;
    default: return FMM_ERR_ARG;
  }
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

int fmm_op_batch(int op, int n, const double *d, const double *in, double *out, int order, int so, int potential,
                 int field, cudaStream_t st) {
  return op_batch<double>(op, n, d, in, out, order, so, potential, field, st);
}

// The same operators in FP32 (the generator's precision="float" variant,
// fmmgen/writer.py:105): float buffers, float arithmetic throughout.
int fmm_op_batch_f32(int op, int n, const float *d, const float *in, float *out, int order, int so, int potential,
                     int field, cudaStream_t st) {
  return op_batch<float>(op, n, d, in, out, order, so, potential, field, st);
}
