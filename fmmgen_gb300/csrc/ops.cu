// ops.cu -- batched device versions of fmmgen's generated operators.
//
// Each entry applies one operator to n independent (displacement, input,
// output) triples with the generated code's "+=" semantics and unscaled
// coefficients, in FP64.  They replace n calls of P2M_p / M2M_p / M2L_p /
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
__device__ __forceinline__ double engine_out_op(const Plan &P, const double *slots, int n) {
  double s = 0;
  for (int k = __ldg(&P.out_seg[n]); k < __ldg(&P.out_seg[n + 1]); k++) s += slots[k];
  return s;
}

// mon[idx(k)] = x^k / k!, |k| <= pmax
__device__ __forceinline__ void op_monomials(double vx, double vy, double vz, int pmax, double *mon, int lane) {
  int cnt = fmm_nterms(pmax);
  for (int i = lane; i < cnt; i += 32) {
    int kx = c_mi[i][0], ky = c_mi[i][1], kz = c_mi[i][2];
    double a = 1, b = 1, d = 1;
    for (int q = 1; q <= kx; q++) a = a * vx / q;
    for (int q = 1; q <= ky; q++) b = b * vy / q;
    for (int q = 1; q <= kz; q++) d = d * vz / q;
    mon[i] = a * b * d;
  }
}

#define OPW 4

// P2M_p: M[n] += (-1)^|n| q x^n/n!  (fmmgen/expansions.py:22-39)
__global__ void k_op_p2m(int n, const double *d, const double *q, double *M, int order, int so) {
  __shared__ double mon[OPW][FMM_NTMAX];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  op_monomials(-d[3 * i], -d[3 * i + 1], -d[3 * i + 2], order, mon[w], lane);
  __syncwarp();
  int off = fmm_nterms(so - 1), ms = fmm_nterms(order) - off;
  for (int j = lane; j < ms; j += 32) M[(size_t)i * ms + j] += q[i] * mon[w][j + off];
}

// M2M_p (fmmgen/expansions.py:42-78) and L2L_p (fmmgen/expansions.py:175-194)
__global__ void k_op_shift(Plan P, int n, const double *d, const double *in, double *out, int order, int so,
                           int insize, int outsize, int pmax) {
  __shared__ double sA[OPW][FMM_NTMAX], sB[OPW][FMM_NTMAX], sS[OPW][FMM_NTMAX + 32];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  op_monomials(d[3 * i], d[3 * i + 1], d[3 * i + 2], pmax, sA[w], lane);
  for (int j = lane; j < insize; j += 32) sB[w][j] = in[(size_t)i * insize + j];
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = 0;
  __syncwarp();
  engine_run_op<double>(P, sA[w], sB[w], sS[w], lane);
  __syncwarp();
  for (int j = lane; j < outsize; j += 32) out[(size_t)i * outsize + j] += engine_out_op(P, sS[w], j);
}

// M2L_p (fmmgen/expansions.py:144-172): derivatives at d, then the contraction
__global__ void k_op_m2l(Plan P, int n, const double *d, const double *M, double *L, int order, int so) {
  // sT is the recurrence's scratch, then holds the source multipole
  __shared__ double sD[OPW][FMM_NTMAX], sT[OPW][FMM_NTMAX], sS[OPW][FMM_NTMAX + 32];
  __shared__ double sb[OPW][FMM_PMAX + 1];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  warp_derivs<double>(d[3 * i], d[3 * i + 1], d[3 * i + 2], order, sD[w], sT[w], sb[w]);
  double *sB = sT[w];
  int ms = fmm_nterms(order) - fmm_nterms(so - 1), ls = fmm_nterms(order - so);
  for (int j = lane; j < ms; j += 32) sB[j] = M[(size_t)i * ms + j];
  for (int k = lane; k < P.nseg; k += 32) sS[w][k] = 0;
  __syncwarp();
  engine_run_op<double>(P, sD[w], sB, sS[w], lane);
  __syncwarp();
  for (int j = lane; j < ls; j += 32) L[(size_t)i * ls + j] += engine_out_op(P, sS[w], j);
}

// L2P_p (fmmgen/expansions.py:197-207)
__global__ void k_op_l2p(int n, const double *d, const double *L, double *F, int order, int so, int potential,
                         int field) {
  __shared__ double mon[OPW][FMM_NTMAX];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int i = blockIdx.x * OPW + w;
  if (i >= n) return;
  int pl = order - so, ls = fmm_nterms(pl);
  op_monomials(d[3 * i], d[3 * i + 1], d[3 * i + 2], pl, mon[w], lane);
  __syncwarp();
  double phi = 0, ex = 0, ey = 0, ez = 0;
  const double *Li = L + (size_t)i * ls;
  for (int j = lane; j < ls; j += 32) {
    int nx = c_mi[j][0], ny = c_mi[j][1], nz = c_mi[j][2];
    double l = Li[j];
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
    double *Fi = F + (size_t)i * os;
    int k = 0;
    if (potential) Fi[k++] += phi;
    if (field) { Fi[k] += ex; Fi[k + 1] += ey; Fi[k + 2] += ez; }
  }
}

// P2P (Coulomb form of example/operators.cpp:54-66; dipole and quadrupole
// fields restated as the gradients of the generated potentials)
__global__ void k_op_p2p(int n, const double *d, const double *S, double *F, int so, int potential, int field) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = d[3 * i], y = d[3 * i + 1], z = d[3 * i + 2];
  double R = sqrt(x * x + y * y + z * z);
  double phi = 0, ex = 0, ey = 0, ez = 0;
  if (so == 2) {
    quadrupole_p2p<double>(x, y, z, S + 6 * (size_t)i, phi, ex, ey, ez);
  } else if (so == 0) {
    double q = S[i];
    double r3 = 1.0 / (R * R * R);
    phi = q / R;
    ex = q * x * r3; ey = q * y * r3; ez = q * z * r3;
  } else {
    const double *s = S + 3 * (size_t)i;
    double rinv = 1.0 / R, r3 = rinv * rinv * rinv, r5 = r3 * rinv * rinv;
    double sr = s[0] * x + s[1] * y + s[2] * z;
    phi = -sr * r3;
    ex = s[0] * r3 - 3.0 * sr * x * r5; ey = s[1] * r3 - 3.0 * sr * y * r5; ez = s[2] * r3 - 3.0 * sr * z * r5;
  }
  int os = (potential ? 1 : 0) + (field ? 3 : 0);
  double *Fi = F + (size_t)i * os;
  int k = 0;
  if (potential) Fi[k++] += phi;
  if (field) { Fi[k] += ex; Fi[k + 1] += ey; Fi[k + 2] += ez; }
}

// op: 0 P2M, 1 M2M, 2 M2L, 3 L2L, 4 L2P, 5 P2P
// M2P_p (fmmgen/generator.py:174-206), one thread per application: the
// potential V = sum_m D_m(d) M_m of fmmgen's M2P and its exact gradient
// E = -sum_m D_(m+e)(d) M_m (the generated field is not that gradient);
// d = particle - cell.  NTQ holds the derivatives to order + 1.
template <int NTQ>
__global__ void k_op_m2p(int n, const double *d, const double *M, double *F, int order, int so, int potential,
                         int field) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double D[NTQ];
  thread_derivs(d[3 * i], d[3 * i + 1], d[3 * i + 2], order + 1, D);
  const int moff = fmm_nterms(so - 1), ms = fmm_nterms(order) - moff;
  const double *Mi = M + (size_t)i * ms;
  double v = 0, gx = 0, gy = 0, gz = 0;
  int j = moff;
  for (int dg = so; dg <= order; dg++)
    for (int mx = dg; mx >= 0; mx--)
      for (int my = dg - mx; my >= 0; my--, j++) {
        const int mz = dg - mx - my;
        const double w = Mi[j - moff];
        v += D[j] * w;
        gx += D[fmm_idx3(mx + 1, my, mz)] * w;
        gy += D[fmm_idx3(mx, my + 1, mz)] * w;
        gz += D[fmm_idx3(mx, my, mz + 1)] * w;
      }
  const int os = (potential ? 1 : 0) + (field ? 3 : 0);
  double *Fi = F + (size_t)i * os;
  int k = 0;
  if (potential) Fi[k++] += v;
  if (field) {
    Fi[k] -= gx;
    Fi[k + 1] -= gy;
    Fi[k + 2] -= gz;
  }
}

int fmm_op_batch(int op, int n, const double *d, const double *in, double *out, int order, int so, int potential,
                 int field, cudaStream_t st) {
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
    case 0: fmm_note_launch(), k_op_p2m<<<nb, 32 * OPW, 0, st>>>(n, d, in, out, order, so); break;
    case 1: fmm_note_launch(), k_op_shift<<<nb, 32 * OPW, 0, st>>>(ps->m2m, n, d, in, out, order, so, ms, ms, order - so); break;
    case 2: fmm_note_launch(), k_op_m2l<<<nb, 32 * OPW, 0, st>>>(ps->m2l, n, d, in, out, order, so); break;
    case 3: fmm_note_launch(), k_op_shift<<<nb, 32 * OPW, 0, st>>>(ps->l2l, n, d, in, out, order, so, ls, ls, order - so); break;
    case 4: fmm_note_launch(), k_op_l2p<<<nb, 32 * OPW, 0, st>>>(n, d, in, out, order, so, potential, field); break;
    case 5: fmm_note_launch(), k_op_p2p<<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, so, potential, field); break;
    case 6:
      if (order + 1 <= 6) fmm_note_launch(), k_op_m2p<84><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, order, so, potential, field);
      else if (order + 1 <= 9) fmm_note_launch(), k_op_m2p<220><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, order, so, potential, field);
      else fmm_note_launch(), k_op_m2p<560><<<fmm_blocks(n, 128), 128, 0, st>>>(n, d, in, out, order, so, potential, field);
      break;
    default: return FMM_ERR_ARG;
  }
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
