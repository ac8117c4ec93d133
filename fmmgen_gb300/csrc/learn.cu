// learn.cu -- learned per-pair expansion order for the M2L (no counterpart in
// the reference, whose FMM uses one order for every pair).
//
// A small MLP (16 -> 64 -> 64 -> 11, ReLU) reads features of an M2L pair
// (B -> A) and predicts the lowest order q in [2, 12] at which the pair's
// contribution stays within a tolerance of its order-p contribution; the
// evaluation then applies each pair at its own order (k_m2l_var, eval.cu).
// Everything here is hand-written CUDA: features, labels (training targets),
// inference, and the training step (forward, backward, weight gradients,
// Adam).  The fixed-order FMM stays the fallback and the judge of the error.
#include <algorithm>
#include <cmath>
#include "internal.h"

#define MLP_IN 16
#define MLP_H 64
#define MLP_OUT 11   // orders 2..12
#define MLP_QMIN 2
#define MLP_NPARAM (MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_OUT * MLP_H + MLP_OUT)
// parameter layout (FP32): W1[64][16], b1[64], W2[64][64], b2[64], W3[11][64], b3[11]
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + MLP_H * MLP_IN)
#define OFF_W2 (OFF_B1 + MLP_H)
#define OFF_B2 (OFF_W2 + MLP_H * MLP_H)
#define OFF_W3 (OFF_B2 + MLP_H)
#define OFF_B3 (OFF_W3 + MLP_OUT * MLP_H)

int fmm_mlp_nparam() { return MLP_NPARAM; }

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
// Per cell: the 2-norm of each degree block of its scaled multipole M~ (degree
// d terms are [NT(d-1), NT(d)) of the full layout; the row starts at degree so).
template <typename T>
__global__ void k_cell_mnorms(const T *M, int mstr, int ncells, int so, int order, float *mn) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (c >= ncells) return;
  const int moff = fmm_nterms(so - 1);
  for (int d = 0; d <= FMM_PMAX; d++) {
    double s = 0;
    if (d >= so && d <= order)
      for (int j = fmm_nterms(d - 1) + lane; j < fmm_nterms(d); j += 32) {
        const double v = (double)M[(size_t)c * mstr + (j - moff)];
        s += v * v;
      }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) mn[(size_t)c * (FMM_PMAX + 1) + d] = (float)sqrt(s);
  }
}

// Geometry of class c in the target's half-widths: separation |d|/s_A and the
// size ratio rho = s_B / s_A = 2^-dlev.
__device__ __forceinline__ void class_geometry(const int *key4, int c, float &sep, float &rho, int &dlev) {
  dlev = key4[4 * c];
  const float gx = (float)key4[4 * c + 1], gy = (float)key4[4 * c + 2], gz = (float)key4[4 * c + 3];
  const float g = sqrtf(gx * gx + gy * gy + gz * gz);  // in half-widths of the finer cell
  sep = dlev > 0 ? ldexpf(g, -dlev) : g;
  rho = ldexpf(1.f, -dlev);
}

// The pair's estimated contribution at the target: sum_d rho^d |M~_d| / sep^(d+1)
// (scaled units), and each degree's part of it.
__device__ __forceinline__ float pair_weight(const float *mn, float sep, float rho, float *part) {
  float w = 0, rp = 1, sp = 1.f / sep;
  for (int d = 0; d <= FMM_PMAX; d++) {
    part[d] = mn[d] * rp * sp;
    w += part[d];
    rp *= rho;
    sp /= sep;
  }
  return w;
}

// ---------------------------------------------------------------------------
// the tolerance scale
// ---------------------------------------------------------------------------
// The error target is global: a relative L2 field error eps over a system's
// particles.  Splitting the squared budget eps^2 sum_i |E_i|^2 equally over
// the system's P pairs, pair k of target A -- whose truncation error reaches
// all n_A particles of A -- may leave a field error of
// eps sqrt(sum_i |E_i|^2 / P) / sqrt(n_A) there; in the scaled units of A's
// local expansion (L^_n = s^(|n|+1) L_n) that is eps T_A with
//   T_A = tscale_sys s_A^2 / sqrt(n_A),   tscale_sys = sqrt(sum_i |E_i|^2 / P).
// |E_i| is the pass's near field (its P2P part), which carries the RMS field
// of point charges, so the scale needs nothing beyond the pass itself.
#define TS_THREADS 256
#define TS_BLOCKS 1024

__device__ __forceinline__ double block_sum(double s, double *red) {
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  s = 0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// sum |E_near|^2 over a contiguous particle range per block (sorted order): one
// chunk of the whole set when nsys == 1, else system blockIdx.x (a system's
// particles are contiguous in the sorted order).  Fixed order: deterministic.
__global__ void __launch_bounds__(TS_THREADS) k_near_sumsq(const double *Fnear, long N, const long *sys_off,
                                                           int nsys, double *part) {
  __shared__ double red[TS_THREADS / 32];
  long lo, hi;
  if (nsys > 1) {
    lo = sys_off[blockIdx.x];
    hi = sys_off[blockIdx.x + 1];
  } else {
    const long ch = (N + gridDim.x - 1) / gridDim.x;
    lo = min(N, (long)blockIdx.x * ch);
    hi = min(N, lo + ch);
  }
  double s = 0;
  for (long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double *f = Fnear + 4 * i;
    s += f[1] * f[1] + f[2] * f[2] + f[3] * f[3];
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_sys_pairs(const int *off, const int *csys, int ncells, int *pairs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int n = off[c + 1] - off[c];
  if (n) atomicAdd(pairs + (csys ? csys[c] : 0), n);
}

__global__ void __launch_bounds__(TS_THREADS) k_sys_tscale(const double *part, int nparts, int nsys,
                                                           const int *pairs, double *tscale) {
  __shared__ double red[TS_THREADS / 32];
  if (nsys == 1) {
    double s = 0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) tscale[0] = sqrt(s / (double)max(pairs[0], 1));
    return;
  }
  for (int i = threadIdx.x; i < nsys; i += blockDim.x) tscale[i] = sqrt(part[i] / (double)max(pairs[i], 1));
}

// T_A of the target cell
__device__ __forceinline__ double cell_tol(const double *tscale, const int *csys, const double *cr, const int *pcount,
                                           int A) {
  const double s = cr[A];
  return tscale[csys ? csys[A] : 0] * s * s / sqrt((double)max(pcount[A], 1));
}

// Features of every M2L pair in list order (one warp per target cell):
//  f0 = lB - lA, f1 = log2(sep / s_A), f2 = log10 of the pair's share of the
//  target's summed estimates, f3..f14 = log10 of the part of degree 1..12 in
//  the pair's estimate, f15 = log10 of the pair's estimated field at A over
//  eps T_A (the estimate w is in the scaled units of A's local expansion, the
//  field about w / sep).
__global__ void k_order_features(const int *off, const int *src, const int *cls, int ncells, const int *key4,
                                 const float *mn, const double *tscale, const int *csys, const double *cr,
                                 const int *pcount, double eps, float *feat) {
  const int A = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (A >= ncells) return;
  const double etol = eps * cell_tol(tscale, csys, cr, pcount, A);
  const int k0 = off[A], k1 = off[A + 1];
  float part[FMM_PMAX + 1];
  float wsum = 0;
  for (int k = k0 + lane; k < k1; k += 32) {
    float sep, rho;
    int dlev;
    class_geometry(key4, cls[k], sep, rho, dlev);
    wsum += pair_weight(mn + (size_t)src[k] * (FMM_PMAX + 1), sep, rho, part);
  }
  for (int o = 16; o; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
  for (int k = k0 + lane; k < k1; k += 32) {
    float sep, rho;
    int dlev;
    class_geometry(key4, cls[k], sep, rho, dlev);
    const float w = pair_weight(mn + (size_t)src[k] * (FMM_PMAX + 1), sep, rho, part);
    float *f = feat + (size_t)k * MLP_IN;
    f[0] = (float)dlev;
    f[1] = log2f(sep);
    f[2] = log10f(fmaxf(w / fmaxf(wsum, 1e-30f), 1e-30f));
    for (int d = 1; d <= 12; d++) f[2 + d] = log10f(fmaxf(part[d] / fmaxf(w, 1e-30f), 1e-30f));
    f[15] = (float)log10(fmax((double)w / ((double)sep * etol), 1e-30));
  }
}

// ---------------------------------------------------------------------------
// labels (training targets)
// ---------------------------------------------------------------------------
// multi-index table and, per output n, g_n = max over the cell box |y_i| <= 1 of
// |grad (y^n / n!)| (the field a unit local coefficient makes in the cell)
__constant__ unsigned char c_lmi[FMM_NTMAX][4];
__constant__ double c_gn[FMM_NTMAX];
static bool g_label_tables[16] = {false};

static int label_tables() {
  int dev = 0;
  FMM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 16) return FMM_ERR_CUDA;
  if (g_label_tables[dev]) return FMM_OK;
  unsigned char mi[FMM_NTMAX][4];
  double gn[FMM_NTMAX];
  double fact[FMM_PMAX + 2];
  fact[0] = 1;
  for (int i = 1; i <= FMM_PMAX + 1; i++) fact[i] = fact[i - 1] * i;
  for (int i = 0; i < FMM_NTMAX; i++) {
    const MI m = fmm_decode(i);
    mi[i][0] = m.x; mi[i][1] = m.y; mi[i][2] = m.z; mi[i][3] = m.d;
    const int n[3] = {m.x, m.y, m.z};
    double g2 = 0;
    for (int a = 0; a < 3; a++) {
      if (!n[a]) continue;
      double f = 1;
      for (int b = 0; b < 3; b++) f *= fact[n[b] - (a == b ? 1 : 0)];
      g2 += 1.0 / (f * f);
    }
    gn[i] = sqrt(g2);
  }
  FMM_CUDA_TRY(cudaMemcpyToSymbol(c_lmi, mi, sizeof(mi)));
  FMM_CUDA_TRY(cudaMemcpyToSymbol(c_gn, gn, sizeof(gn)));
  g_label_tables[dev] = true;
  return FMM_OK;
}

// One warp per pair: for every output n (lanes), the pair's order-p
// contribution split by total degree d = |n| + |m|; err_q = sum_n g_n
// |sum_{d > q} part_{n,d}| bounds the field error in the target cell of
// truncating the pair at order q.  label = lowest q >= 2 with err_q <= eps T_A
// (T_A: the tolerance scale above).  errq (optional) [npairs][11]: err_q / (eps T_A).
#define LBL_WARPS 4
__global__ void __launch_bounds__(32 * LBL_WARPS) k_order_labels(
    const int *src, const int *cls, const int *tgt, long npairs, const double *clsD, int dstr,
    const unsigned char *clevel, const double *M, int mstr, int so, int order, const double *tscale,
    const int *csys, const double *cr, const int *pcount, double eps, unsigned char *label, float *errq) {
  __shared__ double sD[LBL_WARPS][FMM_NTMAX], sM[LBL_WARPS][FMM_NTMAX];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long k = (long)blockIdx.x * LBL_WARPS + w;
  if (k >= npairs) return;
  const int A = tgt[k], B = src[k];
  const int moff = fmm_nterms(so - 1), nt = fmm_nterms(order), ls = fmm_nterms(order - so);
  const int dl = (int)clevel[A] - (int)clevel[B];  // rho = 2^dl
  const double *D = clsD + (size_t)cls[k] * dstr;
  for (int i = lane; i < nt; i += 32) sD[w][i] = D[i];
  for (int j = lane; j < nt - moff; j += 32)
    sM[w][j + moff] = ldexp(M[(size_t)B * mstr + j], dl * (int)c_lmi[j + moff][3]);
  __syncwarp();
  double err[FMM_PMAX + 1];
#pragma unroll
  for (int q = 0; q <= FMM_PMAX; q++) err[q] = 0;
  for (int n = lane; n < ls; n += 32) {
    const int nx = c_lmi[n][0], ny = c_lmi[n][1], nz = c_lmi[n][2], dn = c_lmi[n][3];
    double part[FMM_PMAX + 1];  // part[d]: the terms of total degree d
#pragma unroll
    for (int d = 0; d <= FMM_PMAX; d++) part[d] = 0;
    for (int dm = so; dm <= order - dn; dm++) {  // source degree blocks
      double acc = 0;
      for (int m = fmm_nterms(dm - 1); m < fmm_nterms(dm); m++)
        acc += sD[w][fmm_idx3(nx + c_lmi[m][0], ny + c_lmi[m][1], nz + c_lmi[m][2])] * sM[w][m];
      part[dn + dm] = acc;
    }
    // suffix sums: truncation at q drops the degrees above q
    double suf = 0;
#pragma unroll
    for (int q = FMM_PMAX; q >= 0; q--) {
      err[q] += c_gn[n] * fabs(suf);
      suf += part[q];
    }
  }
#pragma unroll
  for (int q = 0; q <= FMM_PMAX; q++)
    for (int o = 16; o; o >>= 1) err[q] += __shfl_xor_sync(0xffffffffu, err[q], o);
  if (lane == 0) {
    const double tol = eps * cell_tol(tscale, csys, cr, pcount, A);
    int q = order;
    for (int c = MLP_QMIN; c < order; c++)
      if (err[c] <= tol) { q = c; break; }
    label[k] = (unsigned char)(q - MLP_QMIN);
    if (errq)
      for (int c = 0; c < MLP_OUT; c++) {
        const int qq = c + MLP_QMIN;
        errq[(size_t)k * MLP_OUT + c] = qq <= order ? (float)(err[qq] / (tol > 0 ? tol : 1.0)) : 0.f;
      }
  }
}

__global__ void k_expand_tgt(const int *off, int ncells, int *tgt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  for (int k = off[c]; k < off[c + 1]; k++) tgt[k] = c;
}

// ---------------------------------------------------------------------------
// MLP: inference
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mlp_forward(const float *P, const float *x, float *h1, float *h2, float *z) {
  for (int i = 0; i < MLP_H; i++) {
    float a = P[OFF_B1 + i];
#pragma unroll
    for (int j = 0; j < MLP_IN; j++) a = fmaf(P[OFF_W1 + i * MLP_IN + j], x[j], a);
    h1[i] = fmaxf(a, 0.f);
  }
  for (int i = 0; i < MLP_H; i++) {
    float a = P[OFF_B2 + i];
    for (int j = 0; j < MLP_H; j++) a = fmaf(P[OFF_W2 + i * MLP_H + j], h1[j], a);
    h2[i] = fmaxf(a, 0.f);
  }
  for (int i = 0; i < MLP_OUT; i++) {
    float a = P[OFF_B3 + i];
    for (int j = 0; j < MLP_H; j++) a = fmaf(P[OFF_W3 + i * MLP_H + j], h2[j], a);
    z[i] = a;
  }
}

// Order of each pair: the lowest q whose cumulative predicted probability
// P(q* <= q) reaches 1 - delta (delta trades M2L work against the risk of a
// too-low order), clamped to [2, qmax].
__device__ __forceinline__ unsigned char mlp_order(const float *z, float delta, int qmax) {
  float zm = z[0];
  for (int i = 1; i < MLP_OUT; i++) zm = fmaxf(zm, z[i]);
  float s = 0;
  for (int i = 0; i < MLP_OUT; i++) s += __expf(z[i] - zm);
  float cum = 0;
  int q = MLP_QMIN + MLP_OUT - 1;
  for (int i = 0; i < MLP_OUT; i++) {
    cum += __expf(z[i] - zm) / s;
    if (cum >= 1.f - delta) {
      q = MLP_QMIN + i;
      break;
    }
  }
  return (unsigned char)min(max(q, MLP_QMIN), qmax);
}

// The forward pass of two pairs per thread.  The weights sit in shared memory
// (float4 broadcasts, each used for both pairs) and so do the first hidden
// layers (a row per pair, padded so the lanes' float4 reads are conflict
// free): both layers loop at run time over short unrolled bodies -- a fully
// unrolled network (two pairs x 5,824 multiply-adds) outgrows the instruction
// cache.  Units are computed MLP_U at a time (2 MLP_U independent FMA chains;
// 16 reads each hidden-layer float4 once per 16 weight broadcasts: 8 took 7 % longer),
// and each second-layer unit feeds the logits as soon as it is done.  Every
// output is summed in the order of mlp_forward (bias first, inputs
// ascending): the same bits.
#define MLP_U 16
#define MLP_HS (MLP_H + 4)  // padded row of a first hidden layer
constexpr int MLP_PREDICT_SMEM = (MLP_NPARAM + 3) / 4 * 16 + MLP_H * 12 * 4 + 128 * 2 * MLP_HS * 4;
__global__ void __launch_bounds__(128) k_mlp_predict(const float *params, const float *X, long n, float delta,
                                                     int qmax, unsigned char *orders) {
  extern __shared__ float4 mlp_smem[];
  float *P = (float *)mlp_smem;
  float(*W3T)[12] = (float(*)[12])(P + (MLP_NPARAM + 3) / 4 * 4);  // W3 by hidden unit (11 logits + 1 pad)
  float *H = (float *)(W3T + MLP_H) + threadIdx.x * 2 * MLP_HS;     // this thread's two first hidden layers
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) P[i] = params[i];
  for (int i = threadIdx.x; i < MLP_H * 12; i += blockDim.x) {
    const int h = i / 12, o = i - 12 * h;
    W3T[h][o] = o < MLP_OUT ? params[OFF_W3 + o * MLP_H + h] : 0.f;
  }
  __syncthreads();
  const long stride = 2L * gridDim.x * blockDim.x;
  for (long k = 2L * (blockIdx.x * (long)blockDim.x + threadIdx.x); k < n; k += stride) {
    float x[2][MLP_IN];
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const float4 *x4 = (const float4 *)(X + min(k + r, n - 1) * MLP_IN);
#pragma unroll
      for (int j = 0; j < MLP_IN / 4; j++) {
        const float4 u = x4[j];
        x[r][4 * j] = u.x, x[r][4 * j + 1] = u.y, x[r][4 * j + 2] = u.z, x[r][4 * j + 3] = u.w;
      }
    }
#pragma unroll 1
    for (int i = 0; i < MLP_H; i += 4) {
      float a[4][2];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        a[u][0] = a[u][1] = P[OFF_B1 + i + u];
#pragma unroll
        for (int j = 0; j < MLP_IN; j += 4) {
          const float4 w = *(const float4 *)&P[OFF_W1 + (i + u) * MLP_IN + j];
#pragma unroll
          for (int r = 0; r < 2; r++) {
            a[u][r] = fmaf(w.x, x[r][j], a[u][r]);
            a[u][r] = fmaf(w.y, x[r][j + 1], a[u][r]);
            a[u][r] = fmaf(w.z, x[r][j + 2], a[u][r]);
            a[u][r] = fmaf(w.w, x[r][j + 3], a[u][r]);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < 2; r++)
        *(float4 *)&H[r * MLP_HS + i] =
            make_float4(fmaxf(a[0][r], 0.f), fmaxf(a[1][r], 0.f), fmaxf(a[2][r], 0.f), fmaxf(a[3][r], 0.f));
    }
    float z[2][MLP_OUT];
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int o = 0; o < MLP_OUT; o++) z[r][o] = P[OFF_B3 + o];
#pragma unroll 1
    for (int i = 0; i < MLP_H; i += MLP_U) {
      float a[MLP_U][2];
#pragma unroll
      for (int u = 0; u < MLP_U; u++) a[u][0] = a[u][1] = P[OFF_B2 + i + u];
#pragma unroll 2
      for (int j = 0; j < MLP_H; j += 4) {
        const float4 h0 = *(const float4 *)&H[j], h1 = *(const float4 *)&H[MLP_HS + j];
#pragma unroll
        for (int u = 0; u < MLP_U; u++) {
          const float4 w = *(const float4 *)&P[OFF_W2 + (i + u) * MLP_H + j];
          a[u][0] = fmaf(w.x, h0.x, a[u][0]), a[u][1] = fmaf(w.x, h1.x, a[u][1]);
          a[u][0] = fmaf(w.y, h0.y, a[u][0]), a[u][1] = fmaf(w.y, h1.y, a[u][1]);
          a[u][0] = fmaf(w.z, h0.z, a[u][0]), a[u][1] = fmaf(w.z, h1.z, a[u][1]);
          a[u][0] = fmaf(w.w, h0.w, a[u][0]), a[u][1] = fmaf(w.w, h1.w, a[u][1]);
        }
      }
#pragma unroll
      for (int u = 0; u < MLP_U; u++) {
        const float4 t0 = *(const float4 *)&W3T[i + u][0], t1 = *(const float4 *)&W3T[i + u][4],
                     t2 = *(const float4 *)&W3T[i + u][8];
        const float t[12] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
#pragma unroll
        for (int r = 0; r < 2; r++) {
          const float g = fmaxf(a[u][r], 0.f);
#pragma unroll
          for (int o = 0; o < MLP_OUT; o++) z[r][o] = fmaf(t[o], g, z[r][o]);
        }
      }
    }
    orders[k] = mlp_order(z[0], delta, qmax);
    if (k + 1 < n) orders[k + 1] = mlp_order(z[1], delta, qmax);
  }
}

// ---------------------------------------------------------------------------
// MLP: one training step (cross-entropy over a batch, mean)
// ---------------------------------------------------------------------------
// forward: activations H1, H2 [n][64]; G3 = (softmax(z) - onehot(y)) / n [n][11]; loss summed
__global__ void k_mlp_fwd(const float *params, const float *X, const unsigned char *y, int n, float *H1, float *H2,
                          float *G3, float *loss) {
  __shared__ float P[MLP_NPARAM];
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0;
  if (k < n) {
    float x[MLP_IN], h1[MLP_H], h2[MLP_H], z[MLP_OUT];
    for (int j = 0; j < MLP_IN; j++) x[j] = X[(size_t)k * MLP_IN + j];
    mlp_forward(P, x, h1, h2, z);
    for (int i = 0; i < MLP_H; i++) {
      H1[(size_t)k * MLP_H + i] = h1[i];
      H2[(size_t)k * MLP_H + i] = h2[i];
    }
    float zm = z[0];
    for (int i = 1; i < MLP_OUT; i++) zm = fmaxf(zm, z[i]);
    float s = 0;
    for (int i = 0; i < MLP_OUT; i++) s += expf(z[i] - zm);
    const int yk = y[k];
    for (int i = 0; i < MLP_OUT; i++) G3[(size_t)k * MLP_OUT + i] = (expf(z[i] - zm) / s - (i == yk ? 1.f : 0.f)) / n;
    l = (logf(s) + zm - z[yk]) / n;
  }
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// backward through the layers: G2 = (W3^T G3) * [H2 > 0], G1 = (W2^T G2) * [H1 > 0]
__global__ void k_mlp_bwd(const float *params, int n, const float *H1, const float *H2, const float *G3, float *G2,
                          float *G1) {
  __shared__ float P[MLP_NPARAM];
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float g3[MLP_OUT], g2[MLP_H];
  for (int i = 0; i < MLP_OUT; i++) g3[i] = G3[(size_t)k * MLP_OUT + i];
  for (int j = 0; j < MLP_H; j++) {
    float a = 0;
    for (int i = 0; i < MLP_OUT; i++) a = fmaf(P[OFF_W3 + i * MLP_H + j], g3[i], a);
    g2[j] = H2[(size_t)k * MLP_H + j] > 0.f ? a : 0.f;
    G2[(size_t)k * MLP_H + j] = g2[j];
  }
  for (int j = 0; j < MLP_H; j++) {
    float a = 0;
    for (int i = 0; i < MLP_H; i++) a = fmaf(P[OFF_W2 + i * MLP_H + j], g2[i], a);
    G1[(size_t)k * MLP_H + j] = H1[(size_t)k * MLP_H + j] > 0.f ? a : 0.f;
  }
}

// weight gradients, one thread per parameter and row chunk (blockIdx.y):
// dW[i][j] = sum_k G[k][i] A[k][j], db[i] = sum_k G[k][i], chunk sums added
// into grad (zeroed before)
__global__ void k_mlp_wgrad(int n, int chunk, const float *X, const float *H1, const float *H2, const float *G1,
                            const float *G2, const float *G3, float *grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  const int k0 = blockIdx.y * chunk, k1 = min(n, k0 + chunk);
  const float *G, *Aa;
  int gi, gs, aj = -1, as = 0;
  if (p < OFF_B1) { G = G1; gs = MLP_H; gi = (p - OFF_W1) / MLP_IN; Aa = X; as = MLP_IN; aj = (p - OFF_W1) % MLP_IN; }
  else if (p < OFF_W2) { G = G1; gs = MLP_H; gi = p - OFF_B1; Aa = nullptr; }
  else if (p < OFF_B2) { G = G2; gs = MLP_H; gi = (p - OFF_W2) / MLP_H; Aa = H1; as = MLP_H; aj = (p - OFF_W2) % MLP_H; }
  else if (p < OFF_W3) { G = G2; gs = MLP_H; gi = p - OFF_B2; Aa = nullptr; }
  else if (p < OFF_B3) { G = G3; gs = MLP_OUT; gi = (p - OFF_W3) / MLP_H; Aa = H2; as = MLP_H; aj = (p - OFF_W3) % MLP_H; }
  else { G = G3; gs = MLP_OUT; gi = p - OFF_B3; Aa = nullptr; }
  float s = 0;
  if (Aa)
    for (int k = k0; k < k1; k++) s = fmaf(G[(size_t)k * gs + gi], Aa[(size_t)k * as + aj], s);
  else
    for (int k = k0; k < k1; k++) s += G[(size_t)k * gs + gi];
  atomicAdd(grad + p, s);
}

// Adam (bias-corrected), step t >= 1
__global__ void k_adam(float *params, const float *grad, float *m, float *v, int t, float lr, float b1, float b2,
                       float epsa) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  const float g = grad[p];
  const float mm = b1 * m[p] + (1.f - b1) * g, vv = b2 * v[p] + (1.f - b2) * g * g;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.f - powf(b1, (float)t)), vh = vv / (1.f - powf(b2, (float)t));
  params[p] -= lr * mh / (sqrtf(vh) + epsa);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
#define TRY_(x) do { int _rc = (x); if (_rc) return _rc; } while (0)

// the multipole rows of the last evaluation: FP64 (M) or FP32 (Mf, 16-byte rows)
static int mnorms(DevTree *t, cudaStream_t st) {
  const int nc = t->ncells, p = t->order, so = t->so;
  const int msize = fmm_nterms(p) - fmm_nterms(so - 1);
  TRY_(fmm_reserve(t->mnorm, (size_t)nc * (FMM_PMAX + 1)));
  if (t->last_prec == 0)
    fmm_note_launch(), k_cell_mnorms<double><<<fmm_blocks((size_t)nc * 32, 128), 128, 0, st>>>(t->M.p, msize, nc, so,
                                                                                               p, t->mnorm.p);
  else
    fmm_note_launch(), k_cell_mnorms<float><<<fmm_blocks((size_t)nc * 32, 128), 128, 0, st>>>(
        t->Mf.p, fmm_stride4(msize), nc, so, p, t->mnorm.p);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// per-system tolerance scale from the near field of the last pass (t->tscale)
static int tol_scale(DevTree *t, cudaStream_t st) {
  const int nsys = t->nsys, nparts = nsys > 1 ? nsys : TS_BLOCKS;
  TRY_(fmm_reserve(t->tpart, nparts));
  TRY_(fmm_reserve(t->tscale, nsys));
  TRY_(fmm_reserve(t->sys_pairs, nsys));
  FMM_CUDA_TRY(cudaMemsetAsync(t->sys_pairs.p, 0, sizeof(int) * nsys, st));
  fmm_note_launch(), k_near_sumsq<<<nparts, TS_THREADS, 0, st>>>(t->Fnear.p, t->N, nsys > 1 ? t->sys_off.p : nullptr,
                                                                 nsys, t->tpart.p);
  fmm_note_launch(), k_sys_pairs<<<fmm_blocks(t->ncells, 256), 256, 0, st>>>(
      t->m2l_off.p, nsys > 1 ? t->csys.p : nullptr, t->ncells, t->sys_pairs.p);
  fmm_note_launch(), k_sys_tscale<<<1, TS_THREADS, 0, st>>>(t->tpart.p, nparts, nsys, t->sys_pairs.p, t->tscale.p);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

int fmm_order_features(DevTree *t, double eps, float *feat, cudaStream_t st) {
  if (int rc = fmm_m2l_csr(t, st)) return rc;
  if (t->last_prec < 0) return FMM_ERR_STATE;  // the features read the multipoles and near field of a pass
  if (t->nm2l == 0) return FMM_OK;
  TRY_(mnorms(t, st));
  TRY_(tol_scale(t, st));
  fmm_note_launch(), k_order_features<<<fmm_blocks((size_t)t->ncells * 32, 128), 128, 0, st>>>(
      t->m2l_off.p, t->m2l_src.p, t->m2l_cls.p, t->ncells, t->cls_key4.p, t->mnorm.p, t->tscale.p,
      t->nsys > 1 ? t->csys.p : nullptr, t->cr.p, t->pcount.p, eps, feat);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

int fmm_order_labels(DevTree *t, double eps, unsigned char *label, float *errq, cudaStream_t st) {
  if (int rc = fmm_m2l_csr(t, st)) return rc;
  if (t->last_prec != 0) return FMM_ERR_STATE;  // needs the FP64 multipoles
  if (t->nm2l == 0) return FMM_OK;
  TRY_(label_tables());
  const int nc = t->ncells;
  TRY_(fmm_reserve(t->ltgt, t->nm2l));
  TRY_(tol_scale(t, st));
  fmm_note_launch(), k_expand_tgt<<<fmm_blocks(nc, 128), 128, 0, st>>>(t->m2l_off.p, nc, t->ltgt.p);
  const int msize = fmm_nterms(t->order) - fmm_nterms(t->so - 1);
  fmm_note_launch(), k_order_labels<<<fmm_blocks(t->nm2l, LBL_WARPS), 32 * LBL_WARPS, 0, st>>>(
      t->m2l_src.p, t->m2l_cls.p, t->ltgt.p, t->nm2l, t->cls_D.p, fmm_nterms(t->order), t->clevel.p, t->M.p, msize,
      t->so, t->order, t->tscale.p, t->nsys > 1 ? t->csys.p : nullptr, t->cr.p, t->pcount.p, eps, label, errq);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

int fmm_mlp_predict(const float *params, const float *X, long n, float delta, int qmax, unsigned char *orders,
                    cudaStream_t st) {
  if (n <= 0) return FMM_OK;
  const unsigned nb = (unsigned)std::min<long>((n + 255) / 256, 152L * 16);
  FMM_CUDA_TRY(cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_PREDICT_SMEM));
  fmm_note_launch(), k_mlp_predict<<<nb, 128, MLP_PREDICT_SMEM, st>>>(params, X, n, delta, qmax, orders);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// work: n * 267 floats (H1, H2, G1, G2: 64 each; G3: 11); grad [nparam]; loss += mean cross-entropy
int fmm_mlp_train_step(const float *params, const float *X, const unsigned char *y, int n, float *grad, float *loss,
                       float *work, cudaStream_t st) {
  if (n <= 0) return FMM_ERR_ARG;
  float *H1 = work, *H2 = H1 + (size_t)n * MLP_H, *G1 = H2 + (size_t)n * MLP_H, *G2 = G1 + (size_t)n * MLP_H;
  float *G3 = G2 + (size_t)n * MLP_H;
  fmm_note_launch(), k_mlp_fwd<<<fmm_blocks(n, 128), 128, 0, st>>>(params, X, y, n, H1, H2, G3, loss);
  fmm_note_launch(), k_mlp_bwd<<<fmm_blocks(n, 128), 128, 0, st>>>(params, n, H1, H2, G3, G2, G1);
  const int nchunk = std::min(64, (n + 1023) / 1024), chunk = (n + nchunk - 1) / nchunk;
  FMM_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(float) * MLP_NPARAM, st));
  fmm_note_launch(), k_mlp_wgrad<<<dim3(fmm_blocks(MLP_NPARAM, 128), nchunk), 128, 0, st>>>(n, chunk, X, H1, H2, G1,
                                                                                              G2, G3, grad);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

int fmm_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr, cudaStream_t st) {
  if (step < 1) return FMM_ERR_ARG;
  fmm_note_launch(), k_adam<<<fmm_blocks(MLP_NPARAM, 128), 128, 0, st>>>(params, grad, m, v, step, lr, 0.9f, 0.999f,
                                                                         1e-8f);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// In an evaluation with an order model attached (after its P2M, M2M and P2P):
// the features of every M2L pair from this pass's multipoles and near field,
// then the orders (into t->m2l_ord).
int fmm_learned_orders(DevTree *t, cudaStream_t st) {
  if (int rc = fmm_m2l_csr(t, st)) return rc;
  TRY_(fmm_reserve(t->feat, (size_t)(t->nm2l > 0 ? t->nm2l : 1) * MLP_IN));
  TRY_(fmm_reserve(t->m2l_ord, t->nm2l > 0 ? t->nm2l : 1));
  TRY_(fmm_order_features(t, t->model_eps, t->feat.p, st));
  TRY_(fmm_mlp_predict(t->model, t->feat.p, t->nm2l, t->model_delta, t->order, t->m2l_ord.p, st));
  t->ord_serial = t->build_serial;
  return FMM_OK;
}
