// shift.cu -- M2M and L2L of the mixed-precision pass with the eight fixed
// child-shift operators (example/calculate.cpp:163-187 and :219-234 with
// fmmgen's M2M_p / L2L_p, fmmgen/expansions.py:42-78 and :175-194).
//
// A child's centre sits at +-s/2 from its parent's on every axis (s the
// parent's half-width), so in the scaled expansions (M~ = M / s^|m|,
// L^ = s^(|n|+1) L) each shift is one of eight constant operators, fixed by
// the child's octant:
//   M2M:  M~_parent[n] += sum_{k <= n} mono_o(k) 2^-|n-k| M~_child[n-k],  mono_o(k) = (d/s)^k / k!,
//         d = parent - child
//   L2L:  L^_child[n]  += 2^-(|n|+1) sum_{|n|+|k| <= p-so} mono_o(k) L^_parent[n+k],  d = child - parent
// The operators are built once per (order, source order) in FP64 and kept as
// FP32 tables of (coefficient per octant, input term) entries, grouped by output
// term.  One thread computes one output term of one parent (L2L: of all its
// children at once); in L2L the few parents of the upper levels take a warp per
// term.
#include <map>
#include <mutex>
#include <vector>
#include "internal.h"

namespace {

struct ShiftTab {
  int nout = 0, nent = 0;
  const int *off = nullptr;     // [nout + 1] entries of each output term
  const int *in = nullptr;      // [nent] input term (row-relative)
  const float *coef = nullptr;  // [8][nent] coefficient per octant
  const float4 *coef8 = nullptr;  // [nent][2]: the eight octants' coefficients of an entry side by side
  void *dmem = nullptr;
};
struct ShiftSet {
  ShiftTab m2m, l2l;
};

std::mutex g_mu;
ShiftSet *g_sets[16][FMM_PMAX + 1][3] = {};

double mono(int kx, int ky, int kz, double vx, double vy, double vz) {
  double r = 1;
  for (int q = 1; q <= kx; q++) r = r * vx / q;
  for (int q = 1; q <= ky; q++) r = r * vy / q;
  for (int q = 1; q <= kz; q++) r = r * vz / q;
  return r;
}

// octant o: bit a set = the child lies on the + side of its parent along axis a
void sign_of(int o, double &sx, double &sy, double &sz) {
  sx = (o & 1) ? 0.5 : -0.5;
  sy = (o & 2) ? 0.5 : -0.5;
  sz = (o & 4) ? 0.5 : -0.5;
}

int upload(ShiftTab &t, const std::vector<int> &off, const std::vector<int> &in, const std::vector<float> &coef) {
  const size_t nent = in.size();
  std::vector<float> c8(8 * (nent ? nent : 1), 0.f);  // [entry][octant]
  for (size_t e = 0; e < nent; e++)
    for (int o = 0; o < 8; o++) c8[8 * e + o] = coef[(size_t)o * nent + e];
  const size_t b0 = off.size() * 4, b1 = (nent ? nent : 1) * 4, b2 = (coef.size() ? coef.size() : 8) * 4,
               b3 = c8.size() * 4;
  const size_t o1 = (b0 + 255) & ~(size_t)255, o2 = o1 + ((b1 + 255) & ~(size_t)255),
               o3 = o2 + ((b2 + 255) & ~(size_t)255);
  char *d = nullptr;
  if (cudaMalloc((void **)&d, o3 + b3) != cudaSuccess) return FMM_ERR_CUDA;
  if (cudaMemcpy(d, off.data(), b0, cudaMemcpyHostToDevice) != cudaSuccess ||
      (nent && cudaMemcpy(d + o1, in.data(), nent * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
      (coef.size() && cudaMemcpy(d + o2, coef.data(), coef.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
      cudaMemcpy(d + o3, c8.data(), b3, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return FMM_ERR_CUDA;
  }
  t.nout = (int)off.size() - 1;
  t.nent = (int)nent;
  t.off = (const int *)d;
  t.in = (const int *)(d + o1);
  t.coef = (const float *)(d + o2);
  t.coef8 = (const float4 *)(d + o3);
  t.dmem = d;
  return FMM_OK;
}

const ShiftSet *get_shift(int p, int so) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16 || p < 0 || p > FMM_PMAX || so < 0 || so > 2)
    return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_sets[dev][p][so]) return g_sets[dev][p][so];
  const int moff = fmm_nterms(so - 1), msize = fmm_nterms(p) - moff, lsize = fmm_nterms(p - so);
  ShiftSet *S = new ShiftSet();
  // M2M: output n (|n| in [so, p]), inputs j = n - k with k <= n, |j| >= so
  {
    std::vector<int> off(1, 0), in;
    std::vector<std::vector<float>> c8(8);
    for (int n = 0; n < msize; n++) {
      const MI nn = fmm_decode(n + moff);
      for (int kx = 0; kx <= nn.x; kx++)
        for (int ky = 0; ky <= nn.y; ky++)
          for (int kz = 0; kz <= nn.z; kz++) {
            const int jx = nn.x - kx, jy = nn.y - ky, jz = nn.z - kz, jd = jx + jy + jz;
            if (jd < so) continue;
            in.push_back(fmm_idx3(jx, jy, jz) - moff);
            for (int o = 0; o < 8; o++) {
              double sx, sy, sz;
              sign_of(o, sx, sy, sz);  // d = parent - child = -(child offset)
              c8[o].push_back((float)(mono(kx, ky, kz, -sx, -sy, -sz) * std::ldexp(1.0, -jd)));
            }
          }
      off.push_back((int)in.size());
    }
    std::vector<float> coef;
    for (int o = 0; o < 8; o++) coef.insert(coef.end(), c8[o].begin(), c8[o].end());
    if (upload(S->m2m, off, in, coef)) { delete S; return nullptr; }
  }
  // L2L: output n (|n| <= p - so), inputs j = n + k with |j| <= p - so
  {
    std::vector<int> off(1, 0), in;
    std::vector<std::vector<float>> c8(8);
    const int pl = p - so;
    for (int n = 0; n < lsize; n++) {
      const MI nn = fmm_decode(n);
      for (int k = 0; k < fmm_nterms(pl - nn.d); k++) {
        const MI kk = fmm_decode(k);
        in.push_back(fmm_idx3(nn.x + kk.x, nn.y + kk.y, nn.z + kk.z));
        for (int o = 0; o < 8; o++) {
          double sx, sy, sz;
          sign_of(o, sx, sy, sz);  // d = child - parent
          c8[o].push_back((float)(mono(kk.x, kk.y, kk.z, sx, sy, sz) * std::ldexp(1.0, -(nn.d + 1))));
        }
      }
      off.push_back((int)in.size());
    }
    std::vector<float> coef;
    for (int o = 0; o < 8; o++) coef.insert(coef.end(), c8[o].begin(), c8[o].end());
    if (upload(S->l2l, off, in, coef)) { delete S; return nullptr; }
  }
  g_sets[dev][p][so] = S;
  return S;
}

// octant of a child from the FP64 centres (exactly +-s/2 apart on each axis)
__device__ __forceinline__ int child_octant(double px, double py, double pz, double cx, double cy, double cz) {
  return (cx > px ? 1 : 0) | (cy > py ? 2 : 0) | (cz > pz ? 4 : 0);
}

// one thread per (parent of the level, output term)
__global__ void k_m2m_tab(int lo, int hi, int msize, ShiftTab T, const unsigned char *child_mask,
                          const int *child_first, const double *cx, const double *cy, const double *cz, float *M,
                          int mstr) {
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int c = lo + (int)(g / msize), n = (int)(g % msize);
  if (c >= hi) return;
  const unsigned mask = child_mask[c];
  if (!mask) return;
  const int e0 = T.off[n], e1 = T.off[n + 1];
  int ch = child_first[c];
  float acc = 0.f;
  for (int q = __popc(mask); q > 0; q--, ch++) {
    const int o = child_octant(cx[c], cy[c], cz[c], cx[ch], cy[ch], cz[ch]);
    const float *co = T.coef + (size_t)o * T.nent;
    const float *Mc = M + (size_t)ch * mstr;
    for (int e = e0; e < e1; e++) acc = fmaf(co[e], Mc[T.in[e]], acc);
  }
  M[(size_t)c * mstr + n] = acc;
}

// one thread per (parent of the level, output term): each entry's parent term
// is loaded once for all eight octants, and every child's output is added into it
__global__ void k_l2l_tab(int lo, int hi, int lsize, ShiftTab T, const unsigned char *child_mask,
                          const int *child_first, float *L, int lstr) {
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int p = lo + (int)(g / lsize), n = (int)(g % lsize);
  if (p >= hi) return;
  const unsigned mask = child_mask[p];
  if (!mask) return;
  const float *Lp = L + (size_t)p * lstr;
  float a[8];
#pragma unroll
  for (int o = 0; o < 8; o++) a[o] = 0.f;
  for (int e = T.off[n]; e < T.off[n + 1]; e++) {
    const float x = Lp[T.in[e]];
    const float4 c0 = T.coef8[2 * e], c1 = T.coef8[2 * e + 1];
    a[0] = fmaf(c0.x, x, a[0]); a[1] = fmaf(c0.y, x, a[1]); a[2] = fmaf(c0.z, x, a[2]); a[3] = fmaf(c0.w, x, a[3]);
    a[4] = fmaf(c1.x, x, a[4]); a[5] = fmaf(c1.y, x, a[5]); a[6] = fmaf(c1.z, x, a[6]); a[7] = fmaf(c1.w, x, a[7]);
  }
  // children are stored in octant order after child_first
  int ch = child_first[p];
#pragma unroll
  for (int o = 0; o < 8; o++)
    if (mask & (1u << o)) L[(size_t)(ch++) * lstr + n] += a[o];
}

// L2L for the few parents of the upper levels, one warp per (parent, output
// term): the lanes split the term's entries and the warp sums them (a thread
// per term would walk up to NT(p) dependent entries alone).
__global__ void k_l2l_tab_warp(int lo, int hi, int lsize, ShiftTab T, const unsigned char *child_mask,
                               const int *child_first, float *L, int lstr) {
  const long g = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int p = lo + (int)(g / lsize), n = (int)(g % lsize);
  if (p >= hi) return;
  const unsigned mask = child_mask[p];
  if (!mask) return;
  const float *Lp = L + (size_t)p * lstr;
  float a[8];
#pragma unroll
  for (int o = 0; o < 8; o++) a[o] = 0.f;
  for (int e = T.off[n] + lane; e < T.off[n + 1]; e += 32) {
    const float x = Lp[T.in[e]];
    const float4 c0 = T.coef8[2 * e], c1 = T.coef8[2 * e + 1];
    a[0] = fmaf(c0.x, x, a[0]); a[1] = fmaf(c0.y, x, a[1]); a[2] = fmaf(c0.z, x, a[2]); a[3] = fmaf(c0.w, x, a[3]);
    a[4] = fmaf(c1.x, x, a[4]); a[5] = fmaf(c1.y, x, a[5]); a[6] = fmaf(c1.z, x, a[6]); a[7] = fmaf(c1.w, x, a[7]);
  }
#pragma unroll
  for (int o = 0; o < 8; o++)
    for (int d = 16; d; d >>= 1) a[o] += __shfl_xor_sync(0xffffffffu, a[o], d);
  if (lane == 0) {
    int ch = child_first[p];
#pragma unroll
    for (int o = 0; o < 8; o++)
      if (mask & (1u << o)) L[(size_t)(ch++) * lstr + n] += a[o];
  }
}

// levels with fewer parents than this use the warp-per-term L2L
constexpr int SHIFT_WARP_BELOW = 2048;

}  // namespace

bool fmm_shift_tab_supported(int p, int so) { return get_shift(p, so) != nullptr; }

int fmm_m2m_tab(DevTree *t, int lo, int hi, float *M, int mstr, cudaStream_t st) {
  const ShiftSet *S = get_shift(t->order, t->so);
  if (!S) return FMM_ERR_CUDA;
  const int msize = S->m2m.nout;
  const long n = (long)(hi - lo) * msize;
  if (n <= 0) return FMM_OK;
  fmm_note_launch(), k_m2m_tab<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      lo, hi, msize, S->m2m, t->child_mask.p, t->child_first.p, t->cx.p, t->cy.p, t->cz.p, M, mstr);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// L2L into the children [lo, hi) of one level, from their parents (the level above)
int fmm_l2l_tab(DevTree *t, int lo, int hi, float *L, int lstr, cudaStream_t st) {
  const ShiftSet *S = get_shift(t->order, t->so);
  if (!S) return FMM_ERR_CUDA;
  if (hi <= lo) return FMM_OK;
  // the parents of [lo, hi): the cells of the level above
  int l = 1;
  while (l < t->nlevels && t->level_off[l] != lo) l++;
  if (l >= t->nlevels) return FMM_ERR_STATE;
  const int plo = t->level_off[l - 1], phi = t->level_off[l];
  const int lsize = S->l2l.nout;
  const long n = (long)(phi - plo) * lsize;
  if (phi - plo < SHIFT_WARP_BELOW)
    fmm_note_launch(), k_l2l_tab_warp<<<(unsigned)((32 * n + 255) / 256), 256, 0, st>>>(
        plo, phi, lsize, S->l2l, t->child_mask.p, t->child_first.p, L, lstr);
  else
    fmm_note_launch(), k_l2l_tab<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(plo, phi, lsize, S->l2l,
                                                                            t->child_mask.p, t->child_first.p, L,
                                                                            lstr);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
