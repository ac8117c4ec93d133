// p2p.cu -- near-field particle-particle interactions (P2P) over the P2P list
// (P2P_Cells / evaluate_P2P_lazy, example/calculate.cpp:24-40, 208-216), in FP64
// and in the mixed-precision form, plus the per-evaluate FP32 staging.
#include "internal.h"

// ---------------------------------------------------------------------------
// P2P in FP64, one warp per target leaf (example/calculate.cpp:24-40, 208-216)
// ---------------------------------------------------------------------------
#define P2P_WARPS 4
__global__ void __launch_bounds__(32 * P2P_WARPS) k_p2p64(const int *leaf_cells, int nleaves, const int *pstart,
                                                          const int *pcount, const int *off_, const int *src,
                                                          const double *px, const double *py, const double *pz,
                                                          const uint32_t *perm, const double *S, int so,
                                                          double *Fnear) {
  __shared__ double sx[P2P_WARPS][32], sy[P2P_WARPS][32], sz[P2P_WARPS][32], sq[P2P_WARPS][32][3];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int leaf = blockIdx.x * P2P_WARPS + w;
  if (leaf >= nleaves) return;
  const int A = leaf_cells[leaf];
  const int a0 = pstart[A], na = pcount[A];
  const int k0 = off_[A], k1 = off_[A + 1];
  for (int tb = 0; tb < na; tb += 32) {
    const int i = a0 + tb + lane;
    const bool ok = tb + lane < na;
    double xi = 0, yi = 0, zi = 0;
    if (ok) { xi = px[i]; yi = py[i]; zi = pz[i]; }
    double phi = 0, ex = 0, ey = 0, ez = 0;
    for (int k = k0; k < k1; k++) {
      const int B = src[k];
      const int b0 = pstart[B], nb = pcount[B];
      for (int sb = 0; sb < nb; sb += 32) {
        __syncwarp();
        int j = b0 + sb + lane;
        if (sb + lane < nb) {
          sx[w][lane] = px[j]; sy[w][lane] = py[j]; sz[w][lane] = pz[j];
          uint32_t o = perm[j];
          if (so == 0) sq[w][lane][0] = S[o];
          else { sq[w][lane][0] = S[3 * (size_t)o]; sq[w][lane][1] = S[3 * (size_t)o + 1]; sq[w][lane][2] = S[3 * (size_t)o + 2]; }
        }
        __syncwarp();
        const int cnt = min(32, nb - sb);
        if (ok) {
          for (int jj = 0; jj < cnt; jj++) {
            if (b0 + sb + jj == i) continue;  // l2 != l1
            double dx = xi - sx[w][jj], dy = yi - sy[w][jj], dz = zi - sz[w][jj];
            double r2 = dx * dx + dy * dy + dz * dz;
            double rinv = rsqrt(r2);
            double r3 = rinv * rinv * rinv;
            if (so == 0) {
              double q = sq[w][jj][0];
              phi += q * rinv;
              double qr3 = q * r3;
              ex += qr3 * dx; ey += qr3 * dy; ez += qr3 * dz;
            } else {
              double sxj = sq[w][jj][0], syj = sq[w][jj][1], szj = sq[w][jj][2];
              double sr = sxj * dx + syj * dy + szj * dz;
              double r5 = 3.0 * sr * r3 * rinv * rinv;
              phi -= sr * r3;
              ex += sxj * r3 - r5 * dx; ey += syj * r3 - r5 * dy; ez += szj * r3 - r5 * dz;
            }
          }
        }
      }
    }
    if (ok) {
      Fnear[4 * (size_t)i] = phi; Fnear[4 * (size_t)i + 1] = ex;
      Fnear[4 * (size_t)i + 2] = ey; Fnear[4 * (size_t)i + 3] = ez;
    }
  }
}

// ---------------------------------------------------------------------------

// Per evaluate: positions as two-float offsets from the leaf centre (hi in .xyz,
// the charge in .w) plus the low parts; dipole moments in FP32.
__global__ void k_stage_particles(const int *leaf_cells, int nleaves, const int *pstart, const int *pcount,
                                  const double *cx, const double *cy, const double *cz, const double *px,
                                  const double *py, const double *pz, const uint32_t *perm, const double *S, int so,
                                  float4 *phi4, float4 *plo4, float4 *sdip) {
  int leaf = blockIdx.x;
  if (leaf >= nleaves) return;
  int c = leaf_cells[leaf];
  for (int j = threadIdx.x; j < pcount[c]; j += blockDim.x) {
    int i = pstart[c] + j;
    double dx = px[i] - cx[c], dy = py[i] - cy[c], dz = pz[i] - cz[c];
    float hx = (float)dx, hy = (float)dy, hz = (float)dz;
    uint32_t o = perm[i];
    phi4[i] = make_float4(hx, hy, hz, so == 0 ? (float)S[o] : 0.f);
    plo4[i] = make_float4((float)(dx - (double)hx), (float)(dy - (double)hy), (float)(dz - (double)hz), 0.f);
    if (so) sdip[i] = make_float4((float)S[3 * (size_t)o], (float)S[3 * (size_t)o + 1], (float)S[3 * (size_t)o + 2], 0.f);
  }
}


// ---------------------------------------------------------------------------
// P2P in FP32 with compensated accumulation (mixed precision)
// ---------------------------------------------------------------------------
// One warp per target leaf, in chunks of up to 32 target particles.  A chunk of
// m targets uses f = the largest power of two with f*m <= 32 lanes per target,
// each lane taking every f-th source, so a small chunk (a leaf's last few
// particles) does not leave most lanes idle; the f partial sums of a target are
// combined with shuffles.  Positions are two-float offsets from the particle's
// own leaf centre; the offset between the two leaf centres is formed exactly
// from integer cell coordinates, so the displacement keeps ~1e-7 relative
// accuracy even for very close pairs.  Each source leaf's contribution is
// summed in FP32 and folded into a Kahan-compensated FP32 total; the final
// per-particle near + far sum is FP64 (k_finalize).  1/R is the hardware
// approximation (relative error ~1e-7, the size of the FP32 displacement's own
// rounding; measured: 2.3880e-6 field error against 2.3846e-6 for the FP64
// pass at 10^6 charges, p = 8, and 1.645e-6 against 1.619e-6 for 2x10^6
// Plummer dipoles, p = 6).  The potential is summed only when it is an output.
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
  float y = v - c;
  float t = s + y;
  c = (t - s) - y;
  s = t;
}
// Two-float leaf-pair offset: c_A - c_B = d * s_L exactly as (hi, lo), with d
// the integer offset of the centres in half-widths of the finer level L.
__device__ __forceinline__ void offset2(int d, float2 sc, float &hi, float &lo) {
  float df = (float)d;
  hi = df * sc.x;
  lo = fmaf(df, sc.x, -hi) + df * sc.y;
}
// t = (a_hi + a_lo) + (o_hi + o_lo) as (hi, lo), exact two-sum on the high parts
__device__ __forceinline__ void add2(float ah, float al, float oh, float ol, float &th, float &tl) {
  th = ah + oh;
  float bv = th - ah;
  tl = ((ah - (th - bv)) + (oh - bv)) + (al + ol);
}

template <bool SELF, bool POT>
__device__ __forceinline__ void coulomb_one(const float4 &q, const float4 &ql, bool self, float txh, float txl,
                                            float tyh, float tyl, float tzh, float tzl, float &phi, float &ex,
                                            float &ey, float &ez) {
  const float dx = (txh - q.x) + (txl - ql.x);
  const float dy = (tyh - q.y) + (tyl - ql.y);
  const float dz = (tzh - q.z) + (tzl - ql.z);
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  float rinv = rsqrt_approx(r2);
  if (SELF) rinv = self ? 0.f : rinv;  // l2 != l1
  const float qr = q.w * rinv;
  const float qr3 = qr * (rinv * rinv);
  if (POT) phi += qr;
  ex = fmaf(qr3, dx, ex);
  ey = fmaf(qr3, dy, ey);
  ez = fmaf(qr3, dz, ez);
}

// Sources first, first + step, ... < cnt of the staged chunk.  With one lane
// per target (step 1) the loop runs in blocks of 8 with constant shared-memory
// offsets, so nothing but the interaction itself sits in the loop body.
template <bool SELF, bool POT>
__device__ __forceinline__ void p2p_coulomb(const float4 *sh, const float4 *sl, int first, int cnt, int step,
                                            int selfj, float txh, float txl, float tyh, float tyl, float tzh,
                                            float tzl, float &phi, float &ex, float &ey, float &ez) {
  if (step == 1) {
    int jj = 0;
    for (; jj + 8 <= cnt; jj += 8) {
#pragma unroll
      for (int u = 0; u < 8; u++)
        coulomb_one<SELF, POT>(sh[jj + u], sl[jj + u], jj + u == selfj, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey,
                               ez);
    }
    for (; jj < cnt; jj++)
      coulomb_one<SELF, POT>(sh[jj], sl[jj], jj == selfj, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey, ez);
    return;
  }
#pragma unroll 4
  for (int jj = first; jj < cnt; jj += step)
    coulomb_one<SELF, POT>(sh[jj], sl[jj], jj == selfj, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey, ez);
}

template <bool SELF>
__device__ __forceinline__ void p2p_dipole(const float4 *sh, const float4 *sl, const float4 *sd, int first, int cnt,
                                           int step, int selfj, float txh, float txl, float tyh, float tyl,
                                           float tzh, float tzl, float &phi, float &ex, float &ey, float &ez) {
  for (int jj = first; jj < cnt; jj += step) {
    const float4 q = sh[jj];
    const float4 ql = sl[jj];
    const float4 d = sd[jj];
    const float dx = (txh - q.x) + (txl - ql.x);
    const float dy = (tyh - q.y) + (tyl - ql.y);
    const float dz = (tzh - q.z) + (tzl - ql.z);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float rinv = rsqrt_approx(r2);
    if (SELF) rinv = (jj == selfj) ? 0.f : rinv;
    const float r3 = rinv * rinv * rinv;
    const float sr = fmaf(d.x, dx, fmaf(d.y, dy, d.z * dz));
    const float r5 = 3.f * sr * r3 * rinv * rinv;
    phi -= sr * r3;
    ex += d.x * r3 - r5 * dx;
    ey += d.y * r3 - r5 * dy;
    ez += d.z * r3 - r5 * dz;
  }
}

template <bool POT, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_p2p32(const int *leaf_cells, int nleaves, const int *pstart,
                                                          const int *pcount, const int *off_, const int *src,
                                                          const int *ix, const int *iy, const int *iz,
                                                          const unsigned char *clevel, const float2 *crf,
                                                          const float4 *phi4, const float4 *plo4,
                                                          const float4 *sdip, int so, double *Fnear) {
  __shared__ float4 sh[WARPS][32], sl[WARPS][32], sd[WARPS][32];
  const unsigned FULL = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int leaf = blockIdx.x * WARPS + w;
  if (leaf >= nleaves) return;
  const int A = leaf_cells[leaf];
  const int a0 = pstart[A], na = pcount[A];
  const int k0 = off_[A], k1 = off_[A + 1];
  const int la = clevel[A], iax = 2 * ix[A] + 1, iay = 2 * iy[A] + 1, iaz = 2 * iz[A] + 1;
  for (int tb = 0; tb < na; tb += 32) {
    const int m = min(32, na - tb);
    int lf = 0;  // f = 2^lf lanes per target
    while ((2 << lf) * m <= 32) lf++;
    const int f = 1 << lf;
    const int tl = lane >> lf, slice = lane & (f - 1);
    const bool ok = tl < m;
    const int i = a0 + tb + (ok ? tl : 0);
    const float4 th = phi4[i], tlo = plo4[i];
    float s0 = 0, s1 = 0, s2 = 0, s3 = 0, c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int k = k0; k < k1; k++) {
      const int B = src[k];
      const int b0 = pstart[B], nb = pcount[B];
      const int lb = clevel[B], L = max(la, lb);
      const float2 sc = crf[la >= lb ? A : B];  // half-width at the finer level L
      float oxh, oxl, oyh, oyl, ozh, ozl;
      offset2((iax << (L - la)) - ((2 * ix[B] + 1) << (L - lb)), sc, oxh, oxl);
      offset2((iay << (L - la)) - ((2 * iy[B] + 1) << (L - lb)), sc, oyh, oyl);
      offset2((iaz << (L - la)) - ((2 * iz[B] + 1) << (L - lb)), sc, ozh, ozl);
      float txh, txl, tyh, tyl, tzh, tzl;
      add2(th.x, tlo.x, oxh, oxl, txh, txl);
      add2(th.y, tlo.y, oyh, oyl, tyh, tyl);
      add2(th.z, tlo.z, ozh, ozl, tzh, tzl);
      float phi = 0, ex = 0, ey = 0, ez = 0;
      for (int sb = 0; sb < nb; sb += 32) {
        __syncwarp();
        const int j = b0 + sb + lane;
        if (sb + lane < nb) {
          sh[w][lane] = phi4[j];
          sl[w][lane] = plo4[j];
          if (so) sd[w][lane] = sdip[j];
        }
        __syncwarp();
        const int cnt = min(32, nb - sb);
        if (so == 0) {
          if (B == A)
            p2p_coulomb<true, POT>(sh[w], sl[w], slice, cnt, f, i - (b0 + sb), txh, txl, tyh, tyl, tzh, tzl, phi, ex,
                                   ey, ez);
          else
            p2p_coulomb<false, POT>(sh[w], sl[w], slice, cnt, f, -1, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey, ez);
        } else {
          if (B == A)
            p2p_dipole<true>(sh[w], sl[w], sd[w], slice, cnt, f, i - (b0 + sb), txh, txl, tyh, tyl, tzh, tzl, phi,
                             ex, ey, ez);
          else
            p2p_dipole<false>(sh[w], sl[w], sd[w], slice, cnt, f, -1, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey,
                              ez);
        }
      }
      kahan_add(s0, c0, phi); kahan_add(s1, c1, ex); kahan_add(s2, c2, ey); kahan_add(s3, c3, ez);
    }
    // combine the f lanes of each target in FP64
    double r0 = (double)s0 - (double)c0, r1 = (double)s1 - (double)c1;
    double r2 = (double)s2 - (double)c2, r3 = (double)s3 - (double)c3;
    for (int o = 1; o < f; o <<= 1) {
      r0 += __shfl_xor_sync(FULL, r0, o);
      r1 += __shfl_xor_sync(FULL, r1, o);
      r2 += __shfl_xor_sync(FULL, r2, o);
      r3 += __shfl_xor_sync(FULL, r3, o);
    }
    if (ok && slice == 0) {
      Fnear[4 * (size_t)i] = r0;
      Fnear[4 * (size_t)i + 1] = r1;
      Fnear[4 * (size_t)i + 2] = r2;
      Fnear[4 * (size_t)i + 3] = r3;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers used by eval.cu
// ---------------------------------------------------------------------------
int fmm_p2p_launch(DevTree *t, bool mixed, const double *S, cudaStream_t st, bool narrow) {
  const int nl = t->nleaves, so = t->so;
  if (mixed) {
    // narrow blocks (2 warps) when running beside the tensor-core M2L: three
    // fit in the registers its CTA leaves free, against one of 4 warps
    const bool pot = t->pass_potential || so;
    const int wp = narrow ? 2 : P2P_WARPS;
    auto k = narrow ? (pot ? k_p2p32<true, 2> : k_p2p32<false, 2>)
                    : (pot ? k_p2p32<true, P2P_WARPS> : k_p2p32<false, P2P_WARPS>);
    fmm_note_launch(), k<<<fmm_blocks(nl, wp), 32 * wp, 0, st>>>(
        t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->p2p_off.p, t->p2p_src.p, t->ix.p, t->iy.p, t->iz.p,
        t->clevel.p, t->crf.p, t->phi4.p, t->plo4.p, t->sdip.p, so, t->Fnear.p);
  } else {
    fmm_note_launch(), k_p2p64<<<fmm_blocks(nl, P2P_WARPS), 32 * P2P_WARPS, 0, st>>>(
        t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->p2p_off.p, t->p2p_src.p, t->px.p, t->py.p, t->pz.p,
        t->perm.p, S, so, t->Fnear.p);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

int fmm_stage_particles(DevTree *t, const double *S, cudaStream_t st) {
  fmm_note_launch(), k_stage_particles<<<t->nleaves, 128, 0, st>>>(
      t->leaf_cells.p, t->nleaves, t->pstart.p, t->pcount.p, t->cx.p, t->cy.p, t->cz.p, t->px.p, t->py.p, t->pz.p,
      t->perm.p, S, t->so, t->phi4.p, t->plo4.p, t->sdip.p);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
