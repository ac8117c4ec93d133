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
  __shared__ double sx[P2P_WARPS][32], sy[P2P_WARPS][32], sz[P2P_WARPS][32], sq[P2P_WARPS][32][6];
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
          else if (so == 1) { sq[w][lane][0] = S[3 * (size_t)o]; sq[w][lane][1] = S[3 * (size_t)o + 1]; sq[w][lane][2] = S[3 * (size_t)o + 2]; }
          else for (int k = 0; k < 6; k++) sq[w][lane][k] = S[6 * (size_t)o + k];
        }
        __syncwarp();
        const int cnt = min(32, nb - sb);
        if (ok) {
          for (int jj = 0; jj < cnt; jj++) {
            if (b0 + sb + jj == i) continue;  // l2 != l1
            double dx = xi - sx[w][jj], dy = yi - sy[w][jj], dz = zi - sz[w][jj];
            if (so == 2) {  // quadrupole sources
              quadrupole_p2p<double>(dx, dy, dz, sq[w][jj], phi, ex, ey, ez);
              continue;
            }
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

// Per evaluate: positions as two-float offsets from the particle's system root
// centre (hi in .xyz, the charge in .w; lo in .xyz, the particle's own index
// in .w for the self test); dipole moments in FP32.
__global__ void k_stage_particles(const int *leaf_cells, int nleaves, const int *pstart, const int *pcount,
                                  const int *csys, const double *roots, const double *px, const double *py,
                                  const double *pz, const uint32_t *perm, const double *S, int so, float4 *phi4,
                                  float4 *plo4, float4 *sdip) {
  int leaf = blockIdx.x;
  if (leaf >= nleaves) return;
  int c = leaf_cells[leaf];
  const double *root = roots + 4 * (size_t)csys[c];
  const double ox = root[0], oy = root[1], oz = root[2];
  for (int j = threadIdx.x; j < pcount[c]; j += blockDim.x) {
    int i = pstart[c] + j;
    double dx = px[i] - ox, dy = py[i] - oy, dz = pz[i] - oz;
    float hx = (float)dx, hy = (float)dy, hz = (float)dz;
    uint32_t o = perm[i];
    phi4[i] = make_float4(hx, hy, hz, so == 0 ? (float)S[o] : 0.f);
    plo4[i] = make_float4((float)(dx - (double)hx), (float)(dy - (double)hy), (float)(dz - (double)hz),
                          __int_as_float(i));
    if (so) sdip[i] = make_float4((float)S[3 * (size_t)o], (float)S[3 * (size_t)o + 1], (float)S[3 * (size_t)o + 2], 0.f);
  }
}


// ---------------------------------------------------------------------------
// P2P in FP32 with compensated accumulation (mixed precision)
// ---------------------------------------------------------------------------
// One warp per target leaf, in chunks of up to 32 target particles.  The
// source particles of the leaf's P2P list are taken as one stream -- the
// concatenation of the source leaves' particle ranges, up to 32 leaves at a
// time -- and staged in full chunks of 32, so that the per-chunk work (finding
// each lane's source through a prefix sum of the leaves' counts, the staging
// copy, the compensated fold) is spread over 32 sources rather than one leaf's
// ~30.  A chunk of m targets uses f = the largest power of two with f*m <= 32
// lanes per target, each lane taking every f-th source, so a small chunk (a
// leaf's last few particles) does not leave most lanes idle; the f partial sums
// of a target are combined with shuffles.
// Positions are two-float offsets from the system's root centre: the high
// parts of two nearby particles subtract exactly (Sterbenz) or with one
// rounding of the difference, and the low parts carry the rest, so the
// displacement keeps ~1e-7 relative accuracy even for very close pairs.  Each
// chunk's contribution is summed in FP32 and folded into a Kahan-compensated
// FP32 total; the final per-particle near + far sum is FP64 (k_finalize).
// 1/R is the hardware approximation (relative error ~1e-7, the size of the
// FP32 displacement's own rounding).  The potential is summed only when it is
// an output.
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

template <bool SELF, bool POT>
__device__ __forceinline__ void coulomb_one(const float4 &q, const float4 &ql, int i, float txh, float txl, float tyh,
                                            float tyl, float tzh, float tzl, float &phi, float &ex, float &ey,
                                            float &ez) {
  const float dx = (txh - q.x) + (txl - ql.x);
  const float dy = (tyh - q.y) + (tyl - ql.y);
  const float dz = (tzh - q.z) + (tzl - ql.z);
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  float rinv = rsqrt_approx(r2);
  if (SELF) rinv = __float_as_int(ql.w) == i ? 0.f : rinv;  // l2 != l1
  const float qr = q.w * rinv;
  const float qr3 = qr * (rinv * rinv);
  if (POT) phi += qr;
  ex = fmaf(qr3, dx, ex);
  ey = fmaf(qr3, dy, ey);
  ez = fmaf(qr3, dz, ez);
}

template <bool SELF>
__device__ __forceinline__ void dipole_one(const float4 &q, const float4 &ql, const float4 &d, int i, float txh,
                                           float txl, float tyh, float tyl, float tzh, float tzl, float &phi,
                                           float &ex, float &ey, float &ez) {
  const float dx = (txh - q.x) + (txl - ql.x);
  const float dy = (tyh - q.y) + (tyl - ql.y);
  const float dz = (tzh - q.z) + (tzl - ql.z);
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  float rinv = rsqrt_approx(r2);
  if (SELF) rinv = __float_as_int(ql.w) == i ? 0.f : rinv;
  const float r3 = rinv * rinv * rinv;
  const float sr = fmaf(d.x, dx, fmaf(d.y, dy, d.z * dz));
  const float r5 = 3.f * sr * r3 * rinv * rinv;
  phi -= sr * r3;
  ex += d.x * r3 - r5 * dx;
  ey += d.y * r3 - r5 * dy;
  ez += d.z * r3 - r5 * dz;
}

// ---- two sources per instruction (packed FP32x2) ----
// A full chunk with one lane per target (the common case) runs two sources at a
// time through add/sub/mul/fma.rn.f32x2: the same operations, in the same
// precision, as coulomb_one / dipole_one for each source of the pair, with half
// the instructions (the kernel is issue-bound).  Staged chunks are laid out for
// this: pair k of sources (2k, 2k+1) is four 16-byte words
//   X[k] = (xh, xh', yh, yh'), Z[k] = (zh, zh', q, q'),
//   XL[k] = (xl, xl', yl, yl'), ZL[k] = (zl, zl', index, index'),
// and for dipoles D[k] = (mx, mx', my, my'), DZ[k] = (mz, mz', -, -)
// (primes: source 2k + 1).
typedef unsigned long long u64;
__device__ __forceinline__ u64 padd(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 psub(u64 a, u64 b) {
  u64 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 pmul(u64 a, u64 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 pfma(u64 a, u64 b, u64 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ u64 pk2(float a, float b) {
  return ((u64)__float_as_uint(b) << 32) | (u64)__float_as_uint(a);
}
__device__ __forceinline__ float plo(u64 v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float phi_(u64 v) { return __uint_as_float((unsigned)(v >> 32)); }

// staged chunk of one warp (32 sources)
struct P2PStage {
  ulonglong2 X[16], Z[16], XL[16], ZL[16];
};
struct P2PStageD {
  ulonglong2 D[16], DZ[16];
};
__device__ __forceinline__ float *sf(ulonglong2 *a) { return (float *)a; }
__device__ __forceinline__ const float *sf(const ulonglong2 *a) { return (const float *)a; }

// the target's coordinates (hi, lo) duplicated into both halves
struct P2PTgt {
  u64 xh, xl, yh, yl, zh, zl;
};

template <bool SELF, bool POT>
__device__ __forceinline__ void coulomb_two(const P2PStage &sg, int k, int i, const P2PTgt &t, u64 &phi, u64 &ex,
                                            u64 &ey, u64 &ez) {
  const ulonglong2 X = sg.X[k], Z = sg.Z[k], XL = sg.XL[k], ZL = sg.ZL[k];
  const u64 dx = padd(psub(t.xh, X.x), psub(t.xl, XL.x));
  const u64 dy = padd(psub(t.yh, X.y), psub(t.yl, XL.y));
  const u64 dz = padd(psub(t.zh, Z.x), psub(t.zl, ZL.x));
  const u64 r2 = pfma(dx, dx, pfma(dy, dy, pmul(dz, dz)));
  float ra = rsqrt_approx(plo(r2)), rb = rsqrt_approx(phi_(r2));
  if (SELF) {  // l2 != l1
    ra = (int)(unsigned)ZL.y == i ? 0.f : ra;
    rb = (int)(unsigned)(ZL.y >> 32) == i ? 0.f : rb;
  }
  const u64 rinv = pk2(ra, rb);
  const u64 qr = pmul(Z.y, rinv);
  const u64 qr3 = pmul(qr, pmul(rinv, rinv));
  if (POT) phi = padd(phi, qr);
  ex = pfma(qr3, dx, ex);
  ey = pfma(qr3, dy, ey);
  ez = pfma(qr3, dz, ez);
}

template <bool SELF>
__device__ __forceinline__ void dipole_two(const P2PStage &sg, const P2PStageD &sd, int k, int i, const P2PTgt &t,
                                           u64 &phi, u64 &ex, u64 &ey, u64 &ez) {
  const ulonglong2 X = sg.X[k], Z = sg.Z[k], XL = sg.XL[k], ZL = sg.ZL[k], D = sd.D[k];
  const u64 mz = sd.DZ[k].x;
  const u64 dx = padd(psub(t.xh, X.x), psub(t.xl, XL.x));
  const u64 dy = padd(psub(t.yh, X.y), psub(t.yl, XL.y));
  const u64 dz = padd(psub(t.zh, Z.x), psub(t.zl, ZL.x));
  const u64 r2 = pfma(dx, dx, pfma(dy, dy, pmul(dz, dz)));
  float ra = rsqrt_approx(plo(r2)), rb = rsqrt_approx(phi_(r2));
  if (SELF) {
    ra = (int)(unsigned)ZL.y == i ? 0.f : ra;
    rb = (int)(unsigned)(ZL.y >> 32) == i ? 0.f : rb;
  }
  const u64 rinv = pk2(ra, rb);
  const u64 rr = pmul(rinv, rinv);
  const u64 r3 = pmul(rr, rinv);
  const u64 sr = pfma(D.x, dx, pfma(D.y, dy, pmul(mz, dz)));
  const u64 r5 = pmul(pmul(pmul(pk2(3.f, 3.f), sr), r3), rr);
  phi = psub(phi, pmul(sr, r3));
  ex = padd(ex, psub(pmul(D.x, r3), pmul(r5, dx)));
  ey = padd(ey, psub(pmul(D.y, r3), pmul(r5, dy)));
  ez = padd(ez, psub(pmul(mz, r3), pmul(r5, dz)));
}

// one source of the packed layout, for partial chunks
__device__ __forceinline__ void stage_get(const P2PStage &sg, int j, float4 &h, float4 &l) {
  const int o = 4 * (j >> 1) + (j & 1);
  const float *x = sf(sg.X) + o, *z = sf(sg.Z) + o, *xl = sf(sg.XL) + o, *zl = sf(sg.ZL) + o;
  h = make_float4(x[0], x[2], z[0], z[2]);
  l = make_float4(xl[0], xl[2], zl[0], zl[2]);
}
__device__ __forceinline__ float4 stage_getd(const P2PStageD &sd, int j) {
  const int o = 4 * (j >> 1) + (j & 1);
  const float *d = sf(sd.D) + o, *dz = sf(sd.DZ) + o;
  return make_float4(d[0], d[2], dz[0], 0.f);
}

// Sources first, first + step, ... < cnt of the staged chunk.
template <bool SELF, bool POT, int SO>
__device__ __forceinline__ void p2p_chunk(const P2PStage &sg, const P2PStageD &sd, int first, int cnt, int step,
                                          int i, const P2PTgt &t, float txh, float txl, float tyh, float tyl,
                                          float tzh, float tzl, float &phi, float &ex, float &ey, float &ez) {
  if (step == 1 && cnt == 32) {
    u64 p2 = 0, x2 = 0, y2 = 0, z2 = 0;
#pragma unroll 4
    for (int k = 0; k < 16; k++) {
      if (SO == 0)
        coulomb_two<SELF, POT>(sg, k, i, t, p2, x2, y2, z2);
      else
        dipole_two<SELF>(sg, sd, k, i, t, p2, x2, y2, z2);
    }
    if (POT || SO) phi += plo(p2) + phi_(p2);
    ex += plo(x2) + phi_(x2);
    ey += plo(y2) + phi_(y2);
    ez += plo(z2) + phi_(z2);
    return;
  }
#pragma unroll 4
  for (int jj = first; jj < cnt; jj += step) {
    float4 h, l;
    stage_get(sg, jj, h, l);
    if (SO == 0)
      coulomb_one<SELF, POT>(h, l, i, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey, ez);
    else
      dipole_one<SELF>(h, l, stage_getd(sd, jj), i, txh, txl, tyh, tyl, tzh, tzl, phi, ex, ey, ez);
  }
}

// The near field of target leaf A by one warp (sg, sd: its staging area).
template <bool POT, int SO>
__device__ __forceinline__ void p2p_leaf(int A, const int *pstart, const int *pcount, const int *off_,
                                         const int *src, const float4 *phi4, const float4 *plo4,
                                         const float4 *sdip, P2PStage &sg, P2PStageD &sd, double *Fnear) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int a0 = pstart[A], na = pcount[A];
  const int k0 = off_[A], k1 = off_[A + 1];
  const int sk = 4 * (lane >> 1) + (lane & 1);  // this lane's slot when it stages source `lane` of a chunk
  for (int tb = 0; tb < na; tb += 32) {
    const int m = min(32, na - tb);
    int lf = 0;  // f = 2^lf lanes per target
    while ((2 << lf) * m <= 32) lf++;
    const int f = 1 << lf;
    const int tl = lane >> lf, slice = lane & (f - 1);
    const bool ok = tl < m;
    const int i = a0 + tb + (ok ? tl : 0);
    const float4 th = phi4[i], tlo = plo4[i];
    const P2PTgt tg = {pk2(th.x, th.x), pk2(tlo.x, tlo.x), pk2(th.y, th.y),
                       pk2(tlo.y, tlo.y), pk2(th.z, th.z), pk2(tlo.z, tlo.z)};
    float s0 = 0, s1 = 0, s2 = 0, s3 = 0, c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int kb = k0; kb < k1; kb += 32) {
      // up to 32 source leaves: lane q holds leaf kb + q's particle range and
      // the exclusive prefix of the counts (its offset in the stream)
      const int nbat = min(32, k1 - kb);
      int B = -1, start = 0, cnt = 0;
      if (lane < nbat) {
        B = src[kb + lane];
        start = pstart[B];
        cnt = pcount[B];
      }
      int incl = cnt;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += v;
      }
      const int excl = incl - cnt;
      const int total = __shfl_sync(FULL, incl, 31);
      // the target leaf's own range in the stream (self pairs skip i == j)
      const unsigned selfq = __ballot_sync(FULL, B == A);
      const int self_lo = selfq ? __shfl_sync(FULL, excl, __ffs(selfq) - 1) : -1;
      for (int cb = 0; cb < total; cb += 32) {
        // the lane's source: the last leaf q whose stream offset is <= s
        const int s = cb + lane;
        int q = 0;
#pragma unroll
        for (int stp = 16; stp; stp >>= 1) {
          const int cand = q + stp;
          const int v = __shfl_sync(FULL, excl, cand & 31);
          if (cand < nbat && v <= s) q = cand;
        }
        const int jb = __shfl_sync(FULL, start, q), je = __shfl_sync(FULL, excl, q);
        __syncwarp();
        if (s < total) {
          const int j = jb + (s - je);
          const float4 h = phi4[j], l = plo4[j];
          sf(sg.X)[sk] = h.x; sf(sg.X)[sk + 2] = h.y;
          sf(sg.Z)[sk] = h.z; sf(sg.Z)[sk + 2] = h.w;
          sf(sg.XL)[sk] = l.x; sf(sg.XL)[sk + 2] = l.y;
          sf(sg.ZL)[sk] = l.z; sf(sg.ZL)[sk + 2] = l.w;
          if (SO) {
            const float4 d = sdip[j];
            sf(sd.D)[sk] = d.x; sf(sd.D)[sk + 2] = d.y;
            sf(sd.DZ)[sk] = d.z;
          }
        }
        __syncwarp();
        const int n = min(32, total - cb);
        const bool self = self_lo >= 0 && self_lo < cb + n && self_lo + na > cb;
        float phi = 0, ex = 0, ey = 0, ez = 0;
        if (self)
          p2p_chunk<true, POT, SO>(sg, sd, slice, n, f, i, tg, th.x, tlo.x, th.y, tlo.y, th.z, tlo.z, phi, ex, ey,
                                   ez);
        else
          p2p_chunk<false, POT, SO>(sg, sd, slice, n, f, i, tg, th.x, tlo.x, th.y, tlo.y, th.z, tlo.z, phi, ex, ey,
                                    ez);
        if (POT) kahan_add(s0, c0, phi);
        kahan_add(s1, c1, ex); kahan_add(s2, c2, ey); kahan_add(s3, c3, ez);
      }
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

template <bool POT, int WARPS, int SO>
__global__ void __launch_bounds__(32 * WARPS) k_p2p32(const int *leaf_cells, int nleaves, const int *pstart,
                                                      const int *pcount, const int *off_, const int *src,
                                                      const float4 *phi4, const float4 *plo4, const float4 *sdip,
                                                      double *Fnear) {
  __shared__ P2PStage sg[WARPS];
  __shared__ P2PStageD sd[SO ? WARPS : 1];
  const int w = threadIdx.x >> 5;
  const int leaf = blockIdx.x * WARPS + w;
  if (leaf < nleaves)
    p2p_leaf<POT, SO>(leaf_cells[leaf], pstart, pcount, off_, src, phi4, plo4, sdip, sg[w], sd[SO ? w : 0], Fnear);
}

// ---------------------------------------------------------------------------
// launchers used by eval.cu
// ---------------------------------------------------------------------------
int fmm_p2p_launch(DevTree *t, bool mixed, const double *S, cudaStream_t st, bool narrow) {
  const int nl = t->nleaves, so = t->so;
  if (mixed && so <= 1) {  // quadrupole sources take the FP64 kernel in every precision
    // narrow blocks (2 warps) when running beside the tensor-core M2L: they
    // fit in the registers its CTA leaves free
    const bool pot = t->pass_potential || so;
    const int wp = narrow ? 2 : P2P_WARPS;
    decltype(&k_p2p32<true, 2, 0>) k;
    if (so)
      k = narrow ? k_p2p32<true, 2, 1> : k_p2p32<true, P2P_WARPS, 1>;
    else
      k = narrow ? (pot ? k_p2p32<true, 2, 0> : k_p2p32<false, 2, 0>)
                 : (pot ? k_p2p32<true, P2P_WARPS, 0> : k_p2p32<false, P2P_WARPS, 0>);
    const unsigned grid = fmm_blocks(nl, wp);
    if (int rc = fmm_mark_kernel(t, 2, st)) return rc;
    fmm_note_launch(), k<<<grid, 32 * wp, 0, st>>>(t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->p2p_off.p,
                                                   t->p2p_src.p, t->phi4.p, t->plo4.p, t->sdip.p, t->Fnear.p);
  } else {
    if (int rc = fmm_mark_kernel(t, 2, st)) return rc;
    fmm_note_launch(), k_p2p64<<<fmm_blocks(nl, P2P_WARPS), 32 * P2P_WARPS, 0, st>>>(
        t->leaf_cells.p, nl, t->pstart.p, t->pcount.p, t->p2p_off.p, t->p2p_src.p, t->px.p, t->py.p, t->pz.p,
        t->perm.p, S, so, t->Fnear.p);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  return fmm_mark_kernel(t, 3, st);
}

int fmm_stage_particles(DevTree *t, const double *S, cudaStream_t st) {
  if (t->so > 1) return FMM_OK;  // the FP64 P2P reads the sources directly
  fmm_note_launch(), k_stage_particles<<<t->nleaves, 128, 0, st>>>(
      t->leaf_cells.p, t->nleaves, t->pstart.p, t->pcount.p, t->csys.p, t->roots.p, t->px.p, t->py.p, t->pz.p,
      t->perm.p, S, t->so, t->phi4.p, t->plo4.p, t->sdip.p);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
