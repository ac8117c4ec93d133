// tree.cu -- device octree build and interaction lists.
//
// Reproduces build_tree (example/tree.cpp:130-233) and interact_dehnen_lazy
// (example/calculate.cpp:81-133) bit-exactly, without the sequential insertion:
//  * build_tree's final partition does not depend on insertion order: a cell
//    is split iff it holds >= ncrit particles, a child exists iff a particle
//    falls in its octant, and each particle's octant path is fixed by FP64
//    comparisons against centres that depend only on the path.  So every
//    particle gets a 63-bit key of its 21 octant digits, computed with exactly
//    the reference's FP64 centre arithmetic (example/tree.cpp:94-98, 193), the
//    keys are radix-sorted, and the cells are cut level by level from the
//    sorted keys with the count rule.
//  * the dual-tree walk is run breadth-first over a frontier of cell pairs;
//    each pair's decision (MAC, P2P, split A, split B) depends only on the
//    pair, so the visited pairs -- and the M2L/P2P lists as multisets -- are
//    those of the recursive walk.
// All FP64 arithmetic that decides structure uses __d*_rn intrinsics so that no
// FMA contraction changes a rounding relative to the reference source.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include "internal.h"
#include "prims.cuh"
#include "deriv.cuh"

// ---------------------------------------------------------------------------
// root box (example/tree.cpp:139-187)
// ---------------------------------------------------------------------------
// The three sequential sums come from fmm_seqsum3 (seqsum.cu), bit-identical to
// the reference's loop; the maxima are order-independent.
size_t fmm_seqsum_scratch(long N);
int fmm_seqsum3(const double *pos, long N, double *out, void *scratch, cudaStream_t st);

__global__ void k_root_absmax(const double *__restrict__ pos, long N, const double *sums,
                              unsigned long long *mx) {
  double inv_n = (double)N;
  double ax = __ddiv_rn(sums[0], inv_n), ay = __ddiv_rn(sums[1], inv_n), az = __ddiv_rn(sums[2], inv_n);
  double mxx = 0, mxy = 0, mxz = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    mxx = fmax(mxx, fabs(__dsub_rn(pos[3 * i], ax)));
    mxy = fmax(mxy, fabs(__dsub_rn(pos[3 * i + 1], ay)));
    mxz = fmax(mxz, fabs(__dsub_rn(pos[3 * i + 2], az)));
  }
  for (int d = 16; d; d >>= 1) {
    mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, d));
    mxy = fmax(mxy, __shfl_xor_sync(0xffffffffu, mxy, d));
    mxz = fmax(mxz, __shfl_xor_sync(0xffffffffu, mxz, d));
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative doubles order like their bit patterns
    atomicMax(&mx[0], (unsigned long long)__double_as_longlong(mxx));
    atomicMax(&mx[1], (unsigned long long)__double_as_longlong(mxy));
    atomicMax(&mx[2], (unsigned long long)__double_as_longlong(mxz));
  }
}

// root[0..3] = centre, r; lev[2l] = r_l, lev[2l+1] = rmax_l = sqrt(3*r_l*r_l)
__global__ void k_root_final(const double *sums, const unsigned long long *mx, long N, double *root,
                             double *lev, float2 *levf) {
  double n = (double)N;
  double ax = __ddiv_rn(sums[0], n), ay = __ddiv_rn(sums[1], n), az = __ddiv_rn(sums[2], n);
  double xm = __longlong_as_double((long long)mx[0]);
  double ym = __longlong_as_double((long long)mx[1]);
  double zm = __longlong_as_double((long long)mx[2]);
  double r = __dmul_rn((xm > ym ? (xm > zm ? xm : zm) : (ym > zm ? ym : zm)), 1.001);
  root[0] = ax; root[1] = ay; root[2] = az; root[3] = r;
  double rl = r;
  for (int l = 0; l <= FMM_MAXLEVEL; l++) {
    lev[2 * l] = rl;
    lev[2 * l + 1] = __dsqrt_rn(__dmul_rn(__dmul_rn(3.0, rl), rl));  // example/tree.cpp:15
    float hi = (float)rl;
    levf[l] = make_float2(hi, (float)(rl - (double)hi));
    rl = __ddiv_rn(rl, 2.0);
  }
}

// ---------------------------------------------------------------------------
// per-particle octant keys (example/tree.cpp:94-98, 189-204)
// ---------------------------------------------------------------------------
// The digits of levels 1..nlev (the rest of the key is zero): the cells are cut
// from them, and the build asks for all FMM_MAXLEVEL levels only when a cell at
// level nlev still has to be split.
__global__ void k_keys(const double *__restrict__ pos, long N, const double *roots, const int *psys,
                       int nlev, uint64_t *keys, uint32_t *idx) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double *root = roots + 4 * (psys ? psys[i] : 0);  // the particle's system's root cube
  double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
  double cx = root[0], cy = root[1], cz = root[2], r = root[3];
  uint64_t key = 0;
#pragma unroll 3
  for (int l = 0; l < nlev; l++) {
    int oct = (x > cx) + ((y > cy) << 1) + ((z > cz) << 2);
    key = (key << 3) | (uint64_t)oct;
    // r / 2.0 and r * (+-1) are exact: halving and a sign select round identically
    r = __dmul_rn(r, 0.5);
    cx = __dadd_rn(cx, (oct & 1) ? r : -r);
    cy = __dadd_rn(cy, (oct & 2) ? r : -r);
    cz = __dadd_rn(cz, (oct & 4) ? r : -r);
  }
  keys[i] = key << (3 * (FMM_MAXLEVEL - nlev));
  idx[i] = (uint32_t)i;
}

__global__ void k_gather_pos(const double *__restrict__ pos, const uint32_t *perm, long N, double *px,
                             double *py, double *pz) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  uint32_t j = perm[i];
  px[i] = pos[3 * (size_t)j];
  py[i] = pos[3 * (size_t)j + 1];
  pz[i] = pos[3 * (size_t)j + 2];
}

// ---------------------------------------------------------------------------
// level-by-level cell construction
// ---------------------------------------------------------------------------
__device__ __forceinline__ int digit_at(uint64_t key, int level /*1..21*/) {
  return (int)((key >> (3 * (FMM_MAXLEVEL - level))) & 7u);
}
// first index in [lo, hi) whose level-`level` digit is >= d (digits are sorted there)
__device__ __forceinline__ int lower_digit(const uint64_t *keys, int lo, int hi, int level, int d) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (digit_at(keys[mid], level) < d) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// half-width r of a cell, its rmax = sqrt(3 r r) as the reference computes it
// (example/tree.cpp:15), and r as an FP32 (hi, lo) pair
__device__ __forceinline__ void set_radius(int c, double r, double *cr, double *crmax, float2 *crf) {
  cr[c] = r;
  crmax[c] = __dsqrt_rn(__dmul_rn(__dmul_rn(3.0, r), r));
  const float hi = (float)r;
  crf[c] = make_float2(hi, (float)(r - (double)hi));
}

// Level 0: one root cell per system; in sorted order system s holds the
// particles [sys_off[s], sys_off[s + 1]).
__global__ void k_init_roots(int nsys, const double *roots, const long *sys_off, double *cx, double *cy,
                             double *cz, uint64_t *cid, int *ix, int *iy, int *iz, int *pstart, int *pcount,
                             int *parent, int *child_first, unsigned char *child_mask, unsigned char *clevel,
                             double *cr, double *crmax, float2 *crf, int *csys) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const double *rt = roots + 4 * s;
  cx[s] = rt[0]; cy[s] = rt[1]; cz[s] = rt[2];
  cid[s] = 1; ix[s] = iy[s] = iz[s] = 0;
  pstart[s] = (int)sys_off[s]; pcount[s] = (int)(sys_off[s + 1] - sys_off[s]);
  parent[s] = -1; child_first[s] = -1; child_mask[s] = 0; clevel[s] = 0;
  set_radius(s, rt[3], cr, crmax, crf);
  csys[s] = s;
}

// ---------------------------------------------------------------------------
// forests: per-system root cubes (example/tree.cpp:139-187 for each system)
// ---------------------------------------------------------------------------
__global__ void k_fill_psys(const long *sys_off, int *psys) {
  const int s = blockIdx.x;
  for (long i = sys_off[s] + threadIdx.x; i < sys_off[s + 1]; i += blockDim.x) psys[i] = s;
}
// The reference's three sequential FP64 sums, one thread per (system, axis).
__global__ void k_seg_sums(const double *pos, const long *sys_off, int nsys, double *sums) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * nsys) return;
  const int s = t / 3, ax = t - 3 * s;
  double acc = 0.0;
  const long e = sys_off[s + 1];
  for (long i = sys_off[s]; i < e; i++) acc = __dadd_rn(acc, pos[3 * i + ax]);
  sums[t] = acc;
}
// max |x - mean| per system and axis (order-independent), one block per system
__global__ void k_seg_absmax(const double *pos, const long *sys_off, const double *sums, unsigned long long *mx) {
  const int s = blockIdx.x;
  const long b = sys_off[s], e = sys_off[s + 1];
  const double n = (double)(e - b);
  const double ax = __ddiv_rn(sums[3 * s], n), ay = __ddiv_rn(sums[3 * s + 1], n), az = __ddiv_rn(sums[3 * s + 2], n);
  double m0 = 0, m1 = 0, m2 = 0;
  for (long i = b + threadIdx.x; i < e; i += blockDim.x) {
    m0 = fmax(m0, fabs(__dsub_rn(pos[3 * i], ax)));
    m1 = fmax(m1, fabs(__dsub_rn(pos[3 * i + 1], ay)));
    m2 = fmax(m2, fabs(__dsub_rn(pos[3 * i + 2], az)));
  }
  for (int d = 16; d; d >>= 1) {
    m0 = fmax(m0, __shfl_xor_sync(0xffffffffu, m0, d));
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, d));
    m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, d));
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative doubles order like their bit patterns
    atomicMax(&mx[3 * s], (unsigned long long)__double_as_longlong(m0));
    atomicMax(&mx[3 * s + 1], (unsigned long long)__double_as_longlong(m1));
    atomicMax(&mx[3 * s + 2], (unsigned long long)__double_as_longlong(m2));
  }
}
__global__ void k_seg_root_final(int nsys, const long *sys_off, const double *sums, const unsigned long long *mx,
                                 double *roots) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const double n = (double)(sys_off[s + 1] - sys_off[s]);
  const double ax = __ddiv_rn(sums[3 * s], n), ay = __ddiv_rn(sums[3 * s + 1], n), az = __ddiv_rn(sums[3 * s + 2], n);
  const double xm = __longlong_as_double((long long)mx[3 * s]);
  const double ym = __longlong_as_double((long long)mx[3 * s + 1]);
  const double zm = __longlong_as_double((long long)mx[3 * s + 2]);
  roots[4 * s] = ax; roots[4 * s + 1] = ay; roots[4 * s + 2] = az;
  roots[4 * s + 3] = __dmul_rn((xm > ym ? (xm > zm ? xm : zm) : (ym > zm ? ym : zm)), 1.001);
}
// sorted position -> system, for the stable sort by system after the key sort
__global__ void k_sorted_sys(const uint32_t *perm, const int *psys, long N, uint32_t *ks, uint32_t *idx) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  ks[i] = (uint32_t)psys[perm[i]];
  idx[i] = (uint32_t)i;
}
__global__ void k_apply_order(const uint32_t *idx, long N, const uint64_t *kin, const uint32_t *pin, uint64_t *kout,
                              uint32_t *pout) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  kout[i] = kin[idx[i]];
  pout[i] = pin[idx[i]];
}

// One warp per cell of the level: lane o (1..7) finds where digit o starts in
// the cell's sorted keys, so the eight child ranges come from seven searches
// side by side; bnd[9 (c - lo) + o] = first particle of child o (bnd[.. + 8] = end).
__global__ void k_count_children(int lo, int hi, int level, int nlev, long ncrit, const uint64_t *keys,
                                 const int *pstart, const int *pcount, unsigned char *child_mask, uint32_t *cnt,
                                 int *bnd, uint32_t *eflags) {
  const int c = lo + (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (c >= hi) return;
  const int s = pstart[c], e = s + pcount[c];
  const bool split = pcount[c] >= ncrit && level < nlev;
  int b = lane == 0 ? s : e;
  if (split && lane >= 1 && lane <= 7) b = lower_digit(keys, s, e, level + 1, lane);
  if (lane <= 8) bnd[9 * (c - lo) + lane] = b;
  // child o holds [bnd[o], bnd[o + 1])
  const int nb = __shfl_down_sync(0xffffffffu, b, 1);
  const unsigned mask = __ballot_sync(0xffffffffu, split && lane < 8 && nb > b) & 0xffu;
  if (lane == 0) {
    if (pcount[c] >= ncrit && level >= nlev)  // no digits below: give up, or ask for all levels
      atomicOr(eflags, nlev >= FMM_MAXLEVEL ? FMM_EFLAG_DEPTH : FMM_EFLAG_KEYS);
    child_mask[c] = (unsigned char)mask;
    cnt[c - lo] = (uint32_t)__popc(mask);
  }
}

// One warp per cell: lane o writes child o, when it exists.
__global__ void k_write_children(int lo, int hi, int level, const uint32_t *off, const int *bnd, double *cx,
                                 double *cy, double *cz, uint64_t *cid, int *ix, int *iy, int *iz, int *pstart,
                                 int *pcount, int *parent, int *child_first, const unsigned char *child_mask_in,
                                 unsigned char *child_mask, unsigned char *clevel, double *cr, double *crmax,
                                 float2 *crf, int *csys) {
  const int c = lo + (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), o = threadIdx.x & 31;
  if (c >= hi) return;
  const unsigned mask = child_mask_in[c];
  const int first = hi + (int)off[c - lo];
  if (o == 0) child_first[c] = mask ? first : -1;
  if (o >= 8 || !((mask >> o) & 1u)) return;
  const int j = first + __popc(mask & ((1u << o) - 1u));
  const double r = __ddiv_rn(cr[c], 2.0);  // child half-width = parent r / 2.0 (example/tree.cpp:95)
  const int b = bnd[9 * (c - lo) + o], nb = bnd[9 * (c - lo) + o + 1];
  // add_child (example/tree.cpp:95-98)
  cx[j] = __dadd_rn(cx[c], (o & 1) ? r : -r);
  cy[j] = __dadd_rn(cy[c], (o & 2) ? r : -r);
  cz[j] = __dadd_rn(cz[c], (o & 4) ? r : -r);
  cid[j] = (cid[c] << 3) | (uint64_t)o;
  ix[j] = 2 * ix[c] + (o & 1);
  iy[j] = 2 * iy[c] + ((o >> 1) & 1);
  iz[j] = 2 * iz[c] + (o >> 2);
  pstart[j] = b;
  pcount[j] = nb - b;
  parent[j] = c;
  child_first[j] = -1;
  child_mask[j] = 0;
  clevel[j] = (unsigned char)(level + 1);
  set_radius(j, r, cr, crmax, crf);
  csys[j] = csys[c];
}

__global__ void k_leaf_flags(int ncells, long ncrit, const int *pcount, uint32_t *flag) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncells) flag[c] = pcount[c] < ncrit ? 1u : 0u;
}
__global__ void k_leaf_compact(int ncells, long ncrit, const int *pcount, const uint32_t *off, int *leaf_cells,
                               int *cell_leaf) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  if (pcount[c] < ncrit) { leaf_cells[off[c]] = c; cell_leaf[c] = (int)off[c]; }
  else cell_leaf[c] = -1;
}

// ---------------------------------------------------------------------------
// dual-tree walk (example/calculate.cpp:81-133), breadth-first
// ---------------------------------------------------------------------------
#define WALK_BS 256
struct WalkCells {
  const double *cx, *cy, *cz, *crmax;
  const unsigned char *mask, *clevel;
  const int *child_first;
  const int *ix, *iy, *iz;
  const float *margin;  // per cell: relative band around the MAC boundary decided in FP64
  float theta2;
};

// The MAC  R*theta > rmax_A + rmax_B  (example/calculate.cpp:93) is first
// evaluated on the exact integer geometry of the two cells (centres on the
// level grid, rmax = sqrt(3)*r_level):  R^2 theta^2 / (rmax_A + rmax_B)^2 =
// |g_A - g_B|^2 theta^2 / (3 (2^(L-lA) + 2^(L-lB))^2)  with g the doubled
// integer coordinates at the finer level L.  Only when that ratio lies within
// `margin` of 1 -- where the rounding of the FP64 centres can matter -- is the
// reference's own FP64 expression evaluated, with the same roundings.
// Returns 0 = M2L, 1 = P2P, 2 = split A, 3 = split B.
__device__ __forceinline__ int walk_decide(const WalkCells &W, int A, int B, double theta) {
  const int la = W.clevel[A], lb = W.clevel[B], L = max(la, lb);
  const int sa = L - la, sb = L - lb;
  const long long gx = ((long long)(2 * W.ix[A] + 1) << sa) - ((long long)(2 * W.ix[B] + 1) << sb);
  const long long gy = ((long long)(2 * W.iy[A] + 1) << sa) - ((long long)(2 * W.iy[B] + 1) << sb);
  const long long gz = ((long long)(2 * W.iz[A] + 1) << sa) - ((long long)(2 * W.iz[B] + 1) << sb);
  const long long n2 = gx * gx + gy * gy + gz * gz;
  const long long base = (1ll << sa) + (1ll << sb);
  const float rho = (float)n2 * W.theta2 / (3.f * (float)(base * base));
  const float m = W.margin[la >= lb ? A : B];  // the band of the finer cell's level
  bool mac;
  if (rho > 1.f + m) mac = true;
  else if (rho < 1.f - m) mac = false;
  else {
    double dx = __dsub_rn(W.cx[A], W.cx[B]);
    double dy = __dsub_rn(W.cy[A], W.cy[B]);
    double dz = __dsub_rn(W.cz[A], W.cz[B]);
    double R = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    double ra = W.crmax[A], rb = W.crmax[B];
    mac = __dmul_rn(R, theta) > __dadd_rn(ra, rb);
  }
  if (mac) return 0;
  bool leafa = W.mask[A] == 0, leafb = W.mask[B] == 0;
  if (leafa && leafb) return 1;  // the nleaf >= ncrit leaf-leaf branch is unreachable
  if (leafb || (la <= lb && !leafa)) return 2;  // rmax_A >= rmax_B  <=>  lA <= lB
  return 3;
}

// margin of each cell, for pairs in which it is the finer cell: FP32 evaluation
// error plus a bound on how far FP64 centre rounding can move R relative to the
// cell half-width (from its system's root cube)
__global__ void k_cell_margins(int nc, const int *csys, const double *roots, const double *cr, double theta,
                               float *margin) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double *rt = roots + 4 * csys[c];
  const double cmax = fmax(fmax(fabs(rt[0]), fabs(rt[1])), fabs(rt[2])) + rt[3];
  const double s = cr[c];
  const double m = 1e-5 + 64.0 * ldexp(1.0, -52) * cmax / s * fmax(1.0, theta);
  margin[c] = s > 0 && m < 0.01 ? (float)m : 1e30f;  // 1e30: always decide in FP64
}

__global__ void k_root_pairs(int nsys, int *fa, int *fb) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) fa[s] = fb[s] = s;
}

// Output slots of a decided pair: one M2L pair, one P2P pair, or the split
// cell's children as new frontier pairs.
__device__ __forceinline__ U3 walk_slots(const WalkCells &W, int A, int B, int d) {
  U3 c{0u, 0u, 0u};
  if (d == 0) c.x = 1;
  else if (d == 1) c.y = 1;
  else c.z = __popc((unsigned)W.mask[d == 2 ? A : B]);
  return c;
}

// Decisions of the frontier pairs, and each block's slot totals (the per-pair
// slots are recomputed by k_walk_write, so only the block totals are scanned).
__global__ void __launch_bounds__(WALK_BS) k_walk_count(WalkCells W, const int *fa, const int *fb, uint32_t nf,
                                                        double theta, U3 *bsum, unsigned char *dec) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  U3 c{0u, 0u, 0u};
  if (i < nf) {
    const int A = fa[i], B = fb[i];
    const int d = walk_decide(W, A, B, theta);
    dec[i] = (unsigned char)d;
    c = walk_slots(W, A, B, d);
  }
  U3 tot;
  block_exclusive<U3>(c, &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// Writes each pair's outputs at its block's offset (boff, the scanned block
// totals) plus its rank in the block: the walk order of the sequential scan.
__global__ void __launch_bounds__(WALK_BS) k_walk_write(WalkCells W, const int *fa, const int *fb, uint32_t nf,
                                                        const unsigned char *dec, const U3 *boff, U3 base,
                                                        int *m2l_src, int *m2l_tgt, int *p2p_tgt, int *p2p_src,
                                                        int *na, int *nb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  int A = 0, B = 0, d = 0;
  U3 c{0u, 0u, 0u};
  if (i < nf) {
    A = fa[i];
    B = fb[i];
    d = dec[i];
    c = walk_slots(W, A, B, d);
  }
  U3 tot;
  const U3 o = boff[blockIdx.x] + block_exclusive<U3>(c, &tot);
  if (i >= nf) return;
  if (d == 0) {
    m2l_src[base.x + o.x] = B;
    m2l_tgt[base.x + o.x] = A;
  } else if (d == 1) {
    p2p_tgt[base.y + o.y] = A;
    p2p_src[base.y + o.y] = B;
  } else {
    int P = d == 2 ? A : B;
    unsigned m = W.mask[P];
    int ch = W.child_first[P];
    uint32_t k = o.z;
    for (int oc = 0; oc < 8; oc++) {
      if (!(m & (1u << oc))) continue;
      if (d == 2) { na[k] = ch; nb[k] = B; }
      else { na[k] = A; nb[k] = ch; }
      ch++; k++;
    }
  }
}

// ---------------------------------------------------------------------------
// grouping pairs by target cell
// ---------------------------------------------------------------------------
// sort key of a pair: target in the high bits, then (optionally) its class
template <typename K>
__global__ void k_pair_keys(const int *tgt, const int *cls, long n, int cbits, K *keys) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  K k = (K)(uint32_t)tgt[i] << cbits;
  if (cls) k |= (K)(uint32_t)cls[i];
  keys[i] = k;
}
// CSR offsets of pairs sorted by target (off[c] = first pair of target c,
// off[nc] = n), and the class of each sorted pair from the key's low bits.
template <typename K>
__global__ void k_csr_from_sorted(const K *keys, long n, int cbits, int nc, int *off, int *cls) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i > n) return;
  const int cur = i < n ? (int)(keys[i] >> cbits) : nc;
  const int prev = i > 0 ? (int)(keys[i - 1] >> cbits) : -1;
  for (int c = prev + 1; c <= cur; c++) off[c] = (int)i;
  if (cls && i < n) cls[i] = (int)(keys[i] & (((K)1 << cbits) - 1));
}

// ---------------------------------------------------------------------------
// M2L translation classes
// ---------------------------------------------------------------------------
// A pair (B -> A) with levels lA, lB is, up to the scale of A, fixed by
// (dlev = lB - lA, integer offset of the centres in half-widths of the finer
// level).  Classes are shared across levels.  The class key packs
// (dlev + 64, dx + 2^18, dy + 2^18, dz + 2^18) into 7 + 3 x 19 bits, so keys
// order lexicographically by (dlev, dx, dy, dz); class ids are the ranks of
// the distinct keys in that order.
#define CLS_EMPTY 0xffffffffffffffffull
#define CLS_LIM (1LL << 18)
__device__ __forceinline__ uint64_t pair_key(const int *ix, const int *iy, const int *iz, const unsigned char *clevel,
                                             int A, int B) {
  const int la = clevel[A], lb = clevel[B];
  const int L = la > lb ? la : lb;
  const int sa = L - la, sb = L - lb;
  const long long dx = ((2LL * ix[A] + 1) << sa) - ((2LL * ix[B] + 1) << sb);
  const long long dy = ((2LL * iy[A] + 1) << sa) - ((2LL * iy[B] + 1) << sb);
  const long long dz = ((2LL * iz[A] + 1) << sa) - ((2LL * iz[B] + 1) << sb);
  if (llabs(dx) >= CLS_LIM || llabs(dy) >= CLS_LIM || llabs(dz) >= CLS_LIM) return CLS_EMPTY;
  return ((uint64_t)(lb - la + 64) << 57) | ((uint64_t)(dx + CLS_LIM) << 38) | ((uint64_t)(dy + CLS_LIM) << 19) |
         (uint64_t)(dz + CLS_LIM);
}
__device__ __forceinline__ void key_decode(uint64_t k, int *key4) {
  key4[0] = (int)(k >> 57) - 64;
  key4[1] = (int)((long long)((k >> 38) & 0x7FFFF) - CLS_LIM);
  key4[2] = (int)((long long)((k >> 19) & 0x7FFFF) - CLS_LIM);
  key4[3] = (int)((long long)(k & 0x7FFFF) - CLS_LIM);
}
// slot sequence of a key in the open-addressing table (splitmix64 finalizer)
__device__ __forceinline__ uint32_t key_hash(uint64_t k) {
  k ^= k >> 30;
  k *= 0xBF58476D1CE4E5B9ull;
  k ^= k >> 27;
  k *= 0x94D049BB133111EBull;
  k ^= k >> 31;
  return (uint32_t)k;
}
__device__ __forceinline__ long key_find(const uint64_t *tab, uint32_t mask, uint64_t k) {
  uint32_t h = key_hash(k) & mask;
  for (uint32_t probe = 0; probe <= mask; probe++) {
    const uint64_t cur = tab[h];
    if (cur == k) return h;
    if (cur == CLS_EMPTY) return -1;
    h = (h + 1) & mask;
  }
  return -1;
}

// Class key of every pair, inserted into the table; stat[0] counts distinct
// keys, stat[1] flags a table that filled up.
__global__ void k_class_keys(const int *src, const int *tgt, long n, const int *ix, const int *iy, const int *iz,
                             const unsigned char *clevel, uint64_t *keys, uint64_t *tab, uint32_t mask,
                             uint32_t *stat, uint32_t *eflags) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = pair_key(ix, iy, iz, clevel, tgt[i], src[i]);
  keys[i] = k;
  if (k == CLS_EMPTY) {
    atomicOr(eflags, FMM_EFLAG_RANGE);
    return;
  }
  uint32_t h = key_hash(k) & mask;
  for (uint32_t probe = 0; probe <= mask; probe++) {
    uint64_t cur = tab[h];
    if (cur == CLS_EMPTY) {
      cur = atomicCAS((unsigned long long *)&tab[h], CLS_EMPTY, (unsigned long long)k);
      if (cur == CLS_EMPTY) {
        atomicAdd(&stat[0], 1u);
        return;
      }
    }
    if (cur == k) return;
    h = (h + 1) & mask;
  }
  atomicOr(&stat[1], 1u);
}

__global__ void k_class_collect(const uint64_t *tab, uint32_t nslots, uint64_t *uniq, uint32_t *idx,
                                uint32_t *counter) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots || tab[s] == CLS_EMPTY) return;
  const uint32_t r = atomicAdd(counter, 1u);
  uniq[r] = tab[s];
  idx[r] = r;
}

// ids by rank of the sorted distinct keys; the class table entry of each key
__global__ void k_class_rank(const uint64_t *uniq, int nu, const uint64_t *tab, uint32_t mask, int *tabval,
                             int *key4) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nu) return;
  const long s = key_find(tab, mask, uniq[r]);
  if (s >= 0) tabval[s] = r;
  key_decode(uniq[r], key4 + 4 * r);
}

// clears *same unless the two sorted key lists are equal
__global__ void k_keys_equal(const uint64_t *a, const uint64_t *b, int n, uint32_t *same) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && a[i] != b[i]) *same = 0;
}

__global__ void k_class_lookup(const uint64_t *keys, long n, const uint64_t *tab, uint32_t mask, const int *tabval,
                               int *cls) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long s = keys[i] == CLS_EMPTY ? -1 : key_find(tab, mask, keys[i]);
  cls[i] = s >= 0 ? tabval[s] : 0;  // out-of-range pairs were flagged when their keys were made
}

// Key per cell for the M2L processing order: (level, octant within the
// parent, parent index).  A cell's interaction list depends on which octant of
// its parent it is (the children of the parent's neighbours that pass the MAC),
// so grouping the cells of one level by octant, with parents in Morton order
// (cell indices are Morton order within a level), puts cells with
// near-identical class lists side by side: the 128-cell tiles of the tensor-core
// M2L then visit ~1.4x the classes of one list instead of ~3.5x in plain Morton
// order, and the warps of the CUDA-core M2L read the same operator rows.
// Cells are stored level by level in parent order, so a stable sort on
// (level, octant) alone keeps the parents in Morton order.
// grouping 1 keeps plain Morton order within a level (the key is the level alone).
__global__ void k_order_keys(int nc, const uint64_t *cid, const unsigned char *clevel, int grouping, uint64_t *key,
                             uint32_t *idx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  key[c] = ((uint64_t)clevel[c] << 56) | (grouping == 0 ? (cid[c] & 7u) << 48 : 0u);
  idx[c] = (uint32_t)c;
}

// Operator vector of a class: D_k(d / s_A), |k| <= p, in FP64 (one warp per class).
// (skipped when `same` is set: the vectors of the previous build still hold)
__global__ void k_class_derivs(const int *key4, int ncls, int p, double *D64, float *D32, const uint32_t *same) {
  __shared__ double sD[FMM_WARPS][FMM_NTMAX], sT[FMM_WARPS][FMM_NTMAX], sB[FMM_WARPS][FMM_PMAX + 1];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int c = blockIdx.x * FMM_WARPS + w;
  if (c >= ncls || *same) return;
  int dl = key4[4 * c];
  double sc = dl > 0 ? ldexp(1.0, -dl) : 1.0;  // finer-level half-widths -> half-widths of A
  double x = key4[4 * c + 1] * sc, y = key4[4 * c + 2] * sc, z = key4[4 * c + 3] * sc;
  warp_derivs<double>(x, y, z, p, sD[w], sT[w], sB[w]);
  int nt = fmm_nterms(p);
  for (int i = lane; i < nt; i += 32) {
    D64[(size_t)c * nt + i] = sD[w][i];
    D32[(size_t)c * fmm_stride4(nt) + i] = (float)sD[w][i];
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
template <typename T> static int grow_keep(DevBuf<T> &b, size_t need, size_t used, cudaStream_t st) {
  if (need <= b.cap && b.p) return FMM_OK;
  size_t want = need + need / 2 + 64;
  T *p = nullptr;
  FMM_CUDA_TRY(cudaMalloc((void **)&p, want * sizeof(T)));
  if (b.p && used) FMM_CUDA_TRY(cudaMemcpyAsync(p, b.p, used * sizeof(T), cudaMemcpyDeviceToDevice, st));
  if (b.p) {
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(b.p);
  }
  b.p = p;
  b.cap = want;
  return FMM_OK;
}

static int tmp_reserve(DevTree *t, size_t bytes) { return fmm_reserve(t->tmp, bytes); }
static int bits_for(long n);

#define TRY(x) do { int _rc = (x); if (_rc) return _rc; } while (0)

static int rec(DevTree *t, int i, cudaStream_t st) {
  if (!t->ev_ready) return FMM_OK;
  FMM_CUDA_TRY(cudaEventRecord(t->ev[i], st));
  return FMM_OK;
}

__global__ void k_p2p_count(const int *off, const int *src, int nc, const int *pcount, unsigned long long *out);
static int build_cells(DevTree *t, cudaStream_t st, int nlev, bool *deeper);
static int build_lists(DevTree *t, cudaStream_t st);
static int build_classes(DevTree *t, cudaStream_t st);

int fmm_tree_build(DevTree *t, const double *pos, long N, long ncrit, int order, double theta, int so,
                   cudaStream_t st, const long *sys_off, int nsys, bool defer_classes,
                   int (*after_cells)(DevTree *, void *), void *arg) {
  if (N < 1 || N >= (1L << 31) - 1 || ncrit < 1 || order < so + 1 || order > FMM_PMAX || so < 0 || so > 2 ||
      !(theta > 0) || !pos || nsys < 1 || (nsys > 1 && !sys_off))
    return FMM_ERR_ARG;
  if (sys_off) {
    if (sys_off[0] != 0 || sys_off[nsys] != N) return FMM_ERR_ARG;
    for (int k = 0; k < nsys; k++)
      if (sys_off[k + 1] <= sys_off[k]) return FMM_ERR_ARG;  // every system holds particles
  }
  t->N = N; t->ncrit = ncrit; t->order = order; t->so = so; t->theta = theta;
  t->nsys = nsys;
  if (sys_off) t->sys_off_h.assign(sys_off, sys_off + nsys + 1);
  else t->sys_off_h = {0, N};
  FMM_CUDA_TRY(cudaGetDevice(&t->dev));
  if (!t->ev_ready) {
    for (int i = 0; i < 16; i++) FMM_CUDA_TRY(cudaEventCreate(&t->ev[i]));
    for (int i = 0; i < 4; i++) FMM_CUDA_TRY(cudaEventCreate(&t->ev_mk[i]));
    t->ev_ready = true;
  }
  if (!t->h_pinned) {
    FMM_CUDA_TRY(cudaMallocHost((void **)&t->h_pinned, 64));
    memset(t->h_pinned, 0, 64);
  }
  t->build_serial++;
  TRY(rec(t, 0, st));
  TRY(fmm_reserve(t->d_eflags, 4));
  FMM_CUDA_TRY(cudaMemsetAsync(t->d_eflags.p, 0, sizeof(uint32_t), st));
  TRY(fmm_reserve(t->sys_off, (size_t)nsys + 1));
  FMM_CUDA_TRY(cudaMemcpyAsync(t->sys_off.p, t->sys_off_h.data(), sizeof(long) * (nsys + 1),
                               cudaMemcpyHostToDevice, st));
  TRY(fmm_reserve(t->roots, 4 * (size_t)nsys));
  // d_root: [0..2] sums, [3..5] maxima (u64 bits), [6..9] root box, [16..] level r/rmax
  TRY(fmm_reserve(t->d_root, 16 + 2 * (FMM_MAXLEVEL + 1)));
  double *dr = t->d_root.p;
  if (nsys == 1) {
    // one system: the exact sequential mean through fmm_seqsum3 (parallel)
    FMM_CUDA_TRY(cudaMemsetAsync(dr, 0, sizeof(double) * 16, st));
    TRY(tmp_reserve(t, fmm_seqsum_scratch(N)));
    TRY(fmm_seqsum3(pos, N, dr, t->tmp.p, st));
    unsigned nbm = std::min<unsigned>(fmm_blocks(N, 256), 152 * 8);
    fmm_note_launch(), k_root_absmax<<<nbm, 256, 0, st>>>(pos, N, dr, (unsigned long long *)(dr + 3));
    TRY(fmm_reserve(t->levf, FMM_MAXLEVEL + 1));
    fmm_note_launch(), k_root_final<<<1, 1, 0, st>>>(dr, (const unsigned long long *)(dr + 3), N, t->roots.p,
                                                     dr + 16, t->levf.p);
  } else {
    // a forest: each system's sums by one thread (systems run side by side)
    TRY(fmm_reserve(t->psys, N));
    fmm_note_launch(), k_fill_psys<<<nsys, 256, 0, st>>>(t->sys_off.p, t->psys.p);
    TRY(tmp_reserve(t, sizeof(double) * 6 * (size_t)nsys + 64));
    double *sums = (double *)t->tmp.p;
    unsigned long long *mx = (unsigned long long *)(sums + 3 * (size_t)nsys);
    FMM_CUDA_TRY(cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * 3 * nsys, st));
    fmm_note_launch(), k_seg_sums<<<fmm_blocks(3 * (size_t)nsys, 128), 128, 0, st>>>(pos, t->sys_off.p, nsys, sums);
    fmm_note_launch(), k_seg_absmax<<<nsys, 256, 0, st>>>(pos, t->sys_off.p, sums, mx);
    fmm_note_launch(), k_seg_root_final<<<fmm_blocks(nsys, 128), 128, 0, st>>>(nsys, t->sys_off.p, sums, mx,
                                                                                t->roots.p);
  }
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(rec(t, 1, st));

  // keys + stable sort, then the cells; the keys hold the digits of the first
  // FMM_KEYLEVELS levels unless a tree that deep needs more (then all of them)
  TRY(fmm_reserve(t->keys, N)); TRY(fmm_reserve(t->keys2, N));
  TRY(fmm_reserve(t->perm, N)); TRY(fmm_reserve(t->perm2, N));
  for (int nlev = FMM_KEYLEVELS;; nlev = FMM_MAXLEVEL) {
    fmm_note_launch(), k_keys<<<fmm_blocks(N, 256), 256, 0, st>>>(pos, N, t->roots.p, nsys > 1 ? t->psys.p : nullptr,
                                                                   nlev, t->keys.p, t->perm.p);
    FMM_CUDA_TRY(cudaGetLastError());
    size_t nbh = fmm_rs_nblocks(N);
    size_t hist_n = 256 * nbh;
    const size_t sort_bytes = hist_n * 4 + fmm_scan_tmp_elems<uint32_t>(hist_n) * 4 + 1024;
    TRY(tmp_reserve(t, sort_bytes + (nsys > 1 ? 16 * (size_t)N : 0)));
    uint32_t *hist = (uint32_t *)t->tmp.p;
    uint32_t *scantmp = hist + hist_n;
    TRY(fmm_radix_sort(t->keys.p, t->perm.p, t->keys2.p, t->perm2.p, N, 3 * (FMM_MAXLEVEL - nlev),
                       3 * FMM_MAXLEVEL, hist, scantmp, st));
    if (nsys > 1) {
      // stable sort by system: (system, key) order, each system's particles contiguous
      uint32_t *ks = (uint32_t *)(t->tmp.p + sort_bytes);
      uint32_t *idx = ks + N, *ks2 = idx + N, *idx2 = ks2 + N;
      fmm_note_launch(), k_sorted_sys<<<fmm_blocks(N, 256), 256, 0, st>>>(t->perm.p, t->psys.p, N, ks, idx);
      TRY(fmm_radix_sort<uint32_t>(ks, idx, ks2, idx2, N, 0, bits_for(nsys), hist, scantmp, st));
      fmm_note_launch(), k_apply_order<<<fmm_blocks(N, 256), 256, 0, st>>>(idx, N, t->keys.p, t->perm.p,
                                                                           t->keys2.p, t->perm2.p);
      FMM_CUDA_TRY(cudaGetLastError());
      std::swap(t->keys, t->keys2);
      std::swap(t->perm, t->perm2);
    }
    TRY(fmm_reserve(t->px, N)); TRY(fmm_reserve(t->py, N)); TRY(fmm_reserve(t->pz, N));
    fmm_note_launch(), k_gather_pos<<<fmm_blocks(N, 256), 256, 0, st>>>(pos, t->perm.p, N, t->px.p, t->py.p,
                                                                         t->pz.p);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaMemcpyAsync(&t->root, t->roots.p, sizeof(RootBox), cudaMemcpyDeviceToHost, st));  // system 0
    TRY(rec(t, 2, st));
    bool deeper = false;
    TRY(build_cells(t, st, nlev, &deeper));
    if (!deeper) break;
  }
  TRY(rec(t, 3, st));
  if (after_cells) TRY(after_cells(t, arg));  // work that needs the cells only, beside the walk
  TRY(build_lists(t, st));
  TRY(rec(t, 4, st));
  return defer_classes ? FMM_OK : fmm_tree_finish_build(t, st);
}

// The M2L translation classes and the end of the build (fmm_tree_build with
// defer_classes leaves them to this call).
int fmm_tree_finish_build(DevTree *t, cudaStream_t st) {
  TRY(build_classes(t, st));
  TRY(rec(t, 5, st));
  FMM_CUDA_TRY(cudaMemcpyAsync(&t->eflags, t->d_eflags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaStreamSynchronize(st));
  if (t->ev_ready) {
    float ms;
    for (int i = 0; i < 5; i++) {
      cudaEventElapsedTime(&ms, t->ev[i], t->ev[i + 1]);
      t->build_ms[i] = ms;
    }
    cudaEventElapsedTime(&ms, t->ev[0], t->ev[5]);
    t->build_ms[5] = ms;
  }
  if (t->eflags & FMM_EFLAG_DEPTH) return FMM_ERR_DEPTH;
  if (t->eflags & FMM_EFLAG_RANGE) return FMM_ERR_RANGE;
  return FMM_OK;
}

// Cells level by level from keys holding nlev levels of digits; *deeper is set
// (and the error flag cleared) when a cell at level nlev would need the next.
static int build_cells(DevTree *t, cudaStream_t st, int nlev, bool *deeper) {
  long N = t->N;
  const int nsys = t->nsys;
  size_t cap = (size_t)(4 * N / std::max<long>(t->ncrit, 1)) + 1024 + nsys;
  TRY(fmm_reserve(t->cx, cap)); TRY(fmm_reserve(t->cy, cap)); TRY(fmm_reserve(t->cz, cap));
  TRY(fmm_reserve(t->cid, cap)); TRY(fmm_reserve(t->ix, cap)); TRY(fmm_reserve(t->iy, cap));
  TRY(fmm_reserve(t->iz, cap)); TRY(fmm_reserve(t->pstart, cap)); TRY(fmm_reserve(t->pcount, cap));
  TRY(fmm_reserve(t->parent, cap)); TRY(fmm_reserve(t->child_first, cap));
  TRY(fmm_reserve(t->child_mask, cap)); TRY(fmm_reserve(t->clevel, cap));
  TRY(fmm_reserve(t->cr, cap)); TRY(fmm_reserve(t->crmax, cap)); TRY(fmm_reserve(t->crf, cap));
  TRY(fmm_reserve(t->csys, cap));
  fmm_note_launch(), k_init_roots<<<fmm_blocks(nsys, 128), 128, 0, st>>>(
      nsys, t->roots.p, t->sys_off.p, t->cx.p, t->cy.p, t->cz.p, t->cid.p, t->ix.p, t->iy.p, t->iz.p, t->pstart.p,
      t->pcount.p, t->parent.p, t->child_first.p, t->child_mask.p, t->clevel.p, t->cr.p, t->crmax.p, t->crf.p,
      t->csys.p);
  FMM_CUDA_TRY(cudaGetLastError());
  t->level_off.assign(1, 0);
  t->level_off.push_back(nsys);
  int lo = 0, hi = nsys, level = 0;
  uint32_t *h_total = t->h_pinned;
  int rc = FMM_OK;
  while (true) {
    int n = hi - lo;
    const size_t nscan = (size_t)n + 1 + fmm_scan_tmp_elems<uint32_t>(n) + 16;
    size_t need = nscan * 4 + (size_t)n * 9 * 4;
    if ((rc = tmp_reserve(t, need))) break;
    uint32_t *cnt = (uint32_t *)t->tmp.p;
    uint32_t *total = cnt + n;
    uint32_t *stmp = total + 1;
    int *bnd = (int *)(cnt + nscan);  // child boundaries of each cell of the level
    fmm_note_launch(), k_count_children<<<fmm_blocks((size_t)n * 32, 128), 128, 0, st>>>(
        lo, hi, level, nlev, t->ncrit, t->keys.p, t->pstart.p, t->pcount.p, t->child_mask.p, cnt, bnd,
        t->d_eflags.p);
    if ((rc = fmm_scan<uint32_t>(cnt, cnt, n, total, stmp, st))) break;
    cudaMemcpyAsync(h_total, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) { rc = FMM_ERR_CUDA; break; }
    uint32_t nnew = *h_total;
    if (nnew == 0) break;
    size_t need_cells = (size_t)hi + nnew;
    size_t used = hi;
    if ((rc = grow_keep(t->cx, need_cells, used, st)) || (rc = grow_keep(t->cy, need_cells, used, st)) ||
        (rc = grow_keep(t->cz, need_cells, used, st)) || (rc = grow_keep(t->cid, need_cells, used, st)) ||
        (rc = grow_keep(t->ix, need_cells, used, st)) || (rc = grow_keep(t->iy, need_cells, used, st)) ||
        (rc = grow_keep(t->iz, need_cells, used, st)) || (rc = grow_keep(t->pstart, need_cells, used, st)) ||
        (rc = grow_keep(t->pcount, need_cells, used, st)) || (rc = grow_keep(t->parent, need_cells, used, st)) ||
        (rc = grow_keep(t->child_first, need_cells, used, st)) ||
        (rc = grow_keep(t->child_mask, need_cells, used, st)) || (rc = grow_keep(t->clevel, need_cells, used, st)) ||
        (rc = grow_keep(t->cr, need_cells, used, st)) || (rc = grow_keep(t->crmax, need_cells, used, st)) ||
        (rc = grow_keep(t->crf, need_cells, used, st)) || (rc = grow_keep(t->csys, need_cells, used, st)))
      break;
    fmm_note_launch(), k_write_children<<<fmm_blocks((size_t)n * 32, 128), 128, 0, st>>>(
        lo, hi, level, cnt, bnd, t->cx.p, t->cy.p, t->cz.p, t->cid.p, t->ix.p, t->iy.p, t->iz.p, t->pstart.p,
        t->pcount.p, t->parent.p, t->child_first.p, t->child_mask.p, t->child_mask.p, t->clevel.p, t->cr.p,
        t->crmax.p, t->crf.p, t->csys.p);
    if (cudaGetLastError() != cudaSuccess) { rc = FMM_ERR_CUDA; break; }
    lo = hi;
    hi = hi + (int)nnew;
    level++;
    t->level_off.push_back(hi);
  }
  if (rc) return rc;
  t->ncells = hi;
  t->nlevels = level + 1;
  // leaves
  int nc = t->ncells;
  TRY(fmm_reserve(t->leaf_cells, nc));
  TRY(fmm_reserve(t->cell_leaf, nc));
  TRY(tmp_reserve(t, (size_t)nc * 4 + fmm_scan_tmp_elems<uint32_t>(nc) * 4 + 64));
  uint32_t *flag = (uint32_t *)t->tmp.p;
  uint32_t *total = flag + nc;
  uint32_t *stmp = total + 1;
  fmm_note_launch(), k_leaf_flags<<<fmm_blocks(nc, 256), 256, 0, st>>>(nc, t->ncrit, t->pcount.p, flag);
  TRY(fmm_scan<uint32_t>(flag, flag, nc, total, stmp, st));
  fmm_note_launch(), k_leaf_compact<<<fmm_blocks(nc, 256), 256, 0, st>>>(nc, t->ncrit, t->pcount.p, flag, t->leaf_cells.p,
                                                      t->cell_leaf.p);
  FMM_CUDA_TRY(cudaGetLastError());
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned + 1, t->d_eflags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaStreamSynchronize(st));
  t->nleaves = (int)t->h_pinned[0];
  if (t->h_pinned[1] & FMM_EFLAG_KEYS) {
    *deeper = true;
    FMM_CUDA_TRY(cudaMemsetAsync(t->d_eflags.p, 0, sizeof(uint32_t), st));
    return FMM_OK;
  }
  TRY(fmm_reserve(t->cmargin, nc));
  fmm_note_launch(), k_cell_margins<<<fmm_blocks(nc, 256), 256, 0, st>>>(nc, t->csys.p, t->roots.p, t->cr.p,
                                                                          t->theta, t->cmargin.p);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

static int bits_for(long n) {  // bits that hold the values 0..n-1
  int b = 0;
  while ((1L << b) < n) b++;
  return b;
}

template <typename K>
static int sort_pairs(DevTree *t, const int *tgt, const int *cls, int cbits, int end_bit, DevBuf<int> &src_raw,
                      long n, DevBuf<int> &off, int *cls_out, cudaStream_t st) {
  size_t nbh = fmm_rs_nblocks(n);
  size_t hist_n = 256 * nbh;
  size_t bytes = (size_t)n * (2 * sizeof(K) + 4) + hist_n * 4 + fmm_scan_tmp_elems<uint32_t>(hist_n) * 4 + 256;
  TRY(tmp_reserve(t, bytes));
  char *p = t->tmp.p;
  K *k1 = (K *)p; p += (size_t)n * sizeof(K);
  K *k2 = (K *)p; p += (size_t)n * sizeof(K);
  uint32_t *v2 = (uint32_t *)p; p += (size_t)n * 4;
  uint32_t *hist = (uint32_t *)p; p += hist_n * 4;
  uint32_t *stmp = (uint32_t *)p;
  fmm_note_launch(), k_pair_keys<K><<<fmm_blocks(n, 256), 256, 0, st>>>(tgt, cls, n, cbits, k1);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(fmm_radix_sort<K>(k1, (uint32_t *)src_raw.p, k2, v2, n, 0, end_bit, hist, stmp, st));
  fmm_note_launch(), k_csr_from_sorted<K><<<fmm_blocks(n + 1, 256), 256, 0, st>>>(k1, n, cbits, t->ncells, off.p,
                                                                                 cls_out);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// Sort the walk's (tgt, src) pairs by target -- and by class within a target
// when cls is given -- stably, and build the CSR offsets.  The sort runs in
// place on src_raw, which is then swapped into src_out.
static int group_by_target(DevTree *t, DevBuf<int> &tgt_raw, DevBuf<int> &src_raw, const int *cls, int ncls,
                           long n, DevBuf<int> &off, DevBuf<int> &src_out, int *cls_out, cudaStream_t st) {
  int nc = t->ncells;
  TRY(fmm_reserve(off, (size_t)nc + 1));
  if (n == 0) {
    TRY(fmm_reserve(src_out, 1));
    FMM_CUDA_TRY(cudaMemsetAsync(off.p, 0, sizeof(int) * (nc + 1), st));
    return FMM_OK;
  }
  const int cbits = cls ? bits_for(ncls) : 0;
  const int kbits = bits_for(nc) + cbits;
  if (kbits <= 32)
    TRY(sort_pairs<uint32_t>(t, tgt_raw.p, cls, cbits, kbits, src_raw, n, off, cls_out, st));
  else
    TRY(sort_pairs<uint64_t>(t, tgt_raw.p, cls, cbits, kbits, src_raw, n, off, cls_out, st));
  std::swap(src_raw, src_out);
  return FMM_OK;
}

static int build_lists(DevTree *t, cudaStream_t st) {
  int nc = t->ncells;
  WalkCells W{t->cx.p, t->cy.p, t->cz.p, t->crmax.p, t->child_mask.p, t->clevel.p, t->child_first.p,
              t->ix.p, t->iy.p, t->iz.p, t->cmargin.p, (float)(t->theta * t->theta)};
  // raw lists in walk order; the buffers keep their capacity between builds,
  // so a rebuild of a similar tree allocates nothing
  DevBuf<int> &m2l_src_raw = t->m2l_src_raw, &m2l_tgt_raw = t->m2l_tgt_raw;
  DevBuf<int> &p2p_tgt_raw = t->p2p_tgt_raw, &p2p_src_raw = t->p2p_src_raw;
  size_t cap_pairs = (size_t)nc * 64 + 1024 + t->nsys;
  TRY(fmm_reserve(t->fa, cap_pairs)); TRY(fmm_reserve(t->fb, cap_pairs));
  TRY(fmm_reserve(t->fa2, cap_pairs)); TRY(fmm_reserve(t->fb2, cap_pairs));
  TRY(fmm_reserve(m2l_src_raw, cap_pairs)); TRY(fmm_reserve(m2l_tgt_raw, cap_pairs));
  TRY(fmm_reserve(p2p_tgt_raw, cap_pairs)); TRY(fmm_reserve(p2p_src_raw, cap_pairs));
  int rc = FMM_OK;
  long nm2l = 0, np2p = 0;
  // the walk starts from each system's (root, root) pair
  uint32_t nf = (uint32_t)t->nsys;
  U3 *h_tot = (U3 *)t->h_pinned;
  fmm_note_launch(), k_root_pairs<<<fmm_blocks(nf, 256), 256, 0, st>>>((int)nf, t->fa.p, t->fb.p);
  FMM_CUDA_TRY(cudaGetLastError());
  while (nf > 0) {
    const unsigned nblk = fmm_blocks(nf, WALK_BS);
    size_t need = (size_t)nblk * sizeof(U3) + fmm_scan_tmp_elems<U3>(nblk) * sizeof(U3) + 2 * sizeof(U3);
    if ((rc = tmp_reserve(t, need))) break;
    U3 *cnt = (U3 *)t->tmp.p;  // per block: slot totals, then their exclusive scan
    U3 *tot = cnt + nblk;
    U3 *stmp = tot + 1;
    if ((rc = fmm_reserve(t->wdec, nf))) break;
    fmm_note_launch(), k_walk_count<<<nblk, WALK_BS, 0, st>>>(W, t->fa.p, t->fb.p, nf, t->theta, cnt, t->wdec.p);
    if ((rc = fmm_scan<U3>(cnt, cnt, nblk, tot, stmp, st))) break;
    cudaMemcpyAsync(h_tot, tot, sizeof(U3), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) { rc = FMM_ERR_CUDA; break; }
    U3 T = *h_tot;
    if ((rc = grow_keep(m2l_src_raw, nm2l + T.x, nm2l, st)) || (rc = grow_keep(m2l_tgt_raw, nm2l + T.x, nm2l, st)) ||
        (rc = grow_keep(p2p_tgt_raw, np2p + T.y, np2p, st)) || (rc = grow_keep(p2p_src_raw, np2p + T.y, np2p, st)) ||
        (rc = fmm_reserve(t->fa2, T.z + 1)) || (rc = fmm_reserve(t->fb2, T.z + 1)))
      break;
    U3 base{(uint32_t)nm2l, (uint32_t)np2p, 0u};
    fmm_note_launch(), k_walk_write<<<nblk, WALK_BS, 0, st>>>(W, t->fa.p, t->fb.p, nf, t->wdec.p, cnt, base,
                                                     m2l_src_raw.p, m2l_tgt_raw.p, p2p_tgt_raw.p, p2p_src_raw.p,
                                                     t->fa2.p, t->fb2.p);
    if (cudaGetLastError() != cudaSuccess) { rc = FMM_ERR_CUDA; break; }
    nm2l += T.x;
    np2p += T.y;
    nf = T.z;
    std::swap(t->fa, t->fa2);
    std::swap(t->fb, t->fb2);
  }
  if (rc) return rc;
  // the M2L pairs stay in walk order here: build_classes groups them by
  // (target, class) once the classes are known
  t->nm2l = nm2l;
  t->np2p = np2p;
  TRY(group_by_target(t, p2p_tgt_raw, p2p_src_raw, nullptr, 0, np2p, t->p2p_off, t->p2p_src, nullptr, st));
  // the interaction count is a statistic: read when asked for (fmm_p2p_interactions)
  TRY(fmm_reserve(t->d_p2pcount, 1));
  FMM_CUDA_TRY(cudaMemsetAsync(t->d_p2pcount.p, 0, sizeof(unsigned long long), st));
  fmm_note_launch(), k_p2p_count<<<fmm_blocks(nc, 256), 256, 0, st>>>(t->p2p_off.p, t->p2p_src.p, nc, t->pcount.p,
                                                                       t->d_p2pcount.p);
  FMM_CUDA_TRY(cudaGetLastError());
  t->p2p_count_serial = t->build_serial;
  return FMM_OK;
}

long long fmm_p2p_interactions(DevTree *t) {
  if (t->p2p_count_serial == t->build_serial) {
    unsigned long long v = 0;
    // the count kernel ran on the build's stream, which may not block with the default one
    if (cudaDeviceSynchronize() == cudaSuccess &&
        cudaMemcpy(&v, t->d_p2pcount.p, sizeof(v), cudaMemcpyDeviceToHost) == cudaSuccess) {
      t->p2p_interactions = (long long)v;
      t->p2p_count_serial = ~0ull;
    }
  }
  return t->p2p_interactions;
}

// particle-particle interactions of the P2P list (self pairs skip i == j)
__global__ void k_p2p_count(const int *off, const int *src, int nc, const int *pcount, unsigned long long *out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long s = 0;
  if (c < nc)
    for (int k = off[c]; k < off[c + 1]; k++) {
      int b = src[k];
      s += (unsigned long long)pcount[c] * pcount[b] - (b == c ? pcount[c] : 0);
    }
  for (int d = 16; d; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

static int build_classes(DevTree *t, cudaStream_t st) {
  long n = t->nm2l;
  int nc = t->ncells;
  int p = t->order;
  t->csr_serial = ~0ull;  // the target lists of this build are made on demand (fmm_m2l_csr)
  TRY(fmm_reserve(t->m2l_cls_raw, n > 0 ? n : 1));
  if (n == 0) {
    t->nclasses = 0;
    return fmm_m2l_cell_order(t, t->tune.grouping, st);
  }
  // classes of the raw (walk-order) pairs: the distinct keys through an
  // open-addressing table, ids by rank of the sorted distinct keys
  const int *tgt = t->m2l_tgt_raw.p, *src = t->m2l_src_raw.p;
  uint32_t hsize = 1u << 16;
  while ((long)hsize < std::min<long>(n, 1L << 20) / 4) hsize <<= 1;
  uint64_t *keys = nullptr, *U1 = nullptr, *U2 = nullptr;
  uint32_t *stat = nullptr, *I1 = nullptr, *I2 = nullptr, *uhist = nullptr, *uscan = nullptr;
  uint32_t ncls = 0;
  for (int attempt = 0;; attempt++) {
    const size_t umax = hsize / 2;
    const size_t histu = 256 * fmm_rs_nblocks(umax);
    TRY(tmp_reserve(t, (size_t)n * 8 + 64 + umax * 24 + histu * 4 + fmm_scan_tmp_elems<uint32_t>(histu) * 4 + 256));
    char *q = t->tmp.p;
    keys = (uint64_t *)q; q += (size_t)n * 8;
    stat = (uint32_t *)q; q += 64;
    U1 = (uint64_t *)q; q += umax * 8;
    U2 = (uint64_t *)q; q += umax * 8;
    I1 = (uint32_t *)q; q += umax * 4;
    I2 = (uint32_t *)q; q += umax * 4;
    uhist = (uint32_t *)q; q += histu * 4;
    uscan = (uint32_t *)q;
    TRY(fmm_reserve(t->cls_hkeys, hsize));
    FMM_CUDA_TRY(cudaMemsetAsync(t->cls_hkeys.p, 0xff, sizeof(uint64_t) * hsize, st));  // all CLS_EMPTY
    FMM_CUDA_TRY(cudaMemsetAsync(stat, 0, 4 * sizeof(uint32_t), st));
    fmm_note_launch(), k_class_keys<<<fmm_blocks(n, 256), 256, 0, st>>>(src, tgt, n, t->ix.p, t->iy.p, t->iz.p,
                                                                        t->clevel.p, keys, t->cls_hkeys.p,
                                                                        hsize - 1, stat, t->d_eflags.p);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned, stat, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FMM_CUDA_TRY(cudaStreamSynchronize(st));
    ncls = t->h_pinned[0];
    if (!t->h_pinned[1] && ncls <= umax) break;
    if (hsize >= (1u << 28) || attempt >= 4) {
      fmm_set_error_text("M2L translation classes: the class table could not hold the distinct offsets");
      return FMM_ERR_RANGE;
    }
    hsize <<= 4;
  }
  t->nclasses = (int)ncls;
  TRY(fmm_reserve(t->cls_key4, 4 * (size_t)(ncls > 0 ? ncls : 1)));
  TRY(fmm_reserve(t->cls_table, hsize));
  fmm_note_launch(), k_class_collect<<<fmm_blocks(hsize, 256), 256, 0, st>>>(t->cls_hkeys.p, hsize, U1, I1,
                                                                              stat + 2);
  TRY(fmm_radix_sort<uint64_t>(U1, I1, U2, I2, ncls, 0, 64, uhist, uscan, st));
  // same classes as the previous build (same ids): the per-class operator
  // data of that build still holds and its kernels skip their work
  TRY(fmm_reserve(t->d_cls_same, 1));
  if ((int)ncls == t->ncls_prev && p == t->order_prev) {
    FMM_CUDA_TRY(cudaMemsetAsync(t->d_cls_same.p, 0xff, sizeof(uint32_t), st));
    fmm_note_launch(), k_keys_equal<<<fmm_blocks(ncls, 256), 256, 0, st>>>(U1, t->cls_prev.p, (int)ncls,
                                                                          t->d_cls_same.p);
  } else {
    FMM_CUDA_TRY(cudaMemsetAsync(t->d_cls_same.p, 0, sizeof(uint32_t), st));
  }
  TRY(fmm_reserve(t->cls_prev, ncls > 0 ? ncls : 1));
  FMM_CUDA_TRY(cudaMemcpyAsync(t->cls_prev.p, U1, sizeof(uint64_t) * ncls, cudaMemcpyDeviceToDevice, st));
  t->ncls_prev = (int)ncls;
  t->order_prev = p;
  fmm_note_launch(), k_class_rank<<<fmm_blocks(ncls, 256), 256, 0, st>>>(U1, (int)ncls, t->cls_hkeys.p, hsize - 1,
                                                                          t->cls_table.p, t->cls_key4.p);
  // the class of each walk-order pair
  fmm_note_launch(), k_class_lookup<<<fmm_blocks(n, 256), 256, 0, st>>>(keys, n, t->cls_hkeys.p, hsize - 1,
                                                                         t->cls_table.p, t->m2l_cls_raw.p);
  FMM_CUDA_TRY(cudaGetLastError());
  int nt = fmm_nterms(p);
  if (t->cls_D.cap < (size_t)ncls * nt || t->cls_Df.cap < (size_t)ncls * fmm_stride4(nt))  // contents lost
    FMM_CUDA_TRY(cudaMemsetAsync(t->d_cls_same.p, 0, sizeof(uint32_t), st));
  TRY(fmm_reserve(t->cls_D, (size_t)ncls * nt));
  TRY(fmm_reserve(t->cls_Df, (size_t)ncls * fmm_stride4(nt)));
  fmm_note_launch(), k_class_derivs<<<fmm_blocks(ncls, FMM_WARPS), 32 * FMM_WARPS, 0, st>>>(t->cls_key4.p, (int)ncls, p, t->cls_D.p,
                                                                         t->cls_Df.p, t->d_cls_same.p);
  FMM_CUDA_TRY(cudaGetLastError());
  return fmm_m2l_cell_order(t, t->tune.grouping, st);
}

// The M2L pairs grouped by target, sorted by class within a target: a target
// has at most one source per class, so the order within a list is fully
// determined.  The walk-order pairs stay as they are (the sort runs on a copy).
int fmm_m2l_csr(DevTree *t, cudaStream_t st) {
  if (t->csr_serial == t->build_serial) return FMM_OK;
  const long n = t->nm2l;
  const int nc = t->ncells;
  TRY(fmm_reserve(t->m2l_off, (size_t)nc + 1));
  TRY(fmm_reserve(t->m2l_src, n > 0 ? n : 1));
  TRY(fmm_reserve(t->m2l_cls, n > 0 ? n : 1));
  if (n == 0) {
    FMM_CUDA_TRY(cudaMemsetAsync(t->m2l_off.p, 0, sizeof(int) * ((size_t)nc + 1), st));
  } else {
    FMM_CUDA_TRY(cudaMemcpyAsync(t->m2l_src.p, t->m2l_src_raw.p, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    const int cbits = bits_for(t->nclasses), kbits = bits_for(nc) + cbits;
    if (kbits <= 32)
      TRY(sort_pairs<uint32_t>(t, t->m2l_tgt_raw.p, t->m2l_cls_raw.p, cbits, kbits, t->m2l_src, n, t->m2l_off,
                               t->m2l_cls.p, st));
    else
      TRY(sort_pairs<uint64_t>(t, t->m2l_tgt_raw.p, t->m2l_cls_raw.p, cbits, kbits, t->m2l_src, n, t->m2l_off,
                               t->m2l_cls.p, st));
  }
  t->csr_serial = t->build_serial;
  return FMM_OK;
}

// The M2L processing order of the cells (t->m2l_order): level, then by octant
// within the parent (grouping 0) or Morton order (grouping 1).
int fmm_m2l_cell_order(DevTree *t, int grouping, cudaStream_t st) {
  const int nc = t->ncells;
  size_t nbh = fmm_rs_nblocks(nc);
  size_t hist_n = 256 * nbh;
  TRY(tmp_reserve(t, (size_t)nc * 20 + hist_n * 4 + fmm_scan_tmp_elems<uint32_t>(hist_n) * 4 + 256));
  char *q = t->tmp.p;
  uint64_t *k1 = (uint64_t *)q; q += (size_t)nc * 8;
  uint64_t *k2 = (uint64_t *)q; q += (size_t)nc * 8;
  uint32_t *v2 = (uint32_t *)q; q += (size_t)nc * 4;
  uint32_t *hist = (uint32_t *)q; q += hist_n * 4;
  uint32_t *stmp2 = (uint32_t *)q;
  TRY(fmm_reserve(t->m2l_order, nc));
  fmm_note_launch(), k_order_keys<<<fmm_blocks(nc, 256), 256, 0, st>>>(nc, t->cid.p, t->clevel.p, grouping, k1,
                                                                        (uint32_t *)t->m2l_order.p);
  FMM_CUDA_TRY(cudaGetLastError());
  TRY(fmm_radix_sort<uint64_t>(k1, (uint32_t *)t->m2l_order.p, k2, v2, nc, 48, 64, hist, stmp2, st));
  t->grouping_built = grouping;
  t->order_version++;
  return FMM_OK;
}

void fmm_tree_destroy(DevTree *t) {
  if (!t) return;
  fmm_graph_release(t);
  fmm_tcg_release(t);
  for (cudaEvent_t *e : {&t->ev_fork, &t->ev_join, &t->ev_m, &t->ev_c, &t->ev_p, &t->ev_s, &t->ev_l}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  if (t->s_hi) cudaStreamDestroy(t->s_hi);
  if (t->s_near) cudaStreamDestroy(t->s_near);
  t->s_hi = t->s_near = nullptr;
  if (t->gstream) cudaStreamDestroy(t->gstream);
  t->gstream = nullptr;
  fmm_release(t->keys); fmm_release(t->keys2); fmm_release(t->perm); fmm_release(t->perm2);
  fmm_release(t->px); fmm_release(t->py); fmm_release(t->pz);
  fmm_release(t->phi4); fmm_release(t->plo4); fmm_release(t->sdip); fmm_release(t->levf);
  fmm_release(t->cx); fmm_release(t->cy); fmm_release(t->cz); fmm_release(t->cid);
  fmm_release(t->ix); fmm_release(t->iy); fmm_release(t->iz);
  fmm_release(t->pstart); fmm_release(t->pcount); fmm_release(t->parent); fmm_release(t->child_first);
  fmm_release(t->child_mask); fmm_release(t->clevel); fmm_release(t->leaf_cells); fmm_release(t->cell_leaf);
  fmm_release(t->m2l_off); fmm_release(t->m2l_src); fmm_release(t->m2l_cls); fmm_release(t->m2l_order);
  fmm_release(t->m2l_cls_raw);
  t->csr_serial = ~0ull;
  fmm_release(t->p2p_off); fmm_release(t->p2p_src);
  fmm_release(t->cls_key4); fmm_release(t->cls_D); fmm_release(t->cls_Df); fmm_release(t->cls_table);
  fmm_release(t->cls_hkeys); fmm_release(t->cls_prev); fmm_release(t->d_cls_same);
  t->ncls_prev = t->order_prev = -1;
  fmm_release(t->M); fmm_release(t->L); fmm_release(t->Mf); fmm_release(t->Lf);
  fmm_release(t->Fnear); fmm_release(t->Ffar);
  fmm_release(t->fa); fmm_release(t->fb); fmm_release(t->fa2); fmm_release(t->fb2);
  fmm_release(t->m2l_tgt_raw); fmm_release(t->m2l_src_raw);
  fmm_release(t->p2p_tgt_raw); fmm_release(t->p2p_src_raw);
  fmm_release(t->tc_T); fmm_release(t->tc_Mh); fmm_release(t->tc_Ml); fmm_release(t->tc_mexp);
  fmm_release(t->d_tcerr);
  fmm_release(t->tc_sched_off); fmm_release(t->tc_sched_cls); fmm_release(t->tc_bitmap); fmm_release(t->tc_rank);
  fmm_release(t->tc_stab); fmm_release(t->tc_pos); fmm_release(t->cm_otab);
  fmm_release(t->cm_woff); fmm_release(t->cm_wstep); fmm_release(t->tp_perm); fmm_release(t->tp_tgt);
  t->cm_wserial = ~0ull;
  t->sched_serial = ~0ull;
  t->tc_serial = ~0ull;
  fmm_release(t->wdec);
  fmm_release(t->d_p2pcount);
  fmm_release(t->m2l_ord); fmm_release(t->mnorm); fmm_release(t->feat); fmm_release(t->tscale); fmm_release(t->tpart);
  fmm_release(t->sys_pairs);
  fmm_release(t->ltgt);
  fmm_release(t->cr); fmm_release(t->crmax); fmm_release(t->crf); fmm_release(t->cmargin); fmm_release(t->csys);
  fmm_release(t->sys_off); fmm_release(t->psys); fmm_release(t->roots);
  fmm_release(t->tmp); fmm_release(t->d_eflags); fmm_release(t->d_root);
  if (t->h_pinned) cudaFreeHost(t->h_pinned);
  t->h_pinned = nullptr;
  if (t->ev_ready)
    for (int i = 0; i < 16; i++) cudaEventDestroy(t->ev[i]);
  if (t->ev_ready)
    for (int i = 0; i < 4; i++) cudaEventDestroy(t->ev_mk[i]);
  t->ev_ready = false;
}
