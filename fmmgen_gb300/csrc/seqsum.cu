// seqsum.cu -- the reference's sequential FP64 sum, reproduced bit for bit in
// parallel.
//
// build_tree centres the root cube on the mean position, accumulated as
//   s = 0; for i in 0..N-1: s = fl(s + x_i)                 (example/tree.cpp:148-156)
// Every tree decision downstream depends on the bits of that sum, so it must be
// reproduced exactly, not merely accurately.  A single dependent chain of FP64
// adds costs ~70 cycles per element on GB300's narrow FP64 pipe (~40 ms for
// 10^6 particles), so the chain is broken up:
//
//  While s stays inside one binade [2^e, 2^(e+1)) its ulp u = 2^(e-52) is fixed
//  and s is an integer S in units of u.  Adding x then rounds the exact sum to
//  the u grid:  S' = S + round(x / u), with the tie (x/u exactly half-way)
//  going to the even neighbour, i.e. depending only on the parity of S.  So
//  over a chunk of elements the whole chain is an integer map
//      S -> S + A[S mod 2]
//  valid while every intermediate S stays in [2^52, 2^53) (or its negative
//  mirror).  Chunks are analysed in parallel (integer arithmetic on the
//  mantissa bits, no FP64 pipe), with the binade guessed from an ordinary
//  parallel prefix sum; a single thread then chains the chunk maps, checks
//  each map's validity against the exact S, and falls back to plain sequential
//  FP64 adds for any chunk that leaves its binade or was guessed wrong (the
//  first chunk always does).  The result equals the sequential loop exactly.
#include "internal.h"

#define SS_C 256  // elements per chunk
#define SS_PER_LANE (SS_C / 32)

struct ChunkMap {
  long long A0, A1;      // total increment in ulps for start parity 0 / 1
  long long pmin, pmax;  // range of intermediate increments (with margin)
  int e;                 // binade the map is valid in
  int ok;                // 0: no map, run the chunk sequentially
};

// approximate chunk sums (FP64, any order)
__global__ void k_ss_chunksum(const double *__restrict__ pos, long N, long nchunks, double *csum) {
  long k = blockIdx.x * (long)(blockDim.x >> 5) + (threadIdx.x >> 5);
  int a = blockIdx.y, lane = threadIdx.x & 31;
  if (k >= nchunks) return;
  double s = 0;
  for (int j = 0; j < SS_PER_LANE; j++) {
    long i = k * SS_C + lane * SS_PER_LANE + j;
    if (i < N) s += pos[3 * i + a];
  }
  for (int d = 16; d; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
  if (lane == 0) csum[a * nchunks + k] = s;
}

// exclusive prefix of the chunk sums (approximate start values), one block per axis
__global__ void k_ss_prefix(const double *csum, long nchunks, double *start) {
  __shared__ double wsum[32];
  const int a = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5, nt = blockDim.x;
  long per = (nchunks + nt - 1) / nt;
  long b0 = t * per, b1 = min(nchunks, b0 + per);
  double s = 0;
  for (long k = b0; k < b1; k++) s += csum[a * nchunks + k];
  double inc = s;
  for (int d = 1; d < 32; d <<= 1) {
    double o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    double x = lane < (nt >> 5) ? wsum[lane] : 0.0;
    for (int d = 1; d < 32; d <<= 1) {
      double o = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += o;
    }
    wsum[lane] = x;
  }
  __syncthreads();
  double run = (w > 0 ? wsum[w - 1] : 0.0) + inc - s;
  for (long k = b0; k < b1; k++) {
    start[a * nchunks + k] = run;
    run += csum[a * nchunks + k];
  }
}

// element effect in ulps of binade e: non-tie increment, or tie base
struct Elem {
  long long inc;  // rounded increment (non-tie) or the lower candidate (tie)
  int tie;        // 1: exactly half-way, increment is inc or inc+1 by parity
  int bad;        // 1: cannot be expressed (too large, NaN, Inf)
};

__device__ __forceinline__ Elem elem_in_ulps(double x, int e) {
  Elem r{0, 0, 0};
  unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  int ex = (int)((bits >> 52) & 0x7ff);
  unsigned long long m = bits & ((1ull << 52) - 1);
  bool neg = bits >> 63;
  if (ex == 0x7ff) { r.bad = 1; return r; }
  if (ex == 0) ex = 1;       // subnormal: no implicit bit
  else m |= 1ull << 52;
  // x = +-m * 2^(ex - 1075); x / u = +-m * 2^(ex - 1075 - (e - 52)) = +-m * 2^(ex - 1023 - e)
  int sh = ex - 1023 - e;
  long long a = 0;
  if (m == 0) return r;
  if (sh >= 0) {
    if (sh > 9) { r.bad = 1; return r; }  // |x| >= 2^(e+10): leaves the binade anyway
    a = (long long)(m << sh);
  } else {
    int s = -sh;
    if (s >= 64) {
      a = 0;  // |x/u| < 2^-11 < 1/2
    } else {
      unsigned long long q = m >> s;
      unsigned long long rem = m & ((1ull << s) - 1);
      unsigned long long half = 1ull << (s - 1);
      if (rem > half) q += 1;
      else if (rem == half) r.tie = 1;
      a = (long long)q;
    }
  }
  if (neg) {
    // -(q + t): for a tie the candidates are -q and -(q+1); keep the lower one as base
    a = -a;
    if (r.tie) a -= 1;
  }
  r.inc = a;
  return r;
}

// Map of one chunk for start parity p0/p1: (increment, end parity) composed
struct Map2 {
  long long i0, i1;
  int q0, q1;
};
__device__ __forceinline__ Map2 compose(Map2 g, Map2 f) {  // g first, then f
  Map2 r;
  r.i0 = g.i0 + (g.q0 ? f.i1 : f.i0);
  r.q0 = g.q0 ? f.q1 : f.q0;
  r.i1 = g.i1 + (g.q1 ? f.i1 : f.i0);
  r.q1 = g.q1 ? f.q1 : f.q0;
  return r;
}
__device__ __forceinline__ Map2 elem_map(const Elem &el) {
  Map2 m;
  if (!el.tie) {
    m.i0 = m.i1 = el.inc;
    int par = (int)(el.inc & 1);
    m.q0 = par;
    m.q1 = par ^ 1;
  } else {
    // S + inc even: parity p -> increment inc + ((p + inc) & 1), end parity 0
    int b = (int)(el.inc & 1);
    m.i0 = el.inc + (b ? 1 : 0);
    m.i1 = el.inc + (b ? 0 : 1);
    m.q0 = m.q1 = 0;
  }
  return m;
}

__global__ void k_ss_maps(const double *__restrict__ pos, long N, long nchunks, const double *start, ChunkMap *maps) {
  long k = blockIdx.x * (long)(blockDim.x >> 5) + (threadIdx.x >> 5);
  int a = blockIdx.y, lane = threadIdx.x & 31;
  if (k >= nchunks) return;
  double s0 = start[a * nchunks + k];
  ChunkMap cm{0, 0, 0, 0, 0, 0};
  if (s0 == 0.0 || !isfinite(s0)) {
    if (lane == 0) maps[a * nchunks + k] = cm;
    return;
  }
  int e = ilogb(fabs(s0));
  Map2 acc{0, 0, 0, 1};  // identity
  long long run = 0, lmin = 0, lmax = 0;
  int bad = 0;
  for (int j = 0; j < SS_PER_LANE; j++) {
    long i = k * SS_C + lane * SS_PER_LANE + j;
    if (i >= N) break;
    Elem el = elem_in_ulps(pos[3 * i + a], e);
    bad |= el.bad;
    acc = compose(acc, elem_map(el));
    run += el.inc;
    lmin = min(lmin, run);
    lmax = max(lmax, run);
  }
  // inclusive warp scan of the lane maps
  Map2 inc = acc;
  long long base = run;  // parity-0 path approximation for the range
  for (int d = 1; d < 32; d <<= 1) {
    Map2 o;
    o.i0 = __shfl_up_sync(0xffffffffu, inc.i0, d);
    o.i1 = __shfl_up_sync(0xffffffffu, inc.i1, d);
    o.q0 = __shfl_up_sync(0xffffffffu, inc.q0, d);
    o.q1 = __shfl_up_sync(0xffffffffu, inc.q1, d);
    long long ob = __shfl_up_sync(0xffffffffu, base, d);
    if (lane >= d) {
      inc = compose(o, inc);
      base += ob;
    }
  }
  long long excl = base - run;  // increments before this lane
  long long mn = excl + lmin, mx = excl + lmax;
  for (int d = 16; d; d >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, d));
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    bad |= __shfl_xor_sync(0xffffffffu, bad, d);
  }
  if (lane == 31) {
    cm.A0 = inc.i0;
    cm.A1 = inc.i1;
    // ties can move the parity-1 path by at most one ulp per element
    cm.pmin = mn - SS_C - 1;
    cm.pmax = mx + SS_C + 1;
    cm.e = e;
    cm.ok = !bad;
    maps[a * nchunks + k] = cm;
  }
}

// S * 2^(e-52) for |S| in [2^52, 2^53), assembled from its bits (integer
// operations only: the chain runs on one warp per axis, where every FP64
// instruction costs the narrow FP64 pipe a full warp's worth of cycles)
__device__ __forceinline__ double ss_to_double(long long S, int e) {
  const unsigned long long m = (unsigned long long)(S < 0 ? -S : S);
  unsigned long long bits = ((unsigned long long)(e + 1023) << 52) | (m & ((1ull << 52) - 1));
  if (S < 0) bits |= 1ull << 63;
  return __longlong_as_double((long long)bits);
}
// binade e and S = s / 2^(e-52) of a normal double; false for zero,
// subnormals, infinities and NaN (which take plain FP64 adds)
__device__ __forceinline__ bool ss_from_double(double s, int &e, long long &S) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(s);
  const int ex = (int)((bits >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff) return false;
  e = ex - 1023;
  const long long m = (long long)((bits & ((1ull << 52) - 1)) | (1ull << 52));
  S = (bits >> 63) ? -m : m;
  return true;
}

// Chunk maps compose: chunk a then chunk b (same binade) is again
//   S -> S + B[S mod 2],  B[p] = A_a[p] + A_b[(p + A_a[p]) mod 2]
// (the parity after a is that of p + A_a[p]), valid while every intermediate
// increment stays in [min(pmin_a, min A_a + pmin_b), max(pmax_a, max A_a + pmax_b)]
// -- a conservative range, so a composite that checks valid is valid.  e ==
// SS_ANY marks the identity.
#define SS_ANY (-100000)
__device__ __forceinline__ ChunkMap cm_identity() {
  ChunkMap m;
  m.A0 = m.A1 = m.pmin = m.pmax = 0;
  m.e = SS_ANY;
  m.ok = 1;
  return m;
}
__device__ __forceinline__ ChunkMap cm_compose(const ChunkMap &a, const ChunkMap &b) {
  if (a.e == SS_ANY) return b;
  if (b.e == SS_ANY) return a;
  ChunkMap c;
  c.ok = a.ok && b.ok && a.e == b.e;
  c.e = a.e;
  c.A0 = a.A0 + ((a.A0 & 1) ? b.A1 : b.A0);
  c.A1 = a.A1 + ((a.A1 & 1) ? b.A0 : b.A1);
  c.pmin = min(a.pmin, min(a.A0, a.A1) + b.pmin);
  c.pmax = max(a.pmax, max(a.A0, a.A1) + b.pmax);
  return c;
}
__device__ __forceinline__ ChunkMap cm_shfl_up(const ChunkMap &m, int d) {
  const unsigned FULL = 0xffffffffu;
  ChunkMap o;
  o.A0 = __shfl_up_sync(FULL, m.A0, d);
  o.A1 = __shfl_up_sync(FULL, m.A1, d);
  o.pmin = __shfl_up_sync(FULL, m.pmin, d);
  o.pmax = __shfl_up_sync(FULL, m.pmax, d);
  o.e = __shfl_up_sync(FULL, m.e, d);
  o.ok = __shfl_up_sync(FULL, m.ok, d);
  return o;
}

// Chains the chunk maps in order, exactly: one warp per axis (each on its own
// SM), 32 chunks at a time.  The state (s, or S in ulps of binade e) is kept identical in every
// lane.  From the current chunk j of a block, the lanes compose the maps of
// chunks j..lane (a warp scan); the longest run of composites that is valid
// for the exact S is applied in one step.  A chunk that no composite covers
// (its map is missing or invalid for the exact state) is run 32 elements at a
// time: the lanes scan the element maps from the exact S, a ballot finds the
// first element whose result leaves the binade, and only that element takes a
// plain sequential FP64 add.
__global__ void k_ss_chain(const double *__restrict__ pos, long N, long nchunks, const ChunkMap *maps, double *out) {
  __shared__ double sx[1][SS_C];
  const unsigned FULL = 0xffffffffu;
  const int a = blockIdx.x, lane = threadIdx.x & 31;  // one axis per block, so per SM
  const long long LO = 1ll << 52, HI = 1ll << 53;
  double s = 0.0;
  bool imode = false;
  long long S = 0;
  int e = 0;
  // elements of the chunk after the last chunk that ran element by element
  // (such chunks come in runs: their loads overlap the previous one's work)
  long pref_k = -1;
  double pr[SS_PER_LANE];
  ChunkMap nxt = lane < nchunks ? maps[a * nchunks + lane] : cm_identity();
  for (long k0 = 0; k0 < nchunks; k0 += 32) {
    const ChunkMap mo = nxt;  // this lane's chunk k0 + lane
    if (k0 + 32 + lane < nchunks) nxt = maps[a * nchunks + k0 + 32 + lane];  // the next block's, ahead
    const int nb = (int)min(32L, nchunks - k0);
    int j = 0;
    while (j < nb) {
      // the state in the binade of chunk j's map, when it has one
      const int ej = __shfl_sync(FULL, mo.e, j), okj = __shfl_sync(FULL, mo.ok, j);
      if (okj && (!imode || e != ej)) {
        double cur = imode ? ss_to_double(S, e) : s;
        int ce;
        long long cS;
        if (ss_from_double(cur, ce, cS) && ce == ej) {
          S = cS;  // exact: cur is a multiple of its ulp
          e = ej;
          imode = true;
        } else {
          s = cur;
          imode = false;
        }
      }
      if (okj && imode) {
        ChunkMap c = lane >= j && lane < nb ? mo : cm_identity();
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const ChunkMap o = cm_shfl_up(c, d);
          if (lane >= d) c = cm_compose(o, c);
        }
        const bool inr = S > 0 ? (S + c.pmin >= LO && S + c.pmax < HI) : (S + c.pmax <= -LO && S + c.pmin > -HI);
        const bool v = lane >= j && lane < nb && c.ok && c.e == e && inr;
        const unsigned inv = ~__ballot_sync(FULL, v) & (FULL << j);
        const int f = inv ? __ffs(inv) - 1 : 32;  // first chunk not covered
        if (f > j) {
          const long long B0 = __shfl_sync(FULL, c.A0, f - 1), B1 = __shfl_sync(FULL, c.A1, f - 1);
          S += (S & 1) ? B1 : B0;
          j = f;
          continue;
        }
      }
      // ---- warp-parallel exact fallback over chunk k ----
      const long k = k0 + j;
      long i0 = k * SS_C;
      int n = (int)(min(N, (k + 1) * SS_C) - i0);
      __syncwarp();
      if (pref_k == k) {
#pragma unroll
        for (int t = 0; t < SS_PER_LANE; t++) sx[0][lane + 32 * t] = pr[t];
      } else {
        for (int i = lane; i < n; i += 32) sx[0][i] = pos[3 * (i0 + i) + a];
      }
      pref_k = k + 1;
#pragma unroll
      for (int t = 0; t < SS_PER_LANE; t++) {
        const long i = pref_k * SS_C + lane + 32 * t;
        pr[t] = i < N ? pos[3 * i + a] : 0.0;
      }
      __syncwarp();
      for (int b = 0; b < n; b += 32) {
        int cnt = min(32, n - b);
        double xj = lane < cnt ? sx[0][b + lane] : 0.0;
        int c = 0;
        while (c < cnt) {
          if (!imode) {
            if (!ss_from_double(s, e, S)) {
              s = __dadd_rn(s, sx[0][b + c]);
              c++;
              continue;
            }
            imode = true;
          }
          bool act = lane >= c && lane < cnt;
          Elem el = act ? elem_in_ulps(xj, e) : Elem{0, 0, 0};
          Map2 mp = act ? elem_map(el) : Map2{0, 0, 0, 1};
          for (int d = 1; d < 32; d <<= 1) {
            Map2 o;
            o.i0 = __shfl_up_sync(FULL, mp.i0, d);
            o.i1 = __shfl_up_sync(FULL, mp.i1, d);
            o.q0 = __shfl_up_sync(FULL, mp.q0, d);
            o.q1 = __shfl_up_sync(FULL, mp.q1, d);
            if (lane >= d) mp = compose(o, mp);
          }
          long long Sj = S + ((S & 1) ? mp.i1 : mp.i0);
          // strictly inside the binade: a result of exactly 2^52 ulps may be the rounding of a sum
          // just below the power of two, whose true rounding is on the finer grid below it
          bool leaves = el.bad || !(S > 0 ? (Sj > LO && Sj < HI) : (Sj < -LO && Sj > -HI));
          unsigned bal = __ballot_sync(FULL, act && leaves);
          if (bal == 0) {
            S = __shfl_sync(FULL, Sj, cnt - 1);
            c = cnt;
          } else {
            int x = __ffs(bal) - 1;
            long long Sb = __shfl_sync(FULL, Sj, x > 0 ? x - 1 : 0);
            if (x == c) Sb = S;
            s = __dadd_rn(ss_to_double(Sb, e), sx[0][b + x]);
            imode = false;
            c = x + 1;
          }
        }
      }
      j++;
    }
  }
  if (lane == 0) {
    if (imode) s = ss_to_double(S, e);
    out[a] = s;
  }
}

// out[0..2] = the three sequential sums; scratch must hold fmm_seqsum_scratch(N) bytes
size_t fmm_seqsum_scratch(long N) {
  long nch = (N + SS_C - 1) / SS_C;
  return (size_t)nch * 3 * (2 * sizeof(double) + sizeof(ChunkMap)) + 256;
}

int fmm_seqsum3(const double *pos, long N, double *out, void *scratch, cudaStream_t st) {
  long nch = (N + SS_C - 1) / SS_C;
  double *csum = (double *)scratch;
  double *start = csum + 3 * nch;
  ChunkMap *maps = (ChunkMap *)(start + 3 * nch);
  dim3 g((unsigned)((nch + 3) / 4), 3);
  fmm_note_launch(), k_ss_chunksum<<<g, 128, 0, st>>>(pos, N, nch, csum);
  fmm_note_launch(), k_ss_prefix<<<3, 1024, 0, st>>>(csum, nch, start);
  fmm_note_launch(), k_ss_maps<<<g, 128, 0, st>>>(pos, N, nch, start, maps);
  fmm_note_launch(), k_ss_chain<<<3, 32, 0, st>>>(pos, N, nch, maps, out);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}
