// m2l_tc.cu -- M2L on the fifth-generation tensor cores (tcgen05, kind::f16).
//
// The scaled M2L of a pair (B -> A) of translation class c is
//     L^_A[n] += sum_m T_c[m][n] M~_B[m],  T_c[m][n] = D_c[n + m] 2^(-dlev_c |m|),
// |n| + |m| <= p, |m| >= source_order (the contraction of
// fmmgen/expansions.py:144-172 in the scaled form of eval.cu).  For a tile of
// 128 target cells this is a sum of GEMMs, one per class c of the union of the
// tile's class-sorted lists:
//     D[128 x Nout] += A_c[128 x K] * T_c[K x Nout],
// where row i of A_c is the source multipole of target i in class c (zero when
// the target has no source of that class).  K runs over the multipole terms in
// chunks of 16 (one f16 MMA); since |n| <= p - |m|, a chunk whose lowest term
// has degree d only feeds the first NT(p - d) outputs, and its MMA uses that
// prefix as N (~2x the useful multiply-adds instead of ~9x for the square).
//
// FP32 accuracy from FP16 operands ("3xFP16"): each operand is brought near
// 2^14 by an exact power-of-two scale -- per source row for A, per (class,
// output column) for T -- and stored as hi + lo, both FP16, and each chunk
// issues hi*hi + hi*lo + lo*hi (relative product error ~2^-22).  The tensor
// cores' accumulator does not round to nearest, so each class step
// accumulates in a fresh tensor-memory buffer (33 MMAs deep at p = 8) and the
// epilogue warps multiply the step's result by the two scales and add it into
// FP32 registers with round-to-nearest -- the per-pair partial sums of the
// CUDA-core kernels.
//
// Tiles take 128 cells of one level and one octant-within-parent, parents in
// Morton order: those cells have near-identical interaction lists, so a tile
// visits ~1.4x the classes of one list.  The class steps of every tile (the
// sorted union of its rows' classes) and each step's source per row (-1 for a
// row without a source in the class) are scattered once per build straight
// from the walk-order pairs, with no sort (k_tc_bitmap .. k_tc_scatter): the
// kernel's warps then follow that schedule independently, coupled only
// through mbarriers.
//
// Per CTA (one per SM, persistent), 17 warps:
//  * warps 0-7 gather the source rows of each (class, 64-term K-block) step
//    (warps w and w+4: rows 32 (w % 4) .. + 31, one half of the chunks each)
//    into a stage slot with cp.async, in the 128-byte swizzled K-major layout,
//    and arrive on the slot's mbarrier when their copies land
//    (cp.async.mbarrier.arrive); thread 0 also fetches the class's pre-split
//    operator chunks (32-byte swizzled) and column scales with bulk copies.  A
//    row without a source in the class is not copied: its accumulator row
//    holds garbage that the fold leaves out;
//  * warps 8-15 fold each finished class step out of tensor memory (warps w
//    and w+4 take the two column halves of lane quarter w % 4) and store the
//    tile's rows;
//  * warp 16 allocates 512 tensor-memory columns (two accumulators) and one of
//    its lanes issues the MMAs.
// Stage slots and accumulators circulate through mbarriers; every wait is
// bounded and reports a timeout through an error flag instead of hanging.
#include <algorithm>
#include <cstddef>
#include <cuda.h>
#include <cuda_fp16.h>
#include <vector>
#include "internal.h"
#include "prims.cuh"

namespace {

constexpr int TC_ROWS = 128;      // target cells per tile (MMA M)
constexpr int TC_CH = 16;         // multipole terms per K chunk (one kind::f16 MMA)
constexpr int TC_KB = 64;         // terms per K-block: one 128-byte swizzle row of FP16
constexpr int TC_A_BYTES = TC_ROWS * 128;  // one operand half (hi or lo) of a K-block
constexpr int TC_MAXCH = 16;      // K chunks (p <= 9: at most 14)
constexpr int TC_MAXKB = 4;
constexpr int TC_GWARPS = 8;      // gather warps 0-7
constexpr int TC_FWARPS = 8;      // fold warps 8-15
constexpr int TC_MWARP = TC_GWARPS + TC_FWARPS;  // warp 16: tensor memory + MMA issue
constexpr int TC_GATHER = 32 * TC_GWARPS;
constexpr int TC_FOLD = 32 * TC_FWARPS;
constexpr int TC_THREADS = 32 * (TC_MWARP + 1);
constexpr int TC_MAXSLOTS = 4;
constexpr int TC_ACC_COLS = 256;  // tensor-memory columns per accumulator
constexpr int TC_EBIAS = 14;      // operands are scaled to [2^14, 2^15) in magnitude
constexpr unsigned TC_NONE = 0xffffffffu;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

struct TcParams {
  const int *order;               // cells in M2L processing order
  int ncells, ntiles;
  const int *sched_off;           // [ntiles + 1] class steps of each tile
  const unsigned *sched_cls;      // [steps] class of the step
  const int *stab;                // [steps][128] source cell of each tile row in the step, -1: none
  const __half *Mh, *Ml;          // scaled, split source multipoles, row stride kpad
  const int *mexp;                // per cell: row scale exponent (M~ = 2^mexp (Mh + Ml))
  const unsigned char *T;         // per class: split, swizzled operator chunks, then column scales
  float *L;                       // scaled local expansions (FP32), row stride lstride
  int lstride, lsize, kpad, kch, nkb, nslots;
  int cls_bytes, cls_scale, slot_bytes, nout;
  int nch[TC_MAXCH];              // MMA N of each K chunk
  int choff[TC_MAXCH + 1];        // byte offset of each chunk's (hi, lo) block in a class record
  uint32_t *err;                  // [0] bit 0: a gather-side wait timed out, bit 1: an MMA-side wait;
                                  // [2..3] class steps issued (u64, for the executed-work count)
};

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; i++) {
    if (mbar_try(bar, parity)) return true;
    if (i >= 32) __nanosleep(128);
  }
  return false;
}

__device__ __forceinline__ void cp16(uint32_t dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
// arrive on the mbarrier when all cp.async copies this thread issued so far have landed
__device__ __forceinline__ void cp_arrive(uint32_t bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// make this thread's generic-proxy shared-memory writes visible to the async proxy (tensor cores)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptors of K-major operands.  128-byte swizzle:
// rows of 128 bytes, 8-row groups 1024 bytes apart; 32-byte swizzle: rows of
// 32 bytes (one 8-term chunk), 8-row groups 256 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t sbo, uint32_t layout) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                           // leading byte offset (unused: K fits one swizzle row)
  d |= (uint64_t)(sbo >> 4) << 32;                  // stride byte offset: one 8-row group
  d |= (uint64_t)1 << 46;                           // descriptor version
  d |= (uint64_t)layout << 61;                      // swizzle mode
  return d;
}
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) { return smem_desc(saddr, 1024, 2); }
__device__ __forceinline__ uint64_t sw32_desc(uint32_t saddr) { return smem_desc(saddr, 256, 6); }
// Instruction descriptor: kind::f16 with FP16 A and B (both K-major), FP32
// accumulator, M = 128.
__device__ __forceinline__ uint32_t idesc_f16(int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_ROWS >> 4) << 24);
}
__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// arrive on the mbarrier once all MMAs this thread issued so far have completed
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 8 consecutive accumulator columns of this thread's lane (load and wait in
// one statement, so no register is read before the load has landed)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive accumulator columns in one load-and-wait statement
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive accumulator columns in one load-and-wait statement
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// x = 2^e (hi + lo) with hi, lo FP16 and |x 2^-e| in [2^14, 2^15) for the
// largest |x| of its row or column (e from that maximum)
__device__ __forceinline__ int scale_exp(float amax) {
  if (!(amax > 0.f) || !isfinite(amax)) return 0;
  return ilogbf(amax) - TC_EBIAS;
}
__device__ __forceinline__ void split_f16(float x, int e, __half &hi, __half &lo) {
  const float y = ldexpf(x, -e);  // exact: a power-of-two scale
  hi = __float2half_rn(y);
  lo = __float2half_rn(y - __half2float(hi));
}

}  // namespace

namespace {

// control block placed after the stage slots
struct TcShared {
  alignas(16) float colf[2][TC_ACC_COLS];  // column scales 2^g of the class in each accumulator (bulk-copy
                                           // destination: 16-byte aligned)
  uint64_t full[TC_MAXSLOTS];   // slot filled: 256 cp.async arrivals + thread 0's expect_tx arrival
  uint64_t empty[TC_MAXSLOTS];  // slot consumed: MMA commit
  uint64_t accfull[2];          // class step accumulated: MMA commit
  uint64_t accempty[2];         // accumulator folded out: 256 fold arrivals
  uint64_t colfull[2];          // column scales of the class in each accumulator landed (bulk copy)
  uint64_t drain;               // every MMA complete (before tensor memory is released)
  int hdr[TC_MAXSLOTS];         // K-block of the slot's step; -1: end of work
  uint32_t ch_idesc[TC_MAXCH];  // per K chunk: instruction descriptor (N of the chunk)
  uint32_t ch_boff[TC_MAXCH];   // per K chunk: offset of its hi block in the slot's operator area, >> 4
  uint32_t ch_nlo[TC_MAXCH];    // per K chunk: offset of its lo block from its hi block, >> 4
  uint32_t tmem;                // tensor-memory base address
  int sdl[2];                   // level-grid kernel: dlev of the class in each accumulator
  int lexp[8];                  // level-grid kernel: operand scale exponent of each level
};

// the structure starts 1024-byte aligned: bulk-copy destinations need 16
// bytes, mbarriers 8
static_assert(offsetof(TcShared, colf) % 16 == 0 && sizeof(TcShared::colf[0]) % 16 == 0, "colf alignment");
static_assert(offsetof(TcShared, full) % 8 == 0 && offsetof(TcShared, drain) % 8 == 0, "mbarrier alignment");

// Bounded wait of a whole warp: lane 0 waits, the outcome reaches every lane.
__device__ __forceinline__ bool warp_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok = 0;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity) ? 1u : 0u;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// Add class step v's accumulator (this thread's lane, HALF columns from col0),
// times its row scale 2^e and the class's column scales, into the FP32 running
// sums -- rows with a source in the step only -- and hand the accumulator back
// to the MMA issuer.
template <int HALF>
__device__ __forceinline__ bool fold(float *acc, uint32_t tlane, int col0, uint32_t v, int e, bool mine,
                                     uint32_t accfull0, uint32_t accempty0, uint32_t colfull0, TcShared *cs) {
  const uint32_t b = v & 1;
  if (!warp_wait(colfull0 + 8 * b, (v >> 1) & 1) || !warp_wait(accfull0 + 8 * b, (v >> 1) & 1)) return false;
  tc_fence_after();
  __syncwarp();  // tcgen05.ld is warp-collective
  const float rowf = ldexpf(1.f, e);
  const float *cf = cs->colf[b] + col0;
  // columns in loads of 16, then 8 (one wait each)
  constexpr int N16 = HALF / 16, N8 = (HALF % 16) / 8;
#pragma unroll
  for (int j = 0; j < N16; j++) {
    float t[16];
    tmem_ld16(tlane + b * TC_ACC_COLS + 16 * j, t);  // warp-collective: every lane loads
    if (mine)  // a row without a source in the step holds garbage: left out
#pragma unroll
      for (int i = 0; i < 16; i++) acc[16 * j + i] = fmaf(t[i], rowf * cf[16 * j + i], acc[16 * j + i]);
  }
  if (N8) {
    constexpr int c0 = 16 * N16;
    float t[8];
    tmem_ld8(tlane + b * TC_ACC_COLS + c0, t);
    if (mine)
#pragma unroll
      for (int i = 0; i < 8; i++) acc[c0 + i] = fmaf(t[i], rowf * cf[c0 + i], acc[c0 + i]);
  }
  tc_fence_before();
  mbar_arrive(accempty0 + 8 * b);
  return true;
}

template <int NOUT>
__global__ void __launch_bounds__(TC_THREADS, 1) k_m2l_tc(const TcParams P) {
  constexpr int HALF = NOUT / 2;  // accumulator columns folded by each epilogue thread
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const uint32_t raw = su32(tc_smem);
  const uint32_t base = (raw + 1023u) & ~1023u;  // the 128-byte swizzle pattern repeats every 1024 bytes
  TcShared *cs = (TcShared *)(tc_smem + (base - raw) + P.nslots * P.slot_bytes);
  const uint32_t full0 = su32(&cs->full[0]), empty0 = su32(&cs->empty[0]);
  const uint32_t accfull0 = su32(&cs->accfull[0]), accempty0 = su32(&cs->accempty[0]);
  const uint32_t colfull0 = su32(&cs->colfull[0]), drain = su32(&cs->drain);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid < TC_MAXCH) {
    const int ch = tid;
    cs->ch_idesc[ch] = ch < P.kch ? idesc_f16(P.nch[ch]) : 0u;
    cs->ch_boff[ch] = ch < P.kch ? (uint32_t)(P.choff[ch] - P.choff[ch & ~3]) >> 4 : 0u;
    cs->ch_nlo[ch] = ch < P.kch ? (uint32_t)P.nch[ch] * 2u : 0u;  // nch rows x 32 bytes, >> 4
  }
  if (tid == 0) {
    for (int i = 0; i < P.nslots; i++) {
      mbar_init(full0 + 8 * i, TC_GATHER + 1);  // every gather thread + thread 0's expect_tx
      mbar_init(empty0 + 8 * i, 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(accfull0 + 8 * i, 1);
      mbar_init(accempty0 + 8 * i, TC_FOLD);
      mbar_init(colfull0 + 8 * i, 1);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == TC_MWARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&cs->tmem)),
                 "r"(2 * TC_ACC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = cs->tmem;

  if (warp < TC_GWARPS) {
    // ---------------- gather ----------------
    const int quarter = warp & 3, chalf = warp >> 2;  // rows 32 quarter .. + 31, chunks 4 chalf .. + 3
    const int row = 32 * quarter + lane;  // tile row whose list this thread walks
    uint32_t g = 0, u = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < P.ntiles && ok; tile += gridDim.x) {
      const int s0 = P.sched_off[tile], s1 = P.sched_off[tile + 1];
      // the row's source in the next step, loaded a step before it is needed
      int hsrc = s0 < s1 ? P.stab[(size_t)s0 * TC_ROWS + row] : -1;
      for (int st = s0; st < s1; st++, u++) {
        const unsigned c = P.sched_cls[st];
        const int mysrc = hsrc;
        if (st + 1 < s1) hsrc = P.stab[(size_t)(st + 1) * TC_ROWS + row];
        for (int kb = 0; kb < P.nkb; kb++) {
          const int slot = (int)(g % (uint32_t)P.nslots);
          const uint32_t use = g / (uint32_t)P.nslots;
          if (!warp_wait(empty0 + 8 * slot, (use & 1) ^ 1)) { ok = false; break; }
          const uint32_t sa = base + (uint32_t)slot * P.slot_bytes;
          const int qn = min(8, (P.kpad - TC_KB * kb) >> 3);  // valid 16-byte chunks of the K-block
#pragma unroll
          for (int jj = 0; jj < 4; jj++) {
            const int rl = 8 * jj + (lane >> 2), q = 4 * chalf + (lane & 3);  // 8 rows x 4 chunks per instruction
            const int r = 32 * quarter + rl;
            const int sr = __shfl_sync(0xffffffffu, mysrc, rl);
            if (sr >= 0 && q < qn) {
              const size_t e = (size_t)sr * P.kpad + TC_KB * kb + 8 * q;
              const uint32_t o = (uint32_t)r * 128u + ((uint32_t)(q ^ (r & 7)) << 4);
              cp16(sa + o, P.Mh + e, 16u);
              cp16(sa + TC_A_BYTES + o, P.Ml + e, 16u);
            }
          }
          if (tid == 0) {
            cs->hdr[slot] = kb;
            const unsigned char *rec = P.T + (size_t)c * P.cls_bytes;
            const uint32_t b0 = P.choff[4 * kb], b1 = P.choff[min(4 * kb + 4, P.kch)];
            mbar_arrive_tx(full0 + 8 * slot, b1 - b0);
            bulk_g2s(sa + 2 * TC_A_BYTES, rec + b0, b1 - b0, full0 + 8 * slot);
            if (kb == 0) {
              // the class's column scales, for the fold of this step, into
              // buffer u & 1 once the fold of step u - 2 has read it
              const uint32_t cb = colfull0 + 8 * (u & 1), sc = 4u * (uint32_t)P.nout;
              if (!mbar_wait(accempty0 + 8 * (u & 1), ((u >> 1) & 1) ^ 1)) ok = false;
              fence_async_smem();
              mbar_arrive_tx(cb, sc);
              bulk_g2s(su32(cs->colf[u & 1]), rec + P.cls_scale, sc, cb);
            }
          }
          cp_arrive(full0 + 8 * slot);
          g++;
        }
        if (!__all_sync(0xffffffffu, ok)) ok = false;
        if (!ok) break;
      }
    }
    // end of work: one more slot carrying only the end mark
    if (ok) {
      const int slot = (int)(g % (uint32_t)P.nslots);
      const uint32_t use = g / (uint32_t)P.nslots;
      if (warp_wait(empty0 + 8 * slot, (use & 1) ^ 1)) {
        if (tid == 0) {
          cs->hdr[slot] = -1;
          mbar_arrive(full0 + 8 * slot);
        }
        mbar_arrive(full0 + 8 * slot);
      } else {
        ok = false;
      }
    }
    cp_wait_all();
    if (!ok && lane == 0) atomicOr(P.err, 1u);
    if (tid == 0) atomicAdd((unsigned long long *)(P.err + 2), (unsigned long long)u);
  } else if (warp < TC_MWARP) {
    // ---------------- fold + store ----------------
    const int fw = warp - TC_GWARPS;
    const int quarter = warp & 3, half = fw >> 2;  // tensor-memory lanes 32 (warp % 4) .. + 31
    const int row = 32 * quarter + lane;
    const uint32_t tlane = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(half * HALF);
    uint32_t u = 0;
    bool ok = true;
    float acc[HALF];
    for (int tile = blockIdx.x; tile < P.ntiles && ok; tile += gridDim.x) {
      const int rr = tile * TC_ROWS + row;
      const int A = rr < P.ncells ? P.order[rr] : -1;
      float *Lrow = A >= 0 ? P.L + (size_t)A * P.lstride + half * HALF : nullptr;
      const int ncol = min(HALF, P.lsize - half * HALF);  // stored columns of this half
#pragma unroll
      for (int i = 0; i < HALF; i++) acc[i] = 0.f;
      const int s0 = P.sched_off[tile], s1 = P.sched_off[tile + 1];
      int hsrc = s0 < s1 ? P.stab[(size_t)s0 * TC_ROWS + row] : -1;
      for (int st = s0; st < s1; st++, u++) {
        const bool mine = hsrc >= 0;
        const int e = mine ? P.mexp[hsrc] : 0;
        if (st + 1 < s1) hsrc = P.stab[(size_t)(st + 1) * TC_ROWS + row];
        if (!fold<HALF>(acc, tlane, half * HALF, u, e, mine, accfull0, accempty0, colfull0, cs)) {
          ok = false;
          break;
        }
      }
      if (!ok) break;
      if (Lrow)
#pragma unroll
        for (int i = 0; i < HALF; i++)
          if (i < ncol) Lrow[i] = acc[i];
    }
    if (!ok && lane == 0) atomicOr(P.err, 1u);
  } else if (lane == 0) {
    // ---------------- MMA issue (one thread of warp 16) ----------------
    // Per-chunk instruction descriptors and operator offsets live in
    // registers (compile-time indices below), so nothing but descriptor
    // arithmetic sits between consecutive MMAs.
    uint32_t idr[TC_MAXCH], bor[TC_MAXCH], nlr[TC_MAXCH];
#pragma unroll
    for (int ch = 0; ch < TC_MAXCH; ch++) {
      idr[ch] = cs->ch_idesc[ch];
      bor[ch] = cs->ch_boff[ch];
      nlr[ch] = cs->ch_nlo[ch];
    }
    const int kch = P.kch;
    uint32_t g = 0, u = 0;
    bool ok = true;
    while (true) {
      const int slot = (int)(g % (uint32_t)P.nslots);
      if (!mbar_wait(full0 + 8 * slot, (g / (uint32_t)P.nslots) & 1)) { ok = false; break; }
      fence_async_smem();  // the gathered rows were written by cp.async (generic proxy)
      tc_fence_after();
      const int kb = cs->hdr[slot];
      if (kb < 0) break;
      const uint32_t b = u & 1;
      if (kb == 0) {  // a class step starts: its accumulator must have been folded out
        if (!mbar_wait(accempty0 + 8 * b, ((u >> 1) & 1) ^ 1)) { ok = false; break; }
        tc_fence_after();
      }
      // descriptors: the slot's base descriptors plus per-chunk offsets in
      // 16-byte units (all shared addresses stay below 256 KB, so the 14-bit
      // start-address field never carries)
      const uint32_t sa = base + (uint32_t)slot * P.slot_bytes;
      const uint64_t ah0 = sw128_desc(sa), al0 = sw128_desc(sa + TC_A_BYTES);
      const uint64_t b0 = sw32_desc(sa + 2 * TC_A_BYTES);
      const uint32_t d = tmem + b * TC_ACC_COLS;
#define TC_CHUNK(KB, J)                                                                 \
  if (4 * (KB) + (J) < kch) {                                                           \
    const uint64_t bh = b0 + bor[4 * (KB) + (J)], bl = bh + nlr[4 * (KB) + (J)];        \
    const uint64_t ah = ah0 + 2 * (J), al = al0 + 2 * (J); /* 32 bytes along the row */ \
    mma_f16(d, ah, bh, idr[4 * (KB) + (J)], ((KB) == 0 && (J) == 0) ? 0u : 1u);         \
    mma_f16(d, ah, bl, idr[4 * (KB) + (J)], 1u);                                        \
    mma_f16(d, al, bh, idr[4 * (KB) + (J)], 1u);                                        \
  }
#define TC_KBLOCK(KB) \
  TC_CHUNK(KB, 0)     \
  TC_CHUNK(KB, 1)     \
  TC_CHUNK(KB, 2)     \
  TC_CHUNK(KB, 3)
      switch (kb) {
        case 0: { TC_KBLOCK(0) } break;
        case 1: { TC_KBLOCK(1) } break;
        case 2: { TC_KBLOCK(2) } break;
        default: { TC_KBLOCK(3) } break;
      }
#undef TC_KBLOCK
#undef TC_CHUNK
      mma_commit(empty0 + 8 * slot);
      if (kb == P.nkb - 1) {
        mma_commit(accfull0 + 8 * b);
        u++;
      }
      g++;
    }
    // every MMA issued has completed before tensor memory is released
    mma_commit(drain);
    if (!mbar_wait(drain, 0)) ok = false;
    if (!ok) atomicOr(P.err, 2u);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == TC_MWARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_ACC_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Level-grid variant (complete levels): source rows by TMA box loads
// ---------------------------------------------------------------------------
// When every level of a one-system tree is complete (all 8^l cells exist, as
// in the uniform configurations), the sources of a tile's rows in one class
// are a box of one level's cells: tile rows are the 128 targets of one level
// and one octant o whose parents fill an 8 x 4 x 4 box (row x + 8 y + 32 z),
// so for a same-level class (centre offset d = A - B) the sources 2 p + o - d / 2
// share one parity and fill an 8 x 4 x 4 box of that parity's sub-grid, and
// for a class whose source is one level coarser they fill an 8 x 4 x 4 box of
// that level's grid.  The multipoles of every level are kept as such dense
// grids of FP16 (hi, lo) rows, 64-term K-blocks per plane, and one tensor-map
// copy (cp.async.bulk.tensor, 128-byte swizzle) per (K-block, hi or lo)
// lands a class step's operand in the K-major layout the MMA reads; cells
// outside the level read as zeros.  Rows whose target has no pair of the
// class (targets of one octant can differ in their lists) are left out by
// the fold through a per-step row mask.  The operand scale is one power of
// two per level (the largest |M~| of the level brought to [2^14, 2^15)), so
// no per-row scale travels with the rows.
// Each K chunk's three products are issued as hi x lo, hi x hi, lo x hi, so
// that consecutive MMAs share an operand; a chunk whose multipole terms all
// have degree >= TCG_SPLIT_DEG issues hi x hi alone: its part of a local
// expansion is below (sqrt(3) s / R)^6 ~ 2e-4 of the whole at theta = 0.5, so
// the two dropped corrections (2^-11 of it) stay near 1e-7 relative, far
// below the expansion's truncation error (the operand fetch of these narrow
// MMAs, not their arithmetic, sets the kernel's pace).
// Warps: lane 0 of warp w < nslots (0-3) issues the fills of slot w (two
// tensor copies and the operator chunks), lane 1 of warp 0 the column scales
// of every step in order; 4-11 fold; 12 allocates tensor memory and issues
// MMAs.  Every slot and every barrier has one waiter that moves through its
// phases in order, and every role walks the tile schedule itself.
constexpr int TCG_MAXLEV = 8;                      // levels 0..7
constexpr int TCG_PWARPS = 4;                      // producer warps 0-3
constexpr int TCG_MWARP = TCG_PWARPS + TC_FWARPS;  // warp 12
constexpr int TCG_THREADS = 32 * (TCG_MWARP + 1);
constexpr int TCG_SPLIT_DEG = 6;                   // chunks of higher degrees: one product
static_assert(TC_MAXSLOTS <= TCG_PWARPS, "one producer warp per slot");

struct TcgMaps {
  CUtensorMap split[TCG_MAXLEV];  // level l: parity sub-grids (dlev 0 sources)
  CUtensorMap full[TCG_MAXLEV];   // level l: whole grid (sources one level coarser than their targets)
};

struct TcgParams {
  const int *order;           // [ntiles * 128] target cell of each tile row, -1: none
  const int4 *tinfo;          // [ntiles] (level | octant << 8, parent box origin x, y, z)
  int ntiles;
  const int *sched_off;       // [ntiles + 1]
  const unsigned *sched_cls;  // [steps]
  const unsigned *mask;       // [steps][4] rows with a pair of the step's class
  const int *key4;            // [classes][4] dlev, dx, dy, dz
  const unsigned *levmax;     // [TCG_MAXLEV] largest |M~| of each level (FP32 bits)
  const unsigned char *T;
  float *L;
  int lstride, lsize, kch, nkb, nslots, cls_bytes, cls_scale, slot_bytes, nout;
  int nfull;                  // leading K chunks with all three products (the rest: hi x hi only)
  int nch[TC_MAXCH];
  int choff[TC_MAXCH + 1];
  uint32_t *err;              // as TcParams::err
};

__device__ __forceinline__ void tma_box5(uint32_t dst, const CUtensorMap *map, int c1, int c2, int c3, int c4,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(dst),
      "l"(map), "r"(0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

// Fold of the level-grid kernel: as fold(), with the step's row factor 2^e
// (one per source level, from shared memory) and the accumulator read 32
// columns per wait.
template <int HALF>
__device__ __forceinline__ bool fold_g(float *acc, uint32_t tlane, int col0, uint32_t v, bool mine,
                                       uint32_t accfull0, uint32_t accempty0, uint32_t colfull0, int lev,
                                       TcShared *cs) {
  const uint32_t b = v & 1;
  if (!warp_wait(colfull0 + 8 * b, (v >> 1) & 1) || !warp_wait(accfull0 + 8 * b, (v >> 1) & 1)) return false;
  tc_fence_after();
  __syncwarp();  // tcgen05.ld is warp-collective
  const float rowf = ldexpf(1.f, cs->lexp[lev + cs->sdl[b]]);
  const float *cf = cs->colf[b] + col0;
  const uint32_t ta = tlane + b * TC_ACC_COLS;
  constexpr int N32 = HALF > 64 ? 0 : HALF / 32;  // wide loads only where the registers allow
  constexpr int N16 = (HALF - 32 * N32) / 16, R8 = (HALF % 16) / 8;
#pragma unroll
  for (int j = 0; j < N32; j++) {
    float t[32];
    tmem_ld32(ta + 32 * j, t);
    if (mine)  // a row without a pair of the step's class holds garbage: left out
#pragma unroll
      for (int i = 0; i < 32; i++) acc[32 * j + i] = fmaf(t[i], rowf * cf[32 * j + i], acc[32 * j + i]);
  }
#pragma unroll
  for (int j = 0; j < N16; j++) {
    constexpr int c0 = 32 * N32;
    float t[16];
    tmem_ld16(ta + c0 + 16 * j, t);
    if (mine)
#pragma unroll
      for (int i = 0; i < 16; i++) acc[c0 + 16 * j + i] = fmaf(t[i], rowf * cf[c0 + 16 * j + i], acc[c0 + 16 * j + i]);
  }
  if (R8) {
    constexpr int c0 = HALF - 8;
    float t[8];
    tmem_ld8(ta + c0, t);
    if (mine)
#pragma unroll
      for (int i = 0; i < 8; i++) acc[c0 + i] = fmaf(t[i], rowf * cf[c0 + i], acc[c0 + i]);
  }
  tc_fence_before();
  mbar_arrive(accempty0 + 8 * b);
  return true;
}

template <int NOUT>
__global__ void __launch_bounds__(TCG_THREADS, 1) k_m2l_tcg(const __grid_constant__ TcgMaps maps, const TcgParams P) {
  constexpr int HALF = NOUT / 2;
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const uint32_t raw = su32(tc_smem);
  const uint32_t base = (raw + 1023u) & ~1023u;
  TcShared *cs = (TcShared *)(tc_smem + (base - raw) + P.nslots * P.slot_bytes);
  const uint32_t full0 = su32(&cs->full[0]), empty0 = su32(&cs->empty[0]);
  const uint32_t accfull0 = su32(&cs->accfull[0]), accempty0 = su32(&cs->accempty[0]);
  const uint32_t colfull0 = su32(&cs->colfull[0]), drain = su32(&cs->drain);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid < TC_MAXCH) {
    const int ch = tid;
    cs->ch_idesc[ch] = ch < P.kch ? idesc_f16(P.nch[ch]) : 0u;
    cs->ch_boff[ch] = ch < P.kch ? (uint32_t)(P.choff[ch] - P.choff[ch & ~3]) >> 4 : 0u;
    cs->ch_nlo[ch] = ch < P.kch ? (uint32_t)P.nch[ch] * 2u : 0u;
  }
  if (tid == 0) {
    for (int i = 0; i < P.nslots; i++) {
      mbar_init(full0 + 8 * i, 1);  // the producer's expect_tx arrival (+ the copies' bytes)
      mbar_init(empty0 + 8 * i, 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(accfull0 + 8 * i, 1);
      mbar_init(accempty0 + 8 * i, TC_FOLD);
      mbar_init(colfull0 + 8 * i, 1);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < TCG_MAXLEV) cs->lexp[tid] = scale_exp(__uint_as_float(P.levmax[tid]));
  if (warp == TCG_MWARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&cs->tmem)),
                 "r"(2 * TC_ACC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = cs->tmem;

  if (warp < TCG_PWARPS) {
    if (lane == 0 && warp < P.nslots) {
      // ---------------- producer of slot `warp`: fills g with g % nslots == warp ----------------
      uint32_t g = 0, u = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < P.ntiles && ok; tile += gridDim.x) {
        const int4 ti = P.tinfo[tile];
        const int lev = ti.x & 255, o = ti.x >> 8;
        const int ox = o & 1, oy = (o >> 1) & 1, oz = o >> 2;
        const int s0 = P.sched_off[tile], s1 = P.sched_off[tile + 1];
        for (int st = s0; st < s1 && ok; st++, u++) {
          const unsigned c = P.sched_cls[st];
          const int4 k4 = *(const int4 *)(P.key4 + 4 * (size_t)c);
          const CUtensorMap *map;
          int x0, y0, z0, pl0;
          if (k4.x == 0) {  // same level: sources 2 p + o - d / 2 (d even), one parity
            const int ax = ox - (k4.y >> 1), ay = oy - (k4.z >> 1), az = oz - (k4.w >> 1);
            const int px = ax & 1, py = ay & 1, pz = az & 1;
            x0 = ti.y + ((ax - px) >> 1);
            y0 = ti.z + ((ay - py) >> 1);
            z0 = ti.w + ((az - pz) >> 1);
            pl0 = (px + 2 * py + 4 * pz) * 2 * P.nkb;
            map = &maps.split[lev];
          } else {  // one level coarser: sources p + (2 o - 1 - d) / 4
            x0 = ti.y + ((2 * ox - 1 - k4.y) >> 2);
            y0 = ti.z + ((2 * oy - 1 - k4.z) >> 2);
            z0 = ti.w + ((2 * oz - 1 - k4.w) >> 2);
            pl0 = 0;
            map = &maps.full[lev - 1];
          }
          for (int kb = 0; kb < P.nkb; kb++, g++) {
            const int slot = (int)(g % (uint32_t)P.nslots);
            if (slot != warp) continue;
            const uint32_t use = g / (uint32_t)P.nslots;
            if (!mbar_wait(empty0 + 8 * slot, (use & 1) ^ 1)) { ok = false; break; }
            const uint32_t sa = base + (uint32_t)slot * P.slot_bytes, fb = full0 + 8 * slot;
            const unsigned char *rec = P.T + (size_t)c * P.cls_bytes;
            const uint32_t b0 = P.choff[4 * kb], b1 = P.choff[min(4 * kb + 4, P.kch)];
            mbar_arrive_tx(fb, 2u * TC_A_BYTES + (b1 - b0));
            tma_box5(sa, map, x0, y0, z0, pl0 + 2 * kb, fb);
            tma_box5(sa + TC_A_BYTES, map, x0, y0, z0, pl0 + 2 * kb + 1, fb);
            bulk_g2s(sa + 2 * TC_A_BYTES, rec + b0, b1 - b0, fb);
          }
        }
      }
      if (!ok) atomicOr(P.err, 1u);
      if (warp == 0) atomicAdd((unsigned long long *)(P.err + 2), (unsigned long long)u);
    } else if (warp == 0 && lane == 1) {
      // ---------------- column scales of every step, in step order ----------------
      // step u's scales into buffer u & 1 once the fold of step u - 2 has read it
      uint32_t u = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < P.ntiles && ok; tile += gridDim.x) {
        const int s0 = P.sched_off[tile], s1 = P.sched_off[tile + 1];
        for (int st = s0; st < s1; st++, u++) {
          const unsigned c = P.sched_cls[st];
          const int dl = P.key4[4 * (size_t)c];
          const unsigned char *rec = P.T + (size_t)c * P.cls_bytes;
          const uint32_t cb = colfull0 + 8 * (u & 1), sc = 4u * (uint32_t)P.nout;
          if (!mbar_wait(accempty0 + 8 * (u & 1), ((u >> 1) & 1) ^ 1)) { ok = false; break; }
          cs->sdl[u & 1] = dl;  // read by the fold after the scales land (the arrival releases it)
          fence_async_smem();
          mbar_arrive_tx(cb, sc);
          bulk_g2s(su32(cs->colf[u & 1]), rec + P.cls_scale, sc, cb);
        }
      }
      if (!ok) atomicOr(P.err, 1u);
    }
  } else if (warp < TCG_MWARP) {
    // ---------------- fold + store ----------------
    const int fw = warp - TCG_PWARPS;
    const int quarter = warp & 3, half = fw >> 2;  // tensor-memory lanes 32 (warp % 4) .. + 31
    const int row = 32 * quarter + lane;
    const uint32_t tlane = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(half * HALF);
    uint32_t u = 0;
    bool ok = true;
    float acc[HALF];
    for (int tile = blockIdx.x; tile < P.ntiles && ok; tile += gridDim.x) {
      const int A = P.order[(size_t)tile * TC_ROWS + row];
      const int lev = P.tinfo[tile].x & 255;
      float *Lrow = A >= 0 ? P.L + (size_t)A * P.lstride + half * HALF : nullptr;
      const int ncol = min(HALF, P.lsize - half * HALF);
#pragma unroll
      for (int i = 0; i < HALF; i++) acc[i] = 0.f;
      const int s0 = P.sched_off[tile], s1 = P.sched_off[tile + 1];
      // the row mask word of the next step, loaded a step before it is needed
      unsigned mw = s0 < s1 ? P.mask[4 * (size_t)s0 + quarter] : 0u;
      for (int st = s0; st < s1; st++, u++) {
        const bool mine = (mw >> lane) & 1u;
        if (st + 1 < s1) mw = P.mask[4 * (size_t)(st + 1) + quarter];
        if (!fold_g<HALF>(acc, tlane, half * HALF, u, mine, accfull0, accempty0, colfull0, lev, cs)) {
          ok = false;
          break;
        }
      }
      if (!ok) break;
      if (Lrow)
#pragma unroll
        for (int i = 0; i < HALF; i++)
          if (i < ncol) Lrow[i] = acc[i];
    }
    if (!ok && lane == 0) atomicOr(P.err, 1u);
  } else if (lane == 0) {
    // ---------------- MMA issue (one thread of warp 12) ----------------
    uint32_t idr[TC_MAXCH], bor[TC_MAXCH], nlr[TC_MAXCH];
#pragma unroll
    for (int ch = 0; ch < TC_MAXCH; ch++) {
      idr[ch] = cs->ch_idesc[ch];
      bor[ch] = cs->ch_boff[ch];
      nlr[ch] = cs->ch_nlo[ch];
    }
    // the thread walks the schedule itself (a shared-memory load issued behind
    // MMAs that are still reading their operands waits for them)
    const int kch = P.kch, nfull = P.nfull;
    uint32_t g = 0, u = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < P.ntiles && ok; tile += gridDim.x) {
    const int nst = P.sched_off[tile + 1] - P.sched_off[tile];
    for (int st = 0; st < nst && ok; st++) {
    for (int kb = 0; kb < P.nkb; kb++) {
      const int slot = (int)(g % (uint32_t)P.nslots);
      if (!mbar_wait(full0 + 8 * slot, (g / (uint32_t)P.nslots) & 1)) { ok = false; break; }
      tc_fence_after();
      const uint32_t b = u & 1;
      if (kb == 0) {
        if (!mbar_wait(accempty0 + 8 * b, ((u >> 1) & 1) ^ 1)) { ok = false; break; }
        tc_fence_after();
      }
      const uint32_t sa = base + (uint32_t)slot * P.slot_bytes;
      const uint64_t ah0 = sw128_desc(sa), al0 = sw128_desc(sa + TC_A_BYTES);
      const uint64_t b0 = sw32_desc(sa + 2 * TC_A_BYTES);
      const uint32_t d = tmem + b * TC_ACC_COLS;
#define TC_CHUNK(KB, J)                                                                 \
  if (4 * (KB) + (J) < kch) {                                                           \
    const uint64_t bh = b0 + bor[4 * (KB) + (J)], bl = bh + nlr[4 * (KB) + (J)];        \
    const uint64_t ah = ah0 + 2 * (J), al = al0 + 2 * (J); /* 32 bytes along the row */ \
    if (4 * (KB) + (J) < nfull) {                                                       \
      mma_f16(d, ah, bl, idr[4 * (KB) + (J)], ((KB) == 0 && (J) == 0) ? 0u : 1u);       \
      mma_f16(d, ah, bh, idr[4 * (KB) + (J)], 1u);                                      \
      mma_f16(d, al, bh, idr[4 * (KB) + (J)], 1u);                                      \
    } else {                                                                            \
      mma_f16(d, ah, bh, idr[4 * (KB) + (J)], 1u);                                      \
    }                                                                                   \
  }
#define TC_KBLOCK(KB) \
  TC_CHUNK(KB, 0)     \
  TC_CHUNK(KB, 1)     \
  TC_CHUNK(KB, 2)     \
  TC_CHUNK(KB, 3)
      switch (kb) {
        case 0: { TC_KBLOCK(0) } break;
        case 1: { TC_KBLOCK(1) } break;
        case 2: { TC_KBLOCK(2) } break;
        default: { TC_KBLOCK(3) } break;
      }
#undef TC_KBLOCK
#undef TC_CHUNK
      mma_commit(empty0 + 8 * slot);
      if (kb == P.nkb - 1) {
        mma_commit(accfull0 + 8 * b);
        u++;
      }
      g++;
    }
    }
    }
    mma_commit(drain);
    if (!mbar_wait(drain, 0)) ok = false;
    if (!ok) atomicOr(P.err, 2u);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == TCG_MWARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_ACC_COLS)
                 : "memory");
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// operands
// ---------------------------------------------------------------------------
namespace {

struct TcPlan {
  int p, so, msize, lsize, kch, kpad, nkb, nout, cls_scale, cls_bytes, slot_bytes, nslots, smem;
  int nch[TC_MAXCH], choff[TC_MAXCH + 1];
};

bool tc_plan(int p, int so, TcPlan &pl) {
  if (p < 1 || p > 9 || so < 0 || so > 2 || p < so + 1) return false;
  pl.p = p;
  pl.so = so;
  const int moff = fmm_nterms(so - 1);
  pl.msize = fmm_nterms(p) - moff;
  pl.lsize = fmm_nterms(p - so);
  pl.kch = (pl.msize + TC_CH - 1) / TC_CH;
  pl.kpad = TC_CH * pl.kch;
  pl.nkb = (pl.kch + 3) / 4;
  if (pl.kch > TC_MAXCH || pl.nkb > TC_MAXKB) return false;
  pl.choff[0] = 0;
  for (int k = 0; k < pl.kch; k++) {
    const int dm = fmm_decode(moff + TC_CH * k).d;  // lowest degree in the chunk (terms sorted by degree)
    int nout = std::min(pl.lsize, fmm_nterms(p - dm));
    if (nout < 1) nout = 1;
    pl.nch[k] = (nout + 15) / 16 * 16;
    pl.choff[k + 1] = pl.choff[k] + 2 * pl.nch[k] * 32;  // (hi, lo) blocks of nch rows x 16 FP16
  }
  pl.nout = pl.nch[0];
  if (pl.nout > TC_ACC_COLS) return false;
  pl.cls_scale = pl.choff[pl.kch];
  pl.cls_bytes = (pl.cls_scale + 4 * pl.nout + 1023) / 1024 * 1024;
  int bmax = 0;
  for (int b = 0; b < pl.nkb; b++)
    bmax = std::max(bmax, pl.choff[std::min(4 * b + 4, pl.kch)] - pl.choff[4 * b]);
  pl.slot_bytes = (2 * TC_A_BYTES + bmax + 1023) / 1024 * 1024;
  const int budget = 227 * 1024 - 1024 - (int)sizeof(TcShared);
  pl.nslots = std::min(TC_MAXSLOTS, budget / pl.slot_bytes);
  if (pl.nslots < 2) return false;
  pl.smem = 1024 + pl.nslots * pl.slot_bytes + (int)sizeof(TcShared);
  return true;
}

// T_c[m][n] = D_c[n + m] 2^(-dlev |m|) in FP64 (0 outside |n| + |m| <= p)
__device__ __forceinline__ double op_entry(const double *D, int dlev, int p, int moff, int lsize, int msize, int n,
                                           int pos) {
  if (n >= lsize || pos >= msize) return 0.0;
  const MI nn = fmm_decode(n), mm = fmm_decode(moff + pos);
  if (nn.d + mm.d > p) return 0.0;
  return ldexp(D[fmm_idx3(nn.x + mm.x, nn.y + mm.y, nn.z + mm.z)], -dlev * (int)mm.d);
}

// Operator record of a class: per K chunk, the (hi, lo) FP16 blocks of
// 2^-g_n T_c[m][n] (row n, the chunk's 16 terms m) in the 32-byte swizzled
// K-major layout (the two 16-byte halves of row n trade places when bit 2 of n
// is set), then the column scales 2^g_n as FP32.
// (skipped when `same` is given and set: the records of the previous build hold)
__global__ void k_tc_operators(const double *D64, const int *key4, int ncls, TcPlan pl, unsigned char *T,
                               const uint32_t *same) {
  __shared__ int g[TC_ACC_COLS];
  const int c = blockIdx.x;
  if (c >= ncls || (same && *same)) return;
  const int moff = fmm_nterms(pl.so - 1);
  const double *D = D64 + (size_t)c * fmm_nterms(pl.p);
  const int dlev = key4[4 * c];
  unsigned char *rec = T + (size_t)c * pl.cls_bytes;
  for (int n = threadIdx.x; n < pl.nout; n += blockDim.x) {
    double mx = 0.0;
    for (int pos = 0; pos < pl.msize; pos++)
      mx = fmax(mx, fabs(op_entry(D, dlev, pl.p, moff, pl.lsize, pl.msize, n, pos)));
    const int e = mx > 0.0 ? ilogb(mx) - TC_EBIAS : 0;
    g[n] = e;
    ((float *)(rec + pl.cls_scale))[n] = ldexpf(1.f, e);
  }
  __syncthreads();
  for (int k = 0; k < pl.kch; k++) {
    const int nr = pl.nch[k];
    __half *blk = (__half *)(rec + pl.choff[k]);
    for (int i = threadIdx.x; i < nr * 16; i += blockDim.x) {
      const int n = i >> 4, pe = i & 15;
      const int e16 = ((((pe >> 3) ^ (n >> 2)) & 1) << 3) | (pe & 7);  // term of the chunk stored here
      const double y = ldexp(op_entry(D, dlev, pl.p, moff, pl.lsize, pl.msize, n, TC_CH * k + e16), -g[n]);
      const __half hi = __float2half_rn((float)y);
      blk[i] = hi;
      blk[nr * 16 + i] = __float2half_rn((float)(y - (double)__half2float(hi)));
    }
  }
}

// Class steps of every tile, from the walk-order M2L pairs (tgt, src, cls):
//  k_tc_pos     row of each cell in the processing order;
//  k_tc_bitmap  per tile, a bitmap over the classes of its rows' pairs;
//  k_tc_rank    per tile, the exclusive prefix of the words' popcounts (the
//               step of a class is its rank in the tile's bitmap) and the
//               tile's step count;
//  k_tc_steps   the class of every step;
//  k_tc_scatter the source of every pair into its (step, row) slot.
// The steps of a tile are its classes in increasing order, as the union of
// its rows' class-sorted lists would give.
#define TC_SCHED_MAXW 8192  // bitmap words: classes up to 262,144
__global__ void k_tc_pos(const int *order, int ncells, int *pos) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < ncells) pos[order[r]] = r;
}

// Bitmaps of all tiles, each block over a slice of the pairs into a private
// copy in shared memory, written out whole (part[block][nbm]); k_tc_bitmap_or
// then ORs the copies.  (Pairs of one word come from every part of the walk,
// so atomics on one global copy serialise on a few hot words.)
__global__ void k_tc_bitmap_part(const int *tgt, const int *cls, long n, const int *pos, int nwords, int nbm,
                                 unsigned *part) {
  extern __shared__ unsigned sbm[];
  for (int i = threadIdx.x; i < nbm; i += blockDim.x) sbm[i] = 0u;
  __syncthreads();
  const long per = (n + gridDim.x - 1) / gridDim.x, k0 = blockIdx.x * per, k1 = min(n, k0 + per);
  for (long k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const unsigned c = (unsigned)cls[k];
    atomicOr(sbm + (pos[tgt[k]] / TC_ROWS) * nwords + (c >> 5), 1u << (c & 31));
  }
  __syncthreads();
  unsigned *out = part + (size_t)blockIdx.x * nbm;
  for (int i = threadIdx.x; i < nbm; i += blockDim.x) out[i] = sbm[i];
}
__global__ void k_tc_bitmap_or(const unsigned *part, int nparts, int nbm, unsigned *bm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbm) return;
  unsigned v = 0u;
  for (int b = 0; b < nparts; b++) v |= part[(size_t)b * nbm + i];
  bm[i] = v;
}
// the same on one global copy, for bitmaps too large for shared memory
__global__ void k_tc_bitmap(const int *tgt, const int *cls, long n, const int *pos, int nwords, unsigned *bm) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned c = (unsigned)cls[k];
  atomicOr(bm + (size_t)(pos[tgt[k]] / TC_ROWS) * nwords + (c >> 5), 1u << (c & 31));
}

// one block per tile
__global__ void k_tc_rank(const unsigned *bm, int nwords, unsigned *rank, int *count) {
  const unsigned *b = bm + (size_t)blockIdx.x * nwords;
  unsigned *rk = rank + (size_t)blockIdx.x * nwords;
  const int per = (nwords + blockDim.x - 1) / blockDim.x, w0 = threadIdx.x * per;
  unsigned n = 0;
  for (int i = 0; i < per && w0 + i < nwords; i++) n += __popc(b[w0 + i]);
  unsigned tot;
  unsigned run = block_exclusive<unsigned>(n, &tot);
  for (int i = 0; i < per && w0 + i < nwords; i++) {
    rk[w0 + i] = run;
    run += __popc(b[w0 + i]);
  }
  if (threadIdx.x == 0) count[blockIdx.x] = (int)tot;
}

// one block per tile, a thread per bitmap word
__global__ void k_tc_steps(const unsigned *bm, const unsigned *rank, int nwords, const int *sched_off,
                           unsigned *cls_out) {
  const size_t o = (size_t)blockIdx.x * nwords;
  for (int w = threadIdx.x; w < nwords; w += blockDim.x) {
    unsigned m = bm[o + w];
    unsigned st = (unsigned)sched_off[blockIdx.x] + rank[o + w];
    while (m) {
      const int b = __ffs(m) - 1;
      cls_out[st++] = 32u * (unsigned)w + (unsigned)b;
      m &= m - 1;
    }
  }
}

__global__ void k_tc_scatter(const int *tgt, const int *src, const int *cls, long n, const int *pos,
                             const unsigned *bm, const unsigned *rank, int nwords, const int *sched_off, int *stab) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int row = pos[tgt[k]], tile = row / TC_ROWS;
  const unsigned c = (unsigned)cls[k];
  const size_t w = (size_t)tile * nwords + (c >> 5);
  const unsigned st = (unsigned)sched_off[tile] + rank[w] + __popc(bm[w] & ((1u << (c & 31)) - 1u));
  stab[(size_t)st * TC_ROWS + (row % TC_ROWS)] = src[k];
}

// Source multipoles as 2^e (hi + lo), hi and lo FP16 rows of kpad terms, e per
// cell from the row's largest magnitude (one warp per cell).
__global__ void k_tc_split(const float *M, int ncells, int mstr, int msize, int kpad, __half *Mh, __half *Ml,
                           int *mexp) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncells) return;
  const float *row = M + (size_t)w * mstr;
  float mx = 0.f;
  for (int i = lane; i < msize; i += 32) mx = fmaxf(mx, fabsf(row[i]));
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int e = scale_exp(mx);
  if (lane == 0) mexp[w] = e;
  for (int i = lane; i < kpad; i += 32) {
    __half hi, lo;
    split_f16(i < msize ? row[i] : 0.f, e, hi, lo);
    Mh[(size_t)w * kpad + i] = hi;
    Ml[(size_t)w * kpad + i] = lo;
  }
}


// ---- level-grid operands and schedule ----
// raster index of every cell within its (complete) level
__global__ void k_tcg_gidx(const int *ix, const int *iy, const int *iz, const unsigned char *clevel, const int *loff,
                           int ncells, int *gidx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int l = clevel[c], n = 1 << l;
  gidx[loff[l] + (iz[c] * n + iy[c]) * n + ix[c]] = c;
}
// target cell of every tile row and each tile's (level, octant, parent box origin)
__global__ void k_tcg_tiles(const int *gidx, const int *loff, const int *toff, int nlev, int ntiles, int *order,
                            int4 *tinfo) {
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= (long)ntiles * TC_ROWS) return;
  const int tile = (int)(r / TC_ROWS), row = (int)(r % TC_ROWS);
  int l = 1;
  while (l + 1 < nlev && toff[l + 1] <= tile) l++;
  const int P = 1 << (l - 1), tx = (P + 7) / 8, ty = (P + 3) / 4, tz = ty;
  int k = tile - toff[l];
  const int o = k / (tx * ty * tz);
  k %= tx * ty * tz;
  const int bx = k % tx, by = (k / tx) % ty, bz = k / (tx * ty);
  const int px = 8 * bx + (row & 7), py = 4 * by + ((row >> 3) & 3), pz = 4 * bz + (row >> 5);
  int cell = -1;
  if (px < P && py < P && pz < P) {
    const int n = 2 * P;
    const int x = 2 * px + (o & 1), y = 2 * py + ((o >> 1) & 1), z = 2 * pz + (o >> 2);
    cell = gidx[loff[l] + (z * n + y) * n + x];
  }
  order[r] = cell;
  if (row == 0) tinfo[tile] = make_int4(l | (o << 8), 8 * bx, 4 * by, 4 * bz);
}
__global__ void k_tcg_pos(const int *order, long nrows, int *pos) {
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r < nrows && order[r] >= 0) pos[order[r]] = (int)r;
}
// every pair's source must be the cell the tile's box gives it: same level with
// an even offset, or one level coarser with the offset of a parent-level box;
// and no target may be the root (it is no tile row)
__global__ void k_tcg_check(const int *tgt, const int *src, const int *cls, long n, const int *key4, const int *ix,
                            const int *iy, const int *iz, const unsigned char *clevel, uint32_t *bad) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int A = tgt[k], B = src[k];
  const int4 k4 = *(const int4 *)(key4 + 4 * (size_t)cls[k]);
  bool ok;
  if (clevel[A] < 1) {
    ok = false;
  } else if (k4.x == 0) {
    ok = !(k4.y & 1) && !(k4.z & 1) && !(k4.w & 1) && ix[B] == ix[A] - (k4.y >> 1) && iy[B] == iy[A] - (k4.z >> 1) &&
         iz[B] == iz[A] - (k4.w >> 1) && clevel[B] == clevel[A];
  } else if (k4.x == -1) {
    const int qx = 2 * ix[A] - 1 - k4.y, qy = 2 * iy[A] - 1 - k4.z, qz = 2 * iz[A] - 1 - k4.w;
    ok = !(qx & 3) && !(qy & 3) && !(qz & 3) && ix[B] == (qx >> 2) && iy[B] == (qy >> 2) && iz[B] == (qz >> 2) &&
         clevel[B] + 1 == clevel[A];
  } else {
    ok = false;
  }
  if (!ok) atomicOr(bad, 1u);
}
// row masks: the bit of every pair's row in its (tile, class) step
__global__ void k_tcg_mask(const int *tgt, const int *cls, long n, const int *pos, const unsigned *bm,
                           const unsigned *rank, int nwords, const int *sched_off, unsigned *mask) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int row = pos[tgt[k]], tile = row / TC_ROWS, r = row % TC_ROWS;
  const unsigned c = (unsigned)cls[k];
  const size_t w = (size_t)tile * nwords + (c >> 5);
  const unsigned st = (unsigned)sched_off[tile] + rank[w] + __popc(bm[w] & ((1u << (c & 31)) - 1u));
  atomicOr(mask + 4 * (size_t)st + (r >> 5), 1u << (r & 31));
}
// largest |M~| of every level (FP32 bits; non-negative floats order as integers)
__global__ void k_tcg_levmax(const float *M, int ncells, int mstr, int msize, const unsigned char *clevel,
                             unsigned *levmax) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncells) return;
  const float *row = M + (size_t)w * mstr;
  float mx = 0.f;
  for (int i = lane; i < msize; i += 32) mx = fmaxf(mx, fabsf(row[i]));
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0 && mx > 0.f && isfinite(mx) && clevel[w] < TCG_MAXLEV) atomicMax(levmax + clevel[w], __float_as_uint(mx));
}
// Every cell's multipole as FP16 (hi, lo) rows scaled by its level's power of
// two, into the level's parity sub-grids and (levels that are coarser
// sources) its whole grid; thread per (cell, term).
struct TcgGrid {
  long soff[TCG_MAXLEV], foff[TCG_MAXLEV];  // element offsets (-1: none)
  int sx[TCG_MAXLEV], sy[TCG_MAXLEV];       // sub-grid extents (x; y = z)
  int fx[TCG_MAXLEV], fy[TCG_MAXLEV];       // whole-grid extents (x; y = z)
};
__global__ void k_tcg_pack(const float *M, int ncells, int mstr, int msize, int nkb, const int *ix, const int *iy,
                           const int *iz, const unsigned char *clevel, const unsigned *levmax, TcgGrid G,
                           __half *grid) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int kt = 64 * nkb;
  if (i >= (long)ncells * kt) return;
  const int c = (int)(i / kt), t = (int)(i % kt), kb = t >> 6, tt = t & 63;
  const int l = clevel[c];
  if (l >= TCG_MAXLEV) return;
  const int e = scale_exp(__uint_as_float(levmax[l]));
  __half hi, lo;
  split_f16(t < msize ? M[(size_t)c * mstr + t] : 0.f, e, hi, lo);
  const int x = ix[c], y = iy[c], z = iz[c];
  if (G.soff[l] >= 0) {
    const int par = (x & 1) + 2 * (y & 1) + 4 * (z & 1);
    const long pl = ((long)par * nkb + kb) * 2;
    const long sx = G.sx[l], sy = G.sy[l];
    const long cell = (((long)(z >> 1) * sy + (y >> 1)) * sx + (x >> 1));
    const long plane = sx * sy * sy;
    __half *q = grid + G.soff[l] + (pl * plane + cell) * 64 + tt;
    q[0] = hi;
    q[plane * 64] = lo;
  }
  if (G.foff[l] >= 0) {
    const long fx = G.fx[l], fy = G.fy[l];
    const long cell = ((long)z * fy + y) * fx + x;
    const long plane = fx * fy * fy;
    __half *q = grid + G.foff[l] + ((long)kb * 2 * plane + cell) * 64 + tt;
    q[0] = hi;
    q[plane * 64] = lo;
  }
}

int tc_sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  }
  return n;
}

template <int NOUT> int tc_launch(const TcParams &P, int smem, int grid, cudaStream_t st) {
  FMM_CUDA_TRY(cudaFuncSetAttribute(k_m2l_tc<NOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  fmm_note_launch(), k_m2l_tc<NOUT><<<grid, TC_THREADS, smem, st>>>(P);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// level-grid path: host side
// ---------------------------------------------------------------------------
namespace {

typedef CUresult (*TcgEncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

TcgEncodeFn tcg_encoder() {
  static TcgEncodeFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (TcgEncodeFn)p;
  }
  return fn;
}

// a tensor map over planes of (ext_y x ext_y x ext_x) cells of 64 FP16 terms;
// boxes of 8 x 4 x 4 cells of one plane, 128-byte swizzle
bool tcg_encode(CUtensorMap *m, void *base, int ext_x, int ext_y, int planes) {
  TcgEncodeFn enc = tcg_encoder();
  if (!enc) return false;
  const cuuint64_t dims[5] = {64, (cuuint64_t)ext_x, (cuuint64_t)ext_y, (cuuint64_t)ext_y, (cuuint64_t)planes};
  const cuuint64_t strides[4] = {128, 128ull * ext_x, 128ull * ext_x * ext_y, 128ull * ext_x * ext_y * ext_y};
  const cuuint32_t box[5] = {64, 8, 4, 4, 1};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct TcgState {
  uint64_t serial = ~0ull;  // build the state below belongs to
  int eligible = 0, nlev = 0, ntiles = 0, nsteps = 0, nkb = 0;
  TcgGrid G;
  TcgMaps maps;
  DevBuf<int> gidx, order, pos, sched_off, loff, toff;
  DevBuf<int4> tinfo;
  DevBuf<unsigned> sched_cls, bitmap, rank, mask, levmax, part;
  DevBuf<__half> grid;
  DevBuf<uint32_t> flag;
};

TcgState *tcg_state(DevTree *t) {
  if (!t->tcg) t->tcg = new TcgState();
  return (TcgState *)t->tcg;
}

// Schedule, grids and tensor maps of a build whose levels are all complete;
// eligible = 0 when the tree does not qualify (the row-gather kernel runs).
int tcg_prepare(DevTree *t, const TcPlan &pl, cudaStream_t st) {
  TcgState *s = tcg_state(t);
  s->serial = t->build_serial;
  s->nkb = pl.nkb;
  s->eligible = 0;
  const int nlev = t->nlevels, nc = t->ncells;
  if (t->nsys != 1 || nlev < 2 || nlev > TCG_MAXLEV || t->nclasses > 32 * TC_SCHED_MAXW || t->nm2l == 0)
    return FMM_OK;
  for (int l = 0; l < nlev; l++)
    if (t->level_off[l + 1] - t->level_off[l] != (1 << (3 * l))) return FMM_OK;
  // tiles: levels 1 .. nlev-1, eight octants, parent boxes of 8 x 4 x 4
  std::vector<int> toff(nlev + 1, 0);
  for (int l = 1; l < nlev; l++) {
    const int P = 1 << (l - 1), tx = (P + 7) / 8, ty = (P + 3) / 4;
    toff[l + 1] = toff[l] + 8 * tx * ty * ty;
  }
  const int ntiles = toff[nlev];
  s->ntiles = ntiles;
  s->nlev = nlev;
  const long nrows = (long)ntiles * TC_ROWS;
  const int nwords = (t->nclasses + 31) / 32;
  const size_t nbm = (size_t)ntiles * nwords;
  if (fmm_reserve(s->gidx, nc) || fmm_reserve(s->order, nrows) || fmm_reserve(s->pos, nc) ||
      fmm_reserve(s->sched_off, ntiles + 1) || fmm_reserve(s->loff, nlev + 1) || fmm_reserve(s->toff, nlev + 1) ||
      fmm_reserve(s->tinfo, ntiles) || fmm_reserve(s->bitmap, nbm) || fmm_reserve(s->rank, nbm) ||
      fmm_reserve(s->flag, 4) || fmm_reserve(s->levmax, TCG_MAXLEV) ||
      fmm_reserve(t->tmp, sizeof(int) * (ntiles + 1 + fmm_scan_tmp_elems<int>(ntiles))))
    return FMM_ERR_CUDA;
  FMM_CUDA_TRY(cudaMemcpyAsync(s->loff.p, t->level_off.data(), sizeof(int) * (nlev + 1), cudaMemcpyHostToDevice, st));
  FMM_CUDA_TRY(cudaMemcpyAsync(s->toff.p, toff.data(), sizeof(int) * (nlev + 1), cudaMemcpyHostToDevice, st));
  FMM_CUDA_TRY(cudaMemsetAsync(s->pos.p, 0xff, sizeof(int) * nc, st));
  FMM_CUDA_TRY(cudaMemsetAsync(s->flag.p, 0, sizeof(uint32_t) * 4, st));
  fmm_note_launch(), k_tcg_gidx<<<fmm_blocks(nc, 256), 256, 0, st>>>(t->ix.p, t->iy.p, t->iz.p, t->clevel.p,
                                                                     s->loff.p, nc, s->gidx.p);
  fmm_note_launch(), k_tcg_tiles<<<fmm_blocks(nrows, 256), 256, 0, st>>>(s->gidx.p, s->loff.p, s->toff.p, nlev,
                                                                         ntiles, s->order.p, s->tinfo.p);
  fmm_note_launch(), k_tcg_pos<<<fmm_blocks(nrows, 256), 256, 0, st>>>(s->order.p, nrows, s->pos.p);
  const long n = t->nm2l;
  fmm_note_launch(), k_tcg_check<<<fmm_blocks(n, 256), 256, 0, st>>>(t->m2l_tgt_raw.p, t->m2l_src_raw.p,
                                                                     t->m2l_cls_raw.p, n, t->cls_key4.p, t->ix.p,
                                                                     t->iy.p, t->iz.p, t->clevel.p, s->flag.p);
  const int nparts = 2 * tc_sm_count();
  if (nbm * sizeof(unsigned) <= 160 * 1024 && n >= 64L * nparts) {
    // per-block copies in shared memory, OR-reduced (no hot global atomics)
    const int sbytes = (int)(nbm * sizeof(unsigned));
    if (fmm_reserve(s->part, (size_t)nparts * nbm)) return FMM_ERR_CUDA;
    if (sbytes > 48 * 1024)
      FMM_CUDA_TRY(cudaFuncSetAttribute(k_tc_bitmap_part, cudaFuncAttributeMaxDynamicSharedMemorySize, sbytes));
    fmm_note_launch(), k_tc_bitmap_part<<<nparts, 512, sbytes, st>>>(t->m2l_tgt_raw.p, t->m2l_cls_raw.p, n, s->pos.p,
                                                                      nwords, (int)nbm, s->part.p);
    fmm_note_launch(), k_tc_bitmap_or<<<fmm_blocks(nbm, 256), 256, 0, st>>>(s->part.p, nparts, (int)nbm,
                                                                            s->bitmap.p);
  } else {
    FMM_CUDA_TRY(cudaMemsetAsync(s->bitmap.p, 0, sizeof(unsigned) * nbm, st));
    fmm_note_launch(), k_tc_bitmap<<<fmm_blocks(n, 256), 256, 0, st>>>(t->m2l_tgt_raw.p, t->m2l_cls_raw.p, n,
                                                                        s->pos.p, nwords, s->bitmap.p);
  }
  int *cnt = (int *)t->tmp.p, *stmp = cnt + ntiles + 1;
  fmm_note_launch(), k_tc_rank<<<ntiles, 256, 0, st>>>(s->bitmap.p, nwords, s->rank.p, cnt);
  if (int rc = fmm_scan<int>(cnt, s->sched_off.p, ntiles, s->sched_off.p + ntiles, stmp, st)) return rc;
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned + FMM_PINNED_SCRATCH, s->sched_off.p + ntiles, sizeof(int),
                               cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned + FMM_PINNED_SCRATCH + 1, s->flag.p, sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaStreamSynchronize(st));
  if (t->h_pinned[FMM_PINNED_SCRATCH + 1] != 0) return FMM_OK;  // a pair the boxes cannot give
  const int nsteps = (int)t->h_pinned[FMM_PINNED_SCRATCH];
  s->nsteps = nsteps;
  const size_t nst = nsteps > 0 ? (size_t)nsteps : 1;
  if (fmm_reserve(s->sched_cls, nst) || fmm_reserve(s->mask, 4 * nst)) return FMM_ERR_CUDA;
  fmm_note_launch(), k_tc_steps<<<ntiles, 128, 0, st>>>(s->bitmap.p, s->rank.p, nwords, s->sched_off.p,
                                                        s->sched_cls.p);
  FMM_CUDA_TRY(cudaMemsetAsync(s->mask.p, 0, sizeof(unsigned) * 4 * nst, st));
  fmm_note_launch(), k_tcg_mask<<<fmm_blocks(n, 256), 256, 0, st>>>(t->m2l_tgt_raw.p, t->m2l_cls_raw.p, n, s->pos.p,
                                                                     s->bitmap.p, s->rank.p, nwords, s->sched_off.p,
                                                                     s->mask.p);
  // grids: parity sub-grids of levels 1 .. nlev-1, whole grids of levels 0 .. nlev-2
  long off = 0;
  for (int l = 0; l < TCG_MAXLEV; l++) {
    s->G.soff[l] = s->G.foff[l] = -1;
    s->G.sx[l] = s->G.sy[l] = s->G.fx[l] = s->G.fy[l] = 0;
  }
  for (int l = 0; l < nlev; l++) {
    const int n1 = 1 << l;
    if (l >= 1) {
      const int h = n1 / 2;
      s->G.sx[l] = std::max(h, 8);
      s->G.sy[l] = std::max(h, 4);
      s->G.soff[l] = off;
      off += 64L * s->G.sx[l] * s->G.sy[l] * s->G.sy[l] * 16 * pl.nkb;
    }
    if (l <= nlev - 2) {
      s->G.fx[l] = std::max(n1, 8);
      s->G.fy[l] = std::max(n1, 4);
      s->G.foff[l] = off;
      off += 64L * s->G.fx[l] * s->G.fy[l] * s->G.fy[l] * 2 * pl.nkb;
    }
  }
  if (fmm_reserve(s->grid, off)) return FMM_ERR_CUDA;
  // cells outside a level (small levels padded to the box) stay zero
  FMM_CUDA_TRY(cudaMemsetAsync(s->grid.p, 0, sizeof(__half) * off, st));
  memset(&s->maps, 0, sizeof(s->maps));
  for (int l = 0; l < nlev; l++) {
    if (s->G.soff[l] >= 0 &&
        !tcg_encode(&s->maps.split[l], s->grid.p + s->G.soff[l], s->G.sx[l], s->G.sy[l], 16 * pl.nkb))
      return FMM_OK;
    if (s->G.foff[l] >= 0 &&
        !tcg_encode(&s->maps.full[l], s->grid.p + s->G.foff[l], s->G.fx[l], s->G.fy[l], 2 * pl.nkb))
      return FMM_OK;
  }
  FMM_CUDA_TRY(cudaGetLastError());
  s->eligible = 1;
  return FMM_OK;
}

// leading K chunks whose lowest multipole degree is below TCG_SPLIT_DEG (all three products)
int tcg_full_chunks(const TcPlan &pl) {
  const int moff = fmm_nterms(pl.so - 1);
  int n = 0;
  while (n < pl.kch && fmm_decode(moff + TC_CH * n).d < TCG_SPLIT_DEG) n++;
  return n;
}

template <int NOUT> int tcg_launch(const TcgMaps &maps, const TcgParams &P, int smem, int grid, cudaStream_t st) {
  FMM_CUDA_TRY(cudaFuncSetAttribute(k_m2l_tcg<NOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  fmm_note_launch(), k_m2l_tcg<NOUT><<<grid, TCG_THREADS, smem, st>>>(maps, P);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// The level-grid M2L: FMM_OK when it ran, FMM_ERR_STATE when the tree does
// not qualify.  Operator records (t->tc_T) must be current.
int tcg_run(DevTree *t, const TcPlan &pl, const float *M, int mstr, float *L, int lstr, cudaStream_t st) {
  TcgState *s = tcg_state(t);
  if (s->serial != t->build_serial || s->nkb != pl.nkb)
    if (int rc = tcg_prepare(t, pl, st)) return rc;
  if (!s->eligible) return FMM_ERR_STATE;
  const int nc = t->ncells;
  FMM_CUDA_TRY(cudaMemsetAsync(s->levmax.p, 0, sizeof(unsigned) * TCG_MAXLEV, st));
  fmm_note_launch(), k_tcg_levmax<<<fmm_blocks((size_t)nc * 32, 256), 256, 0, st>>>(M, nc, mstr, pl.msize, t->clevel.p,
                                                                                    s->levmax.p);
  const long nel = (long)nc * 64 * pl.nkb;
  fmm_note_launch(), k_tcg_pack<<<fmm_blocks(nel, 256), 256, 0, st>>>(M, nc, mstr, pl.msize, pl.nkb, t->ix.p, t->iy.p,
                                                                      t->iz.p, t->clevel.p, s->levmax.p, s->G,
                                                                      s->grid.p);
  // the root is no tile row: its local expansion starts at zero
  FMM_CUDA_TRY(cudaMemsetAsync(L, 0, sizeof(float) * pl.lsize, st));
  if (fmm_reserve(t->d_tcerr, 4)) return FMM_ERR_CUDA;
  FMM_CUDA_TRY(cudaMemsetAsync(t->d_tcerr.p, 0, 4 * sizeof(uint32_t), st));
  TcgParams P;
  P.order = s->order.p;
  P.tinfo = s->tinfo.p;
  P.ntiles = s->ntiles;
  P.sched_off = s->sched_off.p;
  P.sched_cls = s->sched_cls.p;
  P.mask = s->mask.p;
  P.key4 = t->cls_key4.p;
  P.levmax = s->levmax.p;
  P.T = t->tc_T.p;
  P.L = L;
  P.lstride = lstr;
  P.lsize = pl.lsize;
  P.kch = pl.kch;
  P.nkb = pl.nkb;
  P.nslots = t->tune.nslots >= 2 ? std::min(pl.nslots, t->tune.nslots) : pl.nslots;
  const int smem = 1024 + P.nslots * pl.slot_bytes + (int)sizeof(TcShared);
  P.cls_bytes = pl.cls_bytes;
  P.cls_scale = pl.cls_scale;
  P.slot_bytes = pl.slot_bytes;
  P.nout = pl.nout;
  P.nfull = tcg_full_chunks(pl);
  for (int k = 0; k < TC_MAXCH; k++) P.nch[k] = k < pl.kch ? pl.nch[k] : 0;
  for (int k = 0; k <= TC_MAXCH; k++) P.choff[k] = k <= pl.kch ? pl.choff[k] : pl.cls_scale;
  P.err = t->d_tcerr.p;
  const int grid = std::min(P.ntiles, tc_sm_count());
  int rc;
  if ((rc = fmm_mark_kernel(t, 0, st))) return rc;
  switch (pl.nout) {
    case 16: rc = tcg_launch<16>(s->maps, P, smem, grid, st); break;
    case 32: rc = tcg_launch<32>(s->maps, P, smem, grid, st); break;
    case 48: rc = tcg_launch<48>(s->maps, P, smem, grid, st); break;
    case 64: rc = tcg_launch<64>(s->maps, P, smem, grid, st); break;
    case 96: rc = tcg_launch<96>(s->maps, P, smem, grid, st); break;
    case 128: rc = tcg_launch<128>(s->maps, P, smem, grid, st); break;
    case 176: rc = tcg_launch<176>(s->maps, P, smem, grid, st); break;
    case 224: rc = tcg_launch<224>(s->maps, P, smem, grid, st); break;
    default: return FMM_ERR_ARG;
  }
  if (rc || (rc = fmm_mark_kernel(t, 1, st))) return rc;
  t->tc_ran = 1;
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned + FMM_PINNED_TCERR, t->d_tcerr.p, 4 * sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, st));
  return FMM_OK;
}

}  // namespace

void fmm_tcg_release(DevTree *t) {
  TcgState *s = (TcgState *)t->tcg;
  if (!s) return;
  fmm_release(s->gidx); fmm_release(s->order); fmm_release(s->pos); fmm_release(s->sched_off);
  fmm_release(s->loff); fmm_release(s->toff); fmm_release(s->tinfo); fmm_release(s->sched_cls);
  fmm_release(s->bitmap); fmm_release(s->rank); fmm_release(s->mask); fmm_release(s->levmax);
  fmm_release(s->grid); fmm_release(s->flag); fmm_release(s->part);
  delete s;
  t->tcg = nullptr;
}

bool fmm_m2l_tc_boxes_ok(DevTree *t, cudaStream_t st) {
  TcPlan pl;
  if (!tc_plan(t->order, t->so, pl) || t->nm2l == 0) return false;
  TcgState *s = tcg_state(t);
  if (s->serial != t->build_serial || s->nkb != pl.nkb)
    if (tcg_prepare(t, pl, st) != FMM_OK) return false;
  return s->eligible != 0;
}

bool fmm_m2l_tc_supported(int p, int so) {
  TcPlan pl;
  return tc_plan(p, so, pl);
}

int fmm_m2l_tc_max_slots(int p, int so) {
  TcPlan pl;
  return tc_plan(p, so, pl) ? pl.nslots : 0;
}

// Executed tensor work of one class step of a 128-row tile: MMA instructions
// and flops (each 2 x 128 x 16 x N): 3 products per K chunk in the row-gather
// kernel; in the level-grid kernel (boxes) 3 for the leading chunks, 1 for
// the chunks of degree TCG_SPLIT_DEG and up.
bool fmm_m2l_tc_step_work(int p, int so, bool boxes, long long *mmas, double *flops) {
  TcPlan pl;
  if (!tc_plan(p, so, pl)) return false;
  const int nfull = boxes ? tcg_full_chunks(pl) : pl.kch;
  long long m = 0;
  double n = 0;
  for (int k = 0; k < pl.kch; k++) {
    const int prod = k < nfull ? 3 : 1;
    m += prod;
    n += (double)prod * pl.nch[k];
  }
  *mmas = m;
  *flops = 2.0 * TC_ROWS * TC_CH * n;
  return true;
}

// M2L of the mixed-precision pass on the tensor cores: reads the FP32 scaled
// multipoles M (row stride mstr) and writes every cell's FP32 scaled local
// expansion L (row stride lstr).
// The class-step schedule of the tiles (tiles of TC_ROWS rows in M2L processing
// order): once per build and cell order.  FMM_ERR_RANGE when the classes
// exceed the bitmap's words.
int fmm_tc_schedule(DevTree *t, cudaStream_t st) {
  if (t->sched_serial == t->build_serial && t->sched_version == t->order_version) return FMM_OK;
  const int nc = t->ncells;
  const int ntiles = (nc + TC_ROWS - 1) / TC_ROWS;
  const int nwords = (t->nclasses + 31) / 32;
  if (nwords > TC_SCHED_MAXW) return FMM_ERR_RANGE;
  const size_t nbm = (size_t)ntiles * nwords;
  if (fmm_reserve(t->tc_sched_off, ntiles + 1) || fmm_reserve(t->tc_pos, nc) || fmm_reserve(t->tc_bitmap, nbm) ||
      fmm_reserve(t->tc_rank, nbm) || fmm_reserve(t->tmp, sizeof(int) * (ntiles + 1 + fmm_scan_tmp_elems<int>(ntiles))))
    return FMM_ERR_CUDA;
  int *cnt = (int *)t->tmp.p, *stmp = cnt + ntiles + 1;
  const long n = t->nm2l;
  fmm_note_launch(), k_tc_pos<<<fmm_blocks(nc, 256), 256, 0, st>>>(t->m2l_order.p, nc, t->tc_pos.p);
  const int nparts = 2 * tc_sm_count();
  if (nbm * sizeof(unsigned) <= 160 * 1024 && n >= 64L * nparts) {
    const int sbytes = (int)(nbm * sizeof(unsigned));
    if (fmm_reserve(t->tc_stab, (size_t)nparts * nbm)) return FMM_ERR_CUDA;  // scratch until the table
    if (sbytes > 48 * 1024)
      FMM_CUDA_TRY(cudaFuncSetAttribute(k_tc_bitmap_part, cudaFuncAttributeMaxDynamicSharedMemorySize, sbytes));
    unsigned *part = (unsigned *)t->tc_stab.p;
    fmm_note_launch(), k_tc_bitmap_part<<<nparts, 512, sbytes, st>>>(t->m2l_tgt_raw.p, t->m2l_cls_raw.p, n,
                                                                      t->tc_pos.p, nwords, (int)nbm, part);
    fmm_note_launch(), k_tc_bitmap_or<<<fmm_blocks(nbm, 256), 256, 0, st>>>(part, nparts, (int)nbm,
                                                                            t->tc_bitmap.p);
  } else {
    FMM_CUDA_TRY(cudaMemsetAsync(t->tc_bitmap.p, 0, sizeof(unsigned) * nbm, st));
    fmm_note_launch(), k_tc_bitmap<<<fmm_blocks(n, 256), 256, 0, st>>>(t->m2l_tgt_raw.p, t->m2l_cls_raw.p, n,
                                                                        t->tc_pos.p, nwords, t->tc_bitmap.p);
  }
  fmm_note_launch(), k_tc_rank<<<ntiles, 256, 0, st>>>(t->tc_bitmap.p, nwords, t->tc_rank.p, cnt);
  if (int rc = fmm_scan<int>(cnt, t->tc_sched_off.p, ntiles, t->tc_sched_off.p + ntiles, stmp, st)) return rc;
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned + FMM_PINNED_SCRATCH, t->tc_sched_off.p + ntiles, sizeof(int),
                               cudaMemcpyDeviceToHost, st));
  FMM_CUDA_TRY(cudaStreamSynchronize(st));
  const int nsteps = (int)t->h_pinned[FMM_PINNED_SCRATCH];
  const size_t ntab = (size_t)(nsteps > 0 ? nsteps : 1) * TC_ROWS;
  if (fmm_reserve(t->tc_sched_cls, nsteps > 0 ? nsteps : 1) || fmm_reserve(t->tc_stab, ntab)) return FMM_ERR_CUDA;
  fmm_note_launch(), k_tc_steps<<<ntiles, 128, 0, st>>>(t->tc_bitmap.p, t->tc_rank.p, nwords, t->tc_sched_off.p,
                                                        t->tc_sched_cls.p);
  FMM_CUDA_TRY(cudaMemsetAsync(t->tc_stab.p, 0xff, sizeof(int) * ntab, st));
  fmm_note_launch(), k_tc_scatter<<<fmm_blocks(n, 256), 256, 0, st>>>(
      t->m2l_tgt_raw.p, t->m2l_src_raw.p, t->m2l_cls_raw.p, n, t->tc_pos.p, t->tc_bitmap.p, t->tc_rank.p, nwords,
      t->tc_sched_off.p, t->tc_stab.p);
  FMM_CUDA_TRY(cudaGetLastError());
  t->sched_serial = t->build_serial;
  t->sched_version = t->order_version;
  t->tc_nsteps = nsteps;
  return FMM_OK;
}

int fmm_m2l_tc(DevTree *t, const float *M, int mstr, float *L, int lstr, cudaStream_t st, bool boxes) {
  TcPlan pl;
  if (!tc_plan(t->order, t->so, pl)) return FMM_ERR_ARG;
  const int nc = t->ncells;
  if (t->nm2l == 0) {
    FMM_CUDA_TRY(cudaMemset2DAsync(L, sizeof(float) * lstr, 0, sizeof(float) * pl.lsize, nc, st));
    return FMM_OK;
  }
  // operator records: once per build
  if (t->tc_serial != t->build_serial) {
    const size_t bytes = (size_t)t->nclasses * pl.cls_bytes;
    // the previous build's records stay valid when its classes were the same
    const bool prev = t->tc_serial + 1 == t->build_serial && t->tc_order == t->order && t->tc_so == t->so &&
                      t->tc_T.cap >= bytes;
    if (fmm_reserve(t->tc_T, bytes)) return FMM_ERR_CUDA;
    fmm_note_launch(), k_tc_operators<<<t->nclasses, 256, 0, st>>>(t->cls_D.p, t->cls_key4.p, t->nclasses, pl,
                                                                   t->tc_T.p, prev ? t->d_cls_same.p : nullptr);
    FMM_CUDA_TRY(cudaGetLastError());
    t->tc_serial = t->build_serial;
    t->tc_order = t->order;
    t->tc_so = t->so;
  }
  // complete levels: source rows by tensor-map box loads from level grids
  t->tc_boxes_last = 0;
  if (boxes) {
    const int rc = tcg_run(t, pl, M, mstr, L, lstr, st);
    if (rc != FMM_ERR_STATE) {
      t->tc_boxes_last = rc == FMM_OK;
      return rc;
    }
  }
  // class-step schedule of the tiles: once per build and cell order
  const int ntiles = (nc + TC_ROWS - 1) / TC_ROWS;
  if (int rc = fmm_tc_schedule(t, st)) return rc;
  const size_t nm = (size_t)nc * pl.kpad;
  if (fmm_reserve(t->tc_Mh, nm) || fmm_reserve(t->tc_Ml, nm) || fmm_reserve(t->tc_mexp, nc) ||
      fmm_reserve(t->d_tcerr, 4))
    return FMM_ERR_CUDA;
  fmm_note_launch(), k_tc_split<<<fmm_blocks((size_t)nc * 32, 256), 256, 0, st>>>(
      M, nc, mstr, pl.msize, pl.kpad, (__half *)t->tc_Mh.p, (__half *)t->tc_Ml.p, t->tc_mexp.p);
  FMM_CUDA_TRY(cudaGetLastError());
  FMM_CUDA_TRY(cudaMemsetAsync(t->d_tcerr.p, 0, 4 * sizeof(uint32_t), st));

  TcParams P;
  P.order = t->m2l_order.p;
  P.ncells = nc;
  P.ntiles = ntiles;
  P.sched_off = t->tc_sched_off.p;
  P.sched_cls = t->tc_sched_cls.p;
  P.stab = t->tc_stab.p;
  P.Mh = (const __half *)t->tc_Mh.p;
  P.Ml = (const __half *)t->tc_Ml.p;
  P.mexp = t->tc_mexp.p;
  P.T = t->tc_T.p;
  P.L = L;
  P.lstride = lstr;
  P.lsize = pl.lsize;
  P.kpad = pl.kpad;
  P.kch = pl.kch;
  P.nkb = pl.nkb;
  // pipeline depth: as many row-gather slots as fit, or fewer when tuned so
  P.nslots = t->tune.nslots >= 2 ? std::min(pl.nslots, t->tune.nslots) : pl.nslots;
  const int smem = 1024 + P.nslots * pl.slot_bytes + (int)sizeof(TcShared);
  P.cls_bytes = pl.cls_bytes;
  P.cls_scale = pl.cls_scale;
  P.slot_bytes = pl.slot_bytes;
  P.nout = pl.nout;
  for (int k = 0; k < TC_MAXCH; k++) P.nch[k] = k < pl.kch ? pl.nch[k] : 0;
  for (int k = 0; k <= TC_MAXCH; k++) P.choff[k] = k <= pl.kch ? pl.choff[k] : pl.cls_scale;
  P.err = t->d_tcerr.p;
  const int grid = std::min(P.ntiles, tc_sm_count());
  int rc;
  if ((rc = fmm_mark_kernel(t, 0, st))) return rc;
  switch (pl.nout) {
    case 16: rc = tc_launch<16>(P, smem, grid, st); break;
    case 32: rc = tc_launch<32>(P, smem, grid, st); break;
    case 48: rc = tc_launch<48>(P, smem, grid, st); break;
    case 64: rc = tc_launch<64>(P, smem, grid, st); break;
    case 96: rc = tc_launch<96>(P, smem, grid, st); break;
    case 128: rc = tc_launch<128>(P, smem, grid, st); break;
    case 176: rc = tc_launch<176>(P, smem, grid, st); break;
    case 224: rc = tc_launch<224>(P, smem, grid, st); break;
    default: return FMM_ERR_ARG;
  }
  if (rc || (rc = fmm_mark_kernel(t, 1, st))) return rc;
  t->tc_ran = 1;
  // timeout flags reach the host with the stream (read by fmmgen_tree_times)
  FMM_CUDA_TRY(cudaMemcpyAsync(t->h_pinned + FMM_PINNED_TCERR, t->d_tcerr.p, 4 * sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, st));
  return FMM_OK;
}

// ---------------------------------------------------------------------------
// class-major CUDA-core M2L (generated kernels in m2l_cm_s*.cu) over the same
// class-step schedule: a block per tile, a thread per row, a step gives a warp
// pairs of one class
// ---------------------------------------------------------------------------
namespace {

// Per-pair orders (target-list order) into the schedule's (step, row) slots:
// a warp per target cell, lanes over its pairs.
__global__ void k_cm_otab(const int *off, const int *cls, const unsigned char *ord, int nc, const int *pos,
                          const unsigned *bm, const unsigned *rank, int nwords, const int *sched_off,
                          unsigned char *otab) {
  const int A = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (A >= nc) return;
  const int row = pos[A], tile = row / TC_ROWS;
  const size_t rb = (size_t)tile * nwords;
  const unsigned sb = (unsigned)sched_off[tile];
  for (int k = off[A] + lane; k < off[A + 1]; k += 32) {
    const unsigned c = (unsigned)cls[k];
    const size_t w = rb + (c >> 5);
    const unsigned st = sb + rank[w] + __popc(bm[w] & ((1u << (c & 31)) - 1u));
    otab[(size_t)st * TC_ROWS + row % TC_ROWS] = ord[k];
  }
}

// Per (tile, warp of 32 rows): how many of the tile's steps have a pair in the
// warp's rows, then their list (a block per tile).
__global__ void k_cm_wcount(const int *sched_off, const int *stab, int *cnt) {
  const int tile = blockIdx.x, w = threadIdx.x >> 5;
  int n = 0;
  for (int s = sched_off[tile]; s < sched_off[tile + 1]; s++)
    n += __any_sync(0xffffffffu, stab[(size_t)s * TC_ROWS + threadIdx.x] >= 0) ? 1 : 0;
  if ((threadIdx.x & 31) == 0) cnt[tile * 4 + w] = n;
}
__global__ void k_cm_wlist(const int *sched_off, const int *stab, const int *woff, int *wstep) {
  const int tile = blockIdx.x, w = threadIdx.x >> 5;
  int o = woff[tile * 4 + w];
  for (int s = sched_off[tile]; s < sched_off[tile + 1]; s++)
    if (__any_sync(0xffffffffu, stab[(size_t)s * TC_ROWS + threadIdx.x] >= 0)) {
      if ((threadIdx.x & 31) == 0) wstep[o] = s;
      o++;
    }
}

// Each target list's pair indices by descending per-pair order (orders clamped
// to [qlo, qhi], at most 32 of them), stable within an order: a warp per
// target (row r of the M2L processing order), lane b counting the pairs of
// order qhi - b.  Also the target's sort key: its level, then its number of
// pairs of order >= qhi - 2, descending (warps of targets alike in their
// high-order pairs spend less time on lanes that have none).
__global__ void k_tp_perm(const int *off, const unsigned char *ord, const int *order, const unsigned char *clevel,
                          int nc, int qlo, int qhi, int *perm, unsigned *key, unsigned *val) {
  const int r = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= nc) return;
  const int A = order[r];
  const int k0 = off[A], k1 = off[A + 1], nb = qhi - qlo + 1;
  int cnt = 0;
  for (int k = k0; k < k1; k += 32) {
    const int kk = k + lane;
    const int q = kk < k1 ? min(max((int)ord[kk], qlo), qhi) : -1;
    for (int b = 0; b < nb; b++) {
      const unsigned m = __ballot_sync(0xffffffffu, q == qhi - b);
      if (lane == b) cnt += __popc(m);
    }
  }
  int pos = cnt;  // exclusive prefix over the lanes: the first slot of each order
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, pos, o);
    if (lane >= o) pos += v;
  }
  pos -= cnt;
  const int hi = __shfl_sync(0xffffffffu, pos, min(3, nb));  // pairs of the 3 highest orders
  if (lane == 0) {
    key[r] = ((unsigned)clevel[A] << 24) | (0xffffffu - (unsigned)min(hi, 0xffffff));
    val[r] = (unsigned)A;
  }
  for (int k = k0; k < k1; k += 32) {
    const int kk = k + lane;
    const int q = kk < k1 ? min(max((int)ord[kk], qlo), qhi) : -1;
    const unsigned same = __match_any_sync(0xffffffffu, q);
    const int first = __shfl_sync(0xffffffffu, pos, q >= 0 ? qhi - q : 0);
    if (q >= 0) perm[k0 + first + __popc(same & ((1u << lane) - 1u))] = kk;
    for (int b = 0; b < nb; b++) {
      const unsigned m = __ballot_sync(0xffffffffu, q == qhi - b);
      if (lane == b) pos += __popc(m);
    }
  }
}

}  // namespace

#include "m2l_cm.cuh"

bool fmm_m2l_cm_supported(int p, int so) { return p >= so + 1 && p <= fmm_m2l_cm_pmax(so); }

int fmm_m2l_cm(DevTree *t, const float *M, int mstr, float *L, int lstr, const unsigned char *ord, cudaStream_t st) {
  static_assert(TC_ROWS == 128, "the generated kernels take tiles of 128 rows");
  const int p = t->order, so = t->so, nc = t->ncells;
  if (!fmm_m2l_cm_supported(p, so) || (mstr & 3) || t->nclasses > TC_SCHED_MAXW * 32) return FMM_ERR_STATE;
  const int lsize = fmm_nterms(p - so);
  if (t->nm2l == 0) {
    FMM_CUDA_TRY(cudaMemset2DAsync(L, sizeof(float) * lstr, 0, sizeof(float) * lsize, nc, st));
    return FMM_OK;
  }
  if (int rc = fmm_tc_schedule(t, st)) return rc == FMM_ERR_RANGE ? FMM_ERR_STATE : rc;
  const int ntiles = (nc + TC_ROWS - 1) / TC_ROWS;
  if (t->cm_wserial != t->sched_serial || t->cm_wversion != t->sched_version) {
    const int nw = 4 * ntiles;
    if (fmm_reserve(t->cm_woff, (size_t)nw + 1) ||
        fmm_reserve(t->cm_wstep, (size_t)4 * (t->tc_nsteps > 0 ? t->tc_nsteps : 1)) ||
        fmm_reserve(t->tmp, sizeof(int) * (nw + fmm_scan_tmp_elems<int>(nw))))
      return FMM_ERR_CUDA;
    int *cnt = (int *)t->tmp.p, *stmp = cnt + nw;
    fmm_note_launch(), k_cm_wcount<<<ntiles, TC_ROWS, 0, st>>>(t->tc_sched_off.p, t->tc_stab.p, cnt);
    if (int rc = fmm_scan<int>(cnt, t->cm_woff.p, nw, t->cm_woff.p + nw, stmp, st)) return rc;
    fmm_note_launch(), k_cm_wlist<<<ntiles, TC_ROWS, 0, st>>>(t->tc_sched_off.p, t->tc_stab.p, t->cm_woff.p,
                                                              t->cm_wstep.p);
    FMM_CUDA_TRY(cudaGetLastError());
    t->cm_wserial = t->sched_serial;
    t->cm_wversion = t->sched_version;
  }
  if (ord) {
    if (int rc = fmm_m2l_csr(t, st)) return rc;
    if (fmm_reserve(t->cm_otab, (size_t)(t->tc_nsteps > 0 ? t->tc_nsteps : 1) * TC_ROWS)) return FMM_ERR_CUDA;
    fmm_note_launch(), k_cm_otab<<<fmm_blocks((size_t)nc * 32, 256), 256, 0, st>>>(
        t->m2l_off.p, t->m2l_cls.p, ord, nc, t->tc_pos.p, t->tc_bitmap.p, t->tc_rank.p, (t->nclasses + 31) / 32,
        t->tc_sched_off.p, t->cm_otab.p);
    FMM_CUDA_TRY(cudaGetLastError());
  }
  CmParams P;
  P.woff = t->cm_woff.p;
  P.wstep = t->cm_wstep.p;
  P.sched_cls = t->tc_sched_cls.p;
  P.stab = t->tc_stab.p;
  P.otab = ord ? t->cm_otab.p : nullptr;
  P.order = t->m2l_order.p;
  P.ncells = nc;
  P.p = p;
  P.D = (const float *)t->cls_Df.p;
  P.dstr = fmm_stride4(fmm_nterms(p));
  P.clevel = t->clevel.p;
  P.M = M;
  P.mstr = mstr;
  P.L = L;
  P.lstr = lstr;
  P.lsize = lsize;
  int rc = fmm_mark_kernel(t, 0, st);
  if (!rc) rc = fmm_m2l_cm_launch(so, P, st);
  return rc ? rc : fmm_mark_kernel(t, 1, st);
}

int fmm_m2l_tp(DevTree *t, const float *M, int mstr, float *L, int lstr, const unsigned char *ord, cudaStream_t st) {
  const int p = t->order, so = t->so, nc = t->ncells;
  if (!fmm_m2l_cm_supported(p, so) || (mstr & 3) || p - so > 32) return FMM_ERR_STATE;
  const int lsize = fmm_nterms(p - so);
  if (t->nm2l == 0) {
    FMM_CUDA_TRY(cudaMemset2DAsync(L, sizeof(float) * lstr, 0, sizeof(float) * lsize, nc, st));
    return FMM_OK;
  }
  if (int rc = fmm_m2l_csr(t, st)) return rc;
  if (ord) {
    const size_t nbh = fmm_rs_nblocks(nc), hist_n = 256 * nbh;
    if (fmm_reserve(t->tp_perm, (size_t)t->nm2l) || fmm_reserve(t->tp_tgt, nc) ||
        fmm_reserve(t->tmp, (size_t)nc * 12 + hist_n * 4 + fmm_scan_tmp_elems<uint32_t>(hist_n) * 4 + 256))
      return FMM_ERR_CUDA;
    char *q = t->tmp.p;
    unsigned *k1 = (unsigned *)q; q += (size_t)nc * 4;
    unsigned *k2 = (unsigned *)q; q += (size_t)nc * 4;
    uint32_t *v2 = (uint32_t *)q; q += (size_t)nc * 4;
    uint32_t *hist = (uint32_t *)q; q += hist_n * 4;
    uint32_t *stmp = (uint32_t *)q;
    fmm_note_launch(), k_tp_perm<<<fmm_blocks((size_t)nc * 32, 256), 256, 0, st>>>(
        t->m2l_off.p, ord, t->m2l_order.p, t->clevel.p, nc, so + 1, p, t->tp_perm.p, k1, (unsigned *)t->tp_tgt.p);
    FMM_CUDA_TRY(cudaGetLastError());
    if (int rc = fmm_radix_sort<unsigned>(k1, (uint32_t *)t->tp_tgt.p, k2, v2, nc, 0, 32, hist, stmp, st)) return rc;
  }
  TpParams P;
  P.tgt = ord ? t->tp_tgt.p : t->m2l_order.p;
  P.ntgt = nc;
  P.off = t->m2l_off.p;
  P.src = t->m2l_src.p;
  P.cls = t->m2l_cls.p;
  P.perm = ord ? t->tp_perm.p : nullptr;
  P.ord = ord;
  P.p = p;
  P.D = (const float *)t->cls_Df.p;
  P.dstr = fmm_stride4(fmm_nterms(p));
  P.clevel = t->clevel.p;
  P.M = M;
  P.mstr = mstr;
  P.L = L;
  P.lstr = lstr;
  P.lsize = lsize;
  int rc = fmm_mark_kernel(t, 0, st);
  if (!rc) rc = fmm_m2l_tp_launch(so, P, st);
  return rc ? rc : fmm_mark_kernel(t, 1, st);
}
