// prims.cuh -- device-wide exclusive scan and stable LSD radix sort (u32 or u64
// keys, u32 values), written for this library (no CUB/Thrust on the hot path).
#pragma once
#include "common.cuh"

struct U3 { uint32_t x, y, z; };
__host__ __device__ __forceinline__ U3 operator+(U3 a, U3 b) { return U3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ U3 shfl_up(U3 v, int d) {
  return U3{__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
            __shfl_up_sync(0xffffffffu, v.z, d)};
}
__device__ __forceinline__ uint32_t shfl_up(uint32_t v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ uint64_t shfl_up(uint64_t v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ int shfl_up(int v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
template <typename T> __host__ __device__ __forceinline__ T tzero() { return T{}; }

#define SCAN_BS 1024
#define SCAN_IPT 4
#define SCAN_TILE (SCAN_BS * SCAN_IPT)

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix, writes the block total to *total.
template <typename T> __device__ T block_exclusive(T v, T *total) {
  __shared__ T s_w[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T inc = v;
  for (int d = 1; d < 32; d <<= 1) {
    T o = shfl_up(inc, d);
    if (lane >= d) inc = inc + o;
  }
  if (lane == 31) s_w[w] = inc;
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    T x = lane < nw ? s_w[lane] : tzero<T>();
    T xi = x;
    for (int d = 1; d < 32; d <<= 1) {
      T o = shfl_up(xi, d);
      if (lane >= d) xi = xi + o;
    }
    if (lane < nw) s_w[lane] = xi;  // inclusive warp totals
  }
  __syncthreads();
  T wpre = w > 0 ? s_w[w - 1] : tzero<T>();
  *total = s_w[(blockDim.x >> 5) - 1];
  __syncthreads();
  T exc = inc;
  // exclusive = inclusive - v, computed without subtraction for struct types
  T e = shfl_up(inc, 1);
  exc = lane > 0 ? e : tzero<T>();
  return wpre + exc;
}

template <typename T> __global__ void k_scan_reduce(const T *in, size_t n, T *bsum) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_IPT;
  T s = tzero<T>();
#pragma unroll
  for (int i = 0; i < SCAN_IPT; i++)
    if (base + i < n) s = s + in[base + i];
  T tot;
  block_exclusive(s, &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

template <typename T> __global__ void k_scan_down(const T *in, T *out, size_t n, const T *boff, T *total) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_IPT;
  T v[SCAN_IPT];
  T s = tzero<T>();
#pragma unroll
  for (int i = 0; i < SCAN_IPT; i++) {
    v[i] = (base + i < n) ? in[base + i] : tzero<T>();
    s = s + v[i];
  }
  T tot;
  T pre = block_exclusive(s, &tot);
  T run = (boff ? boff[blockIdx.x] : tzero<T>()) + pre;
#pragma unroll
  for (int i = 0; i < SCAN_IPT; i++) {
    if (base + i < n) out[base + i] = run;
    run = run + v[i];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) *total = run;
}

// Exclusive scan of n elements (in may alias out).  *total (device) receives the
// sum when non-null.  tmp must hold fmm_scan_tmp_elems<T>(n) elements.
template <typename T> size_t fmm_scan_tmp_elems(size_t n) {
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb <= 1) return 1;
  return nb + fmm_scan_tmp_elems<T>(nb);
}
template <typename T> int fmm_scan(const T *in, T *out, size_t n, T *total, T *tmp, cudaStream_t st) {
  if (n == 0) {
    if (total) FMM_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(T), st));
    return FMM_OK;
  }
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 1) {
    fmm_note_launch(), k_scan_down<T><<<1, SCAN_BS, 0, st>>>(in, out, n, nullptr, total);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
  }
  T *bsum = tmp;
  fmm_note_launch(), k_scan_reduce<T><<<(unsigned)nb, SCAN_BS, 0, st>>>(in, n, bsum);
  FMM_CUDA_TRY(cudaGetLastError());
  int rc = fmm_scan<T>(bsum, bsum, nb, nullptr, tmp + nb, st);
  if (rc) return rc;
  fmm_note_launch(), k_scan_down<T><<<(unsigned)nb, SCAN_BS, 0, st>>>(in, out, n, bsum, total);
  FMM_CUDA_TRY(cudaGetLastError());
  return FMM_OK;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  Each block owns a tile of RS_TILE
// consecutive elements.  The scatter ranks the tile's elements by digit in
// element order (so equal digits keep their input order: stability across
// passes), reorders the tile in shared memory, and then writes it out in that
// order: consecutive threads write consecutive positions of one digit's run, so
// the stores coalesce instead of landing one per bucket.
// ---------------------------------------------------------------------------
#define RS_BS 256
#define RS_ROUNDS 12
#define RS_TILE (RS_BS * RS_ROUNDS)

template <typename K> __global__ void k_rs_hist(const K *keys, size_t n, int shift, uint32_t *hist, int nb) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; r++) {
    size_t i = base + (size_t)r * RS_BS + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

template <typename K>
__global__ void __launch_bounds__(RS_BS) k_rs_scatter(const K *kin, const uint32_t *vin, K *kout, uint32_t *vout,
                                                      size_t n, int shift, const uint32_t *offs, int nb) {
  __shared__ uint32_t s_run[256];             // per digit: elements of the tile ranked so far
  __shared__ uint32_t s_wh[RS_BS / 32][256];  // per round: each warp's first rank of a digit
  __shared__ uint32_t s_goff[256];            // per digit: global position of the tile's run - its start in the tile
  __shared__ K s_k[RS_TILE];
  __shared__ uint32_t s_v[RS_TILE];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const unsigned lt = (1u << lane) - 1u;
  const size_t base = (size_t)blockIdx.x * RS_TILE;
  s_run[t] = 0;
  K kr[RS_ROUNDS];
  uint32_t vr[RS_ROUNDS], rk[RS_ROUNDS];
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; r++) {
#pragma unroll
    for (int w = 0; w < RS_BS / 32; w++) s_wh[w][t] = 0;
    __syncthreads();
    const size_t i = base + (size_t)r * RS_BS + t;
    const bool valid = i < n;
    K k = 0;
    uint32_t v = 0, d = 256;
    if (valid) { k = kin[i]; v = vin[i]; d = (uint32_t)((k >> shift) & 255u); }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt);
    if (valid && lane == __ffs(peers) - 1) s_wh[warp][d] = __popc(peers);
    __syncthreads();
    const uint32_t run = s_run[t];
    uint32_t acc = 0;
#pragma unroll
    for (int w = 0; w < RS_BS / 32; w++) {
      const uint32_t c = s_wh[w][t];
      s_wh[w][t] = run + acc;
      acc += c;
    }
    s_run[t] = run + acc;
    __syncthreads();
    kr[r] = k;
    vr[r] = v;
    rk[r] = valid ? s_wh[warp][d] + rank : 0u;  // rank among the tile's elements of digit d
    __syncthreads();                             // before the next round clears s_wh
  }
  // start of each digit's run in the reordered tile, and its global offset
  uint32_t tot;
  const uint32_t start = block_exclusive<uint32_t>(s_run[t], &tot);
  s_goff[t] = offs[(size_t)t * nb + blockIdx.x] - start;
  s_wh[0][t] = start;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; r++) {
    if (base + (size_t)r * RS_BS + t < n) {
      const uint32_t d = (uint32_t)((kr[r] >> shift) & 255u);
      const uint32_t lp = s_wh[0][d] + rk[r];
      s_k[lp] = kr[r];
      s_v[lp] = vr[r];
    }
  }
  __syncthreads();
  const int tile_n = (int)min((size_t)RS_TILE, n - base);
  for (int j = t; j < tile_n; j += RS_BS) {
    const K k = s_k[j];
    const uint32_t pos = s_goff[(k >> shift) & 255u] + (uint32_t)j;
    kout[pos] = k;
    vout[pos] = s_v[j];
  }
}

// Sorts (keys, vals) by bits [begin_bit, end_bit) of the key, stably.  Uses
// (keys2, vals2) as ping-pong space; the result always ends in (keys, vals).
// hist must hold 256 * nblocks u32, scantmp fmm_scan_tmp_elems<uint32_t>(256*nblocks).
static inline size_t fmm_rs_nblocks(size_t n) { return (n + RS_TILE - 1) / RS_TILE; }
template <typename K>
static inline int fmm_radix_sort(K *keys, uint32_t *vals, K *keys2, uint32_t *vals2, size_t n,
                                 int begin_bit, int end_bit, uint32_t *hist, uint32_t *scantmp,
                                 cudaStream_t st) {
  if (n <= 1) return FMM_OK;
  int nb = (int)fmm_rs_nblocks(n);
  K *ka = keys, *kb = keys2;
  uint32_t *va = vals, *vb = vals2;
  int passes = 0;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    fmm_note_launch(), k_rs_hist<K><<<nb, RS_BS, 0, st>>>(ka, n, shift, hist, nb);
    FMM_CUDA_TRY(cudaGetLastError());
    int rc = fmm_scan<uint32_t>(hist, hist, (size_t)256 * nb, nullptr, scantmp, st);
    if (rc) return rc;
    fmm_note_launch(), k_rs_scatter<K><<<nb, RS_BS, 0, st>>>(ka, va, kb, vb, n, shift, hist, nb);
    FMM_CUDA_TRY(cudaGetLastError());
    K *tk = ka; ka = kb; kb = tk;
    uint32_t *tv = va; va = vb; vb = tv;
    passes++;
  }
  if (passes & 1) {
    FMM_CUDA_TRY(cudaMemcpyAsync(keys, ka, n * sizeof(K), cudaMemcpyDeviceToDevice, st));
    FMM_CUDA_TRY(cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  }
  return FMM_OK;
}
