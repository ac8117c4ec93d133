// m2l_cm.cuh -- generated by fmmgen_gb300/gen_m2l_cm.py; do not edit.
// FP32 M2L kernels for every order up to a family's largest (m2l_cm_s*.cu):
// parameters and launchers.  Outputs are written, not accumulated.
#pragma once
#include "internal.h"

// class-major schedule: the tiles of the tensor-core class-step schedule
struct CmParams {
  const int *woff;              // [4 ntiles + 1] first entry of each (tile, warp) in wstep
  const int *wstep;             // steps with a pair in the warp's 32 rows, per (tile, warp), increasing
  const unsigned *sched_cls;    // [steps] class of each step
  const int *stab;              // [steps][128] source cell of each row, -1 without a pair
  const unsigned char *otab;    // [steps][128] per-pair order, or null: every pair at order p
  const int *order;             // [ncells] rows -> cells (M2L processing order)
  int ncells, p;
  const float *D;               // [classes][dstr] FP32 class operators
  int dstr;
  const unsigned char *clevel;  // [ncells] level of each cell
  const float *M;               // [ncells][mstr] scaled multipoles (degrees >= source order)
  int mstr;
  float *L;                     // [ncells][lstr] scaled locals
  int lstr, lsize;
};

// target-major schedule: a thread per target cell over its target list
struct TpParams {
  const int *tgt;               // [ntgt] target cells (null: cells 0 .. ntgt - 1)
  int ntgt;
  const int *off, *src, *cls;   // target lists: pairs of cell A are off[A] .. off[A + 1] - 1
  const int *perm;              // pair indices of each list by descending order, or null (list order)
  const unsigned char *ord;     // per-pair orders (list order, needs perm), or null: every pair at order p
  int p;
  const float *D;
  int dstr;
  const unsigned char *clevel;
  const float *M;
  int mstr;
  float *L;
  int lstr, lsize;
};

static __device__ __forceinline__ void cm_cp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(d), "l"(src) : "memory");
}
static __device__ __forceinline__ void cm_cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> static __device__ __forceinline__ void cm_cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" :: "n"(N) : "memory");
}

int fmm_m2l_cm_s0_p6(const CmParams &P, cudaStream_t st);  // orders 1..6
int fmm_m2l_tp_s0_p6(const TpParams &P, cudaStream_t st);
int fmm_m2l_cm_s0_p8(const CmParams &P, cudaStream_t st);  // orders 1..8
int fmm_m2l_tp_s0_p8(const TpParams &P, cudaStream_t st);
int fmm_m2l_cm_s0_p12(const CmParams &P, cudaStream_t st);  // orders 1..12
int fmm_m2l_tp_s0_p12(const TpParams &P, cudaStream_t st);
int fmm_m2l_cm_s1_p6(const CmParams &P, cudaStream_t st);  // orders 2..6
int fmm_m2l_tp_s1_p6(const TpParams &P, cudaStream_t st);
int fmm_m2l_cm_s1_p8(const CmParams &P, cudaStream_t st);  // orders 2..8
int fmm_m2l_tp_s1_p8(const TpParams &P, cudaStream_t st);
// largest order of the families of each source order (0: none)
static inline int fmm_m2l_cm_pmax(int so) {
  if (so == 0) return 12;
  if (so == 1) return 8;
  return 0;
}
// launch the family of source order so with the smallest largest order >= P.p (FMM_ERR_STATE: none)
static inline int fmm_m2l_cm_launch(int so, const CmParams &P, cudaStream_t st) {
  if (so == 0 && P.p <= 6) return fmm_m2l_cm_s0_p6(P, st);
  if (so == 0 && P.p <= 8) return fmm_m2l_cm_s0_p8(P, st);
  if (so == 0 && P.p <= 12) return fmm_m2l_cm_s0_p12(P, st);
  if (so == 1 && P.p <= 6) return fmm_m2l_cm_s1_p6(P, st);
  if (so == 1 && P.p <= 8) return fmm_m2l_cm_s1_p8(P, st);
  return FMM_ERR_STATE;
}
// launch the family of source order so with the smallest largest order >= P.p (FMM_ERR_STATE: none)
static inline int fmm_m2l_tp_launch(int so, const TpParams &P, cudaStream_t st) {
  if (so == 0 && P.p <= 6) return fmm_m2l_tp_s0_p6(P, st);
  if (so == 0 && P.p <= 8) return fmm_m2l_tp_s0_p8(P, st);
  if (so == 0 && P.p <= 12) return fmm_m2l_tp_s0_p12(P, st);
  if (so == 1 && P.p <= 6) return fmm_m2l_tp_s1_p6(P, st);
  if (so == 1 && P.p <= 8) return fmm_m2l_tp_s1_p8(P, st);
  return FMM_ERR_STATE;
}
