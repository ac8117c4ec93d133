// tune.cu -- autotuner of the M2L phase (no counterpart in the reference, whose
// M2L is one OpenMP loop, example/calculate.cpp:190-206).
//
// Candidates, for the tree's order and source order:
//   implementation: tensor cores (p <= 9) with source rows gathered row by row
//                   or (trees whose levels are all complete) boxed from level
//                   grids, generated CUDA-core kernels (orders that have them),
//                   class-major and target-major generated CUDA-core kernels
//                   (every order up to 12), warp contraction engine;
//   tensor-core pipeline depth: 2 .. the row-gather slots that fit in shared memory;
//   tensor cores alone, or overlapped with the P2P (in 4- or 2-warp blocks);
//   grouping of the cells into tiles / warps: by octant within the parent, or Morton.
// One evaluation pass computes the multipoles and stages the particles; then
// the M2L and P2P phases alone are timed `reps` times per candidate with CUDA
// events on the caller's stream and the candidate with the lowest median is
// kept on the handle.
#include <algorithm>
#include <vector>
#include "internal.h"

#define TRY_(x) do { int _rc = (x); if (_rc) return _rc; } while (0)

int fmm_autotune(DevTree *t, const double *S, int precision, int reps, int max_cand, int *cand4, float *cand_ms,
                 int *ncand, cudaStream_t st) {
  if (t->ord_mode != 0) return FMM_ERR_STATE;  // per-pair orders use their own kernel
  if (reps < 1) reps = 1;
  // the candidates
  struct Cand {
    int impl, nslots, grouping, overlap;
  };
  std::vector<Cand> cands;
  const int maxs = fmm_m2l_tc_max_slots(t->order, t->so);
  const bool gen = fmm_m2l_gen_supported(t->order, t->so);
  const bool cm = fmm_m2l_cm_supported(t->order, t->so) && t->nclasses <= 262144;
  const bool tp = fmm_m2l_cm_supported(t->order, t->so);
  const bool boxes = precision != 0 && maxs > 0 && fmm_m2l_tc_boxes_ok(t, st);
  for (int g = 0; g < 2; g++) {
    if (precision != 0) {
      for (int ov = 0; ov < 3; ov++)
        for (int s = 2; s <= maxs; s++) {
          cands.push_back({0, s, g, ov});
          // level-grid boxes (their tiles do not depend on the grouping)
          if (g == 0 && boxes) cands.push_back({3, s, g, ov});
        }
      if (gen) cands.push_back({1, 0, g, 0});
      if (cm) cands.push_back({4, 0, g, 0});
      if (tp) cands.push_back({5, 0, g, 0});
    }
    cands.push_back({2, 0, g, 0});
  }
  // one pass for the multipoles (the field into a scratch output)
  double *F = nullptr;
  FMM_CUDA_TRY(cudaMalloc((void **)&F, sizeof(double) * 3 * (size_t)std::max(t->N, 1L)));
  const DevTree::M2LTune keep = t->tune;
  t->tune = DevTree::M2LTune();
  int rc = fmm_tree_evaluate(t, S, F, 0, 1, precision, st);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = FMM_ERR_CUDA;
  int best = -1;
  float best_ms = 0.f;
  std::vector<float> med(cands.size(), -1.f);
  for (size_t c = 0; c < cands.size() && !rc; c++) {
    t->tune.impl = cands[c].impl;
    t->tune.nslots = cands[c].nslots;
    t->tune.grouping = cands[c].grouping;
    t->tune.overlap = cands[c].overlap;
    rc = fmm_m2l_p2p_only(t, S, precision, st);  // warm-up (and the grouping's cell order)
    std::vector<float> ms;
    for (int r = 0; r < reps && !rc; r++) {
      if (cudaEventRecord(e0, st) != cudaSuccess) { rc = FMM_ERR_CUDA; break; }
      rc = fmm_m2l_p2p_only(t, S, precision, st);
      if (rc) break;
      float x = 0.f;
      if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&x, e0, e1) != cudaSuccess) {
        rc = FMM_ERR_CUDA;
        break;
      }
      ms.push_back(x);
    }
    if (rc) break;
    std::sort(ms.begin(), ms.end());
    med[c] = ms[ms.size() / 2];
    if (best < 0 || med[c] < best_ms) {
      best = (int)c;
      best_ms = med[c];
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(F);
  if (rc || best < 0) {
    t->tune = keep;
    return rc ? rc : FMM_ERR_STATE;
  }
  // M2L and P2P one after the other unless running them side by side gains more than the noise (2 %):
  // the same step time, and each kernel's own device time stays its own
  if (cands[best].overlap)
    for (size_t c = 0; c < cands.size(); c++)
      if (!cands[c].overlap && cands[c].impl == cands[best].impl && cands[c].nslots == cands[best].nslots &&
          cands[c].grouping == cands[best].grouping && med[c] >= 0.f && med[c] <= 1.02f * best_ms)
        best = (int)c;
  t->tune.impl = cands[best].impl;
  t->tune.nslots = cands[best].nslots;
  t->tune.grouping = cands[best].grouping;
  t->tune.overlap = cands[best].overlap;
  fmm_graph_release(t);
  if (t->grouping_built != t->tune.grouping) TRY_(fmm_m2l_cell_order(t, t->tune.grouping, st));
  const int n = (int)cands.size();
  if (ncand) *ncand = n;
  for (int c = 0; c < std::min(n, max_cand); c++) {
    if (cand4) {
      cand4[4 * c] = cands[c].impl;
      cand4[4 * c + 1] = (cands[c].impl == 0 || cands[c].impl == 3) ? cands[c].nslots : 0;
      cand4[4 * c + 2] = cands[c].grouping;
      cand4[4 * c + 3] = cands[c].overlap;
    }
    if (cand_ms) cand_ms[c] = med[c];
  }
  return FMM_OK;
}
