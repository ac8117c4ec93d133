// plans.cu -- task plans of the warp contraction engine.
//
// M2M, M2L and L2L all have the form out[n] = sum_t A[a_t] * B[b_t] over a
// fixed, order-dependent set of (n, a, b) index triples (the sums of
// fmmgen/expansions.py:42-78, 144-172, 175-194).  Their lengths vary strongly
// with |n| (M2L at p=8: 165 terms for n=0, 1 for |n|=8), so giving each lane
// whole outputs leaves most lanes idle.  A plan flattens the triples in output
// order and cuts the list into 32 equal contiguous lane ranges; each lane keeps
// one running sum per (lane, output) segment and writes it to a private slot,
// and the outputs are then summed from their consecutive slots in a fixed
// order (deterministic, no atomics).
#include <algorithm>
#include <array>
#include <cstring>
#include <mutex>
#include <vector>
#include "internal.h"

namespace {

struct HostPlan {
  std::vector<uint32_t> task;
  std::vector<int> out_seg;
  int iters = 0, nout = 0, nseg = 0;
};

// tasks: (out, a, b), sorted by out.
//
// Within a (lane, output) segment the order of the terms is free, so each
// round's terms are chosen to spread the 32 lanes' shared-memory reads of A and
// of B over distinct banks -- the 32 4-byte banks across the warp for FP32
// operands, and the 16 bank pairs within each half-warp for 8-byte ones (FP64,
// or two FP32 operands side by side); lanes that read the same word share it.
// Lanes are filled in turn, those with the fewest terms left first, each
// taking the remaining term of its current segment that collides with the
// fewest reads already placed in the round.
// Shared-memory bank conflicts otherwise multiply the engine's load wavefronts
// several times over.
HostPlan make_plan(const std::vector<std::array<int, 3>> &tasks, int nout) {
  HostPlan P;
  int T = (int)tasks.size();
  P.nout = nout;
  P.iters = (T + 31) / 32;
  P.task.assign((size_t)P.iters * 32, 0xffffffffu);
  P.out_seg.assign(nout + 1, -1);
  struct Seg {
    int id, t0, t1;  // tasks[t0, t1) of one output
  };
  std::vector<std::vector<Seg>> segs(32);
  int seg = 0;
  for (int l = 0; l < 32; l++) {
    int t0 = (int)((long)l * T / 32), t1 = (int)((long)(l + 1) * T / 32);
    for (int t = t0; t < t1;) {
      int out = tasks[t][0], e = t;
      while (e < t1 && tasks[e][0] == out) e++;
      if (P.out_seg[out] < 0) P.out_seg[out] = seg;
      segs[l].push_back({seg++, t, e});
      t = e;
    }
  }
  P.nseg = seg;
  P.out_seg[nout] = seg;
  // every output owns at least one task, so out_seg is fully set
  std::vector<std::vector<char>> used(32);
  std::vector<size_t> cur(32, 0);  // current segment per lane
  std::vector<int> left(32, 0);    // terms of it not yet placed
  for (int l = 0; l < 32; l++) {
    used[l].assign((size_t)((long)(l + 1) * T / 32 - (long)l * T / 32), 0);
    if (!segs[l].empty()) left[l] = segs[l][0].t1 - segs[l][0].t0;
  }
  for (int it = 0; it < P.iters; it++) {
    // 4-byte reads: 32 banks over the warp; 8-byte reads (FP64, paired FP32):
    // 16 bank pairs within each half-warp
    int bankA[32], bankB[32], pairA[2][16], pairB[2][16];
    for (int k = 0; k < 32; k++) bankA[k] = bankB[k] = pairA[k >> 4][k & 15] = pairB[k >> 4][k & 15] = -1;
    // lanes with the fewest terms left to choose from go first
    int ord[32];
    for (int k = 0; k < 32; k++) ord[k] = k;
    std::stable_sort(ord, ord + 32, [&](int x, int y) { return left[x] < left[y]; });
    for (int li = 0; li < 32; li++) {
      const int l = ord[li];
      if (cur[l] >= segs[l].size()) continue;
      const Seg &S = segs[l][cur[l]];
      const int base = (int)((long)l * T / 32);
      const int h = l >> 4;
      int best = -1, bcost = 5;
      for (int t = S.t0; t < S.t1 && bcost > 0; t++) {
        if (used[l][t - base]) continue;
        const int a = tasks[t][1], b = tasks[t][2];
        const int cost = (bankA[a & 31] >= 0 && bankA[a & 31] != a) + (bankB[b & 31] >= 0 && bankB[b & 31] != b) +
                         (pairA[h][a & 15] >= 0 && pairA[h][a & 15] != a) +
                         (pairB[h][b & 15] >= 0 && pairB[h][b & 15] != b);
        if (cost < bcost) { bcost = cost; best = t; }
      }
      used[l][best - base] = 1;
      const int a = tasks[best][1], b = tasks[best][2];
      if (bankA[a & 31] < 0) bankA[a & 31] = a;
      if (bankB[b & 31] < 0) bankB[b & 31] = b;
      if (pairA[h][a & 15] < 0) pairA[h][a & 15] = a;
      if (pairB[h][b & 15] < 0) pairB[h][b & 15] = b;
      const bool end = --left[l] == 0;
      P.task[(size_t)it * 32 + l] =
          (uint32_t)a | ((uint32_t)b << 10) | ((uint32_t)S.id << 20) | ((end ? 1u : 0u) << 31);
      if (end && ++cur[l] < segs[l].size()) left[l] = segs[l][cur[l]].t1 - segs[l][cur[l]].t0;
    }
  }
  return P;
}

HostPlan plan_m2l(int p, int so) {
  std::vector<std::array<int, 3>> tk;
  int off = fmm_nterms(so - 1), nl = fmm_nterms(p - so), nm = fmm_nterms(p);
  for (int i = 0; i < nl; i++) {
    MI n = fmm_decode(i);
    for (int j = off; j < nm; j++) {
      MI m = fmm_decode(j);
      if (n.d + m.d > p) continue;
      tk.push_back({i, fmm_idx3(n.x + m.x, n.y + m.y, n.z + m.z), j - off});
    }
  }
  return make_plan(tk, nl);
}

HostPlan plan_m2m(int p, int so) {
  std::vector<std::array<int, 3>> tk;
  int off = fmm_nterms(so - 1), nm = fmm_nterms(p);
  for (int i = off; i < nm; i++) {
    MI n = fmm_decode(i);
    for (int kx = 0; kx <= n.x; kx++)
      for (int ky = 0; ky <= n.y; ky++)
        for (int kz = 0; kz <= n.z; kz++) {
          if (n.d - kx - ky - kz < so) continue;
          tk.push_back({i - off, fmm_idx3(kx, ky, kz), fmm_idx3(n.x - kx, n.y - ky, n.z - kz) - off});
        }
  }
  return make_plan(tk, nm - off);
}

HostPlan plan_l2l(int p, int so) {
  std::vector<std::array<int, 3>> tk;
  int pl = p - so, nl = fmm_nterms(pl);
  for (int i = 0; i < nl; i++) {
    MI n = fmm_decode(i);
    for (int j = 0; j < fmm_nterms(pl - n.d); j++) {
      MI k = fmm_decode(j);
      tk.push_back({i, j, fmm_idx3(n.x + k.x, n.y + k.y, n.z + k.z)});
    }
  }
  return make_plan(tk, nl);
}

std::mutex g_mu;
PlanSet *g_plans[16][FMM_PMAX + 1][3] = {};

}  // namespace

const PlanSet *fmm_get_plans(int order, int so) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return nullptr;
  if (order < 0 || order > FMM_PMAX || so < 0 || so > 2) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_plans[dev][order][so]) return g_plans[dev][order][so];
  HostPlan hp[3] = {plan_m2l(order, so), plan_m2m(order, so), plan_l2l(order, so)};
  size_t bytes = 0;
  // each of the two arrays of a plan is padded up to a 256-byte boundary
  for (auto &h : hp) bytes += h.task.size() * 4 + h.out_seg.size() * 4 + 2 * 256;
  char *d = nullptr;
  if (cudaMalloc((void **)&d, bytes) != cudaSuccess) return nullptr;
  std::vector<char> host(bytes, 0);
  PlanSet *ps = new PlanSet();
  ps->order = order;
  ps->so = so;
  ps->dmem = d;
  size_t o = 0;
  Plan *dst[3] = {&ps->m2l, &ps->m2m, &ps->l2l};
  for (int k = 0; k < 3; k++) {
    memcpy(host.data() + o, hp[k].task.data(), hp[k].task.size() * 4);
    dst[k]->task = (const uint32_t *)(d + o);
    o += hp[k].task.size() * 4;
    o = (o + 255) & ~(size_t)255;
    memcpy(host.data() + o, hp[k].out_seg.data(), hp[k].out_seg.size() * 4);
    dst[k]->out_seg = (const int *)(d + o);
    o += hp[k].out_seg.size() * 4;
    o = (o + 255) & ~(size_t)255;
    dst[k]->iters = hp[k].iters;
    dst[k]->nout = hp[k].nout;
    dst[k]->nseg = hp[k].nseg;
  }
  if (cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    delete ps;
    return nullptr;
  }
  g_plans[dev][order][so] = ps;
  return ps;
}
