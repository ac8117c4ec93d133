// internal.h -- the device octree handle and the host-side entry points that
// tree.cu / eval.cu / plans.cu export to capi.cu.
#pragma once
#include <vector>
#include "common.cuh"

// Root cube of build_tree (example/tree.cpp:139-187): mean-centred, half-width
// 1.001 * max |x - mean|.
struct RootBox {
  double cx, cy, cz, r;
};

// Task plan of the warp contraction engine (see plans.cu): one warp applies
//   out[n] (+)= scale(n) * sum_t A[a_t] * B[b_t]
// with the tasks of each output split into per-lane segments.
struct Plan {
  const uint32_t *task = nullptr;  // [iters][32]: a(10) | b(10)<<10 | slot(11)<<20 | end(1)<<31; 0xffffffff = pad
  const int *out_seg = nullptr;    // [nout+1] segment range of each output (segments of one output are consecutive)
  int iters = 0, nout = 0, nseg = 0;
};
struct PlanSet {
  int order = -1, so = -1;
  Plan m2l, m2m, l2l;
  void *dmem = nullptr;  // one allocation holding every table
};
const PlanSet *fmm_get_plans(int order, int so);  // cached per device

struct DevTree {
  // configuration
  long N = 0, ncrit = 0;
  int nsys = 1;                           // independent systems (a forest when > 1)
  std::vector<long> sys_off_h;            // particle offsets of the systems in the caller's order, nsys + 1
  DevBuf<long> sys_off;                   // the same on the device
  DevBuf<int> psys;                       // system of each particle in the caller's order (forests)
  DevBuf<double> roots;                   // per system: root cube (cx, cy, cz, r)
  int order = 0, so = 0;
  double theta = 0;
  int dev = 0;
  RootBox root;
  // levels: cells of level l are [level_off[l], level_off[l+1])
  int nlevels = 0;
  std::vector<int> level_off;
  int ncells = 0, nleaves = 0;
  long nm2l = 0, np2p = 0;
  long long p2p_interactions = 0;  // sum over P2P pairs of n_A n_B, minus self terms (fmm_p2p_interactions)
  DevBuf<unsigned long long> d_p2pcount;  // ... on the device, until read
  uint64_t p2p_count_serial = ~0ull;      // build whose count d_p2pcount holds, not yet read
  int nclasses = 0;
  uint32_t eflags = 0;

  // particles in sorted (leaf-contiguous) order
  DevBuf<uint64_t> keys, keys2;
  DevBuf<uint32_t> perm, perm2;           // sorted position -> caller's particle index
  DevBuf<double> px, py, pz;              // sorted positions (FP64)
  DevBuf<float4> phi4, plo4, sdip;        // FP32 P2P staging: (hi offset from root centre, q), (lo, index), dipole
  DevBuf<float2> levf;                    // per-level half-width as an FP32 (hi, lo) pair
  // cells, level-major, Morton order within a level
  DevBuf<double> cx, cy, cz;
  DevBuf<uint64_t> cid;                   // (1 << 3*level) | octant path
  DevBuf<int> ix, iy, iz;                 // integer cell coordinates at the cell's level
  DevBuf<double> cr, crmax;               // half-width and rmax = sqrt(3 r r) (the reference's FP64 values)
  DevBuf<float2> crf;                     // half-width as an FP32 (hi, lo) pair
  DevBuf<float> cmargin;                  // walk: relative MAC band decided in FP64 for pairs this cell refines
  DevBuf<int> csys;                       // system of the cell (forests of independent systems)
  DevBuf<int> pstart, pcount, parent, child_first;
  DevBuf<unsigned char> child_mask, clevel;
  DevBuf<int> leaf_cells;                 // leaf cell indices
  DevBuf<int> cell_leaf;                  // cell -> leaf ordinal or -1
  // interaction lists, grouped by target cell (CSR over cells)
  DevBuf<int> m2l_off, m2l_src, m2l_cls;  // per target: sorted by class (built on demand: fmm_m2l_csr)
  DevBuf<int> m2l_cls_raw;                // class of each walk-order M2L pair
  uint64_t csr_serial = ~0ull;            // build whose target lists m2l_off/src/cls hold
  DevBuf<int> m2l_order;                  // cells in M2L processing order (level, then the grouping below)
  // M2L choices (set by fmmgen_tree_set_tune / the autotuner; -1 / 0: the default rules)
  struct M2LTune {
    int impl = -1;      // mixed pass: 0 tensor cores, 1 generated CUDA-core kernels, 2 contraction engine
    int nslots = 0;     // tensor-core pipeline depth (row-gather slots), 0: as many as fit
    int grouping = 0;   // cell order within a level: 0 by octant within the parent, 1 Morton
    int overlap = 0;    // tensor-core M2L on a high-priority side stream, P2P beside it on the SMs' spare
                        // room in blocks of 4 (1) or 2 (2) warps
  } tune;
  cudaStream_t s_hi = nullptr;            // the side stream (highest priority)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaStream_t s_near = nullptr;          // build_evaluate: P2M, M2M and P2P beside the class build
  cudaEvent_t ev_m = nullptr, ev_c = nullptr, ev_p = nullptr, ev_s = nullptr, ev_l = nullptr;
  int grouping_built = 0;                 // grouping m2l_order holds
  DevBuf<int> p2p_off, p2p_src;
  // M2L translation classes: operator vectors D^(k)(d/s_target), |k| <= order
  DevBuf<int> cls_key4;                   // [nclasses][4]: dlev, dx, dy, dz
  DevBuf<double> cls_D;                   // [nclasses][Nterms(order)]
  DevBuf<float> cls_Df;
  DevBuf<uint64_t> cls_hkeys;             // open-addressing table of class keys
  DevBuf<int> cls_table;                  // class id of each table slot
  DevBuf<uint64_t> cls_prev;              // sorted class keys of the previous build
  int ncls_prev = -1, order_prev = -1;
  DevBuf<uint32_t> d_cls_same;            // nonzero: this build's classes equal the previous build's
  // expansions (scaled: M~_n = M_n / s^|n|, L^_n = s^(|n|+1) L_n)
  DevBuf<double> M, L;
  DevBuf<float> Mf, Lf;
  DevBuf<double> Fnear, Ffar;             // [N][4] sorted order
  // scratch
  DevBuf<int> fa, fb, fa2, fb2;           // traversal frontiers
  DevBuf<int> m2l_tgt_raw, m2l_src_raw;   // walk output in frontier order (kept between builds)
  DevBuf<int> p2p_tgt_raw, p2p_src_raw;
  uint32_t *h_pinned = nullptr;           // 64 pinned host bytes for count readbacks
#define FMM_PINNED_SCRATCH 8              // h_pinned word 8: the tensor-core schedule's step count
#define FMM_PINNED_TCERR 12               // h_pinned words 12..15: last tensor-core M2L error flags, class steps
  // tensor-core M2L operands (m2l_tc.cu)
  DevBuf<unsigned char> tc_T;             // split, swizzled operator records per class
  DevBuf<uint16_t> tc_Mh, tc_Ml;          // scaled, split source multipoles (FP16 bits)
  DevBuf<int> tc_mexp;                    // per cell: scale exponent of its multipole row
  DevBuf<uint32_t> d_tcerr;               // kernel timeout flags
  uint64_t build_serial = 0, tc_serial = ~0ull;  // tc_T belongs to the build with this serial
  DevBuf<int> tc_sched_off;               // class-step schedule of the tensor-core M2L tiles
  DevBuf<unsigned> tc_sched_cls, tc_bitmap, tc_rank;
  DevBuf<int> tc_stab, tc_pos;            // per class step: each tile row's source (-1: none); row of each cell
  int tc_nsteps = 0;                      // class steps of the schedule
  DevBuf<unsigned char> cm_otab;          // per class step: each tile row's per-pair M2L order
  DevBuf<int> cm_woff, cm_wstep;          // per (tile, warp of 32 rows): its steps with a pair
  uint64_t cm_wserial = ~0ull, cm_wversion = ~0ull;  // ... of this schedule (build, cell order)
  DevBuf<int> tp_perm;                    // per target list: pair indices by descending per-pair order
  DevBuf<int> tp_tgt;                     // targets by level, then by their count of high-order pairs
  void *tcg = nullptr;                    // level-grid tensor-core M2L state (m2l_tc.cu, fmm_tcg_release)
  int tc_boxes_last = 0;                  // the last tensor-core M2L boxed its source rows from level grids
  int tc_ran = 0;                         // the last pass's M2L ran on the tensor cores
  uint64_t sched_serial = ~0ull, sched_version = ~0ull;  // ... of this build and cell order
  uint64_t order_version = 0;             // incremented whenever m2l_order is rewritten
  int tc_order = -1, tc_so = -1;          // ... and to this expansion order and source order
  DevBuf<unsigned char> wdec;             // decision of each frontier pair
  DevBuf<char> tmp;                       // scan / sort / misc scratch
  DevBuf<uint32_t> d_eflags;
  DevBuf<double> d_root;                  // sums / maxima for the root box
  // last evaluate() phase times (ms): P2M, M2M, M2L, P2P, L2L, L2P, finalize, total
  float phase_ms[8] = {0};
  float build_ms[6] = {0};                // root, keys+sort, levels, lists, classes, total
  cudaEvent_t ev[16];
  cudaEvent_t ev_mk[4];                   // around the last pass's M2L kernels (not their preparation), P2P kernel
  float kernel_ms[2] = {-1.f, -1.f};      // ... their device times: M2L, P2P
  bool ev_ready = false;
  // evaluation pass as a CUDA graph (fmmgen_tree_set_graph): replayed while
  // the build, the arrays and the switches are those it was captured with
  bool graph_on = false;
  cudaStream_t gstream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  struct GraphKey {
    const double *S = nullptr;
    double *F = nullptr;
    int potential = -1, field = -1, precision = -1;
    uint64_t serial = 0;
  } gkey;
  long long glaunches = 0;                // kernels in the graph
  // per-pair M2L orders (learn.cu): explicit (fmmgen_tree_set_m2l_orders) or
  // predicted by an order model during each evaluation
  int ord_mode = 0;                       // 0: one order, 1: explicit orders, 2: order model
  DevBuf<unsigned char> m2l_ord;          // order of each M2L pair, list order
  uint64_t ord_serial = 0;                // the build m2l_ord belongs to
  const float *model = nullptr;           // order-model parameters (device, caller-owned)
  float model_delta = 0.f;
  double model_eps = 1e-6;                // error target the model's features are scaled to
  int last_prec = -1;                     // precision of the last evaluation (-1: none)
  bool p2p_first = false;                 // the last pass ran P2P before M2L (phase times swap)
  bool pass_potential = true;             // the pass outputs the potential (the P2P sums it only then)
  DevBuf<float> mnorm, feat;              // per-cell multipole degree norms; per-pair features
  DevBuf<double> tscale, tpart;           // per system: sqrt(sum |E_near|^2 / M2L pairs); partial sums
  DevBuf<int> sys_pairs;                  // per system: M2L pairs
  DevBuf<int> ltgt;                       // target of each M2L pair (labels)
};

// sys_off: nullptr for one system, else nsys + 1 host offsets of the systems'
// particles in pos (a forest: one root cube and tree per system, one pass)
// after_cells(t, arg), when given, runs once the cells exist and before the
// interaction lists are built (its work can run beside the walk)
int fmm_tree_build(DevTree *t, const double *pos, long N, long ncrit, int order, double theta, int so,
                   cudaStream_t st, const long *sys_off = nullptr, int nsys = 1, bool defer_classes = false,
                   int (*after_cells)(DevTree *, void *) = nullptr, void *arg = nullptr);
int fmm_tree_finish_build(DevTree *t, cudaStream_t st);
// build and evaluate in one call, the classes built while P2M, M2M and P2P run
int fmm_tree_build_evaluate(DevTree *t, const double *pos, long N, long ncrit, int order, double theta, int so,
                            const long *sys_off, int nsys, const double *S, double *F, int potential, int field,
                            int precision, cudaStream_t st);
int fmm_tree_evaluate(DevTree *t, const double *S, double *F, int potential, int field, int precision,
                      cudaStream_t st);
int fmm_tree_evaluate_bh(DevTree *t, const double *S, double *F, int potential, int field, cudaStream_t st);
void fmm_tree_destroy(DevTree *t);
void fmm_graph_release(DevTree *t);
bool fmm_m2l_tc_supported(int p, int so);
int fmm_m2l_tc_max_slots(int p, int so);       // 0 when the tensor-core M2L does not support (p, so)
bool fmm_m2l_gen_supported(int p, int so);     // generated CUDA-core M2L kernels exist
int fmm_m2l_cell_order(DevTree *t, int grouping, cudaStream_t st);
// the M2L pairs grouped by target and sorted by class within a target (CSR
// m2l_off / m2l_src / m2l_cls), once per build, for the kernels that read them
int fmm_m2l_csr(DevTree *t, cudaStream_t st);
long long fmm_p2p_interactions(DevTree *t);  // reads the build's count (synchronous)
int fmm_m2l_p2p_only(DevTree *t, const double *S, int precision, cudaStream_t st);  // M2L + P2P alone (after a pass)
int fmm_autotune(DevTree *t, const double *S, int precision, int reps, int max_cand, int *cand4, float *cand_ms,
                 int *ncand, cudaStream_t st);
// learned per-pair orders (learn.cu)
int fmm_mlp_nparam();
int fmm_order_features(DevTree *t, double eps, float *feat, cudaStream_t st);
int fmm_order_labels(DevTree *t, double eps, unsigned char *label, float *errq, cudaStream_t st);
int fmm_mlp_predict(const float *params, const float *X, long n, float delta, int qmax, unsigned char *orders,
                    cudaStream_t st);
int fmm_mlp_train_step(const float *params, const float *X, const unsigned char *y, int n, float *grad, float *loss,
                       float *work, cudaStream_t st);
int fmm_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr, cudaStream_t st);
int fmm_learned_orders(DevTree *t, cudaStream_t st);
bool fmm_m2l_tc_step_work(int p, int so, bool boxes, long long *mmas, double *flops);
// boxes: source rows by tensor-map box loads from level grids where every level is complete
int fmm_m2l_tc(DevTree *t, const float *M, int mstr, float *L, int lstr, cudaStream_t st, bool boxes);
void fmm_tcg_release(DevTree *t);
// marks the start (which 0) / end (1) of the pass's M2L kernels, the start (2) / end (3) of its
// P2P kernel, on their streams
int fmm_mark_kernel(DevTree *t, int which, cudaStream_t st);
// the tiles' class-step schedule (tc_sched_off / tc_sched_cls / tc_stab), once per build and cell order
int fmm_tc_schedule(DevTree *t, cudaStream_t st);
// class-major generated CUDA-core M2L over that schedule (m2l_cm_s*.cu); ord: per-pair orders in target-list
// order or null; FMM_ERR_STATE when no family covers (order, source order) or the schedule cannot be built
int fmm_m2l_cm(DevTree *t, const float *M, int mstr, float *L, int lstr, const unsigned char *ord, cudaStream_t st);
// the same kernel bodies, one thread per target cell over its target list (m2l_cm_s*.cu)
int fmm_m2l_tp(DevTree *t, const float *M, int mstr, float *L, int lstr, const unsigned char *ord, cudaStream_t st);
bool fmm_m2l_cm_supported(int p, int so);
bool fmm_m2l_tc_boxes_ok(DevTree *t, cudaStream_t st);  // the level-grid path can run on this build
// M2M of the parents / L2L into the children of cells [lo, hi), FP32 scaled expansions (shift.cu)
int fmm_m2m_tab(DevTree *t, int lo, int hi, float *M, int mstr, cudaStream_t st);
int fmm_l2l_tab(DevTree *t, int lo, int hi, float *L, int lstr, cudaStream_t st);
int fmm_direct(const double *pos, const double *S, long N, const long *targets, long ntargets, int so,
               int potential, int field, double *F, cudaStream_t st);
