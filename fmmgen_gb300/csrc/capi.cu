// capi.cu -- the extern "C" boundary declared in include/fmmgen_gb300.h.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "../../include/fmmgen_gb300.h"
#include "internal.h"
#include "mi_table.cuh"

struct fmmgen_tree {
  DevTree t;
  bool built = false;
  int last_precision = -1;
};

int fmm_op_batch(int op, int n, const double *d, const double *in, double *out, int order, int so, int potential,
                 int field, cudaStream_t st);
int fmm_op_batch_f32(int op, int n, const float *d, const float *in, float *out, int order, int so, int potential,
                     int field, cudaStream_t st);
void fmm_eval_times(DevTree *t);

namespace {
thread_local std::string g_err;
inline cudaStream_t S(void *s) { return (cudaStream_t)s; }
int ret(int rc) {
  if (rc == FMM_OK) return rc;
  if (g_err.empty()) {
    switch (rc) {
      case FMM_ERR_ARG: g_err = "invalid argument"; break;
      case FMM_ERR_DEPTH: g_err = "octree deeper than 21 levels (>= ncrit coincident particles)"; break;
      case FMM_ERR_RANGE: g_err = "M2L offset range too wide"; break;
      case FMM_ERR_STATE: g_err = "tree handle not built"; break;
      default: g_err = "CUDA error"; break;
    }
  }
  return rc;
}
}  // namespace

void fmm_set_cuda_error(cudaError_t e, const char *what, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
  g_err = buf;
}
void fmm_set_error_text(const char *msg) { g_err = msg; }

static std::atomic<long long> g_launches{0};
void fmm_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long fmm_launches() { return g_launches.load(std::memory_order_relaxed); }
void fmm_add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" {

long long fmmgen_launch_count(void) { return g_launches.load(); }
const char *fmmgen_last_error(void) { return g_err.c_str(); }
const char *fmmgen_version(void) { return "fmmgen_gb300 0.1 (sm_103a)"; }
int fmmgen_max_order(void) { return FMM_PMAX; }

long fmmgen_nterms(int p) { return fmm_nterms(p); }
long fmmgen_msize(int order, int so) { return fmm_nterms(order) - fmm_nterms(so - 1); }
long fmmgen_lsize(int order, int so) { return fmm_nterms(order - so); }
int fmmgen_minorder(int so, int field) { return so + (field ? 1 : 0); }
int fmmgen_sourcesize(int so) { return fmm_nterms(so) - fmm_nterms(so - 1); }
int fmmgen_outputsize(int potential, int field) { return (potential ? 1 : 0) + (field ? 3 : 0); }

#define OPB(opid, n, d, in, out, order, so, pot, fld, st)                                           \
  do {                                                                                              \
    g_err.clear();                                                                                  \
    return ret(fmm_op_batch(opid, n, d, in, out, order, so, pot, fld, S(st)));                     \
  } while (0)
#define OPBF(opid, n, d, in, out, order, so, pot, fld, st)                                          \
  do {                                                                                              \
    g_err.clear();                                                                                  \
    return ret(fmm_op_batch_f32(opid, n, d, in, out, order, so, pot, fld, S(st)));                 \
  } while (0)

int fmmgen_gpu_P2M(int n, const double *d, const double *q, double *M, int order, int so, void *st) {
  OPB(0, n, d, q, M, order, so, 1, 1, st);
}
int fmmgen_gpu_M2M(int n, const double *d, const double *M, double *Ms, int order, int so, void *st) {
  OPB(1, n, d, M, Ms, order, so, 1, 1, st);
}
int fmmgen_gpu_M2L(int n, const double *d, const double *M, double *L, int order, int so, void *st) {
  OPB(2, n, d, M, L, order, so, 1, 1, st);
}
int fmmgen_gpu_L2L(int n, const double *d, const double *L, double *Ls, int order, int so, void *st) {
  OPB(3, n, d, L, Ls, order, so, 1, 1, st);
}
int fmmgen_gpu_L2P(int n, const double *d, const double *L, double *F, int order, int so, int potential, int field,
                   void *st) {
  OPB(4, n, d, L, F, order, so, potential, field, st);
}
int fmmgen_gpu_P2P(int n, const double *d, const double *Sv, double *F, int so, int potential, int field, void *st) {
  OPB(5, n, d, Sv, F, 0, so, potential, field, st);
}
int fmmgen_gpu_M2P(int n, const double *d, const double *M, double *F, int order, int so, int potential, int field,
                   void *st) {
  OPB(6, n, d, M, F, order, so, potential, field, st);
}

int fmmgen_gpu_P2M_f32(int n, const float *d, const float *q, float *M, int order, int so, void *st) {
  OPBF(0, n, d, q, M, order, so, 1, 1, st);
}
int fmmgen_gpu_M2M_f32(int n, const float *d, const float *M, float *Ms, int order, int so, void *st) {
  OPBF(1, n, d, M, Ms, order, so, 1, 1, st);
}
int fmmgen_gpu_M2L_f32(int n, const float *d, const float *M, float *L, int order, int so, void *st) {
  OPBF(2, n, d, M, L, order, so, 1, 1, st);
}
int fmmgen_gpu_L2L_f32(int n, const float *d, const float *L, float *Ls, int order, int so, void *st) {
  OPBF(3, n, d, L, Ls, order, so, 1, 1, st);
}
int fmmgen_gpu_L2P_f32(int n, const float *d, const float *L, float *F, int order, int so, int potential, int field,
                       void *st) {
  OPBF(4, n, d, L, F, order, so, potential, field, st);
}
int fmmgen_gpu_P2P_f32(int n, const float *d, const float *Sv, float *F, int so, int potential, int field, void *st) {
  OPBF(5, n, d, Sv, F, 0, so, potential, field, st);
}
int fmmgen_gpu_M2P_f32(int n, const float *d, const float *M, float *F, int order, int so, int potential, int field,
                       void *st) {
  OPBF(6, n, d, M, F, order, so, potential, field, st);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// scalar twins
// ---------------------------------------------------------------------------
namespace {
template <typename T> int d2h(std::vector<T> &v, const T *p, size_t n) {
  v.resize(n);
  if (n) FMM_CUDA_TRY(cudaMemcpy(v.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost));
  return FMM_OK;
}
struct ScalarCfg {
  int so = 0, potential = 1, field = 1, maxorder = FMM_PMAX;
  std::mutex mu;
  cudaStream_t st = nullptr;
  double *dbuf = nullptr;  // [3 + NTMAX + NTMAX]
};
ScalarCfg g_cfg;

// runs one operator on host arrays through the device path (T = double, or
// float for the precision="float" twins)
template <typename T>
void scalar_op(int op, T x, T y, T z, const T *in, int insize, T *out, int outsize, int order) {
  std::lock_guard<std::mutex> lk(g_cfg.mu);
  if (!g_cfg.st && cudaStreamCreateWithFlags(&g_cfg.st, cudaStreamNonBlocking) != cudaSuccess) return;
  if (!g_cfg.dbuf && cudaMalloc((void **)&g_cfg.dbuf, sizeof(double) * (4 + 2 * FMM_NTMAX)) != cudaSuccess) return;
  T *d = (T *)g_cfg.dbuf, *din = d + 4, *dout = din + FMM_NTMAX;
  T h[3] = {x, y, z};
  cudaMemcpyAsync(d, h, sizeof(h), cudaMemcpyHostToDevice, g_cfg.st);
  cudaMemcpyAsync(din, in, sizeof(T) * insize, cudaMemcpyHostToDevice, g_cfg.st);
  cudaMemcpyAsync(dout, out, sizeof(T) * outsize, cudaMemcpyHostToDevice, g_cfg.st);
  int rc;
  if constexpr (sizeof(T) == 8)
    rc = fmm_op_batch(op, 1, d, din, dout, order, g_cfg.so, g_cfg.potential, g_cfg.field, g_cfg.st);
  else
    rc = fmm_op_batch_f32(op, 1, d, din, dout, order, g_cfg.so, g_cfg.potential, g_cfg.field, g_cfg.st);
  if (rc != FMM_OK) return;
  cudaMemcpyAsync(out, dout, sizeof(T) * outsize, cudaMemcpyDeviceToHost, g_cfg.st);
  cudaStreamSynchronize(g_cfg.st);
}
bool order_ok(int order) {
  return order >= g_cfg.so + (g_cfg.field ? 1 : 0) && order <= g_cfg.maxorder && order <= FMM_PMAX;
}
bool fixed_order_ok(int order) { return order >= g_cfg.so + (g_cfg.field ? 1 : 0) && order <= FMM_PMAX; }
}  // namespace

extern "C" {

int fmmgen_configure(int so, int potential, int field, int maxorder) {
  if (so < 0 || so > 2 || (!potential && !field) || maxorder < so || maxorder > FMM_PMAX) return ret(FMM_ERR_ARG);
  std::lock_guard<std::mutex> lk(g_cfg.mu);
  g_cfg.so = so; g_cfg.potential = potential; g_cfg.field = field; g_cfg.maxorder = maxorder;
  return FMM_OK;
}
void P2M(double x, double y, double z, double q, double *M, int order) {
  if (!order_ok(order)) return;
  scalar_op<double>(0, x, y, z, &q, 1, M, (int)fmmgen_msize(order, g_cfg.so), order);
}
void M2M(double x, double y, double z, double *M, double *Ms, int order) {
  if (!order_ok(order)) return;
  int ms = (int)fmmgen_msize(order, g_cfg.so);
  scalar_op<double>(1, x, y, z, M, ms, Ms, ms, order);
}
void M2L(double x, double y, double z, double *M, double *L, int order) {
  if (!order_ok(order)) return;
  scalar_op<double>(2, x, y, z, M, (int)fmmgen_msize(order, g_cfg.so), L, (int)fmmgen_lsize(order, g_cfg.so), order);
}
void L2L(double x, double y, double z, double *L, double *Ls, int order) {
  if (!order_ok(order)) return;
  int ls = (int)fmmgen_lsize(order, g_cfg.so);
  scalar_op<double>(3, x, y, z, L, ls, Ls, ls, order);
}
void L2P(double x, double y, double z, double *L, double *F, int order) {
  if (!order_ok(order)) return;
  scalar_op<double>(4, x, y, z, L, (int)fmmgen_lsize(order, g_cfg.so), F, fmmgen_outputsize(g_cfg.potential, g_cfg.field),
            order);
}
void M2P(double x, double y, double z, double *M, double *F, int order) {
  if (!order_ok(order)) return;
  scalar_op<double>(6, x, y, z, M, (int)fmmgen_msize(order, g_cfg.so), F, fmmgen_outputsize(g_cfg.potential, g_cfg.field),
            order);
}
void P2P(double x, double y, double z, double *Sv, double *F) {
  scalar_op<double>(5, x, y, z, Sv, fmmgen_sourcesize(g_cfg.so), F, fmmgen_outputsize(g_cfg.potential, g_cfg.field), 0);
}

// precision="float" twins (fmmgen/writer.py:105, fmmgen/printers.py:301-303:
// every double of the generated signatures becomes float)
void P2Mf(float x, float y, float z, float q, float *M, int order) {
  if (!order_ok(order)) return;
  scalar_op<float>(0, x, y, z, &q, 1, M, (int)fmmgen_msize(order, g_cfg.so), order);
}
void M2Mf(float x, float y, float z, float *M, float *Ms, int order) {
  if (!order_ok(order)) return;
  int ms = (int)fmmgen_msize(order, g_cfg.so);
  scalar_op<float>(1, x, y, z, M, ms, Ms, ms, order);
}
void M2Lf(float x, float y, float z, float *M, float *L, int order) {
  if (!order_ok(order)) return;
  scalar_op<float>(2, x, y, z, M, (int)fmmgen_msize(order, g_cfg.so), L, (int)fmmgen_lsize(order, g_cfg.so), order);
}
void L2Lf(float x, float y, float z, float *L, float *Ls, int order) {
  if (!order_ok(order)) return;
  int ls = (int)fmmgen_lsize(order, g_cfg.so);
  scalar_op<float>(3, x, y, z, L, ls, Ls, ls, order);
}
void L2Pf(float x, float y, float z, float *L, float *F, int order) {
  if (!order_ok(order)) return;
  scalar_op<float>(4, x, y, z, L, (int)fmmgen_lsize(order, g_cfg.so), F,
                   fmmgen_outputsize(g_cfg.potential, g_cfg.field), order);
}
void M2Pf(float x, float y, float z, float *M, float *F, int order) {
  if (!order_ok(order)) return;
  scalar_op<float>(6, x, y, z, M, (int)fmmgen_msize(order, g_cfg.so), F,
                   fmmgen_outputsize(g_cfg.potential, g_cfg.field), order);
}
void P2Pf(float x, float y, float z, float *Sv, float *F) {
  scalar_op<float>(5, x, y, z, Sv, fmmgen_sourcesize(g_cfg.so), F, fmmgen_outputsize(g_cfg.potential, g_cfg.field),
                   0);
}

// Per-order functions of the generated code (P2M_p ... M2P_p, fmmgen/writer.py:142-264,
// declared in include/operators.h).  The generator emits them for p in
// [minorder, maxorder); here every p up to 12 exists and applies order p under the
// configured source order and outputs, whatever the dispatchers' highest order is;
// p below the minimum order is a no-op.
#define FMM_PER_ORDER(p)                                                                                         \
  void P2M_##p(double x, double y, double z, double q, double *M) {                                           \
    if (fixed_order_ok(p)) scalar_op<double>(0, x, y, z, &q, 1, M, (int)fmmgen_msize(p, g_cfg.so), p);         \
  }                                                                                                            \
  void M2M_##p(double x, double y, double z, double *M, double *Ms) {                                         \
    int ms = (int)fmmgen_msize(p, g_cfg.so);                                                                   \
    if (fixed_order_ok(p)) scalar_op<double>(1, x, y, z, M, ms, Ms, ms, p);                                    \
  }                                                                                                            \
  void M2L_##p(double x, double y, double z, double *M, double *L) {                                          \
    if (fixed_order_ok(p))                                                                                     \
      scalar_op<double>(2, x, y, z, M, (int)fmmgen_msize(p, g_cfg.so), L, (int)fmmgen_lsize(p, g_cfg.so), p);  \
  }                                                                                                            \
  void L2L_##p(double x, double y, double z, double *L, double *Ls) {                                         \
    int ls = (int)fmmgen_lsize(p, g_cfg.so);                                                                   \
    if (fixed_order_ok(p)) scalar_op<double>(3, x, y, z, L, ls, Ls, ls, p);                                    \
  }                                                                                                            \
  void L2P_##p(double x, double y, double z, double *L, double *F) {                                          \
    if (fixed_order_ok(p))                                                                                     \
      scalar_op<double>(4, x, y, z, L, (int)fmmgen_lsize(p, g_cfg.so), F,                                     \
                        fmmgen_outputsize(g_cfg.potential, g_cfg.field), p);                                   \
  }                                                                                                            \
  void M2P_##p(double x, double y, double z, double *M, double *F) {                                          \
    if (fixed_order_ok(p))                                                                                     \
      scalar_op<double>(6, x, y, z, M, (int)fmmgen_msize(p, g_cfg.so), F,                                     \
                        fmmgen_outputsize(g_cfg.potential, g_cfg.field), p);                                   \
  }
FMM_PER_ORDER(0)
FMM_PER_ORDER(1)
FMM_PER_ORDER(2)
FMM_PER_ORDER(3)
FMM_PER_ORDER(4)
FMM_PER_ORDER(5)
FMM_PER_ORDER(6)
FMM_PER_ORDER(7)
FMM_PER_ORDER(8)
FMM_PER_ORDER(9)
FMM_PER_ORDER(10)
FMM_PER_ORDER(11)
FMM_PER_ORDER(12)
#undef FMM_PER_ORDER

// ---------------------------------------------------------------------------
// tree API
// ---------------------------------------------------------------------------
int fmmgen_tree_build(const double *pos, long N, long ncrit, int order, double theta, int so, void *stream,
                      fmmgen_tree **tree) {
  g_err.clear();
  if (!tree) return ret(FMM_ERR_ARG);
  fmmgen_tree *h = *tree;
  if (!h) h = new fmmgen_tree();
  h->built = false;
  int rc = fmm_tree_build(&h->t, pos, N, ncrit, order, theta, so, S(stream));
  *tree = h;
  if (rc == FMM_OK) h->built = true;
  return ret(rc);
}

int fmmgen_forest_build(const double *pos, const long *sys_off, int nsys, long ncrit, int order, double theta,
                        int so, void *stream, fmmgen_tree **tree) {
  g_err.clear();
  if (!tree || !sys_off || nsys < 1) return ret(FMM_ERR_ARG);
  fmmgen_tree *h = *tree;
  if (!h) h = new fmmgen_tree();
  h->built = false;
  int rc = fmm_tree_build(&h->t, pos, sys_off[nsys], ncrit, order, theta, so, S(stream), sys_off, nsys);
  *tree = h;
  if (rc == FMM_OK) h->built = true;
  return ret(rc);
}

int fmmgen_tree_build_compute(const double *pos, const long *sys_off, int nsys, long N, long ncrit, int order,
                              double theta, int so, const double *Sv, double *F, int potential, int field,
                              int precision, void *stream, fmmgen_tree **tree) {
  g_err.clear();
  if (!tree || nsys < 1 || (nsys > 1 && !sys_off)) return ret(FMM_ERR_ARG);
  if (sys_off && sys_off[nsys] != N) return ret(FMM_ERR_ARG);
  fmmgen_tree *h = *tree;
  if (!h) h = new fmmgen_tree();
  h->built = false;
  h->last_precision = -1;
  int rc = fmm_tree_build_evaluate(&h->t, pos, N, ncrit, order, theta, so, nsys > 1 ? sys_off : nullptr, nsys, Sv, F,
                                   potential, field, precision, S(stream));
  *tree = h;
  if (rc == FMM_OK) {
    h->built = true;
    h->last_precision = precision;
  }
  return ret(rc);
}

int fmmgen_tree_compute_field_fmm(fmmgen_tree *tree, const double *Sv, double *F, int potential, int field,
                                  int precision, void *stream) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  int rc = fmm_tree_evaluate(&tree->t, Sv, F, potential, field, precision, S(stream));
  if (rc == FMM_OK) tree->last_precision = precision;
  return ret(rc);
}

int fmmgen_tree_compute_field_bh(fmmgen_tree *tree, const double *Sv, double *F, int potential, int field,
                                  void *st) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  return ret(fmm_tree_evaluate_bh(&tree->t, Sv, F, potential, field, S(st)));
}

int fmmgen_gpu_direct(const double *pos, const double *Sv, long N, const long *targets, long ntargets, int so,
                      int potential, int field, double *F, void *stream) {
  g_err.clear();
  return ret(fmm_direct(pos, Sv, N, targets, ntargets, so, potential, field, F, S(stream)));
}

int fmmgen_tree_free(fmmgen_tree *tree) {
  if (!tree) return FMM_OK;
  cudaDeviceSynchronize();
  fmm_tree_destroy(&tree->t);
  delete tree;
  return FMM_OK;
}

int fmmgen_tree_counts(fmmgen_tree *tree, long *info) {
  g_err.clear();
  if (!tree || !tree->built || !info) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  info[0] = t.ncells; info[1] = t.nleaves; info[2] = t.nm2l; info[3] = t.np2p;
  info[4] = t.nlevels; info[5] = t.nclasses; info[6] = t.N; info[7] = t.ncrit;
  return FMM_OK;
}

int fmmgen_tree_info(fmmgen_tree *tree, long *info) {
  if (int rc = fmmgen_tree_counts(tree, info)) return rc;
  info[8] = (long)fmm_p2p_interactions(&tree->t);
  return FMM_OK;
}

int fmmgen_tree_set_graph(fmmgen_tree *tree, int enable) {
  g_err.clear();
  if (!tree) return ret(FMM_ERR_STATE);
  tree->t.graph_on = enable != 0;
  if (!enable) fmm_graph_release(&tree->t);
  return FMM_OK;
}

int fmmgen_tree_nsys(fmmgen_tree *tree) {
  if (!tree || !tree->built) return 0;
  return tree->t.nsys;
}

int fmmgen_tree_export_systems(fmmgen_tree *tree, double *roots4, int *cell_system) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  if (roots4) FMM_CUDA_TRY(cudaMemcpy(roots4, t.roots.p, sizeof(double) * 4 * t.nsys, cudaMemcpyDeviceToHost));
  if (cell_system) FMM_CUDA_TRY(cudaMemcpy(cell_system, t.csys.p, sizeof(int) * t.ncells, cudaMemcpyDeviceToHost));
  return FMM_OK;
}

int fmmgen_tree_root(fmmgen_tree *tree, double *root4) {
  if (!tree || !tree->built || !root4) return ret(FMM_ERR_STATE);
  root4[0] = tree->t.root.cx; root4[1] = tree->t.root.cy; root4[2] = tree->t.root.cz; root4[3] = tree->t.root.r;
  return FMM_OK;
}

int fmmgen_tree_export_cells(fmmgen_tree *tree, unsigned long long *cell_id, long *cell_count, double *centre,
                             long *leaf_off, long *leaf_idx) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<uint64_t> cid;
  std::vector<int> ps, pc;
  std::vector<double> x, y, z;
  std::vector<uint32_t> perm;
  size_t nc = t.ncells;
  if (d2h(cid, t.cid.p, nc) || d2h(ps, t.pstart.p, nc) || d2h(pc, t.pcount.p, nc) || d2h(x, t.cx.p, nc) ||
      d2h(y, t.cy.p, nc) || d2h(z, t.cz.p, nc) || d2h(perm, t.perm.p, t.N))
    return ret(FMM_ERR_CUDA);
  long k = 0, o = 0;
  for (size_t c = 0; c < nc; c++) {
    if (cell_id) cell_id[c] = cid[c];
    if (cell_count) cell_count[c] = pc[c];
    if (centre) { centre[3 * c] = x[c]; centre[3 * c + 1] = y[c]; centre[3 * c + 2] = z[c]; }
    if (pc[c] < t.ncrit) {
      if (leaf_off) leaf_off[k] = o;
      for (int i = 0; i < pc[c]; i++) {
        if (leaf_idx) leaf_idx[o] = perm[ps[c] + i];
        o++;
      }
      k++;
    }
  }
  if (leaf_off) leaf_off[k] = o;
  return FMM_OK;
}

int fmmgen_tree_export_lists(fmmgen_tree *tree, unsigned long long *m2l, unsigned long long *p2p) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  if (int rc = fmm_m2l_csr(&t, 0)) return ret(rc);
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  size_t nc = t.ncells;
  std::vector<uint64_t> cid;
  std::vector<int> moff, msrc, poff, psrc;
  if (d2h(cid, t.cid.p, nc) || d2h(moff, t.m2l_off.p, nc + 1) || d2h(msrc, t.m2l_src.p, t.nm2l) ||
      d2h(poff, t.p2p_off.p, nc + 1) || d2h(psrc, t.p2p_src.p, t.np2p))
    return ret(FMM_ERR_CUDA);
  for (size_t c = 0; c < nc; c++) {
    if (m2l)
      for (int k = moff[c]; k < moff[c + 1]; k++) { m2l[2 * k] = cid[msrc[k]]; m2l[2 * k + 1] = cid[c]; }
    if (p2p)
      for (int k = poff[c]; k < poff[c + 1]; k++) { p2p[2 * k] = cid[c]; p2p[2 * k + 1] = cid[psrc[k]]; }
  }
  return FMM_OK;
}

}  // extern "C"

// M_n = M~_n s^|n|, L_n = L^_n / s^(|n|+1)
template <typename T>
__global__ void k_unscale(const T *Ms, const T *Ls, const double *cr, int ncells,
                          int msize, int moff, int lsize, int mstr, int lstr, double *Mo, double *Lo) {
  int c = blockIdx.x;
  if (c >= ncells) return;
  double s = cr[c];
  for (int j = threadIdx.x; j < msize; j += blockDim.x) {
    int d = c_mi[j + moff][3];
    Mo[(size_t)c * msize + j] = (double)Ms[(size_t)c * mstr + j] * pow(s, d);
  }
  for (int j = threadIdx.x; j < lsize; j += blockDim.x) {
    int d = c_mi[j][3];
    Lo[(size_t)c * lsize + j] = (double)Ls[(size_t)c * lstr + j] / pow(s, d + 1);
  }
}

extern "C" int fmmgen_tree_export_expansions(fmmgen_tree *tree, double *M, double *L) {
  g_err.clear();
  if (!tree || !tree->built || tree->last_precision < 0) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  int ms = (int)fmmgen_msize(t.order, t.so), ls = (int)fmmgen_lsize(t.order, t.so), moff = fmm_nterms(t.so - 1);
  size_t nc = t.ncells;
  double *dM = nullptr, *dL = nullptr;
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  FMM_CUDA_TRY(cudaMalloc((void **)&dM, nc * ms * sizeof(double)));
  FMM_CUDA_TRY(cudaMalloc((void **)&dL, nc * ls * sizeof(double)));
  if (tree->last_precision == FMMGEN_PREC_FP64)
    fmm_note_launch(), k_unscale<double><<<(unsigned)nc, 128>>>(t.M.p, t.L.p, t.cr.p, (int)nc, ms, moff, ls, ms, ls, dM, dL);
  else
    fmm_note_launch(), k_unscale<float><<<(unsigned)nc, 128>>>(t.Mf.p, t.Lf.p, t.cr.p, (int)nc, ms, moff, ls, fmm_stride4(ms),
                                                   fmm_stride4(ls), dM, dL);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(M, dM, nc * ms * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(L, dL, nc * ls * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(dM);
  cudaFree(dL);
  if (e != cudaSuccess) {
    fmm_set_cuda_error(e, "export_expansions", __FILE__, __LINE__);
    return FMM_ERR_CUDA;
  }
  return FMM_OK;
}

extern "C" int fmmgen_tree_m2l_work(fmmgen_tree *tree, double *out4) {
  double *out3 = out4;
  if (!tree || !tree->built || !out3) return ret(FMM_ERR_STATE);
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  DevTree &t = tree->t;
  long long mmas = 0;
  double flops = 0;
  unsigned long long steps = 0;
  if (t.h_pinned && t.tc_ran && fmm_m2l_tc_step_work(t.order, t.so, t.tc_boxes_last != 0, &mmas, &flops))
    memcpy(&steps, t.h_pinned + FMM_PINNED_TCERR + 2, sizeof(steps));
  out3[0] = (double)steps;
  out3[1] = (double)steps * (double)mmas;
  out3[2] = (double)steps * flops;
  out4[3] = t.tc_ran && t.tc_boxes_last ? 1.0 : 0.0;
  return FMM_OK;
}

// ---- M2L choices and the autotuner -------------------------------------------
extern "C" {
int fmmgen_tree_set_tune(fmmgen_tree *tree, int impl, int nslots, int grouping, int overlap) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  if (impl < -1 || impl > 5 || nslots < 0 || grouping < 0 || grouping > 1 || overlap < 0 || overlap > 2)
    return ret(FMM_ERR_ARG);
  if ((impl == 0 || impl == 3) && !fmm_m2l_tc_supported(t.order, t.so)) {
    fmm_set_error_text("the tensor-core M2L does not support this order / source order");
    return ret(FMM_ERR_ARG);
  }
  if (impl == 1 && !fmm_m2l_gen_supported(t.order, t.so)) {
    fmm_set_error_text("no generated CUDA-core M2L kernels for this order / source order");
    return ret(FMM_ERR_ARG);
  }
  if ((impl == 4 || impl == 5) && !fmm_m2l_cm_supported(t.order, t.so)) {
    fmm_set_error_text("no class-major CUDA-core M2L kernels for this order / source order");
    return ret(FMM_ERR_ARG);
  }
  fmm_graph_release(&t);  // a recorded pass holds the old choice
  t.tune.impl = impl;
  t.tune.nslots = nslots;
  t.tune.grouping = grouping;
  t.tune.overlap = overlap;
  return FMM_OK;
}

int fmmgen_tree_get_tune(fmmgen_tree *tree, int *tune4) {
  if (!tree || !tree->built || !tune4) return ret(FMM_ERR_STATE);
  tune4[0] = tree->t.tune.impl;
  tune4[1] = tree->t.tune.nslots;
  tune4[2] = tree->t.tune.grouping;
  tune4[3] = tree->t.tune.overlap;
  return FMM_OK;
}

int fmmgen_tree_autotune(fmmgen_tree *tree, const double *Sv, int precision, int reps, int max_cand, int *cand4,
                         float *cand_ms, int *ncand, void *st) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  if (!Sv || precision < 0 || precision > 2 || reps < 1 || max_cand < 0) return ret(FMM_ERR_ARG);
  const int rc = fmm_autotune(&tree->t, Sv, precision, reps, max_cand, cand4, cand_ms, ncand, S(st));
  if (rc == FMM_OK) tree->last_precision = precision;
  return ret(rc);
}
}  // extern "C"

// ---- learned per-pair M2L orders -------------------------------------------
extern "C" {
int fmmgen_order_model_nparam(void) { return fmm_mlp_nparam(); }
int fmmgen_order_nfeatures(void) { return 16; }
int fmmgen_order_nclasses(void) { return 11; }

int fmmgen_tree_order_features(fmmgen_tree *tree, double eps, float *feat, void *st) {
  g_err.clear();
  if (!tree || !tree->built || tree->last_precision < 0) return ret(FMM_ERR_STATE);
  if ((!feat && tree->t.nm2l > 0) || !(eps > 0)) return ret(FMM_ERR_ARG);
  return ret(fmm_order_features(&tree->t, eps, feat, S(st)));
}

int fmmgen_tree_order_labels(fmmgen_tree *tree, double eps, unsigned char *label, float *errq, void *st) {
  g_err.clear();
  if (!tree || !tree->built || tree->last_precision != FMMGEN_PREC_FP64) return ret(FMM_ERR_STATE);
  if (!(eps > 0) || (!label && tree->t.nm2l > 0)) return ret(FMM_ERR_ARG);
  return ret(fmm_order_labels(&tree->t, eps, label, errq, S(st)));
}

int fmmgen_tree_set_m2l_orders(fmmgen_tree *tree, const unsigned char *orders, void *st) {
  g_err.clear();
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  fmm_graph_release(&t);  // a recorded pass holds the old M2L choice
  if (!orders) {
    t.ord_mode = t.model ? 2 : 0;
    return FMM_OK;
  }
  int rc = fmm_reserve(t.m2l_ord, t.nm2l > 0 ? t.nm2l : 1);
  if (rc) return ret(rc);
  if (t.nm2l > 0)
    FMM_CUDA_TRY(cudaMemcpyAsync(t.m2l_ord.p, orders, t.nm2l, cudaMemcpyDeviceToDevice, S(st)));
  t.ord_mode = 1;
  t.ord_serial = t.build_serial;
  return FMM_OK;
}

int fmmgen_tree_set_order_model(fmmgen_tree *tree, const float *params, float delta, double eps) {
  g_err.clear();
  if (!tree) return ret(FMM_ERR_STATE);
  if (params && (!(delta >= 0.f && delta < 1.f) || !(eps > 0))) return ret(FMM_ERR_ARG);
  DevTree &t = tree->t;
  fmm_graph_release(&t);
  t.model = params;
  t.model_delta = delta;
  if (params) t.model_eps = eps;
  t.ord_mode = params ? 2 : 0;
  return FMM_OK;
}

int fmmgen_tree_export_m2l_orders(fmmgen_tree *tree, unsigned char *orders_host) {
  g_err.clear();
  if (!tree || !tree->built || tree->last_precision < 0) return ret(FMM_ERR_STATE);
  DevTree &t = tree->t;
  if (t.nm2l == 0) return FMM_OK;
  if (!orders_host) return ret(FMM_ERR_ARG);
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  if (t.ord_mode == 0 || t.ord_serial != t.build_serial) {
    memset(orders_host, t.order, t.nm2l);
    return FMM_OK;
  }
  std::vector<unsigned char> o;
  if (d2h(o, t.m2l_ord.p, t.nm2l)) return ret(FMM_ERR_CUDA);
  for (long k = 0; k < t.nm2l; k++) orders_host[k] = (unsigned char)std::min(std::max((int)o[k], t.so + 1), t.order);
  return FMM_OK;
}

int fmmgen_mlp_predict(const float *params, const float *X, long n, float delta, int qmax, unsigned char *orders,
                       void *st) {
  g_err.clear();
  if (n < 0 || (n > 0 && (!params || !X || !orders)) || !(delta >= 0.f && delta < 1.f) || qmax < 2)
    return ret(FMM_ERR_ARG);
  return ret(fmm_mlp_predict(params, X, n, delta, qmax, orders, S(st)));
}

long fmmgen_mlp_train_work(int n) { return n > 0 ? 267L * n : 0; }

int fmmgen_mlp_train_step(const float *params, const float *X, const unsigned char *y, int n, float *grad,
                          float *loss, float *work, void *st) {
  g_err.clear();
  if (n <= 0 || !params || !X || !y || !grad || !loss || !work) return ret(FMM_ERR_ARG);
  return ret(fmm_mlp_train_step(params, X, y, n, grad, loss, work, S(st)));
}

int fmmgen_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr, void *st) {
  g_err.clear();
  if (!params || !grad || !m || !v || step < 1) return ret(FMM_ERR_ARG);
  return ret(fmm_mlp_adam(params, grad, m, v, step, lr, S(st)));
}
}  // extern "C"

extern "C" int fmmgen_tree_kernel_ms(fmmgen_tree *tree, float *ms2) {
  if (!tree || !tree->built || !ms2) return ret(FMM_ERR_STATE);
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  ms2[0] = ms2[1] = -1.f;
  if (tree->last_precision >= 0) {
    fmm_eval_times(&tree->t);
    ms2[0] = tree->t.kernel_ms[0];
    ms2[1] = tree->t.kernel_ms[1];
  }
  return FMM_OK;
}

extern "C" int fmmgen_tree_times(fmmgen_tree *tree, float *build_ms6, float *eval_ms8) {
  if (!tree || !tree->built) return ret(FMM_ERR_STATE);
  FMM_CUDA_TRY(cudaDeviceSynchronize());
  if (tree->t.h_pinned && tree->t.h_pinned[FMM_PINNED_TCERR]) {
    fmm_set_error_text("tensor-core M2L: a pipeline wait timed out");
    return ret(FMM_ERR_CUDA);
  }
  if (build_ms6) memcpy(build_ms6, tree->t.build_ms, sizeof(float) * 6);
  if (eval_ms8 && tree->last_precision >= 0) {
    fmm_eval_times(&tree->t);
    memcpy(eval_ms8, tree->t.phase_ms, sizeof(float) * 8);
  }
  return FMM_OK;
}
