/*
 * fmmgen_gb300.h -- C ABI of the GB300 (sm_103a) octree FMM library
 * (libfmmgen_gb300.so).
 *
 * It replaces two interfaces of rpep/fmmgen:
 *   1. the operator ABI that fmmgen.generate_code emits (fmmgen/writer.py:266-330,
 *      signatures from fmmgen/printers.py:296-313; example instance
 *      example/operators.cpp:1376-1489): P2M / M2M / M2L / L2L / L2P / P2P with
 *      "+=" semantics and the FMMGEN_* header macros;
 *   2. the example tree code's API (example/tree.hpp:78-103):
 *      build_tree(pos, S, N, ncrit, order, theta) and
 *      Tree::compute_field_fmm(F) / Tree::compute_field_exact(F).
 *
 * Layouts are fmmgen's: positions [N][3], sources [N][SOURCESIZE]
 * (SOURCESIZE = 1 for charges, 3 for dipoles, 6 for quadrupoles: the degree-
 * source_order multipole coefficients in fmmgen's order), outputs [N][OUTPUTSIZE]
 * (phi, Ex, Ey, Ez as selected by potential/field), multipole/local arrays in
 * the Nterms multi-index order of fmmgen/utils.py:65-118.  All arrays are
 * FP64.  Unless a function says "host", pointers are device pointers and work
 * is stream-ordered on `stream` (a cudaStream_t, NULL = legacy default).
 * Every function returns a status code (0 = OK) and never aborts; the text of
 * the last error is available from fmmgen_last_error().
 */
#ifndef FMMGEN_GB300_H
#define FMMGEN_GB300_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FMMGEN_OK 0
#define FMMGEN_ERR_ARG 1     /* invalid argument (order out of range, N < 1, ...) */
#define FMMGEN_ERR_CUDA 2    /* CUDA runtime error; see fmmgen_last_error() */
#define FMMGEN_ERR_DEPTH 3   /* tree would be deeper than 21 levels (>= ncrit coincident points) */
#define FMMGEN_ERR_RANGE 4   /* an M2L offset beyond 2^18 finer-level half-widths (class key range) */
#define FMMGEN_ERR_STATE 5   /* handle not built */

/* precision modes of fmmgen_tree_compute_field_fmm */
#define FMMGEN_PREC_FP64 0   /* every phase in FP64 */
#define FMMGEN_PREC_MIXED 1  /* FP32 sweeps/M2L/P2P, FP64 operator assembly and final accumulation;
                                M2L on the tensor cores (3 FP16 products per term, FP32
                                accumulation) for orders <= 9 */
#define FMMGEN_PREC_MIXED_SIMT 2  /* as FMMGEN_PREC_MIXED with the M2L on the FP32 CUDA cores */

const char *fmmgen_last_error(void);
const char *fmmgen_version(void);
int fmmgen_max_order(void); /* highest expansion order supported (12) */
long long fmmgen_launch_count(void); /* kernels this library has launched so far (no counterpart in the reference) */

/* ---- layout constants (the FMMGEN_* macros of fmmgen/writer.py:317-328 and
 *      Nterms/Msize/Lsize of fmmgen/utils.py:26-35, example/utils.cpp:3-27) ---- */
long fmmgen_nterms(int p);
long fmmgen_msize(int order, int source_order);
long fmmgen_lsize(int order, int source_order);
int fmmgen_minorder(int source_order, int field);   /* FMMGEN_MINORDER = source_order + field */
int fmmgen_sourcesize(int source_order);            /* FMMGEN_SOURCESIZE */
int fmmgen_outputsize(int potential, int field);    /* FMMGEN_OUTPUTSIZE */

/* ---- batched operators: n independent applications, device pointers ----
 * Each replaces n calls of the generated scalar operator with the same name
 * (fmmgen/writer.py:147-254): application i reads d[3i..3i+2] and the i-th
 * input block and adds into the i-th output block.
 *   P2M: in = q[n],          out = M[n][Msize]     (fmmgen/expansions.py:22-39)
 *   M2M: in = M[n][Msize],   out = Ms[n][Msize]    (fmmgen/expansions.py:42-78)
 *   M2L: in = M[n][Msize],   out = L[n][Lsize]     (fmmgen/expansions.py:108-172)
 *   L2L: in = L[n][Lsize],   out = Ls[n][Lsize]    (fmmgen/expansions.py:175-194)
 *   L2P: in = L[n][Lsize],   out = F[n][OUTPUTSIZE](fmmgen/expansions.py:197-207)
 *   P2P: in = S[n][SOURCESIZE], out = F[n][OUTPUTSIZE] (example/operators.cpp:54-66)
 *   M2P: in = M[n][Msize],   out = F[n][OUTPUTSIZE] (fmmgen/generator.py:174-206: the
 *        potential of fmmgen's M2P and its exact gradient as the field) */
int fmmgen_gpu_P2M(int n, const double *d, const double *q, double *M, int order, int source_order, void *stream);
int fmmgen_gpu_M2M(int n, const double *d, const double *M, double *Ms, int order, int source_order, void *stream);
int fmmgen_gpu_M2L(int n, const double *d, const double *M, double *L, int order, int source_order, void *stream);
int fmmgen_gpu_L2L(int n, const double *d, const double *L, double *Ls, int order, int source_order, void *stream);
int fmmgen_gpu_L2P(int n, const double *d, const double *L, double *F, int order, int source_order, int potential,
                   int field, void *stream);
int fmmgen_gpu_P2P(int n, const double *d, const double *S, double *F, int source_order, int potential, int field,
                   void *stream);
int fmmgen_gpu_M2P(int n, const double *d, const double *M, double *F, int order, int source_order, int potential,
                   int field, void *stream);

/* The same seven operators in FP32: the generator's precision="float" variant
 * (fmmgen/writer.py:105, fmmgen/printers.py:237-303 -- every double of the
 * generated code becomes float).  float buffers, float arithmetic throughout. */
int fmmgen_gpu_P2M_f32(int n, const float *d, const float *q, float *M, int order, int source_order, void *stream);
int fmmgen_gpu_M2M_f32(int n, const float *d, const float *M, float *Ms, int order, int source_order, void *stream);
int fmmgen_gpu_M2L_f32(int n, const float *d, const float *M, float *L, int order, int source_order, void *stream);
int fmmgen_gpu_L2L_f32(int n, const float *d, const float *L, float *Ls, int order, int source_order, void *stream);
int fmmgen_gpu_L2P_f32(int n, const float *d, const float *L, float *F, int order, int source_order, int potential,
                       int field, void *stream);
int fmmgen_gpu_P2P_f32(int n, const float *d, const float *S, float *F, int source_order, int potential, int field,
                       void *stream);
int fmmgen_gpu_M2P_f32(int n, const float *d, const float *M, float *F, int order, int source_order, int potential,
                       int field, void *stream);

/* ---- scalar twins of the generated dispatchers (host pointers, run on the
 *      GPU synchronously).  Signatures of example/operators.cpp:1376-1489;
 *      source_order / potential / field are those set by fmmgen_configure
 *      (the generator fixes them at generation time, fmmgen/writer.py:33-50).
 *      An order outside [minorder, maxorder] is a silent no-op, as the
 *      generated switch has no default case (fmmgen/writer.py:296-309). ---- */
int fmmgen_configure(int source_order, int potential, int field, int maxorder);
void P2M(double x, double y, double z, double q, double *M, int order);
void M2M(double x, double y, double z, double *M, double *Ms, int order);
void M2L(double x, double y, double z, double *M, double *L, int order);
void L2L(double x, double y, double z, double *L, double *Ls, int order);
void L2P(double x, double y, double z, double *L, double *F, int order);
void M2P(double x, double y, double z, double *M, double *F, int order);
void P2P(double x, double y, double z, double *S, double *F);
/* precision="float" scalar twins: the generated float signatures
 * (fmmgen/printers.py:301-303), with an f suffix so that both live in one
 * library; same configuration and order rules as the double twins. */
void P2Mf(float x, float y, float z, float q, float *M, int order);
void M2Mf(float x, float y, float z, float *M, float *Ms, int order);
void M2Lf(float x, float y, float z, float *M, float *L, int order);
void L2Lf(float x, float y, float z, float *L, float *Ls, int order);
void L2Pf(float x, float y, float z, float *L, float *F, int order);
void M2Pf(float x, float y, float z, float *M, float *F, int order);
void P2Pf(float x, float y, float z, float *S, float *F);

/* ---- tree-level API (example/tree.hpp:78-103) ---- */
typedef struct fmmgen_tree fmmgen_tree;

/* build_tree (example/tree.cpp:130-233) on the device: adaptive octree with the
 * reference's root cube, ncrit split rule and FP64 centre arithmetic, and the
 * M2L/P2P interaction lists of interact_dehnen_lazy (example/calculate.cpp:81-133).
 * pos: device [N][3].  *tree may be NULL (a new handle is made) or an existing
 * handle whose device buffers are reused.  Synchronises `stream`. */
int fmmgen_tree_build(const double *pos, long N, long ncrit, int order, double theta, int source_order,
                      void *stream, fmmgen_tree **tree);

/* A forest of independent systems in one handle (no counterpart in the
 * reference, whose Tree holds one system): system s owns the particles
 * [sys_off[s], sys_off[s+1]) of pos (host array of nsys + 1 offsets,
 * sys_off[0] = 0, sys_off[nsys] = N, every system non-empty).  Each system gets
 * exactly the tree, root cube and interaction lists build_tree would give it
 * alone; the build and every evaluation phase run once over all systems (one
 * launch per phase, not per system).  fmmgen_tree_compute_field_fmm then
 * evaluates all systems together (S and F over all N particles).  Same ncrit,
 * order, theta and source order for every system. */
int fmmgen_forest_build(const double *pos, const long *sys_off, int nsys, long ncrit, int order, double theta,
                        int source_order, void *stream, fmmgen_tree **tree);

/* Tree::compute_field_fmm (example/tree.cpp:243-271): F (device
 * [N][OUTPUTSIZE], caller's particle order) is overwritten with phi / E from
 * the sources S (device [N][SOURCESIZE], caller's particle order).  Does not
 * synchronise. */
int fmmgen_tree_compute_field_fmm(fmmgen_tree *tree, const double *S, double *F, int potential, int field,
                                  int precision, void *stream);

/* Graph mode (no counterpart in the reference): with enable != 0 the first
 * fmmgen_tree_compute_field_fmm after a build -- or after S, F, the output
 * switches or the precision change -- runs normally and is then recorded as a
 * CUDA graph; later calls with the same build and arguments replay the whole
 * evaluation pass as one graph launch on `stream`.  The recording uses a
 * private stream, so `stream` may be the legacy default stream.  enable = 0
 * drops the graph. */
int fmmgen_tree_set_graph(fmmgen_tree *tree, int enable);

/* Tree::compute_field_exact / evaluate_direct (example/calculate.cpp:252-264):
 * FP64 O(N^2) sum for the targets listed in `targets` (device, NULL = all N);
 * F is [ntargets][OUTPUTSIZE] in the order of `targets`. */
int fmmgen_gpu_direct(const double *pos, const double *S, long N, const long *targets, long ntargets,
                      int source_order, int potential, int field, double *F, void *stream);

int fmmgen_tree_free(fmmgen_tree *tree);

/* Root cube of build_tree ([cx, cy, cz, r] into the device array root4),
 * bit-identical to the one fmmgen_tree_build computes, WITHOUT allocating any
 * device memory: no counterpart in the reference.  For callers that cannot call
 * cudaMalloc where they need the cube (another allocator already holds the
 * GPU's free memory, or cudaMalloc's implicit synchronisation is not
 * acceptable).  Its scratch is one static device array of ~11 MiB, enough
 * for N <= FMMGEN_NOALLOC_MAX_N; larger N returns FMMGEN_ERR_ARG.  CUDA loads
 * device code lazily by default, so the first call on a device places the
 * array and this function's kernels there and looks the array's address up
 * (cudaGetSymbolAddress): make that first call (a tiny input will do) before
 * another allocator takes the GPU's free memory and before any stream
 * capture; later calls allocate nothing, and the device keeps the array until
 * the process exits.  Not for use on a device after cudaDeviceReset (the
 * address is cached per device).  All calls share the array: calls that
 * overlap on the GPU race. */
#define FMMGEN_NOALLOC_MAX_N 16777216L
int fmmgen_root_box_noalloc(const double *pos, long N, double *root4, void *stream);

/* Introspection (host outputs; synchronises).
 * info: [ncells, nleaves, nm2l, np2p, nlevels, nclasses, N, ncrit, P2P particle interactions].
 * fmmgen_tree_counts fills the first eight without waiting for the device. */
int fmmgen_tree_info(fmmgen_tree *tree, long *info);
int fmmgen_tree_counts(fmmgen_tree *tree, long *info8);
/* build_tree + Tree::compute_field_fmm in one call (fmmgen_tree_build /
 * fmmgen_forest_build, then fmmgen_tree_compute_field_fmm, on the same
 * handle): the near field and the multipoles are computed on a second stream
 * while the build groups the M2L lists by class, and the M2L runs beside the
 * near field's tail.  sys_off / nsys as in fmmgen_forest_build (NULL, 1: one
 * system).  The handle is then built, as after fmmgen_tree_build. */
int fmmgen_tree_build_compute(const double *pos, const long *sys_off, int nsys, long N, long ncrit, int order,
                              double theta, int source_order, const double *S, double *F, int potential, int field,
                              int precision, void *stream, fmmgen_tree **tree);
/* Tree::compute_field_bh (example/tree.cpp:273-293): FP64 P2M and M2M, then
 * for every particle the walk of evaluate_M2P_and_P2P
 * (example/calculate.cpp:266-314) from its system's root: a child c of an
 * opened cell is opened when r_c > theta |x_i - c_c|, else its multipole acts
 * through M2P (fmmgen's M2P potential with its exact gradient as the field --
 * the generated field is wrong), and a leaf's particles through P2P.  S and F
 * as in fmmgen_tree_compute_field_fmm; F is overwritten. */
int fmmgen_tree_compute_field_bh(fmmgen_tree *tree, const double *S, double *F, int potential, int field,
                                 void *stream);
/* Root cube [cx, cy, cz, r] (of system 0 in a forest). */
int fmmgen_tree_root(fmmgen_tree *tree, double *root4);
/* Systems of a handle (1 for fmmgen_tree_build), their root cubes
 * [nsys][4] and the system of every cell (level-major order) -- either output
 * may be NULL. */
int fmmgen_tree_nsys(fmmgen_tree *tree);
int fmmgen_tree_export_systems(fmmgen_tree *tree, double *roots4, int *cell_system);
/* Per cell (level-major order): canonical id (1 << 3*level | octant path),
 * particle count (the reference's nleaf), centre [3]; leaf particle lists as
 * CSR over leaves in cell order (caller's particle indices). */
int fmmgen_tree_export_cells(fmmgen_tree *tree, unsigned long long *cell_id, long *cell_count, double *centre,
                             long *leaf_off, long *leaf_idx);
/* Interaction lists as canonical-id pairs, grouped by target:
 * m2l [nm2l][2] = (source, target), p2p [np2p][2] = (target, source). */
int fmmgen_tree_export_lists(fmmgen_tree *tree, unsigned long long *m2l, unsigned long long *p2p);
/* Scaled expansions of the last FP64 evaluate, unscaled back to fmmgen's
 * convention: M [ncells][Msize], L [ncells][Lsize], cells in level-major order. */
int fmmgen_tree_export_expansions(fmmgen_tree *tree, double *M, double *L);
/* Phase times of the last build ([root, keys+sort, cells, lists, classes, total])
 * and evaluate ([P2M, M2M, M2L, P2P, L2L, L2P, finalize, total]) in ms. */
int fmmgen_tree_times(fmmgen_tree *tree, float *build_ms6, float *eval_ms8);
/* Device times (ms) of the last evaluate's M2L kernels and P2P kernel alone,
 * host ms2 = [M2L, P2P], from events on their streams around the launches (no
 * counterpart in the reference; for roofline accounting): the M2L phase of
 * fmmgen_tree_times also holds its preparation (schedules, operand packing),
 * and the two kernels may run side by side; -1 where none ran. */
int fmmgen_tree_kernel_ms(fmmgen_tree *tree, float *ms2);
/* Work of the last tensor-core M2L (no counterpart in the reference; for
 * roofline accounting), host out4 = [class steps of 128-row tiles, tcgen05 MMA
 * instructions, executed tensor flops, 1 if its source rows were boxed from
 * level grids (else gathered row by row)]; zeros if none ran. */
int fmmgen_tree_m2l_work(fmmgen_tree *tree, double *out4);

/* ---- M2L choices and their autotuner (no counterpart in the reference) ----
 * impl: -1 the default rules (tensor cores for "mixed" where p <= 9 -- as
 * impl 3 --, else the generated CUDA-core kernels where the order has them:
 * impl 1, then impl 5, else the warp contraction engine), 0 tensor cores with the source rows
 * gathered row by row, 1 generated CUDA-core kernels, 2 contraction engine,
 * 3 tensor cores with the source rows boxed from dense level grids by
 * tensor-map copies where every level of the tree is complete (one system,
 * all 8^l cells of every level), else as 0, 4 class-major CUDA-core kernels
 * (a warp takes 32 target cells' pairs of one translation class per step),
 * 5 target-major CUDA-core kernels (a thread per target cell over its list);
 * 4 and 5 cover orders up to 12 for charges, 8 for dipoles (mixed passes;
 * FP64 passes always use the engine).  Per-pair M2L orders
 * (fmmgen_tree_set_m2l_orders, an order model) run in mixed passes on the
 * target-major kernels, on the class-major ones with impl 4, on the engine
 * with impl 2 or where the kernels do not cover the order.
 * nslots: tensor-core pipeline depth (operand slots), 0 = as many as fit.
 * grouping: order of a level's cells in M2L tiles and warps, 0 by octant
 * within the parent, 1 Morton.  overlap: 1 (2) runs the tensor-core M2L on a
 * highest-priority side stream with the P2P beside it on the same SMs, in
 * blocks of 4 (2) warps.
 * Unsupported choices are rejected. */
int fmmgen_tree_set_tune(fmmgen_tree *tree, int impl, int nslots, int grouping, int overlap);
int fmmgen_tree_get_tune(fmmgen_tree *tree, int *tune4);
/* Autotuner: one pass over S at `precision` (for the multipoles and the staged
 * particles), then the M2L and P2P phases alone timed `reps` times per
 * candidate (implementation x pipeline depth x overlap x grouping that this
 * order supports); the handle keeps the candidate with the lowest median, or
 * its serial twin (overlap 0) when that is within 2 % of it.
 * cand4 [max_cand][4] (impl, nslots, grouping, overlap) and cand_ms [max_cand]
 * receive the table (either may be NULL), *ncand its size. */
int fmmgen_tree_autotune(fmmgen_tree *tree, const double *S, int precision, int reps, int max_cand, int *cand4,
                         float *cand_ms, int *ncand, void *stream);

/* ---- learned per-pair M2L orders (no counterpart in the reference, whose
 * FMM applies one order to every pair) ----
 * An M2L pair applied at order q < p keeps the terms |n| + |m| <= q of the
 * order-p translation.  An order model is an MLP 16 -> 64 -> 64 -> 11 (ReLU,
 * FP32 parameters W1[64][16], b1[64], W2[64][64], b2[64], W3[11][64], b3[11])
 * whose 11 outputs are the logits of the orders 2..12.  Pairs are numbered in
 * the order of fmmgen_tree_export_lists; every pointer below is device memory
 * unless it says host. */
int fmmgen_order_model_nparam(void);   /* 5963 */
int fmmgen_order_nfeatures(void);      /* 16 */
int fmmgen_order_nclasses(void);       /* 11: labels 0..10 are the orders 2..12 */
/* The error budget of a pair B -> A for a relative L2 field error eps over
 * its system: eps T_A, T_A = sqrt(sum_i |E_i|^2 / P) s_A^2 / sqrt(n_A) in the
 * scaled units of A's local expansion, with E_i the near field (P2P part) of
 * the system's particles in the last evaluate, P the system's M2L pairs, s_A
 * and n_A A's half-width and particle count (the squared budget split equally
 * over the pairs; A's error reaches all its particles).
 * Features of every M2L pair from the multipoles and near field of the last
 * evaluate, feat [nm2l][16]: lB - lA, log2(separation / s_A), log10 of the
 * pair's share of its target's estimated far field, log10 of the part of
 * degree 1..12 in the pair's estimate, log10 of the pair's estimated field at
 * A over eps T_A. */
int fmmgen_tree_order_features(fmmgen_tree *tree, double eps, float *feat, void *stream);
/* Training labels (needs a last evaluate in FP64): for each pair the lowest
 * order q in [2, p] whose truncation error bound in the target cell,
 * sum_n max_cell |grad y^n / n!| |sum_{|n|+|m| > q} D_(n+m) M_m| (scaled
 * units), stays within eps T_A; label = q - 2.  errq [nm2l][11] (may be NULL):
 * the bound at q = 2..12 over eps T_A. */
int fmmgen_tree_order_labels(fmmgen_tree *tree, double eps, unsigned char *label, float *errq, void *stream);
/* Explicit per-pair orders (uint8 [nm2l], values clamped to [so + 1, p]) for
 * the evaluations of this build; orders == NULL returns to the one order p. */
int fmmgen_tree_set_m2l_orders(fmmgen_tree *tree, const unsigned char *orders, void *stream);
/* Attach an order model (parameters stay caller-owned and must outlive its
 * use): every evaluate then runs P2P before M2L, computes the features for
 * the error target eps from its own multipoles and near field, and applies
 * pair k at the lowest order whose cumulative predicted probability reaches
 * 1 - delta.  params == NULL detaches it. */
int fmmgen_tree_set_order_model(fmmgen_tree *tree, const float *params, float delta, double eps);
/* Host copy of the per-pair orders the last evaluate used (uint8 [nm2l]);
 * all p when it used one order. */
int fmmgen_tree_export_m2l_orders(fmmgen_tree *tree, unsigned char *orders_host);
/* Order-model inference on n feature rows: orders[k] in [2, qmax]. */
int fmmgen_mlp_predict(const float *params, const float *X, long n, float delta, int qmax, unsigned char *orders,
                       void *stream);
/* One training step of the order model: mean cross-entropy of the logits
 * against labels y (0..10) over n rows; grad [nparam] is overwritten with its
 * gradient, *loss (device float) is incremented by its value.  work holds
 * fmmgen_mlp_train_work(n) floats. */
long fmmgen_mlp_train_work(int n);
int fmmgen_mlp_train_step(const float *params, const float *X, const unsigned char *y, int n, float *grad,
                          float *loss, float *work, void *stream);
/* Adam update (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected, step >= 1). */
int fmmgen_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FMMGEN_GB300_H */
