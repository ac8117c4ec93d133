// ref_harness.cpp -- C entry points around the UNMODIFIED reference tree code.
//
// TEST INFRASTRUCTURE ONLY (the checker's reference leg).  oracle/ref/build_ref.py
// compiles this file together with the reference's example/tree.cpp,
// example/calculate.cpp, example/utils.cpp (read in place from the reference
// checkout) and the operators that fmmgen.generate_code emits, into
// oracle/_ref/libref_so<k>.so.  Tests use it to pin the CPU restatement in
// oracle/fmm_oracle.c and to write the golden fixtures under tests/golden/.
//
// The one substitution: fmmgen at HEAD emits a P2P whose field part is zero
// (fmmgen/generator.py:274-284 substitutes R after it has already been replaced
// by Rinv), so the generated P2P is compiled under the name
// fmmgen_generated_P2P and the P2P the example links against is the physics
// below (Coulomb form as in the shipped example/operators.cpp:54-66).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <chrono>
#include <vector>
#include "operators.h"
#include "tree.hpp"
#include "calculate.hpp"
#include "utils.hpp"

void fmmgen_generated_P2P(double x, double y, double z, double *S, double *F);

void P2P(double x, double y, double z, double *S, double *F) {
  double R = sqrt(x * x + y * y + z * z);
#if FMMGEN_SOURCEORDER == 0
  double r3 = 1.0 / (R * R * R);
  double phi = S[0] / R, ex = S[0] * x * r3, ey = S[0] * y * r3, ez = S[0] * z * r3;
#elif FMMGEN_SOURCEORDER == 1
  double rinv = 1.0 / R, r3 = rinv * rinv * rinv, r5 = r3 * rinv * rinv;
  double sr = S[0] * x + S[1] * y + S[2] * z;
  double phi = -sr * r3;
  double ex = S[0] * r3 - 3.0 * sr * x * r5;
  double ey = S[1] * r3 - 3.0 * sr * y * r5;
  double ez = S[2] * r3 - 3.0 * sr * z * r5;
#else
  // quadrupole (source_order 2, S = the degree-2 M coefficients xx xy xz yy yz zz):
  // phi = sum_m S_m d^m (1/R), E_a = -sum_m S_m d^(m+e_a) (1/R), with
  // d_i d_j (1/R) = (3 r_i r_j - delta_ij R^2) / R^5 and
  // d_i d_j d_k (1/R) = -15 r_i r_j r_k / R^7 + 3 (delta_ij r_k + delta_ik r_j + delta_jk r_i) / R^5
  const double r[3] = {x, y, z};
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
  double rinv = 1.0 / R, r2 = R * R, r5 = rinv * rinv * rinv * rinv * rinv, r7 = r5 * rinv * rinv;
  double phi = 0, e[3] = {0, 0, 0};
  for (int m = 0; m < 6; m++) {
    const int i = pi[m], j = pj[m];
    phi += S[m] * (3.0 * r[i] * r[j] - (i == j ? r2 : 0.0)) * r5;
    for (int a = 0; a < 3; a++) {
      double d3 = -15.0 * r[i] * r[j] * r[a] * r7 +
                  3.0 * ((i == j ? r[a] : 0.0) + (i == a ? r[j] : 0.0) + (j == a ? r[i] : 0.0)) * r5;
      e[a] -= S[m] * d3;
    }
  }
  double ex = e[0], ey = e[1], ez = e[2];
#endif
#pragma omp atomic
  F[0] += phi;
#pragma omp atomic
  F[1] += ex;
#pragma omp atomic
  F[2] += ey;
#pragma omp atomic
  F[3] += ez;
}

namespace {
struct Handle {
  Tree tree;
  std::vector<uint64_t> id;
};

void canonical_ids(Handle *h) {
  auto &cells = h->tree.cells;
  h->id.assign(cells.size(), 1);
  // cells are in creation order, so a parent precedes its children
  for (size_t c = 1; c < cells.size(); c++) {
    size_t p = cells[c].parent;
    int oct = -1;
    for (int o = 0; o < 8; o++)
      if ((cells[p].nchild & (1u << o)) && cells[p].child[o] == c) oct = o;
    h->id[c] = (h->id[p] << 3) | (uint64_t)oct;
  }
}
}  // namespace

extern "C" {

int ref_sourceorder() { return FMMGEN_SOURCEORDER; }
int ref_minorder() { return FMMGEN_MINORDER; }
int ref_maxorder() { return FMMGEN_MAXORDER; }

void *ref_build(double *pos, double *S, size_t N, size_t ncrit, size_t order, double theta,
                double *seconds) {
  auto t0 = std::chrono::steady_clock::now();
  Handle *h = new Handle();
  h->tree = build_tree(pos, S, N, ncrit, order, theta);
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  canonical_ids(h);
  return h;
}

void ref_free(void *p) { delete static_cast<Handle *>(p); }

// [ncells, nleaves, nm2l, np2p]
void ref_info(void *p, long *out) {
  Handle *h = static_cast<Handle *>(p);
  long nl = 0;
  for (auto &c : h->tree.cells) nl += (c.nleaf < h->tree.ncrit);
  out[0] = h->tree.cells.size();
  out[1] = nl;
  out[2] = h->tree.M2L_list.size();
  out[3] = h->tree.P2P_list.size();
}

void ref_export_cells(void *p, uint64_t *cell_id, long *cell_nleaf, double *centre, long *level,
                      long *leaf_off, long *leaf_idx) {
  Handle *h = static_cast<Handle *>(p);
  auto &cells = h->tree.cells;
  long k = 0, o = 0;
  for (size_t c = 0; c < cells.size(); c++) {
    cell_id[c] = h->id[c];
    cell_nleaf[c] = cells[c].nleaf;
    level[c] = cells[c].level;
    centre[3 * c] = cells[c].x;
    centre[3 * c + 1] = cells[c].y;
    centre[3 * c + 2] = cells[c].z;
    if (cells[c].nleaf < h->tree.ncrit) {
      leaf_off[k++] = o;
      for (size_t i = 0; i < cells[c].nleaf; i++) leaf_idx[o++] = cells[c].leaf[i];
    }
  }
  leaf_off[k] = o;
}

// m2l as (source, target), p2p as (target, source), canonical ids
void ref_export_lists(void *p, uint64_t *m2l, uint64_t *p2p) {
  Handle *h = static_cast<Handle *>(p);
  size_t i = 0;
  for (auto &pr : h->tree.M2L_list) {
    m2l[2 * i] = h->id[pr.first];
    m2l[2 * i + 1] = h->id[pr.second];
    i++;
  }
  i = 0;
  for (auto &pr : h->tree.P2P_list) {
    p2p[2 * i] = h->id[pr.first];
    p2p[2 * i + 1] = h->id[pr.second];
    i++;
  }
}

// Tree::compute_field_fmm; returns seconds (the region example/main.cpp:154-162 times)
double ref_evaluate(void *p, double *F) {
  Handle *h = static_cast<Handle *>(p);
  auto t0 = std::chrono::steady_clock::now();
  h->tree.compute_field_fmm(F);
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// Tree::compute_field_bh (example/tree.cpp:273-293): the generated M2P's
// potential is right, its field is not the gradient of that potential (the
// generator defect the P2P restatement works around), so only the potential
// of this pass is a pin.
double ref_evaluate_bh(void *p, double *F) {
  Handle *h = static_cast<Handle *>(p);
  auto t0 = std::chrono::steady_clock::now();
  h->tree.compute_field_bh(F);
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

void ref_cell_M(void *p, double *out) {
  Handle *h = static_cast<Handle *>(p);
  memcpy(out, h->tree.M.data(), sizeof(double) * h->tree.M.size());
}
void ref_cell_L(void *p, double *out) {
  Handle *h = static_cast<Handle *>(p);
  memcpy(out, h->tree.L.data(), sizeof(double) * h->tree.L.size());
}

// The generated operator dispatchers (switch over order), unchanged.
void ref_P2M(double x, double y, double z, double q, double *M, int order) { P2M(x, y, z, q, M, order); }
void ref_M2M(double x, double y, double z, double *M, double *Ms, int order) { M2M(x, y, z, M, Ms, order); }
void ref_M2L(double x, double y, double z, double *M, double *L, int order) { M2L(x, y, z, M, L, order); }
void ref_L2L(double x, double y, double z, double *L, double *Ls, int order) { L2L(x, y, z, L, Ls, order); }
void ref_L2P(double x, double y, double z, double *L, double *F, int order) { L2P(x, y, z, L, F, order); }
void ref_M2P(double x, double y, double z, double *M, double *F, int order) { M2P(x, y, z, M, F, order); }
void ref_P2P_generated(double x, double y, double z, double *S, double *F) {
  fmmgen_generated_P2P(x, y, z, S, F);
}
void ref_P2P_restated(double x, double y, double z, double *S, double *F) { P2P(x, y, z, S, F); }

}  // extern "C"
