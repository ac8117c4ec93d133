// A caller of the generated-operator ABI, compiled against include/operators.h
// with the generator's choices given as -D macros (FMMGEN_SOURCEORDER,
// FMMGEN_MAXORDER) and linked against libfmmgen_gb300.so.
//
// It evaluates the FMM of a fixed tree entirely through the scalar operators,
// in the calling pattern of the reference example (example/calculate.cpp:24-40
// for P2P between two leaves, :135-161 P2M as an M2M of each particle's source
// vector, :163-187 M2M child -> parent, :190-206 M2L over the pair list,
// :219-234 L2L parent -> child, :236-250 L2P), with the FMMGEN_* macros
// sizing its arrays as there.  The test feeds it the reference's own tree and
// compares F with the reference's compute_field_fmm.
//
// usage: fmm_caller <input.bin> <output.bin>
//   input: int64 N, ncells, nleafcells, nm2l, np2p, order, source_order, 0;
//          double pos[N][3], S[N][FMMGEN_SOURCESIZE], centre[ncells][3];
//          int64 parent[ncells] (-1 for the root; parents precede children),
//          leafcell[nleafcells], leaf_off[nleafcells + 1], leaf_idx[leaf_off[nleafcells]],
//          m2l[nm2l][2] = (source, target), p2p[np2p][2] = (target, source)
//   output: double F[N][FMMGEN_OUTPUTSIZE]
#include <cstdint>
#include <cstdio>
#include <vector>

#include "operators.h"

namespace {
template <typename T> bool get(FILE *f, std::vector<T> &v, size_t n) {
  v.resize(n);
  return n == 0 || fread(v.data(), sizeof(T), n, f) == n;
}
size_t nterms(int p) { return p < 0 ? 0 : (size_t)(p + 1) * (p + 2) * (p + 3) / 6; }
}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  std::vector<int64_t> h;
  if (!get(f, h, 8)) return 4;
  const size_t N = h[0], ncells = h[1], nleafc = h[2], nm2l = h[3], np2p = h[4];
  const int order = (int)h[5];
  if (h[6] != FMMGEN_SOURCEORDER) return 5;
  std::vector<double> pos, S, centre;
  std::vector<int64_t> parent, leafcell, leaf_off, leaf_idx, m2l, p2p;
  bool ok = get(f, pos, 3 * N) && get(f, S, FMMGEN_SOURCESIZE * N) && get(f, centre, 3 * ncells) &&
            get(f, parent, ncells) && get(f, leafcell, nleafc) && get(f, leaf_off, nleafc + 1) &&
            get(f, leaf_idx, leaf_off.empty() ? 0 : (size_t)leaf_off.back()) && get(f, m2l, 2 * nm2l) &&
            get(f, p2p, 2 * np2p);
  fclose(f);
  if (!ok) return 6;

  // Msize / Lsize of example/utils.cpp (fmmgen/utils.py layout)
  const size_t msize = nterms(order) - nterms(FMMGEN_SOURCEORDER - 1);
  const size_t lsize = nterms(order - FMMGEN_SOURCEORDER);
  std::vector<double> M(ncells * msize, 0.0), L(ncells * lsize, 0.0), F(N * FMMGEN_OUTPUTSIZE, 0.0);
  std::vector<int64_t> leaf_of_cell(ncells, -1);
  for (size_t k = 0; k < nleafc; ++k) leaf_of_cell[leafcell[k]] = (int64_t)k;
  auto c3 = [&](int64_t c) { return &centre[3 * c]; };

  // P2M: each particle's source vector shifted into its leaf's multipole
  std::vector<double> Mp(msize);
  for (size_t k = 0; k < nleafc; ++k) {
    const double *cc = c3(leafcell[k]);
    for (int64_t j = leaf_off[k]; j < leaf_off[k + 1]; ++j) {
      const int64_t i = leaf_idx[j];
      for (size_t t = 0; t < msize; ++t) Mp[t] = t < (size_t)FMMGEN_SOURCESIZE ? S[FMMGEN_SOURCESIZE * i + t] : 0.0;
      M2M(cc[0] - pos[3 * i], cc[1] - pos[3 * i + 1], cc[2] - pos[3 * i + 2], Mp.data(), &M[leafcell[k] * msize],
          order);
    }
  }
  // M2M: children (later cells) into parents
  for (size_t c = ncells; c-- > 1;) {
    const int64_t p = parent[c];
    const double *pc = c3(p), *cc = c3(c);
    M2M(pc[0] - cc[0], pc[1] - cc[1], pc[2] - cc[2], &M[c * msize], &M[p * msize], order);
  }
  // M2L over the interaction list (source B, target A), d = A - B
  for (size_t k = 0; k < nm2l; ++k) {
    const int64_t B = m2l[2 * k], A = m2l[2 * k + 1];
    const double *a = c3(A), *b = c3(B);
    M2L(a[0] - b[0], a[1] - b[1], a[2] - b[2], &M[B * msize], &L[A * lsize], order);
  }
  // L2L: parents into children
  for (size_t c = 1; c < ncells; ++c) {
    const int64_t p = parent[c];
    const double *pc = c3(p), *cc = c3(c);
    L2L(cc[0] - pc[0], cc[1] - pc[1], cc[2] - pc[2], &L[p * lsize], &L[c * lsize], order);
  }
  // L2P at every leaf particle, d = particle - cell
  for (size_t k = 0; k < nleafc; ++k) {
    const double *cc = c3(leafcell[k]);
    for (int64_t j = leaf_off[k]; j < leaf_off[k + 1]; ++j) {
      const int64_t i = leaf_idx[j];
      L2P(pos[3 * i] - cc[0], pos[3 * i + 1] - cc[1], pos[3 * i + 2] - cc[2], &L[leafcell[k] * lsize],
          &F[FMMGEN_OUTPUTSIZE * i], order);
    }
  }
  // P2P between the particles of two leaves (target A, source B), skipping i == j
  for (size_t k = 0; k < np2p; ++k) {
    const int64_t A = leaf_of_cell[p2p[2 * k]], B = leaf_of_cell[p2p[2 * k + 1]];
    if (A < 0 || B < 0) return 7;
    for (int64_t ja = leaf_off[A]; ja < leaf_off[A + 1]; ++ja)
      for (int64_t jb = leaf_off[B]; jb < leaf_off[B + 1]; ++jb) {
        const int64_t i = leaf_idx[ja], s = leaf_idx[jb];
        if (i == s) continue;
        P2P(pos[3 * i] - pos[3 * s], pos[3 * i + 1] - pos[3 * s + 1], pos[3 * i + 2] - pos[3 * s + 2],
            &S[FMMGEN_SOURCESIZE * s], &F[FMMGEN_OUTPUTSIZE * i]);
      }
  }

  FILE *o = fopen(argv[2], "wb");
  if (!o) return 8;
  ok = fwrite(F.data(), sizeof(double), F.size(), o) == F.size();
  fclose(o);
  return ok ? 0 : 9;
}
