/*
 * operators.h -- drop-in for the operators.h that fmmgen.generate_code writes
 * (fmmgen/writer.py:266-330; example instance example/operators.cpp:1376-1489),
 * served by libfmmgen_gb300.so.
 *
 * A caller written against the generated header (the reference's
 * example/calculate.cpp, tree.cpp and main.cpp include "operators.h") compiles
 * unchanged against this one and links -lfmmgen_gb300.  What the generator
 * fixes when it writes the code is chosen here by macros, which a build may
 * set with -D (defaults in brackets):
 *   FMMGEN_SOURCEORDER  source order: 0 charges, 1 dipoles, 2 quadrupoles [0]
 *   FMMGEN_POTENTIAL    1 if the outputs hold the potential [1]
 *   FMMGEN_FIELD        1 if the outputs hold the field [1]
 *   FMMGEN_MAXORDER     one above the highest order, as the generator's
 *                       `order` argument (exclusive) [13]
 * and, derived from them as the generator derives them (fmmgen/writer.py:121-140,
 * 317-328): FMMGEN_MINORDER = source order + field, FMMGEN_SOURCESIZE,
 * FMMGEN_OUTPUTSIZE (1, 3 or 4).
 *
 * The generated code has these choices built in; this library holds them at
 * run time (fmmgen_configure).  In C++ this header configures the library with
 * its macros during static initialisation of every translation unit that
 * includes it; a C caller calls FMMGEN_CONFIGURE() once before the first
 * operator.
 *
 * Operators (all "+=", as generated):
 *   P2M, M2M, M2L, L2L, L2P, M2P (..., int order): the generated dispatchers;
 *     an order outside [FMMGEN_MINORDER, FMMGEN_MAXORDER) is a silent no-op;
 *   P2M_p ... M2P_p (p = 0..12): the generated per-order functions (the
 *     generator emits p in [FMMGEN_MINORDER, FMMGEN_MAXORDER); this library
 *     exports every p up to 12, and one below FMMGEN_MINORDER is a no-op);
 *   P2P (no order).
 * Every call copies its host arrays to the GPU, runs one kernel and copies the
 * outputs back before it returns (a few tens of microseconds): it reproduces
 * the generated operators' results and calling convention, not their speed.
 * Callers that apply many operators should hand whole trees or batches to the
 * device entry points of fmmgen_gb300.h.
 */
#pragma once
#include "fmmgen_gb300.h"

#ifndef FMMGEN_SOURCEORDER
#define FMMGEN_SOURCEORDER 0
#endif
#ifndef FMMGEN_POTENTIAL
#define FMMGEN_POTENTIAL 1
#endif
#ifndef FMMGEN_FIELD
#define FMMGEN_FIELD 1
#endif
#ifndef FMMGEN_MAXORDER
#define FMMGEN_MAXORDER 13
#endif
#define FMMGEN_MINORDER (FMMGEN_SOURCEORDER + ((FMMGEN_FIELD) ? 1 : 0))
#define FMMGEN_SOURCESIZE (((FMMGEN_SOURCEORDER) + 1) * ((FMMGEN_SOURCEORDER) + 2) / 2)
#define FMMGEN_OUTPUTSIZE (((FMMGEN_POTENTIAL) && (FMMGEN_FIELD)) ? 4 : ((FMMGEN_FIELD) ? 3 : 1))

#if FMMGEN_MAXORDER > 13 || FMMGEN_MAXORDER <= FMMGEN_MINORDER
#error "FMMGEN_MAXORDER must lie in (FMMGEN_MINORDER, 13]"
#endif

/* library configuration from the macros (the dispatchers' highest order is
 * FMMGEN_MAXORDER - 1: the generator's bound is exclusive) */
#define FMMGEN_CONFIGURE() \
  fmmgen_configure(FMMGEN_SOURCEORDER, FMMGEN_POTENTIAL, FMMGEN_FIELD, FMMGEN_MAXORDER - 1)

#ifdef __cplusplus
extern "C" {
#endif

#define FMMGEN_DECLARE_ORDER(p)                                                    \
  void P2M_##p(double x, double y, double z, double q, double *M);                \
  void M2M_##p(double x, double y, double z, double *M, double *Ms);              \
  void M2L_##p(double x, double y, double z, double *M, double *L);               \
  void L2L_##p(double x, double y, double z, double *L, double *Ls);              \
  void L2P_##p(double x, double y, double z, double *L, double *F);               \
  void M2P_##p(double x, double y, double z, double *M, double *F);
FMMGEN_DECLARE_ORDER(0)
FMMGEN_DECLARE_ORDER(1)
FMMGEN_DECLARE_ORDER(2)
FMMGEN_DECLARE_ORDER(3)
FMMGEN_DECLARE_ORDER(4)
FMMGEN_DECLARE_ORDER(5)
FMMGEN_DECLARE_ORDER(6)
FMMGEN_DECLARE_ORDER(7)
FMMGEN_DECLARE_ORDER(8)
FMMGEN_DECLARE_ORDER(9)
FMMGEN_DECLARE_ORDER(10)
FMMGEN_DECLARE_ORDER(11)
FMMGEN_DECLARE_ORDER(12)
#undef FMMGEN_DECLARE_ORDER

#ifdef __cplusplus
}  /* extern "C" */

namespace {
/* configures the library from this header's macros before main() runs */
struct fmmgen_operators_h_config {
  fmmgen_operators_h_config() { FMMGEN_CONFIGURE(); }
};
static const fmmgen_operators_h_config fmmgen_operators_h_config_instance{};
}  // namespace
#endif
