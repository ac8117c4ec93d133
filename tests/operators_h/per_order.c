/* C caller of include/operators.h: configures the library from the macros with
 * FMMGEN_CONFIGURE() (C has no static initialisers), then applies each
 * per-order function OP_3 and the dispatcher OP(..., 3) to the same inputs and
 * prints the largest difference between their outputs, and the value of every
 * FMMGEN_* macro.  Output line: "<MINORDER> <MAXORDER> <SOURCEORDER>
 * <SOURCESIZE> <OUTPUTSIZE> <max |difference|> <max |output|>". */
#include <math.h>
#include <stdio.h>

#include "operators.h"

#define NT(p) (((p) + 1) * ((p) + 2) * ((p) + 3) / 6)
#define P 3
#define MS (NT(P) - NT(FMMGEN_SOURCEORDER - 1))
#define LS (NT(P - FMMGEN_SOURCEORDER))

static double maxdiff(const double *a, const double *b, int n, double *amax) {
  double m = 0.0;
  for (int i = 0; i < n; ++i) {
    if (fabs(a[i] - b[i]) > m) m = fabs(a[i] - b[i]);
    if (fabs(a[i]) > *amax) *amax = fabs(a[i]);
  }
  return m;
}

int main(void) {
  if (FMMGEN_CONFIGURE() != 0) return 1;
  double M[MS], L[LS], a[NT(P) + 4], b[NT(P) + 4], d = 0.0, amax = 0.0;
  for (int i = 0; i < MS; ++i) M[i] = 0.3 + 0.1 * i - 0.01 * i * i;
  for (int i = 0; i < LS; ++i) L[i] = -0.2 + 0.07 * i;
  const double x = 0.31, y = -0.17, z = 0.23, X = 2.1, Y = -1.3, Z = 0.9;
#define PAIR(call3, calld, n)                        \
  for (int i = 0; i < (n); ++i) a[i] = b[i] = 0.5; \
  call3;                                             \
  calld;                                             \
  if (maxdiff(a, b, (n), &amax) > d) d = maxdiff(a, b, (n), &amax);
  PAIR(P2M_3(x, y, z, 0.7, a), P2M(x, y, z, 0.7, b, P), MS)
  PAIR(M2M_3(x, y, z, M, a), M2M(x, y, z, M, b, P), MS)
  PAIR(M2L_3(X, Y, Z, M, a), M2L(X, Y, Z, M, b, P), LS)
  PAIR(L2L_3(x, y, z, L, a), L2L(x, y, z, L, b, P), LS)
  PAIR(L2P_3(x, y, z, L, a), L2P(x, y, z, L, b, P), FMMGEN_OUTPUTSIZE)
  PAIR(M2P_3(X, Y, Z, M, a), M2P(X, Y, Z, M, b, P), FMMGEN_OUTPUTSIZE)
  printf("%d %d %d %d %d %.17g %.17g\n", FMMGEN_MINORDER, FMMGEN_MAXORDER, FMMGEN_SOURCEORDER, FMMGEN_SOURCESIZE,
         FMMGEN_OUTPUTSIZE, d, amax);
  return 0;
}
