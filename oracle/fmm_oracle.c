/*
 * fmm_oracle.c -- CPU FP64 restatement of rpep/fmmgen's octree FMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the pytest suite,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it to compare
 * against / time beside the CUDA library.  Nothing in the product library
 * (fmmgen_gb300/) links, loads or calls it.
 *
 * What it restates (all FP64, compiled with -ffp-contract=off so every
 * expression rounds exactly as written):
 *   - the multi-index layout        fmmgen/utils.py:26-35, 65-118; example/utils.cpp:3-27
 *   - the operator mathematics      fmmgen/expansions.py:22-207 (M, M_shift, Phi_derivatives,
 *                                   L, L_shift, phi_deriv) as emitted by fmmgen/generator.py
 *   - P2P (physics restated, the generated field is zero at HEAD)   example/operators.cpp:54-66
 *   - the adaptive octree build     example/tree.cpp:10-21, 91-233
 *   - the dual-tree interaction walk example/calculate.cpp:81-133
 *   - the evaluation sweeps         example/tree.cpp:243-271, example/calculate.cpp:135-250
 *   - the O(N^2) direct sum         example/calculate.cpp:252-264
 *
 * Parity pin: tests compare this file against the reference itself (fmmgen's
 * generated operators and the example tree code compiled by oracle/ref) via
 * the golden vectors under tests/golden/.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PMAX 16
#define OR_MAXLEVEL 21

/* ------------------------------------------------------------------ */
/* multi-index layout (fmmgen/utils.py:26-35, 65-118)                  */
/* ------------------------------------------------------------------ */

/* Nterms(p): number of monomials of total degree <= p (fmmgen/utils.py:26-35). */
long or_nterms(int p) { return p < 0 ? 0 : (long)(p + 1) * (p + 2) * (p + 3) / 6; }

/* Msize/Lsize (example/utils.cpp:18-27). */
long or_msize(int order, int so) { return or_nterms(order) - or_nterms(so - 1); }
long or_lsize(int order, int so) { return or_nterms(order - so); }
/* source components: the degree-so M coefficients (1 charge, 3 dipole, 6 quadrupole) */
long or_sourcesize(int so) { return or_nterms(so) - or_nterms(so - 1); }

/* Flat index of (nx,ny,nz) in the full layout: ordered by total degree, then
 * nx descending, then ny descending (grevlex on [z,y,x], fmmgen/utils.py:103-109). */
static inline int idx3(int nx, int ny, int nz) {
    int d = nx + ny + nz, j = d - nx;
    return (int)or_nterms(d - 1) + j * (j + 1) / 2 + (j - ny);
}

long or_index(int nx, int ny, int nz) { return idx3(nx, ny, nz); }

typedef struct { unsigned char x, y, z, d; } mi_t;
static mi_t g_mi[1140]; /* Nterms(16) = 969 */
static int g_mi_ready = 0;
static void mi_init(void) {
    if (g_mi_ready) return;
    for (int d = 0; d <= OR_PMAX; d++)
        for (int nx = d; nx >= 0; nx--)
            for (int ny = d - nx; ny >= 0; ny--) {
                int nz = d - nx - ny;
                mi_t m = {(unsigned char)nx, (unsigned char)ny, (unsigned char)nz, (unsigned char)d};
                g_mi[idx3(nx, ny, nz)] = m;
            }
    g_mi_ready = 1;
}

static const double g_invfact[OR_PMAX + 1] = {
    1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040, 1.0 / 40320,
    1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800, 1.0 / 479001600, 1.0 / 6227020800.0,
    1.0 / 87178291200.0, 1.0 / 1307674368000.0, 1.0 / 20922789888000.0};

/* t[k] = v^k / k! for k = 0..p */
static void pow_table(double v, int p, double *t) {
    t[0] = 1.0;
    for (int k = 1; k <= p; k++) t[k] = t[k - 1] * v / (double)k;
}

/* ------------------------------------------------------------------ */
/* derivatives of 1/R (fmmgen/expansions.py:108-141)                   */
/* ------------------------------------------------------------------ */
/* D[idx(n)] = d^n (1/R) at (x,y,z) for |n| <= p, via the Hermite-type
 * recurrence  R^{(m)}_{n+e} = x_e R^{(m+1)}_n + n_e R^{(m+1)}_{n-e},
 * R^{(m)}_0 = (-1)^m (2m-1)!! / R^{2m+1}; D_n = R^{(0)}_n.  Same function
 * fmmgen differentiates symbolically; only the evaluation order differs. */
void or_derivs(double x, double y, double z, int p, double *D) {
    mi_init();
    double r2 = x * x + y * y + z * z;
    double rinv = 1.0 / sqrt(r2), rinv2 = rinv * rinv;
    double base[OR_PMAX + 1];
    base[0] = rinv;
    for (int m = 1; m <= p; m++) base[m] = -(double)(2 * m - 1) * rinv2 * base[m - 1];
    double bufa[1140], bufb[1140];
    double *A = bufa, *B = bufb;
    A[0] = base[p];
    for (int m = p - 1; m >= 0; m--) {
        long cnt = or_nterms(p - m);
        for (long i = 0; i < cnt; i++) {
            mi_t n = g_mi[i];
            double v;
            if (n.d == 0) v = base[m];
            else if (n.x > 0) {
                v = x * A[idx3(n.x - 1, n.y, n.z)];
                if (n.x > 1) v += (double)(n.x - 1) * A[idx3(n.x - 2, n.y, n.z)];
            } else if (n.y > 0) {
                v = y * A[idx3(n.x, n.y - 1, n.z)];
                if (n.y > 1) v += (double)(n.y - 1) * A[idx3(n.x, n.y - 2, n.z)];
            } else {
                v = z * A[idx3(n.x, n.y, n.z - 1)];
                if (n.z > 1) v += (double)(n.z - 1) * A[idx3(n.x, n.y, n.z - 2)];
            }
            B[i] = v;
        }
        double *t = A; A = B; B = t;
    }
    memcpy(D, A, sizeof(double) * or_nterms(p));
}

/* ------------------------------------------------------------------ */
/* operators (generated ABI: fmmgen/writer.py:142-264, +=)             */
/* ------------------------------------------------------------------ */

/* P2M_p: M[n] += (-1)^|n| q x^n / n! over the M layout (fmmgen/expansions.py:22-39,
 * fmmgen/generator.py:9-43). */
void or_P2M(double x, double y, double z, double q, double *M, int order, int so) {
    mi_init();
    double px[OR_PMAX + 1], py[OR_PMAX + 1], pz[OR_PMAX + 1];
    pow_table(-x, order, px); pow_table(-y, order, py); pow_table(-z, order, pz);
    long off = or_nterms(so - 1), cnt = or_nterms(order);
    for (long i = off; i < cnt; i++) {
        mi_t n = g_mi[i];
        M[i - off] += q * px[n.x] * py[n.y] * pz[n.z];
    }
}

/* M2M_p: Ms[n] += sum_{k<=n, |n-k|>=so} M[n-k] x^k/k!  (fmmgen/expansions.py:42-78). */
void or_M2M(double x, double y, double z, const double *M, double *Ms, int order, int so) {
    mi_init();
    double px[OR_PMAX + 1], py[OR_PMAX + 1], pz[OR_PMAX + 1];
    pow_table(x, order, px); pow_table(y, order, py); pow_table(z, order, pz);
    long off = or_nterms(so - 1), cnt = or_nterms(order);
    for (long i = off; i < cnt; i++) {
        mi_t n = g_mi[i];
        double acc = 0.0;
        for (int kx = 0; kx <= n.x; kx++)
            for (int ky = 0; ky <= n.y; ky++)
                for (int kz = 0; kz <= n.z; kz++) {
                    int rd = n.d - kx - ky - kz;
                    if (rd < so) continue;
                    acc += M[idx3(n.x - kx, n.y - ky, n.z - kz) - off] * px[kx] * py[ky] * pz[kz];
                }
        Ms[i - off] += acc;
    }
}

/* M2L_p: D = d^k(1/R) at (x,y,z); L[n] += sum_{|m|>=so, |n|+|m|<=order} D_{n+m} M[m]
 * for |n| <= order-so  (fmmgen/expansions.py:144-172, fmmgen/generator.py:82-134). */
void or_M2L(double x, double y, double z, const double *M, double *L, int order, int so) {
    mi_init();
    double D[1140];
    or_derivs(x, y, z, order, D);
    long off = or_nterms(so - 1);
    long lcnt = or_nterms(order - so);
    for (long i = 0; i < lcnt; i++) {
        mi_t n = g_mi[i];
        long mcnt = or_nterms(order - n.d);
        double acc = 0.0;
        for (long j = off; j < mcnt; j++) {
            mi_t m = g_mi[j];
            acc += D[idx3(n.x + m.x, n.y + m.y, n.z + m.z)] * M[j - off];
        }
        L[i] += acc;
    }
}

/* L2L_p: Ls[n] += sum_{k: |n+k|<=order-so} L[n+k] x^k/k!  (fmmgen/expansions.py:175-194). */
void or_L2L(double x, double y, double z, const double *L, double *Ls, int order, int so) {
    mi_init();
    int pl = order - so;
    double px[OR_PMAX + 1], py[OR_PMAX + 1], pz[OR_PMAX + 1];
    pow_table(x, pl, px); pow_table(y, pl, py); pow_table(z, pl, pz);
    long lcnt = or_nterms(pl);
    for (long i = 0; i < lcnt; i++) {
        mi_t n = g_mi[i];
        long kcnt = or_nterms(pl - n.d);
        double acc = 0.0;
        for (long j = 0; j < kcnt; j++) {
            mi_t k = g_mi[j];
            acc += L[idx3(n.x + k.x, n.y + k.y, n.z + k.z)] * px[k.x] * py[k.y] * pz[k.z];
        }
        Ls[i] += acc;
    }
}

/* L2P_p: phi += sum_n L_n x^n/n!, E = -grad phi (fmmgen/expansions.py:197-207,
 * fmmgen/generator.py:209-254).  Output layout [phi][Ex Ey Ez] per the switches. */
void or_L2P(double x, double y, double z, const double *L, double *F, int order, int so,
            int potential, int field) {
    mi_init();
    int pl = order - so;
    double px[OR_PMAX + 1], py[OR_PMAX + 1], pz[OR_PMAX + 1];
    pow_table(x, pl, px); pow_table(y, pl, py); pow_table(z, pl, pz);
    long lcnt = or_nterms(pl);
    double phi = 0, ex = 0, ey = 0, ez = 0;
    for (long i = 0; i < lcnt; i++) {
        mi_t n = g_mi[i];
        double l = L[i];
        phi += l * px[n.x] * py[n.y] * pz[n.z];
        if (n.x) ex -= l * px[n.x - 1] * py[n.y] * pz[n.z];
        if (n.y) ey -= l * px[n.x] * py[n.y - 1] * pz[n.z];
        if (n.z) ez -= l * px[n.x] * py[n.y] * pz[n.z - 1];
    }
    int o = 0;
    if (potential) F[o++] += phi;
    if (field) { F[o] += ex; F[o + 1] += ey; F[o + 2] += ez; }
}

/* M2P_p: the Barnes-Hut far field of a multipole at (x,y,z) = particle - cell
 * (fmmgen/generator.py:174-206): phi = V = sum_{so<=|m|<=order} D_m M[m] (the
 * n = 0 output of M2L_p) and E = -grad V = -sum_m D_{m+e} M[m], the exact
 * gradient (derivatives to order + 1).  The generator's own field is not the
 * gradient of its potential (the same substitution defect as its P2P); this
 * is the physical field. */
void or_M2P(double x, double y, double z, const double *M, double *F, int order, int so, int potential,
            int field) {
    mi_init();
    double D[1140];
    or_derivs(x, y, z, order + 1, D);
    long off = or_nterms(so - 1), cnt = or_nterms(order);
    double phi = 0, ex = 0, ey = 0, ez = 0;
    for (long j = off; j < cnt; j++) {
        mi_t m = g_mi[j];
        double v = M[j - off];
        phi += D[j] * v;
        ex -= D[idx3(m.x + 1, m.y, m.z)] * v;
        ey -= D[idx3(m.x, m.y + 1, m.z)] * v;
        ez -= D[idx3(m.x, m.y, m.z + 1)] * v;
    }
    int o = 0;
    if (potential) F[o++] += phi;
    if (field) { F[o] += ex; F[o + 1] += ey; F[o + 2] += ez; }
}

/* P2P: Coulomb  phi += q/R, E += q r/R^3 (example/operators.cpp:54-66);
 * dipole (source_order=1, S = degree-1 M coefficients):
 *   phi += -S.r/R^3, E += S/R^3 - 3 (S.r) r / R^5  (fmmgen/generator.py:257-288 potential);
 * higher source orders (S = the degree-so M coefficients): the generator's
 * P2P potential V = L_0 of a multipole whose only terms are S
 * (fmmgen/generator.py:257-288), i.e. M2P at order so, with the exact field. */
void or_M2P(double x, double y, double z, const double *M, double *F, int order, int so, int potential,
            int field);
void or_P2P(double x, double y, double z, const double *S, double *F, int so, int potential,
            int field) {
    if (so >= 2) {
        or_M2P(x, y, z, S, F, so, so, potential, field);
        return;
    }
    double R = sqrt(x * x + y * y + z * z);
    double phi, ex, ey, ez;
    if (so == 0) {
        double q = S[0];
        double r3 = 1.0 / (R * R * R);
        phi = q / R;
        ex = q * x * r3; ey = q * y * r3; ez = q * z * r3;
    } else {
        double rinv = 1.0 / R;
        double r3 = rinv * rinv * rinv;
        double sr = S[0] * x + S[1] * y + S[2] * z;
        double r5 = r3 * rinv * rinv;
        phi = -sr * r3;
        ex = S[0] * r3 - 3.0 * sr * x * r5;
        ey = S[1] * r3 - 3.0 * sr * y * r5;
        ez = S[2] * r3 - 3.0 * sr * z * r5;
    }
    int o = 0;
    if (potential) F[o++] += phi;
    if (field) { F[o] += ex; F[o + 1] += ey; F[o + 2] += ez; }
}

/* ------------------------------------------------------------------ */
/* adaptive octree (example/tree.cpp:10-21, 91-233)                     */
/* ------------------------------------------------------------------ */
typedef struct {
    double x, y, z, r, rmax;
    long parent;
    int level;
    unsigned nchild;        /* occupied-octant bitmask */
    long nleaf;             /* particles that entered the cell */
    long child[8];
    long *leaf;             /* capacity ncrit, ascending particle index */
    uint64_t id;            /* canonical id: (1 << 3*level) | octant path */
} ocell_t;

typedef struct {
    long N, ncrit;
    int order, so, err;
    double theta;
    const double *pos, *S;
    ocell_t *cells;
    long ncells, cap;
    long *leafbuf;
    long *m2l; long nm2l, capm2l;   /* pairs (B=source, A=target) */
    long *p2p; long np2p, capp2p;   /* pairs (A=target, B=source) */
    int maxlevel;
    unsigned char *m2l_ord;         /* per M2L pair (list order): its order, or NULL for `order` */
} otree_t;

static long add_cell(otree_t *t, double x, double y, double z, double r, long parent, int level) {
    if (t->ncells == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 1024;
        t->cells = (ocell_t *)realloc(t->cells, sizeof(ocell_t) * t->cap);
    }
    ocell_t *c = &t->cells[t->ncells];
    c->x = x; c->y = y; c->z = z; c->r = r;
    c->rmax = sqrt(3 * r * r);           /* example/tree.cpp:15 */
    c->parent = parent; c->level = level;
    c->nchild = 0; c->nleaf = 0;
    for (int o = 0; o < 8; o++) c->child[o] = 0;
    c->leaf = (long *)malloc(sizeof(long) * t->ncrit);
    c->id = 1;
    if (level > t->maxlevel) t->maxlevel = level;
    return t->ncells++;
}

/* add_child (example/tree.cpp:91-105): child centre = parent +- r/2 per axis. */
static long add_child(otree_t *t, int octant, long p) {
    if (t->cells[p].level + 1 > OR_MAXLEVEL) { t->err = 2; return -1; }
    double r = t->cells[p].r / 2.0;
    double x = t->cells[p].x + r * ((octant & 1) * 2 - 1);
    double y = t->cells[p].y + r * ((octant & 2) - 1);
    double z = t->cells[p].z + r * ((octant & 4) / 2 - 1);
    long c = add_cell(t, x, y, z, r, p, t->cells[p].level + 1);
    t->cells[c].id = (t->cells[p].id << 3) | (uint64_t)octant;
    t->cells[p].child[octant] = c;
    t->cells[p].nchild |= (1u << octant);
    return c;
}

static inline int octant_of(const otree_t *t, long i, long c) {
    const double *r = &t->pos[3 * i];
    const ocell_t *cc = &t->cells[c];
    return (r[0] > cc->x) + ((r[1] > cc->y) << 1) + ((r[2] > cc->z) << 2);
}

/* split_cell (example/tree.cpp:107-128). */
static void split_cell(otree_t *t, long p) {
    for (long i = 0; i < t->ncrit && !t->err; i++) {
        long l = t->cells[p].leaf[i];
        int oct = octant_of(t, l, p);
        if (!(t->cells[p].nchild & (1u << oct))) {
            if (add_child(t, oct, p) < 0) return;
        }
        long c = t->cells[p].child[oct];
        t->cells[c].leaf[t->cells[c].nleaf] = l;
        t->cells[c].nleaf += 1;
        if (t->cells[c].nleaf >= t->ncrit) split_cell(t, c);
    }
}

static void push_pair(long **arr, long *n, long *cap, long a, long b) {
    if (*n == *cap) {
        *cap = *cap ? 2 * *cap : 4096;
        *arr = (long *)realloc(*arr, sizeof(long) * 2 * *cap);
    }
    (*arr)[2 * *n] = a; (*arr)[2 * *n + 1] = b;
    (*n)++;
}

/* interact_dehnen_lazy (example/calculate.cpp:81-133). */
static void interact(otree_t *t, long A, long B) {
    const ocell_t *a = &t->cells[A], *b = &t->cells[B];
    double dx = a->x - b->x, dy = a->y - b->y, dz = a->z - b->z;
    double R = sqrt(dx * dx + dy * dy + dz * dz);
    if (R * t->theta > (a->rmax + b->rmax)) {
        push_pair(&t->m2l, &t->nm2l, &t->capm2l, B, A);
    } else if (a->nchild == 0 && b->nchild == 0) {
        if (b->nleaf >= t->ncrit) push_pair(&t->m2l, &t->nm2l, &t->capm2l, B, A); /* unreachable */
        else push_pair(&t->p2p, &t->np2p, &t->capp2p, A, B);
    } else if (b->nchild == 0 || (a->rmax >= b->rmax && a->nchild != 0)) {
        for (int oa = 0; oa < 8; oa++)
            if (t->cells[A].nchild & (1u << oa)) interact(t, t->cells[A].child[oa], B);
    } else {
        for (int ob = 0; ob < 8; ob++)
            if (t->cells[B].nchild & (1u << ob)) interact(t, A, t->cells[B].child[ob]);
    }
}

/* build_tree (example/tree.cpp:130-233).  Returns NULL on error (*err set):
 * 1 = bad arguments, 2 = tree deeper than OR_MAXLEVEL (coincident points). */
void *or_tree_build(const double *pos, const double *S, long N, long ncrit, int order,
                    double theta, int so, int *err) {
    *err = 0;
    if (N <= 0 || ncrit < 1 || order < 0 || order > OR_PMAX || so < 0 || so > 2) { *err = 1; return NULL; }
    otree_t *t = (otree_t *)calloc(1, sizeof(otree_t));
    t->N = N; t->ncrit = ncrit; t->order = order; t->so = so; t->theta = theta;
    t->pos = pos; t->S = S;
    double xavg = 0, yavg = 0, zavg = 0;
    for (long i = 0; i < N; i++) { xavg += pos[3 * i]; yavg += pos[3 * i + 1]; zavg += pos[3 * i + 2]; }
    xavg /= (double)N; yavg /= (double)N; zavg /= (double)N;
    double xmax = 0, ymax = 0, zmax = 0;
    for (long i = 0; i < N; i++) {
        double x = fabs(pos[3 * i] - xavg), y = fabs(pos[3 * i + 1] - yavg), z = fabs(pos[3 * i + 2] - zavg);
        if (x > xmax) xmax = x;
        if (y > ymax) ymax = y;
        if (z > zmax) zmax = z;
    }
    double r = (xmax > ymax ? (xmax > zmax ? xmax : zmax) : (ymax > zmax ? ymax : zmax)) * 1.001;
    add_cell(t, xavg, yavg, zavg, r, 0, 0);
    for (long i = 0; i < N && !t->err; i++) {
        long curr = 0;
        while (t->cells[curr].nleaf >= ncrit) {
            t->cells[curr].nleaf += 1;
            int oct = octant_of(t, i, curr);
            if (!(t->cells[curr].nchild & (1u << oct))) {
                if (add_child(t, oct, curr) < 0) break;
            }
            curr = t->cells[curr].child[oct];
        }
        if (t->err) break;
        t->cells[curr].leaf[t->cells[curr].nleaf] = i;
        t->cells[curr].nleaf += 1;
        if (t->cells[curr].nleaf >= ncrit) split_cell(t, curr);
    }
    if (t->err) { *err = t->err; return t; }
    interact(t, 0, 0);
    return t;
}

void or_tree_free(void *h) {
    otree_t *t = (otree_t *)h;
    if (!t) return;
    for (long c = 0; c < t->ncells; c++) free(t->cells[c].leaf);
    free(t->cells); free(t->m2l); free(t->p2p); free(t->m2l_ord); free(t);
}

/* Per-pair M2L orders for the following evaluations (list order of
 * or_tree_export_lists), clamped to [so + 1, order]; NULL: one order.  Pair
 * k at order q applies fmmgen's order-q M2L operator, i.e. the terms
 * |n| + |m| <= q of the order-`order` translation (the leading blocks of the
 * degree-major M and L rows).  No counterpart in the reference. */
void or_tree_set_m2l_orders(void *h, const unsigned char *orders) {
    otree_t *t = (otree_t *)h;
    free(t->m2l_ord);
    t->m2l_ord = NULL;
    if (!orders || t->nm2l == 0) return;
    t->m2l_ord = (unsigned char *)malloc((size_t)t->nm2l);
    for (long i = 0; i < t->nm2l; i++) {
        int q = orders[i];
        if (q < t->so + 1) q = t->so + 1;
        if (q > t->order) q = t->order;
        t->m2l_ord[i] = (unsigned char)q;
    }
}

/* counts: [ncells, nleaves, nm2l, np2p, maxlevel] */
void or_tree_info(void *h, long *out) {
    otree_t *t = (otree_t *)h;
    long nl = 0;
    for (long c = 0; c < t->ncells; c++) if (t->cells[c].nleaf < t->ncrit) nl++;
    out[0] = t->ncells; out[1] = nl; out[2] = t->nm2l; out[3] = t->np2p; out[4] = t->maxlevel;
}

/* cell_id[c], cell_nleaf[c], centre[3c..], level[c]; leaf particle lists in
 * CSR (leaf_off[nleaves+1], leaf_idx[...]) in cell creation order. */
void or_tree_export_cells(void *h, uint64_t *cell_id, long *cell_nleaf, double *centre,
                          long *level, long *leaf_cell, long *leaf_off, long *leaf_idx) {
    otree_t *t = (otree_t *)h;
    long k = 0, o = 0;
    for (long c = 0; c < t->ncells; c++) {
        const ocell_t *cc = &t->cells[c];
        cell_id[c] = cc->id; cell_nleaf[c] = cc->nleaf; level[c] = cc->level;
        centre[3 * c] = cc->x; centre[3 * c + 1] = cc->y; centre[3 * c + 2] = cc->z;
        if (cc->nleaf < t->ncrit) {
            leaf_cell[k] = c; leaf_off[k] = o;
            for (long i = 0; i < cc->nleaf; i++) leaf_idx[o++] = cc->leaf[i];
            k++;
        }
    }
    leaf_off[k] = o;
}

/* Interaction lists as canonical-id pairs: m2l as (source, target), p2p as (target, source). */
void or_tree_export_lists(void *h, uint64_t *m2l, uint64_t *p2p) {
    otree_t *t = (otree_t *)h;
    for (long i = 0; i < t->nm2l; i++) {
        m2l[2 * i] = t->cells[t->m2l[2 * i]].id; m2l[2 * i + 1] = t->cells[t->m2l[2 * i + 1]].id;
    }
    for (long i = 0; i < t->np2p; i++) {
        p2p[2 * i] = t->cells[t->p2p[2 * i]].id; p2p[2 * i + 1] = t->cells[t->p2p[2 * i + 1]].id;
    }
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* Group pair list by target into CSR (stable: keeps list order per target). */
static void csr_by_target(long npairs, const long *pairs, int tgt_slot, long ncells, long **off_out,
                          long **src_out, long **pair_out) {
    long *off = (long *)calloc(ncells + 1, sizeof(long));
    long *src = (long *)malloc(sizeof(long) * (npairs ? npairs : 1));
    for (long i = 0; i < npairs; i++) off[pairs[2 * i + tgt_slot] + 1]++;
    for (long c = 0; c < ncells; c++) off[c + 1] += off[c];
    long *fill = (long *)malloc(sizeof(long) * (ncells + 1));
    memcpy(fill, off, sizeof(long) * (ncells + 1));
    long *pidx = (long *)malloc(sizeof(long) * (npairs ? npairs : 1));
    for (long i = 0; i < npairs; i++) {
        long f = fill[pairs[2 * i + tgt_slot]]++;
        src[f] = pairs[2 * i + 1 - tgt_slot];
        pidx[f] = i;
    }
    free(fill);
    *off_out = off; *src_out = src;
    if (pair_out) *pair_out = pidx; else free(pidx);
}

/* P2M (as point-source M2M, example/calculate.cpp:135-161) and M2M, children
 * before parents (example/calculate.cpp:163-187), into M (zeroed, creation
 * order); returns the P2M seconds through *tp2m. */
static void or_tree_multipoles_t(otree_t *t, double *M, double *tp2m) {
    int order = t->order, so = t->so;
    int ssize = (int)or_sourcesize(so);
    long msize = or_msize(order, so);
    long nc = t->ncells, ncrit = t->ncrit;
    double t0 = now_s();
    /* P2M as point-source M2M (example/calculate.cpp:135-161) */
#pragma omp parallel for schedule(dynamic, 16)
    for (long c = 0; c < nc; c++) {
        const ocell_t *cc = &t->cells[c];
        if (cc->nleaf >= ncrit) continue;
        double Mt[1140];
        for (long i = 0; i < cc->nleaf; i++) {
            long l = cc->leaf[i];
            memset(Mt, 0, sizeof(double) * msize);
            for (int k = 0; k < ssize; k++) Mt[k] = t->S[ssize * l + k];
            or_M2M(cc->x - t->pos[3 * l], cc->y - t->pos[3 * l + 1], cc->z - t->pos[3 * l + 2], Mt,
                   &M[(size_t)c * msize], order, so);
        }
    }
    double t1 = now_s();
    if (tp2m) *tp2m = t1 - t0;
    /* M2M, children before parents (example/calculate.cpp:163-187) */
    for (long c = nc - 1; c > 0; c--) {
        long p = t->cells[c].parent;
        or_M2M(t->cells[p].x - t->cells[c].x, t->cells[p].y - t->cells[c].y,
               t->cells[p].z - t->cells[c].z, &M[(size_t)c * msize], &M[(size_t)p * msize], order, so);
    }
}

static void or_tree_multipoles(otree_t *t, double *M) { or_tree_multipoles_t(t, M, NULL); }

/* Tree::compute_field_fmm (example/tree.cpp:243-271).  F is [N][outsize] in the
 * caller's particle order, overwritten.  M/L buffers are returned through
 * Mout/Lout when non-NULL (cells x Msize / Lsize, creation order).
 * sample_stride > 1 restricts the M2L, P2P, L2L-consumer and L2P phases to every
 * sample_stride-th target cell (CPU-baseline sampling; fields incomplete);
 * 1 = the full pass; sample_stride < -1 evaluates the exact fields of the
 * particles of every |sample_stride|-th leaf cell: M2L into those leaves and
 * all their ancestors, P2P and L2P at those leaves (a target subset for
 * checking), other rows of F stay zero.
 * times: [P2M, M2M, M2L, P2P, L2L, L2P] seconds. */
int or_tree_evaluate(void *h, double *F, int potential, int field, long sample_stride,
                     double *Mout, double *Lout, double *times) {
    otree_t *t = (otree_t *)h;
    mi_init();
    int order = t->order, so = t->so;
    int outsize = (potential ? 1 : 0) + (field ? 3 : 0);
    int ssize = (int)or_sourcesize(so);
    long msize = or_msize(order, so), lsize = or_lsize(order, so);
    long nc = t->ncells, N = t->N, ncrit = t->ncrit;
    /* need[c]: M2L into c; leafsel[c]: P2P and L2P at c */
    unsigned char *need = (unsigned char *)malloc((size_t)nc), *leafsel = (unsigned char *)malloc((size_t)nc);
    if (sample_stride < -1) {
        long k = -sample_stride, nleaves = 0;
        memset(need, 0, (size_t)nc);
        memset(leafsel, 0, (size_t)nc);
        for (long c = 0; c < nc; c++) {
            if (t->cells[c].nleaf >= ncrit) continue;
            if (nleaves++ % k) continue;
            leafsel[c] = 1;
            for (long a = c; a >= 0 && !need[a]; a = t->cells[a].parent) need[a] = 1;
        }
    } else {
        if (sample_stride < 1) sample_stride = 1;
        for (long c = 0; c < nc; c++) need[c] = leafsel[c] = (unsigned char)(c % sample_stride == 0);
    }
    double *M = (double *)calloc((size_t)nc * msize, sizeof(double));
    double *L = (double *)calloc((size_t)nc * lsize, sizeof(double));
    memset(F, 0, sizeof(double) * N * outsize);
    double tt[6] = {0};
    double t0 = now_s();
    double tp2m = 0;
    or_tree_multipoles_t(t, M, &tp2m);
    double t1 = t0 + tp2m;
    double t2 = now_s();
    long *moff, *msrc, *mpair, *poff, *psrc;
    csr_by_target(t->nm2l, t->m2l, 1, nc, &moff, &msrc, &mpair);
    csr_by_target(t->np2p, t->p2p, 0, nc, &poff, &psrc, NULL);
    /* M2L (example/calculate.cpp:190-206), grouped by target instead of atomics */
#pragma omp parallel for schedule(dynamic, 8)
    for (long A = 0; A < nc; A++) {
        if (!need[A]) continue;
        for (long k = moff[A]; k < moff[A + 1]; k++) {
            long B = msrc[k];
            int q = t->m2l_ord ? t->m2l_ord[mpair[k]] : order;
            or_M2L(t->cells[A].x - t->cells[B].x, t->cells[A].y - t->cells[B].y,
                   t->cells[A].z - t->cells[B].z, &M[(size_t)B * msize], &L[(size_t)A * lsize], q, so);
        }
    }
    double t3 = now_s();
    /* P2P (example/calculate.cpp:24-40, 208-216) */
#pragma omp parallel for schedule(dynamic, 8)
    for (long A = 0; A < nc; A++) {
        if (!leafsel[A]) continue;
        const ocell_t *ca = &t->cells[A];
        for (long k = poff[A]; k < poff[A + 1]; k++) {
            const ocell_t *cb = &t->cells[psrc[k]];
            for (long p1 = 0; p1 < ca->nleaf; p1++) {
                long l1 = ca->leaf[p1];
                for (long p2 = 0; p2 < cb->nleaf; p2++) {
                    long l2 = cb->leaf[p2];
                    if (l2 == l1) continue;
                    or_P2P(t->pos[3 * l1] - t->pos[3 * l2], t->pos[3 * l1 + 1] - t->pos[3 * l2 + 1],
                           t->pos[3 * l1 + 2] - t->pos[3 * l2 + 2], &t->S[ssize * l2], &F[outsize * l1], so,
                           potential, field);
                }
            }
        }
    }
    double t4 = now_s();
    /* L2L, parents before children (example/calculate.cpp:219-234) */
    for (long p = 0; p < nc; p++) {
        for (int o = 0; o < 8; o++) {
            if (!(t->cells[p].nchild & (1u << o))) continue;
            long c = t->cells[p].child[o];
            or_L2L(t->cells[c].x - t->cells[p].x, t->cells[c].y - t->cells[p].y,
                   t->cells[c].z - t->cells[p].z, &L[(size_t)p * lsize], &L[(size_t)c * lsize], order, so);
        }
    }
    double t5 = now_s();
    /* L2P (example/calculate.cpp:236-250) */
#pragma omp parallel for schedule(dynamic, 16)
    for (long c = 0; c < nc; c++) {
        if (!leafsel[c]) continue;
        const ocell_t *cc = &t->cells[c];
        if (cc->nleaf >= ncrit) continue;
        for (long i = 0; i < cc->nleaf; i++) {
            long k = cc->leaf[i];
            or_L2P(t->pos[3 * k] - cc->x, t->pos[3 * k + 1] - cc->y, t->pos[3 * k + 2] - cc->z,
                   &L[(size_t)c * lsize], &F[outsize * k], order, so, potential, field);
        }
    }
    double t6 = now_s();
    tt[0] = t1 - t0; tt[1] = t2 - t1; tt[2] = t3 - t2; tt[3] = t4 - t3; tt[4] = t5 - t4; tt[5] = t6 - t5;
    if (times) memcpy(times, tt, sizeof(tt));
    if (Mout) memcpy(Mout, M, sizeof(double) * nc * msize);
    if (Lout) memcpy(Lout, L, sizeof(double) * nc * lsize);
    free(M); free(L); free(moff); free(msrc); free(mpair); free(poff); free(psrc); free(need); free(leafsel);
    return 0;
}

/* evaluate_M2P_and_P2P (example/calculate.cpp:266-314) for particle i from
 * cell p: a child c of a non-leaf cell is opened when r_c > theta |x_i - c_c|,
 * else its multipole acts through M2P; a leaf's particles act through P2P. */
static void bh_walk(const otree_t *t, const double *M, long p, long i, double *F, int outsize, int potential,
                    int field) {
    const ocell_t *cp = &t->cells[p];
    long msize = or_msize(t->order, t->so);
    int ssize = (int)or_sourcesize(t->so);
    if (cp->nleaf >= t->ncrit) {
        for (int o = 0; o < 8; o++) {
            if (!(cp->nchild & (1u << o))) continue;
            long c = cp->child[o];
            const ocell_t *cc = &t->cells[c];
            double dx = t->pos[3 * i] - cc->x, dy = t->pos[3 * i + 1] - cc->y, dz = t->pos[3 * i + 2] - cc->z;
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (cc->r > t->theta * r)
                bh_walk(t, M, c, i, F, outsize, potential, field);
            else
                or_M2P(dx, dy, dz, &M[(size_t)c * msize], &F[outsize * i], t->order, t->so, potential, field);
        }
    } else {
        for (long l = 0; l < cp->nleaf; l++) {
            long j = cp->leaf[l];
            if (j == i) continue;
            or_P2P(t->pos[3 * i] - t->pos[3 * j], t->pos[3 * i + 1] - t->pos[3 * j + 1],
                   t->pos[3 * i + 2] - t->pos[3 * j + 2], &t->S[ssize * j], &F[outsize * i], t->so, potential,
                   field);
        }
    }
}

/* Tree::compute_field_bh (example/tree.cpp:273-293) with the physical M2P field. */
void or_tree_evaluate_bh(void *h, double *F, int potential, int field) {
    otree_t *t = (otree_t *)h;
    mi_init();
    int outsize = (potential ? 1 : 0) + (field ? 3 : 0);
    long msize = or_msize(t->order, t->so), nc = t->ncells;
    double *M = (double *)calloc((size_t)nc * msize, sizeof(double));
    memset(F, 0, sizeof(double) * t->N * outsize);
    or_tree_multipoles(t, M);
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < t->N; i++) bh_walk(t, M, 0, i, F, outsize, potential, field);
    free(M);
}

/* evaluate_direct (example/calculate.cpp:252-264) for a subset of targets:
 * F[t][outsize] for targets[t], all N sources, skipping i == j. */
void or_direct(const double *pos, const double *S, long N, const long *targets, long ntargets, int so,
               int potential, int field, double *F) {
    int outsize = (potential ? 1 : 0) + (field ? 3 : 0);
    int ssize = (int)or_sourcesize(so);
    memset(F, 0, sizeof(double) * ntargets * outsize);
#pragma omp parallel for schedule(dynamic, 4)
    for (long t = 0; t < ntargets; t++) {
        long i = targets[t];
        for (long j = 0; j < N; j++) {
            if (i == j) continue;
            or_P2P(pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1], pos[3 * i + 2] - pos[3 * j + 2],
                   &S[ssize * j], &F[outsize * t], so, potential, field);
        }
    }
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
