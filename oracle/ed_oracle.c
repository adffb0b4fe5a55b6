/*
 * ed_oracle.c -- CPU oracle for the exact-diagonalisation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C99, the algorithms
 * of PyHub's Fortran kernels (the .f90 files of pyhub/libs/src) so that the CUDA path in
 * pyhub_gb300/csrc can be checked against them.  Only tests/, the smoke() hook
 * of __graft_entry__.py and the CPU-baseline leg of bench.py may load this
 * library, and only as the checker or as the timed CPU baseline.  Nothing in
 * the pyhub_gb300 package links or calls it.
 *
 * Parity status: the reference cannot be executed in this build environment
 * (Fortran + HDF5, no Fortran compiler), so this restatement is NOT pinned by
 * reference outputs ("parity unpinned" by reference execution).  It is pinned
 * instead against an independent Jordan-Wigner Fock-space construction of the
 * same operators, the examples' cross-consistency relations and physics
 * identities (tests/test_oracle.py).
 *
 * Conventions restated from the reference:
 *   - a spin string is an integer whose bit (NORB-POS) holds site POS (1-based),
 *     i.e. site 1 is the most significant of the NORB bits (funcmod.f90:22-23);
 *   - the sector vector index is d*NSUP + u (0-based here; the reference's
 *     (D-1)*NSUP+U, hprod_hubbard.f90:31);
 *   - the hopping amplitude of a hop J->K is T(J,K) where T is the Fortran
 *     (column-major) view of the row-major t_matrix buffer, i.e. t[K][J]
 *     (the reference reads the h5py-written array column-major,
 *     compute_solver.f90:146-148);
 *   - Fortran REAL*4 literals (1.E-14, 1.E-8 ...) are used as the reference
 *     uses them, promoted to double.
 *
 * Strings are uint32_t (up to 32 sites).  The reference's INTEGER*4 strings
 * overflow at 32 sites; for <= 31 sites the two agree bit for bit.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TOL14 ((double)1.0e-14f) /* REAL*4 literal 1.E-14 as the reference compares */

/* ---------------------------------------------------------------- basis --- */

/* Binomial coefficient C(n,k) (funcmod.f90:7-16 computes it recursively). */
int64_t orc_binom(int n, int k)
{
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

/* C(n,k) for 0 <= n,k <= 32 from a table filled on first use. */
static int64_t binom_tab[33][33];
static int binom_ready = 0;
static inline int64_t bnm(int n, int k)
{
    if (!binom_ready) {
        for (int a = 0; a <= 32; ++a)
            for (int b = 0; b <= 32; ++b) binom_tab[a][b] = orc_binom(a, b);
        binom_ready = 1;
    }
    if (n < 0 || k < 0 || n > 32 || k > 32) return 0;
    return binom_tab[n][k];
}

/* MOVE: shift the particle at bit posf-1 one bit up (compute_basis.f90:127-135). */
static uint32_t hb_move(uint32_t s, int posf)
{
    uint32_t a = (uint32_t)1u << (posf - 1);
    uint32_t b = s ^ a;
    a = (uint32_t)1u << posf;
    return b ^ a;
}

/* BMOVE: carry when the top bits are full (compute_basis.f90:139-167).
 * Returns the next string and writes the new scan position to *posm. */
static uint32_t hb_bmove(int no, uint32_t s, int *posm)
{
    int nstatem = 0;
    uint32_t sf = s;
    while (nstatem < no && (s >> (no - nstatem - 1)) & 1u) nstatem++;
    for (int i = 1; i <= nstatem; ++i) sf -= (uint32_t)1u << (no - i);
    int posle = no;
    while (posle > 0 && !((sf >> (posle - 1)) & 1u)) posle--;
    sf -= (uint32_t)1u << (posle - 1);
    uint32_t sm = sf;
    for (int i = 1; i <= nstatem + 1; ++i) sm += (uint32_t)1u << (posle - 1 + i);
    *posm = posle + 1 + nstatem;
    return sm;
}

/* HILBERT: all ne-of-no bit strings in the reference's enumeration order
 * (compute_basis.f90:67-96).  out must hold C(no,ne) entries. */
void orc_hilbert(int no, int ne, uint32_t *out)
{
    int64_t ns = orc_binom(no, ne);
    if (ns <= 0) return;
    for (int64_t i = 0; i < ns; ++i) out[i] = 0;
    for (int i = 1; i <= ne; ++i) out[0] += (uint32_t)1u << (i - 1);
    int64_t cpt = 1;
    int pos = ne;
    while (cpt < ns) {
        while (pos < no && cpt < ns) {
            out[cpt] = hb_move(out[cpt - 1], pos);
            cpt++;
            pos++;
        }
        if (cpt < ns) {
            out[cpt] = hb_bmove(no, out[cpt - 1], &pos);
            cpt++;
        }
    }
}

/* -------------------------------------------------------- bit primitives --- */

static inline uint32_t site_bit(int norb, int pos) { return (uint32_t)1u << (norb - pos); }

/* KINOP: move a particle from site posi to site posf (funcmod.f90:18-27).
 * Returns 0 when forbidden; returns the string itself when posi==posf and
 * posi is occupied. */
uint32_t orc_kinop(int norb, uint32_t s, int posi, int posf)
{
    uint32_t a = site_bit(norb, posi), b = site_bit(norb, posf);
    uint32_t r = 0;
    if ((s & a) == a && (s & b) == 0) r = s - a + b;
    if ((s & a) == a && posi == posf) r = s;
    return r;
}

/* ANTICOM: (-1)^(number of occupied sites 1..pos-1) (funcmod.f90:29-41). */
double orc_anticom(int norb, int pos, uint32_t s)
{
    double ac = 1.0;
    for (int i = 1; i < pos; ++i)
        if (s & site_bit(norb, i)) ac = -ac;
    return ac;
}

static inline int is_part(int norb, int pos, uint32_t s) { return (s & site_bit(norb, pos)) != 0; }

/* SZ of one site (funcmod.f90:76-84). */
static double sz_site(int norb, int pos, uint32_t up, uint32_t dn)
{
    double sz = 0.0;
    if (is_part(norb, pos, up)) sz += 0.5;
    if (is_part(norb, pos, dn)) sz -= 0.5;
    return sz;
}

/* Linear-search rank, 1-based, 0 when absent (hprod_hubbard.f90:41-47). */
static int64_t lin_rank(uint32_t s, const uint32_t *b, int64_t n)
{
    for (int64_t l = 0; l < n; ++l)
        if (b[l] == s) return l + 1;
    return 0;
}

/* Fortran view T(J,K) of a row-major n*n buffer (1-based J,K). */
#define TF(T, n, J, K) ((T)[((int64_t)(J) - 1) + ((int64_t)(K) - 1) * (n)])

/* ------------------------------------------ Hubbard H*v, reference order --- */

/* Restatement of the live HPROD (hprod_hubbard.f90:17-118) for the local-U
 * path (IS_ULOC=2, UPARTIAL=0): same loop nest, linear-search rank, the
 * NUP==NDOWN transposed down-hop (:52-56) and the separate down loop (:93-114).
 * t: row-major norb*norb buffer as handed to the reference; uloc: per-site U. */
void orc_hprod_hubbard_ref(int norb, int nup, int ndn,
                           const uint32_t *bup, int64_t nsup,
                           const uint32_t *bdn, int64_t nsdn,
                           const double *t, const double *uloc,
                           const double *x, double *y)
{
    int64_t nst = nsup * nsdn;
    for (int64_t i = 0; i < nst; ++i) y[i] = 0.0;
    for (int J = 1; J <= norb; ++J) {
        for (int64_t u = 0; u < nsup; ++u) {
            if (!is_part(norb, J, bup[u])) continue;
            for (int64_t d = 0; d < nsdn; ++d)
                if (is_part(norb, J, bdn[d]))
                    y[d * nsup + u] = y[d * nsup + u] + x[d * nsup + u] * uloc[J - 1];
        }
        for (int K = 1; K <= norb; ++K) {
            double tjk = TF(t, norb, J, K);
            if (!(fabs(tjk) >= TOL14)) continue;
            for (int64_t u = 0; u < nsup; ++u) {
                uint32_t nw = orc_kinop(norb, bup[u], J, K);
                if (nw == 0) continue;
                int64_t pos = lin_rank(nw, bup, nsup);
                if (pos <= 0) continue;
                double ac = orc_anticom(norb, J, bup[u]);
                ac = ac * orc_anticom(norb, K, nw);
                int64_t p = pos - 1;
                if (nup == ndn) {
                    for (int64_t d = 0; d < nsdn; ++d) {
                        y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
                        y[p * nsup + d] = y[p * nsup + d] + ac * x[u * nsup + d] * tjk;
                    }
                } else {
                    for (int64_t d = 0; d < nsdn; ++d)
                        y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
                }
            }
            if (nup != ndn) {
                for (int64_t d = 0; d < nsdn; ++d) {
                    uint32_t nw = orc_kinop(norb, bdn[d], J, K);
                    if (nw == 0) continue;
                    int64_t pos = lin_rank(nw, bdn, nsdn);
                    if (pos <= 0) continue;
                    double ac = orc_anticom(norb, J, bdn[d]);
                    ac = ac * orc_anticom(norb, K, nw);
                    int64_t p = pos - 1;
                    for (int64_t u = 0; u < nsup; ++u)
                        y[p * nsup + u] = y[p * nsup + u] + ac * x[d * nsup + u] * tjk;
                }
            }
        }
    }
}

/* Same restatement, restricted to the ordered site pairs listed in pairs
 * (npairs entries of (J,K), 1-based) and without the U diagonal.  This is the
 * bounded sample used to time the reference loop on large sectors: the work of
 * HPROD is a sum over (J,K) pairs, so the time of a subset scales to the full
 * product by the share of active pairs it covers. */
void orc_hprod_hubbard_ref_pairs(int norb, int nup, int ndn,
                                 const uint32_t *bup, int64_t nsup,
                                 const uint32_t *bdn, int64_t nsdn,
                                 const double *t, const int32_t *pairs, int npairs,
                                 const double *x, double *y)
{
    for (int q = 0; q < npairs; ++q) {
        int J = pairs[2 * q], K = pairs[2 * q + 1];
        double tjk = TF(t, norb, J, K);
        if (!(fabs(tjk) >= TOL14)) continue;
        for (int64_t u = 0; u < nsup; ++u) {
            uint32_t nw = orc_kinop(norb, bup[u], J, K);
            if (nw == 0) continue;
            int64_t pos = lin_rank(nw, bup, nsup);
            if (pos <= 0) continue;
            double ac = orc_anticom(norb, J, bup[u]) * orc_anticom(norb, K, nw);
            int64_t p = pos - 1;
            if (nup == ndn) {
                for (int64_t d = 0; d < nsdn; ++d) {
                    y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
                    y[p * nsup + d] = y[p * nsup + d] + ac * x[u * nsup + d] * tjk;
                }
            } else {
                for (int64_t d = 0; d < nsdn; ++d)
                    y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
            }
        }
        if (nup != ndn) {
            for (int64_t d = 0; d < nsdn; ++d) {
                uint32_t nw = orc_kinop(norb, bdn[d], J, K);
                if (nw == 0) continue;
                int64_t pos = lin_rank(nw, bdn, nsdn);
                if (pos <= 0) continue;
                double ac = orc_anticom(norb, J, bdn[d]) * orc_anticom(norb, K, nw);
                int64_t p = pos - 1;
                for (int64_t u = 0; u < nsup; ++u)
                    y[p * nsup + u] = y[p * nsup + u] + ac * x[d * nsup + u] * tjk;
            }
        }
    }
}

/* orc_hprod_hubbard_ref_pairs on nthreads host threads (0: the OpenMP
 * default), with the same results bit for bit.  For each pair:
 *  1. the rank search of every string (the linear search of
 *     hprod_hubbard.f90:41-47 and :97-103) is split over the threads;
 *  2. the axpys run with each thread owning a block of output rows.  Every
 *     thread walks the strings in the serial order and adds only into its own
 *     rows, so each element of y receives its terms in the serial loop's order
 *     (for one string the column term precedes the row term, as in the
 *     reference's d loop).
 * This is the reference loop with all host cores working on it; the
 * arithmetic and the memory access pattern are the serial loop's. */
void orc_hprod_hubbard_ref_pairs_mt(int norb, int nup, int ndn,
                                    const uint32_t *bup, int64_t nsup,
                                    const uint32_t *bdn, int64_t nsdn,
                                    const double *t, const int32_t *pairs, int npairs,
                                    const double *x, double *y, int nthreads)
{
    int64_t nmax = nsup > nsdn ? nsup : nsdn;
    int64_t *pos = (int64_t *)malloc((size_t)nmax * sizeof(int64_t));
    double *acs = (double *)malloc((size_t)nmax * sizeof(double));
    if (nthreads > 0) omp_set_num_threads(nthreads);
    for (int q = 0; q < npairs; ++q) {
        int J = pairs[2 * q], K = pairs[2 * q + 1];
        double tjk = TF(t, norb, J, K);
        if (!(fabs(tjk) >= TOL14)) continue;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t u = 0; u < nsup; ++u) {
            pos[u] = -1;
            uint32_t nw = orc_kinop(norb, bup[u], J, K);
            if (nw == 0) continue;
            int64_t p = lin_rank(nw, bup, nsup);
            if (p <= 0) continue;
            pos[u] = p - 1;
            acs[u] = orc_anticom(norb, J, bup[u]) * orc_anticom(norb, K, nw);
        }
#pragma omp parallel
        {
            int nt = omp_get_num_threads(), id = omp_get_thread_num();
            int64_t r0 = nsdn * id / nt, r1 = nsdn * (id + 1) / nt;
            for (int64_t u = 0; u < nsup; ++u) {
                int64_t p = pos[u];
                if (p < 0) continue;
                double ac = acs[u];
                for (int64_t d = r0; d < r1; ++d)
                    y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
                if (nup == ndn && p >= r0 && p < r1)
                    for (int64_t d = 0; d < nsdn; ++d)
                        y[p * nsup + d] = y[p * nsup + d] + ac * x[u * nsup + d] * tjk;
            }
        }
        if (nup != ndn) {
#pragma omp parallel for schedule(dynamic, 64)
            for (int64_t d = 0; d < nsdn; ++d) {
                pos[d] = -1;
                uint32_t nw = orc_kinop(norb, bdn[d], J, K);
                if (nw == 0) continue;
                int64_t p = lin_rank(nw, bdn, nsdn);
                if (p <= 0) continue;
                pos[d] = p - 1;
                acs[d] = orc_anticom(norb, J, bdn[d]) * orc_anticom(norb, K, nw);
            }
#pragma omp parallel
            {
                int nt = omp_get_num_threads(), id = omp_get_thread_num();
                int64_t r0 = nsdn * id / nt, r1 = nsdn * (id + 1) / nt;
                for (int64_t d = 0; d < nsdn; ++d) {
                    int64_t p = pos[d];
                    if (p < r0 || p >= r1) continue;
                    double ac = acs[d];
                    for (int64_t u = 0; u < nsup; ++u)
                        y[p * nsup + u] = y[p * nsup + u] + ac * x[d * nsup + u] * tjk;
                }
            }
        }
    }
    free(pos);
    free(acs);
}

/* The on-site U part of the reference loop for site J on nthreads threads
 * (each up string's column belongs to one thread; one term per element, so the
 * result equals the serial loop's). */
void orc_hprod_hubbard_ref_udiag_mt(int norb, const uint32_t *bup, int64_t nsup,
                                    const uint32_t *bdn, int64_t nsdn, int J, double uj,
                                    const double *x, double *y, int nthreads)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static, 16)
    for (int64_t u = 0; u < nsup; ++u) {
        if (!is_part(norb, J, bup[u])) continue;
        for (int64_t d = 0; d < nsdn; ++d)
            if (is_part(norb, J, bdn[d]))
                y[d * nsup + u] = y[d * nsup + u] + x[d * nsup + u] * uj;
    }
}

/* The on-site U part of the reference loop for one site J only
 * (hprod_hubbard.f90:27-35), adding into y: the bounded sample used with
 * orc_hprod_hubbard_ref_pairs to time the reference loop on large sectors. */
void orc_hprod_hubbard_ref_udiag(int norb, const uint32_t *bup, int64_t nsup,
                                 const uint32_t *bdn, int64_t nsdn, int J, double uj,
                                 const double *x, double *y)
{
    for (int64_t u = 0; u < nsup; ++u) {
        if (!is_part(norb, J, bup[u])) continue;
        for (int64_t d = 0; d < nsdn; ++d)
            if (is_part(norb, J, bdn[d]))
                y[d * nsup + u] = y[d * nsup + u] + x[d * nsup + u] * uj;
    }
}

/* ---------------------------------------- Heisenberg H*v, reference order --- */

/* Restatement of HPROD for the Sz=0 Heisenberg sector (hprod_heis.f90:1-61):
 * one up string per state, the down string being its complement (:14). */
void orc_hprod_heis_ref(int norb, const uint32_t *bup, int64_t nsup,
                        const double *jm, const double *x, double *y)
{
    uint32_t full = (norb >= 32) ? 0xFFFFFFFFu : (((uint32_t)1u << norb) - 1u);
    for (int64_t i = 0; i < nsup; ++i) y[i] = 0.0;
    for (int J = 1; J <= norb; ++J) {
        double jjj = TF(jm, norb, J, J);
        if (fabs(jjj) > TOL14) {
            for (int64_t i = 0; i < nsup; ++i) {
                uint32_t dn = full - bup[i];
                int pu = is_part(norb, J, bup[i]), pd = is_part(norb, J, dn);
                if ((pu && !pd) || (!pu && pd)) y[i] = y[i] + x[i] * 0.5 * jjj;
            }
        }
        for (int K = 1; K <= norb; ++K) {
            double jjk = TF(jm, norb, J, K);
            if (fabs(jjk) > TOL14 && J != K) {
                for (int64_t i = 0; i < nsup; ++i) {
                    uint32_t nw = orc_kinop(norb, bup[i], J, K);
                    if (nw == 0) continue;
                    int64_t pos = lin_rank(nw, bup, nsup);
                    if (pos <= 0) continue;
                    uint32_t dn = full - bup[i];
                    double ac = orc_anticom(norb, J, bup[i]);
                    ac = ac * orc_anticom(norb, K, nw);
                    uint32_t nw2 = orc_kinop(norb, dn, K, J);
                    if (nw2 == full - bup[pos - 1]) {
                        ac = ac * orc_anticom(norb, J, dn);
                        ac = ac * orc_anticom(norb, K, nw2);
                        y[pos - 1] = y[pos - 1] - ac * x[i] * jjk;
                    }
                }
            }
            for (int64_t i = 0; i < nsup; ++i) {
                uint32_t dn = full - bup[i];
                y[i] = y[i] + x[i] * sz_site(norb, J, bup[i], dn) * sz_site(norb, K, bup[i], dn) * jjk;
            }
        }
    }
}

/* ------------------------------------------------ rank tables (fast path) --- */

/* Lexicographic rank of a k-subset of {0..n-1} given as a bit string
 * (bit i <-> element i), i.e. the position of s in orc_hilbert(n,k).
 * rank = sum over set bits, in increasing order, of the number of subsets that
 * share the prefix and take a smaller element at this step. */
int64_t orc_rank(int n, int k, uint32_t s)
{
    int64_t r = 0;
    int prev = -1, left = k;
    for (int i = 0; i < n && left > 0; ++i) {
        if (!((s >> i) & 1u)) continue;
        for (int j = prev + 1; j < i; ++j) r += bnm(n - 1 - j, left - 1);
        prev = i;
        left--;
    }
    return r;
}

/* Per-string hop list in gather form: for each target string p, every source
 * string q = p - bit(K) + bit(J) with K occupied and J empty in p and
 * |T(J,K)| >= 1e-14, with coefficient sign(J,q)*sign(K,p)*T(J,K).  This is the
 * same operator as the reference's scatter loop, read from the output side. */
typedef struct {
    int64_t *ptr;  /* n+1 */
    int64_t *src;  /* nnz */
    double *coef;  /* nnz */
    double *diag;  /* n: sum of T(J,J) over occupied J with |T(J,J)| >= 1e-14 */
} hoplist;

static void hoplist_build(int norb, int ne, const uint32_t *b, int64_t n,
                          const double *t, hoplist *h)
{
    h->ptr = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    h->diag = (double *)malloc((size_t)n * sizeof(double));
    int64_t cap = n * (int64_t)(ne * (norb - ne) + 1) + 1;
    h->src = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    h->coef = (double *)malloc((size_t)cap * sizeof(double));
    int64_t nnz = 0;
    for (int64_t p = 0; p < n; ++p) {
        h->ptr[p] = nnz;
        uint32_t s = b[p];
        double dg = 0.0;
        for (int J = 1; J <= norb; ++J) {
            double tjj = TF(t, norb, J, J);
            if (is_part(norb, J, s) && fabs(tjj) >= TOL14) dg += tjj;
        }
        h->diag[p] = dg;
        for (int K = 1; K <= norb; ++K) {
            if (!is_part(norb, K, s)) continue;
            for (int J = 1; J <= norb; ++J) {
                if (J == K || is_part(norb, J, s)) continue;
                double tjk = TF(t, norb, J, K);
                if (!(fabs(tjk) >= TOL14)) continue;
                uint32_t q = s - site_bit(norb, K) + site_bit(norb, J);
                double ac = orc_anticom(norb, J, q) * orc_anticom(norb, K, s);
                h->src[nnz] = orc_rank(norb, ne, q);
                h->coef[nnz] = ac * tjk;
                nnz++;
            }
        }
    }
    h->ptr[n] = nnz;
}

static void hoplist_free(hoplist *h)
{
    free(h->ptr); free(h->src); free(h->coef); free(h->diag);
}

/* Same operator as orc_hprod_hubbard_ref, computed row by row in gather form
 * with combinadic rank, parallel over down strings (OpenMP). */
void orc_hprod_hubbard_fast(int norb, int nup, int ndn,
                            const uint32_t *bup, int64_t nsup,
                            const uint32_t *bdn, int64_t nsdn,
                            const double *t, const double *uloc,
                            const double *x, double *y, int nthreads)
{
    hoplist hu, hd;
    hoplist_build(norb, nup, bup, nsup, t, &hu);
    hoplist_build(norb, ndn, bdn, nsdn, t, &hd);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t d = 0; d < nsdn; ++d) {
        uint32_t sd = bdn[d];
        const double *xr = x + d * nsup;
        double *yr = y + d * nsup;
        for (int64_t u = 0; u < nsup; ++u) {
            uint32_t both = bup[u] & sd;
            double dg = hu.diag[u] + hd.diag[d];
            for (int J = 1; J <= norb; ++J)
                if (both & site_bit(norb, J)) dg += uloc[J - 1];
            double acc = dg * xr[u];
            for (int64_t e = hu.ptr[u]; e < hu.ptr[u + 1]; ++e) acc += hu.coef[e] * xr[hu.src[e]];
            yr[u] = acc;
        }
        for (int64_t e = hd.ptr[d]; e < hd.ptr[d + 1]; ++e) {
            const double *xs = x + hd.src[e] * nsup;
            double c = hd.coef[e];
            for (int64_t u = 0; u < nsup; ++u) yr[u] += c * xs[u];
        }
    }
    hoplist_free(&hu);
    hoplist_free(&hd);
}

/* Same operator as orc_hprod_heis_ref in gather form with combinadic rank,
 * parallel over states (OpenMP). */
void orc_hprod_heis_fast(int norb, const uint32_t *bup, int64_t nsup,
                         const double *jm, const double *x, double *y, int nthreads)
{
    uint32_t full = (norb >= 32) ? 0xFFFFFFFFu : (((uint32_t)1u << norb) - 1u);
    int ne = norb / 2;
    (void)bnm(0, 0); /* fill the binomial table before the parallel region */
    double dconst = 0.0;
    for (int J = 1; J <= norb; ++J) {
        double jjj = TF(jm, norb, J, J);
        if (fabs(jjj) > TOL14) dconst += 0.5 * jjj;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static, 4096)
#endif
    for (int64_t p = 0; p < nsup; ++p) {
        uint32_t s = bup[p], dn = full - s;
        double dg = dconst;
        for (int J = 1; J <= norb; ++J) {
            double sj = is_part(norb, J, s) ? 0.5 : -0.5;
            for (int K = 1; K <= norb; ++K) {
                double sk = is_part(norb, K, s) ? 0.5 : -0.5;
                dg += sj * sk * TF(jm, norb, J, K);
            }
        }
        double acc = dg * x[p];
        /* sources: q = p with K<->J exchanged where K is up in p, J is down in p */
        for (int K = 1; K <= norb; ++K) {
            if (!is_part(norb, K, s)) continue;
            for (int J = 1; J <= norb; ++J) {
                if (J == K || is_part(norb, J, s)) continue;
                double jjk = TF(jm, norb, J, K);
                if (!(fabs(jjk) > TOL14)) continue;
                uint32_t q = s - site_bit(norb, K) + site_bit(norb, J);
                uint32_t qd = full - q;
                double ac = orc_anticom(norb, J, q) * orc_anticom(norb, K, s)
                          * orc_anticom(norb, J, qd) * orc_anticom(norb, K, dn);
                acc -= ac * jjk * x[orc_rank(norb, ne, q)];
            }
        }
        y[p] = acc;
    }
}

/* ------------------------------------------------------------------ RDMs --- */

/* ONE_RDM (static_rq.f90:153-244).  dm is written in the reference's Fortran
 * layout DENS_MAT(J,K,S): element (J,K,S) at (J-1)+(K-1)*N+(S-1)*N*N. */
void orc_one_rdm(int norb, int nup, int ndn,
                 const uint32_t *bup, int64_t nsup,
                 const uint32_t *bdn, int64_t nsdn,
                 const double *bra, const double *ket, double *dm)
{
    int64_t N = norb;
#define DM(J, K, S) dm[((J) - 1) + ((K) - 1) * N + ((S) - 1) * N * N]
    for (int J = 1; J <= norb; ++J) {
        for (int K = 1; K <= J; ++K) {
            DM(J, K, 1) = 0.0;
            for (int64_t i = 0; i < nsup; ++i) {
                uint32_t nw = orc_kinop(norb, bup[i], J, K);
                if (nw == 0) continue;
                int64_t pos = lin_rank(nw, bup, nsup);
                if (pos <= 0) continue;
                double ac = orc_anticom(norb, J, bup[i]) * orc_anticom(norb, K, nw);
                for (int64_t l = 0; l < nsdn; ++l)
                    DM(J, K, 1) = DM(J, K, 1) + ac * bra[l * nsup + i] * ket[l * nsup + pos - 1];
            }
            DM(K, J, 1) = DM(J, K, 1);
            if (nup != ndn) {
                DM(J, K, 2) = 0.0;
                for (int64_t l = 0; l < nsdn; ++l) {
                    uint32_t nw = orc_kinop(norb, bdn[l], J, K);
                    if (nw == 0) continue;
                    int64_t pos = lin_rank(nw, bdn, nsdn);
                    if (pos <= 0) continue;
                    double ac = orc_anticom(norb, J, bdn[l]) * orc_anticom(norb, K, nw);
                    for (int64_t i = 0; i < nsup; ++i)
                        DM(J, K, 2) = DM(J, K, 2) + ac * bra[l * nsup + i] * ket[(pos - 1) * nsup + i];
                }
                DM(K, J, 2) = DM(J, K, 2);
            } else {
                DM(J, K, 2) = DM(J, K, 1);
                DM(K, J, 2) = DM(J, K, 1);
            }
        }
    }
#undef DM
}

/* NI(J) = <n_J,up n_J,down> of TWO_RDM's local-U branch (static_rq.f90:307-316). */
void orc_two_rdm_ni(int norb, const uint32_t *bup, int64_t nsup,
                    const uint32_t *bdn, int64_t nsdn,
                    const double *bra, const double *ket, double *ni)
{
    for (int J = 1; J <= norb; ++J) {
        ni[J - 1] = 0.0;
        for (int64_t u = 0; u < nsup; ++u) {
            if (!is_part(norb, J, bup[u])) continue;
            for (int64_t d = 0; d < nsdn; ++d)
                if (is_part(norb, J, bdn[d]))
                    ni[J - 1] = ni[J - 1] + bra[d * nsup + u] * ket[d * nsup + u];
        }
    }
}

/* J_SPIN: <S_J . S_K> (static_rq.f90:323-395); sm in Fortran layout (J,K). */
void orc_j_spin(int norb, const uint32_t *bup, int64_t nsup,
                const uint32_t *bdn, int64_t nsdn,
                const double *bra, const double *ket, double *sm)
{
    int64_t N = norb;
#define SM(J, K) sm[((J) - 1) + ((K) - 1) * N]
    for (int J = 1; J <= norb; ++J) {
        for (int K = 1; K <= J; ++K) {
            SM(J, K) = 0.0;
            if (J == K) {
                for (int64_t i = 0; i < nsup; ++i)
                    for (int64_t l = 0; l < nsdn; ++l) {
                        int pu = is_part(norb, J, bup[i]), pd = is_part(norb, J, bdn[l]);
                        if (pu && !pd) SM(J, J) = SM(J, J) + 0.5 * bra[l * nsup + i] * ket[l * nsup + i];
                        if (!pu && pd) SM(J, J) = SM(J, J) + 0.5 * bra[l * nsup + i] * ket[l * nsup + i];
                    }
            } else {
                for (int64_t i = 0; i < nsup; ++i) {
                    uint32_t nw = orc_kinop(norb, bup[i], J, K);
                    if (nw == 0) continue;
                    int64_t pos = lin_rank(nw, bup, nsup);
                    if (pos <= 0) continue;
                    double ac = orc_anticom(norb, J, bup[i]) * orc_anticom(norb, K, nw);
                    for (int64_t l = 0; l < nsdn; ++l) {
                        uint32_t nw2 = orc_kinop(norb, bdn[l], K, J);
                        if (nw2 == 0) continue;
                        int64_t pos2 = lin_rank(nw2, bdn, nsdn);
                        if (pos2 <= 0) continue;
                        double ac2 = orc_anticom(norb, K, bdn[l]) * orc_anticom(norb, J, nw2);
                        SM(J, K) = SM(J, K) - ac * ac2 * bra[l * nsup + i] * ket[(pos2 - 1) * nsup + pos - 1];
                    }
                }
            }
            for (int64_t i = 0; i < nsup; ++i)
                for (int64_t l = 0; l < nsdn; ++l)
                    SM(J, K) = SM(J, K) + bra[l * nsup + i] * ket[l * nsup + i]
                             * sz_site(norb, J, bup[i], bdn[l]) * sz_site(norb, K, bup[i], bdn[l]);
            SM(K, J) = SM(J, K);
        }
    }
#undef SM
}

/* J_SPIN for the Sz=0 Heisenberg sector (static_rq_heis.f90:58-116). */
void orc_j_spin_heis(int norb, const uint32_t *bup, int64_t nsup,
                     const double *bra, const double *ket, double *sm)
{
    int64_t N = norb;
    uint32_t full = (norb >= 32) ? 0xFFFFFFFFu : (((uint32_t)1u << norb) - 1u);
#define SM(J, K) sm[((J) - 1) + ((K) - 1) * N]
    for (int J = 1; J <= norb; ++J) {
        for (int K = 1; K <= norb; ++K) {
            SM(J, K) = 0.0;
            if (J == K) {
                for (int64_t i = 0; i < nsup; ++i) {
                    uint32_t dn = full - bup[i];
                    int pu = is_part(norb, J, bup[i]), pd = is_part(norb, J, dn);
                    if (pu && !pd) SM(J, J) = SM(J, J) + 0.5 * bra[i] * ket[i];
                    else if (!pu && pd) SM(J, J) = SM(J, J) + 0.5 * bra[i] * ket[i];
                }
            } else {
                for (int64_t i = 0; i < nsup; ++i) {
                    uint32_t nw = orc_kinop(norb, bup[i], J, K);
                    if (nw == 0) continue;
                    int64_t pos = lin_rank(nw, bup, nsup);
                    if (pos <= 0) continue;
                    uint32_t dn = full - bup[i];
                    double ac = orc_anticom(norb, J, bup[i]) * orc_anticom(norb, K, nw);
                    uint32_t nw2 = orc_kinop(norb, dn, K, J);
                    if (nw2 == full - bup[pos - 1]) {
                        ac = ac * orc_anticom(norb, K, dn);
                        ac = ac * orc_anticom(norb, J, nw2);
                        SM(J, K) = SM(J, K) - ac * bra[pos - 1] * ket[i];
                    }
                }
            }
            for (int64_t i = 0; i < nsup; ++i) {
                uint32_t dn = full - bup[i];
                SM(J, K) = SM(J, K) + bra[i] * ket[i] * sz_site(norb, J, bup[i], dn) * sz_site(norb, K, bup[i], dn);
            }
        }
    }
#undef SM
}

/* ------------------------------------------------ GF start vectors --- */

/* Start vectors of the particle/hole Green's function, one column per site
 * 1..ncomp, written as out[pos*nst_new + index] (the reference's
 * PSI_LCZ(NSTATES,NORB2COMP), column-major).
 *   kind 0: LCZ_H_UP   c_{i,up}|psi>      (spgf_bandlanczos.f90:508-533)
 *   kind 1: LCZ_H_DOWN c_{i,down}|psi>    (:536-560)
 *   kind 2: LCZ_E_UP   c^+_{i,up}|psi>    (:453-478)
 *   kind 3: LCZ_E_DOWN c^+_{i,down}|psi>  (:481-505)
 * (bup0,nsup0,bdn0,nsdn0) is the sector of psi; (bup1,...) the target sector.
 * ndn0 is the down count of psi (the up operators carry (-1)^ndn0). */
void orc_gf_start(int kind, int norb, int ncomp, int ndn0,
                  const uint32_t *bup0, int64_t nsup0, const uint32_t *bdn0, int64_t nsdn0,
                  const uint32_t *bup1, int64_t nsup1, const uint32_t *bdn1, int64_t nsdn1,
                  const double *psi, double *out)
{
    int64_t nst1 = nsup1 * nsdn1;
    for (int64_t i = 0; i < nst1 * ncomp; ++i) out[i] = 0.0;
    for (int pos = 1; pos <= ncomp; ++pos) {
        double *col = out + (int64_t)(pos - 1) * nst1;
        if (kind == 0 || kind == 2) {
            for (int64_t i = 0; i < nsup0; ++i) {
                int occ = is_part(norb, pos, bup0[i]);
                if ((kind == 0 && !occ) || (kind == 2 && occ)) continue;
                uint32_t a = (kind == 0) ? bup0[i] - site_bit(norb, pos) : bup0[i] + site_bit(norb, pos);
                for (int64_t j = 0; j < nsup1; ++j) {
                    if (bup1[j] != a) continue;
                    double ac = orc_anticom(norb, pos, bup0[i]);
                    if (ndn0 % 2 == 1) ac = -ac;
                    for (int64_t k = 0; k < nsdn1; ++k) col[k * nsup1 + j] = ac * psi[k * nsup0 + i];
                }
            }
        } else {
            for (int64_t i = 0; i < nsdn0; ++i) {
                int occ = is_part(norb, pos, bdn0[i]);
                if ((kind == 1 && !occ) || (kind == 3 && occ)) continue;
                uint32_t a = (kind == 1) ? bdn0[i] - site_bit(norb, pos) : bdn0[i] + site_bit(norb, pos);
                for (int64_t j = 0; j < nsdn1; ++j) {
                    if (bdn1[j] != a) continue;
                    double ac = orc_anticom(norb, pos, bdn0[i]);
                    for (int64_t k = 0; k < nsup1; ++k) col[j * nsup1 + k] = ac * psi[i * nsup0 + k];
                }
            }
        }
    }
}

/* -------------------------------------- sampled rows of large sectors --- */

/* The r-th k-subset of {0..n-1} in orc_rank's order (its inverse): at each
 * step the next element j is the first whose C(n-1-j, left-1) subsets
 * (those taking j here) contain r; the others are skipped by subtracting
 * their counts. */
uint32_t orc_unrank(int n, int k, int64_t r)
{
    uint32_t s = 0;
    int prev = -1, left = k;
    while (left > 0) {
        for (int j = prev + 1; j < n; ++j) {
            int64_t c = bnm(n - 1 - j, left - 1);
            if (r < c) {
                s |= (uint32_t)1u << j;
                prev = j;
                break;
            }
            r -= c;
        }
        left--;
    }
    return s;
}

/* Input vectors of the sampled-row checks, as a function of the element
 * index alone, so that a 6e8-element vector never has to exist on the host:
 * h = (i * 2654435761 + seed * 40503) mod 2^32;
 *   kind 0: h / 2^32 - 0.5 (an exact double in [-0.5, 0.5));
 *   kind 1: (h mod 7) - 3 (an integer in [-3, 3]).
 * The device side forms the same numbers with int64 arithmetic. */
double orc_hashval(int64_t i, int64_t seed, int kind)
{
    uint64_t h = ((uint64_t)i * 2654435761ull + (uint64_t)seed * 40503ull) & 0xffffffffull;
    if (kind == 0) return (double)h / 4294967296.0 - 0.5;
    return (double)(int)(h % 7ull) - 3.0;
}

/* HPROD of the Sz=0 Heisenberg sector (hprod_heis.f90:1-61) read from the
 * output side for a list of rows, with x_i = orc_hashval(i, xseed, xkind).
 * The reference scatters every source I into V1(POS); row p receives, in the
 * reference's (J, K) loop order: the J_MATRIX(J,J) single-occupancy term of
 * J (:11-20), then for each K the flip from the one source whose up string
 * maps onto p's (KINOP(BUP(I),J,K) = BUP(p): BUP(I) is BUP(p) with the
 * particle moved back from K to J, :23-49) and the SZ*SZ term (:53-57).
 * The sums are therefore the full restatement's, bit for bit, and the rank
 * is the closed form orc_rank (the reference's linear search finds the same
 * position).  absout[r] = the sum of the terms' magnitudes. */
void orc_hprod_heis_rows(int norb, const double *jm, int64_t nrows, const int64_t *rows,
                         int64_t xseed, int xkind, double *out, double *absout, int nthreads)
{
    const uint32_t full = (norb >= 32) ? 0xFFFFFFFFu : (((uint32_t)1u << norb) - 1u);
    const int ne = norb / 2;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t r = 0; r < nrows; ++r) {
        const int64_t p = rows[r];
        const uint32_t sp = orc_unrank(norb, ne, p), dnp = full - sp;
        const double xp = orc_hashval(p, xseed, xkind);
        double acc = 0.0, aab = 0.0;
        for (int J = 1; J <= norb; ++J) {
            const double jjj = TF(jm, norb, J, J);
            if (fabs(jjj) > TOL14) {
                int pu = is_part(norb, J, sp), pd = is_part(norb, J, dnp);
                if ((pu && !pd) || (!pu && pd)) {
                    acc = acc + xp * 0.5 * jjj;
                    aab += fabs(xp * 0.5 * jjj);
                }
            }
            for (int K = 1; K <= norb; ++K) {
                const double jjk = TF(jm, norb, J, K);
                if (fabs(jjk) > TOL14 && J != K && is_part(norb, K, sp) && !is_part(norb, J, sp)) {
                    const uint32_t s = sp - site_bit(norb, K) + site_bit(norb, J);
                    const int64_t i = orc_rank(norb, ne, s);
                    const uint32_t dn = full - s;
                    double ac = orc_anticom(norb, J, s);
                    ac = ac * orc_anticom(norb, K, sp);
                    const uint32_t nw2 = orc_kinop(norb, dn, K, J);
                    if (nw2 == full - sp) {
                        ac = ac * orc_anticom(norb, J, dn);
                        ac = ac * orc_anticom(norb, K, nw2);
                        const double xi = orc_hashval(i, xseed, xkind);
                        acc = acc - ac * xi * jjk;
                        aab += fabs(xi * jjk);
                    }
                }
                const double t = xp * sz_site(norb, J, sp, dnp) * sz_site(norb, K, sp, dnp) * jjk;
                acc = acc + t;
                aab += fabs(t);
            }
        }
        out[r] = acc;
        if (absout) absout[r] = aab;
    }
}

/* J_SPIN of the Sz=0 Heisenberg sector (static_rq_heis.f90:58-116) for a bra
 * supported on a list of rows R: bra_p = orc_hashval(p, bseed, kind) for p in
 * R and 0 elsewhere, ket_i = orc_hashval(i, kseed, kind) for every i.  Each
 * term of SMATRIX(J,K) carries bra at its row (BRA(I) in the diagonal sums,
 * BRA(POS) in the flip sum), so only rows in R contribute; the flip into row
 * p comes from the source whose up string KINOP maps onto p's, with J_SPIN's
 * sign, ANTICOM(J,BUP(I)) ANTICOM(K,NEW) ANTICOM(K,BDOWNELEM) ANTICOM(J,NEW2)
 * (:84-97).  pairs: npairs (J,K), 1-based; out[q] = SMATRIX(J,K) restricted
 * to R, absout[q] = the sum of its terms' magnitudes. */
void orc_j_spin_heis_rows(int norb, int64_t nrows, const int64_t *rows, int64_t bseed, int64_t kseed, int kind,
                          int npairs, const int32_t *pairs, double *out, double *absout, int nthreads)
{
    const uint32_t full = (norb >= 32) ? 0xFFFFFFFFu : (((uint32_t)1u << norb) - 1u);
    const int ne = norb / 2;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < npairs; ++q) {
        const int J = pairs[2 * q], K = pairs[2 * q + 1];
        double acc = 0.0, aab = 0.0;
        for (int64_t r = 0; r < nrows; ++r) {
            const int64_t p = rows[r];
            const uint32_t sp = orc_unrank(norb, ne, p), dnp = full - sp;
            const double bp = orc_hashval(p, bseed, kind), kp = orc_hashval(p, kseed, kind);
            if (J == K) {
                int pu = is_part(norb, J, sp), pd = is_part(norb, J, dnp);
                if ((pu && !pd) || (!pu && pd)) {
                    acc = acc + 0.5 * bp * kp;
                    aab += fabs(0.5 * bp * kp);
                }
            } else if (is_part(norb, K, sp) && !is_part(norb, J, sp)) {
                const uint32_t s = sp - site_bit(norb, K) + site_bit(norb, J);
                const int64_t i = orc_rank(norb, ne, s);
                const uint32_t dn = full - s;
                double ac = orc_anticom(norb, J, s) * orc_anticom(norb, K, sp);
                const uint32_t nw2 = orc_kinop(norb, dn, K, J);
                if (nw2 == full - sp) {
                    ac = ac * orc_anticom(norb, K, dn);
                    ac = ac * orc_anticom(norb, J, nw2);
                    const double ki = orc_hashval(i, kseed, kind);
                    acc = acc - ac * bp * ki;
                    aab += fabs(bp * ki);
                }
            }
            const double t = bp * kp * sz_site(norb, J, sp, dnp) * sz_site(norb, K, sp, dnp);
            acc = acc + t;
            aab += fabs(t);
        }
        out[q] = acc;
        if (absout) absout[q] = aab;
    }
}

/* ------------------------------------------ U_ijkl interaction (IS_ULOC=3) --- */

/* The reference reads the Python tensor U (C order, U[a][b][c][d]) from HDF5
 * into the Fortran array UL(NORB,NORB,NORB,NORB), so UL(J,K,M,N) =
 * U[N-1][M-1][K-1][J-1]; 'Upartial' = einsum('ijkl,ijkl->ij', U, U) becomes
 * UPARTIAL(J,K) = sum_cd U[K-1][J-1][c][d]^2 (core_solver.py:145-147,
 * compute_solver.f90:129-138). */
#define ULF(ul, n, J, K, M, N) \
    ((ul)[((((int64_t)(N) - 1) * (n) + ((M) - 1)) * (n) + ((K) - 1)) * (n) + ((J) - 1)])

static double upartial(const double *ul, int n, int J, int K)
{
    double s = 0.0;
    const double *p = ul + (((int64_t)(K - 1) * n + (J - 1)) * n) * n;
    for (int64_t q = 0; q < (int64_t)n * n; ++q) s += p[q] * p[q];
    return s;
}

/* HPROD with IS_ULOC=3 (hprod_hubbard.f90:17-118): the hopping terms of
 * every (J,K) with |T(J,K)| >= 1e-14 or UPARTIAL(J,K) >= 1e-14 (:37), and,
 * for UPARTIAL(J,K) >= 1e-14, the up hop J->K times every down hop M->N with
 * |UL(J,K,M,N)| >= 1e-14 (:62-86); no ULDIAG term.  Same loop nest and
 * linear-search rank as orc_hprod_hubbard_ref. */
void orc_hprod_hubbard_uijkl_ref(int norb, int nup, int ndn,
                                 const uint32_t *bup, int64_t nsup,
                                 const uint32_t *bdn, int64_t nsdn,
                                 const double *t, const double *ul,
                                 const double *x, double *y)
{
    int64_t nst = nsup * nsdn;
    for (int64_t i = 0; i < nst; ++i) y[i] = 0.0;
    for (int J = 1; J <= norb; ++J) {
        for (int K = 1; K <= norb; ++K) {
            double tjk = TF(t, norb, J, K);
            double upjk = upartial(ul, norb, J, K);
            if (!((fabs(tjk) >= TOL14) || (upjk >= TOL14))) continue;
            for (int64_t u = 0; u < nsup; ++u) {
                uint32_t nw = orc_kinop(norb, bup[u], J, K);
                if (nw == 0) continue;
                int64_t pos = lin_rank(nw, bup, nsup);
                if (pos <= 0) continue;
                double ac = orc_anticom(norb, J, bup[u]);
                ac = ac * orc_anticom(norb, K, nw);
                int64_t p = pos - 1;
                if (nup == ndn) {
                    for (int64_t d = 0; d < nsdn; ++d) {
                        y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
                        y[p * nsup + d] = y[p * nsup + d] + ac * x[u * nsup + d] * tjk;
                    }
                } else {
                    for (int64_t d = 0; d < nsdn; ++d)
                        y[d * nsup + p] = y[d * nsup + p] + ac * x[d * nsup + u] * tjk;
                }
                if (upjk >= TOL14) {
                    for (int M = 1; M <= norb; ++M)
                        for (int N = 1; N <= norb; ++N) {
                            double uv = ULF(ul, norb, J, K, M, N);
                            if (!(fabs(uv) >= TOL14)) continue;
                            for (int64_t d = 0; d < nsdn; ++d) {
                                uint32_t nw2 = orc_kinop(norb, bdn[d], M, N);
                                if (nw2 == 0) continue;
                                int64_t pos2 = lin_rank(nw2, bdn, nsdn);
                                if (pos2 <= 0) continue;
                                double ac2 = orc_anticom(norb, M, bdn[d]);
                                ac2 = ac2 * orc_anticom(norb, N, nw2);
                                y[(pos2 - 1) * nsup + p] = y[(pos2 - 1) * nsup + p] + ac * ac2 * x[d * nsup + u] * uv;
                            }
                        }
                }
            }
            if (nup != ndn) {
                for (int64_t d = 0; d < nsdn; ++d) {
                    uint32_t nw = orc_kinop(norb, bdn[d], J, K);
                    if (nw == 0) continue;
                    int64_t pos = lin_rank(nw, bdn, nsdn);
                    if (pos <= 0) continue;
                    double ac = orc_anticom(norb, J, bdn[d]);
                    ac = ac * orc_anticom(norb, K, nw);
                    int64_t p = pos - 1;
                    for (int64_t u = 0; u < nsup; ++u)
                        y[p * nsup + u] = y[p * nsup + u] + ac * x[d * nsup + u] * tjk;
                }
            }
        }
    }
}

/* TWO_RDM with DO_RQ_TB (static_rq.f90:247-306): DBL_OCC(J,K,M,N) =
 * sum over the up hop J->K (string I -> POS) and the down hop M->N
 * (L1 -> POS2) of AC*AC2*BRA((L1-1)*NSUP+I)*KET((POS2-1)*NSUP+POS), formed
 * for K <= J and N <= M and copied to (J,K,N,M), (K,J,M,N), (K,J,N,M);
 * NI(J) = DBL_OCC(J,J,J,J).  dbl: Fortran order, DBL_OCC(J,K,M,N) at
 * (J-1) + (K-1) n + (M-1) n^2 + (N-1) n^3. */
void orc_two_rdm_dbl_occ(int norb, const uint32_t *bup, int64_t nsup,
                         const uint32_t *bdn, int64_t nsdn,
                         const double *bra, const double *ket, double *dbl, double *ni)
{
    const int64_t n = norb;
#define DO(J, K, M, N) dbl[((J) - 1) + ((K) - 1) * n + ((M) - 1) * n * n + ((N) - 1) * n * n * n]
    for (int J = 1; J <= norb; ++J)
        for (int K = 1; K <= J; ++K)
            for (int M = 1; M <= norb; ++M)
                for (int N = 1; N <= M; ++N) {
                    double acc = 0.0;
                    for (int64_t i = 0; i < nsup; ++i) {
                        uint32_t nw = orc_kinop(norb, bup[i], J, K);
                        if (nw == 0) continue;
                        int64_t pos = lin_rank(nw, bup, nsup);
                        if (pos <= 0) continue;
                        double ac = orc_anticom(norb, J, bup[i]);
                        ac = ac * orc_anticom(norb, K, nw);
                        for (int64_t l1 = 0; l1 < nsdn; ++l1) {
                            uint32_t nw2 = orc_kinop(norb, bdn[l1], M, N);
                            if (nw2 == 0) continue;
                            int64_t pos2 = lin_rank(nw2, bdn, nsdn);
                            if (pos2 <= 0) continue;
                            double ac2 = orc_anticom(norb, M, bdn[l1]);
                            ac2 = ac2 * orc_anticom(norb, N, nw2);
                            acc = acc + ac * ac2 * bra[l1 * nsup + i] * ket[(pos2 - 1) * nsup + (pos - 1)];
                        }
                    }
                    DO(J, K, M, N) = acc;
                    DO(J, K, N, M) = acc;
                    DO(K, J, M, N) = acc;
                    DO(K, J, N, M) = acc;
                    if (J == K && J == M && J == N) ni[J - 1] = acc;
                }
#undef DO
}
