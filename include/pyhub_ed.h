/*
 * pyhub_ed.h -- C ABI of the GB300 exact-diagonalisation engine.
 *
 * The reference (PyHub) has no in-process native interface: its Python layer
 * writes HDF5 files and runs Fortran executables with os.system
 * (pyhub/core/core_solver.py:107-111), and pyhub/libs/__init__.py:9-23 holds a
 * ctypes loader for a "libsrc" that is never built.  These entry points
 * replace the Fortran routines that process boundary reaches; each
 * declaration names the reference routine it stands in for.
 *
 * Conventions
 *   - Every function returns 0 (ED_OK) on success or a nonzero ED_ERR_* code;
 *     ed_last_error() then describes the failure (thread-local).
 *   - All vectors are caller-owned device memory (e.g. torch tensors), passed
 *     as plain pointers; no hot entry point allocates.  Entry points that
 *     reduce (dot products, norms) take a caller-owned device scratch buffer;
 *     ed_scratch_bytes() gives the size it needs.
 *   - A sector vector is laid out as [nsdn rows][ld columns], element (d,u)
 *     at d*ld + u, d the down-string index and u the up-string index; with
 *     ld == nsup this is exactly the reference's index (D-1)*NSUP+U
 *     (hprod_hubbard.f90:31).  Padding columns u >= nsup must hold zeros.
 *   - Work is enqueued on the given CUDA stream (a cudaStream_t passed as
 *     void*; NULL is the legacy default stream) and is asynchronous unless
 *     stated.  Calls that share a scratch buffer must not overlap in time.
 *   - Scalars produced on the device (dots, norms, RDMs) are FP64.
 */
#ifndef PYHUB_ED_H
#define PYHUB_ED_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ED_OK = 0,
    ED_ERR_ARG = 1,      /* invalid argument (rejected before any launch) */
    ED_ERR_CUDA = 2,     /* CUDA runtime error */
    ED_ERR_MEM = 3,      /* device allocation failed (sector tables only) */
    ED_ERR_RANGE = 4     /* size beyond a stated limit */
};

enum { ED_HUBBARD = 0, ED_HEISENBERG = 1 };
enum { ED_F32 = 0, ED_F64 = 1 };

typedef struct ed_sector ed_sector;
typedef struct ed_opspace ed_opspace;

/* Last error message of the calling thread ("" when none). */
const char *ed_last_error(void);

/* ABI version (major*100+minor). */
int ed_version(void);

/* Binomial coefficient C(n,k); replaces BINOM (funcmod.f90:7-16). */
int64_t ed_binom(int n, int k);

/* Host enumeration of the ne-of-norb spin strings in the reference's order;
 * replaces HILBERT / WRITE_BASIS (compute_basis.f90:67-96, :27-64) and the
 * basis.h5 cache read by READ_BASIS (basismod.f90:38-75).  out holds n
 * entries, n == C(norb,ne). */
int ed_basis(int norb, int ne, uint32_t *out, int64_t n);

/* Index of a spin string in that order (the linear search of
 * hprod_hubbard.f90:41-47 as a closed form); -1 when not an ne-string. */
int64_t ed_rank(int norb, int ne, uint32_t s);

/* Build the device tables of one sector.  Replaces the state that
 * READ_INPUT / READ_BASIS load into HUBMOD (compute_solver.f90:11-19,
 * :39-179).
 *   kind ED_HUBBARD:    t = norb*norb hopping matrix (row-major, as given to
 *                       FermiHubbard; a hop J->K uses t[K][J]), U = per-site
 *                       interaction (norb), J ignored.
 *   kind ED_HEISENBERG: J = norb*norb exchange matrix, nup = norb/2, ndn = 0
 *                       (the reference's heisenberg.py:24 sector), t,U ignored.
 * Sizes beyond 32 sites or 2^31 strings per spin are ED_ERR_RANGE. */
int ed_sector_create(int norb, int nup, int ndn, int kind,
                     const double *t, const double *U, const double *J,
                     ed_sector **out);
int ed_sector_destroy(ed_sector *s);
int ed_sector_dims(const ed_sector *s, int64_t *nsup, int64_t *nsdn, int64_t *dim);
/* Host copies of the two string tables (nsup and nsdn entries). */
int ed_sector_strings(const ed_sector *s, uint32_t *up, uint32_t *dn);
/* Nonzeros per row of the hop tables actually applied (diagnostics). */
int ed_sector_nnz(const ed_sector *s, int64_t *nnz_up, int64_t *nnz_dn);

/* Device scratch bytes needed by the reducing entry points for n elements
 * and nvec vectors. */
int64_t ed_scratch_bytes(int64_t n, int nvec);

/* y = scale * H x.  Replaces HPROD (hprod_hubbard.f90:17-118 for Hubbard,
 * hprod_heis.f90:1-61 for Heisenberg).  dtype ED_F32 or ED_F64 (storage and
 * arithmetic of x and y; FP32 accumulates each element in FP32).  ld >= nsup
 * is the row stride (Heisenberg: ld ignored, vector of nsup entries).
 * If dots != NULL, dots[0] = <x,y> and dots[1] = <y,y> are written (FP64,
 * device pointer), using scratch. */
int ed_hv(ed_sector *s, void *stream, int dtype, int64_t ld,
          const void *x, void *y, double scale,
          double *dots, void *scratch, int64_t scratch_bytes);

/* out[j] = <V_j, w> and, if z != NULL, out[nvec + j] = <V_j, z>, j < nvec.
 * V_j = V + j*ldv elements.  FP64 results (device pointer).  The dot
 * products of the Lanczos loop (lanczos.f90:53,55) and of the
 * reorthogonalisation the reference lacks. */
int ed_multidot(void *stream, int dtype, int64_t n, const void *V, int64_t ldv, int nvec,
                const void *w, const void *z, double *out, void *scratch, int64_t scratch_bytes);

/* out = w - sum_j coef[j] V_j (w may be NULL: out = -sum coef V); coef is a
 * device FP64 array of nvec entries.  out may alias w.  If norm2 != NULL,
 * norm2[0] = <out,out> (FP64, device).  The vector update of lanczos.f90:54
 * generalised to a full projection; with w = NULL it forms a Ritz vector
 * V*c as READ_PSI_HUBBARD does (compute_solver.f90:282). out_dtype may differ
 * from dtype (e.g. an FP64 Ritz vector from an FP32 basis). */
int ed_update(void *stream, int dtype, int out_dtype, int64_t n, const void *V, int64_t ldv, int nvec,
              const double *coef, const void *w, void *out, double *norm2,
              void *scratch, int64_t scratch_bytes);

/* ed_update with the w term scaled by a device scalar:
 * out = wscale[0]*w - sum_j coef[j] V_j (wscale: device FP64, read by the
 * kernel; NULL means 1, which is ed_update).  Lets a Lanczos step scale H*v by
 * a norm that only the device knows. */
int ed_update_wscaled(void *stream, int dtype, int out_dtype, int64_t n, const void *V, int64_t ldv, int nvec,
                      const double *coef, const double *wscale, const void *w, void *out, double *norm2,
                      void *scratch, int64_t scratch_bytes);

/* Scalar work of step k of the full-reorthogonalisation Lanczos, on the
 * device, so that a step needs no host synchronisation (the reference forms
 * alpha and beta on the host, lanczos.f90:50-58, and has no
 * reorthogonalisation).  One step is
 *   ed_hv(u_k -> w, scale 1);  ed_multidot(V, k+1, w, z = u_k -> dots);
 *   ed_lanczos_coef(k, ...);
 *   ed_update_wscaled(V, k+1, coef, wscale = &state[2+k], w -> u_{k+1}, norm2 -> nrm)
 * with V_j = u_j the unnormalised basis, s_j = 1/||u_j|| and G the Gram matrix
 * of the normalised stored vectors, solved through its inverse Cholesky
 * factor, which grows by one row per step.
 * state: device FP64 array of ed_lanczos_state_doubles(mmax) entries, zeroed
 *   before step 0 except state[2] = 1/||u_0||:
 *   [0] stop code: 0 running, j > 0 breakdown after j steps (beta_{j-1} <=
 *       1e-13 max(1,|alpha_{j-1}|), or u_j numerically dependent on the basis: its
 *       Gram pivot below half its squared norm), -j a non-finite norm after j steps;
 *   [1] largest |G - I| entry seen;  [2 .. 2+mmax] s_0 .. s_mmax;
 *   then the inverse Cholesky factor, (mmax+1)^2 entries, row-major, and
 *   four work vectors of mmax+1 entries.
 * dots: [2(k+1)] from the multidot (a_j = <u_j, w>, b_j = <u_j, u_k>); NULL
 *   only closes step k-1 (beta[k-1], s_k and the stop test), as needed after
 *   the last step.
 * nrm: device ||u_k||^2 from the update of step k-1 (ignored at k = 0).
 * Writes alpha[k] = <v_k, H v_k>, beta[k-1] = ||u_k|| (k >= 1; device FP64,
 * mmax entries each) and coef[0..k].  After a stop, coef is zeros and the
 * vectors that follow are zero.  mmax <= 8192. */
int64_t ed_lanczos_state_doubles(int mmax);
int ed_lanczos_coef(void *stream, int k, int mmax, const double *dots, const double *nrm, double *state,
                    double *coef, double *alpha, double *beta);

/* Device scratch bytes needed by ed_rdm for npairs site pairs. */
int64_t ed_rdm_scratch_bytes(int npairs);

/* Raw reduced-density sums of <bra| ... |ket> for a list of site pairs
 * (pairs: host int32 [2*npairs], 1-based (J,K)).  Replaces ONE_RDM,
 * the local-U branch of TWO_RDM and J_SPIN (static_rq.f90:153-395) and the
 * Heisenberg J_SPIN (static_rq_heis.f90:58-116).  out (device FP64,
 * [npairs][6] for Hubbard followed by nothing, [npairs][2] for Heisenberg):
 *   Hubbard    q0: J!=K up hop J->K bra.ket sum / J==K <n_up>;  q1: <Sz_J Sz_K>;
 *              q2: J==K <n_down>;  q3: J==K <n_up n_down>;
 *              q4: J!=K down hop J->K (flags bit 0);
 *              q5: J!=K transverse spin term of J_SPIN (flags bit 1)
 *              (q0..q3 of all pairs come first, then q4,q5 of all pairs);
 *   Heisenberg q0: J!=K transverse term / J==K 0.5<1>;  q1: <Sz_J Sz_K>. */
int ed_rdm(ed_sector *s, void *stream, int dtype, int64_t ld, const void *bra, const void *ket,
           int npairs, const int32_t *pairs, int flags, double *out, void *scratch, int64_t scratch_bytes);

/* The general two-body interaction of a Hubbard sector, the reference's
 * IS_ULOC=3 path (hprod_hubbard.f90:37,62-86): ul (host, norb^4 FP64) is the
 * tensor U exactly as the reference's FermiHubbard takes it (C order
 * U[a][b][c][d]), read as the reference reads it, UL(J,K,M,N) =
 * U[N-1][M-1][K-1][J-1], each (J,K) kept only when UPARTIAL(J,K) =
 * sum_cd U[K-1][J-1][c][d]^2 >= 1e-14 (core_solver.py:143-147,
 * compute_solver.f90:129-138).  After this call ed_hv adds
 * sum UL(J,K,M,N) c+_{K up} c_{J up} c+_{N down} c_{M down} (terms with
 * |UL| >= 1e-14) and the sector's on-site U is dropped (no ULDIAG term on
 * that path).  The work per element is the number of terms: meant for the
 * small clusters this interaction is used on. */
int ed_sector_set_uijkl(ed_sector *s, const double *ul);
/* Device scratch bytes of ed_dbl_occ for nquads site quadruples. */
int64_t ed_dbl_occ_scratch_bytes(const ed_sector *s, int nquads);
/* The two-body density of TWO_RDM with DO_RQ_TB (static_rq.f90:256-306):
 * out[q] (device FP64) = DBL_OCC(J,K,M,N) = <ket| c+_{K up} c_{J up}
 * c+_{N down} c_{M down} |bra> for quads (host int32 [4*nquads], 1-based
 * (J,K,M,N)), summed in FP64.  Synchronises the stream once (the quad list
 * is copied from pageable host memory). */
int ed_dbl_occ(ed_sector *s, void *stream, int dtype, int64_t ld, const void *bra, const void *ket,
               int nquads, const int32_t *quads, double *out, void *scratch, int64_t scratch_bytes);

/* Green's-function start vector out = c_{site,s}|psi> (kind 0: up, 1: down)
 * or c^+_{site,s}|psi> (kind 2: up, 3: down), site 1-based, psi in sector src
 * (row stride ld0), out in sector dst (row stride ld1, written entirely).
 * Replaces LCZ_H_UP/LCZ_H_DOWN/LCZ_E_UP/LCZ_E_DOWN
 * (spgf_bandlanczos.f90:453-560), including their sign (-1)^N_down on the up
 * operators. */
int ed_gf_start(const ed_sector *src, const ed_sector *dst, void *stream, int kind, int site,
                int dtype, int64_t ld0, const void *psi, int out_dtype, int64_t ld1, void *out);
/* ed_gf_start for nsites sites (host array, 1-based, at most 32) in one
 * launch: the vector of sites[j] starts j*out_stride elements into out
 * (out_stride >= one vector of the target sector).  The loop over sites of
 * LCZ_{H,E}_{UP,DOWN} (spgf_bandlanczos.f90:453-560) for one operator. */
int ed_gf_start_sites(const ed_sector *src, const ed_sector *dst, void *stream, int kind, int nsites,
                      const int32_t *sites, int dtype, int64_t ld0, const void *psi, int out_dtype,
                      int64_t ld1, void *out, int64_t out_stride);

/* A batch of independent three-term Lanczos runs, one per instance, each on
 * its own Hubbard sector (e.g. every particle/hole start vector of every
 * cluster of a Green's-function sweep).  Replaces the per-start-block loops
 * of GF_BANDLANCZOS (spgf_bandlanczos.f90:309-448, called from :63-288).
 * Vectors of all instances are concatenated: instance i occupies elements
 * [offsets[i], offsets[i] + nsdn_i*ld_i) with ld_i = nsup_i rounded up to 32
 * (the engine's internal row stride). */
/* ---- composite entry points for a host without the Python layer ----
 * One step k of the full-reorthogonalisation Lanczos: ed_hv(u_k -> w),
 * ed_multidot(V, k+1, w, z = u_k), ed_lanczos_coef(k), ed_update_wscaled(->
 * u_{k+1}), enqueued on one stream with no host synchronisation.  V: device
 * basis rows (stride ldv >= the vector length), row 0 = the start vector;
 * state as ed_lanczos_coef documents it (zeroed, state[2] = 1/||u_0||);
 * alpha, beta device FP64 [mmax]; k < mmax.  The scratch (at least
 * ed_lanczos_step_scratch_bytes) must be the same for every step of a run: it
 * carries ||u_k||^2 from one step to the next.  Replaces the LANCZOS loop body
 * (lanczos.f90:50-58). */
int64_t ed_lanczos_step_scratch_bytes(const ed_sector *s, int mmax);
int ed_lanczos_step(ed_sector *s, void *stream, int dtype, int64_t ld, void *V, int64_t ldv, int k, int mmax,
                    void *w, double *state, double *alpha, double *beta, void *scratch, int64_t scratch_bytes);
/* The reduced quantities of one state as the reference stores them: Hubbard
 * gamma (host [2][N][N], up then down, symmetric), docc (host [N], NI of
 * TWO_RDM) and sisj (host [N][N], J_SPIN) from the pairs K <= J mirrored
 * (static_rq.f90:153-395; the down matrix is the up one when N_up == N_down,
 * :237-239); Heisenberg sisj only (SMATRIX in the Python view,
 * static_rq_heis.f90:58-116; gamma and docc may be NULL).  Synchronises the
 * stream (the sums are copied to the host). */
int64_t ed_rdm1_scratch_bytes(const ed_sector *s);
int ed_rdm1(ed_sector *s, void *stream, int dtype, int64_t ld, const void *psi, double *gamma, double *docc,
            double *sisj, void *scratch, int64_t scratch_bytes);
/* Hellmann-Feynman gradient of <psi|H|psi> for a Hubbard sector: g_t[b] =
 * dE/dt for bond b (bonds: host int32 [2*nbonds], 1-based, t_ij = t_ji one
 * parameter) = sum_s <c+_is c_js + c+_js c_is>; g_u[i] = <n_i,up n_i,down>;
 * g_eps[i] = sum_s <n_is> (the diagonal of t).  Both spins are summed (no
 * N_up == N_down shortcut).  Host outputs; scratch as ed_rdm1; synchronises
 * the stream.  No reference counterpart (the differentiation of the north
 * star). */
int ed_hf_grad(ed_sector *s, void *stream, int dtype, int64_t ld, const void *psi, int nbonds, const int32_t *bonds,
               double *g_t, double *g_u, double *g_eps, void *scratch, int64_t scratch_bytes);

/* ---- generic operator engine (operators.x) ----
 * The vector space of the reference's Operators: the up strings of every
 * listed up-particle number (nups[0..nlist_up-1], each block in HILBERT
 * order, concatenated in list order; compute_operators.f90:8-25 builds BUP
 * the same way from basis.h5), the same for down; state (d, u) at
 * d*nsup + u.  No particle number may be listed twice. */
int ed_opspace_create(int norb, int nlist_up, const int *nups, int nlist_dn, const int *ndns, ed_opspace **out);
int ed_opspace_dims(const ed_opspace *sp, int64_t *nsup, int64_t *nsdn);
int ed_opspace_destroy(ed_opspace *sp);
/* y = sum_t coeff[t] * (O_{t,last} ... O_{t,1}) x, PROGRAM OPERATOR
 * (compute_operators.f90:28-66): terms with |coeff| <= 1e-14 (the single-
 * precision literal 1.E-14, promoted) are skipped; the
 * factors of term t are ops[5*q .. 5*q+4] for q in [term_off[t],
 * term_off[t+1]) = {code, site1, spin1, site2, spin2} exactly as the
 * reference's _write_operator encodes them (_operators.py:420-462; sites
 * 1-based, spin 1 = up, 2 = down), applied in list order, the first factor
 * first: 1 C_DAGGER_C (c+_{site1} c_{site2}, spin1; operators.f90:1-59),
 * 2 NI, 3 identity, 4 NIM1 (1 - n), 5 SZ_OPE, 6 / 7 C_DAGGER_C_UNRES with
 * site1 on both sides (c+_{up} c_{down} / c+_{down} c_{up}), 9
 * C_DAGGER_C_UNRES(site1, site2, spin2) (c+ of the other spin at site1,
 * c_{site2, spin2}), 10 C_DAGGER, 11 C_, and 12 SZ_BASIS (+S^z, the sz of the
 * reference's basis-element mode, operators_basis.f90:134-145; SZ_OPE, code 5,
 * multiplies by (n_down - n_up)/2); code 8 (SISJ) is refused, nothing in the
 * operator algebra produces it.  Results of a factor outside the
 * listed particle numbers are dropped, as the Fortran drops them.  x, y
 * device FP64 [nsup*nsdn]; work device, at least 2*nsup*nsdn doubles; the
 * term list is host memory, read before anything is enqueued. */
int ed_ops_apply(const ed_opspace *sp, void *stream, int nterms, const int32_t *term_off, const int32_t *ops,
                 const double *coeff, const double *x, double *y, double *work, int64_t work_bytes);

typedef struct ed_batch ed_batch;
int ed_batch_create(int ninst, ed_sector *const *secs, ed_batch **out);
/* ed_batch_create with the H*v work split chosen by the caller: rows of one
 * instance per CTA, 4, 8 (the default of ed_batch_create) or 16.  More rows
 * share each hop-table load among more rows but take more shared memory per
 * CTA; pyhub_gb300 times the three on the actual batch and keeps the fastest.
 * No reference counterpart (a launch parameter of this engine). */
int ed_batch_create_rows(int ninst, ed_sector *const *secs, int rows, ed_batch **out);
int ed_batch_rows(const ed_batch *b);
int ed_batch_destroy(ed_batch *b);
/* total elements of one concatenated vector, per-instance offsets and sizes
 * (nsdn_i*ld_i), and the CTA count of one step (scratch sizing). */
int ed_batch_layout(const ed_batch *b, int64_t *total, int64_t *offsets, int64_t *sizes, int64_t *nblocks);
int64_t ed_batch_scratch_bytes(const ed_batch *b);
/* y_i = H_i x_i for every instance in one launch (the batched Lanczos
 * step's H*v kernel alone), x and y concatenated in the batch layout with
 * zero row padding (y's padding is written as zero).  HPROD
 * (hprod_hubbard.f90:17-118) applied to each instance's sector; scratch as
 * for ed_batch_lanczos. */
int ed_batch_hv(ed_batch *b, void *stream, int dtype, const void *x, void *y, void *scratch, int64_t scratch_bytes);
/* Run nsteps Lanczos steps of every instance from the start vectors x0
 * (concatenated, zero padding).  work: 3*total elements (two Krylov vectors
 * and H*v).  alpha: device FP64 [ninst][nsteps]; beta: device FP64
 * [ninst][nsteps+1] with beta[i][0] = ||x0_i|| and beta[i][k] the coupling of
 * steps k-1 and k.  Enqueues kernels only (no host synchronisation), so the
 * call can be captured in a CUDA graph. */
int ed_batch_lanczos(ed_batch *b, void *stream, int dtype, void *work, const void *x0, int nsteps,
                     double *alpha, double *beta, void *scratch, int64_t scratch_bytes);
/* ed_batch_lanczos (kept == NULL; work: 3*total elements) or
 * ed_batch_lanczos_kept (kept: (nsteps+1)*total elements; work: y, total
 * elements) as ONE persistent cooperative launch that runs every step of
 * every instance: CTAs walk a phase-major list of (phase, CTA-block) items,
 * each waiting until its instance has finished the previous phase, and the
 * last CTA of an instance to finish a phase forms that instance's scalars.
 * The instances are split into two groups one phase apart, so the H*v of
 * one group runs beside the update of the other.  alpha/beta are
 * bit-identical to the four-launch form.  Every wait is bounded (10 s of GPU
 * time unless ed_batch_persistent_watchdog sets another limit); a run that
 * gives up sets a status that ed_batch_persistent_status returns (0 = ok)
 * and stops.  Enqueues one memset and one launch, so the
 * call can be captured in a CUDA graph.  The per-start-block loops of
 * GF_BANDLANCZOS (spgf_bandlanczos.f90:309-448) for many instances at once. */
int ed_batch_lanczos_persistent(ed_batch *b, void *stream, int dtype, void *work, const void *x0, int nsteps,
                                double *alpha, double *beta, void *kept, void *scratch, int64_t scratch_bytes);
/* Status of the last persistent run that used this scratch (synchronous
 * copy to the host): 0 = completed, 1 = a wait gave up.  No reference
 * counterpart. */
int ed_batch_persistent_status(const ed_batch *b, const void *scratch, int *status);
/* Settings of the batch's later persistent runs: the limit of every wait in
 * seconds of GPU time (0 < wait_seconds <= 60; 10 when never set), and, to
 * test that limit, an instance whose first H*v phase never completes
 * (stall_instance; -1 = none): the CTAs that wait on it give up after the
 * limit, status 1 is set and the whole grid returns.  Host-side only.  No
 * reference counterpart. */
int ed_batch_persistent_watchdog(ed_batch *b, double wait_seconds, int stall_instance);
/* Replay of ed_batch_lanczos from the same x0 that also accumulates, per
 * instance, the Ritz vector out_i += sum_k coef[i][k] q_k (q_k the
 * normalised Lanczos vectors; coef device FP64 [ninst][nsteps], typically the
 * eigenvector of the instance's tridiagonal matrix for its lowest Ritz
 * value).  out: concatenated, same dtype and layout as x0, accumulated into
 * (zero it first).  The replay recomputes bit-identical q_k, so the pair
 * ed_batch_lanczos + ed_batch_ritz is the batched two-pass ground-state
 * Lanczos of LANCZOS/READ_PSI (lanczos.f90:17-86, compute_solver.f90:270-290). */
int ed_batch_ritz(ed_batch *b, void *stream, int dtype, void *work, const void *x0, int nsteps,
                  double *alpha, double *beta, const double *coef, void *out, void *scratch,
                  int64_t scratch_bytes);
/* ed_batch_lanczos with every Krylov vector kept, as the reference keeps them
 * for READ_PSI (lanczos.f90:42-49): u_k (unnormalised, ||u_k|| = beta[i][k])
 * is written to slot k of basis ((nsteps+1)*total elements, slot k starting at
 * k*total); y (total elements) takes the H*v.  Same alpha/beta as
 * ed_batch_lanczos.  Then ed_batch_ritz_sum forms the Ritz vectors in one pass
 * over the kept slots instead of a replay:
 *   out_i = sum_{k<nsteps} coef[i][k] u_k / beta[i][k]  (terms with beta = 0
 *   dropped; coef device FP64 [ninst][nsteps], beta as written by the run;
 *   out written entirely, same dtype and layout as the basis). */
int ed_batch_lanczos_kept(ed_batch *b, void *stream, int dtype, void *basis, void *y, const void *x0,
                          int nsteps, double *alpha, double *beta, void *scratch, int64_t scratch_bytes);
int ed_batch_ritz_sum(ed_batch *b, void *stream, int dtype, const void *basis, int nsteps,
                      const double *coef, const double *beta, void *out);

/* Green's functions from Lanczos coefficients, as continued fractions:
 *   out[i][j] = beta[i][0]^2 / (z - s a_0 - beta[i][1]^2 / (z - s a_1 - ...)),
 *   z = z_j + shift[i], s = sign[i], a_k = alpha[i][k], m levels,
 * i.e. <phi_i|(z - s H)^-1|phi_i> of each instance's start vector.  The
 * reference evaluates the same G(w) from band-Lanczos poles,
 * sum_p w_p / (w - p + i eta) (pole.py:81-88, positions from
 * reduced_quantities.py:84-92).  alpha [n][m], beta [n][m+1], shift, sign [n]
 * device FP64 (shift NULL: 0, sign NULL: +1); z [nz] and out [n][nz] device
 * complex FP64 as (re, im) pairs, 16-byte aligned.  n <= 65535, m <= 3000. */
int ed_cf_eval(void *stream, int n, int m, const double *alpha, const double *beta, int nz,
               const double *z, const double *shift, const double *sign, double *out);

/* ed_multidot without a scratch buffer, for callers that cannot allocate
 * device memory: a host that hands all GPU memory to another runtime's pool,
 * or a plug-in whose host forbids it to call the CUDA allocator, has no way
 * to provide the scratch that ed_multidot needs.  No counterpart in the
 * reference (its dot products run on the CPU, lanczos.f90:53-55).
 * Same arguments and results as ed_multidot.  The partial sums live in a fixed
 * 1 MiB device array inside the library: nvec is limited to 64 (ED_ERR_RANGE
 * beyond), the array is resident on a device from the library module's first
 * use there until the process exits, and calls that overlap on the GPU race
 * because they share it.  Outside a stream capture every call looks up the
 * array's device address (cudaGetSymbolAddress); inside a capture the
 * address found by an earlier call on that device is used, so make one call
 * before any stream capture (a capture without one is refused with
 * ED_ERR_ARG).  No call allocates or frees device memory. */
int ed_multidot_noalloc(void *stream, int dtype, int64_t n, const void *V, int64_t ldv, int nvec,
                        const void *w, const void *z, double *out);

#ifdef __cplusplus
}
#endif
#endif /* PYHUB_ED_H */
