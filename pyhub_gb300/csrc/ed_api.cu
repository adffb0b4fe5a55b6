// ed_api.cu -- composite entry points of the C ABI for a host that drives
// the engine without the Python layer (the reference's own Fortran, or C):
// one full-reorthogonalisation Lanczos step, the assembled one-body
// densities / double occupancies / spin correlations of ONE_RDM, TWO_RDM and
// J_SPIN, and the Hellmann-Feynman gradient of the energy.  Each one chains
// the kernels of the other files on one stream.
#include "ed_common.cuh"

#include <cstring>
#include <vector>

namespace ed {

static int64_t vec_len(const ed_sector *s, int64_t ld)
{
    return (s->kind == ED_HUBBARD) ? s->nsdn * ld : s->dim;
}

static int64_t rdm1_pairs(const ed_sector *s)
{
    return (s->kind == ED_HUBBARD) ? (int64_t)s->norb * (s->norb + 1) / 2 : (int64_t)s->norb * s->norb;
}

}  // namespace ed

using namespace ed;

extern "C" int64_t ed_lanczos_step_scratch_bytes(const ed_sector *s, int mmax)
{
    if (!s || mmax < 1) return 0;
    const int64_t head = (2 * (int64_t)(mmax + 1) + 2 + (mmax + 1)) * (int64_t)sizeof(double);
    return (head + 255) / 256 * 256 + ed_scratch_bytes(s->nsdn * s->nsup, mmax + 1);
}

extern "C" int ed_lanczos_step(ed_sector *s, void *stream, int dtype, int64_t ld, void *V, int64_t ldv, int k,
                               int mmax, void *w, double *state, double *alpha, double *beta, void *scratch,
                               int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(s != nullptr, "sector is NULL");
    ED_REQUIRE(V != nullptr && w != nullptr && state != nullptr && alpha != nullptr && beta != nullptr &&
                   scratch != nullptr, "NULL argument");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(mmax >= 1 && mmax <= 8192 && k >= 0 && k < mmax, "step k=%d outside 0..mmax-1 (mmax=%d)", k, mmax);
    const int64_t need = ed_lanczos_step_scratch_bytes(s, mmax);
    ED_REQUIRE(scratch_bytes >= need, "scratch of %lld bytes is below %lld", (long long)scratch_bytes,
               (long long)need);
    const int64_t n = vec_len(s, ld);
    ED_REQUIRE(ldv >= n, "basis row stride %lld below the vector length %lld", (long long)ldv, (long long)n);
    const size_t esz = (dtype == ED_F32) ? 4 : 8;
    // scratch: [dots 2(mmax+1)][nrm 2][coef mmax+1] then the kernels' own partials
    double *dots = static_cast<double *>(scratch);
    double *nrm = dots + 2 * (mmax + 1);
    double *coef = nrm + 2;
    const int64_t head = ((2 * (int64_t)(mmax + 1) + 2 + (mmax + 1)) * (int64_t)sizeof(double) + 255) / 256 * 256;
    void *rest = static_cast<unsigned char *>(scratch) + head;
    const int64_t rest_bytes = scratch_bytes - head;
    unsigned char *vb = static_cast<unsigned char *>(V);
    const void *uk = vb + (size_t)k * (size_t)ldv * esz;
    void *unext = vb + (size_t)(k + 1) * (size_t)ldv * esz;
    int rc = ed_hv(s, stream, dtype, ld, uk, w, 1.0, nullptr, rest, rest_bytes);
    if (rc) return rc;
    rc = ed_multidot(stream, dtype, n, V, ldv, k + 1, w, uk, dots, rest, rest_bytes);
    if (rc) return rc;
    rc = ed_lanczos_coef(stream, k, mmax, dots, nrm, state, coef, alpha, beta);
    if (rc) return rc;
    return ed_update_wscaled(stream, dtype, dtype, n, V, ldv, k + 1, coef, state + 2 + k, w, unext, nrm, rest,
                             rest_bytes);
}

extern "C" int64_t ed_rdm1_scratch_bytes(const ed_sector *s)
{
    if (!s) return 0;
    const int64_t np = rdm1_pairs(s);
    return ed_rdm_scratch_bytes((int)np) + (6 * np * (int64_t)sizeof(double) + 255) / 256 * 256;
}

// copy_down: the reference's shortcut for N_up == N_down (the down matrix is the up one,
// static_rq.f90:237-239); without it the down hops are summed too
static int rdm1_impl(ed_sector *s, void *stream, int dtype, int64_t ld, const void *psi, double *gamma,
                     double *docc, double *sisj, void *scratch, int64_t scratch_bytes, bool copy_down)
{
    ED_REQUIRE(s != nullptr && psi != nullptr && scratch != nullptr, "NULL argument");
    ED_REQUIRE(s->kind == ED_HEISENBERG || (gamma != nullptr && docc != nullptr),
               "a Hubbard sector needs gamma and docc");
    ED_REQUIRE(sisj != nullptr, "sisj is NULL");
    const int64_t need = ed_rdm1_scratch_bytes(s);
    ED_REQUIRE(scratch_bytes >= need, "scratch of %lld bytes is below %lld", (long long)scratch_bytes,
               (long long)need);
    const int N = s->norb;
    const int np = (int)rdm1_pairs(s);
    std::vector<int32_t> pairs;
    pairs.reserve(2 * (size_t)np);
    if (s->kind == ED_HUBBARD) {
        for (int J = 1; J <= N; ++J)
            for (int K = 1; K <= J; ++K) { pairs.push_back(J); pairs.push_back(K); }   // K <= J, as ONE_RDM
    } else {
        for (int J = 1; J <= N; ++J)
            for (int K = 1; K <= N; ++K) { pairs.push_back(J); pairs.push_back(K); }
    }
    const int64_t outb = (6 * (int64_t)np * (int64_t)sizeof(double) + 255) / 256 * 256;
    double *out = static_cast<double *>(scratch);
    void *rest = static_cast<unsigned char *>(scratch) + outb;
    const bool dn = !copy_down || s->nup != s->ndn;
    const int flags = (s->kind == ED_HUBBARD) ? (2 | (dn ? 1 : 0)) : 0;
    int rc = ed_rdm(s, stream, dtype, ld, psi, psi, np, pairs.data(), flags, out, rest, scratch_bytes - outb);
    if (rc) return rc;
    const int nq = (s->kind == ED_HUBBARD) ? 6 : 2;
    std::vector<double> h((size_t)nq * np);
    cudaStream_t st = (cudaStream_t)stream;
    ED_CHECK_CUDA(cudaMemcpyAsync(h.data(), out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    ED_CHECK_CUDA(cudaStreamSynchronize(st));
    if (s->kind == ED_HUBBARD) {
        // q[p][0..3] then q[p][4..5] (the layout of ed_rdm); symmetrised as the reference
        // (static_rq.f90:161-241, 307-316, 331-393)
        auto q = [&](int p, int c) { return c < 4 ? h[(size_t)p * 4 + c] : h[(size_t)4 * np + (size_t)p * 2 + (c - 4)]; };
        double *gu = gamma, *gd = gamma + (size_t)N * N;
        std::memset(gamma, 0, sizeof(double) * 2 * (size_t)N * N);
        int p = 0;
        for (int J = 0; J < N; ++J)
            for (int K = 0; K <= J; ++K, ++p) {
                if (J == K) {
                    const double nu = q(p, 0), nd = q(p, 2), d = q(p, 3), zz = q(p, 1);
                    gu[J * N + J] = nu;
                    gd[J * N + J] = nd;
                    docc[J] = d;
                    sisj[J * N + J] = 0.5 * (nu - d) + 0.5 * (nd - d) + zz;
                } else {
                    gu[J * N + K] = gu[K * N + J] = q(p, 0);
                    gd[J * N + K] = gd[K * N + J] = q(p, 4);
                    sisj[J * N + K] = sisj[K * N + J] = q(p, 5) + q(p, 1);
                }
            }
        if (!dn) std::memcpy(gd, gu, sizeof(double) * (size_t)N * N);   // static_rq.f90:237-239
    } else {
        // SMATRIX(J,K) = q0 + q1; the reference's Python reads its transpose (static_rq_heis.f90:66-114)
        for (int J = 0; J < N; ++J)
            for (int K = 0; K < N; ++K) {
                const int p = J * N + K;
                sisj[K * N + J] = h[(size_t)p * 2] + h[(size_t)p * 2 + 1];
            }
    }
    return ED_OK;
}

extern "C" int ed_rdm1(ed_sector *s, void *stream, int dtype, int64_t ld, const void *psi, double *gamma,
                       double *docc, double *sisj, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    return rdm1_impl(s, stream, dtype, ld, psi, gamma, docc, sisj, scratch, scratch_bytes, true);
}

extern "C" int ed_hf_grad(ed_sector *s, void *stream, int dtype, int64_t ld, const void *psi, int nbonds,
                          const int32_t *bonds, double *g_t, double *g_u, double *g_eps, void *scratch,
                          int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(s != nullptr && s->kind == ED_HUBBARD, "the gradient is defined for a Hubbard sector");
    ED_REQUIRE(nbonds >= 0 && (nbonds == 0 || (bonds != nullptr && g_t != nullptr)), "bond list");
    ED_REQUIRE(g_u != nullptr && g_eps != nullptr, "NULL output");
    const int N = s->norb;
    for (int b = 0; b < nbonds; ++b)
        ED_REQUIRE(bonds[2 * b] >= 1 && bonds[2 * b] <= N && bonds[2 * b + 1] >= 1 && bonds[2 * b + 1] <= N &&
                       bonds[2 * b] != bonds[2 * b + 1], "bond %d (%d,%d) outside 1..%d or on one site", b,
                   bonds[2 * b], bonds[2 * b + 1], N);
    std::vector<double> gamma(2 * (size_t)N * N), docc((size_t)N), sm((size_t)N * N);
    const int rc = rdm1_impl(s, stream, dtype, ld, psi, gamma.data(), docc.data(), sm.data(), scratch, scratch_bytes,
                             false);
    if (rc) return rc;
    const double *gu = gamma.data(), *gd = gamma.data() + (size_t)N * N;
    // E = sum_{ij,s} t_ij <c+_is c_js> + sum_i U_i <n_i,up n_i,down> with t_ij = t_ji one parameter
    // per bond and t_ii the on-site energy
    for (int b = 0; b < nbonds; ++b) {
        const int i = bonds[2 * b] - 1, j = bonds[2 * b + 1] - 1;
        g_t[b] = 2.0 * (gu[i * N + j] + gd[i * N + j]);
    }
    for (int i = 0; i < N; ++i) {
        g_u[i] = docc[i];
        g_eps[i] = gu[i * N + i] + gd[i * N + i];
    }
    return ED_OK;
}
