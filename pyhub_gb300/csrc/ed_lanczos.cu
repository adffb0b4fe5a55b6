// ed_lanczos.cu -- the scalar work of a full-reorthogonalisation Lanczos step,
// kept on the device so that a step enqueues without a host synchronisation.
//
// The reference's LANCZOS (lanczos.f90:50-58) forms alpha_k and beta_k from
// two dot products on the host.  The engine's step also projects H v_k on
// every stored basis vector (delayed classical Gram-Schmidt with the exact
// Gram matrix G of the stored, rounded basis):
//   w = H u_k                                   (ed_hv, unscaled)
//   a_j = <u_j, w>, b_j = <u_j, u_k>            (ed_multidot, one pass)
//   g_j = s_j s_k b_j     (row k of G, v_j = s_j u_j the normalised vectors)
//   c_j = s_j s_k a_j     (= <v_j, H v_k>)
//   y = G^{-1} c,  coef_j = y_j s_j
//   u_{k+1} = s_k w - sum_j coef_j u_j          (ed_update_wscaled)
//   beta_k = ||u_{k+1}||,  s_{k+1} = 1 / beta_k,  alpha_k = c_k.
// G is solved through its inverse Cholesky factor Linv (G = L L^T), grown by
// one row per step: with l = Linv g[0:k] and lam = sqrt(g_k - l.l),
//   Linv[k][0:k] = -(l^T Linv) / lam,  Linv[k][k] = 1 / lam,
// and y = Linv^T (Linv c).  G is within rounding of the identity, so the
// explicit inverse is as accurate as the triangular solves it replaces.
#include "ed_common.cuh"

namespace ed {

constexpr int kCoefThreads = 512;
constexpr int kLanczosMax = 8192;   // largest step count a state can hold

// State layout (FP64): [0] stop code, [1] largest |G - I| entry seen,
// [2 .. 2+mmax] scales s_j, then Linv as (mmax+1) x (mmax+1) row-major, then
// four work vectors of mmax+1 entries (Gram row, projections, Linv g, Linv c).
__host__ __device__ inline int64_t lz_linv_off(int mmax) { return 3 + (int64_t)mmax; }
__host__ __device__ inline int64_t lz_work_off(int mmax) { return lz_linv_off(mmax) + (int64_t)(mmax + 1) * (mmax + 1); }

__device__ __forceinline__ double block_sum_d(double v, double *red)
{
    v = warp_sum(v);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

__device__ __forceinline__ double block_max_d(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

// One CTA.  Part 1 (every call, k >= 1): beta_{k-1} and s_k from nrm, with
// the breakdown test of the host loop (beta <= 1e-13 max(1, |alpha|)).
// Part 1 is idempotent: a second call for the same k with the same nrm writes
// the same beta_{k-1} and s_k.  The host's look-ahead relies on it (a run that
// stops at a check has already enqueued the next step, whose part 1 rewrites
// them before the Ritz vector is formed).  Part 2
// (dots != NULL): G row k, Linv row k, coef and alpha_k; it also stops the run
// when u_k is numerically dependent on the basis.  Once stopped, coef is
// written as zeros (and s stays 0), so the vectors that follow are zero and
// finite until the host sees the stop code.
__global__ void __launch_bounds__(kCoefThreads) lanczos_coef_kernel(int k, int mmax, const double *__restrict__ dots,
                                                                    const double *__restrict__ nrm,
                                                                    double *__restrict__ state,
                                                                    double *__restrict__ coef,
                                                                    double *__restrict__ alpha,
                                                                    double *__restrict__ beta)
{
    __shared__ double red[32];
    __shared__ int stop;
    double *s = state + 2;
    double *Linv = state + lz_linv_off(mmax);
    const int64_t ldl = mmax + 1;
    double *g = state + lz_work_off(mmax);   // [k+1] Gram row
    double *c = g + ldl;                     // [k+1] projections
    double *l = c + ldl;                     // [k]   Linv g
    double *z = l + ldl;                     // [k+1] Linv c
    if (threadIdx.x == 0) {
        if (k >= 1 && state[0] == 0.0) {
            const double nb = nrm[0];
            const double bk = sqrt(fmax(nb, 0.0));
            if (!isfinite(nb)) {
                state[0] = -(double)k;
                s[k] = 0.0;
            } else {
                beta[k - 1] = bk;
                if (bk <= 1e-13 * fmax(1.0, fabs(alpha[k - 1]))) {
                    state[0] = (double)k;
                    s[k] = 0.0;
                } else {
                    s[k] = 1.0 / bk;
                }
            }
        }
        stop = (state[0] != 0.0) ? 1 : 0;
    }
    __syncthreads();
    if (dots == nullptr) return;
    if (stop) {
        for (int j = threadIdx.x; j <= k; j += blockDim.x) coef[j] = 0.0;
        return;
    }
    const double sk = s[k];
    for (int j = threadIdx.x; j <= k; j += blockDim.x) {
        const double sj = s[j];
        g[j] = sj * sk * dots[k + 1 + j];
        c[j] = sj * sk * dots[j];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    // l = Linv[0:k][0:k] g[0:k]  (lower triangular, one warp per row)
    for (int i = warp; i < k; i += nwarps) {
        const double *row = Linv + (int64_t)i * ldl;
        double t = 0.0;
        for (int j = lane; j <= i; j += 32) t += row[j] * g[j];
        t = warp_sum(t);
        if (lane == 0) l[i] = t;
    }
    __syncthreads();
    double ll = 0.0, off = 0.0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        ll += l[i] * l[i];
        off = fmax(off, fabs(g[i]));
    }
    if (threadIdx.x == 0) off = fmax(off, fabs(g[k] - 1.0));
    ll = block_sum_d(ll, red);
    off = block_max_d(off, red);
    // a healthy step has lam^2 = g_k - |l|^2 within rounding of 1; below g_k / 2 the stored
    // vector lies mostly inside the span of the basis (a Krylov space exhausted to rounding
    // noise): the run stops with k steps, before the inverse factor would blow up
    if (k >= 1 && !(g[k] - ll >= 0.5 * g[k])) {
        for (int j = threadIdx.x; j <= k; j += blockDim.x) coef[j] = 0.0;
        if (threadIdx.x == 0) state[0] = (double)k;
        return;
    }
    const double lam = sqrt(fmax(g[k] - ll, 1e-300));
    // new row k of Linv: -(l^T Linv[0:k][0:k]) / lam, then 1 / lam
    double *rowk = Linv + (int64_t)k * ldl;
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        double t = 0.0;
        for (int i = j; i < k; ++i) t += l[i] * Linv[(int64_t)i * ldl + j];
        rowk[j] = -t / lam;
    }
    if (threadIdx.x == 0) {
        rowk[k] = 1.0 / lam;
        state[1] = fmax(state[1], off);
    }
    __syncthreads();
    // z = Linv[0:k+1][0:k+1] c
    for (int i = warp; i <= k; i += nwarps) {
        const double *row = Linv + (int64_t)i * ldl;
        double t = 0.0;
        for (int j = lane; j <= i; j += 32) t += row[j] * c[j];
        t = warp_sum(t);
        if (lane == 0) z[i] = t;
    }
    __syncthreads();
    // y = Linv^T z, coef_j = y_j s_j
    for (int j = threadIdx.x; j <= k; j += blockDim.x) {
        double t = 0.0;
        for (int i = j; i <= k; ++i) t += Linv[(int64_t)i * ldl + j] * z[i];
        coef[j] = t * s[j];
    }
    if (threadIdx.x == 0) alpha[k] = c[k];
}

}  // namespace ed

using namespace ed;

extern "C" int64_t ed_lanczos_state_doubles(int mmax)
{
    if (mmax < 1 || mmax > kLanczosMax) return -1;
    return lz_work_off(mmax) + 4 * (int64_t)(mmax + 1);
}

extern "C" int ed_lanczos_coef(void *stream, int k, int mmax, const double *dots, const double *nrm, double *state,
                               double *coef, double *alpha, double *beta)
{
    clear_error();
    ED_REQUIRE(mmax >= 1 && mmax <= kLanczosMax, "mmax=%d outside 1..%d", mmax, kLanczosMax);
    ED_REQUIRE(k >= 0 && k <= mmax, "step %d outside 0..%d", k, mmax);
    ED_REQUIRE(state != nullptr && alpha != nullptr && beta != nullptr, "state, alpha or beta is NULL");
    ED_REQUIRE(k == 0 || nrm != nullptr, "nrm is NULL");
    ED_REQUIRE(dots == nullptr || (coef != nullptr && k < mmax), "coef is NULL or step %d has no next vector", k);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    lanczos_coef_kernel<<<1, kCoefThreads, 0, st>>>(k, mmax, dots, nrm, state, coef, alpha, beta);
    ED_CHECK_LAUNCH();
    return ED_OK;
}
