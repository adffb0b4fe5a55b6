// ed_cf.cu -- continued-fraction Green's functions from Lanczos coefficients.
//
// The reference evaluates G(w) from its band-Lanczos poles as
// sum_p w_p / (w - p + i eta) (pyhub/tools/pole.py:81-88, positions placed by
// reduced_quantities.py:84-92).  For a start vector phi with Lanczos
// coefficients alpha_k, beta_k the same function is the continued fraction
//   <phi|(z - s H)^-1|phi> = beta_0^2 / (z - s a_0 - beta_1^2 / (z - s a_1 - ...)),
// evaluated here bottom-up, one thread per (instance, frequency), all levels in
// registers: FP64 arithmetic and one division per level, no intermediate
// arrays.
#include "ed_common.cuh"

namespace ed {

constexpr int kCfThreads = 256;

// Block (blockIdx.y = instance, blockIdx.x = frequency tile).  alpha [n][m],
// beta [n][m+1] FP64; z [nz] and out [n][nz] complex as interleaved (re, im);
// instance i sees z_j + shift[i] and the sign sign[i] (shift 0, sign +1 when
// the arrays are NULL).
__global__ void __launch_bounds__(kCfThreads) cf_eval_kernel(int m, const double *__restrict__ alpha,
                                                             const double *__restrict__ beta, int nz,
                                                             const double2 *__restrict__ z,
                                                             const double *__restrict__ shift,
                                                             const double *__restrict__ sign,
                                                             double2 *__restrict__ out)
{
    extern __shared__ double cf_smem[];
    double *sa = cf_smem;          // [m]   sign * alpha_k
    double *sb = cf_smem + m;      // [m]   beta_{k+1}^2 (the coupling below level k)
    const int64_t i = blockIdx.y;
    const double sg = sign ? sign[i] : 1.0;
    const double sh = shift ? shift[i] : 0.0;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        sa[k] = sg * alpha[i * m + k];
        const double b = (k + 1 < m) ? beta[i * (m + 1) + k + 1] : 0.0;
        sb[k] = b * b;
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nz) return;
    const double2 zz = make_double2(z[j].x + sh, z[j].y);
    double gr = 0.0, gi = 0.0;   // g = 1 / (z - s a_k - b_{k+1}^2 g_{k+1}), from the bottom
    for (int k = m - 1; k >= 0; --k) {
        const double wr = zz.x - sa[k] - sb[k] * gr;
        const double wi = zz.y - sb[k] * gi;
        const double inv = 1.0 / (wr * wr + wi * wi);   // one division per level (the FP64 pipe binds)
        gr = wr * inv;
        gi = -wi * inv;
    }
    const double b0 = beta[i * (m + 1)];
    out[i * nz + j] = make_double2(b0 * b0 * gr, b0 * b0 * gi);
}

}  // namespace ed

using namespace ed;

extern "C" int ed_cf_eval(void *stream, int n, int m, const double *alpha, const double *beta, int nz,
                          const double *z, const double *shift, const double *sign, double *out)
{
    clear_error();
    ED_REQUIRE(n >= 0 && m >= 1 && nz >= 0, "n=%d m=%d nz=%d", n, m, nz);
    ED_REQUIRE(m <= 3000, "m=%d above 3000 levels", m);   // 2m doubles of shared memory
    ED_REQUIRE(n <= 65535, "n=%d above 65535 instances per call", n);
    if (n == 0 || nz == 0) return ED_OK;
    ED_REQUIRE(alpha != nullptr && beta != nullptr && z != nullptr && out != nullptr, "NULL argument");
    ED_REQUIRE((reinterpret_cast<uintptr_t>(z) % 16) == 0 && (reinterpret_cast<uintptr_t>(out) % 16) == 0,
               "z and out must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 grid((unsigned)((nz + kCfThreads - 1) / kCfThreads), (unsigned)n);
    const size_t smem = sizeof(double) * 2 * (size_t)m;
    cf_eval_kernel<<<grid, kCfThreads, smem, st>>>(m, alpha, beta, nz, reinterpret_cast<const double2 *>(z), shift,
                                                   sign, reinterpret_cast<double2 *>(out));
    ED_CHECK_LAUNCH();
    return ED_OK;
}
