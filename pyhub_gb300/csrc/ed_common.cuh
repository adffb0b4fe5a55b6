// ed_common.cuh -- shared definitions of the GB300 exact-diagonalisation
// engine: error state, the device sector object and small device helpers.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdarg>
#include <cstdio>

#include "../../include/pyhub_ed.h"

namespace ed {

// Thread-local error message behind ed_last_error().
void set_error(const char *fmt, ...);
void clear_error();

#define ED_CHECK_CUDA(expr)                                                              \
    do {                                                                                 \
        cudaError_t _e = (expr);                                                         \
        if (_e != cudaSuccess) {                                                         \
            ::ed::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e),      \
                            __FILE__, __LINE__);                                         \
            return ED_ERR_CUDA;                                                          \
        }                                                                                \
    } while (0)

#define ED_CHECK_LAUNCH()                                                                \
    do {                                                                                 \
        cudaError_t _e = cudaGetLastError();                                             \
        if (_e != cudaSuccess) {                                                         \
            ::ed::set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(_e),  \
                            __FILE__, __LINE__);                                         \
            return ED_ERR_CUDA;                                                          \
        }                                                                                \
    } while (0)

#define ED_REQUIRE(cond, ...)                                                            \
    do {                                                                                 \
        if (!(cond)) {                                                                   \
            ::ed::set_error(__VA_ARGS__);                                                \
            return ED_ERR_ARG;                                                           \
        }                                                                                \
    } while (0)

constexpr int kMaxSites = 32;
// The reference compares |t| against the REAL*4 literal 1.E-14.
constexpr double kTol14 = (double)1.0e-14f;

// Gather-form hop table of one spin species: for every target string p the
// sources q = p - bit(K) + bit(J) (K occupied, J empty in p, |T(J,K)| >= tol)
// with coefficient sign * T(J,K), sign = (-1)^(occupied sites strictly
// between J and K).  CSR over targets.
struct HopTable {
    int norb = 0, ne = 0;
    int64_t n = 0;          // strings
    int64_t nnz = 0;
    uint32_t *str = nullptr;   // [n]
    int32_t *ptr = nullptr;    // [n+1]
    int32_t *src = nullptr;    // [nnz]
    float *cf32 = nullptr;     // [nnz]
    double *cf64 = nullptr;    // [nnz]
    double *ediag = nullptr;   // [n]  sum of T(J,J) over occupied J (|T(J,J)| >= tol)
    bool owner = true;
};

struct HeisTables {
    // colex rank of the empty-site pattern in byte chunks:
    // rank = sum_b lut[b][pop(lower chunks)][byte_b]
    uint32_t *lut = nullptr;   // [4][33][256]
    int nbond = 0;             // unordered pairs {J,K} with a nonzero flip or zz term
    int8_t bj[kMaxSites * kMaxSites];
    int8_t bk[kMaxSites * kMaxSites];
    double flip_jk[kMaxSites * kMaxSites];   // element for the target with K up, J down
    double flip_kj[kMaxSites * kMaxSites];   // element for the target with J up, K down
    double zz[kMaxSites * kMaxSites];        // J(J,K)+J(K,J) for the SzSz sum
    double dconst = 0.0;                     // 0.5*sum J(J,J) (|.|>tol) + 0.25*sum J(J,J)
};

}  // namespace ed

struct ed_sector {
    int kind = ED_HUBBARD;
    int norb = 0, nup = 0, ndn = 0;
    int64_t nsup = 0, nsdn = 0, dim = 0;
    ed::HopTable up, dn;           // dn shares up's arrays when nup == ndn
    double u_site[ed::kMaxSites];  // U per site, indexed by bit (bit b <-> site norb-b)
    bool u_uniform = true;
    double u_value = 0.0;
    ed::HeisTables heis;
    double t_host[ed::kMaxSites * ed::kMaxSites];
    double j_host[ed::kMaxSites * ed::kMaxSites];
    int device = 0;
};

namespace ed {

// ------------------------------------------------------------ device helpers

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sumf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

int num_sms();

}  // namespace ed
