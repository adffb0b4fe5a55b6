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
    float *ediag32 = nullptr;  // [n]  the same, rounded to FP32 (FP32 kernels read it directly)
    // The same table in sliced-ELL form for the row pass: strings in slices of
    // 32; slice s holds width[s] slots, slot-major, so that the 32 lanes of a
    // warp read one slot with one coalesced load.  Padding slots point at the
    // string itself with coefficient 0.
    int64_t nslice = 0, ell_slots = 0;
    int32_t *ell_off = nullptr;    // [nslice+1] first slot of each slice
    int32_t *ell_src = nullptr;    // [ell_slots*32]
    float *ell_cf32 = nullptr;
    double *ell_cf64 = nullptr;
    int2 *ell_pk32 = nullptr;      // [ell_slots*32] {src, FP32 coefficient bits}: one 8-byte load per slot
    // Per ordered site pair (J,K), J != K, at index (J-1)*norb + (K-1): the
    // strings u with J occupied and K empty, as {u, u' | sign << 31} with
    // u' = u - J + K and sign = parity of the occupied sites strictly between
    // J and K (the reduced-density kernels walk only the hops that exist).
    int32_t *pl_off = nullptr;     // [norb*norb + 1]
    int2 *pl_ent = nullptr;
    bool owner = true;
};

struct HeisTables {
    int nbond = 0;             // unordered pairs {J,K} with a nonzero flip or zz term
    int8_t bj[kMaxSites * kMaxSites];
    int8_t bk[kMaxSites * kMaxSites];
    double flip_jk[kMaxSites * kMaxSites];   // element for the target with K up, J down
    double flip_kj[kMaxSites * kMaxSites];   // element for the target with J up, K down
    double zz[kMaxSites * kMaxSites];        // J(J,K)+J(K,J) for the SzSz sum
    double dconst = 0.0;                     // 0.5*sum J(J,J) (|.|>tol) + 0.25*sum J(J,J)
};

constexpr int kMaxHalf = 16;    // sites in one half of a Heisenberg sector
constexpr int kMaxAB = 256;     // bonds between the two halves

// Row tables of a Heisenberg sector (see ed_heis.cu): the vector, in the
// reference order, is one row per B-half hole pattern; the row's entries are
// the A-half hole patterns with m holes in colex order.
struct HeisStruct {
    int nA = 0, nB = 0, H = 0, mlo = 0, mhi = 0;
    int64_t nrows = 0, max_len = 0;
    int64_t col_base[kMaxHalf + 2] = {}, ncol[kMaxHalf + 1] = {}, slice_base[kMaxHalf + 2] = {};
    int64_t row_base[kMaxHalf + 2] = {};
    uint32_t *col_pat = nullptr;     // A patterns, concatenated over m
    int32_t *rankA = nullptr;        // [2^nA] colex rank among the patterns of equal popcount
    double *diagA = nullptr;         // A-A zz energy per column
    int32_t *aa_off = nullptr, *aa_src = nullptr;   // sliced ELL of the A-A flips per m
    float *aa_cf32 = nullptr;
    double *aa_cf64 = nullptr;
    uint32_t *row_pat = nullptr;     // B pattern per row (rows in offset order)
    int32_t *row_m = nullptr, *rowidx = nullptr;    // holes in A per row; [2^nB] row of a pattern or -1
    int64_t *row_off = nullptr;
    double *diagB = nullptr;         // B-B zz energy + constant diagonal per row
    float *diagA32 = nullptr, *diagB32 = nullptr;   // the two diagonals rounded to FP32
    int32_t *bb_ptr = nullptr, *bb_src = nullptr;   // B-B flips: neighbour rows per row (CSR)
    float *bb_cf32 = nullptr;
    double *bb_cf64 = nullptr;
    int32_t *rows_of_m = nullptr;    // rows grouped by m
    int2 *aa_pk32 = nullptr;         // A-A flips packed {column, FP32 coefficient bits}
    bool ab_fast = false;            // at most 32 A-B bonds: bits packed per column / row
    uint32_t *col_abbits = nullptr;  // per column: its A bits at the A-B bonds
    uint32_t *row_bbits = nullptr;   // per row: its B bits at the A-B bonds
    int32_t *ab_rank = nullptr;      // [q][column]: rank after flipping A-B bond q's A bit
    int64_t ncols = 0;               // columns over all m (the stride of ab_rank)
    int nab = 0;
    int8_t ab_pa[kMaxAB] = {}, ab_pb[kMaxAB] = {};  // A bit, B bit (relative to nA)
    double ab_fjk[kMaxAB] = {}, ab_fkj[kMaxAB] = {}, ab_zz[kMaxAB] = {};
};

// The U_ijkl interaction of a Hubbard sector (the reference's IS_ULOC=3):
// terms UL(J,K,M,N) c+_{K up} c_{J up} c+_{N down} c_{M down}, grouped by the
// down pair (M,N); one device allocation.
struct UijklTables {
    int ngroups = 0, nterms = 0;
    int4 *groups = nullptr;    // {M, N, first term, count}
    int2 *jk = nullptr;        // {J, K} per term
    double *val = nullptr;     // UL(J,K,M,N) per term
    float *val32 = nullptr;
    void *pool = nullptr;
};

int uijkl_hv(ed_sector *s, cudaStream_t st, int dtype, int64_t ld, const void *x, void *y, double scale);
void uijkl_free(UijklTables *u);

int heis_struct_build(ed_sector *s);
void heis_struct_free(HeisStruct *hs);
int heis_struct_hv(ed_sector *s, cudaStream_t st, int dtype, const void *x, void *y, double scale, double *dots,
                   double *partials);
int heis_struct_rdm(ed_sector *s, cudaStream_t st, int dtype, const void *bra, const void *ket, int npairs,
                    const int32_t *pairs, double *out, double *scratch, int max_blocks);
int launch_reduce(const double *partials, int nblocks, int m, double *out, cudaStream_t st);

}  // namespace ed

// Product space of the generic operator engine (operators.x,
// compute_operators.f90:8-25): the up strings of every listed up-particle
// number concatenated in list order (each block in HILBERT order), the same
// for down; state (d, u) at d * nsup + u.
struct ed_opspace {
    int norb = 0;
    int64_t nsup = 0, nsdn = 0;
    int64_t up_off[ed::kMaxSites + 1];   // first index of the strings with n up particles, -1 when n is not listed
    int64_t dn_off[ed::kMaxSites + 1];
    uint32_t *ustr = nullptr, *dstr = nullptr;   // device: the concatenated lists
    const uint32_t *lut = nullptr;               // device rank table, shared with the sectors
    void *pool = nullptr;
    int device = 0;
};

struct ed_sector {
    int kind = ED_HUBBARD;
    int norb = 0, nup = 0, ndn = 0;
    int64_t nsup = 0, nsdn = 0, dim = 0;
    ed::HopTable up, dn;           // dn shares up's arrays when nup == ndn
    double u_site[ed::kMaxSites];  // U per site, indexed by bit (bit b <-> site norb-b)
    bool u_uniform = true;
    double u_value = 0.0;
    ed::HeisTables heis;
    ed::HeisStruct *hs = nullptr;  // Heisenberg row tables
    ed::UijklTables *uijkl = nullptr;   // U_ijkl terms (ed_sector_set_uijkl), else NULL
    // colex rank of an empty-site pattern h (bit j: site j+1 empty) in byte
    // chunks, shared by every kernel that ranks strings on the fly:
    // rank = sum_b lut[b][popcount(h & (2^(8b)-1))][byte b of h]
    uint32_t *lut = nullptr;   // [4][33][256], shared by all sectors of the device
    void *pool = nullptr;      // the one device allocation holding this sector's hop tables
    double t_host[ed::kMaxSites * ed::kMaxSites];
    double j_host[ed::kMaxSites * ed::kMaxSites];
    int device = 0;
};

namespace ed {

// ------------------------------------------------------------ device helpers

// Asynchronous global -> shared copy of one element (cp.async, 4 or 8 bytes):
// a thread's copies are all in flight at once; cp_async_wait_all precedes the
// barrier that publishes them to the CTA.
template <typename T> __device__ __forceinline__ void cp_async_elem(T *smem, const T *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

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

// Empty-site pattern of a string of norb sites (site POS in bit norb-POS):
// bit j set when site j+1 is empty.
__device__ __forceinline__ uint32_t holes_dev(uint32_t s, int norb)
{
    const uint32_t full = (norb >= 32) ? 0xFFFFFFFFu : ((1u << norb) - 1u);
    return __brev(~s & full) >> (32 - norb);
}

// Index of a string in the reference order from its empty-site pattern.
__device__ __forceinline__ uint32_t rank_holes(const uint32_t *__restrict__ lut, uint32_t h)
{
    uint32_t r = 0;
    int c = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const uint32_t byte = (h >> (8 * b)) & 255u;
        r += __ldg(lut + (b * 33 + c) * 256 + byte);
        c += __popc(byte);
    }
    return r;
}

}  // namespace ed
