// ed_uijkl.cu -- the general two-body interaction of a Hubbard sector
// (the reference's IS_ULOC=3 path) and its two-body density.
//
// H_U = sum UL(J,K,M,N) c+_{K up} c_{J up} c+_{N down} c_{M down} over the
// (J,K) with UPARTIAL(J,K) >= 1e-14 and |UL(J,K,M,N)| >= 1e-14
// (hprod_hubbard.f90:37,62-86), where the reference reads the Python tensor U
// (C order) as UL(J,K,M,N) = U[N-1][M-1][K-1][J-1] and
// UPARTIAL(J,K) = sum_cd U[K-1][J-1][c][d]^2 (core_solver.py:143-147,
// compute_solver.f90:129-138).  A term moves one up particle J->K and one
// down particle M->N (J == K: n_J), with the sign
// ANTICOM(J,u) ANTICOM(K,u') ANTICOM(M,d) ANTICOM(N,d') of the reference.
//
// The product is formed in gather form: one CTA per output row d' (down
// string), threads over output columns u'; for each down pair (M,N) the
// source row is found once per row (the test is uniform over the CTA), for
// each term of the pair every thread tests its own up string, ranks the
// source column and gathers it.  Work per element is the number of terms, so
// this path suits the small clusters the interaction is used on.
//
// The two-body density DBL_OCC(J,K,M,N) = sum AC AC2 BRA(source) KET(target)
// (TWO_RDM, static_rq.f90:256-306) runs one warp per source row, lanes over
// its columns, one grid row per (J,K,M,N).
#include "ed_common.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace ed {

// (-1)^(occupied sites 1..pos-1) of a string (site p in bit norb-p)
__device__ __forceinline__ int anticom_par(int norb, int pos, uint32_t s)
{
    const uint32_t mask = (uint32_t)((((uint64_t)1 << (pos - 1)) - 1) << (norb - pos + 1));
    return __popc(s & mask) & 1;
}

// Source of the hop a->b onto target string st (KINOP(src, a, b) == st):
// returns false when no string maps onto st.
__device__ __forceinline__ bool hop_source(int norb, uint32_t st, int a, int b, uint32_t &src)
{
    const uint32_t ba = 1u << (norb - a), bb = 1u << (norb - b);
    if (a == b) {
        src = st;
        return (st & ba) != 0;
    }
    if (!(st & bb) || (st & ba)) return false;
    src = st ^ ba ^ bb;
    return true;
}

// Target of the hop a->b from source string s (KINOP(s, a, b)).
__device__ __forceinline__ bool hop_target(int norb, uint32_t s, int a, int b, uint32_t &dst)
{
    const uint32_t ba = 1u << (norb - a), bb = 1u << (norb - b);
    if (!(s & ba)) return false;
    if (a == b) {
        dst = s;
        return true;
    }
    if (s & bb) return false;
    dst = s ^ ba ^ bb;
    return true;
}

template <typename T>
__global__ void __launch_bounds__(256) uijkl_hv_kernel(const T *__restrict__ x, T *__restrict__ y, int64_t ld,
                                                       int64_t nsup, int64_t nsdn, int norb,
                                                       const uint32_t *__restrict__ ustr,
                                                       const uint32_t *__restrict__ dstr,
                                                       const uint32_t *__restrict__ lut,
                                                       const int4 *__restrict__ groups, int ngroups,
                                                       const int2 *__restrict__ jk, const T *__restrict__ val,
                                                       T scale)
{
    for (int64_t d2 = blockIdx.x; d2 < nsdn; d2 += gridDim.x) {
        const uint32_t sd2 = __ldg(dstr + d2);
        for (int64_t u2 = threadIdx.x; u2 < nsup; u2 += blockDim.x) {
            const uint32_t su2 = __ldg(ustr + u2);
            T acc = 0;
            for (int g = 0; g < ngroups; ++g) {
                const int4 gr = __ldg(groups + g);
                uint32_t sd;
                if (!hop_source(norb, sd2, gr.x, gr.y, sd)) continue;
                const int p2 = anticom_par(norb, gr.x, sd) ^ anticom_par(norb, gr.y, sd2);
                const T *xr = x + (int64_t)rank_holes(lut, holes_dev(sd, norb)) * ld;
                for (int q = gr.z; q < gr.z + gr.w; ++q) {
                    const int2 t = __ldg(jk + q);
                    uint32_t su;
                    if (!hop_source(norb, su2, t.x, t.y, su)) continue;
                    const int p = p2 ^ anticom_par(norb, t.x, su) ^ anticom_par(norb, t.y, su2);
                    const T v = __ldg(val + q) * __ldg(xr + rank_holes(lut, holes_dev(su, norb)));
                    acc += p ? -v : v;
                }
            }
            y[d2 * ld + u2] += scale * acc;
        }
    }
}

int uijkl_hv(ed_sector *s, cudaStream_t st, int dtype, int64_t ld, const void *x, void *y, double scale)
{
    const UijklTables *u = s->uijkl;
    if (!u || u->nterms == 0 || s->dim == 0) return ED_OK;
    int64_t blocks = s->nsdn;
    if (blocks > (int64_t)num_sms() * 16) blocks = (int64_t)num_sms() * 16;
    if (dtype == ED_F32)
        uijkl_hv_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
            static_cast<const float *>(x), static_cast<float *>(y), ld, s->nsup, s->nsdn, s->norb, s->up.str,
            s->dn.str, s->lut, u->groups, u->ngroups, u->jk, u->val32, (float)scale);
    else
        uijkl_hv_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
            static_cast<const double *>(x), static_cast<double *>(y), ld, s->nsup, s->nsdn, s->norb, s->up.str,
            s->dn.str, s->lut, u->groups, u->ngroups, u->jk, u->val, scale);
    ED_CHECK_LAUNCH();
    return ED_OK;
}

void uijkl_free(UijklTables *u)
{
    if (!u) return;
    if (u->pool) cudaFree(u->pool);
    delete u;
}

constexpr int kDblWarps = 8;

template <typename T>
__global__ void __launch_bounds__(kDblWarps * 32) dbl_occ_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                                 int64_t ld, int64_t nsup, int64_t nsdn, int norb,
                                                                 const uint32_t *__restrict__ ustr,
                                                                 const uint32_t *__restrict__ dstr,
                                                                 const uint32_t *__restrict__ lut,
                                                                 const int4 *__restrict__ quads, int nquads,
                                                                 double *__restrict__ partials)
{
    const int q = blockIdx.y;
    const int4 c = __ldg(quads + q);   // J, K, M, N
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int64_t d = (int64_t)blockIdx.x * kDblWarps + warp; d < nsdn; d += (int64_t)gridDim.x * kDblWarps) {
        const uint32_t sd = __ldg(dstr + d);
        uint32_t sd2;
        if (!hop_target(norb, sd, c.z, c.w, sd2)) continue;
        const int p2 = anticom_par(norb, c.z, sd) ^ anticom_par(norb, c.w, sd2);
        const T *kr = ket + (int64_t)rank_holes(lut, holes_dev(sd2, norb)) * ld;
        const T *br = bra + d * ld;
        for (int64_t u = lane; u < nsup; u += 32) {
            const uint32_t su = __ldg(ustr + u);
            uint32_t su2;
            if (!hop_target(norb, su, c.x, c.y, su2)) continue;
            const int p = p2 ^ anticom_par(norb, c.x, su) ^ anticom_par(norb, c.y, su2);
            const double v = (double)__ldg(br + u) * (double)__ldg(kr + rank_holes(lut, holes_dev(su2, norb)));
            acc += p ? -v : v;
        }
    }
    __shared__ double red[kDblWarps];
    acc = warp_sum(acc);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kDblWarps; ++w) t += red[w];
        partials[(int64_t)blockIdx.x * nquads + q] = t;
    }
}

static int dbl_occ_blocks(const ed_sector *s)
{
    int64_t b = (s->nsdn + kDblWarps - 1) / kDblWarps;
    return (int)(b > 64 ? 64 : (b < 1 ? 1 : b));
}

}  // namespace ed

using namespace ed;

extern "C" int ed_sector_set_uijkl(ed_sector *s, const double *ul)
{
    clear_error();
    ED_REQUIRE(s != nullptr && ul != nullptr, "NULL argument");
    ED_REQUIRE(s->kind == ED_HUBBARD, "the U_ijkl interaction needs a Hubbard sector");
    const int n = s->norb;
    auto U = [&](int a, int b, int c, int d) { return ul[(((int64_t)a * n + b) * n + c) * n + d]; };
    std::vector<int4> groups;
    std::vector<int2> jk;
    std::vector<double> val;
    for (int M = 1; M <= n; ++M)
        for (int N = 1; N <= n; ++N) {
            const int first = (int)jk.size();
            for (int J = 1; J <= n; ++J)
                for (int K = 1; K <= n; ++K) {
                    double up = 0.0;   // UPARTIAL(J,K) = sum_cd U[K-1][J-1][c][d]^2
                    for (int c = 0; c < n; ++c)
                        for (int d = 0; d < n; ++d) up += U(K - 1, J - 1, c, d) * U(K - 1, J - 1, c, d);
                    if (!(up >= kTol14)) continue;
                    const double v = U(N - 1, M - 1, K - 1, J - 1);   // UL(J,K,M,N)
                    if (!(std::fabs(v) >= kTol14)) continue;
                    jk.push_back(make_int2(J, K));
                    val.push_back(v);
                }
            if ((int)jk.size() > first) groups.push_back(make_int4(M, N, first, (int)jk.size() - first));
        }
    // the interaction replaces the on-site U of the sector (the reference has no ULDIAG term here)
    for (int b = 0; b < kMaxSites; ++b) s->u_site[b] = 0.0;
    s->u_uniform = true;
    s->u_value = 0.0;
    uijkl_free(s->uijkl);
    s->uijkl = nullptr;
    if (jk.empty()) return ED_OK;
    UijklTables *u = new UijklTables();
    u->ngroups = (int)groups.size();
    u->nterms = (int)jk.size();
    const size_t o1 = groups.size() * sizeof(int4);
    const size_t o2 = (o1 + jk.size() * sizeof(int2) + 15) / 16 * 16;
    const size_t o3 = o2 + val.size() * sizeof(double);
    const size_t bytes = o3 + val.size() * sizeof(float);
    std::vector<unsigned char> host(bytes, 0);
    std::vector<float> v32(val.begin(), val.end());
    std::memcpy(host.data(), groups.data(), o1);
    std::memcpy(host.data() + o1, jk.data(), jk.size() * sizeof(int2));
    std::memcpy(host.data() + o2, val.data(), val.size() * sizeof(double));
    std::memcpy(host.data() + o3, v32.data(), v32.size() * sizeof(float));
    if (cudaMalloc(&u->pool, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete u;
        set_error("cudaMalloc of %zu bytes for the U_ijkl terms failed", bytes);
        return ED_ERR_MEM;
    }
    if (cudaMemcpy(u->pool, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        uijkl_free(u);
        set_error("upload of the U_ijkl terms failed");
        return ED_ERR_CUDA;
    }
    unsigned char *b = static_cast<unsigned char *>(u->pool);
    u->groups = reinterpret_cast<int4 *>(b);
    u->jk = reinterpret_cast<int2 *>(b + o1);
    u->val = reinterpret_cast<double *>(b + o2);
    u->val32 = reinterpret_cast<float *>(b + o3);
    s->uijkl = u;
    return ED_OK;
}

extern "C" int64_t ed_dbl_occ_scratch_bytes(const ed_sector *s, int nquads)
{
    if (!s || nquads < 0) return -1;
    return (int64_t)nquads * 16 + (int64_t)dbl_occ_blocks(s) * nquads * 8 + 512;
}

extern "C" int ed_dbl_occ(ed_sector *s, void *stream, int dtype, int64_t ld, const void *bra, const void *ket,
                          int nquads, const int32_t *quads, double *out, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(s != nullptr && bra != nullptr && ket != nullptr && out != nullptr, "NULL argument");
    ED_REQUIRE(s->kind == ED_HUBBARD, "DBL_OCC needs a Hubbard sector");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(nquads >= 1 && nquads <= 65535 && quads != nullptr, "nquads=%d outside 1..65535", nquads);
    ED_REQUIRE(ld >= s->nsup, "ld=%lld below nsup=%lld", (long long)ld, (long long)s->nsup);
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_dbl_occ_scratch_bytes(s, nquads),
               "scratch of %lld bytes is below %lld", (long long)scratch_bytes,
               (long long)ed_dbl_occ_scratch_bytes(s, nquads));
    std::vector<int4> q((size_t)nquads);
    for (int i = 0; i < nquads; ++i) {
        for (int k = 0; k < 4; ++k)
            ED_REQUIRE(quads[4 * i + k] >= 1 && quads[4 * i + k] <= s->norb, "quad %d: site %d outside 1..%d", i,
                       quads[4 * i + k], s->norb);
        q[(size_t)i] = make_int4(quads[4 * i], quads[4 * i + 1], quads[4 * i + 2], quads[4 * i + 3]);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int4 *dq = static_cast<int4 *>(scratch);
    double *part = reinterpret_cast<double *>(static_cast<unsigned char *>(scratch) + (((size_t)nquads * 16 + 255) / 256) * 256);
    ED_CHECK_CUDA(cudaMemcpyAsync(dq, q.data(), (size_t)nquads * sizeof(int4), cudaMemcpyHostToDevice, st));
    // the host copy is pageable: let the transfer finish before q goes out of scope
    ED_CHECK_CUDA(cudaStreamSynchronize(st));
    const int nbx = dbl_occ_blocks(s);
    dim3 grid((unsigned)nbx, (unsigned)nquads);
    if (s->dim == 0) return cudaMemsetAsync(out, 0, sizeof(double) * nquads, st) == cudaSuccess ? ED_OK : ED_ERR_CUDA;
    if (dtype == ED_F32)
        dbl_occ_kernel<float><<<grid, kDblWarps * 32, 0, st>>>(static_cast<const float *>(bra),
                                                                 static_cast<const float *>(ket), ld, s->nsup, s->nsdn,
                                                                 s->norb, s->up.str, s->dn.str, s->lut, dq, nquads, part);
    else
        dbl_occ_kernel<double><<<grid, kDblWarps * 32, 0, st>>>(static_cast<const double *>(bra),
                                                                  static_cast<const double *>(ket), ld, s->nsup,
                                                                  s->nsdn, s->norb, s->up.str, s->dn.str, s->lut, dq,
                                                                  nquads, part);
    ED_CHECK_LAUNCH();
    return launch_reduce(part, nbx, nquads, out, st);
}
