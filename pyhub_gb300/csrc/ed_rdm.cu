// ed_rdm.cu -- reduced density matrices and spin correlations.
//
// Replaces ONE_RDM, TWO_RDM (local-U branch) and J_SPIN
// (static_rq.f90:153-395) and J_SPIN of the Heisenberg solver
// (static_rq_heis.f90:58-116).  The kernels return raw per-pair sums; the
// host assembles them with the reference's symmetrisation (the K<=J half is
// computed and mirrored, and the down matrix is a copy of the up one when
// N_up == N_down, static_rq.f90:212-241).
//
// Hubbard, for each site pair p = (J,K) of the caller's list (1-based sites):
//   q[p][0]  J!=K: sum_{d,u: J in u, K not in u} sign bra[d][u] ket[d][u']   (u' = u-J+K)
//            J==K: sum bra[d][u] ket[d][u] [J in u]                          (<n_J,up>)
//   q[p][1]  sum bra ket Sz_J Sz_K
//   q[p][2]  J==K: sum bra ket [J in d]                                      (<n_J,down>)
//   q[p][3]  J==K: sum bra ket [J in u and J in d]                           (<n_up n_down>)
//   q[p][4]  J!=K: sum_{d: J in d, K not in d} sign sum_u bra[d][u] ket[d'][u] (down hop)
//   q[p][5]  J!=K: -sum sign_u sign_d bra[d][u] ket[d''][u']  (up J->K, down K->J), the
//            transverse part of J_SPIN (static_rq.f90:345-383)
// Heisenberg (complementary down string), per pair:
//   q[p][0]  J!=K: sum_{I: J up, K down} (-1)^(J+K) bra[I'] ket[I]  (I' = I with J,K swapped)
//            J==K: 0.5 sum bra ket
//   q[p][1]  sum bra ket Sz_J Sz_K
#include "ed_common.cuh"

namespace ed {

int launch_reduce(const double *partials, int nblocks, int m, double *out, cudaStream_t st);

constexpr int kRdmQ = 6;
constexpr int kMaxPairs = kMaxSites * kMaxSites;

struct RdmArgs {
    int norb;
    int64_t nsup, nsdn, ld;
    const uint32_t *ustr, *dstr, *lut;
    int npairs;
    int8_t pj[kMaxPairs], pk[kMaxPairs];
};

__device__ __forceinline__ uint32_t bit_of(int norb, int pos) { return 1u << (norb - pos); }

__device__ __forceinline__ uint32_t between_bits(int norb, int a, int b)
{
    // string bits of the sites strictly between a and b
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    if (hi - lo < 2) return 0u;
    // sites lo+1 .. hi-1  <->  bits norb-hi+1 .. norb-lo-1
    const int b0 = norb - hi + 1, b1 = norb - lo - 1;
    const uint32_t upto = (b1 >= 31) ? 0xFFFFFFFFu : ((2u << b1) - 1u);
    return upto & ~((1u << b0) - 1u);
}

// Row-local sums: one thread per site pair, rows of bra and ket in shared memory.
template <typename T>
__global__ void rdm_row_kernel(const T *__restrict__ bra, const T *__restrict__ ket, const RdmArgs a,
                               double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *bs = reinterpret_cast<T *>(smem_raw);
    T *ks = bs + a.nsup;
    const bool same = (bra == ket);
    if (same) ks = bs;
    const int p = threadIdx.x;
    const bool active = p < a.npairs;
    const int J = active ? a.pj[p] : 1, K = active ? a.pk[p] : 1;
    const uint32_t bJ = bit_of(a.norb, J), bK = bit_of(a.norb, K);
    const uint32_t btw = between_bits(a.norb, J, K);
    double q0 = 0.0, q1 = 0.0, q2 = 0.0, q3 = 0.0;
    for (int64_t d = blockIdx.x; d < a.nsdn; d += gridDim.x) {
        for (int64_t i = threadIdx.x; i < a.nsup; i += blockDim.x) {
            bs[i] = bra[d * a.ld + i];
            if (!same) ks[i] = ket[d * a.ld + i];
        }
        __syncthreads();
        if (active) {
            const uint32_t sd = __ldg(a.dstr + d);
            const double szdJ = (sd & bJ) ? 0.5 : 0.0, szdK = (sd & bK) ? 0.5 : 0.0;
            for (int64_t u = 0; u < a.nsup; ++u) {
                const uint32_t su = __ldg(a.ustr + u);
                const double bk = (double)bs[u] * (double)ks[u];
                const double sJ = ((su & bJ) ? 0.5 : 0.0) - szdJ, sK = ((su & bK) ? 0.5 : 0.0) - szdK;
                q1 += bk * sJ * sK;
                if (J == K) {
                    if (su & bJ) q0 += bk;
                    if (sd & bJ) q2 += bk;
                    if ((su & bJ) && (sd & bJ)) q3 += bk;
                } else if ((su & bJ) && !(su & bK)) {
                    const uint32_t u2 = su - bJ + bK;
                    const uint32_t r = rank_holes(a.lut, holes_dev(u2, a.norb));
                    const double sg = (__popc(su & btw) & 1) ? -1.0 : 1.0;
                    q0 += sg * (double)bs[u] * (double)ks[r];
                }
            }
        }
        __syncthreads();
    }
    if (active) {
        double *o = partials + ((int64_t)blockIdx.x * a.npairs + p) * 4;
        o[0] = q0; o[1] = q1; o[2] = q2; o[3] = q3;
    }
}

// Cross-row sums (down hops and the spin-flip term), one CTA per row d.
template <typename T>
__global__ void __launch_bounds__(256) rdm_cross_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                        const RdmArgs a, int want_dn, int want_sx,
                                                        double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *acc = reinterpret_cast<double *>(smem_raw);          // [npairs][2]
    T *kr = reinterpret_cast<T *>(acc + 2 * a.npairs);           // staged ket row
    __shared__ double red[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < 2 * a.npairs; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    for (int64_t d = blockIdx.x; d < a.nsdn; d += gridDim.x) {
        const uint32_t sd = __ldg(a.dstr + d);
        const T *br = bra + d * a.ld;
        for (int p = 0; p < a.npairs; ++p) {
            const int J = a.pj[p], K = a.pk[p];
            if (J == K) continue;
            const uint32_t bJ = bit_of(a.norb, J), bK = bit_of(a.norb, K);
            const uint32_t btw = between_bits(a.norb, J, K);
            if (want_dn && (sd & bJ) && !(sd & bK)) {
                const uint32_t d2 = sd - bJ + bK;
                const int64_t r = rank_holes(a.lut, holes_dev(d2, a.norb));
                const double sg = (__popc(sd & btw) & 1) ? -1.0 : 1.0;
                const T *k2 = ket + r * a.ld;
                double s = 0.0;
                for (int64_t u = threadIdx.x; u < a.nsup; u += blockDim.x) s += (double)br[u] * (double)k2[u];
                s = warp_sum(s);
                if (lane == 0) red[warp] = s;
                __syncthreads();
                if (threadIdx.x == 0) {
                    double t = 0.0;
                    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
                    acc[2 * p] += sg * t;
                }
                __syncthreads();
            }
            if (want_sx && (sd & bK) && !(sd & bJ)) {
                const uint32_t d2 = sd - bK + bJ;
                const int64_t r = rank_holes(a.lut, holes_dev(d2, a.norb));
                const double sgd = (__popc(sd & btw) & 1) ? -1.0 : 1.0;
                const T *k2 = ket + r * a.ld;
                for (int64_t u = threadIdx.x; u < a.nsup; u += blockDim.x) kr[u] = k2[u];
                __syncthreads();
                double s = 0.0;
                for (int64_t u = threadIdx.x; u < a.nsup; u += blockDim.x) {
                    const uint32_t su = __ldg(a.ustr + u);
                    if ((su & bJ) && !(su & bK)) {
                        const uint32_t u2 = su - bJ + bK;
                        const uint32_t ru = rank_holes(a.lut, holes_dev(u2, a.norb));
                        const double sgu = (__popc(su & btw) & 1) ? -1.0 : 1.0;
                        s += sgu * (double)br[u] * (double)kr[ru];
                    }
                }
                s = warp_sum(s);
                if (lane == 0) red[warp] = s;
                __syncthreads();
                if (threadIdx.x == 0) {
                    double t = 0.0;
                    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
                    acc[2 * p + 1] -= sgd * t;
                }
                __syncthreads();
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * a.npairs; i += blockDim.x) partials[(int64_t)blockIdx.x * 2 * a.npairs + i] = acc[i];
}

static constexpr int kRdmBlocks = 256;

template <typename T>
static int rdm_hub(ed_sector *s, cudaStream_t st, int64_t ld, const T *bra, const T *ket, int npairs,
                   const int32_t *pairs, int flags, double *out, double *scratch)
{
    RdmArgs a;
    a.norb = s->norb;
    a.nsup = s->nsup; a.nsdn = s->nsdn; a.ld = ld;
    a.ustr = s->up.str; a.dstr = s->dn.str; a.lut = s->lut;
    a.npairs = npairs;
    for (int p = 0; p < npairs; ++p) { a.pj[p] = (int8_t)pairs[2 * p]; a.pk[p] = (int8_t)pairs[2 * p + 1]; }
    int dev = 0, maxsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    int blocks = (int)std::min<int64_t>(s->nsdn, kRdmBlocks);
    if (blocks < 1) blocks = 1;
    // row-local pass
    const size_t smem1 = (size_t)(bra == ket ? 1 : 2) * s->nsup * sizeof(T);
    if (smem1 > (size_t)maxsm) { set_error("rows of %lld entries exceed shared memory", (long long)s->nsup); return ED_ERR_RANGE; }
    ED_CHECK_CUDA(cudaFuncSetAttribute(rdm_row_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
    const int thr = (npairs + 31) / 32 * 32;
    double *part1 = scratch;
    rdm_row_kernel<T><<<blocks, thr, smem1, st>>>(bra, ket, a, part1);
    ED_CHECK_LAUNCH();
    // reduce per pair: partials are [blocks][npairs][4]
    int rc = launch_reduce(part1, blocks, 4 * npairs, out, st);
    if (rc) return rc;
    const int want_dn = (flags & 1) ? 1 : 0, want_sx = (flags & 2) ? 1 : 0;
    if (want_dn || want_sx) {
        const size_t smem2 = (size_t)2 * npairs * sizeof(double) + (size_t)s->nsup * sizeof(T) + 16;
        if (smem2 > (size_t)maxsm) { set_error("cross-row RDM pass exceeds shared memory"); return ED_ERR_RANGE; }
        ED_CHECK_CUDA(cudaFuncSetAttribute(rdm_cross_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
        double *part2 = scratch + (int64_t)blocks * 4 * npairs;
        rdm_cross_kernel<T><<<blocks, 256, smem2, st>>>(bra, ket, a, want_dn, want_sx, part2);
        ED_CHECK_LAUNCH();
        rc = launch_reduce(part2, blocks, 2 * npairs, out + 4 * npairs, st);
        if (rc) return rc;
    } else {
        ED_CHECK_CUDA(cudaMemsetAsync(out + 4 * npairs, 0, sizeof(double) * 2 * npairs, st));
    }
    return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" int64_t ed_rdm_scratch_bytes(int npairs)
{
    if (npairs < 1) npairs = 1;
    return (int64_t)kRdmBlocks * kRdmQ * npairs * (int64_t)sizeof(double) + 4096;
}

extern "C" int ed_rdm(ed_sector *s, void *stream, int dtype, int64_t ld, const void *bra, const void *ket,
                      int npairs, const int32_t *pairs, int flags, double *out, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(s != nullptr, "sector is NULL");
    ED_REQUIRE(bra != nullptr && ket != nullptr && out != nullptr && pairs != nullptr, "NULL argument");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(npairs >= 1 && npairs <= kMaxPairs, "npairs=%d outside 1..%d", npairs, kMaxPairs);
    for (int p = 0; p < npairs; ++p)
        ED_REQUIRE(pairs[2 * p] >= 1 && pairs[2 * p] <= s->norb && pairs[2 * p + 1] >= 1 && pairs[2 * p + 1] <= s->norb,
                   "pair %d = (%d,%d) outside 1..%d", p, pairs[2 * p], pairs[2 * p + 1], s->norb);
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_rdm_scratch_bytes(npairs),
               "scratch of %lld bytes is below the %lld needed", (long long)scratch_bytes,
               (long long)ed_rdm_scratch_bytes(npairs));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (s->kind == ED_HUBBARD) {
        ED_REQUIRE(ld >= s->nsup, "ld below nsup");
        if (dtype == ED_F32)
            return rdm_hub<float>(s, st, ld, (const float *)bra, (const float *)ket, npairs, pairs, flags, out,
                                  (double *)scratch);
        return rdm_hub<double>(s, st, ld, (const double *)bra, (const double *)ket, npairs, pairs, flags, out,
                               (double *)scratch);
    }
    // partials [blocks][npairs][2] fit in the kRdmBlocks*kRdmQ*npairs doubles of ed_rdm_scratch_bytes
    return heis_struct_rdm(s, st, dtype, bra, ket, npairs, pairs, out, (double *)scratch, kRdmBlocks);
}
