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

#include <algorithm>

namespace ed {

int launch_reduce(const double *partials, int nblocks, int m, double *out, cudaStream_t st);

constexpr int kRdmQ = 6;
constexpr int kMaxPairs = kMaxSites * kMaxSites;

struct RdmArgs {
    int norb;
    int64_t nsup, nsdn, ld;
    const uint32_t *ustr, *dstr, *lut;
    const int32_t *upl_off, *dpl_off;   // pair lists of the up and down strings
    const int2 *upl_ent, *dpl_ent;
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

// ---- diagonal sums (q0 and q3 for J == K, q1 for every pair, q2 for J == K).
// With n_u(J), n_d(J) the occupations of site J in the up and down strings and
// b = bra*ket of an element, Sz_J = (n_u(J) - n_d(J))/2 factorises the sums
// over the (d, u) grid into column sums C(u) = sum_d b, column projections
// T_K(u) = sum_d b n_d(K) and row sums W(d) = sum_u b:
//   sum b Sz_J Sz_K = (sum_u C n_u(J) n_u(K) - sum_u [n_u(J) T_K + n_u(K) T_J]
//                      + sum_d W n_d(J) n_d(K)) / 4,
//   <n_up J> = sum_u C n_u(J),  <n_down J> = sum_d W n_d(J),
//   <n_up n_down J> = sum_u n_u(J) T_J(u),
// so an element costs ~norb FP64 operations for all pairs at once.  A CTA
// owns a tile of 256 columns (one per thread) and a range of rows; each
// tile's sums are complete contributions (everything is linear in them), so
// tiles add up without a global column array.
constexpr int kDiagThreads = 256;

template <typename T, int MS>
__global__ void __launch_bounds__(kDiagThreads) rdm_diag_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                                const RdmArgs a, int nry,
                                                                double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *Ts = reinterpret_cast<double *>(smem_raw);       // [MS][kDiagThreads]
    double *Cs = Ts + MS * kDiagThreads;                      // [kDiagThreads]
    double *accW = Cs + kDiagThreads;                         // [npairs]
    __shared__ double red[kDiagThreads / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ncx = (int)((a.nsup + kDiagThreads - 1) / kDiagThreads);
    const int cx = blockIdx.x % ncx, ry = blockIdx.x / ncx;
    const int64_t u = (int64_t)cx * kDiagThreads + threadIdx.x;
    const bool act = u < a.nsup;
    const int64_t r0 = a.nsdn * ry / nry, r1 = a.nsdn * (ry + 1) / nry;
    for (int q = threadIdx.x; q < a.npairs; q += blockDim.x) accW[q] = 0.0;
    double C = 0.0, Tk[MS];
#pragma unroll
    for (int k = 0; k < MS; ++k) Tk[k] = 0.0;
    const int norb = a.norb;
    for (int64_t d = r0; d < r1; ++d) {
        const uint32_t sd = __ldg(a.dstr + d);
        const double b = act ? (double)__ldg(bra + d * a.ld + u) * (double)__ldg(ket + d * a.ld + u) : 0.0;
        C += b;
#pragma unroll
        for (int k = 0; k < MS; ++k)   // bit k of a string is site norb-k
            if ((sd >> k) & 1u) Tk[k] += b;
        // W(d): the row's sum over this tile's columns
        double w = warp_sum(b);
        __syncthreads();
        if (lane == 0) red[warp] = w;
        __syncthreads();
        w = 0.0;
#pragma unroll
        for (int q = 0; q < kDiagThreads / 32; ++q) w += red[q];
        for (int q = threadIdx.x; q < a.npairs; q += blockDim.x) {
            const uint32_t bJ = bit_of(norb, a.pj[q]), bK = bit_of(norb, a.pk[q]);
            if ((sd & bJ) && (sd & bK)) accW[q] += w;
        }
    }
#pragma unroll
    for (int k = 0; k < MS; ++k) Ts[k * kDiagThreads + threadIdx.x] = Tk[k];
    Cs[threadIdx.x] = C;
    __syncthreads();
    // per pair: sums over the tile's columns (warp w takes pairs w, w+8, ...)
    for (int q = warp; q < a.npairs; q += kDiagThreads / 32) {
        const int J = a.pj[q], K = a.pk[q];
        const uint32_t bJ = bit_of(norb, J), bK = bit_of(norb, K);
        const int kJ = norb - J, kK = norb - K;   // bit positions
        double s_cc = 0.0, s_ct = 0.0, s_c = 0.0, s_t = 0.0;
        for (int t = lane; t < kDiagThreads; t += 32) {
            const int64_t uu = (int64_t)cx * kDiagThreads + t;
            if (uu >= a.nsup) continue;
            const uint32_t su = __ldg(a.ustr + uu);
            const double nJ = (su & bJ) ? 1.0 : 0.0, nK = (su & bK) ? 1.0 : 0.0;
            const double c = Cs[t];
            s_cc += nJ * nK * c;
            s_ct += nJ * Ts[kK * kDiagThreads + t] + nK * Ts[kJ * kDiagThreads + t];
            s_c += nJ * c;
            s_t += nJ * Ts[kJ * kDiagThreads + t];
        }
        s_cc = warp_sum(s_cc);
        s_ct = warp_sum(s_ct);
        s_c = warp_sum(s_c);
        s_t = warp_sum(s_t);
        if (lane == 0) {
            double *o = partials + ((int64_t)blockIdx.x * a.npairs + q) * 4;
            const double wq = accW[q];
            o[0] = (J == K) ? s_c : 0.0;
            o[1] = 0.25 * (s_cc - s_ct + wq);
            o[2] = (J == K) ? wq : 0.0;
            o[3] = (J == K) ? s_t : 0.0;
        }
    }
}

// ---- up hops within a row (q0 for J != K): for each pair, the strings of
// its list, sum sign * bra[d][u] * ket[d][u'].  Rows are staged in shared
// memory; warp w takes pairs w, w+8, ...; per-pair sums accumulate in shared
// memory over the CTA's rows.
template <typename T>
__global__ void __launch_bounds__(256) rdm_uphop_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                        const RdmArgs a, double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *acc = reinterpret_cast<double *>(smem_raw);          // [npairs]
    T *bs = reinterpret_cast<T *>(acc + a.npairs);
    const bool same = (bra == ket);
    T *ks = same ? bs : bs + a.nsup;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = threadIdx.x; q < a.npairs; q += blockDim.x) acc[q] = 0.0;
    for (int64_t d = blockIdx.x; d < a.nsdn; d += gridDim.x) {
        __syncthreads();
        for (int64_t i = threadIdx.x; i < a.nsup; i += blockDim.x) {
            bs[i] = bra[d * a.ld + i];
            if (!same) ks[i] = ket[d * a.ld + i];
        }
        __syncthreads();
        for (int q = warp; q < a.npairs; q += 8) {
            const int J = a.pj[q], K = a.pk[q];
            if (J == K) continue;
            const int pid = (J - 1) * a.norb + (K - 1);
            const int e0 = __ldg(a.upl_off + pid), e1 = __ldg(a.upl_off + pid + 1);
            double s = 0.0;
            for (int e = e0 + lane; e < e1; e += 32) {
                const int2 en = __ldg(a.upl_ent + e);
                const double b = (double)bs[en.x];
                s = fma((en.y < 0) ? -b : b, (double)ks[en.y & 0x7fffffff], s);   // one FP64 op per entry
            }
            s = warp_sum(s);
            if (lane == 0) acc[q] += s;
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < a.npairs; q += blockDim.x) {
        double *o = partials + ((int64_t)blockIdx.x * a.npairs + q) * 4;
        o[0] = acc[q];
        o[1] = o[2] = o[3] = 0.0;
    }
}

// ---- sums across rows (q4: down hop J->K of the row; q5: up hop J->K with
// down hop K->J, the transverse term of J_SPIN).  The bra row is staged in
// shared memory; warp w takes pairs w, w+8, ...: a down hop is a dot product
// with the ket row it reaches (lanes over the row), the transverse term walks
// the up pair list against that ket row.
template <typename T>
__global__ void __launch_bounds__(256) rdm_cross_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                        const RdmArgs a, int want_dn, int want_sx,
                                                        double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *acc = reinterpret_cast<double *>(smem_raw);          // [npairs][2]
    T *bs = reinterpret_cast<T *>(acc + 2 * a.npairs);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < 2 * a.npairs; i += blockDim.x) acc[i] = 0.0;
    for (int64_t d = blockIdx.x; d < a.nsdn; d += gridDim.x) {
        const uint32_t sd = __ldg(a.dstr + d);
        __syncthreads();
        for (int64_t i = threadIdx.x; i < a.nsup; i += blockDim.x) bs[i] = bra[d * a.ld + i];
        __syncthreads();
        for (int q = warp; q < a.npairs; q += 8) {
            const int J = a.pj[q], K = a.pk[q];
            if (J == K) continue;
            const uint32_t bJ = bit_of(a.norb, J), bK = bit_of(a.norb, K);
            const uint32_t btw = between_bits(a.norb, J, K);
            if (want_dn && (sd & bJ) && !(sd & bK)) {
                const int64_t r = rank_holes(a.lut, holes_dev(sd - bJ + bK, a.norb));
                const T *k2 = ket + r * a.ld;
                double s = 0.0;
                for (int64_t u = lane; u < a.nsup; u += 32) s += (double)bs[u] * (double)__ldg(k2 + u);
                s = warp_sum(s);
                if (lane == 0) acc[2 * q] += (__popc(sd & btw) & 1) ? -s : s;
            }
            if (want_sx && (sd & bK) && !(sd & bJ)) {
                const int64_t r = rank_holes(a.lut, holes_dev(sd - bK + bJ, a.norb));
                const T *k2 = ket + r * a.ld;
                const int pid = (J - 1) * a.norb + (K - 1);
                const int e0 = __ldg(a.upl_off + pid), e1 = __ldg(a.upl_off + pid + 1);
                double s = 0.0;
                for (int e = e0 + lane; e < e1; e += 32) {
                    const int2 en = __ldg(a.upl_ent + e);
                    const double b = (double)bs[en.x];
                    s = fma((en.y < 0) ? -b : b, (double)__ldg(k2 + (en.y & 0x7fffffff)), s);
                }
                s = warp_sum(s);
                if (lane == 0) acc[2 * q + 1] -= (__popc(sd & btw) & 1) ? -s : s;
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * a.npairs; i += blockDim.x) partials[(int64_t)blockIdx.x * 2 * a.npairs + i] = acc[i];
}

static constexpr int kRdmBlocks = 256;   // partial rows of the Heisenberg passes (3 x 2 sums per pair each)
static constexpr int kRdmRows = 1024;    // partial rows of each Hubbard part (4 and 2 sums per pair)

template <typename T>
static int rdm_hub(ed_sector *s, cudaStream_t st, int64_t ld, const T *bra, const T *ket, int npairs,
                   const int32_t *pairs, int flags, double *out, double *scratch)
{
    RdmArgs a;
    a.norb = s->norb;
    a.nsup = s->nsup; a.nsdn = s->nsdn; a.ld = ld;
    a.ustr = s->up.str; a.dstr = s->dn.str; a.lut = s->lut;
    a.upl_off = s->up.pl_off; a.upl_ent = s->up.pl_ent;
    a.dpl_off = s->dn.pl_off; a.dpl_ent = s->dn.pl_ent;
    a.npairs = npairs;
    for (int p = 0; p < npairs; ++p) { a.pj[p] = (int8_t)pairs[2 * p]; a.pk[p] = (int8_t)pairs[2 * p + 1]; }
    int dev = 0, maxsm = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    nsm = std::max(nsm, 1);
    // ---- row-local sums: diagonal tiles then up-hop rows, their partials stacked for one reduction.
    // Each pass gets a few CTAs per SM (both are bound by the FP64 pipe of every SM they occupy);
    // the partial rows of the two together stay within kRdmRows.
    constexpr int kMaxTiles = kRdmRows / 2;
    const int ncx = (int)((s->nsup + kDiagThreads - 1) / kDiagThreads);
    if (ncx > kMaxTiles) { set_error("rows of %lld strings are too long for the RDM tiles", (long long)s->nsup); return ED_ERR_RANGE; }
    int nry = (int)std::max<int64_t>(1, std::min<int64_t>(s->nsdn, std::min(2 * nsm, kMaxTiles) / ncx));
    if (ncx * nry > kMaxTiles) nry = std::max(1, kMaxTiles / ncx);
    const int nbA = ncx * nry;
    const bool small = s->norb <= 16;
    const size_t smemA = (size_t)((small ? 16 : 32) + 1) * kDiagThreads * sizeof(double) + (size_t)npairs * sizeof(double);
    const int nbB = (int)std::min<int64_t>(s->nsdn, std::min(4 * nsm, kRdmRows - nbA));
    const size_t smemB = (size_t)npairs * sizeof(double) + (size_t)(bra == ket ? 1 : 2) * s->nsup * sizeof(T);
    if (smemA > (size_t)maxsm || smemB > (size_t)maxsm) {
        set_error("RDM pass of %lld strings exceeds shared memory", (long long)s->nsup);
        return ED_ERR_RANGE;
    }
    double *part1 = scratch;
    if (small) {
        ED_CHECK_CUDA(cudaFuncSetAttribute(rdm_diag_kernel<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemA));
        rdm_diag_kernel<T, 16><<<nbA, kDiagThreads, smemA, st>>>(bra, ket, a, nry, part1);
    } else {
        ED_CHECK_CUDA(cudaFuncSetAttribute(rdm_diag_kernel<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemA));
        rdm_diag_kernel<T, 32><<<nbA, kDiagThreads, smemA, st>>>(bra, ket, a, nry, part1);
    }
    ED_CHECK_LAUNCH();
    if (nbB > 0) {
        ED_CHECK_CUDA(cudaFuncSetAttribute(rdm_uphop_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemB));
        rdm_uphop_kernel<T><<<nbB, 256, smemB, st>>>(bra, ket, a, part1 + (int64_t)nbA * 4 * npairs);
        ED_CHECK_LAUNCH();
    }
    int rc = launch_reduce(part1, nbA + std::max(nbB, 0), 4 * npairs, out, st);
    if (rc) return rc;
    const int want_dn = (flags & 1) ? 1 : 0, want_sx = (flags & 2) ? 1 : 0;
    if (want_dn || want_sx) {
        const size_t smem2 = (size_t)2 * npairs * sizeof(double) + (size_t)s->nsup * sizeof(T) + 16;
        if (smem2 > (size_t)maxsm) { set_error("cross-row RDM pass exceeds shared memory"); return ED_ERR_RANGE; }
        ED_CHECK_CUDA(cudaFuncSetAttribute(rdm_cross_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
        const int nbC = (int)std::min<int64_t>(s->nsdn, std::min(4 * nsm, kRdmRows));
        double *part2 = scratch + (int64_t)kRdmRows * 4 * npairs;
        rdm_cross_kernel<T><<<nbC, 256, smem2, st>>>(bra, ket, a, want_dn, want_sx, part2);
        ED_CHECK_LAUNCH();
        rc = launch_reduce(part2, nbC, 2 * npairs, out + 4 * npairs, st);
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
    // Hubbard: kRdmRows rows of 4 sums and kRdmRows rows of 2 sums per pair; the Heisenberg
    // passes' 3 * kRdmBlocks rows of 2 sums fit in the same space
    static_assert(3 * kRdmBlocks * 2 <= kRdmRows * kRdmQ, "Heisenberg partials exceed the RDM scratch");
    return (int64_t)kRdmRows * kRdmQ * npairs * (int64_t)sizeof(double) + 4096;
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
    // partials [<= 3 * kRdmBlocks][npairs][2] fit in the kRdmRows*kRdmQ*npairs doubles of ed_rdm_scratch_bytes
    return heis_struct_rdm(s, st, dtype, bra, ket, npairs, pairs, out, (double *)scratch, kRdmBlocks);
}
