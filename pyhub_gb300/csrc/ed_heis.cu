// ed_heis.cu -- structured H*v of the Heisenberg sector.
//
// Replaces HPROD of hprod_heis.f90:1-61 (the same Hamiltonian as heis_kernel
// of ed_hv.cu, element for element) with a product that never ranks a full
// 32-bit state.  A state is its empty-site (down-spin) pattern h, bit j for
// site j+1.  Split the sites into A = 1..nA (bits 0..nA-1) and B = the rest.
// The reference order is colex order of h, and colex order keeps all states
// that share their B part contiguous, ordered by the colex rank of their A
// part.  So the sector vector IS a set of rows: one row per B pattern hB
// (row offset = the colex contribution of hB's bits), and the row's entries
// are the A patterns with m = H - popcount(hB) holes in colex order (the
// 16-site combination order for a 4x8 lattice cut in two 4x4 halves).
// With that layout
//   A-A bonds flip within a row     -> gathers from the row staged in shared memory,
//   B-B bonds flip between rows     -> row axpys at equal column (coalesced),
//   A-B bonds flip both             -> a gather from ONE other row per bond; the
//                                      column map (add/remove one fixed bit) is
//                                      monotone, so the gathers stay local.
// Pass R (one CTA per row): diagonal + A-A + A-B, y = s*(...).
// Pass S (column slabs that keep the x slab of one m-block in L2): y += s*B-B,
// with the fused <x,y>, <y,y> partials.
#include "ed_common.cuh"

#include <cstdlib>

#include <algorithm>
#include <cstring>
#include <vector>

namespace ed {

namespace {

int64_t hbinom(int n, int k)
{
    if (k < 0 || n < 0 || k > n) return 0;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

// colex rank of a hole pattern: sum over its set bits p (ascending, i = 1..) of C(p, i)
int64_t colex_rank(uint32_t h, int base_i = 0, int shift = 0)
{
    int64_t r = 0;
    int i = base_i;
    while (h) {
        const int p = __builtin_ctz(h);
        r += hbinom(p + shift, ++i);
        h &= h - 1;
    }
    return r;
}

template <typename T>
int up(T **dst, const std::vector<T> &v)
{
    *dst = nullptr;
    if (v.empty()) return ED_OK;
    if (cudaMalloc(dst, sizeof(T) * v.size()) != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation of %zu bytes failed", sizeof(T) * v.size());
        return ED_ERR_MEM;
    }
    if (cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("upload failed");
        return ED_ERR_CUDA;
    }
    return ED_OK;
}

}  // namespace

int heis_struct_build(ed_sector *s)
{
    const HeisTables &ht = s->heis;
    HeisStruct *hs = new HeisStruct();
    s->hs = hs;
    const int norb = s->norb;
    const int nA = norb / 2, nB = norb - nA, H = norb - s->nup;
    hs->nA = nA;
    hs->nB = nB;
    hs->H = H;
    hs->mlo = std::max(0, H - nB);
    hs->mhi = std::min(nA, H);
    // ---- columns: A patterns by hole count m, colex order
    std::vector<uint32_t> col_pat;
    std::vector<int32_t> rankA((size_t)1 << nA, -1);
    std::vector<double> diagA;
    for (int m = 0; m <= kMaxHalf + 1; ++m) hs->col_base[m] = 0;
    for (int m = 0; m <= nA; ++m) {
        hs->col_base[m] = (int64_t)col_pat.size();
        hs->ncol[m] = hbinom(nA, m);
        std::vector<uint32_t> pats;
        for (uint32_t h = 0; h < (1u << nA); ++h)
            if (__builtin_popcount(h) == m) pats.push_back(h);
        std::sort(pats.begin(), pats.end(), [](uint32_t x, uint32_t y) { return colex_rank(x) < colex_rank(y); });
        for (size_t r = 0; r < pats.size(); ++r) {
            rankA[pats[r]] = (int32_t)r;
            col_pat.push_back(pats[r]);
        }
    }
    hs->col_base[nA + 1] = (int64_t)col_pat.size();
    // bonds by class
    std::vector<int> aa, bb, ab;
    for (int b = 0; b < ht.nbond; ++b) {
        const int pj = ht.bj[b] - 1, pk = ht.bk[b] - 1;   // pj < pk
        if (pk < nA) aa.push_back(b);
        else if (pj >= nA) bb.push_back(b);
        else ab.push_back(b);
    }
    if ((int)ab.size() > kMaxAB) {
        set_error("%zu bonds cross the two halves (at most %d)", ab.size(), kMaxAB);
        return ED_ERR_RANGE;
    }
    // A-A zz energy and hop lists per column, sliced ELL per m (32 columns per slice)
    diagA.resize(col_pat.size());
    std::vector<int32_t> aa_off(1, 0), aa_src;
    std::vector<double> aa_cf;
    int64_t nslices = 0;
    for (int m = 0; m <= nA; ++m) {
        hs->slice_base[m] = nslices;
        const int64_t n = hs->ncol[m], base = hs->col_base[m];
        std::vector<std::vector<std::pair<int32_t, double>>> lists((size_t)n);
        for (int64_t r = 0; r < n; ++r) {
            const uint32_t h = col_pat[(size_t)(base + r)];
            double d = 0.0;
            for (int b : aa) {
                const int pj = ht.bj[b] - 1, pk = ht.bk[b] - 1;
                const uint32_t hj = (h >> pj) & 1u, hk = (h >> pk) & 1u;
                d += (hj == hk ? 0.25 : -0.25) * ht.zz[b];
                if (hj == hk) continue;
                const double c = hj ? ht.flip_jk[b] : ht.flip_kj[b];
                if (c == 0.0) continue;
                lists[(size_t)r].push_back({rankA[h ^ ((1u << pj) | (1u << pk))], c});
            }
            diagA[(size_t)(base + r)] = d;
        }
        const int64_t ns = (n + 31) / 32;
        for (int64_t sl = 0; sl < ns; ++sl) {
            size_t w = 0;
            for (int64_t r = sl * 32; r < std::min(n, sl * 32 + 32); ++r) w = std::max(w, lists[(size_t)r].size());
            for (size_t k = 0; k < w; ++k)
                for (int l = 0; l < 32; ++l) {
                    const int64_t r = sl * 32 + l;
                    if (r < n && k < lists[(size_t)r].size()) {
                        aa_src.push_back(lists[(size_t)r][k].first);
                        aa_cf.push_back(lists[(size_t)r][k].second);
                    } else {
                        aa_src.push_back((int32_t)std::min(r, n - 1));   // own column, weight 0
                        aa_cf.push_back(0.0);
                    }
                }
            aa_off.push_back(aa_off.back() + (int32_t)w);
        }
        nslices += ns;
    }
    hs->slice_base[nA + 1] = nslices;
    // ---- rows: B patterns with H - m holes, m in [mlo, mhi], sorted by offset
    struct Row {
        uint32_t hb;
        int m;
        int64_t off;
    };
    std::vector<Row> rows;
    for (uint32_t hb = 0; hb < (1u << nB); ++hb) {
        const int m = H - __builtin_popcount(hb);
        if (m < hs->mlo || m > hs->mhi) continue;
        // colex contribution of the B holes: running index continues after the m A holes
        rows.push_back({hb, m, colex_rank(hb, m, nA)});
    }
    std::sort(rows.begin(), rows.end(), [](const Row &x, const Row &y) { return x.off < y.off; });
    const int64_t nrows = (int64_t)rows.size();
    hs->nrows = nrows;
    std::vector<uint32_t> row_pat((size_t)nrows);
    std::vector<int32_t> row_m((size_t)nrows), rowidx((size_t)1 << nB, -1);
    std::vector<int64_t> row_off((size_t)nrows);
    std::vector<double> diagB((size_t)nrows);
    int64_t expect = 0;
    hs->max_len = 0;
    for (int64_t r = 0; r < nrows; ++r) {
        const Row &w = rows[(size_t)r];
        if (w.off != expect) {
            set_error("internal: row offsets are not contiguous at row %lld", (long long)r);
            return ED_ERR_ARG;
        }
        expect += hs->ncol[w.m];
        row_pat[(size_t)r] = w.hb;
        row_m[(size_t)r] = w.m;
        row_off[(size_t)r] = w.off;
        rowidx[w.hb] = (int32_t)r;
        hs->max_len = std::max<int64_t>(hs->max_len, hs->ncol[w.m]);
    }
    if (expect != s->nsup) {
        set_error("internal: rows cover %lld of %lld states", (long long)expect, (long long)s->nsup);
        return ED_ERR_ARG;
    }
    // A-B bonds: with at most 32 of them, a column's A bits and a row's B bits at the bonds are
    // packed into one word each; the bonds where they differ are the antiparallel ones
    hs->ab_fast = ab.size() <= 32;
    double ab_zz_sum = 0.0;   // sum of zz/4 over the A-B bonds (every bond taken as "equal")
    for (int b : ab) ab_zz_sum += 0.25 * ht.zz[b];
    std::vector<uint32_t> col_abbits, row_bbits;
    std::vector<int32_t> ab_rank;   // [q][column]: rank of the column's pattern with the bond's A bit flipped
    if (hs->ab_fast) {
        ab_rank.resize(ab.size() * col_pat.size());
        for (size_t q = 0; q < ab.size(); ++q)
            for (size_t c = 0; c < col_pat.size(); ++c)
                ab_rank[q * col_pat.size() + c] = rankA[col_pat[c] ^ (1u << (ht.bj[ab[q]] - 1))];
        hs->ncols = (int64_t)col_pat.size();
        col_abbits.resize(col_pat.size());
        for (size_t c = 0; c < col_pat.size(); ++c) {
            uint32_t w = 0;
            for (size_t q = 0; q < ab.size(); ++q) w |= ((col_pat[c] >> (ht.bj[ab[q]] - 1)) & 1u) << q;
            col_abbits[c] = w;
        }
        row_bbits.resize((size_t)nrows);
        for (int64_t r = 0; r < nrows; ++r) {
            uint32_t w = 0;
            for (size_t q = 0; q < ab.size(); ++q) w |= ((row_pat[(size_t)r] >> (ht.bk[ab[q]] - 1 - nA)) & 1u) << q;
            row_bbits[(size_t)r] = w;
        }
    }
    // B-B zz energy (+ the constant diagonal) and neighbour rows per row
    std::vector<int32_t> bb_ptr(1, 0), bb_src;
    std::vector<double> bb_cf;
    for (int64_t r = 0; r < nrows; ++r) {
        const uint32_t h = row_pat[(size_t)r];
        double d = ht.dconst + (hs->ab_fast ? ab_zz_sum : 0.0);
        for (int b : bb) {
            const int pj = ht.bj[b] - 1 - nA, pk = ht.bk[b] - 1 - nA;
            const uint32_t hj = (h >> pj) & 1u, hk = (h >> pk) & 1u;
            d += (hj == hk ? 0.25 : -0.25) * ht.zz[b];
            if (hj == hk) continue;
            const double c = hj ? ht.flip_jk[b] : ht.flip_kj[b];
            if (c == 0.0) continue;
            bb_src.push_back(rowidx[h ^ ((1u << pj) | (1u << pk))]);
            bb_cf.push_back(c);
        }
        diagB[(size_t)r] = d;
        bb_ptr.push_back((int32_t)bb_src.size());
    }
    // rows grouped by m (offset order within each m) for the slab pass
    std::vector<int32_t> rows_of_m;
    for (int m = 0; m <= kMaxHalf + 1; ++m) hs->row_base[m] = 0;
    for (int m = 0; m <= nA; ++m) {
        hs->row_base[m] = (int64_t)rows_of_m.size();
        for (int64_t r = 0; r < nrows; ++r)
            if (row_m[(size_t)r] == m) rows_of_m.push_back((int32_t)r);
    }
    hs->row_base[nA + 1] = (int64_t)rows_of_m.size();
    // A-B bonds
    hs->nab = (int)ab.size();
    for (int q = 0; q < hs->nab; ++q) {
        const int b = ab[(size_t)q];
        hs->ab_pa[q] = (int8_t)(ht.bj[b] - 1);
        hs->ab_pb[q] = (int8_t)(ht.bk[b] - 1 - nA);
        hs->ab_fjk[q] = ht.flip_jk[b];
        hs->ab_fkj[q] = ht.flip_kj[b];
        hs->ab_zz[q] = 0.25 * ht.zz[b];
    }
    std::vector<float> aa_cf32(aa_cf.begin(), aa_cf.end()), bb_cf32(bb_cf.begin(), bb_cf.end());
    std::vector<float> diagA32(diagA.begin(), diagA.end()), diagB32(diagB.begin(), diagB.end());
    std::vector<int2> aa_pk32(aa_src.size());
    for (size_t q = 0; q < aa_src.size(); ++q) {
        int32_t bits;
        std::memcpy(&bits, &aa_cf32[q], sizeof(bits));
        aa_pk32[q] = make_int2(aa_src[q], bits);
    }
    int rc;
    if ((rc = up(&hs->col_pat, col_pat)) || (rc = up(&hs->rankA, rankA)) || (rc = up(&hs->diagA, diagA)) ||
        (rc = up(&hs->aa_off, aa_off)) || (rc = up(&hs->aa_src, aa_src)) || (rc = up(&hs->aa_cf32, aa_cf32)) ||
        (rc = up(&hs->aa_cf64, aa_cf)) || (rc = up(&hs->row_pat, row_pat)) || (rc = up(&hs->row_m, row_m)) ||
        (rc = up(&hs->row_off, row_off)) || (rc = up(&hs->rowidx, rowidx)) || (rc = up(&hs->diagB, diagB)) ||
        (rc = up(&hs->bb_ptr, bb_ptr)) || (rc = up(&hs->bb_src, bb_src)) || (rc = up(&hs->bb_cf32, bb_cf32)) ||
        (rc = up(&hs->bb_cf64, bb_cf)) || (rc = up(&hs->rows_of_m, rows_of_m)) ||
        (rc = up(&hs->aa_pk32, aa_pk32)) || (rc = up(&hs->col_abbits, col_abbits)) ||
        (rc = up(&hs->row_bbits, row_bbits)) || (rc = up(&hs->diagA32, diagA32)) || (rc = up(&hs->ab_rank, ab_rank)) ||
        (rc = up(&hs->diagB32, diagB32)))
        return rc;
    return ED_OK;
}

void heis_struct_free(HeisStruct *hs)
{
    if (!hs) return;
    void *ptrs[] = {hs->col_pat, hs->rankA, hs->diagA, hs->aa_off, hs->aa_src, hs->aa_cf32,
                    hs->aa_cf64, hs->row_pat, hs->row_m, hs->row_off, hs->rowidx, hs->diagB,
                    hs->bb_ptr, hs->bb_src, hs->bb_cf32, hs->bb_cf64, hs->rows_of_m,
                    hs->aa_pk32, hs->col_abbits, hs->row_bbits, hs->diagA32, hs->diagB32, hs->ab_rank};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete hs;
}

// ------------------------------------------------------------ kernels

struct HsArgs {
    int nA, nB, nab;
    int64_t nrows;
    int64_t col_base[kMaxHalf + 2], ncol[kMaxHalf + 1], slice_base[kMaxHalf + 2], row_base[kMaxHalf + 2];
    const uint32_t *col_pat, *row_pat;
    const int32_t *rankA, *aa_off, *aa_src, *row_m, *rowidx, *bb_ptr, *bb_src, *rows_of_m;
    const int64_t *row_off;
    const void *diagA, *diagB;     // float or double, like the vectors
    const void *aa_cf, *bb_cf;     // float or double
    const int2 *aa_pk32;           // {column, FP32 coefficient bits} of the A-A flips
    const uint32_t *col_abbits, *row_bbits;
    const int32_t *ab_rank;        // [q][column] rank after flipping bond q's A bit (packed path)
    int64_t ncols;
    int ab_fast;
    int8_t ab_pa[kMaxAB], ab_pb[kMaxAB];
    double ab_fjk[kMaxAB], ab_fkj[kMaxAB], ab_zz[kMaxAB];
    double scale;
};

constexpr int kHeisRowThreads = 512;

// bytes of the A-B bond facts ahead of the staged row (16-byte aligned)
__host__ __device__ inline size_t heis_row_head_bytes(int nab, size_t tsize)
{
    const size_t b = (size_t)nab * (sizeof(int64_t) + 3 * tsize + sizeof(uint32_t));
    return (b + 15) / 16 * 16;
}
constexpr int64_t kMaxPartialBlocksHeis = 1024;   // the partials that ed_scratch_bytes provides for

// Pass R: y[row] = s * (diag + A-A flips + A-B flips) of every row.
template <typename T>
__global__ void __launch_bounds__(kHeisRowThreads, 4) heis_row_kernel(const T *__restrict__ x, T *__restrict__ y,
                                                                    const HsArgs a)
{
    // dynamic shared memory: per-row A-B bond facts (nab entries each), then the staged row
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int64_t *ab_src = reinterpret_cast<int64_t *>(smem_raw);      // source row offset, -1 if impossible
    T *ab_c = reinterpret_cast<T *>(ab_src + a.nab);               // flip element for the required A state
    T *ab_dsame = ab_c + a.nab;                                    // zz/4 (generic path)
    T *ab_w2 = ab_dsame + a.nab;                                   // zz/2: drop of an antiparallel bond
    uint32_t *ab_need = reinterpret_cast<uint32_t *>(ab_w2 + a.nab);  // required A bit (1: A site down)
    T *xs = reinterpret_cast<T *>(smem_raw + heis_row_head_bytes(a.nab, sizeof(T)));
    const T *acf = reinterpret_cast<const T *>(a.aa_cf);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = kHeisRowThreads / 32;
    const T sc = (T)a.scale;
    for (int64_t row = blockIdx.x; row < a.nrows; row += gridDim.x) {
        const uint32_t hb = __ldg(a.row_pat + row);
        const int m = __ldg(a.row_m + row);
        const int64_t off = __ldg(a.row_off + row);
        const int len = (int)a.ncol[m];
        const int64_t cbase = a.col_base[m];
        const int64_t sbase = a.slice_base[m];
        const T db = __ldg(static_cast<const T *>(a.diagB) + row);
        const uint32_t rbits = a.ab_fast ? __ldg(a.row_bbits + row) : 0u;
        __syncthreads();   // the previous row's readers are done with xs / ab_*
        // asynchronous copies: the whole row in flight at once
        for (int c = threadIdx.x; c < len; c += blockDim.x) cp_async_elem(xs + c, x + off + c);
        for (int q = threadIdx.x; q < a.nab; q += blockDim.x) {
            const uint32_t hk = (hb >> a.ab_pb[q]) & 1u;
            // the flip needs the A site opposite to the B site: hj = 1 - hk
            const int32_t r2 = __ldg(a.rowidx + (hb ^ (1u << a.ab_pb[q])));
            ab_src[q] = (r2 >= 0) ? __ldg(a.row_off + r2) : (int64_t)-1;
            ab_need[q] = 1u - hk;
            ab_c[q] = (T)(hk ? a.ab_fkj[q] : a.ab_fjk[q]);   // target hj = 1-hk: hj ? fjk : fkj
            ab_dsame[q] = (T)a.ab_zz[q];
            ab_w2[q] = (T)(2.0 * a.ab_zz[q]);
        }
        cp_async_wait_all();
        __syncthreads();
        const int nsl = (len + 31) / 32;
        for (int sl = warp; sl < nsl; sl += nwarps) {
            const int c = sl * 32 + lane;
            const bool ok = c < len;
            const int cc = ok ? c : len - 1;
            const uint32_t ha = __ldg(a.col_pat + cbase + cc);
            T d = __ldg(static_cast<const T *>(a.diagA) + cbase + cc) + db;
            T acc = 0;
            const int s0 = __ldg(a.aa_off + sbase + sl), ns = __ldg(a.aa_off + sbase + sl + 1) - s0;
            if (sizeof(T) == 4) {
#pragma unroll 4
                for (int q = 0; q < ns; ++q) {
                    const int2 pk = __ldg(a.aa_pk32 + (s0 + q) * 32 + lane);
                    acc += (T)__int_as_float(pk.y) * xs[pk.x];
                }
            } else {
#pragma unroll 4
                for (int q = 0; q < ns; ++q) {
                    const int at = (s0 + q) * 32 + lane;
                    acc += __ldg(acf + at) * xs[__ldg(a.aa_src + at)];
                }
            }
            if (a.ab_fast) {
                // antiparallel A-B bonds: the set bits of (column's A bits ^ row's B bits); their
                // zz/4 was counted as "equal" in diagB, so each one drops the diagonal by zz/2
                uint32_t diff = __ldg(a.col_abbits + cbase + cc) ^ rbits;
                while (diff) {
                    const int q = __ffs(diff) - 1;
                    diff &= diff - 1;
                    d -= ab_w2[q];
                    const int64_t src = ab_src[q];
                    if (src >= 0) acc += ab_c[q] * __ldg(x + src + __ldg(a.ab_rank + q * a.ncols + cbase + cc));
                }
            } else
            for (int q = 0; q < a.nab; ++q) {
                const uint32_t hj = (ha >> a.ab_pa[q]) & 1u;
                if (hj != ab_need[q]) {
                    d += ab_dsame[q];          // equal sites
                    continue;
                }
                d -= ab_dsame[q];
                const int64_t src = ab_src[q];
                if (src >= 0) acc += ab_c[q] * __ldg(x + src + __ldg(a.rankA + (ha ^ (1u << a.ab_pa[q]))));
            }
            if (ok) y[off + c] = (d * xs[cc] + acc) * sc;
        }
    }
}

constexpr int kHeisCol4Threads = 1024;

// bytes of the four rows' A-B bond facts ahead of the staged columns (16-byte aligned)
__host__ __device__ inline size_t heis_col4_head_bytes(int nab)
{
    const size_t b = (size_t)nab * (4 * sizeof(int64_t) + 4 * sizeof(float) + sizeof(float));
    return (b + 15) / 16 * 16;
}

// G A-A flip slots of one lane (table entries at, at+32, ...) applied to the
// four staged rows; the G table loads are issued before the first gather.
template <int G>
__device__ __forceinline__ void heis_col4_group(const HsArgs &a, int at, const float4 *xs4, float (&acc)[4])
{
    int q[G];
    float c[G];
#pragma unroll
    for (int i = 0; i < G; ++i) {
        const int2 pk = __ldg(a.aa_pk32 + at + i * 32);
        q[i] = pk.x;
        c[i] = __int_as_float(pk.y);
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
        const float4 v = xs4[q[i]];
        acc[0] += c[i] * v.x;
        acc[1] += c[i] * v.y;
        acc[2] += c[i] * v.z;
        acc[3] += c[i] * v.w;
    }
}

// Pass R for FP32 with four rows of one hole count per CTA (packed A-B path):
// the four rows' entries of column c are staged as one 16-byte column xs4[c],
// so one A-A flip slot (an 8-byte table load) and one 128-bit gather serve all
// four rows.  Each row's sums are the one-row kernel's, in its order (slots,
// then the antiparallel A-B bonds in increasing order), so the product is the same.
// Work items are groups of four rows of rows_of_m, hole count by hole count.
__global__ void __launch_bounds__(kHeisCol4Threads, 1) heis_row_col4_kernel(const float *__restrict__ x,
                                                                          float *__restrict__ y, const HsArgs a,
                                                                          int64_t nitems)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int64_t *ab_src = reinterpret_cast<int64_t *>(smem_raw);      // [4][nab] source row offset, -1 if impossible
    float *ab_c = reinterpret_cast<float *>(ab_src + 4 * a.nab);   // [4][nab] flip element
    float *ab_w2 = ab_c + 4 * a.nab;                               // [nab] zz/2: drop of an antiparallel bond
    float4 *xs4 = reinterpret_cast<float4 *>(smem_raw + heis_col4_head_bytes(a.nab));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = kHeisCol4Threads / 32;
    const float sc = (float)a.scale;
    const float *dA32 = static_cast<const float *>(a.diagA), *dB32 = static_cast<const float *>(a.diagB);
    for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
        int m = 0;
        int64_t g = it;
        for (;;) {
            const int64_t ng = (a.row_base[m + 1] - a.row_base[m] + 3) / 4;
            if (g < ng) break;
            g -= ng;
            ++m;
        }
        const int nr = (int)min((int64_t)4, a.row_base[m + 1] - a.row_base[m] - 4 * g);
        int64_t off[4];
        float db[4];
        uint32_t rbits[4], hb[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int32_t row = __ldg(a.rows_of_m + a.row_base[m] + 4 * g + (r < nr ? r : 0));
            off[r] = __ldg(a.row_off + row);
            db[r] = __ldg(dB32 + row);
            rbits[r] = __ldg(a.row_bbits + row);
            hb[r] = __ldg(a.row_pat + row);
        }
        const int len = (int)a.ncol[m];
        const int64_t cbase = a.col_base[m];
        const int64_t sbase = a.slice_base[m];
        __syncthreads();   // the previous group's readers are done with xs4 / ab_*
        for (int c = threadIdx.x; c < len; c += blockDim.x) {
            float *dst = reinterpret_cast<float *>(xs4 + c);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (r < nr) cp_async_elem(dst + r, x + off[r] + c);
                else dst[r] = 0.f;
            }
        }
        for (int k = threadIdx.x; k < 4 * a.nab; k += blockDim.x) {
            const int r = k / a.nab, q = k - r * a.nab;
            int64_t src = -1;
            float cf = 0.f;
            if (r < nr) {
                const uint32_t h = (r == 0) ? hb[0] : (r == 1) ? hb[1] : (r == 2) ? hb[2] : hb[3];
                const uint32_t hk = (h >> a.ab_pb[q]) & 1u;
                const int32_t r2 = __ldg(a.rowidx + (h ^ (1u << a.ab_pb[q])));
                src = (r2 >= 0) ? __ldg(a.row_off + r2) : (int64_t)-1;
                cf = (float)(hk ? a.ab_fkj[q] : a.ab_fjk[q]);
            }
            ab_src[k] = src;
            ab_c[k] = cf;
            if (r == 0) ab_w2[q] = (float)(2.0 * a.ab_zz[q]);
        }
        cp_async_wait_all();
        __syncthreads();
        const int nsl = (len + 31) / 32;
        for (int sl = warp; sl < nsl; sl += nwarps) {
            const int c = sl * 32 + lane;
            const bool ok = c < len;
            const int cc = ok ? c : len - 1;
            const float dA = __ldg(dA32 + cbase + cc);
            float d[4], acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int r = 0; r < 4; ++r) d[r] = dA + db[r];
            const int s0 = __ldg(a.aa_off + sbase + sl), ns = __ldg(a.aa_off + sbase + sl + 1) - s0;
            // slots in groups: all table loads of a group are in flight before its first gather
            const int at0 = s0 * 32 + lane;
            int q = 0;
            for (; q + 8 <= ns; q += 8) heis_col4_group<8>(a, at0 + q * 32, xs4, acc);
            if (q + 4 <= ns) {
                heis_col4_group<4>(a, at0 + q * 32, xs4, acc);
                q += 4;
            }
            for (; q < ns; ++q) heis_col4_group<1>(a, at0 + q * 32, xs4, acc);
            // antiparallel A-B bonds of each row: the set bits of (column's A bits ^ row's B bits)
            const uint32_t ca = __ldg(a.col_abbits + cbase + cc);
            uint32_t diff[4], any = 0u;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                diff[r] = (r < nr) ? (ca ^ rbits[r]) : 0u;
                any |= diff[r];
            }
            while (any) {
                const int q = __ffs(any) - 1;
                any &= any - 1;
                const int rk = __ldg(a.ab_rank + q * a.ncols + cbase + cc);
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    if (!((diff[r] >> q) & 1u)) continue;
                    d[r] -= ab_w2[q];
                    const int64_t src = ab_src[r * a.nab + q];
                    if (src >= 0) acc[r] += ab_c[r * a.nab + q] * __ldg(x + src + rk);
                }
            }
            if (ok) {
                const float4 xv = xs4[cc];
                const float xr[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (r < nr) y[off[r] + c] = (d[r] * xr[r] + acc[r]) * sc;
            }
        }
    }
}

// Pass S: y += s * (B-B flips), fused <x,y>, <y,y>.  Work items run block
// (m) by block, slab by slab: all row groups of a block read one column slab
// of x while it sits in L2.
struct SlabPlan {
    int nblk;
    int m[kMaxHalf + 1];
    int64_t item_base[kMaxHalf + 2];
    int64_t slab_w[kMaxHalf + 1], ngroups[kMaxHalf + 1];
};

template <typename T>
__global__ void __launch_bounds__(256) heis_slab_kernel(const T *__restrict__ x, T *__restrict__ y, const HsArgs a,
                                                        const SlabPlan p, double *__restrict__ partials)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T *bcf = reinterpret_cast<const T *>(a.bb_cf);
    const T sc = (T)a.scale;
    double dxy = 0.0, dyy = 0.0;
    const int64_t nitems = p.item_base[p.nblk];
    for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
        int bi = 0;
        while (bi + 1 < p.nblk && p.item_base[bi + 1] <= it) ++bi;
        const int m = p.m[bi];
        const int64_t li = it - p.item_base[bi];
        const int64_t slab = li / p.ngroups[bi], g = li - slab * p.ngroups[bi];
        const int len = (int)a.ncol[m];
        const int64_t nr_m = a.row_base[m + 1] - a.row_base[m];
        const int64_t rr = g * 8 + warp;
        if (rr >= nr_m) continue;   // warp-uniform
        const int32_t row = __ldg(a.rows_of_m + a.row_base[m] + rr);
        const int64_t off = __ldg(a.row_off + row);
        const int e0 = __ldg(a.bb_ptr + row), nn = __ldg(a.bb_ptr + row + 1) - e0;
        const int64_t c0 = slab * p.slab_w[bi];
        const int64_t c1 = min((int64_t)len, c0 + p.slab_w[bi]);
        for (int eb = 0; eb < nn || eb == 0; eb += 32) {
            // neighbour rows of this chunk, one per lane
            const int ne = min(32, nn - eb);
            int64_t my_off = 0;
            T my_cf = 0;
            if (lane < ne) {
                my_off = __ldg(a.row_off + __ldg(a.bb_src + e0 + eb + lane));
                my_cf = __ldg(bcf + e0 + eb + lane);
            }
            const bool last = eb + 32 >= nn;
            T sxy = 0, syy = 0;
            // four 32-column chunks per pass: four independent loads per neighbour row
            for (int64_t cb = c0; cb < c1; cb += 128) {
                T acc[4] = {0, 0, 0, 0};
#pragma unroll 2
                for (int e = 0; e < ne; ++e) {
                    const int64_t so = __shfl_sync(0xffffffffu, my_off, e);
                    const T w = __shfl_sync(0xffffffffu, my_cf, e);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int64_t c = cb + 32 * j + lane;
                        if (c < c1) acc[j] += w * __ldg(x + so + c);
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int64_t c = cb + 32 * j + lane;
                    if (c < c1) {
                        const T yv = y[off + c] + acc[j] * sc;
                        y[off + c] = yv;
                        if (last) {
                            sxy += x[off + c] * yv;
                            syy += yv * yv;
                        }
                    }
                }
            }
            dxy += (double)sxy;
            dyy += (double)syy;
        }
    }
    if (partials) {
        __shared__ double red[2][8];
        dxy = warp_sum(dxy);
        dyy = warp_sum(dyy);
        if (lane == 0) {
            red[0][warp] = dxy;
            red[1][warp] = dyy;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sxy = 0.0, syy = 0.0;
            for (int w = 0; w < 8; ++w) {
                sxy += red[0][w];
                syy += red[1][w];
            }
            partials[2 * blockIdx.x] = sxy;
            partials[2 * blockIdx.x + 1] = syy;
        }
    }
}

// ------------------------------------------------------------ spin correlations
//
// J_SPIN of the Heisenberg solver (static_rq_heis.f90:58-116) on the row
// layout, per pair p = (J,K) of the caller's list:
//   q[p][0] = J!=K: sum over states I with J up, K down of (-1)^(J+K) bra[I'] ket[I]
//             (I' = I with J and K swapped);  J==K: 0.5 sum bra ket
//   q[p][1] = sum bra ket Sz_J Sz_K
// The per-pair kernel forms only the transverse (flip) sums q0 of J != K:
// CTAs are (row range, chunk of kRdmP pairs); each thread keeps the chunk's
// sums in registers over all its rows, so one pass over the vector serves
// kRdmP pairs.  The diagonal sums (q1 of every pair, q0 of J == K) come from
// heis_rdm_diag_kernel, factorised: with s_j = +1 / -1 for site j+1 up /
// down and b = bra*ket, sum b s_J s_K is sum_col C(col) s_J s_K for two A
// sites, sum_row W(row) s_J s_K for two B sites and sum_col s_J T_K(col) for
// an A site J and a B site K, where per class m of rows C(col) = sum_row b,
// T_K(col) = sum_row b s_K(row) and W(row) = sum_col b: ~nB FP64 operations
// per element for every pair at once.

constexpr int kRdmP = 8;
constexpr int kRdmThreads = 256;

struct HsRdmArgs {
    int nA, npairs;
    int64_t nrows;
    int64_t col_base[kMaxHalf + 2], ncol[kMaxHalf + 1];
    const uint32_t *col_pat, *row_pat;
    const int32_t *rankA, *row_m, *rowidx;
    const int64_t *row_off;
    int16_t pj[kMaxSites * kMaxSites], pk[kMaxSites * kMaxSites];   // hole-bit positions (site-1)
    // the diagonal pass: rows grouped by m, and its tiles per m (columns x row ranges)
    const int32_t *rows_of_m;
    int64_t row_base[kMaxHalf + 2];
    int tile_base[kMaxHalf + 2], nry[kMaxHalf + 1];
};

template <typename T>
__global__ void __launch_bounds__(kRdmThreads) heis_rdm_row_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                                   const HsRdmArgs a, double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);   // the bra row
    const int p0 = blockIdx.y * kRdmP;
    const int np = min(kRdmP, a.npairs - p0);
    const int nA = a.nA;
    double acc0[kRdmP], acc1[kRdmP];
#pragma unroll
    for (int q = 0; q < kRdmP; ++q) acc0[q] = acc1[q] = 0.0;
    for (int64_t row = blockIdx.x; row < a.nrows; row += gridDim.x) {
        const uint32_t hb = __ldg(a.row_pat + row);
        const int m = __ldg(a.row_m + row);
        const int64_t off = __ldg(a.row_off + row);
        const int len = (int)a.ncol[m];
        const int64_t cbase = a.col_base[m];
        __syncthreads();
        for (int c = threadIdx.x; c < len; c += blockDim.x) xs[c] = bra[off + c];
        __syncthreads();
        // per-row facts of every pair: source row offset of the swapped state (or -1)
        int64_t soff[kRdmP];
#pragma unroll
        for (int q = 0; q < kRdmP; ++q) {
            soff[q] = -1;
            if (q >= np) continue;
            const int J = a.pj[p0 + q], K = a.pk[p0 + q];
            uint32_t mb = 0;
            if (J >= nA) mb |= 1u << (J - nA);
            if (K >= nA) mb |= 1u << (K - nA);
            if (mb) {
                const int32_t r2 = __ldg(a.rowidx + (hb ^ mb));
                if (r2 >= 0) soff[q] = __ldg(a.row_off + r2);
            } else {
                soff[q] = off;
            }
        }
        T r0[kRdmP], r1[kRdmP];
#pragma unroll
        for (int q = 0; q < kRdmP; ++q) r0[q] = r1[q] = 0;
        for (int c = threadIdx.x; c < len; c += blockDim.x) {
            const uint32_t ha = __ldg(a.col_pat + cbase + c);
            const uint64_t h = (uint64_t)ha | ((uint64_t)hb << nA);   // bit j: site j+1 is down
            const T kv = __ldg(ket + off + c);
#pragma unroll
            for (int q = 0; q < kRdmP; ++q) {
                if (q >= np) break;
                const int J = a.pj[p0 + q], K = a.pk[p0 + q];
                const int dJ = (int)((h >> J) & 1u), dK = (int)((h >> K) & 1u);
                if (J == K || dJ || !dK || soff[q] < 0) continue;   // a flip needs J up, K down
                // the swapped state: A part and B part of h ^ (bit J | bit K)
                uint32_t ma = 0;
                if (J < nA) ma |= 1u << J;
                if (K < nA) ma |= 1u << K;
                const int cs = ma ? __ldg(a.rankA + (ha ^ ma)) : c;
                const T bv = (soff[q] == off) ? xs[cs] : __ldg(bra + soff[q] + cs);
                // sign (-1)^((J+1)+(K+1)) folded into the FMA's operand: one operation per flip
                r0[q] = ((J + K) & 1) ? fma(-bv, kv, r0[q]) : fma(bv, kv, r0[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < kRdmP; ++q) {
            acc0[q] += (double)r0[q];
            acc1[q] += (double)r1[q];
        }
    }
    __shared__ double red[kRdmThreads / 32][kRdmP][2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < kRdmP; ++q) {
        const double w0 = warp_sum(acc0[q]), w1 = warp_sum(acc1[q]);
        if (lane == 0) {
            red[warp][q][0] = w0;
            red[warp][q][1] = w1;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 * np) {
        const int q = threadIdx.x >> 1, k = threadIdx.x & 1;
        double t = 0.0;
        for (int w = 0; w < kRdmThreads / 32; ++w) t += red[w][q][k];
        partials[((int64_t)blockIdx.x * a.npairs + p0 + q) * 2 + k] = t;
    }
}

constexpr int kHdThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kHdThreads) heis_rdm_diag_kernel(const T *__restrict__ bra, const T *__restrict__ ket,
                                                                   const HsRdmArgs a, int mlo, int mhi,
                                                                   double *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *Ts = reinterpret_cast<double *>(smem_raw);   // [kMaxHalf][kHdThreads]
    double *Cs = Ts + kMaxHalf * kHdThreads;              // [kHdThreads]
    double *accW = Cs + kHdThreads;                       // [npairs]
    __shared__ double red[kHdThreads / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int m = mlo;
    while (m < mhi && blockIdx.x >= a.tile_base[m + 1]) ++m;
    const int ncx = (int)((a.ncol[m] + kHdThreads - 1) / kHdThreads);
    const int local = blockIdx.x - a.tile_base[m];
    const int cx = local % ncx, ry = local / ncx, nry = a.nry[m];
    const int64_t col = (int64_t)cx * kHdThreads + threadIdx.x;
    const bool act = col < a.ncol[m];
    const int64_t nr_m = a.row_base[m + 1] - a.row_base[m];
    const int64_t q0r = nr_m * ry / nry, q1r = nr_m * (ry + 1) / nry;
    const int nA = a.nA;
    for (int q = threadIdx.x; q < a.npairs; q += blockDim.x) accW[q] = 0.0;
    double C = 0.0, Tk[kMaxHalf];
#pragma unroll
    for (int k = 0; k < kMaxHalf; ++k) Tk[k] = 0.0;
    for (int64_t rr = q0r; rr < q1r; ++rr) {
        const int32_t row = __ldg(a.rows_of_m + a.row_base[m] + rr);
        const uint32_t hb = __ldg(a.row_pat + row);
        const int64_t off = __ldg(a.row_off + row);
        const double b = act ? (double)__ldg(bra + off + col) * (double)__ldg(ket + off + col) : 0.0;
        C += b;
#pragma unroll
        for (int k = 0; k < kMaxHalf; ++k) Tk[k] += ((hb >> k) & 1u) ? -b : b;
        double w = warp_sum(b);
        __syncthreads();
        if (lane == 0) red[warp] = w;
        __syncthreads();
        w = 0.0;
#pragma unroll
        for (int q = 0; q < kHdThreads / 32; ++q) w += red[q];
        for (int q = threadIdx.x; q < a.npairs; q += blockDim.x) {
            const int J = a.pj[q], K = a.pk[q];
            if (J >= nA && K >= nA && J != K) {
                const int sJ = ((hb >> (J - nA)) & 1u) ? -1 : 1, sK = ((hb >> (K - nA)) & 1u) ? -1 : 1;
                accW[q] += (sJ * sK > 0) ? w : -w;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kMaxHalf; ++k) Ts[k * kHdThreads + threadIdx.x] = Tk[k];
    Cs[threadIdx.x] = C;
    __syncthreads();
    for (int q = warp; q < a.npairs; q += kHdThreads / 32) {
        const int J = a.pj[q], K = a.pk[q];
        double s1 = 0.0;
        for (int t = lane; t < kHdThreads; t += 32) {
            const int64_t cc = (int64_t)cx * kHdThreads + t;
            if (cc >= a.ncol[m]) continue;
            const uint32_t ha = __ldg(a.col_pat + a.col_base[m] + cc);
            if (J == K) {
                s1 += Cs[t];
            } else if (J < nA && K < nA) {
                const bool neg = (((ha >> J) ^ (ha >> K)) & 1u) != 0;
                s1 += neg ? -Cs[t] : Cs[t];
            } else if (J < nA || K < nA) {
                const int ja = J < nA ? J : K, kb = (J < nA ? K : J) - nA;
                const double tv = Ts[kb * kHdThreads + t];
                s1 += ((ha >> ja) & 1u) ? -tv : tv;
            }
        }
        s1 = warp_sum(s1);
        if (lane == 0) {
            double *o = partials + ((int64_t)blockIdx.x * a.npairs + q) * 2;
            if (J == K) {
                o[0] = 0.5 * s1;
                o[1] = 0.25 * s1;
            } else {
                o[0] = 0.0;
                o[1] = 0.25 * ((J >= nA && K >= nA) ? accW[q] : s1);
            }
        }
    }
}

template <typename T>
static int heis_struct_rdm_run(ed_sector *s, cudaStream_t st, const T *bra, const T *ket, int npairs,
                               const int32_t *pairs, double *out, double *scratch, int max_blocks)
{
    const HeisStruct &h = *s->hs;
    HsRdmArgs a;
    a.nA = h.nA;
    a.npairs = npairs;
    a.nrows = h.nrows;
    for (int m = 0; m <= kMaxHalf + 1; ++m) {
        a.col_base[m] = h.col_base[m];
        if (m <= kMaxHalf) a.ncol[m] = h.ncol[m];
    }
    a.col_pat = h.col_pat; a.row_pat = h.row_pat;
    a.rankA = h.rankA; a.row_m = h.row_m; a.rowidx = h.rowidx; a.row_off = h.row_off;
    for (int p = 0; p < npairs; ++p) {
        a.pj[p] = (int16_t)(pairs[2 * p] - 1);
        a.pk[p] = (int16_t)(pairs[2 * p + 1] - 1);
    }
    if (h.nB > kMaxHalf) {
        set_error("B half of %d sites (at most %d)", h.nB, kMaxHalf);
        return ED_ERR_RANGE;
    }
    a.rows_of_m = h.rows_of_m;
    for (int m = 0; m <= kMaxHalf + 1; ++m) a.row_base[m] = h.row_base[m];
    // diagonal tiles: per class m, 256-column tiles times row ranges, about max_blocks in all
    const int64_t dim = s->dim;
    int ntiles = 0;
    for (int m = 0; m <= kMaxHalf + 1; ++m) a.tile_base[m] = 0;
    for (int m = h.mlo; m <= h.mhi; ++m) {
        a.tile_base[m] = ntiles;
        const int64_t nr_m = h.row_base[m + 1] - h.row_base[m];
        const int ncx = (int)((h.ncol[m] + kHdThreads - 1) / kHdThreads);
        const double share = dim > 0 ? (double)(h.ncol[m] * nr_m) / (double)dim : 0.0;
        int nry = (int)std::max<double>(1.0, std::floor(share * max_blocks / std::max(ncx, 1)));
        nry = (int)std::min<int64_t>(std::max<int64_t>(nr_m, 1), nry);
        a.nry[m] = nry;
        ntiles += ncx * nry;
    }
    a.tile_base[h.mhi + 1] = ntiles;
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(h.nrows, max_blocks));
    if (gx + ntiles > 3 * max_blocks) {
        set_error("spin-correlation pass needs %d partial rows (scratch holds %d)", gx + ntiles, 3 * max_blocks);
        return ED_ERR_RANGE;
    }
    // flips (q0 of J != K) into partial rows [0, gx), diagonal sums into [gx, gx + ntiles)
    const size_t smem = (size_t)std::max<int64_t>(h.max_len, 1) * sizeof(T);
    ED_CHECK_CUDA(cudaFuncSetAttribute(heis_rdm_row_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const dim3 grid((unsigned)gx, (unsigned)((npairs + kRdmP - 1) / kRdmP));
    heis_rdm_row_kernel<T><<<grid, kRdmThreads, smem, st>>>(bra, ket, a, scratch);
    ED_CHECK_LAUNCH();
    const size_t smemd = (size_t)(kMaxHalf + 1) * kHdThreads * sizeof(double) + (size_t)npairs * sizeof(double);
    ED_CHECK_CUDA(cudaFuncSetAttribute(heis_rdm_diag_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smemd));
    heis_rdm_diag_kernel<T><<<ntiles, kHdThreads, smemd, st>>>(bra, ket, a, h.mlo, h.mhi,
                                                                scratch + (int64_t)gx * 2 * npairs);
    ED_CHECK_LAUNCH();
    return launch_reduce(scratch, gx + ntiles, 2 * npairs, out, st);
}

int heis_struct_rdm(ed_sector *s, cudaStream_t st, int dtype, const void *bra, const void *ket, int npairs,
                    const int32_t *pairs, double *out, double *scratch, int max_blocks)
{
    if (!s->hs) {
        set_error("Heisenberg sector without its row tables");
        return ED_ERR_ARG;
    }
    if (dtype == ED_F32)
        return heis_struct_rdm_run<float>(s, st, static_cast<const float *>(bra), static_cast<const float *>(ket),
                                          npairs, pairs, out, scratch, max_blocks);
    return heis_struct_rdm_run<double>(s, st, static_cast<const double *>(bra), static_cast<const double *>(ket),
                                       npairs, pairs, out, scratch, max_blocks);
}

template <typename T>
static int heis_struct_run(ed_sector *s, cudaStream_t st, const T *x, T *y, double scale, double *dots,
                           double *partials)
{
    const HeisStruct &h = *s->hs;
    HsArgs a;
    a.nA = h.nA;
    a.nB = h.nB;
    a.nab = h.nab;
    a.nrows = h.nrows;
    for (int m = 0; m <= kMaxHalf + 1; ++m) {
        a.col_base[m] = h.col_base[m];
        a.slice_base[m] = h.slice_base[m];
        a.row_base[m] = h.row_base[m];
        if (m <= kMaxHalf) a.ncol[m] = h.ncol[m];
    }
    a.col_pat = h.col_pat; a.row_pat = h.row_pat;
    a.rankA = h.rankA; a.aa_off = h.aa_off; a.aa_src = h.aa_src; a.row_m = h.row_m;
    a.rowidx = h.rowidx; a.bb_ptr = h.bb_ptr; a.bb_src = h.bb_src; a.rows_of_m = h.rows_of_m;
    a.row_off = h.row_off;
    a.diagA = (sizeof(T) == 4) ? (const void *)h.diagA32 : (const void *)h.diagA;
    a.diagB = (sizeof(T) == 4) ? (const void *)h.diagB32 : (const void *)h.diagB;
    a.aa_cf = (sizeof(T) == 4) ? (const void *)h.aa_cf32 : (const void *)h.aa_cf64;
    a.aa_pk32 = h.aa_pk32;
    a.col_abbits = h.col_abbits;
    a.row_bbits = h.row_bbits;
    a.ab_rank = h.ab_rank;
    a.ncols = h.ncols;
    a.ab_fast = h.ab_fast ? 1 : 0;
    a.bb_cf = (sizeof(T) == 4) ? (const void *)h.bb_cf32 : (const void *)h.bb_cf64;
    for (int q = 0; q < h.nab; ++q) {
        a.ab_pa[q] = h.ab_pa[q]; a.ab_pb[q] = h.ab_pb[q];
        a.ab_fjk[q] = h.ab_fjk[q]; a.ab_fkj[q] = h.ab_fkj[q]; a.ab_zz[q] = h.ab_zz[q];
    }
    a.scale = scale;
    const int nsm = num_sms();
    // ---- pass R
    int maxsm = 0;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t smem4 = heis_col4_head_bytes(h.nab) + (size_t)std::max<int64_t>(h.max_len, 1) * 16;
    // FP32 with the packed A-B path: four rows of one hole count per CTA when their columns
    // fit (PYHUB_ED_HEIS_ROWS=1 selects the one-row pass; both give the same product)
    const char *one = std::getenv("PYHUB_ED_HEIS_ROWS");
    if (sizeof(T) == 4 && h.ab_fast && smem4 <= (size_t)maxsm && !(one && one[0] == '1')) {
        int64_t nitems = 0;
        for (int m = 0; m <= h.nA; ++m) nitems += (h.row_base[m + 1] - h.row_base[m] + 3) / 4;
        ED_CHECK_CUDA(cudaFuncSetAttribute(heis_row_col4_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem4));
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, heis_row_col4_kernel, kHeisCol4Threads, smem4);
        if (per_sm < 1) per_sm = 1;
        int64_t blocks = std::min<int64_t>(nitems, (int64_t)nsm * per_sm);
        if (blocks < 1) blocks = 1;
        heis_row_col4_kernel<<<(unsigned)blocks, kHeisCol4Threads, smem4, st>>>(
            reinterpret_cast<const float *>(x), reinterpret_cast<float *>(y), a, nitems);
    } else {
        const size_t smem = heis_row_head_bytes(h.nab, sizeof(T)) + (size_t)std::max<int64_t>(h.max_len, 1) * sizeof(T);
        ED_CHECK_CUDA(cudaFuncSetAttribute(heis_row_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int64_t blocks = std::min<int64_t>(h.nrows, (int64_t)nsm * 4);
        if (blocks < 1) blocks = 1;
        heis_row_kernel<T><<<(unsigned)blocks, kHeisRowThreads, smem, st>>>(x, y, a);
    }
    ED_CHECK_LAUNCH();
    // ---- pass S
    SlabPlan p;
    p.nblk = 0;
    p.item_base[0] = 0;
    for (int m = 0; m <= h.nA; ++m) {
        const int64_t nr = h.row_base[m + 1] - h.row_base[m];
        if (nr == 0) continue;
        const int64_t len = h.ncol[m];
        // the x slab of the block (nr rows x w) should take at most ~48 MB of L2
        int64_t w = (int64_t)(48.0e6 / ((double)nr * sizeof(T)));
        w = w / 32 * 32;
        if (w < 256) w = 256;
        if (w > len) w = len;
        const int b = p.nblk++;
        p.m[b] = m;
        p.slab_w[b] = w;
        p.ngroups[b] = (nr + 7) / 8;
        p.item_base[b + 1] = p.item_base[b] + ((len + w - 1) / w) * p.ngroups[b];
    }
    int64_t blocks2 = std::min<int64_t>((int64_t)nsm * 8, kMaxPartialBlocksHeis);
    if (blocks2 > p.item_base[p.nblk]) blocks2 = p.item_base[p.nblk];
    if (blocks2 < 1) blocks2 = 1;
    heis_slab_kernel<T><<<(unsigned)blocks2, 256, 0, st>>>(x, y, a, p, dots ? partials : nullptr);
    ED_CHECK_LAUNCH();
    if (dots) return launch_reduce(partials, (int)blocks2, 2, dots, st);
    return ED_OK;
}

int heis_struct_hv(ed_sector *s, cudaStream_t st, int dtype, const void *x, void *y, double scale, double *dots,
                   double *partials)
{
    if (!s->hs) {
        set_error("Heisenberg sector without its row tables");
        return ED_ERR_ARG;
    }
    if (dtype == ED_F32)
        return heis_struct_run<float>(s, st, static_cast<const float *>(x), static_cast<float *>(y), scale, dots,
                                      partials);
    return heis_struct_run<double>(s, st, static_cast<const double *>(x), static_cast<double *>(y), scale, dots,
                                   partials);
}

}  // namespace ed
