// ed_batch.cu -- many independent three-term Lanczos runs advanced together.
//
// Replaces the Green's-function Lanczos loops of the reference, which run
// one start block after another (GF_BANDLANCZOS, spgf_bandlanczos.f90:309-448,
// called per particle/hole and spin sector, :63-288).  Here every start
// vector of every cluster is an instance; one step of all instances is two
// kernels over an instance-major grid:
//   step_hv:     s_k = 1/beta_k (reduced from the previous partials),
//                y = s_k H u_k,  partial <u_k, y>
//   step_update: alpha_k = s_k sum partials,
//                u_{k+1} = y - alpha_k s_k u_k - beta_k s_{k-1} u_{k-1},
//                partial ||u_{k+1}||^2
// Stored vectors u_k are unnormalised (norm beta_k); scales stay on the
// device, so a whole run enqueues with no host synchronisation and can be
// captured in a CUDA graph.  alpha/beta are written per instance and step
// for the continued fraction <phi|(z-H)^-1|phi> = beta_0^2/(z-a_0-b_1^2/...).
//
// Sectors here are small (D ~ 1e5..1e6): each CTA stages R rows of u_k in
// shared memory for the up hops and reads the neighbour rows of the down
// hops straight from L2, where the instances in flight keep their vectors.
#include "ed_common.cuh"

#include <algorithm>
#include <mutex>
#include <vector>

namespace ed {

constexpr int kDefaultRows = 8;   // rows of one instance per CTA (4, 8 or 16; chosen per batch)
constexpr int kBatchThreads = 256;

struct BatchInst {
    int64_t nsup, nsdn, ld, off;      // off: first element of this instance in the work arrays
    const uint32_t *ustr, *dstr;
    const int32_t *uptr, *usrc, *dptr, *dsrc;
    const float *ucf32, *dcf32;
    const double *ucf64, *dcf64;
    const double *uediag, *dediag;
    const float *uediag32, *dediag32;
    const double *u_site;             // device, indexed by bit
    const float *u_site32;
    const int32_t *ell_off, *ell_src; // sliced-ELL up-hop table of the sector
    const float *ell_cf32;
    const double *ell_cf64;
    const int2 *ell_pk32;
    int nslice;
    double u_value;
    float u_value32;
    int u_uniform;
    int64_t blk0;                     // first CTA of this instance
    int nblk;
    int rows;                         // rows per CTA of the batch
};

}  // namespace ed

struct ed_batch {
    int ninst = 0;
    int64_t total = 0;                 // elements of one concatenated vector
    int64_t nblocks = 0;
    ed::BatchInst *dev = nullptr;      // [ninst]
    int32_t *blk_inst = nullptr;       // [nblocks] device: instance of every CTA
    double *u_site_all = nullptr;      // [ninst][kMaxSites] device
    float *u_site_all32 = nullptr;     // the same in FP32
    std::vector<int64_t> offsets, dims;
    int max_nsup = 0;
    int max_ld = 0;
    int rows = 8;                      // rows per CTA (4, 8 or 16)
    int32_t *order = nullptr;          // [nblocks] device: persistent-run item order of one super-phase
    int8_t *grp = nullptr;             // [ninst] device: phase offset (0 or 1) of each instance
    double wait_s = 10.0;              // persistent run: limit of every wait, in seconds of GPU time
    int stall_inst = -1;               // persistent run: instance whose first H*v phase never completes (-1: none)
};

namespace ed {

// Per-instance scalars, kept on the device between the kernels of a step.
enum { kS = 0, kSPrev = 1, kBeta = 2, kCCur = 3, kCPrev = 4, kScal = 8 };

__device__ __forceinline__ double sum_partials_warp(const double *__restrict__ part, int64_t b0, int n)
{
    // fixed lane/order pattern: the same partials always give the same sum
    double s = 0.0;
    for (int q = threadIdx.x & 31; q < n; q += 32) s += part[b0 + q];
    return warp_sum(s);
}

template <typename T>
__device__ __forceinline__ T u_energy_b(const BatchInst &a, uint32_t both)
{
    if (a.u_uniform) return ((sizeof(T) == 4) ? (T)a.u_value32 : (T)a.u_value) * (T)__popc(both);
    const T *us = (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.u_site32) : reinterpret_cast<const T *>(a.u_site);
    T e = 0;
    while (both) {
        const int b = __ffs(both) - 1;
        e += us[b];
        both &= both - 1;
    }
    return e;
}

__device__ __forceinline__ void block_partial(double v, double *__restrict__ out)
{
    __shared__ double red[kBatchThreads / 32];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBatchThreads / 32; ++w) t += red[w];
        *out = t;
    }
}

// Norms of the start vectors: partial ||x0||^2 per CTA.
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_norm_kernel(const BatchInst *__restrict__ inst,
                                                                   const int32_t *__restrict__ blk_inst,
                                                                   const T *__restrict__ x, double *__restrict__ part)
{
    const int64_t b = blockIdx.x;
    const BatchInst &a = inst[__ldg(blk_inst + b)];
    const int64_t r0 = (b - a.blk0) * a.rows;
    const int nr = (int)min((int64_t)a.rows, a.nsdn - r0);
    double s = 0.0;
    for (int r = 0; r < nr; ++r) {
        const T *row = x + a.off + (r0 + r) * a.ld;
        for (int64_t c = threadIdx.x; c < a.nsup; c += blockDim.x) s += (double)row[c] * (double)row[c];
    }
    block_partial(s, part + b);
}

// One warp per instance.  mode 0 (after a norm / update pass):
//   beta_k = sqrt(sum), s_{k-1} <- s_k, s_k = 1/beta_k; beta[i][k] written.
// mode 1 (after the H*v pass of step k):
//   alpha_k = s_k sum <u_k, y>; c_cur = alpha_k s_k, c_prev = beta_k s_{k-1}.
__global__ void batch_scalar_kernel(const BatchInst *__restrict__ inst, int ninst, const double *__restrict__ part,
                                    double *__restrict__ scal, double *__restrict__ alpha,
                                    double *__restrict__ beta, int k, int nsteps, int mode)
{
    const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (i >= ninst) return;
    const BatchInst &a = inst[i];
    const double sum = sum_partials_warp(part, a.blk0, a.nblk);
    if ((threadIdx.x & 31) != 0) return;
    double *sc = scal + (int64_t)i * kScal;
    if (mode == 0) {
        const double bk = sqrt(fmax(sum, 0.0));
        sc[kSPrev] = (k == 0) ? 0.0 : sc[kS];
        sc[kS] = (bk > 1e-150) ? 1.0 / bk : 0.0;
        sc[kBeta] = bk;
        beta[(int64_t)i * (nsteps + 1) + k] = bk;
    } else {
        const double al = sc[kS] * sum;
        alpha[(int64_t)i * nsteps + k] = al;
        sc[kCCur] = al * sc[kS];
        sc[kCPrev] = sc[kBeta] * sc[kSPrev];
    }
}

constexpr int kMaxNb = 48;      // down-hop neighbours of a row staged in shared memory


// 16-byte vectors: float4 / double2.
template <typename T> struct V16;
template <> struct V16<float> {
    using type = float4;
    static constexpr int n = 4;
};
template <> struct V16<double> {
    using type = double2;
    static constexpr int n = 2;
};
__device__ __forceinline__ float &vat(float4 &v, int k) { return reinterpret_cast<float *>(&v)[k]; }
__device__ __forceinline__ double &vat(double2 &v, int k) { return reinterpret_cast<double *>(&v)[k]; }

// A down-hop neighbour: element offset of the source row and its coefficient.
template <typename T> struct alignas(sizeof(T) == 4 ? 8 : 16) NbEnt {
    int off;
    T cf;
};

// Column c of the staged block: rows 0..R-1 of string c.  The column stride
// in 16-byte units is made odd (padding by 16 bytes when R rows fill an even
// number), so that column c starts in bank group (odd * c) mod 8: 8
// consecutive or otherwise distinct-mod-8 columns hit 8 different groups.
// FP32: 16, 48, 80 bytes for R = 4, 8, 16; FP64: 48, 80, 144 bytes.
template <typename T, int R> __host__ __device__ constexpr int staged_stride()
{
    return ((R * (int)sizeof(T) / 16) % 2 == 0) ? R + 16 / (int)sizeof(T) : R;
}

template <typename T, int R>
__device__ __forceinline__ void load_column(const T *p, T (&v)[R])
{
    using V = typename V16<T>::type;
#pragma unroll
    for (int q = 0; q < R / V16<T>::n; ++q) {
        const V w = reinterpret_cast<const V *>(p)[q];
#pragma unroll
        for (int k = 0; k < V16<T>::n; ++k) v[q * V16<T>::n + k] = reinterpret_cast<const T *>(&w)[k];
    }
}

// G up-hop slots of one lane (table entries at `at`, `at`+32, ...): the G
// table loads are issued before the first gather.
template <typename T, int G, int R>
__device__ __forceinline__ void up_group(const BatchInst &a, const T *xs, int at, T (&acc)[R])
{
    constexpr int S = staged_stride<T, R>();
    int src[G];
    T w[G];
#pragma unroll
    for (int j = 0; j < G; ++j) {
        if (sizeof(T) == 4) {
            const int2 pk = __ldg(a.ell_pk32 + at + 32 * j);
            src[j] = pk.x;
            w[j] = (T)__int_as_float(pk.y);
        } else {
            src[j] = __ldg(a.ell_src + at + 32 * j);
            w[j] = (T)__ldg(a.ell_cf64 + at + 32 * j);
        }
    }
#pragma unroll
    for (int j = 0; j < G; ++j) {
        T xv[R];
        load_column<T, R>(xs + src[j] * S, xv);
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] += w[j] * xv[r];
    }
}

// G down-hop neighbour rows (16-byte vector v of each): loads issued together
// (COH: ordinary weak loads, for the persistent run).
template <typename T, int G, bool COH>
__device__ __forceinline__ void down_group(const NbEnt<T> *en, const T *__restrict__ ub, int v,
                                           typename V16<T>::type &acc)
{
    using V = typename V16<T>::type;
    V xn[G];
    T cf[G];
#pragma unroll
    for (int j = 0; j < G; ++j) {
        const NbEnt<T> e = en[j];
        cf[j] = e.cf;
        if constexpr (COH) xn[j] = __ldca(reinterpret_cast<const V *>(ub + e.off) + v);
        else xn[j] = __ldg(reinterpret_cast<const V *>(ub + e.off) + v);
    }
#pragma unroll
    for (int j = 0; j < G; ++j)
#pragma unroll
        for (int k = 0; k < V16<T>::n; ++k) vat(acc, k) += cf[j] * reinterpret_cast<const T *>(&xn[j])[k];
}

// Loads of data another CTA may have written earlier in the same launch
// (the persistent run): ordinary weak loads (ld.global.ca, or cp.async for
// the staged rows), each after the CTA's acquire load of the instance's phase
// counter, which the writers published with fence + release.  The PTX memory
// model makes those writes visible to weak loads ordered after the acquire;
// it gives no such guarantee to the non-coherent read-only path (ld.global.nc),
// which only loads of data written before the launch use.
template <bool COH, typename V> __device__ __forceinline__ V ld_data(const V *p)
{
    if constexpr (COH) return __ldca(p);
    else return __ldg(p);
}

// y = s_k H u_k and partial <u_k, y> over R rows of one instance.
// Phase A (diagonal + up hops): the rows are staged in shared memory one
// column per string (asynchronous copies, all in flight together); a warp owns 32-string
// slices, loads each sliced-ELL slot once and applies it to all rows with
// 16-byte shared loads; the sums go to y.  Phase B (down hops): each row
// adds its neighbour rows as 16-byte-vector axpys read from L2 (the
// instances in flight keep their vectors there), then scales, stores and
// forms the dot product.
template <typename T, int R, bool COH>
__device__ __forceinline__ void hv_item(const BatchInst *__restrict__ inst, int64_t b, int i,
                                        const T *__restrict__ u, T *__restrict__ y, double sk,
                                        double *__restrict__ part_out, unsigned char *smem_raw)
{
    using V = typename V16<T>::type;
    constexpr int VN = V16<T>::n;
    constexpr int S = staged_stride<T, R>();
    T *xs = reinterpret_cast<T *>(smem_raw);   // [nsup][S]
    __shared__ NbEnt<T> nb[R][kMaxNb];
    __shared__ int nb_n[R], nb_e0[R];
    __shared__ uint32_t row_str[R];
    __shared__ T row_ed[R];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = kBatchThreads / 32;
    const BatchInst &a = inst[i];
    const int r0 = (int)((b - a.blk0) * R);
    const int nr = (int)min((int64_t)R, a.nsdn - r0);
    const int nsup = (int)a.nsup, ld = (int)a.ld;
    const T *ub = u + a.off;
    T *yb = y + a.off + (int64_t)r0 * ld;
    const T *dcf = (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.dcf32) : reinterpret_cast<const T *>(a.dcf64);
    const T *ued_t = (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.uediag32) : reinterpret_cast<const T *>(a.uediag);
    const T *ded_t = (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.dediag32) : reinterpret_cast<const T *>(a.dediag);
    for (int r = 0; r < R; ++r) {
        const T *src = ub + (int64_t)(r0 + r) * ld;
        for (int c = threadIdx.x; c < nsup; c += blockDim.x) {
            if (r < nr)
                cp_async_elem(xs + c * S + r, src + c);
            else
                xs[c * S + r] = (T)0;
        }
    }
    for (int r = warp; r < R; r += nwarps) {
        int e0 = 0, nn = 0;
        if (r < nr) {
            e0 = __ldg(a.dptr + r0 + r);
            nn = __ldg(a.dptr + r0 + r + 1) - e0;
        }
        for (int e = lane; e < min(nn, kMaxNb); e += 32) {
            nb[r][e].off = __ldg(a.dsrc + e0 + e) * ld;
            nb[r][e].cf = __ldg(dcf + e0 + e);
        }
        if (lane == 0) {
            nb_n[r] = nn;
            nb_e0[r] = e0;
            row_str[r] = (r < nr) ? __ldg(a.dstr + r0 + r) : 0u;
            row_ed[r] = (r < nr) ? __ldg(ded_t + r0 + r) : (T)0;
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // ---- phase A
    for (int sl = warp; sl < a.nslice; sl += nwarps) {
        const int c = sl * 32 + lane;
        const bool ok = c < nsup;
        const int cc = ok ? c : nsup - 1;
        const uint32_t su = __ldg(a.ustr + cc);
        const T ued = __ldg(ued_t + cc);
        T acc[R], xv[R];
        load_column<T, R>(xs + cc * S, xv);
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = (ued + row_ed[r] + u_energy_b<T>(a, su & row_str[r])) * xv[r];
        const int s0 = __ldg(a.ell_off + sl), ns = __ldg(a.ell_off + sl + 1) - s0;
        // slots in groups: all table loads of a group are in flight before
        // its first gather
        int q = 0;
        for (; q + 8 <= ns; q += 8) up_group<T, 8, R>(a, xs, (s0 + q) * 32 + lane, acc);
        if (q + 4 <= ns) {
            up_group<T, 4, R>(a, xs, (s0 + q) * 32 + lane, acc);
            q += 4;
        }
        for (; q < ns; ++q) up_group<T, 1, R>(a, xs, (s0 + q) * 32 + lane, acc);
        if (ok) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (r < nr) yb[r * ld + c] = acc[r];
        }
    }
    __syncthreads();   // phase A's rows of y are visible to the whole CTA
    // ---- phase B
    const T sc = (T)sk;
    const int nvec = ld / VN, chunks = (nvec + 31) / 32;
    T dotp = 0;
    for (int task = warp; task < nr * chunks; task += nwarps) {
        const int r = task / chunks, v = (task - r * chunks) * 32 + lane;
        if (v >= nvec) continue;
        V acc = reinterpret_cast<const V *>(yb + r * ld)[v];
        const int nn = nb_n[r], nl = min(nn, kMaxNb);
        // neighbour rows in groups of loads in flight
        int e = 0;
        for (; e + 8 <= nl; e += 8) down_group<T, 8, COH>(&nb[r][e], ub, v, acc);
        if (e + 4 <= nl) {
            down_group<T, 4, COH>(&nb[r][e], ub, v, acc);
            e += 4;
        }
        for (; e < nl; ++e) down_group<T, 1, COH>(&nb[r][e], ub, v, acc);
        for (int e = kMaxNb; e < nn; ++e) {
            const T cf = __ldg(dcf + nb_e0[r] + e);
            const V xn = ld_data<COH>(reinterpret_cast<const V *>(ub + (int64_t)__ldg(a.dsrc + nb_e0[r] + e) * ld) + v);
#pragma unroll
            for (int k = 0; k < VN; ++k) vat(acc, k) += cf * reinterpret_cast<const T *>(&xn)[k];
        }
        const V xo = ld_data<COH>(reinterpret_cast<const V *>(ub + (int64_t)(r0 + r) * ld) + v);
#pragma unroll
        for (int k = 0; k < VN; ++k) {
            T val = vat(acc, k) * sc;
            if (v * VN + k >= nsup) val = (T)0;   // the row padding stays zero
            vat(acc, k) = val;
            dotp += reinterpret_cast<const T *>(&xo)[k] * val;
        }
        reinterpret_cast<V *>(yb + r * ld)[v] = acc;
    }
    block_partial((double)dotp, part_out + b);
}

template <typename T, int R>
__global__ void __launch_bounds__(kBatchThreads) batch_hv_kernel(const BatchInst *__restrict__ inst,
                                                                 const int32_t *__restrict__ blk_inst,
                                                                 const T *__restrict__ u, T *__restrict__ y,
                                                                 const double *__restrict__ scal,
                                                                 double *__restrict__ part_out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int64_t b = blockIdx.x;
    const int i = __ldg(blk_inst + b);
    hv_item<T, R, false>(inst, b, i, u, y, scal[(int64_t)i * kScal + kS], part_out, smem_raw);
}

// u_next = y - c_cur u_k - c_prev u_prev, written to un (which is u_prev
// itself when only two Krylov vectors are kept, a new basis slot otherwise),
// partial ||u_next||^2, in 16-byte vectors over the CTA's rows (padding is
// zero in all three inputs, so it stays zero).  With ritz_coef, also
// out += ritz_coef[i][k] s_k u_k (the Ritz vector sum_k y_k q_k of a replay).
template <typename T, bool COH>
__device__ __forceinline__ void update_item(const BatchInst &a, int64_t b, T cc, T cp, T cr,
                                            const T *__restrict__ y, const T *__restrict__ u, const T *up, T *un,
                                            double *__restrict__ part_nrm, T *__restrict__ ritz_out)
{
    using V = typename V16<T>::type;
    constexpr int VN = V16<T>::n;
    const int64_t r0 = (b - a.blk0) * a.rows;
    const int nr = (int)min((int64_t)a.rows, a.nsdn - r0);
    const int64_t base = a.off + r0 * a.ld;
    const int nv = nr * (int)(a.ld / VN);
    const V *yv = reinterpret_cast<const V *>(y + base);
    const V *uv = reinterpret_cast<const V *>(u + base);
    const V *pv = reinterpret_cast<const V *>(up + base);
    V *nv_out = reinterpret_cast<V *>(un + base);
    V *ov = ritz_out ? reinterpret_cast<V *>(ritz_out + base) : nullptr;
    T sp = 0;
    for (int q = threadIdx.x; q < nv; q += blockDim.x) {
        const V yy = ld_data<COH>(yv + q), uk = ld_data<COH>(uv + q);
        V pp;
        if constexpr (COH) pp = __ldca(pv + q);
        else pp = pv[q];
        V nv_;
#pragma unroll
        for (int e = 0; e < VN; ++e) {
            const T t = reinterpret_cast<const T *>(&yy)[e] - cc * reinterpret_cast<const T *>(&uk)[e] -
                        cp * reinterpret_cast<const T *>(&pp)[e];
            vat(nv_, e) = t;
            sp += t * t;
        }
        nv_out[q] = nv_;
        if (ov) {
            V o = ov[q];
#pragma unroll
            for (int e = 0; e < VN; ++e) vat(o, e) += cr * reinterpret_cast<const T *>(&uk)[e];
            ov[q] = o;
        }
    }
    block_partial((double)sp, part_nrm + b);
}

template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_update_kernel(const BatchInst *__restrict__ inst,
                                                                     const int32_t *__restrict__ blk_inst,
                                                                     const T *__restrict__ y, const T *__restrict__ u,
                                                                     const T *up, T *un, const double *__restrict__ scal,
                                                                     double *__restrict__ part_nrm,
                                                                     const double *__restrict__ ritz_coef,
                                                                     T *__restrict__ ritz_out, int k, int nsteps)
{
    const int64_t b = blockIdx.x;
    const int i = __ldg(blk_inst + b);
    const BatchInst &a = inst[i];
    const double *sc = scal + (int64_t)i * kScal;
    const T cc = (T)sc[kCCur], cp = (T)sc[kCPrev];
    const T cr = ritz_coef ? (T)(ritz_coef[(int64_t)i * nsteps + k] * sc[kS]) : (T)0;
    update_item<T, false>(a, b, cc, cp, cr, y, u, up, un, part_nrm, ritz_out);
}

// ---------------------------------------------------------------- persistent run
//
// One cooperative launch runs every step of every instance.  The work is a
// list of items (phase, CTA-block of an instance); per instance the phases
// are 0 (copy of x0 and its norm), then for step k: 2k+1 (H*v) and 2k+2
// (update).  The instances are split into two groups whose phases are offset
// by one, and the items of a "super-phase" interleave the two groups' blocks,
// so the H*v of one group (bound by the L1/shared-memory pipe) runs beside
// the update of the other (bound by HBM).  An item waits until its instance has finished the previous phase
// (done[i] >= p; every such item comes earlier in the list, so with all CTAs
// resident the run cannot deadlock); its CTA then arrives on the instance's
// counter, and the last CTA to arrive forms the instance's scalars exactly as
// batch_scalar_kernel does (same partials, same summation order: alpha/beta
// are bit-identical to the four-launch form) and publishes done[i] = p + 1.
// Every wait gives up after wait_ns of GPU time: it sets status[0] and the
// whole grid returns.  CTAs claim items from a queue in list order, so a CTA
// waits only on items already claimed by running CTAs.
struct PersistArgs {
    const BatchInst *inst;
    const int32_t *blk_inst;
    const int32_t *order;     // [nblocks]: the blocks of a super-phase, the two groups interleaved
    const int8_t *grp;        // [ninst]: 0 or 1 (phase offset)
    int ninst;
    int64_t nblocks;
    int nsteps;
    int64_t total;            // elements of one concatenated vector (the kept basis's slot stride)
    int *cnt;                 // [ninst] arrivals
    int *done;                // [ninst] phases completed
    int *status;              // [1] 0 = ok
    unsigned long long *queue;   // next unclaimed item
    double *scal, *pa, *pb, *alpha, *beta;
    unsigned long long wait_ns;  // limit of every wait (default 10 s: far above any phase of one instance)
    int stall_inst;              // watchdog test: this instance never completes phase 1 (-1: none)
};

constexpr int kPersistChunk = 4;   // items claimed at once

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits for done[i] >= p (bounded); the CTA learns the outcome.
__device__ __forceinline__ bool wait_phase(const PersistArgs &P, int i, int p, int *flag)
{
    if (threadIdx.x == 0) {
        int ok = 1;
        if (ld_acquire(P.done + i) < p) {
            const unsigned long long t0 = gtimer();
            unsigned ns = 32;
            while (ld_acquire(P.done + i) < p) {
                if (ld_acquire(P.status) != 0) { ok = 0; break; }
                if (gtimer() - t0 > P.wait_ns) {
                    atomicCAS(P.status, 0, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(ns);
                if (ns < 1024) ns *= 2;
            }
        }
        *flag = ok;
    }
    __syncthreads();
    const bool ok = *flag != 0;
    __syncthreads();
    return ok;
}

// After the CTA's partials are written: count its n arrivals (consecutive
// items of one instance and phase); the last CTA of the instance forms the scalars of phase p (mode 0 after a norm or update
// phase, 1 after an H*v phase) and publishes done[i] = p + 1.
__device__ __forceinline__ void arrive(const PersistArgs &P, const BatchInst &a, int i, int p, int n, int *flag)
{
    __syncthreads();   // the partials (thread 0) and all data stores of the CTA are issued
    if (threadIdx.x == 0) {
        int last = 0;
        if (i != P.stall_inst || p != 1) {   // the watchdog test leaves one counter short: its waiters give up
            __threadfence();
            const int old = atomicAdd(P.cnt + i, n);
            last = (old + n == (p + 1) * a.nblk) ? 1 : 0;
            if (last) __threadfence();
        }
        *flag = last;
    }
    __syncthreads();
    if (*flag && threadIdx.x < 32) {
        const bool upd = (p % 2) == 0;
        const double *part = upd ? P.pb : P.pa;
        double s = 0.0;
        for (int q = threadIdx.x; q < a.nblk; q += 32) s += __ldcg(part + a.blk0 + q);
        s = warp_sum(s);
        if (threadIdx.x == 0) {
            double *sc = P.scal + (int64_t)i * kScal;
            const int nsteps = P.nsteps;
            if (upd) {
                const int k = p / 2;
                const double bk = sqrt(fmax(s, 0.0));
                sc[kSPrev] = (k == 0) ? 0.0 : __ldcg(sc + kS);
                sc[kS] = (bk > 1e-150) ? 1.0 / bk : 0.0;
                sc[kBeta] = bk;
                P.beta[(int64_t)i * (nsteps + 1) + k] = bk;
            } else {
                const int k = (p - 1) / 2;
                const double sk = __ldcg(sc + kS);
                const double al = sk * s;
                P.alpha[(int64_t)i * nsteps + k] = al;
                sc[kCCur] = al * sk;
                sc[kCPrev] = __ldcg(sc + kBeta) * __ldcg(sc + kSPrev);
            }
            __threadfence();
            st_release(P.done + i, p + 1);
        }
    }
    __syncthreads();
}

template <typename T, int R>
__global__ void __launch_bounds__(kBatchThreads, 4) batch_persistent_kernel(const PersistArgs P, const T *__restrict__ x0,
                                                                         T *U0, T *U1, T *Y, T *kept)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int flag;
    __shared__ long long s_base;
    const int64_t tot_items = (int64_t)(2 * P.nsteps + 2) * P.nblocks;
    // items are claimed from a queue, kPersistChunk at a time, in list order: a CTA that drew
    // cheap update items takes more of them instead of waiting behind the H*v items
    for (;;) {
        if (threadIdx.x == 0) {
            flag = ld_acquire(P.status);
            s_base = (long long)atomicAdd(P.queue, (unsigned long long)kPersistChunk);
        }
        __syncthreads();
        const int64_t base = s_base;
        if (flag != 0 || base >= tot_items) return;   // every thread of the CTA saw the same values
        __syncthreads();
        const int64_t id_end = min(base + (int64_t)kPersistChunk, tot_items);
    // consecutive items of one instance and phase are counted with one arrival
    int run_i = -1, run_p = -1, run_n = 0;
    for (int64_t id = base; id < id_end; ++id) {
        const int64_t s = id / P.nblocks;
        const int64_t b = __ldg(P.order + (id - s * P.nblocks));
        const int i = __ldg(P.blk_inst + b);
        const int p = (int)s - (int)__ldg(P.grp + i);
        if (p < 0 || p > 2 * P.nsteps) continue;
        const BatchInst &a = P.inst[i];
        if (run_n > 0 && (i != run_i || p != run_p)) {
            arrive(P, P.inst[run_i], run_i, run_p, run_n, &flag);
            run_n = 0;
        }
        if (p == 0) {
            // u_0 = x0 on the block's rows (and u_{-1} = 0 without a kept basis), partial ||x0||^2
            const int64_t r0 = (b - a.blk0) * a.rows;
            const int nr = (int)min((int64_t)a.rows, a.nsdn - r0);
            const int64_t base_e = a.off + r0 * a.ld, n = (int64_t)nr * a.ld;
            T *u0 = kept ? kept : U0;
            for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
                u0[base_e + q] = x0[base_e + q];
                if (!kept) U1[base_e + q] = (T)0;
            }
            double sn = 0.0;
            for (int r = 0; r < nr; ++r) {
                const T *row = x0 + a.off + (r0 + r) * a.ld;
                for (int64_t c = threadIdx.x; c < a.nsup; c += blockDim.x) sn += (double)row[c] * (double)row[c];
            }
            block_partial(sn, P.pb + b);
        } else {
            if (run_n == 0 && !wait_phase(P, i, p, &flag)) return;
            // with a kept basis u_k is slot k (slot k-1 its predecessor, slot k+1 the next);
            // else u_k lives in U[k % 2] and u_{k+1} overwrites u_{k-1}
            const int k = (p - 1) / 2;
            const T *uk = kept ? kept + (int64_t)k * P.total : ((k & 1) ? U1 : U0);
            if (p % 2 == 1) {
                hv_item<T, R, true>(P.inst, b, i, uk, Y, __ldcg(P.scal + (int64_t)i * kScal + kS), P.pa,
                                    smem_raw);
            } else {
                const T *uprev = kept ? kept + (int64_t)(k > 0 ? k - 1 : 0) * P.total : ((k & 1) ? U0 : U1);
                T *unext = kept ? kept + (int64_t)(k + 1) * P.total : ((k & 1) ? U0 : U1);
                const double *sc = P.scal + (int64_t)i * kScal;
                update_item<T, true>(a, b, (T)__ldcg(sc + kCCur), (T)__ldcg(sc + kCPrev), (T)0, Y, uk, uprev,
                                     unext, P.pb, nullptr);
            }
        }
        run_i = i;
        run_p = p;
        ++run_n;
    }
    if (run_n > 0) arrive(P, P.inst[run_i], run_i, run_p, run_n, &flag);
    }
}

// Ritz vectors from a kept basis: out_i = sum_k coef[i][k] s_k u_k over the
// CTA's rows, s_k = 1 / beta[i][k] (0 after a vanished beta), u_k the basis
// slot k (k*total elements in).  The per-step factors of the instance are
// staged in shared memory; each thread sums its 16-byte vectors over k.
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_ritz_sum_kernel(const BatchInst *__restrict__ inst,
                                                                       const int32_t *__restrict__ blk_inst,
                                                                       const T *__restrict__ basis, int64_t total,
                                                                       int nsteps, const double *__restrict__ coef,
                                                                       const double *__restrict__ beta,
                                                                       T *__restrict__ out)
{
    using V = typename V16<T>::type;
    constexpr int VN = V16<T>::n;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *cs = reinterpret_cast<T *>(smem_raw);   // [nsteps]
    const int64_t b = blockIdx.x;
    const int i = __ldg(blk_inst + b);
    const BatchInst &a = inst[i];
    for (int k = threadIdx.x; k < nsteps; k += blockDim.x) {
        const double bk = beta[(int64_t)i * (nsteps + 1) + k];
        cs[k] = (T)((bk > 1e-150) ? coef[(int64_t)i * nsteps + k] / bk : 0.0);
    }
    __syncthreads();
    const int64_t r0 = (b - a.blk0) * a.rows;
    const int nr = (int)min((int64_t)a.rows, a.nsdn - r0);
    const int64_t base = a.off + r0 * a.ld;
    const int nv = nr * (int)(a.ld / VN);
    for (int q = threadIdx.x; q < nv; q += blockDim.x) {
        V acc;
#pragma unroll
        for (int e = 0; e < VN; ++e) vat(acc, e) = (T)0;
        const V *src = reinterpret_cast<const V *>(basis + base) + q;
        const int64_t step = total / VN;
        int k = 0;
        for (; k + 4 <= nsteps; k += 4) {
            V t[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) t[j] = __ldg(src + (int64_t)(k + j) * step);
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int e = 0; e < VN; ++e) vat(acc, e) += cs[k + j] * reinterpret_cast<const T *>(&t[j])[e];
        }
        for (; k < nsteps; ++k) {
            const V t = __ldg(src + (int64_t)k * step);
#pragma unroll
            for (int e = 0; e < VN; ++e) vat(acc, e) += cs[k] * reinterpret_cast<const T *>(&t)[e];
        }
        reinterpret_cast<V *>(out + base)[q] = acc;
    }
}

// work: two Krylov vectors and y (3*total), or, with kept != NULL, y alone
// (total) while u_k lives in slot k of kept ((nsteps+1)*total).
template <typename T, int R>
static int run_batch(ed_batch *bt, cudaStream_t st, T *work, const T *x0, int nsteps, double *alpha, double *beta,
                     double *scratch, const double *ritz_coef, T *ritz_out, T *kept = nullptr)
{
    const int64_t tot = bt->total;
    T *U[2] = {work, work + tot};
    T *Y = kept ? work : work + 2 * tot;
    double *pa = scratch, *pb = scratch + bt->nblocks, *scal = scratch + 2 * bt->nblocks;
    const size_t smem = (size_t)bt->max_ld * staged_stride<T, R>() * sizeof(T);
    const unsigned nb = (unsigned)bt->nblocks;
    const unsigned ns = (unsigned)((bt->ninst * 32 + 255) / 256);
    // two kept vectors: u_{k+1} overwrites u_{k-1} in place, so u_k lives in slot k % 2
    T *u0 = kept ? kept : U[0];
    ED_CHECK_CUDA(cudaMemcpyAsync(u0, x0, sizeof(T) * tot, cudaMemcpyDeviceToDevice, st));
    if (!kept) ED_CHECK_CUDA(cudaMemsetAsync(U[1], 0, sizeof(T) * tot, st));
    if (nb > 0) {
        batch_norm_kernel<T><<<nb, kBatchThreads, 0, st>>>(bt->dev, bt->blk_inst, u0, pb);
        ED_CHECK_LAUNCH();
    }
    batch_scalar_kernel<<<ns, 256, 0, st>>>(bt->dev, bt->ninst, pb, scal, alpha, beta, 0, nsteps, 0);
    ED_CHECK_LAUNCH();
    for (int k = 0; k < nsteps; ++k) {
        // with a kept basis, step 0's u_{-1} is u_0 itself (its coefficient is 0)
        T *uk = kept ? kept + (int64_t)k * tot : U[k % 2];
        T *uprev = kept ? kept + (int64_t)(k > 0 ? k - 1 : 0) * tot : U[(k + 1) % 2];
        T *unext = kept ? kept + (int64_t)(k + 1) * tot : uprev;
        if (nb > 0) {
            batch_hv_kernel<T, R><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, uk, Y, scal, pa);
            ED_CHECK_LAUNCH();
        }
        batch_scalar_kernel<<<ns, 256, 0, st>>>(bt->dev, bt->ninst, pa, scal, alpha, beta, k, nsteps, 1);
        ED_CHECK_LAUNCH();
        if (nb > 0) {
            batch_update_kernel<T><<<nb, kBatchThreads, 0, st>>>(bt->dev, bt->blk_inst, Y, uk, uprev, unext, scal,
                                                                 pb, ritz_coef, ritz_out, k, nsteps);
            ED_CHECK_LAUNCH();
        }
        batch_scalar_kernel<<<ns, 256, 0, st>>>(bt->dev, bt->ninst, pb, scal, alpha, beta, k + 1, nsteps, 0);
        ED_CHECK_LAUNCH();
    }
    return ED_OK;
}

}  // namespace ed

using namespace ed;

static int rows_index(int rows) { return rows == 4 ? 0 : (rows == 8 ? 1 : 2); }

static size_t hv_smem_bytes(int dtype, int64_t ld, int rows)
{
    static const int s32[3] = {staged_stride<float, 4>(), staged_stride<float, 8>(), staged_stride<float, 16>()};
    static const int s64[3] = {staged_stride<double, 4>(), staged_stride<double, 8>(), staged_stride<double, 16>()};
    const int k = rows_index(rows);
    return (dtype == ED_F32) ? (size_t)ld * s32[k] * sizeof(float) : (size_t)ld * s64[k] * sizeof(double);
}

template <typename T, int R>
static cudaError_t set_hv_smem(size_t bytes)
{
    return cudaFuncSetAttribute(batch_hv_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Dynamic shared memory of the H*v kernels: raised once to the largest need
// (at batch creation, so a later launch inside a stream capture only launches).
static std::mutex g_smem_mu;
static size_t g_smem_set[2][3] = {};

static int ensure_hv_smem(int dtype, int rows, size_t bytes)
{
    std::lock_guard<std::mutex> lk(g_smem_mu);
    const int k = (dtype == ED_F32) ? 0 : 1, r = rows_index(rows);
    if (bytes <= g_smem_set[k][r]) return ED_OK;
    cudaError_t e;
    if (dtype == ED_F32)
        e = (rows == 4) ? set_hv_smem<float, 4>(bytes) : (rows == 8) ? set_hv_smem<float, 8>(bytes)
                                                                     : set_hv_smem<float, 16>(bytes);
    else
        e = (rows == 4) ? set_hv_smem<double, 4>(bytes) : (rows == 8) ? set_hv_smem<double, 8>(bytes)
                                                                      : set_hv_smem<double, 16>(bytes);
    if (e != cudaSuccess) {
        set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return ED_ERR_CUDA;
    }
    g_smem_set[k][r] = bytes;
    return ED_OK;
}

extern "C" int ed_batch_create_rows(int ninst, ed_sector *const *secs, int rows, ed_batch **out)
{
    clear_error();
    ED_REQUIRE(out != nullptr, "out is NULL");
    *out = nullptr;
    ED_REQUIRE(ninst >= 1 && secs != nullptr, "need at least one instance");
    ED_REQUIRE(rows == 4 || rows == 8 || rows == 16, "rows per CTA must be 4, 8 or 16, got %d", rows);
    std::vector<BatchInst> host((size_t)ninst);
    std::vector<double> usite((size_t)ninst * kMaxSites);
    std::vector<float> usite32((size_t)ninst * kMaxSites);
    std::vector<int32_t> binst;
    std::vector<int64_t> offsets, dims;
    int64_t off = 0, blk = 0;
    int max_nsup = 0, max_ld = 0;
    for (int i = 0; i < ninst; ++i) {
        const ed_sector *s = secs[i];
        ED_REQUIRE(s != nullptr && s->kind == ED_HUBBARD, "instance %d is not a Hubbard sector", i);
        const int64_t ld = (s->nsup + 31) / 32 * 32;   // the internal row stride of pyhub_gb300 vectors
        if (hv_smem_bytes(ED_F64, ld, rows) > 200 * 1024) {
            set_error("instance %d: rows of %lld strings are too long for the batched kernel", i, (long long)s->nsup);
            return ED_ERR_RANGE;
        }
        BatchInst &a = host[(size_t)i];
        a.nsup = s->nsup; a.nsdn = s->nsdn;
        a.ld = ld;
        a.off = off;
        a.ustr = s->up.str; a.dstr = s->dn.str;
        a.uptr = s->up.ptr; a.usrc = s->up.src; a.dptr = s->dn.ptr; a.dsrc = s->dn.src;
        a.ucf32 = s->up.cf32; a.dcf32 = s->dn.cf32; a.ucf64 = s->up.cf64; a.dcf64 = s->dn.cf64;
        a.uediag = s->up.ediag; a.dediag = s->dn.ediag;
        a.uediag32 = s->up.ediag32; a.dediag32 = s->dn.ediag32;
        a.ell_off = s->up.ell_off; a.ell_src = s->up.ell_src;
        a.ell_cf32 = s->up.ell_cf32; a.ell_cf64 = s->up.ell_cf64;
        a.ell_pk32 = s->up.ell_pk32;
        a.nslice = (int)s->up.nslice;
        for (int q = 0; q < kMaxSites; ++q) {
            usite[(size_t)i * kMaxSites + q] = s->u_site[q];
            usite32[(size_t)i * kMaxSites + q] = (float)s->u_site[q];
        }
        a.u_site = nullptr;   // set after the upload below
        a.u_value = s->u_value;
        a.u_value32 = (float)s->u_value;
        a.u_uniform = s->u_uniform ? 1 : 0;
        a.blk0 = blk;
        a.nblk = (int)((s->nsdn + rows - 1) / rows);
        a.rows = rows;
        for (int q = 0; q < a.nblk; ++q) binst.push_back(i);
        blk += a.nblk;
        offsets.push_back(off);
        dims.push_back(s->nsdn * ld);
        off += s->nsdn * ld;
        off = (off + 31) / 32 * 32;  // keep every instance 128-byte aligned
        max_nsup = std::max(max_nsup, (int)s->nsup);
        max_ld = std::max(max_ld, (int)ld);
    }
    ED_REQUIRE(blk < (int64_t)INT32_MAX, "batch of %lld CTAs is too large", (long long)blk);
    ed_batch *bt = new ed_batch();
    bt->ninst = ninst;
    bt->total = off;
    bt->nblocks = blk;
    bt->offsets = std::move(offsets);
    bt->dims = std::move(dims);
    bt->max_nsup = max_nsup;
    bt->max_ld = max_ld;
    // one allocation per table: creating a batch of thousands of instances costs a few copies
    // persistent run: instances alternate between two groups whose phases are one apart; the
    // blocks of a super-phase interleave the groups in proportion to their sizes
    std::vector<int8_t> grp((size_t)ninst);
    for (int i = 0; i < ninst; ++i) grp[(size_t)i] = (int8_t)(i & 1);
    std::vector<int32_t> order;
    {
        std::vector<int32_t> g0, g1;
        for (int64_t b = 0; b < blk; ++b) (grp[(size_t)binst[(size_t)b]] ? g1 : g0).push_back((int32_t)b);
        order.reserve((size_t)blk);
        size_t a0 = 0, a1 = 0;
        while (a0 < g0.size() || a1 < g1.size()) {
            // take a run of kPersistChunk blocks from the group that is behind its share (consecutive
            // blocks of one instance, whose arrivals a CTA then counts at once)
            const bool take0 = a1 >= g1.size() ||
                               (a0 < g0.size() && (double)a0 * (double)g1.size() <= (double)a1 * (double)g0.size());
            for (int r = 0; r < kPersistChunk; ++r) {
                if (take0 && a0 < g0.size()) order.push_back(g0[a0++]);
                else if (!take0 && a1 < g1.size()) order.push_back(g1[a1++]);
            }
        }
    }
    if (cudaMalloc(&bt->dev, sizeof(BatchInst) * ninst) != cudaSuccess ||
        cudaMalloc(&bt->grp, (size_t)ninst) != cudaSuccess ||
        (blk > 0 && cudaMalloc(&bt->order, sizeof(int32_t) * (size_t)blk) != cudaSuccess) ||
        cudaMalloc(&bt->u_site_all, sizeof(double) * usite.size()) != cudaSuccess ||
        cudaMalloc(&bt->u_site_all32, sizeof(float) * usite32.size()) != cudaSuccess ||
        (blk > 0 && cudaMalloc(&bt->blk_inst, sizeof(int32_t) * (size_t)blk) != cudaSuccess)) {
        cudaGetLastError();
        set_error("allocation of batch descriptors failed");
        ed_batch_destroy(bt);
        return ED_ERR_MEM;
    }
    bt->rows = rows;
    if (ensure_hv_smem(ED_F32, rows, hv_smem_bytes(ED_F32, max_ld, rows)) != ED_OK ||
        ensure_hv_smem(ED_F64, rows, hv_smem_bytes(ED_F64, max_ld, rows)) != ED_OK) {
        ed_batch_destroy(bt);
        return ED_ERR_CUDA;
    }
    for (int i = 0; i < ninst; ++i) {
        host[(size_t)i].u_site = bt->u_site_all + (size_t)i * kMaxSites;
        host[(size_t)i].u_site32 = bt->u_site_all32 + (size_t)i * kMaxSites;
    }
    if (cudaMemcpy(bt->dev, host.data(), sizeof(BatchInst) * ninst, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(bt->u_site_all, usite.data(), sizeof(double) * usite.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(bt->u_site_all32, usite32.data(), sizeof(float) * usite32.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        (blk > 0 && cudaMemcpy(bt->blk_inst, binst.data(), sizeof(int32_t) * (size_t)blk, cudaMemcpyHostToDevice) !=
                        cudaSuccess) ||
        cudaMemcpy(bt->grp, grp.data(), (size_t)ninst, cudaMemcpyHostToDevice) != cudaSuccess ||
        (blk > 0 && cudaMemcpy(bt->order, order.data(), sizeof(int32_t) * (size_t)blk, cudaMemcpyHostToDevice) !=
                        cudaSuccess)) {
        const cudaError_t e = cudaGetLastError();
        set_error("upload of batch descriptors failed: %s", cudaGetErrorString(e));
        ed_batch_destroy(bt);
        return ED_ERR_CUDA;
    }
    *out = bt;
    return ED_OK;
}

extern "C" int ed_batch_create(int ninst, ed_sector *const *secs, ed_batch **out)
{
    return ed_batch_create_rows(ninst, secs, kDefaultRows, out);
}

extern "C" int ed_batch_rows(const ed_batch *bt) { return bt ? bt->rows : -1; }

extern "C" int ed_batch_destroy(ed_batch *bt)
{
    if (!bt) return ED_OK;
    if (bt->dev) cudaFree(bt->dev);
    if (bt->blk_inst) cudaFree(bt->blk_inst);
    if (bt->u_site_all) cudaFree(bt->u_site_all);
    if (bt->u_site_all32) cudaFree(bt->u_site_all32);
    if (bt->order) cudaFree(bt->order);
    if (bt->grp) cudaFree(bt->grp);
    delete bt;
    return ED_OK;
}

extern "C" int ed_batch_layout(const ed_batch *bt, int64_t *total, int64_t *offsets, int64_t *lds, int64_t *nblocks)
{
    clear_error();
    ED_REQUIRE(bt != nullptr, "batch is NULL");
    if (total) *total = bt->total;
    if (nblocks) *nblocks = bt->nblocks;
    for (int i = 0; i < bt->ninst; ++i) {
        if (offsets) offsets[i] = bt->offsets[(size_t)i];
        if (lds) lds[i] = bt->dims[(size_t)i];
    }
    return ED_OK;
}

extern "C" int64_t ed_batch_scratch_bytes(const ed_batch *bt)
{
    if (!bt) return -1;
    // partials and per-instance scalars (FP64), then the persistent run's counters, phase
    // flags and status (int32)
    return (2 * bt->nblocks + (int64_t)kScal * bt->ninst) * (int64_t)sizeof(double) +
           (2 * (int64_t)bt->ninst + 4) * (int64_t)sizeof(int) + 512;
}

static int batch_launch(ed_batch *bt, void *stream, int dtype, void *work, const void *x0, int nsteps, double *alpha,
                        double *beta, const double *ritz_coef, void *ritz_out, void *scratch, int64_t scratch_bytes,
                        void *kept = nullptr)
{
    ED_REQUIRE(bt != nullptr && work != nullptr && x0 != nullptr && alpha != nullptr && beta != nullptr,
               "NULL argument");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(nsteps >= 1, "nsteps must be positive");
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_batch_scratch_bytes(bt), "scratch of %lld bytes is below %lld",
               (long long)scratch_bytes, (long long)ed_batch_scratch_bytes(bt));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rc = ensure_hv_smem(dtype, bt->rows, hv_smem_bytes(dtype, bt->max_ld, bt->rows));
    if (rc != ED_OK) return rc;
    double *sc = (double *)scratch;
    if (dtype == ED_F32) {
        float *w = (float *)work, *ro = (float *)ritz_out, *kp = (float *)kept;
        const float *x = (const float *)x0;
        if (bt->rows == 4) return run_batch<float, 4>(bt, st, w, x, nsteps, alpha, beta, sc, ritz_coef, ro, kp);
        if (bt->rows == 16) return run_batch<float, 16>(bt, st, w, x, nsteps, alpha, beta, sc, ritz_coef, ro, kp);
        return run_batch<float, 8>(bt, st, w, x, nsteps, alpha, beta, sc, ritz_coef, ro, kp);
    }
    double *w = (double *)work, *ro = (double *)ritz_out, *kp = (double *)kept;
    const double *x = (const double *)x0;
    if (bt->rows == 4) return run_batch<double, 4>(bt, st, w, x, nsteps, alpha, beta, sc, ritz_coef, ro, kp);
    if (bt->rows == 16) return run_batch<double, 16>(bt, st, w, x, nsteps, alpha, beta, sc, ritz_coef, ro, kp);
    return run_batch<double, 8>(bt, st, w, x, nsteps, alpha, beta, sc, ritz_coef, ro, kp);
}

extern "C" int ed_batch_lanczos_kept(ed_batch *bt, void *stream, int dtype, void *basis, void *y, const void *x0,
                                     int nsteps, double *alpha, double *beta, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(basis != nullptr && y != nullptr, "NULL argument");
    return batch_launch(bt, stream, dtype, y, x0, nsteps, alpha, beta, nullptr, nullptr, scratch, scratch_bytes,
                        basis);
}

extern "C" int ed_batch_ritz_sum(ed_batch *bt, void *stream, int dtype, const void *basis, int nsteps,
                                 const double *coef, const double *beta, void *out)
{
    clear_error();
    ED_REQUIRE(bt != nullptr && basis != nullptr && coef != nullptr && beta != nullptr && out != nullptr,
               "NULL argument");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(nsteps >= 1 && nsteps <= 4096, "nsteps=%d outside 1..4096", nsteps);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned nb = (unsigned)bt->nblocks;
    if (nb == 0) return ED_OK;
    const size_t smem = (size_t)nsteps * (dtype == ED_F32 ? sizeof(float) : sizeof(double));
    if (dtype == ED_F32)
        batch_ritz_sum_kernel<float><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst,
                                                                       static_cast<const float *>(basis), bt->total,
                                                                       nsteps, coef, beta, static_cast<float *>(out));
    else
        batch_ritz_sum_kernel<double><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst,
                                                                        static_cast<const double *>(basis), bt->total,
                                                                        nsteps, coef, beta, static_cast<double *>(out));
    ED_CHECK_LAUNCH();
    return ED_OK;
}

namespace ed {
// s_k = 1 for every instance: the H*v kernel's scale when it runs alone.
__global__ void batch_unit_scale_kernel(int ninst, double *__restrict__ scal)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ninst) scal[(int64_t)i * kScal + kS] = 1.0;
}
}  // namespace ed

extern "C" int ed_batch_hv(ed_batch *bt, void *stream, int dtype, const void *x, void *y, void *scratch,
                           int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(bt != nullptr && x != nullptr && y != nullptr, "NULL argument");
    ED_REQUIRE(x != y, "x and y must not alias");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_batch_scratch_bytes(bt), "scratch of %lld bytes is below %lld",
               (long long)scratch_bytes, (long long)ed_batch_scratch_bytes(bt));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rc = ensure_hv_smem(dtype, bt->rows, hv_smem_bytes(dtype, bt->max_ld, bt->rows));
    if (rc != ED_OK) return rc;
    const unsigned nb = (unsigned)bt->nblocks;
    if (nb == 0) return ED_OK;
    double *pa = static_cast<double *>(scratch), *scal = pa + 2 * bt->nblocks;
    batch_unit_scale_kernel<<<(bt->ninst + 255) / 256, 256, 0, st>>>(bt->ninst, scal);
    ED_CHECK_LAUNCH();
    const size_t smem = hv_smem_bytes(dtype, bt->max_ld, bt->rows);
    if (dtype == ED_F32) {
        const float *xx = static_cast<const float *>(x);
        float *yy = static_cast<float *>(y);
        if (bt->rows == 4) batch_hv_kernel<float, 4><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, xx, yy, scal, pa);
        else if (bt->rows == 16) batch_hv_kernel<float, 16><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, xx, yy, scal, pa);
        else batch_hv_kernel<float, 8><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, xx, yy, scal, pa);
    } else {
        const double *xx = static_cast<const double *>(x);
        double *yy = static_cast<double *>(y);
        if (bt->rows == 4) batch_hv_kernel<double, 4><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, xx, yy, scal, pa);
        else if (bt->rows == 16) batch_hv_kernel<double, 16><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, xx, yy, scal, pa);
        else batch_hv_kernel<double, 8><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_inst, xx, yy, scal, pa);
    }
    ED_CHECK_LAUNCH();
    return ED_OK;
}

namespace ed {
// Where the persistent run keeps its counters in the caller's scratch: after
// the FP64 partials and scalars, 16-byte aligned.
static int *persist_ints(const ed_batch *bt, void *scratch)
{
    const size_t off = (size_t)(2 * bt->nblocks + (int64_t)kScal * bt->ninst) * sizeof(double);
    return reinterpret_cast<int *>(static_cast<unsigned char *>(scratch) + (off + 15) / 16 * 16);
}

template <typename T, int R>
static int run_persistent(ed_batch *bt, cudaStream_t st, T *work, const T *x0, int nsteps, double *alpha,
                          double *beta, double *scratch, T *kept)
{
    const int64_t tot = bt->total;
    PersistArgs P;
    P.inst = bt->dev;
    P.blk_inst = bt->blk_inst;
    P.order = bt->order;
    P.grp = bt->grp;
    P.ninst = bt->ninst;
    P.nblocks = bt->nblocks;
    P.nsteps = nsteps;
    P.total = tot;
    P.pa = scratch;
    P.pb = scratch + bt->nblocks;
    P.scal = scratch + 2 * bt->nblocks;
    int *ints = persist_ints(bt, scratch);
    P.cnt = ints;
    P.done = ints + bt->ninst;
    P.status = ints + 2 * bt->ninst;
    P.queue = reinterpret_cast<unsigned long long *>(ints + 2 * bt->ninst + 2);   // 8-byte aligned
    P.alpha = alpha;
    P.beta = beta;
    P.wait_ns = (unsigned long long)(bt->wait_s * 1e9);
    P.stall_inst = bt->stall_inst;
    ED_CHECK_CUDA(cudaMemsetAsync(ints, 0, sizeof(int) * (2 * (size_t)bt->ninst + 4), st));
    if (bt->nblocks == 0) return ED_OK;
    const size_t smem = (size_t)bt->max_ld * staged_stride<T, R>() * sizeof(T);
    auto kfn = batch_persistent_kernel<T, R>;
    ED_CHECK_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ED_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kBatchThreads, smem));
    if (per_sm < 1) {
        set_error("the persistent batched kernel does not fit on an SM");
        return ED_ERR_RANGE;
    }
    int64_t grid = (int64_t)per_sm * num_sms();
    const int64_t items = (int64_t)(2 * nsteps + 2) * bt->nblocks;
    if (grid > items) grid = items;
    T *U0 = kept ? nullptr : work, *U1 = kept ? nullptr : work + tot;
    T *Y = kept ? work : work + 2 * tot;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;   // every CTA resident at once: the waits rely on it
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    ED_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kfn, P, x0, U0, U1, Y, kept));
    return ED_OK;
}
}  // namespace ed

extern "C" int ed_batch_lanczos_persistent(ed_batch *bt, void *stream, int dtype, void *work, const void *x0,
                                           int nsteps, double *alpha, double *beta, void *kept, void *scratch,
                                           int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(bt != nullptr && work != nullptr && x0 != nullptr && alpha != nullptr && beta != nullptr,
               "NULL argument");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(nsteps >= 1, "nsteps must be positive");
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_batch_scratch_bytes(bt), "scratch of %lld bytes is below %lld",
               (long long)scratch_bytes, (long long)ed_batch_scratch_bytes(bt));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *sc = static_cast<double *>(scratch);
    if (dtype == ED_F32) {
        float *w = (float *)work, *kp = (float *)kept;
        const float *x = (const float *)x0;
        if (bt->rows == 4) return run_persistent<float, 4>(bt, st, w, x, nsteps, alpha, beta, sc, kp);
        if (bt->rows == 16) return run_persistent<float, 16>(bt, st, w, x, nsteps, alpha, beta, sc, kp);
        return run_persistent<float, 8>(bt, st, w, x, nsteps, alpha, beta, sc, kp);
    }
    double *w = (double *)work, *kp = (double *)kept;
    const double *x = (const double *)x0;
    if (bt->rows == 4) return run_persistent<double, 4>(bt, st, w, x, nsteps, alpha, beta, sc, kp);
    if (bt->rows == 16) return run_persistent<double, 16>(bt, st, w, x, nsteps, alpha, beta, sc, kp);
    return run_persistent<double, 8>(bt, st, w, x, nsteps, alpha, beta, sc, kp);
}

extern "C" int ed_batch_persistent_watchdog(ed_batch *bt, double wait_seconds, int stall_instance)
{
    clear_error();
    ED_REQUIRE(bt != nullptr, "batch is NULL");
    ED_REQUIRE(wait_seconds > 0.0 && wait_seconds <= 60.0, "wait_seconds=%g outside (0, 60]", wait_seconds);
    ED_REQUIRE(stall_instance >= -1 && stall_instance < bt->ninst, "stall_instance=%d outside -1..%d", stall_instance,
               bt->ninst - 1);
    bt->wait_s = wait_seconds;
    bt->stall_inst = stall_instance;
    return ED_OK;
}

extern "C" int ed_batch_persistent_status(const ed_batch *bt, const void *scratch, int *status)
{
    clear_error();
    ED_REQUIRE(bt != nullptr && scratch != nullptr && status != nullptr, "NULL argument");
    const int *ints = persist_ints(bt, const_cast<void *>(scratch));
    ED_CHECK_CUDA(cudaMemcpy(status, ints + 2 * bt->ninst, sizeof(int), cudaMemcpyDeviceToHost));
    return ED_OK;
}

extern "C" int ed_batch_lanczos(ed_batch *bt, void *stream, int dtype, void *work, const void *x0, int nsteps,
                                double *alpha, double *beta, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    return batch_launch(bt, stream, dtype, work, x0, nsteps, alpha, beta, nullptr, nullptr, scratch, scratch_bytes);
}

extern "C" int ed_batch_ritz(ed_batch *bt, void *stream, int dtype, void *work, const void *x0, int nsteps,
                             double *alpha, double *beta, const double *coef, void *out, void *scratch,
                             int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(coef != nullptr && out != nullptr, "NULL argument");
    return batch_launch(bt, stream, dtype, work, x0, nsteps, alpha, beta, coef, out, scratch, scratch_bytes);
}
