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
// Sectors here are small (D ~ 1e5..1e6): each CTA stages kRows rows of u_k in
// shared memory for the up hops and reads the neighbour rows of the down
// hops straight from L2, where the instances in flight keep their vectors.
#include "ed_common.cuh"

#include <algorithm>
#include <vector>

namespace ed {

constexpr int kRows = 8;          // rows of one instance per CTA
constexpr int kBatchThreads = 256;

struct BatchInst {
    int64_t nsup, nsdn, ld, off;      // off: first element of this instance in the work arrays
    const uint32_t *ustr, *dstr;
    const int32_t *uptr, *usrc, *dptr, *dsrc;
    const float *ucf32, *dcf32;
    const double *ucf64, *dcf64;
    const double *uediag, *dediag;
    const double *u_site;             // device, indexed by bit
    const int32_t *ell_off, *ell_src; // sliced-ELL up-hop table of the sector
    const float *ell_cf32;
    const double *ell_cf64;
    int nslice;
    double u_value;
    int u_uniform;
    int64_t blk0;                     // first CTA of this instance
    int nblk;
};

}  // namespace ed

struct ed_batch {
    int ninst = 0;
    int64_t total = 0;                 // elements of one concatenated vector
    int64_t nblocks = 0;
    ed::BatchInst *dev = nullptr;      // [ninst]
    int64_t *blk_start = nullptr;      // [ninst+1] device
    double **u_site_bufs = nullptr;
    std::vector<int64_t> offsets, dims;
    std::vector<double *> u_site_dev;
    int max_nsup = 0;
    int max_ld = 0;
};

namespace ed {

__device__ __forceinline__ int find_inst(const int64_t *__restrict__ blk_start, int ninst, int64_t b)
{
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(blk_start + mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename T>
__device__ __forceinline__ double inst_reduce(const double *__restrict__ part, int64_t b0, int n)
{
    // every CTA of an instance sums its partials in the same order: identical values
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[b0 + i];
    return s;
}

template <typename T>
__device__ __forceinline__ T u_energy_b(const BatchInst &a, uint32_t both)
{
    if (a.u_uniform) return (T)a.u_value * (T)__popc(both);
    T e = 0;
    while (both) {
        const int b = __ffs(both) - 1;
        e += (T)a.u_site[b];
        both &= both - 1;
    }
    return e;
}

// Norms of the start vectors: partial ||x0||^2 per CTA.
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_norm_kernel(const BatchInst *__restrict__ inst,
                                                                   const int64_t *__restrict__ blk_start, int ninst,
                                                                   const T *__restrict__ x, double *__restrict__ part)
{
    const int64_t b = blockIdx.x;
    const int i = find_inst(blk_start, ninst, b);
    const BatchInst a = inst[i];
    const int64_t r0 = (b - a.blk0) * kRows;
    double s = 0.0;
    for (int r = 0; r < kRows; ++r) {
        const int64_t d = r0 + r;
        if (d >= a.nsdn) break;
        const T *row = x + a.off + d * a.ld;
        for (int64_t u = threadIdx.x; u < a.nsup; u += blockDim.x) s += (double)row[u] * (double)row[u];
    }
    __shared__ double red[kBatchThreads / 32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBatchThreads / 32; ++w) t += red[w];
        part[b] = t;
    }
}

// y = s_k H u_k and partial <u_k, y>; s_k from the partials of the previous
// update (or of the start-vector norms at k = 0).  kRows rows of u_k are
// staged in shared memory; each warp takes 32-string slices of a row: the up
// hops walk the sector's sliced-ELL slots (coalesced) and gather from the
// staged row, the down hops read the neighbour rows' slice from L2 with the
// row's neighbour list held one entry per lane.
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_hv_kernel(const BatchInst *__restrict__ inst,
                                                                 const int64_t *__restrict__ blk_start, int ninst,
                                                                 const T *__restrict__ u, T *__restrict__ y,
                                                                 const double *__restrict__ part_in,
                                                                 double *__restrict__ part_out,
                                                                 double *__restrict__ beta, int k, int nsteps)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);
    __shared__ double red[kBatchThreads / 32];
    __shared__ double s_k;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = kBatchThreads / 32;
    const int64_t b = blockIdx.x;
    const int i = find_inst(blk_start, ninst, b);
    const BatchInst a = inst[i];
    if (threadIdx.x == 0) {
        const double nb = inst_reduce<T>(part_in, a.blk0, a.nblk);
        const double bk = sqrt(fmax(nb, 0.0));
        s_k = (bk > 1e-150) ? 1.0 / bk : 0.0;
        if (b == a.blk0) beta[(int64_t)i * (nsteps + 1) + k] = bk;
    }
    const int64_t r0 = (b - a.blk0) * kRows;
    const int nr = (int)min((int64_t)kRows, a.nsdn - r0);
    const int64_t sld = a.ld;
    const T *ub = u + a.off;
    for (int r = 0; r < nr; ++r)
        for (int64_t c = threadIdx.x; c < a.nsup; c += blockDim.x) xs[r * sld + c] = ub[(r0 + r) * a.ld + c];
    __syncthreads();
    const T sc = (T)s_k;
    const T *ecf = (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.ell_cf32) : reinterpret_cast<const T *>(a.ell_cf64);
    const T *dcf = (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.dcf32) : reinterpret_cast<const T *>(a.dcf64);
    T dotp = 0;
    for (int r = 0; r < nr; ++r) {
        const int64_t d = r0 + r;
        const uint32_t sd = __ldg(a.dstr + d);
        const T ed = (T)__ldg(a.dediag + d);
        const int e0 = __ldg(a.dptr + d), nn = __ldg(a.dptr + d + 1) - e0;
        const int my_src = (lane < nn) ? __ldg(a.dsrc + e0 + lane) : 0;
        const T my_cf = (lane < nn) ? __ldg(dcf + e0 + lane) : (T)0;
        for (int sl = warp; sl < a.nslice; sl += nwarps) {
            const int64_t c = (int64_t)sl * 32 + lane;
            const bool ok = c < a.nsup;
            const int64_t cc = ok ? c : a.nsup - 1;
            const uint32_t su = __ldg(a.ustr + cc);
            const T xv = xs[r * sld + cc];
            T acc = ((T)__ldg(a.uediag + cc) + ed + u_energy_b<T>(a, su & sd)) * xv;
            const int s0 = __ldg(a.ell_off + sl), ns = __ldg(a.ell_off + sl + 1) - s0;
            const int32_t *sp = a.ell_src + (int64_t)s0 * 32 + lane;
            const T *cp = ecf + (int64_t)s0 * 32 + lane;
            for (int q = 0; q < ns; ++q) acc += __ldg(cp + q * 32) * xs[r * sld + __ldg(sp + q * 32)];
            // down hops: the row's neighbour list (<= 32 entries) is spread over the lanes
            for (int e = 0; e < min(nn, 32); ++e) {
                const int src = __shfl_sync(0xffffffffu, my_src, e);
                const T wgt = __shfl_sync(0xffffffffu, my_cf, e);
                acc += wgt * ub[(int64_t)src * a.ld + cc];
            }
            for (int e = 32; e < nn; ++e) acc += __ldg(dcf + e0 + e) * ub[(int64_t)__ldg(a.dsrc + e0 + e) * a.ld + cc];
            acc *= sc;
            if (ok) {
                y[a.off + d * a.ld + c] = acc;
                dotp += xv * acc;
            }
        }
    }
    double dot = warp_sum((double)dotp);
    if (lane == 0) red[warp] = dot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBatchThreads / 32; ++w) t += red[w];
        part_out[b] = t;
    }
}

// u_next = y - alpha_k s_k u_k - beta_k s_{k-1} u_prev (written over u_prev),
// partial ||u_next||^2; alpha_k = s_k sum <u_k,y> partials.
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_update_kernel(const BatchInst *__restrict__ inst,
                                                                     const int64_t *__restrict__ blk_start, int ninst,
                                                                     const T *__restrict__ y, const T *__restrict__ u,
                                                                     T *__restrict__ up,
                                                                     const double *__restrict__ part_dot,
                                                                     double *__restrict__ part_nrm,
                                                                     const double *__restrict__ beta,
                                                                     double *__restrict__ alpha, int k, int nsteps)
{
    __shared__ double red[kBatchThreads / 32];
    __shared__ double c_cur, c_prev;
    const int64_t b = blockIdx.x;
    const int i = find_inst(blk_start, ninst, b);
    const BatchInst a = inst[i];
    if (threadIdx.x == 0) {
        const double bk = beta[(int64_t)i * (nsteps + 1) + k];
        const double sk = (bk > 1e-150) ? 1.0 / bk : 0.0;
        const double al = sk * inst_reduce<T>(part_dot, a.blk0, a.nblk);
        if (b == a.blk0) alpha[(int64_t)i * nsteps + k] = al;
        c_cur = al * sk;
        if (k > 0) {
            const double bp = beta[(int64_t)i * (nsteps + 1) + k - 1];
            const double sp = (bp > 1e-150) ? 1.0 / bp : 0.0;
            c_prev = bk * sp;
        } else {
            c_prev = 0.0;
        }
    }
    __syncthreads();
    const T cc = (T)c_cur, cp = (T)c_prev;
    const int64_t r0 = (b - a.blk0) * kRows;
    const int nr = (int)min((int64_t)kRows, a.nsdn - r0);
    T sp = 0;
    for (int r = 0; r < nr; ++r) {
        const int64_t base = a.off + (r0 + r) * a.ld;
        for (int64_t c = threadIdx.x; c < a.nsup; c += blockDim.x) {
            const T v = y[base + c] - cc * u[base + c] - cp * up[base + c];
            up[base + c] = v;
            sp += v * v;
        }
    }
    double s = warp_sum((double)sp);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBatchThreads / 32; ++w) t += red[w];
        part_nrm[b] = t;
    }
}

// beta of the last step from the last update's partials.
__global__ void batch_last_beta_kernel(const ed::BatchInst *__restrict__ inst, int ninst,
                                       const double *__restrict__ part, double *__restrict__ beta, int nsteps)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ninst; i += gridDim.x * blockDim.x) {
        const BatchInst a = inst[i];
        double s = 0.0;
        for (int q = 0; q < a.nblk; ++q) s += part[a.blk0 + q];
        beta[(int64_t)i * (nsteps + 1) + nsteps] = sqrt(fmax(s, 0.0));
    }
}

template <typename T>
static int run_batch(ed_batch *bt, cudaStream_t st, T *work, const T *x0, int nsteps, double *alpha, double *beta,
                     double *scratch)
{
    const int64_t tot = bt->total;
    T *U[2] = {work, work + tot};
    T *Y = work + 2 * tot;
    double *pa = scratch, *pb = scratch + bt->nblocks;
    const size_t smem = (size_t)kRows * bt->max_ld * sizeof(T);
    const unsigned nb = (unsigned)bt->nblocks;
    // u_{k+1} overwrites u_{k-1} in place, so u_k lives in slot k % 2
    ED_CHECK_CUDA(cudaMemcpyAsync(U[0], x0, sizeof(T) * tot, cudaMemcpyDeviceToDevice, st));
    ED_CHECK_CUDA(cudaMemsetAsync(U[1], 0, sizeof(T) * tot, st));
    batch_norm_kernel<T><<<nb, kBatchThreads, 0, st>>>(bt->dev, bt->blk_start, bt->ninst, U[0], pb);
    ED_CHECK_LAUNCH();
    for (int k = 0; k < nsteps; ++k) {
        T *uk = U[k % 2], *uprev = U[(k + 1) % 2];
        batch_hv_kernel<T><<<nb, kBatchThreads, smem, st>>>(bt->dev, bt->blk_start, bt->ninst, uk, Y, pb, pa, beta,
                                                             k, nsteps);
        ED_CHECK_LAUNCH();
        batch_update_kernel<T><<<nb, kBatchThreads, 0, st>>>(bt->dev, bt->blk_start, bt->ninst, Y, uk, uprev, pa, pb,
                                                             beta, alpha, k, nsteps);
        ED_CHECK_LAUNCH();
    }
    batch_last_beta_kernel<<<(bt->ninst + 127) / 128, 128, 0, st>>>(bt->dev, bt->ninst, pb, beta, nsteps);
    ED_CHECK_LAUNCH();
    return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" int ed_batch_create(int ninst, ed_sector *const *secs, ed_batch **out)
{
    clear_error();
    ED_REQUIRE(out != nullptr, "out is NULL");
    *out = nullptr;
    ED_REQUIRE(ninst >= 1 && secs != nullptr, "need at least one instance");
    ed_batch *bt = new ed_batch();
    bt->ninst = ninst;
    std::vector<BatchInst> host((size_t)ninst);
    std::vector<int64_t> bstart((size_t)ninst + 1);
    int64_t off = 0, blk = 0;
    for (int i = 0; i < ninst; ++i) {
        const ed_sector *s = secs[i];
        if (!s || s->kind != ED_HUBBARD) {
            delete bt;
            set_error("instance %d is not a Hubbard sector", i);
            return ED_ERR_ARG;
        }
        if ((size_t)kRows * ((s->nsup + 31) / 32 * 32) * sizeof(double) > 200 * 1024) {
            delete bt;
            set_error("instance %d: rows of %lld strings are too long for the batched kernel", i, (long long)s->nsup);
            return ED_ERR_RANGE;
        }
        BatchInst &a = host[(size_t)i];
        a.nsup = s->nsup; a.nsdn = s->nsdn;
        a.ld = (s->nsup + 31) / 32 * 32;   // the internal row stride of pyhub_gb300 vectors
        a.off = off;
        a.ustr = s->up.str; a.dstr = s->dn.str;
        a.uptr = s->up.ptr; a.usrc = s->up.src; a.dptr = s->dn.ptr; a.dsrc = s->dn.src;
        a.ucf32 = s->up.cf32; a.dcf32 = s->dn.cf32; a.ucf64 = s->up.cf64; a.dcf64 = s->dn.cf64;
        a.uediag = s->up.ediag; a.dediag = s->dn.ediag;
        a.ell_off = s->up.ell_off; a.ell_src = s->up.ell_src;
        a.ell_cf32 = s->up.ell_cf32; a.ell_cf64 = s->up.ell_cf64;
        a.nslice = (int)s->up.nslice;
        double *us = nullptr;
        if (cudaMalloc(&us, sizeof(double) * kMaxSites) != cudaSuccess ||
            cudaMemcpy(us, s->u_site, sizeof(double) * kMaxSites, cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("allocation of batch parameters failed");
            ed_batch_destroy(bt);
            return ED_ERR_MEM;
        }
        bt->u_site_dev.push_back(us);
        a.u_site = us;
        a.u_value = s->u_value;
        a.u_uniform = s->u_uniform ? 1 : 0;
        a.blk0 = blk;
        a.nblk = (int)((s->nsdn + kRows - 1) / kRows);
        bstart[(size_t)i] = blk;
        blk += a.nblk;
        bt->offsets.push_back(off);
        bt->dims.push_back(s->nsdn * a.ld);
        off += s->nsdn * a.ld;
        off = (off + 31) / 32 * 32;  // keep every instance 128-byte aligned
        bt->max_nsup = std::max(bt->max_nsup, (int)s->nsup);
        bt->max_ld = std::max(bt->max_ld, (int)a.ld);
    }
    bstart[(size_t)ninst] = blk;
    bt->total = off;
    bt->nblocks = blk;
    if (cudaMalloc(&bt->dev, sizeof(BatchInst) * ninst) != cudaSuccess ||
        cudaMalloc(&bt->blk_start, sizeof(int64_t) * (ninst + 1)) != cudaSuccess) {
        set_error("allocation of batch descriptors failed");
        ed_batch_destroy(bt);
        return ED_ERR_MEM;
    }
    ED_CHECK_CUDA(cudaMemcpy(bt->dev, host.data(), sizeof(BatchInst) * ninst, cudaMemcpyHostToDevice));
    ED_CHECK_CUDA(cudaMemcpy(bt->blk_start, bstart.data(), sizeof(int64_t) * (ninst + 1), cudaMemcpyHostToDevice));
    *out = bt;
    return ED_OK;
}

extern "C" int ed_batch_destroy(ed_batch *bt)
{
    if (!bt) return ED_OK;
    for (double *p : bt->u_site_dev) cudaFree(p);
    if (bt->dev) cudaFree(bt->dev);
    if (bt->blk_start) cudaFree(bt->blk_start);
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
    return 2 * bt->nblocks * (int64_t)sizeof(double) + 256;
}

extern "C" int ed_batch_lanczos(ed_batch *bt, void *stream, int dtype, void *work, const void *x0, int nsteps,
                                double *alpha, double *beta, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(bt != nullptr && work != nullptr && x0 != nullptr && alpha != nullptr && beta != nullptr,
               "NULL argument");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(nsteps >= 1, "nsteps must be positive");
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_batch_scratch_bytes(bt), "scratch of %lld bytes is below %lld",
               (long long)scratch_bytes, (long long)ed_batch_scratch_bytes(bt));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == ED_F32) {
        const size_t smem = (size_t)kRows * bt->max_ld * sizeof(float);
        ED_CHECK_CUDA(cudaFuncSetAttribute(batch_hv_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return run_batch<float>(bt, st, (float *)work, (const float *)x0, nsteps, alpha, beta, (double *)scratch);
    }
    const size_t smem = (size_t)kRows * bt->max_ld * sizeof(double);
    ED_CHECK_CUDA(cudaFuncSetAttribute(batch_hv_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return run_batch<double>(bt, st, (double *)work, (const double *)x0, nsteps, alpha, beta, (double *)scratch);
}
