// ed_vec.cu -- Krylov-space vector kernels: many dot products in one pass
// over the basis, and the projection update w - V c with its norm.
//
// These carry the Lanczos scalars of lanczos.f90:53-58 (DOT_PRODUCT, the
// three-term update, NORM2) and the full reorthogonalisation that the
// reference lacks (its LANCZOS_NORM, lanczos.f90:137-161, only measures the
// loss).  FP32 vectors: products are formed and summed in FP32 over 16
// elements per thread, every such partial is promoted to FP64 and all further
// accumulation is FP64, so no FP64 multiply is spent per element.  FP64
// vectors: FP64 throughout.  (The FP32 multi-dot reduces each warp's 512
// products in FP32 before the FP64 stage; see multidot_kernel.)
#include "ed_common.cuh"

namespace ed {

int launch_reduce(const double *partials, int nblocks, int m, double *out, cudaStream_t st);

static constexpr int kVecThreads = 256;
static constexpr int kEPT = 16;                      // elements per thread per chunk
static constexpr int kChunk = kVecThreads * kEPT;    // 4096 elements
static constexpr int kMaxBlocks = 1024;

template <typename T>
__device__ __forceinline__ void load_chunk(T (&r)[kEPT], const T *__restrict__ p, int64_t base, int64_t n)
{
    // thread t owns elements base + t*4 + k*1024 + j (j<4), k < kEPT/4: float4 / double2x2 friendly
#pragma unroll
    for (int k = 0; k < kEPT / 4; ++k) {
        const int64_t i = base + (int64_t)k * (kVecThreads * 4) + threadIdx.x * 4;
        if (i + 3 < n) {
            if constexpr (sizeof(T) == 4) {
                const float4 v = __ldg(reinterpret_cast<const float4 *>(p + i));
                r[4 * k] = v.x; r[4 * k + 1] = v.y; r[4 * k + 2] = v.z; r[4 * k + 3] = v.w;
            } else {
                const double2 v0 = __ldg(reinterpret_cast<const double2 *>(p + i));
                const double2 v1 = __ldg(reinterpret_cast<const double2 *>(p + i + 2));
                r[4 * k] = v0.x; r[4 * k + 1] = v0.y; r[4 * k + 2] = v1.x; r[4 * k + 3] = v1.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) r[4 * k + j] = (i + j < n) ? __ldg(p + i + j) : (T)0;
        }
    }
}

// partials[block][j] (j < nvec) = sum over the block's chunks of <V_j, w>,
// partials[block][nvec + j] the same with z (when z != NULL).
// FP32 vectors: each warp forms its 512 products per chunk and reduces them in
// FP32 (shuffles); only that warp partial is promoted and added in FP64, so
// the FP64 work is one add per 512 elements and vector.  For random-sign
// data the FP32 stage contributes an absolute error ~eps32 |V_j||w|/sqrt(n).
template <typename T>
__global__ void __launch_bounds__(kVecThreads) multidot_kernel(int64_t n, const T *__restrict__ V, int64_t ldv,
                                                               int nvec, const T *__restrict__ w,
                                                               const T *__restrict__ z,
                                                               double *__restrict__ partials)
{
    extern __shared__ double acc[];  // [8 warps][m]
    const int m = z ? 2 * nvec : nvec;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j = threadIdx.x; j < 8 * m; j += blockDim.x) acc[j] = 0.0;
    __syncthreads();
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int64_t base = ch * kChunk;
        T rw[kEPT], rz[kEPT];
        load_chunk<T>(rw, w, base, n);
        if (z) load_chunk<T>(rz, z, base, n);
#pragma unroll 2
        for (int j = 0; j < nvec; ++j) {
            T rv[kEPT];
            load_chunk<T>(rv, V + (int64_t)j * ldv, base, n);
            T pw = 0, pz = 0;
#pragma unroll
            for (int k = 0; k < kEPT; ++k) pw += rv[k] * rw[k];
            if (z) {
#pragma unroll
                for (int k = 0; k < kEPT; ++k) pz += rv[k] * rz[k];
            }
            if constexpr (sizeof(T) == 4) {
                pw = warp_sumf(pw);
                if (z) pz = warp_sumf(pz);
                if (lane == 0) {
                    acc[warp * m + j] += (double)pw;
                    if (z) acc[warp * m + nvec + j] += (double)pz;
                }
            } else {
                const double sw = warp_sum((double)pw);
                const double sz = z ? warp_sum((double)pz) : 0.0;
                if (lane == 0) {
                    acc[warp * m + j] += sw;
                    if (z) acc[warp * m + nvec + j] += sz;
                }
            }
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < 8; ++q) s += acc[q * m + j];
        partials[(int64_t)blockIdx.x * m + j] = s;
    }
}

// out = ws w - sum_j coef_j V_j (w may be NULL; ws = wscale[0], a device
// scalar, or 1 when wscale is NULL), optional partial <out,out>.
// Accumulation type A: FP32 for an FP32 basis with FP32 output, FP64 otherwise.
template <typename T, typename O, typename A>
__global__ void __launch_bounds__(kVecThreads) update_kernel(int64_t n, const T *__restrict__ V, int64_t ldv,
                                                             int nvec, const double *__restrict__ coef,
                                                             const double *__restrict__ wscale, const O *w, O *out,
                                                             double *__restrict__ partials)
{
    extern __shared__ double cs_raw[];
    A *cs = reinterpret_cast<A *>(cs_raw);
    for (int j = threadIdx.x; j < nvec; j += blockDim.x) cs[j] = (A)coef[j];
    const A ws = wscale ? (A)wscale[0] : (A)1;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double nrm = 0.0;
    const int64_t nchunks = (n + kChunk - 1) / kChunk;
    for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int64_t base = ch * kChunk;
        A r[kEPT];
        if (w) {
            O rw[kEPT];
            load_chunk<O>(rw, w, base, n);
#pragma unroll
            for (int k = 0; k < kEPT; ++k) r[k] = ws * (A)rw[k];
        } else {
#pragma unroll
            for (int k = 0; k < kEPT; ++k) r[k] = (A)0;
        }
        for (int j = 0; j < nvec; ++j) {
            T rv[kEPT];
            load_chunk<T>(rv, V + (int64_t)j * ldv, base, n);
            const A c = cs[j];
#pragma unroll
            for (int k = 0; k < kEPT; ++k) r[k] -= c * (A)rv[k];
        }
        O ro[kEPT];
#pragma unroll
        for (int k = 0; k < kEPT; ++k) ro[k] = (O)r[k];
#pragma unroll
        for (int k = 0; k < kEPT / 4; ++k) {
            const int64_t i = base + (int64_t)k * (kVecThreads * 4) + threadIdx.x * 4;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (i + j < n) out[i + j] = ro[4 * k + j];
        }
        if (partials) {
            if constexpr (sizeof(O) == 4) {
                float p = 0.f;
#pragma unroll
                for (int k = 0; k < kEPT; ++k) p += ro[k] * ro[k];
                nrm += (double)p;
            } else {
#pragma unroll
                for (int k = 0; k < kEPT; ++k) nrm += (double)ro[k] * (double)ro[k];
            }
        }
    }
    if (partials) {
        __shared__ double red[8];
        nrm = warp_sum(nrm);
        if (lane == 0) red[warp] = nrm;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int q = 0; q < 8; ++q) s += red[q];
            partials[blockIdx.x] = s;
        }
    }
}

static int grid_for(int64_t n)
{
    int64_t nchunks = (n + kChunk - 1) / kChunk;
    int64_t cap = (int64_t)num_sms() * 4;
    if (cap > kMaxBlocks) cap = kMaxBlocks;
    if (nchunks < cap) cap = nchunks;
    return (int)(cap < 1 ? 1 : cap);
}

}  // namespace ed

using namespace ed;

extern "C" int ed_multidot(void *stream, int dtype, int64_t n, const void *V, int64_t ldv, int nvec, const void *w,
                           const void *z, double *out, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(n >= 0 && nvec >= 0, "negative size");
    ED_REQUIRE(out != nullptr, "out is NULL");
    if (nvec == 0 || n == 0) {
        if (nvec > 0) ED_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (z ? 2 : 1) * nvec, (cudaStream_t)stream));
        return ED_OK;
    }
    ED_REQUIRE(V != nullptr && w != nullptr, "V or w is NULL");
    ED_REQUIRE(ldv >= n, "ldv=%lld below n=%lld", (long long)ldv, (long long)n);
    const size_t esz = dtype == ED_F32 ? 4 : 8;
    ED_REQUIRE((reinterpret_cast<uintptr_t>(V) % 16) == 0 && (reinterpret_cast<uintptr_t>(w) % 16) == 0 &&
                   (!z || (reinterpret_cast<uintptr_t>(z) % 16) == 0) && ((ldv * esz) % 16) == 0,
               "V, w, z and the vector stride must be 16-byte aligned");
    ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_scratch_bytes(n, nvec),
               "scratch of %lld bytes is below the %lld needed", (long long)scratch_bytes,
               (long long)ed_scratch_bytes(n, nvec));
    const int m = z ? 2 * nvec : nvec;
    const size_t smem = sizeof(double) * 8 * (size_t)m;
    ED_REQUIRE(smem <= 200 * 1024, "nvec=%d too large for one pass", nvec);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int grid = grid_for(n);
    double *part = static_cast<double *>(scratch);
    if (dtype == ED_F32) {
        ED_CHECK_CUDA(cudaFuncSetAttribute(multidot_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        multidot_kernel<float><<<grid, kVecThreads, smem, st>>>(n, static_cast<const float *>(V), ldv, nvec,
                                                               static_cast<const float *>(w),
                                                               static_cast<const float *>(z), part);
    } else {
        ED_CHECK_CUDA(cudaFuncSetAttribute(multidot_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        multidot_kernel<double><<<grid, kVecThreads, smem, st>>>(n, static_cast<const double *>(V), ldv, nvec,
                                                                static_cast<const double *>(w),
                                                                static_cast<const double *>(z), part);
    }
    ED_CHECK_LAUNCH();
    return launch_reduce(part, grid, m, out, st);
}

extern "C" int ed_update_wscaled(void *stream, int dtype, int out_dtype, int64_t n, const void *V, int64_t ldv,
                                 int nvec, const double *coef, const double *wscale, const void *w, void *out,
                                 double *norm2, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(out_dtype == ED_F32 || out_dtype == ED_F64, "out_dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(n >= 0 && nvec >= 0, "negative size");
    ED_REQUIRE(out != nullptr, "out is NULL");
    ED_REQUIRE(nvec == 0 || (V != nullptr && coef != nullptr), "V or coef is NULL");
    ED_REQUIRE(nvec == 0 || ldv >= n, "ldv=%lld below n=%lld", (long long)ldv, (long long)n);
    const size_t esz = dtype == ED_F32 ? 4 : 8, osz = out_dtype == ED_F32 ? 4 : 8;
    ED_REQUIRE((nvec == 0 || ((reinterpret_cast<uintptr_t>(V) % 16) == 0 && ((ldv * esz) % 16) == 0)) &&
                   (reinterpret_cast<uintptr_t>(out) % 16) == 0 && (!w || (reinterpret_cast<uintptr_t>(w) % 16) == 0),
               "V, w, out and the vector stride must be 16-byte aligned");
    (void)osz;
    ED_REQUIRE(nvec <= 8192, "nvec=%d too large", nvec);
    if (norm2) {
        ED_REQUIRE(scratch != nullptr && scratch_bytes >= ed_scratch_bytes(n, 1),
                   "scratch of %lld bytes is below the %lld needed", (long long)scratch_bytes,
                   (long long)ed_scratch_bytes(n, 1));
    }
    if (n == 0) return ED_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int grid = grid_for(n);
    double *part = norm2 ? static_cast<double *>(scratch) : nullptr;
    const size_t smem = sizeof(double) * (size_t)(nvec > 0 ? nvec : 1);
    if (dtype == ED_F32 && out_dtype == ED_F32) {
        update_kernel<float, float, float><<<grid, kVecThreads, smem, st>>>(
            n, static_cast<const float *>(V), ldv, nvec, coef, wscale, static_cast<const float *>(w),
            static_cast<float *>(out), part);
    } else if (dtype == ED_F32 && out_dtype == ED_F64) {
        update_kernel<float, double, double><<<grid, kVecThreads, smem, st>>>(
            n, static_cast<const float *>(V), ldv, nvec, coef, wscale, static_cast<const double *>(w),
            static_cast<double *>(out), part);
    } else if (dtype == ED_F64 && out_dtype == ED_F64) {
        update_kernel<double, double, double><<<grid, kVecThreads, smem, st>>>(
            n, static_cast<const double *>(V), ldv, nvec, coef, wscale, static_cast<const double *>(w),
            static_cast<double *>(out), part);
    } else {
        update_kernel<double, float, double><<<grid, kVecThreads, smem, st>>>(
            n, static_cast<const double *>(V), ldv, nvec, coef, wscale, static_cast<const float *>(w),
            static_cast<float *>(out), part);
    }
    ED_CHECK_LAUNCH();
    if (norm2) return launch_reduce(part, grid, 1, norm2, st);
    return ED_OK;
}

extern "C" int ed_update(void *stream, int dtype, int out_dtype, int64_t n, const void *V, int64_t ldv, int nvec,
                         const double *coef, const void *w, void *out, double *norm2, void *scratch,
                         int64_t scratch_bytes)
{
    return ed_update_wscaled(stream, dtype, out_dtype, n, V, ldv, nvec, coef, nullptr, w, out, norm2, scratch,
                             scratch_bytes);
}

// ---------------------------------------------------------------------------
// ed_multidot_noalloc: the multi-dot for callers that cannot allocate device
// memory and so cannot hand ed_multidot a scratch buffer.  Its per-block
// partial sums live in a fixed file-scope device array instead.

#include <mutex>

namespace ed {

constexpr int kNoAllocMaxNvec = 64;
constexpr int64_t kNoAllocDoubles = (int64_t)kMaxBlocks * 2 * kNoAllocMaxNvec;  // 131072 doubles = 1 MiB

// Partial sums of ed_multidot_noalloc.  Every GPU on which this library's
// kernels are loaded holds these 1 MiB until the process exits.  All calls on
// a device share the array: calls that overlap on the GPU race.  The kernel
// writes every partial before the reduction reads it, so nothing is cleared
// between calls.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocDoubles];

constexpr int kNoAllocMaxDevices = 64;
static double *g_noalloc_addr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// Device address of g_noalloc_partials on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// with the device current.  Outside a stream capture it is looked up on every
// call (cheap), so a context that was torn down and rebuilt, where the module
// may have loaded at another address, never gets a stale pointer; inside a
// capture the address cached by an earlier call on this device is used, and a
// capture with no earlier call is refused.
static int noalloc_partials(cudaStream_t st, double **out)
{
    int dev = 0;
    ED_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("device %d is beyond the %d devices ed_multidot_noalloc tracks", dev, kNoAllocMaxDevices);
        return ED_ERR_RANGE;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ED_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (cs == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) {
            set_error("cudaGetSymbolAddress of the fixed scratch array failed: %s", cudaGetErrorString(e));
            return ED_ERR_CUDA;
        }
        g_noalloc_addr[dev] = static_cast<double *>(p);
    } else if (g_noalloc_addr[dev] == nullptr) {
        set_error("ed_multidot_noalloc: call it once on this device outside a stream capture first");
        return ED_ERR_ARG;
    }
    *out = g_noalloc_addr[dev];
    return ED_OK;
}

}  // namespace ed

extern "C" int ed_multidot_noalloc(void *stream, int dtype, int64_t n, const void *V, int64_t ldv, int nvec,
                                   const void *w, const void *z, double *out)
{
    clear_error();
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    ED_REQUIRE(n >= 0 && nvec >= 0, "negative size");
    ED_REQUIRE(out != nullptr, "out is NULL");
    if (nvec > kNoAllocMaxNvec) {
        set_error("nvec=%d exceeds the %d vectors of ed_multidot_noalloc (its scratch is a fixed %lld-byte "
                  "device array); use ed_multidot with a scratch buffer for more",
                  nvec, kNoAllocMaxNvec, (long long)(kNoAllocDoubles * (int64_t)sizeof(double)));
        return ED_ERR_RANGE;
    }
    if (nvec == 0 || n == 0) {
        if (nvec > 0) ED_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (z ? 2 : 1) * nvec, (cudaStream_t)stream));
        return ED_OK;
    }
    ED_REQUIRE(V != nullptr && w != nullptr, "V or w is NULL");
    ED_REQUIRE(ldv >= n, "ldv=%lld below n=%lld", (long long)ldv, (long long)n);
    const size_t esz = dtype == ED_F32 ? 4 : 8;
    ED_REQUIRE((reinterpret_cast<uintptr_t>(V) % 16) == 0 && (reinterpret_cast<uintptr_t>(w) % 16) == 0 &&
                   (!z || (reinterpret_cast<uintptr_t>(z) % 16) == 0) && ((ldv * esz) % 16) == 0,
               "V, w, z and the vector stride must be 16-byte aligned");
    const int m = z ? 2 * nvec : nvec;
    const int grid = grid_for(n);
    if ((int64_t)grid * m > kNoAllocDoubles) {
        set_error("%d blocks x %d sums exceed the fixed scratch of %lld doubles", grid, m, (long long)kNoAllocDoubles);
        return ED_ERR_RANGE;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *part = nullptr;
    const int rc = noalloc_partials(st, &part);
    if (rc) return rc;
    const size_t smem = sizeof(double) * 8 * (size_t)m;  // at most 8 KiB: no opt-in needed
    if (dtype == ED_F32)
        multidot_kernel<float><<<grid, kVecThreads, smem, st>>>(n, static_cast<const float *>(V), ldv, nvec,
                                                               static_cast<const float *>(w),
                                                               static_cast<const float *>(z), part);
    else
        multidot_kernel<double><<<grid, kVecThreads, smem, st>>>(n, static_cast<const double *>(V), ldv, nvec,
                                                                static_cast<const double *>(w),
                                                                static_cast<const double *>(z), part);
    ED_CHECK_LAUNCH();
    return launch_reduce(part, grid, m, out, st);
}
