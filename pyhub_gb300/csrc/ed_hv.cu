// ed_hv.cu -- on-the-fly Hamiltonian-vector products.
//
// Hubbard (replaces HPROD, hprod_hubbard.f90:17-118).  With the vector viewed
// as a matrix X[d][u] (row = down string, contiguous up strings), H = A_up
// acting inside each row + A_dn mixing rows + a diagonal:
//   y[d][u] = diag(d,u) x[d][u] + sum_{q in up(u)} c x[d][q] + sum_{e in dn(d)} c x[e][u]
// Pass 1 (row pass): each CTA stages whole rows of x in shared memory and
//   applies the diagonal and the up hops from there (gathers stay on chip).
// Pass 2 (slab pass): the down hops are row-axpys y[d][:] += c x[e][:].
//   Columns are cut into slabs so that one slab of x (nsdn rows x slab
//   width) stays resident in L2 while every output row of that slab gathers
//   its ~N neighbour rows; x therefore streams from HBM about once.  The pass
//   also forms <x,y> and <y,y> for the Lanczos scalars.
//
// Heisenberg (replaces HPROD, hprod_heis.f90:1-61): ed_heis.cu, on the same
// row/pass structure (rows of B-half patterns over A-half patterns).
#include "ed_common.cuh"

#include <cstdlib>

namespace ed {

struct HubArgs {
    int64_t nsup, nsdn, ld;
    const uint32_t *ustr; const int32_t *uptr; const int32_t *usrc; const void *ucf; const void *uediag;
    const uint32_t *dstr; const int32_t *dptr; const int32_t *dsrc; const void *dcf; const void *dediag;
    int64_t nslice;
    const int32_t *ell_off; const int32_t *ell_src;
    const int2 *ell_pk32;
    double u_site[kMaxSites];
    float u_site32[kMaxSites];
    int u_uniform;
    double u_value;
    double scale;
};

template <typename T>
__device__ __forceinline__ const T *u_sites(const HubArgs &a)
{
    return (sizeof(T) == 4) ? reinterpret_cast<const T *>(a.u_site32) : reinterpret_cast<const T *>(a.u_site);
}

// on-site energy of the doubly occupied bits `both`; uval = U in T (uniform U)
template <typename T>
__device__ __forceinline__ T u_energy(const HubArgs &a, uint32_t both, T uval)
{
    if (a.u_uniform) return uval * (T)__popc(both);
    const T *us = u_sites<T>(a);
    T e = 0;
    while (both) {
        int b = __ffs(both) - 1;
        e += us[b];
        both &= both - 1;
    }
    return e;
}

// Copy n elements from global src to shared dst (dst 16-byte aligned).
template <typename T>
__device__ __forceinline__ void stage_row(T *dst, const T *__restrict__ src, int64_t n, bool vec_ok)
{
    constexpr int VW = 16 / sizeof(T);
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    if (vec_ok) {
        int64_t nv = (n + VW - 1) / VW;  // may read into the zero padding of the row
        const V *s4 = reinterpret_cast<const V *>(src);
        V *d4 = reinterpret_cast<V *>(dst);
        for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) d4[i] = __ldg(s4 + i);
    } else {
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = __ldg(src + i);
    }
}

// G up-hop slots of one lane (table entries at, at+32, ...) applied to the R
// staged rows; the G table loads are issued before the first gather (FP32:
// one packed 8-byte {source, coefficient} load per slot).
template <typename T, int R, int G>
__device__ __forceinline__ void row_group(const HubArgs &a, const T *__restrict__ ecf, int64_t at, const T *xs,
                                          int64_t sld, T (&acc)[R])
{
    int q[G];
    T c[G];
#pragma unroll
    for (int i = 0; i < G; ++i) {
        if (sizeof(T) == 4) {
            const int2 pk = __ldg(a.ell_pk32 + at + i * 32);
            q[i] = pk.x;
            c[i] = (T)__int_as_float(pk.y);
        } else {
            q[i] = __ldg(a.ell_src + at + i * 32);
            c[i] = __ldg(ecf + at + i * 32);
        }
    }
#pragma unroll
    for (int i = 0; i < G; ++i)
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] += c[i] * xs[r * sld + q[i]];
}

// Pass 1: diagonal + up hops, R rows per CTA iteration.  Each warp owns one
// 32-string slice at a time and walks its sliced-ELL slots (coalesced,
// four slots in flight), gathering the sources from the staged rows.
template <typename T, int R>
__global__ void __launch_bounds__(512) hub_row_kernel(const T *__restrict__ x, T *__restrict__ y,
                                                      const HubArgs a, int64_t sld, int vec_ok)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);
    const T *__restrict__ ecf = static_cast<const T *>(a.ucf);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int64_t nsup = a.nsup, ld = a.ld;
    const T uval = (T)a.u_value, sc = (T)a.scale;
    const T *ued_t = static_cast<const T *>(a.uediag), *ded_t = static_cast<const T *>(a.dediag);
    for (int64_t d0 = (int64_t)blockIdx.x * R; d0 < a.nsdn; d0 += (int64_t)gridDim.x * R) {
        const int nr = (int)min((int64_t)R, a.nsdn - d0);
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r < nr) stage_row<T>(xs + r * sld, x + (d0 + r) * ld, nsup, vec_ok != 0);
        __syncthreads();
        uint32_t sd[R];
        T ed[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            sd[r] = (r < nr) ? __ldg(a.dstr + d0 + r) : 0u;
            ed[r] = (r < nr) ? __ldg(ded_t + d0 + r) : (T)0;
        }
        for (int64_t sl = warp; sl < a.nslice; sl += nwarps) {
            const int64_t u = sl * 32 + lane;
            const bool ok = u < nsup;
            const int64_t uu = ok ? u : nsup - 1;
            const uint32_t su = __ldg(a.ustr + uu);
            const T eu = __ldg(ued_t + uu);
            T acc[R];
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r] = (eu + ed[r] + u_energy<T>(a, su & sd[r], uval)) * xs[r * sld + uu];
            const int s0 = __ldg(a.ell_off + sl), ns = __ldg(a.ell_off + sl + 1) - s0;
            const int64_t at0 = (int64_t)s0 * 32 + lane;
            // slots in groups: all table loads of a group are in flight before its first gather
            int k = 0;
            for (; k + 8 <= ns; k += 8) row_group<T, R, 8>(a, ecf, at0 + k * 32, xs, sld, acc);
            if (k + 4 <= ns) {
                row_group<T, R, 4>(a, ecf, at0 + k * 32, xs, sld, acc);
                k += 4;
            }
            for (; k < ns; ++k) row_group<T, R, 1>(a, ecf, at0 + k * 32, xs, sld, acc);
            if (ok) {
#pragma unroll
                for (int r = 0; r < R; ++r)
                    if (r < nr) y[(d0 + r) * ld + u] = acc[r] * sc;
            }
        }
        __syncthreads();
    }
}

// Pass 1 for FP32 with four rows per CTA, column layout: the four rows of
// string u are staged as one 16-byte column xs4[u], so a hop gathers all four
// rows with one 128-bit shared load.  A quarter warp's 8 lanes hit 8 bank
// groups when their sources differ mod 8, which the sliced-ELL slot order
// arranges (ed_sector.cu, ell_order).
template <int G>
__device__ __forceinline__ void col_group(const HubArgs &a, int64_t at, const float4 *xs4, float (&acc)[4])
{
    int q[G];
    float c[G];
#pragma unroll
    for (int i = 0; i < G; ++i) {
        const int2 pk = __ldg(a.ell_pk32 + at + i * 32);
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

__global__ void __launch_bounds__(1024) hub_row_col4_kernel(const float *__restrict__ x, float *__restrict__ y,
                                                            const HubArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *xs4 = reinterpret_cast<float4 *>(smem_raw);   // [nsup]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int64_t nsup = a.nsup, ld = a.ld;
    const float uval = (float)a.u_value, sc = (float)a.scale;
    const float *ued_t = static_cast<const float *>(a.uediag), *ded_t = static_cast<const float *>(a.dediag);
    for (int64_t d0 = (int64_t)blockIdx.x * 4; d0 < a.nsdn; d0 += (int64_t)gridDim.x * 4) {
        const int nr = (int)min((int64_t)4, a.nsdn - d0);
        const float *x0 = x + d0 * ld;
        for (int64_t c = threadIdx.x; c < nsup; c += blockDim.x) {
            float4 v;
            v.x = __ldg(x0 + c);
            v.y = nr > 1 ? __ldg(x0 + ld + c) : 0.f;
            v.z = nr > 2 ? __ldg(x0 + 2 * ld + c) : 0.f;
            v.w = nr > 3 ? __ldg(x0 + 3 * ld + c) : 0.f;
            xs4[c] = v;
        }
        __syncthreads();
        uint32_t sd[4];
        float ed[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            sd[r] = (r < nr) ? __ldg(a.dstr + d0 + r) : 0u;
            ed[r] = (r < nr) ? __ldg(ded_t + d0 + r) : 0.f;
        }
        for (int64_t sl = warp; sl < a.nslice; sl += nwarps) {
            const int64_t u = sl * 32 + lane;
            const bool ok = u < nsup;
            const int64_t uu = ok ? u : nsup - 1;
            const uint32_t su = __ldg(a.ustr + uu);
            const float eu = __ldg(ued_t + uu);
            const float4 xv = xs4[uu];
            const float xr[4] = {xv.x, xv.y, xv.z, xv.w};
            float acc[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[r] = (eu + ed[r] + u_energy<float>(a, su & sd[r], uval)) * xr[r];
            const int s0 = __ldg(a.ell_off + sl), ns = __ldg(a.ell_off + sl + 1) - s0;
            const int64_t at0 = (int64_t)s0 * 32 + lane;
            int k = 0;
            for (; k + 8 <= ns; k += 8) col_group<8>(a, at0 + k * 32, xs4, acc);
            if (k + 4 <= ns) {
                col_group<4>(a, at0 + k * 32, xs4, acc);
                k += 4;
            }
            for (; k < ns; ++k) col_group<1>(a, at0 + k * 32, xs4, acc);
            if (ok) {
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (r < nr) y[(d0 + r) * ld + u] = acc[r] * sc;
            }
        }
        __syncthreads();
    }
}

constexpr int kSlabLoads = 4;   // neighbour-row loads in flight per warp in the slab pass (8 costs occupancy)

// Pass 2: down hops, y[d][slab] += sum_e c_e x[src_e][slab]; optional dots.
// Work items (slab, group of 8 rows) are visited slab-major by a persistent
// grid so that the CTAs in flight share one or two slabs of x in L2.  A warp
// holds its row's neighbour list in registers (one entry per lane) and issues
// the neighbour loads of a chunk back to back.
template <typename T, int VW>
__global__ void __launch_bounds__(256) hub_slab_kernel(const T *__restrict__ x, T *__restrict__ y,
                                                       const HubArgs a, int64_t slab_w, int64_t ngroups,
                                                       int64_t nitems, double *__restrict__ partials)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T *__restrict__ cf = static_cast<const T *>(a.dcf);
    const int64_t nsup = a.nsup, ld = a.ld;
    const T sc = (T)a.scale;
    double dxy = 0.0, dyy = 0.0;
    for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int64_t slab = item / ngroups, g = item - slab * ngroups;
        const int64_t d = g * 8 + warp;
        if (d >= a.nsdn) continue;
        const int64_t c0 = slab * slab_w, c1 = min(c0 + slab_w, nsup);
        const int e0 = __ldg(a.dptr + d), nn = __ldg(a.dptr + d + 1) - e0;
        T *yr = y + d * ld;
        const T *xd = x + d * ld;
        float pxy = 0.f, pyy = 0.f;
        double qxy = 0.0, qyy = 0.0;
        for (int b0 = 0; b0 < nn; b0 += 32) {
            const int nb = min(32, nn - b0);
            const int my_src = (lane < nb) ? __ldg(a.dsrc + e0 + b0 + lane) : 0;
            const T my_cf = (lane < nb) ? __ldg(cf + e0 + b0 + lane) * sc : (T)0;
            const bool last = (b0 + 32 >= nn);
            // chunks of 32*VW columns; the loop is warp-uniform so every lane
            // takes part in the shuffles, lanes past c1 are masked
            for (int64_t cb = c0; cb < c1; cb += 32 * VW) {
                const int64_t c = cb + (int64_t)lane * VW;
                const bool full = c + VW <= c1;
                const int nk = full ? VW : (c < c1 ? (int)(c1 - c) : 0);
                T acc[VW];
#pragma unroll
                for (int k = 0; k < VW; ++k) acc[k] = (k < nk) ? yr[c + k] : (T)0;
                int e = 0;
                for (; e + kSlabLoads <= nb; e += kSlabLoads) {
                    T v[kSlabLoads][VW];
                    T wgt[kSlabLoads];
#pragma unroll
                    for (int i = 0; i < kSlabLoads; ++i) {
                        const int64_t sidx = __shfl_sync(0xffffffffu, my_src, e + i);
                        wgt[i] = __shfl_sync(0xffffffffu, my_cf, e + i);
                        const T *xr = x + sidx * ld + c;
                        if (full) {
                            if constexpr (VW == 4 && sizeof(T) == 4) {
                                const float4 t4 = __ldg(reinterpret_cast<const float4 *>(xr));
                                v[i][0] = t4.x; v[i][1] = t4.y; v[i][2] = t4.z; v[i][3] = t4.w;
                            } else if constexpr (VW == 2 && sizeof(T) == 8) {
                                const double2 t2 = __ldg(reinterpret_cast<const double2 *>(xr));
                                v[i][0] = t2.x; v[i][1] = t2.y;
                            } else {
#pragma unroll
                                for (int k = 0; k < VW; ++k) v[i][k] = __ldg(xr + k);
                            }
                        } else {
#pragma unroll
                            for (int k = 0; k < VW; ++k) v[i][k] = (k < nk) ? __ldg(xr + k) : (T)0;
                        }
                    }
#pragma unroll
                    for (int i = 0; i < kSlabLoads; ++i)
#pragma unroll
                        for (int k = 0; k < VW; ++k) acc[k] += wgt[i] * v[i][k];
                }
                for (; e < nb; ++e) {
                    const int64_t sidx = __shfl_sync(0xffffffffu, my_src, e);
                    const T wg = __shfl_sync(0xffffffffu, my_cf, e);
#pragma unroll
                    for (int k = 0; k < VW; ++k)
                        if (k < nk) acc[k] += wg * __ldg(x + sidx * ld + c + k);
                }
#pragma unroll
                for (int k = 0; k < VW; ++k)
                    if (k < nk) yr[c + k] = acc[k];
                if (partials && last) {
#pragma unroll
                    for (int k = 0; k < VW; ++k) {
                        if (k >= nk) continue;
                        const T xv = __ldg(xd + c + k);
                        if constexpr (sizeof(T) == 4) { pxy += xv * acc[k]; pyy += acc[k] * acc[k]; }
                        else { qxy += xv * acc[k]; qyy += acc[k] * acc[k]; }
                    }
                }
            }
        }
        if (nn == 0 && partials) {
            // no down hops: the dots still need this row's y
            for (int64_t cc = c0 + lane; cc < c1; cc += 32) {
                const T yv = yr[cc], xv = __ldg(xd + cc);
                if constexpr (sizeof(T) == 4) { pxy += xv * yv; pyy += yv * yv; }
                else { qxy += xv * yv; qyy += yv * yv; }
            }
        }
        dxy += (double)pxy + qxy;
        dyy += (double)pyy + qyy;
    }
    if (partials) {
        __shared__ double red[2][8];
        dxy = warp_sum(dxy);
        dyy = warp_sum(dyy);
        if (lane == 0) { red[0][warp] = dxy; red[1][warp] = dyy; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sxy = 0.0, syy = 0.0;
            for (int w = 0; w < 8; ++w) { sxy += red[0][w]; syy += red[1][w]; }
            partials[2 * blockIdx.x] = sxy;
            partials[2 * blockIdx.x + 1] = syy;
        }
    }
}

// Sum nblocks rows of m partials into out[m] (FP64, fixed order).
__global__ void reduce_partials_kernel(const double *__restrict__ partials, int nblocks, int m,
                                       double *__restrict__ out)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    for (int j = blockIdx.x * nw + warp; j < m; j += gridDim.x * nw) {
        double s = 0.0;
        for (int b = lane; b < nblocks; b += 32) s += partials[(int64_t)b * m + j];
        s = warp_sum(s);
        if (lane == 0) out[j] = s;
    }
}

int launch_reduce(const double *partials, int nblocks, int m, double *out, cudaStream_t st)
{
    int threads = 256, per = threads / 32;
    int blocks = (m + per - 1) / per;
    if (blocks > 1024) blocks = 1024;
    reduce_partials_kernel<<<blocks, threads, 0, st>>>(partials, nblocks, m, out);
    ED_CHECK_LAUNCH();
    return ED_OK;
}

// The Heisenberg product lives in ed_heis.cu.

// ------------------------------------------------------------ launchers

static constexpr int kMaxPartialBlocks = 1024;

// L2 budget of one x slab in the slab pass: 48 MB (a third of the 129 MB
// L2, leaving room for the y slab in flight and the tables); the
// environment variable PYHUB_ED_SLAB_L2_BYTES overrides it for tuning.
static double slab_l2_bytes()
{
    static double v = []() {
        const char *e = std::getenv("PYHUB_ED_SLAB_L2_BYTES");
        const double d = e ? std::atof(e) : 0.0;
        return (d >= 1.0e6 && d <= 1.0e9) ? d : 48.0e6;
    }();
    return v;
}

template <typename T>
static int hub_hv(ed_sector *s, cudaStream_t st, int64_t ld, const T *x, T *y, double scale, double *dots,
                  double *partials)
{
    HubArgs a;
    a.nsup = s->nsup; a.nsdn = s->nsdn; a.ld = ld;
    a.ustr = s->up.str; a.uptr = s->up.ptr; a.usrc = s->up.src;
    a.dstr = s->dn.str; a.dptr = s->dn.ptr; a.dsrc = s->dn.src;
    a.uediag = (sizeof(T) == 4) ? (const void *)s->up.ediag32 : (const void *)s->up.ediag;
    a.dediag = (sizeof(T) == 4) ? (const void *)s->dn.ediag32 : (const void *)s->dn.ediag;
    if (sizeof(T) == 4) { a.ucf = s->up.ell_cf32; a.dcf = s->dn.cf32; }
    else { a.ucf = s->up.ell_cf64; a.dcf = s->dn.cf64; }
    a.nslice = s->up.nslice;
    a.ell_off = s->up.ell_off;
    a.ell_src = s->up.ell_src;
    a.ell_pk32 = s->up.ell_pk32;
    for (int b = 0; b < kMaxSites; ++b) {
        a.u_site[b] = s->u_site[b];
        a.u_site32[b] = (float)s->u_site[b];
    }
    a.u_uniform = s->u_uniform ? 1 : 0;
    a.u_value = s->u_value;
    a.scale = scale;
    const int nsm = num_sms();
    constexpr int VWS = 16 / sizeof(T);
    // ---- pass 1
    const int64_t sld = (s->nsup + VWS - 1) / VWS * VWS;
    const bool vec_ok = (ld % VWS == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
    int maxsm = 0;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t row_bytes = (size_t)sld * sizeof(T);
    if (row_bytes > (size_t)maxsm) {
        set_error("up-string row of %lld entries does not fit in shared memory (%d bytes)",
                  (long long)s->nsup, maxsm);
        return ED_ERR_RANGE;
    }
    // FP32: four rows per 1024-thread CTA (one CTA per SM) when they fit, so every
    // hop-table slot serves four rows and one 128-bit gather reads all four;
    // else two rows per CTA with two CTAs per SM; else one.
    constexpr int R2 = 2;
    const bool two = (size_t)R2 * row_bytes * 2 <= (size_t)maxsm;
    const int threads = 512;
    if (sizeof(T) == 4 && (size_t)s->nsup * 16 <= (size_t)maxsm) {
        // four rows per 1024-thread CTA, staged as 16-byte columns
        const size_t smem = (size_t)s->nsup * 16;
        int64_t blocks = (s->nsdn + 3) / 4;
        if (blocks > nsm) blocks = nsm;
        ED_CHECK_CUDA(cudaFuncSetAttribute(hub_row_col4_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
        hub_row_col4_kernel<<<(unsigned)blocks, 1024, smem, st>>>(reinterpret_cast<const float *>(x),
                                                                  reinterpret_cast<float *>(y), a);
    } else if (two) {
        size_t smem = (size_t)R2 * row_bytes;
        ED_CHECK_CUDA(cudaFuncSetAttribute(hub_row_kernel<T, R2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int64_t blocks = (s->nsdn + R2 - 1) / R2;
        int64_t cap = (int64_t)nsm * 2;
        if (blocks > cap) blocks = cap;
        hub_row_kernel<T, R2><<<(unsigned)blocks, threads, smem, st>>>(x, y, a, sld, vec_ok ? 1 : 0);
    } else {
        size_t smem = row_bytes;
        ED_CHECK_CUDA(cudaFuncSetAttribute(hub_row_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int64_t blocks = s->nsdn;
        int64_t cap = (int64_t)nsm * 2;
        if (blocks > cap) blocks = cap;
        hub_row_kernel<T, 1><<<(unsigned)blocks, threads, smem, st>>>(x, y, a, sld, vec_ok ? 1 : 0);
    }
    ED_CHECK_LAUNCH();
    // ---- the U_ijkl terms, if any (before pass 2, whose fused dots need the whole product)
    if (s->uijkl) {
        const int rc = uijkl_hv(s, st, sizeof(T) == 4 ? ED_F32 : ED_F64, ld, x, y, scale);
        if (rc != ED_OK) return rc;
    }
    // ---- pass 2
    // slab width: the x slab (nsdn rows x width) should take at most slab_l2_bytes() of L2
    int64_t slab_w = (int64_t)(slab_l2_bytes() / ((double)s->nsdn * sizeof(T)));
    slab_w = slab_w / 256 * 256;
    if (slab_w < 256) slab_w = 256;
    if (slab_w > s->nsup) slab_w = (s->nsup + VWS - 1) / VWS * VWS;
    const int64_t ngroups = (s->nsdn + 7) / 8;
    const int64_t nslab = (s->nsup + slab_w - 1) / slab_w;
    const int64_t nitems = ngroups * nslab;
    // one wave of resident CTAs: each walks its share of the items, so a grid past the
    // resident count would leave a second, partial wave running whole shares
    const bool vec2pre = (ld % VWS == 0);
    int per_sm = 0;
    if (vec2pre)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hub_slab_kernel<T, VWS>, 256, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hub_slab_kernel<T, 1>, 256, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t blocks2 = (int64_t)nsm * per_sm;
    if (blocks2 > kMaxPartialBlocks) blocks2 = kMaxPartialBlocks;
    if (blocks2 > nitems) blocks2 = nitems;
    if (blocks2 < 1) blocks2 = 1;
    const bool vec2 = (ld % VWS == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0) &&
                      ((reinterpret_cast<uintptr_t>(y) & 15) == 0);
    double *part = dots ? partials : nullptr;
    if (vec2)
        hub_slab_kernel<T, VWS><<<(unsigned)blocks2, 256, 0, st>>>(x, y, a, slab_w, ngroups, nitems, part);
    else
        hub_slab_kernel<T, 1><<<(unsigned)blocks2, 256, 0, st>>>(x, y, a, slab_w, ngroups, nitems, part);
    ED_CHECK_LAUNCH();
    if (dots) return launch_reduce(partials, (int)blocks2, 2, dots, st);
    return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" int64_t ed_scratch_bytes(int64_t n, int nvec)
{
    (void)n;
    if (nvec < 1) nvec = 1;
    return (int64_t)kMaxPartialBlocks * 2 * nvec * (int64_t)sizeof(double) + 4096;
}

extern "C" int ed_hv(ed_sector *s, void *stream, int dtype, int64_t ld, const void *x, void *y, double scale,
                     double *dots, void *scratch, int64_t scratch_bytes)
{
    clear_error();
    ED_REQUIRE(s != nullptr, "sector is NULL");
    ED_REQUIRE(x != nullptr && y != nullptr, "x or y is NULL");
    ED_REQUIRE(x != y, "x and y must not alias");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "dtype must be ED_F32 or ED_F64");
    if (dots) {
        ED_REQUIRE(scratch != nullptr, "dots requested without scratch");
        ED_REQUIRE(scratch_bytes >= ed_scratch_bytes(s->dim, 1), "scratch of %lld bytes is below the %lld needed",
                   (long long)scratch_bytes, (long long)ed_scratch_bytes(s->dim, 1));
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (s->dim == 0) return ED_OK;
    if (s->kind == ED_HUBBARD) {
        ED_REQUIRE(ld >= s->nsup, "ld=%lld below nsup=%lld", (long long)ld, (long long)s->nsup);
        if (dtype == ED_F32)
            return hub_hv<float>(s, st, ld, static_cast<const float *>(x), static_cast<float *>(y), scale, dots,
                                 static_cast<double *>(scratch));
        return hub_hv<double>(s, st, ld, static_cast<const double *>(x), static_cast<double *>(y), scale, dots,
                              static_cast<double *>(scratch));
    }
    return heis_struct_hv(s, st, dtype, x, y, scale, dots, static_cast<double *>(scratch));
}
