// ed_gf.cu -- start vectors of the particle/hole Green's function.
//
// Replaces LCZ_H_UP, LCZ_H_DOWN, LCZ_E_UP, LCZ_E_DOWN
// (spgf_bandlanczos.f90:453-560) and the start vectors of GF_{E,H}_{UP,DOWN}
// (spgf_ed.f90:304-429): out = c_{i,s}|psi> or c^+_{i,s}|psi> in the N-1 /
// N+1 sector, written in gather form (one thread per target element).  Up
// operators carry the extra sign (-1)^(N_down) of the reference
// (spgf_bandlanczos.f90:468,523): down modes are ordered before up modes.
#include "ed_common.cuh"

namespace ed {

struct GfArgs {
    int norb, kind;           // kind 0 h_up, 1 h_down, 2 e_up, 3 e_down (the sites: GfSites)
    int64_t nsup1, nsdn1, ld1, ld0;
    const uint32_t *ustr1, *dstr1, *lut;
    double sgn_dn_parity;     // (-1)^(N_down of psi) for the up operators
};

// Sites of one multi-site launch (blockIdx.y picks one; its vector starts
// blockIdx.y * out_stride elements into out).
struct GfSites {
    int n;
    int site[kMaxSites];
    int64_t out_stride;
};

template <typename T, typename O>
__global__ void gf_start_kernel(const T *__restrict__ psi, O *__restrict__ out, const GfArgs a, const GfSites ss)
{
    const int site = ss.site[blockIdx.y];
    out += (int64_t)blockIdx.y * ss.out_stride;
    const uint32_t bi = 1u << (a.norb - site);
    // string bits of the sites before `site`: bits norb-1 .. norb-site+1
    const uint32_t above = (site >= 2) ? (((a.norb >= 32) ? 0xFFFFFFFFu : ((1u << a.norb) - 1u)) & ~((bi << 1) - 1u)) : 0u;
    const int64_t n = a.nsup1 * a.nsdn1;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = e / a.nsup1, u = e - d * a.nsup1;
        const uint32_t su = __ldg(a.ustr1 + u), sd = __ldg(a.dstr1 + d);
        double v = 0.0;
        if (a.kind == 0 || a.kind == 2) {
            const bool occ = (su & bi) != 0;
            if ((a.kind == 0 && !occ) || (a.kind == 2 && occ)) {
                const uint32_t s0 = (a.kind == 0) ? (su | bi) : (su & ~bi);
                const int64_t u0 = rank_holes(a.lut, holes_dev(s0, a.norb));
                const double sg = ((__popc(s0 & above) & 1) ? -1.0 : 1.0) * a.sgn_dn_parity;
                v = sg * (double)psi[d * a.ld0 + u0];
            }
        } else {
            const bool occ = (sd & bi) != 0;
            if ((a.kind == 1 && !occ) || (a.kind == 3 && occ)) {
                const uint32_t s0 = (a.kind == 1) ? (sd | bi) : (sd & ~bi);
                const int64_t d0 = rank_holes(a.lut, holes_dev(s0, a.norb));
                const double sg = (__popc(s0 & above) & 1) ? -1.0 : 1.0;
                v = sg * (double)psi[d0 * a.ld0 + u];
            }
        }
        out[d * a.ld1 + u] = (O)v;
    }
}

}  // namespace ed

using namespace ed;

static int gf_start_launch(const ed_sector *src, const ed_sector *dst, void *stream, int kind, const GfSites &ss,
                           int dtype, int64_t ld0, const void *psi, int out_dtype, int64_t ld1, void *out)
{
    ED_REQUIRE(src != nullptr && dst != nullptr && psi != nullptr && out != nullptr, "NULL argument");
    ED_REQUIRE(src->kind == ED_HUBBARD && dst->kind == ED_HUBBARD, "Green's function start vectors need Hubbard sectors");
    ED_REQUIRE(src->norb == dst->norb, "sectors of different sizes");
    ED_REQUIRE(kind >= 0 && kind <= 3, "kind must be 0..3");
    for (int j = 0; j < ss.n; ++j)
        ED_REQUIRE(ss.site[j] >= 1 && ss.site[j] <= src->norb, "site %d outside 1..%d", ss.site[j], src->norb);
    const int dup = (kind == 0) ? -1 : (kind == 2 ? 1 : 0);
    const int ddn = (kind == 1) ? -1 : (kind == 3 ? 1 : 0);
    ED_REQUIRE(dst->nup == src->nup + dup && dst->ndn == src->ndn + ddn,
               "target sector (%d,%d) does not match kind %d on (%d,%d)", dst->nup, dst->ndn, kind, src->nup, src->ndn);
    ED_REQUIRE(ld0 >= src->nsup && ld1 >= dst->nsup, "ld below nsup");
    ED_REQUIRE(dtype == ED_F32 || dtype == ED_F64, "bad dtype");
    ED_REQUIRE(out_dtype == ED_F32 || out_dtype == ED_F64, "bad out_dtype");
    if (dst->dim == 0 || ss.n == 0) return ED_OK;
    GfArgs a;
    a.norb = src->norb; a.kind = kind;
    a.nsup1 = dst->nsup; a.nsdn1 = dst->nsdn; a.ld1 = ld1; a.ld0 = ld0;
    a.ustr1 = dst->up.str; a.dstr1 = dst->dn.str; a.lut = dst->lut;
    a.sgn_dn_parity = (src->ndn & 1) ? -1.0 : 1.0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int64_t blocks = (dst->dim + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 16;
    if (blocks > cap) blocks = cap;
    const dim3 grid((unsigned)blocks, (unsigned)ss.n);
    if (dtype == ED_F64 && out_dtype == ED_F64)
        gf_start_kernel<double, double><<<grid, 256, 0, st>>>((const double *)psi, (double *)out, a, ss);
    else if (dtype == ED_F64)
        gf_start_kernel<double, float><<<grid, 256, 0, st>>>((const double *)psi, (float *)out, a, ss);
    else if (out_dtype == ED_F64)
        gf_start_kernel<float, double><<<grid, 256, 0, st>>>((const float *)psi, (double *)out, a, ss);
    else
        gf_start_kernel<float, float><<<grid, 256, 0, st>>>((const float *)psi, (float *)out, a, ss);
    ED_CHECK_LAUNCH();
    return ED_OK;
}

extern "C" int ed_gf_start(const ed_sector *src, const ed_sector *dst, void *stream, int kind, int site,
                           int dtype, int64_t ld0, const void *psi, int out_dtype, int64_t ld1, void *out)
{
    clear_error();
    GfSites ss;
    ss.n = 1;
    ss.site[0] = site;
    ss.out_stride = 0;
    return gf_start_launch(src, dst, stream, kind, ss, dtype, ld0, psi, out_dtype, ld1, out);
}

extern "C" int ed_gf_start_sites(const ed_sector *src, const ed_sector *dst, void *stream, int kind, int nsites,
                                 const int32_t *sites, int dtype, int64_t ld0, const void *psi, int out_dtype,
                                 int64_t ld1, void *out, int64_t out_stride)
{
    clear_error();
    ED_REQUIRE(nsites >= 0 && nsites <= kMaxSites, "nsites=%d outside 0..%d", nsites, kMaxSites);
    ED_REQUIRE(nsites == 0 || sites != nullptr, "sites is NULL");
    ED_REQUIRE(dst != nullptr && (nsites <= 1 || out_stride >= (dst->nsdn - 1) * ld1 + dst->nsup),
               "out_stride below one vector");
    GfSites ss;
    ss.n = nsites;
    for (int j = 0; j < nsites; ++j) ss.site[j] = sites[j];
    ss.out_stride = out_stride;
    return gf_start_launch(src, dst, stream, kind, ss, dtype, ld0, psi, out_dtype, ld1, out);
}
