// ed_ops.cu -- the generic operator engine: a sum of products of the
// elementary operators of operators.x applied to a vector of an operator
// space (ed_opspace: every listed up-particle number times every listed
// down-particle number).
//
// Reference counterparts: PROGRAM OPERATOR (compute_operators.f90:28-66)
// for the term loop, and the elementary routines of operators.f90:
// C_DAGGER_C (:1-59), C_DAGGER_C_UNRES (:62-144), NI (:150-175), NIM1
// (:194-219), SZ_OPE (:223-248), C_DAGGER (:410-465), C_ (:469-523).  Each
// elementary operator maps a basis state to at most one basis state and no
// two states to the same one, so a kernel is one thread per input state
// writing its image (the output is cleared first).  The factors of a product
// act in the order of the term's list, the first one first, as the Fortran
// loop over J applies them.  Signs follow ANTICOM (funcmod.f90:29-41):
// (-1)^(occupied sites 1..POS-1 of the string), 1 for POS = 0.
#include "ed_common.cuh"

#include <algorithm>
#include <cmath>

namespace ed {

// Operator codes of the reference's operator file (_operators.py:438-460).
enum OpCode : int {
    kOpHop = 1,       // c^+_{i s} c_{j s}
    kOpN = 2,         // n_{i s}
    kOpId = 3,        // identity
    kOpNm1 = 4,       // 1 - n_{i s}
    kOpSz = 5,        // SZ_OPE
    kOpSplus = 6,     // c^+_{i up} c_{i down}
    kOpSminus = 7,    // c^+_{i down} c_{i up}
    kOpSisj = 8,      // SISJ: no producer in the Python API
    kOpHopFlip = 9,   // c^+_{i, other spin of s_j} c_{j s_j}
    kOpCdag = 10,     // c^+_{i s}
    kOpC = 11,        // c_{i s}
    kOpSzBasis = 12   // SZ_BASIS (operators_basis.f90:134-145): the basis-element form of sz, + S^z
};

struct OpArgs {
    int norb;
    int64_t nsup, nsdn;
    int64_t up_off[kMaxSites + 1], dn_off[kMaxSites + 1];
    const uint32_t *ustr, *dstr, *lut;
};

// site POS (1-based) is bit norb-POS of a string
__device__ __forceinline__ uint32_t site_bit_dev(int norb, int pos) { return 1u << (norb - pos); }

// ANTICOM(NORB,POS,STATE): (-1)^(occupied sites 1..POS-1); 1 for POS <= 1
__device__ __forceinline__ double anticom_dev(int norb, int pos, uint32_t s)
{
    if (pos <= 1) return 1.0;
    const uint32_t mask = ((1u << (pos - 1)) - 1u) << (norb - pos + 1);
    return (__popc(s & mask) & 1) ? -1.0 : 1.0;
}

// index of a string in the concatenated list of one species, -1 when its
// particle number is not listed (the Fortran's POS = 0: the term is dropped)
__device__ __forceinline__ int64_t list_index(const OpArgs &a, uint32_t s, bool up)
{
    const int64_t off = up ? a.up_off[__popc(s)] : a.dn_off[__popc(s)];
    if (off < 0) return -1;
    return off + (int64_t)rank_holes(a.lut, holes_dev(s, a.norb));
}

__global__ void __launch_bounds__(256) ops_elem_kernel(const OpArgs a, int code, int si, int spi, int sj, int spj,
                                                       const double *__restrict__ in, double *__restrict__ out)
{
    const int64_t nst = a.nsup * a.nsdn;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nst;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = idx / a.nsup, u = idx - d * a.nsup;
        const uint32_t su = __ldg(a.ustr + u), sd = __ldg(a.dstr + d);
        const double x = in[idx];
        const int norb = a.norb;
        switch (code) {
        case kOpHop: {
            // KINOP(NORB, B, K=sj, J=si): the particle at K moves to J (or stays when J = K)
            const bool up = (spi == 1);
            const uint32_t s = up ? su : sd;
            const uint32_t A = site_bit_dev(norb, sj), B = site_bit_dev(norb, si);
            if (!(s & A)) break;
            uint32_t ns;
            if (si != sj) {
                if (s & B) break;
                ns = s - A + B;
            } else {
                ns = s;
            }
            const int64_t pos = list_index(a, ns, up);
            if (pos < 0) break;
            const double ac = anticom_dev(norb, sj, s) * anticom_dev(norb, si, ns);
            out[up ? d * a.nsup + pos : pos * a.nsup + u] = ac * x;
            break;
        }
        case kOpN:
        case kOpNm1: {
            const uint32_t s = (spi == 1) ? su : sd;
            const bool occ = (s & site_bit_dev(norb, si)) != 0;
            if (occ == (code == kOpN)) out[idx] = x;
            break;
        }
        case kOpSz: {
            // SZ_OPE: + x/2 where site i holds no up particle, - x/2 where it holds no down particle
            const uint32_t b = site_bit_dev(norb, si);
            double v = 0.0;
            if (!(su & b)) v = v + x / 2.0;
            if (!(sd & b)) v = v - x / 2.0;
            out[idx] = v;
            break;
        }
        case kOpSzBasis: {
            // VAL = VAL * SZ(NORB, SI, BUP, BDOWN): +1/2 for an up particle, -1/2 for a down one
            const uint32_t b = site_bit_dev(norb, si);
            double sz = 0.0;
            if (su & b) sz = sz + 0.5;
            if (sd & b) sz = sz - 0.5;
            out[idx] = x * sz;
            break;
        }
        case kOpSplus:
        case kOpSminus:
        case kOpHopFlip: {
            // C_DAGGER_C_UNRES(J, K, SPINK): c^+_{J, other spin} c_{K, SPINK}
            const int J = si;
            const int K = (code == kOpHopFlip) ? sj : si;
            const int spink = (code == kOpSplus) ? 2 : (code == kOpSminus) ? 1 : spj;
            const uint32_t bk = site_bit_dev(norb, K), bj = site_bit_dev(norb, J);
            if (spink == 1) {
                if (!(su & bk)) break;
                const uint32_t nu = su - bk;
                const int64_t pos = list_index(a, nu, true);
                if (pos < 0 || (sd & bj)) break;
                const uint32_t nd = sd + bj;
                const int64_t pos2 = list_index(a, nd, false);
                if (pos2 < 0) break;
                const double ac = anticom_dev(norb, K, nu);
                const double ac2 = anticom_dev(norb, J, nd) * anticom_dev(norb, 0, sd);
                out[pos2 * a.nsup + pos] = ac * ac2 * x;
            } else {
                if (!(sd & bk)) break;
                const uint32_t nd = sd - bk;
                const int64_t pos = list_index(a, nd, false);
                if (pos < 0 || (su & bj)) break;
                const uint32_t nu = su + bj;
                const int64_t pos2 = list_index(a, nu, true);
                if (pos2 < 0) break;
                const double ac = anticom_dev(norb, K, nd);
                const double ac2 = anticom_dev(norb, 0, nd) * anticom_dev(norb, J, nu);
                out[pos * a.nsup + pos2] = ac * ac2 * x;
            }
            break;
        }
        case kOpCdag:
        case kOpC: {
            const bool up = (spi == 1);
            const uint32_t s = up ? su : sd, b = site_bit_dev(norb, si);
            const bool occ = (s & b) != 0;
            if (occ == (code == kOpCdag)) break;   // creation needs an empty site, annihilation an occupied one
            const uint32_t ns = (code == kOpCdag) ? s + b : s - b;
            const int64_t pos = list_index(a, ns, up);
            if (pos < 0) break;
            const double ac = anticom_dev(norb, si, s);
            if (up)
                out[d * a.nsup + pos] = ac * anticom_dev(norb, 0, sd) * x;
            else
                out[pos * a.nsup + u] = ac * x;
            break;
        }
        default:
            break;
        }
    }
}

// y = y + c * v, one rounding per operation (PSI_OUT = PSI_OUT + COEFF(I)*PSI_IN)
__global__ void __launch_bounds__(256) ops_axpy_kernel(int64_t n, double c, const double *__restrict__ v,
                                                       double *__restrict__ y)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __dadd_rn(y[i], __dmul_rn(c, v[i]));
}

}  // namespace ed

using namespace ed;

extern "C" int ed_ops_apply(const ed_opspace *sp, void *stream, int nterms, const int32_t *term_off,
                            const int32_t *ops, const double *coeff, const double *x, double *y, double *work,
                            int64_t work_bytes)
{
    clear_error();
    ED_REQUIRE(sp != nullptr, "operator space is NULL");
    ED_REQUIRE(nterms >= 0, "nterms=%d", nterms);
    ED_REQUIRE(nterms == 0 || (term_off != nullptr && ops != nullptr && coeff != nullptr), "NULL term list");
    ED_REQUIRE(x != nullptr && y != nullptr && work != nullptr, "NULL vector");
    const int64_t nst = sp->nsup * sp->nsdn;
    ED_REQUIRE(work_bytes >= 2 * nst * (int64_t)sizeof(double), "work of %lld bytes is below %lld",
               (long long)work_bytes, (long long)(2 * nst * (int64_t)sizeof(double)));
    ED_REQUIRE(x != y && x != work && y != work, "x, y and work must not alias");
    // validate the whole list before anything is enqueued
    for (int t = 0; t < nterms; ++t) {
        ED_REQUIRE(term_off[t] >= 0 && term_off[t] <= term_off[t + 1], "term offsets not ascending at %d", t);
        for (int q = term_off[t]; q < term_off[t + 1]; ++q) {
            const int32_t *o = ops + 5 * (int64_t)q;
            const int code = o[0];
            ED_REQUIRE(code >= 0 && code <= kOpSzBasis, "operator code %d of term %d", code, t);
            ED_REQUIRE(code != kOpSisj, "operator code 8 (SISJ) has no producer in the operator algebra; "
                                        "build S_i.S_j from c_dagger_c and sz terms");
            if (code == 0 || code == kOpId) continue;
            ED_REQUIRE(o[1] >= 1 && o[1] <= sp->norb, "site %d of term %d outside 1..%d", o[1], t, sp->norb);
            const bool two = (code == kOpHop || code == kOpHopFlip);
            if (two) ED_REQUIRE(o[3] >= 1 && o[3] <= sp->norb, "site %d of term %d outside 1..%d", o[3], t, sp->norb);
            const bool spin1 = (code == kOpHop || code == kOpN || code == kOpNm1 || code == kOpCdag || code == kOpC);
            if (spin1) ED_REQUIRE(o[2] == 1 || o[2] == 2, "spin %d of term %d (1 up, 2 down)", o[2], t);
            if (code == kOpHopFlip) ED_REQUIRE(o[4] == 1 || o[4] == 2, "spin %d of term %d (1 up, 2 down)", o[4], t);
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    OpArgs a;
    a.norb = sp->norb;
    a.nsup = sp->nsup;
    a.nsdn = sp->nsdn;
    for (int n = 0; n <= kMaxSites; ++n) {
        a.up_off[n] = sp->up_off[n];
        a.dn_off[n] = sp->dn_off[n];
    }
    a.ustr = sp->ustr;
    a.dstr = sp->dstr;
    a.lut = sp->lut;
    ED_CHECK_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * (size_t)nst, st));
    if (nst == 0) return ED_OK;
    const int nsm = num_sms();
    const unsigned blocks = (unsigned)std::min<int64_t>((nst + 255) / 256, (int64_t)nsm * 8);
    double *A = work, *B = work + nst;
    for (int t = 0; t < nterms; ++t) {
        // IF (ABS(COEFF(I)) .GT. 1.E-14): a default-real literal, compared after promotion
        if (!(fabs(coeff[t]) > (double)1e-14f)) continue;
        ED_CHECK_CUDA(cudaMemcpyAsync(A, x, sizeof(double) * (size_t)nst, cudaMemcpyDeviceToDevice, st));
        for (int q = term_off[t]; q < term_off[t + 1]; ++q) {
            const int32_t *o = ops + 5 * (int64_t)q;
            if (o[0] == 0 || o[0] == kOpId) continue;
            ED_CHECK_CUDA(cudaMemsetAsync(B, 0, sizeof(double) * (size_t)nst, st));
            ops_elem_kernel<<<blocks, 256, 0, st>>>(a, o[0], o[1], o[2], o[3], o[4], A, B);
            ED_CHECK_LAUNCH();
            std::swap(A, B);
        }
        ops_axpy_kernel<<<blocks, 256, 0, st>>>(nst, coeff[t], A, y);
        ED_CHECK_LAUNCH();
    }
    return ED_OK;
}
