// ed_sector.cu -- sector object: spin-string tables, gather-form hop tables,
// diagonal terms and the Heisenberg rank tables; error state; basis and rank
// entry points of the C ABI.
//
// Reference counterparts: HILBERT (compute_basis.f90:67-96) for the string
// order, KINOP/ANTICOM (funcmod.f90:18-41) for hops and signs, the linear
// search of hprod_hubbard.f90:41-47 for the rank, READ_INPUT
// (compute_solver.f90:39-179) for the parameter tables.
#include "ed_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <unordered_map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace ed {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void clear_error() { g_err[0] = '\0'; }

int num_sms()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152;
    return n > 0 ? n : 152;
}

// ------------------------------------------------------------ combinatorics

static int64_t g_binom[kMaxSites + 2][kMaxSites + 2];
static std::once_flag g_binom_once;

// Sectors may be created from several host threads at once: the table is
// filled exactly once.
static void binom_init()
{
    std::call_once(g_binom_once, []() {
        for (int n = 0; n <= kMaxSites + 1; ++n)
            for (int k = 0; k <= kMaxSites + 1; ++k) {
                if (k > n) g_binom[n][k] = 0;
                else if (k == 0 || k == n) g_binom[n][k] = 1;
                else g_binom[n][k] = g_binom[n - 1][k - 1] + g_binom[n - 1][k];
            }
    });
}

static inline int64_t binom(int n, int k)
{
    if (n < 0 || k < 0 || n > kMaxSites + 1 || k > kMaxSites + 1) return 0;
    return g_binom[n][k];
}

// Empty-site pattern of a string: bit j set when site j+1 is empty
// (site POS lives in string bit norb-POS).
static inline uint32_t holes_of(int norb, uint32_t s)
{
    uint32_t h = 0;
    for (int j = 0; j < norb; ++j)
        if (!((s >> (norb - 1 - j)) & 1u)) h |= 1u << j;
    return h;
}

static inline uint32_t string_of_holes(int norb, uint32_t h)
{
    uint32_t s = 0;
    for (int j = 0; j < norb; ++j)
        if (!((h >> j) & 1u)) s |= 1u << (norb - 1 - j);
    return s;
}

// The reference enumerates strings as k-subsets of bit positions in
// lexicographic order.  That index equals the colex rank of the empty-site
// pattern: sum over its set bits p_1 < p_2 < ... of C(p_i, i).
static inline int64_t rank_host(int norb, uint32_t s)
{
    uint32_t h = holes_of(norb, s);
    int64_t r = 0;
    int i = 0;
    for (int p = 0; p < norb; ++p)
        if ((h >> p) & 1u) r += binom(p, ++i);
    return r;
}

static void enumerate_strings(int norb, int ne, uint32_t *out, int64_t n)
{
    int m = norb - ne;  // holes
    uint32_t h = (m >= 32) ? 0xFFFFFFFFu : ((1u << m) - 1u);
    for (int64_t i = 0; i < n; ++i) {
        out[i] = string_of_holes(norb, h);
        if (h == 0) break;
        // next pattern with the same popcount in increasing numeric (colex) order
        uint32_t c = h & (0u - h);
        uint32_t r = h + c;
        h = (((r ^ h) >> 2) / c) | r;
    }
}

// Fortran view T(J,K) of a row-major norb*norb buffer (1-based J,K).
static inline double tf(const double *t, int norb, int J, int K) { return t[(K - 1) * norb + (J - 1)]; }

static inline uint32_t site_bit(int norb, int pos) { return 1u << (norb - pos); }

// Mask of the string bits of the sites strictly between sites a and b.
static inline uint32_t between_mask(int norb, int a, int b)
{
    int lo = a < b ? a : b, hi = a < b ? b : a;
    uint32_t m = 0;
    for (int p = lo + 1; p < hi; ++p) m |= site_bit(norb, p);
    return m;
}

// ------------------------------------------------------------ hop tables

struct HostHop {
    std::vector<uint32_t> str;
    std::vector<int32_t> ptr, src;
    std::vector<double> coef, ediag;
};

static int build_hop_host(int norb, int ne, const double *t, HostHop &h)
{
    int64_t n = binom(norb, ne);
    h.str.resize((size_t)n);
    enumerate_strings(norb, ne, h.str.data(), n);
    h.ptr.resize((size_t)n + 1);
    h.ediag.resize((size_t)n);
    // active (J,K) pairs, J != K
    std::vector<int> pj, pk;
    std::vector<double> pt;
    for (int K = 1; K <= norb; ++K)
        for (int J = 1; J <= norb; ++J) {
            if (J == K) continue;
            double v = tf(t, norb, J, K);
            if (std::fabs(v) >= kTol14) { pj.push_back(J); pk.push_back(K); pt.push_back(v); }
        }
    uint32_t between[kMaxSites * kMaxSites];
    for (size_t a = 0; a < pj.size(); ++a) between[a] = between_mask(norb, pj[a], pk[a]);
    h.src.clear();
    h.coef.clear();
    h.src.reserve((size_t)(n * (int64_t)std::min<size_t>(pj.size(), (size_t)ne * (norb - ne)) + 1));
    h.coef.reserve(h.src.capacity());
    for (int64_t p = 0; p < n; ++p) {
        h.ptr[(size_t)p] = (int32_t)h.src.size();
        uint32_t s = h.str[(size_t)p];
        double dg = 0.0;
        for (int J = 1; J <= norb; ++J) {
            double v = tf(t, norb, J, J);
            if ((s & site_bit(norb, J)) && std::fabs(v) >= kTol14) dg += v;
        }
        h.ediag[(size_t)p] = dg;
        for (size_t a = 0; a < pj.size(); ++a) {
            uint32_t bj = site_bit(norb, pj[a]), bk = site_bit(norb, pk[a]);
            if (!(s & bk) || (s & bj)) continue;  // target needs K occupied, J empty
            uint32_t q = s - bk + bj;
            double sign = (__builtin_popcount(s & between[a]) & 1) ? -1.0 : 1.0;
            h.src.push_back((int32_t)rank_host(norb, q));
            h.coef.push_back(sign * pt[a]);
        }
        if (h.src.size() > (size_t)INT32_MAX) return ED_ERR_RANGE;
    }
    h.ptr[(size_t)n] = (int32_t)h.src.size();
    return ED_OK;
}

// All device tables of one sector live in one allocation: the pieces are
// packed on the host (256-byte aligned) and copied with one cudaMemcpy, so
// creating a sector costs one allocation instead of one per table.
struct TablePool {
    std::vector<unsigned char> host;
    std::vector<std::pair<void **, size_t>> slots;

    template <typename T>
    void add(T **dst, const T *src, size_t count)
    {
        if (count == 0) count = 1;  // keep a valid pointer for empty tables
        const size_t off = (host.size() + 255) / 256 * 256;
        host.resize(off + count * sizeof(T), 0);
        if (src) std::memcpy(host.data() + off, src, count * sizeof(T));
        slots.push_back({reinterpret_cast<void **>(dst), off});
        *dst = nullptr;
    }

    int commit(void **pool)
    {
        *pool = nullptr;
        if (host.empty()) return ED_OK;
        cudaError_t e = cudaMalloc(pool, host.size());
        if (e != cudaSuccess) {
            cudaGetLastError();
            *pool = nullptr;
            set_error("cudaMalloc of %zu bytes for sector tables failed: %s", host.size(), cudaGetErrorString(e));
            return ED_ERR_MEM;
        }
        e = cudaMemcpy(*pool, host.data(), host.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_error("cudaMemcpy to sector tables failed: %s", cudaGetErrorString(e));
            return ED_ERR_CUDA;
        }
        for (auto &sl : slots) *sl.first = static_cast<unsigned char *>(*pool) + sl.second;
        return ED_OK;
    }
};

// Slot layout of a sliced-ELL table: slice offsets and, per (slot, lane),
// the hop-table entry it holds (-1: padding).  It depends only on the hop
// structure (ptr, src), not on the coefficients, so sectors that share a
// lattice and particle number (every cluster of a parameter sweep) share it.
struct EllOrder {
    std::vector<int32_t> ptr, src;   // the structure it was built for
    std::vector<int32_t> off;        // [nslice+1]
    std::vector<int32_t> entry;      // [slots*32]
};

static std::mutex g_ell_mu;
static std::unordered_map<uint64_t, std::vector<std::shared_ptr<const EllOrder>>> g_ell_cache;
static size_t g_ell_count = 0;
constexpr size_t kEllCacheMax = 256;

static uint64_t hash_structure(const HostHop &h)
{
    uint64_t x = 1469598103934665603ull;   // FNV-1a over (n, ptr, src)
    auto mix = [&x](uint32_t v) {
        for (int k = 0; k < 4; ++k) {
            x ^= (v >> (8 * k)) & 0xffu;
            x *= 1099511628211ull;
        }
    };
    mix((uint32_t)h.str.size());
    for (int32_t v : h.ptr) mix((uint32_t)v);
    for (int32_t v : h.src) mix((uint32_t)v);
    return x;
}

static std::shared_ptr<const EllOrder> ell_order(const HostHop &h)
{
    const uint64_t key = hash_structure(h);
    {
        std::lock_guard<std::mutex> lk(g_ell_mu);
        auto it = g_ell_cache.find(key);
        if (it != g_ell_cache.end())
            for (const auto &o : it->second)
                if (o->ptr == h.ptr && o->src == h.src) return o;
    }
    auto o = std::make_shared<EllOrder>();
    o->ptr = h.ptr;
    o->src = h.src;
    const int64_t n = (int64_t)h.str.size();
    const int64_t ns = (n + 31) / 32;
    std::vector<int32_t> &off = o->off;
    off.assign((size_t)ns + 1, 0);
    for (int64_t sl = 0; sl < ns; ++sl) {
        int32_t w = 0;
        for (int64_t u = sl * 32; u < std::min(n, sl * 32 + 32); ++u) w = std::max(w, h.ptr[(size_t)u + 1] - h.ptr[(size_t)u]);
        off[(size_t)sl + 1] = off[(size_t)sl] + w;
    }
    const int64_t slots = off[(size_t)ns];
    o->entry.assign((size_t)std::max<int64_t>(slots * 32, 1), -1);
    // Slot order within a lane is free, so each slot is filled to spread the
    // 32 lanes' sources over the shared-memory banks of the kernels that
    // gather them:
    //   * the batched kernel gathers 16-byte column pieces for 8 lanes at a
    //     time (one quarter warp); a column's bank group is (source mod 8);
    //   * the row kernels gather one 4- or 8-byte word per lane from a staged
    //     row; its bank is (source mod 32) for FP32.
    // Greedy per slot, lanes with the most neighbours left first: prefer a
    // neighbour whose (source mod 32) no lane of the warp and whose
    // (source mod 8) no lane of the quarter uses yet, then one that is new
    // for the quarter only, then one new for the warp only.  Padding slots
    // read the lane's own string (consecutive strings: distinct banks) with
    // weight 0.
    for (int64_t sl = 0; sl < ns; ++sl) {
        const int64_t w = off[(size_t)sl + 1] - off[(size_t)sl];
        std::vector<std::vector<int32_t>> left(32);   // remaining neighbour entries (hop-table positions)
        for (int l = 0; l < 32; ++l) {
            const int64_t u = sl * 32 + l;
            if (u >= n) continue;
            for (int32_t e = h.ptr[(size_t)u]; e < h.ptr[(size_t)u + 1]; ++e) left[(size_t)l].push_back(e);
        }
        for (int64_t k = 0; k < w; ++k) {
            bool used32[32] = {};
            bool used8[4][8] = {};
            int order[32];
            {
                // lanes by remaining neighbours, most first (stable within equal counts)
                int m = 0;
                for (int64_t cnt = w; cnt >= 0 && m < 32; --cnt)
                    for (int l = 0; l < 32; ++l)
                        if ((int64_t)left[(size_t)l].size() == cnt) order[m++] = l;
            }
            for (int oi = 0; oi < 32; ++oi) {
                const int l = order[oi], qw = l >> 3;
                const int64_t u = sl * 32 + l;
                const size_t at = (size_t)((off[(size_t)sl] + k) * 32 + l);
                const int64_t uu = u < n ? u : n - 1;
                std::vector<int32_t> &L = left[(size_t)l];
                const bool must = (int64_t)L.size() >= w - k;   // no spare slot left for this lane
                int pick = -1, best = -1;
                for (size_t j = 0; j < L.size(); ++j) {
                    const int32_t sj = h.src[(size_t)L[j]];
                    const int score = (used8[qw][sj & 7] ? 0 : 2) + (used32[sj & 31] ? 0 : 1);
                    if (score > best) { best = score; pick = (int)j; }
                    if (score == 3) break;
                }
                const int pad_score = (used8[qw][uu & 7] ? 0 : 2) + (used32[uu & 31] ? 0 : 1);
                if (pick >= 0 && !must && best < pad_score) pick = -1;   // padding now is the cleaner choice
                int32_t sat;
                if (pick >= 0) {
                    const int32_t e = L[(size_t)pick];
                    L.erase(L.begin() + pick);
                    o->entry[at] = e;
                    sat = h.src[(size_t)e];
                } else {
                    sat = (int32_t)uu;
                }
                used8[qw][sat & 7] = true;
                used32[sat & 31] = true;
            }
        }
    }
    std::lock_guard<std::mutex> lk(g_ell_mu);
    // a sweep over many different lattices must not grow the cache without bound: past
    // kEllCacheMax structures it starts over (orders in use stay alive through their owners)
    if (g_ell_count >= kEllCacheMax) {
        g_ell_cache.clear();
        g_ell_count = 0;
    }
    g_ell_cache[key].push_back(o);
    ++g_ell_count;
    return o;
}

static int upload_ell(const HostHop &h, HopTable &d, TablePool &pool)
{
    const std::shared_ptr<const EllOrder> o = ell_order(h);
    const int64_t n = (int64_t)h.str.size();
    const int64_t ns = (int64_t)o->off.size() - 1;
    const int64_t slots = o->off[(size_t)ns];
    const std::vector<int32_t> &off = o->off;
    std::vector<int32_t> src((size_t)std::max<int64_t>(slots * 32, 1));
    std::vector<double> c64((size_t)std::max<int64_t>(slots * 32, 1), 0.0);
    for (int64_t sl = 0; sl < ns; ++sl)
        for (int64_t k = off[(size_t)sl]; k < off[(size_t)sl + 1]; ++k)
            for (int l = 0; l < 32; ++l) {
                const size_t at = (size_t)(k * 32 + l);
                const int32_t e = o->entry[at];
                const int64_t u = sl * 32 + l;
                if (e >= 0) {
                    src[at] = h.src[(size_t)e];
                    c64[at] = h.coef[(size_t)e];
                } else {
                    src[at] = (int32_t)(u < n ? u : n - 1);
                    c64[at] = 0.0;
                }
            }
    std::vector<float> c32(c64.begin(), c64.end());
    std::vector<int2> pk(src.size());
    for (size_t q = 0; q < src.size(); ++q) {
        int32_t bits;
        std::memcpy(&bits, &c32[q], sizeof(bits));
        pk[q] = make_int2(src[q], bits);
    }
    d.nslice = ns;
    d.ell_slots = slots;
    pool.add(&d.ell_off, off.data(), off.size());
    pool.add(&d.ell_src, src.data(), src.size());
    pool.add(&d.ell_cf32, c32.data(), c32.size());
    pool.add(&d.ell_cf64, c64.data(), c64.size());
    pool.add(&d.ell_pk32, pk.data(), pk.size());
    return ED_OK;
}

// Pair lists of one spin species (HopTable::pl_off / pl_ent), for every
// ordered pair J != K regardless of T(J,K): the reduced densities need them all.
static int upload_pairs(const HostHop &h, int norb, HopTable &d, TablePool &pool)
{
    const int64_t n = (int64_t)h.str.size();
    std::unordered_map<uint32_t, int32_t> index;
    index.reserve((size_t)n * 2);
    for (int64_t i = 0; i < n; ++i) index[h.str[(size_t)i]] = (int32_t)i;
    std::vector<int32_t> off((size_t)norb * norb + 1, 0);
    std::vector<int2> ent;
    for (int J = 1; J <= norb; ++J)
        for (int K = 1; K <= norb; ++K) {
            const size_t pid = (size_t)(J - 1) * norb + (K - 1);
            off[pid] = (int32_t)ent.size();
            if (J == K) continue;
            const uint32_t bj = site_bit(norb, J), bk = site_bit(norb, K), btw = between_mask(norb, J, K);
            for (int64_t u = 0; u < n; ++u) {
                const uint32_t su = h.str[(size_t)u];
                if (!(su & bj) || (su & bk)) continue;
                const int32_t u2 = index[su - bj + bk];
                const uint32_t sg = (uint32_t)(__builtin_popcount(su & btw) & 1);
                ent.push_back(make_int2((int32_t)u, (int32_t)((uint32_t)u2 | (sg << 31))));
            }
            if (ent.size() > (size_t)INT32_MAX) return ED_ERR_RANGE;
        }
    off[(size_t)norb * norb] = (int32_t)ent.size();
    pool.add(&d.pl_off, off.data(), off.size());
    pool.add(&d.pl_ent, ent.data(), ent.size());
    return ED_OK;
}

// Host side of a hop table: pointers are set when the pool is committed.
static int upload_hop(const HostHop &h, int norb, int ne, HopTable &d, TablePool &pool)
{
    d.norb = norb;
    d.ne = ne;
    d.n = (int64_t)h.str.size();
    d.nnz = (int64_t)h.src.size();
    std::vector<float> c32(h.coef.begin(), h.coef.end());
    std::vector<float> e32(h.ediag.begin(), h.ediag.end());
    pool.add(&d.str, h.str.data(), h.str.size());
    pool.add(&d.ptr, h.ptr.data(), h.ptr.size());
    pool.add(&d.src, h.src.data(), h.src.size());
    pool.add(&d.cf32, c32.data(), c32.size());
    pool.add(&d.cf64, h.coef.data(), h.coef.size());
    pool.add(&d.ediag, h.ediag.data(), h.ediag.size());
    pool.add(&d.ediag32, e32.data(), e32.size());
    d.owner = true;
    const int rc = upload_pairs(h, norb, d, pool);
    if (rc) return rc;
    return upload_ell(h, d, pool);
}

// ------------------------------------------------------------ Heisenberg

// The rank table depends on nothing but the binomials, so every sector of a
// device shares one copy (allocated on first use, kept until the process exits).
static std::mutex g_lut_mu;
static uint32_t *g_lut[64] = {};

static int device_lut(int device, uint32_t **out)
{
    std::lock_guard<std::mutex> lk(g_lut_mu);
    if (device < 0 || device >= 64) {
        set_error("device %d outside 0..63", device);
        return ED_ERR_RANGE;
    }
    if (!g_lut[device]) {
        // lut[b][c][x] = sum over the set bits q of byte x, taken in increasing
        // order with running index i = c+1, c+2, ..., of C(8b+q, i)
        std::vector<uint32_t> lut(4 * 33 * 256, 0u);
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c <= 32; ++c)
                for (int x = 0; x < 256; ++x) {
                    int64_t r = 0;
                    int i = c;
                    for (int q = 0; q < 8; ++q)
                        if ((x >> q) & 1) r += binom(8 * b + q, ++i);
                    lut[(b * 33 + c) * 256 + x] = (uint32_t)r;
                }
        TablePool pool;
        uint32_t *dev = nullptr;
        pool.add(&dev, lut.data(), lut.size());
        void *base = nullptr;
        const int rc = pool.commit(&base);
        if (rc) return rc;
        g_lut[device] = dev;
    }
    *out = g_lut[device];
    return ED_OK;
}

static int build_lut(ed_sector *s)
{
    uint32_t *lut = nullptr;
    const int rc = device_lut(s->device, &lut);
    if (rc == ED_OK) s->lut = lut;
    return rc;
}

static int build_heis(ed_sector *s, const double *J)
{
    int norb = s->norb;
    HeisTables &h = s->heis;
    h.nbond = 0;
    h.dconst = 0.0;
    for (int a = 1; a <= norb; ++a) {
        double jaa = tf(J, norb, a, a);
        if (std::fabs(jaa) > kTol14) h.dconst += 0.5 * jaa;  // hprod_heis.f90:11-21
        h.dconst += 0.25 * jaa;                              // Sz_J Sz_J J(J,J), :54-58
    }
    for (int a = 1; a <= norb; ++a)
        for (int b = a + 1; b <= norb; ++b) {
            double jab = tf(J, norb, a, b), jba = tf(J, norb, b, a);
            if (jab == 0.0 && jba == 0.0) continue;
            int k = h.nbond++;
            h.bj[k] = (int8_t)a;
            h.bk[k] = (int8_t)b;
            // The four ANTICOM factors of hprod_heis.f90:39-45 reduce to
            // (-1)^(J+K) for a complementary down string, so the element that
            // moves the up spin J->K is -(-1)^(J+K) J(J,K) (when |J(J,K)|>tol).
            double par = ((a + b) & 1) ? -1.0 : 1.0;
            h.flip_jk[k] = (std::fabs(jab) > kTol14) ? -par * jab : 0.0;  // target: b up, a down
            h.flip_kj[k] = (std::fabs(jba) > kTol14) ? -par * jba : 0.0;  // target: a up, b down
            h.zz[k] = jab + jba;
        }
    return ED_OK;
}

}  // namespace ed

using namespace ed;

extern "C" {

const char *ed_last_error(void) { return g_err; }

int ed_version(void) { return 100; }

int64_t ed_binom(int n, int k)
{
    binom_init();
    if (n < 0 || k < 0 || k > n || n > kMaxSites) {
        if (n > kMaxSites || n < 0) return -1;
        return 0;
    }
    return binom(n, k);
}

int ed_basis(int norb, int ne, uint32_t *out, int64_t n)
{
    clear_error();
    binom_init();
    ED_REQUIRE(norb >= 1 && norb <= kMaxSites, "norb=%d outside 1..%d", norb, kMaxSites);
    ED_REQUIRE(ne >= 0 && ne <= norb, "ne=%d outside 0..norb", ne);
    ED_REQUIRE(out != nullptr, "out is NULL");
    ED_REQUIRE(n == binom(norb, ne), "n=%lld but C(%d,%d)=%lld", (long long)n, norb, ne,
               (long long)binom(norb, ne));
    enumerate_strings(norb, ne, out, n);
    return ED_OK;
}

int64_t ed_rank(int norb, int ne, uint32_t s)
{
    binom_init();
    if (norb < 1 || norb > kMaxSites || ne < 0 || ne > norb) return -1;
    if (norb < 32 && (s >> norb)) return -1;
    if (__builtin_popcount(s) != ne) return -1;
    return rank_host(norb, s);
}

int ed_sector_create(int norb, int nup, int ndn, int kind, const double *t, const double *U,
                     const double *J, ed_sector **out)
{
    clear_error();
    binom_init();
    ED_REQUIRE(out != nullptr, "out is NULL");
    *out = nullptr;
    if (norb < 1 || norb > kMaxSites) {
        set_error("norb=%d outside 1..%d", norb, kMaxSites);
        return ED_ERR_RANGE;
    }
    ED_REQUIRE(kind == ED_HUBBARD || kind == ED_HEISENBERG, "unknown kind %d", kind);
    ED_REQUIRE(nup >= 0 && nup <= norb && ndn >= 0 && ndn <= norb,
               "particle numbers (%d,%d) outside 0..%d", nup, ndn, norb);
    int64_t nsup = binom(norb, nup), nsdn = binom(norb, ndn);
    if (nsup > INT32_MAX || nsdn > INT32_MAX) {
        set_error("a spin species has more than 2^31 strings");
        return ED_ERR_RANGE;
    }
    if (kind == ED_HEISENBERG) {
        ED_REQUIRE(J != nullptr, "Heisenberg sector needs J");
        if (ndn != 0 || nup != norb / 2) {
            set_error("Heisenberg sector is (norb/2, 0) as in the reference, got (%d,%d)", nup, ndn);
            return ED_ERR_ARG;
        }
    } else {
        ED_REQUIRE(t != nullptr && U != nullptr, "Hubbard sector needs t and U");
    }
    {
        const double *m = (kind == ED_HUBBARD) ? t : J;
        for (int i = 0; i < norb * norb; ++i)
            if (!std::isfinite(m[i])) {
                set_error("%s has a non-finite entry at %d", kind == ED_HUBBARD ? "t" : "J", i);
                return ED_ERR_ARG;
            }
        if (kind == ED_HUBBARD)
            for (int i = 0; i < norb; ++i)
                if (!std::isfinite(U[i])) { set_error("U has a non-finite entry at %d", i); return ED_ERR_ARG; }
    }
    ed_sector *s = new (std::nothrow) ed_sector();
    if (!s) { set_error("host allocation failed"); return ED_ERR_MEM; }
    s->kind = kind;
    s->norb = norb;
    s->nup = nup;
    s->ndn = ndn;
    s->nsup = nsup;
    s->nsdn = nsdn;
    s->dim = nsup * nsdn;
    cudaGetDevice(&s->device);
    int rc = build_lut(s);
    if (rc == ED_OK && kind == ED_HUBBARD) {
        for (int i = 0; i < norb * norb; ++i) {
            if (!std::isfinite(t[i])) { delete s; set_error("t has a non-finite entry at %d", i); return ED_ERR_ARG; }
            s->t_host[i] = t[i];
        }
        s->u_uniform = true;
        s->u_value = U[0];
        for (int p = 1; p <= norb; ++p) {
            if (!std::isfinite(U[p - 1])) { delete s; set_error("U has a non-finite entry at %d", p - 1); return ED_ERR_ARG; }
            s->u_site[norb - p] = U[p - 1];  // bit norb-p holds site p
            if (U[p - 1] != U[0]) s->u_uniform = false;
        }
        TablePool pool;
        HostHop hu;
        rc = build_hop_host(norb, nup, t, hu);
        if (!rc) rc = upload_hop(hu, norb, nup, s->up, pool);
        if (!rc && ndn != nup) {
            HostHop hd;
            rc = build_hop_host(norb, ndn, t, hd);
            if (!rc) rc = upload_hop(hd, norb, ndn, s->dn, pool);
        }
        if (!rc) rc = pool.commit(&s->pool);
        if (!rc && ndn == nup) {
            s->dn = s->up;      // after the commit: the copy carries the device pointers
            s->dn.owner = false;
        }
    } else if (rc == ED_OK) {
        for (int i = 0; i < norb * norb; ++i) {
            if (!std::isfinite(J[i])) { delete s; set_error("J has a non-finite entry at %d", i); return ED_ERR_ARG; }
            s->j_host[i] = J[i];
        }
        rc = build_heis(s, J);
        if (!rc) rc = heis_struct_build(s);
    }
    if (rc) {
        std::string keep = g_err;
        ed_sector_destroy(s);
        set_error("%s", keep.c_str());
        return rc;
    }
    *out = s;
    return ED_OK;
}

int ed_opspace_create(int norb, int nlist_up, const int *nups, int nlist_dn, const int *ndns, ed_opspace **out)
{
    clear_error();
    binom_init();
    ED_REQUIRE(out != nullptr, "out is NULL");
    *out = nullptr;
    ED_REQUIRE(norb >= 1 && norb <= kMaxSites, "norb=%d outside 1..%d", norb, kMaxSites);
    ED_REQUIRE(nlist_up >= 1 && nlist_up <= norb + 1 && nups != nullptr, "up-particle list of %d numbers", nlist_up);
    ED_REQUIRE(nlist_dn >= 1 && nlist_dn <= norb + 1 && ndns != nullptr, "down-particle list of %d numbers", nlist_dn);
    std::unique_ptr<ed_opspace> sp(new (std::nothrow) ed_opspace());
    if (!sp) { set_error("host allocation failed"); return ED_ERR_MEM; }
    sp->norb = norb;
    std::vector<uint32_t> strs[2];
    for (int side = 0; side < 2; ++side) {
        const int nl = side ? nlist_dn : nlist_up;
        const int *ns = side ? ndns : nups;
        int64_t *off = side ? sp->dn_off : sp->up_off;
        for (int n = 0; n <= kMaxSites; ++n) off[n] = -1;
        std::vector<uint32_t> &v = strs[side];
        for (int i = 0; i < nl; ++i) {
            const int n = ns[i];
            ED_REQUIRE(n >= 0 && n <= norb, "particle number %d outside 0..%d", n, norb);
            ED_REQUIRE(off[n] < 0, "particle number %d listed twice", n);
            const int64_t cnt = binom(norb, n);
            ED_REQUIRE((int64_t)v.size() + cnt <= INT32_MAX, "string list of more than 2^31 entries");
            off[n] = (int64_t)v.size();
            v.resize(v.size() + (size_t)cnt);
            enumerate_strings(norb, n, v.data() + off[n], cnt);
        }
    }
    sp->nsup = (int64_t)strs[0].size();
    sp->nsdn = (int64_t)strs[1].size();
    cudaGetDevice(&sp->device);
    uint32_t *lut = nullptr;
    int rc = device_lut(sp->device, &lut);
    if (rc) return rc;
    sp->lut = lut;
    TablePool pool;
    pool.add(&sp->ustr, strs[0].data(), strs[0].size());
    pool.add(&sp->dstr, strs[1].data(), strs[1].size());
    rc = pool.commit(&sp->pool);
    if (rc) return rc;
    *out = sp.release();
    return ED_OK;
}

int ed_opspace_dims(const ed_opspace *sp, int64_t *nsup, int64_t *nsdn)
{
    clear_error();
    ED_REQUIRE(sp != nullptr, "operator space is NULL");
    if (nsup) *nsup = sp->nsup;
    if (nsdn) *nsdn = sp->nsdn;
    return ED_OK;
}

int ed_opspace_destroy(ed_opspace *sp)
{
    if (!sp) return ED_OK;
    if (sp->pool) cudaFree(sp->pool);   // the rank table is shared
    delete sp;
    return ED_OK;
}

int ed_sector_destroy(ed_sector *s)
{
    if (!s) return ED_OK;
    if (s->pool) cudaFree(s->pool);   // every hop table of the sector; the rank table is shared
    heis_struct_free(s->hs);
    uijkl_free(s->uijkl);
    delete s;
    return ED_OK;
}

int ed_sector_dims(const ed_sector *s, int64_t *nsup, int64_t *nsdn, int64_t *dim)
{
    clear_error();
    ED_REQUIRE(s != nullptr, "sector is NULL");
    if (nsup) *nsup = s->nsup;
    if (nsdn) *nsdn = s->nsdn;
    if (dim) *dim = s->dim;
    return ED_OK;
}

int ed_sector_strings(const ed_sector *s, uint32_t *up, uint32_t *dn)
{
    clear_error();
    binom_init();
    ED_REQUIRE(s != nullptr, "sector is NULL");
    if (up) enumerate_strings(s->norb, s->nup, up, s->nsup);
    if (dn) enumerate_strings(s->norb, s->ndn, dn, s->nsdn);
    return ED_OK;
}

int ed_sector_nnz(const ed_sector *s, int64_t *nnz_up, int64_t *nnz_dn)
{
    clear_error();
    ED_REQUIRE(s != nullptr, "sector is NULL");
    if (nnz_up) *nnz_up = s->up.nnz;
    if (nnz_dn) *nnz_dn = s->dn.nnz;
    return ED_OK;
}

}  // extern "C"
