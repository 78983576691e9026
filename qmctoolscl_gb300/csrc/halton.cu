// halton.cu -- fused generalized digital net (e.g. randomised Halton): for
// every dimension j with its own base b_j, digit count tmax_j and generating
// matrix (mmax_j columns), the chain
//
//   gdn_linear_matrix_scramble   qmctoolscl/c_funcs/gdn_linear_matrix_scramble.c:3-46
//   gdn_gen_natural              qmctoolscl/c_funcs/gdn_gen_natural.c:3-53
//   gdn_digital_permutation      qmctoolscl/c_funcs/gdn_digital_permutation.c:3-46
//   gdn_digital_shift            qmctoolscl/c_funcs/gdn_digital_shift.c:3-45
//   gdn_integer_to_float         qmctoolscl/c_funcs/gdn_integer_to_float.c:3-43
//
// called once per dimension (d = 1, r_b = 1, tmax_new = tmax_j: the reference
// takes one tmax per call), with the per-dimension results written into
// x[l, i, j] of one r x n x d array -- bit for bit, without ever storing a
// digit in HBM.
//
// Preparation (one kernel per plan run) packs the scrambled generating
// matrices reduced mod b (the reference's gen step reduces after every
// column; with entries of at most tmax*(b-1) no 64-bit sum wraps, so one
// reduction of reduced terms gives the same digits), the permutations and
// the shifts as 32-bit words, and 1/b^(t+1) as the reference computes it
// (repeated correctly rounded divisions).
//
// Generation: a CTA owns a tile of 32 consecutive points of one
// randomisation and all d dimensions.  Each warp takes whole dimensions
// (assigned longest-first to balance tmax_j * (mmax_j + c) work), one point
// per lane, so the 32 lanes share base, digit count and tables.  The index
// splits as hi * b^K + lo with b^K >= 32: the tile has at most two distinct
// hi, whose contributions to each output digit the lanes compute together,
// and K <= 5 low digits per lane.  Per output digit t: the digit mod b, the
// permutation gather, the shift mod b, and v = RN(v + RN(recip_t * digit)) in
// integer arithmetic on the unpacked sum (digit_sum.cuh); the FP64 unit is
// slow on this GPU and the kernel is bound by integer issue.  Once every
// remaining term is below half an ulp of v the lane stops.  The tile of
// doubles is staged in shared memory and stored as 32 contiguous rows.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "digit_sum.cuh"

namespace {

constexpr int HT_THREADS = 256;
constexpr int HT_WARPS = HT_THREADS / 32;
constexpr u32 HT_MAX_DIMS = 1024;
constexpr u32 HT_MAX_B = 2048;  // bases below 2^11: digit * recip fits the integer product

struct HDim {
    u32 b, tmax, mmax, K;  // K low digits per lane: the smallest K with b^K >= 32
    u64 c_off;     // offset of this dimension's (mmax x tmax) block inside a randomisation's C block
    u64 p_off;     // offset of its (tmax x b) permutation block inside a randomisation's block
    u64 s_off;     // offset of its tmax shifts inside a randomisation's block
    u64 fd_M;      // direct-remainder constant for b
    u64 fdK_M;     // the same for b^K
    u32 bK;
    u32 Klo;       // min(K, mmax): low digits that can be nonzero (C has mmax rows)
};

struct HPlanDev {
    u64 r, n, n_start, d;
    u64 c_per_l, p_per_l, s_per_l;  // words per randomisation
    u32 has_lms, has_perm, has_shift, pad;
    const HDim *dims;
    const u32 *C;                    // r * c_per_l: scrambled matrices mod b
    const u32 *perm;                 // r * p_per_l
    const u32 *shift;                // r * s_per_l
    const u64 *recip;                // s_per_l: bits of 1/b^(t+1), per (j, t)
    const u32 *tail;                 // s_per_l: biased exponent of RN(recip_t * (b-1)), per (j, t)
    const unsigned *flags;           // bit 0: some digit can reach b (permutation values >= b, no shift)
    const u16 *order;                // d dimension ids, warp-balanced: dims of warp w at order[wstart[w]..wstart[w+1])
    const u32 *wstart;               // HT_WARPS + 1
    double *x;
    unsigned *err;
};

// ---------------------------------------------------------------- prep

struct PrepDim {
    u64 b, tmax, mmax;
    const u64 *S, *C, *perms, *shifts;  // caller's per-dimension arrays
};

// the dimension whose block (offset `field` of HDim) holds offset off
template <typename F>
__device__ __forceinline__ u32 dim_of(const HDim *dims, u64 d, u64 off, F field)
{
    u32 lo = 0, hi = (u32)d - 1;
    while (lo < hi) {
        const u32 mid = (lo + hi + 1) >> 1;
        if (field(dims[mid]) <= off)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// one thread per (l, j, k, t) word of C, (l, j, t, c) of perms, (l, j, t) of shifts
__global__ void halton_prep_kernel(HPlanDev P, const PrepDim *pd, u64 total_c, u64 total_p, u64 total_s,
                                   u32 *C, u32 *perm, u32 *shift, unsigned *flags)
{
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 w = (u64)blockIdx.x * blockDim.x + threadIdx.x; w < total_c + total_p + total_s; w += stride) {
        if (w < total_c) {
            const u64 l = w / P.c_per_l, off = w % P.c_per_l;
            const u32 j = dim_of(P.dims, P.d, off, [](const HDim &h) { return h.c_off; });
            const HDim &D = P.dims[j];
            const u64 loc = off - D.c_off, k = loc / D.tmax, t = loc % D.tmax;
            const PrepDim &Q = pd[j];
            if (P.has_lms) {
                // gdn_linear_matrix_scramble.c:36-42 with d = 1, r_C = 1: sum_c (S[l,t,c]*C[k,c]) % b, no
                // final mod; the sum is at most tmax*(b-1) and the generation step reduces it anyway
                const u64 *srow = Q.S + (l * Q.tmax + t) * Q.tmax;
                const u64 *col = Q.C + k * Q.tmax;
                u64 acc = 0;
                for (u64 c = 0; c < Q.tmax; c++) acc += (srow[c] * col[c]) % Q.b;
                C[w] = (u32)(acc % Q.b);
            } else {
                // the generation step multiplies raw entries by digits below b in 64 bits: entries below
                // 2^32 cannot wrap, so reducing them first gives the same digits
                const u64 c = Q.C[k * Q.tmax + t];
                if (c >> 32) atomicOr(P.err, 8u);
                C[w] = (u32)(c % Q.b);
            }
        } else if (w < total_c + total_p) {
            const u64 v = w - total_c;
            const u64 l = v / P.p_per_l, off = v % P.p_per_l;
            const u32 j = dim_of(P.dims, P.d, off, [](const HDim &h) { return h.p_off; });
            const HDim &D = P.dims[j];
            const u64 loc = off - D.p_off;  // t * b + c
            const u64 val = pd[j].perms[l * D.tmax * D.b + loc];
            if (val >> 32) atomicOr(P.err, 8u);
            if (!P.has_shift && val >= D.b) atomicOr(flags, 1u);  // float digits not bounded by b-1
            perm[v] = (u32)val;
        } else {
            const u64 v = w - total_c - total_p;
            const u64 l = v / P.s_per_l, off = v % P.s_per_l;
            const u32 j = dim_of(P.dims, P.d, off, [](const HDim &h) { return h.s_off; });
            const HDim &D = P.dims[j];
            const u64 val = pd[j].shifts[l * D.tmax + (off - D.s_off)];
            if (val >> 32) atomicOr(P.err, 8u);
            shift[v] = (u32)val;
        }
    }
}

// recip_t of gdn_integer_to_float.c:34-38 for every (j, t), and the exponent
// of the largest term recip_t can contribute, RN(recip_t * (b-1))
__global__ void halton_recip_kernel(HPlanDev P, u64 *recip, u32 *tail)
{
    for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < P.d; j += (u64)gridDim.x * blockDim.x) {
        const HDim &D = P.dims[j];
        const double bd = (double)D.b;
        double rc = __ddiv_rn(1.0, bd);
        for (u32 t = 0; t < D.tmax; t++) {
            recip[D.s_off + t] = as_bits(rc);
            tail[D.s_off + t] = (u32)(as_bits(__dmul_rn(rc, (double)(D.b - 1))) >> 52);
            rc = __ddiv_rn(rc, bd);
        }
    }
}

// ---------------------------------------------------------------- generation

// RN(v + RN(rc * s)) for the terms the fast form does not take: the general
// integer routine where it is exact, else the FP64 unit (kept out of line, so
// the FP64 instructions are not if-converted into the fast path)
__device__ __noinline__ u64 halton_step_slow(u64 v, u64 rc, u32 s)
{
    if (dsum::general_ok(v, rc, s)) return dsum::add_bits(v, dsum::mul_bits(rc, s));
    return as_bits(__dadd_rn(as_double(v), __dmul_rn(as_double(rc), (double)s)));
}

// floor(x / b) and x mod b for x < 2^32, b >= 2, from M = floor((2^64-1)/b) + 1
__device__ __forceinline__ u32 hdiv(u64 M, u32 x) { return (u32)__umul64hi(M, (u64)x); }
__device__ __forceinline__ u32 hmod(u64 M, u32 b, u32 x) { return (u32)__umul64hi(M * (u64)x, (u64)b); }

// sum over the base-b digits k >= K of the index (the digits of h = index / b^K)
// of digit * C[k][t], reduced mod b
__device__ __forceinline__ u32 high_part(const HDim &D, const u32 *Cj, u32 h, u32 t)
{
    u32 acc = 0;
    for (u32 k = D.K; h && k < D.mmax; k++) {
        const u32 q = hdiv(D.fd_M, h);
        acc += (h - q * D.b) * Cj[k * D.tmax + t];  // < mmax * b^2 < 2^32
        h = q;
    }
    return hmod(D.fd_M, D.b, acc);
}

// A CTA owns 32 consecutive points of one randomisation (lane = point) and
// all d dimensions; warp w runs dimensions order[wstart[w] .. wstart[w+1]).
// Index split: itrue = hi * b^K + lo with b^K >= 32, so the tile's indices
// have at most two distinct hi (h0, h0 + 1).  Per chunk of 32 output digits
// lane c computes the high-digit sums of digit t0 + c for both, packed into
// one word, and every lane takes its own from lane t - t0 by a shuffle; the
// K <= 5 low digits are per lane.  Lanes stay converged (shuffles); a lane
// whose remaining terms are all below half an ulp of its sum idles, and the
// warp leaves the dimension when all have.
__global__ void __launch_bounds__(HT_THREADS) halton_gen_kernel(HPlanDev P)
{
    extern __shared__ __align__(16) unsigned char sm[];
    double *tile = (double *)sm;  // [32][d]
    const u32 warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const u64 tiles_per_l = (P.n + 31) / 32;
    const u64 ntiles = P.r * tiles_per_l;
    const bool early = !(*P.flags & 1u);
    for (u64 tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
        const u64 l = tt / tiles_per_l, i0 = (tt % tiles_per_l) * 32;
        const bool active = i0 + lane < P.n;  // lanes past the last point compute nothing
        const u32 base = (u32)(P.n_start + i0);
        const u32 itrue = active ? base + lane : base;  // < 2^32 (checked at plan creation)
        const u32 *Cl = P.C + l * P.c_per_l;
        const u32 *Pl = P.perm + l * P.p_per_l;
        const u32 *Sl = P.shift + l * P.s_per_l;
        for (u32 oi = P.wstart[warp]; oi < P.wstart[warp + 1]; oi++) {
            const u32 j = P.order[oi];
            const HDim D = P.dims[j];
            const u32 *Cj = Cl + D.c_off;
            const u32 *Pj = Pl + D.p_off;
            const u32 *Sj = Sl + D.s_off;
            const u64 *Rj = P.recip + D.s_off;
            const u32 *Tj = P.tail + D.s_off;
            const u32 h0 = hdiv(D.fdK_M, base);
            const u32 hi = hdiv(D.fdK_M, itrue);
            const u32 sel = (hi - h0) * 16;  // 0 or 16: which half of the packed word
            u32 dl[5];                        // low digits (zero beyond K)
            {
                u32 x = itrue - hi * D.bK;
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    const u32 q = hdiv(D.fd_M, x);
                    dl[k] = x - q * D.b;
                    x = q;
                }
            }
            bool done = !active;
            dsum::Sum v = dsum::unpack(0);  // the running sum of gdn_integer_to_float, unpacked
            for (u32 t0 = 0; t0 < D.tmax; t0 += 32) {
                if (__all_sync(0xffffffffu, done)) break;
                u32 packed = 0;
                if (t0 + lane < D.tmax)
                    packed = high_part(D, Cj, h0, t0 + lane) | (high_part(D, Cj, h0 + 1, t0 + lane) << 16);
                const u32 tend = min(D.tmax, t0 + 32);
                for (u32 t = t0; t < tend; t++) {
                    if (__all_sync(0xffffffffu, done)) break;
                    const u32 hp = (__shfl_sync(0xffffffffu, packed, t - t0) >> sel) & 0xFFFFu;
                    if (done) continue;
                    // Every later term is at most RN(recip_t*(b-1)) (recip_t only shrinks); once that
                    // lies below half an ulp of v (exponent at most exp(v) - 54), RN(v + term) = v for
                    // the remaining digits.
                    if (early && v.M && Tj[t] + 54 <= v.E) {
                        done = true;
                        continue;
                    }
                    // gdn_gen_natural.c:37-50: digit t of the point, mod b
                    u32 acc = hp;
#pragma unroll
                    for (u32 k = 0; k < 5; k++)
                        if (k < D.Klo) acc += dl[k] * Cj[k * D.tmax + t];
                    const u32 xd = hmod(D.fd_M, D.b, acc);
                    const u32 pv = P.has_perm ? Pj[t * D.b + xd] : xd;  // gdn_digital_permutation.c:36-39
                    u32 sv = pv;
                    if (P.has_shift) {                                 // gdn_digital_shift.c:37-39
                        const u64 sum = (u64)pv + Sj[t];
                        if (sum < 2ull * D.b)
                            sv = (u32)sum >= D.b ? (u32)sum - D.b : (u32)sum;
                        else
                            sv = sum < (1ull << 32) ? hmod(D.fd_M, D.b, (u32)sum) : (u32)(sum % D.b);
                    }
                    if (sv) {                                          // gdn_integer_to_float.c:35-38
                        const u64 rb = Rj[t];
                        const u32 er = (u32)(rb >> 52);
                        if (!((v.M >> 52) && sv < 2048 && er - 1u < 2035u &&
                              dsum::add_term_fast(v, (rb & dsum::FRAC) | dsum::HIDDEN, er, sv)))
                            v = dsum::unpack(halton_step_slow(dsum::pack(v), rb, sv));
                    }
                }
            }
            tile[lane * P.d + j] = as_double(dsum::pack(v));
        }
        __syncthreads();
        // 32 contiguous rows of the output
        const u64 rows = min((u64)32, P.n - i0);
        double *out = P.x + (l * P.n + i0) * P.d;
        for (u64 e = threadIdx.x; e < rows * P.d; e += HT_THREADS) __stcs(out + e, tile[e]);
        __syncthreads();
    }
}

u64 ceil_digits(u64 n_last, u64 b)
{
    u64 k = 0;
    for (u64 x = n_last; x; x /= b) k++;
    return k;
}

}  // namespace

struct qmc_halton_plan {
    HPlanDev P{};
    void *d_dims = nullptr, *d_C = nullptr, *d_perm = nullptr, *d_shift = nullptr, *d_recip = nullptr;
    void *d_order = nullptr, *d_wstart = nullptr, *d_prep = nullptr, *d_tail = nullptr, *d_flags = nullptr;
    std::vector<PrepDim> prep;
    u64 total_c = 0, total_p = 0, total_s = 0;
    size_t smem = 0;
    bool prepared = false;
};

extern "C" {

int qmc_halton_plan_create(uint64_t r, uint64_t n, uint64_t n_start, uint64_t d, const qmc_gdn_dim *dims, double *x,
                           qmc_halton_plan **plan)
{
    QMC_REQUIRE(plan && dims && x, "null argument");
    *plan = nullptr;
    QMC_REQUIRE(d >= 1 && d <= HT_MAX_DIMS && r >= 1 && n >= 1, "need 1 <= d <= %u, r >= 1, n >= 1", HT_MAX_DIMS);
    QMC_REQUIRE(n_start + n <= (1ull << 32) && n_start + n > n_start, "indices must stay below 2^32");
    const u64 smem = 32 * d * sizeof(double);
    QMC_REQUIRE(smem <= 200 * 1024, "d too large for the shared-memory output tile");
    // a step is applied when its array is given, for every dimension alike
    const bool has_lms = dims[0].S != nullptr, has_perm = dims[0].perms != nullptr,
               has_shift = dims[0].shifts != nullptr;
    qmc_halton_plan *p = new qmc_halton_plan();
    std::vector<HDim> hd(d);
    u64 c_off = 0, p_off = 0, s_off = 0;
    for (u64 j = 0; j < d; j++) {
        const qmc_gdn_dim &q = dims[j];
        const char *bad = nullptr;
        if (q.b < 2 || q.b >= HT_MAX_B) bad = "base outside [2, 2048)";
        else if (q.tmax == 0 || q.tmax > 256 || q.mmax == 0 || q.mmax > 64) bad = "tmax in [1,256] and mmax in [1,64]";
        else if (!q.C) bad = "null generating matrix";
        else if ((q.S != nullptr) != has_lms || (q.perms != nullptr) != has_perm ||
                 (q.shifts != nullptr) != has_shift)
            bad = "S, perms and shifts must be given for all dimensions or for none";
        else if (ceil_digits(n_start + n - 1, q.b) > q.mmax) bad = "mmax smaller than the base-b digits of the last index";
        if (bad) {
            delete p;
            qmcgb::set_error("dimension %llu: %s", (unsigned long long)j, bad);
            return q.b < 2 ? QMC_ERR_DOMAIN : QMC_ERR_ARG;
        }
        HDim &h = hd[j];
        h.b = (u32)q.b;
        h.tmax = (u32)q.tmax;
        h.mmax = (u32)q.mmax;
        h.c_off = c_off;
        h.p_off = p_off;
        h.s_off = s_off;
        h.fd_M = fastdiv32_make((u32)q.b).M;
        h.K = 1;
        h.bK = (u32)q.b;
        while (h.bK < 32) {
            h.bK *= (u32)q.b;
            h.K++;
        }
        h.fdK_M = fastdiv32_make(h.bK).M;
        h.Klo = std::min<u32>(h.K, (u32)q.mmax);
        c_off += q.mmax * q.tmax;
        p_off += has_perm ? q.tmax * q.b : 0;
        s_off += q.tmax;
        p->prep.push_back(PrepDim{q.b, q.tmax, q.mmax, (const u64 *)q.S, (const u64 *)q.C, (const u64 *)q.perms,
                                  (const u64 *)q.shifts});
    }
    // longest-first assignment of dimensions to the warps of a CTA
    std::vector<u32> idx(d);
    for (u32 j = 0; j < d; j++) idx[j] = j;
    auto cost = [&](u32 j) { return (double)hd[j].tmax * (hd[j].mmax * 2.0 + 40.0); };
    std::sort(idx.begin(), idx.end(), [&](u32 a, u32 b) { return cost(a) > cost(b); });
    std::vector<std::vector<u32>> per(HT_WARPS);
    std::vector<double> load(HT_WARPS, 0.0);
    for (u32 j : idx) {
        const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        per[w].push_back(j);
        load[w] += cost(j);
    }
    std::vector<u16> order;
    std::vector<u32> wstart(HT_WARPS + 1, 0);
    for (int w = 0; w < HT_WARPS; w++) {
        wstart[w] = (u32)order.size();
        for (u32 j : per[w]) order.push_back((u16)j);
    }
    wstart[HT_WARPS] = (u32)order.size();

    p->P.r = r;
    p->P.n = n;
    p->P.n_start = n_start;
    p->P.d = d;
    p->P.c_per_l = c_off;
    p->P.p_per_l = p_off;
    p->P.s_per_l = s_off;
    p->P.has_lms = has_lms;
    p->P.has_perm = has_perm;
    p->P.has_shift = has_shift;
    p->P.x = x;
    p->P.err = qmcgb::device_error_ptr();
    p->total_c = r * c_off;
    p->total_p = r * p_off;
    p->total_s = has_shift ? r * s_off : 0;
    p->smem = smem;
    int rc = 0;
    auto alloc = [&](void **dst, size_t bytes) {
        if (!rc) rc = qmcgb::cuda_status(cudaMalloc(dst, bytes ? bytes : 16), "cudaMalloc");
    };
    alloc(&p->d_dims, d * sizeof(HDim));
    alloc(&p->d_C, p->total_c * sizeof(u32));
    alloc(&p->d_perm, p->total_p * sizeof(u32));
    alloc(&p->d_shift, p->total_s * sizeof(u32));
    alloc(&p->d_recip, s_off * sizeof(u64));
    alloc(&p->d_order, d * sizeof(u16));
    alloc(&p->d_wstart, (HT_WARPS + 1) * sizeof(u32));
    alloc(&p->d_prep, d * sizeof(PrepDim));
    alloc(&p->d_tail, s_off * sizeof(u32));
    alloc(&p->d_flags, sizeof(unsigned));
    if (!rc) rc = qmcgb::cuda_status(cudaMemcpy(p->d_dims, hd.data(), d * sizeof(HDim), cudaMemcpyHostToDevice), "copy");
    if (!rc) rc = qmcgb::cuda_status(cudaMemcpy(p->d_order, order.data(), d * sizeof(u16), cudaMemcpyHostToDevice), "copy");
    if (!rc)
        rc = qmcgb::cuda_status(cudaMemcpy(p->d_wstart, wstart.data(), wstart.size() * sizeof(u32), cudaMemcpyHostToDevice),
                                "copy");
    if (!rc)
        rc = qmcgb::cuda_status(cudaMemcpy(p->d_prep, p->prep.data(), d * sizeof(PrepDim), cudaMemcpyHostToDevice), "copy");
    if (!rc && !p->P.err) rc = QMC_ERR_CUDA;
    if (!rc && smem > 48 * 1024)
        rc = qmcgb::cuda_status(cudaFuncSetAttribute(halton_gen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)smem), "cudaFuncSetAttribute");
    p->P.dims = (const HDim *)p->d_dims;
    p->P.C = (const u32 *)p->d_C;
    p->P.perm = (const u32 *)p->d_perm;
    p->P.shift = (const u32 *)p->d_shift;
    p->P.recip = (const u64 *)p->d_recip;
    p->P.order = (const u16 *)p->d_order;
    p->P.wstart = (const u32 *)p->d_wstart;
    p->P.tail = (const u32 *)p->d_tail;
    p->P.flags = (const unsigned *)p->d_flags;
    if (rc) {
        qmc_halton_plan_destroy(p);
        return rc;
    }
    *plan = p;
    return QMC_OK;
}

int qmc_halton_plan_prepare(qmc_halton_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p, "null plan");
    cudaStream_t st = QMC_STREAM(s);
    const u64 total = p->total_c + p->total_p + p->total_s;
    if (int rc = qmcgb::cuda_status(cudaMemsetAsync(p->d_flags, 0, sizeof(unsigned), st), "cudaMemsetAsync"))
        return rc;
    halton_prep_kernel<<<qmcgb::grid_for(total, 256, (unsigned)qmcgb::sm_count() * 16), 256, 0, st>>>(
        p->P, (const PrepDim *)p->d_prep, p->total_c, p->total_p, p->total_s, (u32 *)p->d_C, (u32 *)p->d_perm,
        (u32 *)p->d_shift, (unsigned *)p->d_flags);
    if (int rc = qmcgb::launch_status("halton_prep_kernel")) return rc;
    halton_recip_kernel<<<qmcgb::grid_for(p->P.d, 128, 1024), 128, 0, st>>>(p->P, (u64 *)p->d_recip,
                                                                           (u32 *)p->d_tail);
    if (int rc = qmcgb::launch_status("halton_recip_kernel")) return rc;
    p->prepared = true;
    return QMC_OK;
}

int qmc_halton_plan_run(qmc_halton_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p && p->prepared, "null or unprepared plan (call qmc_halton_plan_prepare)");
    const u64 tiles = p->P.r * ((p->P.n + 31) / 32);
    halton_gen_kernel<<<qmcgb::grid_for(tiles, 1, (unsigned)qmcgb::sm_count() * 8), HT_THREADS, p->smem,
                        QMC_STREAM(s)>>>(p->P);
    return qmcgb::launch_status("halton_gen_kernel");
}

int qmc_halton_plan_destroy(qmc_halton_plan *p)
{
    if (!p) return QMC_OK;
    for (void *q : {p->d_dims, p->d_C, p->d_perm, p->d_shift, p->d_recip, p->d_order, p->d_wstart, p->d_prep,
                    p->d_tail, p->d_flags})
        if (q) cudaFree(q);
    delete p;
    return QMC_OK;
}

}  // extern "C"
