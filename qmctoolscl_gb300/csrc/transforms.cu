// transforms.cu -- FP64 radix-2 FFT (bit-reversed input, natural output),
// its inverse (natural input, bit-reversed output) and the Walsh-Hadamard
// transform, all orthonormal and in place along the last axis.
//
// Reference: qmctoolscl/c_funcs/fft_bro_1d_radix2.c:3-80 (decimation in
// time: stage k pairs i1, i1+2^k with twiddle tw[(i1 mod 2^k) * 2^(m-k-1)],
// tw[t] = exp(-2 pi i t/n)), ifft_bro_1d_radix2.c:3-81 (decimation in
// frequency: stage k pairs at distance 2^s, s = m-k-1, twiddle
// tw[(i1 mod 2^s) * 2^k] with the opposite sign), fwht_1d_radix2.c:3-53.
// Every stage of the reference divides by sqrt(2); here the stages are
// unscaled, run two at a time as radix-4 steps (three complex twiddle
// products per four values instead of four, half the shared-memory round
// trips), and the last pass multiplies by 2^(-m/2) once.  The results agree
// with the reference to FP64 rounding (not bit for bit).
//
// Passes.  Stages whose butterflies span the index bits [k0, k1) act on
// independent groups {h*2^k1 + q*2^k0 + c : q < 2^(k1-k0)}; a CTA loads one
// group for CT consecutive c (CT contiguous doubles per q, so loads and
// stores are coalesced runs), runs those stages in shared memory, and
// writes the tile back in place.  Up to 4096 complex (8192 real) values fit
// a tile, so lengths up to 2^12 (2^13 real) take one pass, up to 2^20 two,
// and so on.  The FFT runs the low-bit pass first, the inverse the high-bit
// pass first, matching the order of their stages.
//
// GB300 runs FP64 at about 1.25 TFLOP/s, so these kernels are FP64-bound;
// they are the plain, reference-accurate path.  The tensor-core path
// (tc_fft.cu) is the fast one.
#include <cmath>

#include "common.cuh"

namespace {

constexpr int FT_THREADS = 256;
constexpr u32 TILE_COMPLEX = 4096;
constexpr u32 TILE_REAL = 8192;

enum FtKind { FT_FFT = 0, FT_IFFT = 1, FT_FWHT = 2, FT_CONV = 3, FT_WCONV = 4 };

__global__ void twiddle_kernel(u64 n, double sign, double *twr, double *twi)
{
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (u64)gridDim.x * blockDim.x) {
        double sn, cs;
        // the angle 2*pi*t/n as a multiple of pi is exact for n a power of two
        sincospi(__ddiv_rn(__ull2double_rn(2 * t), __ull2double_rn(n)), &sn, &cs);
        twr[t] = cs;
        twi[t] = sign * sn;
    }
}

struct PassArgs {
    u64 nvec;        // d1*d2 vectors
    u32 m;           // log2 n
    u32 k0, k1;      // index bits spanned by this pass
    u32 ct;          // consecutive c values per tile
    double *xr, *xi;
    const double *twr, *twi;
    double scale;    // applied on write-back when != 1
    // the fused forms: lam (lr, li; li unused for real data), n values shared by
    // the vectors (lam_all = 0) or one per element (lam_all = 1)
    const double *lr, *li;
    u32 lam_all, divide;
    double lam_scale;
};

// the imaginary part of a twiddle; conjugated when the inverse steps read the
// forward transform's table (the fused forms fill only that one)
template <bool CONJ>
__device__ __forceinline__ double tw_im(double v) { return CONJ ? -v : v; }

// The stages of one pass on a tile in shared memory (CT consecutive c per q):
// KIND's butterflies over the index bits [a.k0, a.k1) of group h, columns
// c0 .. c0+ct-1.
template <int KIND, bool CONJ>
__device__ __forceinline__ void ft_stages(const PassArgs &a, double *sr, double *si, u64 h, u64 c0, u32 ct,
                                          u32 tile_elems)
{
    const u32 nb = tile_elems / 2;
    const u32 nbits = a.k1 - a.k0;
    // stages in pairs (radix-4 steps), a single radix-2 stage for an odd bit count: the FFT
    // and WHT go up from bit k0 (the odd stage last), the inverse down from k1-1 (the odd
    // stage last as well, at bit k0)
    for (u32 done = 0; done < nbits;) {
        const u32 w = (nbits - done >= 2) ? 2u : 1u;
        const u32 bit = (KIND == FT_IFFT) ? (a.k1 - done - w) : (a.k0 + done);  // lowest bit of the step
        const u32 hb = bit - a.k0;
        done += w;
        if (w == 2) {
            const u32 S = (1u << hb) * ct;  // member stride in the tile
            // at bit 0 every twiddle is 1: the same step without the products (a separate loop,
            // so the FP64 multiplies are skipped rather than predicated off)
            if (KIND != FT_FWHT && bit == 0) {
                for (u32 b = threadIdx.x; b < tile_elems / 4; b += FT_THREADS) {
                    const u32 p = b / ct, cc = b % ct;
                    const u32 e0 = (p << 2) * ct + cc, e1 = e0 + S, e2 = e1 + S, e3 = e2 + S;
                    const double x0r = sr[e0], x0i = si[e0], x1r = sr[e1], x1i = si[e1];
                    const double x2r = sr[e2], x2i = si[e2], x3r = sr[e3], x3i = si[e3];
                    if (KIND == FT_FFT) {
                        const double ar = x0r + x1r, ai = x0i + x1i, br = x0r - x1r, bi = x0i - x1i;
                        const double cr = x2r + x3r, ci = x2i + x3i, dr = x2r - x3r, di = x2i - x3i;
                        sr[e0] = ar + cr;
                        si[e0] = ai + ci;
                        sr[e2] = ar - cr;
                        si[e2] = ai - ci;
                        sr[e1] = br + di;
                        si[e1] = bi - dr;
                        sr[e3] = br - di;
                        si[e3] = bi + dr;
                    } else {
                        const double ar = x0r + x2r, ai = x0i + x2i, cr = x0r - x2r, ci = x0i - x2i;
                        const double br = x1r + x3r, bi = x1i + x3i, dr = x1r - x3r, di = x1i - x3i;
                        sr[e0] = ar + br;
                        si[e0] = ai + bi;
                        sr[e1] = ar - br;
                        si[e1] = ai - bi;
                        sr[e2] = cr - di;
                        si[e2] = ci + dr;
                        sr[e3] = cr + di;
                        si[e3] = ci - dr;
                    }
                }
                __syncthreads();
                continue;
            }
            for (u32 b = threadIdx.x; b < tile_elems / 4; b += FT_THREADS) {
                const u32 p = b / ct, cc = b % ct;
                const u32 q0 = ((p >> hb) << (hb + 2)) | (p & ((1u << hb) - 1));
                const u32 e0 = q0 * ct + cc, e1 = e0 + S, e2 = e1 + S, e3 = e2 + S;
                if (KIND == FT_FWHT) {
                    const double x0 = sr[e0], x1 = sr[e1], x2 = sr[e2], x3 = sr[e3];
                    const double u0 = x0 + x1, u1 = x0 - x1, u2 = x2 + x3, u3 = x2 - x3;
                    sr[e0] = u0 + u2;
                    sr[e2] = u0 - u2;
                    sr[e1] = u1 + u3;
                    sr[e3] = u1 - u3;
                    continue;
                }
                // the group's offset below bit `bit`; w = tw[c * n / 2^(bit+2)] and its powers
                const u64 i0 = (h << a.k1) + ((u64)q0 << a.k0) + c0 + cc;
                const u64 c = i0 & ((1ull << bit) - 1);
                const u32 sh = a.m - bit - 2;
                const double w1r = a.twr[c << sh], w1i = tw_im<CONJ>(a.twi[c << sh]);
                const double w2r = a.twr[c << (sh + 1)], w2i = tw_im<CONJ>(a.twi[c << (sh + 1)]);
                const double w3r = a.twr[(3 * c) << sh], w3i = tw_im<CONJ>(a.twi[(3 * c) << sh]);
                const double x0r = sr[e0], x0i = si[e0], x1r = sr[e1], x1i = si[e1];
                const double x2r = sr[e2], x2i = si[e2], x3r = sr[e3], x3i = si[e3];
                if (KIND == FT_FFT) {
                    // two decimation-in-time stages: pre-twiddles w^br(p) (br: 0, 2, 1, 3) and the
                    // 4-point DFT of the bit-reversed group
                    const double y1r = fma(x1r, w2r, -x1i * w2i), y1i = fma(x1r, w2i, x1i * w2r);
                    const double y2r = fma(x2r, w1r, -x2i * w1i), y2i = fma(x2r, w1i, x2i * w1r);
                    const double y3r = fma(x3r, w3r, -x3i * w3i), y3i = fma(x3r, w3i, x3i * w3r);
                    const double ar = x0r + y1r, ai = x0i + y1i, br = x0r - y1r, bi = x0i - y1i;
                    const double cr = y2r + y3r, ci = y2i + y3i, dr = y2r - y3r, di = y2i - y3i;
                    sr[e0] = ar + cr;
                    si[e0] = ai + ci;
                    sr[e2] = ar - cr;
                    si[e2] = ai - ci;
                    sr[e1] = br + di;  // (x0 - x1) - i (x2 - x3)
                    si[e1] = bi - dr;
                    sr[e3] = br - di;  // (x0 - x1) + i (x2 - x3)
                    si[e3] = bi + dr;
                } else {
                    // two decimation-in-frequency stages (bits bit+1, then bit): the inverse
                    // 4-point DFT and post-twiddles v^(0, 2, 1, 3) (v = the + sign twiddle)
                    const double ar = x0r + x2r, ai = x0i + x2i, cr = x0r - x2r, ci = x0i - x2i;
                    const double br = x1r + x3r, bi = x1i + x3i, dr = x1r - x3r, di = x1i - x3i;
                    sr[e0] = ar + br;
                    si[e0] = ai + bi;
                    const double z1r = ar - br, z1i = ai - bi;
                    sr[e1] = fma(z1r, w2r, -z1i * w2i);
                    si[e1] = fma(z1r, w2i, z1i * w2r);
                    const double z2r = cr - di, z2i = ci + dr;  // (x0 - x2) + i (x1 - x3)
                    sr[e2] = fma(z2r, w1r, -z2i * w1i);
                    si[e2] = fma(z2r, w1i, z2i * w1r);
                    const double z3r = cr + di, z3i = ci - dr;  // (x0 - x2) - i (x1 - x3)
                    sr[e3] = fma(z3r, w3r, -z3i * w3i);
                    si[e3] = fma(z3r, w3i, z3i * w3r);
                }
            }
            __syncthreads();
            continue;
        }
        const u32 half = 1u << hb;
        for (u32 b = threadIdx.x; b < nb; b += FT_THREADS) {
            const u32 p = b / ct, cc = b % ct;
            const u32 q1 = ((p >> hb) << (hb + 1)) | (p & (half - 1));
            const u32 e1 = q1 * ct + cc, e2 = e1 + half * ct;
            if (KIND == FT_FWHT) {
                const double x1 = sr[e1], x2 = sr[e2];
                sr[e1] = x1 + x2;
                sr[e2] = x1 - x2;
                continue;
            }
            // global index of the upper partner, for the twiddle
            const u64 i1 = (h << a.k1) + ((u64)q1 << a.k0) + c0 + cc;
            const u64 t = (i1 & ((1ull << bit) - 1)) << (a.m - bit - 1);
            const double wr = a.twr[t], wi = tw_im<CONJ>(a.twi[t]);
            const double ar = sr[e1], ai = si[e1], br = sr[e2], bi = si[e2];
            if (KIND == FT_FFT) {
                const double yr = fma(br, wr, -bi * wi), yi = fma(br, wi, bi * wr);
                sr[e1] = ar + yr;
                si[e1] = ai + yi;
                sr[e2] = ar - yr;
                si[e2] = ai - yi;
            } else {
                const double dr = ar - br, di = ai - bi;
                sr[e1] = ar + br;
                si[e1] = ai + bi;
                sr[e2] = fma(dr, wr, -di * wi);
                si[e2] = fma(dr, wi, di * wr);
            }
        }
        __syncthreads();
    }
}

// One pass of a transform on tiles of the data.  KIND: FT_FFT, FT_IFFT
// (CONJ: reading the forward table), FT_FWHT, or the fused forms of the
// highest-bit pass: FT_CONV (forward FFT steps, the pointwise product or
// quotient by lam, inverse FFT steps) and FT_WCONV (WHT steps, pointwise,
// WHT steps).
template <int KIND, bool CONJ>
__global__ void __launch_bounds__(FT_THREADS) ft_pass_kernel(PassArgs a)
{
    constexpr bool REAL = KIND == FT_FWHT || KIND == FT_WCONV;
    extern __shared__ double sm[];
    const u32 Q = 1u << (a.k1 - a.k0);
    const u32 ct = a.ct;
    const u32 tile_elems = Q * ct;
    double *sr = sm;
    double *si = sm + tile_elems;  // unused for real data
    const u64 n = 1ull << a.m;
    const u64 H = n >> a.k1;                 // groups along the high bits
    const u64 cchunks = (1ull << a.k0) / ct;  // c chunks along the low bits
    const u64 tiles_per_vec = H * cchunks;
    const u64 total_tiles = a.nvec * tiles_per_vec;
    for (u64 tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
        const u64 v = tile / tiles_per_vec, rem = tile % tiles_per_vec;
        const u64 h = rem / cchunks, c0 = (rem % cchunks) * ct;
        const u64 base = v * n + (h << a.k1) + c0;
        for (u32 e = threadIdx.x; e < tile_elems; e += FT_THREADS) {
            const u32 q = e / ct, cc = e % ct;
            const u64 gi = base + ((u64)q << a.k0) + cc;
            sr[e] = a.xr[gi];
            if (!REAL) si[e] = a.xi[gi];
        }
        __syncthreads();
        if constexpr (KIND == FT_CONV || KIND == FT_WCONV) {
            ft_stages<KIND == FT_CONV ? (int)FT_FFT : (int)FT_FWHT, false>(a, sr, si, h, c0, ct, tile_elems);
            // y <- y * lam * f or y / lam * f (f = scale / n: the orthonormal factors of both
            // transforms), lam n values shared by the vectors or one per element
            const double f = a.lam_scale;
            for (u32 e = threadIdx.x; e < tile_elems; e += FT_THREADS) {
                const u32 q = e / ct, cc = e % ct;
                const u64 gi = base + ((u64)q << a.k0) + cc;
                const u64 li = a.lam_all ? gi : (gi & (n - 1));
                const double lr = a.lr[li];
                if (REAL) {
                    sr[e] = a.divide ? sr[e] * f / lr : sr[e] * lr * f;
                } else {
                    const double lm = a.li[li], yr = sr[e] * f, yi = si[e] * f;
                    if (a.divide) {
                        const double den = fma(lr, lr, lm * lm);
                        sr[e] = fma(yr, lr, yi * lm) / den;
                        si[e] = fma(yi, lr, -yr * lm) / den;
                    } else {
                        sr[e] = fma(yr, lr, -yi * lm);
                        si[e] = fma(yr, lm, yi * lr);
                    }
                }
            }
            __syncthreads();
            ft_stages<KIND == FT_CONV ? (int)FT_IFFT : (int)FT_FWHT, KIND == FT_CONV>(a, sr, si, h, c0, ct,
                                                                                    tile_elems);
        } else {
            ft_stages<KIND, CONJ>(a, sr, si, h, c0, ct, tile_elems);
        }
        const double sc = a.scale;
        for (u32 e = threadIdx.x; e < tile_elems; e += FT_THREADS) {
            const u32 q = e / ct, cc = e % ct;
            const u64 gi = base + ((u64)q << a.k0) + cc;
            a.xr[gi] = sc != 1.0 ? sr[e] * sc : sr[e];
            if (!REAL) a.xi[gi] = sc != 1.0 ? si[e] * sc : si[e];
        }
        __syncthreads();
    }
}

struct Pass {
    u32 k0, k1, ct;
};

// Bit ranges covered by the passes, low bits first.
int plan_passes(u32 m, u32 tile, Pass *out)
{
    u32 lowbits = 0;
    while ((1u << (lowbits + 1)) <= tile) lowbits++;
    int np = 0;
    u32 k0 = 0;
    const u32 first = m < lowbits ? m : lowbits;
    out[np++] = Pass{0, first, 1};
    k0 = first;
    while (k0 < m) {
        const u32 ct = 16;  // 16 consecutive doubles = 128 bytes per run
        u32 span = 0;
        while ((ct << (span + 1)) <= tile) span++;
        const u32 k1 = (k0 + span < m) ? k0 + span : m;
        out[np++] = Pass{k0, k1, ct < (1u << k0) ? ct : (1u << k0)};
        k0 = k1;
    }
    return np;
}

template <int KIND, bool CONJ>
int launch_one(const PassArgs &a, unsigned grid, size_t smem, cudaStream_t s, const char *what)
{
    if (int rc = qmcgb::raise_smem_limit((const void *)ft_pass_kernel<KIND, CONJ>, smem, what)) return rc;
    ft_pass_kernel<KIND, CONJ><<<grid, FT_THREADS, smem, s>>>(a);
    return qmcgb::launch_status(what);
}

int launch_pass(int kind, bool conj, const PassArgs &a, unsigned grid, size_t smem, cudaStream_t s, const char *what)
{
    switch (kind) {
    case FT_FFT: return launch_one<FT_FFT, false>(a, grid, smem, s, what);
    case FT_IFFT: return conj ? launch_one<FT_IFFT, true>(a, grid, smem, s, what)
                              : launch_one<FT_IFFT, false>(a, grid, smem, s, what);
    case FT_FWHT: return launch_one<FT_FWHT, false>(a, grid, smem, s, what);
    case FT_CONV: return launch_one<FT_CONV, false>(a, grid, smem, s, what);
    default: return launch_one<FT_WCONV, false>(a, grid, smem, s, what);
    }
}

int run_transform(int kind, u64 d1, u64 d2, u64 n_half, double *twr, double *twi, double *xr, double *xi,
                  cudaStream_t s, const char *what)
{
    const u64 nvec = d1 * d2;
    QMC_REQUIRE_DOMAIN(n_half > 0 && (n_half & (n_half - 1)) == 0 && n_half <= (1ull << 40),
                       "%s: n = 2*n_half must be a power of two (n_half=%llu)", what,
                       (unsigned long long)n_half);
    const u64 n = 2 * n_half;
    u32 m = 0;
    while ((1ull << m) < n) m++;
    if (kind != FT_FWHT) {
        QMC_REQUIRE(twr && twi, "%s: null twiddle pointer", what);
        twiddle_kernel<<<qmcgb::grid_for(n, 256, (unsigned)qmcgb::sm_count() * 8), 256, 0, s>>>(
            n, kind == FT_FFT ? -1.0 : 1.0, twr, twi);
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    if (nvec == 0) return QMC_OK;
    QMC_REQUIRE(xr && (kind == FT_FWHT || xi), "%s: null data pointer", what);
    const u32 tile = kind == FT_FWHT ? TILE_REAL : TILE_COMPLEX;
    Pass passes[16];
    const int np = plan_passes(m, tile, passes);
    // orthonormal scaling 2^(-m/2), applied once by the last pass
    const double scale = (m % 2 == 0) ? ldexp(1.0, -(int)(m / 2)) : ldexp(1.0, -(int)(m / 2)) * 0.70710678118654752440;
    for (int pi = 0; pi < np; pi++) {
        const Pass p = (kind == FT_IFFT) ? passes[np - 1 - pi] : passes[pi];
        PassArgs a{};
        a.nvec = nvec;
        a.m = m;
        a.k0 = p.k0;
        a.k1 = p.k1;
        a.ct = p.ct;
        a.xr = xr;
        a.xi = xi;
        a.twr = twr;
        a.twi = twi;
        a.scale = (pi == np - 1) ? scale : 1.0;
        const u32 elems = (1u << (p.k1 - p.k0)) * p.ct;
        const size_t smem = (size_t)elems * sizeof(double) * (kind == FT_FWHT ? 1 : 2);
        const u64 tiles = nvec * (n >> p.k1) * ((1ull << p.k0) / p.ct);
        const unsigned grid = qmcgb::grid_for(tiles, 1, (unsigned)qmcgb::sm_count() * 8);
        if (int rc = launch_pass(kind, false, a, grid, smem, s, what)) return rc;
    }
    return QMC_OK;
}

// y <- IFFT(FFT(y) * lam) * scale (or / lam), or the same with the WHT for real
// data: the forward passes but the last, one fused pass over the highest bits
// (forward steps, the pointwise step, inverse steps), the inverse passes but
// the first; FP64 throughout, the orthonormal factors folded into the
// pointwise scale.  The complex form fills the caller's twiddle arrays with
// the forward table and runs the inverse steps on its conjugates.
int run_fused(int kind, u64 d1, u64 d2, u64 n_half, double *twr, double *twi, const double *lr, const double *li,
              u64 lam_all, int divide, double scale, double *xr, double *xi, cudaStream_t s, const char *what)
{
    const bool real = kind == FT_WCONV;
    const u64 nvec = d1 * d2;
    QMC_REQUIRE_DOMAIN(n_half > 0 && (n_half & (n_half - 1)) == 0 && n_half <= (1ull << 40),
                       "%s: n = 2*n_half must be a power of two (n_half=%llu)", what,
                       (unsigned long long)n_half);
    QMC_REQUIRE(lam_all <= 1, "%s: lam_all is 0 (n values for every vector) or 1 (one per element)", what);
    const u64 n = 2 * n_half;
    u32 m = 0;
    while ((1ull << m) < n) m++;
    if (!real) {
        QMC_REQUIRE(twr && twi, "%s: null twiddle pointer", what);
        twiddle_kernel<<<qmcgb::grid_for(n, 256, (unsigned)qmcgb::sm_count() * 8), 256, 0, s>>>(n, -1.0, twr, twi);
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    if (nvec == 0) return QMC_OK;
    QMC_REQUIRE(xr && lr && (real || (xi && li)), "%s: null data or lam pointer", what);
    const u32 tile = real ? TILE_REAL : TILE_COMPLEX;
    Pass passes[16];
    const int np = plan_passes(m, tile, passes);
    // launch order: forward passes 0 .. np-2, the fused pass np-1, inverse passes np-2 .. 0
    for (int li_ = 0; li_ < 2 * np - 1; li_++) {
        const int pi = li_ < np ? li_ : 2 * np - 2 - li_;
        const int k = real ? (li_ == np - 1 ? FT_WCONV : FT_FWHT)
                           : (li_ < np - 1 ? FT_FFT : li_ == np - 1 ? FT_CONV : FT_IFFT);
        const Pass p = passes[pi];
        PassArgs a{};
        a.nvec = nvec;
        a.m = m;
        a.k0 = p.k0;
        a.k1 = p.k1;
        a.ct = p.ct;
        a.xr = xr;
        a.xi = xi;
        a.twr = twr;
        a.twi = twi;
        a.scale = 1.0;
        a.lr = lr;
        a.li = li;
        a.lam_all = (u32)lam_all;
        a.divide = divide ? 1u : 0u;
        a.lam_scale = scale / (double)n;
        const u32 elems = (1u << (p.k1 - p.k0)) * p.ct;
        const size_t smem = (size_t)elems * sizeof(double) * (real ? 1 : 2);
        const u64 tiles = nvec * (n >> p.k1) * ((1ull << p.k0) / p.ct);
        const unsigned grid = qmcgb::grid_for(tiles, 1, (unsigned)qmcgb::sm_count() * 8);
        if (int rc = launch_pass(k, k == FT_IFFT, a, grid, smem, s, what)) return rc;
    }
    return QMC_OK;
}

}  // namespace

extern "C" {

int qmc_fft_bro_1d_radix2(uint64_t d1, uint64_t d2, uint64_t n_half, double *twiddler, double *twiddlei, double *xr,
                          double *xi, qmc_stream_t s)
{
    return run_transform(FT_FFT, d1, d2, n_half, twiddler, twiddlei, xr, xi, QMC_STREAM(s), "fft_bro_1d_radix2");
}

int qmc_ifft_bro_1d_radix2(uint64_t d1, uint64_t d2, uint64_t n_half, double *twiddler, double *twiddlei, double *xr,
                           double *xi, qmc_stream_t s)
{
    return run_transform(FT_IFFT, d1, d2, n_half, twiddler, twiddlei, xr, xi, QMC_STREAM(s), "ifft_bro_1d_radix2");
}

int qmc_fwht_1d_radix2(uint64_t d1, uint64_t d2, uint64_t n_half, double *x, qmc_stream_t s)
{
    return run_transform(FT_FWHT, d1, d2, n_half, nullptr, nullptr, x, nullptr, QMC_STREAM(s), "fwht_1d_radix2");
}

int qmc_fft_mul_ifft(uint64_t d1, uint64_t d2, uint64_t n_half, double *twiddler, double *twiddlei, const double *lam_r,
                     const double *lam_i, uint64_t lam_per_element, int divide, double scale, double *xr, double *xi,
                     qmc_stream_t s)
{
    return run_fused(FT_CONV, d1, d2, n_half, twiddler, twiddlei, lam_r, lam_i, lam_per_element, divide, scale, xr,
                     xi, QMC_STREAM(s), "fft_mul_ifft");
}

int qmc_fwht_mul_fwht(uint64_t d1, uint64_t d2, uint64_t n_half, const double *lam, uint64_t lam_per_element,
                      int divide, double scale, double *x, qmc_stream_t s)
{
    return run_fused(FT_WCONV, d1, d2, n_half, nullptr, nullptr, lam, nullptr, lam_per_element, divide, scale, x,
                     nullptr, QMC_STREAM(s), "fwht_mul_fwht");
}

}  // extern "C"
