// tc_fft.cu -- tensor-core (tcgen05, BF16 in / FP32 accumulate) paths of
// the fast transforms.
#include "fpconv.cuh"
#include "tc_sm100.cuh"
#include <type_traits>

namespace {
constexpr u32 WAIT_LIMIT = 1u << 22;  // mbarrier polls before giving up (~ a fraction of a second)
}  // namespace

// ===========================================================================
// Tensor-core FFT / inverse FFT / Walsh-Hadamard transform.
//
// Same contract as the FP64 transforms (transforms.cu): orthonormal, in place
// along the last axis of d1*d2 vectors of length n = 2^L, FFT input in
// bit-reversed order and output natural, the inverse the other way round,
// FP64 arrays in HBM.  Arithmetic is FP32 with BF16 tensor-core products;
// the error against the FP64 transform is about 1e-7 relative (tests bound
// it by 1e-6).
//
// Passes.  As in transforms.cu, each pass covers a range of index bits
// [k0, k1) on tiles of 4096 values: pass 1 bits [0, min(L,12)) on contiguous
// blocks (several short vectors per tile), pass 2 bits [12, L) on tiles of
// Q = 2^(L-12) rows by 4096/Q consecutive columns.  The FFT runs pass 1
// first, the inverse pass 2 first.  Between the passes of a complex
// transform the data stay FP32: element f's (re, im) pair is written into the
// eight bytes of xr[f], which only the tile holding f reads or writes, and the
// last pass writes FP64 xr and xi again.
//
// Radix-16 step.  The reference's radix-2 stages k..k+3 on bit-reversed
// input, fused, act on groups of 16 values at positions base + p*2^k
// (p < 16, base with bits k..k+3 clear): with c = base mod 2^k and
// w = exp(-2*pi*i*c/2^(k+4)),
//     Y[m] = sum_p (X[p] * w^br(p)) * exp(-2*pi*i*br(p)*m/16),   br = 4-bit reversal,
// written back to base + m*2^k.  The inverse step applies the conjugate
// 16-point matrix first and the conjugate twiddle w^-br(q) after; the WHT
// step is the 16-point Hadamard matrix with no twiddle.
//
// GEMM.  The 256 groups of a tile form two M = 128 tiles.  A group's 16
// complex inputs are 32 reals; each is split into three BF16 terms
// x = x1 + x2 + x3 (24 significant bits), and so is each entry of the real
// 32 x 32 form of the 16-point matrix.  A holds x1 | x2 | x3 and B
// m1 | m2 | m3 along K; the six products with i + j <= 4 (x1m1, x1m2, x2m1,
// x1m3, x2m2, x3m1) are 12 tcgen05.mma of M=128, N=32, K=16 over the matching
// slices (FP32 accumulation in tensor memory), the step for 128 groups.  The tensor core's accumulation does
// not round to nearest, and chaining all twelve MMAs into one accumulator
// measured about 1e-6 error per step; so the two MMAs of the dominant x1*m1
// product each get their own accumulator and the ten small products a third,
// and the three are added in FP32 (round to nearest) when read back.  Bits
// left over when a pass does not cover a multiple of 4 use FP32 radix-2
// butterflies.
// ===========================================================================

namespace {

constexpr u32 FT_TILE = 4096;          // complex values per tile
constexpr u32 FT_GROUPS = FT_TILE / 16;
constexpr u32 FT_KS = 96;              // K of the operands: 3 splits x 32 reals
constexpr u32 FT_THREADS = 256;
constexpr u32 TMEM_COLS = 128;         // three 32-column FP32 accumulators
constexpr u32 FT_PAD = FT_TILE + FT_TILE / 16;  // shared-memory words per component, padded
// CONV: FFT steps, pointwise, IFFT steps; WCONV: WHT steps, pointwise (real), WHT steps
enum TcKind { TC_FFT = 0, TC_IFFT = 1, TC_WHT = 2, TC_CONV = 3, TC_WCONV = 4 };

// Shared-memory slot of tile element e: one padding word per 16, so that the
// 32 groups a warp handles (16 consecutive elements apart in the first step)
// fall in distinct banks.
__device__ __forceinline__ u32 slot(u32 e) { return e + (e >> 4); }

// FP64 <-> FP32 at every load and store, in integer arithmetic (fpconv.cuh);
// the rare values outside its fast range go through the hardware conversion
__device__ __noinline__ float f64_to_f32_hw(double x) { return __double2float_rn(x); }
__device__ __noinline__ double f32_to_f64_hw(float x) { return (double)x; }

__device__ __forceinline__ float to_f32(u64 b)
{
    u32 o;
    return fpc::f64_to_f32_bits(b, o) ? __uint_as_float(o) : f64_to_f32_hw(__longlong_as_double((long long)b));
}

__device__ __forceinline__ double to_f64(float v)
{
    u64 o;
    return fpc::f32_to_f64_bits(__float_as_uint(v), o) ? __longlong_as_double((long long)o) : f32_to_f64_hw(v);
}

// The same conversions on the FP64 unit or in integer arithmetic (the same bits either way).  The
// passes are bound by instruction issue and leave the FP64 pipe idle, so half the loads' and
// stores' rounds (chosen the same in every lane of a warp) convert there: none 14.64 ms for the
// 4096-vector bench, half 14.40, three quarters 14.43, all 14.56
__device__ __forceinline__ float to_f32_on(u64 b, bool fp64_unit)
{
    return fp64_unit ? __double2float_rn(__longlong_as_double((long long)b)) : to_f32(b);
}

__device__ __forceinline__ double to_f64_on(float v, bool fp64_unit) { return fp64_unit ? (double)v : to_f64(v); }

struct TcPassArgs {
    u64 total;       // nvec * n values
    u32 L;           // log2 n
    u32 k0, k1;      // index bits of this pass
    u32 ct;          // consecutive columns per tile row (1 for pass 1)
    u32 Q;           // tile rows
    double *xr, *xi;
    float scale;     // applied on write-back when != 1
    u32 in32, out32; // the pass reads / writes the FP32 intermediate instead of the FP64 arrays
    // TC_CONV: between the forward and the inverse steps, y <- y * lam * lam_scale (or
    // y / lam * lam_scale with divide); lam is n values shared by all vectors (lam_all = 0) or
    // one per element (lam_all = 1)
    const double *lr, *li;
    u32 lam_all, divide;
    float lam_scale;
};

__device__ __forceinline__ u32 brev4(u32 p) { return __brev(p) >> 28; }

// x = a + b + c, each the RN BF16 of what is left (about 24 significant bits in all)
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &a, __nv_bfloat16 &b, __nv_bfloat16 &c)
{
    a = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(a);
    b = __float2bfloat16_rn(r1);
    c = __float2bfloat16_rn(r1 - __bfloat162float(b));
}

// which split of the data (first) and of the matrix (second) product j uses
__device__ __forceinline__ u32 prod_a(u32 j) { return j == 0 ? 0u : j == 1 ? 0u : j == 2 ? 1u : j == 3 ? 0u : j == 4 ? 1u : 2u; }
__device__ __forceinline__ u32 prod_b(u32 j) { return j == 0 ? 0u : j == 1 ? 1u : j == 2 ? 0u : j == 3 ? 2u : j == 4 ? 1u : 0u; }

// real 32 x 32 form of the 16-point step matrix: row kk = input real index
// (0..15 real parts of input member p, 16..31 imaginary parts), column n =
// output real index (0..15 real, 16..31 imaginary parts of output member m)
template <int KIND>
__device__ __forceinline__ float step_matrix(u32 kk, u32 n)
{
    const u32 p = kk & 15, m = n & 15;
    if (KIND == TC_WHT) {  // real data: only the 16 x 16 block is used
        return (__popc(p & m) & 1) ? -1.0f : 1.0f;
    }
    // forward: F[p][m] = exp(-2 pi i br(p) m / 16); inverse: G[m'][q] with input
    // member p and output member m: exp(+2 pi i br(m) p / 16)
    const u32 e = (KIND == TC_FFT) ? (brev4(p) * m) & 15 : (brev4(m) * p) & 15;
    float s, c;
    sincospif((float)e / 8.0f, &s, &c);
    if (KIND == TC_FFT) s = -s;
    const bool in_im = kk >= 16, out_im = n >= 16;
    if (!in_im && !out_im) return c;   // Re(x) Re(F)
    if (in_im && !out_im) return -s;   // -Im(x) Im(F)
    if (!in_im && out_im) return s;    // Re(x) Im(F)
    return c;                          // Im(x) Re(F)
}

// Twiddle exp(sign * 2 pi i * t / 2^bits) in FP32, t < 2^bits, bits <= 32,
// from a table of exp(-2 pi i r / 4096), r < 1024 (one quarter turn, filled
// once per CTA with sincospif): the angle as a 32-bit fraction of a turn J
// splits into the quarter J >> 30, the table index (J >> 20) mod 1024, and,
// when bits > 12, a remainder below 2 pi / 4096 whose sine and cosine are
// two-term series (the next terms are below 2^-40).
// twiddle_turn takes the angle J / 2^32 of a turn directly (J = t << (32 - bits)).
//
// The table is stored swizzled: entry r at tab_slot(r), its low four bits
// XORed with bits 4-7 and 8-11.  A warp's lookups are often r = s * c for a
// power-of-two stride s (a step's groups differ in c); with 8-byte entries
// unswizzled, strides of 16 or more put them all in one bank pair.
__device__ __forceinline__ u32 tab_slot(u32 r) { return r ^ (((r >> 4) ^ (r >> 8)) & 15u); }

__device__ __forceinline__ void twiddle_turn(const float2 *tab, u32 J, u32 bits, float sign, float &wr, float &wi)
{
    const float2 e = tab[tab_slot((J >> 20) & 1023u)];  // (cos, -sin) of 2 pi r / 4096
    float c = e.x, sn = e.y;
    const u32 quarter = J >> 30;              // times (-i)^quarter
    if (quarter & 1u) {
        const float tmp = c;
        c = sn;
        sn = -tmp;
    }
    if (quarter & 2u) {
        c = -c;
        sn = -sn;
    }
    if (bits > 12) {
        const float th = __uint2float_rn(J & 0xFFFFFu) * 1.4629180792671596e-09f;  // 2 pi / 2^32
        const float th2 = th * th;
        const float ct = fmaf(-0.5f, th2, 1.0f), st = th * fmaf(th2, -0.16666667f, 1.0f);
        const float nc = c * ct + sn * st;  // (c + i sn) * (ct - i st)
        sn = sn * ct - c * st;
        c = nc;
    }
    wr = c;
    wi = sign < 0.0f ? sn : -sn;
}

__device__ __forceinline__ void twiddle(const float2 *tab, u32 t, u32 bits, float sign, float &wr, float &wi)
{
    twiddle_turn(tab, t << (32 - bits), bits, sign, wr, wi);
}

__device__ __forceinline__ void cmul(float ar, float ai, float br, float bi, float &cr, float &ci)
{
    cr = ar * br - ai * bi;
    ci = ar * bi + ai * br;
}

// Twiddles of one half of a radix-16 group: member pp (pp < 8) of half h has br = h + 2j with
// j = brev3(pp), so its twiddle is T_j = u W^j with u = w^h and W = w^2, w = exp(sign 2 pi i c / 2^bits)
// (cg = c << (32 - bits), the angle of w as a fraction of a turn).  Table lookups give W, T_5 and, on
// the upper half, T_1 (T_1 = W on the lower one); the member pair (j, j + 4), that is pp and pp + 1,
// then takes T_j = T_1 f_j and T_(j+4) = T_5 f_j with f_j = conj(W), 1, W, W^2 for j = 0..3.  Every
// twiddle is a lookup times at most a square of one, so the angle error of a looked-up value is
// carried at most twice (powers W^4 and up would carry it four times and more: about 3.5 times the
// error per twiddle).
struct HalfTwiddles {
    float t1r, t1i, t5r, t5i, wr, wi, w2r, w2i;
};

__device__ __forceinline__ HalfTwiddles half_twiddles(const float2 *tab, u32 cg, u32 half, u32 bits, float sign)
{
    HalfTwiddles t;
    twiddle_turn(tab, 2u * cg, bits, sign, t.wr, t.wi);
    if (half) {
        twiddle_turn(tab, 3u * cg, bits, sign, t.t1r, t.t1i);
        twiddle_turn(tab, 11u * cg, bits, sign, t.t5r, t.t5i);
    } else {  // T_1 = W
        t.t1r = t.wr;
        t.t1i = t.wi;
        twiddle_turn(tab, 10u * cg, bits, sign, t.t5r, t.t5i);
    }
    cmul(t.wr, t.wi, t.wr, t.wi, t.w2r, t.w2i);
    return t;
}

// the twiddles of members j and j + 4 (j < 4, known at compile time after unrolling)
__device__ __forceinline__ void pair_twiddles(const HalfTwiddles &t, u32 j, float &ar, float &ai, float &br, float &bi)
{
    if (j == 1) {
        ar = t.t1r;
        ai = t.t1i;
        br = t.t5r;
        bi = t.t5i;
        return;
    }
    const float fr = j == 3 ? t.w2r : t.wr, fi = j == 0 ? -t.wi : j == 3 ? t.w2i : t.wi;
    cmul(t.t1r, t.t1i, fr, fi, ar, ai);
    cmul(t.t5r, t.t5i, fr, fi, br, bi);
}

// bytes [p, p + bytes) of global memory into L2 by the bulk-copy unit (p 16-byte aligned, bytes a
// multiple of 16); the issuing thread does not wait for it
__device__ __forceinline__ void prefetch_l2(const void *p, u32 bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((u64)__cvta_generic_to_global(p)), "r"(bytes)
                 : "memory");
}

// The split step matrices of the forward and the inverse FFT in operand-B layout, for the
// fused pass that runs both kinds of step on one tile (filled by tc_stepB_kernel on the
// caller's stream before every fused transform: the same values each time)
constexpr u32 FT_B_WORDS = 32 * FT_KS * 2 / 16;  // 16-byte words per matrix
__device__ uint4 g_stepB[2][FT_B_WORDS];

__global__ void tc_stepB_kernel()
{
    for (u32 e = threadIdx.x; e < 2 * 32 * FT_KS; e += blockDim.x) {
        const u32 which = e / (32 * FT_KS), r = e % (32 * FT_KS);
        const u32 n = r / FT_KS, rest = r % FT_KS, z = rest / 32, kk = rest % 32;
        __nv_bfloat16 m[3];
        split3(which ? step_matrix<TC_IFFT>(kk, n) : step_matrix<TC_FFT>(kk, n), m[0], m[1], m[2]);
        *(__nv_bfloat16 *)((unsigned char *)g_stepB[which] + tc::kmajor_offset(n, z * 32 + kk, FT_KS)) = m[z];
    }
}

template <int KIND>
__global__ void __launch_bounds__(FT_THREADS, 3) tc_pass_kernel(TcPassArgs a, unsigned *err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    float *sr = (float *)sm;                            // [FT_PAD] real parts (slot(e))
    float *si = sr + FT_PAD;                            // [FT_PAD] imaginary parts
    unsigned char *sA = (unsigned char *)(si + FT_PAD);   // [128 x FT_KS] bf16 operand A: x1 | x2 | x3
    unsigned char *sB = sA + 128 * FT_KS * 2;           // [32 x FT_KS]  bf16 operand B: m1 | m2 | m3
    float2 *tab = (float2 *)(sB + 32 * FT_KS * 2);      // [1024] exp(-2 pi i r / 4096)
    __shared__ __align__(8) u64 bar;
    __shared__ u32 tmem_base;
    constexpr bool REAL = KIND == TC_WHT || KIND == TC_WCONV;
    const u32 warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const u32 NOUT = REAL ? 16u : 32u;      // GEMM N
    const u32 KIN = REAL ? 16u : 32u;       // reals per group and split

    if (warp == 0) tc::tmem_alloc(&tmem_base, TMEM_COLS);
    // operand B: the split step matrix, B[n][KIN*z + kk] = m_z[kk][n] (z = 0, 1, 2)
    for (u32 e = threadIdx.x; e < NOUT * 3 * KIN; e += FT_THREADS) {
        const u32 n = e / (3 * KIN), rest = e % (3 * KIN), z = rest / KIN, kk = rest % KIN;
        __nv_bfloat16 m[3];
        split3(step_matrix<KIND == TC_CONV ? (int)TC_FFT : REAL ? (int)TC_WHT : KIND>(kk, n), m[0], m[1], m[2]);
        *(__nv_bfloat16 *)(sB + tc::kmajor_offset(n, z * KIN + kk, 3 * KIN)) = m[z];
    }
    for (u32 r = threadIdx.x; r < 1024; r += FT_THREADS) {
        float sn, c;
        sincospif((float)r / 2048.0f, &sn, &c);
        tab[tab_slot(r)] = make_float2(c, -sn);
    }
    if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const u32 tmem = tmem_base;
    const u32 KTOT = 3 * KIN;
    const u32 idesc = tc::idesc_bf16_f32(128, NOUT);
    const u32 sbo = (KTOT / 8) * 128;
    u32 phase = 0;
    bool ok = true;

    const u32 Q = a.Q, ct = a.ct;
    // ct, the column and row chunk counts and n are powers of two: index math by shifts
    const u32 ctl = 31 - __clz(ct), ctm = ct - 1;
    const u32 cchl = (a.k0 == 0) ? 0 : a.k0 - ctl;       // log2 column chunks: 2^k0 / ct
    const u32 tpvl = (a.k0 == 0) ? 0 : cchl + (a.L - a.k1);  // log2 tiles per vector
    const u64 ntiles = (a.k0 == 0) ? (a.total + FT_TILE - 1) / FT_TILE : (a.total >> a.L) << tpvl;
    // first element of tile t: pass 1 a block of 4096; later passes Q rows 2^k0 apart of ct
    // consecutive elements
    auto tile_base = [&](u64 t) -> u64 {
        if (a.k0 == 0) return t * FT_TILE;
        const u64 v = t >> tpvl, rem = t & ((1ull << tpvl) - 1);
        return (v << a.L) + ((rem >> cchl) << a.k1) + ((rem & ((1ull << cchl) - 1)) << ctl);
    };
    // tile t's input into L2 while the CTA works on the tile before it, so that the load phase
    // waits on L2 rather than HBM: pass 1 one block per array (an even count of elements from a
    // multiple of 4096), later passes one row of ct (even) elements per thread (Q <= 256 rows);
    // the FP32 intermediate is xr's bytes alone
    auto prefetch_tile = [&](u64 t) {
        if (t >= ntiles) return;
        const u64 b0 = tile_base(t);
        const bool both = !REAL && !a.in32;
        if (a.k0 == 0) {
            if (threadIdx.x == 0) {
                const u32 bytes = (u32)(a.total - b0 < FT_TILE ? a.total - b0 : FT_TILE) * 8;
                prefetch_l2(a.xr + b0, bytes);
                if (both) prefetch_l2(a.xi + b0, bytes);
            }
        } else if (threadIdx.x < Q) {
            const u64 f = b0 + ((u64)threadIdx.x << a.k0);
            prefetch_l2(a.xr + f, ct * 8);
            if (both) prefetch_l2(a.xi + f, ct * 8);
        }
    };
    prefetch_tile(blockIdx.x);

    for (u64 tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const u64 base = tile_base(tile);
        // load (zeros beyond the data): pairs of adjacent elements as 16-byte loads, all of a
        // thread's raw bits in flight before the conversions (whose rare out-of-line fallback
        // would otherwise serialise the loads).  Q * ct is even and ct is 1 (pass 1) or even,
        // so a pair never straddles two rows; a.total is a multiple of n >= 2.
        if (!REAL && a.in32) {
            // the FP32 intermediate of the previous pass: element f's (re, im) in the 8 bytes of xr[f]
            constexpr u32 PAIRS = FT_TILE / (2 * FT_THREADS);  // 8
            float4 b[PAIRS];
#pragma unroll
            for (u32 i = 0; i < PAIRS; i++) {
                const u32 e = 2 * (threadIdx.x + i * FT_THREADS);
                const u64 f = base + ((u64)(e >> ctl) << a.k0) + (e & ctm);
                b[i] = (e < Q * ct && f < a.total) ? *(const float4 *)(a.xr + f) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (u32 i = 0; i < PAIRS; i++) {
                const u32 e = 2 * (threadIdx.x + i * FT_THREADS);
                if (e < Q * ct) {
                    sr[slot(e)] = b[i].x;
                    si[slot(e)] = b[i].y;
                    sr[slot(e + 1)] = b[i].z;
                    si[slot(e + 1)] = b[i].w;
                }
            }
        } else {
            constexpr u32 PAIRS = FT_TILE / (2 * FT_THREADS);  // 8
            ulonglong2 br[PAIRS], bi[PAIRS];
#pragma unroll
            for (u32 i = 0; i < PAIRS; i++) {
                const u32 e = 2 * (threadIdx.x + i * FT_THREADS);
                const u64 f = base + ((u64)(e >> ctl) << a.k0) + (e & ctm);
                const bool in = e < Q * ct && f < a.total;
                br[i] = in ? *(const ulonglong2 *)(a.xr + f) : make_ulonglong2(0, 0);
                bi[i] = (in && !REAL) ? *(const ulonglong2 *)(a.xi + f) : make_ulonglong2(0, 0);
            }
#pragma unroll
            for (u32 i = 0; i < PAIRS; i++) {
                const u32 e = 2 * (threadIdx.x + i * FT_THREADS);
                if (e < Q * ct) {
                    const bool hw = (i & 1u) == 0;  // even rounds on the FP64 unit
                    sr[slot(e)] = to_f32_on(br[i].x, hw);
                    sr[slot(e + 1)] = to_f32_on(br[i].y, hw);
                    if (!REAL) {
                        si[slot(e)] = to_f32_on(bi[i].x, hw);
                        si[slot(e + 1)] = to_f32_on(bi[i].y, hw);
                    }
                }
            }
        }
        __syncthreads();
        prefetch_tile(tile + gridDim.x);
        // the steps over the pass's bits for step kind SK (FFT, IFFT or WHT): false when a wait ran out
        auto steps = [&](auto skc) -> bool {
            constexpr int SK = decltype(skc)::value;
            // steps over the pass's bits: FFT/WHT low to high, inverse high to low
            const u32 nb = a.k1 - a.k0;
            const u32 n16 = nb / 4, nrem = nb % 4;
            for (u32 st = 0; st < n16 + nrem; st++) {
                // step st covers bits [lo, lo + w) of the pass (w = 4 or 1)
                u32 lo, w;
                if (SK == TC_IFFT) {  // remainder radix-2 bits first (highest), then radix-16 downward
                    if (st < nrem) { lo = nb - 1 - st; w = 1; }
                    else { lo = (n16 - 1 - (st - nrem)) * 4; w = 4; }
                } else {
                    if (st < n16) { lo = st * 4; w = 4; }
                    else { lo = n16 * 4 + (st - n16); w = 1; }
                }
                const u32 k = a.k0 + lo;  // global bit of the step
                if (w == 1) {
                    // FP32 radix-2 butterflies on bit k (as the reference's stage)
                    for (u32 b = threadIdx.x; b < Q * ct / 2; b += FT_THREADS) {
                        const u32 cc = b & ctm, pq = b >> ctl;
                        const u32 q1 = ((pq >> lo) << (lo + 1)) | (pq & ((1u << lo) - 1));
                        const u32 e1 = slot(q1 * ct + cc), e2 = slot(q1 * ct + cc + (1u << lo) * ct);
                        if (SK == TC_WHT) {
                            const float x1 = sr[e1], x2 = sr[e2];
                            sr[e1] = x1 + x2;
                            sr[e2] = x1 - x2;
                            continue;
                        }
                        const u32 f1 = (u32)base + (q1 << a.k0) + cc;  // only its low k bits are used
                        float wr, wi;
                        twiddle(tab, f1 & ((1u << k) - 1), k + 1, SK == TC_FFT ? -1.0f : 1.0f, wr, wi);
                        const float ar = sr[e1], ai = si[e1], br = sr[e2], bi = si[e2];
                        if (SK == TC_FFT) {
                            const float yr = br * wr - bi * wi, yi = br * wi + bi * wr;
                            sr[e1] = ar + yr; si[e1] = ai + yi; sr[e2] = ar - yr; si[e2] = ai - yi;
                        } else {
                            const float dr = ar - br, di = ai - bi;
                            sr[e1] = ar + br; si[e1] = ai + bi;
                            sr[e2] = dr * wr - di * wi; si[e2] = dr * wi + di * wr;
                        }
                    }
                    __syncthreads();
                    continue;
                }
                // radix-16 step through the tensor cores, two M-tiles of 128 groups
                for (u32 mt = 0; mt < FT_GROUPS / 128 && ok; mt++) {
                    // build A: thread t handles group 128*mt + t%128, members 8*(t/128) .. +7 at
                    // elements e0 + pp*S; the eight members' BF16 terms of one product sit side by
                    // side along K (one 16-byte row of a core matrix): one 16-byte store per (product,
                    // component).  Members are split two at a time with packed BF16x2 conversions.
                    {
                        const u32 gi = 128 * mt + (threadIdx.x & 127), half = threadIdx.x >> 7;
                        const u32 cc = gi & ctm, qq = gi >> ctl;
                        const u32 qlo = qq & ((1u << lo) - 1), qhi = qq >> lo;
                        const u32 row = threadIdx.x & 127;
                        const u32 S = (1u << lo) * ct;
                        const u32 e0 = (qlo | (qhi << (lo + 4))) * ct + cc + half * 8 * S;
                        // the group's offset below bit k, the same for all its members; member
                        // half*8 + p (p < 8) has br = 2*brev3(p) + half, so its twiddle angle as a
                        // fraction of a turn is J = cg*half + 2*cg*brev3(p) with cg = c << (28 - k)
                        const u32 cgrp = ((u32)base + (qlo << a.k0) + cc) & ((1u << k) - 1);
                        const u32 cg = cgrp << (28 - k);
                        u32 pr[3][4], pim[3][4];  // [split][pair of members]: two BF16 per word
                        // members pp, pp+1 (pp even) have j = brev3(pp) < 4 and j + 4
                        HalfTwiddles tw{};
                        if (SK == TC_FFT && k > 0) tw = half_twiddles(tab, cg, half, k + 4, -1.0f);
#pragma unroll
                        for (u32 pp = 0; pp < 8; pp += 2) {
                            float xr2[2], xi2[2], pwr[2] = {1.0f, 1.0f}, pwi[2] = {0.0f, 0.0f};
                            const u32 jj = ((pp >> 1) & 1u) * 2u + ((pp >> 2) & 1u);  // brev3(pp)
                            if (SK == TC_FFT && k > 0) pair_twiddles(tw, jj, pwr[0], pwi[0], pwr[1], pwi[1]);
#pragma unroll
                            for (u32 h = 0; h < 2; h++) {
                                const u32 e = slot(e0 + (pp + h) * S);
                                xr2[h] = sr[e];
                                xi2[h] = (SK == TC_WHT) ? 0.0f : si[e];
                                if (SK == TC_FFT && k > 0) {  // pre-twiddle w^br(p) (w = 1 on the first step)
                                    const float wr = pwr[h], wi = pwi[h];
                                    const float tr = xr2[h] * wr - xi2[h] * wi;
                                    xi2[h] = xr2[h] * wi + xi2[h] * wr;
                                    xr2[h] = tr;
                                }
                            }
                            // x = x1 + x2 + x3, each RN to BF16 of what is left
                            float ar = xr2[0], br = xr2[1], ai = xi2[0], bi = xi2[1];
#pragma unroll
                            for (u32 z = 0; z < 3; z++) {
                                const __nv_bfloat162 hr = __floats2bfloat162_rn(ar, br);
                                pr[z][pp >> 1] = *(const u32 *)&hr;
                                ar -= __low2float(hr);
                                br -= __high2float(hr);
                                if (SK != TC_WHT) {
                                    const __nv_bfloat162 hi = __floats2bfloat162_rn(ai, bi);
                                    pim[z][pp >> 1] = *(const u32 *)&hi;
                                    ai -= __low2float(hi);
                                    bi -= __high2float(hi);
                                }
                            }
                        }
#pragma unroll
                        for (u32 z = 0; z < 3; z++) {
                            *(uint4 *)(sA + tc::kmajor_offset(row, z * KIN + half * 8, KTOT)) =
                                make_uint4(pr[z][0], pr[z][1], pr[z][2], pr[z][3]);
                            if (SK != TC_WHT)
                                *(uint4 *)(sA + tc::kmajor_offset(row, z * KIN + 16 + half * 8, KTOT)) =
                                    make_uint4(pim[z][0], pim[z][1], pim[z][2], pim[z][3]);
                        }
                    }
                    tc::fence_smem_to_async();
                    tc::fence_before_sync();
                    __syncthreads();
                    tc::fence_after_sync();
                    if (threadIdx.x == 0) {
                        // the six products x_za * m_zb with za + zb <= 2, each KIN/16 MMAs of K = 16 over
                        // the matching slices of A and B; accumulators: D0, D1 the two K-slices of
                        // x1*m1 (one MMA each), D2 the products about 2^-8 smaller; summed in FP32 on
                        // read-back
                        const u32 kin16 = KIN / 16;  // MMAs per product: 2 (FFT), 1 (WHT)
                        u32 issued = 0;
                        for (u32 j = 0; j < 6; j++) {
                            const u32 za = prod_a(j), zb = prod_b(j);
                            for (u32 sl = 0; sl < kin16; sl++) {
                                const u32 dst = j == 0 ? 32u * sl : 64u;
                                const u32 acc = j == 0 ? 0u : (issued > kin16 ? 1u : 0u);
                                tc::mma_bf16(tmem + dst, tc::smem_desc(sA + (za * kin16 + sl) * 256, 128, sbo),
                                             tc::smem_desc(sB + (zb * kin16 + sl) * 256, 128, sbo), idesc, acc);
                                issued++;
                            }
                        }
                        tc::mma_commit(&bar);
                    }
                    ok = __syncthreads_and(tc::mbar_wait(&bar, phase, WAIT_LIMIT) ? 1 : 0);
                    phase ^= 1;
                    tc::fence_after_sync();
                    if (!ok) break;
                    // read back: warps 0-3 the real outputs, warps 4-7 the imaginary ones
                    {
                        const u32 gi = 128 * mt + 32 * (warp & 3) + lane;
                        const u32 cc = gi & ctm, qq = gi >> ctl;
                        const u32 qlo = qq & ((1u << lo) - 1), qhi = qq >> lo;
                        const u32 S = (1u << lo) * ct;
                        const u32 e0 = (qlo | (qhi << (lo + 4))) * ct + cc;
                        const u32 col0 = (SK == TC_WHT) ? 0u : 16u * (warp >> 2);
                        if (SK != TC_WHT || warp < 4) {
                            const u32 lanes = (32 * (warp & 3)) << 16;
                            u32 v0[16], v1[16], v2[16];
                            tc::tmem_ld16(tmem + lanes + col0, v0);
                            if (SK != TC_WHT) tc::tmem_ld16(tmem + lanes + 32 + col0, v1);
                            tc::tmem_ld16(tmem + lanes + 64 + col0, v2);
                            tc::tmem_wait_ld();
                            float *dst = (SK == TC_WHT || warp < 4) ? sr : si;
#pragma unroll
                            for (u32 m = 0; m < 16; m++) {
                                float y = __uint_as_float(v0[m]);
                                if (SK != TC_WHT) y += __uint_as_float(v1[m]);
                                y += __uint_as_float(v2[m]);
                                dst[slot(e0 + m * S)] = y;
                            }
                        }
                    }
                    // the next M-tile's operand build reads only its own groups' elements, and its
                    // MMAs (which overwrite the accumulators read here) start after the barrier that
                    // follows the build: only the last M-tile of a step, and the inverse step's
                    // post-twiddle (other threads' outputs), need a barrier here
                    if (SK == TC_IFFT || mt + 1 == FT_GROUPS / 128) {
                        tc::fence_before_sync();
                        __syncthreads();
                    }
                    if (SK == TC_IFFT) {
                        // post-twiddle w^-br(q) of the inverse step
                        const u32 gi = 128 * mt + (threadIdx.x & 127), half = threadIdx.x >> 7;
                        const u32 cc = gi & ctm, qq = gi >> ctl;
                        const u32 qlo = qq & ((1u << lo) - 1), qhi = qq >> lo;
                        const u32 S = (1u << lo) * ct;
                        const u32 e0 = (qlo | (qhi << (lo + 4))) * ct + cc + half * 8 * S;
                        const u32 cgrp = ((u32)base + (qlo << a.k0) + cc) & ((1u << k) - 1);
                        const u32 cg = cgrp << (28 - k);
                        if (k > 0) {
                            const HalfTwiddles tw = half_twiddles(tab, cg, half, k + 4, 1.0f);  // as in the forward step
#pragma unroll
                            for (u32 pp = 0; pp < 8; pp += 2) {
                                const u32 jj = ((pp >> 1) & 1u) * 2u + ((pp >> 2) & 1u);  // brev3(pp)
                                float pwr[2], pwi[2];
                                pair_twiddles(tw, jj, pwr[0], pwi[0], pwr[1], pwi[1]);
#pragma unroll
                                for (u32 h = 0; h < 2; h++) {
                                    const u32 e = slot(e0 + (pp + h) * S);
                                    const float wr = pwr[h], wi = pwi[h];
                                    const float xr_ = sr[e], xi_ = si[e];
                                    sr[e] = xr_ * wr - xi_ * wi;
                                    si[e] = xr_ * wi + xi_ * wr;
                                }
                            }
                        }
                        __syncthreads();
                    }
                }
                if (!ok) return false;
            }
            return true;
        };
        if constexpr (KIND == TC_CONV) {
            ok = steps(std::integral_constant<int, TC_FFT>{});
            if (ok) {
                // y <- y * lam * s or y / lam * s at the forward transform's output positions f
                for (u32 e = threadIdx.x; e < Q * ct; e += FT_THREADS) {
                    const u64 f = base + ((u64)(e >> ctl) << a.k0) + (e & ctm);
                    if (f >= a.total) continue;
                    const u64 li_ = a.lam_all ? f : (f & ((1ull << a.L) - 1));
                    const float lr = to_f32((u64)__double_as_longlong(a.lr[li_]));
                    const float lm = to_f32((u64)__double_as_longlong(a.li[li_]));
                    const u32 sl = slot(e);
                    const float yr = sr[sl], yi = si[sl];
                    if (a.divide) {
                        const float q = __fdiv_rn(a.lam_scale, fmaf(lr, lr, lm * lm));
                        sr[sl] = (yr * lr + yi * lm) * q;
                        si[sl] = (yi * lr - yr * lm) * q;
                    } else {
                        sr[sl] = (yr * lr - yi * lm) * a.lam_scale;
                        si[sl] = (yr * lm + yi * lr) * a.lam_scale;
                    }
                }
                // operand B: the inverse step matrix for the inverse steps, then the forward one again
                for (u32 i = threadIdx.x; i < FT_B_WORDS; i += FT_THREADS) ((uint4 *)sB)[i] = g_stepB[1][i];
                tc::fence_smem_to_async();
                __syncthreads();
                ok = steps(std::integral_constant<int, TC_IFFT>{});
                for (u32 i = threadIdx.x; i < FT_B_WORDS; i += FT_THREADS) ((uint4 *)sB)[i] = g_stepB[0][i];
                tc::fence_smem_to_async();
                __syncthreads();
            }
        } else if constexpr (KIND == TC_WCONV) {
            ok = steps(std::integral_constant<int, TC_WHT>{});
            if (ok) {
                // y <- y * lam * s or y / lam * s (real lam), then the same WHT steps again
                for (u32 e = threadIdx.x; e < Q * ct; e += FT_THREADS) {
                    const u64 f = base + ((u64)(e >> ctl) << a.k0) + (e & ctm);
                    if (f >= a.total) continue;
                    const u64 li_ = a.lam_all ? f : (f & ((1ull << a.L) - 1));
                    const float lr = to_f32((u64)__double_as_longlong(a.lr[li_]));
                    const u32 sl = slot(e);
                    sr[sl] = a.divide ? sr[sl] * __fdiv_rn(a.lam_scale, lr) : sr[sl] * lr * a.lam_scale;
                }
                __syncthreads();
                ok = steps(std::integral_constant<int, TC_WHT>{});
            }
        } else {
            ok = steps(std::integral_constant<int, KIND>{});
        }
        if (!ok) break;
        // store, pairs of adjacent elements as 16-byte stores
        for (u32 e = 2 * threadIdx.x; e < Q * ct; e += 2 * FT_THREADS) {
            const u64 f = base + ((u64)(e >> ctl) << a.k0) + (e & ctm);
            if (!REAL && a.out32) {
                // FP32 intermediate for the next pass, in the bytes of this tile's own xr elements
                if (f < a.total)
                    *(float4 *)(a.xr + f) = make_float4(sr[slot(e)], si[slot(e)], sr[slot(e + 1)], si[slot(e + 1)]);
            } else if (f < a.total) {
                static_assert(2 * FT_THREADS == 512, "the store loop's round is e >> 9");
                const bool hw = ((e >> 9) & 1u) == 0;  // the loop's round, the same in a warp: even ones on FP64
                *(double2 *)(a.xr + f) =
                    make_double2(to_f64_on(sr[slot(e)] * a.scale, hw), to_f64_on(sr[slot(e + 1)] * a.scale, hw));
                if (!REAL)
                    *(double2 *)(a.xi + f) =
                        make_double2(to_f64_on(si[slot(e)] * a.scale, hw), to_f64_on(si[slot(e + 1)] * a.scale, hw));
            }
        }
        __syncthreads();
    }
    if (!ok && threadIdx.x == 0) atomicOr(err, 4u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// CTAs of a pass: 3 fit on an SM; a long pass takes up to 8 waves of them (24 per SM) as long as
// every CTA still gets about 16 tiles -- later waves start as earlier CTAs finish, which
// shortens the tail and spreads the CTAs' load phases (measured: 2^20-length transforms 4-5 %
// faster), while short passes keep one wave and their setup per CTA small
unsigned tc_grid(u64 tiles)
{
    const u64 sms = (u64)qmcgb::sm_count();
    u64 g = tiles / 16;
    if (g > sms * 24) g = sms * 24;
    g = g / (sms * 3) * (sms * 3);  // whole waves of 3 CTAs per SM
    if (g < sms * 3) g = sms * 3;
    if (g > tiles) g = tiles;
    return (unsigned)(g ? g : 1);
}

int run_tc(int kind, u64 d1, u64 d2, u64 n_half, double *xr, double *xi, cudaStream_t s, const char *what)
{
    QMC_REQUIRE_DOMAIN(n_half > 0 && (n_half & (n_half - 1)) == 0 && n_half <= (1ull << 23),
                       "%s: n = 2*n_half must be a power of two up to 2^24", what);
    const u64 nvec = d1 * d2, n = 2 * n_half;
    if (nvec == 0) return QMC_OK;
    QMC_REQUIRE(xr && (kind == TC_WHT || xi), "%s: null data pointer", what);
    QMC_REQUIRE((((uintptr_t)xr | (uintptr_t)xi) & 15) == 0, "%s: data arrays must be 16-byte aligned", what);
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    u32 L = 0;
    while ((1ull << L) < n) L++;
    // passes: bits [0, min(L,12)), then chunks of at most 8 bits
    struct P { u32 k0, k1; } passes[8];
    int np = 0;
    passes[np++] = {0, L < 12 ? L : 12};
    for (u32 k0 = 12; k0 < L; k0 += 8) passes[np++] = {k0, (k0 + 8 < L) ? k0 + 8 : L};
    const size_t smem = FT_PAD * 8 + 128 * FT_KS * 2 + 32 * FT_KS * 2 + 1024 * 8;
    const float scale = (float)(1.0 / sqrt((double)n));
    for (int pi = 0; pi < np; pi++) {
        const P p = (kind == TC_IFFT) ? passes[np - 1 - pi] : passes[pi];
        TcPassArgs A;
        A.total = nvec * n;
        A.L = L;
        A.k0 = p.k0;
        A.k1 = p.k1;
        if (p.k0 == 0) {
            A.Q = FT_TILE;
            A.ct = 1;
        } else {
            A.Q = 1u << (p.k1 - p.k0);
            A.ct = FT_TILE / A.Q;
            if ((1ull << p.k0) < A.ct) A.ct = (u32)(1ull << p.k0);
        }
        A.xr = xr;
        A.xi = xi;
        A.scale = (pi == np - 1) ? scale : 1.0f;
        // between passes the complex transform keeps FP32 (re, im) pairs in xr's bytes: a
        // quarter less traffic than FP64 arrays and no conversions; the values are the FP32
        // ones the FP64 round trip would restore exactly
        A.in32 = (kind != TC_WHT && pi > 0) ? 1u : 0u;
        A.out32 = (kind != TC_WHT && pi < np - 1) ? 1u : 0u;
        const u64 tiles = (p.k0 == 0) ? (A.total + FT_TILE - 1) / FT_TILE : A.total / (A.Q * (u64)A.ct);
        const unsigned grid = tc_grid(tiles);
        if (kind == TC_FFT) {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_FFT>, smem, what)) return rc;
            tc_pass_kernel<TC_FFT><<<grid, FT_THREADS, smem, s>>>(A, err);
        } else if (kind == TC_IFFT) {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_IFFT>, smem, what)) return rc;
            tc_pass_kernel<TC_IFFT><<<grid, FT_THREADS, smem, s>>>(A, err);
        } else {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_WHT>, smem, what)) return rc;
            tc_pass_kernel<TC_WHT><<<grid, FT_THREADS, smem, s>>>(A, err);
        }
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    return QMC_OK;
}

// y <- IFFT(FFT(y) * lam) * scale, or with / lam: the forward passes but the last, one fused
// pass over the highest bits (forward steps, the pointwise operation, inverse steps), the
// inverse passes but the first; FP32 intermediates throughout, the orthonormal factors 1/n
// folded into the pointwise scale
int run_conv(bool real, u64 d1, u64 d2, u64 n_half, const double *lr, const double *li, u64 lam_all, int divide,
             double scale, double *xr, double *xi, cudaStream_t s, const char *what)
{
    QMC_REQUIRE_DOMAIN(n_half > 0 && (n_half & (n_half - 1)) == 0 && n_half <= (1ull << 23),
                       "%s: n = 2*n_half must be a power of two up to 2^24", what);
    const u64 nvec = d1 * d2, n = 2 * n_half;
    if (nvec == 0) return QMC_OK;
    QMC_REQUIRE(xr && lr && (real || (xi && li)), "%s: null data pointer", what);
    QMC_REQUIRE(lam_all <= 1, "%s: lam_all is 0 (n values for every vector) or 1 (one per element)", what);
    QMC_REQUIRE((((uintptr_t)xr | (uintptr_t)xi) & 15) == 0, "%s: data arrays must be 16-byte aligned", what);
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    u32 L = 0;
    while ((1ull << L) < n) L++;
    struct P { u32 k0, k1; } passes[8];
    int np = 0;
    passes[np++] = {0, L < 12 ? L : 12};
    for (u32 k0 = 12; k0 < L; k0 += 8) passes[np++] = {k0, (k0 + 8 < L) ? k0 + 8 : L};
    const size_t smem = FT_PAD * 8 + 128 * FT_KS * 2 + 32 * FT_KS * 2 + 1024 * 8;
    if (!real) {
        tc_stepB_kernel<<<1, FT_THREADS, 0, s>>>();
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    // launch order: forward passes 0 .. np-2, the fused pass np-1, inverse passes np-2 .. 0
    for (int li_ = 0; li_ < 2 * np - 1; li_++) {
        const int pi = li_ < np ? li_ : 2 * np - 2 - li_;
        const int kind = real ? (li_ == np - 1 ? TC_WCONV : TC_WHT)
                              : (li_ < np - 1 ? TC_FFT : li_ == np - 1 ? TC_CONV : TC_IFFT);
        const P p = passes[pi];
        TcPassArgs A{};
        A.total = nvec * n;
        A.L = L;
        A.k0 = p.k0;
        A.k1 = p.k1;
        if (p.k0 == 0) {
            A.Q = FT_TILE;
            A.ct = 1;
        } else {
            A.Q = 1u << (p.k1 - p.k0);
            A.ct = FT_TILE / A.Q;
            if ((1ull << p.k0) < A.ct) A.ct = (u32)(1ull << p.k0);
        }
        A.xr = xr;
        A.xi = xi;
        A.scale = 1.0f;
        A.in32 = (!real && li_ > 0) ? 1u : 0u;
        A.out32 = (!real && li_ < 2 * np - 2) ? 1u : 0u;
        A.lr = lr;
        A.li = li;
        A.lam_all = (u32)lam_all;
        A.divide = divide ? 1u : 0u;
        A.lam_scale = (float)(scale / (double)n);
        const u64 tiles = (p.k0 == 0) ? (A.total + FT_TILE - 1) / FT_TILE : A.total / (A.Q * (u64)A.ct);
        const unsigned grid = tc_grid(tiles);
        if (kind == TC_FFT) {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_FFT>, smem, what)) return rc;
            tc_pass_kernel<TC_FFT><<<grid, FT_THREADS, smem, s>>>(A, err);
        } else if (kind == TC_IFFT) {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_IFFT>, smem, what)) return rc;
            tc_pass_kernel<TC_IFFT><<<grid, FT_THREADS, smem, s>>>(A, err);
        } else if (kind == TC_WHT) {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_WHT>, smem, what)) return rc;
            tc_pass_kernel<TC_WHT><<<grid, FT_THREADS, smem, s>>>(A, err);
        } else if (kind == TC_WCONV) {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_WCONV>, smem, what)) return rc;
            tc_pass_kernel<TC_WCONV><<<grid, FT_THREADS, smem, s>>>(A, err);
        } else {
            if (int rc = qmcgb::raise_smem_limit((const void *)tc_pass_kernel<TC_CONV>, smem, what)) return rc;
            tc_pass_kernel<TC_CONV><<<grid, FT_THREADS, smem, s>>>(A, err);
        }
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    return QMC_OK;
}

}  // namespace

extern "C" {

int qmc_tc_fft_mul_ifft(uint64_t d1, uint64_t d2, uint64_t n_half, const double *lam_r, const double *lam_i,
                        uint64_t lam_per_element, int divide, double scale, double *xr, double *xi, qmc_stream_t s)
{
    return run_conv(false, d1, d2, n_half, lam_r, lam_i, lam_per_element, divide, scale, xr, xi, QMC_STREAM(s),
                    "tc_fft_mul_ifft");
}

int qmc_tc_fwht_mul_fwht(uint64_t d1, uint64_t d2, uint64_t n_half, const double *lam, uint64_t lam_per_element,
                         int divide, double scale, double *x, qmc_stream_t s)
{
    return run_conv(true, d1, d2, n_half, lam, nullptr, lam_per_element, divide, scale, x, nullptr, QMC_STREAM(s),
                    "tc_fwht_mul_fwht");
}

int qmc_tc_fft_bro_1d(uint64_t d1, uint64_t d2, uint64_t n_half, double *xr, double *xi, qmc_stream_t s)
{
    return run_tc(TC_FFT, d1, d2, n_half, xr, xi, QMC_STREAM(s), "tc_fft_bro_1d");
}

int qmc_tc_ifft_bro_1d(uint64_t d1, uint64_t d2, uint64_t n_half, double *xr, double *xi, qmc_stream_t s)
{
    return run_tc(TC_IFFT, d1, d2, n_half, xr, xi, QMC_STREAM(s), "tc_ifft_bro_1d");
}

int qmc_tc_fwht_1d(uint64_t d1, uint64_t d2, uint64_t n_half, double *x, qmc_stream_t s)
{
    return run_tc(TC_WHT, d1, d2, n_half, x, nullptr, QMC_STREAM(s), "tc_fwht_1d");
}

}  // extern "C"
