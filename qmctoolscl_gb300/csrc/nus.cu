// nus.cu -- nested uniform (Owen) scrambling of base-2 digital nets,
// bit for bit the reference's dnb2_nested_uniform_scramble
// (qmctoolscl/rand_funcs.py:155-253) with numpy's SFC64 generator streams.
//
// The reference walks one binary tree per generator (replication l,
// dimension j), point by point, and draws random bits whenever a point opens
// a new branch.  Its output is fixed by three facts:
//   * the root starts as a leaf for a phantom point with key 0 holding
//     tmax_new random bits, drawn first (rand_funcs.py:191-195);
//   * point v then draws tmax_new - L_v - 1 bits, where L_v is the longest
//     common prefix of v's key (xb << (tmax_new - tmax), tmax_new bits) with
//     any earlier point's key -- nothing when v repeats an earlier key;
//   * bit k (from the top) of a point's scramble comes from the draw of the
//     earliest point that shares the point's first k key bits.
// So per generator (all generators at once, in chunks that fit the caller's
// workspace):
//   1. keys in point order, the phantom (or the history of earlier calls)
//      first: transposed from xb's (r_x, n, d) layout;
//   2. stable LSD radix sort of (key, point) pairs, 8 bits per pass, over
//      the top log2(N) + 4 bits or so, each run of keys equal there finished
//      by an insertion sort (all 8-bit digits when a run is long);
//   3. bottom up, in one pass, the binary radix tree over the sorted pairs
//      (Apetrei's agglomerative construction; keys extended by the point
//      index so that equal keys split too) and each internal node's earliest
//      point; the later of its two children's earliest points first shares
//      a prefix of the node's length with an earlier point, which gives
//      every L_v;
//   4. the draws, one thread per generator in point order (the only serial
//      step: numpy's SFC64 stream and its bounded-integer rule);
//   5. each node's part of the scramble (its earliest point's draw over the
//      depths the node spans) and each leaf's OR over its ancestors;
//   6. xrb = (xb << (tmax_new - tmax)) ^ scramble, transposed back.
#include "nus_dev.cuh"

namespace {

// ---- 1. keys ---------------------------------------------------------------

__global__ void nus_keys_kernel(NusDims m, const u64 *__restrict__ xb, const u64 *__restrict__ hist_keys,
                                const u64 *__restrict__ hist_draws, u64 *__restrict__ key, u64 *__restrict__ draw,
                                u64 *__restrict__ keys_out)
{
    __shared__ u64 tile[32][33];
    const u32 v0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
    for (u32 k = threadIdx.y; k < 32; k += 8) {  // lanes along generators: xb's dimension axis
        const u32 v = v0 + k, g = g0 + threadIdx.x;
        u64 kv = 0;
        if (v < m.N && g < m.S) {
            const u64 s = m.s0 + g;
            if (v < m.H0) {
                kv = m.fresh ? 0 : hist_keys[s * m.h0 + v];
            } else {
                const u64 l = s / m.d, j = s - l * m.d, i = v - m.H0;
                const u64 w = xb[((l % m.r_x) * m.n + i) * m.d + j];
                kv = (m.td >= 64 ? 0 : w << m.td) & m.mask;
            }
        }
        tile[k][threadIdx.x] = kv;
    }
    __syncthreads();
    for (u32 k = threadIdx.y; k < 32; k += 8) {  // lanes along points
        const u32 g = g0 + k, v = v0 + threadIdx.x;
        if (g < m.S && v < m.N) {
            const u64 kv = tile[threadIdx.x][k];
            key[(u64)g * m.NP + v] = kv;
            if (keys_out) keys_out[(m.s0 + g) * m.N + v] = kv;
            if (!m.fresh && v < m.H0) draw[(u64)g * m.NP + v] = hist_draws[(m.s0 + g) * m.h0 + v];
        }
    }
}


// ---- 2-3. the radix sort and the bottom-up tree pass: nus_dev.cuh -------------------

// ---- 4. the draws, one thread per generator --------------------------------------
// One thread per generator, 32 generators (rows of the draw array) per warp.  L_v
// comes in 16 at a time (one 16-byte load per group, rows start 16-byte aligned),
// three groups ahead of the draws.  A group whose 16 draws are all 64-bit draws
// (33..63 bits) or all 32-bit draws (1..32 bits), the usual case, runs unrolled
// without a branch per draw, its draws kept in registers; the warp then writes
// every such row's 128 bytes through shared memory, each 16-byte store
// instruction covering four rows' whole lines (a thread storing its own row would
// touch 32 lines per instruction).  Any other group (the first and last, repeated
// keys, mixed widths) takes the general path and stores its draws one by one.

// the top nb bits (33 <= nb <= 63) of a 64-bit output: a right shift by 64 - nb < 32
__device__ __forceinline__ u64 top_bits64(u64 x, u32 nb)
{
    const u32 sh = 64u - nb, lo = (u32)x, hi = (u32)(x >> 32);
    return ((u64)(hi >> sh) << 32) | __funnelshift_r(lo, hi, sh);
}

__device__ __forceinline__ u32 byte_of(const u32 (&w)[4], int e) { return (w[e >> 2] >> (8 * (e & 3))) & 255u; }

__device__ __forceinline__ u32 max_byte(const uint4 &c)
{
    const u32 m4 = __vmaxu4(__vmaxu4(c.x, c.y), __vmaxu4(c.z, c.w));
    return max(max(m4 & 255u, (m4 >> 8) & 255u), max((m4 >> 16) & 255u, m4 >> 24));
}

__device__ __forceinline__ u32 min_byte(const uint4 &c)
{
    const u32 m4 = __vminu4(__vminu4(c.x, c.y), __vminu4(c.z, c.w));
    return min(min(m4 & 255u, (m4 >> 8) & 255u), min((m4 >> 16) & 255u, m4 >> 24));
}

constexpr int DRAW_AHEAD = 4;

__global__ void __launch_bounds__(32) nus_draw_kernel(NusDims m, u64 *__restrict__ states,
                                                      const unsigned char *__restrict__ Lv, u64 *__restrict__ draw)
{
    // a warp's 32 rows of one group, 128 bytes each plus 16 of padding (the rows' 16-byte
    // chunks then fall in different banks)
    __shared__ uint4 stage[32][9];
    const u32 lane = threadIdx.x, g0 = blockIdx.x * 32, g = g0 + lane;
    const bool active = g < m.S;  // lanes past the last generator stay for the warp's stores
    u64 *st = states + (u64)(active ? m.s0 + g : 0) * 6;
    Sfc64 r{0, 0, 0, 0, 0, 0};
    if (active) r = Sfc64{st[0], st[1], st[2], st[3], st[5], (u32)(st[4] != 0)};
    const u64 off = (u64)(active ? g : 0) * m.NP;
    const int T = (int)m.T;
    u64 *D = draw + off;
    if (active && m.fresh) D[0] = r.bits((u32)T);
    const uint4 *L4 = reinterpret_cast<const uint4 *>(Lv + off);
    const u32 gend = (m.N + 15) >> 4;  // groups covering [0, N); NP keeps the last one in the row
    u32 gq = m.H0 >> 4;
    uint4 ring[DRAW_AHEAD];
#pragma unroll
    for (int k = 0; k < DRAW_AHEAD; k++)
        ring[k] = (active && gq + k < gend) ? L4[gq + k] : make_uint4(0, 0, 0, 0);
    for (; gq < gend; gq++) {  // the same groups in every lane
        const uint4 cur = ring[0];
#pragma unroll
        for (int k = 0; k < DRAW_AHEAD - 1; k++) ring[k] = ring[k + 1];
        ring[DRAW_AHEAD - 1] = (active && gq + DRAW_AHEAD < gend) ? L4[gq + DRAW_AHEAD] : make_uint4(0, 0, 0, 0);
        const u32 w[4] = {cur.x, cur.y, cur.z, cur.w};
        const u32 v0 = gq << 4;
        const bool inside = active && v0 >= m.H0 && v0 + 16 <= m.N;
        const int lmax = (int)max_byte(cur), lmin = (int)min_byte(cur);
        u64 y[16];
        bool staged = false;
        if (inside && lmax <= T - 34) {  // 16 draws of T-1-L in [33, 63] bits
#pragma unroll
            for (int e = 0; e < 16; e++) y[e] = top_bits64(r.next64(), (u32)(T - 1) - byte_of(w, e));
            staged = true;
        } else if (inside && lmin >= T - 33 && lmax <= T - 2) {  // 16 draws of 1..32 bits
            // a draw of nb bits is the top nb bits of a 32-bit half: numpy's buffered half first,
            // then both halves of each output, low first; the last output's high half is kept
#define NUS_SH(e) (32u - ((u32)(T - 1) - byte_of(w, (e))))
            if (r.has) {
                y[0] = (u32)r.half >> NUS_SH(0);
#pragma unroll
                for (int e = 1; e < 15; e += 2) {
                    const u64 x = r.next64();
                    y[e] = (u32)x >> NUS_SH(e);
                    y[e + 1] = (u32)(x >> 32) >> NUS_SH(e + 1);
                }
                const u64 x = r.next64();
                y[15] = (u32)x >> NUS_SH(15);
                r.half = x >> 32;
                r.has = 1;
            } else {
#pragma unroll
                for (int e = 0; e < 16; e += 2) {
                    const u64 x = r.next64();
                    y[e] = (u32)x >> NUS_SH(e);
                    y[e + 1] = (u32)(x >> 32) >> NUS_SH(e + 1);
                    r.half = x >> 32;
                }
            }
#undef NUS_SH
            staged = true;
        } else if (active) {
#pragma unroll 1
            for (int e = 0; e < 16; e++) {
                const u32 v = v0 + e;
                if (v >= m.H0 && v < m.N) {
                    const int L = (int)byte_of(w, e);
                    D[v] = r.bits(L >= T - 1 ? 0u : (u32)(T - 1 - L));
                }
            }
        }
        if (staged) {
#pragma unroll
            for (int c = 0; c < 8; c++)
                stage[lane][c] = make_uint4((u32)y[2 * c], (u32)(y[2 * c] >> 32), (u32)y[2 * c + 1],
                                            (u32)(y[2 * c + 1] >> 32));
        }
        const u32 rows = __ballot_sync(0xFFFFFFFFu, staged);
        __syncwarp();
        if (rows) {
            // store i: rows 4i .. 4i+3, eight lanes (16 bytes each) per row
            const u32 c = lane & 7;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const u32 R = 4 * i + (lane >> 3);
                if ((rows >> R) & 1u)
                    *reinterpret_cast<uint4 *>(draw + (u64)(g0 + R) * m.NP + v0 + 2 * c) = stage[R][c];
            }
        }
        __syncwarp();
    }
    if (!active) return;
    st[0] = r.a;
    st[1] = r.b;
    st[2] = r.c;
    st[3] = r.w;
    st[4] = r.has;
    st[5] = r.half;  // numpy keeps the last buffered half here, used or not
}

// ---- 5. scramble bits: each node's band, each leaf's ancestors -----------------
// A node spans the depths (parent's prefix length, own prefix length]; its
// bits there come from its earliest point's draw.  Depth k is bit T-1-k.

__device__ __forceinline__ u64 band_mask(int kmin, int kmax, int T)
{
    if (kmax > T - 1) kmax = T - 1;
    if (kmin > kmax) return 0;
    const u32 lo = (u32)(T - 1 - kmax), hi = (u32)(T - 1 - kmin);
    const u64 upto_hi = hi >= 63 ? ~0ull : ((2ull << hi) - 1ull);
    return upto_hi & ~((1ull << lo) - 1ull);
}

__global__ void __launch_bounds__(NUS_THREADS) nus_contrib_kernel(NusDims m, const unsigned char *__restrict__ lam,
                                                                  const u32 *__restrict__ pint,
                                                                  const u32 *__restrict__ minv,
                                                                  const u64 *__restrict__ draw,
                                                                  u64 *__restrict__ contrib)
{
    const u32 u = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (u + 1 >= m.N) return;
    const u64 off = (u64)g * m.NP;
    const u32 P = pint[off + u];
    const int dP = P == NONE ? -1 : (int)lam[off + P];
    const u64 mask = band_mask(dP + 1, (int)lam[off + u], (int)m.T);
    contrib[off + u] = mask ? (draw[off + minv[off + u]] & mask) : 0;
}

__global__ void __launch_bounds__(NUS_THREADS) nus_walk_kernel(NusDims m, const u32 *__restrict__ val,
                                                               const unsigned char *__restrict__ lam,
                                                               const u32 *__restrict__ pleaf,
                                                               const u32 *__restrict__ pint,
                                                               const u64 *__restrict__ contrib,
                                                               const u64 *__restrict__ draw, u64 *__restrict__ shv,
                                                               unsigned int *err)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    const u32 v = val[off + p];
    if (v < m.H0) return;  // the phantom and earlier calls' points are not output
    const u32 P = pleaf[off + p];
    const int dP = P == NONE ? -1 : (int)lam[off + P];
    u64 sh = draw[off + v] & band_mask(dP + 1, (int)m.T - 1, (int)m.T);
    int hop = 0;
    for (u32 u = P; u != NONE; u = pint[off + u]) {
        if (++hop > MAX_DEPTH) {
            atomicOr(err, 16u);
            break;
        }
        sh |= contrib[off + u];
    }
    shv[off + v] = sh;
}

// ---- 6. output, transposed back to (r, n, d) --------------------------------------

__global__ void nus_out_kernel(NusDims m, const u64 *__restrict__ xb, const u64 *__restrict__ shv,
                               u64 *__restrict__ xrb)
{
    __shared__ u64 tile[32][33];
    const u32 i0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
    for (u32 k = threadIdx.y; k < 32; k += 8) {  // lanes along points
        const u32 g = g0 + k, i = i0 + threadIdx.x;
        tile[k][threadIdx.x] = (g < m.S && i < m.n) ? shv[(u64)g * m.NP + m.H0 + i] : 0;
    }
    __syncthreads();
    for (u32 k = threadIdx.y; k < 32; k += 8) {  // lanes along generators
        const u32 g = g0 + threadIdx.x, i = i0 + k;
        if (g < m.S && i < m.n) {
            const u64 s = m.s0 + g, l = s / m.d, j = s - l * m.d;
            const u64 w = xb[((l % m.r_x) * m.n + i) * m.d + j];
            xrb[(l * m.n + i) * m.d + j] = (m.td >= 64 ? 0 : w << m.td) ^ tile[threadIdx.x][k];
        }
    }
}

// ---- workspace -------------------------------------------------------------------

inline u64 al256(u64 b) { return (b + 255) & ~255ull; }

struct NusWork {
    u64 *keyA, *keyB, *draw, *shv;
    u32 *valA, *valB, *cnt, *pleaf, *pint, *ctl;
    unsigned long long *slot;
    unsigned char *lam, *Lv;
    u64 bytes;
};

// sub-arrays for `count` generators of N entries (stride NP), 256-byte aligned
NusWork nus_layout(char *base, u64 count, u64 NP, u64 NT)
{
    NusWork w{};
    u64 off = 0;
    auto take = [&](u64 bytes) {
        char *p = base ? base + off : nullptr;
        off += al256(bytes);
        return p;
    };
    const u64 e = count * NP;
    w.keyA = (u64 *)take(e * 8);
    w.keyB = (u64 *)take(e * 8);
    w.draw = (u64 *)take(e * 8);
    w.shv = (u64 *)take(e * 8);
    w.valA = (u32 *)take(e * 4);
    w.valB = (u32 *)take(e * 4);
    w.pleaf = (u32 *)take(e * 4);
    w.pint = (u32 *)take(e * 4);
    w.slot = (unsigned long long *)take(e * 8);
    w.cnt = (u32 *)take(count * 256 * NT * 4);
    w.lam = (unsigned char *)take(e);
    w.Lv = (unsigned char *)take(e);
    w.ctl = (u32 *)take(256);
    w.bytes = off;
    return w;
}

u64 entries_of(u64 n, u64 h0) { return (h0 ? h0 : 1) + n; }
u64 padded(u64 N) { return (N + 15) & ~15ull; }
u64 tiles_of(u64 N) { return (N + WT - 1) / WT; }

}  // namespace

extern "C" {

int qmc_dnb2_nus_workspace_size(uint64_t n, uint64_t h0, uint64_t generators, uint64_t *bytes)
{
    QMC_REQUIRE(bytes, "dnb2_nus_workspace_size: null output pointer");
    const u64 N = entries_of(n, h0);
    QMC_REQUIRE(N < MAX_ENTRIES, "dnb2_nested_uniform_scramble: %llu points and earlier entries per generator "
                "(at most 2^30 - 1)", (unsigned long long)N);
    *bytes = nus_layout(nullptr, generators ? generators : 1, padded(N), tiles_of(N)).bytes;
    return QMC_OK;
}

int qmc_dnb2_nested_uniform_scramble(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t tmax,
                                     uint64_t tmax_new, uint64_t *states, uint64_t h0, const uint64_t *hist_keys,
                                     const uint64_t *hist_draws, const uint64_t *xb, uint64_t *xrb,
                                     uint64_t *keys_out, uint64_t *draws_out, void *work, uint64_t work_bytes,
                                     qmc_stream_t s)
{
    if (r == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE_DOMAIN(tmax_new <= 64, "dnb2_nested_uniform_scramble: tmax_new = %llu (t must be between 0 and 64)",
                       (unsigned long long)tmax_new);
    QMC_REQUIRE(r_x >= 1, "dnb2_nested_uniform_scramble: r_x = 0");
    QMC_REQUIRE(states && work, "dnb2_nested_uniform_scramble: null states or workspace");
    QMC_REQUIRE(n == 0 || (xb && xrb), "dnb2_nested_uniform_scramble: null xb or xrb");
    QMC_REQUIRE(h0 == 0 || (hist_keys && hist_draws), "dnb2_nested_uniform_scramble: null history arrays");
    QMC_REQUIRE(((uintptr_t)work & 255) == 0, "dnb2_nested_uniform_scramble: workspace not 256-byte aligned");
    const u64 N = entries_of(n, h0);
    QMC_REQUIRE(N < MAX_ENTRIES, "dnb2_nested_uniform_scramble: %llu points and earlier entries per generator "
                "(at most 2^30 - 1)", (unsigned long long)N);
    const u64 NP = padded(N), NT = tiles_of(N), G = r * d;
    const u64 per = nus_layout(nullptr, 1, NP, NT).bytes;
    QMC_REQUIRE(work_bytes >= per, "dnb2_nested_uniform_scramble: workspace of %llu bytes, one generator needs %llu",
                (unsigned long long)work_bytes, (unsigned long long)per);
    // the most generators whose sub-arrays fit; work_bytes / per alone comes out one short for
    // a workspace sized for exactly that many, as the fixed words count once in any layout
    const u64 cap = G < 65535 ? G : 65535;
    u64 count = work_bytes / per;
    if (count > cap) count = cap;
    while (count < cap && nus_layout(nullptr, count + 1, NP, NT).bytes <= work_bytes) count++;
    while (count > 1 && nus_layout(nullptr, count, NP, NT).bytes > work_bytes) count--;
    NusWork w = nus_layout((char *)work, count, NP, NT);
    cudaStream_t st = QMC_STREAM(s);
    const u64 *xb_ = (const u64 *)xb, *hk_ = (const u64 *)hist_keys, *hd_ = (const u64 *)hist_draws;
    u64 *xrb_ = (u64 *)xrb, *ko_ = (u64 *)keys_out, *do_ = (u64 *)draws_out, *st_ = (u64 *)states;

    NusDims m{};
    m.n = n;
    m.d = d;
    m.r_x = r_x;
    m.td = tmax_new - tmax;  // wraps when tmax > tmax_new: numpy shifts by >= 64 give 0
    m.T = (u32)tmax_new;
    m.mask = tmax_new >= 64 ? ~0ull : ((1ull << tmax_new) - 1);
    m.h0 = h0;
    m.fresh = h0 == 0;
    m.N = (u32)N;
    m.NP = (u32)NP;
    m.H0 = (u32)(h0 ? h0 : 1);
    m.NT = (u32)NT;
    const u32 passes = m.T ? (m.T + 7) / 8 : 1;
    unsigned int *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");

    for (u64 s0 = 0; s0 < G; s0 += count) {
        m.s0 = s0;
        m.S = (u32)(G - s0 < count ? G - s0 : count);
        const u64 e = (u64)m.S * NP;
        nus_keys_kernel<<<dim3((unsigned)((N + 31) / 32), (m.S + 31) / 32), dim3(32, 8), 0, st>>>(
            m, xb_, hk_, hd_, w.keyA, w.draw, ko_);
        int rc = qmcgb::launch_status("dnb2_nus keys");
        if (rc) return rc;
        const u32 *vfin = nullptr;
        const u64 *kfin = nullptr;
        u64 *kfree = nullptr;
        u32 *vfree = nullptr;
        if (n > 0) {
            const dim3 tg((unsigned)((NT + NUS_WARPS - 1) / NUS_WARPS), m.S);
            if (int rc2 = qmcgb::raise_smem_limit((const void *)nus_scatter_kernel, NUS_SCATTER_SMEM, "dnb2_nus sort"))
                return rc2;
            auto pass = [&](const u64 *kin, const u32 *vin, u32 digit, u64 *kout, u32 *vout) {
                nus_hist_kernel<<<tg, NUS_THREADS, 0, st>>>(m, kin, 8 * digit, w.cnt);
                nus_scan_kernel<<<m.S, 1024, 0, st>>>(m, w.cnt);
                nus_scatter_kernel<<<tg, NUS_THREADS, NUS_SCATTER_SMEM, st>>>(m, kin, vin, 8 * digit, w.cnt, kout, vout);
                return qmcgb::launch_status("dnb2_nus sort");
            };
            // the top digits only: enough for keys that differ in their
            // first log2(N) + 4 bits, finished by the run fixup
            const u32 need_bits = (u32)(64 - __builtin_clzll((unsigned long long)(N - 1) | 1ull)) + 4;
            const u32 top = passes < (need_bits + 7) / 8 ? passes : (need_bits + 7) / 8;
            const u64 *kin = w.keyA;
            const u32 *vin = nullptr;
            for (u32 q = 0; q < top; q++) {
                u64 *kout = (q & 1) ? w.keyA : w.keyB;
                u32 *vout = (q & 1) ? w.valA : w.valB;
                rc = pass(kin, vin, passes - top + q, kout, vout);
                if (rc) return rc;
                kin = kout;
                vin = vout;
            }
            u64 *kf = (top & 1) ? w.keyB : w.keyA, *ko = (top & 1) ? w.keyA : w.keyB;
            u32 *vf = (top & 1) ? w.valB : w.valA, *vo = (top & 1) ? w.valA : w.valB;
            if (top < passes) {
                const dim3 ng((unsigned)((N + NUS_THREADS - 1) / NUS_THREADS), m.S);
                rc = qmcgb::cuda_status(cudaMemsetAsync(w.ctl, 0, 4, st), "dnb2_nus run flag");
                if (rc) return rc;
                nus_fixup_kernel<<<ng, NUS_THREADS, 0, st>>>(m, 8 * (passes - top), kf, vf, w.ctl);
                u32 longrun = 0;
                rc = qmcgb::cuda_status(cudaMemcpyAsync(&longrun, w.ctl, 4, cudaMemcpyDeviceToHost, st),
                                        "dnb2_nus run flag");
                if (rc) return rc;
                rc = qmcgb::cuda_status(cudaStreamSynchronize(st), "dnb2_nus run flag");
                if (rc) return rc;
                if (longrun) {  // every digit, from point order, ending in kf / vf
                    nus_unsort_kernel<<<ng, NUS_THREADS, 0, st>>>(m, kf, vf, w.shv);
                    const u64 *ki = w.shv;
                    const u32 *vi = nullptr;
                    for (u32 q = 0; q < passes; q++) {
                        const bool to_f = ((passes - 1 - q) & 1) == 0;
                        rc = pass(ki, vi, q, to_f ? kf : ko, to_f ? vf : vo);
                        if (rc) return rc;
                        ki = to_f ? kf : ko;
                        vi = to_f ? vf : vo;
                    }
                }
            }
            kfin = kf;
            vfin = vf;
            kfree = ko;
            vfree = vo;
            const dim3 ng((unsigned)((N + NUS_THREADS - 1) / NUS_THREADS), m.S);
            nus_lcp_kernel<<<ng, NUS_THREADS, 0, st>>>(m, kfin, vfin, w.lam);
            rc = qmcgb::cuda_status(cudaMemsetAsync(w.slot, 0xFF, e * 8, st), "dnb2_nus slots");
            if (rc) return rc;
            nus_build_kernel<<<ng, NUS_THREADS, 0, st>>>(m, vfin, w.lam, w.slot, w.pleaf, w.pint, vfree, w.Lv, err);
            rc = qmcgb::launch_status("dnb2_nus tree");
            if (rc) return rc;
        }
        nus_draw_kernel<<<(m.S + 31) / 32, 32, 0, st>>>(m, st_, w.Lv, w.draw);
        rc = qmcgb::launch_status("dnb2_nus draws");
        if (rc) return rc;
        if (draws_out) {
            rc = qmcgb::cuda_status(cudaMemcpy2DAsync(do_ + s0 * N, N * 8, w.draw, NP * 8, N * 8, m.S,
                                                      cudaMemcpyDeviceToDevice, st),
                                    "dnb2_nus draws out");
            if (rc) return rc;
        }
        if (n > 0) {
            const dim3 ng((unsigned)((N + NUS_THREADS - 1) / NUS_THREADS), m.S);
            u64 *contrib = kfree;
            nus_contrib_kernel<<<ng, NUS_THREADS, 0, st>>>(m, w.lam, w.pint, vfree, w.draw, contrib);
            nus_walk_kernel<<<ng, NUS_THREADS, 0, st>>>(m, vfin, w.lam, w.pleaf, w.pint, contrib, w.draw, w.shv, err);
            nus_out_kernel<<<dim3((unsigned)((n + 31) / 32), (m.S + 31) / 32), dim3(32, 8), 0, st>>>(m, xb_, w.shv, xrb_);
            rc = qmcgb::launch_status("dnb2_nus scramble");
            if (rc) return rc;
        }
    }
    return QMC_OK;
}

}  // extern "C"
