// gdn_nus.cu -- nested uniform (Owen) scrambling of generalized (base-b)
// digital nets, bit for bit the reference's gdn_nested_uniform_scramble
// (qmctoolscl/rand_funcs.py:255-356) with numpy's SFC64 generator streams.
//
// The reference walks one b-ary tree per generator (replication l,
// dimension j) point by point; a node holds a permutation of the digits
// 0..b-1 for its level, and a point that opens a branch draws one
// permutation (numpy's Generator.permutation(b)) for every level below it.
// As for base 2 (nus.cu), the output is fixed by three facts:
//   * the root starts as a leaf for a phantom point of zero digits holding
//     tmax_new permutations, drawn first (rand_funcs.py:318-322);
//   * point v draws tmax_new - L_v - 1 permutations, where L_v is the longest
//     common prefix, in digits (zero beyond tmax), of v with any earlier
//     point -- none when v repeats an earlier point;
//   * digit t of a point's result is perm[x_t], perm being the level-t
//     permutation of the earliest point that shares the point's first t
//     digits.
// So per generator: the digits packed w = ceil(log2 b) bits each into
// 128-bit keys (MSB first); the stable radix sort of nus_dev.cuh on the high
// word, finished by an insertion sort of runs on the full key; the prefix
// lengths of sorted neighbours in bits; the bottom-up tree pass of
// nus_dev.cuh (bit-level L; the digit L is L / w); per point the number of
// permutations it draws and their offsets; the draws, one CTA per generator
// (the swap indices of numpy's Fisher-Yates from the stream, fy_stream.cuh),
// then the swaps themselves, one thread per permutation; each point's digits
// through its owners' permutations, level by level on the way up its
// ancestors.
#include "fy_stream.cuh"
#include "nus_dev.cuh"

#include <vector>

namespace {

struct GdnArgs {
    const u64 *bases;
    u64 r_b;
    u32 tmax, tmax_new;
    const u64 *hist_keys;  // (r*d, H0, 2) keys (high, low word) of the trees' earlier entries, or null
};

// base b and bits per digit w of generator s
__device__ __forceinline__ void gdn_base_of(const NusDims &m, const GdnArgs &a, u64 s, u32 &b, u32 &w)
{
    const u64 l = s / m.d, j = s - l * m.d;
    const u64 bb = a.bases[(l % a.r_b) * m.d + j];
    b = (u32)bb;
    w = bb <= 2 ? 1u : (u32)(64 - __clzll((long long)(bb - 1)));
}

// ---- keys: the digits packed MSB first into 128 bits -------------------------------

__global__ void __launch_bounds__(NUS_THREADS) gdn_keys_kernel(NusDims m, GdnArgs a, const u64 *__restrict__ xdig,
                                                               u64 *__restrict__ key, u64 *__restrict__ khi_idx,
                                                               u64 *__restrict__ klo_idx, unsigned int *err)
{
    const u32 v = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (v >= m.N) return;
    const u64 s = m.s0 + g;
    u32 b, w;
    gdn_base_of(m, a, s, b, w);
    u64 hi = 0, lo = 0;
    if (v < m.H0) {  // an entry of an earlier call (the phantom root is entry 0, key 0)
        if (a.hist_keys) {
            const u64 *hk = a.hist_keys + (s * m.H0 + v) * 2;
            hi = hk[0];
            lo = hk[1];
        }
    } else {
        if ((u64)a.tmax * w > 128 || b == 0 || b > 65536) atomicOr(err, 1u);
        const u64 l = s / m.d, j = s - l * m.d, i = v - m.H0;
        const u64 *x = xdig + (((l % m.r_x) * m.n + i) * m.d + j) * a.tmax;
        for (u32 t = 0; t < a.tmax && (t + 1) * w <= 128; t++) {
            u64 dg = x[t];
            if (dg >= b) {  // the reference indexes a permutation with it and raises IndexError
                atomicOr(err, 1u);
                dg = 0;
            }
            const u32 sh = 128 - (t + 1) * w;  // the digit's lowest bit
            if (sh >= 64) {
                hi |= dg << (sh - 64);
            } else {
                lo |= dg << sh;
                if (sh + w > 64) hi |= dg >> (64 - sh);
            }
        }
    }
    const u64 off = (u64)g * m.NP;
    key[off + v] = hi;
    khi_idx[off + v] = hi;
    klo_idx[off + v] = lo;
}

// every entry's key (point order) for a later call on the same trees
__global__ void __launch_bounds__(NUS_THREADS) gdn_keys_out_kernel(NusDims m, const u64 *__restrict__ khi_idx,
                                                                   const u64 *__restrict__ klo_idx,
                                                                   u64 *__restrict__ keys_out)
{
    const u32 v = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (v >= m.N) return;
    const u64 off = (u64)g * m.NP;
    u64 *o = keys_out + ((m.s0 + g) * m.N + v) * 2;
    o[0] = khi_idx[off + v];
    o[1] = klo_idx[off + v];
}

// ---- sort finish: runs equal in the sorted top bits, by the full 128-bit key ----------

__device__ __forceinline__ bool key_less(u64 ah, u64 al, u64 bh, u64 bl) { return ah < bh || (ah == bh && al < bl); }

__global__ void __launch_bounds__(NUS_THREADS) gdn_fixup_kernel(NusDims m, u32 lowbits, u64 *key, u32 *val,
                                                                const u64 *__restrict__ klo_idx, u32 *longrun)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    u64 *k = key + off;
    u32 *v = val + off;
    const u64 *klo = klo_idx + off;
    const u64 top = k[p] >> lowbits;
    if (p > 0 && (k[p - 1] >> lowbits) == top) return;
    if (p + 1 >= m.N || (k[p + 1] >> lowbits) != top) return;
    u32 e = p + 2;
    while (e < m.N && e - p <= RUN_MAX && (k[e] >> lowbits) == top) e++;
    if (e - p > RUN_MAX) {  // a long run is fine only if every key in it is the same (already in point order)
        const u64 h0 = k[p], l0 = klo[v[p]];
        for (u32 q = p + 1; q < m.N && (k[q] >> lowbits) == top; q++)
            if (k[q] != h0 || klo[v[q]] != l0) {
                atomicOr(longrun, 1u);
                return;
            }
        return;
    }
    for (u32 x = p + 1; x < e; x++) {
        const u64 kh = k[x];
        const u32 y = v[x];
        const u64 kl = klo[y];
        u32 c = x;
        while (c > p && key_less(kh, kl, k[c - 1], klo[v[c - 1]])) {
            k[c] = k[c - 1];
            v[c] = v[c - 1];
            c--;
        }
        k[c] = kh;
        v[c] = y;
    }
}

__global__ void __launch_bounds__(NUS_THREADS) gdn_gather_kernel(NusDims m, const u32 *__restrict__ val,
                                                                 const u64 *__restrict__ src, u64 *__restrict__ dst)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    dst[off + p] = src[off + val[off + p]];
}

// ---- prefix lengths (bits) of sorted neighbours, extended by the point index -----------

__global__ void __launch_bounds__(NUS_THREADS) gdn_lcp_kernel(NusDims m, GdnArgs a, const u64 *__restrict__ key,
                                                              const u32 *__restrict__ val,
                                                              const u64 *__restrict__ klo_idx,
                                                              unsigned char *__restrict__ lam)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p + 1 >= m.N) return;
    const u64 off = (u64)g * m.NP;
    u32 b, w;
    gdn_base_of(m, a, m.s0 + g, b, w);
    const u32 va = val[off + p], vb = val[off + p + 1];
    const u64 xh = key[off + p] ^ key[off + p + 1];
    int dl;
    if (xh) {
        dl = __clzll((long long)xh);
    } else {
        const u64 xl = klo_idx[off + va] ^ klo_idx[off + vb];
        dl = xl ? 64 + __clzll((long long)xl) : (int)(a.tmax * w) + __clz((int)(va ^ vb));
    }
    lam[off + p] = (unsigned char)dl;
}

// ---- permutations: how many each point draws, and where -------------------------------

// digit-level common prefix of entry v with earlier entries (bit-level L from
// the tree pass); tmax_new for a repeated point
__device__ __forceinline__ u32 digit_lcp(u32 dl, u32 w, u32 tmax, u32 tmax_new)
{
    return dl >= tmax * w ? tmax_new : dl / w;
}

__device__ __forceinline__ u32 levels_of(u32 v, const unsigned char *Lv, u32 w, const GdnArgs &a)
{
    if (v == 0) return a.tmax_new;  // the phantom root
    const u32 L = digit_lcp(Lv[v], w, a.tmax, a.tmax_new);
    return L + 1 >= a.tmax_new ? 0u : a.tmax_new - 1 - L;
}

// per generator: exclusive offsets (in permutation entries) of each entry's
// permutations, and the generator's total
__global__ void __launch_bounds__(1024) gdn_offsets_kernel(NusDims m, GdnArgs a, const unsigned char *__restrict__ Lv,
                                                           u64 *__restrict__ offs, u64 *__restrict__ tot)
{
    __shared__ u64 wsum[32];
    const u32 g = blockIdx.x;
    const u64 off = (u64)g * m.NP;
    u32 b, w;
    gdn_base_of(m, a, m.s0 + g, b, w);
    const u32 per = (m.N + 1023) / 1024;
    const u32 beg = min(threadIdx.x * per, m.N), end = min(beg + per, m.N);
    u64 sum = 0;
    for (u32 v = beg; v < end; v++) sum += (u64)levels_of(v, Lv + off, w, a) * b;
    const u32 lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    u64 incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const u64 y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (u32)o) incl += y;
    }
    if (lane == 31) wsum[wp] = incl;
    __syncthreads();
    if (wp == 0) {
        u64 x = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const u64 y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (u32)o) x += y;
        }
        wsum[lane] = x;
    }
    __syncthreads();
    u64 run = incl - sum + (wp ? wsum[wp - 1] : 0ull);
    for (u32 v = beg; v < end; v++) {
        offs[off + v] = run;
        run += (u64)levels_of(v, Lv + off, w, a) * b;
    }
    if (threadIdx.x == 1023) tot[g] = run;
}

// the chunk's generators one after another: a base per generator; the total
// in ctl[0] and the most permutation rows of any generator in ctl[1]
__global__ void gdn_bases_kernel(NusDims m, GdnArgs a, const u64 *__restrict__ tot, u64 *__restrict__ base, u64 *ctl)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    u64 run = 0, most = 0;
    for (u32 g = 0; g < m.S; g++) {
        u32 b, w;
        gdn_base_of(m, a, m.s0 + g, b, w);
        base[g] = run;
        run += tot[g];
        const u64 rows = b ? tot[g] / b : 0;
        most = rows > most ? rows : most;
    }
    ctl[0] = run;
    ctl[1] = most;
}

// permutation entries of generator g that earlier calls drew (its entries
// below H0); none for fresh trees, where the phantom root draws here
__device__ __forceinline__ u64 old_entries(const NusDims &m, const u64 *offs, const u64 *tot, u32 g)
{
    if (m.fresh) return 0;
    return m.H0 < m.N ? offs[(u64)g * m.NP + m.H0] : tot[g];
}

// the rows of the trees' earlier entries, copied in front of this call's
// rows; a history whose length disagrees with the entries' levels sets bit 64
// of the device error word and copies nothing
__global__ void __launch_bounds__(NUS_THREADS) gdn_hist_rows_kernel(NusDims m, const u64 *__restrict__ offs,
                                                                    const u64 *__restrict__ tot,
                                                                    const u64 *__restrict__ base,
                                                                    const unsigned short *__restrict__ hist_perms,
                                                                    const u64 *__restrict__ hist_off,
                                                                    unsigned short *__restrict__ perms,
                                                                    unsigned int *err)
{
    const u32 g = blockIdx.y;
    const u64 s = m.s0 + g, beg = hist_off[s], len = hist_off[s + 1] - beg;
    if (len != old_entries(m, offs, tot, g)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, 64u);
        return;
    }
    unsigned short *dst = perms + base[g];
    for (u64 e = (u64)blockIdx.x * NUS_THREADS + threadIdx.x; e < len; e += (u64)gridDim.x * NUS_THREADS)
        dst[e] = hist_perms[beg + e];
}

// ---- the draws: Generator.permutation(b) per level ---------------------------------
// numpy's Generator.shuffle walks i = b-1 .. 1 and swaps position i with
// random_interval(i).  The stream is serial per generator, the swaps are not:
// one CTA per generator runs the stream (fy_stream.cuh: a producer lane and
// decoding warps) and writes each accepted index j_i into entry i of its row
// (rows in draw order: the phantom's, then each point's levels, as the offsets
// lay them out); then one thread per row replays the swaps on arange(b) in
// shared memory and writes the permutation over the indices.

// the rows of one generator this call draws: entry i of row q at row0[q*b + i]
struct GdnRows {
    unsigned short *row0;
    u32 b;
    u64 rows;
    bool given;
    __device__ bool next(u32 &bo, u64 &ro)
    {
        if (given) return false;
        given = true;
        bo = b;
        ro = rows;
        return true;
    }
    __device__ void put(u64 q, u32 i, u32 j) { row0[q * b + i] = (unsigned short)j; }
};

__global__ void __launch_bounds__(FY_THREADS) gdn_stream_kernel(NusDims m, GdnArgs a, u64 *__restrict__ states,
                                                                const u64 *__restrict__ offs,
                                                                const u64 *__restrict__ tot,
                                                                const u64 *__restrict__ base,
                                                                unsigned short *__restrict__ perms, unsigned int *err)
{
    __shared__ FyShared sh;
    const u32 g = blockIdx.x;
    if (g >= m.S) return;
    u32 b, w;
    gdn_base_of(m, a, m.s0 + g, b, w);
    if (b < 2 || b > 65536) {  // reported by the keys pass; nothing to draw from
        if (threadIdx.x == 0) atomicOr(err, 1u);
        return;
    }
    const u64 rows = tot[g] / b;
    const u64 q0 = old_entries(m, offs, tot, g) / b;  // rows before q0 came from earlier calls
    if (q0 >= rows) return;
    GdnRows R{perms + base[g] + q0 * b, b, rows - q0, false};
    if (b <= FY_SMALL_MAX)
        fy_stream_small(sh, states + (m.s0 + g) * 6, b, rows - q0, R, err, 16u);
    else
        fy_stream(sh, states + (m.s0 + g) * 6, R, err, 16u);
}

// rows of one generator per blockIdx.y; thread t of a block holds its row's
// permutation in column t of a (b x T) shared-memory array, so that lanes
// never meet in a bank (T a multiple of 64: entry k of lane t sits in word
// (k*T + t)/2)
__global__ void gdn_shuffle_kernel(NusDims m, GdnArgs a, const u64 *__restrict__ offs, const u64 *__restrict__ tot,
                                   const u64 *__restrict__ base, unsigned short *__restrict__ perms)
{
    extern __shared__ unsigned short col[];
    const u32 g = blockIdx.y, T = blockDim.x, t = threadIdx.x;
    u32 b, w;
    gdn_base_of(m, a, m.s0 + g, b, w);
    if (b < 2 || b > 65536) return;  // reported by the keys pass
    const u64 q = old_entries(m, offs, tot, g) / b + (u64)blockIdx.x * T + t;
    if (q >= tot[g] / b) return;
    unsigned short *row = perms + base[g] + q * b;
    unsigned short *A = col + t;
    for (u32 k = 0; k < b; k++) A[(u64)k * T] = (unsigned short)k;
    for (u32 k = b - 1; k >= 1; k--) {
        const u32 j = row[k];
        const unsigned short x = A[(u64)k * T], y = A[(u64)j * T];
        A[(u64)k * T] = y;
        A[(u64)j * T] = x;
    }
    for (u32 k = 0; k < b; k++) row[k] = A[(u64)k * T];
}

// ---- output: each point's digits through its owners' permutations -------------------
// Level t is owned by the highest ancestor whose prefix covers min(t, tmax)
// digits (bits min(t, tmax) * w); the levels go from the last up, the node
// from the leaf up.

__global__ void __launch_bounds__(NUS_THREADS) gdn_walk_kernel(NusDims m, GdnArgs a, const u32 *__restrict__ val,
                                                               const unsigned char *__restrict__ lam,
                                                               const u32 *__restrict__ pleaf,
                                                               const u32 *__restrict__ pint,
                                                               const u32 *__restrict__ minv,
                                                               const unsigned char *__restrict__ Lv,
                                                               const u64 *__restrict__ offs,
                                                               const u64 *__restrict__ base,
                                                               const unsigned short *__restrict__ perms,
                                                               const u64 *__restrict__ xdig, u64 *__restrict__ xrdig,
                                                               unsigned int *err)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    const u32 v = val[off + p];
    if (v < m.H0) return;  // the phantom
    const u64 s = m.s0 + g, l = s / m.d, j = s - l * m.d, i = v - m.H0;
    u32 b, w;
    gdn_base_of(m, a, s, b, w);
    if (b == 0 || b > 65536) return;  // reported by the keys pass
    const u64 *x = xdig + (((l % m.r_x) * m.n + i) * m.d + j) * a.tmax;
    u64 *out = xrdig + ((l * m.n + i) * m.d + j) * a.tmax_new;
    const unsigned short *pg = perms + base[g];
    u32 owner = v;
    u32 parent = pleaf[off + p];
    int dP = parent == NONE ? -1 : (int)lam[off + parent];
    int hops = 0;
    for (int t = (int)a.tmax_new - 1; t >= 0; t--) {
        const int k = (int)(min((u32)t, a.tmax) * w);
        while (parent != NONE && dP >= k) {
            if (++hops > MAX_DEPTH) {
                atomicOr(err, 16u);
                return;
            }
            owner = minv[off + parent];
            parent = pint[off + parent];
            dP = parent == NONE ? -1 : (int)lam[off + parent];
        }
        const u64 xt = (u32)t < a.tmax ? x[t] : 0;
        const u32 first = owner == 0 ? 0u : digit_lcp(Lv[off + owner], w, a.tmax, a.tmax_new) + 1;
        if (xt >= b || (u32)t < first) {  // a digit outside its base (reported by the keys pass)
            out[t] = 0;
            continue;
        }
        out[t] = pg[offs[off + owner] + (u64)((u32)t - first) * b + xt];
    }
}

// ---- workspace -----------------------------------------------------------------------

inline u64 gal256(u64 b) { return (b + 255) & ~255ull; }

struct GdnWork {
    u64 *keyA, *keyB, *khi, *klo, *offs, *tot, *base, *total;
    u32 *valA, *valB, *cnt, *pleaf, *pint, *ctl;
    unsigned long long *slot;
    unsigned char *lam, *Lv;
    u64 bytes;
};

GdnWork gdn_layout(char *basep, u64 count, u64 NP, u64 NT)
{
    GdnWork w{};
    u64 off = 0;
    auto take = [&](u64 bytes) {
        char *p = basep ? basep + off : nullptr;
        off += gal256(bytes);
        return p;
    };
    const u64 e = count * NP;
    w.keyA = (u64 *)take(e * 8);
    w.keyB = (u64 *)take(e * 8);
    w.khi = (u64 *)take(e * 8);
    w.klo = (u64 *)take(e * 8);
    w.offs = (u64 *)take(e * 8);
    w.slot = (unsigned long long *)take(e * 8);
    w.valA = (u32 *)take(e * 4);
    w.valB = (u32 *)take(e * 4);
    w.pleaf = (u32 *)take(e * 4);
    w.pint = (u32 *)take(e * 4);
    w.cnt = (u32 *)take(count * 256 * NT * 4);
    w.lam = (unsigned char *)take(e);
    w.Lv = (unsigned char *)take(e);
    w.tot = (u64 *)take(count * 8);
    w.base = (u64 *)take(count * 8);
    w.total = (u64 *)take(256);
    w.ctl = (u32 *)take(256);
    w.bytes = off;
    return w;
}

u64 gdn_padded(u64 N) { return (N + 15) & ~15ull; }
u64 gdn_tiles(u64 N) { return (N + WT - 1) / WT; }

}  // namespace

extern "C" {

int qmc_gdn_nus_workspace_size(uint64_t n, uint64_t h0, uint64_t generators, uint64_t *bytes)
{
    QMC_REQUIRE(bytes, "gdn_nus_workspace_size: null output pointer");
    const u64 N = (h0 ? h0 : 1) + n;
    QMC_REQUIRE(N < MAX_ENTRIES, "gdn_nested_uniform_scramble: %llu points per generator (at most 2^30 - 2)",
                (unsigned long long)n);
    *bytes = gdn_layout(nullptr, generators ? generators : 1, gdn_padded(N), gdn_tiles(N)).bytes;
    return QMC_OK;
}

int qmc_gdn_nested_uniform_scramble(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t r_b, uint64_t tmax,
                                    uint64_t tmax_new, uint64_t *states, const uint64_t *bases, uint64_t h0,
                                    const uint64_t *hist_keys, const uint16_t *hist_perms,
                                    const uint64_t *hist_perm_off, const uint64_t *xdig, uint64_t *xrdig,
                                    uint64_t *keys_out, uint16_t *perms, uint64_t perm_capacity, uint64_t *perm_off,
                                    uint64_t *perm_needed, void *work, uint64_t work_bytes, qmc_stream_t s)
{
    if (perm_needed) *perm_needed = 0;
    if (r == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(r_x >= 1 && r_b >= 1, "gdn_nested_uniform_scramble: r_x or r_b = 0");
    QMC_REQUIRE(states && work && bases && perms && perm_off, "gdn_nested_uniform_scramble: null states, bases, "
                "permutation buffer, permutation offsets or workspace");
    QMC_REQUIRE(h0 == 0 || (hist_keys && hist_perms && hist_perm_off),
                "gdn_nested_uniform_scramble: h0 > 0 needs the trees' keys, permutations and offsets");
    QMC_REQUIRE(n == 0 || (xdig && xrdig), "gdn_nested_uniform_scramble: null xdig or xrdig");
    QMC_REQUIRE(tmax_new > tmax && tmax_new <= 255 && tmax >= 1,
                "gdn_nested_uniform_scramble: needs 1 <= tmax < tmax_new <= 255 (tmax = %llu, tmax_new = %llu)",
                (unsigned long long)tmax, (unsigned long long)tmax_new);
    QMC_REQUIRE(((uintptr_t)work & 255) == 0, "gdn_nested_uniform_scramble: workspace not 256-byte aligned");
    const u64 H0 = h0 ? h0 : 1, N = H0 + n;
    QMC_REQUIRE(N < MAX_ENTRIES && N > n, "gdn_nested_uniform_scramble: %llu entries per generator (at most 2^30 - 1)",
                (unsigned long long)N);
    const u64 NP = gdn_padded(N), NT = gdn_tiles(N), G = r * d;
    const u64 per = gdn_layout(nullptr, 1, NP, NT).bytes;
    QMC_REQUIRE(work_bytes >= per, "gdn_nested_uniform_scramble: workspace of %llu bytes, one generator needs %llu",
                (unsigned long long)work_bytes, (unsigned long long)per);
    // the most generators whose sub-arrays fit; work_bytes / per alone comes out one short for
    // a workspace sized for exactly that many, as the fixed words count once in any layout
    const u64 cap = G < 65535 ? G : 65535;
    u64 count = work_bytes / per;
    if (count > cap) count = cap;
    while (count < cap && gdn_layout(nullptr, count + 1, NP, NT).bytes <= work_bytes) count++;
    while (count > 1 && gdn_layout(nullptr, count, NP, NT).bytes > work_bytes) count--;
    GdnWork w = gdn_layout((char *)work, count, NP, NT);
    cudaStream_t st = QMC_STREAM(s);
    unsigned int *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");

    NusDims m{};
    m.n = n;
    m.d = d;
    m.r_x = r_x;
    m.T = 255;  // the tree pass records bit-level prefix lengths as they are
    m.N = (u32)N;
    m.NP = (u32)NP;
    m.H0 = (u32)H0;
    m.NT = (u32)NT;
    m.fresh = h0 == 0;
    GdnArgs a{(const u64 *)bases, r_b, (u32)tmax, (u32)tmax_new, h0 ? (const u64 *)hist_keys : nullptr};
    const u64 *xd = (const u64 *)xdig;
    u64 *xr = (u64 *)xrdig;
    u64 *stw = (u64 *)states;
    unsigned short *pm = (unsigned short *)perms;
    const dim3 ng((unsigned)((N + NUS_THREADS - 1) / NUS_THREADS), 1);
    u64 filled = 0;       // permutation entries of the generators before this chunk
    bool sizing = false;  // the buffer ran short: the remaining chunks only count their entries
    std::vector<u64> tot_h(count);
    perm_off[0] = 0;
    // rows per block of the shuffle: b x T 16-bit entries in shared memory
    u64 bmax = 2;
    {
        std::vector<u64> hb(r_b * d);
        int rc = qmcgb::cuda_status(cudaMemcpyAsync(hb.data(), bases, r_b * d * 8, cudaMemcpyDefault, st),
                                    "gdn_nus bases");
        if (rc) return rc;
        rc = qmcgb::cuda_status(cudaStreamSynchronize(st), "gdn_nus bases");
        if (rc) return rc;
        for (u64 v : hb) bmax = v > bmax ? v : bmax;
    }
    QMC_REQUIRE(bmax <= 65536, "gdn_nested_uniform_scramble: bases above 65536");
    u32 shuffle_T = 128;
    while (shuffle_T > 1 && (u64)shuffle_T * bmax * 2 > 98304) shuffle_T >>= 1;
    const size_t shuffle_smem = (size_t)shuffle_T * bmax * 2;
    if (int rc = qmcgb::raise_smem_limit((const void *)gdn_shuffle_kernel, shuffle_smem, "gdn_nus shuffle smem"))
        return rc;

    for (u64 s0 = 0; s0 < G; s0 += count) {
        m.s0 = s0;
        m.S = (u32)(G - s0 < count ? G - s0 : count);
        const dim3 gg(ng.x, m.S);
        gdn_keys_kernel<<<gg, NUS_THREADS, 0, st>>>(m, a, xd, w.keyA, w.khi, w.klo, err);
        int rc = qmcgb::launch_status("gdn_nus keys");
        if (rc) return rc;
        if (keys_out && !sizing) {
            gdn_keys_out_kernel<<<gg, NUS_THREADS, 0, st>>>(m, w.khi, w.klo, (u64 *)keys_out);
            rc = qmcgb::launch_status("gdn_nus keys out");
            if (rc) return rc;
        }
        u64 *kf = w.keyA, *ko = w.keyB;
        u32 *vf = w.valA, *vo = w.valB;
        if (n > 0) {
            const dim3 tg((unsigned)((NT + NUS_WARPS - 1) / NUS_WARPS), m.S);
            if (int rc2 = qmcgb::raise_smem_limit((const void *)nus_scatter_kernel, NUS_SCATTER_SMEM, "gdn_nus sort"))
                return rc2;
            auto pass = [&](const u64 *kin, const u32 *vin, u32 digit, u64 *kout, u32 *vout) {
                nus_hist_kernel<<<tg, NUS_THREADS, 0, st>>>(m, kin, 8 * digit, w.cnt);
                nus_scan_kernel<<<m.S, 1024, 0, st>>>(m, w.cnt);
                nus_scatter_kernel<<<tg, NUS_THREADS, NUS_SCATTER_SMEM, st>>>(m, kin, vin, 8 * digit, w.cnt, kout, vout);
                return qmcgb::launch_status("gdn_nus sort");
            };
            // the top digits of the high word, then runs finished on the full key
            const u32 need_bits = (u32)(64 - __builtin_clzll((unsigned long long)(N - 1) | 1ull)) + 4;
            const u32 top = 8 < (need_bits + 7) / 8 ? 8u : (need_bits + 7) / 8;
            const u64 *kin = w.keyA;
            const u32 *vin = nullptr;
            for (u32 q = 0; q < top; q++) {
                u64 *kout = (q & 1) ? w.keyA : w.keyB;
                u32 *vout = (q & 1) ? w.valA : w.valB;
                rc = pass(kin, vin, 8 - top + q, kout, vout);
                if (rc) return rc;
                kin = kout;
                vin = vout;
            }
            kf = (top & 1) ? w.keyB : w.keyA;
            ko = (top & 1) ? w.keyA : w.keyB;
            vf = (top & 1) ? w.valB : w.valA;
            vo = (top & 1) ? w.valA : w.valB;
            rc = qmcgb::cuda_status(cudaMemsetAsync(w.ctl, 0, 4, st), "gdn_nus run flag");
            if (rc) return rc;
            gdn_fixup_kernel<<<gg, NUS_THREADS, 0, st>>>(m, 8 * (8 - top), kf, vf, w.klo, w.ctl);
            u32 longrun = 0;
            rc = qmcgb::cuda_status(cudaMemcpyAsync(&longrun, w.ctl, 4, cudaMemcpyDeviceToHost, st),
                                    "gdn_nus run flag");
            if (rc) return rc;
            rc = qmcgb::cuda_status(cudaStreamSynchronize(st), "gdn_nus run flag");
            if (rc) return rc;
            if (longrun) {  // every digit: the low word's from point order, then the high word's
                const u64 *ki = w.klo;
                const u32 *vi = nullptr;
                for (u32 q = 0; q < 8; q++) {
                    u64 *kout = (q & 1) ? kf : ko;
                    u32 *vout = (q & 1) ? vf : vo;
                    rc = pass(ki, vi, q, kout, vout);
                    if (rc) return rc;
                    ki = kout;
                    vi = vout;
                }
                gdn_gather_kernel<<<gg, NUS_THREADS, 0, st>>>(m, vf, w.khi, ko);  // high words in that order
                ki = ko;
                vi = vf;
                for (u32 q = 0; q < 8; q++) {
                    u64 *kout = (q & 1) ? ko : kf;
                    u32 *vout = (q & 1) ? vf : vo;
                    rc = pass(ki, vi, q, kout, vout);
                    if (rc) return rc;
                    ki = kout;
                    vi = vout;
                }
                // the last pass wrote (ko, vf); the keys go back to kf
                rc = qmcgb::cuda_status(cudaMemcpyAsync(kf, ko, (u64)m.S * NP * 8, cudaMemcpyDeviceToDevice, st),
                                        "gdn_nus sort");
                if (rc) return rc;
            }
            gdn_lcp_kernel<<<gg, NUS_THREADS, 0, st>>>(m, a, kf, vf, w.klo, w.lam);
            rc = qmcgb::cuda_status(cudaMemsetAsync(w.slot, 0xFF, (u64)m.S * NP * 8, st), "gdn_nus slots");
            if (rc) return rc;
            nus_build_kernel<<<gg, NUS_THREADS, 0, st>>>(m, vf, w.lam, w.slot, w.pleaf, w.pint, vo, w.Lv, err);
            rc = qmcgb::launch_status("gdn_nus tree");
            if (rc) return rc;
        }
        gdn_offsets_kernel<<<m.S, 1024, 0, st>>>(m, a, w.Lv, w.offs, w.tot);
        gdn_bases_kernel<<<1, 32, 0, st>>>(m, a, w.tot, w.base, w.total);
        u64 sizes[2] = {0, 0};
        rc = qmcgb::cuda_status(cudaMemcpyAsync(sizes, w.total, 16, cudaMemcpyDeviceToHost, st), "gdn_nus sizes");
        if (rc) return rc;
        rc = qmcgb::cuda_status(cudaMemcpyAsync(tot_h.data(), w.tot, (u64)m.S * 8, cudaMemcpyDeviceToHost, st),
                                "gdn_nus sizes");
        if (rc) return rc;
        rc = qmcgb::cuda_status(cudaStreamSynchronize(st), "gdn_nus sizes");
        if (rc) return rc;
        const u64 total = sizes[0], most_rows = sizes[1];
        for (u32 g = 0; g < m.S; g++) perm_off[s0 + g + 1] = perm_off[s0 + g] + tot_h[g];
        if (sizing || filled + total > perm_capacity) {
            sizing = true;
            filled += total;
            continue;
        }
        unsigned short *pc = pm + filled;  // this chunk's rows
        filled += total;
        if (h0) {
            const dim3 hg((unsigned)qmcgb::grid_for(most_rows * bmax, NUS_THREADS, 4096), m.S);
            gdn_hist_rows_kernel<<<hg, NUS_THREADS, 0, st>>>(m, w.offs, w.tot, w.base, (const unsigned short *)hist_perms,
                                                             (const u64 *)hist_perm_off, pc, err);
            rc = qmcgb::launch_status("gdn_nus earlier rows");
            if (rc) return rc;
        }
        gdn_stream_kernel<<<m.S, FY_THREADS, 0, st>>>(m, a, stw, w.offs, w.tot, w.base, pc, err);
        rc = qmcgb::launch_status("gdn_nus draws");
        if (rc) return rc;
        if (most_rows > 0) {
            const dim3 sg((unsigned)((most_rows + shuffle_T - 1) / shuffle_T), m.S);
            gdn_shuffle_kernel<<<sg, shuffle_T, shuffle_smem, st>>>(m, a, w.offs, w.tot, w.base, pc);
            rc = qmcgb::launch_status("gdn_nus permutations");
            if (rc) return rc;
        }
        if (n > 0) {
            gdn_walk_kernel<<<gg, NUS_THREADS, 0, st>>>(m, a, vf, w.lam, w.pleaf, w.pint, vo, w.Lv, w.offs, w.base,
                                                        pc, xd, xr, err);
            rc = qmcgb::launch_status("gdn_nus output");
            if (rc) return rc;
        }
    }
    if (perm_needed) *perm_needed = filled;
    if (sizing) {
        qmcgb::set_error("gdn_nested_uniform_scramble: the permutations of %llu generators need %llu entries, the "
                         "buffer holds %llu", (unsigned long long)G, (unsigned long long)filled,
                         (unsigned long long)perm_capacity);
        return QMC_ERR_ARG;
    }
    return QMC_OK;
}

}  // extern "C"
