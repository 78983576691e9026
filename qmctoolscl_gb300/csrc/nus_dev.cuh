// nus_dev.cuh -- device parts shared by the nested uniform scrambles of
// base-2 nets (nus.cu) and generalized base-b nets (gdn_nus.cu): the launch
// constants and chunk dimensions, the stable LSD radix sort of (key, point)
// pairs on 64-bit keys, Apetrei's bottom-up radix-tree pass with the earliest
// point per node; numpy's SFC64 generator comes from numpy_rng.cuh.  Each
// including file gets its own copy (anonymous namespace).
#pragma once
#include "common.cuh"
#include "numpy_rng.cuh"

namespace {

constexpr u32 NONE = 0xFFFFFFFFu;
constexpr int NUS_THREADS = 256;
constexpr int NUS_WARPS = NUS_THREADS / 32;
constexpr u32 WT = 1024;  // entries per warp tile in the radix passes
constexpr u32 MAX_ENTRIES = 1u << 30;  // points + history per generator
// Prefix lengths of the extended keys (key bits, then 32 bits of the point
// index) grow strictly from the root down and stay below 128 + 32 = 160, so
// no path in a radix tree has more than 161 nodes; the upward loops stop
// there and record bit 16 of the device error word instead of running on.
constexpr int MAX_DEPTH = 161;

struct NusDims {
    u64 n, d, r_x, td, mask, h0, s0;
    u32 T, N, NP, H0, NT, S;
    int fresh;
};

// ---- stable LSD radix sort, 8 bits per pass -----------------------------------
// Each warp owns a tile of WT consecutive entries of one generator.  Pass:
// per-tile digit counts, a per-generator exclusive scan over (digit, tile),
// then each warp sorts its tile by digit in shared memory (ranks among equal
// digits from __match_any_sync, so equal digits keep their order) and writes
// it out in that order: a digit's entries of one tile (about WT/256) land in
// consecutive output slots, so a warp's store covers a few runs of
// consecutive addresses instead of 32 scattered ones.

__global__ void __launch_bounds__(NUS_THREADS) nus_hist_kernel(NusDims m, const u64 *__restrict__ key, u32 shift,
                                                               u32 *__restrict__ cnt)
{
    __shared__ u32 h[NUS_WARPS][256];
    for (u32 k = threadIdx.x; k < NUS_WARPS * 256; k += NUS_THREADS) (&h[0][0])[k] = 0;
    __syncthreads();
    const u32 w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const u32 tile = blockIdx.x * NUS_WARPS + w, g = blockIdx.y;
    if (tile >= m.NT) return;
    const u64 *kp = key + (u64)g * m.NP;
    const u32 beg = tile * WT, end = min(beg + WT, m.N);
    for (u32 p = beg + lane; p < end; p += 32) atomicAdd(&h[w][(u32)(kp[p] >> shift) & 255u], 1u);
    __syncwarp();
    for (u32 dg = lane; dg < 256; dg += 32) cnt[((u64)g * 256 + dg) * m.NT + tile] = h[w][dg];
}

// Exclusive scan of one generator's 256 * NT counts per block: each warp takes a contiguous
// segment, sums it (lanes on consecutive words), and after a scan of the 32 warp sums scans
// its segment in rows of 32 consecutive words (five shuffles a row, the running total carried)
__global__ void __launch_bounds__(1024) nus_scan_kernel(NusDims m, u32 *__restrict__ cnt)
{
    __shared__ u32 wsum[32];
    const u64 total = 256ull * m.NT;
    u32 *c = cnt + (u64)blockIdx.x * total;
    const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const u64 per = ((total + 31) / 32 + 31) & ~31ull;  // a warp's segment, whole rows of 32
    const u64 beg = min((u64)w * per, total), end = min(beg + per, total);
    u32 sum = 0;
    for (u64 k = beg + lane; k < end; k += 32) sum += c[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
    if (lane == 0) wsum[w] = sum;
    __syncthreads();
    if (w == 0) {
        const u32 x0 = wsum[lane];
        u32 x = x0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (u32)o) x += y;
        }
        wsum[lane] = x - x0;  // exclusive: the counts before warp `lane`'s segment
    }
    __syncthreads();
    u32 run = wsum[w];
    for (u64 r0 = beg; r0 < end; r0 += 32) {
        const u64 k = r0 + lane;
        const u32 t = k < end ? c[k] : 0u;
        u32 incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (u32)o) incl += y;
        }
        if (k < end) c[k] = run + incl - t;
        run += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
}

// shared memory of the scatter: per warp the tile's output offsets and staging slots per digit
// (2 x 256 words), then the tile's entries in digit order as indices into the tile (WT x 2 bytes)
constexpr size_t NUS_SCATTER_WARP_BYTES = 2 * 256 * 4 + (size_t)WT * 2;
constexpr size_t NUS_SCATTER_SMEM = NUS_WARPS * NUS_SCATTER_WARP_BYTES;

__global__ void __launch_bounds__(NUS_THREADS) nus_scatter_kernel(NusDims m, const u64 *__restrict__ kin,
                                                                  const u32 *__restrict__ vin, u32 shift,
                                                                  const u32 *__restrict__ cnt, u64 *__restrict__ kout,
                                                                  u32 *__restrict__ vout)
{
    extern __shared__ __align__(16) unsigned char nus_sc_smem[];
    const u32 w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *ws = nus_sc_smem + w * NUS_SCATTER_WARP_BYTES;
    u32 *delta = (u32 *)ws;            // [256] output slot of staged slot j of digit dg: delta[dg] + j
    u32 *lpos = delta + 256;           // [256] the digit's next staging slot
    unsigned short *sx = (unsigned short *)(lpos + 256);  // [WT] the tile's entries in digit order
    const u32 tile = blockIdx.x * NUS_WARPS + w, g = blockIdx.y;
    if (tile >= m.NT) return;  // whole warps leave; nothing below synchronises the block
    // the tile's count of digit dg is the next (digit, tile) offset of the exclusive scan minus
    // its own (the last of all ends at N); lane L takes digits 8L .. 8L+7
    const u64 cb = (u64)g * 256 * m.NT;
    u32 b0[8], c8[8], sum = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const u32 dg = lane * 8 + k;
        const u64 idx = cb + (u64)dg * m.NT + tile;
        b0[k] = cnt[idx];
        const u32 b1 = (dg == 255 && tile == m.NT - 1) ? m.N : cnt[idx + 1];
        c8[k] = b1 - b0[k];
        sum += c8[k];
    }
    u32 incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (u32)o) incl += y;
    }
    u32 run = incl - sum;  // first staging slot of digit 8L
#pragma unroll
    for (int k = 0; k < 8; k++) {
        lpos[lane * 8 + k] = run;
        delta[lane * 8 + k] = b0[k] - run;  // mod 2^32: delta + j is the output slot
        run += c8[k];
    }
    __syncwarp();
    const u64 off = (u64)g * m.NP;
    const u32 beg = tile * WT, end = min(beg + WT, m.N);
    for (u32 p0 = beg; p0 < end; p0 += 32) {
        const u32 p = p0 + lane;
        const bool ok = p < end;
        const u64 k = ok ? kin[off + p] : 0;
        const u32 dg = ok ? ((u32)(k >> shift) & 255u) : 256u + lane;  // idle lanes match nobody
        const u32 peers = __match_any_sync(0xFFFFFFFFu, dg);
        const u32 rank = __popc(peers & ((1u << lane) - 1u));
        const u32 slot = ok ? lpos[dg] + rank : 0;
        __syncwarp();
        if (ok && rank == 0) lpos[dg] += __popc(peers);
        if (ok) sx[slot] = (unsigned short)(p - beg);
        __syncwarp();
    }
    // the key and value again from the tile the warp has just read (still in L1)
    for (u32 j = lane; j < end - beg; j += 32) {
        const u32 p = beg + sx[j];
        const u64 k = kin[off + p];
        const u32 pos = delta[(u32)(k >> shift) & 255u] + j;
        kout[off + pos] = k;
        vout[off + pos] = vin ? vin[off + p] : p;
    }
}

// Keys that agree in the sorted top bits form runs (in point order); runs of
// at most RUN_MAX entries are finished here by an insertion sort on the full
// key, one thread per run.  A longer run sets *longrun and the chunk is sorted
// again on every digit.  Threads compare only the top bits of neighbouring
// runs, which the in-place sorts do not change.
constexpr u32 RUN_MAX = 32;

__global__ void __launch_bounds__(NUS_THREADS) nus_fixup_kernel(NusDims m, u32 lowbits, u64 *key, u32 *val,
                                                                u32 *longrun)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    u64 *k = key + off;
    u32 *v = val + off;
    const u64 hi = k[p] >> lowbits;
    if (p > 0 && (k[p - 1] >> lowbits) == hi) return;        // not the first of its run
    if (p + 1 >= m.N || (k[p + 1] >> lowbits) != hi) return;  // a run of one
    u32 e = p + 2;
    while (e < m.N && e - p <= RUN_MAX && (k[e] >> lowbits) == hi) e++;
    if (e - p > RUN_MAX) {
        atomicOr(longrun, 1u);
        return;
    }
    for (u32 a = p + 1; a < e; a++) {
        const u64 x = k[a];
        const u32 y = v[a];
        u32 b = a;
        while (b > p && k[b - 1] > x) {
            k[b] = k[b - 1];
            v[b] = v[b - 1];
            b--;
        }
        k[b] = x;
        v[b] = y;
    }
}

// back to point order (for the full sort after a long run)
__global__ void __launch_bounds__(NUS_THREADS) nus_unsort_kernel(NusDims m, const u64 *__restrict__ key,
                                                                 const u32 *__restrict__ val, u64 *__restrict__ out)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    out[off + val[off + p]] = key[off + p];
}

// ---- binary radix tree, earliest points and L, in one bottom-up pass -------------
// Apetrei's agglomerative construction (HPG 2014) of the binary radix tree
// over the sorted extended keys (key, point): lam[i] is the common prefix
// length of neighbours i and i+1, and internal node s is the split between
// them (its prefix length is lam[s]).  One thread per leaf climbs: a node
// covering [l, r] has parent r (it is the parent's left child) when
// lam[r] > lam[l-1], else parent l-1.  The first child to arrive at a node
// parks its outer range end and its subtree's earliest point in the node's
// 64-bit slot with one atomic exchange and stops; the second takes them and
// goes on with the merged node.  At each node the later of the two earliest
// points first meets an earlier point at the node's prefix length: its L.
// Two leaves that are each other's sibling are merged by the left one with
// no atomic.

// Common prefix length of the extended keys at sorted positions i and j; -1
// outside [0, N).
__device__ __forceinline__ int nus_delta(const u64 *k, const u32 *v, long long i, long long j, u32 N, u32 T)
{
    if (j < 0 || j >= (long long)N) return -1;
    const u64 x = k[i] ^ k[j];
    if (x) return __clzll((long long)x) - (64 - (int)T);
    return (int)T + __clz((int)(v[i] ^ v[j]));
}

__global__ void __launch_bounds__(NUS_THREADS) nus_lcp_kernel(NusDims m, const u64 *__restrict__ key,
                                                              const u32 *__restrict__ val,
                                                              unsigned char *__restrict__ lam)
{
    const u32 i = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (i + 1 >= m.N) return;
    const u64 off = (u64)g * m.NP;
    lam[off + i] = (unsigned char)nus_delta(key + off, val + off, i, (long long)i + 1, m.N, m.T);
}

constexpr u64 SLOT_EMPTY = ~0ull;  // a parked value has an earliest point below 2^30 in its low word

__global__ void __launch_bounds__(NUS_THREADS) nus_build_kernel(NusDims m, const u32 *__restrict__ val,
                                                                const unsigned char *__restrict__ lam,
                                                                unsigned long long *slot, u32 *__restrict__ pleaf,
                                                                u32 *__restrict__ pint, u32 *__restrict__ minv,
                                                                unsigned char *__restrict__ Lv, unsigned int *err)
{
    const u32 p = blockIdx.x * NUS_THREADS + threadIdx.x, g = blockIdx.y;
    if (p >= m.N) return;
    const u64 off = (u64)g * m.NP;
    const long long last = (long long)m.N - 2;  // the last split
    auto lamv = [&](long long i) -> int { return (i < 0 || i > last) ? -1 : (int)lam[off + i]; };
    auto settle = [&](u32 node, u32 a, u32 b) {  // node's two earliest points are a and b
        minv[off + node] = min(a, b);
        const u32 dl = lam[off + node];
        Lv[off + max(a, b)] = (unsigned char)(dl >= m.T ? m.T : dl);
    };
    // the leaf
    long long lo = p, hi = p;
    bool left = lo == 0 || (hi <= last && lamv(hi) > lamv(lo - 1));
    u32 par = (u32)(left ? hi : lo - 1);
    pleaf[off + p] = par;
    u32 mn = val[off + p], node;
    if (!left && (p - 1 == 0 || lamv((long long)p - 1) > lamv((long long)p - 2))) return;  // merged by leaf p-1
    if (left && ((long long)p == last || lamv((long long)p + 1) < lamv(p))) {  // sibling leaf p+1
        const u32 b = val[off + p + 1];
        settle(p, mn, b);
        mn = min(mn, b);
        node = p;
        hi = (long long)p + 1;
    } else {
        const unsigned long long mine = ((unsigned long long)(u32)(left ? lo : hi) << 32) | mn;
        const unsigned long long prev = atomicExch(&slot[off + par], mine);
        if (prev == SLOT_EMPTY) return;
        const u32 other = (u32)(prev >> 32), omn = (u32)prev;
        if (left) hi = other; else lo = other;
        settle(par, mn, omn);
        mn = min(mn, omn);
        node = par;
    }
    for (int hop = 0;; hop++) {  // the internal node `node` covers [lo, hi]
        if (hop >= MAX_DEPTH) {
            atomicOr(err, 16u);
            return;
        }
        if (lo == 0 && hi == last + 1) {
            pint[off + node] = NONE;
            return;
        }
        left = lo == 0 || (hi <= last && lamv(hi) > lamv(lo - 1));
        par = (u32)(left ? hi : lo - 1);
        pint[off + node] = par;
        const unsigned long long mine = ((unsigned long long)(u32)(left ? lo : hi) << 32) | mn;
        const unsigned long long prev = atomicExch(&slot[off + par], mine);
        if (prev == SLOT_EMPTY) return;
        const u32 other = (u32)(prev >> 32), omn = (u32)prev;
        if (left) hi = other; else lo = other;
        settle(par, mn, omn);
        mn = min(mn, omn);
        node = par;
    }
}

}  // namespace
