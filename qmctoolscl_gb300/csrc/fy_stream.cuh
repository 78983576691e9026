// fy_stream.cuh -- the swap indices of numpy's Generator.permutation(b),
// drawn from one SFC64 stream at the stream's own speed.
//
// numpy's Fisher-Yates walks i = b-1 .. 1 and takes the swap index from
// random_interval(i): a 32-bit output masked to the bits of i, drawn again
// while above i.  The outputs come one after another from one generator, so
// the stream is serial; which of them are accepted, and where they go, can be
// worked out 32 at a time.  One CTA runs a stream:
//
//   * lane 0 of warp 0 (the producer) steps the generator, 16 64-bit outputs
//     per slot of a shared-memory ring, with the generator's state before the
//     slot's first step.  A slot holds 32 candidates: 32-bit halves, low half
//     first, after the half numpy had buffered, as numpy hands them out.
//
//   * runs of rows of any base (fy_stream): warp 1 decodes slot after slot.
//     From the row state at the slot's start (row q, position i), lane L
//     builds its candidate's acceptance mask A_L over the 32 states it can
//     meet (bit k: accepted after k accepts), segment by segment of equal
//     mask; every lane then runs the chain s += A_L & s over the one-hot
//     count s on all 32 masks, which marks the accepted lanes, and each
//     accepted lane stores its index.  A run that ends inside a slot hands
//     the slot's later candidates to the next run.
//
//   * one run of a small base, 2 <= b <= 33 (fy_stream_small): the work per
//     slot that does not depend on the stream's state runs in parallel on
//     FY_WORKERS warps, one slot each.  A candidate's acceptance at each
//     position 1..b-1 is a fixed bit pattern; with the pattern of all 32
//     lanes, lane j follows the 32 candidates from start position j+1 and
//     records which were accepted (E_j), for every start position at once.
//     Lane 0 of warp 1 (the scan) then only picks E_i of the slot's actual
//     start position and moves to the next slot's, one lookup per slot; the
//     worker stores its accepted lanes' indices from the published start.
//
// At the end the generator's state is replayed from the last slot's saved
// state up to the last candidate used and written where numpy leaves it
// (state words a, b, c, w, has_uint32, uinteger).  Every wait on another warp
// is bounded; one that runs out, or a stream that rejects everything for 8
// slots in a row (probability below 2^-256), sets `err_bit` in the device
// error word and stops.  Warps hand slots to one another through
// shared-memory counters, published with release stores and polled with
// acquire loads at CTA scope.
//
// Runs of rows for fy_stream come from a caller object with
//   bool next(u32 &b, u64 &rows)    -- the next run (false: no more); every
//                                      decoder lane calls it with the same result
//   void put(u64 q, u32 i, u32 j)   -- entry i of row q of the current run gets j
// and fy_stream_small takes an object with put() only.
#pragma once
#include "numpy_rng.cuh"

namespace {

constexpr u32 FY_RING = 16;              // slots of 16 outputs (32 candidates)
// Warps: 0 the producer, 1 the decoder of runs or the scan, and the small-base
// workers on warps 2, 3, 6, 7, 10, 11.  Warp w issues on the SM's sub-partition
// w % 4, so the producer, whose SFC64 steps are one dependent chain of 64-bit
// integer operations (about 32 cycles a step), keeps sub-partition 0 to itself
// (warps 4 and 8 leave at once) and the workers share sub-partitions 2 and 3.
constexpr u32 FY_WORKERS = 6;  // small-base decoders
constexpr u32 FY_THREADS = 32 * 12;
__device__ __forceinline__ int fy_worker_of(u32 warp)
{
    return (warp & 3) >= 2 ? (int)((warp >> 2) * 2 + (warp & 3) - 2) : -1;
}
constexpr u32 FY_SMALL_MAX = 33;         // largest base of the small-base decoder
constexpr u32 FY_SPIN_LIMIT = 1u << 26;  // polls per wait (no sleep: a sleeping warp wakes microseconds late)

struct __align__(16) FyShared {
    u64 raw[FY_RING][16];           // the slot's 64-bit outputs
    u64 st[FY_RING][4];             // a, b, c, w before the slot's first step
    u64 ext[FY_WORKERS][32];        // small bases: each worker's lane patterns
    u32 A[32];                      // runs: the lanes' acceptance masks
    u32 E[FY_RING][32];             // small bases: accepted lanes per start position
    u64 start_q[FY_RING];           // small bases: the slot's start row
    u32 start_i[FY_RING];           // and position
    u32 first[FY_RING];             // the buffered half that opens the slot when the stream starts with one
    volatile u32 done[FY_RING];     // small bases: slot c's patterns are in E (c + 1)
    volatile u32 freed[FY_RING];    // slot c's ring entry may be refilled (c + 1)
    volatile u32 produced, scanned, stop;
};

__device__ __forceinline__ u32 fy_mask(u32 i) { return 0xFFFFFFFFu >> __clz((int)i); }

__device__ __forceinline__ u32 fy_recip(u32 d) { return (u32)((0x100000000ull + d - 1) / d); }

// x / d for x < 2^18, 1 <= d < 2^17, with m = fy_recip(d) (unused for d = 1)
__device__ __forceinline__ u32 fy_div(u32 x, u32 d, u32 m)
{
    if (d == 1) return x;
    u32 q = __umulhi(x, m);
    if (q * d > x) q--;
    return q;
}

// a counter written by another warp, read with acquire semantics at CTA scope
__device__ __forceinline__ u32 fy_acquire(const volatile u32 *p)
{
    u32 v;
    asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];"
                 : "=r"(v)
                 : "r"((u32)__cvta_generic_to_shared((const void *)p))
                 : "memory");
    return v;
}

// a counter published to other warps with release semantics at CTA scope: what this
// thread wrote (or saw, after __syncwarp) before is visible to whoever acquires the value
__device__ __forceinline__ void fy_publish(volatile u32 *p, u32 v)
{
    asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"((u32)__cvta_generic_to_shared((const void *)p)),
                 "r"(v)
                 : "memory");
}

// lane 0 waits until *ctr > c; false (for the whole warp) once the stream stopped or the wait
// ran out (recorded)
__device__ __forceinline__ bool fy_wait_above(FyShared &sh, const volatile u32 *ctr, u32 c, u32 lane, unsigned *err,
                                              unsigned err_bit)
{
    u32 go = 1;
    if (lane == 0) {
        u32 spins = 0;
        while (fy_acquire(ctr) <= c) {
            if (sh.stop) {
                go = fy_acquire(ctr) > c;  // published before the stop
                break;
            }
            if (++spins > FY_SPIN_LIMIT) {
                atomicOr(err, err_bit);
                sh.stop = 1;
                go = 0;
                break;
            }
        }
    }
    go = __shfl_sync(0xFFFFFFFFu, go, 0);
    __syncwarp();
    return go != 0;
}

__device__ __forceinline__ u32 fy_candidate(const FyShared &sh, u32 slot, u32 lane, u32 parity)
{
    const int h = (int)lane - (int)parity;
    return h < 0 ? sh.first[slot] : ((const u32 *)sh.raw[slot])[h];
}

// the generator's six state words after candidate h (h = lane - parity) of a slot whose
// state before its first step was st and whose opening half was `first`
__device__ void fy_write_state(u64 *state, const u64 (&st)[4], u32 first, int h)
{
    if (h < 0) {  // the half that opened the slot: the state before the slot, the buffer used
        state[0] = st[0];
        state[1] = st[1];
        state[2] = st[2];
        state[3] = st[3];
        state[4] = 0;
        state[5] = first;
        return;
    }
    Sfc64 r;
    r.a = st[0];
    r.b = st[1];
    r.c = st[2];
    r.w = st[3];
    u64 y = 0;
    for (int k = 0; k <= h / 2; k++) y = r.next64();
    state[0] = r.a;
    state[1] = r.b;
    state[2] = r.c;
    state[3] = r.w;
    state[4] = (h & 1) ? 0u : 1u;  // a low half used: its high half waits in the buffer
    state[5] = y >> 32;
}

__device__ void fy_produce(FyShared &sh, const u64 *state, unsigned *err, unsigned err_bit)
{
    Sfc64 r;
    r.load(state);
    u32 carry = (u32)r.half;
    for (u32 c = 0;; c++) {
        const u32 slot = c % FY_RING;
        // the ring entry's flag is read before the slot's steps and checked after them, so
        // that its latency overlaps the steps' dependent chain
        const u32 fr = c >= FY_RING ? fy_acquire(&sh.freed[slot]) : 0u;
        const u64 s0 = r.a, s1 = r.b, s2 = r.c, s3 = r.w;
        u64 y[16];
#pragma unroll
        for (u32 h = 0; h < 16; h++) y[h] = r.next64();
        if (c >= FY_RING && fr != c - FY_RING + 1) {
            u32 spins = 0;
            while (fy_acquire(&sh.freed[slot]) != c - FY_RING + 1 && !sh.stop) {
                if (++spins > FY_SPIN_LIMIT) {
                    atomicOr(err, err_bit);
                    sh.stop = 1;
                    break;
                }
            }
        }
        if (sh.stop) break;
        sh.st[slot][0] = s0;
        sh.st[slot][1] = s1;
        sh.st[slot][2] = s2;
        sh.st[slot][3] = s3;
        sh.first[slot] = carry;
#pragma unroll
        for (u32 h = 0; h < 16; h++) sh.raw[slot][h] = y[h];
        carry = (u32)(y[15] >> 32);
        fy_publish(&sh.produced, c + 1);
    }
}

__device__ __forceinline__ void fy_init(FyShared &sh)
{
    if (threadIdx.x < FY_RING) {
        sh.done[threadIdx.x] = 0;
        sh.freed[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) {
        sh.produced = 0;
        sh.scanned = 0;
        sh.stop = 0;
    }
    __syncthreads();  // the last CTA-wide barrier
}

// ---- runs of rows of any base ---------------------------------------------------------

// bit k: candidate x accepted after k accepts from row q, position i (rows below nrows)
__device__ __forceinline__ u32 fy_accept_mask(u32 x, u32 i, u64 q, u64 nrows, u32 bm1)
{
    u32 A = 0, k = 0, pos = i;
    u64 row = q;
    while (k < 32 && row < nrows) {  // segments of equal mask; the same for every lane
        const u32 M = fy_mask(pos), lo = (M >> 1) + 1;
        const u32 ln = min(pos - lo + 1, 32 - k);
        const u32 tau = x & M;
        if (pos >= tau) {
            const u32 n = min(ln, pos - tau + 1);
            A |= (u32)(((1ull << n) - 1) << k);
        }
        k += ln;
        pos -= ln;
        if (pos == 0) {
            pos = bm1;
            row++;
        }
    }
    return A;
}

template <class Rows>
__device__ void fy_decode_runs(FyShared &sh, u64 *state, Rows &rows, unsigned *err, unsigned err_bit, u32 parity)
{
    const u32 lane = threadIdx.x & 31;
    u32 b = 0;
    u64 nrows = 0;
    bool have;
    do {
        have = rows.next(b, nrows);
    } while (have && (nrows == 0 || b < 2));  // permutation(0 or 1) draws nothing
    bool used = false, ok = true;
    u32 last_slot = 0, last_lane = 0, c = 0, start = 0, idle = 0;
    u32 bm1 = b - 1, minv = have ? fy_recip(bm1) : 0u;
    u64 q = 0;
    u32 i = bm1;
    while (have) {
        const u32 slot = c % FY_RING;
        if (start == 0 && !fy_wait_above(sh, &sh.produced, c, lane, err, err_bit)) {
            ok = false;
            break;
        }
        const u32 x = fy_candidate(sh, slot, lane, parity);
        const u32 A = lane >= start ? fy_accept_mask(x, i, q, nrows, bm1) : 0u;
        __syncwarp();  // the previous slot's reads of sh.A are done
        sh.A[lane] = A;
        __syncwarp();
        // every lane runs the chain on all 32 masks: E marks the accepted lanes
        u32 E = 0, s = 1;
#pragma unroll
        for (u32 L = 0; L < 32; L += 4) {
            const uint4 a4 = *(const uint4 *)&sh.A[L];
            u32 t = a4.x & s;
            E |= (u32)(t != 0) << L;
            s += t;
            t = a4.y & s;
            E |= (u32)(t != 0) << (L + 1);
            s += t;
            t = a4.z & s;
            E |= (u32)(t != 0) << (L + 2);
            s += t;
            t = a4.w & s;
            E |= (u32)(t != 0) << (L + 3);
            s += t;
        }
        if ((E >> lane) & 1u) {
            const u32 p = (bm1 - i) + __popc(E & ((1u << lane) - 1u)), ad = fy_div(p, bm1, minv);
            const u32 pos = bm1 - (p - ad * bm1);
            rows.put(q + ad, pos, x & fy_mask(pos));
        }
        if (E) {
            used = true;
            last_slot = c;
            last_lane = 31 - __clz((int)E);
            idle = 0;
        } else if (start == 0 && ++idle > 8) {  // an impossible stream: record it, stay bounded
            if (lane == 0) atomicOr(err, err_bit);
            ok = false;
            break;
        }
        const u32 p = (bm1 - i) + __popc(E), ad = fy_div(p, bm1, minv);
        if (q + ad >= nrows) {  // the run is complete (its last draw was the last accepted lane)
            do {
                have = rows.next(b, nrows);
            } while (have && (nrows == 0 || b < 2));
            if (!have) break;
            bm1 = b - 1;
            minv = fy_recip(bm1);
            q = 0;
            i = bm1;
            start = last_lane + 1;
            if (start < 32) continue;  // the same slot's later candidates open the next run
        } else {
            q += ad;
            i = bm1 - (p - ad * bm1);
        }
        __syncwarp();
        if (lane == 0) fy_publish(&sh.freed[slot], c + 1);
        c++;
        start = 0;
    }
    if (lane == 0) {
        sh.stop = 1;
        if (ok && used) {
            const u32 slot = last_slot % FY_RING;
            const u64 st[4] = {sh.st[slot][0], sh.st[slot][1], sh.st[slot][2], sh.st[slot][3]};
            fy_write_state(state, st, sh.first[slot], (int)last_lane - (int)parity);
        }
    }
}

// One CTA of FY_THREADS threads (warps 0 and 1 work) draws the rows of `rows`
// from the generator whose six state words are at `state`, and advances them.
template <class Rows>
__device__ void fy_stream(FyShared &sh, u64 *state, Rows &rows, unsigned *err, unsigned err_bit)
{
    fy_init(sh);
    const u32 warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const u32 parity = (u32)(state[4] != 0);  // numpy's buffered half opens the stream
    if (warp == 0) {
        if (lane == 0) fy_produce(sh, state, err, err_bit);
    } else if (warp == 1) {
        fy_decode_runs(sh, state, rows, err, err_bit, parity);
    }
}

// ---- one run of a small base -----------------------------------------------------------

template <class Put>
__device__ void fy_small_worker(FyShared &sh, u32 w, u32 bm1, u64 nrows, u32 parity, Put &put, unsigned *err,
                                unsigned err_bit)
{
    const u32 lane = threadIdx.x & 31, o = 32 % bm1, minv = fy_recip(bm1);
    for (u32 c = w;; c += FY_WORKERS) {
        const u32 slot = c % FY_RING;
        if (!fy_wait_above(sh, &sh.produced, c, lane, err, err_bit)) return;
        const u32 x = fy_candidate(sh, slot, lane, parity);
        // acceptance at positions 1..bm1 (bit i-1), mask level by mask level
        u32 P = 0;
        for (u32 m = 1; (1u << (m - 1)) <= bm1; m++) {
            const u32 M = (1u << m) - 1, lo = 1u << (m - 1), hi = min(M, bm1), s0 = max(lo, x & M);
            if (s0 <= hi) P |= (u32)((1ull << hi) - (1ull << (s0 - 1)));
        }
        // bit b: acceptance at position b - 31, positions taken mod bm1 into 1..bm1
        u64 X = (u64)P << o;
        for (u32 ln = bm1; ln < 64; ln <<= 1) X |= X << ln;
        if (o) X |= (u64)(P >> (bm1 - o));
        __syncwarp();  // the previous slot's reads of this worker's patterns are done
        sh.ext[w][lane] = X;
        __syncwarp();
        // lane j: the candidates from start position j + 1
        u32 E = 0;
        int pos = (int)lane + 1;
#pragma unroll
        for (u32 L = 0; L < 32; L += 2) {
            const ulonglong2 e2 = *(const ulonglong2 *)&sh.ext[w][L];
            u32 a = (u32)(e2.x >> (pos + 31)) & 1u;
            E |= a << L;
            pos -= (int)a;
            a = (u32)(e2.y >> (pos + 31)) & 1u;
            E |= a << (L + 1);
            pos -= (int)a;
        }
        if (lane < bm1) sh.E[slot][lane] = E;
        __syncwarp();  // every lane's E is in shared memory before lane 0 publishes it
        if (lane == 0) fy_publish(&sh.done[slot], c + 1);
        if (!fy_wait_above(sh, &sh.scanned, c, lane, err, err_bit)) return;
        const u32 ic = sh.start_i[slot];
        const u64 qc = sh.start_q[slot];
        const u32 Ec = sh.E[slot][ic - 1];
        if ((Ec >> lane) & 1u) {
            const u32 p = (bm1 - ic) + __popc(Ec & ((1u << lane) - 1u)), ad = fy_div(p, bm1, minv);
            const u32 ps = bm1 - (p - ad * bm1);
            if (qc + ad < nrows) put.put(qc + ad, ps, x & fy_mask(ps));
        }
        __syncwarp();
        if (lane == 0) fy_publish(&sh.freed[slot], c + 1);
    }
}

__device__ void fy_small_scan(FyShared &sh, u64 *state, u32 bm1, u64 nrows, u32 parity, unsigned *err,
                              unsigned err_bit)
{
    const u32 minv = fy_recip(bm1);
    u32 i = bm1, idle = 0;
    u64 q = 0;
    for (u32 c = 0;; c++) {
        const u32 slot = c % FY_RING;
        u32 spins = 0;
        while (fy_acquire(&sh.done[slot]) != c + 1) {
            if (sh.stop) return;  // stopped by a wait that ran out (recorded)
            if (++spins > FY_SPIN_LIMIT) {
                atomicOr(err, err_bit);
                sh.stop = 1;
                return;
            }
        }
        const u32 E = sh.E[slot][i - 1];
        sh.start_i[slot] = i;
        sh.start_q[slot] = q;
        const u32 N = __popc(E), p = (bm1 - i) + N, ad = fy_div(p, bm1, minv);
        if (q + ad >= nrows) {  // the run ends in this slot, at its need-th accepted lane
            const u64 need = (nrows - q) * bm1 - (bm1 - i);
            u32 e = E;
            for (u64 k = 1; k < need; k++) e &= e - 1;
            const u32 lane_end = __ffs(e) - 1;
            const u64 st[4] = {sh.st[slot][0], sh.st[slot][1], sh.st[slot][2], sh.st[slot][3]};
            const u32 first = sh.first[slot];
            fy_publish(&sh.scanned, c + 1);
            fy_publish(&sh.stop, 1);
            fy_write_state(state, st, first, (int)lane_end - (int)parity);
            return;
        }
        if (N == 0 && ++idle > 8) {  // an impossible stream: record it, stay bounded
            atomicOr(err, err_bit);
            sh.stop = 1;
            return;
        }
        if (N) idle = 0;
        fy_publish(&sh.scanned, c + 1);
        q += ad;
        i = bm1 - (p - ad * bm1);
    }
}

// One CTA of FY_THREADS threads draws nrows rows of Generator.permutation(b),
// 2 <= b <= FY_SMALL_MAX, nrows >= 1, through put.put(q, i, j).
template <class Put>
__device__ void fy_stream_small(FyShared &sh, u64 *state, u32 b, u64 nrows, Put &put, unsigned *err,
                                unsigned err_bit)
{
    fy_init(sh);
    const u32 warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const u32 parity = (u32)(state[4] != 0);
    if (warp == 0) {
        if (lane == 0) fy_produce(sh, state, err, err_bit);
    } else if (warp == 1) {
        if (lane == 0) fy_small_scan(sh, state, b - 1, nrows, parity, err, err_bit);
    } else if (fy_worker_of(warp) >= 0) {
        fy_small_worker(sh, (u32)fy_worker_of(warp), b - 1, nrows, parity, put, err, err_bit);
    }
}

}  // namespace
