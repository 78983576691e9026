"""A pure-Python model of how the GPU computes the nested uniform scrambles
(qmctoolscl_gb300/csrc/nus.cu, gdn_nus.cu, nus_dev.cuh), for the CPU tests.

The reference (qmctoolscl/rand_funcs.py:162-253 and 262-356) walks one tree
per generator point by point.  The GPU form rests on three facts: the root
is a phantom point of zero key drawn first; point v draws for the levels
below L_v, its longest common prefix with any earlier point (nothing for a
repeated point); and level k of a point's result comes from the draw of the
earliest point sharing its first k key bits (digits).  This model computes
exactly what the kernels do, sequentially: a stable sort of (key, point),
the prefix lengths of sorted neighbours, Apetrei's bottom-up radix-tree pass
with the earliest point per node (run with its threads interleaved at random,
one atomic exchange per step), the draws in point order from numpy's SFC64
rules, and each point's walk up its ancestors.  Test infrastructure only.
"""
import random

M64 = (1 << 64) - 1
NONE = 0xFFFFFFFF


class Sfc64:
    """numpy's SFC64 with its buffered 32-bit halves; six state words."""

    def __init__(self, words):
        self.a, self.b, self.c, self.w, self.has, self.half = (int(x) for x in words)

    def words(self):
        return [self.a, self.b, self.c, self.w, self.has, self.half]

    def next64(self):
        out = (self.a + self.b + self.w) & M64
        self.w = (self.w + 1) & M64
        self.a = self.b ^ (self.b >> 11)
        self.b = (self.c + (self.c << 3)) & M64
        self.c = ((((self.c << 24) | (self.c >> 40)) & M64) + out) & M64
        return out

    def next32(self):
        if self.has:
            self.has = 0
            return self.half
        x = self.next64()
        self.has, self.half = 1, x >> 32
        return x & 0xFFFFFFFF

    def bits(self, m):
        """Generator.integers(0, 2**m), and random_tbit_uint64s for m = 64"""
        if m == 0:
            return 0
        if m <= 32:
            return self.next32() >> (32 - m)
        x = self.next64()
        return x if m == 64 else x >> (64 - m)

    def interval(self, mx):
        """numpy's random_interval: masked rejection"""
        if mx == 0:
            return 0
        mask = mx
        for sh in (1, 2, 4, 8, 16, 32):
            mask |= mask >> sh
        while True:
            v = (self.next32() if mx <= 0xFFFFFFFF else self.next64()) & mask
            if v <= mx:
                return v

    def permutation(self, b):
        row = list(range(b))
        for i in range(b - 1, 0, -1):
            j = self.interval(i)
            row[i], row[j] = row[j], row[i]
        return row


def _bottom_up(lam, order, rnd):
    """Apetrei's pass over N sorted entries (lam[i]: prefix length between i and
    i+1): parents, each internal node's earliest point, and the raw prefix
    length at which each later point first meets an earlier one.  Threads are
    generators stepped in a random order; each step is one atomic exchange."""
    N = len(order)
    last = N - 2
    slot, pleaf, pint, minv, L = {}, [None] * N, [None] * (N - 1), [None] * (N - 1), {}

    def lamv(i):
        return -1 if i < 0 or i > last else lam[i]

    def settle(node, a, b):
        minv[node] = min(a, b)
        assert max(a, b) not in L
        L[max(a, b)] = lam[node]

    def thread(p):
        lo = hi = p
        left = lo == 0 or (hi <= last and lamv(hi) > lamv(lo - 1))
        par = hi if left else lo - 1
        pleaf[p] = par
        mn = order[p]
        if not left and (p - 1 == 0 or lamv(p - 1) > lamv(p - 2)):
            return
        if left and (p == last or lamv(p + 1) < lamv(p)):
            b = order[p + 1]
            settle(p, mn, b)
            mn, node, hi = min(mn, b), p, p + 1
        else:
            yield
            prev = slot.get(par)
            slot[par] = (lo if left else hi, mn)
            if prev is None:
                return
            if left:
                hi = prev[0]
            else:
                lo = prev[0]
            settle(par, mn, prev[1])
            mn, node = min(mn, prev[1]), par
        while True:
            if lo == 0 and hi == last + 1:
                pint[node] = NONE
                return
            left = lo == 0 or (hi <= last and lamv(hi) > lamv(lo - 1))
            par = hi if left else lo - 1
            pint[node] = par
            yield
            prev = slot.get(par)
            slot[par] = (lo if left else hi, mn)
            if prev is None:
                return
            if left:
                hi = prev[0]
            else:
                lo = prev[0]
            settle(par, mn, prev[1])
            mn, node = min(mn, prev[1]), par

    threads = [thread(p) for p in range(N)]
    live = list(range(N))
    while live:
        k = rnd.randrange(len(live))
        try:
            next(threads[live[k]])
        except StopIteration:
            live.pop(k)
    return pleaf, pint, minv, L


def _clz64(x):
    return 64 - x.bit_length()


def _clz32(x):
    return 32 - x.bit_length()


def dnb2_scramble(r, n, d, r_x, tmax, tmax_new, states, xb, seed=0):
    """dnb2_nested_uniform_scramble on fresh trees; states (r*d lists of six
    words) are advanced in place; returns xrb as nested lists [l][i][j]."""
    T = tmax_new
    td = (tmax_new - tmax) & M64
    mask = M64 if T >= 64 else (1 << T) - 1
    rnd = random.Random(seed)
    out = [[[0] * d for _ in range(n)] for _ in range(r)]
    for s in range(r * d):
        l, j = divmod(s, d)
        full = [0] + [0 if td >= 64 else (int(xb[l % r_x][i][j]) << td) & M64 for i in range(n)]
        key = [x & mask for x in full]
        N = n + 1
        L = {}
        if n:
            order = sorted(range(N), key=lambda q: (key[q], q))
            k = [key[q] for q in order]

            def delta(a, b):
                x = k[a] ^ k[b]
                return _clz64(x) - (64 - T) if x else T + _clz32(order[a] ^ order[b])

            lam = [delta(p, p + 1) for p in range(N - 1)]
            pleaf, pint, minv, L = _bottom_up(lam, order, rnd)
        g = Sfc64(states[s])
        draw = [g.bits(T)] + [0] * n
        for v in range(1, N):
            draw[v] = g.bits(0 if L[v] >= T - 1 else T - 1 - L[v])
        states[s] = g.words()
        if not n:
            continue

        def band(kmin, kmax):
            kmax = min(kmax, T - 1)
            if kmin > kmax:
                return 0
            return (((1 << (T - kmin)) - 1) >> (T - 1 - kmax)) << (T - 1 - kmax)

        for p in range(N):
            v = order[p]
            if v == 0:
                continue
            P = pleaf[p]
            sh = draw[v] & band(lam[P] + 1, T - 1)
            u = P
            while u != NONE:
                Q = pint[u]
                sh |= draw[minv[u]] & band((lam[Q] if Q != NONE else -1) + 1, lam[u])
                u = Q
            out[l][v - 1][j] = full[v] ^ sh
    return out


def gdn_scramble(r, n, d, r_x, r_b, tmax, tmax_new, bases, states, xdig, seed=0):
    """gdn_nested_uniform_scramble on fresh trees; returns xrdig [l][i][j][t]."""
    rnd = random.Random(seed)
    out = [[[[0] * tmax_new for _ in range(d)] for _ in range(n)] for _ in range(r)]
    for s in range(r * d):
        l, j = divmod(s, d)
        b = int(bases[l % r_b][j])
        w = max(1, (b - 1).bit_length())
        Tg = tmax * w
        digits = [[0] * tmax] + [[int(x) for x in xdig[l % r_x][i][j]] for i in range(n)]
        key = [sum(dg << (128 - (t + 1) * w) for t, dg in enumerate(row)) for row in digits]
        N = n + 1
        L = {}
        if n:
            order = sorted(range(N), key=lambda q: (key[q], q))

            def delta(a, c):
                x = key[order[a]] ^ key[order[c]]
                return 128 - x.bit_length() if x else Tg + _clz32(order[a] ^ order[c])

            lam = [delta(p, p + 1) for p in range(N - 1)]
            pleaf, pint, minv, L = _bottom_up(lam, order, rnd)

        def ldig(v):
            return tmax_new if L[v] >= Tg else L[v] // w

        first = [0] + [ldig(v) + 1 for v in range(1, N)]
        g = Sfc64(states[s])
        perms = [[g.permutation(b) for _ in range(tmax_new)]]
        for v in range(1, N):
            perms.append([g.permutation(b) for _ in range(max(0, tmax_new - first[v]))])
        states[s] = g.words()
        if not n:
            continue
        for p in range(N):
            v = order[p]
            if v == 0:
                continue
            owner, parent = v, pleaf[p]
            dP = lam[parent] if parent != NONE else -1
            for t in range(tmax_new - 1, -1, -1):
                kbits = min(t, tmax) * w
                while parent != NONE and dP >= kbits:
                    owner, parent = minv[parent], pint[parent]
                    dP = lam[parent] if parent != NONE else -1
                xt = digits[v][t] if t < tmax else 0
                out[l][v - 1][j][t] = perms[owner][t - first[owner]][xt]
    return out
