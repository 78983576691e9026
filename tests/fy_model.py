"""A pure-Python model of the permutation-stream decoder of
qmctoolscl_gb300/csrc/fy_stream.cuh, step for step, for the CPU tests.

One producer steps numpy's SFC64 generator, 16 64-bit outputs per slot of
32 candidates (32-bit halves, low half first, after the half numpy had
buffered); a 32-lane decoder takes a slot at a time: the table of states
after k accepts (row q, position i of numpy's Fisher-Yates), each lane's
acceptance mask A_L over those states, the one-hot count chain
s += A_L & s, the stores of accepted lanes, runs of rows that end inside a
slot (the slot's later lanes open the next run), and at the end the state
replayed to where numpy leaves it.  Test infrastructure only.
"""
from .nus_model import Sfc64

M32 = 0xFFFFFFFF


def mask_of(i):
    return (1 << i.bit_length()) - 1


def decode(words, runs):
    """words: the six SFC64 state words; runs: [(b, nrows)].  Returns the
    rows of swap indices (a list per run of rows, entry i = j_i, entry 0
    unused) and the six state words after the last candidate used."""
    parity = 1 if int(words[4]) else 0
    prod = Sfc64(words)
    carry = int(words[5]) & M32
    slots = []  # (state a, b, c, w before the slot, opening half, 16 outputs)

    def slot(c):
        nonlocal carry
        while len(slots) <= c:
            st = (prod.a, prod.b, prod.c, prod.w)
            raw = [prod.next64() for _ in range(16)]
            slots.append((st, carry, raw))
            carry = raw[15] >> 32
        return slots[c]

    def cand(c, lane):
        _st, first, raw = slot(c)
        h = lane - parity
        if h < 0:
            return first
        return (raw[h // 2] >> (32 * (h & 1))) & M32

    out = [[[0] * b for _ in range(n)] for b, n in runs]
    run = 0
    while run < len(runs) and (runs[run][1] == 0 or runs[run][0] < 2):
        run += 1
    used, last = False, (0, 0)
    c, start = 0, 0
    q = 0
    i = runs[run][0] - 1 if run < len(runs) else 0
    while run < len(runs):
        b, nrows = runs[run]
        bm1 = b - 1
        xs = [cand(c, L) for L in range(32)]
        tab = []
        for k in range(33):
            p = (bm1 - i) + k
            ad = p // bm1
            ik = bm1 - (p - ad * bm1)
            past = q + ad >= nrows
            tab.append((-1 if past else ik, 0 if past else mask_of(ik), ad))
        A = [0] * 32
        for L in range(start, 32):
            for k in range(32):
                ti, tm, _ = tab[k]
                if (xs[L] & tm) <= ti:
                    A[L] |= 1 << k
        s, cnts = 1, []
        for L in range(32):
            cnts.append(s.bit_length() - 1)
            s = (s + (A[L] & s)) & M32
        E = 0
        for L in range(32):
            cn = cnts[L]
            if (A[L] >> cn) & 1:
                ti, tm, ad = tab[cn]
                out[run][q + ad][ti] = xs[L] & tm
                E |= 1 << L
        total = cnts[31] + ((A[31] >> cnts[31]) & 1)
        if E:
            used, last = True, (c, E.bit_length() - 1)
        elif start == 0:
            raise AssertionError("a slot with no accepted candidate")
        if tab[total][0] < 0:  # the run is complete
            run += 1
            while run < len(runs) and (runs[run][1] == 0 or runs[run][0] < 2):
                run += 1
            if run == len(runs):
                break
            q, i = 0, runs[run][0] - 1
            start = last[1] + 1
            if start < 32:
                continue
        else:
            q += tab[total][2]
            i = tab[total][0]
        c += 1
        start = 0
    words = [int(x) for x in words]
    if used:
        st, first, _raw = slot(last[0])
        h = last[1] - parity
        if h < 0:
            words = list(st) + [0, first]
        else:
            r = Sfc64(list(st) + [0, 0])
            y = 0
            for _ in range(h // 2 + 1):
                y = r.next64()
            words = [r.a, r.b, r.c, r.w, 0 if h & 1 else 1, y >> 32]
    return out, words


def permutation_of(row):
    """numpy's Fisher-Yates swaps of a row of indices, applied to arange(b)."""
    b = len(row)
    arr = list(range(b))
    for i in range(b - 1, 0, -1):
        j = row[i]
        arr[i], arr[j] = arr[j], arr[i]
    return arr


def accept_mask_segments(x, i, q, nrows, bm1):
    """Acceptance of candidate x over the next 32 states (bit k: accepted
    after k accepts), from the row state (row q, position i) by segments of
    equal mask, as the general decoder computes it."""
    A, k, pos, row = 0, 0, i, q
    while k < 32 and row < nrows:
        M = mask_of(pos)
        lo = (M >> 1) + 1
        ln = min(pos - lo + 1, 32 - k)
        tau = x & M
        if pos >= tau:
            n_acc = min(ln, pos - tau + 1)
            A |= ((1 << n_acc) - 1) << k
        k += ln
        pos -= ln
        if pos == 0:
            pos, row = bm1, row + 1
    return A & M32


def decode_runs(words, runs):
    """The general decoder: per slot the segment masks, the count chain over
    all 32 lanes' masks, the accepted lanes' stores; runs of rows of any base
    one after another.  Same results as decode()."""
    parity = 1 if int(words[4]) else 0
    prod = Sfc64(words)
    carry = int(words[5]) & M32
    slots = []

    def slot(c):
        nonlocal carry
        while len(slots) <= c:
            st = (prod.a, prod.b, prod.c, prod.w)
            raw = [prod.next64() for _ in range(16)]
            slots.append((st, carry, raw))
            carry = raw[15] >> 32
        return slots[c]

    def cand(c, lane):
        _st, first, raw = slot(c)
        h = lane - parity
        return first if h < 0 else (raw[h // 2] >> (32 * (h & 1))) & M32

    def skip(run):
        while run < len(runs) and (runs[run][1] == 0 or runs[run][0] < 2):
            run += 1
        return run

    out = [[[0] * b for _ in range(n)] for b, n in runs]
    run = skip(0)
    used, last = False, (0, 0)
    c, start, q = 0, 0, 0
    i = runs[run][0] - 1 if run < len(runs) else 0
    while run < len(runs):
        b, nrows = runs[run]
        bm1 = b - 1
        xs = [cand(c, L) for L in range(32)]
        A = [accept_mask_segments(xs[L], i, q, nrows, bm1) if L >= start else 0 for L in range(32)]
        s, E = 1, 0
        for L in range(32):
            t = A[L] & s
            if t:
                E |= 1 << L
            s = (s + t) & M32
        for L in range(32):
            if (E >> L) & 1:
                cn = bin(E & ((1 << L) - 1)).count("1")
                p = (bm1 - i) + cn
                ad = p // bm1
                pos = bm1 - (p - ad * bm1)
                out[run][q + ad][pos] = xs[L] & mask_of(pos)
        total = bin(E).count("1")
        if E:
            used, last = True, (c, E.bit_length() - 1)
        elif start == 0:
            raise AssertionError("a slot with no accepted candidate")
        p = (bm1 - i) + total
        ad = p // bm1
        if q + ad >= nrows:
            run = skip(run + 1)
            if run == len(runs):
                break
            q, i = 0, runs[run][0] - 1
            start = last[1] + 1
            if start < 32:
                continue
        else:
            q += ad
            i = bm1 - (p - ad * bm1)
        c += 1
        start = 0
    words = [int(x) for x in words]
    if used:
        words = _replay(slot(last[0]), last[1] - parity, words)
    return out, words


def _replay(slot_rec, h, words):
    st, first, _raw = slot_rec
    if h < 0:
        return list(st) + [0, first]
    r = Sfc64(list(st) + [0, 0])
    y = 0
    for _ in range(h // 2 + 1):
        y = r.next64()
    return [r.a, r.b, r.c, r.w, 0 if h & 1 else 1, y >> 32]


def position_pattern(x, bm1):
    """Acceptance of candidate x at every position i = 1..bm1 (bit i-1), for
    bm1 <= 32, by mask levels."""
    P, m = 0, 1
    while (1 << (m - 1)) <= bm1:
        M = (1 << m) - 1
        lo, hi = 1 << (m - 1), min(M, bm1)
        st = max(lo, x & M)
        if st <= hi:
            P |= ((1 << hi) - (1 << (st - 1)))
        m += 1
    return P & M32


def periodic64(P, bm1):
    """Bit b = acceptance at position b - 31, positions taken mod bm1 into 1..bm1."""
    o = 32 % bm1
    X = (P << o) & ((1 << 64) - 1)
    ln = bm1
    while ln < 64:
        X = (X | (X << ln)) & ((1 << 64) - 1)
        ln *= 2
    if o:
        X |= P >> (bm1 - o)
    return X


def decode_small(words, b, nrows):
    """The small-base decoder (2 <= b <= 33, one run): per slot, for every
    start position j+1 the events E_j of a 32-step chain over the lanes'
    periodic patterns; the scan chains one lookup per slot; the accepted
    lanes store from the slot's start state."""
    parity = 1 if int(words[4]) else 0
    prod = Sfc64(words)
    carry = int(words[5]) & M32
    bm1 = b - 1
    out = [[0] * b for _ in range(nrows)]
    if nrows == 0 or b < 2:
        return out, [int(x) for x in words]
    i, q, c = bm1, 0, 0
    while True:
        st = (prod.a, prod.b, prod.c, prod.w)
        raw = [prod.next64() for _ in range(16)]
        rec = (st, carry, raw)
        carry = raw[15] >> 32
        xs = []
        for L in range(32):
            h = L - parity
            xs.append(rec[1] if h < 0 else (raw[h // 2] >> (32 * (h & 1))) & M32)
        ext = [periodic64(position_pattern(x, bm1), bm1) for x in xs]
        Es = []
        for j in range(bm1):
            pos, E = j + 1, 0
            for L in range(32):
                a = (ext[L] >> (pos + 31)) & 1
                E |= a << L
                pos -= a
            Es.append(E)
        E = Es[i - 1]
        # outputs of this slot from its start state (i, q)
        for L in range(32):
            if (E >> L) & 1:
                cn = bin(E & ((1 << L) - 1)).count("1")
                p = (bm1 - i) + cn
                ad = p // bm1
                pos = bm1 - (p - ad * bm1)
                if q + ad < nrows:
                    out[q + ad][pos] = xs[L] & mask_of(pos)
        N = bin(E).count("1")
        p = (bm1 - i) + N
        ad = p // bm1
        if q + ad >= nrows:
            need = (nrows - q) * bm1 - (bm1 - i)
            e = E
            for _ in range(need - 1):
                e &= e - 1
            lane = (e & -e).bit_length() - 1
            return out, _replay(rec, lane - parity, words)
        q += ad
        i = bm1 - (p - ad * bm1)
        c += 1
