// halton_qrng.cu -- the generalized Halton sequence of the reference's
// halton_qrng (qmctoolscl/c_funcs/halton_qrng.c:3-162; Faure and Lemieux's
// sequence as the R package qrng implements it): for point i and dimension j
// with base b = the dvec[j]-th prime, the 32 base-b digits of i, each mapped to
// (f * digit + s_k) mod b with multiplier f (1, or the generalized table) and
// random digit shift s_k = (int)(b * randu_d_32[j*32 + k]), summed by
// Horner's rule from digit 31 down, every add and divide rounded
// (halton_qrng.c:133-140).  res is d x n, dimension-major.
//
// Bit for bit with less work: the digits at and above the index's digit
// count m are zero, so the Horner steps over them are the same for every
// point with m digits.  Each CTA owns one dimension and computes, once, the
// prefix P[m] after the steps k = 31 .. m (P[0] is the reference's point 0);
// a point then needs only its own m steps, each the reference's rounded add
// and divide.  Three warps in four take them in integer arithmetic
// (qrng_step.cuh), the fourth on the FP64 unit as the reference's own two
// operations: on GB300 an FP64 divide is a sequence of several operations on a
// narrow pipe, so neither kind of unit alone keeps up, and the two run side by
// side (n = 2^20, d = 100: 2.82 ms with integer steps only, 2.51 ms with a
// quarter of the warps on FP64; a third, a fifth, a sixth, or the FP64 warps
// spread over the SM's sub-partitions, measured slower).  The digits come from
// the top down by divisions by b^k (32-bit multiply-high, exact).
#include "common.cuh"
#include "qrng_step.cuh"

namespace {

// the step with the FP64 operations, out of line, for what qstep::step leaves out
__device__ __noinline__ u64 qrng_step_hw(u64 v, u32 c, double bd)
{
    return (u64)__double_as_longlong(__ddiv_rn(__dadd_rn(__longlong_as_double((long long)v), (double)c), bd));
}

constexpr int QRNG_DIMS = 360;

// the first 360 primes (the bases of halton_qrng.c:28-35)
__constant__ int c_qrng_prime[QRNG_DIMS] = {
    2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61,
    67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113, 127, 131, 137, 139, 149, 151,
    157, 163, 167, 173, 179, 181, 191, 193, 197, 199, 211, 223, 227, 229, 233, 239, 241, 251,
    257, 263, 269, 271, 277, 281, 283, 293, 307, 311, 313, 317, 331, 337, 347, 349, 353, 359,
    367, 373, 379, 383, 389, 397, 401, 409, 419, 421, 431, 433, 439, 443, 449, 457, 461, 463,
    467, 479, 487, 491, 499, 503, 509, 521, 523, 541, 547, 557, 563, 569, 571, 577, 587, 593,
    599, 601, 607, 613, 617, 619, 631, 641, 643, 647, 653, 659, 661, 673, 677, 683, 691, 701,
    709, 719, 727, 733, 739, 743, 751, 757, 761, 769, 773, 787, 797, 809, 811, 821, 823, 827,
    829, 839, 853, 857, 859, 863, 877, 881, 883, 887, 907, 911, 919, 929, 937, 941, 947, 953,
    967, 971, 977, 983, 991, 997, 1009, 1013, 1019, 1021, 1031, 1033, 1039, 1049, 1051, 1061, 1063, 1069,
    1087, 1091, 1093, 1097, 1103, 1109, 1117, 1123, 1129, 1151, 1153, 1163, 1171, 1181, 1187, 1193, 1201, 1213,
    1217, 1223, 1229, 1231, 1237, 1249, 1259, 1277, 1279, 1283, 1289, 1291, 1297, 1301, 1303, 1307, 1319, 1321,
    1327, 1361, 1367, 1373, 1381, 1399, 1409, 1423, 1427, 1429, 1433, 1439, 1447, 1451, 1453, 1459, 1471, 1481,
    1483, 1487, 1489, 1493, 1499, 1511, 1523, 1531, 1543, 1549, 1553, 1559, 1567, 1571, 1579, 1583, 1597, 1601,
    1607, 1609, 1613, 1619, 1621, 1627, 1637, 1657, 1663, 1667, 1669, 1693, 1697, 1699, 1709, 1721, 1723, 1733,
    1741, 1747, 1753, 1759, 1777, 1783, 1787, 1789, 1801, 1811, 1823, 1831, 1847, 1861, 1867, 1871, 1873, 1877,
    1879, 1889, 1901, 1907, 1913, 1931, 1933, 1949, 1951, 1973, 1979, 1987, 1993, 1997, 1999, 2003, 2011, 2017,
    2027, 2029, 2039, 2053, 2063, 2069, 2081, 2083, 2087, 2089, 2099, 2111, 2113, 2129, 2131, 2137, 2141, 2143,
    2153, 2161, 2179, 2203, 2207, 2213, 2221, 2237, 2239, 2243, 2251, 2267, 2269, 2273, 2281, 2287, 2293, 2297,
    2309, 2311, 2333, 2339, 2341, 2347, 2351, 2357, 2371, 2377, 2381, 2383, 2389, 2393, 2399, 2411, 2417, 2423,
};

// the scrambling multipliers of the generalized sequence, one per prime
// (halton_qrng.c:37-60): a published table that the parity needs as it is
__constant__ int c_qrng_mult[QRNG_DIMS] = {
    1, 1, 3, 3, 4, 9, 7, 5, 9, 18, 18, 8, 13, 31, 9, 19, 36, 33,
    21, 44, 43, 61, 60, 56, 26, 71, 32, 77, 26, 95, 92, 47, 29, 61, 57, 69,
    115, 63, 92, 31, 104, 126, 50, 80, 55, 152, 114, 80, 83, 97, 95, 150, 148, 55,
    80, 192, 71, 76, 82, 109, 105, 173, 58, 143, 56, 177, 203, 239, 196, 143, 278, 227,
    87, 274, 264, 84, 226, 163, 231, 177, 95, 116, 165, 131, 156, 105, 188, 142, 105, 125,
    269, 292, 215, 182, 294, 152, 148, 144, 382, 194, 346, 323, 220, 174, 133, 324, 215, 246,
    159, 337, 254, 423, 484, 239, 440, 362, 464, 376, 398, 174, 149, 418, 306, 282, 434, 196,
    458, 313, 512, 450, 161, 315, 441, 549, 555, 431, 295, 557, 172, 343, 472, 604, 297, 524,
    251, 514, 385, 531, 663, 674, 255, 519, 324, 391, 394, 533, 253, 717, 651, 399, 596, 676,
    425, 261, 404, 691, 604, 274, 627, 777, 269, 217, 599, 447, 581, 640, 666, 595, 669, 686,
    305, 460, 599, 335, 258, 649, 771, 619, 666, 669, 707, 737, 854, 925, 818, 424, 493, 463,
    535, 782, 476, 451, 520, 886, 340, 793, 390, 381, 274, 500, 581, 345, 363, 1024, 514, 773,
    932, 556, 954, 793, 294, 863, 393, 827, 527, 1007, 622, 549, 613, 799, 408, 856, 601, 1072,
    938, 322, 1142, 873, 629, 1071, 1063, 1205, 596, 973, 984, 875, 918, 1133, 1223, 933, 1110, 1228,
    1017, 701, 480, 678, 1172, 689, 1138, 1022, 682, 613, 635, 984, 526, 1311, 459, 1348, 477, 716,
    1075, 682, 1245, 401, 774, 1026, 499, 1314, 743, 693, 1282, 1003, 1181, 1079, 765, 815, 1350, 1144,
    1449, 718, 805, 1203, 1173, 737, 562, 579, 701, 1104, 1105, 1379, 827, 1256, 759, 540, 1284, 1188,
    776, 853, 1140, 445, 1265, 802, 932, 632, 1504, 856, 1229, 1619, 774, 1229, 1300, 1563, 1551, 1265,
    905, 1333, 493, 913, 1397, 1250, 612, 1251, 1765, 1303, 595, 981, 671, 1403, 820, 1404, 1661, 973,
    1340, 1015, 1649, 855, 1834, 1621, 1704, 893, 1033, 721, 1737, 1507, 1851, 1006, 994, 923, 872, 1860,
};

constexpr u32 QRNG_THREADS = 256;

// eight CTAs per SM (32 registers): each point's digit steps are one dependent chain, so
// occupancy beats the few spilled registers (2, 3, 4, 6 CTAs per SM measured slower)
__global__ void __launch_bounds__(QRNG_THREADS, 8) halton_qrng_kernel(int n, int n0, int generalized, double *res,
                                                                   const double *randu, const int *dvec,
                                                                   unsigned *err)
{
    __shared__ double P[33];          // Horner prefix after the steps k = 31 .. m
    __shared__ u32 s[32];             // digit shifts
    __shared__ FastDiv32 pw[33];      // division by b^k, k < kmax
    __shared__ u64 pwv[33];           // b^k (capped above 2^32)
    __shared__ int b_s, f_s, ok_s;
    const int j = blockIdx.y;
    if (threadIdx.x == 0) {
        const int idx = dvec[j];
        ok_s = idx >= 0 && idx < QRNG_DIMS;
        if (!ok_s) atomicOr(err, 1u);  // halton_qrng.c:70 would read outside its tables
        b_s = ok_s ? c_qrng_prime[idx] : 2;
        f_s = ok_s ? (generalized ? c_qrng_mult[idx] : 1) : 1;
    }
    __syncthreads();
    if (!ok_s) return;
    const int b = b_s;
    const double bd = (double)b;
    if (threadIdx.x < 32) {
        // halton_qrng.c:73: (int)(base * u), then stored as unsigned
        s[threadIdx.x] = (u32)__double2int_rz(__dmul_rn(bd, randu[(u64)j * 32 + threadIdx.x]));
    }
    if (threadIdx.x == 32) {
        u64 v = 1;
        for (int k = 0; k < 33; k++) {
            pwv[k] = v;
            pw[k] = fastdiv32_make((u32)(v >= 2 && v < (1ull << 32) ? v : 2u));  // k = 0 divides by 1 (unused)
            v = v < (1ull << 32) ? v * (u64)b : v;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // halton_qrng.c:74-78: u += s_k; u /= base, k = 31 .. 0
        double u = 0.0;
        P[32] = u;
        for (int k = 31; k >= 0; k--) {
            u = __ddiv_rn(__dadd_rn(u, (double)s[k]), bd);
            P[k] = u;
        }
    }
    __syncthreads();
    const FastDiv32 fb = fastdiv32_make((u32)b);
    const qstep::Div qd = qstep::make_div((u32)b);
    const u32 f = (u32)f_s;
    double *out = res + (u64)j * (u64)n;
    for (u64 q = (u64)blockIdx.x * QRNG_THREADS + threadIdx.x; q < (u64)n; q += (u64)gridDim.x * QRNG_THREADS) {
        const u32 t = (u32)(int)((long long)n0 + (long long)q);  // halton_qrng.c:110: tmp = i
        const bool fp64 = ((q >> 5) & 3u) == 0;                   // the warp's steps on the FP64 unit
        int m = 0;  // base-b digit count of t (at most 32)
        while (m < 32 && pwv[m + 1] <= (u64)t && pwv[m + 1] < (1ull << 32)) m++;
        if (t) m++;
        u64 v = (u64)__double_as_longlong(P[m]);
        for (int k = m - 1; k >= 0; k--) {
            const u32 top = k ? fd_div(pw[k], t) : t;       // t / b^k
            const u32 dig = top - fd_div(fb, top) * (u32)b;  // its lowest digit: digit k of t
            const u32 c = fd_mod(fb, f * dig + s[k]);       // halton_qrng.c:135
            u64 o;                                          // halton_qrng.c:135-136: v = RN(RN(v + c) / b)
            if (fp64 || !qstep::step(v, c, qd, o)) o = qrng_step_hw(v, c, bd);
            v = o;
        }
        out[q] = __longlong_as_double((long long)v);
    }
}

}  // namespace

extern "C" {

int qmc_halton_qrng(int n, int d, int n0, int generalized, double *res, const double *randu_d_32, const int *dvec,
                    qmc_stream_t s)
{
    if (n <= 0 || d <= 0) return QMC_OK;  // the reference's loops do not run
    QMC_REQUIRE_DOMAIN(d <= QRNG_DIMS, "halton_qrng: d = %d above 360 (the reference's tables hold 360 dimensions)",
                       d);
    QMC_REQUIRE_DOMAIN((long long)n + (long long)n0 <= 2147483647LL,
                       "halton_qrng: n + n0 must stay below 2^31 (the reference's int index)");
    QMC_REQUIRE(res && randu_d_32 && dvec, "halton_qrng: null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    // about four waves of CTAs (eight per SM) over all dimensions, at least 64 per dimension:
    // every CTA builds its dimension's tables first (a serial chain of FP64 divides), so
    // fewer, longer CTAs cost less than one per few points (153 per dimension at d = 100
    // measured 3 % slower than 64)
    unsigned per_dim = (unsigned)(qmcgb::sm_count() * 8 * 4 / d);
    if (per_dim < 64) per_dim = 64;
    if (per_dim > (unsigned)qmcgb::sm_count() * 8) per_dim = (unsigned)qmcgb::sm_count() * 8;
    const unsigned gx = qmcgb::grid_for((u64)n, QRNG_THREADS, per_dim);
    halton_qrng_kernel<<<dim3(gx, (unsigned)d, 1), QRNG_THREADS, 0, QMC_STREAM(s)>>>(n, n0, generalized, res,
                                                                                       randu_d_32, dvec, err);
    return qmcgb::launch_status("halton_qrng");
}

}  // extern "C"
