/*
 * qmc_oracle.c -- CPU restatement of the QMCToolsCL point-generation and
 * fast-transform C backend.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the GPU kernels
 * of qmctoolscl_gb300 are checked against it, and bench.py times it as the
 * CPU baseline ("port").  Nothing in the product library links, loads or
 * calls it.
 *
 * Each function restates one reference function, named in its comment as
 * qmctoolscl/c_funcs/<file>.c:<lines>.  Every function takes the reference's
 * scalar arguments minus the three batch-size arguments (the reference's C
 * wrapper sets them to the full extents, qmctoolscl/util.py:107, so every
 * loop below runs over the whole range).  Loop order and the order of every
 * floating-point operation follow the reference, because both decide the
 * rounded results and the CPU timing.
 *
 * Build with -ffp-contract=off: aarch64 gcc would otherwise fuse a*b+c into
 * an FMA and change the rounding of gdn_integer_to_float and the transforms.
 *
 * Shift counts.  Several reference loops shift a 64-bit word by a count that
 * can reach 64 or wrap below zero for unusual arguments (undefined in C).
 * gcc on x86-64 and aarch64 emits a hardware shift that uses the count mod
 * 64; the oracle writes that behaviour out (SHL/SHR below) so it is defined.
 */
#include <math.h>
#include <stdint.h>

typedef uint64_t u64;

#define SHL(v, s) ((u64)(v) << ((u64)(s) & 63u))
#define SHR(v, s) ((u64)(v) >> ((u64)(s) & 63u))

#if defined(__GNUC__)
#define ORACLE_API __attribute__((visibility("default")))
#else
#define ORACLE_API
#endif

/* ------------------------------------------------------------------------ */
/* rank-1 lattices                                                          */
/* ------------------------------------------------------------------------ */

/* qmctoolscl/c_funcs/lat_gen_linear.c:3-33 */
ORACLE_API void oracle_lat_gen_linear(u64 r, u64 n, u64 d, const u64 *g, double *x)
{
    const double nd = (double)n;
    for (u64 i = 0; i < n; i++) {
        const double frac_i = i / nd;
        for (u64 j = 0; j < d; j++)
            for (u64 l = 0; l < r; l++)
                x[l * n * d + i * d + j] = fmod((double)g[l * d + j] * frac_i, 1.0);
    }
}

/* Shared start of the van der Corput recurrence of lat_gen_natural.c:23-34
 * and lat_gen_gray.c:23-34: p = ceil(log2(n0+1)) bits, v = the Gray code of
 * n0 written bit-reversed into p bits. */
static void lat_vdc_start(u64 n0, u64 *p_out, u64 *v_out)
{
    u64 p = (u64)ceil(log2((double)n0 + 1));
    u64 v = 0, t = n0 ^ (n0 >> 1), b = 0;
    for (; t > 0; t >>= 1, b++)
        if (t & 1) v += SHL(1, p - b - 1);
    *p_out = p;
    *v_out = v;
}

/* One step of lat_gen_natural.c:48-57 / lat_gen_gray.c:46-55: advance
 * (p, v) from index itrue-1 to itrue. */
static void lat_vdc_step(u64 itrue, u64 *p, u64 *v)
{
    if ((itrue & (itrue - 1)) == 0) { /* itrue is a power of two */
        *p += 1;
        *v <<= 1;
    }
    u64 b = 0;
    while (!((itrue >> b) & 1)) b++;
    *v ^= SHL(1, *p - b - 1);
}

/* qmctoolscl/c_funcs/lat_gen_natural.c:3-58 */
ORACLE_API void oracle_lat_gen_natural(u64 r, u64 n, u64 d, u64 n_start, const u64 *g, double *x)
{
    u64 p, v;
    lat_vdc_start(n_start, &p, &v);
    for (u64 i = 0; i < n; i++) {
        const double frac_i = ldexp((double)v, -(int)p);
        const u64 itrue = i + n_start;
        const u64 row = ((itrue ^ (itrue >> 1)) - n_start) * d;
        for (u64 j = 0; j < d; j++)
            for (u64 l = 0; l < r; l++)
                x[l * n * d + row + j] = fmod((double)g[l * d + j] * frac_i, 1.0);
        lat_vdc_step(i + n_start + 1, &p, &v);
    }
}

/* qmctoolscl/c_funcs/lat_gen_gray.c:3-56 */
ORACLE_API void oracle_lat_gen_gray(u64 r, u64 n, u64 d, u64 n_start, const u64 *g, double *x)
{
    u64 p, v;
    lat_vdc_start(n_start, &p, &v);
    for (u64 i = 0; i < n; i++) {
        const double frac_i = ldexp((double)v, -(int)p);
        for (u64 j = 0; j < d; j++)
            for (u64 l = 0; l < r; l++)
                x[l * n * d + i * d + j] = fmod((double)g[l * d + j] * frac_i, 1.0);
        lat_vdc_step(i + n_start + 1, &p, &v);
    }
}

/* qmctoolscl/c_funcs/lat_shift_mod_1.c:3-35 */
ORACLE_API void oracle_lat_shift_mod_1(u64 r, u64 n, u64 d, u64 r_x, const double *x,
                                       const double *shifts, double *xr)
{
    const u64 nelem_x = r_x * n * d;
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++) {
                const u64 idx = l * n * d + i * d + j;
                xr[idx] = fmod(x[idx % nelem_x] + shifts[l * d + j], 1.0);
            }
}

/* ------------------------------------------------------------------------ */
/* digital nets in base 2                                                   */
/* ------------------------------------------------------------------------ */

/* Shared body of dnb2_gen_natural.c:23-69 and dnb2_gen_gray.c:23-68.  The
 * first point is the XOR of the columns picked by the bits of its Gray code;
 * each later point flips the column picked by the lowest set bit of its
 * index.  Natural order writes point i at row gray(i)-n_start, Gray order at
 * row i-n_start. */
static void dnb2_gen(u64 r, u64 n, u64 d, u64 n_start, u64 mmax, const u64 *C, u64 *xb,
                     int natural)
{
    u64 itrue = n_start;
    u64 t = itrue ^ (itrue >> 1);
    u64 prev = natural ? (t - n_start) * d : 0;
    if (n > 0) {
        for (u64 j = 0; j < d; j++)
            for (u64 l = 0; l < r; l++)
                xb[l * n * d + prev + j] = 0;
        for (u64 b = 0; t > 0; t >>= 1, b++)
            if (t & 1)
                for (u64 j = 0; j < d; j++)
                    for (u64 l = 0; l < r; l++)
                        xb[l * n * d + prev + j] ^= C[l * d * mmax + j * mmax + b];
    }
    for (u64 i = 1; i < n; i++) {
        itrue = i + n_start;
        const u64 cur = natural ? ((itrue ^ (itrue >> 1)) - n_start) * d : i * d;
        u64 b = 0;
        while (!((itrue >> b) & 1)) b++;
        for (u64 j = 0; j < d; j++)
            for (u64 l = 0; l < r; l++)
                xb[l * n * d + cur + j] = xb[l * n * d + prev + j] ^ C[l * d * mmax + j * mmax + b];
        prev = cur;
    }
}

/* qmctoolscl/c_funcs/dnb2_gen_natural.c:3-70 */
ORACLE_API void oracle_dnb2_gen_natural(u64 r, u64 n, u64 d, u64 n_start, u64 mmax, const u64 *C,
                                        u64 *xb)
{
    dnb2_gen(r, n, d, n_start, mmax, C, xb, 1);
}

/* qmctoolscl/c_funcs/dnb2_gen_gray.c:3-69 */
ORACLE_API void oracle_dnb2_gen_gray(u64 r, u64 n, u64 d, u64 n_start, u64 mmax, const u64 *C,
                                     u64 *xb)
{
    dnb2_gen(r, n, d, n_start, mmax, C, xb, 0);
}

/* qmctoolscl/c_funcs/dnb2_digital_shift.c:3-36 */
ORACLE_API void oracle_dnb2_digital_shift(u64 r, u64 n, u64 d, u64 r_x, const u64 *lshifts,
                                          const u64 *xb, const u64 *shiftsb, u64 *xrb)
{
    const u64 nelem_x = r_x * n * d;
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++) {
                const u64 idx = l * n * d + i * d + j;
                xrb[idx] = SHL(xb[idx % nelem_x], lshifts[l % r_x]) ^ shiftsb[l * d + j];
            }
}

/* qmctoolscl/c_funcs/dnb2_integer_to_float.c:3-32 */
ORACLE_API void oracle_dnb2_integer_to_float(u64 r, u64 n, u64 d, const u64 *tmaxes, const u64 *xb,
                                             double *x)
{
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++) {
                const u64 idx = l * n * d + i * d + j;
                x[idx] = ldexp((double)xb[idx], -(int)tmaxes[l]);
            }
}

/* qmctoolscl/c_funcs/dnb2_linear_matrix_scramble.c:3-51.  The parity of
 * S-row AND C-column is counted bit by bit, as the reference does. */
ORACLE_API void oracle_dnb2_linear_matrix_scramble(u64 r, u64 d, u64 mmax, u64 r_C, u64 tmax_new,
                                                   const u64 *S, const u64 *C, u64 *C_lms)
{
    const u64 nelem_C = r_C * d * mmax;
    for (u64 l = 0; l < r; l++)
        for (u64 j = 0; j < d; j++)
            for (u64 k = 0; k < mmax; k++) {
                const u64 idx = l * d * mmax + j * mmax + k;
                const u64 col = C[idx % nelem_C];
                u64 out = 0;
                for (u64 t = 0; t < tmax_new; t++) {
                    u64 w = S[l * d * tmax_new + j * tmax_new + t] & col, ones = 0;
                    for (; w; w &= w - 1) ones++;
                    if (ones & 1) out += SHL(1, tmax_new - t - 1);
                }
                C_lms[idx] = out;
            }
}

/* qmctoolscl/c_funcs/dnb2_interlace.c:3-45 */
ORACLE_API void oracle_dnb2_interlace(u64 r, u64 d_alpha, u64 mmax, u64 d, u64 tmax, u64 tmax_alpha,
                                      u64 alpha, const u64 *C, u64 *C_alpha)
{
    for (u64 l = 0; l < r; l++)
        for (u64 ja = 0; ja < d_alpha; ja++)
            for (u64 k = 0; k < mmax; k++) {
                u64 out = 0;
                for (u64 ta = 0; ta < tmax_alpha; ta++) {
                    const u64 t = ta / alpha, j = ja * alpha + ta % alpha;
                    if (SHR(C[l * d * mmax + j * mmax + k], tmax - t - 1) & 1)
                        out += SHL(1, tmax_alpha - ta - 1);
                }
                C_alpha[l * d_alpha * mmax + ja * mmax + k] = out;
            }
}

/* qmctoolscl/c_funcs/dnb2_undo_interlace.c:3-45 */
ORACLE_API void oracle_dnb2_undo_interlace(u64 r, u64 d, u64 mmax, u64 d_alpha, u64 tmax,
                                           u64 tmax_alpha, u64 alpha, const u64 *C_alpha, u64 *C)
{
    for (u64 l = 0; l < r; l++)
        for (u64 j = 0; j < d; j++)
            for (u64 k = 0; k < mmax; k++) {
                u64 out = 0;
                for (u64 t = 0; t < tmax; t++) {
                    const u64 ja = j / alpha, ta = t * alpha + j % alpha;
                    if (SHR(C_alpha[l * d_alpha * mmax + ja * mmax + k], tmax_alpha - ta - 1) & 1)
                        out += SHL(1, tmax - t - 1);
                }
                C[l * d * mmax + j * mmax + k] = out;
            }
}

/* qmctoolscl/c_funcs/dnb2_gmat_lsb_to_msb.c:3-44 */
ORACLE_API void oracle_dnb2_gmat_lsb_to_msb(u64 r, u64 d, u64 mmax, const u64 *tmaxes,
                                            const u64 *C_lsb, u64 *C_msb)
{
    for (u64 l = 0; l < r; l++) {
        const u64 tmax = tmaxes[l];
        for (u64 j = 0; j < d; j++)
            for (u64 k = 0; k < mmax; k++) {
                const u64 idx = l * d * mmax + j * mmax + k;
                u64 v = C_lsb[idx], out = 0;
                for (u64 t = 0; v != 0; v >>= 1, t++)
                    if (v & 1) out += SHL(1, tmax - t - 1);
                C_msb[idx] = out;
            }
    }
}

/* ------------------------------------------------------------------------ */
/* generalized digital nets (per-dimension base b)                          */
/* ------------------------------------------------------------------------ */

/* qmctoolscl/c_funcs/gdn_gen_natural.c:3-53.  Digit k of the point index in
 * base b scales column k; the running digit sums are reduced mod b after
 * every column, in 64-bit unsigned arithmetic. */
ORACLE_API void oracle_gdn_gen_natural(u64 r, u64 n, u64 d, u64 r_b, u64 mmax, u64 tmax,
                                       u64 n_start, const u64 *bases, const u64 *C, u64 *xdig)
{
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++) {
            const u64 itrue = i + n_start;
            for (u64 j = 0; j < d; j++) {
                u64 *out = xdig + l * n * d * tmax + i * d * tmax + j * tmax;
                for (u64 t = 0; t < tmax; t++) out[t] = 0;
                const u64 b = bases[(l % r_b) * d + j];
                u64 rest = itrue;
                for (u64 k = 0; rest > 0; k++) {
                    const u64 dig = rest % b;
                    rest = (rest - dig) / b;
                    if (dig > 0) {
                        const u64 *col = C + l * d * mmax * tmax + j * mmax * tmax + k * tmax;
                        for (u64 t = 0; t < tmax; t++) out[t] = (out[t] + dig * col[t]) % b;
                    }
                }
            }
        }
}

/* qmctoolscl/c_funcs/gdn_gen_natural_same_base.c:3-63 */
ORACLE_API void oracle_gdn_gen_natural_same_base(u64 r, u64 n, u64 d, u64 mmax, u64 tmax,
                                                 u64 n_start, u64 b, const u64 *C, u64 *xdig)
{
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++)
                for (u64 t = 0; t < tmax; t++)
                    xdig[l * n * d * tmax + i * d * tmax + j * tmax + t] = 0;
    for (u64 i = 0; i < n; i++) {
        u64 rest = i + n_start;
        for (u64 k = 0; rest > 0; k++) {
            const u64 dig = rest % b;
            rest = (rest - dig) / b;
            if (dig == 0) continue;
            for (u64 l = 0; l < r; l++)
                for (u64 j = 0; j < d; j++) {
                    u64 *out = xdig + l * n * d * tmax + i * d * tmax + j * tmax;
                    const u64 *col = C + l * d * mmax * tmax + j * mmax * tmax + k * tmax;
                    for (u64 t = 0; t < tmax; t++) out[t] = (out[t] + dig * col[t]) % b;
                }
        }
    }
}

/* qmctoolscl/c_funcs/gdn_linear_matrix_scramble.c:3-46.  Each product is
 * reduced mod b but the sum is not. */
ORACLE_API void oracle_gdn_linear_matrix_scramble(u64 r, u64 d, u64 mmax, u64 r_C, u64 r_b,
                                                  u64 tmax, u64 tmax_new, const u64 *bases,
                                                  const u64 *S, const u64 *C, u64 *C_lms)
{
    for (u64 l = 0; l < r; l++)
        for (u64 j = 0; j < d; j++) {
            const u64 b = bases[(l % r_b) * d + j];
            for (u64 k = 0; k < mmax; k++) {
                const u64 *col = C + (l % r_C) * d * mmax * tmax + j * mmax * tmax + k * tmax;
                u64 *out = C_lms + l * d * mmax * tmax_new + j * mmax * tmax_new + k * tmax_new;
                for (u64 t = 0; t < tmax_new; t++) {
                    const u64 *srow = S + l * d * tmax_new * tmax + j * tmax_new * tmax + t * tmax;
                    u64 acc = 0;
                    for (u64 c = 0; c < tmax; c++) acc += (srow[c] * col[c]) % b;
                    out[t] = acc;
                }
            }
        }
}

/* qmctoolscl/c_funcs/gdn_digital_permutation.c:3-46 */
ORACLE_API void oracle_gdn_digital_permutation(u64 r, u64 n, u64 d, u64 r_x, u64 r_b, u64 tmax,
                                               u64 tmax_new, u64 bmax, const u64 *perms,
                                               const u64 *xdig, u64 *xdig_new)
{
    (void)r_b;
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++) {
                const u64 *in = xdig + (l % r_x) * n * d * tmax + i * d * tmax + j * tmax;
                u64 *out = xdig_new + l * n * d * tmax_new + i * d * tmax_new + j * tmax_new;
                const u64 *perm = perms + l * d * tmax_new * bmax + j * tmax_new * bmax;
                for (u64 t = 0; t < tmax; t++) out[t] = perm[t * bmax + in[t]];
                for (u64 t = tmax; t < tmax_new; t++) out[t] = perm[t * bmax];
            }
}

/* qmctoolscl/c_funcs/gdn_digital_shift.c:3-45 */
ORACLE_API void oracle_gdn_digital_shift(u64 r, u64 n, u64 d, u64 r_x, u64 r_b, u64 tmax,
                                         u64 tmax_new, const u64 *bases, const u64 *shifts,
                                         const u64 *xdig, u64 *xdig_new)
{
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++) {
                const u64 *in = xdig + (l % r_x) * n * d * tmax + i * d * tmax + j * tmax;
                u64 *out = xdig_new + l * n * d * tmax_new + i * d * tmax_new + j * tmax_new;
                const u64 *sh = shifts + l * d * tmax_new + j * tmax_new;
                const u64 b = bases[(l % r_b) * d + j];
                for (u64 t = 0; t < tmax; t++) out[t] = (in[t] + sh[t]) % b;
                for (u64 t = tmax; t < tmax_new; t++) out[t] = sh[t];
            }
}

/* qmctoolscl/c_funcs/gdn_integer_to_float.c:3-43.  v += recip*digit and
 * recip /= b, each rounded separately (no FMA). */
ORACLE_API void oracle_gdn_integer_to_float(u64 r, u64 n, u64 d, u64 r_b, u64 tmax,
                                            const u64 *bases, const u64 *xdig, double *x)
{
    for (u64 l = 0; l < r; l++)
        for (u64 i = 0; i < n; i++)
            for (u64 j = 0; j < d; j++) {
                const u64 *in = xdig + l * n * d * tmax + i * d * tmax + j * tmax;
                const double b = (double)bases[(l % r_b) * d + j];
                double v = 0.0, recip = 1 / b;
                for (u64 t = 0; t < tmax; t++) {
                    v += recip * (double)in[t];
                    recip /= b;
                }
                x[l * n * d + i * d + j] = v;
            }
}

/* qmctoolscl/c_funcs/gdn_interlace.c:3-39 */
ORACLE_API void oracle_gdn_interlace(u64 r, u64 d_alpha, u64 mmax, u64 d, u64 tmax, u64 tmax_alpha,
                                     u64 alpha, const u64 *C, u64 *C_alpha)
{
    for (u64 l = 0; l < r; l++)
        for (u64 ja = 0; ja < d_alpha; ja++)
            for (u64 k = 0; k < mmax; k++)
                for (u64 ta = 0; ta < tmax_alpha; ta++) {
                    const u64 t = ta / alpha, j = ja * alpha + ta % alpha;
                    C_alpha[l * d_alpha * mmax * tmax_alpha + ja * mmax * tmax_alpha +
                            k * tmax_alpha + ta] = C[l * d * mmax * tmax + j * mmax * tmax + k * tmax + t];
                }
}

/* qmctoolscl/c_funcs/gdn_undo_interlace.c:3-39 */
ORACLE_API void oracle_gdn_undo_interlace(u64 r, u64 d, u64 mmax, u64 d_alpha, u64 tmax,
                                          u64 tmax_alpha, u64 alpha, const u64 *C_alpha, u64 *C)
{
    for (u64 l = 0; l < r; l++)
        for (u64 j = 0; j < d; j++)
            for (u64 k = 0; k < mmax; k++)
                for (u64 t = 0; t < tmax; t++) {
                    const u64 ja = j / alpha, ta = t * alpha + j % alpha;
                    C[l * d * mmax * tmax + j * mmax * tmax + k * tmax + t] =
                        C_alpha[l * d_alpha * mmax * tmax_alpha + ja * mmax * tmax_alpha +
                                k * tmax_alpha + ta];
                }
}

/* ------------------------------------------------------------------------ */
/* fast transforms along the last axis (length n = 2*n_half)                */
/* ------------------------------------------------------------------------ */

/* Twiddle table of fft_bro_1d_radix2.c:32-42 (sign -1) and
 * ifft_bro_1d_radix2.c:32-42 (sign +1): angle sign*2*pi*t/n, evaluated
 * left to right as the reference writes it. */
static void fill_twiddles(u64 n, double sign, double *twr, double *twi)
{
    const double PI = acos(-1.);
    for (u64 t = 0; t < n; t++) {
        const double ang = sign * 2 * PI * t / n;
        twr[t] = cos(ang);
        twi[t] = sin(ang);
    }
}

/* Partner indices of one butterfly (fft_bro_1d_radix2.c:50-57): the
 * n_half work items each own the pair (i1, i1 + f) whose i1 has bit `bit`
 * clear; items with that bit set take the pair in the upper half. */
static void pair_of(u64 i, u64 n_half, u64 f, u64 bit, u64 *i1, u64 *i2)
{
    if ((i >> bit) & 1) {
        *i2 = i + n_half;
        *i1 = *i2 ^ f;
    } else {
        *i1 = i;
        *i2 = i ^ f;
    }
}

/* qmctoolscl/c_funcs/fft_bro_1d_radix2.c:3-80 (decimation in time,
 * bit-reversed input, natural output, 1/sqrt(2) per stage). */
ORACLE_API void oracle_fft_bro_1d_radix2(u64 d1, u64 d2, u64 n_half, double *twr, double *twi,
                                         double *xr, double *xi)
{
    const u64 n = 2 * n_half, m = (u64)log2((double)n);
    const double sqrt2 = sqrt(2.0);
    fill_twiddles(n, -1.0, twr, twi);
    for (u64 k = 0; k < m; k++) {
        const u64 s = m - k - 1, f = SHL(1, k);
        for (u64 i = 0; i < n_half; i++) {
            u64 i1, i2;
            pair_of(i, n_half, f, k, &i1, &i2);
            const u64 t = (i1 % f) * SHL(1, s);
            const double c = twr[t], sn = twi[t];
            for (u64 j1 = 0; j1 < d1; j1++)
                for (u64 j2 = 0; j2 < d2; j2++) {
                    const u64 base = j1 * d2 * n + j2 * n;
                    const double ar = xr[base + i1], br = xr[base + i2];
                    const double ai = xi[base + i1], bi = xi[base + i2];
                    const double yr = br * c - bi * sn;
                    const double yi = br * sn + bi * c;
                    xr[base + i1] = (ar + yr) / sqrt2;
                    xi[base + i1] = (ai + yi) / sqrt2;
                    xr[base + i2] = (ar - yr) / sqrt2;
                    xi[base + i2] = (ai - yi) / sqrt2;
                }
        }
    }
}

/* qmctoolscl/c_funcs/ifft_bro_1d_radix2.c:3-81 (decimation in frequency,
 * natural input, bit-reversed output, 1/sqrt(2) per stage). */
ORACLE_API void oracle_ifft_bro_1d_radix2(u64 d1, u64 d2, u64 n_half, double *twr, double *twi,
                                          double *xr, double *xi)
{
    const u64 n = 2 * n_half, m = (u64)log2((double)n);
    const double sqrt2 = sqrt(2.0);
    fill_twiddles(n, 1.0, twr, twi);
    for (u64 k = 0; k < m; k++) {
        const u64 s = m - k - 1, f = SHL(1, s);
        for (u64 i = 0; i < n_half; i++) {
            u64 i1, i2;
            pair_of(i, n_half, f, s, &i1, &i2);
            const u64 t = (i1 % f) * SHL(1, k);
            const double c = twr[t], sn = twi[t];
            for (u64 j1 = 0; j1 < d1; j1++)
                for (u64 j2 = 0; j2 < d2; j2++) {
                    const u64 base = j1 * d2 * n + j2 * n;
                    const double ar = xr[base + i1], br = xr[base + i2];
                    const double ai = xi[base + i1], bi = xi[base + i2];
                    const double yr = ar - br, yi = ai - bi;
                    xr[base + i1] = (ar + br) / sqrt2;
                    xi[base + i1] = (ai + bi) / sqrt2;
                    xr[base + i2] = (yr * c - yi * sn) / sqrt2;
                    xi[base + i2] = (yr * sn + yi * c) / sqrt2;
                }
        }
    }
}

/* qmctoolscl/c_funcs/fwht_1d_radix2.c:3-53 */
ORACLE_API void oracle_fwht_1d_radix2(u64 d1, u64 d2, u64 n_half, double *x)
{
    const u64 n = 2 * n_half, m = (u64)log2((double)n);
    const double sqrt2 = sqrt(2.0);
    for (u64 k = 0; k < m; k++) {
        const u64 s = m - k - 1, f = SHL(1, s);
        for (u64 i = 0; i < n_half; i++) {
            u64 i1, i2;
            pair_of(i, n_half, f, s, &i1, &i2);
            for (u64 j1 = 0; j1 < d1; j1++)
                for (u64 j2 = 0; j2 < d2; j2++) {
                    const u64 base = j1 * d2 * n + j2 * n;
                    const double a = x[base + i1], b = x[base + i2];
                    x[base + i1] = (a + b) / sqrt2;
                    x[base + i2] = (a - b) / sqrt2;
                }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* qmctoolscl/c_funcs/halton_qrng.c:3-162: the generalized Halton sequence of
 * Faure and Lemieux in the form of the R package qrng (ghalton): for point i
 * and dimension j with base b = the dvec[j]-th prime, the 32 base-b digits of
 * i, each mapped to (f * digit + s_k) mod b with the multiplier f (1, or the
 * table below when generalized) and the random digit shift
 * s_k = (int)(b * randu_d_32[j*32+k]), summed by Horner's rule from digit 31
 * down, every add and divide rounded (halton_qrng.c:133-140).  Output res is
 * d x n (dimension-major); point 0 (when n0 = 0) is the shift alone
 * (halton_qrng.c:68-83). */

/* the scrambling multipliers of the generalized sequence, one per prime
 * (halton_qrng.c:37-60): a published table that the parity needs as it is */
static const int QRNG_MULT[360] = {
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

static int qrng_prime(int idx)  /* the (idx+1)-th prime, idx < 360 (halton_qrng.c:28-35) */
{
    int count = -1, c = 1;
    while (count < idx) {
        c++;
        int is_p = 1;
        for (int q = 2; q * q <= c; q++)
            if (c % q == 0) {
                is_p = 0;
                break;
            }
        count += is_p;
    }
    return c;
}

ORACLE_API void oracle_halton_qrng(int n, int d, int n0, int generalized, double *res, const double *randu_d_32,
                                   const int *dvec)
{
    for (int j = 0; j < d; j++) {
        const int b = qrng_prime(dvec[j]);
        const unsigned f = generalized ? (unsigned)QRNG_MULT[dvec[j]] : 1u;
        unsigned s[32];
        double u = 0.0;
        for (int k = 31; k >= 0; k--) {
            s[k] = (unsigned)(int)(b * randu_d_32[j * 32 + k]);
            u += s[k];
            u /= b;
        }
        if (n0 == 0) res[(long)j * n] = u;
        for (int i = n0 == 0 ? 1 : n0; i < n + n0; i++) {
            unsigned dg[32] = {0}, t = (unsigned)i;
            for (int k = 0; t > 0 && k < 32; k++) {
                dg[k] = t % (unsigned)b;
                t /= (unsigned)b;
            }
            double v = 0.0;
            for (int k = 31; k >= 0; k--) {
                v += (f * dg[k] + s[k]) % (unsigned)b;
                v /= b;
            }
            res[(long)j * n + (i - n0)] = v;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Nested uniform (Owen) scrambling of base-2 digital nets                   */
/* ------------------------------------------------------------------------ */

/* numpy's SFC64 bit generator: Chris Doty-Humphrey's published SFC64 step
 * (state a, b, c and a counter w) and numpy's 32-bit draw, which hands out
 * the low half of a 64-bit output and keeps the high half for the next
 * 32-bit draw (has_uint32 / uinteger in the generator's state). */
typedef struct {
    u64 a, b, c, w;
    int has;
    u64 half;
} sfc64_t;

static u64 sfc64_next64(sfc64_t *g)
{
    u64 out = g->a + g->b + g->w++;
    g->a = g->b ^ (g->b >> 11);
    g->b = g->c + (g->c << 3);
    g->c = ((g->c << 24) | (g->c >> 40)) + out;
    return out;
}

static u64 sfc64_next32(sfc64_t *g)
{
    if (g->has) {
        g->has = 0;
        return g->half;
    }
    u64 x = sfc64_next64(g);
    g->has = 1;
    g->half = x >> 32;
    return x & 0xFFFFFFFFull;
}

/* Generator.integers(0, 2**m) for 0 <= m <= 63 and random_tbit_uint64s(rng,
 * m, 1) for m <= 64 (qmctoolscl/rand_funcs.py:4-20).  numpy draws from
 * [0, 2^m) with Lemire's multiply-shift on a 32-bit output when 2^m - 1 fits
 * 32 bits and on a 64-bit output otherwise; with a power-of-two range the
 * rejection threshold is zero, so the value is the top m bits of that output
 * and nothing is drawn for m = 0.  m = 64 (the int64 range of
 * random_tbit_uint64s) is one raw 64-bit output. */
static u64 sfc64_bits(sfc64_t *g, unsigned m)
{
    if (m == 0) return 0;
    if (m <= 32) return sfc64_next32(g) >> (32 - m);
    if (m == 64) return sfc64_next64(g);
    return sfc64_next64(g) >> (64 - m);
}

/* One node of the scrambling tree (rand_funcs.py:155-160, NUSNode_dnb2): a
 * leaf holds the trailing bits xb of the one point seen below it and the
 * random bits for all of them; an internal node holds one random bit. */
typedef struct {
    u64 shift_bits, xb;
    int64_t child[2];
    int leaf;
} nus_node_t;

typedef struct {
    nus_node_t *node;
    u64 count, cap;
    int init;
} nus_tree_t;

typedef struct {
    u64 ntrees;
    nus_tree_t *tree;
} nus_forest_t;

#include <stdlib.h>

ORACLE_API void *oracle_nus_forest_new(u64 ntrees)
{
    nus_forest_t *f = (nus_forest_t *)calloc(1, sizeof(nus_forest_t));
    f->ntrees = ntrees;
    f->tree = (nus_tree_t *)calloc(ntrees ? ntrees : 1, sizeof(nus_tree_t));
    return f;
}

ORACLE_API void oracle_nus_forest_free(void *h)
{
    nus_forest_t *f = (nus_forest_t *)h;
    if (!f) return;
    for (u64 k = 0; k < f->ntrees; k++) free(f->tree[k].node);
    free(f->tree);
    free(f);
}

static int64_t nus_new_node(nus_tree_t *t, u64 shift_bits, u64 xb, int leaf)
{
    if (t->count == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->node = (nus_node_t *)realloc(t->node, t->cap * sizeof(nus_node_t));
    }
    nus_node_t *p = &t->node[t->count];
    p->shift_bits = shift_bits;
    p->xb = xb;
    p->child[0] = p->child[1] = -1;
    p->leaf = leaf;
    return (int64_t)t->count++;
}

/* dnb2_nested_uniform_scramble (qmctoolscl/rand_funcs.py:162-253).
 * states: r*d generator states, 6 words each (a, b, c, w, has_uint32,
 * uinteger), advanced in place; forest: r*d trees from oracle_nus_forest_new,
 * kept between calls as the reference keeps its root nodes.  The walk per
 * point follows rand_funcs.py:200-251: bit t-1 of the point picks the child;
 * an internal node adds its bit; a missing child becomes a new leaf with t-1
 * fresh random bits; a leaf holding another point is split, its bits moving
 * down with its point, until the two points part. */
ORACLE_API void oracle_dnb2_nested_uniform_scramble(u64 r, u64 n, u64 d, u64 r_x, u64 tmax, u64 tmax_new,
                                                    u64 *states, void *forest, const u64 *xb, u64 *xrb)
{
    nus_forest_t *f = (nus_forest_t *)forest;
    u64 t_delta = tmax_new - tmax;
    for (u64 l = 0; l < r; l++) {
        u64 l_x = l % r_x;
        for (u64 j = 0; j < d; j++) {
            u64 *st = states + 6 * (l * d + j);
            sfc64_t g = {st[0], st[1], st[2], st[3], (int)st[4], st[5]};
            nus_tree_t *tr = &f->tree[l * d + j];
            if (!tr->init) { /* rand_funcs.py:191-195 */
                tr->count = 0;
                nus_new_node(tr, sfc64_bits(&g, (unsigned)tmax_new), 0, 1);
                tr->init = 1;
            }
            for (u64 i = 0; i < n; i++) {
                /* numpy's uint64 << gives 0 for a count of 64 (tmax = 0) */
                u64 xb_new = t_delta >= 64 ? 0 : xb[l_x * n * d + i * d + j] << t_delta;
                u64 x = xb_new, shift = 0;
                int64_t nd = 0;
                for (u64 t = tmax_new; t > 0; t--) {
                    u64 top = 1ull << (t - 1), mask = top - 1;
                    int b = (int)((x >> (t - 1)) & 1u);
                    u64 x_next = x & mask;
                    nus_node_t *p = &tr->node[nd];
                    if (!p->leaf) {
                        if (p->shift_bits) shift += top;
                        if (p->child[b] < 0) {
                            u64 bits = sfc64_bits(&g, (unsigned)(t - 1));
                            int64_t c = nus_new_node(tr, bits, x_next, 1);
                            tr->node[nd].child[b] = c;
                            shift += bits;
                            break;
                        }
                        nd = p->child[b];
                    } else if (p->xb == x) {
                        shift += p->shift_bits;
                        break;
                    } else {
                        int nb = (int)((p->xb >> (t - 1)) & 1u);
                        u64 nxb = p->xb & mask, nbits = p->shift_bits & mask;
                        u64 lead = (p->shift_bits >> (t - 1)) & 1u;
                        if (lead) shift += top;
                        int64_t moved = nus_new_node(tr, nbits, nxb, 1);
                        p = &tr->node[nd]; /* the pool may have moved */
                        p->child[nb] = moved;
                        p->leaf = 0;
                        p->shift_bits = lead;
                        if (nb != b) {
                            u64 bits = sfc64_bits(&g, (unsigned)(t - 1));
                            int64_t c = nus_new_node(tr, bits, x_next, 1);
                            tr->node[nd].child[b] = c;
                            shift += bits;
                            break;
                        }
                        nd = moved;
                    }
                    x = x_next;
                }
                xrb[l * n * d + i * d + j] = xb_new ^ shift;
            }
            st[0] = g.a; st[1] = g.b; st[2] = g.c; st[3] = g.w; st[4] = (u64)g.has; st[5] = g.half;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Nested uniform scrambling of generalized (base-b) digital nets            */
/* ------------------------------------------------------------------------ */

/* numpy's random_interval(max): a value in [0, max] by masked rejection on
 * 32-bit draws (64-bit ones above 2^32 - 1), as Generator.shuffle uses it */
static u64 sfc64_interval(sfc64_t *g, u64 mx)
{
    if (mx == 0) return 0;
    u64 mask = mx;
    mask |= mask >> 1;
    mask |= mask >> 2;
    mask |= mask >> 4;
    mask |= mask >> 8;
    mask |= mask >> 16;
    mask |= mask >> 32;
    u64 v;
    if (mx <= 0xFFFFFFFFull) {
        do v = sfc64_next32(g) & mask; while (v > mx);
    } else {
        do v = sfc64_next64(g) & mask; while (v > mx);
    }
    return v;
}

/* random_uint64_permutations(rng, m, b) (rand_funcs.py:22-32): m rows, each
 * Generator.permutation(b) -- Fisher-Yates from the top of arange(b) */
static void sfc64_permutations(sfc64_t *g, u64 m, u64 b, u64 *out)
{
    for (u64 k = 0; k < m; k++) {
        u64 *row = out + k * b;
        for (u64 i = 0; i < b; i++) row[i] = i;
        for (u64 i = b; i-- > 1;) {
            u64 j = sfc64_interval(g, i), t = row[i];
            row[i] = row[j];
            row[j] = t;
        }
    }
}

/* One node of the base-b tree (rand_funcs.py:255-260, NUSNode_gdn): a leaf
 * holds the trailing digits of the one point below it and one permutation
 * per remaining level; an internal node holds one permutation and b
 * children.  Leaves that split hand their rows and digits down by pointer. */
typedef struct {
    u64 *perm, *xdig;
    int64_t *child;
    int leaf;
} gnode_t;

typedef struct {
    gnode_t *node;
    u64 count, cap;
    void **bufs;
    u64 nbufs, capbufs;
    int init;
} gtree_t;

typedef struct {
    u64 ntrees;
    gtree_t *tree;
} gforest_t;

ORACLE_API void *oracle_gdn_forest_new(u64 ntrees)
{
    gforest_t *f = (gforest_t *)calloc(1, sizeof(gforest_t));
    f->ntrees = ntrees;
    f->tree = (gtree_t *)calloc(ntrees ? ntrees : 1, sizeof(gtree_t));
    return f;
}

ORACLE_API void oracle_gdn_forest_free(void *h)
{
    gforest_t *f = (gforest_t *)h;
    if (!f) return;
    for (u64 k = 0; k < f->ntrees; k++) {
        gtree_t *t = &f->tree[k];
        for (u64 i = 0; i < t->nbufs; i++) free(t->bufs[i]);
        free(t->bufs);
        free(t->node);
    }
    free(f->tree);
    free(f);
}

static void *gtree_alloc(gtree_t *t, size_t bytes)
{
    if (t->nbufs == t->capbufs) {
        t->capbufs = t->capbufs ? 2 * t->capbufs : 64;
        t->bufs = (void **)realloc(t->bufs, t->capbufs * sizeof(void *));
    }
    void *p = malloc(bytes ? bytes : 1);
    t->bufs[t->nbufs++] = p;
    return p;
}

static int64_t gtree_leaf(gtree_t *t, u64 *perm, u64 *xdig)
{
    if (t->count == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->node = (gnode_t *)realloc(t->node, t->cap * sizeof(gnode_t));
    }
    gnode_t *p = &t->node[t->count];
    p->perm = perm;
    p->xdig = xdig;
    p->child = NULL;
    p->leaf = 1;
    return (int64_t)t->count++;
}

/* gdn_nested_uniform_scramble (qmctoolscl/rand_funcs.py:262-356).  states:
 * r*d generator states as for the base-2 scramble; forest: r*d trees from
 * oracle_gdn_forest_new, kept between calls.  xdig (r_x, n, d, tmax) digits,
 * xrdig (r, n, d, tmax_new).  Returns 0, or 1 where the reference raises
 * IndexError: a digit at or above its base, or a walk that runs out of
 * digits (tmax_new = tmax and a point that repeats an earlier one down to
 * its last digit). */
ORACLE_API int oracle_gdn_nested_uniform_scramble(u64 r, u64 n, u64 d, u64 r_x, u64 r_b, u64 tmax, u64 tmax_new,
                                                  u64 *states, void *forest, const u64 *bases, const u64 *xdig,
                                                  u64 *xrdig)
{
    gforest_t *f = (gforest_t *)forest;
    u64 *xd = (u64 *)malloc((tmax_new + 1) * sizeof(u64));
    int bad = 0;
    for (u64 l = 0; l < r && !bad; l++) {
        u64 l_b = l % r_b, l_x = l % r_x;
        for (u64 j = 0; j < d && !bad; j++) {
            u64 *st = states + 6 * (l * d + j);
            sfc64_t g = {st[0], st[1], st[2], st[3], (int)st[4], st[5]};
            gtree_t *tr = &f->tree[l * d + j];
            u64 b = bases[l_b * d + j];
            if (!tr->init) { /* rand_funcs.py:318-322 */
                tr->count = 0;
                u64 *perm = (u64 *)gtree_alloc(tr, tmax_new * b * sizeof(u64));
                u64 *z = (u64 *)gtree_alloc(tr, tmax_new * sizeof(u64));
                for (u64 k = 0; k < tmax_new; k++) z[k] = 0;
                sfc64_permutations(&g, tmax_new, b, perm);
                gtree_leaf(tr, perm, z);
                tr->init = 1;
            }
            for (u64 i = 0; i < n && !bad; i++) {
                const u64 *x = xdig + ((l_x * n + i) * d + j) * tmax;
                u64 *out = xrdig + ((l * n + i) * d + j) * tmax_new;
                int64_t nd = 0;
                for (u64 t = 0; t <= tmax; t++) {
                    if (t >= tmax_new) { bad = 1; break; } /* _xdig[0] of an empty array */
                    u64 len = tmax_new - t;
                    for (u64 k = 0; k < len; k++) xd[k] = (t + k < tmax) ? x[t + k] : 0;
                    u64 dig = xd[0];
                    if (dig >= b) { bad = 1; break; }
                    gnode_t *p = &tr->node[nd];
                    if (!p->leaf) {
                        out[t] = p->perm[dig];
                        if (p->child[dig] < 0) {
                            u64 m = len - 1;
                            u64 *perm = (u64 *)gtree_alloc(tr, m * b * sizeof(u64));
                            u64 *rest = (u64 *)gtree_alloc(tr, m * sizeof(u64));
                            sfc64_permutations(&g, m, b, perm);
                            for (u64 k = 0; k < m; k++) rest[k] = xd[1 + k];
                            for (u64 k = 0; k < m; k++) {
                                if (rest[k] >= b) { bad = 1; break; }
                                out[t + 1 + k] = perm[k * b + rest[k]];
                            }
                            int64_t c = gtree_leaf(tr, perm, rest);
                            tr->node[nd].child[dig] = c;
                            break;
                        }
                        nd = p->child[dig];
                        continue;
                    }
                    int same = 1;
                    for (u64 k = 0; k < len; k++)
                        if (p->xdig[k] != xd[k]) { same = 0; break; }
                    if (same) {
                        for (u64 k = 0; k < len; k++) {
                            if (xd[k] >= b) { bad = 1; break; }
                            out[t + k] = p->perm[k * b + xd[k]];
                        }
                        break;
                    }
                    u64 node_dig = p->xdig[0];
                    if (node_dig >= b) { bad = 1; break; }
                    out[t] = p->perm[dig];
                    u64 *rows = p->perm, *digs = p->xdig;
                    int64_t *kids = (int64_t *)gtree_alloc(tr, b * sizeof(int64_t));
                    for (u64 k = 0; k < b; k++) kids[k] = -1;
                    int64_t moved = gtree_leaf(tr, rows + b, digs + 1);
                    p = &tr->node[nd]; /* the pool may have moved */
                    p->leaf = 0;
                    p->perm = rows; /* its first row: the permutation of this level */
                    p->xdig = NULL;
                    p->child = kids;
                    kids[node_dig] = moved;
                    if (node_dig == dig) {
                        nd = moved;
                        continue;
                    }
                    u64 m = len - 1;
                    u64 *perm = (u64 *)gtree_alloc(tr, m * b * sizeof(u64));
                    u64 *rest = (u64 *)gtree_alloc(tr, m * sizeof(u64));
                    sfc64_permutations(&g, m, b, perm);
                    for (u64 k = 0; k < m; k++) rest[k] = xd[1 + k];
                    for (u64 k = 0; k < m; k++) {
                        if (rest[k] >= b) { bad = 1; break; }
                        out[t + 1 + k] = perm[k * b + rest[k]];
                    }
                    kids[dig] = gtree_leaf(tr, perm, rest);
                    break;
                }
            }
            st[0] = g.a; st[1] = g.b; st[2] = g.c; st[3] = g.w; st[4] = (u64)g.has; st[5] = g.half;
        }
    }
    free(xd);
    return bad;
}
