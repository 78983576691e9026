/*
 * qmcgb.h -- C ABI of libqmcgb.so, the GB300 (sm_103a) implementation of the
 * QMCToolsCL point-generation and fast-transform hot path.
 *
 * One entry point per reference C function.  Each takes the reference's
 * scalar arguments in the reference's order WITHOUT the three batch-size
 * arguments bs_r/bs_n/bs_d (the reference's C wrapper sets them to the full
 * extents, qmctoolscl/util.py:107), then the reference's arrays as DEVICE
 * pointers, then a CUDA stream.  Array layouts are the reference's:
 * C-contiguous in the order of the size strings of the reference comments
 * (e.g. x is r*n*d with d fastest).  Outputs are written in place; the
 * transforms work in place and also fill both twiddle arrays.
 *
 * Every per-function entry point (and the fused qmc_lat_gen_shift,
 * qmc_dnb2_gen_fused, the tensor-core transforms and qmc_net_gen_noalloc) is
 * stream-ordered and asynchronous, allocates nothing, keeps no host state
 * between calls and is safe to call from several host threads.  The plan
 * objects (qmc_*_plan_create) allocate their device tables when created and
 * free them when destroyed; running a plan allocates nothing.  Every call
 * returns QMC_OK or a negative status; qmc_last_error() gives the message
 * for the calling thread.
 *
 * Where the reference's behaviour is undefined (shift counts >= 64 in C,
 * reads past an array) the kernels follow what gcc builds of the reference
 * do on x86-64 and aarch64 (shift counts mod 64) or report QMC_ERR_DOMAIN.
 */
#ifndef QMCGB_H
#define QMCGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void *qmc_stream_t; /* a cudaStream_t; NULL is the legacy default stream */

enum qmc_status {
    QMC_OK = 0,
    QMC_ERR_ARG = -1,    /* bad size, null pointer or unsupported argument combination */
    QMC_ERR_DOMAIN = -2, /* arguments for which the reference's result is undefined */
    QMC_ERR_CUDA = -3,   /* a CUDA runtime or launch error */
    QMC_ERR_DEVICE = -4  /* a kernel recorded an error in the device error word (bits: 1 an index the
                            reference would read out of its array, 2 a base below 2, 4 a tensor-core
                            completion wait that ran out, 8 a fused generalized-net matrix entry >= 2^32,
                            16 a nested-uniform scrambling tree deeper than its keys allow) */
};

/* message of the last failing call on this host thread ("" if none) */
const char *qmc_last_error(void);
/* ABI version: major*10000 + minor*100 + patch */
int qmc_version(void);
/* clears the device error word on stream s */
int qmc_device_error_reset(qmc_stream_t s);
/* synchronises s, then returns QMC_ERR_DEVICE (and clears the word) if a
 * kernel recorded an error since the last reset */
int qmc_device_error_check(qmc_stream_t s);

/* device-side address of pinned host memory (cudaHostAlloc / cudaHostRegister)
 * that kernels may write directly; QMC_ERR_ARG for pageable memory.  No
 * reference counterpart: used to write results straight into host buffers. */
int qmc_host_pointer_for_device(const void *host, void **dev);
/* pageable-memory access, whether it uses the host page tables, SM count of
 * the current device.  No reference counterpart. */
int qmc_device_attributes(int *pageable_access, int *uses_host_page_tables, int *sms);

/* ---- rank-1 lattices ---------------------------------------------------- */

/* qmctoolscl/c_funcs/lat_gen_linear.c:3-13: x[l,i,j] = fmod(g[l,j]*(i/n), 1) */
int qmc_lat_gen_linear(uint64_t r, uint64_t n, uint64_t d, const uint64_t *g, double *x,
                       qmc_stream_t s);
/* qmctoolscl/c_funcs/lat_gen_natural.c:3-14: x[l,k,j] = fmod(g[l,j]*vdc(n_start+k), 1);
 * n_start and n_start+n must be 0 or powers of two (qmctoolscl/util.py:84-86) */
int qmc_lat_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, const uint64_t *g,
                        double *x, qmc_stream_t s);
/* qmctoolscl/c_funcs/lat_gen_gray.c:3-14: x[l,i,j] = fmod(g[l,j]*vdc(gray(n_start+i)), 1) */
int qmc_lat_gen_gray(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, const uint64_t *g,
                     double *x, qmc_stream_t s);
/* qmctoolscl/c_funcs/lat_shift_mod_1.c:3-15: xr[l,i,j] = fmod(x[l%r_x,i,j]+shifts[l,j], 1) */
int qmc_lat_shift_mod_1(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, const double *x,
                        const double *shifts, double *xr, qmc_stream_t s);

/* ---- digital nets in base 2 --------------------------------------------- */

/* qmctoolscl/c_funcs/dnb2_gen_natural.c:3-15; [n_start, n_start+n) must map onto
 * itself under the Gray code and n_start+n <= 2^mmax */
int qmc_dnb2_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, uint64_t mmax,
                         const uint64_t *C, uint64_t *xb, qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_gen_gray.c:3-15; gray(n_start+n-1) < 2^mmax */
int qmc_dnb2_gen_gray(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, uint64_t mmax,
                      const uint64_t *C, uint64_t *xb, qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_digital_shift.c:3-16 */
int qmc_dnb2_digital_shift(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x,
                           const uint64_t *lshifts, const uint64_t *xb, const uint64_t *shiftsb,
                           uint64_t *xrb, qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_integer_to_float.c:3-14 */
int qmc_dnb2_integer_to_float(uint64_t r, uint64_t n, uint64_t d, const uint64_t *tmaxes,
                              const uint64_t *xb, double *x, qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_linear_matrix_scramble.c:3-16 */
int qmc_dnb2_linear_matrix_scramble(uint64_t r, uint64_t d, uint64_t mmax, uint64_t r_C,
                                    uint64_t tmax_new, const uint64_t *S, const uint64_t *C,
                                    uint64_t *C_lms, qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_interlace.c:3-17 */
int qmc_dnb2_interlace(uint64_t r, uint64_t d_alpha, uint64_t mmax, uint64_t d, uint64_t tmax,
                       uint64_t tmax_alpha, uint64_t alpha, const uint64_t *C, uint64_t *C_alpha,
                       qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_undo_interlace.c:3-17 */
int qmc_dnb2_undo_interlace(uint64_t r, uint64_t d, uint64_t mmax, uint64_t d_alpha, uint64_t tmax,
                            uint64_t tmax_alpha, uint64_t alpha, const uint64_t *C_alpha,
                            uint64_t *C, qmc_stream_t s);
/* qmctoolscl/c_funcs/dnb2_gmat_lsb_to_msb.c:3-14 */
int qmc_dnb2_gmat_lsb_to_msb(uint64_t r, uint64_t d, uint64_t mmax, const uint64_t *tmaxes,
                             const uint64_t *C_lsb, uint64_t *C_msb, qmc_stream_t s);

/* ---- generalized digital nets (base b per dimension) -------------------- */

/* qmctoolscl/c_funcs/gdn_gen_natural.c:3-18 */
int qmc_gdn_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t r_b, uint64_t mmax,
                        uint64_t tmax, uint64_t n_start, const uint64_t *bases, const uint64_t *C,
                        uint64_t *xdig, qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_gen_natural_same_base.c:3-17 */
int qmc_gdn_gen_natural_same_base(uint64_t r, uint64_t n, uint64_t d, uint64_t mmax, uint64_t tmax,
                                  uint64_t n_start, uint64_t b, const uint64_t *C, uint64_t *xdig,
                                  qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_linear_matrix_scramble.c:3-19 */
int qmc_gdn_linear_matrix_scramble(uint64_t r, uint64_t d, uint64_t mmax, uint64_t r_C,
                                   uint64_t r_b, uint64_t tmax, uint64_t tmax_new,
                                   const uint64_t *bases, const uint64_t *S, const uint64_t *C,
                                   uint64_t *C_lms, qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_digital_permutation.c:3-19; a digit >= bmax reads
 * the flat entry the reference reads while that entry lies inside perms
 * (r*d*tmax_new*bmax elements); beyond it the kernel writes 0 and records
 * QMC_ERR_DEVICE for qmc_device_error_check */
int qmc_gdn_digital_permutation(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t r_b,
                                uint64_t tmax, uint64_t tmax_new, uint64_t bmax,
                                const uint64_t *perms, const uint64_t *xdig, uint64_t *xdig_new,
                                qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_digital_shift.c:3-19 */
int qmc_gdn_digital_shift(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t r_b,
                          uint64_t tmax, uint64_t tmax_new, const uint64_t *bases,
                          const uint64_t *shifts, const uint64_t *xdig, uint64_t *xdig_new,
                          qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_integer_to_float.c:3-16 */
int qmc_gdn_integer_to_float(uint64_t r, uint64_t n, uint64_t d, uint64_t r_b, uint64_t tmax,
                             const uint64_t *bases, const uint64_t *xdig, double *x,
                             qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_interlace.c:3-17 */
int qmc_gdn_interlace(uint64_t r, uint64_t d_alpha, uint64_t mmax, uint64_t d, uint64_t tmax,
                      uint64_t tmax_alpha, uint64_t alpha, const uint64_t *C, uint64_t *C_alpha,
                      qmc_stream_t s);
/* qmctoolscl/c_funcs/gdn_undo_interlace.c:3-17 */
int qmc_gdn_undo_interlace(uint64_t r, uint64_t d, uint64_t mmax, uint64_t d_alpha, uint64_t tmax,
                           uint64_t tmax_alpha, uint64_t alpha, const uint64_t *C_alpha,
                           uint64_t *C, qmc_stream_t s);

/* ---- fast transforms along the last axis, n = 2*n_half a power of two -- */

/* qmctoolscl/c_funcs/fft_bro_1d_radix2.c:3-17: orthonormal DFT of
 * bit-reversed input, natural-order output, in place; fills twiddler/twiddlei[0:n] */
int qmc_fft_bro_1d_radix2(uint64_t d1, uint64_t d2, uint64_t n_half, double *twiddler,
                          double *twiddlei, double *xr, double *xi, qmc_stream_t s);
/* qmctoolscl/c_funcs/ifft_bro_1d_radix2.c:3-17: the inverse (natural in,
 * bit-reversed out) */
int qmc_ifft_bro_1d_radix2(uint64_t d1, uint64_t d2, uint64_t n_half, double *twiddler,
                           double *twiddlei, double *xr, double *xi, qmc_stream_t s);
/* qmctoolscl/c_funcs/fwht_1d_radix2.c:3-14: orthonormal Walsh-Hadamard, in place */
int qmc_fwht_1d_radix2(uint64_t d1, uint64_t d2, uint64_t n_half, double *x, qmc_stream_t s);

/* ---- fused pipelines (no single reference counterpart) -------------------
 * Each equals a chain of reference calls, bit for bit, in one kernel. */

/* qmctoolscl/c_funcs/lat_gen_natural.c:3-58 (gray=0) or lat_gen_gray.c:3-56
 * (gray=1), followed by lat_shift_mod_1.c:3-35 with r_x = r: writes only xr
 * (r*n*d), never the unshifted points */
int qmc_lat_gen_shift(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, int gray, const uint64_t *g,
                      const double *shifts, double *xr, qmc_stream_t s);
/* dnb2_gen_natural / dnb2_gen_gray (qmctoolscl/c_funcs/dnb2_gen_natural.c:3-70,
 * dnb2_gen_gray.c:3-69), then, when shiftsb != NULL, dnb2_digital_shift.c:3-36
 * ((point << lshifts[l % r_x]) ^ shiftsb[l,j]), then, when x != NULL,
 * dnb2_integer_to_float.c:3-32 (ldexp(value, -tmaxes[l])).  C holds r_C*d*mmax
 * columns (randomisation l uses set l % r_C); xrb may be NULL when x is set. */
int qmc_dnb2_gen_fused(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, uint64_t mmax, const uint64_t *C,
                       uint64_t r_C, int gray, const uint64_t *lshifts, uint64_t r_x, const uint64_t *shiftsb,
                       const uint64_t *tmaxes, uint64_t *xrb, double *x, qmc_stream_t s);

/* ---- tensor-core transforms ---------------------------------------------
 * The contracts of qmc_fft_bro_1d_radix2 / qmc_ifft_bro_1d_radix2 /
 * qmc_fwht_1d_radix2 (qmctoolscl/c_funcs/fft_bro_1d_radix2.c:3-80,
 * ifft_bro_1d_radix2.c:3-81, fwht_1d_radix2.c:3-53: orthonormal, in place along
 * the last axis, same input/output orders) computed with radix-16 steps as
 * BF16 tensor-core products (three-term BF16 splits of data and matrix, FP32
 * accumulation): relative L2 error about 1e-7 against the FP64 transform
 * instead of FP64 rounding.  No twiddle arrays are written.  n = 2*n_half up
 * to 2^24; the data arrays must be 16-byte aligned (QMC_ERR_ARG otherwise). */
int qmc_tc_fft_bro_1d(uint64_t d1, uint64_t d2, uint64_t n_half, double *xr, double *xi, qmc_stream_t s);
int qmc_tc_ifft_bro_1d(uint64_t d1, uint64_t d2, uint64_t n_half, double *xr, double *xi, qmc_stream_t s);
int qmc_tc_fwht_1d(uint64_t d1, uint64_t d2, uint64_t n_half, double *x, qmc_stream_t s);

/* ---- generalized Halton (qrng) ---------------------------------------------
 * qmctoolscl/c_funcs/halton_qrng.c:3-162, the raw ctypes binding halton_qrng_c
 * of the reference (pdm_build.py:84-94): n points (indices n0 .. n0+n-1) of d
 * dimensions of the generalized Halton sequence in the form of the R package
 * qrng, res d x n (dimension-major), randu_d_32 d x 32 uniforms for the digit
 * shifts, dvec the prime index of each dimension; bit for bit the reference's
 * values.  d above 360 or n + n0 above 2^31 - 1 (undefined in the reference)
 * return QMC_ERR_DOMAIN; a dvec entry outside [0, 360) sets bit 1 of the device
 * error word and leaves that dimension unwritten. */
int qmc_halton_qrng(int n, int d, int n0, int generalized, double *res, const double *randu_d_32, const int *dvec,
                    qmc_stream_t s);

/* The fast kernel matrix-vector product and solve of the reference's
 * documentation (docs/index.md:1825-1884: u = ifft(fft(y) * kt), v =
 * ifft(fft(y) / kt), with fft = fft_bro_1d_radix2 and ifft =
 * ifft_bro_1d_radix2) in one call, in place on (xr, xi):
 *     y <- IFFT(FFT(y) * lam) * scale      (divide = 0)
 *     y <- IFFT(FFT(y) / lam) * scale      (divide != 0)
 * with the tensor-core transforms above (orthonormal; y in the FFT's input
 * order, lam in its natural output order).  lam = (lam_r, lam_i) holds n
 * values applied to every vector (lam_per_element = 0) or d1*d2*n values, one
 * per element (lam_per_element = 1).  The forward transform's last pass, the
 * pointwise step and the inverse transform's first pass run as one kernel on
 * each tile, with FP32 intermediates between passes: about half the HBM
 * traffic of the three steps done separately. */
int qmc_tc_fft_mul_ifft(uint64_t d1, uint64_t d2, uint64_t n_half, const double *lam_r, const double *lam_i,
                        uint64_t lam_per_element, int divide, double scale, double *xr, double *xi, qmc_stream_t s);

/* The Walsh-Hadamard analog (docs/index.md:1929-1978: u = fwht(fwht(y) * kt),
 * v = fwht(fwht(y) / kt), fwht = fwht_1d_radix2) in one call, in place on x:
 *     y <- FWHT(FWHT(y) * lam) * scale     (divide = 0)
 *     y <- FWHT(FWHT(y) / lam) * scale     (divide != 0)
 * with the tensor-core WHT above; lam real, n values for every vector or one
 * per element.  The first transform's last pass, the pointwise step and the
 * second transform's first pass run as one kernel on each tile. */
int qmc_tc_fwht_mul_fwht(uint64_t d1, uint64_t d2, uint64_t n_half, const double *lam, uint64_t lam_per_element,
                         int divide, double scale, double *x, qmc_stream_t s);

/* The same two fused forms in FP64 (the arithmetic of qmc_fft_bro_1d_radix2 /
 * qmc_ifft_bro_1d_radix2 / qmc_fwht_1d_radix2, to FP64 rounding of numpy's
 * result): forward passes but the last, one fused pass (forward steps, the
 * pointwise product or quotient, inverse steps), inverse passes but the first.
 * qmc_fft_mul_ifft writes the forward twiddle table into twiddler/twiddlei (n
 * doubles each, as qmc_fft_bro_1d_radix2 does) and runs the inverse steps on
 * its conjugates. */
int qmc_fft_mul_ifft(uint64_t d1, uint64_t d2, uint64_t n_half, double *twiddler, double *twiddlei, const double *lam_r,
                     const double *lam_i, uint64_t lam_per_element, int divide, double scale, double *xr, double *xi,
                     qmc_stream_t s);
int qmc_fwht_mul_fwht(uint64_t d1, uint64_t d2, uint64_t n_half, const double *lam, uint64_t lam_per_element,
                      int divide, double scale, double *x, qmc_stream_t s);

/* ---- batched plans: many requests of uneven size, one persistent launch -----
 * No single reference counterpart: a plan runs, for every request, the chain
 * of reference calls written next to each struct, bit for bit, in two
 * launches in total (matrix preparation, then generation), and can replay
 * them from a CUDA graph.  A plan keeps device copies of the request
 * descriptors plus scratch for the prepared matrices and a work counter
 * (allocated when the plan is created).  The arrays the requests point to
 * are read at run time, so their contents may change between runs; the
 * pointers may not. */

/* One base-2 digital-net request with r randomisations:
 *   dnb2_linear_matrix_scramble (if S)  qmctoolscl/c_funcs/dnb2_linear_matrix_scramble.c:3-51
 *   dnb2_interlace (if alpha > 1)       qmctoolscl/c_funcs/dnb2_interlace.c:3-45
 *   dnb2_gen_natural / dnb2_gen_gray    qmctoolscl/c_funcs/dnb2_gen_natural.c:3-70, dnb2_gen_gray.c:3-69
 *   dnb2_digital_shift (if shifts)      qmctoolscl/c_funcs/dnb2_digital_shift.c:3-36 with r_x = r
 *   dnb2_integer_to_float (if x)        qmctoolscl/c_funcs/dnb2_integer_to_float.c:3-32 */
typedef struct qmc_net_request {
    uint64_t r;          /* randomisations */
    uint64_t n;          /* points */
    uint64_t d;          /* output dimension (d_pre / alpha) */
    uint64_t n_start;    /* index of the first point */
    uint64_t mmax;       /* generating-matrix columns */
    uint64_t d_pre;      /* dimension of C and S (d * alpha) */
    uint64_t alpha;      /* interlacing factor, 1 = none */
    uint64_t tmax;       /* bits of the columns of C (used when S is NULL) */
    uint64_t tmax_new;   /* bits after scrambling (used when S is set) */
    uint64_t tmax_alpha; /* bits after interlacing (alpha > 1) */
    uint64_t r_C;        /* matrix sets in C; randomisation l uses l % r_C */
    int32_t gray;        /* 0: natural order, 1: Gray order */
    int32_t reserved;
    const uint64_t *C;       /* r_C * d_pre * mmax */
    const uint64_t *S;       /* r * d_pre * tmax_new scrambling rows, or NULL */
    const uint64_t *lshifts; /* r left shifts (with shifts) */
    const uint64_t *shifts;  /* r * d digital shifts, or NULL */
    const uint64_t *tmaxes;  /* r float scalings (with x) */
    uint64_t *xb;            /* r * n * d integers out, or NULL */
    double *x;               /* r * n * d floats out, or NULL */
} qmc_net_request;

/* One rank-1 lattice request with r randomisations:
 *   lat_gen_natural / lat_gen_gray      qmctoolscl/c_funcs/lat_gen_natural.c:3-58, lat_gen_gray.c:3-56
 *   lat_shift_mod_1 (if shifts)         qmctoolscl/c_funcs/lat_shift_mod_1.c:3-35 with r_x = r */
typedef struct qmc_lat_request {
    uint64_t r, n, d, n_start;
    int32_t gray;          /* 0: natural order, 1: Gray order */
    int32_t reserved;
    const uint64_t *g;     /* r * d generating vectors */
    const double *shifts;  /* r * d shifts, or NULL */
    double *x;             /* r * n * d points out */
} qmc_lat_request;

typedef struct qmc_plan qmc_plan;

int qmc_net_plan_create(const qmc_net_request *reqs, int nreq, qmc_plan **plan);
int qmc_lat_plan_create(const qmc_lat_request *reqs, int nreq, qmc_plan **plan);
/* launch the plan on s (two launches for net plans, one for lattice plans) */
int qmc_plan_run(qmc_plan *plan, qmc_stream_t s);
/* the same work from a CUDA graph: captured on s at the first call (s must not be
 * the legacy default stream), replayed afterwards */
int qmc_plan_graph_launch(qmc_plan *plan, qmc_stream_t s);
/* launch shape of the generation kernel: CTAs per SM, tiles taken per work-queue
 * grab, coordinates per tile (rounded to whole rows); 0 keeps a value.  Drops any
 * captured graph. */
int qmc_plan_set_tuning(qmc_plan *plan, int ctas_per_sm, int chunk, uint64_t tile_coords);
/* tiles, coordinates and output bytes of one run, kernel launches per run */
int qmc_plan_info(const qmc_plan *plan, uint64_t *tiles, uint64_t *coords, uint64_t *bytes_out, int *launches);
int qmc_plan_destroy(qmc_plan *plan);

/* ---- fused generalized digital net (per-dimension bases, e.g. Halton) -------
 * For every dimension j the reference chain
 *   gdn_linear_matrix_scramble  qmctoolscl/c_funcs/gdn_linear_matrix_scramble.c:3-46
 *   gdn_gen_natural             qmctoolscl/c_funcs/gdn_gen_natural.c:3-53
 *   gdn_digital_permutation     qmctoolscl/c_funcs/gdn_digital_permutation.c:3-46
 *   gdn_digital_shift           qmctoolscl/c_funcs/gdn_digital_shift.c:3-45
 *   gdn_integer_to_float        qmctoolscl/c_funcs/gdn_integer_to_float.c:3-43
 * called with d = 1, r_b = 1, r_C = 1 and tmax_new = tmax, its result going to
 * x[l, i, j] of one r*n*d array; digits never reach HBM.  A step whose array
 * is NULL (S, perms or shifts, the same for every dimension) is left out of
 * the chain.  Bases in [2, 2048), n_start + n <= 2^32, mmax at least the
 * base-b digits of the last index; without S, generating-matrix entries
 * below 2^32 (larger ones set bit 8 of the device error word).  Create
 * allocates the packed tables; prepare fills them from the arrays the dims
 * point to (read at that time, on the stream); run generates x.
 * set_fp64_share picks the share of the digit adds that run on the FP64
 * unit (the rest run in integer arithmetic, same bits either way), a tuning
 * knob for the balance between the two pipes (default 1.0: all FP64, the fastest
 * measured on GB300). */
typedef struct qmc_gdn_dim {
    uint64_t b, tmax, mmax;
    const uint64_t *S;      /* r * tmax * tmax scrambling matrices */
    const uint64_t *C;      /* mmax * tmax generating matrix */
    const uint64_t *perms;  /* r * tmax * b digit permutations */
    const uint64_t *shifts; /* r * tmax digital shifts */
} qmc_gdn_dim;
typedef struct qmc_halton_plan qmc_halton_plan;
int qmc_halton_plan_create(uint64_t r, uint64_t n, uint64_t n_start, uint64_t d, const qmc_gdn_dim *dims, double *x,
                           qmc_halton_plan **plan);
/* Many requests of uneven (r, n, n_start, d, bases, digit counts) in one plan:
 * preparation and generation each one launch over all requests (generation
 * walks one list of point tiles).  Each request's dims, arrays and x as for
 * qmc_halton_plan_create. */
typedef struct qmc_halton_request {
    uint64_t r, n, n_start, d;
    const qmc_gdn_dim *dims;
    double *x;
} qmc_halton_request;
int qmc_halton_batch_create(const qmc_halton_request *reqs, int nreq, qmc_halton_plan **plan);
int qmc_halton_plan_prepare(qmc_halton_plan *plan, qmc_stream_t s);
int qmc_halton_plan_run(qmc_halton_plan *plan, qmc_stream_t s);
/* prepare + run from a CUDA graph captured on s at the first call (s must not be the
 * legacy default stream); later calls replay it */
int qmc_halton_plan_graph_launch(qmc_halton_plan *plan, qmc_stream_t s);
int qmc_halton_plan_set_fp64_share(qmc_halton_plan *plan, double share);
int qmc_halton_plan_destroy(qmc_halton_plan *plan);

/* ---- one digital-net request without any allocation -------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * -- their device memory belongs to another allocator (a framework's caching
 * pool, a serving process's fixed arena), or they run a latency-bound loop
 * that must not take cudaMalloc's implicit device synchronisation.  Runs the
 * chain of one qmc_net_request (as a one-request plan does) on stream s,
 * allocating nothing: the scrambled/interlaced matrices go to a fixed array
 * of QMC_NOALLOC_MATRIX_WORDS words (1 MiB) inside the library, present on
 * every device that loads it until the process exits.  Requests needing
 * more (r*d*mmax words when S is set or alpha > 1) are rejected with
 * QMC_ERR_ARG.  The first call on a device looks the array up and should come
 * before any stream capture.  Calls share the array: calls whose kernels
 * overlap on the GPU race, so order them on one stream. */
#define QMC_NOALLOC_MATRIX_WORDS 131072
int qmc_net_gen_noalloc(const qmc_net_request *req, qmc_stream_t s);

/* ---- nested uniform (Owen) scrambling of base-2 digital nets ----------------
 * Replaces the reference's Python routine dnb2_nested_uniform_scramble
 * (qmctoolscl/rand_funcs.py:162-253), which the reference binds only in
 * Python (no C function exists for it); bit for bit its output and its
 * generators' advanced states.  One generator per (replication l, dimension
 * j), g = l*d + j, each numpy's SFC64 in six words (a, b, c, w, has_uint32,
 * uinteger) in `states` (r*d*6 words, device, updated in place).  The
 * reference keeps a tree per generator between calls; here a generator's
 * history is the keys (xb << (tmax_new - tmax), tmax_new bits) and draws of
 * every entry seen so far, phantom root entry first:
 *   h0 = 0: fresh trees (the phantom's tmax_new-bit draw comes first);
 *   h0 > 0: hist_keys / hist_draws hold r*d*h0 words, generator-major.
 * keys_out / draws_out (each r*d*(max(h0,1)+n) words, or NULL) receive the
 * history after the call, the history for the next call on the same trees.
 * xb (r_x, n, d), xrb (r, n, d) as in the reference (xrb[l] uses xb[l % r_x]).
 * All arrays are device memory.  `work` is a 256-byte aligned device
 * workspace of work_bytes: generators run in chunks of as many as fit
 * (qmc_dnb2_nus_workspace_size gives the bytes for a chunk of `generators`).
 * Stream-ordered, allocates nothing.  QMC_ERR_DOMAIN for tmax_new > 64 (the
 * reference asserts t <= 64); QMC_ERR_ARG for more than 2^30 - 1 entries per
 * generator or a workspace smaller than one generator needs. */
int qmc_dnb2_nus_workspace_size(uint64_t n, uint64_t h0, uint64_t generators, uint64_t *bytes);
int qmc_dnb2_nested_uniform_scramble(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t tmax,
                                     uint64_t tmax_new, uint64_t *states, uint64_t h0, const uint64_t *hist_keys,
                                     const uint64_t *hist_draws, const uint64_t *xb, uint64_t *xrb,
                                     uint64_t *keys_out, uint64_t *draws_out, void *work, uint64_t work_bytes,
                                     qmc_stream_t s);

/* ---- nested uniform (Owen) scrambling of generalized (base-b) nets ----------
 * Replaces the reference's Python routine gdn_nested_uniform_scramble
 * (qmctoolscl/rand_funcs.py:262-356): bit for bit its xrdig and its
 * generators' advanced states.  Generator g = l*d + j with base
 * bases[(l % r_b)*d + j] (2..65536) and numpy's SFC64 state in six words
 * (states, r*d*6, updated in place).  xdig (r_x, n, d, tmax) digits, xrdig
 * (r, n, d, tmax_new); needs 1 <= tmax < tmax_new <= 255 and
 * tmax * ceil(log2 b) <= 128 (the digits are compared as 128-bit keys).
 *
 * Trees.  h0 = 0 starts fresh trees (the call adds the phantom root as entry
 * 0).  A later call on the same trees passes what the earlier calls left:
 * h0 entries per tree (the phantom root and every earlier point, in call
 * order), their keys hist_keys (r*d, h0, 2) as the earlier call wrote them to
 * keys_out, and their permutation rows: generator g's at
 * hist_perms[hist_perm_off[g] .. hist_perm_off[g+1]) (device memory, r*d+1
 * offsets), as perm_off gave them.  The new points then continue each tree
 * exactly as the reference's nodes continue (draws from the generators'
 * current states).
 *
 * Outputs besides xrdig: keys_out (r*d, h0 + n, 2) (or h0 = 1 when fresh; may
 * be NULL) and every tree's rows, earlier ones copied in front: generator g's
 * at perms[perm_off[g] .. perm_off[g+1]), perm_off a HOST array of r*d+1
 * entries.  When perm_capacity 16-bit entries are too few, the call counts the
 * rest without drawing and returns QMC_ERR_ARG with the entries needed in
 * *perm_needed -- states of the generators drawn so far are then already
 * advanced, so a caller retries from its own copy.
 * A digit at or above its base sets bit 1 of the device error word (the
 * reference raises IndexError); history rows whose length disagrees with the
 * tree set bit 64.  Device memory throughout; `work` is a 256-byte aligned
 * workspace of work_bytes (qmc_gdn_nus_workspace_size with the same n and
 * h0); synchronises its stream twice per chunk of generators. */
int qmc_gdn_nus_workspace_size(uint64_t n, uint64_t h0, uint64_t generators, uint64_t *bytes);
int qmc_gdn_nested_uniform_scramble(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t r_b, uint64_t tmax,
                                    uint64_t tmax_new, uint64_t *states, const uint64_t *bases, uint64_t h0,
                                    const uint64_t *hist_keys, const uint16_t *hist_perms,
                                    const uint64_t *hist_perm_off, const uint64_t *xdig, uint64_t *xrdig,
                                    uint64_t *keys_out, uint16_t *perms, uint64_t perm_capacity, uint64_t *perm_off,
                                    uint64_t *perm_needed, void *work, uint64_t work_bytes, qmc_stream_t s);

/* ---- randomisation inputs on the GPU ----------------------------------------
 * The reference's numpy helpers (qmctoolscl/rand_funcs.py:4-153) bit for bit:
 * the same draws in the same order from one numpy Generator on an SFC64 bit
 * generator, whose six state words (a, b, c, w, has_uint32, uinteger -- the
 * fields of numpy's SFC64 state) are read from and written back to `state`
 * (device memory) in stream order.  One GPU thread runs the stream (it is
 * serial); fills and the permutations' swaps run wide.  Outputs are device
 * arrays laid out as the helpers return them; uint64 results as their bits.
 *   qmc_lat_get_shifts               rand_funcs.py:34-41   Generator.random((r, d))
 *   qmc_random_tbit_uint64s          rand_funcs.py:4-20    count values of t bits (0 <= t <= 64)
 *   qmc_dnb2_get_digital_shifts      rand_funcs.py:43-51   (r, d) values of tmax_new bits
 *   qmc_dnb2_get_linear_scramble_matrix  rand_funcs.py:53-78  (r, d, tmax_new); 1 <= tmax <= tmax_new
 *                                    (numpy's broadcasting refuses tmax > tmax_new)
 *   qmc_gdn_get_linear_scramble_matrix   rand_funcs.py:80-104 (r, d, tmax_new, tmax), bases r_b*d
 *   qmc_gdn_get_digital_shifts       rand_funcs.py:115-132 (r, d, tmax_new)
 *   qmc_gdn_get_digital_permutations rand_funcs.py:134-153 (r, d, tmax_new, bmax), zero padded;
 *                                    bmax = the largest base, at most 65536
 *   qmc_random_uint64_permutations   rand_funcs.py:22-32   (n, b), b at most 65536
 * Bases live in device memory.  A base numpy would refuse (below 2 for the
 * scrambling matrices, 0 for the shifts) or one above bmax sets bit 128 of
 * the device error word and stops the stream; a rejection loop that runs out
 * sets bit 32. */
int qmc_lat_get_shifts(uint64_t *state, uint64_t r, uint64_t d, double *shifts, qmc_stream_t s);
int qmc_random_tbit_uint64s(uint64_t *state, uint64_t t, uint64_t count, uint64_t *out, qmc_stream_t s);
int qmc_dnb2_get_digital_shifts(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax_new, uint64_t *shifts,
                                qmc_stream_t s);
int qmc_dnb2_get_linear_scramble_matrix(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax, uint64_t tmax_new,
                                        uint64_t *S, qmc_stream_t s);
int qmc_gdn_get_linear_scramble_matrix(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax, uint64_t tmax_new,
                                       uint64_t r_b, const uint64_t *bases, uint64_t *S, qmc_stream_t s);
int qmc_gdn_get_digital_shifts(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax_new, uint64_t r_b,
                               const uint64_t *bases, uint64_t *shifts, qmc_stream_t s);
int qmc_gdn_get_digital_permutations(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax_new, uint64_t r_b,
                                     const uint64_t *bases, uint64_t bmax, uint64_t *perms, qmc_stream_t s);
int qmc_random_uint64_permutations(uint64_t *state, uint64_t n, uint64_t b, uint64_t *out, qmc_stream_t s);

#ifdef __cplusplus
}
#endif

#endif /* QMCGB_H */
