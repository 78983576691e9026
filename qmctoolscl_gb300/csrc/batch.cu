// batch.cu -- many generation requests of uneven size (n, d, order, matrix
// sets) in one persistent launch, with CUDA-graph capture and replay.
//
// A plan holds one descriptor per request in device memory.  Each request is
// cut into tiles of about the same number of coordinates (a randomisation,
// a column tile of up to 64 columns for digital nets, and a run of rows), so
// every tile is about the same work whatever the request's shape.  A
// persistent grid (a few CTAs per SM) pulls chunks of consecutive tiles from
// a global counter with atomicAdd; consecutive tiles of a chunk usually share
// their (request, randomisation, column tile), so a CTA rebuilds its
// shared-memory table only when that changes.  No CTA ever waits for
// another: the last CTA to finish resets the counter for the next run, so a
// plan can be relaunched or replayed from a graph with no host work.
//
// Digital-net plans first run one matrix-preparation kernel over all
// requests (linear matrix scrambling and interlacing, one thread per output
// column word) into plan scratch, then the generation kernel.
//
// Reference chains reproduced, bit for bit: see qmc_net_request /
// qmc_lat_request in include/qmcgb.h.
#include <mutex>
#include <vector>

#include "lattice_dev.cuh"
#include "net_dev.cuh"

struct BatchCtrl {
    unsigned long long next;  // next tile to hand out
    unsigned int done;        // CTAs that have finished this run
    unsigned int pad;
};

namespace {

constexpr int THREADS = 256;

struct PrepDesc {
    u64 r, d, d_pre, mmax, alpha, nbits, tmax_alpha, r_C;
    const u64 *C, *S;
    u64 *out;        // r*d*mmax prepared matrices
    u64 word_begin;  // first global output word of this request
};

struct NetDesc {
    u64 r, n, d, n_start, mmax, r_C;
    const u64 *C;  // r_C*d*mmax, prepared or the caller's
    const u64 *lshifts, *shifts, *tmaxes;
    u64 *xb;
    double *x;
    u32 gray, K, col_tiles, pad;
    u64 rows_per_tile, row_tiles, tile_begin;
};

struct LatDesc {
    u64 r, n, d, n_start;
    const u64 *g;
    const double *shifts;
    double *x;
    u32 gray, p, narrow, vec2;
    u64 rows_per_tile, row_tiles, tile_begin;
};

// ------------------------------------------------------------ prep kernel

// index of the last descriptor whose `first` <= t (descriptors sorted)
template <typename D, typename F>
__device__ __forceinline__ int find_desc(const D *ds, int nd, u64 t, F first)
{
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first(ds[mid]) <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ u64 lms_word(const u64 *srow, u64 col, u64 tmax_new)
{
    u64 out = 0;
    for (u64 t = 0; t < tmax_new; t++)
        if (__popcll(srow[t] & col) & 1) out += shl64(1ull, tmax_new - t - 1);
    return out;
}

constexpr int MAX_ALPHA = 16;

// Word loc of one request's prepared matrices: LMS of the alpha source
// columns (dnb2_linear_matrix_scramble.c:32-48), then interlacing.
__device__ __forceinline__ void prep_word(const PrepDesc &P, u64 loc)
{
    {
        const u64 k = loc % P.mmax, ja = (loc / P.mmax) % P.d, l = loc / (P.mmax * P.d);
        const u64 *Cl = P.C + (l % P.r_C) * P.d_pre * P.mmax;
        u64 words[MAX_ALPHA];
        for (u64 a = 0; a < P.alpha; a++) {
            const u64 j = ja * P.alpha + a;
            const u64 col = Cl[j * P.mmax + k];
            words[a] = P.S ? lms_word(P.S + (l * P.d_pre + j) * P.nbits, col, P.nbits) : col;
        }
        u64 out;
        if (P.alpha == 1) {
            out = words[0];
        } else {  // dnb2_interlace.c:33-41 with tmax = nbits
            out = 0;
            for (u64 ta = 0; ta < P.tmax_alpha; ta++) {
                const u64 t = ta / P.alpha;
                if (shr64(words[ta % P.alpha], P.nbits - t - 1) & 1) out += shl64(1ull, P.tmax_alpha - ta - 1);
            }
        }
        P.out[loc] = out;
    }
}

__global__ void net_prep_kernel(const PrepDesc *ps, int np, u64 total)
{
    for (u64 w = (u64)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (u64)gridDim.x * blockDim.x) {
        const PrepDesc &P = ps[find_desc(ps, np, w, [](const PrepDesc &p) { return p.word_begin; })];
        prep_word(P, w - P.word_begin);
    }
}

// ------------------------------------------------------ generation kernels

__device__ __forceinline__ void finish_run(BatchCtrl *ctrl)
{
    // the last CTA to get here resets the queue; all others have already
    // taken their final (empty) grab, so nobody touches the counter after it
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int done = atomicAdd(&ctrl->done, 1u);
        if (done == gridDim.x - 1) {
            ctrl->next = 0;
            ctrl->done = 0;
            __threadfence();
        }
    }
}

__device__ __forceinline__ u64 grab(BatchCtrl *ctrl, u32 chunk, u64 *slot)
{
    if (threadIdx.x == 0) *slot = atomicAdd(&ctrl->next, (unsigned long long)chunk);
    __syncthreads();
    const u64 t0 = *slot;
    __syncthreads();
    return t0;
}

__global__ void __launch_bounds__(THREADS) net_batch_kernel(const NetDesc *reqs, int nreq, u64 total_tiles,
                                                            BatchCtrl *ctrl, u32 chunk)
{
    extern __shared__ u64 smem[];
    __shared__ u64 slot;
    int cur_q = -1;
    u64 cur_l = ~0ull;
    u32 cur_ct = ~0u;
    for (;;) {
        const u64 t0 = grab(ctrl, chunk, &slot);
        if (t0 >= total_tiles) break;
        const u64 t1 = min(t0 + chunk, total_tiles);
        for (u64 t = t0; t < t1; t++) {
            const int q = find_desc(reqs, nreq, t, [](const NetDesc &d) { return d.tile_begin; });
            const NetDesc &R = reqs[q];
            const u64 lt = t - R.tile_begin;
            const u64 per_l = (u64)R.col_tiles * R.row_tiles;
            const u64 l = lt / per_l, rem = lt % per_l;
            const u32 ct = (u32)(rem / R.row_tiles);
            const u64 rt = rem % R.row_tiles;
            const u64 j0 = (u64)ct * net::MAX_COLS;
            const u32 ncols = (u32)min((u64)net::MAX_COLS, R.d - j0);
            u64 *T = smem;
            u64 *H = smem + ((u64)1 << R.K) * ncols;
            if (q != cur_q || l != cur_l || ct != cur_ct) {
                __syncthreads();  // every thread is done with the previous table
                const u32 ls = R.shifts ? (u32)(R.lshifts[l] & 63) : 0u;
                net::build_table(T, H, R.C + (l % R.r_C) * R.d * R.mmax, R.mmax, j0, ncols, R.K, ls,
                                 R.shifts ? R.shifts + l * R.d : nullptr);
                cur_q = q;
                cur_l = l;
                cur_ct = ct;
            }
            const u64 row0 = rt * R.rows_per_tile, row1 = min(R.n, row0 + R.rows_per_tile);
            const int e_float = R.x ? (int)(u32)(0ull - R.tmaxes[l]) : 0;
            u64 *xb_l = R.xb ? R.xb + l * R.n * R.d + j0 : nullptr;
            double *x_l = R.x ? R.x + l * R.n * R.d + j0 : nullptr;
            if (R.gray)
                net::gen_rows<true>(T, H, R.K, ncols, R.n_start, R.d, row0, row1, xb_l, x_l, e_float);
            else
                net::gen_rows<false>(T, H, R.K, ncols, R.n_start, R.d, row0, row1, xb_l, x_l, e_float);
        }
    }
    finish_run(ctrl);
}

template <int ORDER, bool SHIFT, int VEC>
__device__ __forceinline__ void lat_tile(const LatDesc &R, u64 l, u64 row0, u64 row1)
{
    const u64 ngroups = (R.d + VEC - 1) / VEC;
    u32 bx = 1;
    while (bx < ngroups && bx < 32) bx <<= 1;
    const u32 by = THREADS / bx;
    const u32 cg = threadIdx.x % bx, ry = threadIdx.x / bx;
    for (u64 jg = cg; jg < ngroups; jg += bx)
        lat::rows<ORDER, SHIFT, VEC>(R.g + l * R.d, SHIFT ? R.shifts + l * R.d : nullptr, R.x + l * R.n * R.d, R.d,
                                     R.n, R.n_start, R.p, jg, row0 + ry, row1, by, R.narrow != 0);
}

__global__ void __launch_bounds__(THREADS) lat_batch_kernel(const LatDesc *reqs, int nreq, u64 total_tiles,
                                                            BatchCtrl *ctrl, u32 chunk)
{
    __shared__ u64 slot;
    for (;;) {
        const u64 t0 = grab(ctrl, chunk, &slot);
        if (t0 >= total_tiles) break;
        const u64 t1 = min(t0 + chunk, total_tiles);
        for (u64 t = t0; t < t1; t++) {
            const LatDesc &R = reqs[find_desc(reqs, nreq, t, [](const LatDesc &d) { return d.tile_begin; })];
            const u64 lt = t - R.tile_begin;
            const u64 l = lt / R.row_tiles, rt = lt % R.row_tiles;
            const u64 row0 = rt * R.rows_per_tile, row1 = min(R.n, row0 + R.rows_per_tile);
            const int sel = (R.gray ? 4 : 0) | (R.shifts ? 2 : 0) | (R.vec2 ? 1 : 0);
            switch (sel) {
            case 0: lat_tile<lat::NATURAL, false, 1>(R, l, row0, row1); break;
            case 1: lat_tile<lat::NATURAL, false, 2>(R, l, row0, row1); break;
            case 2: lat_tile<lat::NATURAL, true, 1>(R, l, row0, row1); break;
            case 3: lat_tile<lat::NATURAL, true, 2>(R, l, row0, row1); break;
            case 4: lat_tile<lat::GRAY, false, 1>(R, l, row0, row1); break;
            case 5: lat_tile<lat::GRAY, false, 2>(R, l, row0, row1); break;
            case 6: lat_tile<lat::GRAY, true, 1>(R, l, row0, row1); break;
            default: lat_tile<lat::GRAY, true, 2>(R, l, row0, row1); break;
            }
        }
    }
    finish_run(ctrl);
}

bool gray_closed(u64 lo, u64 hi)
{
    u64 a = lo;
    while (a < hi) {
        u32 k = a ? (u32)__builtin_ctzll(a) : 63;
        while (k > 0 && (a + (1ull << k) > hi || a + (1ull << k) < a)) k--;
        const u64 q = a >> k, g = q ^ (q >> 1);
        if ((g << k) < lo || (g << k) + (1ull << k) > hi) return false;
        a += 1ull << k;
    }
    return true;
}

}  // namespace

// ------------------------------------------------------------------- plan

struct qmc_plan {
    int kind = 0;  // 1: digital net, 2: lattice
    int device = 0;
    std::vector<NetDesc> net;
    std::vector<LatDesc> lat;
    std::vector<PrepDesc> prep;
    std::vector<u64> tile_rows_base;  // rows_per_tile chosen from tile_coords
    void *d_desc = nullptr, *d_prep = nullptr;
    u64 *d_scratch = nullptr;
    BatchCtrl *d_ctrl = nullptr;
    u64 total_tiles = 0, prep_words = 0, coords = 0, bytes_out = 0;
    size_t smem = 0;
    int ctas_per_sm = 4;
    u32 chunk = 4;
    u64 tile_coords = 1ull << 16;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

void drop_graph(qmc_plan *p)
{
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
}

// Cut every request into tiles of about tile_coords coordinates and upload
// the descriptors.
int layout_tiles(qmc_plan *p)
{
    u64 tile = 0;
    if (p->kind == 1) {
        for (auto &R : p->net) {
            const u32 ncols = (u32)(R.d < (u64)net::MAX_COLS ? R.d : (u64)net::MAX_COLS);
            u64 rows = p->tile_coords / ncols;
            const u64 min_rows = 1ull << R.K;  // a table's worth of rows at least
            if (rows < min_rows) rows = min_rows;
            if (rows > R.n) rows = R.n;
            R.rows_per_tile = rows ? rows : 1;
            R.row_tiles = (R.n + R.rows_per_tile - 1) / R.rows_per_tile;
            R.tile_begin = tile;
            tile += R.r * R.col_tiles * R.row_tiles;
        }
    } else {
        for (auto &R : p->lat) {
            u64 rows = p->tile_coords / (R.d ? R.d : 1);
            if (rows < 8) rows = 8;
            if (rows > R.n) rows = R.n;
            R.rows_per_tile = rows ? rows : 1;
            R.row_tiles = (R.n + R.rows_per_tile - 1) / R.rows_per_tile;
            R.tile_begin = tile;
            tile += R.r * R.row_tiles;
        }
    }
    p->total_tiles = tile;
    const size_t bytes = p->kind == 1 ? p->net.size() * sizeof(NetDesc) : p->lat.size() * sizeof(LatDesc);
    const void *src = p->kind == 1 ? (const void *)p->net.data() : (const void *)p->lat.data();
    return qmcgb::cuda_status(cudaMemcpy(p->d_desc, src, bytes, cudaMemcpyHostToDevice), "uploading descriptors");
}

int alloc_common(qmc_plan *p, size_t desc_bytes)
{
    cudaGetDevice(&p->device);
    if (int rc = qmcgb::cuda_status(cudaMalloc(&p->d_desc, desc_bytes ? desc_bytes : 16), "cudaMalloc")) return rc;
    if (int rc = qmcgb::cuda_status(cudaMalloc((void **)&p->d_ctrl, sizeof(BatchCtrl)), "cudaMalloc")) return rc;
    return qmcgb::cuda_status(cudaMemset(p->d_ctrl, 0, sizeof(BatchCtrl)), "cudaMemset");
}

int launch(qmc_plan *p, cudaStream_t s)
{
    const int sms = qmcgb::sm_count();
    if (p->kind == 1 && p->prep_words) {
        net_prep_kernel<<<qmcgb::grid_for(p->prep_words, 256, (unsigned)sms * 8), 256, 0, s>>>(
            (const PrepDesc *)p->d_prep, (int)p->prep.size(), p->prep_words);
        if (int rc = qmcgb::launch_status("net_prep_kernel")) return rc;
    }
    if (p->total_tiles == 0) return QMC_OK;
    u64 grid = (u64)sms * (u64)p->ctas_per_sm;
    const u64 grabs = (p->total_tiles + p->chunk - 1) / p->chunk;
    if (grid > grabs) grid = grabs;
    if (p->kind == 1) {
        net_batch_kernel<<<(unsigned)grid, THREADS, p->smem, s>>>((const NetDesc *)p->d_desc, (int)p->net.size(),
                                                                   p->total_tiles, p->d_ctrl, p->chunk);
    } else {
        lat_batch_kernel<<<(unsigned)grid, THREADS, 0, s>>>((const LatDesc *)p->d_desc, (int)p->lat.size(),
                                                             p->total_tiles, p->d_ctrl, p->chunk);
    }
    return qmcgb::launch_status("batch kernel");
}

u32 bitlen(u64 v) { return v ? 64u - (u32)__builtin_clzll(v) : 0u; }

}  // namespace

extern "C" {

int qmc_net_plan_create(const qmc_net_request *reqs, int nreq, qmc_plan **plan)
{
    QMC_REQUIRE(plan && (nreq == 0 || reqs) && nreq >= 0, "bad plan arguments");
    *plan = nullptr;
    qmc_plan *p = new qmc_plan();
    p->kind = 1;
    u64 scratch_words = 0;
    for (int q = 0; q < nreq; q++) {
        const qmc_net_request &Q = reqs[q];
        const u64 alpha = Q.alpha ? Q.alpha : 1;
        if (Q.r == 0 || Q.n == 0 || Q.d == 0) continue;
        const char *bad = nullptr;
        if (!Q.C || (!Q.xb && !Q.x)) bad = "null matrices or no output";
        else if (Q.shifts && !Q.lshifts) bad = "shifts without lshifts";
        else if (Q.x && !Q.tmaxes) bad = "float output without tmaxes";
        else if (alpha > 16) bad = "alpha above 16";
        else if (Q.d_pre != Q.d * alpha) bad = "d_pre must equal d*alpha";
        else if (Q.mmax > 64) bad = "mmax above 64";
        else if (Q.r_C == 0) bad = "r_C is 0";
        if (bad) {
            delete p;
            qmcgb::set_error("request %d: %s", q, bad);
            return QMC_ERR_ARG;
        }
        if ((!Q.gray && !gray_closed(Q.n_start, Q.n_start + Q.n)) || bitlen(Q.n_start + Q.n - 1) > Q.mmax ||
            Q.n_start + Q.n < Q.n_start) {
            delete p;
            qmcgb::set_error("request %d: index range not covered by the generating matrices (or not Gray-closed "
                             "in natural order)", q);
            return QMC_ERR_DOMAIN;
        }
        NetDesc R{};
        R.r = Q.r;
        R.n = Q.n;
        R.d = Q.d;
        R.n_start = Q.n_start;
        R.mmax = Q.mmax;
        R.lshifts = Q.shifts ? (const u64 *)Q.lshifts : nullptr;
        R.shifts = (const u64 *)Q.shifts;
        R.tmaxes = Q.x ? (const u64 *)Q.tmaxes : nullptr;
        R.xb = (u64 *)Q.xb;
        R.x = Q.x;
        R.gray = Q.gray ? 1u : 0u;
        const u32 ncols = (u32)(Q.d < (u64)net::MAX_COLS ? Q.d : (u64)net::MAX_COLS);
        R.K = net::pick_K(Q.mmax, ncols);
        R.col_tiles = (u32)((Q.d + net::MAX_COLS - 1) / net::MAX_COLS);
        const size_t sm = net::table_words(R.K, Q.mmax, ncols) * sizeof(u64);
        if (sm > p->smem) p->smem = sm;
        if (Q.S || alpha > 1) {
            PrepDesc P{};
            P.r = Q.r;
            P.d = Q.d;
            P.d_pre = Q.d_pre;
            P.mmax = Q.mmax;
            P.alpha = alpha;
            P.nbits = Q.S ? Q.tmax_new : Q.tmax;
            P.tmax_alpha = Q.tmax_alpha;
            P.r_C = Q.r_C;
            P.C = (const u64 *)Q.C;
            P.S = (const u64 *)Q.S;
            P.word_begin = p->prep_words;
            P.out = (u64 *)(uintptr_t)(scratch_words);  // offset; made a pointer below
            p->prep.push_back(P);
            R.C = (const u64 *)(uintptr_t)(scratch_words);
            R.r_C = Q.r;
            R.pad = 1;  // C is an offset into plan scratch
            scratch_words += Q.r * Q.d * Q.mmax;
            p->prep_words += Q.r * Q.d * Q.mmax;
        } else {
            R.C = (const u64 *)Q.C;
            R.r_C = Q.r_C;
        }
        p->coords += Q.r * Q.n * Q.d;
        p->bytes_out += Q.r * Q.n * Q.d * ((Q.xb ? 8 : 0) + (Q.x ? 8 : 0));
        p->net.push_back(R);
    }
    int rc = alloc_common(p, p->net.size() * sizeof(NetDesc));
    if (!rc && scratch_words)
        rc = qmcgb::cuda_status(cudaMalloc((void **)&p->d_scratch, scratch_words * sizeof(u64)), "cudaMalloc");
    if (!rc && !p->prep.empty()) {
        for (auto &P : p->prep) P.out = p->d_scratch + (uintptr_t)P.out;
        rc = qmcgb::cuda_status(cudaMalloc(&p->d_prep, p->prep.size() * sizeof(PrepDesc)), "cudaMalloc");
        if (!rc)
            rc = qmcgb::cuda_status(cudaMemcpy(p->d_prep, p->prep.data(), p->prep.size() * sizeof(PrepDesc),
                                               cudaMemcpyHostToDevice), "uploading prep descriptors");
    }
    for (auto &R : p->net)
        if (R.pad) {
            R.C = p->d_scratch + (uintptr_t)R.C;
            R.pad = 0;
        }
    if (!rc) rc = qmcgb::raise_smem_limit((const void *)net_batch_kernel, p->smem, "net_batch_kernel smem");
    if (!rc) rc = layout_tiles(p);
    if (rc) {
        qmc_plan_destroy(p);
        return rc;
    }
    *plan = p;
    return QMC_OK;
}

int qmc_lat_plan_create(const qmc_lat_request *reqs, int nreq, qmc_plan **plan)
{
    QMC_REQUIRE(plan && (nreq == 0 || reqs) && nreq >= 0, "bad plan arguments");
    *plan = nullptr;
    qmc_plan *p = new qmc_plan();
    p->kind = 2;
    for (int q = 0; q < nreq; q++) {
        const qmc_lat_request &Q = reqs[q];
        if (Q.r == 0 || Q.n == 0 || Q.d == 0) continue;
        if (!Q.g || !Q.x) {
            delete p;
            qmcgb::set_error("request %d: null g or x", q);
            return QMC_ERR_ARG;
        }
        if (!Q.gray && ((Q.n_start & (Q.n_start - 1)) || ((Q.n + Q.n_start) & (Q.n + Q.n_start - 1)))) {
            delete p;
            qmcgb::set_error("request %d: lat_gen_natural requires n_start and n+n_start are either 0 or powers of 2",
                             q);
            return QMC_ERR_ARG;
        }
        LatDesc R{};
        R.r = Q.r;
        R.n = Q.n;
        R.d = Q.d;
        R.n_start = Q.n_start;
        R.g = (const u64 *)Q.g;
        R.shifts = Q.shifts;
        R.x = Q.x;
        R.gray = Q.gray ? 1u : 0u;
        R.p = bitlen(Q.n_start + Q.n - 1);
        R.narrow = (Q.n_start + Q.n <= (1ull << 32) && Q.n_start + Q.n >= Q.n_start) ? 1u : 0u;
        R.vec2 = (Q.d % 2 == 0 && ((uintptr_t)Q.x & 15) == 0) ? 1u : 0u;
        p->coords += Q.r * Q.n * Q.d;
        p->bytes_out += Q.r * Q.n * Q.d * 8;
        p->lat.push_back(R);
    }
    int rc = alloc_common(p, p->lat.size() * sizeof(LatDesc));
    if (!rc) rc = layout_tiles(p);
    if (rc) {
        qmc_plan_destroy(p);
        return rc;
    }
    *plan = p;
    return QMC_OK;
}

int qmc_plan_run(qmc_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p, "null plan");
    return launch(p, QMC_STREAM(s));
}

int qmc_plan_graph_launch(qmc_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p, "null plan");
    QMC_REQUIRE(s != nullptr, "graph capture needs a stream other than the legacy default stream");
    cudaStream_t st = QMC_STREAM(s);
    if (!p->exec) {
        if (int rc = qmcgb::cuda_status(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "capture"))
            return rc;
        const int lrc = launch(p, st);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        if (lrc) {
            if (g) cudaGraphDestroy(g);
            return lrc;
        }
        if (int rc = qmcgb::cuda_status(e, "end capture")) return rc;
        p->graph = g;
        if (int rc = qmcgb::cuda_status(cudaGraphInstantiate(&p->exec, g, 0), "instantiate")) {
            drop_graph(p);
            return rc;
        }
    }
    return qmcgb::cuda_status(cudaGraphLaunch(p->exec, st), "cudaGraphLaunch");
}

int qmc_plan_set_tuning(qmc_plan *p, int ctas_per_sm, int chunk, uint64_t tile_coords)
{
    QMC_REQUIRE(p, "null plan");
    QMC_REQUIRE(ctas_per_sm >= 0 && ctas_per_sm <= 32 && chunk >= 0 && chunk <= 1024, "tuning out of range");
    if (ctas_per_sm) p->ctas_per_sm = ctas_per_sm;
    if (chunk) p->chunk = (u32)chunk;
    drop_graph(p);
    if (tile_coords && tile_coords != p->tile_coords) {
        p->tile_coords = tile_coords;
        // the previous run may still read the descriptors
        if (int rc = qmcgb::cuda_status(cudaDeviceSynchronize(), "synchronise before re-tiling")) return rc;
        return layout_tiles(p);
    }
    return QMC_OK;
}

int qmc_plan_info(const qmc_plan *p, uint64_t *tiles, uint64_t *coords, uint64_t *bytes_out, int *launches)
{
    QMC_REQUIRE(p, "null plan");
    if (tiles) *tiles = p->total_tiles;
    if (coords) *coords = p->coords;
    if (bytes_out) *bytes_out = p->bytes_out;
    if (launches) *launches = (p->prep_words ? 1 : 0) + (p->total_tiles ? 1 : 0);
    return QMC_OK;
}

int qmc_plan_destroy(qmc_plan *p)
{
    if (!p) return QMC_OK;
    drop_graph(p);
    if (p->d_desc) cudaFree(p->d_desc);
    if (p->d_prep) cudaFree(p->d_prep);
    if (p->d_scratch) cudaFree(p->d_scratch);
    if (p->d_ctrl) cudaFree(p->d_ctrl);
    delete p;
    return QMC_OK;
}

}  // extern "C"

// ------------------------------------------------- entry point without allocation
//
// qmc_net_gen_noalloc runs one digital-net request -- the same chain as a
// one-request plan -- without allocating any device memory.  It exists for
// callers that cannot call cudaMalloc: a process whose device memory is
// already handed to another allocator (a framework's caching pool, a fixed
// arena in a serving process), where a raw cudaMalloc fails or escapes the
// pool's accounting, and latency-bound loops that must not pay cudaMalloc's
// implicit device synchronisation.  Inputs and outputs stay the caller's.
//
// The only scratch it needs, the scrambled and interlaced generating
// matrices, lives in the file-scope array below: QMC_NOALLOC_MATRIX_WORDS
// 64-bit words (1 MiB) on every device that loads this library, held until
// the process exits.  Host code reaches it through the address that
// cudaGetSymbolAddress returns for the current device (the array's name in
// host code is only a stand-in, not a device address); the lookup is done by
// the first call on each device, so that first call should come before any
// stream capture.  Every call shares the array and it keeps the last call's
// contents; the preparation kernel overwrites every word a call reads, so
// nothing has to start at zero.  Calls whose kernels overlap on the GPU (on
// different streams, or from different host threads without ordering) race
// on the array: order them on one stream.

static __device__ __align__(256) unsigned long long g_noalloc_matrices[QMC_NOALLOC_MATRIX_WORDS];

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
u64 *g_noalloc_ptr[NOALLOC_MAX_DEVICES];

// device address of g_noalloc_matrices on the current device, looked up once
int noalloc_scratch(u64 **out)
{
    int dev = 0;
    if (int rc = qmcgb::cuda_status(cudaGetDevice(&dev), "cudaGetDevice")) return rc;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        qmcgb::set_error("device %d is beyond the %d devices this entry point serves", dev, NOALLOC_MAX_DEVICES);
        return QMC_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_matrices);
        if (e != cudaSuccess) return qmcgb::cuda_status(e, "cudaGetSymbolAddress of the matrix scratch");
        g_noalloc_ptr[dev] = (u64 *)p;
    }
    *out = g_noalloc_ptr[dev];
    return QMC_OK;
}

__global__ void net_prep_one_kernel(PrepDesc P, u64 total)
{
    for (u64 w = (u64)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (u64)gridDim.x * blockDim.x)
        prep_word(P, w);
}

}  // namespace

extern "C" int qmc_net_gen_noalloc(const qmc_net_request *req, qmc_stream_t s)
{
    QMC_REQUIRE(req, "null request");
    const qmc_net_request &Q = *req;
    if (Q.r == 0 || Q.n == 0 || Q.d == 0) return QMC_OK;
    const u64 alpha = Q.alpha ? Q.alpha : 1;
    QMC_REQUIRE(Q.C && (Q.xb || Q.x), "null matrices or no output");
    QMC_REQUIRE(!Q.shifts || Q.lshifts, "shifts without lshifts");
    QMC_REQUIRE(!Q.x || Q.tmaxes, "float output without tmaxes");
    QMC_REQUIRE(alpha <= (u64)MAX_ALPHA && Q.d <= UINT64_MAX / alpha && Q.d_pre == Q.d * alpha && Q.mmax <= 64 &&
                    Q.r_C > 0,
                "bad alpha, d_pre, mmax or r_C");
    if ((!Q.gray && !gray_closed(Q.n_start, Q.n_start + Q.n)) || bitlen(Q.n_start + Q.n - 1) > Q.mmax ||
        Q.n_start + Q.n < Q.n_start) {
        qmcgb::set_error("index range not covered by the generating matrices (or not Gray-closed in natural order)");
        return QMC_ERR_DOMAIN;
    }
    const bool prep = Q.S || alpha > 1;
    // r*d*mmax bounded factor by factor, so that no product can wrap below the limit
    const u64 per_r = Q.d <= (u64)QMC_NOALLOC_MATRIX_WORDS ? Q.d * (Q.mmax ? Q.mmax : 1) : UINT64_MAX;
    QMC_REQUIRE(!prep || (per_r <= (u64)QMC_NOALLOC_MATRIX_WORDS && Q.r <= (u64)QMC_NOALLOC_MATRIX_WORDS / per_r),
                "qmc_net_gen_noalloc: the request needs r*d*mmax words of matrix scratch (r=%llu, d=%llu, "
                "mmax=%llu), above the %d this entry point holds; use a plan (qmc_net_plan_create) for it",
                (unsigned long long)Q.r, (unsigned long long)Q.d, (unsigned long long)Q.mmax,
                QMC_NOALLOC_MATRIX_WORDS);
    const u64 words = Q.r * Q.d * Q.mmax;
    cudaStream_t st = QMC_STREAM(s);
    const u64 *C = (const u64 *)Q.C;
    u64 r_C = Q.r_C;
    if (prep) {
        u64 *scratch = nullptr;
        if (int rc = noalloc_scratch(&scratch)) return rc;
        PrepDesc P{};
        P.r = Q.r;
        P.d = Q.d;
        P.d_pre = Q.d_pre;
        P.mmax = Q.mmax;
        P.alpha = alpha;
        P.nbits = Q.S ? Q.tmax_new : Q.tmax;
        P.tmax_alpha = Q.tmax_alpha;
        P.r_C = Q.r_C;
        P.C = (const u64 *)Q.C;
        P.S = (const u64 *)Q.S;
        P.out = scratch;
        net_prep_one_kernel<<<qmcgb::grid_for(words, 256, (unsigned)qmcgb::sm_count() * 8), 256, 0, st>>>(P, words);
        if (int rc = qmcgb::launch_status("net_prep_one_kernel")) return rc;
        C = scratch;
        r_C = Q.r;
    }
    return qmcgb::dnb2_gen_fused(Q.r, Q.n, Q.d, Q.n_start, Q.mmax, C, r_C, Q.gray ? 1 : 0,
                                 Q.shifts ? (const u64 *)Q.lshifts : nullptr, Q.r, (const u64 *)Q.shifts,
                                 Q.x ? (const u64 *)Q.tmaxes : nullptr, (u64 *)Q.xb, Q.x, st);
}
