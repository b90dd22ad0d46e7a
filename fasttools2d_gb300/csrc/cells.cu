// cells.cu -- device cell list for the real-space sums.
//
// Restates the reference's Assign (PeriodicEwald/src/mex/common/ewald_tools.cpp:7-80):
// boxes are nside_x x nside_y, numbered box_y*nside_x + box_x, points are
// binned with floor(nside (x/L + 0.5)) clamped to the box range.  On the GPU
// the counting sort is a histogram with atomics (which also hands each point
// its slot inside its box), an exclusive scan, and a scatter that writes the
// sorted positions together with the per-source densities the near-field
// kernels read (f for the Stokeslet, S = f (x) n folded to three numbers for
// the stresslet).  The order of points inside a box is not the input order
// (the reference keeps input order); only the summation order differs.
#include "fte_internal.cuh"

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_assign(const double* __restrict__ p, int64_t n, int nsx, int nsy, double Lx, double Ly,
                         int* __restrict__ box, int* __restrict__ rank, int* __restrict__ counts) {
    const double rLx = __drcp_rn(Lx), rLy = __drcp_rn(Ly);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = p[2 * i], y = p[2 * i + 1];
        int b = fte_cell_1d(y, Ly, rLy, nsy) * nsx + fte_cell_1d(x, Lx, rLx, nsx);
        box[i] = b;
        rank[i] = atomicAdd(&counts[b], 1);
    }
}

// block-wide exclusive scan of kScanTile ints; writes the tile total
__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, int n, int* __restrict__ tile_sums) {
    __shared__ int warp_tot[kScanThreads / 32];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int x = (base + k < n) ? in[base + k] : 0;
        v[k] = s;
        s += x;
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += u;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = ti - t;
        if (lane == kScanThreads / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = ti;
    }
    __syncthreads();
    int excl = warp_tot[warp] + incl - s;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) out[base + k] = excl + v[k];
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ tile_offs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_offs[i / kScanTile];
}

template <int KIND>
__global__ void k_scatter_src(const double* __restrict__ p, const double* __restrict__ f,
                              const double* __restrict__ nrm, const double* __restrict__ wts, int64_t n,
                              const int* __restrict__ box, const int* __restrict__ rank, const int* __restrict__ off,
                              double2* __restrict__ spos, double* __restrict__ q0, double* __restrict__ q1,
                              double* __restrict__ q2, int* __restrict__ sidx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int d = off[box[i]] + rank[i];
        spos[d] = make_double2(p[2 * i], p[2 * i + 1]);
        sidx[d] = (int)i;
        double f1 = f[2 * i], f2 = f[2 * i + 1];
        if (wts) {
            f1 *= wts[i];
            f2 *= wts[i];
        }
        if (KIND == FTE_KIND_SLP) {
            q0[d] = f1;
            q1[d] = f2;
        } else {
            double n1 = nrm[2 * i], n2 = nrm[2 * i + 1];
            q0[d] = f1 * n1;
            q1[d] = f1 * n2 + f2 * n1;
            q2[d] = f2 * n2;
        }
    }
}

__global__ void k_scatter_tar(const double* __restrict__ p, int64_t n, const int* __restrict__ box,
                              const int* __restrict__ rank, const int* __restrict__ off, double2* __restrict__ tpos,
                              int* __restrict__ tidx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int d = off[box[i]] + rank[i];
        tpos[d] = make_double2(p[2 * i], p[2 * i + 1]);
        tidx[d] = (int)i;
    }
}

// Grid tile of a point for the k-space kernels: floor((x + L/2)/h), the node
// index FindClosestNode starts from, divided by the tile size, clamped.
// With W > 0 (target bins of the tiled gathers, W = the staged region's row
// length) a point also gets the residue mod 16 of its window's first row in
// the staged region, counted per (tile, residue): k_tile_scatter then orders
// each tile's points round-robin over the residues, so that the 16 threads
// of a half-warp, which read the region at those rows' offsets, mostly hit
// distinct shared-memory banks (8-byte values).  The order is a heuristic:
// the node it assumes ignores the tie-break of FindClosestNode.
__global__ void k_tile_assign(const double* __restrict__ p, int64_t n, double Lx, double Ly, double hx, double hy,
                              int ts, int ntx, int nty, int* __restrict__ tile, int* __restrict__ rank,
                              int* __restrict__ counts, int W, int* __restrict__ counts16) {
    const double lhx = __dmul_rn(Lx, 0.5), lhy = __dmul_rn(Ly, 0.5), rhx = __drcp_rn(hx), rhy = __drcp_rn(hy);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double ax = floor(fte_div_rcp(__dadd_rn(p[2 * i], lhx), hx, rhx));
        double ay = floor(fte_div_rcp(__dadd_rn(p[2 * i + 1], lhy), hy, rhy));
        ax = fmin(fmax(ax, 0.0), (double)(ntx * ts - 1));
        ay = fmin(fmax(ay, 0.0), (double)(nty * ts - 1));
        int tx = min((int)ax / ts, ntx - 1), ty = min((int)ay / ts, nty - 1);
        int t = ty * ntx + tx;
        tile[i] = t;
        const int rk = atomicAdd(&counts[t], 1);
        if (W > 0) {
            const int r = (((int)ax - tx * ts + 2) * W + ((int)ay - ty * ts + 2)) & 15;
            rank[i] = (r << 26) | atomicAdd(&counts16[16 * t + r], 1);
        } else {
            rank[i] = rk;
        }
    }
}

// W > 0: position in the tile = the points of earlier rounds (sum over
// residues of min(count, round)) + the earlier residues present in this
// round; a bijection onto the tile's slots
__global__ void k_tile_scatter(int64_t n, const int* __restrict__ tile, const int* __restrict__ rank,
                               const int* __restrict__ off, int* __restrict__ perm, int W,
                               const int* __restrict__ counts16) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int t = tile[i];
        int pos = rank[i];
        if (W > 0) {
            const int r = pos >> 26, q = pos & ((1 << 26) - 1);
            const int* c = counts16 + 16 * t;
            pos = 0;
#pragma unroll
            for (int b = 0; b < 16; b++) {
                const int cb = c[b];
                pos += min(cb, q) + ((b < r && cb > q) ? 1 : 0);
            }
        }
        perm[off[t] + pos] = (int)i;
    }
}

inline int grid_for(int64_t n, int threads, int max_blocks) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

}  // namespace

int fte_scan_exclusive(fte_context* ctx, WsCarver& wc, const int* in, int* out, int n) {
    if (n <= 0) return FTE_OK;
    int tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        FTE_LAUNCH(ctx, k_scan_tiles, 1, kScanThreads, 0, in, out, n, (int*)nullptr);
        return FTE_OK;
    }
    int* sums = wc.take<int>(tiles);
    int* offs = wc.take<int>(tiles);
    FTE_WS_CHECK(wc);
    FTE_LAUNCH(ctx, k_scan_tiles, tiles, kScanThreads, 0, in, out, n, sums);
    FTE_TRY(fte_scan_exclusive(ctx, wc, sums, offs, tiles));
    FTE_LAUNCH(ctx, k_scan_add, (n + 255) / 256, 256, 0, out, n, (const int*)offs);
    return FTE_OK;
}

size_t fte_cells_ws(int64_t nsrc, int64_t ntar, int nb) {
    size_t s = 0;
    s += 2 * ws_bytes(nb + 1, sizeof(int));                      // counts
    s += 2 * ws_bytes(nb + 1, sizeof(int));                      // offsets
    s += 2 * ws_bytes((size_t)(nsrc + 1), sizeof(int));          // src box, rank
    s += 2 * ws_bytes((size_t)(ntar + 1), sizeof(int));          // tar box, rank
    s += ws_bytes((size_t)(nsrc + 1), sizeof(double2));          // spos
    s += 3 * ws_bytes((size_t)(nsrc + 1), sizeof(double));       // q0..q2
    s += ws_bytes((size_t)(ntar + 1), sizeof(double2));          // tpos
    s += ws_bytes((size_t)(ntar + 1), sizeof(int));              // tidx
    s += ws_bytes((size_t)(nsrc + 1), sizeof(int));              // sidx
    s += 4 * ws_bytes((size_t)(nb + 1) / 4096 + 8, sizeof(int)); // scan partials
    return s + 4096;
}

int fte_cells_build(fte_context* ctx, WsCarver& wc, int kind, const double* psrc, int64_t nsrc, const double* ptar,
                    int64_t ntar, const double* f, const double* nrm, const double* wts, int nsx, int nsy, double Lx,
                    double Ly, CellList* cl) {
    int nb = nsx * nsy;
    cl->nsx = nsx;
    cl->nsy = nsy;
    cl->nb = nb;
    cl->nsrc = nsrc;
    int* scnt = wc.take<int>(nb + 1);
    int* tcnt = wc.take<int>(nb + 1);
    cl->src_off = wc.take<int>(nb + 1);
    cl->tar_off = wc.take<int>(nb + 1);
    int* sbox = wc.take<int>(nsrc + 1);
    int* srank = wc.take<int>(nsrc + 1);
    int* tbox = wc.take<int>(ntar + 1);
    int* trank = wc.take<int>(ntar + 1);
    cl->spos = wc.take<double2>(nsrc + 1);
    cl->q0 = wc.take<double>(nsrc + 1);
    cl->q1 = wc.take<double>(nsrc + 1);
    cl->q2 = wc.take<double>(nsrc + 1);
    cl->tpos = wc.take<double2>(ntar + 1);
    cl->tidx = wc.take<int>(ntar + 1);
    cl->max_neigh = 0;
    cl->qstride = 0;
    cl->sidx = wc.take<int>(nsrc + 1);
    FTE_WS_CHECK(wc);
    FTE_WS_CHECK(wc);
    FTE_CUDA_TRY(cudaMemsetAsync(scnt, 0, sizeof(int) * (nb + 1), ctx->stream));
    FTE_CUDA_TRY(cudaMemsetAsync(tcnt, 0, sizeof(int) * (nb + 1), ctx->stream));
    int maxb = ctx->num_sms * 8;
    if (nsrc > 0)
        FTE_LAUNCH(ctx, k_assign, grid_for(nsrc, 256, maxb), 256, 0, psrc, nsrc, nsx, nsy, Lx, Ly, sbox, srank, scnt);
    if (ntar > 0)
        FTE_LAUNCH(ctx, k_assign, grid_for(ntar, 256, maxb), 256, 0, ptar, ntar, nsx, nsy, Lx, Ly, tbox, trank, tcnt);
    FTE_TRY(fte_scan_exclusive(ctx, wc, scnt, cl->src_off, nb + 1));
    FTE_TRY(fte_scan_exclusive(ctx, wc, tcnt, cl->tar_off, nb + 1));
    if (nsrc > 0) {
        if (kind == FTE_KIND_SLP)
            FTE_LAUNCH(ctx, k_scatter_src<FTE_KIND_SLP>, grid_for(nsrc, 256, maxb), 256, 0, psrc, f, nrm, wts, nsrc,
                       (const int*)sbox, (const int*)srank, (const int*)cl->src_off, cl->spos, cl->q0, cl->q1, cl->q2,
                       cl->sidx);
        else
            FTE_LAUNCH(ctx, k_scatter_src<FTE_KIND_DLP>, grid_for(nsrc, 256, maxb), 256, 0, psrc, f, nrm, wts, nsrc,
                       (const int*)sbox, (const int*)srank, (const int*)cl->src_off, cl->spos, cl->q0, cl->q1, cl->q2,
                       cl->sidx);
    }
    if (ntar > 0)
        FTE_LAUNCH(ctx, k_scatter_tar, grid_for(ntar, 256, maxb), 256, 0, ptar, ntar, (const int*)tbox,
                   (const int*)trank, (const int*)cl->tar_off, cl->tpos, cl->tidx);
    return FTE_OK;
}

size_t fte_tiles_ws(int64_t n, int ntiles) {
    return 4 * ws_bytes(ntiles + 1, sizeof(int)) + ws_bytes(16 * (size_t)ntiles + 1, sizeof(int)) +
           3 * ws_bytes((size_t)(n + 1), sizeof(int)) +
           4 * ws_bytes((size_t)(ntiles + 1) / 4096 + 8, sizeof(int)) + 4096;
}

int fte_tiles_build(fte_context* ctx, WsCarver& wc, const double* p, int64_t n, double Lx, double Ly, double hx,
                    double hy, int ts, int ntx, int nty, TileBins* out, int region_w) {
    int nt = ntx * nty;
    out->ntx = ntx;
    out->nty = nty;
    out->ts = ts;
    int* cnt = wc.take<int>(nt + 1);
    out->off = wc.take<int>(nt + 1);
    int* tile = wc.take<int>(n + 1);
    int* rank = wc.take<int>(n + 1);
    out->perm = wc.take<int>(n + 1);
    if (n >= (int64_t(1) << 26)) region_w = 0;  // ranks within a residue class are packed in 26 bits
    int* cnt16 = region_w > 0 ? wc.take<int>(16 * (size_t)nt + 1) : nullptr;
    FTE_WS_CHECK(wc);
    FTE_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (nt + 1), ctx->stream));
    if (cnt16) FTE_CUDA_TRY(cudaMemsetAsync(cnt16, 0, sizeof(int) * 16 * (size_t)nt, ctx->stream));
    int maxb = ctx->num_sms * 8;
    if (n > 0)
        FTE_LAUNCH(ctx, k_tile_assign, grid_for(n, 256, maxb), 256, 0, p, n, Lx, Ly, hx, hy, ts, ntx, nty, tile,
                   rank, cnt, region_w, cnt16);
    FTE_TRY(fte_scan_exclusive(ctx, wc, cnt, out->off, nt + 1));
    if (n > 0)
        FTE_LAUNCH(ctx, k_tile_scatter, grid_for(n, 256, maxb), 256, 0, n, (const int*)tile, (const int*)rank,
                   (const int*)out->off, out->perm, region_w, (const int*)cnt16);
    return FTE_OK;
}
