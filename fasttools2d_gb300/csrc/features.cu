// features.cu -- point-layout statistics on the device for the learned
// parameter selector (no counterpart in the reference, whose drivers use only
// N, the box and the tolerance).
//
// fte_nn_sample: the distance from each of a sample of the sources to its
// nearest other source in the periodic box.  The sources go into a device cell
// list with about four per cell (the same counting sort as the real-space
// sums); each sampled source searches the rings of cells around its own,
// nearest ring first, until the unsearched rings lie farther than the best
// distance found.  The sample is every stride-th source, stride =
// max(1, nsrc / nsample), so it is deterministic.
#include <cmath>

#include "fte_internal.cuh"

namespace {

constexpr int kMaxRing = 16;

__global__ void k_nn_pack(const double* __restrict__ x, const double* __restrict__ y, int64_t n, double Lx, double Ly,
                          double* __restrict__ p) {
    const double rLx = __drcp_rn(Lx), rLy = __drcp_rn(Ly);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        p[2 * i] = fte_wrap_coord(x[i], Lx, rLx);
        p[2 * i + 1] = fte_wrap_coord(y[i], Ly, rLy);
    }
}

__global__ void k_nn_sample(const double* __restrict__ p, int ns, int64_t stride, double* __restrict__ t) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x) {
        const int64_t i = (int64_t)j * stride;
        t[2 * j] = p[2 * i];
        t[2 * j + 1] = p[2 * i + 1];
    }
}

// one thread per sampled source (cell-sorted target j, original sample index
// tidx[j], source index tidx[j] * stride)
__global__ void k_nn_search(CellList cl, int64_t stride, double Lx, double Ly, double* __restrict__ out) {
    const int nt = cl.tar_off[cl.nb];
    const double bx = Lx / cl.nsx, by = Ly / cl.nsy, bmin = fmin(bx, by);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nt; j += gridDim.x * blockDim.x) {
        const double2 q = cl.tpos[j];
        const int self = cl.tidx[j];
        const int64_t self_src = (int64_t)self * stride;
        const int cx = min(max((int)floor((q.x + 0.5 * Lx) / bx), 0), cl.nsx - 1);
        const int cy = min(max((int)floor((q.y + 0.5 * Ly) / by), 0), cl.nsy - 1);
        double best2 = INFINITY;
        const int rmax = min(kMaxRing, max(max(cl.nsx, cl.nsy) / 2, 1));
        for (int r = 0; r <= rmax; r++) {
            // every source of ring r lies at least (r - 1) cell sides away
            if (r >= 2 && (double)(r - 1) * bmin * (double)(r - 1) * bmin > best2) break;
            for (int oy = -r; oy <= r; oy++) {
                const int step = (oy == -r || oy == r) ? 1 : 2 * r;  // ring cells only
                for (int ox = -r; ox <= r; ox += (r == 0 ? 1 : step)) {
                    int gx = cx + ox, gy = cy + oy;
                    // periodic image: floor division by the cell counts (a
                    // ring may wrap more than once around a narrow box)
                    const int kx = gx >= 0 ? gx / cl.nsx : -((cl.nsx - 1 - gx) / cl.nsx);
                    const int ky = gy >= 0 ? gy / cl.nsy : -((cl.nsy - 1 - gy) / cl.nsy);
                    gx -= kx * cl.nsx;
                    gy -= ky * cl.nsy;
                    const double sx = kx * Lx, sy = ky * Ly;
                    const int b = gy * cl.nsx + gx;
                    for (int k = cl.src_off[b]; k < cl.src_off[b + 1]; k++) {
                        if (cl.sidx[k] == self_src) continue;
                        const double2 s = cl.spos[k];
                        const double dx = s.x + sx - q.x, dy = s.y + sy - q.y;
                        const double d2 = dx * dx + dy * dy;
                        best2 = d2 < best2 ? d2 : best2;
                    }
                }
            }
        }
        out[self] = sqrt(best2);
    }
}

int grid_of(const fte_context* c, int64_t n) {
    int64_t b = (n + 255) / 256;
    const int64_t cap = (int64_t)c->num_sms * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

extern "C" int fte_nn_sample(fte_context* c, const double* xsrc, const double* ysrc, int64_t nsrc, double Lx,
                             double Ly, int nsample, double* out, unsigned flags) {
    if (!c) {
        fte_set_error("fte_nn_sample: null context");
        return FTE_ERR_INVALID;
    }
    if (nsrc < 2 || nsrc > 2000000000LL || nsample < 1 || !xsrc || !ysrc || !out) {
        fte_set_error("fte_nn_sample: need at least two sources, a positive sample size and non-null arrays");
        return FTE_ERR_INVALID;
    }
    if (!(Lx > 0) || !(Ly > 0) || !std::isfinite(Lx) || !std::isfinite(Ly)) {
        fte_set_error("fte_nn_sample: box sides must be positive and finite");
        return FTE_ERR_INVALID;
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    const int64_t stride = nsrc / nsample > 1 ? nsrc / nsample : 1;
    const int ns = (int)((nsrc + stride - 1) / stride < nsample ? (nsrc + stride - 1) / stride : nsample);
    // about four sources per cell, cells nearly square
    const double side = std::sqrt(4.0 * Lx * Ly / (double)nsrc);
    int nsx = (int)std::lround(Lx / side), nsy = (int)std::lround(Ly / side);
    nsx = nsx < 1 ? 1 : (nsx > 8192 ? 8192 : nsx);
    nsy = nsy < 1 ? 1 : (nsy > 8192 ? 8192 : nsy);
    size_t need = ws_bytes(2 * (size_t)(nsrc + 1), 8) + ws_bytes(2 * (size_t)(ns + 1), 8) +
                  ws_bytes((size_t)ns + 1, 8) + fte_cells_ws(nsrc, ns, nsx * nsy) + 4096;
    if (host) need += 2 * ws_bytes((size_t)nsrc + 1, 8);
    FTE_TRY(fte_ws_reserve(c, need));
    WsCarver wc{c->ws, 0, c->ws_size};
    const double* dx = xsrc;
    const double* dy = ysrc;
    if (host) {
        double* hx = wc.take<double>(nsrc + 1);
        double* hy = wc.take<double>(nsrc + 1);
        FTE_WS_CHECK(wc);
        FTE_CUDA_TRY(cudaMemcpyAsync(hx, xsrc, nsrc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        FTE_CUDA_TRY(cudaMemcpyAsync(hy, ysrc, nsrc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        dx = hx;
        dy = hy;
    }
    double* ps = wc.take<double>(2 * (nsrc + 1));
    double* pt = wc.take<double>(2 * (ns + 1));
    double* dist = host ? wc.take<double>(ns + 1) : out;
    FTE_WS_CHECK(wc);
    FiniteSet fin;
    fin.add(dx, nsrc);
    fin.add(dy, nsrc);
    FTE_TRY(fte_check_finite(c, fin, "fte_nn_sample"));
    FTE_LAUNCH(c, k_nn_pack, grid_of(c, nsrc), 256, 0, dx, dy, nsrc, Lx, Ly, ps);
    FTE_LAUNCH(c, k_nn_sample, grid_of(c, ns), 256, 0, (const double*)ps, ns, stride, pt);
    CellList cl;
    // the positions stand in for the densities the cell list also sorts
    FTE_TRY(fte_cells_build(c, wc, FTE_KIND_SLP, ps, nsrc, pt, ns, ps, nullptr, nullptr, nsx, nsy, Lx, Ly, &cl));
    FTE_LAUNCH(c, k_nn_search, grid_of(c, ns), 256, 0, cl, stride, Lx, Ly, dist);
    if (host)
        FTE_CUDA_TRY(cudaMemcpyAsync(out, dist, ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}
