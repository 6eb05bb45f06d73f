// kg_dem.cu -- vertex heights from a georeferenced elevation raster.
//
// The raster branch of GetTileHeights: TileHeightData and GetRasterData
// (src/dem.f90:203-356) with Bicubic_r (src/Interp2d.f90:214-282).  For every tile the
// reference reads its own raster section -- the pixels from two left of / above the
// tile's north-west cell corner, extending ceiling(tile width / pixel) + 5 pixels -- and
// puts at each vertex the mean of four bicubic samples at the corners of the cell-sized
// square around it, in section pixel coordinates.  Seam vertices computed by two tiles
// from different sections can differ in the last bits; the reference then keeps the
// value of the tile to the right / above (EqualiseTopographicBoundaryData), which the
// engine applies at activation exactly as for any other topography.
//
// One CTA per tile, all tiles at once: a section is a few hundred pixels, read through
// L1/L2 (neighbouring tiles' sections overlap by 5 pixels), and a vertex costs four
// bicubic patches in FP64 (the kernel is bound by the FP64 pipe).  The FP64 arithmetic follows the reference's
// operation order with no contraction (-fmad=false), so the heights equal the host
// restatement's bit for bit.
#include <cuda_runtime.h>

#include "kg_engine.cuh"

namespace kg {


// Bicubic_r's coefficients a = m f (src/Interp2d.f90:53-70, matmul order j = 1..16) with
// f = (corner values, x-derivatives, y-derivatives, cross derivatives) at (0,0), (1,0),
// (0,1), (1,1).  Only the non-zero entries of m are summed: a product with a zero entry is
// +-0 and adding it never changes a partial sum that starts at +0 (x + -x rounds to +0),
// so for finite data the sums equal the full 16-term products bit for bit, at a third of
// the FP64 operations.
__device__ __forceinline__ void bicubic_coeffs(const double* f, double* a) {
    a[0] = 0.0 + f[0];
    a[1] = 0.0 + f[8];
    a[2] = (((0.0 + -3.0 * f[0]) + 3.0 * f[2]) + -2.0 * f[8]) - f[10];
    a[3] = (((0.0 + 2.0 * f[0]) + -2.0 * f[2]) + f[8]) + f[10];
    a[4] = 0.0 + f[4];
    a[5] = 0.0 + f[12];
    a[6] = (((0.0 + -3.0 * f[4]) + 3.0 * f[6]) + -2.0 * f[12]) - f[14];
    a[7] = (((0.0 + 2.0 * f[4]) + -2.0 * f[6]) + f[12]) + f[14];
    a[8] = (((0.0 + -3.0 * f[0]) + 3.0 * f[1]) + -2.0 * f[4]) - f[5];
    a[9] = (((0.0 + -3.0 * f[8]) + 3.0 * f[9]) + -2.0 * f[12]) - f[13];
    a[10] = (((((((((((((((0.0 + 9.0 * f[0]) + -9.0 * f[1]) + -9.0 * f[2]) + 9.0 * f[3]) + 6.0 * f[4]) + 3.0 * f[5]) +
                    -6.0 * f[6]) + -3.0 * f[7]) + 6.0 * f[8]) + -6.0 * f[9]) + 3.0 * f[10]) + -3.0 * f[11]) + 4.0 * f[12]) +
              2.0 * f[13]) + 2.0 * f[14]) + f[15];
    a[11] = (((((((((((((((0.0 + -6.0 * f[0]) + 6.0 * f[1]) + 6.0 * f[2]) + -6.0 * f[3]) + -4.0 * f[4]) + -2.0 * f[5]) +
                    4.0 * f[6]) + 2.0 * f[7]) + -3.0 * f[8]) + 3.0 * f[9]) + -3.0 * f[10]) + 3.0 * f[11]) + -2.0 * f[12]) -
              f[13]) + -2.0 * f[14]) - f[15];
    a[12] = (((0.0 + 2.0 * f[0]) + -2.0 * f[1]) + f[4]) + f[5];
    a[13] = (((0.0 + 2.0 * f[8]) + -2.0 * f[9]) + f[12]) + f[13];
    a[14] = (((((((((((((((0.0 + -6.0 * f[0]) + 6.0 * f[1]) + 6.0 * f[2]) + -6.0 * f[3]) + -3.0 * f[4]) + -3.0 * f[5]) +
                    3.0 * f[6]) + 3.0 * f[7]) + -4.0 * f[8]) + 4.0 * f[9]) + -2.0 * f[10]) + 2.0 * f[11]) + -2.0 * f[12]) +
              -2.0 * f[13]) - f[14]) - f[15];
    a[15] = (((((((((((((((0.0 + 4.0 * f[0]) + -4.0 * f[1]) + -4.0 * f[2]) + 4.0 * f[3]) + 2.0 * f[4]) + 2.0 * f[5]) +
                    -2.0 * f[6]) + -2.0 * f[7]) + 2.0 * f[8]) + -2.0 * f[9]) + 2.0 * f[10]) + -2.0 * f[11]) + f[12]) +
              f[13]) + f[14]) + f[15];
}

// Section of one tile (GetRasterData, src/dem.f90:203-256, and the section geotransform of
// src/RasterData.cpp:190-199).
struct Section {
    int xoff, yoff, xsize, ysize;
    double ox, oy;
};
__device__ __forceinline__ Section tile_section(const RasterGeo& g, const double* xv, const double* yv) {
    double nwE = g.ce + (xv[0] - 0.5 * g.dx), nwN = g.cn + (yv[g.nY] + 0.5 * g.dy);
    double seE = g.ce + (xv[g.nX] + 0.5 * g.dx), seN = g.cn + (yv[0] - 0.5 * g.dy);
    Section S;
    S.xoff = (int)floor((nwE - g.ox) / g.pw) - 2;
    S.yoff = (int)floor((nwN - g.oy) / g.ph) - 2;
    S.xsize = (int)ceil((seE - nwE) / g.pw) + 5;
    S.ysize = (int)ceil((seN - nwN) / g.ph) + 5;
    S.ox = g.ox + S.xoff * g.pw;
    S.oy = g.oy + S.yoff * g.ph;
    return S;
}

// Bicubic_r at section coordinates (x, y) (1-based); z(i, j) is section pixel (i, j).
// Returns false (and leaves h) if a needed pixel lies outside the section.
__device__ __forceinline__ bool bicubic(const double* __restrict__ R, long long nx, const Section& S, double x, double y,
                                        double& h) {
    int x0 = (int)floor(x), x1 = (int)ceil(x), y0 = (int)floor(y), y1 = (int)ceil(y);
    if (x0 - 1 < 1 || x1 + 1 > S.xsize || y0 - 1 < 1 || y1 + 1 > S.ysize) return false;
    auto z = [&](int i, int j) { return R[(long long)(S.yoff + j - 1) * nx + (S.xoff + i - 1)]; };
    // The finite-difference spacings x1 - x0 + 1 and y1 - y0 + 1 are 1 (on a pixel line)
    // or 2, and the patch width x1 - x0 is 1 off a pixel line: dividing by 1 or 2 is
    // exactly multiplying by 1 or 0.5, so no FP64 divide is needed.
    const double sx = (x1 == x0) ? 1.0 : 0.5, sy = (y1 == y0) ? 1.0 : 0.5;
    double f[16];
    f[0] = z(x0, y0);
    f[1] = z(x1, y0);
    f[2] = z(x0, y1);
    f[3] = z(x1, y1);
    f[4] = (z(x1, y0) - z(x0 - 1, y0)) * sx;
    f[5] = (z(x1 + 1, y0) - z(x0, y0)) * sx;
    f[6] = (z(x1, y1) - z(x0 - 1, y1)) * sx;
    f[7] = (z(x1 + 1, y1) - z(x0, y1)) * sx;
    f[8] = (z(x0, y1) - z(x0, y0 - 1)) * sy;
    f[9] = (z(x1, y1) - z(x1, y0 - 1)) * sy;
    f[10] = (z(x0, y1 + 1) - z(x0, y0)) * sy;
    f[11] = (z(x1, y1 + 1) - z(x1, y0)) * sy;
    f[12] = ((z(x1, y1) - z(x0 - 1, y1)) - (z(x1, y0 - 1) - z(x0 - 1, y0 - 1))) * sx * sy;
    f[13] = ((z(x1 + 1, y1) - z(x0, y1)) - (z(x1 + 1, y0 - 1) - z(x0, y0 - 1))) * sx * sy;
    f[14] = ((z(x1, y1 + 1) - z(x0 - 1, y1 + 1)) - (z(x1, y0) - z(x0 - 1, y0))) * sx * sy;
    f[15] = ((z(x1 + 1, y1 + 1) - z(x0, y1 + 1)) - (z(x1 + 1, y0) - z(x0, y0))) * sx * sy;
    double a[16];
    bicubic_coeffs(f, a);
    double t = (x == (double)x0) ? 0.0 : (x - x0);
    double u = (y == (double)y0) ? 0.0 : (y - y0);
    double ans = 0.0;
    for (int i = 3; i >= 0; --i) ans = t * ans + ((a[i * 4 + 3] * u + a[i * 4 + 2]) * u + a[i * 4 + 1]) * u + a[i * 4 + 0];
    h = ans;
    return true;
}

// Heights of every tile: out[(tile - 1) * SV + b * (nX + 1) + a]; status[tile - 1] = 0 (ok),
// 1 (section outside the raster), 2 (no-data in the section), 3 (a sample outside its
// section).  xv / yv hold the vertex coordinates of each tile column / row.
__global__ void __launch_bounds__(256) k_raster_heights(const double* __restrict__ R, RasterGeo g, const double* __restrict__ XV,
                                                        const double* __restrict__ YV, double* __restrict__ out,
                                                        int* __restrict__ status) {
    const int ntiles = g.nXt * g.nYt, SV = (g.nX + 1) * (g.nY + 1);
    __shared__ int st;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int gi = t % g.nXt, gj = t / g.nXt;
        const double* xv = XV + (size_t)gi * (g.nX + 1);
        const double* yv = YV + (size_t)gj * (g.nY + 1);
        const Section S = tile_section(g, xv, yv);
        __syncthreads();
        if (threadIdx.x == 0) {
            bool inside = S.xoff >= 0 && S.yoff >= 0 && (long long)S.xoff + S.xsize <= g.nx &&
                          (long long)S.yoff + S.ysize <= g.ny && S.xsize > 0 && S.ysize > 0;
            st = inside ? 0 : 1;
        }
        __syncthreads();
        if (st == 0) {
            bool nod = false;
            for (int k = threadIdx.x; k < S.xsize * S.ysize; k += blockDim.x) {
                int i = k % S.xsize, j = k / S.xsize;
                if (R[(long long)(S.yoff + j) * g.nx + (S.xoff + i)] == g.nodata) nod = true;
            }
            if (nod) atomicMax(&st, 2);
        }
        __syncthreads();
        if (st == 0) {
            bool bad = false;
            for (int v = threadIdx.x; v < SV; v += blockDim.x) {
                const int a = v % (g.nX + 1), b = v / (g.nX + 1);
                double hc[4];
                for (int ii = 1; ii <= 2; ++ii)
                    for (int jj = 1; jj <= 2; ++jj) {
                        const int k = jj + 2 * (ii - 1);
                        double E = (g.ce + xv[a]) + ((double)(ii - 1) - 0.5) * g.dx;
                        double N = (g.cn + yv[b]) + ((double)(jj - 1) - 0.5) * g.dy;
                        double x = (E - S.ox) / g.pw + 1.0, y = (N - S.oy) / g.ph + 1.0;
                        if (!bicubic(R, g.nx, S, x, y, hc[k - 1])) { bad = true; hc[k - 1] = 0.0; }
                    }
                out[(size_t)t * SV + v] = 0.25 * (((hc[0] + hc[1]) + hc[2]) + hc[3]);
            }
            if (bad) atomicMax(&st, 3);
        }
        __syncthreads();
        if (threadIdx.x == 0) status[t] = st;
    }
}

cudaError_t launch_raster_heights(const double* R, const RasterGeo& g, const double* XV, const double* YV, double* out, int* status,
                                  cudaStream_t st) {
    int ntiles = g.nXt * g.nYt;
    if (ntiles <= 0) return cudaSuccess;
    int grid = ntiles < 152 * 8 ? ntiles : 152 * 8;
    k_raster_heights<<<grid, 256, 0, st>>>(R, g, XV, YV, out, status);
    return cudaGetLastError();
}

}  // namespace kg
