// ko_grid.hpp -- TEST INFRASTRUCTURE (the oracle).  Grid, tile navigation, topography and
// the hydraulic operator, restated from src/Grid.f90, src/dem.f90, src/TopogFuncs.f90,
// src/MorphodynamicRHS.f90 (topographic interpolation) and src/HydraulicRHS.f90.
#pragma once
#include "ko_model.hpp"
#include <stdexcept>

namespace ko {

struct KoError : std::runtime_error {
    int code;
    KoError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// An elevation raster as GDAL presents the reference's DEM.vrt (src/RasterData.cpp:160-215):
// values row-major from the top row, the geotransform origin and pixel sizes, the no-data
// value, and the projected domain centre (RunParams%centerUTM).
struct Raster {
    std::vector<double> values;
    int64_t nx = 0, ny = 0;
    double originX = 0, originY = 0, pixelWidth = 0, pixelHeight = 0, nodata = 0, centerE = 0, centerN = 0;
};

typedef std::vector<Tile> Tiles;

// GridType, src/Grid.f90:128-158.
struct Grid {
    int dim = 2;
    int nXtiles, nYtiles, nTiles;
    double deltaX, deltaY, deltaXRecip, deltaYRecip, Xtilesize, Ytilesize;
    Tiles tileContainer, intermed0, intermed1, intermed2, intermed3;
    std::vector<int> activeTiles, ghostTiles;  // %List (activeTiles sorted ascending)
    double xmin, xmax, ymin, ymax;
    double t = 0.0, t0 = 0.0, dt = 1.0e-5;
    std::vector<double> b0_upload;  // global vertex grid when topog == KG_TOPO_UPLOAD
    int64_t nx1 = 0, ny1 = 0;
    Raster raster;                  // when topog == KG_TOPO_RASTER
    Tile& tc(int id) { return tileContainer[(size_t)id - 1]; }
};
inline Tile& TL(Tiles& t, int id) { return t[(size_t)id - 1]; }

// ---------------------------------------------------------------- Grid.f90 navigation
inline int TileRow(int tile, const Grid& g) { return (tile - 1) / g.nXtiles + 1; }
inline int TileCol(int tile, const Grid& g) { return (tile - 1) % g.nXtiles + 1; }
inline void GridCoords(int id, const Grid& g, int& i, int& j) { i = TileCol(id, g); j = TileRow(id, g); }
inline int TileID(const Grid& g, int gi, int gj) { return gi + (gj - 1) * g.nXtiles; }
inline bool TileInBounds(const Grid& g, int id) { return !(id < 1 || id > g.nTiles); }
inline int NorthTile(int id, const Grid& g) { return id + g.nXtiles; }
inline int SouthTile(int id, const Grid& g) { return id - g.nXtiles; }
inline int EastTile(int id) { return id + 1; }
inline int WestTile(int id) { return id - 1; }
inline bool OnDomainEdge(const Grid& g, int id) {
    int i, j;
    GridCoords(id, g, i, j);
    bool on = (i == 1 || i == g.nXtiles);
    on = on || (g.nYtiles > 1 && (j == 1 || j == g.nYtiles));
    return on;
}
// src/Grid.f90:339-353
inline void GridToPhysical(const RunSet& rp, const Grid& g, int gi, int gj, int ti, int tj, double& x, double& y) {
    x = -0.5 * rp.xSize + g.deltaX * ((gi - 1.0) * rp.nXpertile + (ti - 0.5));
    y = -0.5 * rp.ySize + g.deltaY * ((gj - 1.0) * rp.nYpertile + (tj - 0.5));
}
inline bool InVector(const std::vector<int>& v, int val) {
    for (int x : v) if (x == val) return true;
    return false;
}
// src/Grid.f90:359-377
inline bool IsActiveGhostTile(Grid& g, int id) {
    if (!g.ghostTiles.empty() && InVector(g.ghostTiles, id))
        if (g.tc(id).isGhostTile) return true;
    return false;
}

// ---------------------------------------------------------------- topography
// The remaining analytic surfaces of src/TopogFuncs.f90 at one vertex (X, Y): x2slopes
// (:101-135), usgs (:145-183), flume (:197-242), channel_powerlaw (:255-276),
// channel_trapezium (:288-308), xbislope (:315-337), xtrislope (:346-388).
inline double OtherTopogFunc(int kind, const double* P, double X, double Y) {
    const double pi = PI;
    switch (kind) {
        case KG_TOPO_X2SLOPES: {
            double alpha = P[0], beta = P[1], R = P[2];
            double xc0 = (std::sqrt(1.0 + alpha * alpha) - std::sqrt(1.0 + beta * beta)) * R / (alpha - beta);
            double zc0 = (alpha * std::sqrt(1.0 + beta * beta) - beta * std::sqrt(1.0 + alpha * alpha)) * R / (alpha - beta);
            double x1 = xc0 - alpha * R / std::sqrt(1.0 + alpha * alpha);
            double x2 = xc0 - beta * R / std::sqrt(1.0 + beta * beta);
            if (X < x1) return -alpha * X;
            if (X > x2) return -beta * X;
            return zc0 - std::sqrt(R * R - (X - xc0) * (X - xc0));
        }
        case KG_TOPO_USGS:
        case KG_TOPO_FLUME: {
            double th0 = 31.0, th1 = 2.4, xwall = 8.5, ww = 2.0, wallH = P[0], sigma = P[1];
            if (kind == KG_TOPO_FLUME) { th0 = P[0]; th1 = P[1]; xwall = P[2]; ww = P[3]; wallH = P[4]; sigma = P[5]; }
            double alpha = 8.5 / (std::asinh(-std::tan(4.0 * pi / 180.0)) - std::asinh(-std::tan(th0 * pi / 180.0)));
            double xc0 = -alpha * std::asinh(-std::tan(th0 * pi / 180.0));
            double zc0 = -alpha * std::cosh((-xc0) / alpha);
            double x1 = xc0 + alpha * std::asinh(-std::tan(th1 * pi / 180.0));
            double b;
            if (X < 0.0) b = -std::tan(th0 * pi / 180.0) * X;
            else if (X > x1) b = zc0 + alpha * std::cosh((x1 - xc0) / alpha) - std::tan(th1 * pi / 180.0) * (X - x1);
            else b = zc0 + alpha * std::cosh((X - xc0) / alpha);
            if (X < xwall) {
                if (kind == KG_TOPO_USGS)
                    b = b + 0.5 * wallH * (std::tanh(sigma * (Y - 1.0)) - std::tanh(sigma * (Y - 2.0)) + std::tanh(sigma * (Y + 2.0)) -
                                           std::tanh(sigma * (Y + 1.0)));
                else
                    b = b + 0.5 * wallH * (std::tanh(sigma * (Y - 0.5 * ww)) - std::tanh(sigma * (Y - 1.5 * ww)) +
                                           std::tanh(sigma * (Y + 1.5 * ww)) - std::tanh(sigma * (Y + 0.5 * ww)));
            }
            return b;
        }
        case KG_TOPO_CHANNEL_POWERLAW: {
            double slope = P[0], W = P[1], alpha = P[2];
            double costheta = std::cos(std::atan(slope));
            return slope * X + costheta * std::pow(std::fabs(Y) / W, alpha);
        }
        case KG_TOPO_CHANNEL_TRAPEZIUM: {
            double slope = P[0], W = P[1], Sb = P[2];
            double costheta = std::cos(std::atan(slope));
            return slope * X + costheta * std::max(0.0, Sb * (std::fabs(Y) - 0.5 * W));
        }
        case KG_TOPO_XBISLOPE: {
            double phi1 = P[0] * pi / 180.0, phi2 = P[1] * pi / 180.0, lam = P[2];
            double a1 = std::tan(phi1), a2 = std::tan(phi2);
            return -0.5 * (a1 + a2) * X + 0.5 * (a1 - a2) * lam * std::log(std::cosh(X / lam));
        }
        case KG_TOPO_XTRISLOPE: {
            double phi1 = P[0] * pi / 180.0, phi2 = P[1] * pi / 180.0, phi3 = P[2] * pi / 180.0;
            double lam = P[3], x1 = P[4], x2 = P[5];
            double s1 = std::tan(phi1), s2 = std::tan(phi2), s3 = std::tan(phi3);
            double c2 = (x1 - 0.5 * lam) * 0.5 * (s1 - s2);
            double c3 = (x1 + 0.5 * lam) * 0.5 * (s1 - s2) + c2;
            double c4 = (x2 - 0.5 * lam) * 0.5 * (s2 - s3) + c3;
            double c5 = (x2 + 0.5 * lam) * 0.5 * (s2 - s3) + c4;
            if (X < x1 - 0.5 * lam) return s1 * X;
            if (X < x1 + 0.5 * lam) {
                double A = 0.5 * (s2 - s1) * lam / pi;
                return A * std::sin((X - x1) * pi / lam - 0.5 * pi) + 0.5 * (s1 + s2) * X + c2;
            }
            if (X < x2 - 0.5 * lam) return s2 * X + c3;
            if (X < x2 + 0.5 * lam) {
                double A = 0.5 * (s3 - s2) * lam / pi;
                return A * std::sin((X - x2) * pi / lam - 0.5 * pi) + 0.5 * (s2 + s3) * X + c4;
            }
            return s3 * X + c5;
        }
    }
    return 0.0;
}

// TopogFuncs.f90 analytic surfaces evaluated on vertex coordinates (x, y), plus the
// uploaded-grid replacement of GetTileHeights for the synthetic terrains.
inline void TopogFunc(const RunSet& rp, const Grid& g, int tileid, const std::vector<double>& x,
                      const std::vector<double>& y, A2& b0) {
    const double* P = rp.p.topog_params;
    int nx = (int)x.size(), ny = (int)y.size();
    for (int jj = 1; jj <= ny; ++jj)
        for (int ii = 1; ii <= nx; ++ii) {
            double X = x[ii - 1], Y = y[jj - 1], b = 0.0;
            switch (rp.p.topog) {
                case KG_TOPO_FLAT: b = 0.0; break;
                case KG_TOPO_XSLOPE: b = P[0] * X; break;
                case KG_TOPO_YSLOPE: b = P[0] * Y; break;
                case KG_TOPO_XYSLOPE: b = P[0] * X + P[1] * Y; break;
                case KG_TOPO_XSINSLOPE: {
                    double Lx = rp.Xtilesize * rp.nXtiles;
                    double k = 2.0 * PI / Lx;
                    b = P[0] * std::sin(X * k);
                    break;
                }
                case KG_TOPO_XYSINSLOPE: {
                    double Lx = rp.Xtilesize * rp.nXtiles, Ly = rp.Ytilesize * rp.nYtiles;
                    double kx = 2.0 * PI / Lx, ky = 2.0 * PI / Ly;
                    b = P[0] * std::sin(X * kx) * std::sin(Y * ky);
                    break;
                }
                case KG_TOPO_XHUMP:
                    b = ((X > -P[1]) && (X < P[1])) ? 0.5 * P[0] * (1.0 + std::cos(PI * X / P[1])) : 0.0;
                    break;
                case KG_TOPO_XTANH: b = P[1] * (1.0 + std::tanh((X - P[0]) / P[2])); break;
                case KG_TOPO_XPARAB: b = P[0] * X * X; break;
                case KG_TOPO_XYPARAB: b = P[0] * X * X + P[1] * Y * Y; break;
                case KG_TOPO_X2SLOPES:
                case KG_TOPO_USGS:
                case KG_TOPO_FLUME:
                case KG_TOPO_CHANNEL_POWERLAW:
                case KG_TOPO_CHANNEL_TRAPEZIUM:
                case KG_TOPO_XBISLOPE:
                case KG_TOPO_XTRISLOPE: b = OtherTopogFunc(rp.p.topog, P, X, Y); break;
                case KG_TOPO_UPLOAD: {
                    int gi, gj;
                    GridCoords(tileid, g, gi, gj);
                    int64_t vx = (int64_t)(gi - 1) * rp.nXpertile + (ii - 1);
                    int64_t vy = (int64_t)(gj - 1) * rp.nYpertile + (jj - 1);
                    b = g.b0_upload[(size_t)(vx + g.nx1 * vy)];
                    break;
                }
            }
            b0(ii, jj) = b;
        }
}

// A raster section read the way GetRasterData reads one (src/dem.f90:203-256):
// bandSection(i, j) = pixel (xoff + i - 1, yoff + j - 1) of the full raster, with the
// section's own geotransform origin (src/RasterData.cpp:190-199).
struct BandSection {
    int xoff, yoff, xsize, ysize;
    double rOX, rOY;
    const Raster* r;
    double operator()(int i, int j) const { return r->values[(size_t)((int64_t)(yoff + j - 1) * r->nx + (xoff + i - 1))]; }
};

// Bicubic_r, src/Interp2d.f90:214-282 (coefficient matrix m at :53-70).
inline double Bicubic(double x, double y, const BandSection& z) {
    static const double m[16][16] = {
        {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0},
        {-3, 0, 3, 0, 0, 0, 0, 0, -2, 0, -1, 0, 0, 0, 0, 0},
        {2, 0, -2, 0, 0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0},
        {0, 0, 0, 0, -3, 0, 3, 0, 0, 0, 0, 0, -2, 0, -1, 0},
        {0, 0, 0, 0, 2, 0, -2, 0, 0, 0, 0, 0, 1, 0, 1, 0},
        {-3, 3, 0, 0, -2, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, -3, 3, 0, 0, -2, -1, 0, 0},
        {9, -9, -9, 9, 6, 3, -6, -3, 6, -6, 3, -3, 4, 2, 2, 1},
        {-6, 6, 6, -6, -4, -2, 4, 2, -3, 3, -3, 3, -2, -1, -2, -1},
        {2, -2, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 2, -2, 0, 0, 1, 1, 0, 0},
        {-6, 6, 6, -6, -3, -3, 3, 3, -4, 4, -2, 2, -2, -2, -1, -1},
        {4, -4, -4, 4, 2, 2, -2, -2, 2, -2, 2, -2, 1, 1, 1, 1}};
    int x0 = (int)std::floor(x), x1 = (int)std::ceil(x), y0 = (int)std::floor(y), y1 = (int)std::ceil(y);
    if (x0 - 1 < 1 || x1 + 1 > z.xsize || y0 - 1 < 1 || y1 + 1 > z.ysize)
        throw KoError(KG_ERR_PARAM, "bicubic sample outside its raster section");
    double fVec[16];
    fVec[0] = z(x0, y0);
    fVec[1] = z(x1, y0);
    fVec[2] = z(x0, y1);
    fVec[3] = z(x1, y1);
    fVec[4] = (z(x1, y0) - z(x0 - 1, y0)) / (double)(x1 - x0 + 1);
    fVec[5] = (z(x1 + 1, y0) - z(x0, y0)) / (double)(x1 + 1 - x0);
    fVec[6] = (z(x1, y1) - z(x0 - 1, y1)) / (double)(x1 - x0 + 1);
    fVec[7] = (z(x1 + 1, y1) - z(x0, y1)) / (double)(x1 + 1 - x0);
    fVec[8] = (z(x0, y1) - z(x0, y0 - 1)) / (double)(y1 - y0 + 1);
    fVec[9] = (z(x1, y1) - z(x1, y0 - 1)) / (double)(y1 - y0 + 1);
    fVec[10] = (z(x0, y1 + 1) - z(x0, y0)) / (double)(y1 + 1 - y0);
    fVec[11] = (z(x1, y1 + 1) - z(x1, y0)) / (double)(y1 + 1 - y0);
    fVec[12] = ((z(x1, y1) - z(x0 - 1, y1)) - (z(x1, y0 - 1) - z(x0 - 1, y0 - 1))) / (double)(x1 - x0 + 1) / (double)(y1 - y0 + 1);
    fVec[13] = ((z(x1 + 1, y1) - z(x0, y1)) - (z(x1 + 1, y0 - 1) - z(x0, y0 - 1))) / (double)(x1 + 1 - x0) / (double)(y1 - y0 + 1);
    fVec[14] = ((z(x1, y1 + 1) - z(x0 - 1, y1 + 1)) - (z(x1, y0) - z(x0 - 1, y0))) / (double)(x1 - x0 + 1) / (double)(y1 + 1 - y0);
    fVec[15] = ((z(x1 + 1, y1 + 1) - z(x0, y1 + 1)) - (z(x1 + 1, y0) - z(x0, y0))) / (double)(x1 + 1 - x0) / (double)(y1 + 1 - y0);
    double aVec[16];
    for (int i = 0; i < 16; ++i) {  // matmul(m, fVec)
        aVec[i] = 0.0;
        for (int j = 0; j < 16; ++j) aVec[i] = aVec[i] + m[i][j] * fVec[j];
    }
    double a[4][4];  // reshape(aVec, (/4,4/), order=(/2,1/))
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) a[i][j] = aVec[i * 4 + j];
    double t = (x == (double)x0) ? 0.0 : (x - x0) / (double)(x1 - x0);
    double u = (y == (double)y0) ? 0.0 : (y - y0) / (double)(y1 - y0);
    double ans = 0.0;
    for (int i = 3; i >= 0; --i) ans = t * ans + ((a[i][3] * u + a[i][2]) * u + a[i][1]) * u + a[i][0];
    return ans;
}

// TileHeightData, src/dem.f90:260-356, with its raster read (GetRasterData, :203-256;
// GeoTiffArraySectionRead's failures, src/GeoTiffRead.f90:213-214, become errors).
inline void TileHeightData(const RunSet& rp, const Grid& g, const std::vector<double>& xtile, const std::vector<double>& ytile,
                           A2& b0) {
    const Raster& R = g.raster;
    int nX = rp.nXpertile, nY = rp.nYpertile;
    double nwE = R.centerE + (xtile[0] - 0.5 * g.deltaX), nwN = R.centerN + (ytile[nY] + 0.5 * g.deltaY);
    double seE = R.centerE + (xtile[nX] + 0.5 * g.deltaX), seN = R.centerN + (ytile[0] - 0.5 * g.deltaY);
    BandSection z;
    z.r = &R;
    double imgx = (nwE - R.originX) / R.pixelWidth, imgy = (nwN - R.originY) / R.pixelHeight;
    z.xoff = (int)std::floor(imgx) - 2;
    z.yoff = (int)std::floor(imgy) - 2;
    z.xsize = (int)std::ceil((seE - nwE) / R.pixelWidth) + 5;
    z.ysize = (int)std::ceil((seN - nwN) / R.pixelHeight) + 5;
    if (z.xoff < 0 || z.yoff < 0 || z.xoff + (int64_t)z.xsize > R.nx || z.yoff + (int64_t)z.ysize > R.ny)
        throw KoError(KG_ERR_PARAM, "Could not read raster file: tile section outside the raster");
    z.rOX = R.originX + z.xoff * R.pixelWidth;
    z.rOY = R.originY + z.yoff * R.pixelHeight;
    for (int j = 1; j <= z.ysize; ++j)
        for (int i = 1; i <= z.xsize; ++i)
            if (z(i, j) == R.nodata) throw KoError(KG_ERR_PARAM, "No-data value found in raster file");
    for (int i = 1; i <= nX + 1; ++i)
        for (int j = 1; j <= nY + 1; ++j) {
            double hcorner[4];
            for (int ii = 1; ii <= 2; ++ii)
                for (int jj = 1; jj <= 2; ++jj) {
                    int k = jj + 2 * (ii - 1);
                    double E = R.centerE + xtile[i - 1] + ((double)(ii - 1) - 0.5) * g.deltaX;
                    double N = R.centerN + ytile[j - 1] + ((double)(jj - 1) - 0.5) * g.deltaY;
                    double ix = (E - z.rOX) / R.pixelWidth + 1;
                    double iy = (N - z.rOY) / R.pixelHeight + 1;
                    hcorner[k - 1] = Bicubic(ix, iy, z);
                }
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s = s + hcorner[k];
            b0(i, j) = 0.25 * s;
        }
}

// GetHeights, src/dem.f90:360-391 (2D branch).
inline void GetHeights(const RunSet& rp, Grid& g, int tID) {
    Tile& T = g.tc(tID);
    int nX = rp.nXpertile, nY = rp.nYpertile;
    A2 b0;
    b0.allocate(nX + 1, nY + 1, 0.0);
    if (rp.p.topog == KG_TOPO_RASTER) TileHeightData(rp, g, T.x_vertex, T.y_vertex, b0);
    else TopogFunc(rp, g, tID, T.x_vertex, T.y_vertex, b0);
    T.b0 = b0;
    for (int i = 1; i <= nY; ++i)
        for (int a = 1; a <= nX + 1; ++a) {
            T.uPlusX(ib0, a, i) = 0.5 * (b0(a, i) + b0(a, i + 1));
            T.uMinusX(ib0, a, i) = 0.5 * (b0(a, i) + b0(a, i + 1));
        }
    for (int i = 1; i <= nX; ++i)
        for (int a = 1; a <= nY + 1; ++a) {
            T.uPlusY(ib0, i, a) = 0.5 * (b0(i, a) + b0(i + 1, a));
            T.uMinusY(ib0, i, a) = 0.5 * (b0(i, a) + b0(i + 1, a));
        }
}

// ComputeCellCentredTopographicData_tileID, src/MorphodynamicRHS.f90:308-366 (2D).
inline void ComputeCellCentredTopographicData(const RunSet& rp, Grid& g, Tiles& tiles, int tID) {
    Tile& T = TL(tiles, tID);
    double dxR = g.deltaXRecip, dyR = g.deltaYRecip;
    for (int i = 1; i <= rp.nXpertile; ++i)
        for (int j = 1; j <= rp.nYpertile; ++j) {
            double a1[4] = {T.b0(i, j), T.b0(i + 1, j), T.b0(i, j + 1), T.b0(i + 1, j + 1)};
            double b0c = 0.25 * KahanSumL(a1);
            double a2[4] = {T.bt(i, j), T.bt(i + 1, j), T.bt(i, j + 1), T.bt(i + 1, j + 1)};
            double btc = 0.25 * KahanSumL(a2);
            T.u(ib0, i, j) = b0c;
            T.u(ibt, i, j) = btc;
            double a3[8] = {T.b0(i + 1, j), T.bt(i + 1, j), -T.b0(i, j), -T.bt(i, j),
                            T.b0(i + 1, j + 1), T.bt(i + 1, j + 1), -T.b0(i, j + 1), -T.bt(i, j + 1)};
            T.u(idbdx, i, j) = 0.5 * dxR * KahanSumL(a3);
            double a4[8] = {T.b0(i, j + 1), T.bt(i, j + 1), -T.b0(i, j), -T.bt(i, j),
                            T.b0(i + 1, j + 1), T.bt(i + 1, j + 1), -T.b0(i + 1, j), -T.bt(i + 1, j)};
            T.u(idbdy, i, j) = 0.5 * dyR * KahanSumL(a4);
        }
}
// ComputeCellCentredTopographicData_ij, src/MorphodynamicRHS.f90:371-414 (2D).
inline void ComputeCellCentredTopographicDataIJ(const RunSet& rp, Grid& g, Tiles& tiles, int tID, int i, int j) {
    (void)rp;
    Tile& T = TL(tiles, tID);
    double dxR = g.deltaXRecip, dyR = g.deltaYRecip;
    double a2[4] = {T.bt(i, j), T.bt(i + 1, j), T.bt(i, j + 1), T.bt(i + 1, j + 1)};
    T.u(ibt, i, j) = 0.25 * KahanSumL(a2);
    double a3[8] = {T.b0(i + 1, j), T.bt(i + 1, j), -T.b0(i, j), -T.bt(i, j),
                    T.b0(i + 1, j + 1), T.bt(i + 1, j + 1), -T.b0(i, j + 1), -T.bt(i, j + 1)};
    T.u(idbdx, i, j) = 0.5 * dxR * KahanSumL(a3);
    double a4[8] = {T.b0(i, j + 1), T.bt(i, j + 1), -T.b0(i, j), -T.bt(i, j),
                    T.b0(i + 1, j + 1), T.bt(i + 1, j + 1), -T.b0(i + 1, j), -T.bt(i + 1, j)};
    T.u(idbdy, i, j) = 0.5 * dyR * KahanSumL(a4);
}

// ComputeInterfacialTopographicData, src/MorphodynamicRHS.f90:419-540 (2D).
inline void ComputeInterfacialTopographicData(const RunSet& rp, Grid& g, Tiles& tiles, int tID) {
    Tile& T = TL(tiles, tID);
    int nX = rp.nXpertile, nY = rp.nYpertile;
    double dxR = g.deltaXRecip, dyR = g.deltaYRecip;
    for (int i = 2; i <= nX; ++i)
        for (int j = 1; j <= nY; ++j) {
            double a[8] = {T.b0(i + 1, j), T.bt(i + 1, j), T.b0(i + 1, j + 1), T.bt(i + 1, j + 1),
                           -T.b0(i - 1, j), -T.bt(i - 1, j), -T.b0(i - 1, j + 1), -T.bt(i - 1, j + 1)};
            double d = 0.25 * dxR * KahanSumL(a);
            T.uMinusX(idbdx, i, j) = d;
            T.uPlusX(idbdx, i, j) = d;
        }
    {
        Tile& P = TL(tiles, T.West());
        for (int j = 1; j <= nY; ++j) {
            double a[8] = {T.b0(2, j), T.bt(2, j), T.b0(2, j + 1), T.bt(2, j + 1),
                           -P.b0(nX, j), -P.bt(nX, j), -P.b0(nX, j + 1), -P.bt(nX, j + 1)};
            double d = 0.25 * dxR * KahanSumL(a);
            T.uMinusX(idbdx, 1, j) = d;
            T.uPlusX(idbdx, 1, j) = d;
        }
    }
    {
        Tile& N = TL(tiles, T.East());
        for (int j = 1; j <= nY; ++j) {
            double a[8] = {N.b0(2, j), N.bt(2, j), N.b0(2, j + 1), N.bt(2, j + 1),
                           -T.b0(nX, j), -T.bt(nX, j), -T.b0(nX, j + 1), -T.bt(nX, j + 1)};
            double d = 0.25 * dxR * KahanSumL(a);
            T.uMinusX(idbdx, nX + 1, j) = d;
            T.uPlusX(idbdx, nX + 1, j) = d;
        }
    }
    for (int i = 1; i <= nX + 1; ++i)
        for (int j = 1; j <= nY; ++j) {
            double bt = 0.5 * (T.bt(i, j) + T.bt(i, j + 1));
            double a[4] = {T.b0(i, j + 1), T.bt(i, j + 1), -T.b0(i, j), -T.bt(i, j)};
            double dbdy = dyR * KahanSumL(a);
            T.uPlusX(ibt, i, j) = bt;
            T.uMinusX(ibt, i, j) = bt;
            T.uPlusX(idbdy, i, j) = dbdy;
            T.uMinusX(idbdy, i, j) = dbdy;
        }
    for (int i = 1; i <= nX; ++i)
        for (int j = 1; j <= nY + 1; ++j) {
            double bt = 0.5 * (T.bt(i, j) + T.bt(i + 1, j));
            double a[4] = {T.b0(i + 1, j), T.bt(i + 1, j), -T.b0(i, j), -T.bt(i, j)};
            double dbdx = dxR * KahanSumL(a);
            T.uPlusY(ibt, i, j) = bt;
            T.uMinusY(ibt, i, j) = bt;
            T.uPlusY(idbdx, i, j) = dbdx;
            T.uMinusY(idbdx, i, j) = dbdx;
        }
    for (int i = 1; i <= nX; ++i)
        for (int j = 2; j <= nY; ++j) {
            double a[8] = {T.b0(i + 1, j + 1), T.bt(i + 1, j + 1), T.b0(i, j + 1), T.bt(i, j + 1),
                           -T.b0(i + 1, j - 1), -T.bt(i + 1, j - 1), -T.b0(i, j - 1), -T.bt(i, j - 1)};
            double d = 0.25 * dyR * KahanSumL(a);
            T.uPlusY(idbdy, i, j) = d;
            T.uMinusY(idbdy, i, j) = d;
        }
    {
        Tile& S = TL(tiles, T.South());
        for (int i = 1; i <= nX; ++i) {
            double a[8] = {T.b0(i + 1, 2), T.bt(i + 1, 2), T.b0(i, 2), T.bt(i, 2),
                           -S.b0(i + 1, nY), -S.bt(i + 1, nY), -S.b0(i, nY), -S.bt(i, nY)};
            double d = 0.25 * dyR * KahanSumL(a);
            T.uPlusY(idbdy, i, 1) = d;
            T.uMinusY(idbdy, i, 1) = d;
        }
    }
    {
        Tile& N = TL(tiles, T.North());
        for (int i = 1; i <= nX; ++i) {
            double a[8] = {N.b0(i + 1, 2), N.bt(i + 1, 2), N.b0(i, 2), N.bt(i, 2),
                           -T.b0(i + 1, nY), -T.bt(i + 1, nY), -T.b0(i, nY), -T.bt(i, nY)};
            double d = 0.25 * dyR * KahanSumL(a);
            T.uPlusY(idbdy, i, nY + 1) = d;
            T.uMinusY(idbdy, i, nY + 1) = d;
        }
    }
}

// ---------------------------------------------------------------- HydraulicRHS.f90
// CalculateLimitedDerivsBoundary, :326-386 (2D branches).
inline void CalculateLimitedDerivsBoundary(const RunSet& rp, Grid& g, int d, int i, int j, Tiles& tiles, int tID, char bid) {
    Tile& T = TL(tiles, tID);
    switch (bid) {
        case 'N': {
            double uN = TL(tiles, T.North()).u(d, i, 1);
            T.uLimY(d, i, j) = g.deltaYRecip * limiter(rp, uN - T.u(d, i, j), T.u(d, i, j) - T.u(d, i, j - 1));
            break;
        }
        case 'S': {
            double uS = TL(tiles, T.South()).u(d, i, rp.nYpertile);
            T.uLimY(d, i, j) = g.deltaYRecip * limiter(rp, T.u(d, i, j + 1) - T.u(d, i, j), T.u(d, i, j) - uS);
            break;
        }
        case 'E': {
            double uE = TL(tiles, T.East()).u(d, 1, j);
            T.uLimX(d, i, j) = g.deltaXRecip * limiter(rp, uE - T.u(d, i, j), T.u(d, i, j) - T.u(d, i - 1, j));
            break;
        }
        default: {
            double uW = TL(tiles, T.West()).u(d, rp.nXpertile, j);
            T.uLimX(d, i, j) = g.deltaXRecip * limiter(rp, T.u(d, i + 1, j) - T.u(d, i, j), T.u(d, i, j) - uW);
            break;
        }
    }
}

// CalculateLimitedDerivs, :181-321.
inline void CalculateLimitedDerivs(const RunSet& rp, Grid& g, const int* vars, int nVars, Tiles& tiles, int tID) {
    Tile& T = TL(tiles, tID);
    int nXP = rp.nXpertile, nYP = rp.nYpertile;
    for (int j = 1; j <= nYP; ++j)
        for (int i = 2; i <= nXP - 1; ++i)
            for (int k = 0; k < nVars; ++k) {
                int d = vars[k];
                T.uLimX(d, i, j) = g.deltaXRecip * limiter(rp, T.u(d, i + 1, j) - T.u(d, i, j), T.u(d, i, j) - T.u(d, i - 1, j));
            }
    for (int j = 2; j <= nYP - 1; ++j)
        for (int i = 1; i <= nXP; ++i)
            for (int k = 0; k < nVars; ++k) {
                int d = vars[k];
                T.uLimY(d, i, j) = g.deltaYRecip * limiter(rp, T.u(d, i, j + 1) - T.u(d, i, j), T.u(d, i, j) - T.u(d, i, j - 1));
            }
    // South boundary, then the south neighbour's north row if that tile is on.
    for (int i = 1; i <= nXP; ++i)
        for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], i, 1, tiles, tID, 'S');
    int nb = g.tc(tID).South();
    if (g.tc(nb).TileOn)
        for (int i = 1; i <= nXP; ++i)
            for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], i, nYP, tiles, nb, 'N');
    for (int i = 1; i <= nXP; ++i)
        for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], i, nYP, tiles, tID, 'N');
    nb = g.tc(tID).North();
    if (g.tc(nb).TileOn)
        for (int i = 1; i <= nXP; ++i)
            for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], i, 1, tiles, nb, 'S');
    for (int j = 1; j <= nYP; ++j)
        for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], 1, j, tiles, tID, 'W');
    nb = g.tc(tID).West();
    if (g.tc(nb).TileOn)
        for (int j = 1; j <= nYP; ++j)
            for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], nXP, j, tiles, nb, 'E');
    for (int j = 1; j <= nYP; ++j)
        for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], nXP, j, tiles, tID, 'E');
    nb = g.tc(tID).East();
    if (g.tc(nb).TileOn)
        for (int j = 1; j <= nYP; ++j)
            for (int k = 0; k < nVars; ++k) CalculateLimitedDerivsBoundary(rp, g, vars[k], 1, j, tiles, nb, 'W');
}

// Reconstruct, :397-552 (2D).
inline void Reconstruct(const RunSet& rp, Grid& g, const int* dims, int nd, bool isFlux, Tiles& tiles, int tID) {
    Tile& T = TL(tiles, tID);
    int nXP = rp.nXpertile, nYP = rp.nYpertile;
    double dx = g.deltaX, dy = g.deltaY;
    {
        Tile& P = TL(tiles, T.West());
        for (int k = 0; k < nd; ++k) {
            int d = dims[k];
            for (int j = 1; j <= nYP; ++j) {
                T.uPlusX(d, 1, j) = T.u(d, 1, j) - T.uLimX(d, 1, j) * 0.5 * dx;
                T.uMinusX(d, 1, j) = P.u(d, nXP, j) + P.uLimX(d, nXP, j) * 0.5 * dx;
            }
        }
    }
    for (int k = 0; k < nd; ++k) {
        int d = dims[k];
        for (int j = 1; j <= nYP; ++j)
            for (int i = 2; i <= nXP; ++i) {
                T.uPlusX(d, i, j) = T.u(d, i, j) - T.uLimX(d, i, j) * 0.5 * dx;
                T.uMinusX(d, i, j) = T.u(d, i - 1, j) + T.uLimX(d, i - 1, j) * 0.5 * dx;
            }
    }
    {
        Tile& N = TL(tiles, T.East());
        for (int k = 0; k < nd; ++k) {
            int d = dims[k];
            for (int j = 1; j <= nYP; ++j) {
                T.uPlusX(d, nXP + 1, j) = N.u(d, 1, j) - N.uLimX(d, 1, j) * 0.5 * dx;
                T.uMinusX(d, nXP + 1, j) = T.u(d, nXP, j) + T.uLimX(d, nXP, j) * 0.5 * dx;
            }
        }
    }
    {
        Tile& P = TL(tiles, T.South());
        for (int k = 0; k < nd; ++k) {
            int d = dims[k];
            for (int i = 1; i <= nXP; ++i) {
                T.uPlusY(d, i, 1) = T.u(d, i, 1) - T.uLimY(d, i, 1) * 0.5 * dy;
                T.uMinusY(d, i, 1) = P.u(d, i, nYP) + P.uLimY(d, i, nYP) * 0.5 * dy;
            }
        }
    }
    for (int k = 0; k < nd; ++k) {
        int d = dims[k];
        for (int j = 2; j <= nYP; ++j)
            for (int i = 1; i <= nXP; ++i) {
                T.uPlusY(d, i, j) = T.u(d, i, j) - T.uLimY(d, i, j) * 0.5 * dy;
                T.uMinusY(d, i, j) = T.u(d, i, j - 1) + T.uLimY(d, i, j - 1) * 0.5 * dy;
            }
    }
    {
        Tile& N = TL(tiles, T.North());
        for (int k = 0; k < nd; ++k) {
            int d = dims[k];
            for (int i = 1; i <= nXP; ++i) {
                T.uPlusY(d, i, nYP + 1) = N.u(d, i, 1) - N.uLimY(d, i, 1) * 0.5 * dy;
                T.uMinusY(d, i, nYP + 1) = T.u(d, i, nYP) + T.uLimY(d, i, nYP) * 0.5 * dy;
            }
        }
    }
    if (isFlux) return;
    // Face Hn from the face w and bed (:494-517).
    for (int i = 1; i <= nXP + 1; ++i)
        for (int j = 1; j <= nYP; ++j) {
            double gam = Gam(rp, T.uPlusX.col(i, j));
            T.uPlusX(iHn, i, j) = ComputeHn(T.uPlusX(iw, i, j), T.uPlusX(ib0, i, j), T.uPlusX(ibt, i, j), gam);
            gam = Gam(rp, T.uMinusX.col(i, j));
            T.uMinusX(iHn, i, j) = ComputeHn(T.uMinusX(iw, i, j), T.uMinusX(ib0, i, j), T.uMinusX(ibt, i, j), gam);
        }
    for (int i = 1; i <= nXP; ++i)
        for (int j = 1; j <= nYP + 1; ++j) {
            double gam = Gam(rp, T.uPlusY.col(i, j));
            T.uPlusY(iHn, i, j) = ComputeHn(T.uPlusY(iw, i, j), T.uPlusY(ib0, i, j), T.uPlusY(ibt, i, j), gam);
            gam = Gam(rp, T.uMinusY.col(i, j));
            T.uMinusY(iHn, i, j) = ComputeHn(T.uMinusY(iw, i, j), T.uMinusY(ib0, i, j), T.uMinusY(ibt, i, j), gam);
        }
    // Face momenta rho*Hn*u (:521-551).
    auto remom = [&](A3& F, int ni, int nj) {
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                F(irhoHnu, i, j) = F(irho, i, j) * F(iHn, i, j) * F(iu, i, j);
            }
    };
    auto remomv = [&](A3& F, int ni, int nj) {
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) F(irhoHnv, i, j) = F(irho, i, j) * F(iHn, i, j) * F(iv, i, j);
    };
    remom(T.uPlusX, nXP + 1, nYP);
    remom(T.uMinusX, nXP + 1, nYP);
    remom(T.uPlusY, nXP, nYP + 1);
    remom(T.uMinusY, nXP, nYP + 1);
    remomv(T.uPlusX, nXP + 1, nYP);
    remomv(T.uMinusX, nXP + 1, nYP);
    remomv(T.uPlusY, nXP, nYP + 1);
    remomv(T.uMinusY, nXP, nYP + 1);
}

// InterpolateB, :741-753.
inline double InterpolateB(double b0_0, double b0_1, double bt_0, double bt_1) {
    double b = bt_0 + bt_1;
    b = b + b0_0;
    b = b + b0_1;
    b = b * 0.5;
    return b;
}

// CorrectSlopes, :560-736 (2D).  Tile-seam handling depends on which neighbours were
// already processed; that order dependence is kept as written.
inline void CorrectSlopes(const RunSet& rp, Grid& g, Tiles& tiles, int tID) {
    Tile& T = TL(tiles, tID);
    int nXP = rp.nXpertile, nYP = rp.nYpertile;
    for (int j = 1; j <= nYP; ++j) {
        {
            int pid = T.West();
            Tile& P = TL(tiles, pid);
            double bl = InterpolateB(P.b0(nXP, j), P.b0(nXP, j + 1), P.bt(nXP, j), P.bt(nXP, j + 1));
            double br = InterpolateB(P.b0(nXP + 1, j), P.b0(nXP + 1, j + 1), P.bt(nXP + 1, j), P.bt(nXP + 1, j + 1));
            if ((P.uMinusX(iw, nXP + 1, j) < br) || (P.uPlusX(iw, nXP, j) < bl)) {
                T.uMinusX(iw, 1, j) = P.u(iw, nXP, j) + 0.5 * (br - bl);
            } else if (!(((T.uMinusX(iw, 1, j) != P.uMinusX(iw, nXP + 1, j)) && g.tc(pid).isGhostTile))) {
                // Fortran: "a /= b .and. isGhost .eqv. .false." parses as ((a/=b).and.isGhost).eqv..false.
                T.uMinusX(iw, 1, j) = P.uMinusX(iw, nXP + 1, j);
            }
            if (T.uMinusX(iHnpsi, 1, j) < 0.0) T.uMinusX(iHnpsi, 1, j) = P.u(iHnpsi, nXP, j);
        }
        for (int i = 1; i <= nXP; ++i) {
            double bl = InterpolateB(T.b0(i, j), T.b0(i, j + 1), T.bt(i, j), T.bt(i, j + 1));
            double br = InterpolateB(T.b0(i + 1, j), T.b0(i + 1, j + 1), T.bt(i + 1, j), T.bt(i + 1, j + 1));
            if ((T.uMinusX(iw, i + 1, j) < br) || (T.uPlusX(iw, i, j) < bl)) {
                T.uMinusX(iw, i + 1, j) = T.u(iw, i, j) + 0.5 * (br - bl);
                T.uPlusX(iw, i, j) = T.u(iw, i, j) + 0.5 * (bl - br);
            }
            if ((T.uMinusX(iHnpsi, i + 1, j) < 0.0) || (T.uPlusX(iHnpsi, i, j) < 0.0)) {
                T.uMinusX(iHnpsi, i + 1, j) = T.u(iHnpsi, i, j);
                T.uPlusX(iHnpsi, i, j) = T.u(iHnpsi, i, j);
            }
        }
        {
            int nid = T.East();
            Tile& N = TL(tiles, nid);
            double bl = InterpolateB(N.b0(1, j), N.b0(1, j + 1), N.bt(1, j), N.bt(1, j + 1));
            double br = InterpolateB(N.b0(2, j), N.b0(2, j + 1), N.bt(2, j), N.bt(2, j + 1));
            if ((N.uMinusX(iw, 2, j) < br) || (N.uPlusX(iw, 1, j) < bl)) {
                T.uPlusX(iw, nXP + 1, j) = N.u(iw, 1, j) + 0.5 * (bl - br);
            } else if (!(((T.uPlusX(iw, nXP + 1, j) != N.uPlusX(iw, 1, j)) && g.tc(nid).isGhostTile))) {
                T.uPlusX(iw, nXP + 1, j) = N.uPlusX(iw, 1, j);
            }
            if (T.uPlusX(iHnpsi, nXP + 1, j) < 0.0) T.uPlusX(iHnpsi, nXP + 1, j) = N.u(iHnpsi, 1, j);
        }
    }
    for (int i = 1; i <= nXP; ++i) {
        {
            int pid = T.South();
            Tile& P = TL(tiles, pid);
            double bb = InterpolateB(P.b0(i, nYP), P.b0(i + 1, nYP), P.bt(i, nYP), P.bt(i + 1, nYP));
            double bt_ = InterpolateB(P.b0(i, nYP + 1), P.b0(i + 1, nYP + 1), P.bt(i, nYP + 1), P.bt(i + 1, nYP + 1));
            if ((P.uMinusY(iw, i, nYP + 1) < bt_) || (P.uPlusY(iw, i, nYP) < bb)) {
                T.uMinusY(iw, i, 1) = P.u(iw, i, nYP) + 0.5 * (bt_ - bb);
            } else if (!(((T.uMinusY(iw, i, 1) != P.uMinusY(iw, i, nYP + 1)) && g.tc(pid).isGhostTile))) {
                T.uMinusY(iw, i, 1) = P.uMinusY(iw, i, nYP + 1);
            }
            if (T.uMinusY(iHnpsi, i, 1) < 0.0) T.uMinusY(iHnpsi, i, 1) = P.u(iHnpsi, i, nYP);
        }
        for (int j = 1; j <= nYP; ++j) {
            double bb = InterpolateB(T.b0(i, j), T.b0(i + 1, j), T.bt(i, j), T.bt(i + 1, j));
            double bt_ = InterpolateB(T.b0(i, j + 1), T.b0(i + 1, j + 1), T.bt(i, j + 1), T.bt(i + 1, j + 1));
            if ((T.uMinusY(iw, i, j + 1) < bt_) || (T.uPlusY(iw, i, j) < bb)) {
                T.uMinusY(iw, i, j + 1) = T.u(iw, i, j) + 0.5 * (bt_ - bb);
                T.uPlusY(iw, i, j) = T.u(iw, i, j) + 0.5 * (bb - bt_);
            }
            if ((T.uMinusY(iHnpsi, i, j + 1) < 0.0) || (T.uPlusY(iHnpsi, i, j) < 0.0)) {
                T.uMinusY(iHnpsi, i, j + 1) = T.u(iHnpsi, i, j);
                T.uPlusY(iHnpsi, i, j) = T.u(iHnpsi, i, j);
            }
        }
        {
            int nid = T.North();
            Tile& N = TL(tiles, nid);
            double bb = InterpolateB(N.b0(i, 1), N.b0(i + 1, 1), N.bt(i, 1), N.bt(i + 1, 1));
            double bt_ = InterpolateB(N.b0(i, 2), N.b0(i + 1, 2), N.bt(i, 2), N.bt(i + 1, 2));
            if ((N.uMinusY(iw, i, 2) < bt_) || (N.uPlusY(iw, i, 1) < bb)) {
                T.uPlusY(iw, i, nYP + 1) = N.u(iw, i, 1) + 0.5 * (bb - bt_);
            } else if (!(((T.uPlusY(iw, i, nYP + 1) != N.uPlusY(iw, i, 1)) && g.tc(nid).isGhostTile))) {
                T.uPlusY(iw, i, nYP + 1) = N.uPlusY(iw, i, 1);
            }
            if (T.uPlusY(iHnpsi, i, nYP + 1) < 0.0) T.uPlusY(iHnpsi, i, nYP + 1) = N.u(iHnpsi, i, 1);
        }
    }
}

// ComputeDesingularisedVariables, :762-878.
inline void ComputeDesingularisedVariables(const RunSet& rp, Tiles& tiles, int tID, bool computeVelocities) {
    Tile& T = TL(tiles, tID);
    double Hneps = rp.heightThreshold;
    for (int i = 1; i <= rp.nXpertile; ++i)
        for (int j = 1; j <= rp.nYpertile; ++j) {
            double rhoHnu = T.u(irhoHnu, i, j);
            double Hnpsi = T.u(iHnpsi, i, j);
            double gam = Gam(rp, T.u.col(i, j));
            double Hn = ComputeHn(T.u(iw, i, j), T.u(ib0, i, j), T.u(ibt, i, j), gam);
            if (Hn < 0.0) Hn = 0.0;
            if (Hnpsi < 0.0) Hnpsi = 0.0;
            double psi = std::min(2.0 * Hn * Hnpsi / (Hn * Hn + std::max(Hn * Hn, Hneps * Hneps)), rp.p.maxPack);
            double rho = Density(rp, psi);
            T.u(iHn, i, j) = Hn;
            T.u(ipsi, i, j) = psi;
            T.u(irho, i, j) = rho;
            if (computeVelocities) {
                double u = 2.0 * Hn * rhoHnu / (Hn * Hn + std::max(Hn * Hn, Hneps * Hneps)) / rho;
                T.u(iu, i, j) = u;
                double rhoHnv = T.u(irhoHnv, i, j);
                double v = 2.0 * Hn * rhoHnv / (Hn * Hn + std::max(Hn * Hn, Hneps * Hneps)) / rho;
                T.u(iv, i, j) = v;
            }
        }
}

// CalculateFluxes, :896-1182 (2D, dims = iFlux).
inline void CalculateFluxes(const RunSet& rp, Grid& g, Tiles& tiles, int tID, double& unitCFL) {
    Tile& T = TL(tiles, tID);
    int nXP = rp.nXpertile, nYP = rp.nYpertile;
    double dx = g.deltaX, dy = g.deltaY;
    unitCFL = HUGE_;
    double gam_ratio = 1.0;
    double cP[4], cM[4], hP[4], hM[4], dP[4], dM[4];
    for (int j = 1; j <= nYP; ++j)
        for (int i = 1; i <= nXP + 1; ++i) {
            const double* up = T.uPlusX.col(i, j);
            const double* um = T.uMinusX.col(i, j);
            double wsP = XMaxWaveSpeeds(rp, up), wsM = XMaxWaveSpeeds(rp, um);
            double aPos = (wsP > wsM) ? wsP : wsM;
            if (aPos < 0.0) aPos = 0.0;
            wsP = XMinWaveSpeeds(rp, up);
            wsM = XMinWaveSpeeds(rp, um);
            double aNeg = (wsP < wsM) ? wsP : wsM;
            if (aNeg > 0.0) aNeg = 0.0;
            if (aPos > EPS) {
                if (i == 1) {
                    Tile& P = TL(tiles, T.West());
                    gam_ratio = std::min(Gam(rp, P.u.col(nXP, j)) / Gam(rp, up), 1.0);
                } else {
                    gam_ratio = std::min(Gam(rp, T.u.col(i - 1, j)) / Gam(rp, up), 1.0);
                }
                unitCFL = std::min(gam_ratio * gam_ratio * dx / aPos, unitCFL);
            }
            if (std::fabs(aNeg) > EPS) {
                if (i == nXP + 1) {
                    Tile& N = TL(tiles, T.East());
                    gam_ratio = std::min(Gam(rp, N.u.col(1, j)) / Gam(rp, um), 1.0);
                } else {
                    gam_ratio = std::min(Gam(rp, T.u.col(i, j)) / Gam(rp, um), 1.0);
                }
                unitCFL = std::min(gam_ratio * gam_ratio * dx / std::fabs(aNeg), unitCFL);
            }
            XConvectionFlux(rp, up, cP);
            XConvectionFlux(rp, um, cM);
            HydrostaticFlux(rp, up, hP);
            HydrostaticFlux(rp, um, hM);
            if (i == nXP + 1) {
                DiffusionFlux(rp, up, TL(tiles, T.East()).uLimX.col(1, j), dP);
                DiffusionFlux(rp, um, T.uLimX.col(i - 1, j), dM);
            } else if (i == 1) {
                DiffusionFlux(rp, up, T.uLimX.col(i, j), dP);
                DiffusionFlux(rp, um, TL(tiles, T.West()).uLimX.col(nXP, j), dM);
            } else {
                DiffusionFlux(rp, up, T.uLimX.col(i, j), dP);
                DiffusionFlux(rp, um, T.uLimX.col(i - 1, j), dM);
            }
            double dif = aPos - aNeg;
            for (int k = 0; k < 4; ++k) {
                int d = IFLUX[k];
                double hX;
                if (dif < 1e-10) {
                    T.hXFlux(d, i, j) = 0.0; T.gXFlux(d, i, j) = 0.0; T.pXFlux(d, i, j) = 0.0;
                } else if (d == iw) {
                    double gp = Gam(rp, up), gn = Gam(rp, um);
                    hX = up[iHn - 1] * gp - um[iHn - 1] * gn;
                    hX = hX * aPos * aNeg;
                    hX = hX + (aPos * cM[k] - aNeg * cP[k]);
                    hX = hX / dif;
                    T.hXFlux(d, i, j) = hX; T.gXFlux(d, i, j) = 0.0; T.pXFlux(d, i, j) = 0.0;
                } else if (d == iHnpsi) {
                    double gp = Gam(rp, up), gn = Gam(rp, um);
                    hX = up[d - 1] * gp - um[d - 1] * gn;
                    hX = hX * aPos * aNeg;
                    hX = hX + (aPos * cM[k] - aNeg * cP[k]);
                    hX = hX / dif;
                    T.hXFlux(d, i, j) = hX; T.gXFlux(d, i, j) = 0.0; T.pXFlux(d, i, j) = 0.0;
                } else {
                    hX = up[d - 1] - um[d - 1];
                    hX = hX * aPos * aNeg;
                    hX = hX + (aPos * cM[k] - aNeg * cP[k]);
                    hX = hX / dif;
                    T.hXFlux(d, i, j) = hX;
                    T.gXFlux(d, i, j) = (aPos * hM[k] - aNeg * hP[k]) / dif;
                    T.pXFlux(d, i, j) = 0.5 * (dP[k] + dM[k]);
                }
            }
        }
    for (int j = 1; j <= nYP + 1; ++j)
        for (int i = 1; i <= nXP; ++i) {
            const double* up = T.uPlusY.col(i, j);
            const double* um = T.uMinusY.col(i, j);
            double wsP = YMaxWaveSpeeds(rp, up), wsM = YMaxWaveSpeeds(rp, um);
            double aPos = (wsP > wsM) ? wsP : wsM;
            if (aPos < 0.0) aPos = 0.0;
            wsP = YMinWaveSpeeds(rp, up);
            wsM = YMinWaveSpeeds(rp, um);
            double aNeg = (wsP < wsM) ? wsP : wsM;
            if (aNeg > 0.0) aNeg = 0.0;
            if (aPos > EPS) {
                if (j == 1) {
                    Tile& P = TL(tiles, T.South());
                    gam_ratio = std::min(Gam(rp, P.u.col(i, nYP)) / Gam(rp, up), 1.0);
                } else {
                    gam_ratio = std::min(Gam(rp, T.u.col(i, j - 1)) / Gam(rp, up), 1.0);
                }
                unitCFL = std::min(gam_ratio * gam_ratio * dy / aPos, unitCFL);
            }
            if (std::fabs(aNeg) > EPS) {
                if (j == nYP + 1) {
                    Tile& N = TL(tiles, T.North());
                    gam_ratio = std::min(Gam(rp, N.u.col(i, 1)) / Gam(rp, um), 1.0);
                } else {
                    gam_ratio = std::min(Gam(rp, T.u.col(i, j)) / Gam(rp, um), 1.0);
                }
                unitCFL = std::min(gam_ratio * gam_ratio * dy / std::fabs(aNeg), unitCFL);
            }
            YConvectionFlux(rp, up, cP);
            YConvectionFlux(rp, um, cM);
            HydrostaticFlux(rp, up, hP);
            HydrostaticFlux(rp, um, hM);
            if (j == nYP + 1) {
                DiffusionFlux(rp, up, TL(tiles, T.North()).uLimY.col(i, 1), dP);
                DiffusionFlux(rp, um, T.uLimY.col(i, j - 1), dM);
            } else if (j == 1) {
                DiffusionFlux(rp, up, T.uLimY.col(i, j), dP);
                DiffusionFlux(rp, um, TL(tiles, T.South()).uLimY.col(i, nYP), dM);
            } else {
                DiffusionFlux(rp, up, T.uLimY.col(i, j), dP);
                DiffusionFlux(rp, um, T.uLimY.col(i, j - 1), dM);
            }
            double dif = aPos - aNeg;
            for (int k = 0; k < 4; ++k) {
                int d = IFLUX[k];
                double hY;
                if (dif < 1e-10) {
                    T.hYFlux(d, i, j) = 0.0; T.gYFlux(d, i, j) = 0.0; T.pYFlux(d, i, j) = 0.0;
                } else if (d == iw) {
                    double gp = Gam(rp, up), gn = Gam(rp, um);
                    hY = up[iHn - 1] * gp - um[iHn - 1] * gn;
                    hY = hY * aPos * aNeg;
                    hY = hY + (aPos * cM[k] - aNeg * cP[k]);
                    hY = hY / dif;
                    T.hYFlux(d, i, j) = hY; T.gYFlux(d, i, j) = 0.0; T.pYFlux(d, i, j) = 0.0;
                } else if (d == iHnpsi) {
                    double gp = Gam(rp, up), gn = Gam(rp, um);
                    hY = up[d - 1] * gp - um[d - 1] * gn;
                    hY = hY * aPos * aNeg;
                    hY = hY + (aPos * cM[k] - aNeg * cP[k]);
                    hY = hY / dif;
                    T.hYFlux(d, i, j) = hY; T.gYFlux(d, i, j) = 0.0; T.pYFlux(d, i, j) = 0.0;
                } else {
                    hY = up[d - 1] - um[d - 1];
                    hY = hY * aPos * aNeg;
                    hY = hY + (aPos * cM[k] - aNeg * cP[k]);
                    hY = hY / dif;
                    T.hYFlux(d, i, j) = hY;
                    T.gYFlux(d, i, j) = (aPos * hM[k] - aNeg * hP[k]) / dif;
                    T.pYFlux(d, i, j) = 0.5 * (dP[k] + dM[k]);
                }
            }
        }
}

}  // namespace ko
