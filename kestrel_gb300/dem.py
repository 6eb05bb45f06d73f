"""Elevation rasters for the raster topography (kg_upload_raster).

The reference reads its DEM through GDAL (src/RasterData.cpp, src/GeoTiffRead.f90): it
warps the user's raster to UTM at the grid spacing into DEM.vrt and reads one section per
tile.  GDAL and PROJ are not available to this package, so the raster arrives already in
the projected coordinates of the run, either as an array with its geotransform or as an
ESRI ASCII grid (one of the formats GDAL reads, as its AAIGrid driver georeferences it:
origin at the upper-left corner of the upper-left pixel, square pixels, north-up).  The
projected domain centre, which the reference obtains from the input's latitude and
longitude through PROJ (src/TopogSettings.f90:387), is passed explicitly.
"""
from __future__ import annotations

import math
import os

import numpy as np


def read_ascii_grid(path: str) -> dict:
    """An ESRI ASCII grid as the keyword arguments of Simulation.upload_raster (without the
    centre): values (nrows, ncols) from the north row, origin, pixel and nodata.  A grid
    without NODATA_value gets NaN, which no value equals."""
    header = {}
    with open(path) as f:
        pos = f.tell()
        line = f.readline()
        while line:
            parts = line.split()
            if len(parts) == 2 and parts[0][0].isalpha():
                header[parts[0].lower()] = float(parts[1])
                pos = f.tell()
                line = f.readline()
            else:
                break
        f.seek(pos)
        data = np.array(f.read().split(), dtype=np.float64)
    nc, nr = int(header["ncols"]), int(header["nrows"])
    if data.size != nc * nr:
        raise ValueError(f"{path}: expected {nc * nr} values, found {data.size}")
    cs = header["cellsize"]
    if "xllcorner" in header:
        x0 = header["xllcorner"]
    else:
        x0 = header["xllcenter"] - 0.5 * cs
    if "yllcorner" in header:
        y0 = header["yllcorner"]
    else:
        y0 = header["yllcenter"] - 0.5 * cs
    return dict(values=data.reshape(nr, nc), origin=(x0, y0 + nr * cs), pixel=(cs, -cs),
                nodata=header.get("nodata_value", math.nan))


def write_ascii_grid(path: str, values: np.ndarray, origin, cellsize: float, nodata: float = -9999.0):
    """Write values (nrows, ncols, north row first) as an ESRI ASCII grid whose upper-left
    corner is origin = (x, y); values are written in Python's shortest round-trip form, so
    reading the file back gives the same doubles."""
    v = np.asarray(values, dtype=np.float64)
    nr, nc = v.shape
    with open(path, "w") as f:
        f.write(f"ncols {nc}\nnrows {nr}\nxllcorner {float(origin[0])!r}\nyllcorner {float(origin[1]) - nr * cellsize!r}\n"
                f"cellsize {float(cellsize)!r}\nNODATA_value {float(nodata)!r}\n")
        for row in v:
            f.write(" ".join(repr(float(x)) for x in row) + "\n")


def raster_input(parsed, base_dir: str = ".", center=(0.0, 0.0)) -> dict | None:
    """The raster of a parsed input with Topog type Raster/DEM: the 'Raster File' (under
    'DEM directory' when given) read as an ESRI ASCII grid, with the domain centre."""
    t = parsed.topog
    if t.get("type") not in ("dem", "raster"):
        return None
    name = t.get("raster file")
    if not name:
        raise ValueError("Topog type Raster needs 'Raster File'")
    path = os.path.join(base_dir, t.get("dem directory", ""), name)
    r = read_ascii_grid(path)
    r["center"] = (float(center[0]), float(center[1]))
    return r
