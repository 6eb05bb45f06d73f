"""Synthetic benchmark workloads, written with the reference's input keys.

No public dataset is involved: the reference measures on none and publishes no numbers.
Terrain for the larger configurations is a seeded spectral synthesis (power spectrum
k^-3, relief scaled to [0, 800] m, plus a regional tilt) injected as a vertex grid
through kg_upload_b0, since the reference could only read such a surface as a GDAL
raster.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi, config


def cap_release_256(tend: float = 30.0, nout: int = 1) -> abi.Params:
    """Plain FP64 hydraulic cap release: 256 x 256 cells at dx = 1 m on a 5-degree planar
    slope, cylindrical cap of radius 40 m and height 4 m centred at (128 m, 64 m) from the
    south-west corner, clear water, Chezy Cd = 0.01, no erosion, CFL 0.25, to t = 30 s.
    Laid out as 16 x 16 tiles of 16 x 16 cells with sponge edges."""
    slope = -math.tan(5.0 * math.pi / 180.0)
    text = f"""
Domain:
nXtiles = 16
nYtiles = 16
nXpertile = 16
nYpertile = 16
Xtilesize = 16
Boundary Conditions = sponge
Cap:
  capX = 0
  capY = -64
  capRadius = 40
  capHeight = 4
  capShape = flat
  capConc = 0
Parameters:
Drag = Chezy
Chezy Co = 0.01
Erosion = Off
Eddy Viscosity = 0
Solver:
T end = {tend}
cfl = 0.25
Output:
N out = {nout}
Topog:
Type = Function
Topog function = ySlope
Topog params = ({slope!r})
"""
    return config.parse(text).params


def fractal_terrain(nx1: int, ny1: int, dx: float, seed: int, relief: float = 800.0, tilt_deg: float = 8.0) -> np.ndarray:
    """Vertex heights (ny1, nx1): spectral synthesis with P(k) ~ k^-3 (amplitude ~ k^-1.5),
    min-max scaled to [0, relief], plus a planar tilt descending towards +y."""
    rng = np.random.default_rng(seed)
    kx = np.fft.rfftfreq(nx1)
    ky = np.fft.fftfreq(ny1)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    k[0, 0] = 1.0
    amp = k ** -1.5
    amp[0, 0] = 0.0
    phase = rng.uniform(0.0, 2.0 * np.pi, size=amp.shape)
    spec = amp * (rng.standard_normal(amp.shape) + 0j) * np.exp(1j * phase)
    field = np.fft.irfft2(spec, s=(ny1, nx1))
    field = (field - field.min()) / (field.max() - field.min()) * relief
    y = np.arange(ny1) * dx
    field = field - math.tan(tilt_deg * math.pi / 180.0) * (y - y.mean())[:, None]
    return np.ascontiguousarray(field, dtype=np.float64)


def morpho_flux_2048(tend: float = 600.0, nout: int = 1, seed: int = 12345):
    """2D morphodynamic flux release: 2048 x 2048 cells at dx = 5 m (32 x 32 tiles of
    64 x 64 cells) on seeded fractal terrain (P(k) ~ k^-3, relief 0-800 m, 8-degree tilt),
    a point inflow of radius 6 m with a triangular hydrograph (0 -> 200 -> 0 m^3/s over
    300 s, sediment concentration 0.3), Voellmy drag (mu = 0.1, xi = 500 m/s^2, i.e.
    Chezy Co = g / xi), mixed erosion/deposition with erodible depth 2 m and eddy
    viscosity 1e-2, to t = 600 s.  Sponge edges keep a flow that reaches the domain edge
    from halting the run.  Returns (params, b0 vertex grid)."""
    text = f"""
Domain:
nXtiles = 32
nYtiles = 32
nXpertile = 64
nYpertile = 64
Xtilesize = 320
Boundary Conditions = sponge
Source:
  sourceX = 0
  sourceY = -3000
  sourceRadius = 6
  sourceTime = (0,150,300)
  sourceFlux = (0,200,0)
  sourceConc = (0.3,0.3,0.3)
Parameters:
Drag = Voellmy
Coulomb Co = 0.1
Chezy Co = {9.81 / 500.0!r}
Erosion = On
Erosion Depth = 2
Eddy Viscosity = 1e-2
Solver:
T end = {tend}
cfl = 0.25
Output:
N out = {nout}
Topog:
Type = Function
Topog function = flat
"""
    p = config.parse(text).params
    p.topog = abi.TOPO["upload"]
    nx1 = p.nXtiles * p.nXpertile + 1
    ny1 = p.nYtiles * p.nYpertile + 1
    b0 = fractal_terrain(nx1, ny1, p.Xtilesize / p.nXpertile, seed)
    return p, b0


WORKLOADS = {
    "cap_release_256_fp64": dict(
        desc="plain FP64 2D hydraulic cap release, 256x256 cells, dx=1 m, 5 deg slope, cap r=40 m h=4 m at "
             "(128,64), Chezy 0.01, no erosion, CFL 0.25, to t=30 s (16x16 tiles of 16x16 cells)",
        params=cap_release_256, prec=abi.PREC_FP64, b0=None, spinup=0.0),
    "morpho_flux_2048_fp64": dict(
        desc="2D morphodynamic flux release, 2048x2048 cells at dx=5 m on seeded fractal terrain (k^-3, relief "
             "0-800 m, 8 deg tilt), inflow r=6 m with hydrograph 0-200-0 m^3/s over 300 s (conc 0.3), Voellmy "
             "(mu=0.1, xi=500), mixed erosion with 2 m erodible depth, eddy viscosity 1e-2, to t=600 s; "
             "FP64 plain; timed after a spin-up to t=120 s",
        params=morpho_flux_2048, prec=abi.PREC_FP64, spinup=120.0),
    "cap_release_256_fp32": dict(
        desc="2D hydraulic cap release, 256x256 cells, dx=1 m, 5 deg slope, cap r=40 m h=4 m at (128,64), Chezy "
             "0.01, no erosion, CFL 0.25, to t=30 s (16x16 tiles of 16x16 cells); FP32 form (FP64 free surface, "
             "bed, mass/solids rows and dt)",
        params=cap_release_256, prec=abi.PREC_FP32, b0=None, spinup=0.0),
    "morpho_flux_2048_fp32": dict(
        desc="2D morphodynamic flux release, 2048x2048 cells at dx=5 m on seeded fractal terrain (k^-3, relief "
             "0-800 m, 8 deg tilt), inflow r=6 m with hydrograph 0-200-0 m^3/s over 300 s (conc 0.3), Voellmy "
             "(mu=0.1, xi=500), mixed erosion with 2 m erodible depth, eddy viscosity 1e-2, to t=600 s; "
             "FP32 form (FP64 free surface, bed, mass/solids rows and dt); timed after a spin-up to t=120 s",
        params=morpho_flux_2048, prec=abi.PREC_FP32, spinup=120.0),
}
