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


def fractal_terrain(nx1: int, ny1: int, dx: float, seed: int, relief: float = 800.0, tilt_deg: float = 8.0,
                    smooth: float = 0.0) -> np.ndarray:
    """Vertex heights (ny1, nx1): spectral synthesis with P(k) ~ k^-3 (amplitude ~ k^-1.5),
    optionally low-passed by a Gaussian of standard deviation `smooth` metres, min-max
    scaled to [0, relief], plus a planar tilt descending towards +y."""
    rng = np.random.default_rng(seed)
    kx = np.fft.rfftfreq(nx1)
    ky = np.fft.fftfreq(ny1)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    k[0, 0] = 1.0
    amp = k ** -1.5
    amp[0, 0] = 0.0
    if smooth > 0.0:
        amp = amp * np.exp(-2.0 * math.pi ** 2 * (smooth / dx) ** 2 * k ** 2)
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


def morpho_flux_window(size: int = 256, tile: int = 32, tend: float = 600.0, nout: int = 1, seed: int = 12345,
                       src_from_south: float = 300.0):
    """The 2048^2 morphodynamic flux release cut down to a size x size window of its own
    terrain: the same seeded 2049^2 vertex grid (same dx = 5 m, relief, tilt), of which the
    window holds the source with `src_from_south` metres of terrain south of it and the
    rest downhill (north); the same source (radius 6 m, hydrograph 0 -> 200 -> 0 m^3/s over
    300 s, concentration 0.3), Voellmy drag, mixed erosion with 2 m erodible depth, eddy
    viscosity 1e-2, sponge edges, in tiles of tile^2 cells.  Returns (params, b0)."""
    pf, bf = morpho_flux_2048(tend=tend, nout=nout, seed=seed)
    dx = pf.Xtilesize / pf.nXpertile
    half_full = 0.5 * pf.nXtiles * pf.Xtilesize
    sx, sy = pf.sources[0].x, pf.sources[0].y
    L = size * dx
    x_lo, y_lo = sx - 0.5 * L, sy - src_from_south
    c0, r0 = int(round((x_lo + half_full) / dx)), int(round((y_lo + half_full) / dx))
    b0 = np.ascontiguousarray(bf[r0:r0 + size + 1, c0:c0 + size + 1])
    p, _ = morpho_flux_2048(tend=tend, nout=nout, seed=seed)
    p.nXtiles = p.nYtiles = size // tile
    p.nXpertile = p.nYpertile = tile
    p.Xtilesize = p.Ytilesize = tile * dx
    # window centred at (0, 0): the source keeps its place on the terrain
    p.sources[0].x = sx - (c0 * dx - half_full + 0.5 * L)
    p.sources[0].y = sy - (r0 * dx - half_full + 0.5 * L)
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


# ---- ensembles (the batched and served forms) ---------------------------------------

DRAGS = ("Chezy", "Voellmy", "Manning")


def ensemble_member(seed: int, side: int | None = None, tend: float | None = None, tile: int | None = None,
                    side_range=(128, 1024), tend_range=(60.0, 600.0), dx: float = 5.0, volume: float | None = None,
                    drag: str | None = None, morpho: bool | None = None, kind: str | None = None):
    """One ensemble solve, drawn from `seed`: grid side log-uniform in side_range (rounded to
    a multiple of 64 cells) unless given, dx = 5 m, its own seeded fractal terrain, a cap or
    a flux source (half each) of volume log-uniform in [1e3, 1e6] m^3 placed 20% of the way
    from the centre to the upper (southern) edge, always inside an interior tile row, drag drawn from Chezy / Voellmy / Manning with coefficients uniform over
    physical ranges, morphodynamics on for half, sponge edges.  The terrain's relief scales
    with the domain (800 m over the 10.24 km of the 2048^2 configuration; the 8-degree tilt
    is kept), so every size sees the same slopes.  `tile` is the tile side (the
    autotuner's choice; by default the largest that leaves interior tiles); volume / drag /
    morpho / kind ("cap" or "flux") override the draws.  Returns (params, b0, description
    dict)."""
    rng = np.random.default_rng(seed)
    if side is None:
        side = int(round(math.exp(rng.uniform(math.log(side_range[0]), math.log(side_range[1]))) / 64.0)) * 64
        side = max(64, side)
    if tend is None:
        tend = float(rng.uniform(*tend_range))
    if not tile:
        # largest tile side that leaves an interior of tiles (edge tiles never activate
        # under sponge edges)
        tile = max([t for t in (16, 32, 64) if side % t == 0 and side // t >= 4] or [16])
    if side % tile:
        raise ValueError(f"tile {tile} does not divide side {side}")
    L = side * dx
    v_draw = math.exp(float(rng.uniform(math.log(1e3), math.log(1e6))))
    d_draw = DRAGS[int(rng.integers(0, 3))]
    m_draw = bool(rng.integers(0, 2))
    volume = v_draw if volume is None else volume
    drag = d_draw if drag is None else drag
    morpho = m_draw if morpho is None else morpho
    y0 = -0.2 * L
    if drag == "Chezy":
        dtext = f"Drag = Chezy\nChezy Co = {float(rng.uniform(0.005, 0.05))!r}"
    elif drag == "Voellmy":
        dtext = f"Drag = Voellmy\nCoulomb Co = {float(rng.uniform(0.05, 0.3))!r}\nChezy Co = {9.81 / float(rng.uniform(200.0, 2000.0))!r}"
    else:
        dtext = f"Drag = Manning\nManning Co = {float(rng.uniform(0.02, 0.1))!r}"
    k_draw = "cap" if rng.integers(0, 2) else "flux"
    if (kind or k_draw) == "cap":
        h = float(rng.uniform(1.0, 5.0))
        r = math.sqrt(volume / (math.pi * h))
        r = min(r, 0.12 * L)
        h = volume / (math.pi * r * r)
        stext = f"Cap:\n  capX = 0\n  capY = {y0!r}\n  capRadius = {r!r}\n  capHeight = {h!r}\n  capShape = flat\n  capConc = 0.2"
        src = ("cap", r, h)
    else:
        T = float(rng.uniform(60.0, 300.0))
        q = 2.0 * volume / T
        stext = (f"Source:\n  sourceX = 0\n  sourceY = {y0!r}\n  sourceRadius = {2.5 * dx!r}\n"
                 f"  sourceTime = (0,{T / 2!r},{T!r})\n  sourceFlux = (0,{q!r},0)\n  sourceConc = (0.2,0.2,0.2)")
        src = ("flux", T, q)
    mtext = (f"Erosion = On\nErosion Depth = {float(rng.uniform(0.5, 3.0))!r}" if morpho else "Erosion = Off")
    text = f"""
Domain:
nXtiles = {side // tile}
nYtiles = {side // tile}
nXpertile = {tile}
nYpertile = {tile}
Xtilesize = {tile * dx!r}
Boundary Conditions = sponge
{stext}
Parameters:
{dtext}
{mtext}
Solver:
T end = {tend!r}
cfl = 0.25
Output:
N out = 1
Topog:
Type = Function
Topog function = flat
"""
    p = config.parse(text).params
    p.topog = abi.TOPO["upload"]
    b0 = fractal_terrain(side + 1, side + 1, dx, seed + 7919, relief=800.0 * min(1.0, L / 10240.0))
    return p, b0, dict(seed=seed, side=side, tile=tile, tend=tend, volume=volume, drag=drag, morpho=morpho, source=src)


def ensemble(n: int = 256, seed: int = 2024, tiles=None, **kw):
    """The batched ensemble of n members (seeds seed .. seed + n - 1); `tiles` maps a grid
    side to its tile side (a dict, or a function such as the autotuner's choice)."""
    out = []
    for k in range(n):
        side = None
        rng = np.random.default_rng(seed + k)
        lo, hi = kw.get("side_range", (128, 1024))
        side = max(64, int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))) / 64.0)) * 64)
        tile = tiles(side) if callable(tiles) else (tiles or {}).get(side)
        out.append(ensemble_member(seed + k, side=side, tile=tile, **{k2: v for k2, v in kw.items() if k2 != "side_range"}))
    return out


def serve_requests(n: int, rate: float = 20.0, seed: int = 77, sides=(256, 512, 1024, 2048), tend_range=(60.0, 600.0),
                   tiles=None):
    """A served request stream: Poisson arrivals at `rate` per second, grid sides uniform
    over `sides`, end times uniform over tend_range, everything else as the ensemble.
    Returns [(arrival_s, params, b0, desc)]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += float(rng.exponential(1.0 / rate))
        side = int(sides[int(rng.integers(0, len(sides)))])
        tend = float(rng.uniform(*tend_range))
        tile = tiles(side) if callable(tiles) else (tiles or {}).get(side)
        p, b0, d = ensemble_member(seed * 1000 + k, side=side, tend=tend, tile=tile)
        out.append((t, p, b0, d))
    return out


def sparse_tiles(size: int = 8192, tile: int = 64, dx: float = 2.0, tend: float = 300.0, nout: int = 1, seed: int = 31337,
                 relief: float = 400.0, tilt_deg: float = 6.0, smooth: float = 20.0, radius: float = 100.0,
                 qpeak: tuple = (20000.0, 60000.0)):
    """Large sparse tiled domain: size x size cells at dx (8192^2 at 2 m by default, in
    tiles of tile^2 cells) on fractal terrain with its own seed, low-passed at 20 m (relief
    0-400 m plus a 6-degree tilt: median slope about 12 degrees, 99th percentile about 28),
    three flux sources of radius 100 m at seeded positions in the middle 60% of the domain
    with triangular hydrographs (peak 20,000-60,000 m^3/s over 100-300 s, concentration
    0.2-0.4: large enough that the flows cover about 5% of the tiles by t = 300 s),
    Pouliquen-Forterre drag with the reference's defaults, morphodynamics on, sponge edges,
    to t = 300 s.  Returns (params, b0)."""
    rng = np.random.default_rng(seed)
    L = size * dx
    srcs = []
    for k in range(3):
        x, y = (float(v) for v in rng.uniform(-0.3 * L, 0.3 * L, size=2))
        T = float(rng.uniform(100.0, 300.0))
        q = float(rng.uniform(*qpeak))
        cc = float(rng.uniform(0.2, 0.4))
        srcs.append(f"Source:\n  sourceX = {x!r}\n  sourceY = {y!r}\n  sourceRadius = {float(radius)!r}\n"
                    f"  sourceTime = (0,{T / 2!r},{T!r})\n  sourceFlux = (0,{q!r},0)\n  sourceConc = ({cc!r},{cc!r},{cc!r})")
    text = f"""
Domain:
nXtiles = {size // tile}
nYtiles = {size // tile}
nXpertile = {tile}
nYpertile = {tile}
Xtilesize = {tile * dx!r}
Boundary Conditions = sponge
{chr(10).join(srcs)}
Parameters:
Drag = Pouliquen
Erosion = On
Solver:
T end = {tend!r}
cfl = 0.25
Output:
N out = {nout}
Topog:
Type = Function
Topog function = flat
"""
    p = config.parse(text).params
    p.topog = abi.TOPO["upload"]
    b0 = fractal_terrain(size + 1, size + 1, dx, seed + 104729, relief=relief, tilt_deg=tilt_deg, smooth=smooth)
    return p, b0


WORKLOADS["sparse_8192_fp32"] = dict(
    desc="large sparse tiled domain: 8192x8192 cells at dx=2 m (128x128 tiles of 64x64), seeded fractal terrain "
         "(k^-3 low-passed at 20 m, relief 0-400 m, 6 deg tilt), three seeded flux sources (r=100 m, peak "
         "20000-60000 m^3/s over 100-300 s, conc 0.2-0.4), Pouliquen-Forterre drag, mixed erosion, to t=300 s; FP32 "
         "form; timed after a spin-up to t=290 s",
    params=sparse_tiles, prec=abi.PREC_FP32, spinup=290.0, timeline=20.0, twin_restart=True)
WORKLOADS["sparse_8192_fp64"] = dict(
    desc="large sparse tiled domain: 8192x8192 cells at dx=2 m (128x128 tiles of 64x64), seeded fractal terrain "
         "(k^-3 low-passed at 20 m, relief 0-400 m, 6 deg tilt), three seeded flux sources (r=100 m, peak "
         "20000-60000 m^3/s over 100-300 s, conc 0.2-0.4), Pouliquen-Forterre drag, mixed erosion, to t=300 s; FP64 "
         "plain; timed after a spin-up to t=290 s",
    params=sparse_tiles, prec=abi.PREC_FP64, spinup=290.0, timeline=20.0)


def dem_2048(seed: int = 1, pixel: float = 2.5, center=(500000.0, 4000000.0)):
    """The 2048^2 morphodynamic configuration with its bed read from an elevation raster
    (topog = raster): seeded fractal terrain (k^-3, relief 0-800 m, 8-degree tilt) sampled
    at `pixel` metres over the domain plus a 40 m margin, north-up, centred on `center`.
    Returns (params, raster keyword arguments of Simulation.upload_raster)."""
    p, _ = morpho_flux_2048()
    p.topog = abi.TOPO["raster"]
    half = 0.5 * p.nXtiles * p.Xtilesize + 40.0
    n = int(round(2.0 * half / pixel))
    z = fractal_terrain(n, n, pixel, seed + 7, relief=800.0, tilt_deg=8.0)[::-1]  # north row first
    return p, dict(values=np.ascontiguousarray(z), origin=(center[0] - half, center[1] + half), pixel=(pixel, -pixel),
                   nodata=-9999.0, center=center)
