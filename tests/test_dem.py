"""Raster topography (TileHeightData / GetRasterData / Bicubic_r, src/dem.f90:203-356,
src/Interp2d.f90:214-282): the oracle's restatement against properties the reference's
interpolation has by construction, its error behaviour, the input keys and the ASCII grid
reader; on the GPU, the library's heights and a short morphodynamic run against the
oracle, bit for bit."""
import math

import numpy as np
import pytest

import _oracle
from kestrel_gb300 import abi, config, dem, lib

E0, N0 = 500000.0, 4000000.0  # projected domain centre


def raster_case(tiles=4, n=16, dx=2.0, morpho=False, tend=2.0):
    text = f"""
Domain:
nXtiles = {tiles}
nYtiles = {tiles}
nXpertile = {n}
nYpertile = {n}
Xtilesize = {n * dx!r}
Boundary Conditions = sponge
Source:
  sourceX = 0.0
  sourceY = 0.0
  sourceRadius = {3 * dx!r}
  sourceTime = (0,20)
  sourceFlux = (4,4)
  sourceConc = (0.2,0.2)
Parameters:
Drag = Voellmy
Erosion = {'On' if morpho else 'Off'}
Solver:
T end = {tend!r}
Output:
N out = 1
Topog:
Type = Raster
Raster File = dem.asc
"""
    return config.parse(text)


def surface(kind, half=80.0, pix=1.0, seed=5):
    """A raster around the centre: (values, origin, pixel) with half-width `half` metres."""
    n = int(round(2 * half / pix))
    X = -half + pix * (np.arange(n) + 0.5)          # pixel centres, west to east
    Y = half - pix * (np.arange(n) + 0.5)           # north to south
    XX, YY = np.meshgrid(X, Y)
    if kind == "plane":
        z = 40.0 + 0.25 * XX - 0.125 * YY
    else:
        rng = np.random.default_rng(seed)
        z = 50.0 - 0.3 * YY + 2.0 * np.sin(XX / 7.0) * np.cos(YY / 11.0) + 0.05 * rng.standard_normal(XX.shape)
    return dict(values=z, origin=(E0 - half, N0 + half), pixel=(pix, -pix), nodata=-9999.0, center=(E0, N0))


def vertex_positions(p, tile):
    """Vertex (x, y) of a tile relative to the domain centre (src/UpdateTiles.f90:308-325)."""
    gi, gj = (tile - 1) % p.nXtiles, (tile - 1) // p.nXtiles
    dx = p.Xtilesize / p.nXpertile
    x = -0.5 * p.nXtiles * p.Xtilesize + dx * (gi * p.nXpertile + np.arange(p.nXpertile + 1))
    y = -0.5 * p.nYtiles * p.Ytilesize + dx * (gj * p.nYpertile + np.arange(p.nYpertile + 1))
    return np.meshgrid(x, y)


def test_input_keys():
    parsed = raster_case()
    assert parsed.params.topog == abi.TOPO["raster"]
    assert parsed.topog["raster file"] == "dem.asc"
    with pytest.raises(config.InputError):
        config.parse("Domain:\nnXtiles = 2\nnYtiles = 2\nnXpertile = 4\nnYpertile = 4\nXtilesize = 4\n"
                     "Solver:\nT end = 1\nTopog:\nType = SRTM\n")


def test_ascii_grid_round_trip(tmp_path):
    r = surface("rough", half=20.0)
    path = str(tmp_path / "dem.asc")
    dem.write_ascii_grid(path, r["values"], r["origin"], r["pixel"][0])
    back = dem.raster_input(raster_case(), base_dir=str(tmp_path), center=(E0, N0))
    assert np.array_equal(back["values"], r["values"])
    assert back["origin"] == r["origin"] and back["pixel"] == r["pixel"] and back["nodata"] == -9999.0
    assert back["center"] == (E0, N0)


def test_ascii_grid_header_forms(tmp_path):
    """The centre form of the ESRI header (xllcenter/yllcenter: half a cell inside the
    corner), a grid without NODATA_value (NaN, which no value equals), and a grid whose
    value count disagrees with its header."""
    path = tmp_path / "c.asc"
    path.write_text("ncols 3\nnrows 2\nxllcenter 101.0\nyllcenter 201.0\ncellsize 2.0\n1 2 3\n4 5 6\n")
    r = dem.read_ascii_grid(str(path))
    assert r["origin"] == (100.0, 204.0) and r["pixel"] == (2.0, -2.0)
    assert np.isnan(r["nodata"]) and r["values"].tolist() == [[1, 2, 3], [4, 5, 6]]
    path.write_text("ncols 3\nnrows 2\nxllcorner 0\nyllcorner 0\ncellsize 1\n1 2 3\n4 5\n")
    with pytest.raises(ValueError, match="expected 6 values, found 5"):
        dem.read_ascii_grid(str(path))


def test_oracle_reproduces_a_plane():
    """Bicubic_r's finite-difference derivatives are exact for a linear surface and its
    Hermite patch is then that surface, so every vertex height is the plane at the vertex
    (the mean of four samples around it), to rounding -- shifted by half a pixel: the
    reference puts pixel (i, j)'s value at pixel coordinate (i, j) = the pixel's upper-left
    corner (imgx = (E - originX) / pixelWidth + 1, src/dem.f90:335-336), while a raster's
    values describe the pixel centres, so a vertex takes the surface half a pixel east and
    half a pixel south of it."""
    p = raster_case().params
    sim = _oracle.simulation(p, raster=surface("plane"))
    for t in sim.active_tiles():
        X, Y = vertex_positions(p, t)
        want = 40.0 + 0.25 * (X + 0.5) - 0.125 * (Y - 0.5)
        got = sim.vertex(t, 0)
        assert np.max(np.abs(got - want)) < 1e-10, t


def test_oracle_seams_single_valued():
    """Seam vertices shared by two tiles hold one value after activation
    (EqualiseTopographicBoundaryData keeps the right / upper tile's)."""
    p = raster_case().params
    sim = _oracle.simulation(p, raster=surface("rough"))
    tiles = set(sim.active_tiles())
    for t in tiles:
        if t + 1 in tiles and t % p.nXtiles != 0:
            assert np.array_equal(sim.vertex(t, 0)[:-1, -1], sim.vertex(t + 1, 0)[:-1, 0]), t
        if t + p.nXtiles in tiles:
            assert np.array_equal(sim.vertex(t, 0)[-1, :-1], sim.vertex(t + p.nXtiles, 0)[0, :-1]), t


def test_oracle_errors():
    p = raster_case().params
    small = surface("rough", half=20.0)  # the source's tiles need sections beyond 20 m
    with pytest.raises(Exception, match="raster"):
        _oracle.simulation(p, raster=small)
    holes = surface("rough")
    holes["values"] = holes["values"].copy()
    holes["values"][80, 80] = -9999.0  # the centre pixel: inside the source tiles' sections
    with pytest.raises(Exception, match="No-data"):
        _oracle.simulation(p, raster=holes)
    bad = surface("rough")
    bad["pixel"] = (1.0, 1.0)  # south-up rasters are refused
    with pytest.raises(Exception):
        _oracle.simulation(p, raster=bad)


@pytest.mark.gpu
def test_gpu_heights_bitexact():
    p = raster_case().params
    r = surface("rough")
    g, o = lib.simulation(p, raster=r), _oracle.simulation(p, raster=r)
    assert g.active_tiles() == o.active_tiles() and g.ghost_tiles() == o.ghost_tiles()
    for t in o.active_tiles():
        assert np.array_equal(g.vertex(t, 0), o.vertex(t, 0)), t
        for f in (10, 12, 13):
            assert np.array_equal(g.field(t, f), o.field(t, f)), (t, f)


@pytest.mark.gpu
def test_gpu_run_on_raster_bitexact():
    """A short morphodynamic run on the raster bed: same steps, activation and fields."""
    p = raster_case(morpho=True, tend=1.5).params
    r = surface("rough")
    g, o = lib.simulation(p, raster=r), _oracle.simulation(p, raster=r)
    sg, so = g.integrate_to(p.tend), o.integrate_to(p.tend)
    assert (sg.steps, sg.rejected) == (so.steps, so.rejected)
    assert g.active_tiles() == o.active_tiles()
    for t in o.active_tiles():
        for f in (1, 2, 3, 4, 11):
            a, b = g.field(t, f), o.field(t, f)
            scale = max(np.max(np.abs(b)), 1e-300)
            assert np.max(np.abs(a - b)) / scale <= 1e-10, (t, f)


@pytest.mark.gpu
def test_gpu_raster_errors():
    p = raster_case().params
    with pytest.raises(Exception, match="raster"):
        lib.simulation(p, raster=surface("rough", half=20.0))
    holes = surface("rough")
    holes["values"] = holes["values"].copy()
    holes["values"][80, 80] = -9999.0
    with pytest.raises(Exception, match="No-data"):
        lib.simulation(p, raster=holes)


# ---- the analytic surfaces of src/TopogFuncs.f90 not covered by the reference's inputs ----

def surface_case(name, params, tiles=4, n=8, dx=1.0):
    text = f"""
Domain:
nXtiles = {tiles}
nYtiles = {tiles}
nXpertile = {n}
nYpertile = {n}
Xtilesize = {n * dx!r}
Boundary Conditions = sponge
Cap:
  capX = 0.0
  capY = 0.0
  capRadius = {2.5 * dx!r}
  capHeight = 0.5
  capShape = flat
Parameters:
Drag = Chezy
Solver:
T end = 0.5
Output:
N out = 1
Topog:
Type = Function
Topog function = {name}
Topog params = ({','.join(repr(float(v)) for v in params)})
"""
    return config.parse(text).params


def numpy_surface(name, P, X, Y):
    """Vectorised restatement of the same surfaces (an independent check of the oracle)."""
    pi = math.pi
    if name == "x2slopes":
        a, b, R = P
        xc0 = (math.sqrt(1 + a * a) - math.sqrt(1 + b * b)) * R / (a - b)
        zc0 = (a * math.sqrt(1 + b * b) - b * math.sqrt(1 + a * a)) * R / (a - b)
        x1, x2 = xc0 - a * R / math.sqrt(1 + a * a), xc0 - b * R / math.sqrt(1 + b * b)
        mid = zc0 - np.sqrt(np.maximum(R * R - (X - xc0) ** 2, 0.0))
        return np.where(X < x1, -a * X, np.where(X > x2, -b * X, mid))
    if name in ("usgs", "flume"):
        if name == "usgs":
            t0, t1, xw, lo, hi, H, s = 31.0, 2.4, 8.5, 1.0, 2.0, P[0], P[1]
        else:
            t0, t1, xw, H, s = P[0], P[1], P[2], P[4], P[5]
            lo, hi = 0.5 * P[3], 1.5 * P[3]
        al = 8.5 / (math.asinh(-math.tan(4 * pi / 180)) - math.asinh(-math.tan(t0 * pi / 180)))
        xc0 = -al * math.asinh(-math.tan(t0 * pi / 180))
        zc0 = -al * math.cosh(-xc0 / al)
        x1 = xc0 + al * math.asinh(-math.tan(t1 * pi / 180))
        b = np.where(X < 0, -math.tan(t0 * pi / 180) * X,
                     np.where(X > x1, zc0 + al * math.cosh((x1 - xc0) / al) - math.tan(t1 * pi / 180) * (X - x1),
                              zc0 + al * np.cosh((X - xc0) / al)))
        wall = 0.5 * H * (np.tanh(s * (Y - lo)) - np.tanh(s * (Y - hi)) + np.tanh(s * (Y + hi)) - np.tanh(s * (Y + lo)))
        return b + np.where(X < xw, wall, 0.0)
    if name == "channel power law":
        sl, W, al = P
        return sl * X + math.cos(math.atan(sl)) * (np.abs(Y) / W) ** al
    if name == "channel trapezium":
        sl, W, Sb = P
        return sl * X + math.cos(math.atan(sl)) * np.maximum(0.0, Sb * (np.abs(Y) - 0.5 * W))
    if name == "xbislope":
        a1, a2, lam = math.tan(P[0] * pi / 180), math.tan(P[1] * pi / 180), P[2]
        return -0.5 * (a1 + a2) * X + 0.5 * (a1 - a2) * lam * np.log(np.cosh(X / lam))
    if name == "xtrislope":
        s1, s2, s3 = (math.tan(v * pi / 180) for v in P[:3])
        lam, x1, x2 = P[3:]
        c2 = (x1 - 0.5 * lam) * 0.5 * (s1 - s2)
        c3 = (x1 + 0.5 * lam) * 0.5 * (s1 - s2) + c2
        c4 = (x2 - 0.5 * lam) * 0.5 * (s2 - s3) + c3
        c5 = (x2 + 0.5 * lam) * 0.5 * (s2 - s3) + c4
        A1, A2 = 0.5 * (s2 - s1) * lam / pi, 0.5 * (s3 - s2) * lam / pi
        return np.select([X < x1 - 0.5 * lam, X < x1 + 0.5 * lam, X < x2 - 0.5 * lam, X < x2 + 0.5 * lam],
                         [s1 * X, A1 * np.sin((X - x1) * pi / lam - 0.5 * pi) + 0.5 * (s1 + s2) * X + c2, s2 * X + c3,
                          A2 * np.sin((X - x2) * pi / lam - 0.5 * pi) + 0.5 * (s2 + s3) * X + c4], s3 * X + c5)
    raise KeyError(name)


SURFACES = [("x2slopes", (0.6, 0.1, 5.0)), ("usgs", (0.3, 20.0)), ("flume", (25.0, 3.0, 6.0, 1.5, 0.4, 15.0)),
            ("channel power law", (-0.2, 3.0, 2.0)), ("channel trapezium", (-0.2, 2.0, 0.7)),
            ("xbislope", (20.0, 5.0, 3.0)), ("xtrislope", (30.0, 15.0, 5.0, 2.0, -4.0, 6.0))]


@pytest.mark.parametrize("name,params", SURFACES)
def test_oracle_analytic_surfaces(name, params):
    p = surface_case(name, params)
    sim = _oracle.simulation(p)
    for t in sim.active_tiles():
        X, Y = vertex_positions(p, t)
        want = numpy_surface(name, params, X, Y)
        assert np.allclose(sim.vertex(t, 0), want, rtol=1e-12, atol=1e-12), (name, t)


def test_surface_parameter_counts():
    with pytest.raises(config.InputError, match="six"):
        surface_case("flume", (25.0, 3.0))
    with pytest.raises(config.InputError):
        surface_case("no such surface", (1.0,))


@pytest.mark.gpu
@pytest.mark.parametrize("name,params", SURFACES)
def test_gpu_analytic_surfaces_bitexact(name, params):
    """A cap release on each surface: the bed equals the oracle's bit for bit, the same
    steps are accepted and refused, and the state agrees to 1e-12 of each field's scale.
    (On these curved beds a handful of cells near the wet front differ in the last bit
    after the first step, although the RHS of any given state is bit-identical; on the
    linear beds of the other parity tests the whole state is bit-identical.)"""
    p = surface_case(name, params)
    g, o = lib.simulation(p), _oracle.simulation(p)
    sg, so = g.integrate_to(p.tend), o.integrate_to(p.tend)
    assert (sg.steps, sg.rejected) == (so.steps, so.rejected)
    assert g.active_tiles() == o.active_tiles()
    for t in o.active_tiles():
        assert np.array_equal(g.vertex(t, 0), o.vertex(t, 0)), t
        for f in (1, 2, 3, 4):
            a, b = g.field(t, f), o.field(t, f)
            assert np.max(np.abs(a - b)) <= 1e-12 * max(np.max(np.abs(b)), 1e-300), (t, f)
