"""The reference's text outputs, written from a simulation's read-back state.

Restates the formats of src/Output.f90: the per-output snapshot NNNNNN.txt and its vertex
file NNNNNN.txt_topo (OutputSolutionData_txt, :754-931), Volume.txt (CalculateVolume,
:617-737) and Maximums.txt (OutputMaximums_txt, :1270-1355), with Fortran's ES/F edit
descriptors and the blank record after every tile row, so the reference's own readers
(src/Restart.f90:151-328) and checks read them unchanged.  ``run_with_output`` mirrors
Run (src/TimeStepper.f90:72-113): output 0 at t_start, then one snapshot, one Volume line
and the maxima after each output interval.  Latitude and longitude columns are 0 (the path
is not georeferenced).  Works with any implementation behind the ABI (the GPU library or
the oracle).
"""
from __future__ import annotations

import math
import os

import numpy as np

from .solver import Simulation


def fortran_es(x: float, w: int, d: int, e: int | None = None) -> str:
    """Fortran ESw.d (e = None) or ESw.dEe of one value, right-justified in w columns."""
    x = float(x)
    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    m, ex = f"{x:.{d}E}".split("E")
    n = int(ex)
    if x == 0.0:
        n = 0
    if e is None:
        expo = f"E{'-' if n < 0 else '+'}{abs(n):02d}" if abs(n) <= 99 else f"{'-' if n < 0 else '+'}{abs(n):03d}"
    else:
        expo = f"E{'-' if n < 0 else '+'}{abs(n):0{e}d}"
    s = m + expo
    return s.rjust(w) if len(s) <= w else "*" * w


def es18(x: float) -> str:
    return fortran_es(x, 18, 10, 3)


def cell_centres(p, tile: int):
    """x(i), y(j) of a tile's cells (src/Grid.f90:348-351), domain centred at (0, 0)."""
    gi, gj = (tile - 1) % p.nXtiles + 1, (tile - 1) // p.nXtiles + 1
    dx, dy = p.Xtilesize / p.nXpertile, p.Ytilesize / p.nYpertile
    xs, ys = p.nXtiles * p.Xtilesize, p.nYtiles * p.Ytilesize
    i = np.arange(1, p.nXpertile + 1)
    j = np.arange(1, p.nYpertile + 1)
    x = -0.5 * xs + dx * ((gi - 1.0) * p.nXpertile + (i - 0.5))
    y = -0.5 * ys + dy * ((gj - 1.0) * p.nYpertile + (j - 0.5))
    return x, y


def flow_speed(p, Hn, u, v, dbdx, dbdy):
    """sqrt(FlowSquaredSpeedSlopeAligned) where Hn > heightThreshold, else 0."""
    if p.geometric_factors:
        m = u * u * (1.0 + dbdx * dbdx)
        m = m + v * v * (1.0 + dbdy * dbdy) + 2.0 * dbdx * dbdy * u * v
    else:
        m = u * u
        m = m + v * v
    return np.where(Hn > p.heightThreshold, np.sqrt(np.maximum(m, 0.0)), 0.0)


def output_filename(n: int, width: int = 6, ext: str = ".txt") -> str:
    return f"{n:0{width}d}{ext}"


SNAP_HEADER = ("    tile", "                 x", "                 y", "          latitude", "         longitude",
               "        flow_depth", "        flow_speed", "        x_velocity", "        y_velocity",
               "           density", "   solids_fraction", "            x_flux", "            y_flux",
               "             Hnpsi", "                 w", "    base_elevation", "  elevation_change",
               "           x_slope", "           y_slope")


def write_snapshot(sim: Simulation, path: str):
    """NNNNNN.txt (cell-centred solution) and NNNNNN.txt_topo (vertex b0, bt)."""
    p = sim.params
    with open(path, "w") as f, open(path + "_topo", "w") as g:
        f.write(", ".join(SNAP_HEADER) + "\n")
        g.write("    tile, " + "         B0_vertex, " + "         Bt_vertex" + "\n")
        for t in sim.active_tiles():
            F = {k: sim.field(t, k) for k in range(1, 14)}
            x, y = cell_centres(p, t)
            spd = flow_speed(p, F[5], F[6], F[7], F[12], F[13])
            for j in range(p.nYpertile):
                for i in range(p.nXpertile):
                    cols = [x[i], y[j], 0.0, 0.0, F[5][j, i], spd[j, i], F[6][j, i], F[7][j, i], F[9][j, i],
                            F[8][j, i], F[2][j, i], F[3][j, i], F[4][j, i], F[1][j, i], F[10][j, i], F[11][j, i],
                            F[12][j, i], F[13][j, i]]
                    f.write(f"{t:8d}, " + ", ".join(es18(c) for c in cols) + "\n")
                f.write("\n")
            b0, bt = sim.vertex(t, 0), sim.vertex(t, 1)
            for j in range(p.nYpertile + 1):
                for i in range(p.nXpertile + 1):
                    g.write(f"{t:8d}, {es18(b0[j, i])}, {es18(bt[j, i])}\n")
                g.write("\n")


VOLUME_HEADER = ("        time", "                  volume", "        total_bed_volume", "              total_mass",
                 "                bed_mass", "       total_solids_mass", "         bed_solids_mass")


def volume_line(sim: Simulation, t: float) -> str:
    p = sim.params
    vol, bed, mass, solids = sim.volume()
    rhob = p.rhow * p.BedPorosity + p.rhos * (1.0 - p.BedPorosity)
    vals = [vol, bed, mass, bed * rhob, solids * p.rhos, bed * p.rhos * (1.0 - p.BedPorosity)]
    return f"{t:12.2f}" + "".join(", " + fortran_es(v, 24, 15) for v in vals) + "\n"


def write_volume(sim: Simulation, path: str, t: float, create: bool = False):
    new = create or not os.path.exists(path)
    with open(path, "w" if new else "a") as f:
        if new:
            f.write(", ".join(VOLUME_HEADER) + "\n")
        f.write(volume_line(sim, t))


MAX_HEADER = ("    tile", "        x_distance", "        y_distance", "          latitude", "         longitude",
              "         max_depth", "       t_max_depth", "         max_speed", "       t_max_speed",
              "       max_erosion", "     t_max_erosion", "       max_deposit", "     t_max_deposit",
              "   max_solids_frac", " t_max_solids_frac", "   inundation_time")


def write_maxima(sim: Simulation, path: str):
    p = sim.params
    with open(path, "w") as f:
        f.write(", ".join(MAX_HEADER) + "\n")
        for t in sim.active_tiles():
            M = [sim.maxima(t, w) for w in range(6)]
            x, y = cell_centres(p, t)
            for j in range(p.nYpertile):
                for i in range(p.nXpertile):
                    cols = [x[i], y[j], 0.0, 0.0]
                    for w in range(5):
                        cols += [M[w][0, j, i], M[w][1, j, i]]
                    cols.append(M[5][0, j, i])
                    f.write(f"{t:8d}, " + ", ".join(es18(c) for c in cols) + "\n")
                f.write("\n")
            f.write("\n")


def run_with_output(sim: Simulation, out_dir: str):
    """Run (src/TimeStepper.f90:72-113) with the text outputs: output 0 and the first Volume
    line at t_start, then after every output interval a snapshot, a Volume line and
    Maximums.txt."""
    p = sim.params
    os.makedirs(out_dir, exist_ok=True)
    nout = p.Nout if p.Nout > 0 else 100
    write_snapshot(sim, os.path.join(out_dir, output_filename(0)))
    write_volume(sim, os.path.join(out_dir, "Volume.txt"), p.tstart, create=True)
    dT = (p.tend - p.tstart) / nout
    for k in range(1, nout + 1):
        t = p.tstart + k * dT
        sim.integrate_to(t)
        write_snapshot(sim, os.path.join(out_dir, output_filename(k)))
        write_volume(sim, os.path.join(out_dir, "Volume.txt"), t)
        write_maxima(sim, os.path.join(out_dir, "Maximums.txt"))


def read_snapshot(path: str, nX: int, nY: int):
    """Parse a snapshot and its _topo file the way LoadInitialCondition_txt does
    (src/Restart.f90:151-328): {tile: {column name: (nY, nX) array}} and
    {tile: (b0, bt) vertex arrays (nY+1, nX+1)}."""
    cells: dict = {}
    with open(path) as f:
        header = [h.strip() for h in f.readline().split(",")]
        rows = [ln for ln in f if ln.strip()]
    for ln in rows:
        parts = [s.strip() for s in ln.split(",")]
        t = int(parts[0])
        cells.setdefault(t, []).append([float(v) for v in parts[1:]])
    out = {}
    for t, vals in cells.items():
        a = np.array(vals).reshape(nY, nX, len(header) - 1)
        out[t] = {header[k + 1]: a[:, :, k] for k in range(len(header) - 1)}
    verts: dict = {}
    with open(path + "_topo") as g:
        g.readline()
        for ln in g:
            if not ln.strip():
                continue
            parts = [s.strip() for s in ln.split(",")]
            verts.setdefault(int(parts[0]), []).append((float(parts[1]), float(parts[2])))
    topo = {t: (np.array([v[0] for v in vv]).reshape(nY + 1, nX + 1), np.array([v[1] for v in vv]).reshape(nY + 1, nX + 1))
            for t, vv in verts.items()}
    return out, topo


def restart_from_snapshot(lib, params, path: str, t: float, precision: int = 0, b0: np.ndarray | None = None,
                          prefix: str = "kg"):
    """A new simulation restarted from snapshot `path` (and `path`_topo) at time t, as
    LoadInitialCondition does (src/Restart.f90:55-328): the saved tiles are activated in
    order with their w, momenta, Hnpsi and vertex bt; the running maxima start afresh.
    `lib` is a loaded library (None: the GPU library) and `prefix` its entry-point prefix."""
    from . import lib as _lib
    sim = _lib.simulation(params, precision=precision, b0=b0, load_sources=False) if lib is None else \
        Simulation(lib, prefix, params, precision=precision, b0=b0, load_sources=False)
    cells, topo = read_snapshot(path, params.nXpertile, params.nYpertile)
    ids = sorted(cells)
    state = np.stack([np.stack([cells[t_]["w"], cells[t_]["x_flux"], cells[t_]["y_flux"], cells[t_]["Hnpsi"]])
                      for t_ in ids])
    btv = np.stack([topo[t_][1] for t_ in ids])
    sim.load_state(ids, state, btv, t)
    return sim
