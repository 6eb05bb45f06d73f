"""Host-side mirror of the reference's Run / IntegrateTo interface over the C ABI.

``Simulation`` drives any library that exports the kg_ API of include/kestrel_gpu.h (the
GPU library built from kestrel_gb300/csrc).  It follows the call order of
src/main.f90:148-171: read input -> InitialiseGrid/LoadDEM (kg_create, kg_upload_b0) ->
LoadSourceConditions (kg_load_sources) -> Run (kg_run / kg_integrate_to).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class KestrelError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{abi.KG_ERR.get(code, code)}: {msg}")
        self.code = code


class Simulation:
    """One simulation on one context.  ``lib``/``prefix`` select the implementation."""

    def __init__(self, lib, prefix: str, params: abi.Params, precision: int = abi.PREC_FP64,
                 b0: np.ndarray | None = None, load_sources: bool = True, raster: dict | None = None):
        self.lib, self.pre = lib, prefix
        self.params = params
        self.nX, self.nY = params.nXpertile, params.nYpertile
        h = C.c_void_p()
        if prefix == "kg":
            rc = self._f("create")(C.byref(params), precision, C.byref(h))
        else:
            rc = self._f("create")(C.byref(params), C.byref(h))
        if rc != abi.KG_OK:
            msg = self._f("last_error")(None)
            raise KestrelError(rc, "create failed: " + (msg.decode() if msg else ""))
        self.h = h
        if b0 is not None:
            self.upload_b0(b0)
        if raster is not None:
            self.upload_raster(**raster)
        if load_sources:
            self._check(self._f("load_sources")(self.h))

    @classmethod
    def view(cls, lib, handle, params: abi.Params):
        """A non-owning view of a context owned elsewhere (a batch member): every getter
        works; closing the view leaves the context alone."""
        self = cls.__new__(cls)
        self.lib, self.pre, self.params = lib, "kg", params
        self.nX, self.nY = params.nXpertile, params.nYpertile
        self.h = C.c_void_p(handle)
        self._owned = False
        return self

    def _f(self, name):
        return getattr(self.lib, f"{self.pre}_{name}")

    def _check(self, rc):
        if rc != abi.KG_OK:
            msg = self._f("last_error")(self.h)
            raise KestrelError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if self.h and getattr(self, "_owned", True):
            self._f("destroy")(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set-up --------------------------------------------------------------------
    def upload_b0(self, b0: np.ndarray):
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        ny1, nx1 = b0.shape
        self._check(self._f("upload_b0")(self.h, b0.ctypes.data_as(C.POINTER(C.c_double)), nx1, ny1))

    def upload_raster(self, values: np.ndarray, origin, pixel, nodata: float, center=(0.0, 0.0)):
        """kg_upload_raster: an elevation raster (ny, nx), row 0 the north row, with its
        geotransform origin (x, y) of the upper-left corner, pixel sizes (w, h) with h < 0,
        no-data value and the projected domain centre (E, N)."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        ny, nx = v.shape
        g = abi.Raster(nx=nx, ny=ny, origin_x=float(origin[0]), origin_y=float(origin[1]), pixel_w=float(pixel[0]),
                       pixel_h=float(pixel[1]), nodata=float(nodata), center_e=float(center[0]), center_n=float(center[1]))
        self._check(self._f("upload_raster")(self.h, v.ctypes.data_as(C.POINTER(C.c_double)), C.byref(g)))

    def load_state(self, ids, state: np.ndarray, bt_vertex: np.ndarray | None, t: float):
        """load_state: restart from saved tiles (state (n, 4, nY, nX): w, rhoHnu, rhoHnv,
        Hnpsi; bt_vertex (n, nY+1, nX+1) or None) at time t, instead of loading sources."""
        ids = (C.c_int32 * len(ids))(*ids)
        st = np.ascontiguousarray(state, dtype=np.float64)
        bt = None if bt_vertex is None else np.ascontiguousarray(bt_vertex, dtype=np.float64)
        f = self._f("load_state")
        f.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                      C.c_double]
        f.restype = C.c_int
        self._check(f(self.h, ids, len(ids), st.ctypes.data_as(C.POINTER(C.c_double)),
                      None if bt is None else bt.ctypes.data_as(C.POINTER(C.c_double)), t))

    # -- stepping ------------------------------------------------------------------
    def step(self, t_stop: float) -> abi.StepStats:
        st = abi.StepStats()
        self._check(self._f("step")(self.h, t_stop, C.byref(st)))
        return st

    def integrate_to(self, t_end: float) -> abi.StepStats:
        st = abi.StepStats()
        self._check(self._f("integrate_to")(self.h, t_end, C.byref(st)))
        return st

    def run(self) -> abi.StepStats:
        st = abi.StepStats()
        self._check(self._f("run")(self.h, C.byref(st)))
        return st

    def hydraulic_rhs(self, t: float, substep: int = 1) -> float:
        adv = C.c_double()
        self._check(self._f("hydraulic_rhs")(self.h, t, substep, C.byref(adv)))
        return adv.value

    def redistribution_stats(self):
        """(cells walked, dependency waves, walks) of RedistributeGrid so far."""
        v = [C.c_int64() for _ in range(3)]
        self._check(self._f("redistribution_stats")(self.h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    # -- state access --------------------------------------------------------------
    @property
    def time(self):
        t, dt = C.c_double(), C.c_double()
        self._check(self._f("get_time")(self.h, C.byref(t), C.byref(dt)))
        return t.value, dt.value

    def _ids(self, name):
        n = C.c_int32(0)
        self._f(name)(self.h, None, C.byref(n))
        buf = (C.c_int32 * max(n.value, 1))()
        self._check(self._f(name)(self.h, buf, C.byref(n)))
        return [buf[i] for i in range(n.value)]

    def active_tiles(self):
        return self._ids("get_active_tiles")

    def ghost_tiles(self):
        return self._ids("get_ghost_tiles")

    def field(self, tile: int, field: int) -> np.ndarray:
        out = np.empty(self.nX * self.nY, dtype=np.float64)
        self._check(self._f("get_tile_field")(self.h, tile, field, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(self.nY, self.nX)

    def get_state(self):
        """(tile ids, state (n, 4, nY, nX), vertex bt (n, nY+1, nX+1), t): the whole active
        state in one call (kg_get_state), in the form load_state takes back."""
        n = C.c_int32(0)
        self._check(self._f("get_state")(self.h, None, C.byref(n), None, None))
        na = n.value
        ids = (C.c_int32 * max(na, 1))()
        st = np.empty((na, 4, self.nY, self.nX), dtype=np.float64)
        bt = np.empty((na, self.nY + 1, self.nX + 1), dtype=np.float64)
        self._check(self._f("get_state")(self.h, ids, C.byref(n), st.ctypes.data_as(C.POINTER(C.c_double)),
                                         bt.ctypes.data_as(C.POINTER(C.c_double))))
        return [ids[i] for i in range(na)], st, bt, self.time[0]

    def set_field(self, tile: int, field: int, values: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        self._check(self._f("set_tile_field")(self.h, tile, field, v.ctypes.data_as(C.POINTER(C.c_double))))

    def vertex(self, tile: int, which: int) -> np.ndarray:
        out = np.empty((self.nX + 1) * (self.nY + 1), dtype=np.float64)
        self._check(self._f("get_tile_vertex")(self.h, tile, which, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(self.nY + 1, self.nX + 1)

    def rhs(self, tile: int, k: int) -> np.ndarray:
        out = np.empty(self.nX * self.nY, dtype=np.float64)
        self._check(self._f("get_tile_rhs")(self.h, tile, k, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(self.nY, self.nX)

    def maxima(self, tile: int, which: int) -> np.ndarray:
        n = self.nX * self.nY * (1 if which == 5 else 2)
        out = np.empty(n, dtype=np.float64)
        self._check(self._f("get_tile_maxima")(self.h, tile, which, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(-1, self.nY, self.nX)

    def volume(self) -> np.ndarray:
        out = (C.c_double * 4)()
        self._check(self._f("volume")(self.h, out))
        return np.array(list(out))

    def state(self, fields=range(1, 14)) -> dict:
        """{tile_id: array (len(fields), nY, nX)} for every active tile."""
        return {t: np.stack([self.field(t, f) for f in fields]) for t in self.active_tiles()}

    def global_field(self, field: int, fill=np.nan) -> np.ndarray:
        """Assemble one field over the whole domain (inactive tiles filled)."""
        p = self.params
        out = np.full((p.nYtiles * self.nY, p.nXtiles * self.nX), fill)
        for t in self.active_tiles():
            gi, gj = (t - 1) % p.nXtiles, (t - 1) // p.nXtiles
            out[gj * self.nY:(gj + 1) * self.nY, gi * self.nX:(gi + 1) * self.nX] = self.field(t, field)
        return out
