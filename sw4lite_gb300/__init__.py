"""sw4lite_gb300: GB300-native (sm_103a) elastic-wave time step behind sw4lite's
kernel/phase API.

The compute path is libsw4g.so (CUDA kernels + C ABI, include/sw4g.h), built in-tree
by ``python -m sw4lite_gb300.builder``.  This module loads it with ctypes and offers a
thin Python view of the C ABI for tests and benchmarks; PyTorch is used only for
device memory and streams.  There is no CPU fallback: every call that computes
runs on the GPU, and loading fails loudly when the library is missing.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libsw4g.so"
HEADER = _PKG.parent / "include" / "sw4g.h"
DEV_HEADER = _PKG.parent / "include" / "sw4g_dev.h"

_lib = None

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_VP = C.c_void_p


class Sw4gError(RuntimeError):
    pass


class NonFiniteError(Sw4gError):
    """A step's new level held NaN or infinite values (SW4G_NAN_DETECTED); .report is
    the object's nan_report() dict."""

    def __init__(self, msg, report):
        super().__init__(msg)
        self.report = report


class GridDesc(C.Structure):
    """sw4g_grid (include/sw4g.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double),
                ("zmin", C.c_double), ("bc", C.c_int * 6), ("sg_gp", C.c_int),
                ("sg_damping", C.c_double), ("sg_order", C.c_int), ("soa", C.c_int),
                ("precision", C.c_int)]


class SourceDesc(C.Structure):
    """sw4g_source (include/sw4g.h)."""
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("moment", C.c_int),
                ("fx", C.c_double), ("fy", C.c_double), ("fz", C.c_double),
                ("mxx", C.c_double), ("mxy", C.c_double), ("mxz", C.c_double),
                ("myy", C.c_double), ("myz", C.c_double), ("mzz", C.c_double),
                ("freq", C.c_double), ("t0", C.c_double), ("kind", C.c_int)]


class TopoDesc(C.Structure):
    """sw4g_topography (include/sw4g.h)."""
    _fields_ = [("amp", C.c_double), ("xc", C.c_double), ("yc", C.c_double), ("lx", C.c_double),
                ("ly", C.c_double), ("zeta_break", C.c_double), ("order", C.c_int)]


class GeoDesc(C.Structure):
    """sw4g_geo (include/sw4g.h): the grid's geographic mapping."""
    _fields_ = [("lon_origin", C.c_double), ("lat_origin", C.c_double), ("az", C.c_double),
                ("meters_per_degree", C.c_double), ("meters_per_longitude", C.c_double),
                ("const_meters_per_longitude", C.c_int)]


class SacEvent(C.Structure):
    """sw4g_sac_event (include/sw4g.h): the event a SAC header names."""
    _fields_ = [("lat", C.c_double), ("lon", C.c_double), ("depth", C.c_double),
                ("time_offset", C.c_double)]


class UsgsStation(C.Structure):
    """sw4g_usgs_station (include/sw4g.h): one receiver file's header fields."""
    _fields_ = [("station", C.c_char_p), ("x", C.c_double), ("y", C.c_double),
                ("gp_x", C.c_double), ("gp_y", C.c_double), ("utc", C.c_int * 7),
                ("mode", C.c_int), ("xyz", C.c_int), ("t_shift", C.c_double), ("dt", C.c_double)]


def topo_desc(amp, xc, yc, lx, ly, zeta_break=0.95, order=4) -> TopoDesc:
    t = TopoDesc()
    t.amp, t.xc, t.yc, t.lx, t.ly, t.zeta_break, t.order = amp, xc, yc, lx, ly, zeta_break, order
    return t


# time-function kinds
GAUSSIAN, C6SMOOTHBUMP, RICKER, VERYSMOOTHBUMP = 0, 1, 2, 3
# boundary kinds (the reference's boundaryConditionType numbering)
FREE, DIRICHLET, SUPERGRID, PERIODIC, INTERFACE = 0, 1, 2, 3, 4
MODE_PHASES, MODE_FUSED = 0, 1
# receiver record modes (the reference's TimeSeries::receiverMode numbering)
REC_DISPLACEMENT, REC_DIV, REC_CURL, REC_STRAINS, REC_VELOCITY, REC_GRADIENT = 0, 1, 2, 3, 4, 5
# sw4g_status codes
OK, BAD_ARGUMENT, CUDA_ERROR, NAN_DETECTED, NOT_SUPPORTED, TIMEOUT, IO_ERROR = range(7)

_SIGS = {
    "sw4g_version": ([], C.c_char_p),
    "sw4g_status_string": ([C.c_int], C.c_char_p),
    "sw4g_stencil_coefficients": ([_D, _D, _D, _D], C.c_int),
    "sw4g_rhs4sg": ([C.c_int] * 8 + [_I, _VP, _VP, _VP, _VP, C.c_double, _VP, _VP, _VP, _VP],
                    C.c_int),
    "sw4g_predfort": ([C.c_int] * 7 + [_VP] * 6 + [C.c_double, _VP], C.c_int),
    "sw4g_corrfort": ([C.c_int] * 7 + [_VP] * 4 + [C.c_double, _VP], C.c_int),
    "sw4g_dpdmtfort": ([C.c_int] * 6 + [_VP] * 4 + [C.c_double, _VP], C.c_int),
    "sw4g_addsgd4fort": ([C.c_int] * 7 + [_VP] * 13 + [C.c_double, _VP], C.c_int),
    "sw4g_addsgd6fort": ([C.c_int] * 7 + [_VP] * 13 + [C.c_double, _VP], C.c_int),
    "sw4g_bcfortsg": ([C.c_int] * 7 + [_I, C.c_int, C.c_int, C.c_int, _VP, C.c_double, _I, _D,
                                       _VP, _VP, C.POINTER(_VP), _VP, _VP, _VP], C.c_int),
    "sw4g_supergrid_profile": ([C.POINTER(GridDesc), C.c_int, _D, _D, _D], C.c_int),
    "sw4g_boundary_windows": ([C.POINTER(GridDesc), _I, _I], C.c_int),
    "sw4g_discretize_source": ([C.POINTER(GridDesc), C.POINTER(SourceDesc), C.c_int, _I, _D, _I],
                               C.c_int),
    "sw4g_ew_create": ([C.POINTER(GridDesc), _VP, C.POINTER(_VP)], C.c_int),
    "sw4g_ew_create_subdomain": ([C.POINTER(GridDesc), C.c_int, C.c_int, C.c_int, C.c_int, _VP,
                                  C.POINTER(_VP)], C.c_int),
    "sw4g_ew_step_part": ([_VP, C.c_int], C.c_int),
    "sw4g_ew_halo_bytes": ([_VP, C.c_int], C.c_longlong),
    "sw4g_ew_halo_pack": ([_VP, C.c_int, C.c_int, _VP], C.c_int),
    "sw4g_ew_halo_unpack": ([_VP, C.c_int, C.c_int, _VP], C.c_int),
    "sw4g_ew_step_group": ([C.POINTER(_VP), C.c_int, _I, C.c_int], C.c_int),
    "sw4g_halo_len": ([C.c_int] * 6 + [C.c_int], C.c_longlong),
    "sw4g_halo_pack": ([C.c_int] * 9 + [_VP, _VP, _VP], C.c_int),
    "sw4g_halo_unpack": ([C.c_int] * 9 + [_VP, _VP, _VP], C.c_int),
    "sw4g_ew_create_topo": ([C.POINTER(GridDesc), C.POINTER(TopoDesc), _VP, C.POINTER(_VP)],
                            C.c_int),
    "sw4g_ew_num_grids": ([_VP], C.c_int),
    "sw4g_ew_gradient": ([_VP, C.c_int, C.c_int, _VP, C.c_int, _D, _VP, _VP, _VP, C.c_int],
                         C.c_int),
    "sw4g_ew_grid_dims": ([_VP, C.c_int, _I, _I, _I, C.POINTER(C.c_longlong)], C.c_int),
    "sw4g_ew_set_material_grid": ([_VP, C.c_int, _VP, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_set_fields_grid": ([_VP, C.c_int, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_get_fields_grid": ([_VP, C.c_int, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_curvilinear_arrays": ([_VP, _VP, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_destroy": ([_VP], C.c_int),
    "sw4g_ew_npts": ([_VP], C.c_longlong),
    "sw4g_ew_set_material": ([_VP, _VP, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_add_source": ([_VP, C.POINTER(SourceDesc)], C.c_int),
    "sw4g_ew_add_grid_point_sources": ([_VP, C.c_int, _I, _D, _D, _D, _I], C.c_int),
    "sw4g_ew_clear_sources": ([_VP], C.c_int),
    "sw4g_ew_num_grid_point_sources": ([_VP], C.c_int),
    "sw4g_ew_set_time_step": ([_VP, C.c_double, C.c_double], C.c_int),
    "sw4g_ew_compute_time_step": ([_VP, C.c_double, C.c_double, _D, _I], C.c_int),
    "sw4g_ew_time": ([_VP], C.c_double),
    "sw4g_ew_set_graphs": ([_VP, C.c_int], C.c_int),
    "sw4g_ew_set_gradient_memory": ([_VP, C.c_longlong], C.c_int),
    "sw4g_ew_set_source_discretization": ([_VP, C.c_int], C.c_int),
    "sw4g_ew_write_checkpoint": ([_VP, C.c_char_p, C.c_int], C.c_int),
    "sw4g_ew_read_checkpoint": ([_VP, C.c_char_p, _I], C.c_int),
    "sw4g_discretize_source_topo": ([_VP, _VP, C.c_int, _D, _VP, C.c_int, _I, _D, _I, _I, _D, _I], C.c_int),
    "sw4g_ew_grid_point_sources": ([_VP, C.c_int, C.c_int, _I, _D, _I], C.c_int),
    "sw4g_ew_set_fields": ([_VP, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_get_fields": ([_VP, _VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_field": ([_VP, C.c_int], _VP),
    "sw4g_ew_step": ([_VP, C.c_int, C.c_int], C.c_int),
    "sw4g_ew_set_nan_check": ([_VP, C.c_int], C.c_int),
    "sw4g_ew_nan_report": ([_VP, _I, _I, _I, _I, _I, C.POINTER(C.c_longlong), _D], C.c_int),
    "sw4g_ew_status": ([_VP], C.c_int),
    "sw4g_ew_enforce_bc": ([_VP, _VP], C.c_int),
    "sw4g_rhs4sgcurv": ([C.c_int] * 7 + [_I] + [_VP] * 8 + [_VP], C.c_int),
    "sw4g_metric": ([C.c_int] * 7 + [C.c_double, _VP, _VP, _VP, _VP], C.c_int),
    "sw4g_gaussian_hill_grid": ([C.c_int] * 7 + [C.c_double] * 3 + [C.c_int] + [C.c_double] * 5
                                + [_VP, _VP], C.c_int),
    "sw4g_freesurfcurvisg": ([C.c_int] * 9 + [_VP] * 4 + [_D] + [_VP] * 3 + [_VP], C.c_int),
    "sw4g_addsgd4cfort": ([C.c_int] * 7 + [_VP] * 11 + [C.c_double, _VP], C.c_int),
    "sw4g_addsgd6cfort": ([C.c_int] * 7 + [_VP] * 11 + [C.c_double, _VP], C.c_int),
    "sw4g_curvilinear_time_step": ([C.c_int] * 7 + [_VP] * 5 + [C.c_double, _D, _VP], C.c_int),
    "sw4g_nearest_grid_point": ([C.POINTER(GridDesc), C.c_double, C.c_double, C.c_double, _I],
                                C.c_int),
    "sw4g_ew_set_receivers": ([_VP, C.c_int, _I, _I, C.c_int], C.c_int),
    "sw4g_ew_set_receivers_grid": ([_VP, C.c_int, _I, _I, _I, C.c_int], C.c_int),
    "sw4g_ew_nearest_grid_point": ([_VP, C.c_double, C.c_double, C.c_double, _I, _I], C.c_int),
    "sw4g_ew_topography_z": ([_VP, C.c_double, C.c_double, C.POINTER(C.c_double)], C.c_int),
    "sw4g_ew_record_shape": ([_VP, _I, _I], C.c_int),
    "sw4g_ew_get_records": ([_VP, _VP, C.c_int], C.c_int),
    "sw4g_ew_launches_per_step": ([_VP, C.c_int], C.c_int),
    "sw4g_ew_profile_kernels": ([_VP, C.c_int, _D], C.c_int),
    "sw4g_dev_set_stage_chunks": ([C.c_int], C.c_int),
    "sw4g_dev_set_mixed_tma": ([C.c_int], C.c_int),
    "sw4g_dev_set_rows_overlap": ([C.c_int], C.c_int),
    "sw4g_dev_set_adjoint_pipeline": ([C.c_int], C.c_int),
    "sw4g_dev_stage_kchunk": ([C.c_longlong, C.c_int, C.c_int, C.c_int, _I], C.c_int),
    "sw4g_geo_default": ([C.POINTER(GeoDesc)], C.c_int),
    "sw4g_geographic_coord": ([C.POINTER(GeoDesc), C.c_double, C.c_double, _D, _D], C.c_int),
    "sw4g_write_usgs": ([C.c_char_p, C.POINTER(GeoDesc), C.POINTER(UsgsStation), _D, C.c_longlong,
                         C.c_longlong], C.c_int),
    "sw4g_write_sac": ([C.c_char_p, C.POINTER(GeoDesc), C.POINTER(UsgsStation), C.POINTER(SacEvent), _D,
                        C.c_longlong, C.c_longlong, C.c_int], C.c_int),
    "sw4g_corr_rows_scratch_len": ([C.c_int] * 4, C.c_longlong),
    "sw4g_pred_rows": ([C.c_int] * 8 + [_VP] * 9 + [C.c_double, C.c_double, _VP], C.c_int),
    "sw4g_corr_rows": ([C.c_int] * 8 + [_VP] * 16 + [C.c_double] * 3 + [_VP, C.c_longlong, _VP],
                       C.c_int),
    "sw4g_corr_rows_noalloc": ([C.c_int] * 8 + [_VP] * 16 + [C.c_double] * 3 + [_VP], C.c_int),
}


def build(force: bool = False) -> Path:
    import importlib
    return importlib.import_module(__name__ + ".builder").build(force=force)


def lib():
    """The loaded libsw4g.so.  Raises Sw4gError if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise Sw4gError(f"{LIB_PATH} is missing: build it with `python -m sw4lite_gb300.builder`"
                            " (there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = lib().sw4g_status_string(status).decode()
        raise Sw4gError(f"{what}: sw4g status {status} ({msg})")


def header_functions() -> list[str]:
    """Names of every function the C ABI headers declare (the drop-in header and
    the developer header)."""
    import re
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text() + DEV_HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(sw4g_[a-z0-9_]+)\s*\(", text)))


def stencil_coefficients():
    import numpy as np
    acof, ghcof, bope, sbop = np.zeros(384), np.zeros(6), np.zeros(48), np.zeros(5)
    check(lib().sw4g_stencil_coefficients(*[a.ctypes.data_as(_D) for a in (acof, ghcof, bope, sbop)]))
    return acof, ghcof, bope, sbop


FP64, MIXED = 0, 1
OK, BAD_ARGUMENT, CUDA_ERROR, NAN_DETECTED, NOT_SUPPORTED, TIMEOUT, IO_ERROR = range(7)


def grid_desc(nx, ny, nz, h, bc=(SUPERGRID,) * 4 + (FREE, SUPERGRID), zmin=0.0, sg_gp=20,
              sg_damping=0.02, sg_order=4, soa=1, precision=FP64) -> GridDesc:
    g = GridDesc()
    g.nx, g.ny, g.nz, g.h, g.zmin = nx, ny, nz, h, zmin
    for s in range(6):
        g.bc[s] = int(bc[s])
    g.sg_gp, g.sg_damping, g.sg_order, g.soa = sg_gp, sg_damping, sg_order, soa
    g.precision = precision
    return g


def source_desc(x, y, z, *, force=None, moment=None, freq=1.0, t0=0.0, kind=GAUSSIAN) -> SourceDesc:
    s = SourceDesc()
    s.x, s.y, s.z = x, y, z
    if moment is not None:
        s.moment = 1
        s.mxx, s.mxy, s.mxz, s.myy, s.myz, s.mzz = moment
    else:
        s.moment = 0
        s.fx, s.fy, s.fz = force if force is not None else (0.0, 0.0, 0.0)
    s.freq, s.t0, s.kind = freq, t0, kind
    return s


def _ptr(t) -> int:
    """Device (or host) address of a torch tensor / numpy array."""
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def _stream_ptr(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream or None
    return getattr(stream, "cuda_stream", stream) or None


class EW:
    """One Cartesian grid's time loop on the GPU (sw4g_ew_* in include/sw4g.h)."""

    def __init__(self, grid: GridDesc, stream=None, topo: TopoDesc = None, subdomain=None):
        """subdomain=(i0, i1, j0, j1): the object of that block of interior points of the
        global grid `grid` (sw4g_ew_create_subdomain); self.grid is then the local grid."""
        self._stream = _stream_ptr(stream)
        h = _VP()
        if subdomain is not None:
            i0, i1, j0, j1 = subdomain
            check(lib().sw4g_ew_create_subdomain(C.byref(grid), i0, i1, j0, j1, self._stream,
                                                 C.byref(h)), "sw4g_ew_create_subdomain")
            loc = GridDesc.from_buffer_copy(grid)
            loc.nx, loc.ny = i1 - i0 + 1, j1 - j0 + 1
            grid = loc
            self.subdomain = tuple(subdomain)
        elif topo is None:
            check(lib().sw4g_ew_create(C.byref(grid), self._stream, C.byref(h)), "sw4g_ew_create")
        else:
            check(lib().sw4g_ew_create_topo(C.byref(grid), C.byref(topo), self._stream,
                                            C.byref(h)), "sw4g_ew_create_topo")
        self.grid = grid
        self._h = h
        self.npts = lib().sw4g_ew_npts(h)
        self.shape = (grid.nz + 4, grid.ny + 4, grid.nx + 4)

    # --- subdomains of a decomposed grid ---
    def step_part(self, part):
        check(lib().sw4g_ew_step_part(self._h, part), "step_part")

    def halo_bytes(self, axis) -> int:
        return lib().sw4g_ew_halo_bytes(self._h, axis)

    def halo_pack(self, axis, side, buf):
        """Pack side (0 low, 1 high) along axis of the level to exchange into buf (a
        device tensor of halo_bytes(axis) bytes)."""
        with self._ordered(buf):
            check(lib().sw4g_ew_halo_pack(self._h, axis, side, _ptr(buf)), "halo_pack")

    def halo_unpack(self, axis, side, buf):
        with self._ordered(buf):
            check(lib().sw4g_ew_halo_unpack(self._h, axis, side, _ptr(buf)), "halo_unpack")

    @contextlib.contextmanager
    def _ordered(self, *arrays):
        """Stream order around a call that takes or fills device tensors: the
        library's stream waits for torch's current stream before the call, and
        torch's current stream waits for the library's stream after it (the rule
        torch applies between its own streams)."""
        if not any(getattr(a, "is_cuda", False) for a in arrays if a is not None):
            yield
            return
        import torch
        cur = torch.cuda.current_stream()
        own = torch.cuda.ExternalStream(self._stream) if self._stream else torch.cuda.default_stream()
        if own.cuda_stream == cur.cuda_stream:
            yield
            return
        own.wait_stream(cur)
        yield
        cur.wait_stream(own)

    def close(self):
        if getattr(self, "_h", None):
            lib().sw4g_ew_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_material(self, rho, mu, la):
        on_dev = int(hasattr(rho, "is_cuda") and rho.is_cuda)
        with self._ordered(rho, mu, la):
            check(lib().sw4g_ew_set_material(self._h, _ptr(rho), _ptr(mu), _ptr(la), on_dev),
                  "set_material")

    def add_source(self, src: SourceDesc):
        check(lib().sw4g_ew_add_source(self._h, C.byref(src)), "add_source")

    def add_grid_point_sources(self, ijk, amp, freq, t0, kind):
        import numpy as np
        ijk = np.ascontiguousarray(ijk, dtype=np.int32)
        amp = np.ascontiguousarray(amp, dtype=np.float64)
        freq = np.ascontiguousarray(freq, dtype=np.float64)
        t0 = np.ascontiguousarray(t0, dtype=np.float64)
        kind = np.ascontiguousarray(kind, dtype=np.int32)
        n = len(freq)
        check(lib().sw4g_ew_add_grid_point_sources(self._h, n, ijk.ctypes.data_as(_I),
                                                   amp.ctypes.data_as(_D), freq.ctypes.data_as(_D),
                                                   t0.ctypes.data_as(_D), kind.ctypes.data_as(_I)),
              "add_grid_point_sources")

    def grid_point_sources(self, grid=0):
        """(ijk, amp) of the discretised grid-point sources of grid 0 or 1."""
        import numpy as np
        n = C.c_int()
        check(lib().sw4g_ew_grid_point_sources(self._h, grid, 0, None, None, C.byref(n)),
              "grid_point_sources")
        ijk = np.zeros(3 * max(n.value, 1), dtype=np.int32)
        amp = np.zeros(3 * max(n.value, 1))
        check(lib().sw4g_ew_grid_point_sources(self._h, grid, n.value, ijk.ctypes.data_as(_I),
                                               amp.ctypes.data_as(_D), C.byref(n)),
              "grid_point_sources")
        return ijk[:3 * n.value].reshape(-1, 3), amp[:3 * n.value].reshape(-1, 3)

    def clear_sources(self):
        check(lib().sw4g_ew_clear_sources(self._h), "clear_sources")

    def num_grid_point_sources(self) -> int:
        return lib().sw4g_ew_num_grid_point_sources(self._h)

    def set_time_step(self, dt, t0=0.0):
        check(lib().sw4g_ew_set_time_step(self._h, dt, t0), "set_time_step")

    def set_graphs(self, on=True):
        """Replay the fused time loop (and the gradient's loops) as CUDA graphs."""
        check(lib().sw4g_ew_set_graphs(self._h, int(bool(on))), "set_graphs")

    def set_source_discretization(self, on_device=True):
        """Compute add_source's grid-point sources on the device (the whole batch,
        the same bits as the host path); Cartesian grid only."""
        check(lib().sw4g_ew_set_source_discretization(self._h, int(bool(on_device))),
              "set_source_discretization")

    def set_gradient_memory(self, max_bytes):
        """Device memory gradient() may add for segments kept from its forward run
        (their recompute is skipped): < 0 all free memory but a reserve, 0 none
        beyond the last segment."""
        check(lib().sw4g_ew_set_gradient_memory(self._h, int(max_bytes)), "set_gradient_memory")

    def write_checkpoint(self, path, cycle):
        """Both levels and the time in the reference's restart-file format."""
        check(lib().sw4g_ew_write_checkpoint(self._h, os.fsencode(path), int(cycle)), "write_checkpoint")

    def read_checkpoint(self, path):
        """Restart from a file in the reference's format; returns its cycle."""
        cyc = C.c_int()
        check(lib().sw4g_ew_read_checkpoint(self._h, os.fsencode(path), C.byref(cyc)), "read_checkpoint")
        return cyc.value

    def compute_time_step(self, cfl, tmax):
        dt = C.c_double()
        n = C.c_int()
        check(lib().sw4g_ew_compute_time_step(self._h, cfl, tmax, C.byref(dt), C.byref(n)),
              "compute_time_step")
        return dt.value, n.value

    @property
    def time(self) -> float:
        return lib().sw4g_ew_time(self._h)

    def set_fields(self, u, um):
        on_dev = int(hasattr(u, "is_cuda") and u.is_cuda)
        with self._ordered(u, um):
            check(lib().sw4g_ew_set_fields(self._h, _ptr(u), _ptr(um), on_dev), "set_fields")

    def get_fields(self, u, um):
        on_dev = int(hasattr(u, "is_cuda") and u.is_cuda)
        with self._ordered(u, um):
            check(lib().sw4g_ew_get_fields(self._h, _ptr(u), _ptr(um) if um is not None else None,
                                           on_dev), "get_fields")

    def field_ptr(self, which=0) -> int:
        return lib().sw4g_ew_field(self._h, which)

    def step(self, nsteps=1, mode=MODE_FUSED):
        st = lib().sw4g_ew_step(self._h, nsteps, mode)
        if st == NAN_DETECTED:
            r = self.nan_report()
            raise NonFiniteError(f"step: {r['count']} non-finite values on grid {r['grid']}, first "
                                 f"at component {r['c']} point {r['ijk']} (t = {r['t']})", r)
        check(st, "step")

    def set_nan_check(self, every=1):
        """Scan the new level for NaN/Inf every `every` steps (0: off)."""
        check(lib().sw4g_ew_set_nan_check(self._h, int(every)), "set_nan_check")

    def nan_report(self) -> dict:
        v = [C.c_int() for _ in range(5)]
        cnt, t = C.c_longlong(), C.c_double()
        check(lib().sw4g_ew_nan_report(self._h, *[C.byref(x) for x in v], C.byref(cnt), C.byref(t)),
              "nan_report")
        return {"grid": v[0].value, "c": v[1].value, "ijk": (v[2].value, v[3].value, v[4].value),
                "count": cnt.value, "t": t.value}

    def status(self) -> int:
        """Synchronises the object's stream; SW4G status of its bounded waits (0 or
        TIMEOUT)."""
        return lib().sw4g_ew_status(self._h)

    def enforce_bc(self, u):
        with self._ordered(u):
            check(lib().sw4g_ew_enforce_bc(self._h, _ptr(u)), "enforce_bc")

    def gradient(self, nsteps, checkpoint_every, observed, g_rho, g_mu, g_la):
        """Misfit of the receiver records against `observed` ((nsteps+1) x nvals) over
        nsteps steps from the current levels, and its gradient with respect to
        (rho, mu, lambda) written into g_rho, g_mu, g_la (npts each; host arrays or
        device tensors).  Returns the misfit."""
        J = C.c_double()
        od = int(hasattr(observed, "is_cuda") and observed.is_cuda)
        gd = int(hasattr(g_rho, "is_cuda") and g_rho.is_cuda)
        with self._ordered(observed, g_rho, g_mu, g_la):
            check(lib().sw4g_ew_gradient(self._h, nsteps, checkpoint_every, _ptr(observed), od,
                                         C.byref(J), _ptr(g_rho), _ptr(g_mu), _ptr(g_la), gd),
                  "gradient")
        return J.value

    @property
    def num_grids(self) -> int:
        return lib().sw4g_ew_num_grids(self._h)

    def grid_dims(self, grid=0):
        """(nx, ny, nz, npts) of grid 0 (Cartesian) or 1 (curvilinear)."""
        nx, ny, nz, n = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        check(lib().sw4g_ew_grid_dims(self._h, grid, C.byref(nx), C.byref(ny), C.byref(nz),
                                      C.byref(n)), "grid_dims")
        return nx.value, ny.value, nz.value, n.value

    def set_material_grid(self, grid, rho, mu, la):
        on_dev = int(hasattr(rho, "is_cuda") and rho.is_cuda)
        with self._ordered(rho, mu, la):
            check(lib().sw4g_ew_set_material_grid(self._h, grid, _ptr(rho), _ptr(mu), _ptr(la),
                                                  on_dev), "set_material_grid")

    def set_fields_grid(self, grid, u, um):
        on_dev = int(hasattr(u, "is_cuda") and u.is_cuda)
        with self._ordered(u, um):
            check(lib().sw4g_ew_set_fields_grid(self._h, grid, _ptr(u), _ptr(um), on_dev),
                  "set_fields_grid")

    def get_fields_grid(self, grid, u, um=None):
        on_dev = int(hasattr(u, "is_cuda") and u.is_cuda)
        with self._ordered(u, um):
            check(lib().sw4g_ew_get_fields_grid(self._h, grid, _ptr(u),
                                                _ptr(um) if um is not None else None, on_dev),
                  "get_fields_grid")

    def curvilinear_arrays(self, z=None, met=None, jac=None):
        ref = next(a for a in (z, met, jac) if a is not None)
        on_dev = int(hasattr(ref, "is_cuda") and ref.is_cuda)
        p = lambda a: _ptr(a) if a is not None else None
        with self._ordered(z, met, jac):
            check(lib().sw4g_ew_curvilinear_arrays(self._h, p(z), p(met), p(jac), on_dev),
                  "curvilinear_arrays")

    def set_receivers(self, ijk, modes, capacity, grids=None):
        """Receivers at 1-based grid points ijk (n x 3) with record modes (REC_*);
        room for `capacity` record rows (initial data + one per step).  grids: per
        receiver 0 (Cartesian, the default) or 1 (the curvilinear grid)."""
        import numpy as np
        ijk = np.ascontiguousarray(np.asarray(ijk, dtype=np.int32).reshape(-1, 3))
        modes = np.ascontiguousarray(np.asarray(modes, dtype=np.int32).reshape(-1))
        n = len(modes)
        if ijk.shape[0] != n:
            raise Sw4gError("set_receivers: one mode per receiver")
        if grids is None:
            check(lib().sw4g_ew_set_receivers(self._h, n, ijk.ctypes.data_as(_I),
                                              modes.ctypes.data_as(_I), capacity), "set_receivers")
            return
        grids = np.ascontiguousarray(np.asarray(grids, dtype=np.int32).reshape(-1))
        if len(grids) != n:
            raise Sw4gError("set_receivers: one grid per receiver")
        check(lib().sw4g_ew_set_receivers_grid(self._h, n, ijk.ctypes.data_as(_I),
                                               modes.ctypes.data_as(_I), grids.ctypes.data_as(_I),
                                               capacity), "set_receivers")

    def nearest_grid_point(self, x, y, z):
        """((i, j, k), grid) of the grid point nearest to (x, y, z) on this object's
        grids (grid 1: the curvilinear grid)."""
        ijk, g = (C.c_int * 3)(), C.c_int()
        check(lib().sw4g_ew_nearest_grid_point(self._h, x, y, z, ijk, C.byref(g)), "nearest_grid_point")
        return tuple(ijk), g.value

    def topography_z(self, x, y):
        """z of the topography surface at (x, y) (0 without topography)."""
        z = C.c_double()
        check(lib().sw4g_ew_topography_z(self._h, x, y, C.byref(z)), "topography_z")
        return z.value

    def record_shape(self):
        rows, nvals = C.c_int(), C.c_int()
        check(lib().sw4g_ew_record_shape(self._h, C.byref(rows), C.byref(nvals)), "record_shape")
        return rows.value, nvals.value

    def records(self, out=None):
        """The record array, rows x values: into `out` (host array or device tensor)
        or a new host array."""
        rows, nvals = self.record_shape()
        if out is None:
            import numpy as np
            out = np.zeros((rows, nvals))
        on_dev = int(hasattr(out, "is_cuda") and out.is_cuda)
        with self._ordered(out):
            check(lib().sw4g_ew_get_records(self._h, _ptr(out), on_dev), "get_records")
        return out

    def launches_per_step(self, mode=MODE_FUSED) -> int:
        return lib().sw4g_ew_launches_per_step(self._h, mode)

    def profile_kernels(self, nrep=5):
        ms = (C.c_double * 4)()
        check(lib().sw4g_ew_profile_kernels(self._h, nrep, ms), "profile_kernels")
        return dict(pred_stage=ms[0], corr_stage=ms[1], rows=ms[2], bc_force=ms[3])


def discretize_source_topo(g, topo, nzc, jac, src):
    """Grid-point sources of `src` on the two grids of g (bc[4] = INTERFACE) and the
    topography `topo` with nzc curvilinear planes and curvilinear Jacobian `jac`
    (host, full array).  Returns ((ijk, amp) of grid 0, (ijk, amp) of grid 1)."""
    import numpy as np
    cap = 4096
    jac = np.ascontiguousarray(jac, dtype=np.float64)
    a_ijk, b_ijk = np.zeros(3 * cap, dtype=np.int32), np.zeros(3 * cap, dtype=np.int32)
    a_amp, b_amp = np.zeros(3 * cap), np.zeros(3 * cap)
    na, nb = C.c_int(), C.c_int()
    check(lib().sw4g_discretize_source_topo(C.byref(g), C.byref(topo), nzc, jac.ctypes.data_as(_D),
                                            C.byref(src), cap, a_ijk.ctypes.data_as(_I),
                                            a_amp.ctypes.data_as(_D), C.byref(na),
                                            b_ijk.ctypes.data_as(_I), b_amp.ctypes.data_as(_D),
                                            C.byref(nb)), "discretize_source_topo")
    return ((a_ijk[:3 * na.value].reshape(-1, 3), a_amp[:3 * na.value].reshape(-1, 3)),
            (b_ijk[:3 * nb.value].reshape(-1, 3), b_amp[:3 * nb.value].reshape(-1, 3)))


def nearest_grid_point(g, x, y, z):
    """1-based (i, j, k) of the grid point nearest to (x, y, z) on grid g."""
    ijk = (C.c_int * 3)()
    check(lib().sw4g_nearest_grid_point(C.byref(g), x, y, z, ijk), "nearest_grid_point")
    return tuple(ijk)


def geo_desc(**kw) -> GeoDesc:
    """The reference's default geographic mapping (lon -118, lat 37, azimuth 0),
    with any field replaced by a keyword."""
    g = GeoDesc()
    check(lib().sw4g_geo_default(C.byref(g)), "geo_default")
    for k, v in kw.items():
        setattr(g, k, v)
    return g


def geographic_coord(geo, x, y):
    """(longitude, latitude) in degrees of grid point (x, y)."""
    lon, lat = C.c_double(), C.c_double()
    check(lib().sw4g_geographic_coord(C.byref(geo), x, y, C.byref(lon), C.byref(lat)), "geographic_coord")
    return lon.value, lat.value


def write_usgs(path, values, *, station, x, y, gp_x, gp_y, dt, mode=REC_DISPLACEMENT, xyz=True,
               t_shift=0.0, utc=(1970, 1, 1, 0, 0, 0, 0), geo=None):
    """Writes one receiver's records (rows x values, e.g. its columns of
    EW.records()) as a USGS text file, byte for byte as the reference does.
    Returns the status: 0, or NOT_SUPPORTED (header only) for curl, strains and
    gradient records in geographic components."""
    v = _rows(values)
    st = _station(station, x, y, gp_x, gp_y, dt, mode, xyz, t_shift, utc)
    geo = geo_desc() if geo is None else geo
    rc = lib().sw4g_write_usgs(str(path).encode(), C.byref(geo), C.byref(st), v.ctypes.data_as(_D),
                               v.shape[0], v.strides[0] // 8)
    if rc not in (0, NOT_SUPPORTED):
        check(rc, "write_usgs")
    return rc


def _station(station, x, y, gp_x, gp_y, dt, mode, xyz, t_shift, utc):
    st = UsgsStation()
    st.station = station.encode()
    st.x, st.y, st.gp_x, st.gp_y = x, y, gp_x, gp_y
    st.utc[:] = list(utc)
    st.mode, st.xyz, st.t_shift, st.dt = mode, int(bool(xyz)), t_shift, dt
    return st


def _rows(values):
    import numpy as np
    v = np.asarray(values, dtype=np.float64)
    if v.ndim == 1:
        v = v.reshape(-1, 1)
    if v.strides[1] != 8:
        v = np.ascontiguousarray(v)
    return v


def write_sac(prefix, values, *, station, x, y, dt, mode=REC_DISPLACEMENT, xyz=True, t_shift=0.0,
              utc=(1970, 1, 1, 0, 0, 0, 0), event=(0.0, 0.0, 0.0, 0.0), geo=None,
              flush_subnormals=False) -> None:
    """Writes one receiver's records as binary SAC files prefix + suffix (one per
    value of the mode), as the reference does.  event = (lat, lon, depth m, origin
    time offset s); flush_subnormals writes FP32 subnormal samples as signed zeros
    (a flush-to-zero build of the reference)."""
    v = _rows(values)
    st = _station(station, x, y, x, y, dt, mode, xyz, t_shift, utc)
    ev = SacEvent(*event)
    geo = geo_desc() if geo is None else geo
    check(lib().sw4g_write_sac(str(prefix).encode(), C.byref(geo), C.byref(st), C.byref(ev),
                               v.ctypes.data_as(_D), v.shape[0], v.strides[0] // 8, int(bool(flush_subnormals))),
          "write_sac")


def stage_kchunk(cols, nk, resident, min_planes=12) -> int:
    """Planes per k chunk of the automatic stage launch shape."""
    p = C.c_int()
    check(lib().sw4g_dev_stage_kchunk(cols, nk, resident, min_planes, C.byref(p)), "stage_kchunk")
    return p.value


def set_stage_chunks(chunks=0) -> None:
    """Tuning: k chunks of every stage kernel launch (0: the automatic choice)."""
    check(lib().sw4g_dev_set_stage_chunks(int(chunks)), "set_stage_chunks")


def set_adjoint_pipeline(on=True) -> None:
    """Comparison switch: the gradient's backward sweep recomputes the next segment
    beside the current one's adjoint steps (default) or after them."""
    check(lib().sw4g_dev_set_adjoint_pipeline(1 if on else 0), "set_adjoint_pipeline")


def set_rows_overlap(on=True) -> None:
    """Comparison switch: the one-sided rows beside each stage kernel on a second
    stream (default) or after it."""
    check(lib().sw4g_dev_set_rows_overlap(1 if on else 0), "set_rows_overlap")


def set_mixed_tma(on=True) -> None:
    """Comparison switch: FP32-mixed stages on the tensor-copy kernels (default) or
    on the synchronous kernels."""
    check(lib().sw4g_dev_set_mixed_tma(1 if on else 0), "set_mixed_tma")


def step_group(subs, neighbors, nsteps):
    """nsteps lockstep steps of subdomain EW objects with their halo exchanges;
    neighbors[s] = (x-low, x-high, y-low, y-high) indices into subs or -1."""
    n = len(subs)
    hs = (_VP * n)(*[e._h for e in subs])
    nb = (C.c_int * (4 * n))(*[int(x) for row in neighbors for x in row])
    check(lib().sw4g_ew_step_group(hs, n, nb, nsteps), "step_group")

