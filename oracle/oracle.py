"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product package never imports this module.

Two libraries:
  * liboracle.so      -- the plain-C restatement in oracle/sw4_oracle.c (always built
                         by ``make -C oracle``; builds on x86_64 and aarch64 alike);
  * _ref/libsw4ref.so -- the reference's own kernels compiled in place from the
                         reference sources (``make -C oracle ref``), present only
                         where the reference tree exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_D)


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_I)


def reference_src():
    """The reference's source directory as the oracle recipe resolves it
    (SW4_REFERENCE_SRC, else the recipe's default), or None where it is absent."""
    r = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref-src"], capture_output=True,
                       text=True)
    path = r.stdout.strip() if r.returncode == 0 else ""
    return path if path and os.path.isdir(path) else None


def build(ref: bool = False) -> None:
    """Build liboracle.so (and the reference kernels when asked and possible)."""
    target = "ref" if ref else "all"
    subprocess.run(["make", "-s", "-C", str(HERE), target], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            build()
        _lib = C.CDLL(str(path))
        _lib.sw4o_timefunc.restype = C.c_double
        _lib.sw4o_timefunc_tt.restype = C.c_double
    return _lib


def ref_available() -> bool:
    return (HERE / "_ref" / "libsw4ref.so").exists()


def ref():
    """The reference's own kernels, or None where they were not built."""
    global _ref
    if _ref is None and ref_available():
        _ref = C.CDLL(str(HERE / "_ref" / "libsw4ref.so"))
    return _ref


# --------------------------------------------------------------------------
# Thin wrappers.  `which` is "oracle" (the restatement) or "ref" (the reference).
# Arrays are flat float64 numpy arrays in the layout selected by `soa`.
# --------------------------------------------------------------------------
def stencil_coefficients(which="oracle"):
    acof = np.zeros(384)
    ghcof = np.zeros(6)
    bope = np.zeros(48)
    sbop = np.zeros(5)
    if which == "ref":
        ref().sw4ref_stencil_coefficients(_dp(acof), _dp(ghcof), _dp(bope), _dp(sbop))
    else:
        lib().sw4o_stencil_coefficients(_dp(acof), _dp(ghcof), _dp(bope), _dp(sbop))
    return acof, ghcof, bope, sbop


def rhs4sg(soa, bounds, nk, onesided, lu, u, mu, la, h, strx, stry, strz, which="oracle"):
    acof, ghcof, bope, _ = stencil_coefficients("oracle")
    os_arr, os_p = _ip(onesided)
    fn = ref().sw4ref_rhs4sg if which == "ref" else lib().sw4o_rhs4sg
    fn(C.c_int(soa), *[C.c_int(b) for b in bounds], C.c_int(nk), os_p, _dp(acof), _dp(bope),
       _dp(ghcof), _dp(lu), _dp(u), _dp(mu), _dp(la), C.c_double(h), _dp(strx), _dp(stry),
       _dp(strz))


def predfort(soa, bounds, up, u, um, lu, fo, rho, dt2, which="oracle"):
    fn = ref().sw4ref_predfort if which == "ref" else lib().sw4o_predfort
    fn(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(up), _dp(u), _dp(um), _dp(lu), _dp(fo),
       _dp(rho), C.c_double(dt2))


def corrfort(soa, bounds, up, lu, fo, rho, dt4, which="oracle"):
    fn = ref().sw4ref_corrfort if which == "ref" else lib().sw4o_corrfort
    fn(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(up), _dp(lu), _dp(fo), _dp(rho),
       C.c_double(dt4))


def dpdmtfort(bounds, up, u, um, u2, dt2i, which="oracle"):
    fn = ref().sw4ref_dpdmtfort if which == "ref" else lib().sw4o_dpdmtfort
    fn(*[C.c_int(b) for b in bounds], _dp(up), _dp(u), _dp(um), _dp(u2), C.c_double(dt2i))


def addsgd(order, soa, bounds, up, u, um, rho, dc, st, co, beta, which="oracle"):
    if which == "ref":
        fn = ref().sw4ref_addsgd6 if order == 6 else ref().sw4ref_addsgd4
    else:
        fn = lib().sw4o_addsgd6 if order == 6 else lib().sw4o_addsgd4
    fn(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(up), _dp(u), _dp(um), _dp(rho),
       _dp(dc[0]), _dp(dc[1]), _dp(dc[2]), _dp(st[0]), _dp(st[1]), _dp(st[2]), _dp(co[0]),
       _dp(co[1]), _dp(co[2]), C.c_double(beta))


def rhs4sgcurv(soa, bounds, onesided, lu, u, mu, la, met, jac, strx, stry, which="oracle"):
    """Curvilinear operator (rhs4sgcurv_rev.C / rhs4sgcurv.C)."""
    os_arr, os_p = _ip(onesided)
    if which == "ref":
        acof, ghcof, bope, _ = stencil_coefficients("ref")
        ref().sw4ref_rhs4sgcurv(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(u), _dp(mu),
                                _dp(la), _dp(met), _dp(jac), _dp(lu), os_p, _dp(acof), _dp(bope),
                                _dp(ghcof), _dp(strx), _dp(stry))
    else:
        lib().sw4o_rhs4sgcurv(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(u), _dp(mu),
                              _dp(la), _dp(met), _dp(jac), _dp(lu), os_p, _dp(strx), _dp(stry))


def metric(soa, bounds, h, z, met, jac, which="oracle"):
    """Numerical metric from z (EW::metric_rev); returns the status (0 ok)."""
    if which == "ref":
        ib, ie, jb, je, kb, ke = bounds
        shape = (ke - kb + 1, je - jb + 1, ie - ib + 1)
        k, j, i = np.meshgrid(np.arange(kb, ke + 1), np.arange(jb, je + 1), np.arange(ib, ie + 1),
                              indexing="ij")
        x = np.ascontiguousarray(((i - 1) * h).reshape(-1), dtype=np.float64)
        y = np.ascontiguousarray(((j - 1) * h).reshape(-1), dtype=np.float64)
        assert x.size == int(np.prod(shape))
        ref().sw4ref_metric.restype = C.c_int
        return ref().sw4ref_metric(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(x), _dp(y),
                                   _dp(z), _dp(met), _dp(jac))
    lib().sw4o_metric.restype = C.c_int
    return lib().sw4o_metric(C.c_int(soa), *[C.c_int(b) for b in bounds], C.c_double(h), _dp(z),
                             _dp(met), _dp(jac))


def gaussian_hill_z(bounds, nz, h, zmax, amp, xc, yc, lx, ly, zeta_break=0.95, order=4):
    """z of the curvilinear grid over a Gaussian hill (EW::grid_mapping)."""
    ib, ie, jb, je, kb, ke = bounds
    z = np.zeros((ie - ib + 1) * (je - jb + 1) * (ke - kb + 1))
    lib().sw4o_gaussian_hill_z(*[C.c_int(b) for b in bounds], C.c_int(nz), C.c_double(h),
                               C.c_double(zmax), C.c_double(zeta_break), C.c_int(order),
                               C.c_double(amp), C.c_double(xc), C.c_double(yc), C.c_double(lx),
                               C.c_double(ly), _dp(z))
    return z


def freesurfcurvisg(soa, bounds, nz, side, u, mu, la, met, sbop, forcing, strx, stry,
                    which="oracle"):
    ib, ie, jb, je, kb, ke = bounds
    if forcing is None and which == "ref":
        forcing = np.zeros(3 * (ie - ib + 1) * (je - jb + 1))
    fn = ref().sw4ref_freesurfcurvisg if which == "ref" else lib().sw4o_freesurfcurvisg
    fn(C.c_int(soa), *[C.c_int(b) for b in bounds], C.c_int(nz), C.c_int(side), _dp(u), _dp(mu),
       _dp(la), _dp(met), _dp(sbop), _dp(forcing) if forcing is not None else _D(), _dp(strx),
       _dp(stry))


def addsgd4c(soa, bounds, up, u, um, rho, dcx, dcy, strx, stry, jac, cox, coy, beta,
             which="oracle", order=4):
    if order == 6:
        fn = ref().sw4ref_addsgd6c if which == "ref" else lib().sw4o_addsgd6c
    else:
        fn = ref().sw4ref_addsgd4c if which == "ref" else lib().sw4o_addsgd4c
    fn(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(up), _dp(u), _dp(um), _dp(rho), _dp(dcx),
       _dp(dcy), _dp(strx), _dp(stry), _dp(jac), _dp(cox), _dp(coy), C.c_double(beta))


def sym3_min_eig(a6):
    a = np.ascontiguousarray(a6, dtype=np.float64)
    lib().sw4o_sym3_min_eig.restype = C.c_double
    return lib().sw4o_sym3_min_eig(_dp(a))


def curv_dt(soa, bounds, rho, mu, la, met, jac, cfl):
    lib().sw4o_curv_dt.restype = C.c_double
    return lib().sw4o_curv_dt(C.c_int(soa), *[C.c_int(b) for b in bounds], _dp(rho), _dp(mu),
                              _dp(la), _dp(met), _dp(jac), C.c_double(cfl))


def boundary_windows(bounds, nxyz, bccnd):
    wind = np.zeros(36, dtype=np.int32)
    npts = np.zeros(6, dtype=np.int32)
    bc, bcp = _ip(bccnd)
    lib().sw4o_boundary_windows(*[C.c_int(b) for b in bounds], *[C.c_int(n) for n in nxyz], bcp,
                                wind.ctypes.data_as(_I), npts.ctypes.data_as(_I))
    return wind, npts


def bcfortsg(soa, bounds, wind, nxyz, u, h, bccnd, sbop, mu, la, bforce, strx, stry,
             which="oracle"):
    w, wp = _ip(wind)
    bc, bcp = _ip(bccnd)
    bf = [None if b is None else np.ascontiguousarray(b, dtype=np.float64) for b in bforce]
    if which == "ref":
        # the reference kernel dereferences every forcing array it is given for
        # sides with bccnd 1/2/0; hand it zero arrays of the window size where None
        bf = [np.zeros(3 * max(1, _wsize(w, s))) if b is None else b for s, b in enumerate(bf)]
        ref().sw4ref_bcfortsg(C.c_int(soa), *[C.c_int(b) for b in bounds], wp,
                              *[C.c_int(n) for n in nxyz], _dp(u), C.c_double(h), bcp, _dp(sbop),
                              _dp(mu), _dp(la), C.c_double(0.0), *[_dp(b) for b in bf],
                              _dp(strx), _dp(stry))
    else:
        arr = (_D * 6)(*[(_dp(b) if b is not None else _D()) for b in bf])
        lib().sw4o_bcfortsg(C.c_int(soa), *[C.c_int(b) for b in bounds], wp,
                            *[C.c_int(n) for n in nxyz], _dp(u), C.c_double(h), bcp, _dp(sbop),
                            _dp(mu), _dp(la), arr, _dp(strx), _dp(stry))


def _wsize(w, s):
    ww = w[6 * s:6 * s + 6]
    return max(0, (ww[1] - ww[0] + 1) * (ww[3] - ww[2] + 1) * (ww[5] - ww[4] + 1))


def supergrid_profile(first, last, h, xmin, left, right, x0, x1, width):
    n = last - first + 1
    dc, st, co = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().sw4o_supergrid_profile(C.c_int(first), C.c_int(last), C.c_double(h), C.c_double(xmin),
                                 C.c_int(int(left)), C.c_int(int(right)), C.c_double(x0),
                                 C.c_double(x1), C.c_double(width), _dp(dc), _dp(st), _dp(co))
    return dc, st, co


def timefunc(kind, freq, t, tt=False):
    f = lib().sw4o_timefunc_tt if tt else lib().sw4o_timefunc
    return f(C.c_int(kind), C.c_double(freq), C.c_double(t))


class Problem(C.Structure):
    """Mirror of sw4o_problem (oracle/sw4_oracle.h)."""
    _fields_ = [("ib", C.c_int), ("ie", C.c_int), ("jb", C.c_int), ("je", C.c_int),
                ("kb", C.c_int), ("ke", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("nz", C.c_int), ("h", C.c_double), ("dt", C.c_double),
                ("onesided", C.c_int * 6), ("bccnd", C.c_int * 6), ("wind", C.c_int * 36),
                ("sg_beta", C.c_double), ("sg_order", C.c_int),
                ("mu", _D), ("la", _D), ("rho", _D),
                ("strx", _D), ("stry", _D), ("strz", _D), ("dcx", _D), ("dcy", _D),
                ("dcz", _D), ("cox", _D), ("coy", _D), ("coz", _D),
                ("nsrc", C.c_int), ("src_ijk", _I), ("src_amp", _D), ("src_freq", _D),
                ("src_t0", _D), ("src_kind", _I)]


def step(problem: Problem, soa, t, up, u, um, lu, f, uacc, which="oracle"):
    fn = ref().sw4ref_step if which == "ref" else lib().sw4o_step
    fn(C.byref(problem), C.c_int(soa), C.c_double(t), _dp(up), _dp(u), _dp(um), _dp(lu), _dp(f),
       _dp(uacc))


class Curv(C.Structure):
    """Mirror of sw4o_curv (oracle/sw4_oracle.h)."""
    _fields_ = [("ib", C.c_int), ("ie", C.c_int), ("jb", C.c_int), ("je", C.c_int),
                ("kb", C.c_int), ("ke", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("nz", C.c_int), ("h", C.c_double), ("bccnd", C.c_int * 6),
                ("wind", C.c_int * 36), ("rho", _D), ("mu", _D), ("la", _D), ("met", _D),
                ("jac", _D), ("strx", _D), ("stry", _D), ("dcx", _D), ("dcy", _D), ("cox", _D),
                ("coy", _D), ("nsrc", C.c_int), ("src_ijk", _I), ("src_amp", _D),
                ("src_freq", _D), ("src_t0", _D), ("src_kind", _I)]


def step_topo(problem: Problem, curv: Curv, t, cart_arrays, curv_arrays, which="oracle"):
    """One two-grid step; *_arrays = (up, u, um, lu, f, uacc) of each grid."""
    fn = ref().sw4ref_step_topo if which == "ref" else lib().sw4o_step_topo
    fn(C.byref(problem), C.byref(curv), C.c_double(t), *[_dp(a) for a in cart_arrays],
       *[_dp(a) for a in curv_arrays])


def step_pred(problem: Problem, t, up, u, um, lu, f, uacc, pred):
    """sw4o_step that also returns the predicted level in pred."""
    lib().sw4o_step_pred(C.byref(problem), C.c_int(1), C.c_double(t), _dp(up), _dp(u), _dp(um),
                         _dp(lu), _dp(f), _dp(uacc), _dp(pred))


def apply_lt(bounds, nz, y, mu, la, h, strx, stry, strz):
    """L^T y = W L (W^-1 y) on the interior (zero ghosts), W = 1/(sx sy sz)."""
    lt = np.zeros_like(y)
    lib().sw4o_apply_lt(*[C.c_int(b) for b in bounds], C.c_int(nz), _dp(y), _dp(mu), _dp(la),
                        C.c_double(h), _dp(strx), _dp(stry), _dp(strz), _dp(lt))
    return lt


def apply_lt_fs(bounds, nxyz, onesided, y, mu, la, h, strx, stry, strz):
    """L^T y = D L (D^-1 y) on the interior with free-surface z sides, D = H W (H the
    SBP norm weights next to those sides)."""
    lt = np.zeros_like(y)
    os_arr, os_p = _ip(onesided)
    lib().sw4o_apply_lt_fs(*[C.c_int(b) for b in bounds], *[C.c_int(n) for n in nxyz], os_p, _dp(y),
                           _dp(mu), _dp(la), C.c_double(h), _dp(strx), _dp(stry), _dp(strz), _dp(lt))
    return lt


def sg_adjoint(bounds, y, rho, dc, st, co):
    """SG^T (y / rho) on the interior."""
    z = np.zeros_like(y)
    lib().sw4o_sg_adjoint(*[C.c_int(b) for b in bounds], _dp(y), _dp(rho), *[_dp(a) for a in dc],
                          *[_dp(a) for a in st], *[_dp(a) for a in co], _dp(z))
    return z


def coef_gradient(bounds, v, w, h, st, gmu, gla):
    """gmu, gla += gradient of v . L(w) with respect to mu, lambda."""
    lib().sw4o_coef_gradient(*[C.c_int(b) for b in bounds], _dp(v), _dp(w), C.c_double(h),
                             *[_dp(a) for a in st], _dp(gmu), _dp(gla))


def coef_gradient_fs(bounds, nz, onesided, v, w, h, st, gmu, gla):
    """gmu, gla += gradient of v . L(w) with free-surface z sides (one-sided rows and
    the ghost plane from the traction condition)."""
    os_arr, os_p = _ip(onesided)
    lib().sw4o_coef_gradient_fs(*[C.c_int(b) for b in bounds], C.c_int(nz), os_p, _dp(v), _dp(w),
                                C.c_double(h), *[_dp(a) for a in st], _dp(gmu), _dp(gla))


def sg6_adjoint(bounds, y, rho, dc, st, co):
    """SG6^T (y / rho) on the interior (sixth-order damping)."""
    z = np.zeros_like(y)
    lib().sw4o_sg6_adjoint(*[C.c_int(b) for b in bounds], _dp(y), _dp(rho), *[_dp(a) for a in dc],
                           *[_dp(a) for a in st], *[_dp(a) for a in co], _dp(z))
    return z


def sg6_rho_gradient(bounds, a1, d, rho, dc, st, co, beta, grho):
    """grho += -beta * d/drho [(R a1) . SG6(d)] at fixed R (sixth-order damping)."""
    lib().sw4o_sg6_rho_gradient(*[C.c_int(b) for b in bounds], _dp(a1), _dp(d), _dp(rho),
                                *[_dp(a) for a in dc], *[_dp(a) for a in st], *[_dp(a) for a in co],
                                C.c_double(beta), _dp(grho))


def sg_rho_gradient(bounds, a1, d, rho, dc, st, co, beta, grho):
    """grho += -beta * d/drho [(R a1) . SG(d)] at fixed R."""
    lib().sw4o_sg_rho_gradient(*[C.c_int(b) for b in bounds], _dp(a1), _dp(d), _dp(rho),
                               *[_dp(a) for a in dc], *[_dp(a) for a in st], *[_dp(a) for a in co],
                               C.c_double(beta), _dp(grho))


def nearest_grid_point(h, zmin, x, y, z):
    """EW::computeNearestGridPoint (src/EW.C:5149-5177) for one Cartesian grid:
    1-based (i, j, k) of the nearest point, a half-way point going to the lower index."""
    i = int(np.floor(x / h)) + 1
    if x - ((i - 0.5) * h) > 0.0:
        i += 1
    j = int(np.floor(y / h)) + 1
    if y - ((j - 0.5) * h) > 0.0:
        j += 1
    k = int(np.floor((z - zmin) / h)) + 1
    if z - (zmin + (k - 0.5) * h) > 0.0:
        k += 1
    return i, j, k


REC_VALUES = {0: 3, 1: 1, 2: 3, 3: 6, 4: 3, 5: 9}


def record(mode, ijk, u, um, dt, h, dims, initial=False):
    """Values one receiver records (EW::extractRecordData, src/EW.C:5854-6072,
    Cartesian formulas).  u, um: SoA 3-component fields over the array of an
    nx x ny x nz grid (index -1 .. n+2 per axis); dims = (nx, ny, nz).  Velocity
    is not recorded for the initial data (src/EW.C:2489-2491): zeros there."""
    nx, ny, nz = dims
    U = np.asarray(u).reshape(3, nz + 4, ny + 4, nx + 4)
    Um = np.asarray(um).reshape(3, nz + 4, ny + 4, nx + 4)
    i, j, k = ijk

    def at(A, c, ii, jj, kk):
        return A[c, kk + 1, jj + 1, ii + 1]

    if mode == 0:
        return [at(U, c, i, j, k) for c in range(3)]
    if mode == 4:
        if initial:
            return [0.0, 0.0, 0.0]
        return [(at(U, c, i, j, k) - at(Um, c, i, j, k)) / (2 * dt) for c in range(3)]
    f = 1.0 / (2 * h)
    if mode == 1:
        return [(at(U, 0, i + 1, j, k) - at(U, 0, i - 1, j, k) + at(U, 1, i, j + 1, k) -
                 at(U, 1, i, j - 1, k) + at(U, 2, i, j, k + 1) - at(U, 2, i, j, k - 1)) * f]
    g = [[(at(U, c, i + 1, j, k) - at(U, c, i - 1, j, k)) * f,
          (at(U, c, i, j + 1, k) - at(U, c, i, j - 1, k)) * f,
          (at(U, c, i, j, k + 1) - at(U, c, i, j, k - 1)) * f] for c in range(3)]
    if mode == 2:
        return [g[2][1] - g[1][2], g[0][2] - g[2][0], g[1][0] - g[0][1]]
    if mode == 3:
        return [g[0][0], g[1][1], g[2][2], 0.5 * (g[1][0] + g[0][1]), 0.5 * (g[2][0] + g[0][2]),
                0.5 * (g[1][2] + g[2][1])]
    return [g[c][a] for c in range(3) for a in range(3)]


def exact_point_source(bounds, h, zmin, rho, cp, cs, x0, y0, z0, t, *, force=None, moment=None,
                       kind=1, freq=1.0, t0=0.0):
    """Analytic whole-space displacement (SoA, over the array `bounds`) of one force
    or moment-tensor point source; the field of the reference's point-source test
    (EW::get_exact_point_source, src/EW.C:3899-4524)."""
    ib, ie, jb, je, kb, ke = bounds
    npts = (ie - ib + 1) * (je - jb + 1) * (ke - kb + 1)
    u = np.zeros(3 * npts)
    f = np.ascontiguousarray(force if force is not None else np.zeros(3), dtype=np.float64)
    m = np.ascontiguousarray(moment if moment is not None else np.zeros(6), dtype=np.float64)
    lib().sw4o_exact_point_source(ib, ie, jb, je, kb, ke, C.c_double(h), C.c_double(zmin),
                                  C.c_double(rho), C.c_double(cp), C.c_double(cs), C.c_double(x0),
                                  C.c_double(y0), C.c_double(z0), int(moment is not None), _dp(f),
                                  _dp(m), kind, C.c_double(freq), C.c_double(t0), C.c_double(t),
                                  _dp(u))
    return u


def solerr3(bounds, h, zmin, uex, u, x0, y0, z0, radius, region):
    """(Linf, L2, max uex) of u - uex over region = (imin, imax, jmin, jmax, kmin, kmax)
    outside the ball of `radius` around (x0, y0, z0) (EW::solerr3fort,
    src/ew-cfromfort.C:144; EW::normOfDifference, src/EW.C:4537)."""
    ib, ie, jb, je, kb, ke = bounds
    li, l2, xli = C.c_double(), C.c_double(), C.c_double()
    lib().sw4o_solerr3(ib, ie, jb, je, kb, ke, C.c_double(h), C.c_double(zmin), _dp(uex), _dp(u),
                       C.c_double(x0), C.c_double(y0), C.c_double(z0), C.c_double(radius),
                       *[int(r) for r in region], C.byref(li), C.byref(l2), C.byref(xli))
    return li.value, l2.value, xli.value


def set_threads(n: int) -> None:
    os.environ["OMP_NUM_THREADS"] = str(n)


# --------------------------------------------------------------------------
# Source discretisation and a whole Cartesian problem, built from plain values
# (no product types), for the parity tests and the CPU baseline.
# --------------------------------------------------------------------------
def source_weights(which, a):
    """The 6 weights of a source at fractional position a: which 0 delta, 1 delta',
    2 and 3 their five-point free-surface variants (sw4_oracle_src.c)."""
    w = np.zeros(6)
    lib().sw4o_source_weights(C.c_int(which), C.c_double(a), _dp(w))
    return w


def discretize_source(nx, ny, nz, h, zmin, top_onesided, bot_onesided, x, y, z, *, force=None,
                      moment=None, cap=512):
    """Grid-point sources of one point force or moment tensor (m: xx xy xz yy yz zz) on
    a Cartesian grid: (ijk int32 [3n], amp [3n]) in the reference's emission order."""
    ijk = np.zeros(3 * cap, dtype=np.int32)
    amp = np.zeros(3 * cap)
    f = np.asarray(force if force is not None else (0.0, 0.0, 0.0), dtype=np.float64)
    m = np.asarray(moment if moment is not None else (0.0,) * 6, dtype=np.float64)
    n = lib().sw4o_discretize_source(
        C.c_int(nx), C.c_int(ny), C.c_int(nz), C.c_double(h), C.c_double(zmin),
        C.c_int(int(top_onesided)), C.c_int(int(bot_onesided)), C.c_double(x), C.c_double(y),
        C.c_double(z), C.c_int(int(moment is not None)), _dp(f), _dp(m), C.c_int(cap),
        ijk.ctypes.data_as(_I), _dp(amp))
    if n < 0:
        raise ValueError("more grid-point sources than cap")
    return ijk[:3 * n].copy(), amp[:3 * n].copy()


class PointSource:
    """A point force (force=(fx, fy, fz)) or moment tensor (moment=(xx, xy, xz, yy, yz,
    zz)) at (x, y, z) with time function `kind` (0 Gaussian, 1 C6SmoothBump, 3
    VerySmoothBump), frequency and offset."""

    def __init__(self, x, y, z, *, force=None, moment=None, freq=1.0, t0=0.0, kind=0):
        self.x, self.y, self.z = x, y, z
        self.force, self.moment = force, moment
        self.freq, self.t0, self.kind = freq, t0, kind


class CartProblem:
    """sw4o_problem of one Cartesian grid: nx, ny, nz interior points with 2 ghost
    points per side, bc[6] (0 free surface, 1 Dirichlet, 2 supergrid, 3 periodic),
    supergrid width sg_gp points with damping sg_damping and order sg_order, the
    material over the whole array, dt, and PointSource sources discretised here."""

    def __init__(self, nx, ny, nz, h, bc, rho, mu, la, dt, sources=(), *, zmin=0.0, sg_gp=20,
                 sg_damping=0.02, sg_order=4):
        self.nx, self.ny, self.nz, self.h, self.zmin = nx, ny, nz, h, zmin
        self.bounds = (-1, nx + 2, -1, ny + 2, -1, nz + 2)
        self.keep = [rho, mu, la]
        bc = list(bc)
        used = 2 in bc
        prof = []
        for ax, n, b0, b1 in [(0, nx, bc[0], bc[1]), (1, ny, bc[2], bc[3]), (2, nz, bc[4], bc[5])]:
            if used:
                x0 = zmin if ax == 2 else 0.0
                p = supergrid_profile(-1, n + 2, h, x0, b0 == 2, b1 == 2, 0.0, x0 + (n - 1) * h,
                                      sg_gp * h)
            else:
                p = (np.zeros(n + 4), np.ones(n + 4), np.ones(n + 4))
            prof.append(p)
        self.prof = prof
        self.keep += [a for p in prof for a in p]
        wind, _ = boundary_windows(self.bounds, (nx, ny, nz), bc)
        P = Problem()
        P.ib, P.ie, P.jb, P.je, P.kb, P.ke = self.bounds
        P.nx, P.ny, P.nz = nx, ny, nz
        P.h, P.dt = h, dt
        for s in range(6):
            P.bccnd[s] = bc[s]
        P.onesided[4] = int(bc[4] == 0)
        P.onesided[5] = int(bc[5] == 0)
        for q in range(36):
            P.wind[q] = int(wind[q])
        P.sg_beta = sg_damping if used else 0.0
        P.sg_order = sg_order
        P.rho, P.mu, P.la = _dp(rho), _dp(mu), _dp(la)
        P.dcx, P.strx, P.cox = [_dp(a) for a in prof[0]]
        P.dcy, P.stry, P.coy = [_dp(a) for a in prof[1]]
        P.dcz, P.strz, P.coz = [_dp(a) for a in prof[2]]
        self.P = P
        ijk, amp, freq, t0, kind = [], [], [], [], []
        for src in sources:
            a, b = discretize_source(nx, ny, nz, h, zmin, bc[4] == 0, bc[5] == 0, src.x, src.y, src.z,
                                     force=src.force, moment=src.moment)
            n = len(a) // 3
            ijk.append(a)
            amp.append(b)
            freq += [src.freq] * n
            t0 += [src.t0] * n
            kind += [src.kind] * n
        self.set_grid_point_sources(np.concatenate(ijk) if ijk else np.zeros(0),
                                    np.concatenate(amp) if amp else np.zeros(0), freq, t0, kind)
        self.npts = (nx + 4) * (ny + 4) * (nz + 4)

    def set_grid_point_sources(self, ijk, amp, freq, t0, kind):
        """Grid-point sources (flat ijk and amp, 3 per source) of this problem."""
        self.src = (np.ascontiguousarray(ijk, dtype=np.int32).reshape(-1),
                    np.ascontiguousarray(amp, dtype=np.float64).reshape(-1),
                    np.asarray(freq, dtype=np.float64), np.asarray(t0, dtype=np.float64),
                    np.asarray(kind, dtype=np.int32))
        self.keep += list(self.src)
        P = self.P
        P.nsrc = len(self.src[2])
        P.src_ijk = self.src[0].ctypes.data_as(_I)
        P.src_amp = self.src[1].ctypes.data_as(_D)
        P.src_freq = self.src[2].ctypes.data_as(_D)
        P.src_t0 = self.src[3].ctypes.data_as(_D)
        P.src_kind = self.src[4].ctypes.data_as(_I)

    def run(self, u, um, t0, nsteps, which="oracle", receivers=None):
        """nsteps steps from (u, um) (which: "oracle" the restatement, "ref" the
        reference's kernels); with receivers [(ijk, mode), ...] also returns the record
        rows (initial data, then one row per step)."""
        n3 = 3 * self.npts
        u, um = u.copy(), um.copy()
        up, lu, f, uacc = (np.zeros(n3) for _ in range(4))
        t = t0
        dims = (self.nx, self.ny, self.nz)

        def row(a, b, initial):
            return np.concatenate([record(m, ijk, a, b, self.P.dt, self.h, dims, initial)
                                   for ijk, m in receivers])

        rows = [row(u, um, True)] if receivers else []
        for _ in range(nsteps):
            step(self.P, 1, t, up, u, um, lu, f, uacc, which=which)
            if receivers:
                rows.append(row(up, um, False))
            um, u, up = u, up, um
            t += self.P.dt
        if receivers:
            return u, um, np.array(rows)
        return u, um

