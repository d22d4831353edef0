"""ctypes wrapper of the FP64 CPU oracle (oracle/_build/libswm_oracle.so).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference Fortran
shallow-water hot path (vvshashkin/cubedsphere_sbp_swm) in C++; see
swm_oracle.cpp for the file:line each routine follows.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
and only as the checker or as the timed CPU baseline.

Arrays use the reference layout: shape (6, N+1, N+1) = (panel, j, i), FP64,
C-contiguous (i fastest).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libswm_oracle.so")
_lib = None

_D = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (portable flags, a few seconds)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(
            os.path.getmtime(os.path.join(_HERE, f))
            for f in ("swm_oracle.cpp", "swm_oracle_c.cpp", "swm_oracle.h",
                      "swm_oracle_common.h", "Makefile",
                      "../cubedsphere_sbp_swm_gb300/csrc/swm_narrow_tables.h")
        )
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, _D]
        L.orc_destroy.argtypes = [vp]
        L.orc_npts.argtypes = [vp]
        L.orc_npts.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        L.orc_geometry.argtypes = [vp] + [_D] * 8
        L.orc_bases.argtypes = [vp] + [_D] * 4
        L.orc_sync_weights.argtypes = [vp] + [_D] * 4
        for name, n in (("orc_co2contra", 4), ("orc_contra2co", 4), ("orc_grad", 3),
                        ("orc_div", 3), ("orc_curl", 3), ("orc_sync_scalar", 1),
                        ("orc_sync_vector_cov", 2), ("orc_coriolis", 6),
                        ("orc_apply", 7), ("orc_diagnostics", 5)):
            getattr(L, name).argtypes = [vp] + [_D] * n
        L.orc_rk4.argtypes = [vp, _D, _D, _D, _D, ctypes.c_double, ctypes.c_int]
        L.orc_l2norm.argtypes = [vp, _D]
        L.orc_l2norm.restype = ctypes.c_double
        L.orc_mass.argtypes = [vp, _D]
        L.orc_mass.restype = ctypes.c_double
        for name in ("orc_golden_div", "orc_golden_grad", "orc_golden_curl"):
            getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_int, _D]
            getattr(L, name).restype = ctypes.c_int
        for name in ("orc_golden_co2contra", "orc_golden_contra2co", "orc_golden_coriolis",
                     "orc_golden_ke"):
            getattr(L, name).argtypes = [ctypes.c_int, _D]
            getattr(L, name).restype = ctypes.c_int
        L.orc_golden_quadrature.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_golden_quadrature.restype = ctypes.c_double
        L.orc_golden_rk4_iomega.restype = ctypes.c_double
        L.orc_vector_test_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
        L.orc_vector_test_field.restype = ctypes.c_int
        L.orc_scalar_test_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, _D]
        L.orc_scalar_test_field.restype = ctypes.c_int
        L.orc_latlon_scalar.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
        L.orc_latlon_scalar.restype = ctypes.c_int
        L.orc_latlon_vector.argtypes = [vp] + [ctypes.c_int] * 4 + [_D] * 4
        L.orc_latlon_vector.restype = ctypes.c_int
        L.orc_golden_regrid.argtypes = [ctypes.c_int, ctypes.c_int, _D]
        L.orc_golden_regrid.restype = ctypes.c_int
        for name, args in (("orc_laplace", [vp, ctypes.c_int, _D, _D]),
                           ("orc_hordiff_scalar", [vp, ctypes.c_int, ctypes.c_double, _D, _D]),
                           ("orc_hordiff_vec_xyz", [vp, ctypes.c_int, ctypes.c_double] + [_D] * 4),
                           ("orc_diffusion_apply", [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                    ctypes.c_double] + [_D] * 6),
                           ("orc_diffusion_step", [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                   ctypes.c_double, _D, _D, _D, ctypes.c_double])):
            getattr(L, name).argtypes = args
            getattr(L, name).restype = ctypes.c_int
        # C grid (swm_oracle_c.cpp)
        L.orcc_create.restype = vp
        L.orcc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_double, _D]
        L.orcc_destroy.argtypes = [vp]
        L.orcc_size.argtypes = [vp, ctypes.c_int]
        L.orcc_size.restype = ctypes.c_int
        L.orcc_points.argtypes = [vp, ctypes.c_int] + [_D] * 3
        L.orcc_metric.argtypes = [vp, ctypes.c_int] + [_D] * 5
        L.orcc_bases.argtypes = [vp, ctypes.c_int] + [_D] * 4
        for name, n in (("orcc_co2contra", 4), ("orcc_massflux", 5), ("orcc_ke", 5),
                        ("orcc_grad", 3), ("orcc_div", 3), ("orcc_curl", 3),
                        ("orcc_coriolis", 6), ("orcc_apply", 7)):
            getattr(L, name).argtypes = [vp] + [_D] * n
        L.orcc_rk4.argtypes = [vp, _D, _D, _D, _D, ctypes.c_double, ctypes.c_int]
        L.orcc_grad_perp.argtypes = [vp, _D, _D, _D]
        L.orcc_ecs_o_halo.argtypes = [vp, _D, ctypes.c_int, _D]
        L.orcc_ecs_o_halo.restype = ctypes.c_int
        L.orcc_grad_a2_ecs.argtypes = [vp, _D, _D, _D]
        L.orcc_ecs_a_vec_halo.argtypes = [vp, _D, _D, ctypes.c_int, _D, _D]
        L.orcc_ecs_a_vec_halo.restype = ctypes.c_int
        L.orcc_div_a2_ecs.argtypes = [vp, _D, _D, _D]
        L.orcc_grad_c2_ecs.argtypes = [vp, _D, _D, _D]
        L.orcc_ecs_xy_halo.argtypes = [vp, _D, ctypes.c_int, _D]
        L.orcc_ecs_xy_halo.restype = ctypes.c_int
        L.orcc_laplace_ch.argtypes = [vp, ctypes.c_int, _D, _D]
        L.orcc_laplace_ch.restype = ctypes.c_int
        L.orcc_contra2co.argtypes = [vp, _D, _D, _D, _D]
        L.orcc_hordiff.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double] + [_D] * 6
        L.orcc_model_step.argtypes = [vp, _D, _D, _D, _D, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double]
        for name in ("orcc_mass", "orcc_l2norm"):
            getattr(L, name).argtypes = [vp, ctypes.c_int, _D]
            getattr(L, name).restype = ctypes.c_double
        L.orcc_vector_test_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
        L.orcc_vector_test_field.restype = ctypes.c_int
        L.orcc_scalar_test_field.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D]
        L.orcc_scalar_test_field.restype = ctypes.c_int
        L.orcc_golden.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D]
        L.orcc_golden.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


class OracleDomain:
    """FP64 oracle domain: geometry + SBP operator of one configuration."""

    def __init__(self, N, sbp_order=42, radius=6.371e6, grav=9.80616,
                 omega=7.292e-5, axis=(0.0, 0.0, 1.0)):
        L = lib()
        ax = np.asarray(axis, dtype=np.float64)
        self._h = L.orc_create(int(N), int(sbp_order), float(radius), float(grav),
                               float(omega), _p(ax))
        if not self._h:
            raise ValueError(f"oracle: unsupported N={N} / sbp_order={sbp_order}")
        self.N, self.n, self.sbp_order = int(N), int(N) + 1, int(sbp_order)
        self.shape = (6, self.n, self.n)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def zeros(self):
        return np.zeros(self.shape)

    def geometry(self):
        out = {k: self.zeros() for k in ("J", "Qi1", "Qi2", "Qi3", "f", "rx", "ry", "rz")}
        lib().orc_geometry(self._h, *(_p(out[k]) for k in
                                      ("J", "Qi1", "Qi2", "Qi3", "f", "rx", "ry", "rz")))
        return out

    def bases(self):
        out = {k: np.zeros(self.shape + (3,)) for k in ("a1", "a2", "b1", "b2")}
        lib().orc_bases(self._h, *(_p(out[k]) for k in ("a1", "a2", "b1", "b2")))
        return out

    def sync_weights(self):
        out = [np.zeros(self.n) for _ in range(4)]
        lib().orc_sync_weights(self._h, *(_p(o) for o in out))
        return dict(zip(("qb", "qt", "ql", "qr"), out))

    def co2contra(self, u, v):
        ut, vt = self.zeros(), self.zeros()
        lib().orc_co2contra(self._h, _p(u), _p(v), _p(ut), _p(vt))
        return ut, vt

    def grad(self, f):
        gx, gy = self.zeros(), self.zeros()
        lib().orc_grad(self._h, _p(f), _p(gx), _p(gy))
        return gx, gy

    def div(self, u, v):
        out = self.zeros()
        lib().orc_div(self._h, _p(u), _p(v), _p(out))
        return out

    def curl(self, u, v):
        out = self.zeros()
        lib().orc_curl(self._h, _p(u), _p(v), _p(out))
        return out

    def sync_scalar(self, f):
        f = np.array(f, dtype=np.float64, order="C")
        lib().orc_sync_scalar(self._h, _p(f))
        return f

    def sync_vector_cov(self, gx, gy):
        gx = np.array(gx, dtype=np.float64, order="C")
        gy = np.array(gy, dtype=np.float64, order="C")
        lib().orc_sync_vector_cov(self._h, _p(gx), _p(gy))
        return gx, gy

    def coriolis(self, hu, hv, h, curl):
        cu, cv = self.zeros(), self.zeros()
        lib().orc_coriolis(self._h, _p(hu), _p(hv), _p(h), _p(curl), _p(cu), _p(cv))
        return cu, cv

    def apply(self, h, u, v, hs=None):
        th, tu, tv = self.zeros(), self.zeros(), self.zeros()
        lib().orc_apply(self._h, _p(hs), _p(h), _p(u), _p(v), _p(th), _p(tu), _p(tv))
        return th, tu, tv

    def rk4(self, h, u, v, dt, nsteps=1, hs=None):
        h, u, v = (np.array(a, dtype=np.float64, order="C") for a in (h, u, v))
        lib().orc_rk4(self._h, _p(hs), _p(h), _p(u), _p(v), float(dt), int(nsteps))
        return h, u, v

    def rk4_inplace(self, h, u, v, dt, nsteps=1, hs=None):
        """rk4 on the caller's C-contiguous FP64 arrays, updated in place (no
        copies: the timed CPU baseline uses this)."""
        for a in (h, u, v):
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] and a.shape == self.shape
        lib().orc_rk4(self._h, _p(hs), _p(h), _p(u), _p(v), float(dt), int(nsteps))

    def diagnostics(self, h, u, v, hs=None):
        out = np.zeros(7)
        lib().orc_diagnostics(self._h, _p(hs), _p(h), _p(u), _p(v), _p(out))
        return out

    # hyperdiffusion (narrow = 21, 42 or 63: the narrow Laplacian's SBP order)
    def laplace(self, f, narrow=42):
        out = self.zeros()
        assert lib().orc_laplace(self._h, int(narrow), _p(np.ascontiguousarray(f)), _p(out)) == 0
        return out

    def hordiff_scalar(self, f, coeff, narrow=42):
        out = self.zeros()
        assert lib().orc_hordiff_scalar(self._h, int(narrow), float(coeff),
                                        _p(np.ascontiguousarray(f)), _p(out)) == 0
        return out

    def hordiff_vec_xyz(self, u, v, coeff, narrow=42):
        ut, vt = self.zeros(), self.zeros()
        assert lib().orc_hordiff_vec_xyz(self._h, int(narrow), float(coeff),
                                         _p(np.ascontiguousarray(u)), _p(np.ascontiguousarray(v)),
                                         _p(ut), _p(vt)) == 0
        return ut, vt

    def diffusion_apply(self, h, u, v, uv_coeff, h_coeff, uv_narrow=42, h_narrow=42):
        th, tu, tv = self.zeros(), self.zeros(), self.zeros()
        assert lib().orc_diffusion_apply(self._h, int(uv_narrow), float(uv_coeff), int(h_narrow),
                                         float(h_coeff), *(_p(np.ascontiguousarray(a)) for a in (h, u, v)),
                                         _p(th), _p(tu), _p(tv)) == 0
        return th, tu, tv

    def diffusion_step(self, h, u, v, dt, uv_coeff, h_coeff, uv_narrow=42, h_narrow=42):
        h, u, v = (np.array(a, dtype=np.float64, order="C") for a in (h, u, v))
        assert lib().orc_diffusion_step(self._h, int(uv_narrow), float(uv_coeff), int(h_narrow),
                                        float(h_coeff), _p(h), _p(u), _p(v), float(dt)) == 0
        return h, u, v

    # lat-lon regrid of Ah fields (width 2 linear, 4 cubic); (Nlat, Nlon) arrays
    def latlon_scalar(self, f, nlon, nlat, width=4):
        out = np.zeros((nlat, nlon))
        assert lib().orc_latlon_scalar(self._h, int(nlon), int(nlat), int(width),
                                       _p(np.ascontiguousarray(f)), _p(out)) == 0
        return out

    def latlon_vector(self, u, v, nlon, nlat, width=4, contravariant=False):
        uo, vo = np.zeros((nlat, nlon)), np.zeros((nlat, nlon))
        assert lib().orc_latlon_vector(self._h, int(nlon), int(nlat), int(width),
                                       1 if contravariant else 0, _p(np.ascontiguousarray(u)),
                                       _p(np.ascontiguousarray(v)), _p(uo), _p(vo)) == 0
        return uo, vo

    VECTOR_FIELDS = {"solid_rotation": 0, "cross_polar": 1, "xyz_grad": 2, "vsh_curl_free_10": 3}
    SCALAR_FIELDS = {"xyz": 10, "cross_polar_div": 11, "cross_polar_zeta": 12}

    def vector_test_field(self, kind, level=0, contravariant=False):
        u, v = self.zeros(), self.zeros()
        rc = lib().orc_vector_test_field(self._h, self.VECTOR_FIELDS[kind], int(level),
                                         1 if contravariant else 0, _p(u), _p(v))
        assert rc == 0
        return u, v

    def scalar_test_field(self, kind, level=0):
        f = self.zeros()
        assert lib().orc_scalar_test_field(self._h, self.SCALAR_FIELDS[kind], int(level), _p(f)) == 0
        return f

    def l2norm(self, f):
        return lib().orc_l2norm(self._h, _p(np.ascontiguousarray(f, dtype=np.float64)))

    def mass(self, f):
        return lib().orc_mass(self._h, _p(np.ascontiguousarray(f, dtype=np.float64)))


class OracleCDomain:
    """FP64 oracle of the C-grid SBP vector-invariant operator
    (&shallow_water_model_c, sbp_order 21 or 42).  Fields are dense arrays
    per mesh: h (6, N, N) on the cell centres, u (6, N, N+1) on the x-faces,
    v (6, N+1, N) on the y-faces, the curl (6, N+1, N+1) on the corners."""

    MESHES = {"p": 0, "u": 1, "v": 2, "q": 3}

    def __init__(self, N, sbp_order=42, radius=6.371e6, grav=9.80616,
                 omega=7.292e-5, axis=(0.0, 0.0, 1.0)):
        L = lib()
        ax = np.asarray(axis, dtype=np.float64)
        self._h = L.orcc_create(int(N), int(sbp_order), float(radius), float(grav),
                                float(omega), _p(ax))
        if not self._h:
            raise ValueError(f"oracle: unsupported C grid N={N} / sbp_order={sbp_order}")
        self.N, self.sbp_order = int(N), int(sbp_order)
        n = self.N
        self.shapes = {"p": (6, n, n), "u": (6, n, n + 1), "v": (6, n + 1, n), "q": (6, n + 1, n + 1)}

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orcc_destroy(self._h)
            self._h = None

    def zeros(self, mesh):
        return np.zeros(self.shapes[mesh])

    def points(self, mesh):
        x, y, z = (self.zeros(mesh) for _ in range(3))
        lib().orcc_points(self._h, self.MESHES[mesh], _p(x), _p(y), _p(z))
        return x, y, z

    def metric(self, mesh):
        out = {k: self.zeros(mesh) for k in ("J", "Qi1", "Qi2", "Qi3", "f")}
        lib().orcc_metric(self._h, self.MESHES[mesh], *(_p(out[k]) for k in ("J", "Qi1", "Qi2", "Qi3", "f")))
        return out

    def bases(self, mesh):
        sh = self.shapes[mesh] + (3,)
        out = {k: np.zeros(sh) for k in ("a1", "a2", "b1", "b2")}
        lib().orcc_bases(self._h, self.MESHES[mesh], *(_p(out[k]) for k in ("a1", "a2", "b1", "b2")))
        return out

    @staticmethod
    def _c(a):
        return np.ascontiguousarray(a, dtype=np.float64)

    def co2contra(self, u, v):
        ut, vt = self.zeros("u"), self.zeros("v")
        lib().orcc_co2contra(self._h, _p(self._c(u)), _p(self._c(v)), _p(ut), _p(vt))
        return ut, vt

    def massflux(self, h, ut, vt):
        hu, hv = self.zeros("u"), self.zeros("v")
        lib().orcc_massflux(self._h, _p(self._c(h)), _p(self._c(ut)), _p(self._c(vt)), _p(hu), _p(hv))
        return hu, hv

    def ke(self, u, v, ut, vt):
        k = self.zeros("p")
        lib().orcc_ke(self._h, *(_p(self._c(a)) for a in (u, v, ut, vt)), _p(k))
        return k

    def grad(self, f):
        gx, gy = self.zeros("u"), self.zeros("v")
        lib().orcc_grad(self._h, _p(self._c(f)), _p(gx), _p(gy))
        return gx, gy

    def div(self, hu, hv):
        d = self.zeros("p")
        lib().orcc_div(self._h, _p(self._c(hu)), _p(self._c(hv)), _p(d))
        return d

    def curl(self, u, v):
        c = self.zeros("q")
        lib().orcc_curl(self._h, _p(self._c(u)), _p(self._c(v)), _p(c))
        return c

    def coriolis(self, hu, hv, h, curl):
        cu, cv = self.zeros("u"), self.zeros("v")
        lib().orcc_coriolis(self._h, *(_p(self._c(a)) for a in (hu, hv, h, curl)), _p(cu), _p(cv))
        return cu, cv

    def apply(self, h, u, v, hs=None):
        th, tu, tv = self.zeros("p"), self.zeros("u"), self.zeros("v")
        hs_p = None if hs is None else _p(self._c(hs))
        lib().orcc_apply(self._h, hs_p, *(_p(self._c(a)) for a in (h, u, v)), _p(th), _p(tu), _p(tv))
        return th, tu, tv

    def rk4(self, h, u, v, dt, nsteps=1, hs=None):
        h, u, v = (np.array(a, dtype=np.float64, order="C") for a in (h, u, v))
        hs_p = None if hs is None else _p(self._c(hs))
        lib().orcc_rk4(self._h, hs_p, _p(h), _p(u), _p(v), float(dt), int(nsteps))
        return h, u, v

    def grad_perp(self, w):
        gu, gv = self.zeros("u"), self.zeros("v")
        lib().orcc_grad_perp(self._h, _p(self._c(w)), _p(gu), _p(gv))
        return gu, gv

    def ecs_o_halo(self, f, halo_width=2):
        """The ECS_O halo of a cell-centre field: (6, N+2hw, N+2hw) extended
        tiles, 1-based (i, j) of the reference at [j + hw - 1, i + hw - 1]."""
        W = self.N + 2 * int(halo_width)
        e = np.zeros((6, W, W))
        assert lib().orcc_ecs_o_halo(self._h, _p(self._c(f)), int(halo_width), _p(e)) == 0
        return e

    def grad_a2_ecs(self, f):
        """gradient_a2_ecs at the cell centres (covariant gx, gy, both p-shaped)."""
        gx, gy = self.zeros("p"), self.zeros("p")
        lib().orcc_grad_a2_ecs(self._h, _p(self._c(f)), _p(gx), _p(gy))
        return gx, gy

    def ecs_a_vec_halo(self, u, v, halo_width=2):
        """The ecs_A_vec halo of contravariant (u, v) at the cell centres:
        two (6, N+2hw, N+2hw) arrays laid out as ecs_o_halo."""
        W = self.N + 2 * int(halo_width)
        eu, ev = np.zeros((6, W, W)), np.zeros((6, W, W))
        assert lib().orcc_ecs_a_vec_halo(self._h, _p(self._c(u)), _p(self._c(v)), int(halo_width),
                                         _p(eu), _p(ev)) == 0
        return eu, ev

    def ecs_xy_halo(self, f, halo_width=3):
        """The ECS_xy halo of a corner-mesh field: (6, n+2hw, n+2hw), n = N+1."""
        W = self.N + 1 + 2 * int(halo_width)
        e = np.zeros((6, W, W))
        assert lib().orcc_ecs_xy_halo(self._h, _p(self._c(f)), int(halo_width), _p(e)) == 0
        return e

    def laplace_ch(self, f, order=4):
        """laplace_ch_halo2 / laplace_ch_halo4 of a corner-mesh field."""
        out = self.zeros("q")
        assert lib().orcc_laplace_ch(self._h, int(order), _p(self._c(f)), _p(out)) == 0
        return out

    def grad_c2_ecs(self, f):
        """gradient_c2_ecs: gx on the x-faces, gy on the y-faces."""
        gx, gy = self.zeros("u"), self.zeros("v")
        lib().orcc_grad_c2_ecs(self._h, _p(self._c(f)), _p(gx), _p(gy))
        return gx, gy

    def div_a2_ecs(self, u, v):
        """divergence_a2_ecs of contravariant (u, v) at the cell centres."""
        d = self.zeros("p")
        lib().orcc_div_a2_ecs(self._h, _p(self._c(u)), _p(self._c(v)), _p(d))
        return d

    def contra2co(self, ut, vt):
        u, v = self.zeros("u"), self.zeros("v")
        lib().orcc_contra2co(self._h, _p(self._c(ut)), _p(self._c(vt)), _p(u), _p(v))
        return u, v

    # hordiff_uv_name of the C grid -> the parts of the vector hyperdiffusion
    HORDIFF_UV = {"hordiff_c_biharm_div": 1, "hordiff_c_biharm_curl": 2, "hordiff_c_biharm_curl_div": 3}

    def hordiff(self, h, u, v, uv_name="hordiff_c_biharm_curl_div", uv_coeff=0.03, h_coeff=0.03):
        """Tendency of operator_swm_diff_t%apply with the C-grid operators."""
        th, tu, tv = self.zeros("p"), self.zeros("u"), self.zeros("v")
        lib().orcc_hordiff(self._h, self.HORDIFF_UV[uv_name], float(uv_coeff), float(h_coeff),
                           *(_p(self._c(a)) for a in (h, u, v)), _p(th), _p(tu), _p(tv))
        return th, tu, tv

    def model_step(self, h, u, v, dt, nsteps=1, hs=None, uv_name="hordiff_c_biharm_curl_div",
                   uv_coeff=0.03, h_coeff=0.03):
        """nsteps of one RK4 step followed by one explicit Euler step of the
        hyperdiffusion."""
        h, u, v = (np.array(a, dtype=np.float64, order="C") for a in (h, u, v))
        hs_p = None if hs is None else _p(self._c(hs))
        lib().orcc_model_step(self._h, hs_p, _p(h), _p(u), _p(v), float(dt), int(nsteps),
                              self.HORDIFF_UV[uv_name], float(uv_coeff), float(h_coeff))
        return h, u, v

    VECTOR_FIELDS = {"solid_rotation": 0, "cross_polar": 1, "xyz_grad": 2, "vsh_curl_free_10": 3}
    SCALAR_FIELDS = {"xyz": 10, "cross_polar_div": 11, "cross_polar_zeta": 12}

    def vector_test_field(self, kind, level=0, contravariant=False):
        u, v = self.zeros("u"), self.zeros("v")
        assert lib().orcc_vector_test_field(self._h, self.VECTOR_FIELDS[kind], int(level),
                                            1 if contravariant else 0, _p(u), _p(v)) == 0
        return u, v

    def scalar_test_field(self, kind, level=0, mesh="p"):
        f = self.zeros(mesh)
        assert lib().orcc_scalar_test_field(self._h, self.SCALAR_FIELDS[kind], int(level),
                                            self.MESHES[mesh], _p(f)) == 0
        return f

    def mass(self, f, mesh="p"):
        return lib().orcc_mass(self._h, self.MESHES[mesh], _p(self._c(f)))

    def l2norm(self, f, mesh="p"):
        return lib().orcc_l2norm(self._h, self.MESHES[mesh], _p(self._c(f)))


def golden_c(kind: str, N: int = 32, sbp_order: int = 42) -> np.ndarray:
    """Values printed by the reference known-answer test of a C-grid
    operator at (N, nz=3): kind div, grad, curl, coriolis, ke, co2contra or
    contra2co (the transform2co of co2contra_c_sbp*_new), or grad_a2_ecs
    (gradient_a2_ecs on the A grid's cell centres, with the ECS_O halo)."""
    k = {"div": 0, "grad": 1, "curl": 2, "coriolis": 3, "ke": 4, "co2contra": 5, "contra2co": 6,
         "grad_a2_ecs": 7, "div_a2_ecs": 8, "grad_c2_ecs": 9}[kind]
    out = np.zeros(4)
    if lib().orcc_golden(k, int(N), int(sbp_order), _p(out)) != 0:
        raise ValueError(f"oracle C-grid golden {kind} failed for order {sbp_order}")
    return out[:4] if kind in ("div", "curl", "ke", "div_a2_ecs") else out[:2]


def golden(kind: str, N: int = 32, sbp_order: int = 42):
    """Values printed by the reference known-answer test at (N, nz=3)."""
    L = lib()
    if kind in ("div", "curl"):
        out = np.zeros(4)
        rc = getattr(L, f"orc_golden_{kind}")(int(N), int(sbp_order), _p(out))
    elif kind == "grad":
        out = np.zeros(2)
        rc = L.orc_golden_grad(int(N), int(sbp_order), _p(out))
    elif kind in ("co2contra", "contra2co", "coriolis"):
        out = np.zeros(2)
        rc = getattr(L, f"orc_golden_{kind}")(int(N), _p(out))
    elif kind == "ke":
        out = np.zeros(4)
        rc = L.orc_golden_ke(int(N), _p(out))
    else:
        raise ValueError(kind)
    if rc != 0:
        raise ValueError(f"oracle golden {kind} failed for order {sbp_order}")
    return out


def golden_regrid(kind: str, interp: str) -> np.ndarray:
    """test_regrid_mod.f90's maximum errors on the Ah grid at N=32: kind
    "scalar", "covariant" or "contravariant"; interp "linear" or "cubic"."""
    out = np.zeros(2)
    k = {"scalar": 0, "covariant": 1, "contravariant": 2}[kind]
    assert lib().orc_golden_regrid(k, 2 if interp == "linear" else 4, _p(out)) == 0
    return out[:1] if k == 0 else out


def quadrature_error(N: int, sbp_order: int, max_order: int) -> float:
    return lib().orc_golden_quadrature(int(N), int(sbp_order), int(max_order))


def rk4_iomega_error() -> float:
    return lib().orc_golden_rk4_iomega()
