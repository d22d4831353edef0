"""GB300-native shallow-water time-stepping hot path (cubed sphere, Ah-grid SBP).

Host-side mirror of the reference's plugin surface
(vvshashkin/cubedsphere_sbp_swm), over the C-ABI of include/swm_gpu.h:

  OperatorSWM      operator_t / operator_swm_t  (apply, get_diagnostics)
  StvecSWM         stvec_t / stvec_swm_t        (assign/update/dot/norm2)
  RK4              timescheme_t / rk4_t         (step)
  HaloAhScalarSync, EcsAhVecSyncCovariant       halo_t / halo_vec_t
  GridField        grid_field_t (FP64 field; single operators)

Host arrays are float64 with shape (6, N+1, N+1) = (panel, j, i): one tile
per panel as in the reference Ah grid, edge nodes duplicated on both panels.
All compute runs in libswm_gb300.so on the GPU; nothing here falls back to
the CPU.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _abi
from ._abi import SWM_FP32_FUSED, SWM_FP64_PLAIN, SwmError

__all__ = [
    "ModelConfig", "OperatorSWM", "StvecSWM", "GridField", "RK4", "OperatorSWMDiff",
    "ExplicitEul1", "LatLonRegrid", "LatLonOutputer", "PaneledOutputer", "HaloAhScalarSync",
    "EcsAhVecSyncCovariant", "create_timescheme", "create_halo_procedure",
    "create_vector_halo_procedure", "Ensemble", "SwmError", "EARTH", "c_grid_names", "MESHES",
]

_D = ctypes.POINTER(ctypes.c_double)

# constants of the benchmark configurations (not the reference's const_mod)
EARTH = dict(radius=6.371e6, grav=9.80616, omega=7.292e-5)

_PREC = {"fp64": SWM_FP64_PLAIN, "fp64_plain": SWM_FP64_PLAIN,
         "fp32": SWM_FP32_FUSED, "fp32_fused": SWM_FP32_FUSED}

DIAG_KEYS = ("hmin", "hmax", "mass", "TE", "KE", "PE", "Enstrophy")


@dataclass
class ModelConfig:
    """&domain / &metric / &shallow_water_model keys of the hot path."""
    N: int
    sbp_order: int = 42
    radius: float = EARTH["radius"]
    grav: float = EARTH["grav"]
    omega: float = EARTH["omega"]
    rotation_axis: tuple = (0.0, 0.0, 1.0)
    precision: str = "fp64"
    device: int = 0
    # operator names of the &shallow_water_model namelist (None: derived
    # from sbp_order)
    names: dict | None = field(default=None)

    def c_struct(self) -> _abi.SwmConfig:
        c = _abi.SwmConfig()
        c.N = int(self.N)
        c.sbp_order = int(self.sbp_order)
        c.radius, c.grav, c.omega = float(self.radius), float(self.grav), float(self.omega)
        for k in range(3):
            c.rotation_axis[k] = float(self.rotation_axis[k])
        if self.precision not in _PREC:
            raise ValueError(f"unknown precision {self.precision!r}")
        c.precision = _PREC[self.precision]
        c.device = int(self.device)
        return c


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _host(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def _check_c_f64(a, shape):
    """An array an asynchronous transfer reads or writes after the call
    returns: no temporary copy may stand in for it."""
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
            and a.shape == shape):
        raise ValueError(f"asynchronous transfers need C-contiguous float64 arrays of shape {shape}")


MESHES = {"p": _abi.SWM_MESH_P, "u": _abi.SWM_MESH_U, "v": _abi.SWM_MESH_V, "q": _abi.SWM_MESH_Q}


def c_grid_names(sbp_order: int = 42) -> dict:
    """Operator names of the C-grid family (the &shallow_water_model_c
    namelist, namelist_swm:80-102) at SBP order 21 or 42."""
    o = int(sbp_order)
    return {"div_op_name": f"divergence_c_sbp{o}", "grad_op_name": f"gradient_c_sbp{o}",
            "curl_op_name": f"curl_c_sbp{o}", "coriolis_op_name": f"coriolis_Cgrid_sbp{o}",
            "KE_op_name": f"KE_Cgrid_sbp{o}", "co2contra_op_name": f"co2contra_c_sbp{o}",
            "massflux_op_name": f"massflux_c_sbp{o}", "quadrature_name": f"SBP_C{o}_quadrature"}


class OperatorSWM:
    """operator_swm_t on one GPU: domain geometry, the vector-invariant RHS,
    its cube-edge syncs, the fused RK4 driver and FP64 diagnostics.

    The staggering follows the operator names: the Ah family (default) keeps
    h, u, v on the (N+1) x (N+1) nodes; the C family (c_grid_names) keeps h
    on the N x N cell centres, u on the x-faces and v on the y-faces
    (shapes in mesh_shape / state_shapes)."""

    def __init__(self, config: ModelConfig | None = None, **kw):
        if config is None:
            config = ModelConfig(**kw)
        self.config = config
        self._L = _abi.load()
        c = config.c_struct()
        h = ctypes.c_void_p()
        if config.names:
            nm = config.names
            keys = ("div_op_name", "grad_op_name", "curl_op_name", "coriolis_op_name",
                    "KE_op_name", "co2contra_op_name", "massflux_op_name", "quadrature_name")
            args = [(nm.get(k) or "").encode() for k in keys]
            rc = self._L.swm_ctx_create_named(ctypes.byref(c), *args, ctypes.byref(h))
        else:
            rc = self._L.swm_ctx_create(ctypes.byref(c), ctypes.byref(h))
        _abi.check(rc, None)
        self._h = h
        self.N = config.N
        self.n = config.N + 1
        self.staggering = "C" if self._L.swm_ctx_grid(h) == _abi.SWM_GRID_C else "Ah"
        self._mesh_shapes = {}
        for name, m in MESHES.items():
            nx, ny = ctypes.c_int(), ctypes.c_int()
            _abi.check(self._L.swm_mesh_dims(h, m, ctypes.byref(nx), ctypes.byref(ny)), h)
            self._mesh_shapes[name] = (6, ny.value, nx.value)
        # host shape of h, u and v (all (6, N+1, N+1) on the Ah grid)
        self.state_shapes = tuple(self._mesh_shapes[k] for k in ("p", "u", "v"))
        self.shape = self._mesh_shapes["p"]

    def mesh_shape(self, mesh: str = "p") -> tuple:
        """Host array shape (6, ny, nx) of a field on mesh p, u, v or q."""
        return self._mesh_shapes[mesh]

    # lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.swm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _abi.check(rc, self._h)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return self._L.swm_ctx_stream(self._h) or 0

    def synchronize(self):
        self._check(self._L.swm_ctx_synchronize(self._h))

    @property
    def npts(self) -> int:
        return int(self._L.swm_ctx_npts(self._h))

    # factories ----------------------------------------------------------
    def create_stvec(self) -> "StvecSWM":
        return StvecSWM(self)

    def create_field(self, mesh: str = "p") -> "GridField":
        return GridField(self, mesh)

    def set_orography(self, hs):
        hs = _host(hs, self.shape)
        self._check(self._L.swm_set_orography(self._h, _ptr(hs)))

    # operator_t ---------------------------------------------------------
    def apply(self, vout: "StvecSWM", vin: "StvecSWM"):
        """vout = A(vin) (operator_mod.f90:18-25)."""
        self._check(self._L.swm_apply(self._h, vout._h, vin._h))

    def apply_unfused(self, vout: "StvecSWM", vin: "StvecSWM"):
        self._check(self._L.swm_apply_unfused(self._h, vout._h, vin._h))

    def laplace(self, out: "GridField", f: "GridField", narrow_order: int = 42):
        """out = L(f): the narrow-stencil SBP Laplacian laplace_ah_sbp21_narrow /
        _sbp42_narrow / _sbp63_narrow (laplace_Ah_sbp42_narrow_mod.f90:23-58,
        laplace_Ah_sbp21_narrow_mod.f90:23-243), edge-synced."""
        self._check(self._L.swm_laplace(self._h, out._h, f._h, int(narrow_order)))

    _BOX_MODES = {"auto": 0, "strip": 1, "widest": 2}
    _BOX_NAMES = {1: "strip", 2: "widest"}

    def tune_stage(self, v: "StvecSWM", dt: float, steps: int = 10) -> dict:
        """Time the stage kernel's launch shapes (consumer width, rows per
        unit, persistent grid, TMA box mode) on a copy of v and keep the
        fastest (bit-identical results)."""
        c, r, g, b, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._check(self._L.swm_tune_stage(self._h, v._h, float(dt), int(steps), ctypes.byref(c),
                                           ctypes.byref(r), ctypes.byref(g), ctypes.byref(b),
                                           ctypes.byref(ms)))
        return {"width": c.value, "seg_rows": r.value, "grid": g.value,
                "box": self._BOX_NAMES[b.value], "ms": ms.value}

    @property
    def stage_shape(self) -> dict:
        c, r, g, b, n = (ctypes.c_int() for _ in range(5))
        self._check(self._L.swm_get_stage_shape(self._h, ctypes.byref(c), ctypes.byref(r),
                                                ctypes.byref(g), ctypes.byref(b), ctypes.byref(n)))
        return {"width": c.value, "seg_rows": r.value, "grid": g.value,
                "box": self._BOX_NAMES[b.value], "units": n.value}

    def set_stage_shape(self, width: int = 128, seg_rows: int = 0, grid: int = 0, box: str = "auto"):
        """box: "strip" (the narrowest TMA box covering every column strip),
        "widest" (the width's widest box, compiled in; needs a field pitch of
        at least that box) or "auto" (the widest where it fits and keeps the
        resident CTAs per SM)."""
        if box not in self._BOX_MODES:
            raise SwmError(_abi.SWM_E_INVALID, f"unknown box mode {box!r}")
        self._check(self._L.swm_set_stage_shape(self._h, int(width), int(seg_rows), int(grid),
                                                self._BOX_MODES[box]))

    def model_step(self, v0: "StvecSWM", dt: float, nsteps: int = 1):
        """nsteps of the drivers' time step (ts2_mod.f90:143-146): RK4, then the
        diffusion step when an OperatorSWMDiff is attached to this operator."""
        self._check(self._L.swm_model_step(self._h, v0._h, float(dt), int(nsteps)))

    def get_diagnostics(self, v: "StvecSWM") -> dict:
        out = np.zeros(7)
        self._check(self._L.swm_diagnostics(self._h, v._h, _ptr(out)))
        return dict(zip(DIAG_KEYS, out.tolist()))

    # single operators on GridFields ------------------------------------
    def co2contra(self, ut, vt, u, v):
        self._check(self._L.swm_op_co2contra(self._h, ut._h, vt._h, u._h, v._h))

    def massflux(self, hu, hv, h, ut, vt):
        self._check(self._L.swm_op_massflux(self._h, hu._h, hv._h, h._h, ut._h, vt._h))

    def calc_KE(self, ke, u, v, ut, vt):
        self._check(self._L.swm_op_ke(self._h, ke._h, u._h, v._h, ut._h, vt._h))

    def calc_grad(self, gx, gy, f):
        self._check(self._L.swm_op_grad(self._h, gx._h, gy._h, f._h))

    def calc_div(self, div, u, v):
        self._check(self._L.swm_op_div(self._h, div._h, u._h, v._h))

    def calc_curl(self, curl, u, v):
        self._check(self._L.swm_op_curl(self._h, curl._h, u._h, v._h))

    def calc_coriolis_vec_inv(self, cor_u, cor_v, hu, hv, h, curl):
        self._check(self._L.swm_op_coriolis(self._h, cor_u._h, cor_v._h, hu._h, hv._h,
                                            h._h, curl._h))

    def calc_grad_perp(self, gu, gv, w):
        """grad_perp_c_sbp (C grid): w on mesh q, gu on u, gv on v."""
        self._check(self._L.swm_op_grad_perp(self._h, gu._h, gv._h, w._h))

    def contra2co(self, u, v, ut, vt):
        """transform2co of co2contra_c_sbp*_new (C grid)."""
        self._check(self._L.swm_op_contra2co(self._h, u._h, v._h, ut._h, vt._h))

    def calc_grad_a2_ecs(self, gx, gy, f):
        """gradient_a2_ecs on the cell centres (C grid): gx, gy and f on mesh p."""
        self._check(self._L.swm_op_grad_a2_ecs(self._h, gx._h, gy._h, f._h))

    def ecs_o_halo(self, f, halo_width: int = 2) -> np.ndarray:
        """The ECS_O halo of a cell-centre field (C grid): the (6, N+2hw,
        N+2hw) extended tiles, the reference's 1-based (i, j) at
        [:, j + hw - 1, i + hw - 1]."""
        W = self.N + 2 * int(halo_width)
        out = np.empty((6, W, W))
        self._check(self._L.swm_halo_ecs_o(self._h, f._h, int(halo_width), _ptr(out)))
        return out

    def calc_grad_c2_ecs(self, gx, gy, f):
        """gradient_c2_ecs (C grid): f on mesh p, gx on u, gy on v."""
        self._check(self._L.swm_op_grad_c2_ecs(self._h, gx._h, gy._h, f._h))

    def ecs_xy_halo(self, f, halo_width: int = 3) -> np.ndarray:
        """The ECS_xy halo of a corner-mesh field (C grid): (6, n+2hw, n+2hw)
        extended tiles, n = N+1, laid out as ecs_o_halo's."""
        W = self.N + 1 + 2 * int(halo_width)
        out = np.empty((6, W, W))
        self._check(self._L.swm_halo_ecs_xy(self._h, f._h, int(halo_width), _ptr(out)))
        return out

    def laplace_ch(self, out, f, order: int = 4):
        """laplace_ch_halo2 / laplace_ch_halo4 of a corner-mesh field (C grid)."""
        self._check(self._L.swm_laplace_ch(self._h, out._h, f._h, int(order)))

    def calc_div_a2_ecs(self, div, u, v):
        """divergence_a2_ecs on the cell centres (C grid): contravariant u, v
        and div on mesh p."""
        self._check(self._L.swm_op_div_a2_ecs(self._h, div._h, u._h, v._h))

    def ecs_a_vec_halo(self, u, v, halo_width: int = 2):
        """The ecs_A_vec halo of contravariant (u, v) on the cell centres (C
        grid): two extended-tile arrays laid out as ecs_o_halo's."""
        W = self.N + 2 * int(halo_width)
        eu, ev = np.empty((6, W, W)), np.empty((6, W, W))
        self._check(self._L.swm_halo_ecs_a_vec(self._h, u._h, v._h, int(halo_width), _ptr(eu), _ptr(ev)))
        return eu, ev

    def quadrature_mass(self, f) -> float:
        out = ctypes.c_double()
        self._check(self._L.swm_quadrature_mass(self._h, f._h, ctypes.byref(out)))
        return out.value

    # measurement --------------------------------------------------------
    def timing_enable(self, on: bool = True):
        self._check(self._L.swm_timing_enable(self._h, 1 if on else 0))

    def timing_read(self):
        sm, em = ctypes.c_double(), ctypes.c_double()
        sl, el = ctypes.c_long(), ctypes.c_long()
        self._check(self._L.swm_timing_read(self._h, ctypes.byref(sm), ctypes.byref(sl),
                                            ctypes.byref(em), ctypes.byref(el)))
        return sm.value, sl.value, em.value, el.value


class StvecSWM:
    """stvec_swm_t: the (h, u, v) state on the device (covariant u, v)."""

    def __init__(self, op: OperatorSWM, _similar_to: "StvecSWM" | None = None):
        self.op = op
        h = ctypes.c_void_p()
        if _similar_to is None:
            rc = op._L.swm_state_create(op._h, ctypes.byref(h))
        else:
            rc = op._L.swm_state_create_similar(op._h, _similar_to._h, ctypes.byref(h))
        op._check(rc)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.op._L.swm_state_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def create_similar(self) -> "StvecSWM":
        return StvecSWM(self.op, _similar_to=self)

    def upload(self, h, u, v):
        h, u, v = (_host(a, sh) for a, sh in zip((h, u, v), self.op.state_shapes))
        self.op._check(self.op._L.swm_state_upload(self.op._h, self._h, _ptr(h), _ptr(u), _ptr(v)))
        self.op.synchronize()

    def upload_async(self, h, u, v):
        """Upload from caller-owned C-contiguous float64 arrays
        (swm_state_upload_async): the copy engine moves them through a
        device staging buffer on the context's upload stream and the state
        takes their values for every later call; the arrays must stay
        unchanged until OperatorSWM.synchronize().  Page-locked arrays let
        the copy overlap the context's kernels."""
        for a, sh in zip((h, u, v), self.op.state_shapes):
            _check_c_f64(a, sh)
        self.op._check(self.op._L.swm_state_upload_async(self.op._h, self._h, _ptr(h), _ptr(u), _ptr(v)))

    def download(self, out=None):
        if out is None:
            out = tuple(np.empty(sh) for sh in self.op.state_shapes)
        self.op._check(self.op._L.swm_state_download(self.op._h, self._h, *(_ptr(a) for a in out)))
        return out

    def download_async(self, out):
        """Download into caller-owned C-contiguous float64 arrays
        (swm_state_download_async): the state as the calls queued before
        leave it, moved by the copy engine on the context's download stream;
        `out` holds it once OperatorSWM.synchronize() returns."""
        for a, sh in zip(out, self.op.state_shapes):
            _check_c_f64(a, sh)
        self.op._check(self.op._L.swm_state_download_async(self.op._h, self._h, *(_ptr(a) for a in out)))
        return out

    def save(self, path: str, time: float = 0.0):
        """Write the state to a restart file (FP64 fields and a header)."""
        self.op._check(self.op._L.swm_state_save(self.op._h, self._h, str(path).encode(), float(time)))

    def load(self, path: str) -> float:
        """Read a restart file of the same N; returns the stored model time."""
        t = ctypes.c_double()
        self.op._check(self.op._L.swm_state_load(self.op._h, self._h, str(path).encode(),
                                                 ctypes.byref(t)))
        return t.value

    def assign_s1(self, s1):
        self.op._check(self.op._L.swm_assign_s1(self.op._h, self._h, float(s1)))

    def assign_s1v1(self, s1, v1):
        self.op._check(self.op._L.swm_assign_s1v1(self.op._h, self._h, float(s1), v1._h))

    def assign_s1v1s2v2(self, s1, v1, s2, v2):
        self.op._check(self.op._L.swm_assign_s1v1s2v2(self.op._h, self._h, float(s1), v1._h,
                                                       float(s2), v2._h))

    def update_s1v1(self, s1, v1):
        self.op._check(self.op._L.swm_update_s1v1(self.op._h, self._h, float(s1), v1._h))

    def update_s1v1s2v2(self, s1, v1, s2, v2):
        self.op._check(self.op._L.swm_update_s1v1s2v2(self.op._h, self._h, float(s1), v1._h,
                                                       float(s2), v2._h))

    def algebraic_dot(self, other) -> float:
        out = ctypes.c_double()
        self.op._check(self.op._L.swm_dot(self.op._h, self._h, other._h, ctypes.byref(out)))
        return out.value

    def algebraic_norm2(self) -> float:
        out = ctypes.c_double()
        self.op._check(self.op._L.swm_norm2(self.op._h, self._h, ctypes.byref(out)))
        return out.value


class GridField:
    """grid_field_t: one FP64 field on the device, on mesh p, u, v or q."""

    def __init__(self, op: OperatorSWM, mesh: str = "p"):
        self.op = op
        self.mesh = mesh
        self.shape = op.mesh_shape(mesh)
        h = ctypes.c_void_p()
        op._check(op._L.swm_field_create_mesh(op._h, MESHES[mesh], ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.op._L.swm_field_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, a):
        a = _host(a, self.shape)
        self.op._check(self.op._L.swm_field_upload(self.op._h, self._h, _ptr(a)))
        self.op.synchronize()

    def download(self) -> np.ndarray:
        out = np.empty(self.shape)
        self.op._check(self.op._L.swm_field_download(self.op._h, self._h, _ptr(out)))
        return out


class RK4:
    """rk4_t (time_schemes/rk4_mod.f90:12-42): classic RK4 with the stage
    combinations fused into the RHS kernels, replayed as a CUDA graph."""

    def step(self, v0: StvecSWM, operator: OperatorSWM, dt: float, nsteps: int = 1):
        operator._check(operator._L.swm_rk4_step(operator._h, v0._h, float(dt), int(nsteps)))


class OperatorSWMDiff:
    """operator_swm_diff_t (models/shallow_water/operator/operator_swm_diff_mod.f90
    :25-46), created like create_swm_diff_operator
    (operator_swm_diff_factory_mod.f90:27-30) from the namelist's
    hordiff_uv_name / uv_diff_coeff / hordiff_h_name / h_diff_coeff.  It lives
    on the model operator's context (its grid, stream and work fields)."""

    # the namelist defaults of &shallow_water_model (Ah) and
    # &shallow_water_model_c (namelist_swm:20-25, 90-94)
    DEFAULTS = {"Ah": ("hordiff_vec_xyz_Ah_sbp_42_narrow", 0.03, "hordiff_scalar_Ah_sbp_42_narrow", 0.01),
                "C": ("hordiff_c_biharm_curl_div", 0.03, "hordiff_scalar_C", 0.03)}

    def __init__(self, op: OperatorSWM, hordiff_uv_name: Optional[str] = None,
                 uv_diff_coeff: Optional[float] = None, hordiff_h_name: Optional[str] = None,
                 h_diff_coeff: Optional[float] = None):
        d = self.DEFAULTS[op.staggering]
        hordiff_uv_name = d[0] if hordiff_uv_name is None else hordiff_uv_name
        uv_diff_coeff = d[1] if uv_diff_coeff is None else uv_diff_coeff
        hordiff_h_name = d[2] if hordiff_h_name is None else hordiff_h_name
        h_diff_coeff = d[3] if h_diff_coeff is None else h_diff_coeff
        self.op = op
        op._check(op._L.swm_diffusion_set(op._h, hordiff_uv_name.encode(), float(uv_diff_coeff),
                                          hordiff_h_name.encode(), float(h_diff_coeff)))

    def apply(self, vout: StvecSWM, vin: StvecSWM):
        """vout = D(vin)."""
        self.op._check(self.op._L.swm_apply_diffusion(self.op._h, vout._h, vin._h))


class ExplicitEul1:
    """explicit_Eul1_t (time_schemes/explicit_Eul1_mod.f90:20-30) for the
    diffusion operator: v0 += dt * D(v0), replayed as a CUDA graph."""

    def step(self, v0: StvecSWM, operator: OperatorSWMDiff, dt: float, nsteps: int = 1):
        op = operator.op
        op._check(op._L.swm_diffusion_step(op._h, v0._h, float(dt), int(nsteps)))


class LatLonRegrid:
    """Lat-lon regrid of the context's Ah fields: create_latlon_regrid and
    create_latlon_vector_regrid with grid type "Ah"
    (regridders/regrid_factory_mod.f90:9-190).  Outputs are (Nlat, Nlon)
    arrays (longitude fastest, latitude from -90 to 90 degrees); vectors come
    out as (east, north) components."""

    def __init__(self, op: OperatorSWM, Nlon: int, Nlat: int, interp_type: str = "cubic",
                 components_type: str = "covariant"):
        self.op, self.Nlon, self.Nlat = op, int(Nlon), int(Nlat)
        h = ctypes.c_void_p()
        op._check(op._L.swm_latlon_create(op._h, self.Nlon, self.Nlat, interp_type.encode(),
                                          components_type.encode(), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.op._L.swm_latlon_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _out(self):
        return np.empty((self.Nlat, self.Nlon))

    def do_regrid(self, f: "GridField") -> np.ndarray:
        out = self._out()
        self.op._check(self.op._L.swm_latlon_regrid_field(self.op._h, self._h, f._h, _ptr(out)))
        return out

    def do_regrid_vec(self, u: "GridField", v: "GridField"):
        uo, vo = self._out(), self._out()
        self.op._check(self.op._L.swm_latlon_regrid_vector(self.op._h, self._h, u._h, v._h,
                                                          _ptr(uo), _ptr(vo)))
        return uo, vo

    def regrid_state(self, s: "StvecSWM"):
        h, u, v = self._out(), self._out(), self._out()
        self.op._check(self.op._L.swm_latlon_regrid_state(self.op._h, self._h, s._h, _ptr(h),
                                                          _ptr(u), _ptr(v)))
        return h, u, v


class LatLonOutputer:
    """latlon_outputer_t and latlon_vec_outputer_t for a state
    (outputer/latlon_outputer_mod.f90:38-190, created as in
    outputer_factory_mod.f90:45-218 with cubic interpolation): FP32
    direct-access records of Nlon*Nlat values."""

    def __init__(self, op: OperatorSWM, Nlat: int, Nlon: int):
        self.regrid = LatLonRegrid(op, Nlon, Nlat, "cubic", "covariant")
        self.op = op

    def write(self, s: "StvecSWM", h_file: str | None = "h.dat", u_file: str | None = "u.dat",
              v_file: str | None = "v.dat", rec_num: int = 1):
        enc = lambda x: x.encode() if x else None
        self.op._check(self.op._L.swm_latlon_write(self.op._h, self.regrid._h, s._h, enc(h_file),
                                                   enc(u_file), enc(v_file), int(rec_num)))


class PaneledOutputer:
    """master_paneled_outputer_t (outputer/master_paneled_outputer_mod.f90:24-77):
    FP32 direct-access records of the six panels' (N+1)^2 values."""

    def __init__(self, op: OperatorSWM):
        self.op = op

    def write(self, s: "StvecSWM", component: int, file_name: str, rec_num: int = 1):
        self.op._check(self.op._L.swm_paneled_write(self.op._h, s._h, int(component),
                                                    file_name.encode(), int(rec_num)))


class HaloAhScalarSync:
    """halo_t "Ah_scalar_sync" (halo/halo_Ah_scalar_sync_mod.f90)."""

    def __init__(self, op: OperatorSWM):
        self.op = op

    def get_halo_scalar(self, f: GridField, halo_width: int = 1):
        self.op._check(self.op._L.swm_sync_scalar(self.op._h, f._h))


class EcsAhVecSyncCovariant:
    """halo_vec_t "ecs_Ah_vec_sync_covariant" (equiang_cs/ecs_Ah_vec_sync_mod.f90)."""

    def __init__(self, op: OperatorSWM):
        self.op = op

    def get_halo_vector(self, u: GridField, v: GridField, halo_width: int = 0):
        self.op._check(self.op._L.swm_sync_vector_cov(self.op._h, u._h, v._h))


class Ensemble:
    """Independent members (own N, initial state and time step each; shared
    SBP order, constants and precision) advanced together: one RK4 step of
    all members is one CUDA graph with one stage-kernel and one edge-kernel
    launch per RK stage.  No reference counterpart (the reference runs one
    instance per job)."""

    def __init__(self, config: ModelConfig, member_N, member_dt):
        member_N = [int(x) for x in member_N]
        member_dt = [float(x) for x in member_dt]
        if len(member_N) != len(member_dt):
            raise ValueError("member_N and member_dt differ in length")
        self._L = _abi.load()
        self.config = config
        self.member_N = member_N
        self.member_dt = member_dt
        Ns = (ctypes.c_int * len(member_N))(*member_N)
        dts = (ctypes.c_double * len(member_dt))(*member_dt)
        h = ctypes.c_void_p()
        rc = self._L.swm_ensemble_create(ctypes.byref(config.c_struct()), len(member_N), Ns, dts,
                                         ctypes.byref(h))
        _abi.check_ensemble(rc, None)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.swm_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.member_N)

    def _check(self, rc):
        _abi.check_ensemble(rc, self._h)

    def shape(self, m):
        n = self.member_N[m] + 1
        return (6, n, n)

    def upload(self, m, h, u, v):
        sh = self.shape(m)
        h, u, v = (_host(a, sh) for a in (h, u, v))
        self._check(self._L.swm_ensemble_upload(self._h, int(m), _ptr(h), _ptr(u), _ptr(v)))

    def download(self, m):
        out = tuple(np.empty(self.shape(m)) for _ in range(3))
        self._check(self._L.swm_ensemble_download(self._h, int(m), *(_ptr(a) for a in out)))
        return out

    def get_diagnostics(self, m) -> dict:
        out = np.zeros(7)
        self._check(self._L.swm_ensemble_diagnostics(self._h, int(m), _ptr(out)))
        return dict(zip(DIAG_KEYS, out.tolist()))

    def step(self, nsteps: int = 1):
        self._check(self._L.swm_ensemble_step(self._h, int(nsteps)))

    def synchronize(self):
        self._check(self._L.swm_ensemble_synchronize(self._h))

    @property
    def stream(self) -> int:
        return self._L.swm_ensemble_stream(self._h) or 0

    def member(self, m):
        """(context handle, state handle) of member m, for single-instance calls."""
        c, s = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(self._L.swm_ensemble_member(self._h, int(m), ctypes.byref(c), ctypes.byref(s)))
        return c, s

    def set_shape(self, seg_rows: int, grid: int):
        self._check(self._L.swm_ensemble_set_shape(self._h, int(seg_rows), int(grid)))

    def get_shape(self) -> dict:
        a, b, c, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._L.swm_ensemble_get_shape(self._h, ctypes.byref(a), ctypes.byref(b),
                                                   ctypes.byref(c)))
        self._check(self._L.swm_ensemble_get_width(self._h, ctypes.byref(w)))
        return {"seg_rows": a.value, "grid": b.value, "units": c.value, "width": w.value}

    def set_width(self, cols: int):
        """Consumer width of the members' FP32 stage kernel (64, 96, 128, 160, 192)."""
        self._check(self._L.swm_ensemble_set_width(self._h, int(cols)))

    def tune(self, steps: int = 5) -> dict:
        a, b, ms, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        self._check(self._L.swm_ensemble_tune(self._h, int(steps), ctypes.byref(a), ctypes.byref(b),
                                              ctypes.byref(ms)))
        self._check(self._L.swm_ensemble_get_width(self._h, ctypes.byref(w)))
        return {"seg_rows": a.value, "grid": b.value, "width": w.value, "ms_per_step": ms.value}


def create_timescheme(name: str):
    """timescheme factory (time_schemes/timescheme_factory_mod.f90:13-59):
    "rk4" for the model operator, "explicit_Eul1" for the diffusion
    operator (the drivers' diff_time_scheme)."""
    if name == "rk4":
        return RK4()
    if name == "explicit_Eul1":
        return ExplicitEul1()
    raise SwmError(_abi.SWM_E_UNSUPPORTED, f"unsupported time scheme: {name}")


def create_halo_procedure(op: OperatorSWM, name: str):
    if name == "Ah_scalar_sync":
        return HaloAhScalarSync(op)
    raise SwmError(_abi.SWM_E_UNSUPPORTED, f"unsupported halo procedure: {name}")


def create_vector_halo_procedure(op: OperatorSWM, name: str):
    if name == "ecs_Ah_vec_sync_covariant":
        return EcsAhVecSyncCovariant(op)
    raise SwmError(_abi.SWM_E_UNSUPPORTED, f"unsupported vector halo procedure: {name}")
