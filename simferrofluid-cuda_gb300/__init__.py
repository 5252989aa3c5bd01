"""sf-gb300: GB300-native (sm_103a) drop-in for the two grid solves of a SimFerrofluid substep.

Host-side mirror of the reference's solver classes over the C ABI (include/sfgpu.h):

* :class:`Pressure` -- ``Pressure(StaggeredGrid)``, ``SetPressureJump``, ``Project``, ``Reproject``
  (core/Pressure.h:8-22).
* :class:`MagneticField` -- ``MagneticField(StaggeredGrid, chi, bandWidth)``, ``SetSusceptibility``,
  ``SetBandWidth``, ``Solve`` (core/MagneticField.h:24-36); the potential and the total field, private in
  the reference, are exposed as ``potential`` and ``total_field``.
* :class:`StaggeredGrid` -- the geometry of core/StaggeredGrid.h:8-21 (cell grid and face grids).

Arrays are numpy float64 in the reference's layout (C-contiguous ``(nx, ny, nz)`` cells, face grid ``a`` of
shape ``res + e_a``) for the host entry points, or CUDA tensors / objects with ``data_ptr()`` for the
device entry points (``device=True``).  Every call runs the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import SF_PREC_FP64, SF_PREC_LEARNED, SF_PREC_MIXED  # noqa: F401

__all__ = ["StaggeredGrid", "Context", "Pressure", "MagneticField", "Network", "SolveError", "options",
           "load_library", "SF_PREC_FP64", "SF_PREC_MIXED", "SF_PREC_LEARNED"]


def load_library():
    return _abi.load()


class SolveError(RuntimeError):
    def __init__(self, status, msg, stats=None):
        super().__init__(f"{msg} (status {status})")
        self.status = status
        self.stats = stats


@dataclass(frozen=True)
class StaggeredGrid:
    """StaggeredGrid(boundaryWidth, spacing, resolution, center) (core/StaggeredGrid.h:10-21)."""
    boundary_width: int
    spacing: float
    resolution: tuple
    center: tuple = (0.0, 0.0, 0.0)

    @property
    def origin(self):
        # m_Origin = center - resolution * spacing / 2
        return tuple(float(c) - float(r) * float(self.spacing) / 2 for c, r in zip(self.center, self.resolution))

    @property
    def shape(self):
        return tuple(int(r) for r in self.resolution)

    @property
    def num_cells(self):
        nx, ny, nz = self.shape
        return nx * ny * nz

    def face_shape(self, axis):
        s = list(self.shape)
        s[axis] += 1
        return tuple(s)

    def domain_origin(self):
        return tuple(o + self.boundary_width * self.spacing for o in self.origin)

    @staticmethod
    def from_origin(spacing, resolution, origin=(0.0, 0.0, 0.0), boundary_width=0):
        """Grid whose corner is ``origin`` (center computed back from it)."""
        center = tuple(float(o) + float(r) * float(spacing) / 2 for o, r in zip(origin, resolution))
        g = StaggeredGrid(boundary_width, spacing, tuple(resolution), center)
        return g

    def c_grid(self, origin=None):
        g = _abi.sf_grid()
        g.nx, g.ny, g.nz = self.shape
        g.h = float(self.spacing)
        o = self.origin if origin is None else origin
        for a in range(3):
            g.origin[a] = float(o[a])
        return g


def options(which="pressure", **kw):
    """sf_solve_opts with the library defaults (tol 1e-8 pressure, 1e-6 magnetic) updated by ``kw``.

    ``precision`` accepts "fp64" / "mixed" or the SF_PREC_* constants."""
    lib = load_library()
    o = _abi.sf_solve_opts()
    lib.sf_default_opts(C.byref(o), 0 if which == "pressure" else 1)
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = {"fp64": SF_PREC_FP64, "mixed": SF_PREC_MIXED, "learned": SF_PREC_LEARNED}[v]
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class Context:
    """One CUDA stream and the device workspaces of both solvers (sf_create / sf_destroy)."""

    def __init__(self, device: int = 0, stream=None):
        self.lib = load_library()
        h = C.c_void_p()
        s = self.lib.sf_create(int(device), C.c_void_p(int(stream) if stream is not None else 0), C.byref(h))
        if s != _abi.SF_OK:
            raise SolveError(s, "sf_create failed: " + self.lib.sf_status_string(s).decode())
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self.network = None
            self.lib.sf_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self):
        return self.lib.sf_last_error(self.handle).decode()

    def device_bytes(self):
        return int(self.lib.sf_device_bytes(self.handle))

    def upload_collider(self, grid, fraction, solid_velocity=None):
        """Keep the collider's face fractions (and velocity) on the device (sf_collider_upload); pressure calls
        given fraction=None read them.  Arrays: numpy (host) or CUDA tensors."""
        ptr = lambda a: int(a.data_ptr()) if hasattr(a, "data_ptr") else np.ascontiguousarray(a, np.float64).ctypes.data  # noqa: E731
        keep = [a if hasattr(a, "data_ptr") else np.ascontiguousarray(a, np.float64) for a in fraction]
        us = None
        if solid_velocity is not None:
            keep += [a if hasattr(a, "data_ptr") else np.ascontiguousarray(a, np.float64) for a in solid_velocity]
            us = _abi.p3_ref([ptr(a) for a in keep[3:]])
        s = self.lib.sf_collider_upload(self.handle, C.byref(grid.c_grid()), _abi.p3([ptr(a) for a in keep[:3]]),
                                        us[0] if us else None)
        if s != _abi.SF_OK:
            raise SolveError(s, "sf_collider_upload: " + self.last_error())

    def upload_level_set(self, grid, level_set):
        """Keep a cell level set on the device for the substep's solves (sf_levelset_upload); calls given
        level_set=None read it.  Array: numpy (host) or a CUDA tensor."""
        a = level_set if hasattr(level_set, "data_ptr") else np.ascontiguousarray(level_set, np.float64)
        p = int(a.data_ptr()) if hasattr(a, "data_ptr") else a.ctypes.data
        s = self.lib.sf_levelset_upload(self.handle, C.byref(grid.c_grid()), C.c_void_p(p))
        if s != _abi.SF_OK:
            raise SolveError(s, "sf_levelset_upload: " + self.last_error())

    def prefetch_applied_field(self, grid, field):
        """Copy a later magnetic call's applied field asynchronously (sf_applied_field_prefetch): the copy runs
        under the next pressure projection; MagneticField.solve with external_field=None reads it.  Arrays: numpy
        (host; pinned memory gives a truly asynchronous copy) or CUDA tensors.  They are kept referenced here and
        must stay unchanged until that magnetic call returns."""
        keep = [a if hasattr(a, "data_ptr") else np.ascontiguousarray(a, np.float64) for a in field]
        ptr = lambda a: int(a.data_ptr()) if hasattr(a, "data_ptr") else a.ctypes.data  # noqa: E731
        s = self.lib.sf_applied_field_prefetch(self.handle, C.byref(grid.c_grid()), _abi.p3([ptr(a) for a in keep]))
        if s != _abi.SF_OK:
            raise SolveError(s, "sf_applied_field_prefetch: " + self.last_error())
        self._prefetched_field = keep

    def set_network(self, net):
        """Attach the U-Net used by precision="learned" solves (None detaches)."""
        s = self.lib.sf_set_network(self.handle, net.handle if net is not None else None)
        if s != _abi.SF_OK:
            raise SolveError(s, self.last_error())
        self.network = net

    def system_operator(self, which, shape):
        """(diag, [lower_x, lower_y, lower_z], rhs) of the last assembled system (0 pressure, 1 potential), as
        host arrays of the cell grid's shape (sf_system_operator)."""
        diag, rhs = np.empty(shape), np.empty(shape)
        lower = [np.empty(shape) for _ in range(3)]
        lp = _abi.p3_ref([a.ctypes.data for a in lower])
        s = self.lib.sf_system_operator(self.handle, int(which), C.c_void_p(diag.ctypes.data), lp[0],
                                        C.c_void_p(rhs.ctypes.data))
        if s != _abi.SF_OK:
            raise SolveError(s, "sf_system_operator: " + self.last_error())
        return diag, lower, rhs

    def system_features(self, which, features=None, solution=None):
        """Network features (BF16 [n][16], device) and FP32 solution of the last pressure (0) / potential (1)
        system assembled on this context; arguments are CUDA tensors or None."""
        s = self.lib.sf_system_features_dev(self.handle, int(which),
                                            C.c_void_p(features.data_ptr()) if features is not None else None,
                                            C.c_void_p(solution.data_ptr()) if solution is not None else None)
        if s != _abi.SF_OK:
            raise SolveError(s, self.last_error())


class Network:
    """The learned solver's 3D U-Net on a context (sf_unet_*).  Features and outputs are CUDA tensors."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        s = ctx.lib.sf_unet_create(ctx.handle, C.byref(h))
        if s != _abi.SF_OK:
            raise SolveError(s, "sf_unet_create: " + ctx.last_error())
        self.handle = h
        self.num_params = int(ctx.lib.sf_unet_num_params(h))

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.sf_unet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, s, what):
        if s != _abi.SF_OK:
            raise SolveError(s, f"{what}: {self.ctx.last_error()}")

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, dtype=np.float32)
        self._ok(self.ctx.lib.sf_unet_set_params(self.handle, flat.ctypes.data, flat.size), "set_params")

    def get_params(self):
        out = np.empty(self.num_params, np.float32)
        self._ok(self.ctx.lib.sf_unet_get_params(self.handle, out.ctypes.data, out.size), "get_params")
        return out

    def forward(self, grid: StaggeredGrid, features, out):
        self._ok(self.ctx.lib.sf_unet_forward_dev(self.handle, C.byref(grid.c_grid()), features.data_ptr(),
                                                   out.data_ptr()), "forward")
        return out

    def gradients(self, grid: StaggeredGrid, features, dout):
        g = np.empty(self.num_params, np.float32)
        self._ok(self.ctx.lib.sf_unet_backward_dev(self.handle, C.byref(grid.c_grid()), features.data_ptr(),
                                                    dout.data_ptr(), g.ctypes.data), "backward")
        return g

    def train_step(self, grid: StaggeredGrid, features, target, lr):
        loss = C.c_double()
        self._ok(self.ctx.lib.sf_unet_train_step_dev(self.handle, C.byref(grid.c_grid()), features.data_ptr(),
                                                      target.data_ptr(), float(lr), C.byref(loss)), "train_step")
        return loss.value

    def set_mode(self, mode):
        """Convolution kernels: "tcgen05" (default: TMA + TMEM for the forward, input-gradient and weight-gradient
        convolutions), "mma" (warp-level mma.sync) or "tcgen05_wgrad" (tcgen05 for the weight gradient alone)."""
        m = {"mma": 0, "tcgen05": 1, "tcgen05_wgrad": 2}.get(mode, mode)
        self._ok(self.ctx.lib.sf_unet_set_mode(self.handle, int(m)), "set_mode")

    def tc_launches(self):
        return int(self.ctx.lib.sf_unet_tc_launches(self.handle))

    def save(self, path):
        self.get_params().tofile(path)

    def load(self, path):
        flat = np.fromfile(path, dtype=np.float32)
        if flat.size != self.num_params:
            raise ValueError(f"{path}: {flat.size} parameters, expected {self.num_params}")
        self.set_params(flat)


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _host_f64(a, shape, name, writable=False):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        if writable:
            raise TypeError(f"{name}: must be a C-contiguous float64 numpy array (updated in place)")
        a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != tuple(shape) and a.size != int(np.prod(shape)):
        raise ValueError(f"{name}: shape {a.shape}, expected {tuple(shape)}")
    return a


def _ptr(a, shape, name, device, writable=False, keep=None):
    if a is None:
        return None
    if device:
        n = a.numel() if hasattr(a, "numel") else None
        if n is not None and n != int(np.prod(shape)):
            raise ValueError(f"{name}: {n} elements, expected {int(np.prod(shape))}")
        return int(a.data_ptr())
    a = _host_f64(a, shape, name, writable)
    if keep is not None:
        keep.append(a)
    return a.ctypes.data


def _check(ctx, status, stats, what, raise_on_nonconv):
    if status == _abi.SF_OK or status == _abi.SF_STALLED_FALLBACK:
        return
    if status == _abi.SF_NOT_CONVERGED and not raise_on_nonconv:
        return
    raise SolveError(status, f"{what}: {ctx.last_error()}", stats)


class Pressure:
    """Ghost-fluid pressure projection (core/Pressure.h:8-56) on the GPU."""

    def __init__(self, sgrid: StaggeredGrid, ctx: Context | None = None):
        self.grid = sgrid
        self.ctx = ctx or default_context()
        self.jump = None
        self.pressure = None
        self.stats = None

    def set_pressure_jump(self, jump):
        """Per-face J(axis, face) = p_liquid - p_air on liquid-air faces (three face arrays), or None.

        The reference takes a callback J(axis, face, theta) (core/Pressure.h:20-22); the shipped one ignores
        theta (core/Simulation.cpp:216-235), so an array of its values per face is equivalent."""
        self.jump = jump

    def _call(self, fn, velocity, level_set, fraction, solid_velocity, vol_error, opts, device, p_out,
              raise_on_nonconv):
        g = self.grid
        keep = []
        fs = [g.face_shape(a) for a in range(3)]
        vel = [_ptr(velocity[a], fs[a], f"velocity[{a}]", device, True, keep) for a in range(3)]
        fr = None if fraction is None else [_ptr(fraction[a], fs[a], f"fraction[{a}]", device, False, keep)
                                             for a in range(3)]
        phi = _ptr(level_set, g.shape, "level_set", device, False, keep)
        us = None if solid_velocity is None else [_ptr(solid_velocity[a], fs[a], "solid_velocity", device,
                                                       False, keep) for a in range(3)]
        jp = None if self.jump is None else [_ptr(self.jump[a], fs[a], "jump", device, False, keep)
                                             for a in range(3)]
        if p_out is None and not device:
            p_out = np.zeros(g.shape)
        elif p_out is False:  # no pressure output (the reference keeps p private)
            p_out = None
        pp = _ptr(p_out, g.shape, "p_out", device, True) if p_out is not None else None
        us_ref = _abi.p3_ref(us)
        jp_ref = _abi.p3_ref(jp)
        fr_ref = _abi.p3_ref(fr)
        st = _abi.sf_solve_stats()
        o = opts if opts is not None else options("pressure")
        s = fn(self.ctx.handle, C.byref(g.c_grid()), _abi.p3(vel), C.c_void_p(phi), fr_ref[0] if fr_ref else None,
               us_ref[0] if us_ref else None, jp_ref[0] if jp_ref else None, float(vol_error),
               C.c_void_p(pp) if pp else None, C.byref(o), C.byref(st))
        self.stats = st.as_dict()
        _check(self.ctx, s, self.stats, "pressure projection", raise_on_nonconv)
        self.pressure = p_out
        self.status = s
        return self.stats

    def project(self, velocity, level_set, fraction, solid_velocity=None, vol_error=0.0, opts=None, device=False,
                p_out=None, raise_on_nonconv=True):
        """Pressure::Project: velocity (3 face arrays) is updated in place; returns the solve statistics.
        level_set / fraction None: the context's uploaded level set / collider (Context.upload_*)."""
        fn = self.ctx.lib.sf_pressure_project_dev if device else self.ctx.lib.sf_pressure_project
        return self._call(fn, velocity, level_set, fraction, solid_velocity, vol_error, opts, device, p_out,
                          raise_on_nonconv)

    def reproject(self, velocity, level_set, fraction, solid_velocity=None, vol_error=0.0, opts=None, device=False,
                  p_out=None, raise_on_nonconv=True):
        """Pressure::Reproject: same unknowns and matrix as the last project(), new right-hand side."""
        fn = self.ctx.lib.sf_pressure_reproject_dev if device else self.ctx.lib.sf_pressure_reproject
        return self._call(fn, velocity, level_set, fraction, solid_velocity, vol_error, opts, device, p_out,
                          raise_on_nonconv)


class MagneticField:
    """FDM magnetostatic potential (core/MagneticField.h:15-71) on the GPU."""

    def __init__(self, sgrid: StaggeredGrid, susceptibility: float, band_width: float, ctx: Context | None = None):
        self.grid = sgrid
        self.ctx = ctx or default_context()
        self.chi = float(susceptibility)
        self.band_width = float(band_width)
        self.potential = None
        self.total_field = None
        self.stats = None
        self.ctx.lib.sf_magnetic_reset(self.ctx.handle)  # m_Sol starts at zero (core/MagneticField.cpp:26)

    def set_susceptibility(self, chi):
        self.chi = float(chi)

    def set_band_width(self, bw):
        self.band_width = float(bw)

    def solve(self, level_set, external_field, opts=None, device=False, psi_out=None, H_out=None,
              raise_on_nonconv=True):
        """MagneticField::Solve: returns statistics; ``potential`` and ``total_field`` hold the results.
        level_set None: the context's uploaded level set; external_field None: the context's prefetched applied
        field (Context.prefetch_applied_field); psi_out False: no potential output."""
        g = self.grid
        keep = []
        fs = [g.face_shape(a) for a in range(3)]
        phi = _ptr(level_set, g.shape, "level_set", device, False, keep)
        he = None if external_field is None else \
            [_ptr(external_field[a], fs[a], f"external_field[{a}]", device, False, keep) for a in range(3)]
        if not device:
            if psi_out is None:
                psi_out = np.zeros(g.shape)
            if H_out is None:
                H_out = [np.zeros(fs[a]) for a in range(3)]
        if psi_out is False:  # no potential output (the reference keeps psi private)
            psi_out = None
        pp = _ptr(psi_out, g.shape, "psi_out", device, True) if psi_out is not None else None
        hp = None if H_out is None else [_ptr(H_out[a], fs[a], "H_out", device, True) for a in range(3)]
        hp_ref = _abi.p3_ref(hp)
        he_ref = _abi.p3_ref(he)
        st = _abi.sf_solve_stats()
        o = opts if opts is not None else options("magnetic")
        fn = self.ctx.lib.sf_magnetic_solve_dev if device else self.ctx.lib.sf_magnetic_solve
        s = fn(self.ctx.handle, C.byref(g.c_grid()), C.c_void_p(phi), self.chi, self.band_width,
               he_ref[0] if he_ref else None,
               C.c_void_p(pp) if pp else None, hp_ref[0] if hp_ref else None, C.byref(o), C.byref(st))
        self.stats = st.as_dict()
        _check(self.ctx, s, self.stats, "magnetic solve", raise_on_nonconv)
        self.potential = psi_out
        self.total_field = H_out
        self.status = s
        return self.stats

    def calculate_vertex_pressures(self, positions, normals, H=None, device=False, out=None):
        """MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48) at the mesh vertices
        (positions, normals: nverts x 3) from H (default: the total field of the last solve)."""
        g, keep = self.grid, []
        H = self.total_field if H is None else H
        if H is None:
            raise ValueError("no total field: solve first or pass H")
        fs = [g.face_shape(a) for a in range(3)]
        hp = [_ptr(H[a], fs[a], f"H[{a}]", device, False, keep) for a in range(3)]
        nv = int(positions.shape[0]) if hasattr(positions, "shape") else len(positions) // 3
        if not device:
            positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
            normals = np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, 3)
            if out is None:
                out = np.empty(nv)
        pp = _ptr(positions, (nv, 3), "positions", device, False, keep)
        np_ = _ptr(normals, (nv, 3), "normals", device, False, keep)
        op = _ptr(out, (nv,), "out", device, True)
        fn = self.ctx.lib.sf_magnetic_vertex_pressures_dev if device else self.ctx.lib.sf_magnetic_vertex_pressures
        st = fn(self.ctx.handle, C.byref(g.c_grid()), self.chi, _abi.p3(hp), C.c_void_p(pp), C.c_void_p(np_), nv,
                C.c_void_p(op))
        _check(self.ctx, st, None, "vertex pressures", True)
        return out


def pressure_jump(sgrid: StaggeredGrid, edge_mark, curvature=None, mag_pressure=None, st_coeff=0.0, density=1.0,
                  dt=1.0, ctx: Context | None = None, device=False, out=None):
    """The pressure jump of core/Simulation.cpp:216-235 on every face (three face arrays) from the contour's edge
    marks (int32 per cell-grid edge, -1 = no vertex), vertex curvatures and vertex magnetic pressures."""
    ctx = ctx or default_context()
    g, keep = sgrid, []
    fs = [g.face_shape(a) for a in range(3)]
    es = [tuple(g.shape[b] - (b == a) for b in range(3)) for a in range(3)]
    if device:
        em = [int(edge_mark[a].data_ptr()) for a in range(3)]
    else:
        ems = [np.ascontiguousarray(edge_mark[a], dtype=np.int32) for a in range(3)]
        for a in range(3):
            if ems[a].size != int(np.prod(es[a])):
                raise ValueError(f"edge_mark[{a}]: {ems[a].size} entries, expected {int(np.prod(es[a]))}")
        keep += ems
        em = [e.ctypes.data for e in ems]
    nv = 0
    for v in (curvature, mag_pressure):
        if v is not None:
            nv = int(v.numel()) if hasattr(v, "numel") else int(np.asarray(v).size)
    kp = _ptr(curvature, (nv,), "curvature", device, False, keep) if curvature is not None else None
    mp = _ptr(mag_pressure, (nv,), "mag_pressure", device, False, keep) if mag_pressure is not None else None
    if out is None and not device:
        out = [np.zeros(fs[a]) for a in range(3)]
    jp = [_ptr(out[a], fs[a], f"jump[{a}]", device, True) for a in range(3)]
    fn = ctx.lib.sf_pressure_jump_dev if device else ctx.lib.sf_pressure_jump
    st = fn(ctx.handle, C.byref(g.c_grid()), _abi.p3(em), C.c_void_p(kp) if kp else None,
            C.c_void_p(mp) if mp else None, nv, float(st_coeff), float(density), float(dt), _abi.p3(jp))
    _check(ctx, st, None, "pressure jump", True)
    return out


# ------------------------------------------------------------------------------------------------ velocity pipeline
def collider_face_normals(sgrid: StaggeredGrid, node_level_set):
    """Collider::Finish normals (core/Collider.cpp:30-44) from the collider's node level set (host)."""
    lib = load_library()
    ls = np.ascontiguousarray(node_level_set, dtype=np.float64)
    normal = [np.empty(sgrid.face_shape(a)) for a in range(3)]
    s = lib.sf_collider_face_normals(C.byref(sgrid.c_grid()), C.c_void_p(ls.ctypes.data),
                                     _abi.p3([n.ctypes.data for n in normal]))
    if s != _abi.SF_OK:
        raise SolveError(s, "sf_collider_face_normals: " + lib.sf_status_string(s).decode())
    return normal


class Extrapolation:
    """Extrapolation::Solve of the projected velocity (core/Extrapolation.cpp:4-30) with the simulation's
    validity predicate (core/Simulation.cpp:237-240), on the GPU."""

    def __init__(self, sgrid: StaggeredGrid, ctx: Context | None = None):
        self.grid = sgrid
        self.ctx = ctx or default_context()

    def solve(self, velocity, level_set, fraction, clear_val=0.0, max_steps=6, device=False):
        g, keep = self.grid, []
        fs = [g.face_shape(a) for a in range(3)]
        vel = [_ptr(velocity[a], fs[a], f"velocity[{a}]", device, True, keep) for a in range(3)]
        fr = None if fraction is None else [_ptr(fraction[a], fs[a], f"fraction[{a}]", device, False, keep)
                                             for a in range(3)]
        phi = _ptr(level_set, g.shape, "level_set", device, False, keep)
        fn = self.ctx.lib.sf_extrapolate_velocity_dev if device else self.ctx.lib.sf_extrapolate_velocity
        s = fn(self.ctx.handle, C.byref(g.c_grid()), _abi.p3(vel), C.c_void_p(phi), _abi.p3(fr), float(clear_val),
               int(max_steps))
        _check(self.ctx, s, None, "velocity extrapolation", True)


class ColliderEnforce:
    """Collider::Enforce (core/Collider.cpp:75-86) with the collider's fractions and face normals, on the GPU."""

    def __init__(self, sgrid: StaggeredGrid, fraction, normal, solid_velocity=None, ctx: Context | None = None):
        self.grid = sgrid
        self.ctx = ctx or default_context()
        self.fraction, self.normal, self.solid_velocity = fraction, normal, solid_velocity

    def enforce(self, velocity, device=False):
        g, keep = self.grid, []
        fs = [g.face_shape(a) for a in range(3)]
        vel = [_ptr(velocity[a], fs[a], f"velocity[{a}]", device, True, keep) for a in range(3)]
        fr = [_ptr(self.fraction[a], fs[a], f"fraction[{a}]", device, False, keep) for a in range(3)]
        nm = [_ptr(self.normal[a], fs[a], f"normal[{a}]", device, False, keep) for a in range(3)]
        us = None if self.solid_velocity is None else [
            _ptr(self.solid_velocity[a], fs[a], "solid_velocity", device, False, keep) for a in range(3)]
        us_ref = _abi.p3_ref(us)
        fn = self.ctx.lib.sf_collider_enforce_dev if device else self.ctx.lib.sf_collider_enforce
        s = fn(self.ctx.handle, C.byref(g.c_grid()), _abi.p3(vel), _abi.p3(fr), _abi.p3(nm),
               us_ref[0] if us_ref else None)
        _check(self.ctx, s, None, "collider enforce", True)


# ------------------------------------------------------------------------------------------------ level set
class Advection:
    """Advection::Solve<2> (core/Advection.h:33-59) on the GPU: semi-Lagrangian with the TVD RK2 trace."""

    def __init__(self, sgrid: StaggeredGrid, ctx: Context | None = None):
        self.grid = sgrid
        self.ctx = ctx or default_context()

    def solve_levelset(self, level_set, velocity, dt, device=False):
        """Advection::Solve<2>(levelSet, velocity, dt): the level set (updated in place), tricubic."""
        g, keep = self.grid, []
        fs = [g.face_shape(a) for a in range(3)]
        phi = _ptr(level_set, g.shape, "level_set", device, True, keep)
        vel = [_ptr(velocity[a], fs[a], f"velocity[{a}]", device, False, keep) for a in range(3)]
        fn = self.ctx.lib.sf_advect_levelset_dev if device else self.ctx.lib.sf_advect_levelset
        s = fn(self.ctx.handle, C.byref(g.c_grid()), C.c_void_p(phi), _abi.p3(vel), float(dt))
        _check(self.ctx, s, None, "level-set advection", True)

    def solve_velocity(self, velocity, dt, device=False):
        """Advection::Solve<2>(velocity, velocity, dt): the velocity advected by itself (in place), trilinear."""
        g, keep = self.grid, []
        fs = [g.face_shape(a) for a in range(3)]
        vel = [_ptr(velocity[a], fs[a], f"velocity[{a}]", device, True, keep) for a in range(3)]
        fn = self.ctx.lib.sf_advect_velocity_dev if device else self.ctx.lib.sf_advect_velocity
        s = fn(self.ctx.handle, C.byref(g.c_grid()), _abi.p3(vel), float(dt))
        _check(self.ctx, s, None, "velocity advection", True)


class Reinitialization:
    """Reinitialization::Solve (core/Reinitialization.cpp:36-76) on the GPU: WENO5 + TVD-RK3, dt = h/2."""

    def __init__(self, sgrid: StaggeredGrid, ctx: Context | None = None):
        self.grid = sgrid
        self.ctx = ctx or default_context()

    def solve(self, level_set, max_steps=10, device=False):
        g, keep = self.grid, []
        phi = _ptr(level_set, g.shape, "level_set", device, True, keep)
        fn = self.ctx.lib.sf_reinitialize_dev if device else self.ctx.lib.sf_reinitialize
        s = fn(self.ctx.handle, C.byref(g.c_grid()), C.c_void_p(phi), int(max_steps))
        _check(self.ctx, s, None, "reinitialization", True)
