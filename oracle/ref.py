"""ctypes wrapper over ``oracle/_ref/libsfref.so``: the reference's own hot-path C++ sources compiled
unmodified against the stand-in headers in ``oracle/refshim`` (recipe: ``oracle/ref.mk``, driver:
``oracle/ref_driver.cpp``).

TEST INFRASTRUCTURE ONLY: it pins the C oracle to the reference's code.  It is built only where the
reference's sources are present; tests that need it skip elsewhere, and ``tests/golden/make_ref_golden.py``
records its outputs as committed fixtures so that the pin is checked everywhere.

Arrays use the reference's layout (core/Grid.h:28), as in ``oracle.py``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libsfref.so")
REF_DEFAULT = "/root/reference"

_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_D3 = _D * 3


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double),
                ("ox", C.c_double), ("oy", C.c_double), ("oz", C.c_double)]


def ref_sources(ref: str | None = None) -> str | None:
    ref = ref or os.environ.get("SF_REFERENCE_DIR", REF_DEFAULT)
    return ref if os.path.exists(os.path.join(ref, "core", "Pressure.cpp")) else None


def build(ref: str | None = None) -> str | None:
    """make -f oracle/ref.mk where the reference's sources exist; returns the library path or None."""
    src = ref_sources(ref)
    if src is None:
        return LIB if os.path.exists(LIB) else None
    subprocess.check_call(["make", "-s", "-f", os.path.join(HERE, "ref.mk"), f"REF={src}", "-j8"],
                          cwd=os.path.dirname(HERE))
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FileNotFoundError(LIB)
        L = C.CDLL(LIB)
        G = C.POINTER(_Grid)
        V = C.c_void_p
        L.ref_session_new.argtypes = [G, C.c_int]
        L.ref_session_new.restype = V
        L.ref_session_free.argtypes = [V]
        L.ref_collider_finish.argtypes = [V, _D, V, V]
        L.ref_collider_set.argtypes = [V, V, V, V]
        L.ref_pressure_project.argtypes = [V, C.c_int, _D, V, C.c_double, _D3, C.c_int, V, C.c_double,
                                           V, V, V, V, V, V, V, V]
        L.ref_pressure_project.restype = C.c_int64
        L.ref_magnetic_solve.argtypes = [V, C.c_double, C.c_double, _D, _D3, C.c_int, V, C.c_double,
                                         V, V, V, V, V, V, V, V, V, V]
        L.ref_vertex_pressures.argtypes = [V, C.c_double, _D3, _D, _D, C.c_int64, _D]
        L.ref_extrapolate_velocity.argtypes = [V, _D3, _D, C.c_double, C.c_int]
        L.ref_collider_enforce.argtypes = [V, _D3]
        L.ref_advect_levelset.argtypes = [V, _D, _D3, C.c_double]
        L.ref_advect_velocity.argtypes = [V, _D3, C.c_double]
        L.ref_reinitialize.argtypes = [V, _D, C.c_int]
        L.ref_fast_marching.argtypes = [V, _D, C.c_int]
        L.ref_last_solve_iters.restype = C.c_int64
        L.ref_csg_union.argtypes = [V, _D, C.c_int, _D, _D, C.c_double]
        L.ref_domain.argtypes = [V, _D, _D]
        _lib = L
    return _lib


def available() -> bool:
    return os.path.exists(LIB)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t=_D):
    return a.ctypes.data_as(t)


def _vp(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _faces_ptr(arrs):
    """(kept arrays, void* to a double*[3]) or (None, None)."""
    if arrs is None:
        return None, None
    arrs = [_f64(a) for a in arrs]
    p = _D3(*[_p(a) for a in arrs])
    return (arrs, p), C.cast(C.pointer(p), C.c_void_p)


class Session:
    """A simulation grid of the reference with its Collider, Pressure and MagneticField objects."""

    def __init__(self, nx, ny, nz, h, origin=(0.0, 0.0, 0.0), bw=0):
        self.shape = (nx, ny, nz)
        self.N = nx * ny * nz
        self.g = _Grid(nx, ny, nz, float(h), *map(float, origin))
        self.h = lib().ref_session_new(C.byref(self.g), int(bw))

    def close(self):
        if self.h:
            lib().ref_session_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def face_shape(self, a):
        s = list(self.shape)
        s[a] += 1
        return tuple(s)

    def node_shape(self):
        return tuple(n + 1 for n in self.shape)

    def _faces_out(self):
        arrs = [np.zeros(self.face_shape(a)) for a in range(3)]
        p = _D3(*[_p(a) for a in arrs])
        return arrs, p

    # ------------------------------------------------------------------------------------ collider
    def collider_finish(self):
        ls = np.empty(self.node_shape())
        frac, fp = self._faces_out()
        nrm, npp = self._faces_out()
        lib().ref_collider_finish(self.h, _p(ls), C.cast(C.pointer(fp), C.c_void_p),
                                  C.cast(C.pointer(npp), C.c_void_p))
        return ls, frac, nrm

    def collider_set(self, frac=None, normal=None, solid_vel=None):
        k1, f = _faces_ptr(frac)
        k2, n = _faces_ptr(normal)
        k3, s = _faces_ptr(solid_vel)
        lib().ref_collider_set(self.h, f, n, s)

    # ------------------------------------------------------------------------------------ pressure
    def pressure_project(self, phi, vel, jump=None, vol_error=0.0, mode=2, p_inject=None, tol=1e-13,
                         reproject=False):
        """Pressure::Project / Reproject.  mode 0: keep the initial guess, 1: inject p_inject (reduced),
        2: Jacobi-PCG to tol.  Returns a dict: u (new face velocities), n, A (rowptr, col, val; Project
        only), rhs, x0, p (reduced), grid2mat, tol (the tolerance handed to amgcl)."""
        phi = _f64(phi)
        u = [_f64(a).copy() for a in vel]
        up = _D3(*[_p(a) for a in u])
        kj, jp = _faces_ptr(jump)
        n_max = self.N
        rowptr = np.zeros(n_max + 1, np.int64)
        col = np.zeros(7 * n_max, np.int32)
        val = np.zeros(7 * n_max)
        rhs = np.zeros(max(n_max, 1))
        x0 = np.zeros(max(n_max, 1))
        sol = np.zeros(max(n_max, 1))
        g2m = np.zeros(self.N, np.int32)
        tol_seen = C.c_double(-1.0)
        pin = None if p_inject is None else _f64(p_inject)
        n = lib().ref_pressure_project(self.h, int(reproject), _p(phi), jp, float(vol_error), up, int(mode),
                                       _vp(pin), float(tol), _vp(rowptr), _vp(col), _vp(val), _vp(rhs),
                                       _vp(x0), _vp(sol), _vp(g2m), C.c_void_p(C.addressof(tol_seen)))
        out = dict(u=u, n=int(n), rhs=rhs[:n].copy(), x0=x0[:n].copy(), p=sol[:n].copy(), grid2mat=g2m,
                   tol=tol_seen.value, iters=int(lib().ref_last_solve_iters()))
        if not reproject:
            nnz = int(rowptr[n])
            out.update(rowptr=rowptr[:n + 1].copy(), col=col[:nnz].copy(), val=val[:nnz].copy())
        return out

    # ------------------------------------------------------------------------------------ magnetic
    def magnetic_solve(self, chi, band_width, phi, hext, mode=2, psi_inject=None, tol=1e-13):
        """MagneticField::Solve on the session's MagneticField (warm start m_Sol kept across calls).
        Returns mu, A (rowptr, col, val), rhs, x0, psi, H, tol (handed to amgcl) and the field grid's corner."""
        phi = _f64(phi)
        he = [_f64(a) for a in hext]
        hp = _D3(*[_p(a) for a in he])
        N = self.N
        mu, mup = self._faces_out()
        H, Hp = self._faces_out()
        rowptr = np.zeros(N + 1, np.int64)
        col = np.zeros(7 * N, np.int32)
        val = np.zeros(7 * N)
        rhs = np.zeros(N)
        x0 = np.zeros(N)
        psi = np.zeros(self.shape)
        tol_seen = C.c_double(-1.0)
        org = np.zeros(3)
        pin = None if psi_inject is None else _f64(psi_inject)
        lib().ref_magnetic_solve(self.h, float(chi), float(band_width), _p(phi), hp, int(mode), _vp(pin),
                                 float(tol), C.cast(C.pointer(mup), C.c_void_p), _vp(rowptr), _vp(col),
                                 _vp(val), _vp(rhs), _vp(x0), _vp(psi), C.cast(C.pointer(Hp), C.c_void_p),
                                 C.c_void_p(C.addressof(tol_seen)), _vp(org))
        nnz = int(rowptr[N])
        return dict(mu=mu, rowptr=rowptr, col=col[:nnz].copy(), val=val[:nnz].copy(), rhs=rhs, x0=x0,
                    psi=psi, H=H, tol=tol_seen.value, origin_ext=org, iters=int(lib().ref_last_solve_iters()))

    def vertex_pressures(self, chi, H, positions, normals):
        hh = [_f64(a) for a in H]
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        nrm = np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, 3)
        out = np.empty(pos.shape[0])
        lib().ref_vertex_pressures(self.h, float(chi), _D3(*[_p(a) for a in hh]), _p(pos), _p(nrm),
                                   pos.shape[0], _p(out))
        return out

    # ------------------------------------------------------------------------------------ neighbours
    def extrapolate_velocity(self, vel, phi, clear_val=0.0, max_steps=6):
        u = [_f64(a).copy() for a in vel]
        lib().ref_extrapolate_velocity(self.h, _D3(*[_p(a) for a in u]), _p(_f64(phi)), float(clear_val),
                                       int(max_steps))
        return u

    def collider_enforce(self, vel):
        u = [_f64(a).copy() for a in vel]
        lib().ref_collider_enforce(self.h, _D3(*[_p(a) for a in u]))
        return u

    def advect_levelset(self, phi, vel, dt):
        out = _f64(phi).copy()
        uu = [_f64(a) for a in vel]
        lib().ref_advect_levelset(self.h, _p(out), _D3(*[_p(a) for a in uu]), float(dt))
        return out

    def advect_velocity(self, vel, dt):
        u = [_f64(a).copy() for a in vel]
        lib().ref_advect_velocity(self.h, _D3(*[_p(a) for a in u]), float(dt))
        return u

    def reinitialize(self, phi, max_steps=10):
        out = _f64(phi).copy()
        lib().ref_reinitialize(self.h, _p(out), int(max_steps))
        return out

    def csg_union(self, phi, kind, a, b=(0.0, 0.0, 0.0), r=0.0):
        """CSG::Union of the cell level set with a plane (kind 0: point a, direction b), a sphere (1: centre a,
        radius r) or a box (2: min corner a, lengths b); phi=None starts from +infinity."""
        out = np.full(self.shape, np.inf) if phi is None else _f64(phi).copy()
        aa = _f64(np.asarray(a, dtype=np.float64))
        bb = _f64(np.asarray(b, dtype=np.float64))
        lib().ref_csg_union(self.h, _p(out), int(kind), _p(aa), _p(bb), float(r))
        return out

    def domain(self):
        o, l = np.zeros(3), np.zeros(3)
        lib().ref_domain(self.h, _p(o), _p(l))
        return o, l

    def fast_marching(self, node_ls, max_steps=-1):
        out = _f64(node_ls).copy()
        lib().ref_fast_marching(self.h, _p(out), int(max_steps))
        return out
