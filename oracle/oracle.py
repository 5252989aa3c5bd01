"""ctypes wrapper over the C oracle (``sf_oracle.c``).

TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA library.  Tests, the smoke check and the
CPU-baseline leg of the benchmark import this module; the product never does.

Parity pinned: every function here reproduces the reference's own compiled code bit for bit
(``oracle/_ref``, ``tests/test_ref_pin.py``; see the header of ``sf_oracle.c``).  Arrays use the reference's layout (core/Grid.h:28): cell arrays are C-contiguous
``(nx, ny, nz)`` float64, face arrays of axis a are ``(nx+(a==0), ny+(a==1), nz+(a==2))``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP, no FMA contraction) into oracle/_build/liboracle.so."""
    srcs = [os.path.join(HERE, f) for f in ("sf_oracle.c", "sf_amg.c", "sf_mgcpu.c")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
                           "-o", tmp, *srcs, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class _AmgInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("resid", C.c_double), ("levels", C.c_int), ("setup_s", C.c_double)]


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double),
                ("ox", C.c_double), ("oy", C.c_double), ("oz", C.c_double)]


@dataclass(frozen=True)
class Grid:
    """Cell grid of a staggered grid: resolution, spacing and the corner (StaggeredGrid::GetOrigin)."""
    nx: int
    ny: int
    nz: int
    h: float
    origin: tuple = (0.0, 0.0, 0.0)

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz)

    @property
    def N(self):
        return self.nx * self.ny * self.nz

    def face_shape(self, a):
        s = list(self.shape)
        s[a] += 1
        return tuple(s)

    def c(self):
        return _Grid(self.nx, self.ny, self.nz, self.h, *map(float, self.origin))


_lib = None
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_D3 = _D * 3


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        G = C.POINTER(_Grid)
        L.or_pressure_unknowns.argtypes = [G, _D, _I32, _I64]
        L.or_pressure_unknowns.restype = C.c_int64
        L.or_pressure_assemble.argtypes = [G, _D, _D3, _D3, C.c_void_p, C.c_void_p, C.c_double, _I32, _I64,
                                           C.c_int64, _I64, _I32, _D, _D]
        L.or_pressure_assemble.restype = C.c_int64
        L.or_pressure_rhs.argtypes = [G, _D3, _D3, C.c_void_p, C.c_double, _I64, C.c_int64, _D]
        L.or_pressure_apply.argtypes = [G, _D, _D3, C.c_void_p, _I32, _D, _D3]
        L.or_magnetic_coeff.argtypes = [G, _D, C.c_double, C.c_double, _D3]
        L.or_magnetic_assemble.argtypes = [G, _D3, _I64, _I32, _D]
        L.or_magnetic_assemble.restype = C.c_int64
        L.or_magnetic_rhs.argtypes = [G, _D3, _D3, _D, _D]
        L.or_magnetic_total_field.argtypes = [G, _D, _D3, _D3]
        L.or_magnetic_grid_origin.argtypes = [G, _D]
        L.or_csr_spmv.argtypes = [C.c_int64, _I64, _I32, _D, _D, _D]
        L.or_csr_pcg.argtypes = [C.c_int64, _I64, _I32, _D, _D, _D, C.c_double, C.c_int, _D]
        L.or_csr_pcg.restype = C.c_int
        L.or_fast_marching.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _D]
        L.or_collider_box_levelset.argtypes = [G, C.c_int, _D]
        L.or_collider_face_fractions.argtypes = [G, _D, _D3]
        L.or_num_threads.restype = C.c_int
        L.or_extrapolate_velocity.argtypes = [G, _D3, _D, _D3, C.c_double, C.c_int]
        L.or_collider_face_normals.argtypes = [G, _D, _D3]
        L.or_collider_enforce.argtypes = [G, _D3, _D3, _D3, C.c_void_p]
        L.or_vertex_pressures.argtypes = [G, C.c_double, _D3, _D, _D, C.c_int64, _D]
        L.or_advect_levelset.argtypes = [G, _D, _D3, C.c_double, _D]
        L.or_advect_velocity.argtypes = [G, _D3, C.c_double, _D3]
        L.or_reinitialize.argtypes = [G, _D, C.c_int]
        L.or_pressure_jump.argtypes = [G, C.c_void_p * 3, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                       C.c_double, _D3]
        L.or_amg_solve.argtypes = [C.c_int, C.c_int64, _I64, _I32, _D, _D, _D, C.c_double, C.c_int,
                                   C.POINTER(_AmgInfo)]
        L.or_amg_solve.restype = C.c_int
        L.or_pressure_face_form.argtypes = [C.c_int, C.c_int, C.c_int, _I64, C.c_int64, _I64, _I32, _D, _D, _D, _D,
                                            _D, _D]
        L.or_magnetic_face_form.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D, _D, _D, _D, _D, _D]
        L.or_mgpcg_solve.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D, _D, _D, _D, _D, C.c_double, C.c_int,
                                     C.c_int, C.POINTER(C.c_double)]
        L.or_mgpcg_solve.restype = C.c_int
    return _lib


def _p(a, t=_D):
    return a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _faces(arrs):
    arrs = [_f64(a) for a in arrs]
    return arrs, _D3(*[_p(a) for a in arrs])


def _opt_faces(arrs):
    if arrs is None:
        return None, None
    arrs, p = _faces(arrs)
    return arrs, C.cast(C.pointer(p), C.c_void_p)


class CSR:
    def __init__(self, n, rowptr, col, val):
        self.n, self.rowptr, self.col, self.val = n, rowptr, col, val

    def matvec(self, x):
        x = _f64(x)
        y = np.empty(self.n)
        lib().or_csr_spmv(self.n, _p(self.rowptr, _I64), _p(self.col, _I32), _p(self.val), _p(x), _p(y))
        return y

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rowptr), shape=(self.n, self.n))

    def solve(self, b, x0=None, tol=1e-12, maxit=20000):
        """Jacobi-PCG to ||b - Ax|| <= tol ||b||; returns (x, iterations, true relative residual)."""
        x = np.zeros(self.n) if x0 is None else _f64(x0).copy()
        b = _f64(b)
        rr = C.c_double()
        it = lib().or_csr_pcg(self.n, _p(self.rowptr, _I64), _p(self.col, _I32), _p(self.val), _p(b), _p(x),
                              tol, maxit, C.byref(rr))
        return x, it, rr.value

    def amg_solve(self, b, kind, x0=None, tol=1e-8, maxit=100):
        """Restated amgcl path: SA-AMG (SPAI-0) preconditioning BiCGStab (kind 0) or CG (kind 1).

        Returns (x, info dict with iters, resid, levels, setup_s, converged)."""
        x = np.zeros(self.n) if x0 is None else _f64(x0).copy()
        b = _f64(b)
        inf = _AmgInfo()
        rc = lib().or_amg_solve(int(kind), self.n, _p(self.rowptr, _I64), _p(self.col, _I32), _p(self.val), _p(b),
                                _p(x), float(tol), int(maxit), C.byref(inf))
        return x, dict(iters=inf.iters, resid=inf.resid, levels=inf.levels, setup_s=inf.setup_s, converged=rc == 0)


# ------------------------------------------------------------------------------------------------ CPU MGPCG
def mgpcg_solve(g: Grid, form, b, tol, maxit=200, pairs=48):
    """The library's plain FP64 method (geometric-MG PCG, sf_mgcpu.c) on the host cores, from x = 0.
    form = (ax, ay, az, dex, D) on the cell grid; b on the cell grid.  Returns (x, iters, relres)."""
    ax, ay, az, dex, D = [_f64(a).reshape(-1) for a in form]
    b = _f64(b).reshape(-1)
    x = np.empty(g.N)
    rr = C.c_double()
    it = lib().or_mgpcg_solve(g.nx, g.ny, g.nz, _p(ax), _p(ay), _p(az), _p(dex), _p(D), _p(b), _p(x), float(tol),
                              int(maxit), int(pairs), C.byref(rr))
    if it < 0:
        raise MemoryError("or_mgpcg_solve: allocation failed")
    return x, it, rr.value


def _empty_form(g: Grid):
    return [np.empty(g.N) for _ in range(5)]


# ------------------------------------------------------------------------------------------------ pressure
def pressure_unknowns(g: Grid, phi):
    phi = _f64(phi)
    g2m = np.empty(g.N, np.int32)
    m2g = np.empty(g.N, np.int64)
    n = lib().or_pressure_unknowns(C.byref(g.c()), _p(phi), _p(g2m, _I32), _p(m2g, _I64))
    return g2m, m2g[:n].copy()


def pressure_assemble(g: Grid, phi, frac, u, us=None, jump=None, vol_error=0.0):
    """Pressure::SetUnKnowns + BuildProjectionMatrix.  Returns (CSR, rhs, grid2mat, mat2grid)."""
    phi = _f64(phi)
    g2m, m2g = pressure_unknowns(g, phi)
    n = len(m2g)
    fr, frp = _faces(frac)
    uu, up = _faces(u)
    usa, usp = _opt_faces(us)
    ja, jp = _opt_faces(jump)
    rowptr = np.zeros(n + 1, np.int64)
    col = np.empty(7 * max(n, 1), np.int32)
    val = np.empty(7 * max(n, 1))
    rhs = np.empty(max(n, 1))
    nnz = lib().or_pressure_assemble(C.byref(g.c()), _p(phi), frp, up, usp, jp, float(vol_error), _p(g2m, _I32),
                                     _p(m2g, _I64), n, _p(rowptr, _I64), _p(col, _I32), _p(val), _p(rhs))
    return CSR(n, rowptr, col[:nnz].copy(), val[:nnz].copy()), rhs[:n].copy(), g2m, m2g


def pressure_rhs(g: Grid, frac, u, us, vol_error, m2g):
    fr, frp = _faces(frac)
    uu, up = _faces(u)
    usa, usp = _opt_faces(us)
    rhs = np.empty(max(len(m2g), 1))
    lib().or_pressure_rhs(C.byref(g.c()), frp, up, usp, float(vol_error), _p(m2g, _I64), len(m2g), _p(rhs))
    return rhs[:len(m2g)].copy()


def pressure_apply(g: Grid, phi, frac, jump, g2m, p_reduced, u):
    """Pressure::ApplyProjection; returns new face velocities (inputs untouched)."""
    phi = _f64(phi)
    fr, frp = _faces(frac)
    ja, jp = _opt_faces(jump)
    out = [_f64(a).copy() for a in u]
    op = _D3(*[_p(a) for a in out])
    pr = _f64(p_reduced) if len(p_reduced) else np.zeros(1)
    lib().or_pressure_apply(C.byref(g.c()), _p(phi), frp, jp, _p(g2m, _I32), _p(pr), op)
    return out


def pressure_project(g: Grid, phi, frac, u, us=None, jump=None, vol_error=0.0, tol=1e-12, maxit=20000,
                     solver="pcg"):
    """Pressure::Project with the linear system solved to ``tol``: solver "pcg" (Jacobi-PCG, the parity
    reference) or "amg" (the restated amgcl SA-AMG + BiCGStab of core/Pressure.cpp:125-135, maxit 100).

    Returns (u_new, p_grid, info): p_grid is the pressure on every cell (0 in air cells)."""
    A, b, g2m, m2g = pressure_assemble(g, phi, frac, u, us, jump, vol_error)
    p_grid = np.zeros(g.N)
    if A.n == 0:
        return [_f64(a).copy() for a in u], p_grid.reshape(g.shape), dict(n=0, iters=0, relres=0.0)
    if solver == "amg":
        p, inf = A.amg_solve(b, 0, tol=tol, maxit=min(maxit, 100))
        it = inf["iters"]
        rr = float(np.linalg.norm(b - A.matvec(p)) / max(np.linalg.norm(b), 1e-300))
    elif solver == "mgpcg":
        form = _empty_form(g)
        lib().or_pressure_face_form(g.nx, g.ny, g.nz, _p(m2g, _I64), A.n, _p(A.rowptr, _I64), _p(A.col, _I32),
                                    _p(A.val), *[_p(a) for a in form])
        bg = np.zeros(g.N)
        bg[m2g] = b
        x, it, _ = mgpcg_solve(g, form, bg, tol, maxit=min(maxit, 200))
        p = x[m2g]
        rr = float(np.linalg.norm(b - A.matvec(p)) / max(np.linalg.norm(b), 1e-300))
    else:
        p, it, rr = A.solve(b, tol=tol, maxit=maxit)
    u_new = pressure_apply(g, phi, frac, jump, g2m, p, u)
    p_grid[m2g] = p
    return u_new, p_grid.reshape(g.shape), dict(n=A.n, iters=it, relres=rr, A=A, b=b, g2m=g2m, m2g=m2g)


# ------------------------------------------------------------------------------------------------ magnetic
def magnetic_grid_origin(g: Grid):
    out = np.zeros(3)
    lib().or_magnetic_grid_origin(C.byref(g.c()), _p(out))
    return out


def magnetic_coeff(g: Grid, phi, chi, band_width):
    phi = _f64(phi)
    mu = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_magnetic_coeff(C.byref(g.c()), _p(phi), float(chi), float(band_width), _D3(*[_p(a) for a in mu]))
    return mu


def magnetic_assemble(g: Grid, mu):
    m, mp = _faces(mu)
    rowptr = np.zeros(g.N + 1, np.int64)
    col = np.empty(7 * g.N, np.int32)
    val = np.empty(7 * g.N)
    nnz = lib().or_magnetic_assemble(C.byref(g.c()), mp, _p(rowptr, _I64), _p(col, _I32), _p(val))
    return CSR(g.N, rowptr, col[:nnz].copy(), val[:nnz].copy())


def magnetic_rhs(g: Grid, mu, hext):
    m, mp = _faces(mu)
    hx, hp = _faces(hext)
    rhs = np.empty(g.N)
    r0 = C.c_double()
    lib().or_magnetic_rhs(C.byref(g.c()), mp, hp, _p(rhs), C.byref(r0))
    return rhs, r0.value


def magnetic_total_field(g: Grid, psi, hext):
    psi = _f64(psi)
    hx, hp = _faces(hext)
    H = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_magnetic_total_field(C.byref(g.c()), _p(psi), hp, _D3(*[_p(a) for a in H]))
    return H


def magnetic_solve(g: Grid, phi, chi, band_width, hext, psi0=None, tol=1e-12, maxit=20000, solver="pcg"):
    """MagneticField::Solve with the pinned system solved to ``tol`` ("pcg", or "amg" = the restated amgcl
    SA-AMG + CG of core/MagneticField.cpp:92-94,120-123, warm start psi0; or "mgpcg" = the library's plain FP64
    method on the host cores, on the Neumann system, shifted so that psi_0 = 0, from zero).  Returns
    (psi, H, info)."""
    mu = magnetic_coeff(g, phi, chi, band_width)
    if solver == "mgpcg":
        b, b0n = magnetic_rhs(g, mu, hext)
        b[0] = b0n  # row 0's natural right-hand side: the consistent Neumann system
        form = _empty_form(g)
        lib().or_magnetic_face_form(g.nx, g.ny, g.nz, *[_p(_f64(m)) for m in mu], *[_p(a) for a in form])
        x, it, rr = mgpcg_solve(g, form, b, tol, maxit=min(maxit, 200))
        psi = x - x[0]
        H = magnetic_total_field(g, psi, hext)
        return psi.reshape(g.shape), H, dict(iters=it, relres=rr, mu=mu, rhs0_neumann=b0n)
    A = magnetic_assemble(g, mu)
    b, b0n = magnetic_rhs(g, mu, hext)
    x0 = None if psi0 is None else _f64(psi0).reshape(-1)
    if solver == "amg":
        psi, inf = A.amg_solve(b, 1, x0=x0, tol=tol, maxit=min(maxit, 100))
        it = inf["iters"]
        rr = float(np.linalg.norm(b - A.matvec(psi)) / max(np.linalg.norm(b), 1e-300))
    else:
        psi, it, rr = A.solve(b, x0=x0, tol=tol, maxit=maxit)
    H = magnetic_total_field(g, psi, hext)
    return psi.reshape(g.shape), H, dict(iters=it, relres=rr, A=A, b=b, mu=mu, rhs0_neumann=b0n)


# ------------------------------------------------------------------------------------------------ collider
def box_collider_fractions(g: Grid, bw: int = 0):
    """Collider(sgrid) + Finish: node level set of the domain box walls, fast marching, face fractions."""
    ls = np.empty((g.nx + 1, g.ny + 1, g.nz + 1))
    lib().or_collider_box_levelset(C.byref(g.c()), int(bw), _p(ls))
    lib().or_fast_marching(g.nx + 1, g.ny + 1, g.nz + 1, float(g.h), _p(ls))
    frac = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_collider_face_fractions(C.byref(g.c()), _p(ls), _D3(*[_p(a) for a in frac]))
    return frac


def box_collider(g: Grid, bw: int = 0):
    """Collider(sgrid) + Finish: node level set (after fast marching), face fractions and face normals."""
    ls = np.empty((g.nx + 1, g.ny + 1, g.nz + 1))
    lib().or_collider_box_levelset(C.byref(g.c()), int(bw), _p(ls))
    lib().or_fast_marching(g.nx + 1, g.ny + 1, g.nz + 1, float(g.h), _p(ls))
    frac = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_collider_face_fractions(C.byref(g.c()), _p(ls), _D3(*[_p(a) for a in frac]))
    normal = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_collider_face_normals(C.byref(g.c()), _p(ls), _D3(*[_p(a) for a in normal]))
    return ls, frac, normal


def extrapolate_velocity(g: Grid, u, phi, frac, clear_val=0.0, max_steps=6):
    """Extrapolation::Solve of the projected velocity (core/Simulation.cpp:237-241); returns new arrays."""
    u = [np.array(a, dtype=np.float64, copy=True) for a in u]
    fr, fp = _faces(frac)
    lib().or_extrapolate_velocity(C.byref(g.c()), _D3(*[_p(a) for a in u]), _p(_f64(phi)), fp, float(clear_val),
                                  int(max_steps))
    return u


def collider_enforce(g: Grid, u, frac, normal, us=None):
    """Collider::Enforce (core/Collider.cpp:75-86); returns new arrays."""
    u = [np.array(a, dtype=np.float64, copy=True) for a in u]
    fr, fp = _faces(frac)
    nr, npp = _faces(normal)
    ur, up = _opt_faces(us)
    lib().or_collider_enforce(C.byref(g.c()), _D3(*[_p(a) for a in u]), fp, npp, up)
    return u


def vertex_pressures(g: Grid, chi, H, positions, normals):
    """MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48) from the total field H."""
    hr, hp = _faces(H)
    pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
    nrm = np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, 3)
    out = np.empty(pos.shape[0])
    lib().or_vertex_pressures(C.byref(g.c()), float(chi), hp, _p(pos), _p(nrm), pos.shape[0], _p(out))
    return out


def pressure_jump(g: Grid, edge_mark, kappa=None, pm=None, sigma=0.0, rho=1.0, dt=1.0):
    """The jump callback of core/Simulation.cpp:216-235 on every face (three face arrays)."""
    em = [np.ascontiguousarray(e, dtype=np.int32) for e in edge_mark]
    kp = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    pp = None if pm is None else np.ascontiguousarray(pm, dtype=np.float64)
    jump = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_pressure_jump(C.byref(g.c()), (C.c_void_p * 3)(*[e.ctypes.data for e in em]),
                           None if kp is None else kp.ctypes.data, None if pp is None else pp.ctypes.data,
                           float(sigma), float(rho), float(dt), _D3(*[_p(a) for a in jump]))
    return jump


def advect_levelset(g: Grid, phi, u, dt):
    """Advection::Solve<2>(levelSet, velocity, dt) (core/Advection.h:40-49); returns the new level set."""
    phi = _f64(phi)
    ur, up = _faces(u)
    out = np.empty(g.shape)
    lib().or_advect_levelset(C.byref(g.c()), _p(phi), up, float(dt), _p(out))
    return out


def advect_velocity(g: Grid, u, dt):
    """Advection::Solve<2>(velocity, velocity, dt) (core/Advection.h:51-59); returns the new face arrays."""
    ur, up = _faces(u)
    out = [np.empty(g.face_shape(a)) for a in range(3)]
    lib().or_advect_velocity(C.byref(g.c()), up, float(dt), _D3(*[_p(a) for a in out]))
    return out


def reinitialize(g: Grid, phi, max_steps=10):
    """Reinitialization::Solve (core/Reinitialization.cpp:36-46); returns the new level set."""
    out = np.array(phi, dtype=np.float64, copy=True)
    lib().or_reinitialize(C.byref(g.c()), _p(out), int(max_steps))
    return out


def num_threads() -> int:
    return int(lib().or_num_threads())
