"""Test infrastructure only (the oracle): ctypes wrapper of oracle/liboracle.so,
the C restatement of the reference algorithm.  Imported by tests/,
__graft_entry__.smoke() and bench.py's CPU baseline; never by the product."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
_L = None


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def load():
    global _L
    if _L is None:
        src = os.path.join(HERE, "pda_oracle.c")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = C.CDLL(LIB)
        L.orc_last_error.restype = C.c_char_p
        L.orc_mesh_load.restype = C.c_void_p
        L.orc_mesh_load.argtypes = [C.c_char_p]
        L.orc_mesh_from_arrays.restype = C.c_void_p
        L.orc_mesh_from_arrays.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_mesh_free.argtypes = [C.c_void_p]
        L.orc_mesh_counts.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_problem_create.restype = C.c_void_p
        L.orc_problem_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.POINTER(C.c_char_p), C.POINTER(C.c_double)]
        L.orc_problem_free.argtypes = [C.c_void_p]
        L.orc_sizes.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_initial_condition.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_velocity.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
        L.orc_velocity_and_jacobian.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p]
        L.orc_ssprk3.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64]
        L.orc_rk4.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64]
        L.orc_ssprk3_py.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64]
        L.orc_weno5.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_weno3.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_set_cube_mode.argtypes = [C.c_int]
        L.orc_round14.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_set_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _L = L
    return Oracle(_L)


class Mesh:
    def __init__(self, L, h):
        self.L, self.h = L, h
        c = np.zeros(4, dtype=np.int64)
        L.orc_mesh_counts(C.c_void_p(h), _vp(c))
        self.counts = tuple(int(x) for x in c)

    def __del__(self):
        if self.h:
            self.L.orc_mesh_free(C.c_void_p(self.h))
            self.h = None


class Problem:
    def __init__(self, L, mesh, h):
        self.L, self.mesh, self.h = L, mesh, h
        s = np.zeros(4, dtype=np.int64)
        L.orc_sizes(C.c_void_p(h), _vp(s))
        self.ndpc, self.dofs_sample, self.dofs_stencil, self.nnz = (int(x) for x in s)

    def __del__(self):
        if self.h:
            self.L.orc_problem_free(C.c_void_p(self.h))
            self.h = None

    def initial_condition(self):
        u = np.empty(self.dofs_stencil)
        self.L.orc_initial_condition(C.c_void_p(self.h), _vp(u))
        return u

    def velocity(self, U, t=0.0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.empty(self.dofs_sample)
        self.L.orc_velocity(C.c_void_p(self.h), _vp(U), t, _vp(V))
        return V

    def velocity_and_jacobian(self, U, t=0.0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.empty(self.dofs_sample)
        rp = np.empty(self.dofs_sample + 1, dtype=np.int32)
        ci = np.empty(self.nnz, dtype=np.int32)
        jv = np.empty(self.nnz)
        self.L.orc_velocity_and_jacobian(C.c_void_p(self.h), _vp(U), t, _vp(V), _vp(rp), _vp(ci), _vp(jv))
        return V, rp, ci, jv

    def ssprk3(self, U, t0, dt, n):
        self.L.orc_ssprk3(C.c_void_p(self.h), _vp(U), t0, dt, n)

    def rk4(self, U, t0, dt, n):
        self.L.orc_rk4(C.c_void_p(self.h), _vp(U), t0, dt, n)

    def ssprk3_py(self, U, t0, dt, n):
        """SSP-RK3 with the update order of the reference's Python driver."""
        self.L.orc_ssprk3_py(C.c_void_p(self.h), _vp(U), t0, dt, n)


class Oracle:
    def __init__(self, L):
        self.L = L

    def mesh_load(self, d):
        h = self.L.orc_mesh_load(os.fsencode(d))
        if not h:
            raise RuntimeError(self.L.orc_last_error().decode())
        return Mesh(self.L, h)

    def mesh_from_arrays(self, dim, stencil, graph, x, y, z, dx):
        graph = np.ascontiguousarray(graph, dtype=np.int32)
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        dxa = np.ascontiguousarray(dx, dtype=np.float64)
        h = self.L.orc_mesh_from_arrays(dim, stencil, graph.shape[0], len(x), _vp(graph), _vp(x), _vp(y),
                                        _vp(z), _vp(dxa))
        return Mesh(self.L, h)

    def problem(self, mesh, family, problem, scheme, icflag=1, params=None):
        names = list((params or {}).keys())
        cn = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
        cv = (C.c_double * max(1, len(names)))(*[float(params[n]) for n in names])
        h = self.L.orc_problem_create(C.c_void_p(mesh.h), family, problem, scheme, icflag, len(names), cn, cv)
        if not h:
            raise RuntimeError(self.L.orc_last_error().decode())
        return Problem(self.L, mesh, h)

    def weno5(self, q7):
        o = np.empty(4)
        self.L.orc_weno5(_vp(np.ascontiguousarray(q7, dtype=np.float64)), _vp(o))
        return o

    def weno3(self, q5):
        o = np.empty(4)
        self.L.orc_weno3(_vp(np.ascontiguousarray(q5, dtype=np.float64)), _vp(o))
        return o

    def set_cube_mode(self, correctly_rounded):
        """0: x^3 by pow (the reference); 1: correctly rounded (the library)."""
        self.L.orc_set_cube_mode(int(bool(correctly_rounded)))

    def round14(self, v):
        """strtod(sprintf("%.14f", v)) element-wise: a mesh-script coordinate as read back."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.empty_like(v)
        self.L.orc_round14(_vp(v), _vp(out), v.size)
        return out

    def set_threads(self, n):
        return self.L.orc_set_threads(n)
