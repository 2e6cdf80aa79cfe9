"""GB300-native finite-volume residual / Jacobian engine with the
pressio-demoapps problem API.

This module is the Python face of ``libpda_gb300.so`` (C ABI declared in
``include/pda_gb300.h``).  It mirrors the reference's Python bindings
(src_py/main_binder.cc, adapter_py.hpp): ``load_cellcentered_uniform_mesh``,
``create_problem``, and problem objects with ``initialCondition``,
``createState``, ``createVelocity``/``createRightHandSide``, ``velocity``/
``rightHandSide``, ``createJacobian``, ``jacobian``,
``rightHandSideAndJacobian``, ``applyJacobian`` ... operating on CUDA tensors
(float64) that stay resident on the GPU.  PyTorch supplies device memory and
streams only; all arithmetic runs in the library's own CUDA kernels.

There is no CPU fallback: if the shared library is missing the import of a
problem fails with a RuntimeError naming the build step.
"""
from __future__ import annotations

import ctypes as C
import enum
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libpda_gb300.so")

# ------------------------------------------------------------------- enums


class Euler1d(enum.IntEnum):
    PeriodicSmooth = 0
    Sod = 1
    Lax = 2
    ShuOsher = 3


class Euler2d(enum.IntEnum):
    PeriodicSmooth = 0
    KelvinHelmholtz = 1
    SedovFull = 2
    SedovSymmetry = 3
    Riemann = 4
    NormalShock = 5
    DoubleMachReflection = 6
    CrossShock = 7
    testingonlyneumann = 8


class Euler3d(enum.IntEnum):
    PeriodicSmooth = 0
    SedovSymmetry = 1


class Swe2d(enum.IntEnum):
    SlipWall = 0
    CustomBCs = 1


class InviscidFluxReconstruction(enum.IntEnum):
    FirstOrder = 0
    Weno3 = 1
    Weno5 = 2


class InviscidFluxScheme(enum.IntEnum):
    Rusanov = 0


_FAMILY = {Euler1d: 0, Euler2d: 1, Euler3d: 2, Swe2d: 3}

# -------------------------------------------------------------- the library

_lib = None

_SIGS = {
    "pda_last_error": (C.c_char_p, []),
    "pda_version": (C.c_char_p, []),
    "pda_mesh_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "pda_mesh_create_full": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int,
                                       C.POINTER(C.c_int), C.POINTER(C.c_void_p)]),
    "pda_mesh_create_sample": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.c_int64,
                                         C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "pda_mesh_write": (C.c_int, [C.c_void_p, C.c_char_p]),
    "pda_mesh_write_binary": (C.c_int, [C.c_void_p, C.c_char_p]),
    "pda_mesh_load_binary": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "pda_mesh_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "pda_mesh_arrays": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]),
    "pda_mesh_free": (None, [C.c_void_p]),
    "pda_problem_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.c_int,
                                     C.c_void_p, C.POINTER(C.c_void_p)]),
    "pda_problem_create_swe_slip_wall": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double,
                                                   C.c_double, C.c_void_p, C.POINTER(C.c_void_p)]),
    "pda_problem_create_cross_shock": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double,
                                                 C.c_void_p, C.POINTER(C.c_void_p)]),
    "pda_problem_free": (None, [C.c_void_p]),
    "pda_problem_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64)]),
    "pda_query_parameter": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]),
    "pda_initial_condition": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pda_initial_condition_host": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pda_velocity": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "pda_velocity_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "pda_jacobian_shape": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                     C.POINTER(C.c_int64)]),
    "pda_jacobian_pattern": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "pda_jacobian_pattern_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "pda_velocity_and_jacobian": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                            C.c_void_p]),
    "pda_velocity_and_jacobian_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                                 C.c_void_p]),
    "pda_jacobian": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "pda_apply_jacobian": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_int,
                                     C.c_void_p]),
    "pda_advance_ssprk3": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64,
                                     C.c_int]),
    "pda_advance_rk4": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64,
                                  C.c_int]),
    "pda_problem_launch_count": (C.c_int64, [C.c_void_p]),
    "pda_profile_velocity": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.POINTER(C.c_double)]),
    "pda_measure_fp64_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "pda_check_divsqrt": (C.c_int, [C.c_int, C.c_uint64, C.c_int64, C.c_void_p]),
    "pda_check_products": (C.c_int, [C.c_int, C.c_uint64, C.c_int64, C.c_void_p]),
    "pda_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "pda_batch_free": (None, [C.c_void_p]),
    "pda_batch_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64)]),
    "pda_batch_offsets": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pda_batch_initial_condition": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pda_batch_velocity": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "pda_batch_advance_ssprk3": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64,
                                           C.c_int]),
    "pda_batch_num_tile_shapes": (C.c_int, [C.c_void_p]),
    "pda_batch_set_tile_shape": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "pda_batch_tile_shape": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]),
    "pda_batch_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "pda_batch_launch_count": (C.c_int64, [C.c_void_p]),
    "pda_tc_gemm_bf16": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pda_ae_create": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_void_p,
                                C.POINTER(C.c_void_p)]),
    "pda_ae_free": (None, [C.c_void_p]),
    "pda_ae_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_double, C.c_uint64,
                               C.c_void_p]),
    "pda_ae_set_fused": (C.c_int, [C.c_void_p, C.c_int]),
    "pda_ae_reconstruct": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "pda_ae_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_void_p]),
    "pda_ae_layer": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pda_ae_set_layer": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "pda_lspg_create_affine": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                         C.POINTER(C.c_void_p)]),
    "pda_lspg_create_mlp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_int, C.POINTER(C.c_void_p)]),
    "pda_lspg_free": (None, [C.c_void_p]),
    "pda_advance_implicit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64, C.c_int,
                                       C.c_double, C.c_int, C.c_double, C.c_int, C.c_void_p]),
    "pda_lspg_decode": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "pda_lspg_set_fused": (C.c_int, [C.c_void_p, C.c_int]),
    "pda_lspg_set_jacobian_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "pda_lspg_advance_bdf1": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int64, C.c_int, C.c_double,
                                        C.c_int, C.c_void_p]),
    "pda_lspg_advance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int64, C.c_int, C.c_double,
                                   C.c_int, C.c_int64, C.c_int, C.c_void_p]),
}


def lib():
    """Load libpda_gb300.so (built by build_lib.py); raise if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} not found: build it first (python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class PdaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pda error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc != 0:
        raise PdaError(rc, lib().pda_last_error().decode())


def _ptr(t):
    return C.c_void_p(t.data_ptr())


# -------------------------------------------------------------------- meshes


class CellCenteredUniformMesh:
    """Mesh handle (mirror of pressiodemoapps.CellCenteredUniformMesh)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        dims = (C.c_int * 3)()
        sizes = (C.c_int64 * 4)()
        dx = (C.c_double * 3)()
        dxi = (C.c_double * 3)()
        flags = (C.c_int * 2)()
        _check(lib().pda_mesh_info(self._h, dims, sizes, dx, dxi, flags))
        self._dim, self._stencil, self._ncols = dims[0], dims[1], dims[2]
        self._sizes = tuple(sizes)
        self._dx = tuple(dx)
        self._dxinv = tuple(dxi)
        self._fully_periodic = bool(flags[0])
        self._structured = bool(flags[1])

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pda_mesh_free(self._h)
            self._h = None

    def dimensionality(self):
        return self._dim

    def stencilSize(self):
        return self._stencil

    def stencilMeshSize(self):
        return self._sizes[0]

    def sampleMeshSize(self):
        return self._sizes[1]

    def numCellsInner(self):
        return self._sizes[2]

    def numCellsNearBd(self):
        return self._sizes[3]

    def isFullyPeriodic(self):
        return self._fully_periodic

    def isStructured(self):
        return self._structured

    def dx(self):
        return self._dx[0]

    def dy(self):
        return self._dx[1]

    def dz(self):
        return self._dx[2]

    def dxInv(self):
        return self._dxinv[0]

    def dyInv(self):
        return self._dxinv[1]

    def dzInv(self):
        return self._dxinv[2]

    def _arrays(self):
        import numpy as np
        g = np.empty((self._sizes[1], self._ncols), dtype=np.int32)
        x = np.empty(self._sizes[0])
        y = np.empty(self._sizes[0])
        z = np.empty(self._sizes[0])
        inner = np.empty(self._sizes[2], dtype=np.int32)
        near = np.empty(self._sizes[3], dtype=np.int32)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        _check(lib().pda_mesh_arrays(self._h, vp(g), vp(x), vp(y), vp(z), vp(inner), vp(near)))
        return g, x, y, z, inner, near

    def graph(self):
        return self._arrays()[0]

    def viewX(self):
        return self._arrays()[1]

    def viewY(self):
        return self._arrays()[2]

    def viewZ(self):
        return self._arrays()[3]

    def graphRowsOfCellsAwayFromBd(self):
        return self._arrays()[4]

    def graphRowsOfCellsNearBd(self):
        return self._arrays()[5]

    def write(self, directory):
        _check(lib().pda_mesh_write(self._h, os.fsencode(directory)))

    def write_binary(self, path):
        """Write the mesh as one binary file (load_mesh_binary reads it)."""
        _check(lib().pda_mesh_write_binary(self._h, os.fsencode(str(path))))


def load_cellcentered_uniform_mesh(directory) -> CellCenteredUniformMesh:
    h = C.c_void_p()
    _check(lib().pda_mesh_load(os.fsencode(str(directory)), C.byref(h)))
    return CellCenteredUniformMesh(h)


def load_mesh_binary(path) -> CellCenteredUniformMesh:
    """Load a mesh written by CellCenteredUniformMesh.write_binary."""
    h = C.c_void_p()
    _check(lib().pda_mesh_load_binary(os.fsencode(str(path)), C.byref(h)))
    return CellCenteredUniformMesh(h)


def create_full_mesh(n, bounds, stencil_size=3, periodic=(False, False, False)):
    """In-memory equivalent of meshing_scripts/create_full_mesh.py."""
    nn = list(n) + [1] * (3 - len(n))
    bb = list(bounds) + [0.0] * (6 - len(bounds))
    pp = [int(bool(p)) for p in periodic] + [0] * (3 - len(periodic))
    h = C.c_void_p()
    _check(lib().pda_mesh_create_full((C.c_int * 3)(*nn), (C.c_double * 6)(*bb), int(stencil_size),
                                      (C.c_int * 3)(*pp), C.byref(h)))
    return CellCenteredUniformMesh(h)


def create_sample_mesh(full: CellCenteredUniformMesh, sample_gids):
    """Equivalent of meshing_scripts/create_sample_mesh.py; returns
    (sample mesh, stencil-mesh gids w.r.t. the full mesh)."""
    import numpy as np
    g = np.ascontiguousarray(np.asarray(sample_gids, dtype=np.int64))
    st = np.empty(full.stencilMeshSize(), dtype=np.int64)
    h = C.c_void_p()
    _check(lib().pda_mesh_create_sample(full._h, g.ctypes.data_as(C.POINTER(C.c_int64)), len(g),
                                        C.byref(h), st.ctypes.data_as(C.POINTER(C.c_int64))))
    m = CellCenteredUniformMesh(h)
    return m, st[: m.stencilMeshSize()].copy()


# ------------------------------------------------------------------- problems


class CsrJacobian:
    """Device CSR matrix with the reference's Eigen row-major layout."""

    def __init__(self, rowptr, colidx, values, shape):
        self.rowptr = rowptr
        self.colidx = colidx
        self.values = values
        self.shape = shape

    def nonZeros(self):
        return int(self.values.numel())

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values.cpu().numpy(), self.colidx.cpu().numpy(),
                              self.rowptr.cpu().numpy()), shape=self.shape)


class Problem:
    """Device problem object (mirror of PublicProblemEigenMixinCpp /
    the reference's Python problem classes)."""

    def __init__(self, mesh, family, handle, stream):
        self._mesh = mesh  # the mesh must outlive the problem
        self._family = family
        self._h = handle
        self._stream = stream
        nd = C.c_int()
        ds = C.c_int64()
        dst = C.c_int64()
        _check(lib().pda_problem_sizes(self._h, C.byref(nd), C.byref(ds), C.byref(dst)))
        self._ndpc, self._ds, self._dst = nd.value, ds.value, dst.value
        self._pattern = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pda_problem_free(self._h)
            self._h = None

    # sizes
    def numDofPerCell(self):
        return self._ndpc

    def totalDofSampleMesh(self):
        return self._ds

    def totalDofStencilMesh(self):
        return self._dst

    def queryParameter(self, name):
        v = C.c_double()
        _check(lib().pda_query_parameter(self._h, name.encode(), C.byref(v)))
        return v.value

    def gamma(self):
        return self.queryParameter("gamma")

    def gravity(self):
        return self.queryParameter("gravity")

    def coriolis(self):
        return self.queryParameter("coriolis")

    # buffers
    def _empty(self, n):
        import torch
        return torch.empty(n, dtype=torch.float64, device="cuda")

    def initialCondition(self):
        import torch
        u = torch.empty(self._dst, dtype=torch.float64, device="cuda")
        _check(lib().pda_initial_condition(self._h, _ptr(u)))
        return u

    def initialConditionHost(self):
        import numpy as np
        u = np.empty(self._dst)
        _check(lib().pda_initial_condition_host(self._h, u.ctypes.data_as(C.c_void_p)))
        return u

    def createState(self):
        import torch
        return torch.zeros(self._dst, dtype=torch.float64, device="cuda")

    def createVelocity(self):
        import torch
        return torch.zeros(self._ds, dtype=torch.float64, device="cuda")

    createRightHandSide = createVelocity
    createRhs = createVelocity

    @staticmethod
    def _check_vec(t, n, what):
        import torch
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64
                and t.is_contiguous() and t.numel() == n):
            raise ValueError(f"{what}: expected a contiguous float64 CUDA tensor of {n} entries")

    # evaluation
    def velocity(self, state, t, V):
        self._check_vec(state, self._dst, "state")
        self._check_vec(V, self._ds, "velocity")
        _check(lib().pda_velocity(self._h, _ptr(state), float(t), _ptr(V)))

    rightHandSide = velocity
    rhs = velocity

    def __call__(self, state, t, V, J=None, computeJacobian=False):
        if J is not None and computeJacobian:
            self.rightHandSideAndJacobian(state, t, V, J)
        else:
            self.velocity(state, t, V)

    def velocity_host(self, state_np, t, V_np):
        """Host-buffer call through the C ABI (H2D, kernels, D2H)."""
        _check(lib().pda_velocity_host(self._h, state_np.ctypes.data_as(C.c_void_p), float(t),
                                       V_np.ctypes.data_as(C.c_void_p)))

    def _shape(self):
        r, c, n = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().pda_jacobian_shape(self._h, C.byref(r), C.byref(c), C.byref(n)))
        return r.value, c.value, n.value

    def createJacobian(self) -> CsrJacobian:
        import torch
        rows, cols, nnz = self._shape()
        rp = torch.empty(rows + 1, dtype=torch.int32, device="cuda")
        ci = torch.empty(nnz, dtype=torch.int32, device="cuda")
        _check(lib().pda_jacobian_pattern(self._h, _ptr(rp), _ptr(ci)))
        vals = torch.zeros(nnz, dtype=torch.float64, device="cuda")
        return CsrJacobian(rp, ci, vals, (rows, cols))

    def jacobianPatternHost(self):
        import numpy as np
        rows, cols, nnz = self._shape()
        rp = np.empty(rows + 1, dtype=np.int32)
        ci = np.empty(nnz, dtype=np.int32)
        _check(lib().pda_jacobian_pattern_host(self._h, rp.ctypes.data_as(C.c_void_p),
                                               ci.ctypes.data_as(C.c_void_p)))
        return rp, ci

    def rightHandSideAndJacobian(self, state, t, V, J: CsrJacobian):
        self._check_vec(state, self._dst, "state")
        self._check_vec(V, self._ds, "velocity")
        _check(lib().pda_velocity_and_jacobian(self._h, _ptr(state), float(t), _ptr(V),
                                               _ptr(J.values)))

    def jacobian(self, state, t, J: CsrJacobian):
        self._check_vec(state, self._dst, "state")
        _check(lib().pda_jacobian(self._h, _ptr(state), float(t), _ptr(J.values)))

    def applyJacobian(self, state, operand, t, result):
        """result = J(state) @ operand; operand/result column-major
        (n x k tensors are passed transposed-contiguous as k columns)."""
        import torch
        if operand.dim() == 1:
            B = operand.contiguous()
            k = 1
            R = result
        else:
            B = operand.t().contiguous()
            k = operand.shape[1]
            R = torch.empty((k, self._ds), dtype=torch.float64, device="cuda")
        _check(lib().pda_apply_jacobian(self._h, _ptr(state), float(t), _ptr(B), k, _ptr(R)))
        if operand.dim() != 1:
            result.copy_(R.t())

    # time integration
    def advance_ssprk3(self, state, t0, dt, nsteps, use_graph=True):
        self._check_vec(state, self._dst, "state")
        _check(lib().pda_advance_ssprk3(self._h, _ptr(state), float(t0), float(dt), int(nsteps),
                                        int(bool(use_graph))))

    def advance_rk4(self, state, t0, dt, nsteps, use_graph=True):
        self._check_vec(state, self._dst, "state")
        _check(lib().pda_advance_rk4(self._h, _ptr(state), float(t0), float(dt), int(nsteps),
                                     int(bool(use_graph))))

    def launch_count(self):
        return lib().pda_problem_launch_count(self._h)

    def advance_implicit(self, state, t0, dt, nsteps, scheme="cn", newton_tol=1e-5, newton_max_iters=100,
                         linear_tol=1e-12, linear_max_iters=2000):
        """Crank-Nicolson ("cn") or BDF1 ("bdf1") steps with Newton-Raphson and
        Jacobi-preconditioned BiCGSTAB on the device (Pressio's implicit stepper
        + create_newton_solver + iterative::Bicgstab)."""
        import numpy as np
        self._check_vec(state, self._dst, "state")
        info = np.zeros(4)
        _check(lib().pda_advance_implicit(self._h, _ptr(state), float(t0), float(dt), int(nsteps),
                                          1 if scheme == "cn" else 0, float(newton_tol), int(newton_max_iters),
                                          float(linear_tol), int(linear_max_iters),
                                          info.ctypes.data_as(C.c_void_p)))
        return {"newton_iters": int(info[0]), "max_newton_per_step": int(info[1]), "linear_iters": int(info[2]),
                "worst_linear_relres": float(info[3])}

    def profile_velocity(self, state, V, reps=10):
        """Mean device ms of the velocity kernels: faces x/y/z, balance, near-boundary rows."""
        ms = (C.c_double * 5)()
        _check(lib().pda_profile_velocity(self._h, _ptr(state), _ptr(V), int(reps), ms))
        return dict(faces_x=ms[0], faces_y=ms[1], faces_z=ms[2], balance=ms[3], near_rows=ms[4])


def measure_fp64_peak():
    """Measured FP64 FMA throughput of the current GPU in FLOP/s."""
    v = C.c_double()
    _check(lib().pda_measure_fp64_peak(C.byref(v)))
    return v.value


def check_divsqrt(mode, seed=1, per_thread=4096):
    """Bit-for-bit comparison of the kernels' integer-pipe division and square
    root with the FP64 pipe's IEEE operations on seeded operands; returns
    (operand sets, division mismatches, square-root mismatches)."""
    import numpy as np
    c = np.zeros(3, dtype=np.int64)
    _check(lib().pda_check_divsqrt(int(mode), int(seed), int(per_thread), c.ctypes.data_as(C.c_void_p)))
    return tuple(int(v) for v in c)


def check_products(mode, seed=1, per_thread=4096):
    """Bit-for-bit comparison of the kernels' integer-pipe products by
    constants (3x, 5x, 7x, 11x, 13x; x/2, x/4; x c for literals c) and
    density guard (x + 1e-30) with the FP64 pipe's operations on seeded
    operands; returns (operands, small-integer product mismatches,
    power-of-two mismatches, guard mismatches, constant product
    mismatches)."""
    import numpy as np
    c = np.zeros(5, dtype=np.int64)
    _check(lib().pda_check_products(int(mode), int(seed), int(per_thread), c.ctypes.data_as(C.c_void_p)))
    return tuple(int(v) for v in c)


def _stream_handle(stream):
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return C.c_void_p(torch.cuda.current_stream().cuda_stream)
        except Exception:
            pass
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def create_problem(mesh, problem_enum, scheme=InviscidFluxReconstruction.FirstOrder, icFlag=1,
                   params=None, stream=None) -> Problem:
    """Mirror of pressiodemoapps.create_problem(mesh, enum, scheme[, icFlag[, params]])."""
    fam = _FAMILY[type(problem_enum)]
    names = list((params or {}).keys())
    vals = [float(params[k]) for k in names]
    cn = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
    cv = (C.c_double * max(1, len(vals)))(*vals)
    h = C.c_void_p()
    s = _stream_handle(stream)
    _check(lib().pda_problem_create(mesh._h, fam, int(problem_enum), int(scheme), int(icFlag), cn, cv,
                                    len(names), s, C.byref(h)))
    return Problem(mesh, fam, h, s)


def create_slip_wall_swe_2d_problem(mesh, scheme, gravity, coriolis, pulse_magnitude, stream=None):
    """Mirror of create_slip_wall_swe_2d_problem_eigen (swe2d.hpp:278-308)."""
    h = C.c_void_p()
    s = _stream_handle(stream)
    _check(lib().pda_problem_create_swe_slip_wall(mesh._h, int(scheme), float(gravity), float(coriolis),
                                                  float(pulse_magnitude), s, C.byref(h)))
    return Problem(mesh, 3, h, s)


def create_cross_shock_problem(mesh, scheme, density=0.1, inletXVel=10.0, bottomYVel=1.0, stream=None):
    """Mirror of create_cross_shock_problem (euler2d.hpp:258-299; the Python
    binding's name, src_py/main_binder.cc:476)."""
    h = C.c_void_p()
    s = _stream_handle(stream)
    _check(lib().pda_problem_create_cross_shock(mesh._h, int(scheme), float(density), float(inletXVel),
                                                float(bottomYVel), s, C.byref(h)))
    return Problem(mesh, 1, h, s)


class ProblemBatch:
    """Many independent problems (one family and scheme, uneven meshes and
    parameters) advanced together: one launch per residual phase over all
    instances.  No counterpart in the reference, whose callers loop over
    problem objects.  The state is one packed device vector; instance i owns
    ``U[offsets[i] : offsets[i] + problems[i].totalDofStencilMesh()]``."""

    def __init__(self, problems, stream=None):
        self._problems = list(problems)  # the problems must outlive the batch
        n = len(self._problems)
        arr = (C.c_void_p * max(1, n))(*[p._h.value for p in self._problems])
        h = C.c_void_p()
        self._stream = _stream_handle(stream)
        _check(lib().pda_batch_create(arr, n, self._stream, C.byref(h)))
        self._h = h
        nn, td, tc = C.c_int(), C.c_int64(), C.c_int64()
        _check(lib().pda_batch_sizes(self._h, C.byref(nn), C.byref(td), C.byref(tc)))
        self.size, self.totalDofs, self.totalCells = nn.value, td.value, tc.value
        off = (C.c_int64 * (n + 1))()
        _check(lib().pda_batch_offsets(self._h, off))
        self.offsets = [int(x) for x in off]

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pda_batch_free(self._h)
            self._h = None

    def createState(self):
        import torch
        return torch.zeros(self.totalDofs, dtype=torch.float64, device="cuda")

    def initialCondition(self):
        u = self.createState()
        _check(lib().pda_batch_initial_condition(self._h, _ptr(u)))
        return u

    def instance(self, U, i):
        """View of instance i inside a packed vector."""
        return U[self.offsets[i]: self.offsets[i] + self._problems[i].totalDofStencilMesh()]

    def velocity(self, U, t, V):
        Problem._check_vec(U, self.totalDofs, "state")
        Problem._check_vec(V, self.totalDofs, "velocity")
        _check(lib().pda_batch_velocity(self._h, _ptr(U), float(t), _ptr(V)))

    def advance_ssprk3(self, U, t0, dt, n_steps, use_graph=True):
        Problem._check_vec(U, self.totalDofs, "state")
        _check(lib().pda_batch_advance_ssprk3(self._h, _ptr(U), float(t0), float(dt), int(n_steps),
                                              int(bool(use_graph))))

    def num_tile_shapes(self):
        return lib().pda_batch_num_tile_shapes(self._h)

    def set_tile_shape(self, axis, shape):
        _check(lib().pda_batch_set_tile_shape(self._h, int(axis), int(shape)))

    def tile_shape(self, axis):
        s, la, li = C.c_int(), C.c_int(), C.c_int()
        _check(lib().pda_batch_tile_shape(self._h, int(axis), C.byref(s), C.byref(la), C.byref(li)))
        return s.value, la.value, li.value

    def autotune(self, U, reps=3):
        """Time every compiled tile shape per axis on U and keep the fastest;
        returns the mean times [axis][shape] in ms."""
        import numpy as np
        ns = self.num_tile_shapes()
        ms = np.zeros(3 * ns)
        _check(lib().pda_batch_autotune(self._h, _ptr(U), int(reps), ms.ctypes.data_as(C.c_void_p)))
        return ms.reshape(3, ns)

    def launch_count(self):
        return int(lib().pda_batch_launch_count(self._h))


def create_batch(problems, stream=None) -> ProblemBatch:
    return ProblemBatch(problems, stream)


def tc_gemm_bf16(A, B, bias=None, epilogue=0, out_f32=True, out_bf16=False, preact=False, stream=None):
    """C = A @ B.T (+ bias, ELU) on the tcgen05 tensor cores; A [M,K], B [N,K]
    bf16 CUDA tensors, K a multiple of 64.  Returns (C_f32, C_bf16, preact)."""
    import torch
    M, K = A.shape
    N = B.shape[0]
    oF = torch.empty(M, N, dtype=torch.float32, device=A.device) if out_f32 else None
    oB = torch.empty(M, N, dtype=torch.bfloat16, device=A.device) if out_bf16 else None
    pa = torch.empty(M, N, dtype=torch.float32, device=A.device) if preact else None
    vp = lambda t: C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)
    _check(lib().pda_tc_gemm_bf16(vp(A), vp(B), M, N, K, vp(bias), int(epilogue), vp(oF), vp(oB), vp(pa),
                                  _stream_handle(stream)))
    return oF, oB, pa


# ------------------------------------------------------- learned-manifold ROM
def _vp(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


class AutoEncoder:
    """MLP autoencoder trained on the device (tcgen05 BF16 GEMMs, fp32
    accumulation, Adam): n -> ha -> hb -> latent -> hb -> ha -> n, ELU.
    No counterpart in the reference."""

    LAYERS = 6

    def __init__(self, n, latent, ha=1024, hb=256, seed=0, stream=None):
        h = C.c_void_p()
        self._stream = _stream_handle(stream)
        _check(lib().pda_ae_create(int(n), int(latent), int(ha), int(hb), int(seed), self._stream, C.byref(h)))
        self._h = h
        self.n, self.latent, self.ha, self.hb = int(n), int(latent), int(ha), int(hb)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pda_ae_free(self._h)
            self._h = None

    def train(self, data, batch=256, epochs=1, lr=1e-3, seed=0):
        import numpy as np
        import torch
        assert data.dtype == torch.bfloat16 and data.is_cuda and data.is_contiguous() and data.shape[1] == self.n
        losses = np.zeros(max(1, epochs))
        _check(lib().pda_ae_train(self._h, _vp(data), data.shape[0], int(batch), int(epochs), float(lr), int(seed),
                                  losses.ctypes.data_as(C.c_void_p)))
        return losses[:epochs]

    def set_fused(self, fused=True):
        """Adam inside the weight-gradient GEMM epilogues (default) or as a
        separate pass over stored gradients; the weights agree bit for bit."""
        _check(lib().pda_ae_set_fused(self._h, 1 if fused else 0))

    def reconstruct(self, X):
        import torch
        rows = X.shape[0]
        Y = torch.empty(rows, self.n, dtype=torch.float32, device=X.device)
        Z = torch.empty(rows, self.latent, dtype=torch.float32, device=X.device)
        _check(lib().pda_ae_reconstruct(self._h, _vp(X), rows, _vp(Y), _vp(Z)))
        return Y, Z

    def layer_shape(self, l):
        import numpy as np
        oi = np.zeros(2, dtype=np.int64)
        _check(lib().pda_ae_layer(self._h, int(l), C.c_void_p(0), C.c_void_p(0), oi.ctypes.data_as(C.c_void_p)))
        return int(oi[0]), int(oi[1])

    def layer(self, l):
        import torch
        o, i = self.layer_shape(l)
        W = torch.empty(o, i, dtype=torch.float32, device="cuda")
        b = torch.empty(o, dtype=torch.float32, device="cuda")
        _check(lib().pda_ae_layer(self._h, int(l), _vp(W), _vp(b), C.c_void_p(0)))
        return W, b

    def set_layer(self, l, W, b):
        _check(lib().pda_ae_set_layer(self._h, int(l), _vp(W.contiguous()), _vp(b.contiguous())))

    def gradients(self, X):
        import torch
        total = sum(o * i + o for o, i in (self.layer_shape(l) for l in range(self.LAYERS)))
        g = torch.empty(total, dtype=torch.float32, device=X.device)
        loss = C.c_double()
        _check(lib().pda_ae_gradients(self._h, _vp(X), X.shape[0], C.byref(loss), _vp(g)))
        return loss.value, g

    def decoder(self):
        """Decoder weights with real sizes: W1 [hb x k], W2 [ha x hb], W3 [n x ha]."""
        W1, b1 = self.layer(3)
        W2, b2 = self.layer(4)
        W3, b3 = self.layer(5)
        return (W1[:, : self.latent].contiguous(), b1, W2, b2, W3, b3)


class LspgRom:
    """Hyper-reduced LSPG (BDF1, Gauss-Newton, FP64 normal equations) on a
    sample-mesh problem with an affine or MLP-decoder trial manifold."""

    def __init__(self, handle, problem, keep):
        self._h, self._problem, self._keep = handle, problem, keep

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pda_lspg_free(self._h)
            self._h = None

    @staticmethod
    def affine(sample_problem, sample_to_stencil, uref, phi):
        import numpy as np
        s2 = np.ascontiguousarray(sample_to_stencil, dtype=np.int64)
        k = phi.shape[1]
        h = C.c_void_p()
        _check(lib().pda_lspg_create_affine(sample_problem._h, s2.ctypes.data_as(C.c_void_p), int(k), _vp(uref),
                                            _vp(phi.contiguous()), C.byref(h)))
        return LspgRom(h, sample_problem, (s2, k, uref.numel()))

    @staticmethod
    def mlp(sample_problem, sample_to_stencil, uref, scale, W1, b1, W2, b2, W3, b3, tensor_cores=False):
        """tensor_cores=True: the output layer as a bf16 tcgen05 GEMM (the
        trained network's numerics; W3 must hold bf16 values)."""
        import numpy as np
        s2 = np.ascontiguousarray(sample_to_stencil, dtype=np.int64)
        k = W1.shape[1]
        h = C.c_void_p()
        ts = [t.contiguous() for t in (W1, b1, W2, b2, W3, b3)]
        _check(lib().pda_lspg_create_mlp(sample_problem._h, s2.ctypes.data_as(C.c_void_p), int(k),
                                         int(W1.shape[0]), int(W2.shape[0]), _vp(uref), _vp(scale),
                                         *[_vp(t) for t in ts], int(bool(tensor_cores)), C.byref(h)))
        return LspgRom(h, sample_problem, (s2, k, uref.numel()))

    def set_fused(self, fused=True):
        """Fused Gauss-Newton iteration (default) or the assembled sample-mesh
        Jacobian path; the same LSPG iteration, equal to rounding."""
        _check(lib().pda_lspg_set_fused(self._h, 1 if fused else 0))

    def set_jacobian_precision(self, bits=64):
        """64 (default): the exact Jacobian of the sample-mesh residual; 32: its
        terms in single precision (an inexact Gauss-Newton step on the same
        double-precision residual and normal equations; fused form only)."""
        _check(lib().pda_lspg_set_jacobian_precision(self._h, int(bits)))

    def decode(self, x):
        import torch
        y = torch.empty(self._keep[2], dtype=torch.float64, device="cuda")
        _check(lib().pda_lspg_decode(self._h, _vp(x), _vp(y)))
        return y

    def advance_bdf1(self, x, dt, n_steps, gn_iters=5, tol=1e-10, use_graph=True):
        return self.advance(x, dt, n_steps, gn_iters, tol, order=1, first_step=1, use_graph=use_graph)

    def advance(self, x, dt, n_steps, gn_iters=5, tol=1e-10, order=1, first_step=1, use_graph=True):
        """n_steps BDF1 (order 1) or BDF2 (order 2) LSPG steps; first_step is
        the 1-based index of the first of them in the trajectory (BDF2 takes
        step 1 with BDF1, as Pressio does)."""
        import numpy as np
        info = np.zeros(4)
        _check(lib().pda_lspg_advance(self._h, _vp(x), float(dt), int(n_steps), int(gn_iters), float(tol),
                                      int(order), int(first_step), int(bool(use_graph)),
                                      info.ctypes.data_as(C.c_void_p)))
        return {"last_correction": info[0], "iters_last_step": int(info[1]), "residual": info[2],
                "max_residual": info[3]}
