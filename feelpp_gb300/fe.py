"""Feel++-style host API over the GB300 C-ABI.

Mirrors the user-level names of the reference hot path
(``form2 / form1 / integrate / on / solve``, ``Pch / Pchv``, ``elements /
boundaryfaces / markedfaces``, ``gradt / grad / idt / id / inner``) so that
code written against Feel++ (C++ API or its pyfeelpp bindings,
``python/pyfeelpp/feelpp/forms.cpp``) reads the same. Every operation is a
call into ``libfgpu.so``; nothing here computes element values.

Supported integrands (everything the assembly kernels implement):

* ``k * inner(gradt(u), grad(v)) + m * idt(u) * id(v)`` on ``Pch<1..3>``, with
  ``k`` a constant or a per-element array (a P0 coefficient) and ``m`` a constant;
* ``inner(stress(u, lam, mu), grad(v))`` on ``Pchv<1..2>`` (linear elasticity);
* load vectors ``f * id(v)`` with ``f`` a constant, ``cst_vec(a, b, c)`` (Pchv)
  or ``sine_source()`` = 3 pi^2 sin(pi x) sin(pi y) sin(pi z).
"""
import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import check

# ---------------------------------------------------------------------------
# context (Environment + backend)
# ---------------------------------------------------------------------------


class Environment:
    """Owns an ``fgpu_ctx`` (device, launch stream, profiling)."""

    def __init__(self, device=0, stream=None, profile=False, host_threads=0):
        self.lib = _ffi.load()
        cfg = _ffi.Config(device, stream, 1 if profile else 0, host_threads)
        h = C.c_void_p()
        rc = self.lib.fgpu_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise _ffi.FgpuError(rc, "fgpu_create failed (no CUDA device?)")
        self.h = h

    def check(self, rc):
        check(rc, self.h)

    def sync(self):
        self.check(self.lib.fgpu_sync(self.h))

    def launches(self):
        return int(self.lib.fgpu_launch_count(self.h))

    def prof(self, name):
        n = C.c_int64()
        ms = C.c_double()
        self.check(self.lib.fgpu_prof_get(self.h, name.encode(), C.byref(n), C.byref(ms)))
        return int(n.value), float(ms.value)

    def prof_reset(self):
        self.check(self.lib.fgpu_prof_reset(self.h))

    def close(self):
        if self.h:
            self.lib.fgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_env = None


def environment():
    global _default_env
    if _default_env is None:
        _default_env = Environment()
    return _default_env


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------------------
# mesh and spaces
# ---------------------------------------------------------------------------


class Mesh:
    """Tetrahedral mesh: vertex coordinates (V x 3) and elements (T x 4) in insertion order."""

    def __init__(self, xyz, tets, env=None):
        self.env = env or environment()
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32)
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_mesh_upload(self.env.h, len(self.xyz), _ptr(self.xyz), len(self.tets),
                                                     _ptr(self.tets), C.byref(h)))
        self.h = h

    @property
    def num_elements(self):
        return len(self.tets)

    def set_coords(self, xyz):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.env.check(self.env.lib.fgpu_mesh_set_coords(self.h, _ptr(self.xyz)))

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_mesh_destroy(self.h)
        except Exception:
            pass


class FunctionSpace:
    """Continuous Lagrange space Pch<order> (ncomp = 1) or Pchv<order> (ncomp = 3)."""

    def __init__(self, mesh, order, ncomp=1):
        self.mesh = mesh
        self.env = mesh.env
        self.order = order
        self.ncomp = ncomp
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_space_create(self.env.h, mesh.h, order, ncomp, C.byref(h)))
        self.h = h
        n = C.c_int64()
        nl = C.c_int()
        self.env.check(self.env.lib.fgpu_space_ndof(self.h, C.byref(n), C.byref(nl)))
        self.ndof = int(n.value)
        self.nloc = int(nl.value)

    def nDof(self):
        return self.ndof

    def dof_l2g(self):
        out = np.zeros((self.mesh.num_elements, self.nloc), dtype=np.int32)
        self.env.check(self.env.lib.fgpu_space_l2g(self.h, _ptr(out)))
        return out

    def boundary_dofs(self, xmax=None):
        cnt = C.c_int64()
        on = 0 if xmax is None else 1
        xm = 0.0 if xmax is None else float(xmax)
        self.env.check(self.env.lib.fgpu_space_boundary_dofs(self.h, on, xm, C.byref(cnt), None))
        out = np.zeros(cnt.value, dtype=np.int32)
        self.env.check(self.env.lib.fgpu_space_boundary_dofs(self.h, on, xm, C.byref(cnt), _ptr(out)))
        return out

    def element(self, name="u"):
        return Element(self, name)

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_space_destroy(self.h)
        except Exception:
            pass


def Pch(mesh, order=1):
    return FunctionSpace(mesh, order, 1)


def Pchv(mesh, order=1):
    return FunctionSpace(mesh, order, 3)


class DeviceVector:
    def __init__(self, env, n):
        self.env = env
        self.n = n
        h = C.c_void_p()
        env.check(env.lib.fgpu_vector_create(env.h, n, C.byref(h)))
        self.h = h

    def upload(self, host):
        host = np.ascontiguousarray(host, dtype=np.float64)
        assert host.size == self.n
        self.env.check(self.env.lib.fgpu_vector_upload(self.h, _ptr(host)))

    def to_numpy(self, out=None):
        out = np.zeros(self.n) if out is None else out
        self.env.check(self.env.lib.fgpu_vector_download(self.h, _ptr(out)))
        return out

    def zero(self):
        self.env.check(self.env.lib.fgpu_vector_zero(self.h))

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_vector_destroy(self.h)
        except Exception:
            pass


class Element(DeviceVector):
    """An element of a function space (coefficient vector resident on the device)."""

    def __init__(self, space, name="u"):
        super().__init__(space.env, space.ndof)
        self.space = space
        self.name = name

    def errors_sine(self, quad=0):
        """(normL2, normH1-seminorm) of self - sin(pi x) sin(pi y) sin(pi z)."""
        l2, h1 = C.c_double(), C.c_double()
        self.env.check(self.env.lib.fgpu_norms_sine(self.env.h, self.space.h, self.h, quad, C.byref(l2), C.byref(h1)))
        return float(l2.value), float(h1.value)


# ---------------------------------------------------------------------------
# ranges and expressions
# ---------------------------------------------------------------------------


class _Range:
    def __init__(self, mesh, kind, xmax=None):
        self.mesh, self.kind, self.xmax = mesh, kind, xmax


def elements(mesh):
    return _Range(mesh, "elements")


def boundaryfaces(mesh):
    return _Range(mesh, "boundaryfaces")


def markedfaces(mesh, xmax):
    """Boundary faces whose vertices all satisfy x <= xmax (the "Dirichlet" marker of a box)."""
    return _Range(mesh, "markedfaces", xmax)


class _Op:
    def __init__(self, kind, f):
        self.kind, self.f = kind, f

    def __mul__(self, other):
        if isinstance(other, _Op) and {self.kind, other.kind} == {"idt", "id"}:
            return Expr([("mass", 1.0)])
        if isinstance(other, _Op) and self.kind == "id":
            return other.__mul__(self)
        return NotImplemented

    def __rmul__(self, coef):
        if self.kind == "id":
            return LinearExpr(_source(coef))
        return NotImplemented


def gradt(u):
    return _Op("gradt", u)


def grad(v):
    return _Op("grad", v)


def idt(u):
    return _Op("idt", u)


def id(v):  # noqa: A001 - Feel++ name
    return _Op("id", v)


class _Stress:
    def __init__(self, u, lam, mu):
        self.u, self.lam, self.mu = u, float(lam), float(mu)


def stress(u, lam, mu):
    """sigma(u) = lam tr(sym(gradt(u))) I + 2 mu sym(gradt(u))."""
    return _Stress(u, lam, mu)


class Expr:
    """Sum of bilinear terms: ("stiff", k), ("mass", m), ("elast", (lam, mu))."""

    __array_ufunc__ = None  # let ndarray * Expr dispatch to Expr.__rmul__

    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        return Expr(self.terms + other.terms)

    def __rmul__(self, coef):
        out = []
        for kind, c in self.terms:
            if kind == "elast":
                raise ValueError("scale the Lame coefficients instead")
            if isinstance(coef, np.ndarray) or isinstance(c, np.ndarray):
                out.append((kind, np.asarray(coef, dtype=np.float64) * c))
            else:
                out.append((kind, float(coef) * c))
        return Expr(out)

    __mul__ = __rmul__


def inner(a, b):
    if isinstance(a, _Op) and isinstance(b, _Op) and {a.kind, b.kind} == {"gradt", "grad"}:
        return Expr([("stiff", 1.0)])
    if isinstance(a, _Stress) and isinstance(b, _Op) and b.kind == "grad":
        return Expr([("elast", (a.lam, a.mu))])
    if isinstance(b, _Op) and b.kind == "id":
        return LinearExpr(_source(a))
    raise ValueError("unsupported inner product")


class _Source:
    def __init__(self, kind, c=(0.0, 0.0, 0.0)):
        self.kind, self.c = kind, c


def _source(coef):
    if isinstance(coef, _Source):
        return coef
    return _Source(_ffi.RHS_CONST, (float(coef), 0.0, 0.0))


def sine_source():
    """f = 3 pi^2 sin(pi x) sin(pi y) sin(pi z) (the manufactured source of u = sin sin sin)."""
    return _Source(_ffi.RHS_SINE)


def cst(c):
    return float(c)


def cst_vec(a, b, c):
    return _Source(_ffi.RHS_CONST_VEC, (float(a), float(b), float(c)))


class LinearExpr:
    def __init__(self, source):
        self.source = source


class _Integral:
    def __init__(self, rng, expr, quad):
        self.range, self.expr, self.quad = rng, expr, quad


def integrate(range, expr, quad=0):  # noqa: A002 - Feel++ keyword
    if range.kind != "elements":
        raise ValueError("only element integrals are on the device path")
    return _Integral(range, expr, quad)


class _On:
    def __init__(self, rng, rhs, element, expr, type_):
        self.range, self.rhs, self.element, self.expr, self.type = rng, rhs, element, expr, type_


ON_TYPES = {"elimination": _ffi.ON_ELIMINATION, "elimination_symmetric": _ffi.ON_ELIMINATION_SYMMETRIC,
            "elimination_keep_diagonal": _ffi.ON_ELIMINATION_KEEP_DIAGONAL}


def on(range, rhs, element, expr=0.0, type="elimination"):  # noqa: A002
    return _On(range, rhs, element, float(expr), ON_TYPES[type])


# ---------------------------------------------------------------------------
# forms
# ---------------------------------------------------------------------------


class Form1:
    def __init__(self, test):
        self.space = test
        self.env = test.env
        self.vec = DeviceVector(self.env, test.ndof)

    def __iadd__(self, integral):
        self._assemble(integral, accumulate=1)
        return self

    def assign(self, integral):
        self._assemble(integral, accumulate=0)
        return self

    def _assemble(self, integral, accumulate):
        src = integral.expr.source
        d = _ffi.RhsDesc()
        d.kind = src.kind
        for k in range(3):
            d.c[k] = src.c[k]
        d.quad_degree = integral.quad
        self.env.check(self.env.lib.fgpu_assemble_vector(self.env.h, self.space.h, C.byref(d), self.vec.h, accumulate))

    def to_numpy(self):
        return self.vec.to_numpy()

    def zero(self):
        self.vec.zero()


class Form2:
    """Bilinear form backed by a device CSR matrix with the Feel++ GraphCSR pattern."""

    def __init__(self, test, trial=None, precision="f64"):
        self.space = test
        self.env = test.env
        self.precision = _ffi.F64 if precision == "f64" else _ffi.F32
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_matrix_create(self.env.h, test.h, (trial or test).h, self.precision,
                                                       C.byref(h)))
        self.h = h
        nr = C.c_int64()
        nnz = C.c_int64()
        self.env.check(self.env.lib.fgpu_matrix_info(self.h, C.byref(nr), C.byref(nnz), None))
        self.nrows = int(nr.value)
        self.nnz = int(nnz.value)
        self._kappa_dev = None
        self.algo = _ffi.ALGO_AUTO

    def __iadd__(self, item):
        if isinstance(item, _On):
            self._on(item)
        else:
            self._assemble(item, accumulate=1)
        return self

    def assign(self, integral):
        self._assemble(integral, accumulate=0)
        return self

    def zero(self):
        self.env.check(self.env.lib.fgpu_matrix_zero(self.h))

    def _desc(self, integral):
        return Form2._desc_of(integral, self.algo)

    @staticmethod
    def _desc_of(integral, algo):
        d = _ffi.FormDesc()
        d.kind = _ffi.FORM_LAPLACE_MASS
        d.kappa = 0.0
        d.kappa_elem = None
        d.mass = 0.0
        d.lam, d.mu = 0.0, 0.0
        d.quad_degree = integral.quad
        d.algo = algo
        kappa_arr = None
        for kind, c in integral.expr.terms:
            if kind == "stiff":
                if isinstance(c, np.ndarray):
                    kappa_arr = np.ascontiguousarray(c, dtype=np.float64)
                    d.kappa = 0.0
                else:
                    d.kappa += c
            elif kind == "mass":
                if isinstance(c, np.ndarray):
                    raise ValueError("the mass coefficient must be constant")
                d.mass += c
            elif kind == "elast":
                d.kind = _ffi.FORM_ELASTICITY
                d.lam, d.mu = c
        return d, kappa_arr

    def _assemble(self, integral, accumulate):
        d, kappa_arr = self._desc(integral)
        self._kappa_host = kappa_arr  # keep alive during the call
        if kappa_arr is not None:
            d.kappa_elem = kappa_arr.ctypes.data_as(C.c_void_p)
        self.env.check(self.env.lib.fgpu_assemble_matrix(self.env.h, self.h, C.byref(d), accumulate))

    def _on(self, item):
        dofs = self.space.boundary_dofs(item.range.xmax if item.range.kind == "markedfaces" else None)
        vals = None
        if item.expr != 0.0:
            vals = np.full(len(dofs), item.expr)
        self.env.check(self.env.lib.fgpu_dirichlet(self.env.h, self.h, item.rhs.vec.h, len(dofs), _ptr(dofs),
                                                   _ptr(vals), item.type, 1.0))

    def csr(self):
        ia = np.zeros(self.nrows + 1, dtype=np.int64)
        ja = np.zeros(self.nnz, dtype=np.int32)
        val = np.zeros(self.nnz)
        self.env.check(self.env.lib.fgpu_matrix_get_csr(self.h, _ptr(ia), _ptr(ja), _ptr(val)))
        return ia, ja, val

    def values(self):
        val = np.zeros(self.nnz)
        self.env.check(self.env.lib.fgpu_matrix_get_csr(self.h, None, None, _ptr(val)))
        return val

    def mult(self, x, y):
        self.env.check(self.env.lib.fgpu_matrix_mult(self.env.h, self.h, x.h, y.h))

    def solve(self, rhs, solution, rtol=1e-10, maxit=100000, pc="jacobi", mixed=False, inner_rtol=0.1,
              check_every=16, arith="f64"):
        """CG + Jacobi (ksp-type=cg, pc-type=jacobi). mixed=True: binary32 CG whose iterate is folded
        into the binary64 solution, and its residual replaced by the binary64 one, each time the
        recurrence residual has dropped by `inner_rtol`; arith="df64": double-float arithmetic for
        the plain solve."""
        cfg = _ffi.SolverCfg(rtol, maxit, _ffi.PC_JACOBI if pc == "jacobi" else _ffi.PC_NONE, 1 if mixed else 0,
                             inner_rtol, check_every, _ffi.ARITH_DF64 if arith == "df64" else _ffi.ARITH_F64)
        st = _ffi.SolveStats()
        self.env.check(self.env.lib.fgpu_solve_cg(self.env.h, self.h, None, rhs.vec.h, solution.h, C.byref(cfg),
                                                  C.byref(st)))
        return {"iterations": st.iterations, "outer": st.outer, "rel_residual": st.rel_residual,
                "time_ms": st.time_ms}

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_matrix_destroy(self.h)
        except Exception:
            pass


class Operator:
    """Matrix-free operator of a Laplace/mass integral on a scalar space.

    precision: "f32", "f64" (native FP64) or "df64" (double-float). Dirichlet dofs set
    with set_dirichlet() are eliminated symmetrically, as on(..., type="elimination_symmetric")
    does on the assembled matrix."""

    PREC = {"f32": _ffi.F32, "f64": _ffi.F64, "df64": _ffi.DF64}

    def __init__(self, space, integral, precision="f32"):
        self.space = space
        self.env = space.env
        d, kappa_arr = Form2._desc_of(integral, _ffi.ALGO_AUTO)
        self._kappa = kappa_arr
        if kappa_arr is not None:
            d.kappa_elem = kappa_arr.ctypes.data_as(C.c_void_p)
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_operator_create(self.env.h, space.h, C.byref(d), self.PREC[precision], C.byref(h)))
        self.h = h
        self.precision = precision

    def use_tensor_cores(self, on=True):
        """binary32 P2/P3 operators: element phase on the tensor cores (tcgen05, 3xTF32)."""
        self.env.check(self.env.lib.fgpu_operator_set_tensor_cores(self.h, 1 if on else 0))

    def set_dirichlet(self, dofs):
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        self.env.check(self.env.lib.fgpu_operator_set_dirichlet(self.h, len(dofs), _ptr(dofs)))

    def apply(self, x, y):
        self.env.check(self.env.lib.fgpu_operator_apply(self.env.h, self.h, x.h, y.h))

    def solve(self, rhs, solution, rtol=1e-10, maxit=100000, pc="jacobi", inner=None, inner_rtol=0.1, check_every=16):
        """Matrix-free PCG; with `inner` (a binary32 Operator) the mixed method is used
        (binary32 CG with binary64 residual replacement every `inner_rtol` reduction)."""
        cfg = _ffi.SolverCfg(rtol, maxit, _ffi.PC_JACOBI if pc == "jacobi" else _ffi.PC_NONE, 1 if inner else 0,
                             inner_rtol, check_every, _ffi.ARITH_F64)
        st = _ffi.SolveStats()
        vec = rhs.vec if isinstance(rhs, Form1) else rhs
        self.env.check(self.env.lib.fgpu_solve_cg_operator(self.env.h, self.h, inner.h if inner else None, vec.h,
                                                           solution.h, C.byref(cfg), C.byref(st)))
        return {"iterations": st.iterations, "outer": st.outer, "rel_residual": st.rel_residual,
                "time_ms": st.time_ms}

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_operator_destroy(self.h)
        except Exception:
            pass


def operator(test, integral, precision="f32"):
    return Operator(test, integral, precision)


def form1(test):
    return Form1(test)


def form2(test, trial=None, precision="f64"):
    return Form2(test, trial, precision)
