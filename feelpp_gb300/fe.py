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

    def __init__(self, device=0, stream=None, profile=False, host_threads=0, host_setup=False, tune=True, tune_cache=None):
        self.lib = _ffi.load()
        cfg = _ffi.Config(device, stream, 1 if profile else 0, host_threads, 1 if host_setup else 0, 0 if tune else -1,
                          tune_cache.encode() if tune_cache else None)
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

    def set_tensor_cores(self, on=True, df64=False):
        """Binary32 quadrature-form element matrices (curved tetrahedra, hexahedra) on the tensor cores
        (on, the default) or on the CUDA cores; df64: the FP64-accurate affine Laplace/mass element
        matrices of the two-phase assembly on the tensor cores too (exact bf16 slices; default off,
        the CUDA-core df64 kernel is faster)."""
        self.check(self.lib.fgpu_set_tensor_cores(self.h, (_ffi.TC_F32 if on else 0) | (_ffi.TC_DF64 if df64 else 0)))

    def set_host_transfer(self, mode="auto"):
        """How host-output assembly moves values: "auto", "copy" (copy engines) or "direct" (kernel stores
        into the page-locked host buffer)."""
        m = {"auto": _ffi.HOST_TRANSFER_AUTO, "copy": _ffi.HOST_TRANSFER_COPY, "direct": _ffi.HOST_TRANSFER_DIRECT}[mode]
        self.check(self.lib.fgpu_set_host_transfer(self.h, m))

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
    """Tetrahedral mesh: vertex coordinates (V x 3) and elements (T x 4) in insertion order; with `ho`
    (T x 6 x 3 edge nodes, local edge order (1,2) (2,0) (0,1) (0,3) (1,3) (2,3)) the elements are curved
    (P2 geometry, as a gmsh order-2 mesh read with GEOMAP_HO). Elements given as T x 8 vertex ids make a
    hexahedral mesh (Mesh<Hypercube<3,1>>, reference vertex order: the z = -1 face counter-clockwise from
    (-1,-1,-1), then the z = +1 face); its spaces are scalar Q1/Q2."""

    def __init__(self, xyz, tets, env=None, ho=None):
        self.env = env or environment()
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32)
        if self.tets.ndim != 2 or self.tets.shape[1] not in (4, 8):
            raise ValueError("elements: T x 4 (tetrahedra) or T x 8 (hexahedra) vertex ids")
        self.cell = "hex" if self.tets.shape[1] == 8 else "tet"
        upload = self.env.lib.fgpu_mesh_upload_hex if self.cell == "hex" else self.env.lib.fgpu_mesh_upload
        h = C.c_void_p()
        self.env.check(upload(self.env.h, len(self.xyz), _ptr(self.xyz), len(self.tets), _ptr(self.tets), C.byref(h)))
        self.h = h
        self.ho = None
        if ho is not None:
            self.set_ho_nodes(ho)

    def set_ho_nodes(self, ho):
        """Curved elements from their edge nodes (None: affine again)."""
        if ho is None:
            self.ho = None
            self.env.check(self.env.lib.fgpu_mesh_set_ho_nodes(self.h, None))
            return
        self.ho = np.ascontiguousarray(ho, dtype=np.float64).reshape(len(self.tets), 6, 3)
        self.env.check(self.env.lib.fgpu_mesh_set_ho_nodes(self.h, _ptr(self.ho)))

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

    def rigid_body_modes(self):
        """The six rigid body modes of a Pchv space at its dof nodes (translations x, y, z; rotations
        (-y, x, 0), (0, -z, y), (z, 0, -x) about the vertex centroid): the elasticity near null space."""
        vs = [DeviceVector(self.env, self.ndof) for _ in range(6)]
        arr = (C.c_void_p * 6)(*[v.h.value for v in vs])
        self.env.check(self.env.lib.fgpu_space_rigid_body_modes(self.h, arr))
        return vs

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


    def device_ptr(self):
        d = C.c_void_p()
        self.env.check(self.env.lib.fgpu_vector_device(self.h, C.byref(d)))
        return d

    def axpby(self, a, x, b=1.0):
        """self = a x + b self (VectorPetsc::add / scale)."""
        self.env.check(self.env.lib.fgpu_vector_axpby(self.env.h, float(a), x.h, float(b), self.h))
        return self

    def copy_from(self, x):
        self.env.check(self.env.lib.fgpu_vector_copy(self.env.h, x.h, self.h))
        return self


class _Scaled:
    """factor * (device scalar): a coefficient read by the kernels when they run."""

    def __init__(self, factor, dev):
        self.factor, self.dev = float(factor), dev

    def __rmul__(self, coef):
        if not isinstance(coef, (int, float)):
            return NotImplemented
        return _Scaled(float(coef) * self.factor, self.dev)

    __mul__ = __rmul__


class DeviceScalar(DeviceVector):
    """A scalar kept in device memory, e.g. a time-dependent coefficient kappa(t):
    `dt * kt * inner(gradt(u), grad(v))` scales the stiffness term by its value at the
    time the assembly kernels run, so a captured graph follows set()."""

    def __init__(self, env, value=0.0):
        super().__init__(env, 1)
        self.set(value)

    def set(self, value):
        self.upload(np.array([float(value)]))

    def __rmul__(self, coef):
        if not isinstance(coef, (int, float)):
            return NotImplemented
        return _Scaled(float(coef), self)

    def __mul__(self, other):
        if isinstance(other, (int, float)):
            return _Scaled(float(other), self)
        if isinstance(other, Expr):
            return other.__rmul__(self)
        return NotImplemented


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


def _range_code(rng):
    """(FGPU_RANGE_*, xmax) of an integration range; integrate() without a range means elements."""
    if rng is None or rng.kind == "elements":
        return _ffi.RANGE_ELEMENTS, 0.0
    if rng.kind == "boundaryfaces":
        return _ffi.RANGE_BOUNDARY_FACES, 0.0
    return _ffi.RANGE_MARKED_FACES, float(rng.xmax)


def boundaryfaces(mesh):
    return _Range(mesh, "boundaryfaces")


def markedfaces(mesh, xmax):
    """Boundary faces whose vertices all satisfy x <= xmax (the "Dirichlet" marker of a box)."""
    return _Range(mesh, "markedfaces", xmax)


class _Normal:
    """N(): the unit outward normal of a boundary face."""


class _HFace:
    """hFace(): the longest edge of a boundary face (feelpp/feel/feelmesh/geond.hpp:737-757)."""


def N():  # noqa: N802 - Feel++ name
    return _Normal()


def hFace():  # noqa: N802 - Feel++ name
    return _HFace()


def _is_num(c):
    return isinstance(c, (int, float, np.floating, np.integer))


class _Op:
    """gradt(u), grad(v), idt(u), id(v), optionally times a coefficient and (for the gradients) N()."""

    __array_ufunc__ = None  # ndarray * _Op -> _Op.__rmul__ (per-element coefficients)

    def __init__(self, kind, f, coef=1.0):
        self.kind, self.f, self.coef = kind, f, coef

    def __mul__(self, other):
        if isinstance(other, _Normal) and self.kind in ("gradt", "grad"):
            return _Op(self.kind + "_n", self.f, self.coef)
        if isinstance(other, _Op) and {self.kind, other.kind} == {"idt", "id"}:
            return Expr([("mass", self.coef * other.coef)])
        if isinstance(other, _Op) and self.kind == "id":
            return other.__mul__(self)
        if _is_num(other) or isinstance(other, np.ndarray):
            return self.__rmul__(other)
        return NotImplemented

    def __rmul__(self, coef):
        if self.kind == "id":
            return LinearExpr(_source(coef))
        if _is_num(coef) or isinstance(coef, np.ndarray):
            return _Op(self.kind, self.f, coef * self.coef)
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
    """Sum of bilinear terms: ("stiff", k), ("mass", m), ("elast", (lam, mu)); on faces also
    ("mass_h", m) for m*idt(u)*id(v)/hFace(), ("dn_trial", c) for c*inner(gradt(u)*N(), id(v)) and
    ("dn_test", c) for c*inner(grad(v)*N(), idt(u))."""

    __array_ufunc__ = None  # let ndarray * Expr dispatch to Expr.__rmul__

    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        return Expr(self.terms + other.terms)

    def __neg__(self):
        return (-1.0) * self

    def __sub__(self, other):
        return self + (-other)

    def __truediv__(self, other):
        if isinstance(other, _HFace):
            out = []
            for kind, c in self.terms:
                if kind != "mass":
                    raise ValueError("only idt(u)*id(v) may be divided by hFace()")
                out.append(("mass_h", c))
            return Expr(out)
        return (1.0 / float(other)) * self

    def __rmul__(self, coef):
        out = []
        if isinstance(coef, DeviceScalar):
            coef = _Scaled(1.0, coef)
        for kind, c in self.terms:
            if kind == "elast":
                raise ValueError("scale the Lame coefficients instead")
            if isinstance(coef, _Scaled) or isinstance(c, _Scaled):
                if kind != "stiff":
                    raise ValueError("a device coefficient scales the stiffness term only")
                if isinstance(coef, _Scaled) and isinstance(c, _Scaled):
                    raise ValueError("one device coefficient per term")
                out.append((kind, coef * c if isinstance(coef, _Scaled) else _Scaled(float(coef) * c.factor, c.dev)))
                continue
            if isinstance(coef, np.ndarray) or isinstance(c, np.ndarray):
                out.append((kind, np.asarray(coef, dtype=np.float64) * c))
            else:
                out.append((kind, float(coef) * c))
        return Expr(out)

    __mul__ = __rmul__


def inner(a, b):
    if isinstance(a, _Op) and isinstance(b, _Op):
        kinds = {a.kind, b.kind}
        c = a.coef * b.coef
        if kinds == {"gradt", "grad"}:
            return Expr([("stiff", c)])
        if kinds == {"gradt_n", "id"}:
            return Expr([("dn_trial", c)])
        if kinds == {"grad_n", "idt"}:
            return Expr([("dn_test", c)])
    if isinstance(a, _Stress) and isinstance(b, _Op) and b.kind == "grad":
        return Expr([("elast", (a.lam, a.mu))])
    if isinstance(b, _Op) and b.kind == "grad_n" and _is_num(a):
        a, b = b, a
    if isinstance(a, _Op) and a.kind == "grad_n" and _is_num(b):
        return LinearExpr(terms=[("dn", float(a.coef) * float(b))])
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
    """Sum of linear terms: ("src", _Source) for f*id(v); on faces also ("src_h", g) for
    g*id(v)/hFace() and ("dn", c) for c*inner(grad(v)*N(), 1)."""

    __array_ufunc__ = None

    def __init__(self, source=None, terms=None):
        self.terms = list(terms) if terms is not None else [("src", source)]

    @property
    def source(self):
        if len(self.terms) != 1 or self.terms[0][0] != "src":
            raise ValueError("not a single source term")
        return self.terms[0][1]

    def __add__(self, other):
        return LinearExpr(terms=self.terms + other.terms)

    def __neg__(self):
        return (-1.0) * self

    def __sub__(self, other):
        return self + (-other)

    def __rmul__(self, coef):
        f = float(coef)
        out = []
        for kind, c in self.terms:
            if kind == "src":
                if c.kind == _ffi.RHS_SINE and f != 1.0:
                    raise ValueError("the sine source takes no coefficient")
                out.append(("src", _Source(c.kind, tuple(f * x for x in c.c))))
            else:
                out.append((kind, f * c))
        return LinearExpr(terms=out)

    __mul__ = __rmul__

    def __truediv__(self, other):
        if isinstance(other, _HFace):
            out = []
            for kind, c in self.terms:
                if kind != "src" or c.kind != _ffi.RHS_CONST:
                    raise ValueError("only a constant g*id(v) may be divided by hFace()")
                out.append(("src_h", c.c[0]))
            return LinearExpr(terms=out)
        return (1.0 / float(other)) * self


class _Integral:
    def __init__(self, rng, expr, quad):
        self.range, self.expr, self.quad = rng, expr, quad


def integrate(range, expr, quad=0):  # noqa: A002 - Feel++ keyword
    """integrate(_range=elements(mesh) | boundaryfaces(mesh) | markedfaces(mesh, xmax), _expr=...).
    On faces, with constant coefficients: alpha*idt(u)*id(v) (Robin), beta*idt(u)*id(v)/hFace(),
    c*inner(gradt(u)*N(), id(v)) and c*inner(grad(v)*N(), idt(u)) (Nitsche) in a form2; g*id(v),
    g*id(v)/hFace() and c*inner(grad(v)*N(), g) in a form1."""
    if range.kind not in ("elements", "boundaryfaces", "markedfaces"):
        raise ValueError("unknown integration range")
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
        expr = integral.expr
        if isinstance(expr, _Op) and expr.kind == "id":
            expr = LinearExpr(_source(1.0))
        rng, xmax = _range_code(integral.range)
        descs = []
        face = [0.0, 0.0, 0.0]          # FGPU_RHS_FACE: id(v), id(v)/hFace(), inner(grad(v), N())
        has_face = False
        for kind, c in expr.terms:
            if kind == "src" and not (rng != _ffi.RANGE_ELEMENTS and c.kind == _ffi.RHS_CONST):
                descs.append((c.kind, c.c))
            elif kind == "src":
                face[0] += c.c[0]
            elif kind == "src_h":
                face[1] += c
                has_face = True
            else:
                face[2] += c
                has_face = True
        if rng == _ffi.RANGE_ELEMENTS and has_face:
            raise ValueError("hFace() and N() terms need a face range")
        if rng != _ffi.RANGE_ELEMENTS:
            if descs:
                raise ValueError("face loads: constant coefficients only")
            descs.append((_ffi.RHS_FACE, tuple(face)) if has_face else (_ffi.RHS_CONST, (face[0], 0.0, 0.0)))
        for k, (kind, cc) in enumerate(descs):
            d = _ffi.RhsDesc()
            d.kind = kind
            for j in range(3):
                d.c[j] = cc[j]
            d.quad_degree = integral.quad
            d.range, d.range_xmax = rng, xmax
            self.env.check(self.env.lib.fgpu_assemble_vector(self.env.h, self.space.h, C.byref(d), self.vec.h,
                                                             accumulate if k == 0 else 1))

    def to_numpy(self):
        return self.vec.to_numpy()

    def zero(self):
        self.vec.zero()


_PC = {"none": _ffi.PC_NONE, "jacobi": _ffi.PC_JACOBI, "cheb_jacobi": _ffi.PC_CHEB_JACOBI, "gamg": _ffi.PC_GAMG,
       "pmg": _ffi.PC_PMG}


def _solver_cfg(rtol, maxit, pc, mixed, inner_rtol, check_every, arith, cheb_degree, cheb_ratio):
    """ksp-rtol, ksp-max-it, pc-type ("jacobi", "cheb_jacobi", "gamg" or "none")."""
    if pc not in _PC:
        raise ValueError("pc must be one of %s" % sorted(_PC))
    return _ffi.SolverCfg(rtol, maxit, _PC[pc], 1 if mixed else 0, inner_rtol, check_every,
                          _ffi.ARITH_DF64 if arith == "df64" else _ffi.ARITH_F64, cheb_degree, cheb_ratio)


def _stats(st):
    return {"iterations": st.iterations, "outer": st.outer, "rel_residual": st.rel_residual,
            "time_ms": st.time_ms, "eig_max": st.eig_max, "fallback": st.fallback,
            "fallback_iterations": st.fallback_iterations}


class Form2:
    """Bilinear form backed by a device CSR matrix with the Feel++ GraphCSR pattern."""

    def __init__(self, test, trial=None, precision="f64"):
        self._version = 0
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
        self._version = getattr(self, "_version", 0) + 1
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
        d.kappa_scale = None
        d.mass_h = d.dn_trial = d.dn_test = 0.0
        d.range, d.range_xmax = _range_code(integral.range)
        kappa_arr = None
        for kind, c in integral.expr.terms:
            if kind == "stiff" and isinstance(c, _Scaled):
                if d.kappa != 0.0 or kappa_arr is not None or d.kappa_scale:
                    raise ValueError("a device-scaled stiffness term must be the only one")
                d.kappa = c.factor
                d.kappa_scale = c.dev.device_ptr()
                continue
            if kind == "stiff":
                if d.kappa_scale:
                    raise ValueError("a device-scaled stiffness term must be the only one")
                if isinstance(c, np.ndarray):
                    kappa_arr = np.ascontiguousarray(c, dtype=np.float64)
                    d.kappa = 0.0
                else:
                    d.kappa += c
            elif kind in ("mass", "mass_h", "dn_trial", "dn_test"):
                if isinstance(c, np.ndarray):
                    raise ValueError("the %s coefficient must be constant" % kind)
                setattr(d, kind, getattr(d, kind) + c)
            elif kind == "elast":
                d.kind = _ffi.FORM_ELASTICITY
                d.lam, d.mu = c
        return d, kappa_arr

    def _assemble(self, integral, accumulate):
        self._version = getattr(self, "_version", 0) + 1
        d, kappa_arr = self._desc(integral)
        self._kappa_host = kappa_arr  # keep alive during the call
        if kappa_arr is not None:
            d.kappa_elem = kappa_arr.ctypes.data_as(C.c_void_p)
        self.env.check(self.env.lib.fgpu_assemble_matrix(self.env.h, self.h, C.byref(d), accumulate))

    def _on(self, item):
        self._version = getattr(self, "_version", 0) + 1
        dofs = self.space.boundary_dofs(item.range.xmax if item.range.kind == "markedfaces" else None)
        vals = None
        if item.expr != 0.0:
            vals = np.full(len(dofs), item.expr)
        self.env.check(self.env.lib.fgpu_dirichlet(self.env.h, self.h, item.rhs.vec.h, len(dofs), _ptr(dofs),
                                                   _ptr(vals), item.type, 1.0))

    def apply_bc(self, bc, rhs=None, type="elimination_symmetric", diag=1.0):  # noqa: A002
        """Apply a DirichletBC (device-resident rows; capturable in graphs)."""
        t = {"elimination": 0, "elimination_symmetric": 1, "elimination_keep_diagonal": 2}[type]
        self._version = getattr(self, "_version", 0) + 1
        vec = rhs.vec if isinstance(rhs, Form1) else rhs
        self.env.check(self.env.lib.fgpu_bc_apply(self.env.h, bc.h, self.h, vec.h if vec is not None else None, t, diag))

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
              check_every=16, arith="f64", cheb_degree=0, cheb_ratio=0.0, gamg=None, ksp="cg", restart=30):
        """CG + Jacobi (ksp-type=cg, pc-type=jacobi). mixed=True: binary32 CG whose iterate is folded
        into the binary64 solution, and its residual replaced by the binary64 one, each time the
        recurrence residual has dropped by `inner_rtol`; arith="df64": double-float arithmetic for
        the plain solve. pc="gamg": smoothed-aggregation AMG V-cycle, the hierarchy built on first use
        (options in `gamg`, see AMG) and rebuilt when the matrix changed since. ksp="gmres": restarted
        GMRES(restart) with right preconditioning (pc "none", "jacobi" or "gamg"), for non-symmetric
        matrices."""
        cfg = _solver_cfg(rtol, maxit, pc, mixed, inner_rtol, check_every, arith, cheb_degree, cheb_ratio)
        st = _ffi.SolveStats()
        vec = rhs.vec if isinstance(rhs, Form1) else rhs
        if ksp == "gmres":
            amg = self.gamg(**(gamg or {})) if pc == "gamg" else None
            self.env.check(self.env.lib.fgpu_solve_gmres(self.env.h, self.h, amg.h if amg else None, vec.h, solution.h,
                                                         C.byref(cfg), int(restart), C.byref(st)))
            return _stats(st)
        if ksp != "cg":
            raise ValueError("ksp: 'cg' or 'gmres'")
        if pc == "gamg":
            amg = self.gamg(**(gamg or {}))
            self.env.check(self.env.lib.fgpu_solve_cg_amg(self.env.h, self.h, amg.h, vec.h, solution.h, C.byref(cfg),
                                                          C.byref(st)))
            out = _stats(st)
            out["gamg"] = amg.info()
            return out
        self.env.check(self.env.lib.fgpu_solve_cg(self.env.h, self.h, None, vec.h, solution.h, C.byref(cfg),
                                                  C.byref(st)))
        return _stats(st)

    def solve_refined(self, rhs, solution, solution_lo=None, rtol=1e-10, maxit=100000, pc="jacobi", mixed=False,
                      inner_reduction=1e-6, gamg=None, cheb_degree=0):
        """CG with iterative refinement in double-double: the solution is solution + solution_lo (two
        binary64 vectors, about 106 bits) and the outer residual b - A (solution + solution_lo) is formed
        in double-double, so rtol may lie below the binary64 floor of a stiff system. Each outer step
        solves for the correction with CG (pc "jacobi", "cheb_jacobi", "none" or "gamg"; mixed allowed
        without gamg) to the relative reduction inner_reduction. The returned rel_residual is the
        double-double one; "outer" counts the outer steps."""
        cfg = _solver_cfg(rtol, maxit, pc, mixed, 0.1, 16, "f64", cheb_degree, 0.0)
        st = _ffi.SolveStats()
        vec = rhs.vec if isinstance(rhs, Form1) else rhs
        amg = self.gamg(**(gamg or {})) if pc == "gamg" else None
        self.env.check(self.env.lib.fgpu_solve_cg_refine_dd(self.env.h, self.h, amg.h if amg else None, vec.h, solution.h,
                                                            solution_lo.h if solution_lo is not None else None,
                                                            C.byref(cfg), float(inner_reduction), C.byref(st)))
        return _stats(st)

    def gamg(self, reuse=False, **opts):
        """The AMG hierarchy of this matrix (built, or rebuilt when the values changed since). reuse=True
        keeps an existing hierarchy after the values changed (PETSc's -pc_gamg_reuse_interpolation /
        a preconditioner kept across time steps): the V-cycle then acts with the older operator, the CG
        with the current one."""
        amg = getattr(self, "_amg", None)
        full = dict(threshold=0.0, max_levels=0, coarse_eq_lim=0, agg_smooths=0, smoother_degree=0, setup_on_host=False,
                    near_null_space=None, block_size=0)
        full.update(opts)
        if amg is not None and amg.opts != full:
            amg = None
        if amg is None:
            amg = AMG(self, **opts)
            self._amg = amg
            self._amg_version = self._version
        elif self._amg_version != self._version and not reuse:
            amg.update()
            self._amg_version = self._version
        return amg

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_matrix_destroy(self.h)
        except Exception:
            pass


class AMG:
    """Smoothed-aggregation AMG hierarchy of an assembled FP64 form (pc-type=gamg; PETSc PCGAMG "agg"
    options of the reference: threshold (pc-gamg-threshold), max_levels (pc-mg-levels), coarse_eq_lim
    (pc-gamg-coarse-eq-lim), agg_smooths (pc-gamg-nsmooths; -1 = unsmoothed), smoother_degree
    (Chebyshev degree of the level smoothers). 0 selects the default. setup_on_host: build the hierarchy
    on the host instead of the device (the same hierarchy bit for bit). near_null_space: None (the
    constant vector), "rigid" (the rigid body modes of the form's Pchv space, block size 3) or a list of
    DeviceVectors with block_size rows per node (PETSc MatSetNearNullSpace)."""

    def __init__(self, form, threshold=0.0, max_levels=0, coarse_eq_lim=0, agg_smooths=0, smoother_degree=0,
                 setup_on_host=False, near_null_space=None, block_size=0):
        self.env, self.form = form.env, form
        self.opts = dict(threshold=threshold, max_levels=max_levels, coarse_eq_lim=coarse_eq_lim, agg_smooths=agg_smooths,
                         smoother_degree=smoother_degree, setup_on_host=setup_on_host, near_null_space=near_null_space,
                         block_size=block_size)
        cfg = _ffi.AmgCfg(float(threshold), max_levels, coarse_eq_lim, agg_smooths, smoother_degree, int(bool(setup_on_host)))
        self._nns = None
        if near_null_space is not None:
            if isinstance(near_null_space, str):
                if near_null_space != "rigid":
                    raise ValueError("near_null_space: 'rigid' or a list of DeviceVectors")
                vecs, block_size = form.space.rigid_body_modes(), 3
            else:
                vecs = list(near_null_space)
            arr = (C.c_void_p * len(vecs))(*[v.h.value for v in vecs])
            self._nns = (vecs, arr)
            cfg.block_size, cfg.nns_count = int(block_size), len(vecs)
            cfg.nns = C.cast(arr, C.c_void_p)
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_amg_create(self.env.h, form.h, C.byref(cfg), C.byref(h)))
        self.h = h

    def update(self):
        self.env.check(self.env.lib.fgpu_amg_update(self.h))

    def info(self):
        nl = C.c_int()
        rows = np.zeros(16, dtype=np.int64)
        nnz = np.zeros(16, dtype=np.int64)
        ms = C.c_double()
        self.env.check(self.env.lib.fgpu_amg_info(self.h, C.byref(nl), _ptr(rows), _ptr(nnz), C.byref(ms)))
        dl = C.c_int()
        ph = np.zeros(9)
        self.env.check(self.env.lib.fgpu_amg_setup_info(self.h, C.byref(dl), _ptr(ph)))
        names = ("graph", "aggregate", "lanczos", "prolong", "galerkin", "host_levels", "layout", "total")
        return {"levels": nl.value, "rows": rows[:nl.value].tolist(), "nnz": nnz[:nl.value].tolist(),
                "setup_ms": ms.value, "device_levels": dl.value,
                "setup_phases_ms": {k: round(float(x), 3) for k, x in zip(names, ph[:8])}, "handoff": int(ph[8])}

    def __del__(self):
        if getattr(self, "h", None):
            try:
                self.env.lib.fgpu_amg_destroy(self.h)
            except Exception:
                pass
            self.h = None


class PMG:
    """p-multigrid preconditioner of a matrix-free operator: Chebyshev smoothing on the binary32 operator
    `smoother`, the P1 Form2 `coarse` (same mesh, Dirichlet rows eliminated) with its AMG hierarchy below."""

    def __init__(self, smoother, coarse, smoother_degree=0, coarse_cycles=0):
        self.env, self.smoother, self.coarse = smoother.env, smoother, coarse
        self.amg = coarse.gamg()
        cfg = _ffi.PmgCfg(smoother_degree, coarse_cycles)
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_pmg_create(self.env.h, smoother.h, coarse.h, self.amg.h, C.byref(cfg), C.byref(h)))
        self.h = h

    def info(self):
        lmax, ms = C.c_double(), C.c_double()
        nc = C.c_int64()
        self.env.check(self.env.lib.fgpu_pmg_info(self.h, C.byref(lmax), C.byref(nc), C.byref(ms)))
        return {"lmax": lmax.value, "coarse_rows": nc.value, "setup_ms": ms.value, "coarse_amg": self.amg.info()}

    def __del__(self):
        if getattr(self, "h", None):
            try:
                self.env.lib.fgpu_pmg_destroy(self.h)
            except Exception:
                pass
            self.h = None


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

    def set_algo(self, algo):
        """"gather" (element buffer + node gather) or "colour" (graph-coloured scatter, binary32)."""
        self.env.check(self.env.lib.fgpu_operator_set_algo(self.h, {"gather": _ffi.ALGO_GATHER,
                                                                    "colour": _ffi.ALGO_COLOUR}[algo]))

    def set_dirichlet(self, dofs):
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        self.env.check(self.env.lib.fgpu_operator_set_dirichlet(self.h, len(dofs), _ptr(dofs)))

    def apply(self, x, y):
        self.env.check(self.env.lib.fgpu_operator_apply(self.env.h, self.h, x.h, y.h))

    def solve(self, rhs, solution, rtol=1e-10, maxit=100000, pc="jacobi", inner=None, inner_rtol=0.1, check_every=16,
              cheb_degree=0, cheb_ratio=0.0, coarse=None, smoother=None, smoother_degree=0, coarse_cycles=0):
        """Matrix-free PCG; with `inner` (a binary32 Operator) the mixed method is used
        (binary32 CG with binary64 residual replacement every `inner_rtol` reduction).
        pc="pmg": p-multigrid V-cycle with `coarse` = the assembled P1 Form2 on the same mesh (same
        coefficients, Dirichlet rows eliminated) and its AMG hierarchy as coarse level; the smoother runs
        on `smoother` (a binary32 Operator; default `inner`), Chebyshev degree `smoother_degree` (0: 3), `coarse_cycles`
        AMG V-cycles per coarse solve (0: 4)."""
        cfg = _solver_cfg(rtol, maxit, pc, inner is not None, inner_rtol, check_every, "f64", cheb_degree, cheb_ratio)
        st = _ffi.SolveStats()
        vec = rhs.vec if isinstance(rhs, Form1) else rhs
        if pc == "pmg":
            pm = self.pmg(coarse, smoother or inner, smoother_degree, coarse_cycles)
            self.env.check(self.env.lib.fgpu_solve_cg_operator_pmg(self.env.h, self.h, inner.h if inner else None, pm.h, vec.h,
                                                                   solution.h, C.byref(cfg), C.byref(st)))
            out = _stats(st)
            out["pmg"] = pm.info()
            return out
        self.env.check(self.env.lib.fgpu_solve_cg_operator(self.env.h, self.h, inner.h if inner else None, vec.h,
                                                           solution.h, C.byref(cfg), C.byref(st)))
        return _stats(st)

    def pmg(self, coarse, smoother, smoother_degree=0, coarse_cycles=0):
        """The p-multigrid preconditioner (kept while the coarse matrix is unchanged)."""
        if coarse is None or smoother is None:
            raise ValueError("pc='pmg' needs coarse= (the P1 Form2) and a binary32 smoother operator")
        key = (id(coarse), id(smoother), getattr(coarse, "_version", 0), smoother_degree, coarse_cycles)
        pm = getattr(self, "_pmg", None)
        if pm is None or pm.key != key:
            pm = PMG(smoother, coarse, smoother_degree, coarse_cycles)
            pm.key = key
            self._pmg = pm
        return pm

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_operator_destroy(self.h)
        except Exception:
            pass


def export_ensight(space, prefix, fields):
    """Write the mesh and nodal fields ({name: Element}) of a scalar space as EnSight Gold files
    prefix.case, prefix.geo, prefix.<name>.scl (values at the vertices), the reference's default
    exporter format."""
    names = list(fields)
    arr_n = (C.c_char_p * max(len(names), 1))(*[n.encode() for n in names])
    arr_f = (C.c_void_p * max(len(names), 1))(*[fields[n].h for n in names])
    space.env.check(space.env.lib.fgpu_export_ensight(space.h, str(prefix).encode(), len(names),
                                                      C.cast(arr_n, C.c_void_p), C.cast(arr_f, C.c_void_p)))


def operator(test, integral, precision="f32"):
    return Operator(test, integral, precision)


def form1(test):
    return Form1(test)


def form2(test, trial=None, precision="f64"):
    return Form2(test, trial, precision)


class DirichletBC:
    """Dirichlet rows held on the device (on() applied repeatedly, e.g. every time step)."""

    def __init__(self, space, dofs, values=None):
        self.env = space.env
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        vals = None if values is None else np.ascontiguousarray(values, dtype=np.float64)
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_bc_create(self.env.h, space.ndof, len(dofs), _ptr(dofs), _ptr(vals), C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_bc_destroy(self.h)
        except Exception:
            pass


class Graph:
    """CUDA graph of library calls: `with fpp.capture(env) as g: ...` records, g.launch(n) replays."""

    def __init__(self, env):
        self.env = env
        self.h = None

    def __enter__(self):
        self.env.check(self.env.lib.fgpu_graph_begin(self.env.h))
        return self

    def __exit__(self, et, ev, tb):
        h = C.c_void_p()
        rc = self.env.lib.fgpu_graph_end(self.env.h, C.byref(h))
        if et is None:
            self.env.check(rc)
            self.h = h
        return False

    def launch(self, count=1):
        self.env.check(self.env.lib.fgpu_graph_launch(self.env.h, self.h, int(count)))

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_graph_destroy(self.h)
        except Exception:
            pass


def capture(env):
    return Graph(env)


class Batch:
    """Independent scalar Laplace/mass problems assembled together: one geometry launch and
    one persistent gather launch for all of them (meshes, orders 1-3, kappas may differ)."""

    def __init__(self, forms, integrals):
        if len(forms) != len(integrals) or not forms:
            raise ValueError("one integral per form")
        self.env = forms[0].env
        n = len(forms)
        self.forms = list(forms)
        descs = (_ffi.FormDesc * n)()
        self._kappa = []
        kp = (C.c_void_p * n)()
        for k, (f, integral) in enumerate(zip(forms, integrals)):
            d, karr = Form2._desc_of(integral, _ffi.ALGO_AUTO)
            if d.kind != _ffi.FORM_LAPLACE_MASS or d.kappa_scale:
                raise ValueError("batches hold Laplace/mass forms with constant or per-element kappa")
            descs[k] = d
            if karr is not None:
                dv = DeviceVector(self.env, len(karr))
                dv.upload(karr)
                self._kappa.append(dv)
                kp[k] = dv.device_ptr().value
        mats = (C.c_void_p * n)(*[f.h.value for f in forms])
        h = C.c_void_p()
        self.env.check(self.env.lib.fgpu_batch_create(self.env.h, n, mats, descs, kp, C.byref(h)))
        self.h = h

    def assemble(self, accumulate=False):
        self.env.check(self.env.lib.fgpu_batch_assemble(self.env.h, self.h, 1 if accumulate else 0))

    def set_launch(self, threads, chunk):
        self.env.check(self.env.lib.fgpu_batch_set_launch(self.h, threads, chunk))

    def set_algo(self, algo):
        """"gather" (fused persistent row-owner gather) or "two_phase" (element buffers + gather maps)."""
        self.env.check(self.env.lib.fgpu_batch_set_algo(self.h, {"gather": _ffi.ALGO_GATHER,
                                                                 "two_phase": _ffi.ALGO_TWO_PHASE}[algo]))

    def launch_config(self):
        t, c, tu = C.c_int(), C.c_int(), C.c_int()
        self.env.check(self.env.lib.fgpu_batch_get_launch(self.h, C.byref(t), C.byref(c), C.byref(tu)))
        return {"threads": t.value, "chunk": c.value, "tuned": bool(tu.value), "two_phase": c.value == 0}

    def __del__(self):
        try:
            if self.h:
                self.env.lib.fgpu_batch_destroy(self.h)
        except Exception:
            pass
