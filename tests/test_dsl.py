"""Host-side checks of the expression mirror (no device): how integrands map to form descriptors."""
import numpy as np
import pytest

from feelpp_gb300 import _ffi, fe


class _FakeDev:
    """Stands in for a DeviceScalar (only its device pointer is read)."""

    def device_ptr(self):
        import ctypes as C
        return C.c_void_p(0x1000)


def _integral(expr):
    return fe._Integral(None, expr, 0)


def _stiff():
    return fe.inner(fe.gradt(None), fe.grad(None))


def _mass():
    return fe.idt(None) * fe.id(None)


def test_laplace_plus_mass():
    d, karr = fe.Form2._desc_of(_integral(2.5 * _stiff() + 0.5 * _mass()), _ffi.ALGO_AUTO)
    assert d.kind == _ffi.FORM_LAPLACE_MASS and d.kappa == 2.5 and d.mass == 0.5 and karr is None
    assert not d.kappa_scale


def test_per_element_kappa():
    k = np.array([1.0, 2.0, 3.0])
    d, karr = fe.Form2._desc_of(_integral(k * _stiff() + _mass()), _ffi.ALGO_AUTO)
    assert np.array_equal(karr, k) and d.mass == 1.0


def test_device_scaled_stiffness():
    dev = _FakeDev()
    scaled = fe._Scaled(1.0, dev)
    e = (0.05 * scaled) * _stiff() + _mass()
    d, karr = fe.Form2._desc_of(_integral(e), _ffi.ALGO_AUTO)
    assert d.kappa == pytest.approx(0.05) and d.kappa_scale == 0x1000 and d.mass == 1.0
    e2 = 0.5 * (scaled * _stiff())
    d2, _ = fe.Form2._desc_of(_integral(e2), _ffi.ALGO_AUTO)
    assert d2.kappa == pytest.approx(0.5)


def test_device_scale_rejects_mass_and_double_scaling():
    scaled = fe._Scaled(1.0, _FakeDev())
    with pytest.raises(ValueError):
        scaled * _mass()
    with pytest.raises(ValueError):
        fe.Form2._desc_of(_integral(scaled * _stiff() + 2.0 * _stiff()), _ffi.ALGO_AUTO)


def test_elasticity_and_sources():
    d, _ = fe.Form2._desc_of(_integral(fe.inner(fe.stress(None, 1.0, 0.5), fe.grad(None))), _ffi.ALGO_AUTO)
    assert d.kind == _ffi.FORM_ELASTICITY and (d.lam, d.mu) == (1.0, 0.5)
    le = fe.inner(fe.cst_vec(0, 0, -1), fe.id(None))
    assert le.source.kind == _ffi.RHS_CONST_VEC and le.source.c == (0.0, 0.0, -1.0)
    assert (fe.sine_source() * fe.id(None)).source.kind == _ffi.RHS_SINE


def test_solver_cfg_names():
    cfg = fe._solver_cfg(1e-10, 100, "cheb_jacobi", True, 0.1, 16, "f64", 3, 0.03)
    assert cfg.pc == _ffi.PC_CHEB_JACOBI and cfg.mixed == 1 and cfg.cheb_degree == 3
    assert fe._solver_cfg(1e-10, 100, "gamg", False, 0.1, 16, "f64", 0, 0.0).pc == _ffi.PC_GAMG
    with pytest.raises(ValueError):
        fe._solver_cfg(1e-10, 100, "ilu", False, 0.1, 16, "f64", 0, 0.0)


def test_face_ranges():
    class _M:
        pass
    m = _M()
    d, _ = fe.Form2._desc_of(fe._Integral(fe.boundaryfaces(m), 2.0 * _mass(), 0), _ffi.ALGO_AUTO)
    assert d.range == _ffi.RANGE_BOUNDARY_FACES and d.mass == 2.0
    d, _ = fe.Form2._desc_of(fe._Integral(fe.markedfaces(m, 0.5), _mass(), 0), _ffi.ALGO_AUTO)
    assert d.range == _ffi.RANGE_MARKED_FACES and d.range_xmax == 0.5
    d, _ = fe.Form2._desc_of(fe._Integral(fe.elements(m), _stiff(), 0), _ffi.ALGO_AUTO)
    assert d.range == _ffi.RANGE_ELEMENTS


def test_nitsche_bilinear_terms():
    """cg_laplacian.hpp's weak-Dirichlet integrand maps to the face descriptor fields."""
    k = 1.5
    u, v = None, None
    e = (-fe.inner(k * fe.gradt(u) * fe.N(), fe.id(v)) - fe.inner(k * fe.grad(v) * fe.N(), fe.idt(u))
         + 2 * k * fe.idt(u) * fe.id(v) / fe.hFace() + 0.25 * fe.idt(u) * fe.id(v))
    d, karr = fe.Form2._desc_of(_integral(e), _ffi.ALGO_AUTO)
    assert d.dn_trial == -k and d.dn_test == -k and d.mass_h == 2 * k and d.mass == 0.25 and d.kappa == 0.0
    assert karr is None
    # k*gradt(u) inside inner(., grad(v)) is the stiffness coefficient
    d2, _ = fe.Form2._desc_of(_integral(fe.inner(k * fe.gradt(u), fe.grad(v))), _ffi.ALGO_AUTO)
    assert d2.kappa == k


def test_nitsche_linear_terms():
    k, g = 2.0, 0.3
    le = -fe.inner(k * fe.grad(None) * fe.N(), g) + 2 * k * g * fe.id(None) / fe.hFace()
    kinds = dict(le.terms)
    assert kinds["dn"] == pytest.approx(-k * g) and kinds["src_h"] == pytest.approx(2 * k * g)
    with pytest.raises(ValueError):
        fe.sine_source() * fe.id(None) / fe.hFace()
    with pytest.raises(ValueError):
        (fe.inner(fe.gradt(None), fe.grad(None))) / fe.hFace()
