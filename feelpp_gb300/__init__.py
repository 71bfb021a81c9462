"""feelpp_gb300 — GB300-native device backend for the Feel++ assembly + solve hot path.

The compute path is ``_lib/libfgpu.so`` (hand-written sm_103a CUDA behind the
C-ABI of ``include/fgpu.h``); this package is its host-side mirror of the
Feel++ user API (``form2``, ``form1``, ``integrate``, ``on``, ``solve``).
"""
from . import meshgen  # noqa: F401
from ._ffi import FgpuError  # noqa: F401
from .fe import (  # noqa: F401
    Environment, Mesh, FunctionSpace, Pch, Pchv, Element, DeviceVector, Form1, Form2, form1, form2, integrate,
    elements, boundaryfaces, markedfaces, gradt, grad, idt, id, inner, stress, on, cst, cst_vec, sine_source,
    environment, Operator, operator, DeviceScalar, DirichletBC, Graph, capture, Batch, N, hFace, AMG, PMG, export_ensight,
)

__all__ = [
    "Environment", "Mesh", "FunctionSpace", "Pch", "Pchv", "Element", "DeviceVector", "Form1", "Form2", "form1",
    "form2", "integrate", "elements", "boundaryfaces", "markedfaces", "gradt", "grad", "idt", "id", "inner", "stress",
    "on", "cst", "cst_vec", "sine_source", "environment", "meshgen", "FgpuError", "Operator", "operator",
    "DeviceScalar", "DirichletBC", "Graph", "capture", "Batch", "N", "hFace", "AMG", "PMG", "export_ensight",
]
