"""Python handle on the CPU oracle (oracle/tx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
bench's CPU-baseline leg, never by the tianxin_gb300 package.  The oracle
restates the reference path (Tianxin/Panzer, one rank) in FP64 with forward-
mode AD Jacobians; see the header of tx_oracle.cpp for the file:line map.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from tianxin_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (g++, seconds)."""
    src = os.path.join(HERE, "tx_oracle.cpp")
    hdr = os.path.join(HERE, "..", "include", "tianxin_gb300.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int32, C.c_double
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(_abi.MeshDesc), C.POINTER(_abi.EquationSetDesc), C.c_char_p, C.c_int]
        L.orc_destroy.argtypes = [P]
        for name in ("orc_n_dofs", "orc_nnz", "orc_n_elements"):
            getattr(L, name).restype = I64
            getattr(L, name).argtypes = [P]
        L.orc_n_blocks.argtypes = [P]
        L.orc_n_fields.argtypes = [P]
        L.orc_block_n_elems.restype = I64
        L.orc_block_n_elems.argtypes = [P, C.c_int]
        L.orc_block_gid_count.argtypes = [P, C.c_int]
        L.orc_block_elements.argtypes = [P, C.c_int, P]
        L.orc_owned_gids.argtypes = [P, P]
        L.orc_element_gids.argtypes = [P, C.c_int, P]
        L.orc_element_lids.argtypes = [P, C.c_int, P]
        L.orc_element_conn.argtypes = [P, I64, P, C.POINTER(C.c_int)]
        L.orc_field_offsets.argtypes = [P, C.c_int, C.c_int, P]
        L.orc_graph.argtypes = [P, P, P]
        L.orc_coordinates.argtypes = [P, P]
        L.orc_dof_coordinates.argtypes = [P, P]
        L.orc_eval.argtypes = [P, P, P, P, D, D, D, P, P, C.c_int, I64, I64, C.c_int, C.c_char_p, C.c_int]
        L.orc_dirichlet_dofs.restype = I64
        L.orc_dirichlet_dofs.argtypes = [P, C.c_uint32, C.c_uint32, P]
        L.orc_dirichlet_apply.argtypes = [P, I64, P, P, P, P, P]
        L.orc_response.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P]
        L.orc_neumann.restype = I64
        L.orc_response_extreme.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P]
        L.orc_response_side.argtypes = [P, C.c_int, C.c_uint32, C.c_int, P, P, P]
        L.orc_response_probe.restype = I64
        L.orc_response_probe.argtypes = [P, P, C.c_int, P, P, P]
        L.orc_neumann.argtypes = [P, C.c_int, C.c_uint32, C.c_int, D, P]
        L.orc_spmv.argtypes = [I64, P, P, P, P, P, D, D]
        L.orc_cg.argtypes = [I64, P, P, P, P, P, D, C.c_int, C.POINTER(D)]
        L.orc_cubature.argtypes = [C.c_int, C.c_int, P, P]
        L.orc_cell_values.argtypes = [C.c_int, C.c_int, P, P, P]
        L.orc_basis_subcell.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_basis_eval.argtypes = [C.c_int, C.c_int, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One mesh + equation set, numbered and graphed the way the reference does it."""

    def __init__(self, mesh, eqset):
        L = lib()
        err = C.create_string_buffer(512)
        self.mesh, self.eqset = mesh, eqset
        self.h = L.orc_create(C.byref(mesh), C.byref(eqset), err, 512)
        if not self.h:
            raise RuntimeError("oracle: " + err.value.decode())
        self.n_dofs = L.orc_n_dofs(self.h)
        self.nnz = L.orc_nnz(self.h)
        self.n_blocks = L.orc_n_blocks(self.h)
        self.n_fields = L.orc_n_fields(self.h)
        self.n_elements = L.orc_n_elements(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def block_n_elems(self, b):
        return lib().orc_block_n_elems(self.h, b)

    def block_gid_count(self, b):
        return lib().orc_block_gid_count(self.h, b)

    def block_elements(self, b):
        out = np.zeros(self.block_n_elems(b), np.int64)
        lib().orc_block_elements(self.h, b, _p(out))
        return out

    def owned_gids(self):
        out = np.zeros(self.n_dofs, np.int64)
        lib().orc_owned_gids(self.h, _p(out))
        return out

    def element_gids(self, b):
        out = np.zeros((self.block_n_elems(b), self.block_gid_count(b)), np.int64)
        lib().orc_element_gids(self.h, b, _p(out))
        return out

    def element_lids(self, b):
        out = np.zeros((self.block_n_elems(b), self.block_gid_count(b)), np.int32)
        lib().orc_element_lids(self.h, b, _p(out))
        return out

    def element_conn(self, e):
        out = np.zeros(64, np.int64)
        n = C.c_int()
        lib().orc_element_conn(self.h, e, _p(out), C.byref(n))
        return out[: n.value]

    def field_offsets(self, b, f):
        out = np.zeros(64, np.int32)
        n = lib().orc_field_offsets(self.h, b, f, _p(out))
        return out[:n]

    def graph(self):
        rowptr = np.zeros(self.n_dofs + 1, np.int64)
        colind = np.zeros(self.nnz, np.int32)
        lib().orc_graph(self.h, _p(rowptr), _p(colind))
        return rowptr, colind

    def coordinates(self):
        n = (self.mesh.nx * self.mesh.bx + 1) * (self.mesh.ny * self.mesh.by + 1) * (self.mesh.nz * self.mesh.bz + 1)
        out = np.zeros((n, 3))
        lib().orc_coordinates(self.h, _p(out))
        return out

    def dof_coordinates(self):
        out = np.zeros((self.n_dofs, 3))
        lib().orc_dof_coordinates(self.h, _p(out))
        return out

    def evaluate(self, x, x_dot=None, aux=None, alpha=0.0, beta=1.0, t=0.0, jacobian=True, residual=True,
                 block=-1, elem_range=(0, -1), threads=1):
        """Residual f and CRS values (summed from zero), like evalModel(f, W)."""
        x = np.ascontiguousarray(x, np.float64)
        xd = None if x_dot is None else np.ascontiguousarray(x_dot, np.float64)
        ax = None if aux is None else np.ascontiguousarray(aux, np.float64)
        f = np.zeros(self.n_dofs) if residual else None
        vals = np.zeros(self.nnz) if jacobian else None
        err = C.create_string_buffer(512)
        rc = lib().orc_eval(self.h, _p(x), _p(xd), _p(ax), alpha, beta, t, _p(f), _p(vals), block,
                            elem_range[0], elem_range[1], threads, err, 512)
        if rc:
            raise RuntimeError("oracle eval: " + err.value.decode())
        return f, vals

    def dirichlet_dofs(self, side_mask, field_mask=0x7):
        n = lib().orc_dirichlet_dofs(self.h, side_mask, field_mask, None)
        out = np.zeros(n, np.int32)
        lib().orc_dirichlet_dofs(self.h, side_mask, field_mask, _p(out))
        return out

    def dirichlet_apply(self, lids, g, x, f=None, vals=None):
        lids = np.ascontiguousarray(lids, np.int32)
        g = None if g is None else np.ascontiguousarray(g, np.float64)
        lib().orc_dirichlet_apply(self.h, len(lids), _p(lids), _p(g), _p(np.ascontiguousarray(x, np.float64)),
                                  _p(f), _p(vals))


    def neumann(self, block, side_mask, field, value, f=None):
        """f += the "Flux" Neumann residual of `value` on block's sides in side_mask; returns (f, #sides)."""
        if f is None:
            f = np.zeros(self.n_dofs)
        n = lib().orc_neumann(self.h, block, side_mask, field, float(value), _p(f))
        if n < 0:
            raise RuntimeError("oracle neumann failed")
        return f, int(n)


def _response_impl(self, integrand, field=0, block=-1, degree=0, x=None, gradient=False):
    """Integral response at x: "Field", "L2 Error" or "H1 Error" (against sin(pi x) sin(pi y) sin(pi z));
    returns value, or (value, dvalue/dx) with gradient=True."""
    kind = {"Field": _abi.TX_INTEGRAND_FIELD, "L2 Error": _abi.TX_INTEGRAND_L2_ERROR,
            "H1 Error": _abi.TX_INTEGRAND_H1_ERROR}[integrand]
    x = np.ascontiguousarray(x, np.float64)
    val = C.c_double()
    g = np.zeros(self.n_dofs) if gradient else None
    if lib().orc_response(self.h, block, field, kind, degree, _p(x), C.byref(val), _p(g)):
        raise RuntimeError("oracle response failed")
    return (val.value, g) if gradient else val.value


Oracle.response = _response_impl


def _extreme_impl(self, use_max=True, field=0, block=-1, degree=0, x=None, gradient=False):
    """ExtremeValue response at x: max (or min) of the field at the cubature points; optional gradient."""
    x = np.ascontiguousarray(x, np.float64)
    val = C.c_double()
    g = np.zeros(self.n_dofs) if gradient else None
    if lib().orc_response_extreme(self.h, block, field, int(use_max), degree, _p(x), C.byref(val), _p(g)):
        raise RuntimeError("oracle extreme value failed")
    return (val.value, g) if gradient else val.value


def _side_impl(self, side_mask, field=0, block=-1, x=None, gradient=False):
    """Integral of the field over the block sides on the box sides of side_mask; optional gradient."""
    x = np.ascontiguousarray(x, np.float64)
    val = C.c_double()
    g = np.zeros(self.n_dofs) if gradient else None
    if lib().orc_response_side(self.h, block, side_mask, field, _p(x), C.byref(val), _p(g)):
        raise RuntimeError("oracle side response failed")
    return (val.value, g) if gradient else val.value


def _probe_impl(self, point, field=0, x=None, gradient=False):
    """Probe response: (value, element) of the field at point (element -1: outside); optional gradient."""
    x = np.ascontiguousarray(x, np.float64)
    pt = np.ascontiguousarray(point, np.float64)
    val = C.c_double(np.nan)
    g = np.zeros(self.n_dofs) if gradient else None
    e = lib().orc_response_probe(self.h, _p(pt), field, _p(x), C.byref(val), _p(g))
    return (val.value, int(e), g) if gradient else (val.value, int(e))


Oracle.extreme = _extreme_impl
Oracle.side_response = _side_impl
Oracle.probe = _probe_impl


def workset_functor(value_type, value=0.0, times=None, values=None, t=0.0):
    """WorksetFunctor values (disc-fe/src/evaluators/TianXin_WorksetFunctor_impl.hpp:56-121):
    Constant; Linear, whose elapse time is read from the same "Value" entry as the value (:67-82);
    TimeTable, linear between the table points, an error past the last time (:88-121)."""
    if value_type == "Constant":
        return value
    if value_type == "Linear":
        elapse = value
        if t >= elapse:
            return value
        if t <= 0.0:
            return 0.0
        return value * t / elapse
    if value_type == "TimeTable":
        if t > times[-1]:
            raise ValueError("Time is growing unbounded!")
        i = 0
        while times[i] < t:
            i += 1
        if i == 0:
            return values[0]
        slope = (values[i] - values[i - 1]) / (times[i] - times[i - 1])
        return values[i - 1] + slope * (t - times[i - 1])
    raise ValueError(value_type)


def spmv(rowptr, colind, vals, x, y=None, alpha=1.0, beta=0.0):
    n = len(rowptr) - 1
    y = np.zeros(n) if y is None else y
    lib().orc_spmv(n, _p(rowptr), _p(colind), _p(vals), _p(np.ascontiguousarray(x, np.float64)), _p(y), alpha, beta)
    return y


def cg(rowptr, colind, vals, b, x0=None, rtol=1e-12, maxit=100000):
    n = len(rowptr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    rr = C.c_double()
    it = lib().orc_cg(n, _p(rowptr), _p(colind), _p(vals), _p(np.ascontiguousarray(b, np.float64)), _p(x), rtol,
                      maxit, C.byref(rr))
    return x, it, rr.value


def cubature(topo, degree):
    n = lib().orc_cubature(topo, degree, None, None)
    xi = np.zeros((n, 3))
    w = np.zeros(n)
    lib().orc_cubature(topo, degree, _p(xi), _p(w))
    return xi, w


def cell_values(topo, degree, X):
    X = np.ascontiguousarray(X, np.float64)
    n = lib().orc_cubature(topo, degree, None, None)
    wdet = np.zeros(n)
    ip = np.zeros((n, 3))
    lib().orc_cell_values(topo, degree, _p(X), _p(wdet), _p(ip))
    return wdet, ip


def basis_subcell(topo, basis, dim, c):
    return lib().orc_basis_subcell(topo, basis, dim, c)


def basis_eval(topo, basis, xi):
    val = np.zeros(12 * 3 if basis == _abi.TX_HCURL_I1 else 27)
    grad = np.zeros(27 * 3 if basis != _abi.TX_HCURL_I1 else 36)
    n = lib().orc_basis_eval(topo, basis, _p(np.ascontiguousarray(xi, np.float64)), _p(val), _p(grad))
    if basis == _abi.TX_HCURL_I1:
        return val.reshape(12, 3), grad.reshape(12, 3)
    return val[:n], grad[: 3 * n].reshape(n, 3)


def max_threads():
    return lib().orc_max_threads()
