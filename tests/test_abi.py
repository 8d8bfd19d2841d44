"""The C-ABI library loads and exports every symbol the header declares (CPU only)."""
import ctypes
import os
import re

from tianxin_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(HEADER):
        if fn.endswith(".h"):
            txt = open(os.path.join(HEADER, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"^\s*(?:int|void|const char\*)\s+(tx_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_python_signatures_cover_header():
    assert declared_symbols() <= set(_lib.SIGNATURES)


def test_no_device_needed_to_describe_a_mesh():
    lib = _lib.load()
    from tianxin_gb300 import _abi
    d = _abi.mesh_desc((2, 2, 2))
    h = ctypes.c_void_p()
    assert lib.tx_mesh_create(ctypes.byref(d), ctypes.byref(h)) == 0
    lib.tx_destroy(h)
    bad = _abi.mesh_desc((2, 2, 2))
    bad.bx = 0
    assert lib.tx_mesh_create(ctypes.byref(bad), ctypes.byref(h)) == _abi.TX_EINVAL


def test_neumann_value_functors_match_the_oracle():
    # tx_neumann_value is host logic: the WorksetFunctor values, checked
    # against the oracle's restatement, including the reference's Linear
    # ramp whose elapse time is its own "Value" and the TimeTable error.
    import pytest
    from oracle import oracle as O
    import tianxin_gb300 as tx
    from tianxin_gb300 import _abi as A
    tt, tv = [0.0, 0.5, 2.0, 3.0], [1.0, -2.0, 4.0, 4.0]
    for t in (-1.0, 0.0, 0.25, 0.5, 1.0, 2.0, 2.9, 3.0):
        assert tx.neumann_value("TimeTable", times=tt, values=tv, t=t) == O.workset_functor("TimeTable", times=tt,
                                                                                              values=tv, t=t)
    for v, t in [(3.0, 1.0), (3.0, 3.0), (3.0, 7.0), (3.0, -2.0), (0.5, 0.25)]:
        assert tx.neumann_value("Linear", v, t=t) == O.workset_functor("Linear", v, t=t)
        assert tx.neumann_value("Constant", v, t=t) == v
    with pytest.raises(tx.TxError) as e:
        tx.neumann_value("TimeTable", times=tt, values=tv, t=3.5)
    assert e.value.code == A.TX_ERANGE


def test_spmv_shape_validation_needs_no_device():
    import tianxin_gb300 as tx
    from tianxin_gb300 import _abi as A
    conn = tx.CartesianConnManager(1, 1, 1)
    lib = _lib.load()
    assert lib.tx_set_spmv_shape(conn.h, 16, 2) == 0
    assert lib.tx_set_spmv_shape(conn.h, 0, 0) == 0
    assert lib.tx_set_spmv_shape(conn.h, 12, 2) == A.TX_EINVAL
    assert lib.tx_set_spmv_shape(conn.h, 8, 3) == A.TX_EINVAL
    assert lib.tx_set_spmv_shape(conn.h, 8, 16) == 0
    assert lib.tx_set_spmv_entity_shape(conn.h, 8, 2) == 0
    assert lib.tx_set_spmv_entity_shape(conn.h, 0, 0) == 0
    assert lib.tx_set_spmv_entity_shape(conn.h, 8, 4) == 0
    assert lib.tx_set_spmv_entity_shape(conn.h, 16, 4) == A.TX_EINVAL
    assert lib.tx_set_spmv_entity_shape(conn.h, 3, 3) == 0
    assert lib.tx_set_spmv_entity_shape(conn.h, 3, 4) == A.TX_EINVAL
    assert lib.tx_set_spmv_entity_shape(conn.h, 2, 1) == A.TX_EINVAL


def test_two_phase_fit_is_a_host_query():
    """TX_EVAL_GATHER holds linear elasticity's rows, not quadratic elasticity's
    (81 element DOFs, 125-entity rows): the query answers without a device."""
    import ctypes as C
    import tianxin_gb300 as tx
    from tianxin_gb300 import _abi as A
    lib = _lib.load()
    conn = tx.CartesianConnManager(2, 2, 2)
    ok = C.c_int32(-1)
    assert lib.tx_eval_gather_supported(conn.h, C.byref(ok)) == A.TX_ESTATE
    params = (1.0, 0.3, 0.0, 0.0, -1.0, 0.0)
    for basis, fits in ((A.TX_HGRAD_C1, 1), (A.TX_HGRAD_C2, 0)):
        tx.DOFManager(conn, A.equation_set(A.TX_PHYS_ELASTICITY, basis, params=params), require_device=False)
        assert lib.tx_eval_gather_supported(conn.h, C.byref(ok)) == 0 and ok.value == fits
    tx.DOFManager(conn, A.equation_set(A.TX_PHYS_HEAT, A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0)), require_device=False)
    assert lib.tx_eval_gather_supported(conn.h, C.byref(ok)) == 0 and ok.value == 1


def test_size_limits_are_refused_before_allocation():
    """Index widths: vertex and DOF numbers are int32 on the device (CRS column indices), so a lattice with
    2^31 or more vertices is refused at creation, from its sizes alone, and block counts above
    TX_MAX_BLOCKS likewise."""
    import time

    import pytest
    import tianxin_gb300 as tx
    from tianxin_gb300 import _abi as A
    t0 = time.perf_counter()
    with pytest.raises(tx.TxError) as e:
        tx.CartesianConnManager(1291, 1291, 1291)  # 1292^3 = 2.16e9 vertices
    assert e.value.code == A.TX_EINVAL and "2^31" in str(e.value)
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(tx.TxError) as e:
        tx.CartesianConnManager(2, 2, 2, 3, 3, 1)  # nine blocks
    assert "too many blocks" in str(e.value)
