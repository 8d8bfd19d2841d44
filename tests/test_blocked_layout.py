"""Blocked DOF numbering on the host (no device calls): block sizes, block
nonzero counts and block GIDs.  A field block numbers its DOFs as a
DOFManager built on its fields alone would: ascending entity GID, the
block's fields interleaved in field order (disc-fe/src/Panzer_BlockedDOFManager
builds one DOFManager per field block)."""
import ctypes as C

import numpy as np
import pytest

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A


def _dof(n=(3, 2, 2), topo=A.TX_TOPO_HEX):
    conn = tx.CartesianConnManager(*n, topology=topo)
    return tx.DOFManager(conn, A.equation_set(A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1,
                                              params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0)), require_device=False)


@pytest.mark.parametrize("blocks", [[["UX"], ["UY"], ["UZ"]], [["UX", "UZ"], ["UY"]], [["UZ", "UX", "UY"]]])
def test_block_sizes_and_gids(blocks):
    dof = _dof()
    bd = tx.BlockedDOFManager(dof, blocks)
    ne = dof.n_dofs // 3
    g = dof.getOwnedIndices()
    for i, names in enumerate(blocks):
        n_rows, n_cols, nnz = C.c_int64(), C.c_int64(), C.c_int64()
        assert dof.lib.tx_blocked_sizes(dof.h, i, i, C.byref(n_rows), C.byref(n_cols), C.byref(nnz)) == 0
        b = len(names)
        assert n_rows.value == b * ne and bd.getBlockSize(i) == b * ne
        assert nnz.value == b * b * dof.nnz // 9
        # block GIDs: entity rank (GID order) times b plus the field's place, fields in field order
        order = sorted(names, key=dof.getFieldNum)
        want = []
        for lid in range(0, dof.n_dofs, 3):
            rank = g[lid] // 3
            want += [rank * b + k for k, _ in enumerate(order)]
        assert np.array_equal(bd.getOwnedIndices(i), np.array(want))


def test_blocked_layout_validation():
    dof = _dof()
    lib = dof.lib
    bad = np.array([0, 2, 0], np.int32)  # block 1 empty
    assert lib.tx_blocked_layout(dof.h, 3, bad.ctypes.data) == A.TX_EINVAL
    assert lib.tx_blocked_layout(dof.h, 4, np.zeros(3, np.int32).ctypes.data) == A.TX_EINVAL
    n = C.c_int64()
    assert lib.tx_blocked_sizes(dof.h, 0, 0, C.byref(n), None, None) in (0, A.TX_ESTATE)
