"""Loader for libtianxin_gb300.so (the in-tree CUDA library) and its C-ABI.

There is no CPU fallback: if the library cannot be built or loaded, every
entry point raises.
"""
import ctypes as C
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtianxin_gb300.so")

# name -> (restype, argtypes); mirrors include/tianxin_gb300.h
P, I32, I64, U32, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_double
SIGNATURES = {
    "tx_mesh_create": (C.c_int, [C.POINTER(_abi.MeshDesc), C.POINTER(P)]),
    "tx_destroy": (None, [P]),
    "tx_last_error": (C.c_char_p, [P]),
    "tx_mesh_sizes": (C.c_int, [P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I32)]),
    "tx_mesh_coordinates": (C.c_int, [P, P]),
    "tx_mesh_block_elements": (C.c_int, [P, I32, C.POINTER(I64), P]),
    "tx_dof_build": (C.c_int, [P, C.POINTER(_abi.EquationSetDesc)]),
    "tx_dof_sizes": (C.c_int, [P, C.POINTER(I64), C.POINTER(I32), C.POINTER(I64), C.POINTER(I32)]),
    "tx_dof_owned_gids": (C.c_int, [P, P]),
    "tx_dof_element_gids": (C.c_int, [P, I32, P]),
    "tx_dof_element_lids": (C.c_int, [P, I32, P]),
    "tx_dof_block_gid_count": (C.c_int, [P, I32, C.POINTER(I32)]),
    "tx_dof_field_offsets": (C.c_int, [P, I32, I32, C.POINTER(I32), P]),
    "tx_dirichlet_dofs": (C.c_int, [P, U32, U32, C.POINTER(I64), P]),
    "tx_graph_build": (C.c_int, [P, P, P]),
    "tx_eval": (C.c_int, [P, C.POINTER(_abi.EvalArgs)]),
    "tx_eval_gather_supported": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "tx_eval_gather_form": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "tx_dirichlet_apply": (C.c_int, [P, I64, P, P, P, P, P]),
    "tx_spmv": (C.c_int, [P, I32, I64, P, P, P, P, P, D, D]),
    "tx_solve_cg_ir": (C.c_int, [P, C.POINTER(_abi.SolveArgs)]),
    "tx_neumann_value": (C.c_int, [C.POINTER(_abi.NeumannDesc), D, C.POINTER(D)]),
    "tx_neumann_create": (C.c_int, [P, C.POINTER(_abi.NeumannDesc), C.POINTER(I32), C.POINTER(I64)]),
    "tx_neumann_eval": (C.c_int, [P, I32, D, P]),
    "tx_eval_dfdp": (C.c_int, [P, C.POINTER(_abi.EvalArgs), I32, P]),
    "tx_response_create": (C.c_int, [P, C.POINTER(_abi.ResponseDesc), C.POINTER(I32)]),
    "tx_response_eval": (C.c_int, [P, I32, P, P, P]),
    "tx_ip_coordinates": (C.c_int, [P, I32, I32, C.POINTER(I32), P]),
    "tx_set_worksets": (C.c_int, [P, I64, I64, C.c_uint64]),
    "tx_set_grid_cap": (C.c_int, [P, I32]),
    "tx_set_spmv_shape": (C.c_int, [P, I32, I32]),
    "tx_set_spmv_entity_shape": (C.c_int, [P, I32, I32]),
    "tx_set_assembly_variant": (C.c_int, [P, I32]),
    "tx_set_cta_threads": (C.c_int, [P, C.c_int32]),
    "tx_graph_capture_begin": (C.c_int, [P]),
    "tx_graph_capture_end": (C.c_int, [P, C.POINTER(I32)]),
    "tx_graph_launch": (C.c_int, [P, I32]),
    "tx_graph_destroy": (C.c_int, [P, I32]),
    "tx_batch_create": (C.c_int, [P, I32, C.POINTER(P)]),
    "tx_batch_set_worksets": (C.c_int, [P, I64, I64, C.c_uint64, I32]),
    "tx_batch_eval": (C.c_int, [P, P]),
    "tx_batch_last_error": (C.c_char_p, [P]),
    "tx_batch_destroy": (None, [P]),
    "tx_eval_noalloc": (C.c_int, [P, C.POINTER(_abi.EvalArgs)]),
    "tx_blocked_layout": (C.c_int, [P, I32, P]),
    "tx_blocked_sizes": (C.c_int, [P, I32, I32, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)]),
    "tx_blocked_graph_build": (C.c_int, [P, I32, I32, P, P]),
    "tx_blocked_split_vector": (C.c_int, [P, P, P]),
    "tx_blocked_merge_vector": (C.c_int, [P, P, P]),
    "tx_blocked_split_matrix": (C.c_int, [P, P, P]),
    "tx_blocked_spmv": (C.c_int, [P, P, P, P, D, D]),
    "tx_mesh_element_vertices": (C.c_int, [P, I32, C.POINTER(I32), P]),
    "tx_mesh_create_explicit": (C.c_int, [C.POINTER(_abi.MeshExplicitDesc), C.POINTER(P), C.c_char_p, I32]),
    "tx_mesh_create_exodus": (C.c_int, [C.c_char_p, I32, C.POINTER(P), C.c_char_p, I32]),
    "tx_exodus_inspect": (C.c_int, [C.c_char_p, C.POINTER(_abi.ExodusSummary), C.c_char_p, I32]),
    "tx_mesh_set_info": (C.c_int, [P, I32, I32, C.POINTER(I64), C.c_char_p, I32, C.POINTER(I64)]),
    "tx_mesh_set_entries": (C.c_int, [P, I32, I32, P]),
    "tx_dirichlet_dofs_node_set": (C.c_int, [P, I32, U32, C.POINTER(I64), P]),
    "tx_set_stream": (C.c_int, [P, P]),
    "tx_synchronize": (C.c_int, [P]),
    "tx_selftest_wait_timeout": (C.c_int, [P]),
}

_lib = None


class TxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"tianxin_gb300 error {code}: {msg}")
        self.code = code


def load(build_if_missing=True):
    """Load (building first if the sources are newer) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _build
        try:
            _build.build()
        except (OSError, RuntimeError) as e:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"libtianxin_gb300.so is missing and could not be built: {e}") from e
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libtianxin_gb300.so not found at {LIB_PATH}; run tianxin_gb300/build.py")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(h, rc, what=""):
    if rc != 0:
        msg = load().tx_last_error(h) if h else b""
        raise TxError(rc, (what + ": " if what else "") + (msg.decode() if msg else ""))
