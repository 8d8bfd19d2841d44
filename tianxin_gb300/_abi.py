"""ctypes mirror of the structs and constants in include/tianxin_gb300.h."""
import ctypes as C

TX_OK = 0
TX_EINVAL = 22
TX_ERANGE = 34
TX_ENOMEM = 12
TX_ETIMEDOUT = 110
TX_ECUDA = 1000
TX_ESTATE = 1001

TX_MAX_BLOCKS = 8
TX_MAX_FIELDS = 3

TX_TOPO_HEX = 0
TX_TOPO_TET = 1

TX_PHYS_POISSON = 1
TX_PHYS_ELASTICITY = 2
TX_PHYS_HEAT = 3
TX_PHYS_MAXWELL = 5

TX_HGRAD_C1 = 1
TX_HGRAD_C2 = 2
TX_HCURL_I1 = 3

TX_SOURCE_CONST = 0
TX_SOURCE_SINE = 1
TX_SOURCE_AFFINE = 2

TX_EVAL_MIXED = 0x1
TX_EVAL_DETERMINISTIC = 0x2
TX_EVAL_PERSISTENT = 0x4
TX_EVAL_SCATTER_DIRECT = 0x8
TX_EVAL_TANGENT = 0x10
TX_EVAL_GATHER = 0x20
TX_GATHER_TWO_PHASE = 1
TX_GATHER_LATTICE = 2
TX_MAX_TANGENTS = 4

TX_SPMV_F64 = 0
TX_SPMV_F32 = 1
TX_SPMV_ENTITY_BLOCKS = 0x10

TX_SOLVE_MATRIX_FREE_RESIDUAL = 0x1
TX_SOLVE_FIXED_ITERATIONS = 0x2
TX_SOLVE_REUSE_OPERATOR = 0x4
TX_SOLVE_ENTITY_BLOCKS = 0x8
TX_SOLVE_BLOCK_JACOBI = 0x10

TX_INTEGRAND_FIELD = 1
TX_INTEGRAND_L2_ERROR = 2
TX_INTEGRAND_H1_ERROR = 3
TX_INTEGRAND_MAX = 4
TX_INTEGRAND_MIN = 5
TX_INTEGRAND_PROBE = 6

TX_VALUE_CONSTANT = 1
TX_VALUE_LINEAR = 2
TX_VALUE_TIME_TABLE = 3

# side bits for Dirichlet sets
SIDE_XMIN, SIDE_XMAX, SIDE_YMIN, SIDE_YMAX, SIDE_ZMIN, SIDE_ZMAX = (1 << i for i in range(6))
ALL_SIDES = 0x3F


class MeshDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("bx", C.c_int32), ("by", C.c_int32), ("bz", C.c_int32),
        ("block_topology", C.c_int32 * TX_MAX_BLOCKS),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("jitter", C.c_double),
        ("seed", C.c_uint64),
    ]


class EquationSetDesc(C.Structure):
    _fields_ = [
        ("physics", C.c_int32),
        ("block_basis", C.c_int32 * TX_MAX_BLOCKS),
        ("integration_order", C.c_int32 * TX_MAX_BLOCKS),
        ("source_kind", C.c_int32),
        ("params", C.c_double * 8),
    ]


class EvalArgs(C.Structure):
    _fields_ = [
        ("x", C.c_void_p), ("x_dot", C.c_void_p), ("aux", C.c_void_p),
        ("alpha", C.c_double), ("beta", C.c_double), ("t", C.c_double),
        ("f", C.c_void_p), ("crs_vals", C.c_void_p),
        ("block", C.c_int32),
        ("elem_begin", C.c_int64), ("elem_end", C.c_int64),
        ("flags", C.c_uint32),
        ("tangent", C.c_void_p), ("dfdp", C.c_void_p), ("n_tangent", C.c_int32),
    ]


class SolveArgs(C.Structure):
    _fields_ = [
        ("rowptr", C.c_void_p), ("colind", C.c_void_p), ("vals", C.c_void_p),
        ("b", C.c_void_p), ("x", C.c_void_p),
        ("n_dirichlet", C.c_int64), ("dirichlet_lids", C.c_void_p), ("dirichlet_g", C.c_void_p),
        ("rtol", C.c_double), ("inner_rtol", C.c_double),
        ("max_outer", C.c_int32), ("max_inner", C.c_int32),
        ("flags", C.c_uint32),
        ("x_dot", C.c_void_p),
        ("alpha", C.c_double), ("beta", C.c_double), ("t", C.c_double),
        ("stats", C.c_double * 4),
        ("stats_device", C.c_void_p),
        ("x_pred", C.c_void_p), ("x_dot_coef", C.c_double),
        ("n_neumann", C.c_int32), ("neumann_ids", C.c_void_p),
    ]


class ResponseDesc(C.Structure):
    _fields_ = [("block", C.c_int32), ("field", C.c_int32), ("integrand", C.c_int32), ("cubature_degree", C.c_int32),
                ("side_mask", C.c_uint32), ("side_set", C.c_int32), ("point", C.c_double * 3)]


class NeumannDesc(C.Structure):
    _fields_ = [
        ("block", C.c_int32), ("side_mask", C.c_uint32), ("field", C.c_int32), ("value_type", C.c_int32),
        ("value", C.c_double),
        ("n_table", C.c_int32), ("table_t", C.c_void_p), ("table_v", C.c_void_p),
        ("side_set", C.c_int32),
    ]


class ExplicitBlock(C.Structure):
    _fields_ = [("topology", C.c_int32), ("n_elem", C.c_int64), ("conn", C.c_void_p), ("id", C.c_int64),
                ("name", C.c_char_p), ("nodes_per_elem", C.c_int32)]


class ExplicitSet(C.Structure):
    _fields_ = [("n", C.c_int64), ("entries", C.c_void_p), ("id", C.c_int64), ("name", C.c_char_p)]


class MeshExplicitDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("coords", C.c_void_p),
                ("n_blocks", C.c_int32), ("blocks", C.POINTER(ExplicitBlock)),
                ("n_side_sets", C.c_int32), ("side_sets", C.POINTER(ExplicitSet)),
                ("n_node_sets", C.c_int32), ("node_sets", C.POINTER(ExplicitSet))]


class ExodusSummary(C.Structure):
    _fields_ = [("version", C.c_int32), ("dim", C.c_int64), ("n_nodes", C.c_int64), ("n_elem", C.c_int64),
                ("n_blocks", C.c_int64), ("n_side_sets", C.c_int64), ("n_node_sets", C.c_int64)]


def mesh_desc(n, blocks=(1, 1, 1), topology=TX_TOPO_HEX, lengths=(1.0, 1.0, 1.0), jitter=0.0, seed=0):
    """Brick lattice of n=(nx,ny,nz) bricks per block; topology is one value or one per block."""
    if isinstance(n, int):
        n = (n, n, n)
    d = MeshDesc()
    d.nx, d.ny, d.nz = n
    d.bx, d.by, d.bz = blocks
    nb = blocks[0] * blocks[1] * blocks[2]
    topo = [topology] * nb if isinstance(topology, int) else list(topology)
    for i, t in enumerate(topo[:TX_MAX_BLOCKS]):  # more blocks: the library refuses the description
        d.block_topology[i] = t
    d.lx, d.ly, d.lz = lengths
    d.jitter = jitter
    d.seed = seed
    return d


def equation_set(physics, basis=TX_HGRAD_C1, params=(), source_kind=TX_SOURCE_CONST, integration_order=None,
                 n_blocks=TX_MAX_BLOCKS):
    q = EquationSetDesc()
    q.physics = physics
    bas = [basis] * TX_MAX_BLOCKS if isinstance(basis, int) else list(basis) + [basis[-1]] * (TX_MAX_BLOCKS - len(basis))
    for i in range(TX_MAX_BLOCKS):
        q.block_basis[i] = bas[i]
    io = integration_order
    for i in range(TX_MAX_BLOCKS):
        if io is None:
            q.integration_order[i] = 0
        elif isinstance(io, int):
            q.integration_order[i] = io
        else:
            q.integration_order[i] = io[i] if i < len(io) else io[-1]
    q.source_kind = source_kind
    for i, p in enumerate(params):
        q.params[i] = p
    return q


def field_names(physics):
    return {TX_PHYS_POISSON: ["U"], TX_PHYS_ELASTICITY: ["UX", "UY", "UZ"], TX_PHYS_HEAT: ["T"],
            TX_PHYS_MAXWELL: ["E"]}[physics]
