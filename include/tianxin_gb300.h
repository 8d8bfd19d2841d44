/*
 * tianxin_gb300.h -- C-ABI of the GB300-native finite-element assembly path.
 *
 * The library replaces, for the Residual and Jacobian evaluation types, the
 * Tianxin/Panzer volume-assembly path:
 *
 *   Cartesian topology      CartesianConnManager::initialize / buildConnectivity
 *                           (dof-mgr/test/cartesian_topology/CartesianConnManager.cpp:159-331)
 *   DOF numbering           DOFManager::buildGlobalUnknowns
 *                           (dof-mgr/src/Panzer_DOFManager.cpp:449-716)
 *   CRS graph               TpetraLinearObjFactory::buildGhostedGraph
 *                           (disc-fe/src/lof/Panzer_TpetraLinearObjFactory_impl.hpp:559-651)
 *   evaluation (f, W)       ModelEvaluator::evalModelImpl_basic -> AssemblyEngine::evaluate
 *                           (disc-fe/src/Panzer_ModelEvaluator_impl.hpp:1714-1882,
 *                            disc-fe/src/Panzer_AssemblyEngine_impl.hpp:65-182)
 *   Dirichlet rows          TianXin::DirichletEvalautor<Jacobian>::evaluateFields
 *                           (disc-fe/src/evaluators/TianXin_Dirichlet_impl.hpp:55-81)
 *   Neumann flux            AssemblyEngine::evaluateNeumannCondition -> TianXin::Flux
 *                           (disc-fe/src/Panzer_AssemblyEngine_impl.hpp:324-364,
 *                            disc-fe/src/evaluators/TianXin_Neumann_impl.hpp:146-166)
 *   SpMV                    Tpetra::CrsMatrix::apply as called by Belos
 *                           (adapters-stk/example/PoissonExample/main.cpp:402-419)
 *
 * Conventions
 *   - All vector/matrix pointers passed to compute entry points are DEVICE
 *     pointers owned by the caller (like the Tpetra container views that
 *     GatherSolution/ScatterResidual borrow in preEvaluate).  They are
 *     borrowed for the duration of the call only.
 *   - f and the CRS values are SUMMED INTO; the caller zeroes them first,
 *     exactly as ModelEvaluator does before AssemblyEngine::evaluate
 *     (disc-fe/src/Panzer_ModelEvaluator_impl.hpp:1788-1789).
 *   - Every entry point returns 0 on success or a TX_E* status; the message
 *     is available from tx_last_error().  A handle is not thread safe; all
 *     work of a handle is ordered on the handle's CUDA stream.
 *   - Row/column indices are local ids (LIDs): the position of a DOF in the
 *     owned (+ghosted) list.  The CRS layout is Tpetra's local layout after
 *     fillComplete: rowptr int64[N+1], colind int32[nnz] ascending per row.
 */
#ifndef TIANXIN_GB300_H
#define TIANXIN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define TX_OK 0
#define TX_EINVAL 22     /* bad argument / shape                            */
#define TX_ERANGE 34     /* index or size out of range                      */
#define TX_ENOMEM 12     /* device or host allocation failed                */
#define TX_ETIMEDOUT 110 /* a bounded device wait gave up                   */
#define TX_ECUDA 1000    /* CUDA runtime error                              */
#define TX_ESTATE 1001   /* call out of order (e.g. eval before dof_build)  */

/* ------------------------------------------------------------- limits */
#define TX_MAX_BLOCKS 8
#define TX_MAX_FIELDS 3

/* Element topology of the bricks of a block (CartesianConnManager elemTopo:
 * Hexahedron<8>, or Tetrahedron<4> = each brick split into 6 tets). */
enum tx_topology { TX_TOPO_HEX = 0, TX_TOPO_TET = 1 };

/* Equation sets.  POISSON follows Example::PoissonEquationSet
 * (adapters-stk/example/PoissonExample/Example_PoissonEquationSet_impl.hpp:
 * 135-188); MAXWELL follows mini-em's curl-curl + sigma mass
 * (mini-em/src/eqn_sets/MiniEM_EquationSet_Maxwell_impl.hpp:74-245).
 * ELASTICITY, HEAT (k(T) field multiplier) and ELASTODYNAMICS have no
 * equation set in the reference; they are built from the same integrators
 * (GradBasisDotVector with a stress/flux closure, BasisTimesScalar). */
enum tx_physics {
  TX_PHYS_POISSON = 1,        /* field U: k grad u.grad v + c u v - s v (+ udot v)     */
  TX_PHYS_ELASTICITY = 2,     /* fields UX,UY,UZ: sigma(u):grad v - b.v (+ rho udd.v)  */
  TX_PHYS_HEAT = 3,           /* field T: (k0 + k2 T^2) grad T.grad v - q v             */
  TX_PHYS_MAXWELL = 5         /* field E (edges): curl E.curl v / mu + sigma E.v - J.v  */
};

/* Basis family per block (IntrepidBasisFactory names in brackets). */
enum tx_basis {
  TX_HGRAD_C1 = 1, /* HEX: HGRAD_HEX_C1 (8)  TET: HGRAD_TET_C1 (4)  */
  TX_HGRAD_C2 = 2, /* HEX: HGRAD_HEX_C2 (27) TET: HGRAD_TET_C2 (10) */
  TX_HCURL_I1 = 3  /* HEX: HCURL_HEX_I1 (12 edges)                  */
};

/* Brick lattice, CartesianConnManager::initialize(comm, nx,ny,nz, px,py,pz,
 * bx,by,bz, elemTopo) on one rank.  Blocks are enumerated in the
 * reference's getElementBlockIds order: eblock-i_j_k with i slowest. */
typedef struct tx_mesh_desc {
  int32_t nx, ny, nz;                   /* bricks per block per direction           */
  int32_t bx, by, bz;                   /* blocks per direction                     */
  int32_t block_topology[TX_MAX_BLOCKS];/* tx_topology per block                    */
  double lx, ly, lz;                    /* domain [0,lx]x[0,ly]x[0,lz]              */
  double jitter;                        /* interior vertices moved U(-j,j)*h        */
  uint64_t seed;                        /* jitter seed                              */
} tx_mesh_desc;

/* Equation set: fields follow from the physics (field order is
 * alphabetical, DOFManagerFactory, disc-fe/src/Panzer_DOFManagerFactory.cpp:82-94). */
typedef struct tx_equation_set_desc {
  int32_t physics;                      /* tx_physics                               */
  int32_t block_basis[TX_MAX_BLOCKS];   /* tx_basis per block                       */
  int32_t integration_order[TX_MAX_BLOCKS]; /* cubature degree per block; <=0: default
                                           (HEX C1: 2, HEX C2: 4, TET: 2, HCURL: 2)  */
  int32_t source_kind;                  /* see TX_SOURCE_*                          */
  double params[8];                     /* physics coefficients, see below          */
} tx_equation_set_desc;
/* params:
 *  POISSON        [0] k  [1] reaction c  [2] transient multiplier (udot term)
 *                 [3] source constant
 *  ELASTICITY     [0] E  [1] nu  [2..4] body force  [5] rho (mass term on the
 *                 time-derivative vector, see TX_FLAG notes)
 *  HEAT           [0] k0 [1] k2 [2] q
 *  MAXWELL        [0] 1/mu [1] sigma   (J is read from tx_eval_args.aux)    */
enum tx_source {
  TX_SOURCE_CONST = 0,     /* s = params[3] (POISSON)                           */
  TX_SOURCE_SINE = 1,      /* s = 3 pi^2 sin(pi x) sin(pi y) sin(pi z)          */
  TX_SOURCE_AFFINE = 2     /* s = c*(1 + x + 2y + 3z)  (patch/reproduction test)*/
};

/* Evaluation flags. */
#define TX_EVAL_MIXED 0x1u          /* FP32 element contractions, FP64 scatter   */
#define TX_EVAL_DETERMINISTIC 0x2u  /* fixed summation order: coloured scatter, no atomics  */
#define TX_EVAL_PERSISTENT 0x4u     /* every block's worksets in one persistent launch      */
#define TX_EVAL_SCATTER_DIRECT 0x8u /* per-thread row reductions instead of the staged,
                                       row-coalesced CTA scatter (comparison / tuning)     */
/* Tangent evaluation type (GatherSolution_Tpetra<Tangent> seeds the
 * derivative slots from tangent vectors, Panzer_GatherSolution_Tpetra_impl.hpp:
 * 336-389; ScatterResidual_Tpetra<Tangent> sums the derivative slots into the
 * dfdp vectors and leaves f alone, Panzer_ScatterResidual_Tpetra_impl.hpp:
 * 237-270): dfdp[i] += (beta dR/dx + alpha dR/dxdot) tangent[i] for
 * i < n_tangent, without assembling the matrix.  beta = 1, alpha = 0 gives the
 * dx/dp tangents; beta = 0, alpha = 1 those of x_dot.  FP64; f and crs_vals
 * are not touched (pass NULL); not with PERSISTENT or MIXED. */
#define TX_EVAL_TANGENT 0x10u
/* Two-phase evaluation: the element kernels write every element residual and
 * Jacobian to scratch (held by the handle, about E * NE^2 values), then one
 * warp per entity row sums its elements' rows in a fixed order and writes
 * the row once.  f and crs_vals are OVERWRITTEN (no zeroing needed, no
 * atomics, bitwise reproducible).  Needs crs_vals; whole-handle evaluations
 * only (block = -1, all elements); not with TANGENT, PERSISTENT or
 * DETERMINISTIC.  TX_EINVAL when the rows do not fit the gather: an entity
 * row (nf^2 x row length > TX_GATHER_ROW_MAX) or an element's rows
 * (nf^2 x basis count > 128), e.g. quadratic elasticity; see
 * tx_eval_gather_supported. */
#define TX_EVAL_GATHER 0x20u
#define TX_GATHER_ROW_MAX 512
#define TX_MAX_TANGENTS 4

typedef struct tx_eval_args {
  const double* x;         /* solution, LID order (GED "... - X")                       */
  const double* x_dot;     /* time derivative (GED "... - Xdot"); may be NULL           */
  const double* aux;       /* DOF-indexed auxiliary input (MAXWELL: J coefficients)     */
  double alpha, beta, t;   /* d/d x_dot seed, d/d x seed, time                          */
  double* f;               /* residual (summed into); NULL: no residual                 */
  double* crs_vals;        /* Jacobian values (summed into); NULL: Residual type only   */
  int32_t block;           /* -1: every block                                           */
  int64_t elem_begin;      /* workset range inside the block (block >= 0)               */
  int64_t elem_end;        /* -1: to the end of the block                               */
  uint32_t flags;          /* TX_EVAL_*                                                 */
  const double* tangent;   /* TX_EVAL_TANGENT: n_tangent directions, [n_tangent][N]     */
  double* dfdp;            /* TX_EVAL_TANGENT: [n_tangent][N], summed into              */
  int32_t n_tangent;       /* 1 .. TX_MAX_TANGENTS                                      */
} tx_eval_args;

typedef struct tx_handle_s* tx_handle;

/* -------------------------------------------------------------- setup */
/* CartesianConnManager::initialize (CartesianConnManager.cpp:159-294). */
int tx_mesh_create(const tx_mesh_desc* desc, tx_handle* out);
void tx_destroy(tx_handle h);
/* The handle's last error message; tx_last_error(NULL): the calling thread's
 * last failed tx_mesh_create (no handle was made), else "null handle". */
const char* tx_last_error(tx_handle h);

/* Mesh sizes: bricks, elements, vertices (global), blocks. */
int tx_mesh_sizes(tx_handle h, int64_t* n_elements, int64_t* n_vertices, int32_t* n_blocks);
/* Vertex coordinates, node GID order, xyz interleaved (host array of 3*n_vertices). */
int tx_mesh_coordinates(tx_handle h, double* xyz_host);
/* Element ids of a block in the block's element order (ConnManager::getElementBlock). */
int tx_mesh_block_elements(tx_handle h, int32_t block, int64_t* n, int64_t* elems_host);

/* DOFManager::buildGlobalUnknowns (Panzer_DOFManager.cpp:449-716) for the
 * fields of an equation set, plus the CRS graph pattern
 * (TpetraLinearObjFactory::buildGhostedGraph) and the device-side maps. */
int tx_dof_build(tx_handle h, const tx_equation_set_desc* eqset);

/* N = owned DOFs, ndof_max = largest element GID count, nnz of the graph,
 * n_fields of the equation set. */
int tx_dof_sizes(tx_handle h, int64_t* n_dofs, int32_t* ndof_max, int64_t* nnz, int32_t* n_fields);
/* GlobalIndexer::getOwnedIndices: owned_[LID] = GID (host array of N). */
int tx_dof_owned_gids(tx_handle h, int64_t* gids_host);
/* GlobalIndexer::getElementGIDs / getElementLIDs for every element of a block
 * (host arrays n_block_elems x getElementBlockGIDCount(block)). */
int tx_dof_element_gids(tx_handle h, int32_t block, int64_t* gids_host);
int tx_dof_element_lids(tx_handle h, int32_t block, int32_t* lids_host);
int tx_dof_block_gid_count(tx_handle h, int32_t block, int32_t* count);
/* GlobalIndexer::getGIDFieldOffsets(blockId, fieldNum) (Panzer_FieldAggPattern.cpp:369-413). */
int tx_dof_field_offsets(tx_handle h, int32_t block, int32_t field, int32_t* n, int32_t* offsets_host);

/* Dirichlet DOF set: LIDs (sorted, unique; PointEvaluatorBase std::set,
 * TianXin_PointEvaluator_impl.hpp:104,196-202) of the fields in field_mask
 * living on entities that lie on the box sides in side_mask
 * (bit 0 x=0, 1 x=lx, 2 y=0, 3 y=ly, 4 z=0, 5 z=lz).  Call with lids_host
 * NULL to get the count. */
int tx_dirichlet_dofs(tx_handle h, uint32_t side_mask, uint32_t field_mask, int64_t* n, int32_t* lids_host);

/* Graph (Tpetra local layout) into caller DEVICE arrays rowptr[N+1], colind[nnz]. */
int tx_graph_build(tx_handle h, int64_t* rowptr, int32_t* colind);

/* -------------------------------------------------------------- compute */
/* ModelEvaluator::evalModel for f and W, volume fill only
 * (AssemblyEngine::evaluateVolume, Panzer_AssemblyEngine_impl.hpp:134-182):
 * gather -> IntegrationValues2/BasisValues2 -> integrators -> scatter.
 * crs_vals == NULL gives the Residual evaluation type.  Uses the handle's
 * graph (rowptr/colind of tx_graph_build).  In FP64 (without TX_EVAL_MIXED)
 * with the staged scatter (without TX_EVAL_SCATTER_DIRECT) the element
 * matrices of elasticity, Poisson and Nedelec Maxwell blocks are formed
 * symmetric: block (b, a) is the transpose of block (a, b) bit for bit, so
 * the assembled Jacobian is symmetric up to the order of the FP64 sums into
 * each entry. */
int tx_eval(tx_handle h, const tx_eval_args* args);

/* *supported = 1 when TX_EVAL_GATHER holds this handle's rows (after
 * tx_dof_build), else 0; a host query, no device work. */
int tx_eval_gather_supported(tx_handle h, int32_t* supported);

/* The form TX_EVAL_GATHER takes on this handle with TX_EVAL_MIXED:
 * TX_GATHER_LATTICE for one hex8 elasticity block on the whole brick lattice
 * (owner-computes: each CTA owns a column of nodes, sums the rows of its
 * nodes from the eight elements around each in shared memory and registers,
 * and writes every f entry and CRS value once; no element scratch), else
 * TX_GATHER_TWO_PHASE (element rows to scratch, then the row gather), or 0
 * when TX_EVAL_GATHER does not apply.  FP64 evaluations always take the
 * two-phase form.  The replaced step is the atomic sumIntoValues scatter
 * into a zeroed matrix (Panzer_ScatterResidual_Tpetra_impl.hpp:390-439,
 * Panzer_ModelEvaluator_impl.hpp:1788-1789).  A host query. */
#define TX_GATHER_TWO_PHASE 1
#define TX_GATHER_LATTICE 2
int tx_eval_gather_form(tx_handle h, int32_t* form);

/* DirichletEvalautor<Jacobian>/<Residual> through the container's
 * applyDirichletBoundaryCondition (TianXin_Dirichlet_impl.hpp:75-81,
 * lof/Panzer_TpetraLinearObjContainer.hpp:228-238): with a residual f,
 * f[d] = x[d] - g[i] and the Jacobian rows d become unit rows (columns
 * untouched, pivot 1.0: applyDirichletBoundaryConditionToLocalMatrixRows);
 * with f == NULL the columns d are cleared as well, the diagonal kept at 1
 * (applyDirichletBoundaryConditionToLocalMatrixRowsAndColumns).  lids/g are
 * DEVICE arrays of n entries; g may be NULL (g = 0); crs_vals may be NULL. */
int tx_dirichlet_apply(tx_handle h, int64_t n, const int32_t* lids, const double* g,
                       const double* x, double* f, double* crs_vals);

/* ------------------------------------------------------------ Neumann flux
 * A "Neumann Conditions" entry of Type "Flux" (FieldManagerBuilder::
 * setupNeumannFieldManagers, disc-fe/src/Panzer_FieldManagerBuilder.cpp:
 * 417-535): on the side workset of one element block (the block's elements
 * with a local side on the side set, panzer_stk::buildBCWorkset,
 * adapters-stk/src/Panzer_STK_SetupUtilities.cpp:306-392), the residual of
 * DOF field `field` gains
 *     R_b += val(t) * sum_q N_b(xi_q) * w_q * |J t_u x J t_v|
 * (TianXin::Flux::evaluateFields, TianXin_Neumann_impl.hpp:146-166; side
 * cubature of the block's integration order mapped to the element's
 * reference side, face measure = norm of the mapped tangents' cross
 * product).  The flux does not depend on the solution, so a Jacobian
 * evaluation leaves the matrix unchanged and sums the same values into f.
 * Side sets are box sides (bits as tx_dirichlet_dofs).  Each side takes its
 * own local side ordinal; the reference's single side workset uses the
 * first cell's ordinal for all cells (Panzer_STK_SetupUtilities.cpp:383),
 * which agrees whenever a side set's cells share one ordinal (every hex
 * block here). */
enum tx_value_type {       /* WorksetFunctor "Value Type"
                              (disc-fe/src/evaluators/TianXin_WorksetFunctor_impl.hpp) */
  TX_VALUE_CONSTANT = 1,   /* val = value                                              */
  TX_VALUE_LINEAR = 2,     /* ramp to value; the elapse time is read from the same
                              "Value" entry as the value, as the reference does (:67-82) */
  TX_VALUE_TIME_TABLE = 3  /* piecewise linear in (table_t, table_v); t past the last
                              time is an error (:88-121)                                 */
};
typedef struct tx_neumann_desc {
  int32_t block;           /* "Element Block Name" (block index)                        */
  uint32_t side_mask;      /* "SideSet Name": box sides, bit 0 x=0 ... bit 5 z=lz       */
  int32_t field;           /* "DOF Name" (field number); HGRAD blocks                   */
  int32_t value_type;      /* tx_value_type                                             */
  double value;            /* CONSTANT / LINEAR "Value"                                 */
  int32_t n_table;         /* TIME_TABLE points                                         */
  const double* table_t;   /* "Time Values" (HOST, ascending, copied at creation)       */
  const double* table_v;   /* "BC Values" (HOST)                                        */
  int32_t side_set;        /* explicit meshes: side set index + 1 ("SideSet Name" of a  */
                           /* file); 0 = the box sides of side_mask (lattice meshes)    */
} tx_neumann_desc;
/* The functor value at time t (host only, no handle). */
int tx_neumann_value(const tx_neumann_desc* d, double t, double* value);
/* Build the side workset and side tables of a Neumann set (allocates);
 * *id names it in tx_neumann_eval, *n_sides = cells x local sides in it. */
int tx_neumann_create(tx_handle h, const tx_neumann_desc* d, int32_t* id, int64_t* n_sides);
/* f += the set's flux at time t (f DEVICE, LID order).  Launch only. */
int tx_neumann_eval(tx_handle h, int32_t id, double t, double* f);

/* ------------------------------------------------------------ responses
 * Integral responses over element blocks: value = sum over cells and
 * cubature points of integrand(q) * w_q * |det J_q| (TianXin::Response_Integral,
 * disc-fe/src/responses/TianXin_Response_Integral_impl.hpp:106-130; the
 * weighted measure of IntegrationValues2), and for the Jacobian evaluation
 * type the gradient dvalue/dx at the field's LIDs, as panzer's functional
 * response scatters it (disc-fe/src/responses/
 * Panzer_ResponseScatterEvaluator_Functional_impl.hpp:143-171; TianXin's own
 * Response_Integral<Jacobian> sums a placeholder constant instead, :186-200).
 * The error integrands are the Poisson example's "L2 Error" / "H1 Error"
 * functionals (adapters-stk/example/PoissonExample/main.cpp:269-295,
 * Example_ClosureModel_Factory_impl.hpp:147-230) against the manufactured
 * solution of TX_SOURCE_SINE, u* = sin(pi x) sin(pi y) sin(pi z) (the 3-D
 * form of Example_SimpleSolution_impl.hpp:98-100). */
enum tx_integrand {
  TX_INTEGRAND_FIELD = 1,     /* u_field(q)                                          */
  TX_INTEGRAND_L2_ERROR = 2,  /* (u(q) - u*(q))^2                                    */
  TX_INTEGRAND_H1_ERROR = 3,  /* (u(q) - u*(q))^2 + |grad u(q) - grad u*(q)|^2        */
  /* ExtremeValue ("Use Max" true / false; ResponseScatterEvaluator_ExtremeValue,
   * disc-fe/src/responses/Panzer_ResponseScatterEvaluator_ExtremeValue_impl.hpp:136-146):
   * the max / min of u at the cubature points of the covered cells; among
   * equal values the lowest (block, cell, point) wins; d/dx = N_b(q*) at the
   * winning cell's DOFs. */
  TX_INTEGRAND_MAX = 4,
  TX_INTEGRAND_MIN = 5,
  /* Probe (disc-fe/src/responses/Panzer_ResponseScatterEvaluator_Probe_impl.hpp:
   * the containing cell by checkPointwiseInclusion :144 and the reference
   * point by mapToReferenceFrame :187, evaluateFields :262): u at point, in
   * the first cell (blocks in order, cells in order) holding it;
   * d/dx = N_b(xi). */
  TX_INTEGRAND_PROBE = 6
};
typedef struct tx_response_desc {
  int32_t block;           /* element block, -1: every block                          */
  int32_t field;           /* DOF field number (HGRAD blocks)                         */
  int32_t integrand;       /* tx_integrand                                            */
  int32_t cubature_degree; /* <= 0: each block's integration order; hex up to 7, tet 2 */
  /* FIELD over sides instead of cells (a sideset response): the block's sides
   * on these box sides (lattice meshes) or in side set side_set - 1
   * (explicit meshes); the side rule is the block's integration order, as for
   * the Neumann flux.  0 / 0: the cells. */
  uint32_t side_mask;
  int32_t side_set;
  double point[3];         /* PROBE: the point (HOST copy at creation)                */
} tx_response_desc;
/* Build the response (per-block cubature tables; allocates).  PROBE locates
 * the point here: TX_ERANGE when no cell holds it. */
int tx_response_create(tx_handle h, const tx_response_desc* d, int32_t* id);
/* *value (DEVICE double) = the integral at x, summed in a fixed order (the
 * same bits on every call); dvalue_dx (DEVICE [N], may be NULL) += its
 * gradient.  Launch only. */
int tx_response_eval(tx_handle h, int32_t id, const double* x, double* value, double* dvalue_dx);
/* IPCoordinates (disc-fe/src/responses/Panzer_ResponseEvaluatorFactory_IPCoordinates_impl.hpp:79,
 * Panzer_ResponseScatterEvaluator_IPCoordinates_impl.hpp:105): the physical
 * cubature points of a block at cubature_degree (<= 0: its integration
 * order), [n_elem][*nq][3] into xyz (DEVICE; NULL: sizes only).  The tables
 * are cached on the handle, so later calls are launch-only. */
int tx_ip_coordinates(tx_handle h, int32_t block, int32_t cubature_degree, int32_t* nq, double* xyz);

/* y = alpha*A*x + beta*y over a Tpetra-layout CRS (CrsMatrix::apply).
 * vals/x/y are FP64 (TX_SPMV_F64) or FP32 (TX_SPMV_F32). */
#define TX_SPMV_F64 0
#define TX_SPMV_F32 1
/* OR into precision: rowptr/colind/vals lie on the graph tx_graph_build
 * wrote for this handle (n_rows = its DOF count, TX_EINVAL otherwise).  Its
 * nf rows of one entity share one column pattern of nf x nf blocks, so with
 * nf = 3 the product reads one column index per block from the handle's
 * entity graph instead of one per entry (12 -> 8.4 bytes an FP64 entry,
 * 8 -> 4.4 FP32); other nf use the CRS form.  Results equal to rounding. */
#define TX_SPMV_ENTITY_BLOCKS 0x10
int tx_spmv(tx_handle h, int32_t precision, int64_t n_rows, const int64_t* rowptr,
            const int32_t* colind, const void* vals, const void* x, void* y,
            double alpha, double beta);

/* Solve A dx = b with FP64 iterative refinement around an FP32 Jacobi-CG
 * inner solve.  A is the FP64 Tpetra-layout Jacobian (Dirichlet rows unit);
 * the outer residual is either r = b - A x (FP64 SpMV) or, with
 * TX_SOLVE_MATRIX_FREE_RESIDUAL, r = -f(x) from an FP64 Residual evaluation
 * of the handle's equation set, the Neumann sets listed in neumann_ids
 * (at time t) and the Dirichlet residual x_d - g_d.
 * x must satisfy the Dirichlet values on entry (the corrections at those
 * rows are then zero); dirichlet lids (device) are eliminated symmetrically
 * for the CG solve.  Relative residuals are taken against ||r(x0)||.
 * On return stats[0] = outer iterations, stats[1] = total inner CG
 * iterations, stats[2] = final ||r||/||b||. */
#define TX_SOLVE_MATRIX_FREE_RESIDUAL 0x1u
/* Exactly max_outer x max_inner iterations with no host reads (capturable
 * in a CUDA graph after one uncaptured call has sized the work space);
 * statistics go to stats_device. */
#define TX_SOLVE_FIXED_ITERATIONS 0x2u
/* Reuse the FP32 operator of the previous solve (A unchanged). */
#define TX_SOLVE_REUSE_OPERATOR 0x4u
/* The operator lies on the handle's graph: the solver's SpMVs take the
 * entity-block form of TX_SPMV_ENTITY_BLOCKS. */
#define TX_SOLVE_ENTITY_BLOCKS 0x8u
/* Inner preconditioner with TX_SOLVE_ENTITY_BLOCKS and three fields an
 * entity: the inverses of the 3x3 entity diagonal blocks (block Jacobi,
 * Dirichlet rows and columns eliminated, inverted in FP64, applied in FP32)
 * instead of the diagonal; otherwise ignored.  Same solution, fewer inner
 * iterations on vector problems such as elasticity. */
#define TX_SOLVE_BLOCK_JACOBI 0x10u
typedef struct tx_solve_args {
  const int64_t* rowptr; const int32_t* colind; const double* vals;
  const double* b;         /* right-hand side (ignored with MATRIX_FREE: b = -f(x0)) */
  double* x;               /* in: initial guess / state, out: solution        */
  int64_t n_dirichlet; const int32_t* dirichlet_lids;
  const double* dirichlet_g; /* Dirichlet values (device, n_dirichlet) or NULL = 0 */
  double rtol;             /* outer relative residual target, e.g. 1e-10      */
  double inner_rtol;       /* inner FP32 CG relative tolerance, e.g. 1e-5     */
  int32_t max_outer, max_inner;
  uint32_t flags;          /* TX_SOLVE_*                                      */
  const double* x_dot;     /* state for MATRIX_FREE residuals (may be NULL)   */
  double alpha, beta, t;   /* coefficients for MATRIX_FREE residuals          */
  double stats[4];
  double* stats_device;    /* FIXED_ITERATIONS: device double[4] (or NULL)    */
  /* Implicit time integration (MATRIX_FREE only): when x_pred is given the
   * residual is evaluated with x_dot = x_dot_coef * (x - x_pred), the form a
   * Newmark or backward-Euler wrapper presents to evalModel. */
  const double* x_pred;
  double x_dot_coef;
  /* Neumann sets (ids from tx_neumann_create, HOST array) whose flux enters
   * MATRIX_FREE residuals, as evalModel adds them before the Dirichlet rows. */
  int32_t n_neumann;
  const int32_t* neumann_ids;
} tx_solve_args;
int tx_solve_cg_ir(tx_handle h, tx_solve_args* args);

/* ------------------------------------------------------------ CUDA graphs
 * Record the handle's stream work into an executable CUDA graph owned by the
 * handle and replay it: one time step or one Newton step (tx_eval,
 * tx_neumann_eval, tx_dirichlet_apply, tx_spmv, and tx_solve_cg_ir with
 * TX_SOLVE_FIXED_ITERATIONS after one uncaptured call) becomes one launch.
 * Between begin and end only launch-only calls are legal; the captured
 * calls' pointers and scalars are frozen into the graph.  The stream must be
 * a non-default stream (tx_set_stream). */
int tx_graph_capture_begin(tx_handle h);
int tx_graph_capture_end(tx_handle h, int32_t* graph_id);
int tx_graph_launch(tx_handle h, int32_t graph_id);
int tx_graph_destroy(tx_handle h, int32_t graph_id);

/* ------------------------------------------------------------ explicit meshes
 * Unstructured meshes for nodal fields: TX_HGRAD_C1 on hex8 / tet4 blocks, and
 * TX_HGRAD_C2 on hex27 / tet10 blocks (the quadratic nodes carry the DOFs; the
 * geometry is the vertices' trilinear / linear map),
 * from arrays or from an Exodus II file (STK_ExodusReaderFactory::buildMesh,
 * adapters-stk/src/stk_interface/Panzer_STK_ExodusReaderFactory.cpp:111-197,
 * with its element block, side set and node set registration at :178-180).  Node numbers are
 * 0-based and are the vertex GIDs of the numbering: DOF GIDs ascend in node
 * number, fields interleaved, LIDs by first touch as on lattice meshes.
 * Element vertices follow the Exodus/shards order.  Elements are numbered
 * over the whole mesh, blocks in order.  Side sets list (element, side)
 * pairs with the 0-based shards side ordinal (Exodus side - 1: hex faces
 * {0,1,5,4} {1,2,6,5} {2,3,7,6} {0,4,7,3} {0,3,2,1} {4,5,6,7}; tet faces
 * {0,1,3} {1,2,3} {0,3,2} {0,2,1}).  Dirichlet DOFs come from node sets
 * (tx_dirichlet_dofs_node_set) and Neumann sides from side sets
 * (tx_neumann_desc.side_set); the box-side forms give TX_EINVAL here. */
typedef struct tx_explicit_block {
  int32_t topology;        /* TX_TOPO_HEX (8 vertices) or TX_TOPO_TET (4)          */
  int64_t n_elem;
  const int64_t* conn;     /* [n_elem][nodes_per_elem] node numbers (HOST)         */
  int64_t id;              /* element block id                                     */
  const char* name;        /* block name or NULL                                   */
  int32_t nodes_per_elem;  /* 0 or 8 / 4: the vertices; 27 (HEX27) / 10 (TETRA10):  */
                           /* quadratic nodes in shards order, which carry the      */
                           /* TX_HGRAD_C2 DOFs (basis b <-> node b)                 */
} tx_explicit_block;
typedef struct tx_explicit_set {
  int64_t n;               /* side sets: n (element, side) pairs; node sets: n nodes */
  const int64_t* entries;  /* HOST                                                   */
  int64_t id;
  const char* name;        /* or NULL                                                */
} tx_explicit_set;
typedef struct tx_mesh_explicit_desc {
  int64_t n_nodes;
  const double* coords;    /* [n_nodes][3] (HOST)                                  */
  int32_t n_blocks;        /* 1..TX_MAX_BLOCKS                                      */
  const tx_explicit_block* blocks;
  int32_t n_side_sets;
  const tx_explicit_set* side_sets;
  int32_t n_node_sets;
  const tx_explicit_set* node_sets;
} tx_mesh_explicit_desc;
/* err (may be NULL) receives the reason of a failure. */
/* Vertex node numbers [n_elem][*nv] of a block's elements in shards vertex
 * order (lattice and explicit meshes; vertices may be NULL to get *nv). */
int tx_mesh_element_vertices(tx_handle h, int32_t block, int32_t* nv, int64_t* vertices);
int tx_mesh_create_explicit(const tx_mesh_explicit_desc* d, tx_handle* out, char* err, int32_t err_len);
/* A 3-D Exodus II file in the NetCDF classic container (CDF-1/2/5; NetCDF-4
 * files: TX_EINVAL).  Blocks are HEX* or TET*; HEX27 and TETRA10 keep their
 * quadratic nodes (for TX_HGRAD_C2 fields), or with linear != 0 only their
 * vertices (Panzer_STK_QuadraticToLinearMeshFactory's conversion, also the
 * only form of HEX20).  Nodes are
 * renumbered in ascending node_num_map order when the file has one. */
int tx_mesh_create_exodus(const char* path, int32_t linear, tx_handle* out, char* err, int32_t err_len);
typedef struct tx_exodus_summary {
  int32_t version;         /* NetCDF container version 1, 2 or 5                   */
  int64_t dim, n_nodes, n_elem, n_blocks, n_side_sets, n_node_sets;
} tx_exodus_summary;
/* Sizes of an Exodus file of any dimension, without building a mesh. */
int tx_exodus_inspect(const char* path, tx_exodus_summary* s, char* err, int32_t err_len);
/* Sets of an explicit mesh: kind 0 element blocks, 1 side sets, 2 node sets.
 * tx_mesh_set_info: count of sets of that kind in *n when k < 0, else the
 * set's id, name (NUL-terminated, truncated to name_len) and entry count
 * (elements, pairs or nodes); tx_mesh_set_entries copies the entries
 * (side sets: 2n values).  Lattice meshes have no sets (TX_ESTATE). */
int tx_mesh_set_info(tx_handle h, int32_t kind, int32_t k, int64_t* id, char* name, int32_t name_len, int64_t* n);
int tx_mesh_set_entries(tx_handle h, int32_t kind, int32_t k, int64_t* entries);
/* Dirichlet DOF LIDs of the fields in field_mask at the nodes of a node set
 * (ascending; the explicit-mesh form of tx_dirichlet_dofs). */
int tx_dirichlet_dofs_node_set(tx_handle h, int32_t node_set, uint32_t field_mask, int64_t* n, int32_t* lids);

/* ------------------------------------------------------------ blocked layout
 * BlockedDOFManager + BlockedTpetraLinearObjFactory
 * (dof-mgr/src/Panzer_BlockedDOFManager.hpp:68; disc-fe/src/lof/
 * Panzer_BlockedTpetraLinearObjFactory_impl.hpp: getGraph :709,
 * buildTpetraGraph :799, getTpetraMatrix :903, getTpetraDomainVector :933,
 * getBlockRowCount :969, addExcludedPair :295): the
 * equation set's fields are grouped into n_blocks field blocks
 * (field_block[f] = block of field f, fields in field order, every block
 * non-empty).  Block i with b_i fields numbers its DOFs b_i * entity + k (k =
 * the field's place in the block, entities in the interleaved numbering's LID
 * order), block vectors are the product vector's pieces, and block (i, j) of
 * the operator is a Tpetra-layout CRS whose row (entity r, k) holds the b_j
 * columns b_j * m + l of every neighbour entity m of r, ascending.  Host
 * calls; the data calls (graph, split, merge, spmv) are launch-only on the
 * handle's stream.  Pointer arrays (xb, yb, blk_vals) are HOST arrays of
 * DEVICE pointers; blk_vals has n_blocks^2 entries, row-major, NULL for an
 * excluded pair (BlockedTpetraLinearObjFactory::addExcludedPair). */
int tx_blocked_layout(tx_handle h, int32_t n_blocks, const int32_t* field_block);
int tx_blocked_sizes(tx_handle h, int32_t i, int32_t j, int64_t* n_rows, int64_t* n_cols, int64_t* nnz);
/* rowptr [n_rows + 1] int64, colind [nnz] int32 of block (i, j) (getGraph(i, j)) */
int tx_blocked_graph_build(tx_handle h, int32_t i, int32_t j, int64_t* rowptr, int32_t* colind);
/* interleaved vector x [N] -> block vectors xb[k] [n_rows(k)], and back */
int tx_blocked_split_vector(tx_handle h, const double* x, double* const* xb);
int tx_blocked_merge_vector(tx_handle h, const double* const* xb, double* x);
/* interleaved CRS values (tx_graph_build's graph) -> block CRS values */
int tx_blocked_split_matrix(tx_handle h, const double* crs_vals, double* const* blk_vals);
/* y_i = alpha sum_j A_ij x_j + beta y_i over the blocks not excluded (the
 * blocked Thyra operator's apply), FP64 */
int tx_blocked_spmv(tx_handle h, const double* const* blk_vals, const double* const* xb, double* const* yb,
                    double alpha, double beta);

/* Parameter sensitivity of the residual (the dfdp vectors that
 * ScatterResidual_Tpetra<Tangent> fills for an active scalar parameter,
 * Panzer_ScatterResidual_Tpetra_impl.hpp:218-270): dfdp += df/dparams[param]
 * at args' x, x_dot, aux, t over args' blocks and element range, in FP64.
 * param indexes tx_equation_set_desc.params; Dirichlet rows are not
 * touched (zero them for a Dirichlet value independent of the parameter).
 * TX_ERANGE for an index the physics does not use. */
int tx_eval_dfdp(tx_handle h, const tx_eval_args* args, int32_t param, double* dfdp);

/* Worksets (WorksetContainer::setWorksetSize, disc-fe/src/Panzer_WorksetContainer.hpp:104)
 * of the TX_EVAL_PERSISTENT evaluation: consecutive element ranges of every
 * block with sizes drawn uniformly in [min_size, max_size] from seed
 * (min == max: even worksets). */
int tx_set_worksets(tx_handle h, int64_t min_size, int64_t max_size, uint64_t seed);
/* Upper bound on the CTAs of assembly launches (0: occupancy-derived); the
 * tile-shape knob the autotuner sets (HierarchicParallelism's role,
 * disc-fe/src/Panzer_HierarchicParallelism.hpp:78-128). */
int tx_set_grid_cap(tx_handle h, int32_t max_ctas);
/* Launch shape of this handle's CRS SpMV (tx_spmv, the solver's inner and
 * outer products): lanes per row 4/8/16/32 and entries each lane loads per
 * pass 1/2/4, or 16 for aligned 16-byte vector loads (2 FP64 / 4 FP32
 * entries a load; unaligned arrays fall back to 1); (0, 0) picks the lanes
 * from the mean row length.  The
 * autotuner's knob for the SpMV; results equal to rounding for every shape. */
int tx_set_spmv_shape(tx_handle h, int32_t lanes, int32_t unroll);
/* Launch shape of the entity-block form (TX_SPMV_ENTITY_BLOCKS,
 * TX_SOLVE_ENTITY_BLOCKS): lanes per entity 3 (blocks per pass 1/2/3; ten
 * entities a warp, two lanes idle), 4 or 8 (1/2/4) or 16/32 (1/2); (0, 0) =
 * FP64 4 lanes, 4 blocks, FP32 16 lanes, 2. */
int tx_set_spmv_entity_shape(tx_handle h, int32_t lanes, int32_t unroll);
/* Assembly kernel of the per-block mixed evaluation: 0 automatic (the
 * warp-per-element kernel where the element family has one, hex8 elasticity;
 * the CTA-staged kernel elsewhere), 1 always the CTA-staged kernel, 2 the
 * warp-per-element kernel where available, 3 the tensor-core kernel where
 * available (hex8 elasticity R+J: the element contractions P = sum_q W grad N
 * grad N^T and M = sum_q W N N^T as tcgen05 TF32 MMAs with hi/lo splitting,
 * relative error about 1e-6; a bounded MMA wait that gives up is reported by
 * tx_synchronize as TX_ETIMEDOUT).  Results agree to the FP32 summation order
 * (the tensor-core kernel to its splitting error); the autotuner's third
 * knob.  The reference has one AD kernel per integrator and no such choice. */
#define TX_VARIANT_AUTO 0
#define TX_VARIANT_CTA 1
#define TX_VARIANT_WARP 2
#define TX_VARIANT_TENSOR 3
int tx_set_assembly_variant(tx_handle h, int32_t variant);
/* Tile shape of the CTA-staged Jacobian kernel: threads a CTA, 64, 128 (the
 * default; 0 restores it) or 256.  Each element takes TPE threads (its basis
 * count rounded up to a power of two), so a CTA assembles threads / TPE
 * elements: hex8 8, 16 or 32, tet10 4, 8 or 16, hex27 2, 4 or 8.  Blocks of
 * hex8 elasticity, hex27 heat and tet10 heat take the shape; other families
 * keep 128 (TX_EINVAL when no block of the handle has it).  Replaces the
 * team size of Panzer's HierarchicParallelism
 * (disc-fe/src/Panzer_HierarchicParallelism.hpp:78-128); the autotuner's
 * fourth knob. */
int tx_set_cta_threads(tx_handle h, int32_t threads);

/* Many independent meshes in one persistent launch: the volume fill of every
 * block of every handle, cut into worksets, is one work list.  args holds one
 * tx_eval_args per handle (same precision and evaluation type for all).  The
 * reference evaluates meshes one ModelEvaluator at a time; this has no
 * single counterpart there. */
typedef struct tx_batch_s* tx_batch;
int tx_batch_create(const tx_handle* handles, int32_t n, tx_batch* out);
int tx_batch_set_worksets(tx_batch b, int64_t min_size, int64_t max_size, uint64_t seed, int32_t max_ctas);
int tx_batch_eval(tx_batch b, const tx_eval_args* args);
const char* tx_batch_last_error(tx_batch b);
void tx_batch_destroy(tx_batch b);

/* Volume fill that allocates no device memory.  It has no counterpart in the
 * reference.  It exists for callers that may not allocate: applications that
 * reserve all device memory up front in their own pool (a driver allocation
 * outside the pool fails or starves a neighbour), and step loops that must not
 * stall the device, which a cudaFree of grown scratch does.
 * Same result as tx_eval with TX_EVAL_PERSISTENT (every block, even worksets
 * of the size set by tx_set_worksets' min_size, each cut into the same work
 * items; TX_EVAL_MIXED honoured, TX_EVAL_DETERMINISTIC refused, block must
 * be -1), up to the order of the FP64 sums.  Its scratch (work counter,
 * parameter tables, work list) is one static device array holding at most
 * TX_NOALLOC_MAX_WORKSETS work items (about 1.6 MB, kept by every GPU that
 * loads the library until exit); larger work lists are rejected with
 * TX_ERANGE.  The parameter tables reach the device as kernel arguments, not
 * host copies.  The first call on a device looks the array's address up
 * (make that first call before any stream capture).  All calls share the
 * array and each rewrites it: calls that overlap on the GPU race. */
#define TX_NOALLOC_MAX_WORKSETS 65536
int tx_eval_noalloc(tx_handle h, const tx_eval_args* args);

/* Stream the handle's work is ordered on (cudaStream_t as void*); set NULL
 * to use the legacy default stream. */
int tx_set_stream(tx_handle h, void* stream);
/* Waits for the handle's stream; TX_ETIMEDOUT when a bounded device wait of
 * the work since the last call gave up (the tensor-core kernel's MMA waits),
 * TX_ECUDA on a CUDA error. */
int tx_synchronize(tx_handle h);
/* Failure-path check of the bounded device waits: launches one warp that
 * waits on an mbarrier nothing arrives at, gives up after a few thousand
 * polls and sets the handle's status word, so the next tx_synchronize returns
 * TX_ETIMEDOUT (and the one after it TX_OK).  No counterpart in the
 * reference; no GPU fault or hang is involved. */
int tx_selftest_wait_timeout(tx_handle h);

#ifdef __cplusplus
}
#endif
#endif /* TIANXIN_GB300_H */
