// tx_device.cuh -- kernel-side declarations shared by the .cu files.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "tx_internal.h"

namespace tx {

// Everything one assembly launch reads besides the block view.
struct EvalParams {
  const double* coords;      // [n_nodes][3]
  const double* x;           // [N]
  const double* xdot;        // [N] or nullptr
  const double* aux;         // [N] or nullptr
  double alpha, beta, t;
  double* f;                 // [N] or nullptr
  double* vals;              // [nnz] or nullptr
  const int64_t* rowptr;     // [N+1] DOF-level Tpetra rowptr
  int64_t e0, e1;            // element range within the block
  int physics, source_kind;
  double p[8];
  double lam, mu;            // Lame parameters from p[0] (E), p[1] (nu), computed in FP64 on the host
  // Tangent evaluation: dfdp[i][:] += (beta dR/dx + alpha dR/dxdot) tan[i][:], i < ntan
  const double* tan;         // [ntan][n] or nullptr
  double* dfdp;              // [ntan][n]
  int ntan;
  int64_t n;                 // DOF count (the stride of tan and dfdp)
  // Two-phase (gather) evaluation, staged Jacobian kernels only: the element
  // residual and matrix go to scratch (element arithmetic's type) instead of
  // the scatter: kscr[(e * NE + row) * NE + col], rscr[e * NE + row], e the
  // block-local element; launch_gather_rows then writes every row once.
  void* kscr;
  void* rscr;
};
constexpr int kMaxTangents = 4;

// Launch the fused gather -> geometry -> integrators -> scatter kernel for
// elements [e_lo, e_hi) of one block (through perm when given).  atomic=false
// is the coloured, deterministic scatter (one launch per colour).  Returns
// cudaErrorInvalidValue for element families without a kernel.
cudaError_t launch_assemble(const BlockView& B, const EvalParams& P, bool mixed, const int32_t* perm, int64_t e_lo,
                            int64_t e_hi, bool atomic, bool stage, cudaStream_t s, int grid_cap);

// Two-phase (gather) evaluation: the scratch of each mesh block (element
// matrices and residuals of the first phase) and its element-to-row map.
constexpr int kGatherRowMax = TX_GATHER_ROW_MAX;  // nf * nf * (entity row length) the gather kernel holds
constexpr int kGatherElemRowMax = 128;  // nf * (element DOFs): the values of one entity's element rows
struct GatherBlock {
  const void* k;        // [E][NE][NE] element Jacobians (Real)
  const void* r;        // [E][NE] element residuals (Real)
  const uint8_t* epos;  // [E][nb][nb]
  int nb;
};
struct GatherBlocks {
  GatherBlock b[TX_MAX_BLOCKS];
};
// One warp per entity: f[nf*a + c] and the CRS rows of entity a written
// once from the element rows listed in inc (block << 56 | element << 8 |
// local basis, entity-major, CSR by inc_ptr).
cudaError_t launch_gather_rows(int64_t n_ent, int nf, const int64_t* inc_ptr, const int64_t* inc,
                               const GatherBlocks& G, bool mixed, const int64_t* erp, const int64_t* rowptr,
                               double* vals, double* f, cudaStream_t s);

// One chunk of elements of one block view (views[view], params[view]).
struct WorkItem {
  int32_t kind;   // assemble_kind() of the view
  int32_t view;
  int64_t e0, e1;
};
// Element family id of (topology, basis, cubature points, physics); -1 if none.
int assemble_kind(int topo, int basis, int nq, int physics);
// Dynamic shared memory of one family in the batched kernel.
size_t batched_smem_bytes(int kind, bool mixed, bool stage);
// Elements one CTA of the persistent kernel assembles per pass for a family.
int batched_elements_per_pass(int kind);
// Persistent launch over a work list (device arrays); counter is a device int.
cudaError_t launch_assemble_batched(const BlockView* views, const EvalParams* params, const WorkItem* items,
                                    int n_items, int* counter, size_t smem, bool mixed, bool jac, bool stage,
                                    int grid, cudaStream_t s);

// The CTA-staged Jacobian kernel at 64 or 256 threads a CTA (tx_assemble_tiles.cu),
// for the families tile_shape_supported lists (element family ids of assemble_kind).
bool tile_shape_supported(int kind, int threads);
cudaError_t launch_assemble_tile(const BlockView& B, const EvalParams& P, bool mixed, int threads, int64_t e_lo,
                                 int64_t e_hi, cudaStream_t s, int grid_cap);

// Mixed R+J of hex8 elasticity with the element contraction on the tensor
// cores (tcgen05 TF32, hi/lo split; tx_assemble_tc.cu), atomic scatter.  A
// bounded MMA wait that gives up sets bit 0 of *status.
bool tc_supported(const BlockView& B, const EvalParams& P);
cudaError_t launch_assemble_tc(const BlockView& B, const EvalParams& P, int64_t e_lo, int64_t e_hi, int* status,
                               cudaStream_t s, int grid_cap);
// One warp waiting on an mbarrier that never completes: the bounded wait's
// give-up path (sets bit 0 of *status).
cudaError_t launch_wait_selftest(int* status, cudaStream_t s);

// ---- owner-computes lattice assembly (tx_lattice.cu)
// One node of a single-block hex8 brick lattice, in node GID order: FP32
// hi/lo coordinates (x = hi + lo), its entity LID, the first CRS value of
// its three rows (nf = 3) and the position of neighbour (dx, dy, dz) in its
// sorted entity row at npos[(dx + 1) + 3 (dy + 1) + 9 (dz + 1)] (0xff: none).
struct __align__(16) LatticeNode {
  float xh[3];
  int32_t lid;
  float xl[3];
  int32_t pad0;
  int64_t rowstart;
  int64_t pad1;
  uint8_t npos[32];
};
static_assert(sizeof(LatticeNode) == 80, "LatticeNode layout");
struct LatticeArgs {
  int64_t nx = 0, ny = 0, nz = 0;   // bricks per direction
  int64_t zchunk = 0;               // node layers per task (set by launch_lattice_gather)
  int grid = 0;                     // CTA cap (0: one wave of resident CTAs)
  const LatticeNode* nodes = nullptr;
  const float* u = nullptr;         // [nodes][4] FP32 (set by the launcher)
  const float* ud = nullptr;
  const double* ref = nullptr;      // packed RefTables of the block
  float lam = 0, mu = 0, rho = 0, alpha = 0, beta = 0;
  float body[3] = {0, 0, 0};
  double* f = nullptr;              // overwritten (may be null)
  double* vals = nullptr;           // overwritten
};
// Mixed R+J of elasticity on the lattice: f and vals written once.  u_work and
// ud_work hold nodes x 4 floats each (the gathered x and x_dot).
cudaError_t launch_lattice_gather(LatticeArgs A, float4* u_work, float4* ud_work, const double* x, const double* xdot,
                                  cudaStream_t s);
size_t lattice_gather_smem();

// ---- linear algebra (tx_linalg.cu)
cudaError_t launch_expand_rowptr(const int64_t* erowptr, int64_t n_ent, int nf, int64_t* rowptr, cudaStream_t s);
cudaError_t launch_expand_colind(const int64_t* erowptr, const int32_t* ecol, int64_t n_ent, int nf,
                                 const int64_t* rowptr, int32_t* colind, cudaStream_t s);
cudaError_t launch_dirichlet(int64_t n, const int32_t* lids, const double* g, const double* x, double* f,
                             const int64_t* rowptr, const int64_t* erowptr, const int32_t* ecol, int nf,
                             double* vals, cudaStream_t s);
// f[nf*dconn[e][b] + field] += val * sum_q N_b(q) w_q |J t_u x J t_v| over a
// side workset (entries e << 3 | local side), one warp per side.
cudaError_t launch_neumann(const BlockView& B, const double* coords, const int64_t* sides, int64_t n_sides,
                           const double* tables, int stride, int nqf, int nf, int field, double val, double* f,
                           cudaStream_t s);
// CRS SpMV launch shape: lanes per row (4, 8, 16, 32) and entries each lane
// loads per pass (1, 2, 4); {0, 0} picks lanes from the mean row length.
struct SpmvShape {
  int lanes = 0, unroll = 0;
};
bool spmv_shape_valid(SpmvShape sh);
// The entity graph behind the CRS the library expands from it (row nf*r + c
// holds the nf columns nf*m .. nf*m+nf-1 of every neighbour entity m of r, in
// ascending m): the entity-block SpMV reads one column index per nf x nf
// block from it.  Built for nf = kEntityNf (3D elasticity); other nf use the
// CRS form.  Shapes: lanes per entity 4/8/16/32, blocks per lane pass 1/2.
constexpr int kEntityNf = 3;
struct EntityGraph {
  const int64_t* erp = nullptr;
  const int32_t* ecol = nullptr;
  int64_t n_ent = 0;
};
bool entity_shape_valid(SpmvShape sh);
cudaError_t launch_spmv_entity_f64(const EntityGraph& eg, const double* vals, const double* x, double* y, double a,
                                   double b, cudaStream_t s, SpmvShape shape = SpmvShape());
cudaError_t launch_spmv_entity_f32(const EntityGraph& eg, const float* vals, const float* x, float* y, float a,
                                   float b, cudaStream_t s, SpmvShape shape = SpmvShape());
// Warp-per-element mixed assembly (hex8 elasticity, FP32 element math, atomic
// FP64 scatter): the same results as launch_assemble's staged FP32 kernel up to
// the summation order.
bool wpe_supported(const BlockView& B, const EvalParams& P);
cudaError_t launch_assemble_wpe(const BlockView& B, const EvalParams& P, int64_t e_lo, int64_t e_hi, cudaStream_t s,
                                int grid_cap);

// Integral responses: one launch per block writes response_grid(n_elem)
// partial sums (and adds the gradient into dgdx when given); the sum kernel
// adds n partials in order into *value.
constexpr int kResponseCtas = 1024;
int response_grid(int64_t n_elem);
cudaError_t launch_response(const BlockView& B, int nq, const double* coords, const double* x, int nf, int field,
                            int integrand, double* partial, double* dgdx, cudaStream_t s);
cudaError_t launch_response_sum(const double* partial, int64_t n, double* value, cudaStream_t s);
// ExtremeValue: per-CTA best (value, key = block << 48 | cell << 6 | point);
// the final pass picks the winner in index order; the gradient pass adds the
// winner's basis values when it lies in the given block.
cudaError_t launch_response_extreme(const BlockView& B, int nq, const double* x, int nf, int field, bool use_max,
                                    int blk_key, double* pval, int64_t* pidx, cudaStream_t s);
cudaError_t launch_response_extreme_final(const double* pval, const int64_t* pidx, int64_t n, bool use_max,
                                          double* value, int64_t* winner, cudaStream_t s);
cudaError_t launch_response_extreme_grad(const BlockView& B, int nq, int blk_key, const int64_t* winner, int nf,
                                         int field, double* dgdx, cudaStream_t s);
// Integral of a field over a side workset (response_grid(n) partials).
cudaError_t launch_response_side(const BlockView& B, const double* coords, const int64_t* sides, int64_t n,
                                 const double* tables, int stride, int nqf, const double* x, int nf, int field,
                                 double* partial, double* dgdx, cudaStream_t s);
cudaError_t launch_response_probe(const int32_t* lids, const double* N, int nb, const double* x, double* value,
                                  double* dgdx, cudaStream_t s);
// Physical cubature points [E][nq][3] of a block (ref = packed RefTables).
cudaError_t launch_ip_coordinates(const BlockView& B, int nq, const double* coords, double* xyz, cudaStream_t s);
cudaError_t launch_spmv_f64(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* vals,
                            const double* x, double* y, double alpha, double beta, int64_t nnz_hint, cudaStream_t s,
                            SpmvShape shape = SpmvShape());
cudaError_t launch_spmv_f32(int64_t n, const int64_t* rowptr, const int32_t* colind, const float* vals,
                            const float* x, float* y, float alpha, float beta, int64_t nnz_hint, cudaStream_t s,
                            SpmvShape shape = SpmvShape());

// Blocked layout (BlockedTpetraLinearObjFactory): field f lives in block
// fblock[f] at place fpos[f]; block k has bnf[k] fields.
constexpr int kMaxFieldBlocks = 8;
struct BlockedMap {
  int nf = 0, nb = 0;
  int fblock[kMaxFieldBlocks] = {}, fpos[kMaxFieldBlocks] = {}, bnf[kMaxFieldBlocks] = {};
};
// Block vectors (nb pointers) or block matrices (nb * nb, row-major; null =
// excluded pair), passed to kernels by value.
struct BlockPtrs {
  double* p[kMaxFieldBlocks * kMaxFieldBlocks];
};
// CRS graph of block (i, j) with bi and bj fields: the entity graph expanded by bi x bj.
cudaError_t launch_block_graph(const int64_t* erp, const int32_t* ecol, int64_t n_ent, int bi, int bj, int64_t* rp,
                               int32_t* col, cudaStream_t s);
// split: blocks.p[k] <- x (interleaved); else dst (interleaved) <- blocks.p[k].
cudaError_t launch_block_vector(int64_t n_ent, const BlockedMap& M, const double* src, BlockPtrs blocks, double* dst,
                                bool split, cudaStream_t s);
// block CRS values blk.p[i * nb + j] <- interleaved CRS values.
cudaError_t launch_block_split_matrix(const int64_t* erp, int64_t n_ent, const BlockedMap& M, const double* vals,
                                      BlockPtrs blk, cudaStream_t s);

// Work space of the iterative-refinement solver (owned by the handle).
struct SolverWork {
  int64_t n = 0, nnz = 0;
  float* vals32 = nullptr;     // FP32 Jacobian with symmetric Dirichlet elimination
  float* dinv = nullptr;       // Jacobi preconditioner
  float* binv = nullptr;       // block Jacobi: inverses of the 3x3 entity diagonal blocks [n / 3][9]
  bool binv_valid = false;     // binv belongs to the current FP32 operator
  float *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *d = nullptr;
  double* r64 = nullptr;       // outer residual
  double* xdw = nullptr;       // x_dot work vector of implicit integration
  uint8_t* mask = nullptr;     // Dirichlet mask
  double* red = nullptr;       // reduction partials [kRedSlots * kRedBlocks]
  double* scal = nullptr;      // device scalars
  double* host_scal = nullptr; // pinned mirror
  SpmvShape spmv;              // shape of the inner FP32 SpMV
  SpmvShape spmv_eb;           // its shape in the entity-block form
};
constexpr int kRedBlocks = 1024;
constexpr int kRedSlots = 4;

cudaError_t solver_alloc(SolverWork& w, int64_t n, int64_t nnz);
void solver_free(SolverWork& w);

// Outer-residual callback: r = b - A x (or -f(x)); returns 0 or a TX status.
typedef int (*ResidualFn)(void* ctx, const double* x, double* r);

// FP64 iterative refinement around FP32 Jacobi-CG.  stats as tx_solve_args.
int solve_cg_ir(SolverWork& w, const int64_t* rowptr, const int32_t* colind, const double* vals,
                int64_t n_dir, const int32_t* dir_lids, double* x, ResidualFn resid, void* ctx,
                double rtol, double inner_rtol, int max_outer, int max_inner, double* stats,
                cudaStream_t s, std::string& err, bool fixed, bool reuse_op, double* stats_dev,
                const EntityGraph* eg = nullptr, bool block_jacobi = false);

// Vector helpers used by the API layer
cudaError_t launch_fill(double* p, double v, int64_t n, cudaStream_t s);
cudaError_t launch_axpby(double* y, const double* x, double a, double b, int64_t n, cudaStream_t s);
// out = c * (x - xp)
cudaError_t launch_scaled_diff(double* out, const double* x, const double* xp, double c, int64_t n, cudaStream_t s);
// sum of squares of x (FP64) into *out (device), using w.red as scratch
cudaError_t launch_norm2sq(const double* x, int64_t n, double* red, double* out, cudaStream_t s);

}  // namespace tx
