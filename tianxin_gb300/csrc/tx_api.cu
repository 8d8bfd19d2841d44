// tx_api.cu -- the extern "C" boundary of libtianxin_gb300 (declared in
// include/tianxin_gb300.h).  Host set-up lives in tx_setup.cpp, kernels in
// tx_assemble.cu and tx_linalg.cu.
#include <cuda_runtime.h>

#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "tx_device.cuh"

namespace {

struct DevBlock {
  int topo = 0, basis = 0, nq = 0, nb = 0, nv = 0;
  int64_t n_elem = 0;
  int32_t* vconn = nullptr;
  int32_t* dconn = nullptr;
  uint8_t* epos = nullptr;
  int8_t* esign = nullptr;
  double* ref = nullptr;
};

template <typename T>
cudaError_t upload(T*& d, const std::vector<T>& h) {
  if (h.empty()) { d = nullptr; return cudaSuccess; }
  cudaError_t e = cudaMalloc((void**)&d, sizeof(T) * h.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
}

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};
inline void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

struct tx_handle_s {
  tx::Mesh mesh;
  tx::Dofs dofs;
  bool have_dofs = false;       // numbering + device maps ready
  bool have_host_dofs = false;  // numbering ready (host queries work without a GPU)
  double* d_coords = nullptr;
  std::vector<DevBlock> blocks;
  int64_t* d_erowptr = nullptr;
  int32_t* d_ecol = nullptr;
  int64_t* d_rowptr = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  tx::SolverWork solver;
  int grid_cap = 0;

  void free_dofs() {
    for (auto& b : blocks) {
      cudaFree(b.vconn); cudaFree(b.dconn); cudaFree(b.epos); cudaFree(b.esign); cudaFree(b.ref);
    }
    blocks.clear();
    cudaFree(d_erowptr); cudaFree(d_ecol); cudaFree(d_rowptr);
    d_erowptr = nullptr; d_ecol = nullptr; d_rowptr = nullptr;
    tx::solver_free(solver);
    have_dofs = false;
    have_host_dofs = false;
  }
  ~tx_handle_s() {
    free_dofs();
    cudaFree(d_coords);
  }
};

namespace {

int fail(tx_handle h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

template <typename F>
int guarded(tx_handle h, F&& body) {
  try {
    return body();
  } catch (CudaError& e) {
    return fail(h, TX_ECUDA, e.what());
  } catch (std::invalid_argument& e) {
    return fail(h, TX_EINVAL, e.what());
  } catch (std::bad_alloc&) {
    return fail(h, TX_ENOMEM, "host allocation failed");
  } catch (std::exception& e) {
    return fail(h, TX_EINVAL, e.what());
  }
}

// Evaluate every requested block/range (volume fill).
int eval_blocks(tx_handle h, const tx_eval_args& a) {
  const tx::Dofs& D = h->dofs;
  tx::EvalParams P{};
  P.coords = h->d_coords;
  P.x = a.x; P.xdot = a.x_dot; P.aux = a.aux;
  P.alpha = a.alpha; P.beta = a.beta; P.t = a.t;
  P.f = a.f; P.vals = a.crs_vals;
  P.rowptr = h->d_rowptr;
  P.physics = D.eq.physics;
  P.source_kind = D.eq.source_kind;
  for (int i = 0; i < 8; ++i) P.p[i] = D.eq.params[i];
  const bool mixed = (a.flags & TX_EVAL_MIXED) != 0;
  const int b0 = a.block < 0 ? 0 : a.block;
  const int b1 = a.block < 0 ? (int)h->blocks.size() : a.block + 1;
  for (int b = b0; b < b1; ++b) {
    const DevBlock& db = h->blocks[b];
    tx::BlockView V{db.topo, db.basis, db.nq, db.nb, db.nv, db.n_elem, db.vconn, db.dconn, db.epos, db.esign, db.ref};
    P.e0 = 0; P.e1 = db.n_elem;
    if (a.block >= 0) {
      P.e0 = a.elem_begin;
      P.e1 = a.elem_end < 0 ? db.n_elem : a.elem_end;
      if (P.e0 < 0 || P.e1 > db.n_elem || P.e0 > P.e1) return fail(h, TX_ERANGE, "tx_eval: element range outside the block");
    }
    cudaError_t e = tx::launch_assemble(V, P, mixed, h->stream, h->grid_cap);
    if (e == cudaErrorInvalidValue) return fail(h, TX_EINVAL, "tx_eval: no kernel for this element family / cubature");
    if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval: ") + cudaGetErrorString(e));
  }
  return TX_OK;
}

struct MfCtx {
  tx_handle h;
  const double* x_dot;
  double alpha, beta, t;
  int64_t n_dir;
  const int32_t* dir;
  const double* g;
  const double* b;           // matrix-based: r = b - A x
  const int64_t* rowptr;
  const int32_t* colind;
  const double* vals;
  bool matrix_free;
};

int outer_residual(void* vctx, const double* x, double* r) {
  MfCtx* c = (MfCtx*)vctx;
  tx_handle h = c->h;
  const int64_t n = h->dofs.n_dofs;
  if (c->matrix_free) {
    // r = -f(x): FP64 Residual evaluation + Dirichlet residual x_d - g_d
    if (cudaMemsetAsync(r, 0, sizeof(double) * n, h->stream) != cudaSuccess) return TX_ECUDA;
    tx_eval_args a{};
    a.x = x; a.x_dot = c->x_dot; a.alpha = c->alpha; a.beta = c->beta; a.t = c->t;
    a.f = r; a.crs_vals = nullptr; a.block = -1; a.elem_end = -1; a.flags = 0;
    int rc = eval_blocks(h, a);
    if (rc) return rc;
    if (tx::launch_dirichlet(c->n_dir, c->dir, c->g, x, r, nullptr, nullptr, nullptr, h->dofs.nf, nullptr,
                             h->stream) != cudaSuccess)
      return TX_ECUDA;
    if (tx::launch_axpby(r, r, 0.0, -1.0, n, h->stream) != cudaSuccess) return TX_ECUDA;
    return TX_OK;
  }
  if (cudaMemcpyAsync(r, c->b, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess) return TX_ECUDA;
  if (tx::launch_spmv_f64(n, c->rowptr, c->colind, c->vals, x, r, -1.0, 1.0, h->dofs.nnz, h->stream) != cudaSuccess)
    return TX_ECUDA;
  return TX_OK;
}

}  // namespace

extern "C" {

int tx_mesh_create(const tx_mesh_desc* desc, tx_handle* out) {
  if (!desc || !out) return TX_EINVAL;
  *out = nullptr;
  std::unique_ptr<tx_handle_s> h(new (std::nothrow) tx_handle_s);
  if (!h) return TX_ENOMEM;
  int rc = guarded(h.get(), [&]() {
    tx::build_mesh(h->mesh, *desc);
    return TX_OK;
  });
  if (rc) return rc;  // message is lost with the handle; sizes were invalid
  *out = h.release();
  return TX_OK;
}

void tx_destroy(tx_handle h) { delete h; }

const char* tx_last_error(tx_handle h) { return h ? h->err.c_str() : "null handle"; }

int tx_mesh_sizes(tx_handle h, int64_t* n_elements, int64_t* n_vertices, int32_t* n_blocks) {
  if (!h) return TX_EINVAL;
  if (n_elements) *n_elements = h->mesh.n_elements;
  if (n_vertices) *n_vertices = h->mesh.n_nodes;
  if (n_blocks) *n_blocks = h->mesh.nblocks;
  return TX_OK;
}

int tx_mesh_coordinates(tx_handle h, double* xyz) {
  if (!h || !xyz) return TX_EINVAL;
  std::memcpy(xyz, h->mesh.coords.data(), sizeof(double) * h->mesh.coords.size());
  return TX_OK;
}

int tx_mesh_block_elements(tx_handle h, int32_t block, int64_t* n, int64_t* elems) {
  if (!h || !n) return TX_EINVAL;
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "block out of range");
  const auto& v = h->mesh.block_elems[block];
  *n = (int64_t)v.size();
  if (elems) std::memcpy(elems, v.data(), sizeof(int64_t) * v.size());
  return TX_OK;
}

int tx_dof_build(tx_handle h, const tx_equation_set_desc* eq) {
  if (!h || !eq) return TX_EINVAL;
  return guarded(h, [&]() {
    h->free_dofs();
    tx::build_dofs(h->mesh, h->dofs, *eq);
    h->have_host_dofs = true;
    const tx::Dofs& D = h->dofs;
    if (!h->d_coords) ck(upload(h->d_coords, h->mesh.coords), "upload coordinates");
    for (int b = 0; b < h->mesh.nblocks; ++b) {
      const tx::BlockDofs& B = D.blocks[b];
      DevBlock db;
      db.topo = B.topo; db.basis = B.basis; db.nq = B.ref.nq; db.nb = B.nb; db.nv = B.nv;
      db.n_elem = (int64_t)h->mesh.block_elems[b].size();
      h->blocks.push_back(db);
      DevBlock& d = h->blocks.back();
      ck(upload(d.vconn, B.vconn), "upload vconn");
      ck(upload(d.dconn, B.dconn), "upload dconn");
      ck(upload(d.epos, B.epos), "upload epos");
      ck(upload(d.esign, B.esign), "upload esign");
      ck(upload(d.ref, B.ref.packed()), "upload reference tables");
    }
    ck(upload(h->d_erowptr, D.erowptr), "upload entity rowptr");
    ck(upload(h->d_ecol, D.ecol), "upload entity columns");
    ck(cudaMalloc((void**)&h->d_rowptr, sizeof(int64_t) * (D.n_dofs + 1)), "alloc rowptr");
    ck(tx::launch_expand_rowptr(h->d_erowptr, D.n_entities, D.nf, h->d_rowptr, h->stream), "expand rowptr");
    ck(cudaStreamSynchronize(h->stream), "dof_build sync");
    h->have_dofs = true;
    return TX_OK;
  });
}

int tx_dof_sizes(tx_handle h, int64_t* n_dofs, int32_t* ndof_max, int64_t* nnz, int32_t* n_fields) {
  if (!h) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "tx_dof_sizes before tx_dof_build");
  if (n_dofs) *n_dofs = h->dofs.n_dofs;
  if (nnz) *nnz = h->dofs.nnz;
  if (n_fields) *n_fields = h->dofs.nf;
  if (ndof_max) {
    int m = 0;
    for (int b = 0; b < h->mesh.nblocks; ++b) m = std::max(m, tx::dof_block_gid_count(h->dofs, b));
    *ndof_max = m;
  }
  return TX_OK;
}

int tx_dof_owned_gids(tx_handle h, int64_t* gids) {
  if (!h || !gids) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  tx::dof_owned_gids(h->dofs, gids);
  return TX_OK;
}

int tx_dof_block_gid_count(tx_handle h, int32_t block, int32_t* count) {
  if (!h || !count) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "block out of range");
  *count = tx::dof_block_gid_count(h->dofs, block);
  return TX_OK;
}

int tx_dof_element_gids(tx_handle h, int32_t block, int64_t* gids) {
  if (!h || !gids) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "block out of range");
  tx::dof_element_gids(h->mesh, h->dofs, block, gids);
  return TX_OK;
}

int tx_dof_element_lids(tx_handle h, int32_t block, int32_t* lids) {
  if (!h || !lids) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "block out of range");
  tx::dof_element_lids(h->mesh, h->dofs, block, lids);
  return TX_OK;
}

int tx_dof_field_offsets(tx_handle h, int32_t block, int32_t field, int32_t* n, int32_t* offsets) {
  if (!h || !n) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "block out of range");
  if (field < 0 || field >= h->dofs.nf) return fail(h, TX_ERANGE, "field out of range");
  *n = h->dofs.blocks[block].nb;
  if (offsets) tx::dof_field_offsets(h->dofs, block, field, offsets);
  return TX_OK;
}

int tx_dirichlet_dofs(tx_handle h, uint32_t side_mask, uint32_t field_mask, int64_t* n, int32_t* lids) {
  if (!h || !n) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  return guarded(h, [&]() {
    std::vector<int32_t> v = tx::dirichlet_dofs(h->dofs, h->mesh, side_mask, field_mask);
    *n = (int64_t)v.size();
    if (lids) std::memcpy(lids, v.data(), sizeof(int32_t) * v.size());
    return TX_OK;
  });
}

int tx_graph_build(tx_handle h, int64_t* rowptr, int32_t* colind) {
  if (!h || !rowptr || !colind) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_graph_build before tx_dof_build");
  const tx::Dofs& D = h->dofs;
  cudaError_t e = cudaMemcpyAsync(rowptr, h->d_rowptr, sizeof(int64_t) * (D.n_dofs + 1), cudaMemcpyDeviceToDevice,
                                  h->stream);
  if (e == cudaSuccess) e = tx::launch_expand_colind(h->d_erowptr, h->d_ecol, D.n_entities, D.nf, h->d_rowptr, colind, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_graph_build: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_eval(tx_handle h, const tx_eval_args* args) {
  if (!h || !args) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_eval before tx_dof_build");
  if (!args->x) return fail(h, TX_EINVAL, "tx_eval: x is required");
  if (args->block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "tx_eval: block out of range");
  if (h->dofs.eq.physics == TX_PHYS_MAXWELL && !args->aux && args->f)
    return fail(h, TX_EINVAL, "tx_eval: MAXWELL needs the current density J in aux");
  return eval_blocks(h, *args);
}

int tx_dirichlet_apply(tx_handle h, int64_t n, const int32_t* lids, const double* g, const double* x, double* f,
                       double* crs_vals) {
  if (!h) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  if (n < 0 || (n > 0 && !lids)) return fail(h, TX_EINVAL, "tx_dirichlet_apply: lids");
  if (f && !x) return fail(h, TX_EINVAL, "tx_dirichlet_apply: residual needs x");
  cudaError_t e = tx::launch_dirichlet(n, lids, g, x, f, h->d_rowptr, h->d_erowptr, h->d_ecol, h->dofs.nf, crs_vals,
                                       h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_dirichlet_apply: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_spmv(tx_handle h, int32_t precision, int64_t n_rows, const int64_t* rowptr, const int32_t* colind,
            const void* vals, const void* x, void* y, double alpha, double beta) {
  if (!h || !rowptr || !colind || !vals || !x || !y) return TX_EINVAL;
  if (n_rows < 0) return fail(h, TX_EINVAL, "tx_spmv: negative row count");
  const int64_t hint = (h->have_dofs && n_rows == h->dofs.n_dofs) ? h->dofs.nnz : 0;
  cudaError_t e;
  if (precision == TX_SPMV_F64)
    e = tx::launch_spmv_f64(n_rows, rowptr, colind, (const double*)vals, (const double*)x, (double*)y, alpha, beta,
                            hint, h->stream);
  else if (precision == TX_SPMV_F32)
    e = tx::launch_spmv_f32(n_rows, rowptr, colind, (const float*)vals, (const float*)x, (float*)y, (float)alpha,
                            (float)beta, hint, h->stream);
  else
    return fail(h, TX_EINVAL, "tx_spmv: precision must be TX_SPMV_F64 or TX_SPMV_F32");
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_spmv: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_solve_cg_ir(tx_handle h, tx_solve_args* a) {
  if (!h || !a) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_solve_cg_ir before tx_dof_build");
  if (!a->rowptr || !a->colind || !a->vals || !a->x) return fail(h, TX_EINVAL, "tx_solve_cg_ir: missing operand");
  const bool mf = (a->flags & TX_SOLVE_MATRIX_FREE_RESIDUAL) != 0;
  if (!mf && !a->b) return fail(h, TX_EINVAL, "tx_solve_cg_ir: b is required without MATRIX_FREE_RESIDUAL");
  if (a->n_dirichlet > 0 && !a->dirichlet_lids) return fail(h, TX_EINVAL, "tx_solve_cg_ir: dirichlet lids");
  const int64_t n = h->dofs.n_dofs;
  cudaError_t e = tx::solver_alloc(h->solver, n, h->dofs.nnz);
  if (e != cudaSuccess) return fail(h, TX_ENOMEM, std::string("tx_solve_cg_ir: ") + cudaGetErrorString(e));
  MfCtx ctx{h, a->x_dot, a->alpha, a->beta, a->t, a->n_dirichlet, a->dirichlet_lids, a->dirichlet_g,
            a->b, a->rowptr, a->colind, a->vals, mf};
  std::string err;
  int rc = tx::solve_cg_ir(h->solver, a->rowptr, a->colind, a->vals, a->n_dirichlet, a->dirichlet_lids, a->x,
                           outer_residual, &ctx, a->rtol > 0 ? a->rtol : 1e-10,
                           a->inner_rtol > 0 ? a->inner_rtol : 1e-5, a->max_outer > 0 ? a->max_outer : 50,
                           a->max_inner > 0 ? a->max_inner : 100000, a->stats, h->stream, err);
  if (rc == TX_ETIMEDOUT) return fail(h, rc, "tx_solve_cg_ir: did not reach rtol within max_outer iterations");
  if (rc) return fail(h, rc, err);
  return TX_OK;
}

int tx_set_stream(tx_handle h, void* stream) {
  if (!h) return TX_EINVAL;
  h->stream = (cudaStream_t)stream;
  return TX_OK;
}

int tx_synchronize(tx_handle h) {
  if (!h) return TX_EINVAL;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_synchronize: ") + cudaGetErrorString(e));
  return TX_OK;
}

}  // extern "C"
