// tx_api.cu -- the extern "C" boundary of libtianxin_gb300 (declared in
// include/tianxin_gb300.h).  Host set-up lives in tx_setup.cpp, kernels in
// tx_assemble.cu and tx_linalg.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "tx_device.cuh"

namespace {

struct DevBlock {
  int topo = 0, basis = 0, nq = 0, nb = 0, nv = 0, kind = -1;
  int64_t n_elem = 0;
  int32_t* vconn = nullptr;
  int32_t* dconn = nullptr;
  uint8_t* epos = nullptr;
  int8_t* esign = nullptr;
  double* ref = nullptr;
  float* ref32 = nullptr;
  int32_t* color_perm = nullptr;
  std::vector<int64_t> color_offsets;
  tx::BlockView view() const {
    return tx::BlockView{topo, basis, nq, nb, nv, n_elem, vconn, dconn, epos, esign, ref, ref32};
  }
};

// Pinned staging for small per-call tables (kernel parameters of batched
// launches): the copy is stream ordered; before the host buffer is reused
// the previous copy is waited for.
struct Staging {
  void* host = nullptr;
  void* dev = nullptr;
  size_t cap = 0;
  cudaEvent_t ev = nullptr;
  bool pending = false;
  cudaError_t put(const void* src, size_t n, cudaStream_t s) {
    cudaError_t e;
    if (pending && (e = cudaEventSynchronize(ev)) != cudaSuccess) return e;
    if (n > cap) {
      cudaFreeHost(host);
      cudaFree(dev);
      cap = n < 4096 ? 4096 : 2 * n;
      if ((e = cudaMallocHost(&host, cap)) != cudaSuccess) return e;
      if ((e = cudaMalloc(&dev, cap)) != cudaSuccess) return e;
      if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
    }
    std::memcpy(host, src, n);
    if ((e = cudaMemcpyAsync(dev, host, n, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    pending = true;
    return cudaEventRecord(ev, s);
  }
  void release() {
    if (pending && ev) cudaEventSynchronize(ev);
    cudaFreeHost(host);
    cudaFree(dev);
    if (ev) cudaEventDestroy(ev);
    *this = Staging();
  }
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

// One Neumann "Flux" set: its side workset and side tables on the device.
struct NeumannSet {
  tx_neumann_desc desc{};
  std::vector<double> table_t, table_v;  // TIME_TABLE copy
  int64_t n_sides = 0;
  int64_t* sides = nullptr;
  double* tables = nullptr;
  int stride = 0, nqf = 0;
};

// One integral response: per-block cubature tables and the partial sums.
struct ResponseSet {
  tx_response_desc desc{};
  std::vector<int> blocks, nq;     // blocks it covers and their point counts
  std::vector<double*> tables;     // packed RefTables per covered block
  std::vector<int64_t> offset;     // first partial of each covered block
  double* partial = nullptr;
  int64_t n_partial = 0;
  int64_t* pidx = nullptr;          // ExtremeValue: per-partial winner keys
  int64_t* winner = nullptr;        // ExtremeValue: the final winner key
  bool side = false;                // FIELD over a side workset per covered block
  std::vector<int64_t*> sides;
  std::vector<int64_t> n_sides;
  std::vector<int> stride, nqf;
  int32_t* probe_lids = nullptr;    // PROBE: the cell's field DOFs and N_b(xi)
  double* probe_n = nullptr;
  int probe_nb = 0;
};

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
  // worksets of the persistent (one launch) evaluation
  int64_t ws_min = 512, ws_max = 512;
  uint64_t ws_seed = 0;
  std::vector<tx::WorkItem> items;   // host copy, rebuilt when the worksets change
  tx::WorkItem* d_items = nullptr;
  int* d_counter = nullptr;
  Staging stage;
  std::vector<NeumannSet> neumann;
  std::vector<ResponseSet> responses;
  tx::SpmvShape spmv;     // SpMV launch shape ({0, 0}: automatic)
  tx::SpmvShape spmv_eb;  // the same for the entity-block form
  int variant = 0;     // assembly kernel: 0 automatic, 1 CTA-staged, 2 warp per element, 3 tensor cores
  int* d_wait_status = nullptr;  // bounded device waits that gave up (bit 0: the tensor-core kernel's MMA waits)
  int cta_threads = 0; // threads a CTA of the staged Jacobian kernel (0: 128); tx_set_cta_threads
  std::vector<cudaGraphExec_t> graphs;  // tx_graph_capture_end; destroyed slots are null
  bool capturing = false;
  // two-phase evaluation: entity -> (block, element, local basis) incidence
  // (CSR, device) and the element scratch of the first phase
  int64_t* d_inc_ptr = nullptr;
  int64_t* d_inc = nullptr;
  unsigned char* gather_scratch = nullptr;
  size_t gather_bytes = 0;
  // owner-computes lattice assembly (single-block hex8 elasticity lattices):
  // per-node records and the gathered x / x_dot of a call
  tx::LatticeNode* d_lat = nullptr;
  float4* d_lat_u = nullptr;
  float4* d_lat_ud = nullptr;
  // cubature tables of tx_ip_coordinates per (block, degree)
  struct IpTables { int block, degree, nq; double* tables; };
  std::vector<IpTables> ip_tables;
  // blocked layout (tx_blocked_layout) and the device graphs of its blocks,
  // one per (fields in row block, fields in column block)
  tx::BlockedMap blocked;
  struct BlockGraph { int64_t* rp = nullptr; int32_t* col = nullptr; };
  BlockGraph block_graphs[tx::kMaxFieldBlocks + 1][tx::kMaxFieldBlocks + 1];

  void free_block_graphs() {
    for (auto& row : block_graphs)
      for (auto& g : row) { cudaFree(g.rp); cudaFree(g.col); g = BlockGraph(); }
  }

  void free_dofs() {
    for (auto& ns : neumann) { cudaFree(ns.sides); cudaFree(ns.tables); }
    neumann.clear();
    for (auto& rs : responses) {
      for (double* t : rs.tables) cudaFree(t);
      for (int64_t* sd : rs.sides) cudaFree(sd);
      cudaFree(rs.partial); cudaFree(rs.pidx); cudaFree(rs.winner);
      cudaFree(rs.probe_lids); cudaFree(rs.probe_n);
    }
    responses.clear();
    for (auto& t : ip_tables) cudaFree(t.tables);
    ip_tables.clear();
    cudaFree(d_inc_ptr); cudaFree(d_inc); cudaFree(gather_scratch);
    d_inc_ptr = nullptr; d_inc = nullptr; gather_scratch = nullptr; gather_bytes = 0;
    cudaFree(d_lat); cudaFree(d_lat_u); cudaFree(d_lat_ud);
    d_lat = nullptr; d_lat_u = nullptr; d_lat_ud = nullptr;
    for (auto& b : blocks) {
      cudaFree(b.vconn); cudaFree(b.dconn); cudaFree(b.epos); cudaFree(b.esign); cudaFree(b.ref); cudaFree(b.ref32);
      cudaFree(b.color_perm);
    }
    cudaFree(d_items); cudaFree(d_counter);
    d_items = nullptr; d_counter = nullptr;
    items.clear();
    stage.release();
    blocks.clear();
    cudaFree(d_erowptr); cudaFree(d_ecol); cudaFree(d_rowptr);
    d_erowptr = nullptr; d_ecol = nullptr; d_rowptr = nullptr;
    tx::solver_free(solver);
    free_block_graphs();
    blocked = tx::BlockedMap();
    have_dofs = false;
    have_host_dofs = false;
  }
  ~tx_handle_s() {
    for (auto g : graphs)
      if (g) cudaGraphExecDestroy(g);
    free_dofs();
    cudaFree(d_coords);
    cudaFree(d_wait_status);
  }
};

namespace {

// The calling thread's last failed tx_mesh_create message.
std::string& create_error() {
  thread_local std::string e;
  return e;
}

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
  } catch (std::out_of_range& e) {
    return fail(h, TX_ERANGE, e.what());
  } catch (std::bad_alloc&) {
    return fail(h, TX_ENOMEM, "host allocation failed");
  } catch (std::exception& e) {
    return fail(h, TX_EINVAL, e.what());
  }
}

// Coefficients that replace the equation set's in a parameter-derivative evaluation.
struct CoefOverride {
  double p[8];
  double lam, mu;
  int source_kind;
  bool zero_aux;
};

tx::EvalParams make_params(tx_handle h, const tx_eval_args& a, const CoefOverride* ov = nullptr) {
  const tx::Dofs& D = h->dofs;
  tx::EvalParams P{};
  P.coords = h->d_coords;
  P.x = a.x; P.xdot = a.x_dot; P.aux = a.aux;
  P.alpha = a.alpha; P.beta = a.beta; P.t = a.t;
  P.f = a.f; P.vals = a.crs_vals;
  P.rowptr = h->d_rowptr;
  P.n = D.n_dofs;
  if (a.flags & TX_EVAL_TANGENT) {
    P.tan = a.tangent; P.dfdp = a.dfdp; P.ntan = a.n_tangent;
    P.f = nullptr; P.vals = nullptr;
  }
  P.physics = D.eq.physics;
  P.source_kind = D.eq.source_kind;
  for (int i = 0; i < 8; ++i) P.p[i] = D.eq.params[i];
  if (D.eq.physics == TX_PHYS_ELASTICITY) {
    const double E = D.eq.params[0], nu = D.eq.params[1];
    P.lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    P.mu = E / (2.0 * (1.0 + nu));
  }
  if (ov) {
    for (int i = 0; i < 8; ++i) P.p[i] = ov->p[i];
    P.lam = ov->lam; P.mu = ov->mu;
    P.source_kind = ov->source_kind;
    if (ov->zero_aux) P.aux = nullptr;
  }
  return P;
}

// The residual is affine in every coefficient of these equation sets except
// Poisson's ratio (through the Lame parameters), so dR/dp_i is the residual
// evaluated with a derivative coefficient set: p_i -> 1 and the rest -> 0
// (sources kept only where they scale with p_i), and for E and nu the Lame
// derivatives.  Returns false for a parameter the physics does not use.
bool derivative_coefficients(const tx_equation_set_desc& q, int i, CoefOverride& ov) {
  for (int k = 0; k < 8; ++k) ov.p[k] = 0.0;
  ov.lam = ov.mu = 0.0;
  ov.source_kind = TX_SOURCE_CONST;
  ov.zero_aux = false;
  switch (q.physics) {
    case TX_PHYS_POISSON:
      if (i > 3) return false;
      if (i == 3 && q.source_kind != TX_SOURCE_CONST) return true;  // the source does not scale with p3
      ov.p[i] = 1.0;
      if (i == 1 && q.source_kind == TX_SOURCE_AFFINE) ov.source_kind = TX_SOURCE_AFFINE;  // s = c (1 + x + 2y + 3z)
      return true;
    case TX_PHYS_ELASTICITY: {
      if (i > 5) return false;
      const double E = q.params[0], nu = q.params[1];
      if (i == 0) {  // lambda, mu proportional to E
        ov.lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
        ov.mu = 1.0 / (2.0 * (1.0 + nu));
      } else if (i == 1) {
        const double d = (1.0 + nu) * (1.0 - 2.0 * nu);
        ov.lam = E * (1.0 + 2.0 * nu * nu) / (d * d);
        ov.mu = -E / (2.0 * (1.0 + nu) * (1.0 + nu));
      } else {
        ov.p[i] = 1.0;  // body force component or rho
      }
      return true;
    }
    case TX_PHYS_HEAT:
      if (i > 2) return false;
      ov.p[i] = 1.0;
      return true;
    case TX_PHYS_MAXWELL:
      if (i > 1) return false;
      ov.p[i] = 1.0;
      ov.zero_aux = true;  // the current density does not scale with 1/mu or sigma
      return true;
    default:
      return false;
  }
}

// Work list of a handle: every block cut into worksets, and each workset into
// device work items of at most kItemPasses CTA passes of its element family, so
// that a workset of heavy elements (4 hex27 per CTA pass) is shared by several
// CTAs instead of serialising one of them.
constexpr int kItemPasses = 8;
void build_items(tx_handle h, std::vector<tx::WorkItem>& out, int view_base) {
  for (size_t b = 0; b < h->blocks.size(); ++b) {
    const DevBlock& db = h->blocks[b];
    const int64_t cap = (int64_t)tx::batched_elements_per_pass(db.kind) * kItemPasses;
    std::vector<int64_t> wb = tx::workset_bounds(db.n_elem, h->ws_min, h->ws_max, h->ws_seed + 7919 * b);
    for (size_t k = 0; k + 1 < wb.size(); ++k)
      for (int64_t e0 = wb[k]; e0 < wb[k + 1]; e0 += cap)
        out.push_back(tx::WorkItem{db.kind, (int32_t)(view_base + b), e0, std::min(e0 + cap, wb[k + 1])});
  }
}

int eval_persistent(tx_handle h, const tx_eval_args& a) {
  const bool mixed = (a.flags & TX_EVAL_MIXED) != 0;
  const bool stage = a.crs_vals != nullptr && (a.flags & TX_EVAL_SCATTER_DIRECT) == 0;
  if (h->items.empty()) {
    build_items(h, h->items, 0);
    cudaFree(h->d_items);
    if (cudaMalloc((void**)&h->d_items, sizeof(tx::WorkItem) * h->items.size()) != cudaSuccess ||
        cudaMemcpy(h->d_items, h->items.data(), sizeof(tx::WorkItem) * h->items.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess)
      return fail(h, TX_ENOMEM, "tx_eval: work list allocation");
    if (!h->d_counter && cudaMalloc((void**)&h->d_counter, sizeof(int)) != cudaSuccess)
      return fail(h, TX_ENOMEM, "tx_eval: counter allocation");
  }
  const size_t nb = h->blocks.size();
  std::vector<unsigned char> tab(nb * (sizeof(tx::BlockView) + sizeof(tx::EvalParams)));
  size_t smem = 0;
  tx::EvalParams P = make_params(h, a);
  for (size_t b = 0; b < nb; ++b) {
    tx::BlockView V = h->blocks[b].view();
    std::memcpy(&tab[b * sizeof(tx::BlockView)], &V, sizeof V);
    std::memcpy(&tab[nb * sizeof(tx::BlockView) + b * sizeof(tx::EvalParams)], &P, sizeof P);
    smem = std::max(smem, tx::batched_smem_bytes(h->blocks[b].kind, mixed, stage));
  }
  cudaError_t e = h->stage.put(tab.data(), tab.size(), h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval: staging ") + cudaGetErrorString(e));
  const tx::BlockView* dv = (const tx::BlockView*)h->stage.dev;
  const tx::EvalParams* dp = (const tx::EvalParams*)((unsigned char*)h->stage.dev + nb * sizeof(tx::BlockView));
  e = tx::launch_assemble_batched(dv, dp, h->d_items, (int)h->items.size(), h->d_counter, smem, mixed,
                                  a.crs_vals != nullptr, stage, h->grid_cap, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval: ") + cudaGetErrorString(e));
  return TX_OK;
}

// Whether the two-phase form holds this handle's rows: nf^2 x the longest
// entity row in the gather kernel's shared row, nf^2 x an element's basis
// count in its per-entity element-row window.
const char* gather_misfit(const tx::Dofs& D) {
  int64_t maxdeg = 0;
  for (int64_t r = 0; r < D.n_entities; ++r) maxdeg = std::max(maxdeg, D.erowptr[r + 1] - D.erowptr[r]);
  if (maxdeg * D.nf * D.nf > tx::kGatherRowMax) return "tx_eval: an entity row is too long for TX_EVAL_GATHER";
  for (const tx::BlockDofs& B : D.blocks)
    if (D.nf * D.nf * B.nb > tx::kGatherElemRowMax) return "tx_eval: element rows too long for TX_EVAL_GATHER";
  return nullptr;
}

// Whether the handle is one hex8 elasticity block on the whole brick lattice
// (the owner-computes lattice assembly applies).
bool lattice_gather_applies(tx_handle h) {
  const tx::Mesh& m = h->mesh;
  const tx::Dofs& D = h->dofs;
  if (m.is_explicit || m.nblocks != 1 || D.blocks.size() != 1) return false;
  const tx::BlockDofs& B = D.blocks[0];
  return B.topo == TX_TOPO_HEX && B.basis == TX_HGRAD_C1 && B.ref.nq == 8 && D.eq.physics == TX_PHYS_ELASTICITY &&
         D.nf == 3 && D.n_entities == m.n_nodes && (int64_t)B.dconn.size() == 8 * m.NX * m.NY * m.NZ &&
         (int64_t)D.ent_lattice.size() == 3 * D.n_entities;
}

// Per-node records of the lattice assembly (node GID order): FP32 hi/lo
// coordinates, entity LID, first CRS value of the node's rows and the
// position of each lattice neighbour in the node's sorted entity row.
void build_lattice_nodes(tx_handle h) {
  const tx::Mesh& m = h->mesh;
  const tx::Dofs& D = h->dofs;
  const int64_t NX = m.NX, NY = m.NY, NZ = m.NZ, nn = (NX + 1) * (NY + 1) * (NZ + 1);
  std::vector<int32_t> lid_of(nn, -1);
  for (int64_t l = 0; l < D.n_entities; ++l) {
    const int32_t* p = &D.ent_lattice[3 * l];
    if ((p[0] | p[1] | p[2]) & 1) throw std::invalid_argument("lattice assembly: an entity is not a vertex");
    lid_of[p[0] / 2 + (NX + 1) * (p[1] / 2 + (NY + 1) * (int64_t)(p[2] / 2))] = (int32_t)l;
  }
  std::vector<tx::LatticeNode> rec(nn);
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t g = 0; g < nn; ++g) {
    tx::LatticeNode& r = rec[g];
    std::memset(&r, 0, sizeof r);
    std::memset(r.npos, 0xff, sizeof r.npos);
    const int64_t i = g % (NX + 1), j = (g / (NX + 1)) % (NY + 1), k = g / ((NX + 1) * (NY + 1));
    const int32_t l = lid_of[g];
    if (l < 0) { bad = 1; continue; }
    r.lid = l;
    r.rowstart = 9 * D.erowptr[l];
    for (int d = 0; d < 3; ++d) {
      const double X = m.coords[3 * g + d];
      const float hi = (float)X;
      r.xh[d] = hi;
      r.xl[d] = (float)(X - (double)hi);
    }
    const int32_t* row = D.ecol.data() + D.erowptr[l];
    const int64_t len = D.erowptr[l + 1] - D.erowptr[l];
    int64_t found = 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int64_t a = i + dx, b = j + dy, c = k + dz;
          if (a < 0 || a > NX || b < 0 || b > NY || c < 0 || c > NZ) continue;
          const int32_t lm = lid_of[a + (NX + 1) * (b + (NY + 1) * c)];
          const int32_t* pos = std::lower_bound(row, row + len, lm);
          if (pos == row + len || *pos != lm) { bad = 1; continue; }
          r.npos[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)] = (uint8_t)(pos - row);
          ++found;
        }
    if (found != len) bad = 1;
  }
  if (bad) throw std::invalid_argument("lattice assembly: the entity graph is not the lattice's");
  ck(upload(h->d_lat, rec), "upload lattice nodes");
  ck(cudaMalloc((void**)&h->d_lat_u, sizeof(float4) * nn), "alloc lattice u");
  ck(cudaMalloc((void**)&h->d_lat_ud, sizeof(float4) * nn), "alloc lattice u_dot");
}

// Owner-computes mixed R+J of a lattice hex8 elasticity block: f and the CRS
// values overwritten, each once.
int eval_lattice(tx_handle h, const tx_eval_args& a, const tx::EvalParams& P) {
  int rc = guarded(h, [&]() {
    if (!h->d_lat) build_lattice_nodes(h);
    return TX_OK;
  });
  if (rc) return rc;
  const tx::Mesh& m = h->mesh;
  tx::LatticeArgs L;
  L.nx = m.NX; L.ny = m.NY; L.nz = m.NZ;
  L.grid = h->grid_cap;  // the z chunk length is picked by the launcher for its grid
  L.nodes = h->d_lat;
  L.ref = h->blocks[0].ref;
  L.lam = (float)P.lam; L.mu = (float)P.mu; L.rho = (float)P.p[5];
  L.alpha = (float)P.alpha; L.beta = (float)P.beta;
  for (int d = 0; d < 3; ++d) L.body[d] = (float)P.p[2 + d];
  L.f = a.f;
  L.vals = a.crs_vals;
  cudaError_t e = tx::launch_lattice_gather(L, h->d_lat_u, h->d_lat_ud, a.x, a.x_dot, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval: ") + cudaGetErrorString(e));
  return TX_OK;
}

// Evaluate every requested block/range (volume fill).
// Two-phase evaluation (TX_EVAL_GATHER): incidence lists built on first use,
// element scratch grown to the precision's need, then per block the first
// phase and one gather launch over every entity row.
int eval_gather(tx_handle h, const tx_eval_args& a, const tx::EvalParams& P0) {
  const bool mixed = (a.flags & TX_EVAL_MIXED) != 0;
  if (!a.crs_vals) return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_GATHER needs crs_vals");
  if (a.block >= 0) return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_GATHER evaluates every block (block = -1)");
  if (a.flags & (TX_EVAL_TANGENT | TX_EVAL_PERSISTENT | TX_EVAL_DETERMINISTIC))
    return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_GATHER is not combined with TANGENT, PERSISTENT or DETERMINISTIC");
  if (mixed && lattice_gather_applies(h)) return eval_lattice(h, a, P0);
  const tx::Dofs& D = h->dofs;
  const int nf = D.nf;
  if (const char* why = gather_misfit(D)) return fail(h, TX_EINVAL, why);
  int rc = guarded(h, [&]() {
    if (!h->d_inc_ptr) {
      const int64_t ne = D.n_entities;
      std::vector<int64_t> ptr(ne + 1, 0);
      for (const tx::BlockDofs& B : D.blocks)
        for (int32_t ent : B.dconn) ++ptr[ent + 1];
      for (int64_t i = 0; i < ne; ++i) ptr[i + 1] += ptr[i];
      std::vector<int64_t> inc(ptr[ne]), fill(ptr.begin(), ptr.end() - 1);
      for (size_t b = 0; b < D.blocks.size(); ++b) {
        const tx::BlockDofs& B = D.blocks[b];
        const int64_t E = (int64_t)B.dconn.size() / B.nb;
        for (int64_t e = 0; e < E; ++e)
          for (int k = 0; k < B.nb; ++k)
            inc[fill[B.dconn[e * B.nb + k]]++] = ((int64_t)b << 56) | (e << 8) | k;
      }
      ck(upload(h->d_inc_ptr, ptr), "upload incidence");
      ck(upload(h->d_inc, inc), "upload incidence");
    }
    size_t need = 0;
    for (const DevBlock& db : h->blocks) {
      const size_t E = (size_t)db.n_elem, NE = (size_t)nf * db.nb, w = mixed ? 4 : 8;
      need += ((E * NE * NE * w + 255) & ~size_t(255)) + ((E * NE * w + 255) & ~size_t(255));
    }
    if (need > h->gather_bytes) {
      cudaFree(h->gather_scratch);
      h->gather_scratch = nullptr;
      h->gather_bytes = 0;
      ck(cudaMalloc((void**)&h->gather_scratch, need), "alloc two-phase scratch");
      h->gather_bytes = need;
    }
    return TX_OK;
  });
  if (rc) return rc;
  tx::GatherBlocks G{};
  size_t off = 0;
  cudaError_t e = cudaSuccess;
  for (size_t b = 0; b < h->blocks.size() && e == cudaSuccess; ++b) {
    const DevBlock& db = h->blocks[b];
    const size_t E = (size_t)db.n_elem, NE = (size_t)nf * db.nb, w = mixed ? 4 : 8;
    tx::EvalParams P = P0;
    P.kscr = h->gather_scratch + off;
    off += (E * NE * NE * w + 255) & ~size_t(255);
    P.rscr = h->gather_scratch + off;
    off += (E * NE * w + 255) & ~size_t(255);
    G.b[b] = tx::GatherBlock{P.kscr, P.rscr, db.epos, db.nb};
    e = tx::launch_assemble(db.view(), P, mixed, nullptr, 0, db.n_elem, true, true, h->stream, h->grid_cap);
  }
  if (e == cudaSuccess)
    e = tx::launch_gather_rows(D.n_entities, nf, h->d_inc_ptr, h->d_inc, G, mixed, h->d_erowptr, h->d_rowptr,
                               a.crs_vals, a.f, h->stream);
  if (e == cudaErrorInvalidValue) return fail(h, TX_EINVAL, "tx_eval: no kernel for this element family / cubature");
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval: ") + cudaGetErrorString(e));
  return TX_OK;
}

int eval_blocks(tx_handle h, const tx_eval_args& a, const CoefOverride* ov = nullptr) {
  tx::EvalParams P = make_params(h, a, ov);
  if (a.flags & TX_EVAL_GATHER) return eval_gather(h, a, P);
  const bool mixed = (a.flags & TX_EVAL_MIXED) != 0;
  const bool det = (a.flags & TX_EVAL_DETERMINISTIC) != 0;
  const bool stage = (a.flags & TX_EVAL_SCATTER_DIRECT) == 0;
  if (a.flags & TX_EVAL_TANGENT) {
    if (!a.tangent || !a.dfdp || a.n_tangent < 1 || a.n_tangent > TX_MAX_TANGENTS)
      return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_TANGENT needs tangent, dfdp and 1 <= n_tangent <= 4");
    if (a.flags & (TX_EVAL_PERSISTENT | TX_EVAL_MIXED))
      return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_TANGENT is an FP64 per-block evaluation");
  }
  if ((a.flags & TX_EVAL_PERSISTENT) && !det) {
    if (a.block >= 0) return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_PERSISTENT evaluates every block (block = -1)");
    for (const auto& db : h->blocks)
      if (db.kind < 0) return fail(h, TX_EINVAL, "tx_eval: no kernel for this element family / cubature");
    return eval_persistent(h, a);
  }
  const int b0 = a.block < 0 ? 0 : a.block;
  const int b1 = a.block < 0 ? (int)h->blocks.size() : a.block + 1;
  for (int b = b0; b < b1; ++b) {
    const DevBlock& db = h->blocks[b];
    tx::BlockView V = db.view();
    int64_t e0 = 0, e1 = db.n_elem;
    if (a.block >= 0) {
      e0 = a.elem_begin;
      e1 = a.elem_end < 0 ? db.n_elem : a.elem_end;
      if (e0 < 0 || e1 > db.n_elem || e0 > e1) return fail(h, TX_ERANGE, "tx_eval: element range outside the block");
    }
    cudaError_t e = cudaSuccess;
    const bool tiled = !det && stage && P.vals && !P.tan && h->cta_threads != 0 &&
                       tx::tile_shape_supported(db.kind, h->cta_threads);
    const bool tens = !det && !tiled && mixed && stage && P.vals && h->variant == 3 && h->cta_threads == 0 &&
                      tx::tc_supported(V, P);
    const bool wpe = !det && !tiled && !tens && mixed && stage && h->variant != 1 && h->cta_threads == 0 &&
                     tx::wpe_supported(V, P);
    if (tens && !h->d_wait_status) {
      if (cudaMalloc((void**)&h->d_wait_status, sizeof(int)) != cudaSuccess ||
          cudaMemset(h->d_wait_status, 0, sizeof(int)) != cudaSuccess)
        return fail(h, TX_ECUDA, "tx_eval: status word of the tensor-core kernel");
    }
    if (tens) {
      e = tx::launch_assemble_tc(V, P, e0, e1, h->d_wait_status, h->stream, h->grid_cap);
    } else if (tiled) {
      e = tx::launch_assemble_tile(V, P, mixed, h->cta_threads, e0, e1, h->stream, h->grid_cap);
    } else if (wpe) {
      e = tx::launch_assemble_wpe(V, P, e0, e1, h->stream, h->grid_cap);
    } else if (!det) {
      e = tx::launch_assemble(V, P, mixed, nullptr, e0, e1, true, stage, h->stream, h->grid_cap);
    } else {
      if (e0 != 0 || e1 != db.n_elem)
        return fail(h, TX_EINVAL, "tx_eval: TX_EVAL_DETERMINISTIC evaluates whole blocks");
      // one launch per colour, plain read-modify-write: fixed summation order
      for (size_t c = 0; c + 1 < db.color_offsets.size() && e == cudaSuccess; ++c)
        e = tx::launch_assemble(V, P, mixed, db.color_perm, db.color_offsets[c], db.color_offsets[c + 1], false,
                                stage, h->stream, h->grid_cap);
    }
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
  const double* x_pred;      // implicit integration: x_dot = coef * (x - x_pred)
  double coef;
  double* xdot_work;
  int32_t n_neumann;
  const int32_t* neumann_ids;
  const tx::EntityGraph* eg;  // matrix-based residual in the entity-block form (or null)
};

int neumann_eval(tx_handle h, int32_t id, double t, double* f);

int outer_residual(void* vctx, const double* x, double* r) {
  MfCtx* c = (MfCtx*)vctx;
  tx_handle h = c->h;
  const int64_t n = h->dofs.n_dofs;
  if (c->matrix_free) {
    // r = -f(x): FP64 Residual evaluation + Dirichlet residual x_d - g_d
    if (cudaMemsetAsync(r, 0, sizeof(double) * n, h->stream) != cudaSuccess) return TX_ECUDA;
    const double* xdot = c->x_dot;
    if (c->x_pred) {
      if (tx::launch_scaled_diff(c->xdot_work, x, c->x_pred, c->coef, n, h->stream) != cudaSuccess) return TX_ECUDA;
      xdot = c->xdot_work;
    }
    tx_eval_args a{};
    a.x = x; a.x_dot = xdot; a.alpha = c->alpha; a.beta = c->beta; a.t = c->t;
    a.f = r; a.crs_vals = nullptr; a.block = -1; a.elem_end = -1; a.flags = 0;
    int rc = eval_blocks(h, a);
    if (rc) return rc;
    for (int32_t k = 0; k < c->n_neumann; ++k)
      if ((rc = neumann_eval(h, c->neumann_ids[k], c->t, r)) != TX_OK) return rc;
    if (tx::launch_dirichlet(c->n_dir, c->dir, c->g, x, r, nullptr, nullptr, nullptr, h->dofs.nf, nullptr,
                             h->stream) != cudaSuccess)
      return TX_ECUDA;
    if (tx::launch_axpby(r, r, 0.0, -1.0, n, h->stream) != cudaSuccess) return TX_ECUDA;
    return TX_OK;
  }
  if (cudaMemcpyAsync(r, c->b, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess) return TX_ECUDA;
  const cudaError_t e =
      c->eg ? tx::launch_spmv_entity_f64(*c->eg, c->vals, x, r, -1.0, 1.0, h->stream, h->spmv_eb)
            : tx::launch_spmv_f64(n, c->rowptr, c->colind, c->vals, x, r, -1.0, 1.0, h->dofs.nnz, h->stream, h->spmv);
  if (e != cudaSuccess) return TX_ECUDA;
  return TX_OK;
}

// Neumann sets

// WorksetFunctor values (disc-fe/src/evaluators/TianXin_WorksetFunctor_impl.hpp).
int neumann_value(const tx_neumann_desc& d, const double* tt, const double* tv, double t, double* out,
                  std::string& err) {
  switch (d.value_type) {
    case TX_VALUE_CONSTANT:
      *out = d.value;
      return TX_OK;
    case TX_VALUE_LINEAR: {
      // the elapse time is the "Value" entry itself, as LinearWorksetFunctor reads it
      const double elapse = d.value;
      if (t >= elapse) *out = d.value;
      else if (t <= 0.0) *out = 0.0;
      else *out = d.value * t / elapse;
      return TX_OK;
    }
    case TX_VALUE_TIME_TABLE: {
      if (d.n_table < 1 || !tt || !tv) { err = "TIME_TABLE needs n_table >= 1 and both tables"; return TX_EINVAL; }
      if (t > tt[d.n_table - 1]) { err = "time is past the last TIME_TABLE time"; return TX_ERANGE; }
      int i = 0;
      while (tt[i] < t) ++i;
      if (i == 0) *out = tv[0];
      else *out = tv[i - 1] + (tv[i] - tv[i - 1]) / (tt[i] - tt[i - 1]) * (t - tt[i - 1]);
      return TX_OK;
    }
    default:
      err = "unknown value_type";
      return TX_EINVAL;
  }
}

int neumann_eval(tx_handle h, int32_t id, double t, double* f) {
  if (id < 0 || id >= (int32_t)h->neumann.size()) return fail(h, TX_ERANGE, "tx_neumann_eval: unknown set");
  const NeumannSet& ns = h->neumann[id];
  double val = 0.0;
  std::string err;
  int rc = neumann_value(ns.desc, ns.table_t.data(), ns.table_v.data(), t, &val, err);
  if (rc) return fail(h, rc, "tx_neumann_eval: " + err);
  cudaError_t e = tx::launch_neumann(h->blocks[ns.desc.block].view(), h->d_coords, ns.sides, ns.n_sides, ns.tables,
                                     ns.stride, ns.nqf, h->dofs.nf, ns.desc.field, val, f, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_neumann_eval: ") + cudaGetErrorString(e));
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
  if (rc) {  // no handle: the message stays with the calling thread (tx_last_error(NULL))
    create_error() = h->err;
    return rc;
  }
  *out = h.release();
  return TX_OK;
}

}  // extern "C"

namespace {
void copy_err(char* err, int32_t len, const std::string& msg) {
  if (!err || len <= 0) return;
  const size_t n = std::min<size_t>(msg.size(), (size_t)len - 1);
  std::memcpy(err, msg.data(), n);
  err[n] = 0;
}

// Builds a handle around an explicit mesh made by make(); failures go to err.
template <typename F>
int create_explicit(tx_handle* out, char* err, int32_t err_len, F make) {
  if (!out) return TX_EINVAL;
  *out = nullptr;
  copy_err(err, err_len, "");
  std::unique_ptr<tx_handle_s> h(new (std::nothrow) tx_handle_s);
  if (!h) return TX_ENOMEM;
  try {
    tx::build_mesh_explicit(h->mesh, make());
  } catch (const std::invalid_argument& e) {
    copy_err(err, err_len, e.what());
    return TX_EINVAL;
  } catch (const std::exception& e) {
    copy_err(err, err_len, e.what());
    return TX_EINVAL;
  }
  *out = h.release();
  return TX_OK;
}
}  // namespace

extern "C" {

int tx_mesh_create_explicit(const tx_mesh_explicit_desc* d, tx_handle* out, char* err, int32_t err_len) {
  if (!d || !out) return TX_EINVAL;
  return create_explicit(out, err, err_len, [&]() {
    tx::ExplicitMesh M;
    if (d->n_nodes < 1 || !d->coords) throw std::invalid_argument("explicit mesh: nodes and coordinates");
    if (d->n_blocks < 1 || !d->blocks) throw std::invalid_argument("explicit mesh: element blocks");
    M.n_nodes = d->n_nodes;
    M.coords.assign(d->coords, d->coords + 3 * d->n_nodes);
    for (int32_t b = 0; b < d->n_blocks; ++b) {
      const tx_explicit_block& B = d->blocks[b];
      tx::ExplicitBlock E;
      E.topology = B.topology; E.n_elem = B.n_elem; E.id = B.id;
      E.name = B.name ? B.name : "block_" + std::to_string(B.id);
      E.npe = B.nodes_per_elem > 0 ? B.nodes_per_elem : (B.topology == TX_TOPO_TET ? 4 : 8);
      if (E.npe != 4 && E.npe != 8 && E.npe != 10 && E.npe != 27)
        throw std::invalid_argument("explicit mesh: nodes per element");
      if (B.n_elem < 0 || (B.n_elem > 0 && !B.conn)) throw std::invalid_argument("explicit mesh: connectivity");
      if (B.n_elem > 0) E.conn.assign(B.conn, B.conn + B.n_elem * E.npe);
      M.blocks.push_back(std::move(E));
    }
    auto sets = [](int32_t n, const tx_explicit_set* in, int per, std::vector<tx::ExplicitSet>& dst) {
      if (n > 0 && !in) throw std::invalid_argument("explicit mesh: sets");
      for (int32_t k = 0; k < n; ++k) {
        tx::ExplicitSet S;
        S.id = in[k].id;
        S.name = in[k].name ? in[k].name : std::to_string(in[k].id);
        if (in[k].n < 0 || (in[k].n > 0 && !in[k].entries)) throw std::invalid_argument("explicit mesh: set entries");
        if (in[k].n > 0) S.entries.assign(in[k].entries, in[k].entries + in[k].n * per);
        dst.push_back(std::move(S));
      }
    };
    sets(d->n_side_sets, d->side_sets, 2, M.side_sets);
    sets(d->n_node_sets, d->node_sets, 1, M.node_sets);
    return M;
  });
}

int tx_mesh_create_exodus(const char* path, int32_t linear, tx_handle* out, char* err, int32_t err_len) {
  if (!path || !out) return TX_EINVAL;
  return create_explicit(out, err, err_len, [&]() { return tx::read_exodus(path, linear != 0); });
}

int tx_exodus_inspect(const char* path, tx_exodus_summary* s, char* err, int32_t err_len) {
  if (!path || !s) return TX_EINVAL;
  copy_err(err, err_len, "");
  try {
    const tx::ExodusSummary x = tx::exodus_summary(path);
    s->version = x.version; s->dim = x.dim; s->n_nodes = x.n_nodes; s->n_elem = x.n_elem;
    s->n_blocks = x.n_blocks; s->n_side_sets = x.n_side_sets; s->n_node_sets = x.n_node_sets;
  } catch (const std::exception& e) {
    copy_err(err, err_len, e.what());
    return TX_EINVAL;
  }
  return TX_OK;
}

int tx_mesh_set_info(tx_handle h, int32_t kind, int32_t k, int64_t* id, char* name, int32_t name_len, int64_t* n) {
  if (!h || kind < 0 || kind > 2) return TX_EINVAL;
  if (!h->mesh.is_explicit) return fail(h, TX_ESTATE, "tx_mesh_set_info: lattice meshes have no sets");
  const tx::ExplicitMesh& M = h->mesh.ex;
  const int64_t count = kind == 0 ? (int64_t)M.blocks.size() : kind == 1 ? (int64_t)M.side_sets.size()
                                                                         : (int64_t)M.node_sets.size();
  if (k < 0) {
    if (n) *n = count;
    return TX_OK;
  }
  if (k >= count) return fail(h, TX_ERANGE, "tx_mesh_set_info: set out of range");
  const std::string* nm;
  if (kind == 0) {
    if (id) *id = M.blocks[k].id;
    if (n) *n = M.blocks[k].n_elem;
    nm = &M.blocks[k].name;
  } else {
    const tx::ExplicitSet& S = kind == 1 ? M.side_sets[k] : M.node_sets[k];
    if (id) *id = S.id;
    if (n) *n = (int64_t)S.entries.size() / (kind == 1 ? 2 : 1);
    nm = &S.name;
  }
  copy_err(name, name_len, *nm);
  return TX_OK;
}

int tx_mesh_set_entries(tx_handle h, int32_t kind, int32_t k, int64_t* entries) {
  if (!h || !entries || kind < 0 || kind > 2) return TX_EINVAL;
  if (!h->mesh.is_explicit) return fail(h, TX_ESTATE, "tx_mesh_set_entries: lattice meshes have no sets");
  const tx::ExplicitMesh& M = h->mesh.ex;
  if (kind == 0) {
    if (k < 0 || k >= (int32_t)M.blocks.size()) return fail(h, TX_ERANGE, "tx_mesh_set_entries: block out of range");
    const int64_t first = h->mesh.block_first[k];
    for (int64_t i = 0; i < M.blocks[k].n_elem; ++i) entries[i] = first + i;
    return TX_OK;
  }
  const std::vector<tx::ExplicitSet>& sets = kind == 1 ? M.side_sets : M.node_sets;
  if (k < 0 || k >= (int32_t)sets.size()) return fail(h, TX_ERANGE, "tx_mesh_set_entries: set out of range");
  std::copy(sets[k].entries.begin(), sets[k].entries.end(), entries);
  return TX_OK;
}

void tx_destroy(tx_handle h) { delete h; }

const char* tx_last_error(tx_handle h) {
  if (h) return h->err.c_str();
  return create_error().empty() ? "null handle" : create_error().c_str();
}

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

int tx_mesh_element_vertices(tx_handle h, int32_t block, int32_t* nv, int64_t* vertices) {
  if (!h || !nv) return TX_EINVAL;
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "block out of range");
  *nv = h->mesh.desc.block_topology[block] == TX_TOPO_HEX ? 8 : 4;
  if (vertices) tx::element_vertices(h->mesh, block, vertices);
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
      db.kind = tx::assemble_kind(db.topo, db.basis, db.nq, D.eq.physics);
      db.color_offsets = B.color_offsets;
      h->blocks.push_back(db);
      DevBlock& d = h->blocks.back();
      ck(upload(d.vconn, B.vconn), "upload vconn");
      ck(upload(d.dconn, B.dconn), "upload dconn");
      ck(upload(d.epos, B.epos), "upload epos");
      ck(upload(d.esign, B.esign), "upload esign");
      const std::vector<double> ref = B.ref.packed();
      ck(upload(d.ref, ref), "upload reference tables");
      ck(upload(d.ref32, std::vector<float>(ref.begin(), ref.end())), "upload FP32 reference tables");
      ck(upload(d.color_perm, B.color_perm), "upload colouring");
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

int tx_dirichlet_dofs_node_set(tx_handle h, int32_t node_set, uint32_t field_mask, int64_t* n, int32_t* lids) {
  if (!h || !n) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "before tx_dof_build");
  if (!h->mesh.is_explicit) return fail(h, TX_EINVAL, "tx_dirichlet_dofs_node_set: lattice meshes use side masks");
  if (node_set < 0 || node_set >= (int32_t)h->mesh.ex.node_sets.size())
    return fail(h, TX_ERANGE, "tx_dirichlet_dofs_node_set: node set out of range");
  return guarded(h, [&]() {
    std::vector<int32_t> v = tx::node_set_dofs(h->dofs, h->mesh, node_set, field_mask);
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

int tx_eval_gather_form(tx_handle h, int32_t* form) {
  if (!h || !form) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "tx_eval_gather_form before tx_dof_build");
  *form = lattice_gather_applies(h) ? TX_GATHER_LATTICE : gather_misfit(h->dofs) ? 0 : TX_GATHER_TWO_PHASE;
  return TX_OK;
}

int tx_eval_gather_supported(tx_handle h, int32_t* supported) {
  if (!h || !supported) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "tx_eval_gather_supported before tx_dof_build");
  *supported = gather_misfit(h->dofs) ? 0 : 1;
  return TX_OK;
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

// The handle's entity graph when the caller declares (TX_SPMV_ENTITY_BLOCKS,
// TX_SOLVE_ENTITY_BLOCKS) that its CRS is the one tx_graph_build wrote, the
// DOFs carry kEntityNf fields each and the rows number n_dofs; else null (the
// CRS form serves, e.g. for nf = 1, where both forms read the same bytes).
const tx::EntityGraph* entity_graph(tx_handle h, int64_t n_rows, tx::EntityGraph& eg) {
  if (!h->have_dofs || h->dofs.nf != tx::kEntityNf || n_rows != h->dofs.n_dofs || !h->d_erowptr) return nullptr;
  eg = tx::EntityGraph{h->d_erowptr, h->d_ecol, h->dofs.n_entities};
  return &eg;
}

int tx_spmv(tx_handle h, int32_t precision, int64_t n_rows, const int64_t* rowptr, const int32_t* colind,
            const void* vals, const void* x, void* y, double alpha, double beta) {
  if (!h || !rowptr || !colind || !vals || !x || !y) return TX_EINVAL;
  if (n_rows < 0) return fail(h, TX_EINVAL, "tx_spmv: negative row count");
  const int64_t hint = (h->have_dofs && n_rows == h->dofs.n_dofs) ? h->dofs.nnz : 0;
  const bool entity = (precision & TX_SPMV_ENTITY_BLOCKS) != 0;
  precision &= ~TX_SPMV_ENTITY_BLOCKS;
  if (entity && (!h->have_dofs || n_rows != h->dofs.n_dofs))
    return fail(h, TX_EINVAL, "tx_spmv: TX_SPMV_ENTITY_BLOCKS needs the handle's graph (n_rows = its DOF count)");
  tx::EntityGraph egs;
  const tx::EntityGraph* eg = entity ? entity_graph(h, n_rows, egs) : nullptr;
  cudaError_t e;
  if (eg && precision == TX_SPMV_F64)
    e = tx::launch_spmv_entity_f64(*eg, (const double*)vals, (const double*)x, (double*)y, alpha, beta, h->stream,
                                   h->spmv_eb);
  else if (eg && precision == TX_SPMV_F32)
    e = tx::launch_spmv_entity_f32(*eg, (const float*)vals, (const float*)x, (float*)y, (float)alpha, (float)beta,
                                   h->stream, h->spmv_eb);
  else if (precision == TX_SPMV_F64)
    e = tx::launch_spmv_f64(n_rows, rowptr, colind, (const double*)vals, (const double*)x, (double*)y, alpha, beta,
                            hint, h->stream, h->spmv);
  else if (precision == TX_SPMV_F32)
    e = tx::launch_spmv_f32(n_rows, rowptr, colind, (const float*)vals, (const float*)x, (float*)y, (float)alpha,
                            (float)beta, hint, h->stream, h->spmv);
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
  tx::EntityGraph egs;
  const tx::EntityGraph* eg = (a->flags & TX_SOLVE_ENTITY_BLOCKS) ? entity_graph(h, n, egs) : nullptr;
  MfCtx ctx{h, a->x_dot, a->alpha, a->beta, a->t, a->n_dirichlet, a->dirichlet_lids, a->dirichlet_g,
            a->b, a->rowptr, a->colind, a->vals, mf, a->x_pred, a->x_dot_coef, h->solver.xdw,
            a->n_neumann, a->neumann_ids, eg};
  if (a->x_pred && !mf) return fail(h, TX_EINVAL, "tx_solve_cg_ir: x_pred needs MATRIX_FREE_RESIDUAL");
  if (a->n_neumann < 0 || (a->n_neumann > 0 && !a->neumann_ids))
    return fail(h, TX_EINVAL, "tx_solve_cg_ir: neumann ids");
  for (int32_t k = 0; k < a->n_neumann; ++k)
    if (a->neumann_ids[k] < 0 || a->neumann_ids[k] >= (int32_t)h->neumann.size())
      return fail(h, TX_ERANGE, "tx_solve_cg_ir: unknown Neumann set");
  std::string err;
  h->solver.spmv = h->spmv;
  h->solver.spmv_eb = h->spmv_eb;
  int rc = tx::solve_cg_ir(h->solver, a->rowptr, a->colind, a->vals, a->n_dirichlet, a->dirichlet_lids, a->x,
                           outer_residual, &ctx, a->rtol > 0 ? a->rtol : 1e-10,
                           a->inner_rtol > 0 ? a->inner_rtol : 1e-5, a->max_outer > 0 ? a->max_outer : 50,
                           a->max_inner > 0 ? a->max_inner : 100000, a->stats, h->stream, err,
                           (a->flags & TX_SOLVE_FIXED_ITERATIONS) != 0, (a->flags & TX_SOLVE_REUSE_OPERATOR) != 0,
                           a->stats_device, eg, (a->flags & TX_SOLVE_BLOCK_JACOBI) != 0);
  if (rc == TX_ETIMEDOUT) return fail(h, rc, "tx_solve_cg_ir: did not reach rtol within max_outer iterations");
  if (rc) return fail(h, rc, err);
  return TX_OK;
}


int tx_neumann_value(const tx_neumann_desc* d, double t, double* value) {
  if (!d || !value) return TX_EINVAL;
  std::string err;
  return neumann_value(*d, d->table_t, d->table_v, t, value, err);
}

int tx_neumann_create(tx_handle h, const tx_neumann_desc* d, int32_t* id, int64_t* n_sides) {
  if (!h || !d || !id) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_neumann_create before tx_dof_build");
  if (d->block < 0 || d->block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "tx_neumann_create: block out of range");
  if (d->field < 0 || d->field >= h->dofs.nf) return fail(h, TX_ERANGE, "tx_neumann_create: field out of range");
  if (h->mesh.is_explicit) {
    if (d->side_set < 1 || d->side_set > (int32_t)h->mesh.ex.side_sets.size())
      return fail(h, TX_EINVAL, "tx_neumann_create: explicit meshes name a side set (side_set = index + 1)");
  } else if (d->side_set != 0) {
    return fail(h, TX_EINVAL, "tx_neumann_create: lattice meshes use side_mask (side_set = 0)");
  } else if (d->side_mask == 0 || (d->side_mask & ~0x3fu)) {
    return fail(h, TX_EINVAL, "tx_neumann_create: side_mask");
  }
  if (h->blocks[d->block].basis == TX_HCURL_I1)
    return fail(h, TX_EINVAL, "tx_neumann_create: the flux integrates a scalar (HGRAD) basis");
  double v0;
  std::string verr;
  int rc = neumann_value(*d, d->table_t, d->table_v, d->value_type == TX_VALUE_TIME_TABLE && d->table_t ?
                         d->table_t[0] : 0.0, &v0, verr);
  if (rc) return fail(h, rc, "tx_neumann_create: " + verr);
  if (d->value_type == TX_VALUE_TIME_TABLE)
    for (int32_t i = 1; i < d->n_table; ++i)
      if (!(d->table_t[i] > d->table_t[i - 1]))
        return fail(h, TX_EINVAL, "tx_neumann_create: TIME_TABLE times must increase");
  return guarded(h, [&]() {
    NeumannSet ns;
    ns.desc = *d;
    if (d->value_type == TX_VALUE_TIME_TABLE) {
      ns.table_t.assign(d->table_t, d->table_t + d->n_table);
      ns.table_v.assign(d->table_v, d->table_v + d->n_table);
    }
    ns.desc.table_t = nullptr;
    ns.desc.table_v = nullptr;
    const tx::BlockDofs& B = h->dofs.blocks[d->block];
    std::vector<int64_t> sides = d->side_set > 0 ? tx::side_set_workset(h->mesh, d->block, d->side_set - 1)
                                                 : tx::side_workset(h->mesh, d->block, d->side_mask);
    tx::SideTables S = tx::make_side_tables(B.topo, B.basis, B.degree);
    ns.n_sides = (int64_t)sides.size();
    ns.stride = S.stride;
    ns.nqf = S.nqf;
    try {
      ck(upload(ns.sides, sides), "upload side workset");
      ck(upload(ns.tables, S.packed), "upload side tables");
    } catch (...) {
      cudaFree(ns.sides); cudaFree(ns.tables);
      throw;
    }
    h->neumann.push_back(ns);
    *id = (int32_t)h->neumann.size() - 1;
    if (n_sides) *n_sides = ns.n_sides;
    return TX_OK;
  });
}

int tx_neumann_eval(tx_handle h, int32_t id, double t, double* f) {
  if (!h || !f) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_neumann_eval before tx_dof_build");
  return neumann_eval(h, id, t, f);
}

int tx_set_worksets(tx_handle h, int64_t min_size, int64_t max_size, uint64_t seed) {
  if (!h) return TX_EINVAL;
  if (min_size < 1 || max_size < min_size) return fail(h, TX_EINVAL, "tx_set_worksets: need 1 <= min <= max");
  h->ws_min = min_size; h->ws_max = max_size; h->ws_seed = seed;
  h->items.clear();  // rebuilt at the next persistent evaluation
  return TX_OK;
}

int tx_eval_dfdp(tx_handle h, const tx_eval_args* args, int32_t param, double* dfdp) {
  if (!h || !args || !dfdp) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_eval_dfdp before tx_dof_build");
  if (!args->x) return fail(h, TX_EINVAL, "tx_eval_dfdp: x is required");
  if (args->block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "tx_eval_dfdp: block out of range");
  CoefOverride ov;
  if (param < 0 || !derivative_coefficients(h->dofs.eq, param, ov))
    return fail(h, TX_ERANGE, "tx_eval_dfdp: the equation set has no parameter with this index");
  tx_eval_args a = *args;
  a.f = dfdp;
  a.crs_vals = nullptr;
  a.flags &= TX_EVAL_DETERMINISTIC | TX_EVAL_SCATTER_DIRECT;  // FP64 residual type, per block
  return eval_blocks(h, a, &ov);
}

int tx_response_create(tx_handle h, const tx_response_desc* d, int32_t* id) {
  if (!h || !d || !id) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_response_create before tx_dof_build");
  if (d->block < -1 || d->block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "tx_response_create: block");
  if (d->field < 0 || d->field >= h->dofs.nf) return fail(h, TX_ERANGE, "tx_response_create: field");
  if (d->integrand < TX_INTEGRAND_FIELD || d->integrand > TX_INTEGRAND_PROBE)
    return fail(h, TX_EINVAL, "tx_response_create: integrand");
  const bool side = d->side_mask != 0 || d->side_set != 0;
  if (side) {
    if (d->integrand != TX_INTEGRAND_FIELD)
      return fail(h, TX_EINVAL, "tx_response_create: side responses integrate the field (TX_INTEGRAND_FIELD)");
    if (h->mesh.is_explicit ? (d->side_set < 1 || d->side_set > (int32_t)h->mesh.ex.side_sets.size())
                            : (d->side_set != 0 || (d->side_mask & ~0x3fu)))
      return fail(h, TX_EINVAL, "tx_response_create: side_mask (lattice meshes) or side_set (explicit meshes)");
  }
  const bool extreme = d->integrand == TX_INTEGRAND_MAX || d->integrand == TX_INTEGRAND_MIN;
  return guarded(h, [&]() {
    ResponseSet rs;
    rs.desc = *d;
    rs.side = side;
    auto release = [&]() {
      for (double* t : rs.tables) cudaFree(t);
      for (int64_t* sd : rs.sides) cudaFree(sd);
      cudaFree(rs.partial); cudaFree(rs.pidx); cudaFree(rs.winner);
      cudaFree(rs.probe_lids); cudaFree(rs.probe_n);
    };
    try {
      if (d->integrand == TX_INTEGRAND_PROBE) {
        int b = -1;
        int64_t i = -1;
        double xi[3];
        if (!tx::locate_point(h->mesh, h->dofs, d->point, b, i, xi))
          throw std::out_of_range("tx_response_create: no cell holds the probe point");
        const tx::BlockDofs& B = h->dofs.blocks[b];
        if (B.basis == TX_HCURL_I1) throw std::invalid_argument("tx_response_create: HGRAD blocks only");
        const tx::RefTables R = tx::tables_at(B.topo, B.basis, xi, 1);
        std::vector<int32_t> lids(B.nb);
        std::vector<double> n(B.nb);
        for (int k = 0; k < B.nb; ++k) {
          lids[k] = h->dofs.nf * B.dconn[i * B.nb + k] + d->field;
          n[k] = R.val[k];
        }
        ck(upload(rs.probe_lids, lids), "upload probe DOFs");
        ck(upload(rs.probe_n, n), "upload probe basis values");
        rs.probe_nb = B.nb;
      } else {
        for (int b = 0; b < h->mesh.nblocks; ++b) {
          if (d->block >= 0 && b != d->block) continue;
          const tx::BlockDofs& B = h->dofs.blocks[b];
          if (B.basis == TX_HCURL_I1) throw std::invalid_argument("tx_response_create: HGRAD blocks only");
          double* t = nullptr;
          if (side) {
            std::vector<int64_t> sd = d->side_set > 0 ? tx::side_set_workset(h->mesh, b, d->side_set - 1)
                                                      : tx::side_workset(h->mesh, b, d->side_mask);
            const tx::SideTables S = tx::make_side_tables(B.topo, B.basis, B.degree);
            if (S.nqf > 32) throw std::invalid_argument("tx_response_create: at most 32 side points");
            int64_t* dsd = nullptr;
            ck(upload(dsd, sd), "upload side workset");
            rs.sides.push_back(dsd);
            rs.n_sides.push_back((int64_t)sd.size());
            rs.stride.push_back(S.stride);
            rs.nqf.push_back(S.nqf);
            ck(upload(t, S.packed), "upload side tables");
            rs.tables.push_back(t);
            rs.nq.push_back(S.nqf);
            rs.offset.push_back(rs.n_partial);
            rs.n_partial += tx::response_grid((int64_t)sd.size());
          } else {
            const int deg = d->cubature_degree > 0 ? d->cubature_degree : B.degree;
            tx::RefTables R = tx::make_ref_tables(B.topo, B.basis, deg);
            if (R.nq > 64) throw std::invalid_argument("tx_response_create: at most 64 cubature points");
            ck(upload(t, R.packed()), "upload response tables");
            rs.tables.push_back(t);
            rs.nq.push_back(R.nq);
            rs.offset.push_back(rs.n_partial);
            rs.n_partial += tx::response_grid((int64_t)h->mesh.block_elems[b].size());
          }
          rs.blocks.push_back(b);
        }
        const size_t np = (size_t)(rs.n_partial > 0 ? rs.n_partial : 1);
        ck(cudaMalloc((void**)&rs.partial, sizeof(double) * np), "alloc partials");
        ck(cudaMemset(rs.partial, 0, sizeof(double) * np), "zero partials");
        if (extreme) {
          ck(cudaMalloc((void**)&rs.pidx, sizeof(int64_t) * np), "alloc partial keys");
          ck(cudaMemset(rs.pidx, 0xff, sizeof(int64_t) * np), "clear partial keys");
          ck(cudaMalloc((void**)&rs.winner, sizeof(int64_t)), "alloc winner");
        }
      }
    } catch (...) {
      release();
      throw;
    }
    h->responses.push_back(rs);
    *id = (int32_t)h->responses.size() - 1;
    return TX_OK;
  });
}

int tx_response_eval(tx_handle h, int32_t id, const double* x, double* value, double* dvalue_dx) {
  if (!h || !x || !value) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_response_eval before tx_dof_build");
  if (id < 0 || id >= (int32_t)h->responses.size()) return fail(h, TX_ERANGE, "tx_response_eval: unknown response");
  const ResponseSet& rs = h->responses[id];
  const int nf = h->dofs.nf, field = rs.desc.field, kind = rs.desc.integrand;
  cudaError_t e = cudaSuccess;
  if (kind == TX_INTEGRAND_PROBE) {
    e = tx::launch_response_probe(rs.probe_lids, rs.probe_n, rs.probe_nb, x, value, dvalue_dx, h->stream);
  } else if (kind == TX_INTEGRAND_MAX || kind == TX_INTEGRAND_MIN) {
    const bool use_max = kind == TX_INTEGRAND_MAX;
    for (size_t k = 0; k < rs.blocks.size() && e == cudaSuccess; ++k) {
      tx::BlockView v = h->blocks[rs.blocks[k]].view();
      v.ref = rs.tables[k];
      e = tx::launch_response_extreme(v, rs.nq[k], x, nf, field, use_max, (int)k, rs.partial + rs.offset[k],
                                      rs.pidx + rs.offset[k], h->stream);
    }
    if (e == cudaSuccess)
      e = tx::launch_response_extreme_final(rs.partial, rs.pidx, rs.n_partial, use_max, value, rs.winner, h->stream);
    for (size_t k = 0; dvalue_dx && k < rs.blocks.size() && e == cudaSuccess; ++k) {
      tx::BlockView v = h->blocks[rs.blocks[k]].view();
      v.ref = rs.tables[k];
      e = tx::launch_response_extreme_grad(v, rs.nq[k], (int)k, rs.winner, nf, field, dvalue_dx, h->stream);
    }
  } else {
    for (size_t k = 0; k < rs.blocks.size() && e == cudaSuccess; ++k) {
      tx::BlockView v = h->blocks[rs.blocks[k]].view();
      v.ref = rs.tables[k];
      e = rs.side ? tx::launch_response_side(v, h->d_coords, rs.sides[k], rs.n_sides[k], rs.tables[k], rs.stride[k],
                                             rs.nqf[k], x, nf, field, rs.partial + rs.offset[k], dvalue_dx, h->stream)
                  : tx::launch_response(v, rs.nq[k], h->d_coords, x, nf, field, kind, rs.partial + rs.offset[k],
                                        dvalue_dx, h->stream);
    }
    if (e == cudaSuccess) e = tx::launch_response_sum(rs.partial, rs.n_partial, value, h->stream);
  }
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_response_eval: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_ip_coordinates(tx_handle h, int32_t block, int32_t cubature_degree, int32_t* nq, double* xyz) {
  if (!h || !nq) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_ip_coordinates before tx_dof_build");
  if (block < 0 || block >= h->mesh.nblocks) return fail(h, TX_ERANGE, "tx_ip_coordinates: block");
  return guarded(h, [&]() {
    const tx::BlockDofs& B = h->dofs.blocks[block];
    const int deg = cubature_degree > 0 ? cubature_degree : B.degree;
    tx_handle_s::IpTables* t = nullptr;
    for (auto& c : h->ip_tables)
      if (c.block == block && c.degree == deg) t = &c;
    if (!t) {
      const tx::RefTables R = tx::make_ref_tables(B.topo, TX_HGRAD_C1, deg);
      tx_handle_s::IpTables c{block, deg, R.nq, nullptr};
      ck(upload(c.tables, R.packed()), "upload cubature tables");
      h->ip_tables.push_back(c);
      t = &h->ip_tables.back();
    }
    *nq = t->nq;
    if (xyz) {
      tx::BlockView v = h->blocks[block].view();
      v.ref = t->tables;
      ck(tx::launch_ip_coordinates(v, t->nq, h->d_coords, xyz, h->stream), "ip coordinates");
    }
    return TX_OK;
  });
}

int tx_graph_capture_begin(tx_handle h) {
  if (!h) return TX_EINVAL;
  if (h->capturing) return fail(h, TX_ESTATE, "tx_graph_capture_begin: a capture is open");
  if (!h->stream) return fail(h, TX_EINVAL, "tx_graph_capture_begin: set a non-default stream first");
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_graph_capture_begin: ") + cudaGetErrorString(e));
  h->capturing = true;
  return TX_OK;
}

int tx_graph_capture_end(tx_handle h, int32_t* graph_id) {
  if (!h || !graph_id) return TX_EINVAL;
  if (!h->capturing) return fail(h, TX_ESTATE, "tx_graph_capture_end: no capture is open");
  h->capturing = false;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(h, TX_ECUDA, std::string("tx_graph_capture_end: ") + cudaGetErrorString(e));
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_graph_capture_end: ") + cudaGetErrorString(e));
  h->graphs.push_back(x);
  *graph_id = (int32_t)h->graphs.size() - 1;
  return TX_OK;
}

int tx_graph_launch(tx_handle h, int32_t graph_id) {
  if (!h) return TX_EINVAL;
  if (graph_id < 0 || graph_id >= (int32_t)h->graphs.size() || !h->graphs[graph_id])
    return fail(h, TX_ERANGE, "tx_graph_launch: unknown graph");
  cudaError_t e = cudaGraphLaunch(h->graphs[graph_id], h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_graph_launch: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_graph_destroy(tx_handle h, int32_t graph_id) {
  if (!h) return TX_EINVAL;
  if (graph_id < 0 || graph_id >= (int32_t)h->graphs.size() || !h->graphs[graph_id])
    return fail(h, TX_ERANGE, "tx_graph_destroy: unknown graph");
  cudaGraphExecDestroy(h->graphs[graph_id]);
  h->graphs[graph_id] = nullptr;
  return TX_OK;
}

int tx_set_cta_threads(tx_handle h, int32_t threads) {
  if (!h) return TX_EINVAL;
  if (threads == 128) threads = 0;
  if (threads != 0 && threads != 64 && threads != 256)
    return fail(h, TX_EINVAL, "tx_set_cta_threads: 0 (or 128), 64 or 256");
  if (threads != 0) {
    bool any = false;
    for (const DevBlock& db : h->blocks) any = any || tx::tile_shape_supported(db.kind, threads);
    if (!any) return fail(h, TX_EINVAL, "tx_set_cta_threads: no block of this handle has that tile shape");
  }
  h->cta_threads = threads;
  return TX_OK;
}

int tx_set_assembly_variant(tx_handle h, int32_t variant) {
  if (!h) return TX_EINVAL;
  if (variant < 0 || variant > 3) return fail(h, TX_EINVAL, "tx_set_assembly_variant: 0, 1, 2 or 3");
  h->variant = variant;
  return TX_OK;
}

int tx_set_spmv_shape(tx_handle h, int32_t lanes, int32_t unroll) {
  if (!h) return TX_EINVAL;
  const tx::SpmvShape sh{lanes, unroll};
  if (!tx::spmv_shape_valid(sh))
    return fail(h, TX_EINVAL, "tx_set_spmv_shape: lanes 4/8/16/32 and unroll 1/2/4, or both 0");
  h->spmv = sh;
  return TX_OK;
}

// ---------------------------------------------------------------- blocked layout

int tx_blocked_layout(tx_handle h, int32_t n_blocks, const int32_t* field_block) {
  if (!h || !field_block) return TX_EINVAL;
  if (!h->have_host_dofs) return fail(h, TX_ESTATE, "tx_blocked_layout before tx_dof_build");
  const int nf = h->dofs.nf;
  if (n_blocks < 1 || n_blocks > nf || nf > tx::kMaxFieldBlocks)
    return fail(h, TX_EINVAL, "tx_blocked_layout: 1 <= n_blocks <= number of fields");
  tx::BlockedMap M;
  M.nf = nf;
  M.nb = n_blocks;
  for (int f = 0; f < nf; ++f) {
    const int b = field_block[f];
    if (b < 0 || b >= n_blocks) return fail(h, TX_EINVAL, "tx_blocked_layout: field block out of range");
    M.fblock[f] = b;
    M.fpos[f] = M.bnf[b]++;
  }
  for (int b = 0; b < n_blocks; ++b)
    if (M.bnf[b] == 0) return fail(h, TX_EINVAL, "tx_blocked_layout: empty field block");
  h->blocked = M;
  return TX_OK;
}

int tx_blocked_sizes(tx_handle h, int32_t i, int32_t j, int64_t* n_rows, int64_t* n_cols, int64_t* nnz) {
  if (!h) return TX_EINVAL;
  const tx::BlockedMap& M = h->blocked;
  if (M.nb == 0) return fail(h, TX_ESTATE, "tx_blocked_sizes before tx_blocked_layout");
  if (i < 0 || i >= M.nb || j < 0 || j >= M.nb) return fail(h, TX_ERANGE, "tx_blocked_sizes: block out of range");
  const int64_t ne = h->dofs.n_entities;
  if (n_rows) *n_rows = (int64_t)M.bnf[i] * ne;
  if (n_cols) *n_cols = (int64_t)M.bnf[j] * ne;
  if (nnz) *nnz = (int64_t)M.bnf[i] * M.bnf[j] * h->dofs.erowptr[ne];
  return TX_OK;
}

}  // extern "C"

namespace {
// The device graph of blocks with bi x bj fields, built on first use.
int block_graph(tx_handle h, int bi, int bj, tx_handle_s::BlockGraph*& out) {
  tx_handle_s::BlockGraph& g = h->block_graphs[bi][bj];
  if (!g.rp) {
    const int64_t ne = h->dofs.n_entities, nnz = (int64_t)bi * bj * h->dofs.erowptr[ne];
    if (cudaMalloc((void**)&g.rp, sizeof(int64_t) * (bi * ne + 1)) != cudaSuccess ||
        cudaMalloc((void**)&g.col, sizeof(int32_t) * (nnz > 0 ? nnz : 1)) != cudaSuccess) {
      cudaFree(g.rp); cudaFree(g.col); g = tx_handle_s::BlockGraph();
      return fail(h, TX_ENOMEM, "blocked graph: out of device memory");
    }
    if (tx::launch_block_graph(h->d_erowptr, h->d_ecol, ne, bi, bj, g.rp, g.col, h->stream) != cudaSuccess)
      return fail(h, TX_ECUDA, "blocked graph: launch failed");
  }
  out = &g;
  return TX_OK;
}

int blocked_ready(tx_handle h, const char* who) {
  if (!h->have_dofs) return fail(h, TX_ESTATE, std::string(who) + " before tx_dof_build");
  if (h->blocked.nb == 0) return fail(h, TX_ESTATE, std::string(who) + " before tx_blocked_layout");
  return TX_OK;
}
}  // namespace

extern "C" {

int tx_blocked_graph_build(tx_handle h, int32_t i, int32_t j, int64_t* rowptr, int32_t* colind) {
  if (!h || !rowptr || !colind) return TX_EINVAL;
  int rc = blocked_ready(h, "tx_blocked_graph_build");
  if (rc) return rc;
  const tx::BlockedMap& M = h->blocked;
  if (i < 0 || i >= M.nb || j < 0 || j >= M.nb) return fail(h, TX_ERANGE, "tx_blocked_graph_build: block out of range");
  tx_handle_s::BlockGraph* g = nullptr;
  if ((rc = block_graph(h, M.bnf[i], M.bnf[j], g))) return rc;
  const int64_t ne = h->dofs.n_entities, nnz = (int64_t)M.bnf[i] * M.bnf[j] * h->dofs.erowptr[ne];
  cudaError_t e = cudaMemcpyAsync(rowptr, g->rp, sizeof(int64_t) * (M.bnf[i] * ne + 1), cudaMemcpyDeviceToDevice,
                                  h->stream);
  if (e == cudaSuccess && nnz > 0)
    e = cudaMemcpyAsync(colind, g->col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_blocked_graph_build: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_blocked_split_vector(tx_handle h, const double* x, double* const* xb) {
  if (!h || !x || !xb) return TX_EINVAL;
  int rc = blocked_ready(h, "tx_blocked_split_vector");
  if (rc) return rc;
  tx::BlockPtrs P{};
  for (int k = 0; k < h->blocked.nb; ++k) {
    if (!xb[k]) return fail(h, TX_EINVAL, "tx_blocked_split_vector: null block vector");
    P.p[k] = xb[k];
  }
  if (tx::launch_block_vector(h->dofs.n_entities, h->blocked, x, P, nullptr, true, h->stream) != cudaSuccess)
    return fail(h, TX_ECUDA, "tx_blocked_split_vector: launch failed");
  return TX_OK;
}

int tx_blocked_merge_vector(tx_handle h, const double* const* xb, double* x) {
  if (!h || !x || !xb) return TX_EINVAL;
  int rc = blocked_ready(h, "tx_blocked_merge_vector");
  if (rc) return rc;
  tx::BlockPtrs P{};
  for (int k = 0; k < h->blocked.nb; ++k) {
    if (!xb[k]) return fail(h, TX_EINVAL, "tx_blocked_merge_vector: null block vector");
    P.p[k] = const_cast<double*>(xb[k]);
  }
  if (tx::launch_block_vector(h->dofs.n_entities, h->blocked, nullptr, P, x, false, h->stream) != cudaSuccess)
    return fail(h, TX_ECUDA, "tx_blocked_merge_vector: launch failed");
  return TX_OK;
}

int tx_blocked_split_matrix(tx_handle h, const double* crs_vals, double* const* blk_vals) {
  if (!h || !crs_vals || !blk_vals) return TX_EINVAL;
  int rc = blocked_ready(h, "tx_blocked_split_matrix");
  if (rc) return rc;
  tx::BlockPtrs P{};
  const int nb = h->blocked.nb;
  for (int k = 0; k < nb * nb; ++k) P.p[k] = blk_vals[k];
  if (tx::launch_block_split_matrix(h->d_erowptr, h->dofs.n_entities, h->blocked, crs_vals, P, h->stream) !=
      cudaSuccess)
    return fail(h, TX_ECUDA, "tx_blocked_split_matrix: launch failed");
  return TX_OK;
}

int tx_blocked_spmv(tx_handle h, const double* const* blk_vals, const double* const* xb, double* const* yb,
                    double alpha, double beta) {
  if (!h || !blk_vals || !xb || !yb) return TX_EINVAL;
  int rc = blocked_ready(h, "tx_blocked_spmv");
  if (rc) return rc;
  const tx::BlockedMap& M = h->blocked;
  const int64_t ne = h->dofs.n_entities;
  for (int i = 0; i < M.nb; ++i) {
    if (!yb[i] || !xb[i]) return fail(h, TX_EINVAL, "tx_blocked_spmv: null block vector");
    const int64_t rows = (int64_t)M.bnf[i] * ne;
    bool first = true;
    for (int j = 0; j < M.nb; ++j) {
      const double* v = blk_vals[i * M.nb + j];
      if (!v) continue;  // excluded pair
      tx_handle_s::BlockGraph* g = nullptr;
      if ((rc = block_graph(h, M.bnf[i], M.bnf[j], g))) return rc;
      const int64_t nnz = (int64_t)M.bnf[i] * M.bnf[j] * h->dofs.erowptr[ne];
      if (tx::launch_spmv_f64(rows, g->rp, g->col, v, xb[j], yb[i], alpha, first ? beta : 1.0, nnz, h->stream,
                              h->spmv) != cudaSuccess)
        return fail(h, TX_ECUDA, "tx_blocked_spmv: launch failed");
      first = false;
    }
    if (first) {  // a block row with every pair excluded: y_i = beta y_i
      cudaError_t e = beta == 0.0 ? tx::launch_fill(yb[i], 0.0, rows, h->stream)
                                  : tx::launch_axpby(yb[i], yb[i], 0.0, beta, rows, h->stream);
      if (e != cudaSuccess) return fail(h, TX_ECUDA, "tx_blocked_spmv: launch failed");
    }
  }
  return TX_OK;
}

int tx_set_spmv_entity_shape(tx_handle h, int32_t lanes, int32_t unroll) {
  if (!h) return TX_EINVAL;
  const tx::SpmvShape sh{lanes, unroll};
  if (!tx::entity_shape_valid(sh))
    return fail(h, TX_EINVAL, "tx_set_spmv_entity_shape: lanes 3 (unroll 1-3), 4/8 (1/2/4), 16/32 (1/2), or both 0");
  h->spmv_eb = sh;
  return TX_OK;
}

int tx_set_grid_cap(tx_handle h, int32_t max_ctas) {
  if (!h || max_ctas < 0) return TX_EINVAL;
  h->grid_cap = max_ctas;
  return TX_OK;
}

int tx_set_stream(tx_handle h, void* stream) {
  if (!h) return TX_EINVAL;
  h->stream = (cudaStream_t)stream;
  return TX_OK;
}

int tx_selftest_wait_timeout(tx_handle h) {
  if (!h) return TX_EINVAL;
  if (!h->d_wait_status) {
    if (cudaMalloc((void**)&h->d_wait_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(h->d_wait_status, 0, sizeof(int)) != cudaSuccess)
      return fail(h, TX_ECUDA, "tx_selftest_wait_timeout: status word");
  }
  cudaError_t e = tx::launch_wait_selftest(h->d_wait_status, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_selftest_wait_timeout: ") + cudaGetErrorString(e));
  return TX_OK;
}

int tx_synchronize(tx_handle h) {
  if (!h) return TX_EINVAL;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_synchronize: ") + cudaGetErrorString(e));
  if (h->d_wait_status) {
    int st = 0;
    e = cudaMemcpy(&st, h->d_wait_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_synchronize: ") + cudaGetErrorString(e));
    if (st) {
      cudaMemset(h->d_wait_status, 0, sizeof(int));
      return fail(h, TX_ETIMEDOUT, "tx_synchronize: a tensor-core MMA wait gave up; the results of that evaluation are incomplete");
    }
  }
  return TX_OK;
}

// ---------------------------------------------------------------- batches
struct tx_batch_s {
  std::vector<tx_handle> hs;
  std::vector<tx::WorkItem> items;
  tx::WorkItem* d_items = nullptr;
  int* d_counter = nullptr;
  Staging stage;
  int64_t ws_min = 512, ws_max = 512;
  uint64_t seed = 0;
  int grid_cap = 0;
  std::string err;
  ~tx_batch_s() {
    cudaFree(d_items);
    cudaFree(d_counter);
    stage.release();
  }
};

int tx_batch_create(const tx_handle* handles, int32_t n, tx_batch* out) {
  if (!handles || n < 1 || !out) return TX_EINVAL;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!handles[i] || !handles[i]->have_dofs) return TX_ESTATE;
  tx_batch b = new (std::nothrow) tx_batch_s;
  if (!b) return TX_ENOMEM;
  b->hs.assign(handles, handles + n);
  *out = b;
  return TX_OK;
}

void tx_batch_destroy(tx_batch b) { delete b; }

const char* tx_batch_last_error(tx_batch b) { return b ? b->err.c_str() : "null batch"; }

int tx_batch_set_worksets(tx_batch b, int64_t min_size, int64_t max_size, uint64_t seed, int32_t max_ctas) {
  if (!b || min_size < 1 || max_size < min_size || max_ctas < 0) return TX_EINVAL;
  b->ws_min = min_size; b->ws_max = max_size; b->seed = seed; b->grid_cap = max_ctas;
  b->items.clear();
  return TX_OK;
}

int tx_batch_eval(tx_batch b, const tx_eval_args* args) {
  if (!b || !args) return TX_EINVAL;
  const int n = (int)b->hs.size();
  const bool mixed = (args[0].flags & TX_EVAL_MIXED) != 0;
  const bool jac = args[0].crs_vals != nullptr;
  const bool stage = jac && (args[0].flags & TX_EVAL_SCATTER_DIRECT) == 0;
  for (int i = 0; i < n; ++i) {
    if (!args[i].x) { b->err = "tx_batch_eval: x is required for every instance"; return TX_EINVAL; }
    if (((args[i].flags & TX_EVAL_MIXED) != 0) != mixed || (args[i].crs_vals != nullptr) != jac) {
      b->err = "tx_batch_eval: every instance needs the same precision and evaluation type";
      return TX_EINVAL;
    }
    for (const auto& db : b->hs[i]->blocks)
      if (db.kind < 0) { b->err = "tx_batch_eval: no kernel for an element family of the batch"; return TX_EINVAL; }
  }
  cudaStream_t s = b->hs[0]->stream;
  if (b->items.empty()) {
    int base = 0;
    for (int i = 0; i < n; ++i) {
      tx_handle h = b->hs[i];
      int64_t mn = h->ws_min, mx = h->ws_max;
      uint64_t sd = h->ws_seed;
      h->ws_min = b->ws_min; h->ws_max = b->ws_max; h->ws_seed = b->seed + 104729ull * i;
      build_items(h, b->items, base);
      h->ws_min = mn; h->ws_max = mx; h->ws_seed = sd;
      base += (int)h->blocks.size();
    }
    cudaFree(b->d_items);
    if (cudaMalloc((void**)&b->d_items, sizeof(tx::WorkItem) * b->items.size()) != cudaSuccess ||
        cudaMemcpy(b->d_items, b->items.data(), sizeof(tx::WorkItem) * b->items.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      b->err = "tx_batch_eval: work list allocation";
      return TX_ENOMEM;
    }
    if (!b->d_counter && cudaMalloc((void**)&b->d_counter, sizeof(int)) != cudaSuccess) {
      b->err = "tx_batch_eval: counter allocation";
      return TX_ENOMEM;
    }
  }
  size_t nviews = 0;
  for (int i = 0; i < n; ++i) nviews += b->hs[i]->blocks.size();
  std::vector<unsigned char> tab(nviews * (sizeof(tx::BlockView) + sizeof(tx::EvalParams)));
  size_t smem = 0, v = 0;
  for (int i = 0; i < n; ++i) {
    tx_handle h = b->hs[i];
    tx::EvalParams P = make_params(h, args[i]);
    for (const auto& db : h->blocks) {
      tx::BlockView V = db.view();
      std::memcpy(&tab[v * sizeof(tx::BlockView)], &V, sizeof V);
      std::memcpy(&tab[nviews * sizeof(tx::BlockView) + v * sizeof(tx::EvalParams)], &P, sizeof P);
      smem = std::max(smem, tx::batched_smem_bytes(db.kind, mixed, stage));
      ++v;
    }
  }
  cudaError_t e = b->stage.put(tab.data(), tab.size(), s);
  if (e == cudaSuccess) {
    const tx::BlockView* dv = (const tx::BlockView*)b->stage.dev;
    const tx::EvalParams* dp = (const tx::EvalParams*)((unsigned char*)b->stage.dev + nviews * sizeof(tx::BlockView));
    e = tx::launch_assemble_batched(dv, dp, b->d_items, (int)b->items.size(), b->d_counter, smem, mixed, jac,
                                    stage, b->grid_cap, s);
  }
  if (e != cudaSuccess) {
    b->err = std::string("tx_batch_eval: ") + cudaGetErrorString(e);
    return TX_ECUDA;
  }
  return TX_OK;
}

}  // extern "C"
// ---------------------------------------------------------------- no-alloc
// Volume fill for callers that cannot allocate device memory.
//
// tx_eval's persistent form keeps its scratch -- the work counter, the
// per-block parameter tables and the work list -- in device memory that the
// handle allocates on first use.  Some callers cannot accept that:
// applications that reserve all device memory up front in their own pool (a
// solver embedded in a larger simulation with a fixed memory budget, where a
// driver allocation outside the pool fails or pushes a neighbour out of
// memory), and time-step loops that must not stall the device, which a
// cudaFree of grown scratch does.  tx_eval_noalloc runs the same kernel with
// that scratch in one file-scope static device array of fixed size, so a call
// allocates nothing.
namespace {

constexpr int64_t kNoAllocMaxItems = TX_NOALLOC_MAX_WORKSETS;
constexpr size_t al256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kNaCounter = 0;
constexpr size_t kNaViews = 256;
constexpr size_t kNaParams = al256(kNaViews + sizeof(tx::BlockView) * TX_MAX_BLOCKS);
constexpr size_t kNaItems = al256(kNaParams + sizeof(tx::EvalParams) * TX_MAX_BLOCKS);
constexpr size_t kNaBytes = kNaItems + sizeof(tx::WorkItem) * kNoAllocMaxItems;

// The scratch: [counter | views | params | work items].  Every call shares it
// and it keeps the last call's contents; each call rewrites the tables and
// the work list and clears the counter before the persistent launch.
__device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];
// Device address of g_noalloc_scratch per device ordinal, looked up once per
// device by the first call (the host-side name of a __device__ array is only
// a stand-in, not a device address).  Threads that race on the first call
// look up the same address, so a relaxed atomic suffices.
std::atomic<unsigned char*> g_noalloc_addr[256] = {};

// Everything the persistent launch reads, passed by value so that no host
// buffer is copied: the block views, the evaluation parameters and the work
// list's shape.  Items follow tx_eval's persistent work list: each block's
// even worksets of `ws` elements, each cut into items of at most `cap[b]`
// elements (a few CTA passes of the family).
struct NaTables {
  tx::BlockView views[TX_MAX_BLOCKS];
  tx::EvalParams params;
  int64_t first[TX_MAX_BLOCKS + 1];  // first item of each block
  int64_t n_elem[TX_MAX_BLOCKS];
  int64_t cap[TX_MAX_BLOCKS];        // elements an item
  int64_t per_ws[TX_MAX_BLOCKS];     // items of a full workset
  int32_t kind[TX_MAX_BLOCKS];
  int32_t nblocks;
  int64_t ws;
};

// Writes the parameter tables and the work list into the scratch.  Item j of
// block b lies in workset w = j / per_ws[b], as chunk c = j % per_ws[b]:
// elements [w ws + c cap, min(w ws + (c + 1) cap, (w + 1) ws, n_elem)).
__global__ void k_noalloc_setup(unsigned char* base, int64_t n_items, NaTables t) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid < t.nblocks) {
    ((tx::BlockView*)(base + kNaViews))[tid] = t.views[tid];
    ((tx::EvalParams*)(base + kNaParams))[tid] = t.params;
  }
  tx::WorkItem* items = (tx::WorkItem*)(base + kNaItems);
  for (int64_t i = tid; i < n_items; i += (int64_t)gridDim.x * blockDim.x) {
    int b = 0;
    while (b + 1 < t.nblocks && i >= t.first[b + 1]) ++b;
    const int64_t j = i - t.first[b];
    const int64_t w = j / t.per_ws[b], c = j % t.per_ws[b];
    const int64_t w1 = (w + 1) * t.ws < t.n_elem[b] ? (w + 1) * t.ws : t.n_elem[b];
    const int64_t e0 = w * t.ws + c * t.cap[b];
    const int64_t e1 = e0 + t.cap[b] < w1 ? e0 + t.cap[b] : w1;
    items[i] = tx::WorkItem{t.kind[b], b, e0, e1};
  }
}

}  // namespace

extern "C" int tx_eval_noalloc(tx_handle h, const tx_eval_args* a) {
  if (!h || !a) return TX_EINVAL;
  if (!h->have_dofs) return fail(h, TX_ESTATE, "tx_eval_noalloc before tx_dof_build");
  if (!a->x) return fail(h, TX_EINVAL, "tx_eval_noalloc: x is required");
  if (a->block != -1) return fail(h, TX_EINVAL, "tx_eval_noalloc evaluates every block (block = -1)");
  if (a->flags & TX_EVAL_DETERMINISTIC) return fail(h, TX_EINVAL, "tx_eval_noalloc: no deterministic form");
  if (a->flags & TX_EVAL_TANGENT) return fail(h, TX_EINVAL, "tx_eval_noalloc: no tangent form");
  if (a->flags & TX_EVAL_GATHER) return fail(h, TX_EINVAL, "tx_eval_noalloc: the two-phase form allocates scratch");
  if (h->dofs.eq.physics == TX_PHYS_MAXWELL && !a->aux && a->f)
    return fail(h, TX_EINVAL, "tx_eval_noalloc: MAXWELL needs the current density J in aux");
  const int nb = (int)h->blocks.size();
  const int64_t ws = h->ws_min;
  const bool mixed = (a->flags & TX_EVAL_MIXED) != 0;
  const bool stage = a->crs_vals != nullptr && (a->flags & TX_EVAL_SCATTER_DIRECT) == 0;
  NaTables t{};
  t.nblocks = nb;
  t.ws = ws;
  t.params = make_params(h, *a);
  size_t smem = 0;
  for (int b = 0; b < nb; ++b) {
    const DevBlock& db = h->blocks[b];
    if (db.kind < 0) return fail(h, TX_EINVAL, "tx_eval_noalloc: no kernel for this element family");
    t.views[b] = db.view();
    t.kind[b] = db.kind;
    t.n_elem[b] = db.n_elem;
    t.cap[b] = std::min<int64_t>(ws, (int64_t)tx::batched_elements_per_pass(db.kind) * kItemPasses);
    t.per_ws[b] = (ws + t.cap[b] - 1) / t.cap[b];
    const int64_t rem = db.n_elem % ws;
    t.first[b + 1] = t.first[b] + (db.n_elem / ws) * t.per_ws[b] + (rem + t.cap[b] - 1) / t.cap[b];
    smem = std::max(smem, tx::batched_smem_bytes(db.kind, mixed, stage));
  }
  const int64_t n_items = t.first[nb];
  if (n_items > kNoAllocMaxItems)
    return fail(h, TX_ERANGE,
                "tx_eval_noalloc: " + std::to_string(n_items) + " work items exceed the static limit of " +
                    std::to_string(kNoAllocMaxItems) + "; raise the workset size with tx_set_worksets");
  // set-up, once per device, with that device current
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 256) return fail(h, TX_ECUDA, "tx_eval_noalloc: no current device");
  unsigned char* base = g_noalloc_addr[dev].load(std::memory_order_relaxed);
  if (!base) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval_noalloc: ") + cudaGetErrorString(e));
    base = (unsigned char*)p;
    g_noalloc_addr[dev].store(base, std::memory_order_relaxed);
  }
  if (n_items == 0) return TX_OK;
  const int64_t blocks = std::min<int64_t>((n_items + 255) / 256, 1024);
  k_noalloc_setup<<<(unsigned)blocks, 256, 0, h->stream>>>(base, n_items, t);
  e = cudaGetLastError();
  if (e == cudaSuccess)  // clears the counter, then one persistent launch
    e = tx::launch_assemble_batched((const tx::BlockView*)(base + kNaViews), (const tx::EvalParams*)(base + kNaParams),
                                    (const tx::WorkItem*)(base + kNaItems), (int)n_items, (int*)(base + kNaCounter),
                                    smem, mixed, a->crs_vals != nullptr, stage, h->grid_cap, h->stream);
  if (e != cudaSuccess) return fail(h, TX_ECUDA, std::string("tx_eval_noalloc: ") + cudaGetErrorString(e));
  return TX_OK;
}
