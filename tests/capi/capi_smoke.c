/* Plain-C caller of the C-ABI (no torch, no Python): mesh -> numbering ->
 * graph -> evalModel(f, W) with Dirichlet rows -> SpMV -> solve.  Prints one
 * line "capi ok N nnz |f|_1 |W|_1 relres" for the GPU test to compare with
 * the Python path. */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tianxin_gb300.h"

#define CK(call)                                                                       \
  do {                                                                                 \
    int rc_ = (call);                                                                  \
    if (rc_) {                                                                         \
      fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, h ? tx_last_error(h) : ""); \
      return 1;                                                                        \
    }                                                                                  \
  } while (0)

int main(int argc, char** argv) {
  int n = argc > 1 ? atoi(argv[1]) : 6;
  tx_handle h = NULL;
  tx_mesh_desc m;
  memset(&m, 0, sizeof m);
  m.nx = m.ny = m.nz = n;
  m.bx = m.by = m.bz = 1;
  m.block_topology[0] = TX_TOPO_HEX;
  m.lx = m.ly = m.lz = 1.0;
  m.jitter = 0.05;
  m.seed = 2024;
  CK(tx_mesh_create(&m, &h));
  tx_equation_set_desc q;
  memset(&q, 0, sizeof q);
  q.physics = TX_PHYS_ELASTICITY;
  q.block_basis[0] = TX_HGRAD_C1;
  q.params[0] = 1.0; q.params[1] = 0.3; q.params[4] = -1.0;
  CK(tx_dof_build(h, &q));
  int64_t N, nnz;
  int32_t ndm, nf;
  CK(tx_dof_sizes(h, &N, &ndm, &nnz, &nf));

  int64_t *rowptr;
  int32_t *colind, *dlids;
  double *vals, *f, *x, *y;
  if (cudaMalloc((void**)&rowptr, 8 * (N + 1)) || cudaMalloc((void**)&colind, 4 * nnz) ||
      cudaMalloc((void**)&vals, 8 * nnz) || cudaMalloc((void**)&f, 8 * N) || cudaMalloc((void**)&x, 8 * N) ||
      cudaMalloc((void**)&y, 8 * N))
    return 2;
  CK(tx_graph_build(h, rowptr, colind));
  cudaMemset(vals, 0, 8 * nnz);
  cudaMemset(f, 0, 8 * N);
  cudaMemset(x, 0, 8 * N);
  tx_eval_args a;
  memset(&a, 0, sizeof a);
  a.x = x; a.beta = 1.0; a.f = f; a.crs_vals = vals; a.block = -1; a.elem_end = -1;
  a.flags = TX_EVAL_MIXED;
  CK(tx_eval(h, &a));
  int64_t nd;
  CK(tx_dirichlet_dofs(h, 1u << 4, 0x7, &nd, NULL));
  int32_t* hl = (int32_t*)malloc(4 * nd);
  CK(tx_dirichlet_dofs(h, 1u << 4, 0x7, &nd, hl));
  if (cudaMalloc((void**)&dlids, 4 * nd)) return 2;
  cudaMemcpy(dlids, hl, 4 * nd, cudaMemcpyHostToDevice);
  CK(tx_dirichlet_apply(h, nd, dlids, NULL, x, f, vals));
  CK(tx_spmv(h, TX_SPMV_F64, N, rowptr, colind, vals, f, y, 1.0, 0.0));
  CK(tx_synchronize(h));

  double* hf = (double*)malloc(8 * N);
  double* hv = (double*)malloc(8 * nnz);
  cudaMemcpy(hf, f, 8 * N, cudaMemcpyDeviceToHost);
  cudaMemcpy(hv, vals, 8 * nnz, cudaMemcpyDeviceToHost);
  double sf = 0, sv = 0;
  for (int64_t i = 0; i < N; ++i) sf += fabs(hf[i]);
  for (int64_t i = 0; i < nnz; ++i) sv += fabs(hv[i]);

  /* Newton step from x = 0: W dx = -f, FP64 matrix-free refinement */
  tx_solve_args s;
  memset(&s, 0, sizeof s);
  s.rowptr = rowptr; s.colind = colind; s.vals = vals; s.x = x;
  s.n_dirichlet = nd; s.dirichlet_lids = dlids;
  s.rtol = 1e-10; s.inner_rtol = 1e-5; s.max_outer = 30; s.max_inner = 100000;
  s.flags = TX_SOLVE_MATRIX_FREE_RESIDUAL; s.beta = 1.0;
  CK(tx_solve_cg_ir(h, &s));
  printf("capi ok %lld %lld %.17g %.17g %.3e\n", (long long)N, (long long)nnz, sf, sv, s.stats[2]);
  tx_destroy(h);
  return 0;
}
