"""Newmark-beta elastodynamics through evalModel, one CUDA graph per step.

M a + K u = F with the reference's second-time-derivative wiring: the
D2XDT2 fields are gathered from the time-derivative vector with the alpha
seed (disc-fe/src/Panzer_EquationSet_DefaultImpl_impl.hpp:283-305 ->
disc-fe/src/evaluators/Panzer_GatherSolution_Tpetra_impl.hpp:554-556), so
the acceleration is passed in the x_dot slot and

    f(u, a) = K u + rho M a - F,     W = beta dF/du + alpha dF/da = K + alpha rho M.

For a step with a = c (u - u_pred), c = 1/(beta_N dt^2), evalModel with
alpha = c, beta = 1 gives the effective Jacobian K_eff = K + c M.  The step
(predictor, FP64-refined FP32 CG on K_eff, block-Jacobi preconditioned on the
entity-block form, corrector) has no host
synchronisation and is captured once as a CUDA graph, then replayed.

The refinement residual is FP64.  For a linear problem (linear=True, the
default: K, M and F do not depend on u) K_eff and M are assembled once in
FP64 and each step forms b = F + c M u_pred and r = b - K_eff x with FP64
SpMVs; otherwise (linear=False) r = -f(x) is a matrix-free FP64 Residual
evaluation, which also covers nonlinear closures.
"""
import torch


class NewmarkElastodynamics:
    def __init__(self, me, dt, beta=0.25, gamma=0.5, mixed=True, outer=3, inner=24, linear=True, block_jacobi=True):
        self.me, self.dt, self.beta_n, self.gamma_n = me, dt, beta, gamma
        self.mixed, self.outer, self.inner, self.linear = mixed, outer, inner, linear
        self.block_jacobi = block_jacobi  # 3x3 block-Jacobi inner CG on the entity-block form
        self.c = 1.0 / (beta * dt * dt)
        lof = me.lof
        z = lof.getTpetraVector
        self.u, self.v, self.a = z(), z(), z()
        self.u_pred, self.v_pred, self.x, self.f, self.zero = z(), z(), z(), z(), z()
        self.F, self.b, self.Mu = z(), z(), z()
        self.W = me.create_W_op()
        self.M = None
        self.stats = torch.zeros(4, dtype=torch.float64, device="cuda")
        self.graph = None

    def assemble_effective_jacobian(self):
        """K_eff = K + c M (linear problem: once; in FP64 when it also gives the refinement residual)."""
        self.me.evalModel(self.u, x_dot=self.zero, alpha=self.c, beta=1.0, f=self.f, W=self.W,
                          mixed=self.mixed and not self.linear)

    def initialize(self, u0, v0=None):
        """u, v given; a0 from M a0 = F - K u0 (FP64 mass matrix, refined CG)."""
        self.u.copy_(u0)
        if v0 is not None:
            self.v.copy_(v0)
        M = self.me.create_W_op()
        f = self.me.lof.getTpetraVector()
        self.me.evalModel(self.u, x_dot=self.zero, alpha=1.0, beta=0.0, f=f, W=M)  # W = rho M, f = K u - F
        a0 = self.me.lof.getTpetraVector()
        self.me.solve(M, a0, b=-f, rtol=1e-13)
        self.a.copy_(a0)
        self.M = M
        if self.linear:  # F = -f(0) at zero acceleration
            fz = self.me.lof.getTpetraVector()
            self.me.evalModel(self.zero, x_dot=self.zero, alpha=0.0, beta=1.0, f=fz)
            torch.neg(fz, out=self.F)
        self.assemble_effective_jacobian()
        # size the solver work space and build the FP32 operator outside any capture
        self.x.copy_(self.u)
        if self.linear:
            self._rhs(self.u)
            self.me.solve(self.W, self.x, b=self.b, fixed=True, max_outer=1, max_inner=1, stats_device=self.stats, block_jacobi=self.block_jacobi)
        else:
            self.me.solve(self.W, self.x, matrix_free=True, fixed=True, max_outer=1, max_inner=1,
                          stats_device=self.stats, block_jacobi=self.block_jacobi, x_pred=self.u, x_dot_coef=self.c, alpha=self.c, beta=1.0)

    def _rhs(self, u_pred):
        """b = F + c M u_pred (FP64 SpMV)."""
        self.M.apply(u_pred, self.Mu)
        torch.add(self.F, self.Mu, alpha=self.c, out=self.b)

    def _step_body(self):
        dt, b, g = self.dt, self.beta_n, self.gamma_n
        torch.add(self.u, self.v, alpha=dt, out=self.u_pred)
        self.u_pred.add_(self.a, alpha=dt * dt * (0.5 - b))
        torch.add(self.v, self.a, alpha=dt * (1.0 - g), out=self.v_pred)
        self.x.copy_(self.u_pred)
        if self.linear:
            self._rhs(self.u_pred)
            self.me.solve(self.W, self.x, b=self.b, fixed=True, reuse_operator=True, max_outer=self.outer,
                          max_inner=self.inner, stats_device=self.stats, block_jacobi=self.block_jacobi)
        else:
            self.me.solve(self.W, self.x, matrix_free=True, fixed=True, reuse_operator=True, max_outer=self.outer,
                          max_inner=self.inner, stats_device=self.stats, block_jacobi=self.block_jacobi, x_pred=self.u_pred, x_dot_coef=self.c,
                          alpha=self.c, beta=1.0)
        torch.sub(self.x, self.u_pred, out=self.a)
        self.a.mul_(self.c)
        torch.add(self.v_pred, self.a, alpha=g * dt, out=self.v)
        self.u.copy_(self.x)

    def capture(self):
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):  # torch's recommended warm-up on a side stream
            pass
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        saved = [t.clone() for t in (self.u, self.v, self.a)]
        with torch.cuda.graph(g):
            self._step_body()
        for t, sv in zip((self.u, self.v, self.a), saved):  # capture does not execute; restore to be safe
            t.copy_(sv)
        self.graph = g

    def step(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self._step_body()
        return self.stats
