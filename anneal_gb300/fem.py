"""Voxel FEM with the interface of anneal's fem.py (anneal 0.3.0), solved on the GPU.

``Grid``, ``hex8_matrices``, ``FEM`` and ``SolverError`` keep the reference's names,
arguments and return types (fem.py:20-263), so callers written for the reference run
unchanged. What changes underneath: there is no CSR matrix. ``FEM.assemble`` returns a
lightweight operator that holds the element scales on the device, and ``FEM.solve`` runs
the multigrid-preconditioned CG of the CUDA library (libanneal_gb300.so). Solves with
rtol >= 1e-7 run in FP32 with FP64 CG scalars and solution; tighter tolerances run in FP64
(``precision="fp32"`` or ``"fp64"`` forces one). FP32 solves certify their tolerance on
the true residual of the FP64 operator; one that stops improving above its tolerance is
finished by the FP64 solver.
"""
import time

import numpy as np
import torch

from .context import Context, require_cuda, to_dev
from . import _native as N

LOCAL = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])

FP32_RTOL_FLOOR = 1e-7


class SolverError(RuntimeError):
    """Raised where the reference raises it (fem.py:24-25, 138-139, 225-229)."""


SOLVER_MESSAGE = ("The solver did not converge in {maxiter} iterations. Usual causes: the part can move "
                  "or turn freely (add a fixed anchor, or fix more directions on one), or the design has "
                  "pieces held only by near-empty voxels (raise volumeFraction or iterations).")


def elasticity_D(nu):
    """Isotropic D for E = 1, Voigt order xx yy zz xy yz zx, engineering shear (fem.py:36-43)."""
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] = lam + 2 * mu
    D[np.arange(3, 6), np.arange(3, 6)] = mu
    return D


def _strain_matrix(point, h):
    """6x24 strain-displacement matrix of the trilinear brick at a point of [-1, 1]^3."""
    s = 2.0 * LOCAL - 1.0
    xi = np.asarray(point, float)
    # dN_a/dxi_d = s_ad/8 * prod over the other two axes (1 + s_a xi)
    g = np.empty((8, 3))
    for d in range(3):
        o1, o2 = [a for a in range(3) if a != d]
        g[:, d] = s[:, d] * (1 + s[:, o1] * xi[o1]) * (1 + s[:, o2] * xi[o2]) / 8.0
    g /= h / 2.0
    B = np.zeros((6, 24))
    cols = 3 * np.arange(8)
    B[0, cols] = g[:, 0]
    B[1, cols + 1] = g[:, 1]
    B[2, cols + 2] = g[:, 2]
    B[3, cols], B[3, cols + 1] = g[:, 1], g[:, 0]
    B[4, cols + 1], B[4, cols + 2] = g[:, 2], g[:, 1]
    B[5, cols], B[5, cols + 2] = g[:, 2], g[:, 0]
    return B


def hex8_matrices(nu, h=1.0):
    """(Ke, B0, D) for a cube of side h, E = 1: Ke by 2x2x2 Gauss quadrature, B0 at the
    centre (fem.py:71-84)."""
    D = elasticity_D(nu)
    g = 1.0 / np.sqrt(3.0)
    pts = np.array(np.meshgrid([-g, g], [-g, g], [-g, g], indexing="ij")).reshape(3, -1).T
    ke = np.zeros((24, 24))
    for p in pts:
        B = _strain_matrix(p, h)
        ke += B.T @ D @ B * (h / 2.0) ** 3
    return ke, _strain_matrix((0.0, 0.0, 0.0), h), D


class Grid:
    """Regular voxel grid; element (i,j,k) spans origin + h*[i,i+1] x ... (fem.py:87-127).
    Elements and nodes are numbered x fastest."""

    def __init__(self, shape, h, origin):
        self.shape = tuple(int(s) for s in shape)
        self.nx, self.ny, self.nz = self.shape
        self.h = float(h)
        self.origin = np.asarray(origin, dtype=float)
        self.nelem = self.nx * self.ny * self.nz
        self.nnode = (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        self._noff = LOCAL[:, 0] + (self.nx + 1) * (LOCAL[:, 1] + (self.ny + 1) * LOCAL[:, 2])

    def elem_ijk(self, e):
        e = np.asarray(e)
        return e % self.nx, (e // self.nx) % self.ny, e // (self.nx * self.ny)

    def element_nodes(self, e):
        i, j, k = self.elem_ijk(e)
        first = i + (self.nx + 1) * (j + (self.ny + 1) * k)
        return first[:, None] + self._noff[None, :]

    def node_coords(self, n):
        n = np.asarray(n)
        ijk = np.stack([n % (self.nx + 1), (n // (self.nx + 1)) % (self.ny + 1),
                        n // ((self.nx + 1) * (self.ny + 1))], axis=-1)
        return self.origin + self.h * ijk

    def elem_centers(self, e=None):
        e = np.arange(self.nelem) if e is None else e
        return self.origin + self.h * (np.stack(self.elem_ijk(e), axis=-1) + 0.5)

    def to3d(self, flat):
        """Flat element array (x fastest) -> array indexed [i, j, k]."""
        return np.asarray(flat).reshape(self.nz, self.ny, self.nx).transpose(2, 1, 0)

    def to1d(self, arr3):
        return np.asarray(arr3).transpose(2, 1, 0).ravel()


class StiffnessOperator:
    """What ``FEM.assemble`` returns: the element scales on the device, applied matrix-free.
    ``K @ u_red`` works on reduced (free-DOF) vectors like the reference's CSR matrix."""

    def __init__(self, fem, Ee):
        self.fem = fem
        self.Ee = np.asarray(Ee, float)
        full = np.zeros(fem.grid.nelem)
        full[fem.act] = self.Ee
        self.escale = to_dev(full, torch.float32)
        self.shape = (fem.nfree, fem.nfree)

    def __matmul__(self, u_red):
        ctx = self.fem._ctx(fp64=True)
        u = torch.zeros(ctx.ndof, dtype=torch.float64, device="cuda")
        u[self.fem._free_t] = to_dev(u_red, torch.float64)
        y = torch.empty_like(u)
        ctx.apply_K(self.escale, u, y)
        return y[self.fem._free_t].cpu().numpy()

    dot = __matmul__


class FEM:
    """Linear elastic solve on the active voxels of a grid (fem.py:130-263)."""

    def __init__(self, grid, active, fixed_dofs, nu, log=None, precision="auto", multi="batch"):
        require_cuda()
        if precision not in ("auto", "fp32", "fp64"):
            raise ValueError(f"precision must be 'auto', 'fp32' or 'fp64', not {precision!r}")
        if multi not in ("batch", "lanes"):
            raise ValueError(f"multi must be 'batch' or 'lanes', not {multi!r}")
        self.precision = precision
        self.multi = multi
        t0 = time.time()
        self.grid = grid
        self.nu = float(nu)
        self.log = log or (lambda *a: None)
        self.act = np.flatnonzero(active)
        if self.act.size == 0:
            raise SolverError("No active voxels: the design space is empty.")
        self.ke, self.B0, self.D = hex8_matrices(nu, grid.h)
        act = np.zeros(grid.nelem, np.uint8)
        act[self.act] = 1
        fixed = np.zeros(3 * grid.nnode, np.uint8)
        fixed[np.asarray(fixed_dofs, dtype=np.int64)] = 1
        self.active_t = to_dev(act, torch.uint8)
        self.fixed_t = to_dev(fixed, torch.uint8)
        self._ctxs = {}
        ctx = self._ctx(fp64=False)
        self._mask_t = ctx.free_mask().bool()
        self.free = np.flatnonzero(self._mask_t.cpu().numpy())
        self._free_t = torch.as_tensor(self.free, device="cuda")
        self.nfree = self.free.size
        self.nnz = None  # no assembled matrix
        self.amg_builds = 0
        self.cg_iters = []
        self.relres = []
        self.log(f"  system: {self.act.size:,} elements, {self.nfree:,} free dofs, "
                 f"matrix-free on the GPU, built in {time.time() - t0:.1f} s")

    def _ctx(self, fp64, lane=0, nrhs=1):
        """The solver context of a precision; lanes > 0 are extra contexts that solve other
        load cases at the same time, each on its own stream; nrhs > 1 is an FP32 context
        that solves that many cases together."""
        key = ("fp64" if fp64 else "fp32", lane, nrhs)
        if key not in self._ctxs:
            c = Context(self.grid.shape, self.grid.h, self.nu, fp64=fp64, nrhs=nrhs)
            c.set_domain(self.active_t, self.fixed_t)
            self._ctxs[key] = c
        return self._ctxs[key]

    @property
    def edof(self):
        en = self.grid.element_nodes(self.act)
        return (3 * en[:, :, None] + np.arange(3)).reshape(-1, 24)

    def assemble(self, Ee):
        """Ee: stiffness scale per active element (fem.py:198-201)."""
        return StiffnessOperator(self, Ee)

    def reduce_load(self, F_global):
        return np.asarray(F_global)[self.free]

    def expand(self, u_red):
        u = np.zeros(3 * self.grid.nnode)
        u[self.free] = u_red
        return u

    def solve_device(self, escale, F, X, rtol=1e-8, maxiter=2000, rebuild=True):
        """Device-level solve: F, X (nrhs, 3*nnode) float64 CUDA tensors, X holds the
        initial guesses and receives the solutions. Raises SolverError like fem.py:225-229.

        The reference solves its load cases one after the other (fem.py:217-231). Here the
        cases are solved as a batch: a case whose load is a scalar multiple of another's
        (for example the +x / -x pair of a load set) takes that multiple of its solution,
        because the problem is linear; the remaining distinct cases run at the same time.
        With ``multi="batch"`` (the default) an FP32 solve advances all of them in the same
        kernels (one context with a slot per case: the latency-bound coarse levels of the
        V-cycle get that many times the work per launch); with ``multi="lanes"``, and for
        FP64 solves, each case runs in its own context and stream."""
        fp64 = self.fp64_for(rtol)
        nrhs = F.shape[0] if F.dim() == 2 else 1
        if nrhs == 1:
            st, iters, relres = self._ctx(fp64).solve(escale, F, X, rtol, maxiter, rebuild)
            if st == N.ANL_ERR_STAGNATION:  # finish in FP64 from the FP32 iterate
                st, it2, relres = self._ctx(True).solve(escale, F, X, rtol, maxiter, rebuild)
                iters = [iters[0] + it2[0]]
            sts = [st]
        else:
            groups = self._multiple_groups(F, fp64)
            reps = [g[0] for g in groups]
            if not fp64 and self.multi == "batch" and len(reps) > 1:
                res = self._solve_batch(escale, F, X, reps, rtol, maxiter, rebuild)
            else:
                res = self._solve_lanes(escale, F, X, reps, rtol, maxiter, rebuild, fp64)
            iters, relres, sts = [0] * nrhs, [0.0] * nrhs, []
            for (rep, members), (st, it, rr) in zip(groups, res):
                sts.append(st)
                iters[rep], relres[rep] = it, rr
                for m, scale in members:
                    X[m].copy_(X[rep]).mul_(scale)
                    iters[m], relres[m] = it, rr
        if rebuild:
            self.amg_builds += 1
        if any(st != N.ANL_OK for st in sts):
            raise SolverError(SOLVER_MESSAGE.format(maxiter=maxiter))
        worst = max(relres)
        if worst > rtol * (1 + 1e-9):
            # only an FP64 solve at the attainable accuracy of its arithmetic gets here
            self.log(f"  solve stopped at relative residual {worst:.2e} (FP64 floor; asked {rtol:.1e})")
        self.cg_iters.extend(iters)
        self.relres.extend(relres)
        return iters

    def fp64_for(self, rtol):
        """Whether a solve to ``rtol`` runs on the FP64 operator."""
        if self.precision != "auto":
            return self.precision == "fp64"
        return rtol < FP32_RTOL_FLOOR

    def _multiple_groups(self, F, fp64):
        """[(representative, [(case, scale), ...]), ...]: cases whose load is a scalar
        multiple of an earlier case's (collinear to 1e-12 in FP64) join that case."""
        ctx = self._ctx(fp64)
        n = F.shape[0]
        norm2 = [ctx.dot(F[i], F[i]) for i in range(n)]
        groups = []
        for i in range(n):
            placed = False
            for g in groups:
                r = g[0]
                if norm2[r] == 0.0 or norm2[i] == 0.0:
                    continue
                d = ctx.dot(F[r], F[i])
                if d * d >= (1.0 - 1e-12) * norm2[r] * norm2[i]:
                    g[1].append((i, d / norm2[r]))
                    placed = True
                    break
            if not placed:
                groups.append((i, []))
        return groups

    def _solve_batch(self, escale, F, X, reps, rtol, maxiter, rebuild):
        """Solves F[reps] together in one FP32 context with len(reps) slots; a case that
        stagnates above rtol in FP32 is finished in FP64 from its FP32 iterate. Returns
        [(status, iters, relres)]."""
        R = len(reps)
        idx = torch.as_tensor(reps, device=F.device)
        Fb = F.index_select(0, idx).contiguous()
        Xb = X.index_select(0, idx).contiguous()
        ctx = self._ctx(False, nrhs=R)
        st, its, rrs = ctx.solve(escale, Fb, Xb, rtol, maxiter, rebuild)
        out = []
        for k in range(R):
            sk = ctx.solve_status(k) if st != N.ANL_OK else N.ANL_OK
            it, rr = its[k], rrs[k]
            if sk == N.ANL_ERR_STAGNATION:  # finish in FP64 from the FP32 iterate
                sk, it2, r2 = self._ctx(True).solve(escale, Fb[k:k + 1], Xb[k:k + 1], rtol, maxiter, rebuild)
                it, rr = it + it2[0], r2[0]
            out.append((sk, it, rr))
        X.index_copy_(0, idx, Xb)
        return out

    def _solve_lanes(self, escale, F, X, reps, rtol, maxiter, rebuild, fp64):
        """Solves F[reps[k]] in context lane k on stream k, concurrently (host threads; the
        library releases the GIL in every call). Returns [(status, iters, relres)]."""
        import concurrent.futures as cf
        main = torch.cuda.current_stream()
        dev = torch.cuda.current_device()
        ctxs = [self._ctx(fp64, lane=k) for k in range(len(reps))]
        if not hasattr(self, "_streams"):
            self._streams = []
        while len(self._streams) < len(reps):
            self._streams.append(torch.cuda.Stream(device=dev))
        streams = self._streams[:len(reps)]
        for st in streams:
            st.wait_stream(main)

        def work(k):
            torch.cuda.set_device(dev)
            with torch.cuda.stream(streams[k]):
                r = reps[k]
                st, it, rr = ctxs[k].solve(escale, F[r:r + 1], X[r:r + 1], rtol, maxiter, rebuild)
                if st == N.ANL_ERR_STAGNATION:  # finish in FP64 from the FP32 iterate
                    st, it2, rr = self._ctx(True, lane=k).solve(escale, F[r:r + 1], X[r:r + 1], rtol, maxiter,
                                                                rebuild)
                    it = [it[0] + it2[0]]
                return st, it[0], rr[0]
        if len(reps) == 1:
            out = [work(0)]
        else:
            with cf.ThreadPoolExecutor(max_workers=len(reps)) as ex:
                out = list(ex.map(work, range(len(reps))))
        for st in streams:
            main.wait_stream(st)
        return out

    def solve(self, K, F_list, x0_list=None, rebuild=True, rtol=1e-8, maxiter=2000):
        """fem.py:206-232: reduced loads in, reduced displacements out."""
        nd = 3 * self.grid.nnode
        F = torch.zeros((len(F_list), nd), dtype=torch.float64, device="cuda")
        X = torch.zeros_like(F)
        for i, f in enumerate(F_list):
            F[i, self._free_t] = to_dev(f, torch.float64)
            if x0_list is not None and x0_list[i] is not None:
                X[i, self._free_t] = to_dev(x0_list[i], torch.float64)
        self.solve_device(K.escale, F, X, rtol=rtol, maxiter=maxiter, rebuild=rebuild)
        Xh = X[:, self._free_t].cpu().numpy()
        if not np.all(np.isfinite(Xh)):
            raise SolverError(SOLVER_MESSAGE.format(maxiter=maxiter))
        return [Xh[i].copy() for i in range(len(F_list))]

    def element_energy(self, u_full):
        """u_e^T ke u_e per active element (fem.py:239-242)."""
        ctx = self._ctx(fp64=False)
        ce = torch.empty(self.grid.nelem, dtype=torch.float32, device="cuda")
        ctx.element_energy(to_dev(u_full, torch.float64), ce)
        return ce.cpu().numpy().astype(float)[self.act]

    def _stress_device(self, u_full, E_material, want_sig, want_vm):
        ctx = self._ctx(fp64=False)
        u = to_dev(np.asarray(u_full, float), torch.float64)
        ne = self.grid.nelem
        if np.ndim(E_material):
            Ef = np.zeros(ne)
            Ef[self.act] = np.asarray(E_material, float)
            E = to_dev(Ef, torch.float64)
        else:
            E = float(E_material)
        sig = torch.empty((ne, 6), dtype=torch.float64, device="cuda") if want_sig else None
        vm = torch.empty(ne, dtype=torch.float64, device="cuda") if want_vm else None
        ctx.element_stress(u, E, sig, vm)
        return sig, vm

    def stress(self, u_full, E_material):
        """Element-centre stress, Voigt order xx yy zz xy yz zx, shape (n_active, 6)
        (fem.py:244-250), computed on the GPU."""
        sig, _ = self._stress_device(u_full, E_material, True, False)
        return sig.cpu().numpy()[self.act]

    @staticmethod
    def normal_stress(sig, d):
        """Normal stress on planes across direction d, d^T sigma d (fem.py:252-257)."""
        d = np.asarray(d, float)
        d = d / np.linalg.norm(d)
        S = np.asarray(sig)
        T = np.stack([np.stack([S[:, 0], S[:, 3], S[:, 5]], -1), np.stack([S[:, 3], S[:, 1], S[:, 4]], -1),
                      np.stack([S[:, 5], S[:, 4], S[:, 2]], -1)], -2)
        return np.einsum("i,nij,j->n", d, T, d)

    def von_mises(self, u_full, E_material):
        """Element-centre von Mises stress (fem.py:259-263), computed on the GPU."""
        _, vm = self._stress_device(u_full, E_material, False, True)
        return vm.cpu().numpy()[self.act]

    def close(self):
        for c in self._ctxs.values():
            c.close()
        self._ctxs = {}
