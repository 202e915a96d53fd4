"""Learned warm start for the SIMP solve: a 3D U-Net that predicts the displacement field.

No counterpart in the reference, which starts each CG from the previous iterate's
displacement (optimize.py:122, ``x0_list=U``). Here a network maps (filtered density,
nodal load, support mask) to a normalised displacement shape. The solve then starts from the
energy-optimal combination of the previous iterate and the prediction:

    x0 = a u_prev + b u_net,   [a b] from the 2x2 Galerkin system of K on span{u_prev, u_net}

This minimises the initial energy-norm error over the two directions, so the start is never
worse than the previous iterate in that norm, and a useless prediction gets b ~ 0. The CG
still runs to the same relative residual and alone decides convergence.

Network (the learned-warm-start configuration): 4 levels, base channels doubling per level,
two 3x3x3 convolutions with GELU per level, 2x average pooling down, 2x nearest upsampling
up with skip concatenation, a final 1x1x1 convolution to 3 channels. It runs on the node grid
zero-padded to a multiple of 8. Every layer is a kernel of the CUDA library (``anl_nn_*``:
convolution forward and backward, GELU, pooling, upsampling, masked MSE, Adam). Weights and
activations are FP32 (master weights and optimiser state FP32 as well).
"""
import ctypes
import math
import time

import numpy as np
import torch

from . import _native as N
from .context import require_cuda

F32 = torch.float32


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class UNet:
    """The U-Net's parameters, optimiser state and buffers for one input size."""

    def __init__(self, base=16, levels=4, cin=5, cout=3, seed=0):
        require_cuda()
        self.base, self.levels, self.cin, self.cout = base, levels, cin, cout
        self.ch = [base * 2 ** l for l in range(levels)]
        # (name, cin, cout, k) in a fixed order
        specs = []
        for l in range(levels):
            specs.append((f"e1_{l}", cin if l == 0 else self.ch[l - 1], self.ch[l], 3))
            specs.append((f"e2_{l}", self.ch[l], self.ch[l], 3))
        for l in range(levels - 2, -1, -1):
            specs.append((f"d1_{l}", self.ch[l + 1] + self.ch[l], self.ch[l], 3))
            specs.append((f"d2_{l}", self.ch[l], self.ch[l], 3))
        specs.append(("out", self.ch[0], cout, 1))
        self.specs = specs
        sizes = []
        for _, ci, co, k in specs:
            sizes += [co * ci * k ** 3, co]
        self.nparam = int(sum(sizes))
        self.params = torch.zeros(self.nparam, dtype=F32, device="cuda")
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0
        self.w, self.b, self.gw, self.gb = {}, {}, {}, {}
        off = 0
        g = torch.Generator(device="cpu").manual_seed(seed)
        for name, ci, co, k in specs:
            nw = co * ci * k ** 3
            self.w[name] = self.params[off:off + nw].view(co, ci, k, k, k)
            self.gw[name] = self.grads[off:off + nw].view(co, ci, k, k, k)
            off += nw
            self.b[name] = self.params[off:off + co]
            self.gb[name] = self.grads[off:off + co]
            off += co
            fan_in = ci * k ** 3
            std = math.sqrt(2.0 / fan_in) if name != "out" else math.sqrt(1.0 / fan_in)
            self.w[name].copy_((torch.randn(co, ci, k, k, k, generator=g) * std).to("cuda"))
        maxw = max(co * ci * k ** 3 for _, ci, co, k in specs)
        maxper = max(co * ci * k ** 3 + co for _, ci, co, k in specs)
        self.wt_work = torch.empty(maxw, dtype=F32, device="cuda")
        self.part_floats = 64 * maxper
        self.part_work = torch.empty(self.part_floats, dtype=F32, device="cuda")
        self.red = torch.zeros(2 * 1216 + 4, dtype=torch.float64, device="cuda")
        self.counter = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.loss_out = torch.zeros(2, dtype=torch.float64, device="cuda")
        self._dims = None

    # ---------------------------------------------------------------- buffers

    def _alloc(self, dims):
        if self._dims == dims:
            return
        D, H, W = dims
        self._dims = dims
        L = self.levels
        self.vol = [(D >> l) * (H >> l) * (W >> l) for l in range(L)]
        self.dims = [(D >> l, H >> l, W >> l) for l in range(L)]
        e = lambda c, l: torch.empty(c * self.vol[l], dtype=F32, device="cuda")
        self.act = {}
        for l in range(L):
            c = self.ch[l]
            self.act[f"z1e_{l}"], self.act[f"a1e_{l}"] = e(c, l), e(c, l)
            self.act[f"z2e_{l}"] = e(c, l)
            if l < L - 1:
                # the concatenation buffer of decoder level l: [upsampled (ch[l+1]); skip (ch[l])]
                cat = e(self.ch[l + 1] + c, l)
                self.act[f"cat_{l}"] = cat
                self.act[f"a2e_{l}"] = cat[self.ch[l + 1] * self.vol[l]:]
                self.act[f"pool_{l}"] = e(c, l + 1)
                self.act[f"z1d_{l}"], self.act[f"a1d_{l}"] = e(c, l), e(c, l)
                self.act[f"z2d_{l}"], self.act[f"a2d_{l}"] = e(c, l), e(c, l)
            else:
                self.act[f"a2e_{l}"] = e(c, l)
        self.act["y"] = e(self.cout, 0)
        maxc = max(self.ch[l] * 2 + self.ch[min(l + 1, L - 1)] for l in range(L))
        self.g1 = torch.empty(maxc * self.vol[0], dtype=F32, device="cuda")
        self.g2 = torch.empty_like(self.g1)
        self.g3 = torch.empty_like(self.g1)
        self.dskip = {l: e(self.ch[l], l) for l in range(L - 1)}

    # ---------------------------------------------------------------- layers

    def _conv(self, name, x, z, a, dims, act=True):
        ci, co, k = self._spec(name)
        D, H, W = dims
        N.call("anl_nn_conv3d", _p(x), _p(self.w[name]), _p(self.b[name]), _p(z), _p(a) if act else None, ci, co,
               D, H, W, k, 1 if act else 0, 0, _stream())

    def _conv_back(self, name, x, dz, dx, dims, need_dx=True):
        ci, co, k = self._spec(name)
        D, H, W = dims
        N.call("anl_nn_conv3d_bwd_weight", _p(x), _p(dz), _p(self.part_work), self.part_floats, _p(self.gw[name]),
               _p(self.gb[name]), ci, co, D, H, W, k, 0, _stream())
        if need_dx:
            N.call("anl_nn_conv3d_bwd_data", _p(dz), _p(self.w[name]), _p(self.wt_work), _p(dx), ci, co, D, H, W, k,
                   0, _stream())

    def _spec(self, name):
        for n, ci, co, k in self.specs:
            if n == name:
                return ci, co, k
        raise KeyError(name)

    def _gelu_back(self, z, da, dz):
        N.call("anl_nn_gelu_bwd", _p(z), _p(da), _p(dz), z.numel(), _stream())

    # ---------------------------------------------------------------- passes

    def forward(self, x, dims):
        """x: (cin * D*H*W,) FP32 CUDA tensor on the padded node grid. Returns y (cout * vol)."""
        self._alloc(tuple(dims))
        A, L = self.act, self.levels
        inp = x
        for l in range(L):
            d = self.dims[l]
            self._conv(f"e1_{l}", inp, A[f"z1e_{l}"], A[f"a1e_{l}"], d)
            self._conv(f"e2_{l}", A[f"a1e_{l}"], A[f"z2e_{l}"], A[f"a2e_{l}"], d)
            if l < L - 1:
                N.call("anl_nn_pool2", _p(A[f"a2e_{l}"]), _p(A[f"pool_{l}"]), self.ch[l], *d, 0, 0, _stream())
                inp = A[f"pool_{l}"]
        h = A[f"a2e_{L - 1}"]
        for l in range(L - 2, -1, -1):
            d = self.dims[l]
            N.call("anl_nn_up2", _p(h), _p(A[f"cat_{l}"]), self.ch[l + 1], *d, 0, _stream())
            self._conv(f"d1_{l}", A[f"cat_{l}"], A[f"z1d_{l}"], A[f"a1d_{l}"], d)
            self._conv(f"d2_{l}", A[f"a1d_{l}"], A[f"z2d_{l}"], A[f"a2d_{l}"], d)
            h = A[f"a2d_{l}"]
        self._conv("out", h, A["y"], None, self.dims[0], act=False)
        self._x = x
        return A["y"]

    def backward(self, dy):
        """Gradients of the parameters for dy = dLoss/dy of the last forward (overwrites grads)."""
        A, L = self.act, self.levels
        g1, g2, g3 = self.g1, self.g2, self.g3
        c0 = self.ch[0]
        v = self.vol
        # output 1x1x1 conv
        self._conv_back("out", A["a2d_0"] if L > 1 else A[f"a2e_0"], dy, g1[:c0 * v[0]], self.dims[0])
        dh = g1[:c0 * v[0]]
        for l in range(L - 1):
            d, c = self.dims[l], self.ch[l]
            dz2 = g2[:c * v[l]]
            self._gelu_back(A[f"z2d_{l}"], dh, dz2)
            da1 = g3[:c * v[l]]
            self._conv_back(f"d2_{l}", A[f"a1d_{l}"], dz2, da1, d)
            dz1 = g2[:c * v[l]]
            self._gelu_back(A[f"z1d_{l}"], da1, dz1)
            cu = self.ch[l + 1]
            dcat = g3[:(cu + c) * v[l]]
            self._conv_back(f"d1_{l}", A[f"cat_{l}"], dz1, dcat, d)
            self.dskip[l].copy_(dcat[cu * v[l]:])
            dnext = g1[:cu * v[l + 1]]
            N.call("anl_nn_up2", _p(dcat[:cu * v[l]]), _p(dnext), cu, *d, 1, _stream())
            dh = dnext
        # encoder, bottleneck first; dh is the gradient of the bottleneck output
        da2 = dh
        for l in range(L - 1, -1, -1):
            d, c = self.dims[l], self.ch[l]
            if l < L - 1:
                # skip gradient plus the pooling path's gradient
                da2 = g1[:c * v[l]]
                da2.copy_(self.dskip[l])
                N.call("anl_nn_pool2", _p(dpool), _p(da2), c, *d, 1, 1, _stream())
            dz2 = g2[:c * v[l]]
            self._gelu_back(A[f"z2e_{l}"], da2, dz2)
            da1 = g3[:c * v[l]]
            self._conv_back(f"e2_{l}", A[f"a1e_{l}"], dz2, da1, d)
            dz1 = g2[:c * v[l]]
            self._gelu_back(A[f"z1e_{l}"], da1, dz1)
            inp = self._x if l == 0 else A[f"pool_{l - 1}"]
            if l > 0:
                dpool_new = g3[:self.ch[l - 1] * v[l]]
                self._conv_back(f"e1_{l}", inp, dz1, dpool_new, d)
                # keep it away from the buffers the next level overwrites
                dpool = torch.empty_like(dpool_new).copy_(dpool_new)
            else:
                self._conv_back(f"e1_{l}", inp, dz1, None, d, need_dx=False)

    def loss_and_grad(self, y, target, mask):
        """Masked MSE over the 3 output channels; returns (loss (device), dy)."""
        vol = mask.numel()
        dy = torch.empty_like(y)
        N.call("anl_nn_mse", _p(y), _p(target), _p(mask), _p(dy), self.cout, vol, _p(self.red),
               _p(self.counter), _p(self.loss_out), _stream())
        return self.loss_out, dy

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        N.call("anl_nn_adam", _p(self.params), _p(self.grads), _p(self.m), _p(self.v), self.nparam, lr, b1, b2,
               eps, self.step_count, _stream())

    def state_dict(self):
        return {"base": self.base, "levels": self.levels, "params": self.params.cpu().numpy()}

    @classmethod
    def from_state(cls, st):
        net = cls(base=int(st["base"]), levels=int(st["levels"]))
        net.params.copy_(torch.as_tensor(st["params"]).to("cuda"))
        return net


# -------------------------------------------------------------------- features

def padded_dims(shape, mult=8):
    nx, ny, nz = shape
    r = lambda n: ((n + 1 + mult - 1) // mult) * mult
    return (r(nz), r(ny), r(nx))   # (D, H, W) of the node grid, padded


def node_features(shape, escale, E0, emin, p, F, fixed_mask, free_mask):
    """Network input (5 channels) and the loss mask on the padded node grid.
    escale: (ne,) element stiffness scales (CUDA); F: (3*nn,) loads; fixed_mask, free_mask:
    (3*nn,) uint8/bool. Returns (x (5*vol,), mask (vol,), dims, scale of F)."""
    nx, ny, nz = shape
    D, H, W = padded_dims(shape)
    dev = escale.device
    rho = ((escale.double() / E0 - emin) / (1 - emin)).clamp(min=0).pow(1.0 / p).float()
    r3 = rho.view(nz, ny, nx)
    node = torch.zeros(nz + 2, ny + 2, nx + 2, dtype=F32, device=dev)
    cnt = torch.zeros_like(node)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                node[dz:dz + nz, dy:dy + ny, dx:dx + nx] += r3
                cnt[dz:dz + nz, dy:dy + ny, dx:dx + nx] += 1
    node = (node / cnt.clamp(min=1))[:nz + 1, :ny + 1, :nx + 1]
    x = torch.zeros(5, D, H, W, dtype=F32, device=dev)
    x[0, :nz + 1, :ny + 1, :nx + 1] = node
    Fn = F.view(nz + 1, ny + 1, nx + 1, 3).float()
    fs = float(Fn.abs().max()) or 1.0
    for c in range(3):
        x[1 + c, :nz + 1, :ny + 1, :nx + 1] = Fn[..., c] / fs
    x[4, :nz + 1, :ny + 1, :nx + 1] = fixed_mask.view(nz + 1, ny + 1, nx + 1, 3).any(dim=-1).float()
    mask = torch.zeros(D, H, W, dtype=F32, device=dev)
    mask[:nz + 1, :ny + 1, :nx + 1] = free_mask.view(nz + 1, ny + 1, nx + 1, 3).any(dim=-1).float()
    return x.reshape(-1), mask.reshape(-1), (D, H, W), fs


def node_target(shape, u, dims):
    """Normalised displacement (3 channels) on the padded node grid, and its scale."""
    nx, ny, nz = shape
    D, H, W = dims
    U = u.view(nz + 1, ny + 1, nx + 1, 3).float()
    s = float(U.abs().max()) or 1.0
    t = torch.zeros(3, D, H, W, dtype=F32, device=u.device)
    for c in range(3):
        t[c, :nz + 1, :ny + 1, :nx + 1] = U[..., c] / s
    return t.reshape(-1), s


def unpad_displacement(shape, y, dims):
    """Network output (3 * vol,) -> full DOF vector (3 * nn,) float64."""
    nx, ny, nz = shape
    D, H, W = dims
    Y = y.view(3, D, H, W)[:, :nz + 1, :ny + 1, :nx + 1]
    return Y.permute(1, 2, 3, 0).reshape(-1).double().contiguous()


# -------------------------------------------------------------------- warm start

def galerkin_start(ctx, escale, F, u_prev, u_net, free, with_gain=False):
    """x0 = a u_prev + b u_net minimising the energy error over the two directions.
    free: (3 nn,) float64 0/1 mask. Returns (x0, a, b), plus with ``with_gain`` the drop of
    the energy Pi(x) = x.Kx/2 - F.x from the previous iterate to x0, relative to |Pi(u_prev)|
    (Pi - Pi(u*) is half the squared energy error, so this is the share of it removed)."""
    vecs = [v * free for v in (u_prev, u_net) if v is not None and float(v.abs().max()) > 0]
    if not vecs:
        z = torch.zeros_like(F)
        return (z, 0.0, 0.0, 0.0) if with_gain else (z, 0.0, 0.0)
    Kv = []
    for v in vecs:
        y = torch.empty(v.numel(), dtype=F32, device="cuda")
        ctx.apply_K(escale, v.float().contiguous(), y)
        Kv.append(y.double())
    n = len(vecs)
    G = np.array([[float(vecs[i] @ Kv[j]) for j in range(n)] for i in range(n)])
    G = 0.5 * (G + G.T)
    rhs = np.array([float(F @ v) for v in vecs])
    try:
        c = np.linalg.solve(G + 1e-14 * np.trace(G) * np.eye(n), rhs)
    except np.linalg.LinAlgError:
        c = np.zeros(n)
    x0 = sum(ci * v for ci, v in zip(c, vecs))
    coef = list(c) + [0.0] * (2 - n)
    prev_ok = u_prev is not None and float(u_prev.abs().max()) > 0
    if not prev_ok:
        coef = [0.0, coef[0]]
    if not with_gain:
        return x0, coef[0], coef[1]
    pi0 = 0.5 * G[0, 0] - rhs[0] if prev_ok else 0.0
    pi1 = -0.5 * float(c @ rhs)
    gain = (pi0 - pi1) / abs(pi0) if prev_ok and pi0 != 0 else 1.0
    return x0, coef[0], coef[1], gain


def energy(ctx, escale, F, x):
    """Pi(x) = x.Kx / 2 - F.x with the FP32 operator (one K u)."""
    y = torch.empty(x.numel(), dtype=F32, device="cuda")
    ctx.apply_K(escale, x.float().contiguous(), y)
    return 0.5 * float(x @ y.double()) - float(F @ x)


class WarmStart:
    """Wraps a trained UNet: ``predict`` gives the displacement direction for a solve."""

    def __init__(self, net, shape, E0, emin, p):
        self.net, self.shape, self.E0, self.emin, self.p = net, tuple(shape), E0, emin, p

    def predict(self, escale, F, fixed_mask, free_mask):
        x, mask, dims, _ = node_features(self.shape, escale, self.E0, self.emin, self.p, F, fixed_mask, free_mask)
        y = self.net.forward(x, dims)
        return unpad_displacement(self.shape, y, dims)


# -------------------------------------------------------------------- data and training

def simp_snapshots(work, iters, rtol=1e-6, log=lambda *a: None):
    """Runs the GPU SIMP loop on a workload and returns one (escale, u, F) snapshot per
    iteration (the displacement of that iteration's solve)."""
    from . import optimize as OPT
    from .fem import Grid
    grid = Grid(work.shape, work.h, (0, 0, 0))
    old = OPT.EMIN
    OPT.EMIN = work.emin
    try:
        run = OPT.SimpRunner(grid, work.fill, work.active, work.frozen, work.fixed, work.loads, work.weights,
                             work.E0, work.nu, work.vf, iters=iters, r_mm=work.r_vox, p_final=3.0, move=0.2,
                             x0=np.full(work.nelem, work.vf), beta_max=0.0, rtol=rtol, log=log)
        snaps = []
        for _ in range(iters):
            run.step()
            snaps.append((run.escale_t.clone(), run.U_t[0].clone(), run.F_t[0].clone()))
        fixed = torch.zeros(3 * grid.nnode, dtype=torch.uint8, device="cuda")
        fixed[torch.as_tensor(np.asarray(work.fixed), device="cuda")] = 1
        free = run.fem._mask_t.to(torch.uint8)
        run.close()
    finally:
        OPT.EMIN = old
    return snaps, fixed, free


def seeded_problem(seed, shape):
    """A cantilever with a random end load or (for nx >= 32, where its clamp patches still
    hold the part) an L-bracket with a random load direction, seeded."""
    from . import problems as P
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    vf = float(rng.uniform(0.2, 0.4))
    if rng.random() < 0.5 or nx < 32:
        w = P.cantilever(nx, ny, nz, vf=vf, r_vox=1.5)
        n = np.arange(w.nnode)
        i, j, k = n % (nx + 1), (n // (nx + 1)) % (ny + 1), n // ((nx + 1) * (ny + 1))
        kk = int(rng.integers(0, nz + 1))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        tip = n[(i == nx) & (k == kk)]
        F = np.zeros(3 * w.nnode)
        for c in range(3):
            F[3 * tip + c] = d[c] / tip.size
        w.loads = {"c": F}
        return w
    return P.lbracket(scale=nx / 192.0, vf=vf, r_vox=1.5, load_dirs=[tuple(rng.normal(size=3))])


def train(samples, net, epochs=10, lr=1e-3, log=print, seed=0):
    """samples: list of (x, target, mask, dims). Returns the per-epoch mean losses."""
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(len(samples))
        tot = 0.0
        t0 = time.time()
        for i in order:
            x, t, m, dims = samples[i]
            y = net.forward(x, dims)
            loss, dy = net.loss_and_grad(y, t, m)
            net.backward(dy)
            net.adam(lr)
            tot += float(loss[0]) / max(1.0, float(loss[1]))
        hist.append(tot / len(samples))
        log(f"  epoch {ep + 1}: loss {hist[-1]:.4e} ({time.time() - t0:.1f}s)")
    return hist
