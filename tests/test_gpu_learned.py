"""The warm-start network's CUDA layers and the U-Net's passes against the FP64 CPU oracle
(oracle/unet_oracle.py: torch autograd in float64), through the C ABI; then training and the
warm start itself. Tolerances: FP32 kernels against FP64, relative to each tensor's scale."""
import ctypes

import numpy as np
import pytest
import torch
import torch.nn.functional as Fn

from oracle import unet_oracle as UO

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _close(got, want, tol):
    got = got.detach().double().cpu()
    want = want.detach().double().cpu()
    scale = max(float(want.abs().max()), 1e-30)
    err = float((got - want).abs().max()) / scale
    assert err <= tol, f"relative error {err:.2e} > {tol:.0e}"


@pytest.mark.parametrize("k,cin,cout,dims,act", [(3, 5, 20, (5, 9, 12), 1), (3, 16, 16, (8, 8, 8), 0),
                                                 (1, 16, 3, (6, 7, 9), 0), (3, 3, 33, (4, 17, 10), 1)])
def test_conv3d_forward_and_backward(k, cin, cout, dims, act):
    from anneal_gb300 import _native as N
    g = torch.Generator().manual_seed(k * 100 + cin + cout)
    x = torch.randn(cin, *dims, generator=g, dtype=torch.float64)
    w = torch.randn(cout, cin, k, k, k, generator=g, dtype=torch.float64) / (cin * k ** 3) ** 0.5
    b = torch.randn(cout, generator=g, dtype=torch.float64)
    xw = x.clone().requires_grad_(True)
    ww = w.clone().requires_grad_(True)
    bb = b.clone().requires_grad_(True)
    z_ref = Fn.conv3d(xw[None], ww, bb, padding=k // 2)[0]
    a_ref = Fn.gelu(z_ref) if act else z_ref
    da = torch.randn_like(a_ref)
    (a_ref * da).sum().backward()
    D, H, W = dims
    xd, wd, bd = x.float().cuda(), w.float().cuda(), b.float().cuda()
    z = torch.empty(cout, *dims, device="cuda")
    a = torch.empty_like(z)
    N.call("anl_nn_conv3d", _p(xd), _p(wd), _p(bd), _p(z), _p(a) if act else None, cin, cout, D, H, W, k, act, 0, None)
    _close(z, z_ref, 2e-6)
    if act:
        _close(a, a_ref, 2e-6)
    dz = torch.empty_like(z)
    dad = da.float().cuda()
    if act:
        N.call("anl_nn_gelu_bwd", _p(z), _p(dad), _p(dz), z.numel(), None)
    else:
        dz.copy_(dad)
    dx = torch.empty_like(xd)
    wt = torch.empty(wd.numel(), device="cuda")
    N.call("anl_nn_conv3d_bwd_data", _p(dz), _p(wd), _p(wt), _p(dx), cin, cout, D, H, W, k, 0, None)
    _close(dx, xw.grad, 5e-6)
    part = torch.empty(64 * (wd.numel() + cout), device="cuda")
    dw = torch.empty_like(wd)
    db = torch.empty_like(bd)
    N.call("anl_nn_conv3d_bwd_weight", _p(xd), _p(dz), _p(part), part.numel(), _p(dw), _p(db), cin, cout, D, H, W, k,
           0, None)
    _close(dw, ww.grad, 5e-6)
    _close(db, bb.grad, 5e-6)


def test_pool_and_upsample():
    from anneal_gb300 import _native as N
    g = torch.Generator().manual_seed(3)
    x = torch.randn(6, 8, 6, 10, generator=g, dtype=torch.float64)
    xd = x.float().cuda()
    y = torch.empty(6, 4, 3, 5, device="cuda")
    N.call("anl_nn_pool2", _p(xd), _p(y), 6, 8, 6, 10, 0, 0, None)
    _close(y, Fn.avg_pool3d(x[None], 2)[0], 1e-6)
    gy = torch.randn(6, 4, 3, 5, generator=g, dtype=torch.float64)
    gx = torch.zeros_like(xd)
    N.call("anl_nn_pool2", _p(gy.float().cuda()), _p(gx), 6, 8, 6, 10, 1, 1, None)
    xr = x.clone().requires_grad_(True)
    (Fn.avg_pool3d(xr[None], 2)[0] * gy).sum().backward()
    _close(gx, xr.grad, 1e-6)
    h = torch.randn(6, 4, 3, 5, generator=g, dtype=torch.float64)
    up = torch.empty(6, 8, 6, 10, device="cuda")
    N.call("anl_nn_up2", _p(h.float().cuda()), _p(up), 6, 8, 6, 10, 0, None)
    _close(up, Fn.interpolate(h[None], scale_factor=2, mode="nearest")[0], 1e-6)
    gu = torch.randn(6, 8, 6, 10, generator=g, dtype=torch.float64)
    gh = torch.empty(6, 4, 3, 5, device="cuda")
    N.call("anl_nn_up2", _p(gu.float().cuda()), _p(gh), 6, 8, 6, 10, 1, None)
    hr = h.clone().requires_grad_(True)
    (Fn.interpolate(hr[None], scale_factor=2, mode="nearest")[0] * gu).sum().backward()
    _close(gh, hr.grad, 1e-6)


def test_unet_loss_and_gradients_match_oracle():
    from anneal_gb300.learned import UNet
    net = UNet(base=4, levels=3, seed=1)
    dims = (8, 12, 16)
    g = torch.Generator().manual_seed(0)
    x = torch.randn(5, *dims, generator=g, dtype=torch.float64)
    t = torch.randn(3, *dims, generator=g, dtype=torch.float64)
    m = (torch.rand(*dims, generator=g) > 0.3).double()
    y = net.forward(x.float().cuda().reshape(-1), dims)
    loss, dy = net.loss_and_grad(y, t.float().cuda().reshape(-1), m.float().cuda().reshape(-1))
    net.backward(dy)
    P = UO.unflatten(net.params.cpu().double(), net.specs)
    y_ref = UO.forward(P, x, 3)
    l_ref = UO.loss(y_ref, t, m)
    l_ref.backward()
    _close(y.view(3, *dims), y_ref, 2e-5)
    assert abs(float(loss[0]) / float(loss[1]) / float(l_ref.detach()) - 1) < 1e-5
    for name, _, _, _ in net.specs:
        _close(net.gw[name], P[name][0].grad, 2e-4)
        _close(net.gb[name], P[name][1].grad, 2e-4)


def test_adam_step():
    from anneal_gb300 import _native as N
    g = torch.Generator().manual_seed(4)
    p = torch.randn(1000, generator=g)
    gr = torch.randn(1000, generator=g)
    m = torch.zeros(1000)
    v = torch.zeros(1000)
    pd, md, vd = p.cuda(), m.cuda(), v.cuda()
    for step in (1, 2, 3):
        N.call("anl_nn_adam", _p(pd), _p(gr.cuda()), _p(md), _p(vd), 1000, 1e-3, 0.9, 0.999, 1e-8, step, None)
        m = 0.9 * m + 0.1 * gr
        v = 0.999 * v + 0.001 * gr * gr
        p = p - 1e-3 * (m / (1 - 0.9 ** step)) / ((v / (1 - 0.999 ** step)).sqrt() + 1e-8)
    _close(pd, p, 1e-5)


def test_training_and_warm_start_never_hurt():
    """Trains a small net on SIMP snapshots of seeded cantilevers and L-brackets, then
    compares CG iterations on an unseen problem: previous iterate vs the Galerkin
    combination with the prediction (which must never need more than a few extra iterations
    and must not raise the initial energy error)."""
    from anneal_gb300 import learned as LW
    from anneal_gb300.context import Context
    shape = (32, 16, 16)
    samples = []
    for seed in range(3):
        w = LW.seeded_problem(seed, shape)
        snaps, fixed, free = LW.simp_snapshots(w, 6)
        for esc, u, F in snaps:
            x, mask, dims, _ = LW.node_features(shape, esc, w.E0, w.emin, 3.0, F, fixed, free)
            tgt, _ = LW.node_target(shape, u, dims)
            samples.append((x, tgt, mask, dims))
    net = LW.UNet(base=8, levels=3, seed=0)
    hist = LW.train(samples, net, epochs=20, lr=2e-3, log=lambda *a: None)
    assert hist[-1] < 0.6 * hist[0], hist
    # unseen problem: one solve from the previous iterate and one from the combination
    w = LW.seeded_problem(11, shape)
    snaps, fixed, free = LW.simp_snapshots(w, 3)
    (e_prev, u_prev, F), (e_cur, u_cur, _) = snaps[1], snaps[2]
    ws = LW.WarmStart(net, shape, w.E0, w.emin, 3.0)
    u_net = ws.predict(e_cur, F, fixed, free)
    ctx = Context(shape, 1.0, 0.3, fp64=False)
    ctx.set_domain(torch.as_tensor(w.active.astype(np.uint8)).cuda(), fixed)
    freef = free.double()
    x0, a, b = LW.galerkin_start(ctx, e_cur, F, u_prev, u_net, freef)

    def energy_err(x):
        y = torch.empty(x.numel(), device="cuda")
        ctx.apply_K(e_cur, (x - u_cur).float().contiguous(), y)
        return float((x - u_cur) @ y.double())
    assert energy_err(x0) <= energy_err(u_prev * freef) * (1 + 1e-6)
    its = {}
    for name, start in (("prev", u_prev.clone()), ("learned", x0.clone())):
        X = start.view(1, -1).clone()
        st, it, _ = ctx.solve(e_cur, F.view(1, -1), X, 1e-6, 2000, True)
        its[name] = it[0]
    ctx.close()
    assert its["learned"] <= its["prev"] + 2, its
