"""FP64 CPU reference of the warm-start network (torch autograd on the CPU).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA layers (anl_nn_*) and of the U-Net's
forward and backward passes in anneal_gb300/learned.py. The network has no counterpart in
the reference (it replaces the previous-iterate start of optimize.py:122), so its oracle is
a plain float64 restatement of the same layers: 3x3x3 / 1x1x1 convolutions with zero
padding, exact (erf) GELU, 2x average pooling, 2x nearest upsampling with skip
concatenation, and the masked mean-squared error.
"""
import torch
import torch.nn.functional as Fn


def unflatten(params, specs):
    """Flat parameter vector (the GPU layout) -> {name: (w, b)} float64 tensors."""
    out, off = {}, 0
    p = torch.as_tensor(params, dtype=torch.float64)
    for name, ci, co, k in specs:
        nw = co * ci * k ** 3
        w = p[off:off + nw].view(co, ci, k, k, k).clone().requires_grad_(True)
        off += nw
        b = p[off:off + co].clone().requires_grad_(True)
        off += co
        out[name] = (w, b)
    return out


def forward(P, x, levels):
    """x: (cin, D, H, W) float64. Returns the (cout, D, H, W) output."""
    def conv(name, t, act=True):
        w, b = P[name]
        k = w.shape[-1]
        z = Fn.conv3d(t[None], w, b, padding=k // 2)[0]
        return Fn.gelu(z) if act else z
    skips = []
    h = x
    for l in range(levels):
        h = conv(f"e2_{l}", conv(f"e1_{l}", h))
        if l < levels - 1:
            skips.append(h)
            h = Fn.avg_pool3d(h[None], 2)[0]
    for l in range(levels - 2, -1, -1):
        up = Fn.interpolate(h[None], scale_factor=2, mode="nearest")[0]
        h = conv(f"d2_{l}", conv(f"d1_{l}", torch.cat([up, skips[l]], 0)))
    return conv("out", h, act=False)


def loss(y, t, mask):
    d = (y - t) ** 2 * mask[None]
    return d.sum() / torch.clamp(mask.sum(), min=1.0)
