"""Float64 CPU oracle of the surrogate's 3^3 circular convolutions -- TEST INFRASTRUCTURE ONLY.

Only the tests import it.  It restates the kernels' definition with torch CPU float64 ops:
out[z, y, x, co] = sum_{tap, ci} W[tap, co, ci] in[(z + dz) % n, (y + dy) % n, (x + dx) % n, ci] + b[co]
with tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1); gradients come from float64 autograd.
"""
import torch
import torch.nn.functional as F


def _to_conv(w):
    # [27, cout, cin] -> conv3d weight [cout, cin, 3, 3, 3] (cross-correlation, tap offsets -1..1)
    t, co, ci = w.shape
    return w.reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)


def conv3d(x, w, b=None):
    """x [n, n, n, cin] -> [n, n, n, cout], float64, circular padding."""
    xc = x.permute(3, 0, 1, 2).unsqueeze(0)
    xc = F.pad(xc, (1, 1, 1, 1, 1, 1), mode="circular")
    y = F.conv3d(xc, _to_conv(w), b)
    return y[0].permute(1, 2, 3, 0)


def conv3d_planes(x, w, b, planes):
    """conv3d's output on the z-planes `planes` only: [len(planes), n, n, cout], float64."""
    n = x.shape[0]
    outs = []
    for z in planes:
        slab = x[[(z - 1) % n, z, (z + 1) % n]].double()          # [3, n, n, cin]
        xc = slab.permute(3, 0, 1, 2).unsqueeze(0)
        xc = torch.cat([xc[..., -1:], xc, xc[..., :1]], dim=-1)   # circular in x
        xc = torch.cat([xc[..., -1:, :], xc, xc[..., :1, :]], dim=-2)  # circular in y
        y = F.conv3d(xc, _to_conv(w.double()), None if b is None else b.double())
        outs.append(y[0, :, 0].permute(1, 2, 0))
    return torch.stack(outs)


def net_forward(feats, ws, bs):
    """Hidden layers ReLU, last layer sigmoid of channel 0; returns (pred, activations)."""
    acts = [feats]
    x = feats
    for w, b in zip(ws[:-1], bs[:-1]):
        x = torch.relu(conv3d(x, w, b))
        acts.append(x)
    z = conv3d(x, ws[-1], bs[-1])
    return torch.sigmoid(z[..., 0]), acts


def net_grads(feats, ws, bs, target):
    """Gradients of the summed binary cross-entropy w.r.t. every weight and bias (float64)."""
    ws = [w.detach().clone().double().requires_grad_(True) for w in ws]
    bs = [b.detach().clone().double().requires_grad_(True) for b in bs]
    pred, _ = net_forward(feats.double(), ws, bs)
    p = pred.clamp(1e-12, 1 - 1e-12)
    t = target.double()
    loss = -(t * torch.log(p) + (1 - t) * torch.log(1 - p)).sum()
    loss.backward()
    return [w.grad for w in ws], [b.grad for b in bs], pred.detach()
