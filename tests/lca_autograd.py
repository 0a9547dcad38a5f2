"""Differentiable LCA in the test harness: torch.autograd.Function wrappers around the C-ABI
delivery kernels and their adjoints (test infrastructure; the product exposes only the C ABI).

Adjoint pairs (all through libpvgpu.so):
  reconstruction  y = W^T a   (pvgpu_deliver_pre, V1 -> error, presynaptic perspective)
      dL/da = W g             (pvgpu_deliver_post, the transpose delivery)
      dL/dW = sum a (x) g     (pvgpu_hebbian_dw with pre = a, post = g: the pre x post correlation
                               of HebbianUpdater::updateInd_dW, dWMax = 1)
  drive           z = W r     (pvgpu_deliver_post, error -> V1, postsynaptic perspective)
      dL/dr = W^T h           (pvgpu_deliver_pre)
      dL/dW = sum h (x) r     (pvgpu_hebbian_dw with pre = h, post = r)

Tensors are in the reference layouts: V1 activity extended [nb][nyExt][nxExt][nf], error
restricted [nb][ny][nx][c]; weights [F][P][P][C] (V1 -> error, pre weights).
"""
import numpy as np
import torch
import torch.utils.checkpoint

from openpv_gb300 import capi


class Geometry:
    """V1 (stride S over an error layer of ny x nx x c) with square patches P, as LCA uses."""

    def __init__(self, nb, in_shape, v1_shape, P):
        iy, ix, ic = in_shape
        vy, vx, vf = v1_shape
        s = ix // vx
        self.nb, self.P, self.S = nb, P, s
        m_v1 = (P // s) // 2                     # requiredConvolveMargin, one-to-many
        m_err = (P // s - 1) * s // 2            # requiredConvolveMargin of the transpose
        self.v1 = capi.Loc.make(nb, vx, vy, vf, m_v1)
        self.err = capi.Loc.make(nb, ix, iy, ic, m_err)
        self.err_res = capi.Loc.make(nb, ix, iy, ic, 0)
        self.v1_res = capi.Loc.make(nb, vx, vy, vf, 0)
        self.pre = capi.conn_desc(self.v1, self.err_res, P, P)            # recon into restricted GSyn
        self.post = capi.conn_desc(self.err, self.v1_res, P // s, P // s)  # error -> V1
        self.pre_h = capi.conn_desc(self.v1, self.err, P, P)              # Hebbian reads post extended

    def extend_v1(self, a):
        h = self.v1.halo.lt
        return torch.nn.functional.pad(a, (0, 0, h, h, h, h)).contiguous()

    def extend_err(self, r):
        h = self.err.halo.lt
        return torch.nn.functional.pad(r, (0, 0, h, h, h, h)).contiguous()


def _hebbian(geo, pre_ext, post_ext, nk):
    dw = torch.zeros(nk, device=pre_ext.device)
    capi.hebbian_dw(geo.pre_h, 1.0, pre_ext, post_ext, dw)
    return dw


class Recon(torch.autograd.Function):
    """y = W^T a (restricted error layer) from the V1 activity a (restricted)."""

    @staticmethod
    def forward(ctx, a, w, geo):
        ae = geo.extend_v1(a)
        y = torch.zeros(geo.err_res.res_shape(), device=a.device)
        capi.deliver_pre(geo.pre, w.contiguous(), y, a_ext=ae)
        ctx.save_for_backward(ae, w)
        ctx.geo = geo
        return y

    @staticmethod
    def backward(ctx, g):
        ae, w = ctx.saved_tensors
        geo = ctx.geo
        ge = geo.extend_err(g.contiguous())
        ga = torch.zeros(geo.v1_res.res_shape(), device=g.device)
        capi.deliver_post(geo.post, ge, w.contiguous(), ga)
        gw = _hebbian(geo, ae, ge, w.numel()).view_as(w)
        return ga, gw, None


class Drive(torch.autograd.Function):
    """z = W r (V1 GSyn, restricted) from the residual r (restricted error layer)."""

    @staticmethod
    def forward(ctx, r, w, geo):
        re = geo.extend_err(r)
        z = torch.zeros(geo.v1_res.res_shape(), device=r.device)
        capi.deliver_post(geo.post, re, w.contiguous(), z)
        ctx.save_for_backward(re, w)
        ctx.geo = geo
        return z

    @staticmethod
    def backward(ctx, h):
        re, w = ctx.saved_tensors
        geo = ctx.geo
        he = geo.extend_v1(h.contiguous())
        gr = torch.zeros(geo.err_res.res_shape(), device=h.device)
        capi.deliver_pre(geo.pre, w.contiguous(), gr, a_ext=he)
        gw = _hebbian(geo, he, re, w.numel()).view_as(w)
        return gr, gw, None


def soft_threshold(v, vthresh):
    """ANNActivityBuffer with AMin = 0, AShift = VThresh, VWidth = 0 (the LCA soft threshold)."""
    return torch.where(v >= vthresh, v - vthresh, torch.zeros_like(v))


def lca_segment(v, w, x, geo, steps, e, vthresh):
    for _ in range(steps):
        a = soft_threshold(v, vthresh)
        r = x - Recon.apply(a, w, geo)
        v = e * v + (1.0 - e) * (Drive.apply(r, w, geo) + a)
    return v


def unrolled_lca_loss(w, x, geo, steps, vthresh, lam, tau=100.0, checkpoint_every=10):
    """a_T from `steps` LCA timesteps from V = 0 (checkpointed every `checkpoint_every` steps),
    then L = 0.5 ||x - W^T a_T||^2 + lam ||a_T||_1 summed over the batch."""
    e = float(np.float32(np.exp(-1.0 / tau)))
    v = torch.zeros(geo.v1_res.res_shape(), device=x.device)
    done = 0
    while done < steps:
        k = min(checkpoint_every, steps - done)
        v = torch.utils.checkpoint.checkpoint(lca_segment, v, w, x, geo, k, e, vthresh, use_reentrant=False)
        done += k
    a = soft_threshold(v, vthresh)
    r = x - Recon.apply(a, w, geo)
    return 0.5 * (r * r).sum() + lam * a.abs().sum()
