"""Points sharded over several processes, one GPU each.

The forward path has no exchange step: every point's AO and MO values depend on that point alone
(the reference's kernels work per point: src/qmckl_ao_sycl.cpp:40-95 and :337-422,
src/qmckl_mo_sycl.cpp:24-50), so each rank evaluates its own contiguous range of points and keeps
its rows. The adjoint's parameter gradients (MO coefficients, primitive exponents) are sums over
points, so a sharded vector-Jacobian product needs one all-reduce of A*M + K doubles; the
coordinates' gradients stay with their rank. torch.distributed carries the all-reduce (gloo with
host tensors, or NCCL with device tensors); no kernel waits on another rank.
"""
import numpy as np


def point_range(point_num, rank, world, block=1):
    """The contiguous range [lo, hi) of `point_num` points that `rank` of `world` evaluates, in whole
    blocks of `block` points (a walker's electrons, say), as equal as whole blocks allow."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %r outside a world of %r" % (rank, world))
    if block < 1 or point_num % block:
        raise ValueError("point_num %r is not a whole number of blocks of %r" % (point_num, block))
    blocks = point_num // block
    lo = rank * blocks // world
    hi = (rank + 1) * blocks // world
    return lo * block, hi * block


def vjp_mo_vgl_allreduce(ctx, w, prim_num, group=None):
    """Gradients of L = sum over all ranks' points of w * mo_vgl, for a context that holds this
    rank's points and w their [P][5][M] weights: the local qmckl_vjp_mo_vgl_device call, then one
    all-reduce (sum) of the coefficient and exponent gradients. Returns {'coef': [M][A] (all
    ranks), 'expo': [K] (all ranks), 'coord': [P][3] (this rank's points)}."""
    import torch
    import torch.distributed as dist

    g = ctx.vjp_mo_vgl(w, prim_num=prim_num)
    coef, expo = g["coef"], g["expo"]
    flat = torch.from_numpy(np.concatenate([coef.ravel(), expo.ravel()]))
    if dist.get_backend(group) == "nccl":
        t = flat.to("cuda")
        dist.all_reduce(t, group=group)
        flat = t.cpu()
    else:
        dist.all_reduce(flat, group=group)
    out = flat.numpy()
    return {"coef": out[:coef.size].reshape(coef.shape), "expo": out[coef.size:].copy(), "coord": g["coord"]}
