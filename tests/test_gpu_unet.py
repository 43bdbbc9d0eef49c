"""The learned warm start: BF16 tensor-core U-Net forward and backward
kernels against the numpy oracle (oracle/unet_oracle.py), training, and the
learned guess inside the solver.

Tolerances: the oracle rounds weights, inputs, activations and activation
gradients to BF16 where the GPU does, so the remaining differences come from
FP32 accumulation order and the rounding boundaries it moves: output within
1e-2 of its scale; each layer's weight and bias gradient within 5e-2 of the
BF16 oracle's norm plus the BF16 noise of that layer (the distance between
the BF16 oracle and the same oracle in exact arithmetic, which reaches
4-20 % on small grids); a wrong tap, padding or layout gives O(1) errors."""
import os

import numpy as np
import pytest

from _util import params_of, periodic_case, rel_err

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("dims,per,levels", [((8, 8, 8), (1, 1, 1), 2), ((16, 8, 8), (1, 0, 1), 3)])
def test_unet_forward_and_gradients_match_oracle(o3d, dims, per, levels):
    torch = pytest.importorskip("torch")
    from oracle import unet_oracle as U
    nvox = dims[0] * dims[1] * dims[2]
    net = o3d.UNet(dims, periodic=per, base=16, levels=levels, in_channels=2, seed=7)
    p = net.get_params()
    rng = np.random.default_rng(3)
    inp = rng.standard_normal((2, nvox)).astype(np.float32)
    tgt = rng.standard_normal(nvox).astype(np.float32)
    d_in, d_tgt = _dev(inp.reshape(-1)), _dev(tgt)
    d_out = torch.zeros(nvox, dtype=torch.float32, device="cuda")
    net.forward(d_in.data_ptr(), d_out.data_ptr())
    torch.cuda.synchronize()
    out_ref, loss_ref, g_ref = U.forward_backward(p.astype(np.float64), inp.astype(np.float64),
                                                  tgt.astype(np.float64), dims, per, 16, levels)
    _, _, g_exact = U.forward_backward(p.astype(np.float64), inp.astype(np.float64), tgt.astype(np.float64),
                                       dims, per, 16, levels, bf16_round=False)
    assert rel_err(d_out.cpu().numpy(), out_ref) < 1e-2
    loss, g = net.gradients(d_in.data_ptr(), d_tgt.data_ptr())
    assert loss == pytest.approx(loss_ref, rel=1e-2)
    L = U.Layout(16, levels)
    for name, (w0, b0, K, N) in L.layers.items():
        for sl in (slice(w0, b0), slice(b0, b0 + N)):
            ref, ex = g_ref[sl], g_exact[sl]
            # rounding flips move the GPU away from the BF16 oracle by at most
            # the BF16 noise itself (the oracle's distance to exact arithmetic)
            bound = 5e-2 * np.linalg.norm(ref) + np.linalg.norm(ref - ex) + 1e-12
            assert np.linalg.norm(g[sl] - ref) <= bound, name
    hw = slice(L.head_w, L.head_b + 1)
    assert np.linalg.norm(g[hw] - g_ref[hw]) <= 2e-2 * np.linalg.norm(g_ref[hw])
    net.close()


def test_unet_forward_unsplit_matches_oracle(o3d):
    """The guess grid of a 256^3 run (32^3): its level-0 convolutions fill
    the GPU without splitting the (tap, channel) reduction, so they take the
    fused-epilogue path that the small grids above do not reach; the output
    agrees with the BF16 oracle as on the small grids."""
    torch = pytest.importorskip("torch")
    from oracle import unet_oracle as U
    dims, per, levels = (32, 32, 32), (1, 1, 1), 2
    nvox = dims[0] * dims[1] * dims[2]
    net = o3d.UNet(dims, periodic=per, base=16, levels=levels, in_channels=2, seed=11)
    p = net.get_params()
    rng = np.random.default_rng(5)
    inp = rng.standard_normal((2, nvox)).astype(np.float32)
    d_in = _dev(inp.reshape(-1))
    d_out = torch.zeros(nvox, dtype=torch.float32, device="cuda")
    net.forward(d_in.data_ptr(), d_out.data_ptr())
    torch.cuda.synchronize()
    out_ref, _, _ = U.forward_backward(p.astype(np.float64), inp.astype(np.float64), np.zeros(nvox), dims, per, 16,
                                       levels)
    assert rel_err(d_out.cpu().numpy(), out_ref) < 1e-2
    net.close()


def test_unet_training_reduces_loss(o3d):
    """A few hundred Adam steps on a fixed smooth sample fit it."""
    torch = pytest.importorskip("torch")
    dims = (16, 16, 16)
    nvox = 16 ** 3
    x = np.arange(16) * 2 * np.pi / 16
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    f = lambda a: np.ravel(a, order="F")
    inp = np.stack([f(np.sin(X) * np.cos(Y)), f(np.cos(Z))]).astype(np.float32)
    tgt = f(0.5 * np.sin(X) * np.cos(Y) + 0.25 * np.cos(Z)).astype(np.float32)
    net = o3d.UNet(dims, periodic=(1, 1, 1), base=16, levels=3, seed=11)
    d_in, d_tgt = _dev(inp.reshape(-1)), _dev(tgt)
    first = net.train_step(d_in.data_ptr(), d_tgt.data_ptr(), 1e-3)
    for _ in range(300):
        last = net.train_step(d_in.data_ptr(), d_tgt.data_ptr(), 1e-3)
    assert last < 0.05 * first, (first, last)
    net.close()


def test_learned_guess_in_the_step(oracle, o3d):
    """With an attached (untrained) network the solver still converges to eps,
    so the step matches the FP64 oracle; the sampler writes finite features."""
    torch = pytest.importorskip("torch")
    from _util import perturbed
    c = periodic_case(oracle, 32, omega=1.6, eps=1e-11, kmax=100000)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    for a in range(3):
        s.u[a][...] = perturbed(s.u[a], 40 + a)
    runner = oracle.Runner(c, s)
    with o3d.Context(params_of(o3d, c, solver=o3d.SOLVER_MG, kmax=200, guess=o3d.GUESS_LEARNED)) as ctx:
        dims = ctx.guess_grid()
        assert dims == (16, 16, 16)
        net = o3d.UNet(dims, periodic=(1, 1, 1), base=16, levels=2, seed=5)
        ctx.attach_unet(net)
        n2 = dims[0] * dims[1] * dims[2]
        feat = torch.zeros(2 * n2, dtype=torch.float32, device="cuda")
        tgt = torch.zeros(n2, dtype=torch.float32, device="cuda")
        ctx.set_sample_buffers(feat.data_ptr(), tgt.data_ptr())
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        ctx.upload("pp", s.pp)
        for it in range(1, 5):
            runner.step(it)
            info = ctx.step(it)
            assert info.poisson_status == 0
            assert ctx.sample_ready() == (it > 1)
        for a, name in enumerate(("ux", "uy", "uz")):
            assert rel_err(ctx.download(name), s.u[a]) < 1e-9, name
        torch.cuda.synchronize()
        assert torch.isfinite(feat).all() and torch.isfinite(tgt).all()
        assert float(tgt.abs().max()) > 0
        ctx.set_sample_buffers(None, None)
        ctx.attach_unet(None)
        net.close()


def _cycles(o3d, guess, n, steps, warmup, weights=None):
    """Mean V-cycles per step (steps after warm-up) and the final velocity of
    the n^3 Taylor-Green run, Poisson eps = 1e-8, mixed precision."""
    from osinco3d_gb300 import learn

    p = o3d.tgv_params(n, re=1600.0, precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG, eps=1e-8, kmax=100,
                       guess=guess)
    with o3d.Context(p) as ctx:
        net = None
        if weights:
            net = learn.load(weights, ctx.guess_grid())
            ctx.attach_unet(net)
        for nm, f in zip(("ux", "uy", "uz", "pp"), o3d.tgv_fields(p)):
            ctx.upload(nm, f)
        cyc = []
        for it in range(1, warmup + steps + 1):
            info = ctx.step(it)
            assert info.poisson_status == 0
            if it > warmup:
                cyc.append(info.poisson_cycles)
        u = ctx.download("ux")
        if net:
            ctx.attach_unet(None)
            net.close()
    return float(np.mean(cyc)), u


@pytest.mark.slow
def test_trained_network_saves_v_cycles(o3d):
    """The committed network (trained on 128^3 solver samples) against the
    same solver without it, at 256^3: the extrapolated guess alone, and the
    previous step's pressure (the reference's start).  Every run iterates to
    the same eps, so the velocity agrees; the network must save V-cycles."""
    from osinco3d_gb300 import learn

    if not os.path.exists(learn.WEIGHTS):
        pytest.skip("no trained weights")
    n, steps, warmup = 256, 6, 3
    c_prev, u_prev = _cycles(o3d, o3d.GUESS_PREVIOUS, n, steps, warmup)
    c_ex, u_ex = _cycles(o3d, o3d.GUESS_EXTRAPOLATED, n, steps, warmup)
    c_nn, u_nn = _cycles(o3d, o3d.GUESS_LEARNED, n, steps, warmup, weights=learn.WEIGHTS)
    print(f"V-cycles per step at {n}^3: previous {c_prev:.2f}, extrapolated {c_ex:.2f}, learned {c_nn:.2f}")
    assert c_nn < c_ex <= c_prev
    scale = np.abs(u_ex).max()
    assert np.abs(u_nn - u_ex).max() < 1e-6 * scale
    assert np.abs(u_prev - u_ex).max() < 1e-6 * scale
