"""Training data, training and evaluation of the learned Poisson warm start.

The network maps the restricted FP64 residual of the extrapolated pressure
p_ex = 2 p^n - p^(n-1) and the last pressure increment to the coarse part of
the remaining correction p^(n+1) - p_ex (see o3d.h, "learned Poisson warm
start").  Samples come from the solver itself: a multigrid context with the
extrapolated (or learned) guess and sample buffers writes (features,
target) for every solve that has a previous pressure.  Training runs the library's own BF16 forward/backward kernels and
Adam (o3d_unet_train_step); PyTorch only holds the device buffers.

  python -m osinco3d_gb300.learn train --n 128 --runs 8 --steps 150 --epochs 6 --out weights.npz
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import o3d

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_tgv.npz")


def _perturbation(shape, seed, amp):
    """Smooth, periodic, seeded velocity perturbation (three modes per component)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    x = np.arange(nx) * 2 * math.pi / nx
    y = np.arange(ny) * 2 * math.pi / ny
    z = np.arange(nz) * 2 * math.pi / nz
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    out = []
    for _ in range(3):
        f = np.zeros(shape)
        for _m in range(3):
            k = rng.integers(1, 5, 3)
            ph = rng.uniform(0, 2 * math.pi, 3)
            f += rng.standard_normal() * np.sin(k[0] * X + ph[0]) * np.sin(k[1] * Y + ph[1]) * np.sin(k[2] * Z + ph[2])
        out.append(np.asfortranarray(amp * f))
    return out


def generate(n: int, runs: int, steps: int, seed: int = 0, re_range=(800.0, 3000.0), noise=(0.0, 0.05)):
    """Runs `runs` seeded Taylor-Green simulations at n^3 (Re and perturbation
    amplitude drawn from the ranges) with the mixed-precision multigrid solver
    and collects one sample per solve.  Returns device tensors (feat, tgt)."""
    import torch

    rng = np.random.default_rng(seed)
    feats, tgts = [], []
    for r in range(runs):
        re = float(rng.uniform(*re_range))
        amp = float(rng.uniform(*noise))
        p = o3d.tgv_params(n, re=re, precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG, eps=1e-8, kmax=100,
                           guess=o3d.GUESS_EXTRAPOLATED)
        with o3d.Context(p) as ctx:
            dims = ctx.guess_grid()
            n2 = dims[0] * dims[1] * dims[2]
            ux, uy, uz, pp = o3d.tgv_fields(p)
            du = _perturbation(ux.shape, seed * 1000 + r, amp)
            for nm, f in zip(("ux", "uy", "uz"), (ux + du[0], uy + du[1], uz + du[2])):
                ctx.upload(nm, np.asfortranarray(f))
            ctx.upload("pp", pp)
            fb = torch.zeros(2 * n2, dtype=torch.float32, device="cuda")
            tb = torch.zeros(n2, dtype=torch.float32, device="cuda")
            ctx.set_sample_buffers(fb.data_ptr(), tb.data_ptr())
            for it in range(1, steps + 1):
                ctx.step(it)
                if ctx.sample_ready():
                    torch.cuda.synchronize()
                    feats.append(fb.clone())
                    tgts.append(tb.clone())
            ctx.set_sample_buffers(None, None)
    return torch.stack(feats), torch.stack(tgts), dims


def train(net: "o3d.UNet", feat, tgt, epochs: int, lr: float = 1e-3, seed: int = 0, log=None):
    """Adam on single samples in shuffled order; returns the mean loss per epoch."""
    import torch

    rng = np.random.default_rng(seed)
    hist = []
    if log:
        log(f"zero-prediction loss {float((tgt.double() ** 2).mean()):.4e}")
    for ep in range(epochs):
        order = rng.permutation(feat.shape[0])
        tot = 0.0
        lr_ep = lr * (0.5 ** (ep // 3))
        for i in order:
            tot += net.train_step(feat[i].data_ptr(), tgt[i].data_ptr(), lr_ep)
        torch.cuda.synchronize()
        hist.append(tot / len(order))
        if log:
            log(f"epoch {ep} loss {hist[-1]:.4e}")
    return hist


def to_bf16_bits(a: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 bit patterns (round to nearest, ties to even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def save(net: "o3d.UNet", path: str) -> None:
    """Parameters as BF16 (the precision the convolutions use; the biases and
    the head, which run in FP32, are rounded too), with the architecture."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params_bf16=to_bf16_bits(net.get_params()), base=net.base, levels=net.levels,
                        in_channels=net.in_channels)


def load(path: str, dims, periodic=(1, 1, 1)) -> "o3d.UNet":
    d = np.load(path)
    net = o3d.UNet(dims, periodic=periodic, base=int(d["base"]), levels=int(d["levels"]),
                   in_channels=int(d["in_channels"]))
    net.set_params(from_bf16_bits(d["params_bf16"]) if "params_bf16" in d else d["params"])
    return net


def inference_ms(net: "o3d.UNet", reps: int = 20) -> float:
    """Wall time of one forward pass on random input (launches included)."""
    import torch

    n = net.dims[0] * net.dims[1] * net.dims[2]
    x = torch.randn(net.in_channels * n, device="cuda")
    y = torch.empty(n, device="cuda")
    for _ in range(3):
        net.forward(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        net.forward(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    return 1e3 * (time.perf_counter() - t0) / reps


def compare_guesses(n: int, steps: int, warmup: int, weights: str | None, precision=o3d.PREC_MIXED, re=1600.0,
                    seed: int = 17, t0: float = 0.0, cycle: dict | None = None, guesses=None, amp: float = 0.02):
    """Poisson V-cycles and time per step on the n^3 Taylor-Green run for the
    zero, previous, extrapolated and (with weights) learned initial guesses,
    all iterating to eps = 1e-8.  The measured steps start at time t0 (the
    run gets there first); `cycle` sets mg_pre, mg_post and mg_omega; `amp`
    is the amplitude of the seeded smooth perturbation of the initial state."""
    results = {}
    all_guesses = [("zero", o3d.GUESS_ZERO), ("previous", o3d.GUESS_PREVIOUS),
                   ("extrapolated", o3d.GUESS_EXTRAPOLATED)]
    if weights and os.path.exists(weights):
        all_guesses.append(("learned", o3d.GUESS_LEARNED))
    guesses = [gg for gg in all_guesses if guesses is None or gg[0] in guesses]
    for name, g in guesses:
        p = o3d.tgv_params(n, re=re, precision=precision, solver=o3d.SOLVER_MG, eps=1e-8, kmax=100, guess=g,
                           **(cycle or {}))
        warmup = max(warmup, int(round(t0 / p.dt)))
        with o3d.Context(p) as ctx:
            net = None
            if g == o3d.GUESS_LEARNED:
                net = load(weights, ctx.guess_grid())
                ctx.attach_unet(net)
            ux, uy, uz, pp = o3d.tgv_fields(p)
            du = _perturbation(ux.shape, seed, amp)
            for nm, f in zip(("ux", "uy", "uz"), (ux + du[0], uy + du[1], uz + du[2])):
                ctx.upload(nm, np.asfortranarray(f))
            ctx.upload("pp", pp)
            cyc, pms, sms = [], [], []
            for it in range(1, warmup + steps + 1):
                info = ctx.step(it)
                if it > warmup:
                    cyc.append(info.poisson_cycles)
                    pms.append(info.poisson_ms)
                    sms.append(info.step_ms)
            results[name] = {"vcycles_per_step": float(np.mean(cyc)), "poisson_ms": float(np.mean(pms)),
                             "step_ms": float(np.mean(sms)), "t_first": (warmup + 1) * p.dt}
            if net:
                results[name]["inference_ms"] = inference_ms(net)
                results[name]["grid"] = list(net.dims)
                ctx.attach_unet(None)
                net.close()
    return results


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd")
    t = sub.add_parser("train")
    t.add_argument("--n", type=int, default=128)
    t.add_argument("--runs", type=int, default=8)
    t.add_argument("--steps", type=int, default=150)
    t.add_argument("--epochs", type=int, default=6)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--out", default=WEIGHTS)
    e = sub.add_parser("eval")
    e.add_argument("--n", type=int, default=256)
    e.add_argument("--steps", type=int, default=10)
    e.add_argument("--weights", default=WEIGHTS)
    e.add_argument("--t0", type=float, default=0.0, help="time at which the measured steps start")
    e.add_argument("--pre", type=int, default=0)
    e.add_argument("--post", type=int, default=0)
    e.add_argument("--omega", type=float, default=0.0)
    e.add_argument("--amp", type=float, default=0.02, help="initial perturbation amplitude")
    e.add_argument("--guesses", default="", help="comma-separated subset of zero,previous,extrapolated,learned")
    args = ap.parse_args()
    if args.cmd == "train":
        t0 = time.time()
        feat, tgt, dims = generate(args.n, args.runs, args.steps)
        print(f"samples {feat.shape[0]} on {dims} in {time.time() - t0:.1f} s", flush=True)
        net = o3d.UNet(dims, periodic=(1, 1, 1), base=16, levels=4, seed=1234)
        t1 = time.time()
        hist = train(net, feat, tgt, args.epochs, args.lr, log=lambda s: print(s, flush=True))
        print(f"training {time.time() - t1:.1f} s, loss {hist[0]:.4e} -> {hist[-1]:.4e}", flush=True)
        save(net, args.out)
    elif args.cmd == "eval":
        cyc = {k: v for k, v in (("mg_pre", args.pre), ("mg_post", args.post), ("mg_omega", args.omega)) if v}
        sel = [x for x in args.guesses.split(",") if x] or None
        res = compare_guesses(args.n, args.steps, 3, args.weights, t0=args.t0, cycle=cyc, guesses=sel, amp=args.amp)
        print(json.dumps({"n": args.n, "t0": args.t0, "cycle": cyc, "amp": args.amp, "guesses": res}))


if __name__ == "__main__":
    main()
