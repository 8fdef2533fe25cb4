"""Train and evaluate the learned surrogate on pairs generated by the plain engine.

    python -m 21cmpy_gb300.Programs.train_surrogate [--n 128] [--box-len 200] [--train 2048]
        [--held 128] [--epochs 60] [--lr 3e-4] [--decay 0.95] [--out weights.pt] [--report report.json]
    python -m 21cmpy_gb300.Programs.train_surrogate --conv-only [--n 128]

Training pairs: Gaussian random fields of seeds 1000..(1000 + train - 1) at n^3 with parameter
points drawn uniformly (zeta in [10, 80], R_mfp in [5, 50] Mpc, log10 Tvir in [4, 5.3], z in
[6, 10]); labels are the plain engine's x_HI.  Evaluation: held-out seeds 5000.. against the plain
engine (mean |dx_HI|, flag agreement at x_HI = 0.5, P21(k) ratio on k in [0.1, 1] /Mpc), the
untrained network and the constant mean predictor, plus inference speed in boxes/s next to the
plain engine's, and a parameter sweep through SurrogateSweep (surrogate with engine fallback).
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np
import torch

from .. import surrogate as S


def main(argv=None):
    ap = argparse.ArgumentParser(prog="train_surrogate")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--box-len", type=float, default=200.0)
    ap.add_argument("--train", type=int, default=2048)
    ap.add_argument("--held", type=int, default=128)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--decay", type=float, default=0.95, help="step-size factor per epoch")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--smooth", default=",".join(f"{r:g}" for r in S.SMOOTH_CELLS),
                    help="radii (cells) of the smoothed input channels, comma-separated; empty for none")
    ap.add_argument("--out", default=None)
    ap.add_argument("--report", default=None)
    ap.add_argument("--conv-only", action="store_true",
                    help="time one 32 -> 32 channel 3^3 convolution layer at n^3 (2 + 3 launches) and exit")
    args = ap.parse_args(argv)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    if args.conv_only:
        return conv_only(args.n)

    gen = S.DataGenerator(n=args.n, box_len=args.box_len)
    rng = np.random.default_rng(args.seed)
    t0 = time.time()
    train = [gen.sample(1000 + i, S.draw_params(rng)) for i in range(args.train)]
    held_rng = np.random.default_rng(args.seed + 1)
    held = [gen.sample(5000 + i, S.draw_params(held_rng)) for i in range(args.held)]
    torch.cuda.synchronize()
    t_data = time.time() - t0
    log(f"generated {len(train)} + {len(held)} pairs in {t_data:.1f} s")

    smoothing = tuple(float(v) for v in args.smooth.split(",") if v.strip())
    net = S.SurrogateNet(seed=args.seed, smoothing=smoothing)
    untrained = S.evaluate(net, held, gen.plan)
    order_rng = np.random.default_rng(args.seed + 2)
    t0 = time.time()
    losses = []
    for ep in range(args.epochs):
        perm = order_rng.permutation(len(train))
        losses.extend(S.train(net, [train[i] for i in perm], epochs=1, lr=args.lr * (args.decay ** ep),
                              log=lambda m, ep=ep: log(m.replace("epoch 0:", f"epoch {ep}:", 1))))
    torch.cuda.synchronize()
    t_train = time.time() - t0
    trained = S.evaluate(net, held, gen.plan)
    mean_pred = float(np.mean([s.xH.mean().item() for s in train]))
    const_err = float(np.mean([(s.xH - mean_pred).abs().mean().item() for s in held]))

    # inference speed next to the plain engine (inputs resident on the device)
    s = held[0]
    f = net.features(s.delta, s.z, s.zeta, s.R_max, s.t_vir)
    st = S.schedule.ionize_setup(gen.n, gen.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir, R_max=s.R_max,
                                 cosmo=gen.cosmo, table=gen.table)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def best_ms(fn, rounds=3, reps=10):
        """Fastest of a few timed rounds (both sides alike), after warm-up."""
        for _ in range(3):
            fn()
        times = []
        for _ in range(rounds):
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / reps)
        return min(times)

    sg_ms = best_ms(lambda: net.forward(f))
    sg_in_ms = best_ms(lambda: net.forward(net.features(s.delta, s.z, s.zeta, s.R_max, s.t_vir)))
    eng_ms = best_ms(lambda: gen.plan.run(s.delta, st))
    from ..autotune import cached as tuned_config
    flop = 2 * gen.n ** 3 * sum(27 * ci * co for ci, co in S.LAYERS)

    sweep = S.SurrogateSweep(net, gen, max_abs_err=0.05, check_every=8)
    kinds = [sweep(x.delta, dict(z=x.z, zeta=x.zeta, R_max=x.R_max, t_vir=x.t_vir))[1] for x in held]
    report = {
        "n": gen.n, "box_len_mpc": gen.box_len, "train_pairs": len(train), "held_out": len(held),
        "epochs": args.epochs, "data_seconds": t_data, "train_seconds": t_train,
        "final_bce": float(np.mean(losses[-len(train):])) if losses else None,
        "trained": trained, "untrained": untrained, "constant_mean_abs_dxHI": const_err,
        "smoothing_cells": list(smoothing),
        "surrogate_ms_per_box": sg_ms, "surrogate_boxes_per_s": 1e3 / sg_ms,
        "surrogate_with_features_ms_per_box": sg_in_ms,
        "surrogate_tflops": flop / sg_ms / 1e9,
        "engine_ms_per_box": eng_ms, "engine_boxes_per_s": 1e3 / eng_ms, "engine_radii": st.n_radii,
        "engine_config": tuned_config(gen.plan.device, gen.n),
        "speed_ratio_surrogate_over_engine": eng_ms / sg_ms,
        "sweep": {"points": len(kinds), "surrogate": kinds.count("surrogate"), "engine": kinds.count("engine")},
    }
    print(json.dumps(report), flush=True)
    if args.report:
        with open(args.report, "w") as fh:
            json.dump(report, fh, indent=1)
    if args.out:
        torch.save(net.state(), args.out)
    return 0


def conv_only(n: int) -> int:
    """One 32 -> 32 channel layer on random BF16 activations: two warm-up launches, then three timed
    ones; prints us / launch."""
    net = S.SurrogateNet(seed=0)
    g = torch.Generator(device=net.device).manual_seed(1)
    x = torch.randn((n, n, n, 32), device=net.device, generator=g).to(torch.bfloat16)
    w = (torch.randn((27, 32, 32), device=net.device, generator=g) * 0.1).to(torch.bfloat16)
    b = torch.zeros(32, device=net.device)
    out = torch.empty_like(x)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        net._conv(n, 32, 32, 0, x, w, b, out)
    e0.record()
    for _ in range(3):
        net._conv(n, 32, 32, 0, x, w, b, out)
    e1.record()
    e1.synchronize()
    net.check()
    us = e0.elapsed_time(e1) / 3 * 1e3
    print(json.dumps({"n": n, "layer": "32->32", "us_per_launch": us,
                      "tflops": 2 * n ** 3 * 27 * 32 * 32 / us / 1e6}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
