"""Trains the learned denoiser on image pairs that the path tracer renders
itself: for each seeded view (scenes.training_views), a converged target
and noisy renders at 1 to 256 samples per pixel with an independent
sample stream. Training runs on the GPU through the library's own
forward, backward and Adam kernels (raymond_net_train_step); PyTorch only
holds the device memory and cuts the random crops.

    python -m raymond_gb300.train_denoiser --views 160 --steps 4000 --out weights.npz

Each --loss variant (w_log,w_rel: the weights of the L1 log-radiance and
the relative squared-radiance terms) trains from the same initial weights on
the same data; the one with the lowest held-out RMSE at 4 spp is saved.
The report (--report) gives, for held-out views at 1, 4 and 16 spp, the
RMSE against the converged render of the noisy image, of the à-trous
filter and of the network."""

from __future__ import annotations

import argparse
import json
import math
import os
import shlex
import sys
import time

import numpy as np

from . import _native, scenes
from .denoiser import DEFAULT_WEIGHTS, Denoiser, make_batch
from .renderer import Canvas, Renderer

NOISY_SPP = (1, 2, 4, 8, 16, 32, 64, 128, 256)
NOISE_SEED = 0x5BD1E995


def rmse(a, b) -> float:
    """Root mean square RGB difference (the reference's rmse)."""
    d = np.asarray(a, np.float64)[..., :3] - np.asarray(b, np.float64)[..., :3]
    return float(np.sqrt(np.mean(d * d)))


def render_view(scene, camera, size, target_spp, bounces=8):
    """(target mean radiance, [(spp, accum, albedo, normal) sums at each of NOISY_SPP])."""
    canvas = Canvas(size, size)
    ref = Renderer.create(canvas)
    ref.scene, ref.camera = scene, camera
    ref.maxBounces = bounces
    ref.denoise = False
    ref.caustics = False
    per_frame = min(64, target_spp)
    ref.samplesPerFrame = per_frame
    for _ in range(target_spp // per_frame):
        ref.render()
    target = ref.readPixels().reshape(size, size, 4)
    ref.dispose()

    noisy = Renderer.create(canvas, seed=NOISE_SEED)
    noisy.scene, noisy.camera = scene, camera
    noisy.maxBounces = bounces
    noisy.denoise = False
    noisy.caustics = False
    out = []
    for spp in NOISY_SPP:
        # frames of at most 64 samples (samplesPerFrame's range), up to spp in all
        while noisy.samples < spp:
            noisy.samplesPerFrame = min(64, spp - noisy.samples)
            noisy.render()
        a, g, n = noisy.readGuides()
        out.append((noisy.samples, a, g, n))
    noisy.dispose()
    return target, out


def build_dataset(views, size, target_spp, log=print):
    t0 = time.time()
    targets, inputs = [], []
    for k, (scene, camera, info) in enumerate(views):
        target, noisy = render_view(scene, camera, size, target_spp)
        targets.append(target)
        inputs.append(noisy)
        if (k + 1) % 16 == 0:
            log(f"  rendered {k + 1}/{len(views)} views ({time.time() - t0:.1f} s)")
    return targets, inputs


def atrous(accum, albedo, normal, spp, torch):
    """The à-trous filter (raymond_denoise_static) on one noisy render."""
    h, w = accum.shape[:2]
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (accum, albedo, normal)]
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    _native.check(_native.lib().raymond_denoise_static(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), w, h,
                                                       spp, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def learned(net, accum, albedo, normal, spp, torch):
    h, w = accum.shape[:2]
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda()[None] for x in (accum, albedo, normal)]
    out = torch.empty((1, h, w, 4), dtype=torch.float32, device="cuda")
    net.infer(make_batch(*dev, samples_all=float(spp)), out)
    net.sync()
    return out[0].cpu().numpy()


def evaluate(net, targets, inputs, spp=4):
    import torch

    rows = []
    for target, noisy in zip(targets, inputs):
        s, a, g, n = next(x for x in noisy if x[0] == spp)
        rows.append({"noisy": rmse(a / s, target), "atrous": rmse(atrous(a, g, n, s, torch), target),
                     "learned": rmse(learned(net, a, g, n, s, torch), target)})
    mean = {k: float(np.mean([r[k] for r in rows])) for k in rows[0]}
    return mean, rows


def parse_losses(text):
    """Variants "w_log,w_rel[,rel_eps]" separated by ';'."""
    out = []
    for item in text.split(";"):
        vals = [float(v) for v in item.split(",")]
        out.append((vals[0], vals[1], vals[2] if len(vals) > 2 else 0.01))
    return out


def train(net, targets, inputs, steps, batch, crop, lr, seed=1, log=print):
    import torch

    rng = np.random.default_rng(seed)
    levels = len(NOISY_SPP)
    # The crops are cut on a torch stream and the network runs on the same
    # one, so each step reads finished crops and torch's allocator reuses
    # their memory only after the step.
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    net.use_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        out = _train_loop(net, targets, inputs, steps, batch, crop, lr, rng, levels, log, torch)
    net.sync()
    net.use_stream(None)
    return out


def _train_loop(net, targets, inputs, steps, batch, crop, lr, rng, levels, log, torch):
    acc = torch.from_numpy(np.stack([[x[1] for x in v] for v in inputs])).cuda()  # [V, L, H, W, 4]
    alb = torch.from_numpy(np.stack([[x[2] for x in v] for v in inputs])).cuda()
    nrm = torch.from_numpy(np.stack([[x[3] for x in v] for v in inputs])).cuda()
    tgt = torch.from_numpy(np.stack(targets)).cuda()  # [V, H, W, 4]
    spp = torch.tensor(NOISY_SPP, dtype=torch.float32, device="cuda")
    V, size = acc.shape[0], acc.shape[2]
    losses = []
    # Divergence guard: the parameters of the best 1,000-step window of the
    # logged loss are kept, and restored if the last window ends more than
    # twice as high (a long run at a high rate has collapsed into a pass-
    # through: blend weight 0 everywhere).
    window, best = [], (math.inf, None, -1)
    t0 = time.time()
    for step in range(steps):
        vi = torch.from_numpy(rng.integers(0, V, batch)).cuda()
        li = torch.from_numpy(rng.integers(0, levels, batch)).cuda()
        y0, x0 = (int(v) for v in rng.integers(0, size - crop + 1, 2))
        sl = (slice(y0, y0 + crop), slice(x0, x0 + crop))
        a = acc[vi, li][:, sl[0], sl[1]]
        g = alb[vi, li][:, sl[0], sl[1]]
        n = nrm[vi, li][:, sl[0], sl[1]]
        t = tgt[vi][:, sl[0], sl[1]]
        flip = rng.integers(0, 4)
        if flip & 1:
            a, g, n, t = (z.flip(2) for z in (a, g, n, t))
        if flip & 2:
            a, g, n, t = (z.flip(1) for z in (a, g, n, t))
        a, g, n, t = (z.contiguous() for z in (a, g, n, t))
        s = spp[li].contiguous()
        warm = min(1.0, (step + 1) / 100.0)
        rate = lr * warm * (0.02 + 0.98 * 0.5 * (1.0 + math.cos(math.pi * step / steps)))
        want = step % 100 == 0 or step == steps - 1
        loss = net.train_step(make_batch(a, g, n, t, samples=s), rate, want_loss=want)
        if want:
            losses.append((step, loss))
            log(f"  step {step:5d}  loss {loss:.4f}  lr {rate:.2e}  {time.time() - t0:.1f} s")
            window.append(loss)
            if len(window) == 10:
                mean = float(np.mean(window))
                if mean < best[0]:
                    best = (mean, net.get_params(), step)
                window = []
    net.sync()
    tail = float(np.mean([v for _, v in losses[-10:]])) if losses else math.inf
    if best[1] is not None and tail > 2.0 * best[0]:
        log(f"  loss ended at {tail:.4f}, twice the best window's {best[0]:.4f}: restoring step {best[2]}")
        net.set_params(best[1])
        losses.append(("restored", best[2]))
    return losses, time.time() - t0


def choose_tau(net, targets, inputs, eval_spp, taus, log):
    """Held-out scores (mean learned/noisy error ratio over eval_spp) for each
    display guard τ, and the best τ."""
    scores = {}
    for tau in (float(v) for v in taus.split(",")):
        net.blend = tau
        ratios = []
        for spp in eval_spp:
            mean, _ = evaluate(net, targets, inputs, spp)
            ratios.append(mean["learned"] / mean["noisy"])
        scores[str(tau)] = {"score": float(np.mean(ratios)), "ratios": dict(zip(map(str, eval_spp), ratios))}
        log(f"tau {tau}: {scores[str(tau)]}")
    best = min(scores, key=lambda k: scores[k]["score"])
    return scores, float(best)


def tune_only(args, argv, log):
    """Held-out evaluation of saved weights at each --tau, the best τ saved
    with them (the held-out views are the training run's: the same seeded
    list, after its --views)."""
    field_spheres = tuple(int(v) for v in args.field_spheres.split(","))
    field_frequency = tuple(int(v) for v in args.field_frequency.split(","))
    views = scenes.training_views(args.views + args.holdout, seed=args.seed, spheres=field_spheres,
                                  frequency=field_frequency)
    h_targets, h_inputs = build_dataset(views[args.views:], args.size, args.target_spp, log)
    eval_spp = [int(v) for v in args.eval_spp.split(",")]
    net = Denoiser(weights=args.weights)
    scores, tau = choose_tau(net, h_targets, h_inputs, eval_spp, args.tau or str(net.blend), log)
    net.blend = tau
    net.save(args.out)
    net.dispose()
    report = {"command": "python -m raymond_gb300.train_denoiser " + shlex.join(argv if argv is not None else sys.argv[1:]),
              "tau_scores": scores, "tau": tau}
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    return report


def main(argv=None):
    global NOISY_SPP
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--views", type=int, default=160)
    ap.add_argument("--holdout", type=int, default=8)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--target-spp", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--loss", default="0.5,1", help="variants w_log,w_rel[,rel_eps] separated by ';'")
    ap.add_argument("--eval-spp", default="1,4,16", help="held-out evaluation sample counts")
    ap.add_argument("--noisy-spp", default=",".join(str(v) for v in NOISY_SPP),
                    help="sample counts of the noisy inputs (increasing)")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--field-spheres", default="300,3000", help="sphere-field views: spheres, min,max")
    ap.add_argument("--field-frequency", default="10,55", help="sphere-field views: centre-mesh frequency, min,max")
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--report", default=None)
    ap.add_argument("--tau", default=None,
                    help="display guards τ to try on the held-out views after training (comma-separated); "
                         "the one with the lowest mean learned/noisy error ratio is saved with the weights")
    ap.add_argument("--weights", default=None,
                    help="skip training: load these weights and only evaluate (and choose τ) on the held-out views")
    args = ap.parse_args(argv)
    NOISY_SPP = tuple(int(v) for v in args.noisy_spp.split(","))

    def log(msg):
        print(msg, flush=True)

    if args.weights:
        return tune_only(args, argv, log)
    t0 = time.time()
    field_spheres = tuple(int(v) for v in args.field_spheres.split(","))
    field_frequency = tuple(int(v) for v in args.field_frequency.split(","))
    views = scenes.training_views(args.views + args.holdout, seed=args.seed, spheres=field_spheres,
                                  frequency=field_frequency)
    train_views, held = views[:args.views], views[args.views:]
    log(f"{len(train_views)} training views, {len(held)} held out; {args.size}² at {args.target_spp} spp")
    targets, inputs = build_dataset(train_views, args.size, args.target_spp, log)
    h_targets, h_inputs = build_dataset(held, args.size, args.target_spp, log)
    t_data = time.time() - t0
    variants = []
    best = None
    eval_spp = [int(v) for v in args.eval_spp.split(",")]
    for w_log, w_rel, rel_eps in parse_losses(args.loss):
        net = Denoiser(seed=args.seed)
        net.set_loss(w_log, w_rel, rel_eps)
        log(f"loss variant w_log={w_log} w_rel={w_rel} rel_eps={rel_eps}")
        losses, t_train = train(net, targets, inputs, args.steps, args.batch, args.crop, args.lr, seed=args.seed,
                                log=log)
        result = {"w_log": w_log, "w_rel": w_rel, "rel_eps": rel_eps, "seconds_train": t_train, "loss": losses}
        for spp in eval_spp:
            result[f"holdout_rmse_{spp}spp"], rows = evaluate(net, h_targets, h_inputs, spp)
            if spp == 4:
                result["holdout_rows_4spp"] = rows
        log(json.dumps({k: v for k, v in result.items() if k.startswith("holdout_rmse") or k in ("w_log", "w_rel",
                                                                                                "rel_eps")}))
        variants.append(result)
        # chosen: the lowest mean ratio of learned to noisy error over the evaluated sample counts
        score = float(np.mean([result[f"holdout_rmse_{spp}spp"]["learned"] / result[f"holdout_rmse_{spp}spp"]["noisy"]
                               for spp in eval_spp]))
        result["score"] = score
        if best is None or score < best[0]:
            if best is not None:
                best[1].dispose()
            best = (score, net, result)
        else:
            net.dispose()
    if args.tau:
        best[2]["tau_scores"], tau = choose_tau(best[1], h_targets, h_inputs, eval_spp, args.tau, log)
        best[1].blend = tau
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    best[1].save(args.out)
    report = {"command": "python -m raymond_gb300.train_denoiser " + shlex.join(argv if argv is not None else sys.argv[1:]),
              "views": args.views, "holdout": args.holdout, "size": args.size, "target_spp": args.target_spp,
              "noisy_spp": list(NOISY_SPP), "steps": args.steps, "batch": args.batch, "crop": args.crop,
              "lr": args.lr, "seed": args.seed, "field_spheres": list(field_spheres),
              "field_frequency": list(field_frequency), "seconds_data": t_data, "variants": variants,
              "eval_spp": eval_spp,
              "chosen": {"w_log": best[2]["w_log"], "w_rel": best[2]["w_rel"], "rel_eps": best[2]["rel_eps"]},
              "weights": os.path.basename(args.out)}
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
