"""Train the denoiser on the GPU with the library's own kernels.

    python -m pt_gb300.train_denoiser [--scenes 128] [--steps 2000] [--out pt_gb300/weights/unet.bin]

1. For each seeded procedural scene (pt_gb300.trainset), the tracer renders
   a target (FP64 accumulation, --target-spp samples) and inputs at several
   low sample counts, each packed with its first-hit features into the
   16-channel bf16 network input and an FP32 residual base (log(1 + noisy
   radiance)).  Everything stays on the device.
2. The U-Net trains on random batches with Adam (lr 1e-3, cosine decay),
   using the library's BF16 tensor-core forward and backward passes.
3. Held-out scenes report the MSE of the noisy input and of the denoised
   output against their targets, per sample count.

With --checkpoint PATH the parameters, Adam state, step and batch sampler
RNG are saved every --checkpoint-every steps; a run started again with the
same PATH and --resume continues from the last save (the training set is
re-rendered, bit-identically, from its seeds).
"""
from __future__ import annotations

import argparse
import json
import math
import time
from pathlib import Path

import numpy as np

from . import abi
from .core import Context, HostScene
from .denoise import WEIGHTS_DIR, UNet, init_params, save_params
from . import checkpoint, trainset


def render_set(ctx, seeds, size, target_spp, input_spps):
    """Returns (inputs [len(seeds) * len(input_spps), size, size, 16] bf16,
    residual bases [same, 4] fp32, targets [len(seeds), size, size, 4] fp32,
    noisy images [same as inputs, 4] fp32).  Bounce limit and Russian
    roulette per scene from trainset.render_settings."""
    import torch

    k = len(input_spps)
    X = torch.empty((len(seeds) * k, size, size, 16), dtype=torch.bfloat16, device="cuda")
    B = torch.empty((len(seeds) * k, size, size, 4), dtype=torch.float32, device="cuda")
    N = torch.empty((len(seeds) * k, size, size, 4), dtype=torch.float32, device="cuda")
    Y = torch.empty((len(seeds), size, size, 4), dtype=torch.float32, device="cuda")
    for i, seed in enumerate(seeds):
        raw, cam = trainset.training_scene(seed)
        hs = HostScene.from_raw(raw, cam)
        ctx.upload(hs.pack())
        ctx.build_accel()
        bounces, rr = trainset.render_settings(seed)
        ctx.render(hs.render_params(size, size, target_spp, bounces, rr_start=rr, accum_mode=abi.PT_ACCUM_FP32_FP64),
                   stats=False)
        y = ctx.read_image(fp64=True).astype(np.float32)
        y[..., 3] = 1.0
        Y[i].copy_(torch.from_numpy(y))
        for j, spp in enumerate(input_spps):
            ctx.render_noisy(hs.render_params(size, size, spp, bounces, rr_start=rr))
            ctx.denoise_input(spp, X[i * k + j].data_ptr(), B[i * k + j].data_ptr())
            N[i * k + j].copy_(torch.from_numpy(ctx.read_image()))
    torch.cuda.synchronize()
    return X, B, Y, N


def mse(a, b) -> float:
    """meansq of the reference (util/meansq/meansq.cpp:34-43): RGB, n - 1."""
    d = (a[..., :3].double() - b[..., :3].double())
    return float((d * d).sum() / (d.numel() - 1))


def evaluate(net_eval, X, B, Y, N, k, input_spps):
    import torch

    out = {}
    for j, spp in enumerate(input_spps):
        m_noisy, m_den = [], []
        for i in range(Y.shape[0]):
            net_eval.input_tensor().copy_(X[i * k + j:i * k + j + 1])
            net_eval.base_tensor().copy_(B[i * k + j:i * k + j + 1])
            net_eval.forward()
            o = net_eval.output_tensor()[..., :3].float()
            den = torch.expm1(torch.clamp(o, min=0.0))
            m_noisy.append(mse(N[i * k + j], Y[i]))
            m_den.append(mse(den[0], Y[i]))
        out[spp] = {"noisy": float(np.mean(m_noisy)), "denoised": float(np.mean(m_den))}
    return out


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--scenes", type=int, default=128)
    ap.add_argument("--eval-scenes", type=int, default=8)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--target-spp", type=int, default=1024)
    ap.add_argument("--input-spp", type=str, default="2,4,8,16")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--init", type=str, default="", help="start from these parameters instead of a fresh init")
    ap.add_argument("--out", type=str, default=str(WEIGHTS_DIR / "unet.bin"))
    ap.add_argument("--checkpoint", type=str, default="", help="training checkpoint file (.npz)")
    ap.add_argument("--checkpoint-every", type=int, default=500)
    ap.add_argument("--resume", action="store_true", help="continue from --checkpoint when it exists")
    args = ap.parse_args(argv)
    spps = [int(s) for s in args.input_spp.split(",")]
    k = len(spps)
    torch.manual_seed(args.seed)
    ctx = Context(0)

    t0 = time.perf_counter()
    X, B, Y, N = render_set(ctx, range(1000, 1000 + args.scenes), args.size, args.target_spp, spps)
    Xe, Be, Ye, Ne = render_set(ctx, range(900000, 900000 + args.eval_scenes), args.size, args.target_spp, spps)
    t_data = time.perf_counter() - t0
    print(f"rendered {args.scenes} + {args.eval_scenes} scenes in {t_data:.1f} s", flush=True)

    net = UNet(args.batch, args.size, args.size)
    params = np.fromfile(args.init, dtype="<f4") if args.init else init_params(args.seed)
    net.set_params(params)
    tgt = torch.empty((args.batch, args.size, args.size, 4), dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cpu").manual_seed(args.seed)
    first = 0
    if args.resume and args.checkpoint and Path(args.checkpoint).exists():
        first, rng, _ = checkpoint.load_training(args.checkpoint, net)
        gen.set_state(torch.from_numpy(rng))
        print(f"resumed from {args.checkpoint} at step {first}", flush=True)
    losses = []
    t1 = time.perf_counter()
    for step in range(first, args.steps):
        idx = torch.randint(0, X.shape[0], (args.batch,), generator=gen)
        net.input_tensor().copy_(X[idx.cuda()])
        net.base_tensor().copy_(B[idx.cuda()])
        tgt.copy_(Y[(idx // k).cuda()])
        net.forward()
        losses.append(net.backward(tgt.data_ptr()))
        lr = 0.05 * args.lr + 0.95 * args.lr * 0.5 * (1 + math.cos(math.pi * step / max(1, args.steps)))
        net.adam(lr)
        if step % 100 == 0 or step == args.steps - 1:
            print(f"step {step:5d} loss {np.mean(losses[-100:]):.5f} lr {lr:.2e}", flush=True)
        if args.checkpoint and ((step + 1) % args.checkpoint_every == 0 or step == args.steps - 1):
            checkpoint.save_training(args.checkpoint, net, step + 1, gen.get_state(), {"seed": args.seed})
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    params = net.params()
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    save_params(out, params)

    ev = UNet(1, args.size, args.size)
    ev.set_params(params)
    res = evaluate(ev, Xe, Be, Ye, Ne, k, spps)
    summary = {"scenes": args.scenes, "size": args.size, "target_spp": args.target_spp, "input_spp": spps,
               "steps": args.steps, "batch": args.batch, "lr": args.lr, "data_seconds": round(t_data, 2),
               "train_seconds": round(t_train, 2),
               "ms_per_step": round(1000 * t_train / max(1, args.steps - first), 3),
               "final_loss": float(np.mean(losses[-100:])) if losses else None, "eval_mse": res}
    if first:
        summary["resumed_at_step"] = first
    out.with_suffix(".json").write_text(json.dumps(summary, indent=1) + "\n")
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
