"""Train the learned-initial-guess network on stamps rendered by this library and save it.

    python -m astrophot_gb300.train_cnn --stamps 48000000 --out astrophot_gb300/weights/init_cnn.npz

Each stamp is rendered once (``ap_render``), given noise and used for one Adam step; the
held-out loss is reported on stamps of a seed the training never draws.  The committed
weights file is the output of this command with its defaults.
"""

from __future__ import annotations

import argparse
import json
import time

import torch

from . import cnn


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--stamps", type=int, default=48_000_000)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--chunk", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=cnn.WEIGHTS_PATH)
    ap.add_argument("--log-every", type=int, default=16)
    args = ap.parse_args(argv)

    net = cnn.InitNet(seed=args.seed)
    held = cnn.make_stamps(4096, seed=987654321)
    before = net.loss(held, 4096)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.train(n_stamps=args.stamps, batch=args.batch, chunk=args.chunk, lr=args.lr, seed=args.seed,
              log_every=args.log_every)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    held = cnn.make_stamps(4096, seed=987654321)
    after = net.loss(held, 4096)
    net.save(args.out)
    print(json.dumps({"stamps": args.stamps, "seconds": round(dt, 2), "stamps_per_s": round(args.stamps / dt, 1),
                      "held_out_loss_before": before, "held_out_loss_after": after, "out": args.out}))


if __name__ == "__main__":
    main()
