"""Train and evaluate the FNO surrogate on its workload, all on one GPU.

    python -m litho_gb300.train_surrogate --out DIR [--train 20000 --eval 2000 ...]

1. Optics: quasar source (~2000 lit points), NA 0.8, 193 nm, in focus, 256 x 256
   masks -> FP64 TCC and FP64 eigensolve on the GPU -> K = 24 SOCS kernels.
2. Pairs: seeded rectangle masks (litho_rect_masks) imaged by the plain GPU SOCS
   path; disjoint seeds for the training, calibration and held-out sets.
3. Training: Adam (lr step-decayed), mini-batches from the device-resident set,
   forward/backward/update by the library's own kernels.
4. Calibration: alpha of the error estimate = the `coverage` quantile of
   (true error / raw estimate) on the calibration set.
5. Held-out evaluation: litho_surrogate_image with the threshold; SOCS images of
   every held-out mask judge the returned images.  Throughput of plain SOCS, of
   the network path and of the whole surrogate-with-fallback path is measured
   with CUDA events on the same stream.
Writes DIR/surrogate_report.json and DIR/surrogate_params.npy.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np


def _events_ms(fn, reps: int):
    import torch
    st = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        fn()
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def main(argv=None):
    import torch

    import litho_gb300 as LG
    from litho_gb300 import surrogate as S

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--calib", type=int, default=1000)
    ap.add_argument("--eval", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--decay-every", type=int, default=15)
    ap.add_argument("--threshold", type=float, default=1e-2)
    ap.add_argument("--coverage", type=float, default=0.99)
    ap.add_argument("--seed", type=int, default=2026)
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    ctx = LG.Context(0)
    ks, info = S.c5_kernel_set(ctx)
    L = S.C5["L"]
    rep = {"optics": {k: v for k, v in info.items() if k not in ("krn", "scales")}, "args": vars(a)}
    t0 = time.time()
    tm, ti = S.make_pairs(ctx, ks, seed=a.seed, first=0, count=a.train, L=L)
    cm, ci = S.make_pairs(ctx, ks, seed=a.seed + 1, first=0, count=a.calib, L=L)
    em, ei = S.make_pairs(ctx, ks, seed=a.seed + 2, first=0, count=a.eval, L=L)
    torch.cuda.synchronize()
    rep["pairs_s"] = time.time() - t0

    model = S.Surrogate(ctx, L=L, seed=a.seed)
    t0 = time.time()
    hist = S.train(model, tm, ti, epochs=a.epochs, batch=a.batch, lr=a.lr, decay_every=a.decay_every,
                   seed=a.seed, log=lambda s: print(s, flush=True))
    torch.cuda.synchronize()
    rep["train_s"] = time.time() - t0
    rep["loss_history"] = hist
    del tm, ti

    # calibration of the estimate
    model.set_alpha(1.0)
    raw_err, raw_est = [], []
    for s0 in range(0, a.calib, 256):
        img, est = model.predict(ks, cm[s0:s0 + 256])
        raw_err.append(S.rel_l2_per_image(img, ci[s0:s0 + 256]).cpu().numpy())
        raw_est.append(est.cpu().numpy())
    raw_err, raw_est = np.concatenate(raw_err), np.concatenate(raw_est)
    alpha = float(np.quantile(raw_err / raw_est, a.coverage))
    model.set_alpha(alpha)
    rep["alpha"] = alpha
    rep["calib_err_quantiles"] = np.quantile(raw_err, [0.5, 0.9, 0.99, 1.0]).tolist()

    # held-out evaluation against SOCS images
    errs, ests, used = [], [], []
    for s0 in range(0, a.eval, 256):
        img, est, u = model.image(ks, em[s0:s0 + 256], a.threshold)
        errs.append(S.rel_l2_per_image(img, ei[s0:s0 + 256]).cpu().numpy())
        ests.append(est)
        used.append(u)
    errs, ests, used = np.concatenate(errs), np.concatenate(ests), np.concatenate(used)
    net_err = []
    for s0 in range(0, a.eval, 256):
        img, _ = model.predict(ks, em[s0:s0 + 256])
        net_err.append(S.rel_l2_per_image(img, ei[s0:s0 + 256]).cpu().numpy())
    net_err = np.concatenate(net_err)
    acc = ~used
    rep["eval"] = {
        "n": int(a.eval),
        "threshold": a.threshold,
        "accepted_fraction": float(acc.mean()),
        "network_err_quantiles": np.quantile(net_err, [0.5, 0.9, 0.99, 1.0]).tolist(),
        "network_err_below_threshold": float((net_err <= a.threshold).mean()),
        "accepted_err_max": float(errs[acc].max()) if acc.any() else None,
        "accepted_err_median": float(np.median(errs[acc])) if acc.any() else None,
        "false_accepts": int(((net_err > a.threshold) & acc).sum()),
        "returned_err_max": float(errs.max()),
        "spearman_est_vs_err": float(
            np.corrcoef(np.argsort(np.argsort(net_err)), np.argsort(np.argsort(ests)))[0, 1]),
    }

    # throughput at batch 256: plain SOCS, network path, surrogate with fallback
    B = 256
    mb = em[:B].contiguous()
    out = torch.empty_like(mb)

    def socs():
        with S.torch_stream(ctx):
            ctx.image_batch(ks, mb, out)

    t_socs = _events_ms(socs, 20)
    t_net = _events_ms(lambda: model.predict(ks, mb, out), 10)
    t_sur = _events_ms(lambda: model.image(ks, mb, a.threshold, out), 10)
    rep["throughput_img_s"] = {"plain_socs": B / t_socs * 1e3, "surrogate_network": B / t_net * 1e3,
                               "surrogate_with_fallback": B / t_sur * 1e3, "batch": B}
    rep["train_step_ms"] = _events_ms(lambda: model.train_step(mb[:a.batch].contiguous(), out[:a.batch].contiguous(),
                                                               1e-9, want_loss=False), 10)
    model.save(os.path.join(a.out, "surrogate_params.npy"))
    with open(os.path.join(a.out, "surrogate_report.json"), "w") as fh:
        json.dump(rep, fh, indent=1)
    print(json.dumps({k: v for k, v in rep.items() if k != "loss_history"}, indent=1))
    return rep


if __name__ == "__main__":
    main()
