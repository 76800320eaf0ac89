#!/usr/bin/env python
"""Aerial-image throughput of the SOCS path on GB300 (one JSON line on stdout).

Workload (one "step"): a batch of B seeded 1024x1024 float32 Manhattan masks
(line/space gratings and contact arrays, ~50 % density) imaged with K=24 fixed
SOCS kernels.  The kernels come from this library's own GPU TCC + FP64
eigensolver for a quasar source (4 poles at 45/135/225/315 deg, sigma 0.7-0.9,
~2000 lit points), NA 0.8, lambda 193 nm, defocus 0.  B=1024 masks are 4 GiB in
and 4 GiB out per step, far larger than the 129 MB L2, so no flush is needed.
Smaller steps pay a fixed per-step cost (the previous step's image writes still
dirty in L2, kernel ramps, tails and launch gaps) over fewer masks: 256 masks per
step run at ~0.9 of the 1024-mask throughput, 64 masks at ~0.75.

  value : images/s with masks resident in HBM (litho_image_batch on device
          pointers), timed with CUDA events over K steps on the library's stream.
  e2e   : images/s through the same C-ABI call with pinned host buffers
          (host->device copy of the masks and device->host copy of the images
          inside every step).
  roofline : the dominant kernel's algorithmic bytes per launch / its average
          launch time (CUDA events recorded by the library around each launch on
          the launching stream) vs the measured HBM copy bandwidth.
  cpu_baseline : the reference CPU algorithm (FT_r2c_padded + calcSOCS + FI in
          FP64, multi-threaded scipy port) on a bounded sample of the same masks,
          which also yields the GPU result's rel-L2 vs FP64.

--impl reference times that CPU port alone on all host cores (the reference's
own CPU implementation of the path cannot travel to the GPU host: it is built
from the reference checkout with a project-written FFTW shim).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fpga-litho-accel_gb300"))

METRIC = "aerial images/s at 1024^2 K=24: mixed/batched/surrogate vs plain GPU at stated rel-L2"
L_SIZE, K_KERNELS, NA, WAVELENGTH, DEFOCUS = 1024, 24, 0.8, 193.0, 0.0
# DRAM bytes (read + write) per mask of the mixed form's two HBM-bound kernels, from an
# ncu capture of one launch of each on 48 masks of this workload (the traffic scales with
# the masks).  The FI kernel's figure is what DRAM saw during its launch: part of its
# image writes is still in L2 when it ends and drains during the next launch.
TRAFFIC_PER_IMAGE = {("mixed", "win_dft"): (201.65e6 + 3.31e6) / 48,
                     ("mixed", "fi_out"): (13.07e6 + 140.29e6) / 48}
TRAFFIC_KERNEL = {"win_dft": "win_dft_tc", "fi_out": "fi_tc"}
WORKLOAD = ("1024x1024 float32 Manhattan masks (L/S + contacts, ~50% density), K=24 SOCS kernels from a "
            "~2000-point quasar source (sigma 0.7-0.9), NA 0.8, 193 nm; fixed kernels, batch of masks per step")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--batch", type=int, default=1024)
    p.add_argument("--cpu-budget-s", type=float, default=12.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--precision", default="auto", choices=["auto", "fp32", "mixed"])
    p.add_argument("--no-surrogate", action="store_true")
    p.add_argument("--no-large-tcc", action="store_true")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--profile-tcc", action="store_true",
                   help="the large-TCC workload's GPU stages only (split-BF16 TCC twice, FP64 TCC, top-48 FP64 "
                        "eigensolve), for ncu captures")
    p.add_argument("--profile-batched", action="store_true",
                   help="the batched workload only (plan creation with its autotuning, then --steps graph launches "
                        "per form), for ncu captures")
    p.add_argument("--profile-surrogate", action="store_true",
                   help="the surrogate's kernels only (forward passes, predictions with the error estimate and "
                        "Adam steps on seeded 256^2 masks, --batch masks), for ncu captures")
    p.add_argument("--profile", action="store_true",
                   help="warm-up + timed steps of both forms only (no clock sampling, e2e, CPU or surrogate legs)")
    p.add_argument("--surrogate-epochs", type=int, default=10)
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(dist, x, device):
    """The largest x over all ranks (every rank passes its own); x itself without a
    process group.  A step's time is the slowest rank's."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_images_per_s(world, batch, steps, seconds):
    """Whole-job throughput: every rank images its own batch per step (weak scaling,
    replicas), over the slowest rank's time."""
    return world * batch * steps / seconds


def load_synth():
    """The seeded mask and source generators (litho_gb300/synth.py, numpy only), loaded by
    file path so that the package's __init__ -- which maps liblitho_gb300.so -- does not run:
    the reference arm must not load the product library."""
    import importlib.util
    path = os.path.join(ROOT, "fpga-litho-accel_gb300", "litho_gb300", "synth.py")
    spec = importlib.util.spec_from_file_location("litho_bench_synth", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_masks(n, seed0=100):
    import numpy as np
    synth = load_synth()
    base = [synth.manhattan_mask(L_SIZE, seed=seed0 + i) for i in range(min(n, 8))]
    return np.stack([base[i % len(base)] for i in range(n)])


def grey_levels(masks):
    """8-bit grey-level versions of binary masks (device tensor in, device tensor out): pattern
    pixels at levels 200-255, background at 0-55, divided by 255 as the reference's PNG masks are."""
    import torch
    g = torch.Generator(device=masks.device)
    g.manual_seed(7)
    lv = torch.randint(0, 56, masks.shape, generator=g, device=masks.device, dtype=torch.int32)
    return ((masks * 200.0 + lv.float()) / 255.0).to(torch.float32)


def bench_config(nx, npts, batch, form):
    """The workload's config, identical in both arms' lines."""
    gib = batch * 4 * L_SIZE * L_SIZE / 2 ** 30
    return {"workload": WORKLOAD, "L": L_SIZE, "K": K_KERNELS, "Nx": nx, "source_points": npts,
            "batch_per_step": batch, "form": form,
            "forms": "mixed = split-BF16 tcgen05 TCC + FP64 eigensolve + split-TF32 tcgen05 DFTs; "
                     "plain = FP64 TCC + FP64 eigensolve + FP32 CUDA-core DFTs; both FP32 FFTs",
            "l2": f"inputs larger than L2 ({gib:g} GiB in + {gib:g} GiB out per step), no flush"}


class Clocks:
    """nvidia-smi sampling during the timed region (read-only queries)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"litho_bench_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def setup_kernels(ctx):
    """Kernels of both forms from this library's GPU path for the quasar source:
    plain = FP64 TCC + FP64 eigensolve; mixed = split-BF16 tensor-core TCC + FP64 eigensolve."""
    import litho_gb300 as L
    from litho_gb300 import synth
    src, S, npts = synth.quasar_source(2000)
    sig = L.outer_sigma(src)
    nx = L.optics_n(NA, L_SIZE, sig, WAVELENGTH)
    out = {"src": src, "sigma": sig, "nx": nx, "npts": npts}
    for form, prec in (("plain", L.TCC_FP64), ("mixed", L.TCC_SPLIT_BF16)):
        tcc = ctx.calc_tcc(src, sig, WAVELENGTH, NA, DEFOCUS, L_SIZE, L_SIZE, nx, nx, precision=prec)
        krn, s32, s64 = ctx.calc_kernels(tcc, K_KERNELS)
        out[form] = {"tcc": tcc, "krn": krn, "s32": s32, "s64": s64}
    return out


def cpu_leg(setup, masks_h, gpu_images, budget):
    """The reference CPU algorithm (FP64) on a bounded sample: timing, and the
    GPU forms' errors vs FP64 for TCC, scales, kernels (per-cluster projectors) and image."""
    import numpy as np
    from oracle import cpu_socs
    from oracle import np_ref as R
    nx = setup["nx"]
    tcc = R.calc_tcc(setup["src"], setup["sigma"], WAVELENGTH, NA, DEFOCUS, L_SIZE, L_SIZE, nx, nx)
    krn, s32, w64 = R.calc_kernels(tcc, K_KERNELS)
    ips, n, el, ref = cpu_socs.time_images(masks_h, krn, s32, nx, nx, budget_s=budget)
    w_all = np.linalg.eigvalsh(tcc)[::-1]
    err = {}
    for form, imgs in gpu_images.items():
        f = setup[form]
        proj = 0.0
        i = 0
        while i < K_KERNELS:   # clusters of (near-)equal eigenvalues inside the kept set
            j = i + 1
            while j < len(w_all) and abs(w_all[j - 1] - w_all[j]) <= 1e-6 * w_all[0]:
                j += 1
            if j <= K_KERNELS:
                a, b = f["krn"][i:j].T, krn[i:j].T
                proj = max(proj, float(np.linalg.norm(a @ a.conj().T - b @ b.conj().T)))
            i = j
        err[form] = {"image": max(R.rel_l2(imgs[k], ref[k]) for k in range(min(len(ref), len(imgs)))),
                     "tcc": float(np.linalg.norm(f["tcc"] - tcc) / np.linalg.norm(tcc)),
                     "scales": float(np.max(np.abs(f["s64"] - w64) / np.abs(w64))),
                     "kernel_projector": proj}
    return ips, n, el, err


def run_reference(args, ws, rank):
    """The reference CPU algorithm on the host cores, one bounded sample per step.

    The path is litho.cpp's Modules 3 + 7 (FT_r2c_padded + calcSOCS + FI) restated
    in FP64 with scipy.fft on all host cores (oracle/cpu_socs.py); the reference's own
    build cannot travel to the GPU host.  The kernels come from the FP64 oracle of
    calcTCC + calcKernels for the same quasar source.  Only rank 0 works."""
    if rank != 0:
        return
    from oracle import np_ref as R
    from oracle import cpu_socs
    synth = load_synth()
    src, S, npts = synth.quasar_source(2000)
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(NA, L_SIZE, sig, WAVELENGTH)
    tcc = R.calc_tcc(src, sig, WAVELENGTH, NA, DEFOCUS, L_SIZE, L_SIZE, nx, nx)
    krn, scales, _ = R.calc_kernels(tcc, K_KERNELS)
    per_step = 2
    masks = make_masks(per_step)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        for m in masks:
            cpu_socs.socs_image(m, krn, scales, nx, nx, workers=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for m in masks:
            cpu_socs.socs_image(m, krn, scales, nx, nx, workers=cores)
    el = time.perf_counter() - t0
    v = per_step * args.steps / el
    head = "plain" if args.precision == "fp32" else "mixed"
    line = {"metric": METRIC, "value": v, "unit": "images/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": bench_config(nx, npts, args.batch, head),
            "cpu_baseline": {"value": v, "unit": "images/s", "cores": cores, "kind": "port",
                             "sample": f"{per_step} masks of the workload per step x {args.steps} steps: "
                                       "FT_r2c_padded (r2c + half-spectrum rebuild) + calcSOCS (128^2 conv grid, "
                                       f"embed 94) + FI in FP64, scipy.fft workers={cores}"},
            "e2e": {"value": v, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measured_peaks():
    """The HBM copy rate and bf16 rates measured on this GPU model (empty: use the fallback)."""
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def batched_leg(ctx, setup, reps=20, forms=("plain", "mixed")):
    """The batched workload: 256 seeded masks with sides drawn from {256, 512, 768, 1024, 2048}
    and 20-60 % density (rectangles with sides L/64..L/8, count set by the drawn density),
    imaged per size class in one CUDA graph (litho_batch_plan_*, autotuned).  Masks up to 1024
    are centred in a 1024 period and use the K=24 kernels above; 2048 masks use a 2048-period
    kernel set of the same optics (Nx = 16, tcc 1089, K = 24)."""
    import math
    import numpy as np
    import torch
    import litho_gb300 as LG
    from litho_gb300 import surrogate as S
    ctx.set_stream(None)
    rng = np.random.default_rng(31)
    sizes = rng.choice([256, 512, 768, 1024, 2048], size=256)
    dens = rng.uniform(0.2, 0.6, size=256)
    sig, src = setup["sigma"], setup["src"]
    nx2 = LG.optics_n(NA, 2048, sig, WAVELENGTH)
    t2 = ctx.calc_tcc(src, sig, WAVELENGTH, NA, DEFOCUS, 2048, 2048, nx2, nx2)
    k2, s2, _ = ctx.calc_kernels(t2, K_KERNELS)
    res = {"config": {"masks": 256, "sizes": {int(v): int((sizes == v).sum()) for v in (256, 512, 768, 1024, 2048)},
                      "periods": [1024, 2048], "Nx": [setup["nx"], nx2], "K": K_KERNELS}}
    items = [(0 if m <= 1024 else 1, int(m), int(m)) for m in sizes]
    masks = []
    for i, (m, d) in enumerate(zip(sizes, dens)):
        lo, hi = max(1, int(m) // 64), max(2, int(m) // 8)
        area = ((lo + hi) / 2.0) ** 2
        n = int(min(256, max(1, round(-math.log(1.0 - d) * m * m / area))))
        masks.append(S.rect_masks(ctx, 31, i, 1, int(m), nmin=n, nmax=n, wmin=lo, wmax=hi)[0])
    torch.cuda.synchronize()
    res["config"]["density_mean"] = float(np.mean([float(x.mean()) for x in masks]))
    pix = float(sum(int(m) ** 2 for m in sizes))
    # compulsory HBM bytes of a batch: every mask read once, every period-sized image written once
    io_bytes = 4.0 * (pix + sum((1024 if m <= 1024 else 2048) ** 2 for m in sizes))
    hbm = float(measured_peaks().get("hbm_gbs", 6800.0))
    res["config"]["io_bytes_per_batch"] = io_bytes
    for form, prec in (("plain", LG.PREC_FP32), ("mixed", LG.PREC_MIXED)):
        if form not in forms:
            continue
        f = setup[form]
        sets = [ctx.kernel_set(f["krn"], f["s32"], setup["nx"], setup["nx"]), ctx.kernel_set(k2, s2, nx2, nx2)]
        t0 = time.perf_counter()
        plan = LG.BatchPlan(ctx, sets, [1024, 2048], items, precision=prec)
        t_plan = time.perf_counter() - t0
        for i, m in enumerate(masks):
            plan.mask(i).copy_(m)
        torch.cuda.synchronize()
        plan.run()
        ctx.synchronize()
        st = torch.cuda.Stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ctx.set_stream(st.cuda_stream)
        try:
            torch.cuda.nvtx.range_push("batched_timed")  # the range an ncu launch list selects
            e0.record(st)
            for _ in range(reps):
                plan.run()
            e1.record(st)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
        finally:
            ctx.set_stream(None)
        ms = e0.elapsed_time(e1) / reps
        io_gbs = io_bytes / (ms * 1e-3) / 1e9
        res[form] = {"images_per_s": 256 / (ms * 1e-3), "ms_per_batch": ms, "mask_mpix_per_s": pix / (ms * 1e-3) / 1e6,
                     "io_gb_per_s": io_gbs, "io_frac_of_measured_hbm": io_gbs / hbm,
                     "plan_create_s": t_plan, "tuned": plan.describe().get("classes")}
        plan.close()
        for k in sets:
            k.close()
    return res


def profile_tcc(device):
    """The launch sequence an ncu capture of the large-TCC kernels needs: the workload of
    large_tcc_leg, split-BF16 TCC twice, the FP64 TCC once and its top-48 eigensolve."""
    import litho_gb300 as LG
    from litho_gb300 import synth
    ctx = LG.Context(device)
    src = synth.annular_source(113, 0.7, 0.95)
    sig = LG.outer_sigma(src)
    nx = LG.optics_n(1.35, 2048, sig, 193.0)
    for _ in range(2):
        ctx.calc_tcc(src, sig, 193.0, 1.35, 0.0, 2048, 2048, nx, nx, precision=LG.TCC_SPLIT_BF16, n_medium=1.44)
    tcc = ctx.calc_tcc(src, sig, 193.0, 1.35, 0.0, 2048, 2048, nx, nx, precision=LG.TCC_FP64, n_medium=1.44)
    ctx.calc_kernels(tcc, 48)
    ctx.close()
    print(json.dumps({"profile_tcc": True, "tcc": int(tcc.shape[0]), "K": 48}), flush=True)


def profile_surrogate(device, batch, steps):
    """The launch sequence an ncu capture of the surrogate kernels needs: forward passes,
    predictions with the error estimate and Adam steps of a 256^2 FNO on seeded masks."""
    import torch
    import litho_gb300 as LG
    from litho_gb300 import surrogate as S
    ctx = LG.Context(device)
    ks, _ = S.c5_kernel_set(ctx, 256)
    model = S.Surrogate(ctx, L=256, seed=1)
    m = S.rect_masks(ctx, 1, 0, batch, 256)
    out = torch.empty_like(m)
    for _ in range(steps):
        model.forward(m, out)
    for _ in range(steps):
        model.predict(ks, m, out)
    tb = min(32, batch)
    mt, tt = m[:tb].contiguous(), torch.rand_like(m[:tb])
    for _ in range(steps):
        model.train_step(mt, tt, 1e-4, want_loss=False)
    torch.cuda.synchronize()
    model.close()
    ks.close()
    ctx.close()
    print(json.dumps({"profile_surrogate": True, "batch": batch, "steps": steps}), flush=True)


def large_tcc_leg(ctx):
    """The large-TCC workload: 2048^2 period at 1 nm/px, NA 1.35 (immersion, n = 1.44),
    193 nm, annular source sigma 0.7-0.95 on a 113^2 grid (4,044 points): Nx = 27 by the
    reference's formula, a 3025^2 TCC, top K = 48 eigenpairs.  Split-BF16 tensor-core TCC and
    FP64 TCC, FP64 eigensolve of both; device times from the library's stage events;
    errors of the split-BF16 form against the FP64 form."""
    import numpy as np
    import litho_gb300 as LG
    from litho_gb300 import synth
    ctx.set_stream(None)
    NA_, LAM, L_, NMED, K = 1.35, 193.0, 2048, 1.44, 48
    src = synth.annular_source(113, 0.7, 0.95)
    sig = LG.outer_sigma(src)
    nx = LG.optics_n(NA_, L_, sig, LAM)
    npts = int((src > 0).sum())
    res = {"config": {"L": L_, "NA": NA_, "wavelength": LAM, "n_medium": NMED, "source": "annular 0.7-0.95",
                      "source_points": npts, "Nx": nx, "tcc": (2 * nx + 1) ** 2, "K": K}}
    out = {}
    for form, prec in (("fp64", LG.TCC_FP64), ("split_bf16", LG.TCC_SPLIT_BF16)):
        ctx.calc_tcc(src, sig, LAM, NA_, 0.0, L_, L_, nx, nx, precision=prec, n_medium=NMED)  # warm
        ctx.stage_times(reset=True)
        ctx.enable_timing(True)
        t0 = time.perf_counter()
        tcc = ctx.calc_tcc(src, sig, LAM, NA_, 0.0, L_, L_, nx, nx, precision=prec, n_medium=NMED)
        t1 = time.perf_counter()
        k64, s32, s64 = ctx.calc_kernels(tcc, K)
        t2 = time.perf_counter()
        st = ctx.stage_times(reset=True)
        ctx.enable_timing(False)
        n = tcc.shape[0]
        flops = 8.0 * npts * n * n
        res[form] = {"tcc_device_ms": st["tcc"][0], "tcc_call_s": t1 - t0, "eig_device_ms": st["eig"][0],
                     "eig_call_s": t2 - t1,
                     "tcc_tflops_effective": flops / (st["tcc"][0] * 1e-3) / 1e12 if st["tcc"][0] else None}
        out[form] = (tcc, k64, s64)
    t64, k64, w64 = out["fp64"]
    tbf, kbf, wbf = out["split_bf16"]
    err = {"tcc": float(np.linalg.norm(tbf - t64) / np.linalg.norm(t64)),
           "eigenvalues": float(np.max(np.abs(wbf - w64) / np.abs(w64)))}
    V, W = k64[:, ::-1].T, kbf[:, ::-1].T
    proj, i = 0.0, 0
    while i < K:
        j = i + 1
        while j < K and abs(w64[j - 1] - w64[j]) <= 1e-6 * w64[0]:
            j += 1
        if j < K:
            a, b = W[:, i:j], V[:, i:j]
            proj = max(proj, float(np.linalg.norm(a @ a.conj().T - b @ b.conj().T)))
        i = j
    err["kernel_projector"] = proj
    res["split_bf16_vs_fp64"] = err
    res["gemm_tuning"] = [t for t in ctx.tcc_gemm_tuning() if t["n"] == (2 * nx + 1) ** 2]
    return res


def surrogate_leg(ctx, epochs):
    """The FNO surrogate on its own workload: 256x256 seeded rectangle masks, the
    quasar-source optics above (Nx=2), K=24.  A short training schedule (4096 GPU-SOCS
    pairs) by the library's kernels, calibration of the error estimate on 256 masks,
    512 held-out masks imaged with SOCS fallback and judged by SOCS, and throughput of
    plain SOCS, the network path and the surrogate-with-fallback path on the same 256
    masks (CUDA events)."""
    import numpy as np
    import torch
    from litho_gb300 import surrogate as S
    ctx.set_stream(None)
    ks, info = S.c5_kernel_set(ctx)
    L = S.C5["L"]
    thr = 1e-2
    tm, ti = S.make_pairs(ctx, ks, seed=11, first=0, count=4096, L=L)
    cm, ci = S.make_pairs(ctx, ks, seed=12, first=0, count=256, L=L)
    em, ei = S.make_pairs(ctx, ks, seed=13, first=0, count=512, L=L)
    model = S.Surrogate(ctx, L=L, seed=5)
    t0 = time.perf_counter()
    S.train(model, tm, ti, epochs=epochs, batch=32, lr=1e-3, decay_every=max(1, epochs // 3))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    img, est = model.predict(ks, cm)
    alpha = float(np.quantile(S.rel_l2_per_image(img, ci).cpu().numpy() / est.cpu().numpy(), 0.99))
    model.set_alpha(alpha)
    out, est, used = model.image(ks, em, thr)
    err = S.rel_l2_per_image(out, ei).cpu().numpy()
    net, _ = model.predict(ks, em)
    nerr = S.rel_l2_per_image(net, ei).cpu().numpy()

    def ms(fn, reps):
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

    mb = em[:256].contiguous()
    buf = torch.empty_like(mb)
    with S.torch_stream(ctx):
        t_socs = ms(lambda: ctx.image_batch(ks, mb, buf), 20)
    t_net = ms(lambda: model.predict(ks, mb, buf), 10)
    t_sur = ms(lambda: model.image(ks, mb, thr, buf), 10)
    model.close()
    ks.close()
    served = ~used
    return {"images_per_s": 256 / t_sur * 1e3, "network_images_per_s": 256 / t_net * 1e3,
            "plain_socs_same_config_images_per_s": 256 / t_socs * 1e3, "vs_plain_same_config": t_socs / t_sur,
            "config": {"L": L, "K": info["nk"], "Nx": info["Nx"], "masks": "seeded rectangles 8-32 of 8-64 px",
                       "train_pairs": 4096, "epochs": epochs, "train_s": t_train, "threshold": thr,
                       "alpha": alpha, "held_out": 512, "batch_timed": 256},
            "served_fraction": float(served.mean()),
            "network_rel_l2_median": float(np.median(nerr)), "network_rel_l2_max": float(nerr.max()),
            "returned_rel_l2_max": float(err.max()),
            "served_rel_l2_max": float(err[served].max()) if served.any() else None}


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.profile_tcc:
        return profile_tcc(local)
    if args.profile_surrogate:
        return profile_surrogate(local, args.batch, args.steps)
    if args.profile_batched:
        import litho_gb300 as LG
        ctx = LG.Context(local)
        res = batched_leg(ctx, setup_kernels(ctx), reps=args.steps, forms=("mixed",))
        ctx.close()
        res["mixed"].pop("tuned", None)
        print(json.dumps({"profile_batched": True, **res}), flush=True)
        return
    import numpy as np
    import torch
    import litho_gb300 as L

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = L.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    setup = setup_kernels(ctx)
    nx, npts = setup["nx"], setup["npts"]
    ks = {f: ctx.kernel_set(setup[f]["krn"], setup[f]["s32"], nx, nx) for f in ("plain", "mixed")}
    prec = {"plain": L.PREC_FP32, "mixed": L.PREC_MIXED}
    head = "plain" if args.precision == "fp32" else "mixed"
    B = args.batch
    masks_h = make_masks(B)
    masks = torch.from_numpy(masks_h).cuda()
    images = {f: torch.empty_like(masks) for f in ("plain", "mixed")}
    torch.cuda.synchronize()

    def step(form, m=None):
        ctx.image_batch(ks[form], masks if m is None else m, images[form], precision=prec[form])

    def timed(form, steps, stages, m=None):
        """K steps bracketed by barrier + synchronize, CUDA events on the library's stream.
        stages=True also brackets every kernel launch with CUDA events (per-kernel durations);
        the returned counts are launches either way."""
        ctx.stage_times(reset=True)
        ctx.enable_timing(stages)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(form, m)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(dist, e0.elapsed_time(e1), "cuda")
        ctx.enable_timing(False)
        return ms, ctx.stage_times(reset=True)

    for form in ("plain", "mixed"):
        for _ in range(max(args.warmup, 3)):
            step(form)
    torch.cuda.synchronize()
    if args.profile:  # the launch sequence an ncu capture needs, nothing else
        for form in ("plain", "mixed"):
            for _ in range(args.steps):
                step(form)
        torch.cuda.synchronize()
        print(json.dumps({"profile": True, "batch": B, "steps": args.steps}), flush=True)
        return
    # clocks are sampled from here through both timed regions and the e2e region;
    # a short untimed pre-roll keeps the GPU under load until the sampler is live
    clocks = Clocks(local)
    clocks.start()
    t_pre = time.perf_counter()
    while time.perf_counter() - t_pre < 0.6:
        for _ in range(8):
            step(head)
        torch.cuda.synchronize()
    other = "plain" if head == "mixed" else "mixed"
    ms_o, _ = timed(other, args.steps, False)
    ms, st_v = timed(head, args.steps, False)
    value = job_images_per_s(ws, B, args.steps, ms / 1e3)
    value_o = job_images_per_s(ws, B, args.steps, ms_o / 1e3)
    launches = sum(n for _, n in st_v.values())
    # the same masks as 8-bit grey levels / 255 (the reference's PNG-mask convention): no tile of
    # these is exact in TF32, so the mixed window DFT runs its residual products on every tile
    grey = grey_levels(masks)
    for _ in range(3):
        step("mixed", grey)
    ms_g, _ = timed("mixed", args.steps, False, grey)
    value_g = job_images_per_s(ws, B, args.steps, ms_g / 1e3)
    del grey
    # the same step with the band formed by per-kernel 2-D inverse FFTs on the conv grid
    # (LITHO_BAND_FFT) instead of the default TCC bilinear form
    ctx.set_band_method(L.BAND_FFT)
    for _ in range(3):
        step("mixed")
    ms_fft, _ = timed("mixed", args.steps, False)
    _, st_fft = timed("mixed", max(10, args.steps // 5), True)
    ctx.set_band_method(L.BAND_AUTO)
    value_fft = job_images_per_s(ws, B, args.steps, ms_fft / 1e3)
    # per-kernel durations: a shorter pass with every launch bracketed by CUDA events
    ksteps = max(10, args.steps // 5)
    _, st_o = timed(other, ksteps, True)
    _, st = timed(head, ksteps, True)

    # roofline of the dominant kernel (algorithmic bytes per launch)
    img_bytes = 4 * L_SIZE * L_SIZE
    kb = K_KERNELS * (2 * nx + 1) ** 2 * 8 + 4 * K_KERNELS
    alg = {"win_dft": B * img_bytes, "fi_out": B * img_bytes, "socs": B * kb,
           "fi_prep": B * (4 * nx + 1) * L_SIZE * 4}
    names = ("win_dft", "socs", "fi_prep", "fi_out")
    dom = max(names, key=lambda s: st[s][0])
    dom_ms = st[dom][0] / max(1, st[dom][1])
    peaks = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg[dom] / (dom_ms / 1e3) / 1e9
    tot = sum(st[k][0] for k in names)
    shares = {s: round(st[s][0] / max(1e-9, tot), 4) for s in names}
    kern_gbs = {s: alg[s] / (st[s][0] / max(1, st[s][1]) / 1e3) / 1e9 for s in ("win_dft", "fi_out")}

    # e2e through the C ABI with pinned host buffers (headline form)
    pin_in = torch.from_numpy(masks_h).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    hin, hout = pin_in.numpy(), pin_out.numpy()
    ctx.set_stream(None)
    for _ in range(2):
        ctx.image_batch(ks[head], hin, hout, precision=prec[head])
    if dist:
        dist.barrier()
    e2e_steps = max(3, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.image_batch(ks[head], hin, hout, precision=prec[head])
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0, "cuda")
    e2e = job_images_per_s(ws, B, e2e_steps, e2e_s)
    clk = clocks.stop()

    forms = {"mixed_grey_masks": {"images_per_s": value_g, "ms_per_step": ms_g / args.steps,
                                  "masks": "the step's masks as 8-bit grey levels / 255 (binary pattern x "
                                           "levels 200-255 on a background of levels 0-55)"},
             "mixed_band_fft": {"images_per_s": value_fft, "ms_per_step": ms_fft / args.steps,
                                "band_ms_per_step": st_fft["socs"][0] / max(10, args.steps // 5),
                                "band": "per-kernel 2-D inverse FFTs on the 64^2 conv grid, sum of s_k |E_k|^2, "
                                        "forward FFT (LITHO_BAND_FFT); the head forms use the TCC bilinear form"},
             head: {"images_per_s": value, "ms_per_step": ms / args.steps,
                    "stage_ms_per_step_serial": {s: st[s][0] / ksteps for s in names}},
             other: {"images_per_s": value_o, "ms_per_step": ms_o / args.steps,
                     "stage_ms_per_step_serial": {s: st_o[s][0] / ksteps for s in names}}}
    line = {"metric": METRIC, "value": value, "unit": "images/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "tf32x3/f32" if head == "mixed" else "f32", "data": "synthetic",
            "config": bench_config(nx, npts, B, head),
            "gpu_launches": int(launches),
            "forms": forms,
            "mixed_over_plain": forms["mixed"]["images_per_s"] / forms["plain"]["images_per_s"],
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm,
                         "traffic": (B * TRAFFIC_PER_IMAGE[(head, dom)]) if (head, dom) in TRAFFIC_PER_IMAGE else None,
                         "traffic_source": (f"ncu dram__bytes_read+write of one {TRAFFIC_KERNEL.get(dom, dom)} launch "
                                            "at 1024^2, K=24, 48 masks, scaled per mask to the batch"),
                         "peak_source": "measured (MEASURED_PEAKS.json)" if peaks else "fallback",
                         "shares": shares, "kernel_gbs": kern_gbs,
                         "bytes_per_image": 2 * img_bytes + kb,
                         "path_frac": value / ws * (2 * img_bytes + kb) / 1e9 / hbm},
            "e2e": {"value": e2e, "unit": "images/s", "h2d_bytes_per_step": int(masks_h.nbytes),
                    "d2h_bytes_per_step": int(masks_h.nbytes)},
            "clocks": clk}

    if rank == 0 and not args.no_cpu:
        nsamp = min(16, B)
        gpu_imgs = {f: images[f][:nsamp].cpu().numpy() for f in ("plain", "mixed")}
        ips, n, el, err = cpu_leg(setup, masks_h[:nsamp], gpu_imgs, args.cpu_budget_s)
        line["cpu_baseline"] = {"value": ips, "unit": "images/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{n} images ({nsamp} distinct masks of the step) in {el:.1f} s: "
                                          "FT_r2c_padded + calcSOCS (128^2 conv grid, embed 94) + FI in FP64, "
                                          "scipy.fft on all host cores"}
        line["rel_l2_vs_fp64"] = err
    if rank == 0 and not args.no_surrogate:
        line["forms"]["surrogate"] = surrogate_leg(ctx, args.surrogate_epochs)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_leg(ctx, setup)
    if rank == 0 and not args.no_large_tcc:
        line["large_tcc"] = large_tcc_leg(ctx)
    if rank == 0:
        print(json.dumps(line), flush=True)
    for k in ks.values():
        k.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
