#!/usr/bin/env python
"""Headline benchmark: DR iterations/s and gridding GFLOP/s at a 256^3 object
(512^3 Fourier grid), mixed precision against the FP64 GPU path.

Workload (seeded synthetic, no dataset): 256^3 volume of 2000 Gaussian atoms
(sigma 1, amplitudes U[0.3,1]) in a 110/110/80 ellipsoid, 90 projections
256 x 256 at random Euler angles (theta in [-72, 72]), 0.3 degree angle
jitter given to the reconstructor, oversampling 2, cutoff 0.125, mode 3,
positivity and the ellipsoid support on.

A "step" is one iteration of the Fourier-constraint loop (reconstruct.m:117-186)
on the 512^3 grid.  `value` is mixed-precision iterations/s with inputs
resident in HBM, timed with CUDA events on the library's stream; `e2e` is the
same metric through the host-pointer C ABI (genfire_reconstruct), host<->device
copies included.  `--impl reference` times the CPU restatement of the
reference (the oracle) on the host cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "DR iters/s + gridding GFLOP/s at 256³: mixed vs FP64 GPU at equal R-factor"
WORKLOAD = "euler256"


def parse():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=30, help="timed FP64 iterations")
    ap.add_argument("--rfactor-iters", type=int, default=None,
                    help="iterations for the equal-R-factor comparison (default: the workload's own count, "
                         "1000 for the 256^3 headline)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-problems leg")
    ap.add_argument("--batch-steps", type=int, default=300, help="iterations per problem in the batched leg")
    ap.add_argument("--quick", action="store_true", help="small workload (for checking the script)")
    ap.add_argument("--workload", default=WORKLOAD, choices=["tilt64", "euler128", "euler256", "euler512"],
                    help="synthetic workload (default: the 256^3 headline; euler512 is the 512^3 object on a "
                         "1024^3 grid, best run with --no-cpu-baseline --no-e2e --no-batch)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
        pg = dist
    return ws, rank, local, pg


def max_over_ranks(t_local, pg, device):
    """The whole job's time: the slowest rank's, after a barrier (replicas only;
    no collective runs inside the timed region)."""
    if not pg:
        return t_local
    import torch
    pg.barrier()
    t = torch.tensor([t_local], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, t_max, ws):
    """Units all ranks processed per second of the slowest rank's time."""
    return units_per_rank * ws / t_max


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(workload=WORKLOAD):
    """dram bytes per launch of the dominant kernel from the committed ncu
    summary of this workload's iteration, if any."""
    path = os.path.join(HERE, "profiles", "dr_iteration_%s_traffic.txt" % workload)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch"):
                return float(line.split("=")[1].split()[0])
    except Exception:
        pass
    return None


# ---------------------------------------------------------------------------
def gridding_flops(nk, D1, D2):
    """Useful DFT flops: sum_p (4 Nk D1 D2 + 8 Nk D2) (E_u P products and the E_v contraction)."""
    nk = np.asarray(nk, dtype=np.float64)
    return float((4.0 * nk * D1 * D2 + 8.0 * nk * D2).sum())


def make_inputs(G, ctx, quick, workload=WORKLOAD):
    from genfire_gb300 import synth

    def proj(vol, angles, vectors):
        return ctx.project(vol.astype(np.float64), angles, vectors=np.asarray(vectors, float).reshape(-1))
    if quick:
        return synth.make_workload(workload, proj, D=64, n_proj=30, atoms=120)
    return synth.make_workload(workload, proj)


def params_for(G, w, precision, iters):
    p = G.default_params()
    D = w["D"]
    p.Dim1, p.Dim2, p.NumProjs = D, D, w["projections"].shape[2]
    p.oversamplingRatio = w["os"]
    p.interpolationCutoffDistance = 0.125
    for k, v in zip(("vector1", "vector2", "vector3"), w["vectors"]):
        getattr(p, k)[:] = [float(x) for x in v]
    p.numIterations = iters
    p.constraintEnforcementMode = 3
    p.constraintPositivity = 1
    p.constraintSupport = 1
    p.precision = precision
    return p


def run_ours(args, ws, rank, local, pg):
    import torch
    import __graft_entry__ as ge
    ge.build()
    import genfire_gb300 as G

    torch.cuda.set_device(local)
    ctx = G.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    w = make_inputs(G, ctx, args.quick, args.workload)
    D = w["D"]
    P = w["projections"].shape[2]
    n1, _ = G.grid_size(params_for(G, w, G.PREC_FP64, 1))
    N3 = n1 ** 3
    d_proj = torch.from_numpy(np.ascontiguousarray(w["projections"].reshape(-1, order="F"))).cuda()
    d_sup = torch.from_numpy(np.ascontiguousarray(w["support"].reshape(-1, order="F").astype(np.uint8))).cuda()
    d_M32 = torch.empty(N3, dtype=torch.complex64, device="cuda")
    d_M64 = torch.empty(N3, dtype=torch.complex128, device="cuda")
    angles = w["angles_in"]

    def time_call(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    # ---- gridding (fillInFourierGrid_DFT incl. recIFFT), device-resident projections
    pm = params_for(G, w, G.PREC_MIXED, 1)
    pf = params_for(G, w, G.PREC_FP64, 1)
    ctx.grid_dft_device(pm, d_proj.data_ptr(), angles, d_M32.data_ptr())          # warm-up
    nk, t_grid_mixed = time_call(lambda: ctx.grid_dft_device(pm, d_proj.data_ptr(), angles, d_M32.data_ptr()))
    nk64, t_grid_fp64 = time_call(lambda: ctx.grid_dft_device(pf, d_proj.data_ptr(), angles, d_M64.data_ptr()))
    flops = gridding_flops(nk, D, D)
    stages = ctx.grid_profile(pm, d_proj.data_ptr(), angles, d_M32.data_ptr())
    ctx.grid_dft_device(pm, d_proj.data_ptr(), angles, d_M32.data_ptr())   # restore (the profile skips recIFFT)
    grid_err = float(torch.linalg.vector_norm(d_M32.to(torch.complex128) - d_M64) / torch.linalg.vector_norm(d_M64))
    # split-FP16 gridding with per-projection scaling (GENFIRE_PREC_FP16_SCALED), same projections
    ph = params_for(G, w, G.PREC_FP16_SCALED, 1)
    ctx.grid_dft_device(ph, d_proj.data_ptr(), angles, d_M32.data_ptr())                 # warm-up
    _, t_grid_fp16 = time_call(lambda: ctx.grid_dft_device(ph, d_proj.data_ptr(), angles, d_M32.data_ptr()))
    grid_err_fp16 = float(torch.linalg.vector_norm(d_M32.to(torch.complex128) - d_M64) / torch.linalg.vector_norm(d_M64))
    stages_fp16 = ctx.grid_profile(ph, d_proj.data_ptr(), angles, d_M32.data_ptr())
    # the second tensor-core form (GENFIRE_DFT_KERNEL=n256: Re and Im stacked in
    # rows, N = 256 MMAs, 64-point tiles), opt-in, split BF16
    os.environ["GENFIRE_DFT_KERNEL"] = "n256"
    try:
        ctx.grid_dft_device(pm, d_proj.data_ptr(), angles, d_M32.data_ptr())             # warm-up
        _, t_grid_n256 = time_call(lambda: ctx.grid_dft_device(pm, d_proj.data_ptr(), angles, d_M32.data_ptr()))
        grid_err_n256 = float(torch.linalg.vector_norm(d_M32.to(torch.complex128) - d_M64)
                              / torch.linalg.vector_norm(d_M64))
        stages_n256 = ctx.grid_profile(pm, d_proj.data_ptr(), angles, d_M32.data_ptr())
    finally:
        del os.environ["GENFIRE_DFT_KERNEL"]
    ctx.grid_dft_device(pm, d_proj.data_ptr(), angles, d_M32.data_ptr())   # the MIXED grid for the loop below

    # ---- DR loop, mixed (value): warm-up, then exactly K timed iterations
    K, W = args.steps, args.warmup
    pmr = params_for(G, w, G.PREC_MIXED, W + K + 20)
    rec = ctx.recon(pmr, d_M32.data_ptr(), support=d_sup.data_ptr(), on_device=True)
    rec.iterate(W)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    rec.iterate(K)
    ev1.record(stream)
    ev1.synchronize()
    t_dr = ev0.elapsed_time(ev1) / 1e3
    clk = clocks.stop()
    t_dr = max_over_ranks(t_dr, pg, "cuda")
    names, ms, by = rec.profile(20)
    tuned = rec.tuning()
    rec.close()

    # ---- e2e: the host-pointer C ABI (genfire_reconstruct), copies included.  One call
    # runs the configuration's own iteration count (what a user's reconstruct does);
    # a call of the timed step count is reported beside it, and the staged API
    # splits the call into its host->device copy, setup, iterations and readback.
    e2e = None
    if not args.no_e2e:
        hM = d_M32.cpu().numpy().reshape((n1, n1, n1), order="F")
        hM = np.asfortranarray(hM)
        hS = np.asfortranarray(w["support"].astype(np.uint8))
        h2d = hM.nbytes + hS.nbytes

        def e2e_call(steps):
            pe = params_for(G, w, G.PREC_MIXED, steps)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            vol_e, errK_e, _, _, _ = ctx.reconstruct(pe, hM, support=hS)
            return time.perf_counter() - t0, vol_e.nbytes + errK_e.nbytes
        K_e2e = K if args.quick else max(K, w["iters"])
        t_short, d2h = e2e_call(K)
        t_e2e, d2h = e2e_call(K_e2e) if K_e2e != K else (t_short, d2h)
        # split, from the staged calls: the setup alone (the same inputs already in
        # device memory), then from host buffers (copies + setup), the iterations
        # and the readback
        pe = params_for(G, w, G.PREC_MIXED, K_e2e)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.recon(pe, hM, support=hS)
        t_create = time.perf_counter() - t0
        t0 = time.perf_counter()
        r.iterate(K_e2e)
        torch.cuda.synchronize()
        t_iter = time.perf_counter() - t0
        t0 = time.perf_counter()
        r.result()
        t_d2h = time.perf_counter() - t0
        r.close()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.recon(pe, d_M32.data_ptr(), support=d_sup.data_ptr(), on_device=True)
        t_setup = time.perf_counter() - t0
        r.close()
        e2e = {"value": K_e2e / t_e2e, "unit": "iters/s", "steps": K_e2e, "h2d_bytes_per_step": h2d / K_e2e,
               "d2h_bytes_per_step": d2h / K_e2e,
               "at_timed_steps": {"steps": K, "value": K / t_short, "h2d_bytes_per_step": h2d / K,
                                  "d2h_bytes_per_step": d2h / K},
               "split_ms": {"h2d_copy": (t_create - t_setup) * 1e3, "setup": t_setup * 1e3, "iterate": t_iter * 1e3,
                            "d2h_result": t_d2h * 1e3, "staged_total": (t_create + t_iter + t_d2h) * 1e3},
               "note": "one genfire_reconstruct call of the configuration's %d iterations from host buffers: "
                       "measuredK (%d^3 complex64, pageable) and the support copied in, reconstruction and errK "
                       "copied out, setup (constraint table, autotuned pass choice, graph) included" % (K_e2e, n1)}

    # ---- DR loop, FP64
    K64 = max(3, min(args.fp64_steps, K))
    pfr = params_for(G, w, G.PREC_FP64, 3 + K64)
    rec64 = ctx.recon(pfr, d_M64.data_ptr(), support=d_sup.data_ptr(), on_device=True)
    rec64.iterate(3)
    torch.cuda.synchronize()
    ev0.record(stream)
    rec64.iterate(K64)
    ev1.record(stream)
    ev1.synchronize()
    t_dr64 = ev0.elapsed_time(ev1) / 1e3
    rec64.close()

    # ---- equal-iteration R-factors (reconstruct.m:176 form, ZYZ projector at the input angles)
    NR_ = args.rfactor_iters if args.rfactor_iters else (50 if args.quick else w["iters"])
    out = {}
    for prec, dM in ((G.PREC_MIXED, d_M32), (G.PREC_FP64, d_M64)):
        pr = params_for(G, w, prec, NR_)
        r = ctx.recon(pr, dM.data_ptr(), support=d_sup.data_ptr(), on_device=True)
        r.iterate(NR_)
        vol, errK, _, _, _ = r.result()
        r.close()
        errR, _, _ = ctx.rfactor(vol.astype(np.float64), angles, w["projections"], vectors=None)
        out[prec] = (errR, float(errK[-1]), vol)
    r_mixed, r_fp64 = out[G.PREC_MIXED][0], out[G.PREC_FP64][0]
    vol_err = float(np.linalg.norm(out[G.PREC_MIXED][2] - out[G.PREC_FP64][2]) / np.linalg.norm(out[G.PREC_FP64][2]))
    gt_err = float(np.linalg.norm(out[G.PREC_MIXED][2] - w["vol"]) / np.linalg.norm(w["vol"]))

    # ---- projector (the R-factor of reconstruct.m:176) on the device, MIXED
    projector = projector_leg(G, ctx, out[G.PREC_MIXED][2], w)

    # ---- FFT gridding (fillInFourierGrid, griddingMethod 1) on the same projections
    pfm = params_for(G, w, G.PREC_MIXED, 1)
    pfm.griddingMethod = 1
    pfm.allowMultipleGridMatches = 1
    ctx.grid_fft_device(pfm, d_proj.data_ptr(), angles, d_M32.data_ptr())             # warm-up
    npairs, t_fft_grid = time_call(lambda: ctx.grid_fft_device(pfm, d_proj.data_ptr(), angles, d_M32.data_ptr()))
    fft_grid = {"ms": t_fft_grid * 1e3, "pairs": int(npairs), "precision": "mixed",
                "interpolationCutoffDistance": 0.125, "allowMultipleGridMatches": 1}

    # ---- batched problems: one graph launch per iteration of all problems
    batch = None
    if not args.no_batch and rank == 0 and ws == 1:
        batch = batch_leg(G, ctx, args.batch_steps, args.quick)

    # ---- roofline of the dominant kernel (live CUDA events per kernel)
    peak, peak_kind = measured_peaks()
    k = int(np.argmax(ms))
    achieved = by[k] / (ms[k] * 1e-3) / 1e9
    roof = {"kernel": names[k], "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": "of " + peak_kind,
            "traffic": None if args.quick else committed_traffic(args.workload),
            "algorithmic_bytes_per_launch": by[k], "ms_per_launch": ms[k],
            "per_kernel": [{"kernel": names[i], "ms": ms[i], "bytes": by[i],
                            "GB/s": (by[i] / (ms[i] * 1e-3) / 1e9) if ms[i] > 0 else None} for i in range(len(ms))]}

    # ---- CPU baseline (oracle, bounded sample), rank 0 at N=1 only
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(w, d_M64)
        except Exception as e:  # reported, not fatal
            cpu = {"value": None, "error": str(e)[:200]}

    iters_per_s = whole_job_rate(K, t_dr, ws)
    res = {
        "metric": METRIC, "value": iters_per_s, "unit": "iters/s", "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": t_dr / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "%s: %d^3 object, %d^3 Fourier grid, %d projections %dx%d, mixed precision "
                               "(complex64 FFT passes, FP64 errK/weight/phase sums)" % (args.workload, D, n1, P, D, D),
                   "oversamplingRatio": w["os"], "interpolationCutoffDistance": 0.125,
                   "constraintEnforcementMode": 3, "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": ("per-iteration working set (object, half spectra, constraint table) exceeds the 129 MB L2"
                          if n1 >= 512 else "per-iteration working set partly L2-resident (no flush)")},
        "gridding_gflops": flops / t_grid_mixed / 1e9,
        "gridding_stages_ms": stages,
        "gridding_roofline": gridding_roofline(flops, nk, D, stages),
        "gridding_ms": t_grid_mixed * 1e3,
        "gridding_rel_l2_vs_fp64": grid_err,
        "gridding_fp16_scaled": {"gridding_ms": t_grid_fp16 * 1e3, "gridding_gflops": flops / t_grid_fp16 / 1e9,
                                 "rel_l2_vs_fp64": grid_err_fp16, "stages_ms": stages_fp16,
                                 "roofline": gridding_roofline(flops, nk, D, stages_fp16),
                                 "note": "split-FP16 operands (3 products), each projection scaled by a power of "
                                         "two; the same kernel as split BF16"},
        "gridding_n256_form": {"gridding_ms": t_grid_n256 * 1e3, "rel_l2_vs_fp64": grid_err_n256,
                               "stages_ms": stages_n256,
                               "roofline": gridding_roofline(flops, nk, D, stages_n256, tile=64),
                               "note": "opt-in second tensor-core form (GENFIRE_DFT_KERNEL=n256), split BF16"},
        "projector_roofline": projector,
        "fp64": {"dr_iters_per_s": K64 / t_dr64, "gridding_gflops": flops / t_grid_fp64 / 1e9,
                 "gridding_ms": t_grid_fp64 * 1e3, "timed_iterations": K64},
        "mixed_over_fp64_dr": (K / t_dr) / (K64 / t_dr64),
        "rfactor": {"iterations": NR_, "mixed": r_mixed, "fp64": r_fp64, "abs_diff": abs(r_mixed - r_fp64),
                    "errK_mixed": out[G.PREC_MIXED][1], "errK_fp64": out[G.PREC_FP64][1],
                    "volume_rel_l2_mixed_vs_fp64": vol_err, "volume_rel_l2_vs_ground_truth": gt_err},
        "gridded_points": int(np.sum(nk)),
        "e2e": e2e,
        "fft_gridding": fft_grid,
        "batch": batch,
        "roofline": roof,
        "fft_pass_variants": {"F2": tuned[0], "F3": tuned[1], "I2": tuned[2],
                              "legend": "autotuned at setup: 0 generic shared-memory engine, 1 radix-8 register "
                                        "engine one column per thread, 2 the same with two columns per thread, "
                                        "3 mixed-radix engine, 4 radix-32 engine (512 or 1024 points, one exchange)"},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": len(ms) * K,
    }
    ctx.close()
    return res


def gridding_roofline(flops, nk, D, stages, tile=128):
    """The tcgen05 DFT kernel against the measured bf16 tensor peak: useful
    flops (sum_p 4 Nk D1 D2 + 8 Nk D2) and executed tensor flops (the 3 split
    products, Re and Im, over tiles of `tile` points: 128 for the default
    form, 64 for the N = 256 form whose 128 MMA rows are the Re and Im of 64
    points) per its CUDA-event duration."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        peak, kind = float(pk["bf16_tflops"]), "measured"
    except Exception:
        peak, kind = 1900.0, "fallback"
    ms = stages["dft_kernel"]
    tiles = float(np.sum(np.ceil(np.asarray(nk, dtype=np.float64) / tile)))
    k_pad, n_pad = -(-D // 32) * 32, -(-D // 16) * 16
    executed = tiles * tile * k_pad * n_pad * 2.0 * 6
    ach = flops / (ms * 1e-3) / 1e12
    return {"kernel": "k_dft_tcgen05" if tile == 128 else "k_dft_tcgen05_w", "bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak, "peak_kind": "of " + kind, "ms_per_launch": ms,
            "executed_tflops": executed / (ms * 1e-3) / 1e12, "executed_frac": executed / (ms * 1e-3) / 1e12 / peak,
            "note": "achieved counts the useful DFT flops; executed counts the split products the tensor cores "
                    "run (3 per complex-real product, Re and Im: 6 products of 2 flops per MAC, on whole tiles "
                    "and the projection padded to 32 rows and 16 columns)"}


def projector_leg(G, ctx, vol, w, reps=5):
    """The MIXED R-factor call of reconstruct.m:176 (projector + fused sums) on
    device-resident data through genfire_rfactor_noalloc, CUDA events on the
    library's stream.  Algorithmic bytes P (4 D^3 + 4 D^2): the volume read once
    per projection and one float per pixel."""
    import ctypes
    import torch
    from genfire_gb300 import _lib
    L = _lib.load()
    D = vol.shape[0]
    P = w["projections"].shape[2]
    d_vol = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(vol, dtype=np.float32).reshape(-1, order="F"))).cuda()
    d_meas = torch.from_numpy(np.ascontiguousarray(w["projections"].reshape(-1, order="F"))).cuda()
    A = np.asfortranarray(w["angles_in"], dtype=np.float64)
    vec = np.ascontiguousarray(np.asarray(w["vectors"], dtype=np.float64).reshape(9))
    R1, R2, eR = np.zeros(P), np.zeros(P), ctypes.c_double()
    stream = torch.cuda.ExternalStream(ctx.stream)
    dp = ctypes.POINTER(ctypes.c_double)

    def call():
        st = L.genfire_rfactor_noalloc(ctx.handle, G.PREC_MIXED, ctypes.c_void_p(d_vol.data_ptr()), D, D, D, P,
                                       A.ctypes.data_as(dp), vec.ctypes.data_as(dp), ctypes.c_void_p(d_meas.data_ptr()),
                                       R1.ctypes.data_as(dp), R2.ctypes.data_as(dp), ctypes.byref(eR))
        assert st == 0
    torch.cuda.synchronize()
    call()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ts = []
    for _ in range(reps):
        ev0.record(stream)
        call()
        ev1.record(stream)
        ev1.synchronize()
        ts.append(ev0.elapsed_time(ev1))
    ms = float(np.median(ts))
    peak, kind = measured_peaks()
    by = float(P) * (4.0 * D ** 3 + 4.0 * D ** 2)
    ach = by / (ms * 1e-3) / 1e9
    return {"kernel": "k_project<float, trilinear> + k_project_sums", "bound": "hbm", "achieved": ach, "peak": peak,
            "unit": "GB/s", "frac": ach / peak, "peak_kind": "of " + kind, "ms_per_call": ms,
            "algorithmic_bytes": by, "errR": eR.value, "projections": P,
            "note": "the 256^3 float volume (67 MB) stays resident in the 129 MB L2, so the gathers are served "
                    "from L2; frac is against HBM as the formula's bytes define it"}


def batch_leg(G, ctx, K, quick):
    """Independent problems of different sizes (the batched workload of
    genfire_gb300.synth) iterated K times each: all problems per graph launch
    (genfire_recon_batch) against the same problems iterated one after the
    other; aggregate problem-iterations per second for both."""
    from genfire_gb300 import synth

    def proj(vol, angles, vectors):
        return ctx.project(vol.astype(np.float64), angles, vectors=np.asarray(vectors, float).reshape(-1))
    probs = synth.make_batch_workload(proj, count=4 if quick else 24, sizes=(48, 64) if quick else synth.BATCH_SIZES,
                                      iters=K)
    W = 3
    recons = []
    for w in probs:
        p = params_for(G, w, G.PREC_MIXED, W + 2 * K)
        M, _, _ = ctx.grid_dft(p, w["projections"], w["angles_in"], want_rec=False)
        recons.append(ctx.recon(p, M, support=w["support"]))
    b = G.ReconBatch(ctx, recons)
    b.iterate(W)
    t0 = time.perf_counter()
    b.iterate(K)
    t_batch = time.perf_counter() - t0
    b.close()
    t0 = time.perf_counter()
    for r in recons:
        r.iterate(K)
    t_seq = time.perf_counter() - t0
    for r in recons:
        r.close()
    n = len(probs)
    return {"problems": n, "sizes": [w["D"] for w in probs], "projections": [int(w["projections"].shape[2]) for w in probs],
            "iterations_per_problem": K, "precision": "mixed",
            "batched_problem_iters_per_s": n * K / t_batch, "sequential_problem_iters_per_s": n * K / t_seq,
            "batched_over_sequential": t_seq / t_batch, "batched_ms": t_batch * 1e3, "sequential_ms": t_seq * 1e3,
            "note": "wall time with a stream synchronize at the end of each leg; one graph launch per batched "
                    "iteration runs every problem's iteration as an independent child graph"}


def cpu_baseline(w, d_M64):
    """The oracle (FP64 CPU restatement) on the host cores: one iteration of the
    full 512^3 loop, and the gridding of 4 of the 90 projections."""
    from oracle import oracle as O
    D = w["D"]
    n1 = O.oversampled(D, w["os"])
    prm = O.make_params(D, D, 4, oversamplingRatio=w["os"], interpolationCutoffDistance=0.125,
                        vector1=w["vectors"][0], vector2=w["vectors"][1], vector3=w["vectors"][2],
                        numIterations=1, constraintEnforcementMode=3)
    sub = [0, 30, 60, 89] if w["projections"].shape[2] >= 90 else [0, 1, 2, 3]
    t0 = time.perf_counter()
    FS, nk = O.grid_fs(prm, w["projections"][:, :, sub], w["angles_in"][sub])
    t_grid = time.perf_counter() - t0
    M = d_M64.cpu().numpy().reshape((n1, n1, n1), order="F")
    O.reconstruct(prm, M, support=w["support"])
    t_loop = O.last_loop_seconds()
    return {"value": 1.0 / t_loop, "unit": "iters/s", "cores": O.num_threads(), "kind": "port",
            "sample": "1 iteration of the %d^3 FP64 loop (full complex FFTs, as reconstruct.m); gridding of "
                      "projections %s" % (n1, sub),
            "gridding_gflops": gridding_flops(nk, D, D) / t_grid / 1e9, "cpu": cpu_model()}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if "Model name" in line:
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return None


def run_reference(args, ws, rank):
    """The reference's CPU path restated (the oracle), all host threads, on the same workload."""
    if rank != 0:
        return None
    from oracle import oracle as O
    import genfire_gb300.synth as synth
    # inputs: the same seeded workload, projected by the oracle's own projector
    from genfire_gb300.synth import WORKLOADS
    wl = WORKLOADS[args.workload]

    def proj(vol, angles, vectors):
        v = np.asarray(vectors, float).reshape(-1)
        return np.stack([O.project(vol.astype(np.float64), *a, vectors=v) for a in angles], axis=2)
    kw = dict(D=64, n_proj=30, atoms=120) if args.quick else {}
    w = synth.make_workload(args.workload, proj, **kw)
    D = w["D"]
    P = w["projections"].shape[2]
    steps = max(1, min(args.steps, 2 if not args.quick else 5))
    # warm-up iterations inside the same loop (the arrays already touched),
    # at most 5 so that the run stays within a few minutes
    warm = max(0, min(args.warmup, 5))
    prm = O.make_params(D, D, P, oversamplingRatio=wl["os"], interpolationCutoffDistance=0.125,
                        vector1=w["vectors"][0], vector2=w["vectors"][1], vector3=w["vectors"][2],
                        numIterations=warm + steps, constraintEnforcementMode=3)
    t0 = time.perf_counter()
    M, _, nk = O.grid_dft(prm, w["projections"], w["angles_in"], want_rec=False)
    t_grid = time.perf_counter() - t0
    O.reconstruct(prm, M, support=w["support"])
    t_loop = O.last_loop_seconds_from(warm)
    v = steps / t_loop
    n1 = O.oversampled(D, wl["os"])
    sample = ("%d iterations of the %d^3 FP64 loop after %d warm-up iterations; gridding of all %d projections"
              % (steps, n1, warm, P))
    return {"metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": ws, "steps": steps, "warmup": warm,
            "ms_per_step": t_loop / steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "%s: %d^3 object, %d^3 Fourier grid, %d projections (CPU restatement of the "
                                   "reference's host path, FP64)" % (args.workload, D, n1, P)},
            "gridding_gflops": gridding_flops(nk, D, D) / t_grid / 1e9,
            "cpu_baseline": {"value": v, "unit": "iters/s", "cores": O.num_threads(), "kind": "port",
                             "sample": sample, "cpu": cpu_model()},
            "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    ws, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        res = run_reference(args, ws, rank)
    else:
        res = run_ours(args, ws, rank, local, pg)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
