"""Benchmark of the multiview deconvolution hot path: voxel-updates/s.

One step = one deconvolution iteration (every view's conv1 -> quotient -> conv2 -> update) of
the 4-view efficient-Bayesian workload 512x512x256, PSF 31x31x61 (sigma 2,2,7) rotated per view
(0/45/90/135 deg about y, so the 45 and 135 degree views carry 65x31x65 PSFs), cosine-blended
VIRTUAL weights; synthetic seeded inputs.  voxel-updates/s = voxels * views * steps / time.
The 4-view 256x256x192 workload and the 6-view workload cropped to random boxes in a 256^3
volume (15x15x41 PSFs, 128^3 reference blocks) are measured as well, each in its own object
(``workloads``); so is the same workload with the tensor-core DFT stages (``tensor_dft``).

Besides the timed value the line carries the error of the timed handle's own tile plans against
the FP64 oracle after 10 iterations (``accuracy_vs_fp64``, computed after the timed region), the
plain FP32 form (the reference's block structure, one block per launch sequence), the e2e job
through the C ABI from host buffers, and the CPU restatement timed on the host cores.

Arms:
  (default)          the sm_103a library: fused tiled passes, all tiles of a view in one launch
                     per pass, one CUDA graph per iteration, inputs resident in HBM.
  --impl reference   the reference algorithm on the host cores (the CPU restatement of the Java
                     MVDeconvolution / MVDeconFFT path, float32, scipy FFT on every core); the
                     reference's own Java code cannot run on this machine.

Multi-GPU: the path does not shard across GPUs (views are sequential, and the deployment is one
GPU per machine); with --gpus N each rank runs an independent replica on its own GPU ("weak" scaling,
value = all ranks' voxel-updates / max time over ranks).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-updates/s, 4-view decon, batched+split vs plain FP32 form at relL2<=1e-4"

WORKLOADS = {
    # name: (cfg id, shape xyz, psf xyz, reference block for the plain form)
    "cfg2_4view_eb_256x256x192": (2, (256, 256, 192), (15, 15, 41), (128, 128, 128)),
    "cfg3_6view_crops_256": (3, (256, 256, 256), (15, 15, 41), (128, 128, 128)),
    "cfg4_4view_eb_512x512x256": (4, (512, 512, 256), (31, 31, 61), None),
    "cfg1_2view_128x128x64": (1, (128, 128, 64), (9, 9, 25), None),
}
DEFAULT_WORKLOAD = "cfg4_4view_eb_512x512x256"
# reported beside the headline workload, each in its own object
SECONDARY_WORKLOADS = ("cfg2_4view_eb_256x256x192", "cfg3_6view_crops_256")
REFERENCE_MAX_SECONDS = 150.0  # bound on the reference arm's timed view stages


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 form measurement")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="planner's default tiles instead of timed ones")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 accuracy check")
    ap.add_argument("--no-secondary", action="store_true", help="skip the other workloads' objects")
    ap.add_argument("--no-psf-refine", action="store_true", help="skip the PSF refinement object")
    ap.add_argument("--no-tensor-dft", action="store_true", help="skip the tensor-core DFT stage object")
    ap.add_argument("--tensor-dft", action="store_true",
                    help="time the handle with the tensor-core middle DFT stages as the line's value")
    ap.add_argument("--only", choices=["inputs", "separable", "stage"],
                    help="measure only the input preparation or the separable convolution at the workload's size; "
                         "'stage': run --warmup + --steps iterations of the workload (untimed, for profilers)")
    ap.add_argument("--volume", default=None,
                    help="x,y,z size of the workload's synthetic volume (default: the workload's own)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_problem(workload, volume=None):
    """The workload's seeded inputs; MVD_PROBLEM_CACHE=<dir> keeps them between runs."""
    from spim_registration_gb300 import synthetic as S

    cfg, shape, psf, _ = WORKLOADS[workload]
    if volume is not None:
        shape = tuple(int(v) for v in volume.split(","))
        workload = f"{workload}_at_{shape[0]}x{shape[1]}x{shape[2]}"
    cache = os.environ.get("MVD_PROBLEM_CACHE")
    path = os.path.join(cache, workload + ".npz") if cache else None
    if path and os.path.exists(path):
        z = np.load(path)
        nv = int(z["nv"])
        return S.Problem(name=workload, views=[z[f"v{i}"] for i in range(nv)], weights=[z[f"w{i}"] for i in range(nv)],
                         psfs=[z[f"p{i}"] for i in range(nv)], psftype=int(z["psftype"]),
                         iterations=int(z["iterations"]), lam=float(z["lam"]), block=None)
    prob = S.make_problem(cfg, shape_xyz=shape, psf_size_xyz=psf)
    if path:
        os.makedirs(cache, exist_ok=True)
        arrs = {"nv": len(prob.views), "psftype": prob.psftype, "iterations": prob.iterations, "lam": prob.lam}
        for i in range(len(prob.views)):
            arrs[f"v{i}"], arrs[f"w{i}"], arrs[f"p{i}"] = prob.views[i], prob.weights[i], prob.psfs[i]
        np.savez(path, **arrs)
    return prob


def bytes_per_iteration(dec, n_views, n_voxels):
    """Algorithmic HBM bytes of one fused iteration per pass kind, from the live tile plans.
    Per view, with P the tile voxels, H the complex values of the tiles' half spectra and N the
    volume's voxels: forward plane pass 4 P + 8 H and z pass 8 H + 8 H_eff + one OTF read (it
    reads every slice and stores the effective ones), each twice (two convolutions); inverse
    pass with the quotient 8 H_eff + 8 N; inverse pass with the update 8 H_eff + 12 N."""
    out = {"plane_fwd": 0, "zpass": 0, "plane_inv_quotient": 0, "plane_inv_update": 0}
    for v in range(n_views):
        p = dec.plan(v)
        tx, ty, tz = p["tile"]
        ex, ey, ez = p["effective"]
        nt = p["tiles"][0] * p["tiles"][1] * p["tiles"][2]
        half = (tx // 2 + 1) * ty  # complex values per spectrum slice
        P = nt * tx * ty * tz      # real voxels transformed
        H = nt * half * tz         # complex values of the half spectrum
        Heff = nt * half * min(ez, tz)
        # forward plane: gather P reals, write H complex (x2 convolutions)
        out["plane_fwd"] += 2 * (4 * P + 8 * H)
        # z pass: read H, write the effective slices, read the OTF once (all tiles of a view
        # share its shape) (x2)
        out["zpass"] += 2 * (8 * H + 8 * Heff + 8 * half * tz)
        # inverse plane: read effective spectrum slices; quotient reads img, writes q
        out["plane_inv_quotient"] += 8 * Heff + 8 * n_voxels
        # update reads psi, weight, writes psi
        out["plane_inv_update"] += 8 * Heff + 12 * n_voxels
    return out


def reference_block_bytes(prob, block):
    """Algorithmic HBM bytes of one iteration per pass kind under the reference's block
    structure, the roofline's byte contract: per view, blocks of image + kernel - 1 (one block,
    MVDeconFFT.java:144-165) or of the given block size (BlockGeneratorFixedSizePrecise.java:
    46-122, count ceil(n / (B - k + 1)) per axis), P = the block's voxels, H = (X / 2 + 1) Y Z.
    Per block and convolution: the forward pass reads 4 P and writes 8 H, the z pass reads and
    writes 8 H each, the inverse pass reads 8 H; the epilogues move 8 (quotient) and 12 (update)
    bytes per voxel of the volume.  Padding of the tiles this library runs is not credited."""
    nx, ny, nz = prob.dims_xyz
    n = nx * ny * nz
    out = {"plane_fwd": 0, "zpass": 0, "plane_inv_quotient": 0, "plane_inv_update": 0}
    for psf in prob.psfs:
        kz, ky, kx = psf.shape
        if block is None:
            dims, count = (nx + kx - 1, ny + ky - 1, nz + kz - 1), 1
        else:
            dims = tuple(block)
            count = 1
            for nd, kd, bd in zip((nx, ny, nz), (kx, ky, kz), block):
                count *= -(-nd // (bd - kd + 1))
        P = dims[0] * dims[1] * dims[2]
        H = (dims[0] // 2 + 1) * dims[1] * dims[2]
        out["plane_fwd"] += 2 * count * (4 * P + 8 * H)
        out["zpass"] += 2 * count * 16 * H
        out["plane_inv_quotient"] += count * 8 * H + 8 * n
        out["plane_inv_update"] += count * 8 * H + 12 * n
    return out


def max_over_ranks(ms: float, world: int) -> float:
    """Slowest rank's timed region (ms); every rank gets the same value."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, ms_max: float, world: int) -> float:
    """Whole-job throughput of `world` independent replicas: all ranks' units / the max time."""
    return units_per_rank * world / (ms_max / 1e3)


def run_stage(prob, local, args):
    """Iterations of the workload for a profiler: the handle with the bench's flags, --warmup +
    --steps iterations, nothing timed; prints the plans."""
    from spim_registration_gb300 import FLAG_AUTOTUNE, FLAG_TENSOR_DFT, Deconvolution

    flags = (0 if args.no_autotune else FLAG_AUTOTUNE) | (FLAG_TENSOR_DFT if args.tensor_dft else 0)
    with Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, local, flags) as dec:
        dec.run(args.warmup + args.steps)
        dec.synchronize()
        return {"workload": args.workload, "volume_xyz": list(prob.dims_xyz), "iterations": args.warmup + args.steps,
                "plans": [dec.plan(v) for v in range(len(prob.views))]}


def time_iterations(dec, stream, steps, world=1, clocks=None):
    """CUDA-event time (ms) of `steps` iterations on the handle's stream, max over ranks; the
    kernel launches issued meanwhile; the clock record if a sampler is given."""
    import torch

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.start()
        time.sleep(0.3)  # let the sampler start before the timed region
    launches0 = dec.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        dec.run_iteration()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clock_info = clocks.stop() if clocks is not None else None
    return max_over_ranks(ms, world), dec.launch_count() - launches0, clock_info


def accuracy_vs_fp64(dec, prob, device, iterations=10):
    """Error of the handle's own tile plans against the FP64 oracle, after the timed region: psi
    is reset to the first-iteration average, `iterations` iterations run, and the result is
    compared with the oracle's float64 deconvolution of the same inputs (the oracle's torch
    restatement on this GPU; the check, not the thing measured)."""
    import torch

    from oracle import fp64_torch as T

    dec.set_psi(np.full(prob.views[0].shape, np.float32(dec.initial_average()), dtype=np.float32))
    dec.run(iterations)
    got = dec.get_psi()
    got_masked = dec.get_psi(masked=True)
    ref = T.Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, device=f"cuda:{device}")
    ref.run(iterations)
    e = T.errors(got, ref.psi)
    em = T.errors(got_masked, ref.masked_psi())
    del ref
    torch.cuda.empty_cache()
    return {"iterations": iterations, "rel_l2": e["rel_l2"], "max_abs": e["max_abs"],
            "max_abs_rel_to_max": e["max_abs_rel"], "rel_l2_masked": em["rel_l2"], "gate": 1e-4,
            "passes": e["rel_l2"] <= 1e-4,
            "oracle": "FP64 restatement of the reference loop (one whole-image block, float64 FFTs)"}


def plain_form(prob, block, local, steps):
    """The plain FP32 form: the reference's block structure (MVDeconFFT.java:128-165: the given
    block size, or one block of image + kernel - 1), one block per launch sequence (copy, three
    FFT passes, paste), separate quotient and update kernels, no graph."""
    import torch

    from spim_registration_gb300 import FLAG_PLAIN, Deconvolution

    plain = Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, local, FLAG_PLAIN, block)
    pstream = torch.cuda.ExternalStream(plain.stream(), device=local)
    plain.run_iteration()
    plain.synchronize()
    pms, _, _ = time_iterations(plain, pstream, steps)
    psi = plain.get_psi()
    plans = [plain.plan(v) for v in range(len(prob.views))]
    plain.close()
    return pms / steps, psi, plans


def run_ours(args, rank, world, local):
    import torch

    from spim_registration_gb300 import FLAG_AUTOTUNE, FLAG_TENSOR_DFT, Deconvolution
    from spim_registration_gb300 import native

    torch.cuda.set_device(local)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    prob = make_problem(args.workload, args.volume)
    if args.only == "stage":
        return run_stage(prob, local, args)
    if args.only:
        part = {"inputs": ("input_preparation", run_inputs), "separable": ("separable_convolution", run_separable)}
        key, fn = part[args.only]
        return {"workload": args.workload, key: fn(prob, local, hbm_peak)}
    n_vox = prob.n_voxels
    V = len(prob.views)
    native.load()

    flags = (0 if args.no_autotune else FLAG_AUTOTUNE) | (FLAG_TENSOR_DFT if args.tensor_dft else 0)
    dec = Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, local, flags)
    stream = torch.cuda.ExternalStream(dec.stream(), device=local)

    # warm-up (captures the graph on the first iteration)
    for _ in range(args.warmup):
        dec.run_iteration()
    dec.synchronize()
    ms, launches, clock_info = time_iterations(dec, stream, args.steps, world, ClockSampler(local))
    ms_per_step = ms / args.steps
    value = replica_value(n_vox * V * args.steps, ms, world)

    # per-pass device time (CUDA events on the library's stream) for the roofline
    prof = dec.profile_iteration()
    algo = reference_block_bytes(prob, WORKLOADS[args.workload][3])  # the byte contract
    tile = bytes_per_iteration(dec, V, n_vox)  # bytes of the tiles actually transformed
    dom = max(("plane_fwd", "zpass", "plane_inv_quotient", "plane_inv_update"), key=lambda k: prof[k][0])
    dom_ms, dom_launches = prof[dom]
    achieved = algo[dom] / (dom_ms / 1e3) / 1e9
    per_pass = {k: {"ms": round(prof[k][0], 4), "launches": prof[k][1],
                    "gbs": round(algo[k] / (prof[k][0] / 1e3) / 1e9, 1) if k in algo and prof[k][0] > 0 else None,
                    "gbs_tile_bytes": round(tile[k] / (prof[k][0] / 1e3) / 1e9, 1)
                    if k in tile and prof[k][0] > 0 else None}
                for k in prof}
    iter_bytes = sum(algo.values())
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(args.workload, {}).get(dom)
        except Exception:
            traffic = None
    plans = [dec.plan(v) for v in range(V)]

    out = {
        "metric": METRIC,
        "value": value,
        "unit": "voxel-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded blobs, Poisson noise, rotated Gaussian PSFs)",
        "config": {"workload": args.workload, "views": V, "volume_xyz": list(prob.dims_xyz),
                   "psf_xyz": [list(p.shape[::-1]) for p in prob.psfs], "psftype": "EFFICIENT_BAYESIAN",
                   "lambda": prob.lam, "step": "one iteration over all views",
                   "plans": plans, "flags": "planner default tiles" if args.no_autotune else "autotuned tile plans",
                   "l2": "working set per iteration > 129 MB L2 (no flush needed)",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": launches,
        "clocks": clock_info,
        "per_pass": per_pass,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_launch": algo[dom] / max(dom_launches, 1),
                     "bytes_model": "the reference's block structure (one block of image + kernel - 1 per view, "
                                    "or the workload's block size): forward pass 4 P + 8 H per block and "
                                    "convolution; the padding of this library's tiles is not credited",
                     "avg_launch_ms": dom_ms / max(dom_launches, 1), "traffic": traffic,
                     "tile_bytes_per_launch": tile[dom] / max(dom_launches, 1),
                     "frac_with_tile_bytes": tile[dom] / (dom_ms / 1e3) / 1e9 / hbm_peak,
                     "iteration": {"bytes": iter_bytes, "achieved": iter_bytes / (ms_per_step / 1e3) / 1e9,
                                   "frac": iter_bytes / (ms_per_step / 1e3) / 1e9 / hbm_peak}},
    }
    if args.tensor_dft:
        out["config"]["flags"] += ", middle DFT stages of the 320 / 288 z passes on the tensor cores"
    if rank == 0 and not args.no_accuracy:
        out["accuracy_vs_fp64"] = accuracy_vs_fp64(dec, prob, local, iterations=10)
    dec.close()
    if rank == 0 and not args.no_tensor_dft and not args.tensor_dft:
        out["tensor_dft"] = run_tensor_dft(prob, local, flags, value, args)

    if rank == 0 and not args.no_plain:
        _, _, _, block = WORKLOADS[args.workload]
        psteps = max(1, min(3, args.steps))
        pms, ppsi, pplans = plain_form(prob, block, local, psteps)
        pvalue = n_vox * V / (pms / 1e3)
        # the fused form after the same iterations (1 + psteps), default plans
        fused = Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, local, 0)
        fused.run(1 + psteps)
        f = fused.get_psi()
        fused.close()
        out["plain_fp32_form"] = {
            "value": pvalue, "ms_per_step": pms, "steps": psteps,
            "block_xyz": block if block is not None else "one block of image + kernel - 1 per view",
            "plans": pplans, "speedup_of_value": value / world / pvalue,
            "rel_l2_fused_vs_plain": float(np.linalg.norm(f - ppsi) / np.linalg.norm(ppsi))}

    if rank == 0 and not args.no_e2e:
        out["e2e"] = run_e2e(prob, local)
    if rank == 0:
        out["input_preparation"] = run_inputs(prob, local, hbm_peak)
        out["separable_convolution"] = run_separable(prob, local, hbm_peak)
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(prob)
    if rank == 0 and not args.no_psf_refine:
        out["psf_refinement"] = run_psf_refinement(local)
    if rank == 0 and not args.no_secondary:
        del prob
        out["workloads"] = {w: run_secondary(w, local, args) for w in SECONDARY_WORKLOADS if w != args.workload}
    return out


def run_tensor_dft(prob, local, flags, simt_value, args, steps=50):
    """The same workload with the middle 16-point DFTs of the 320- and 288-long z passes on the
    tensor cores (tcgen05 TF32 products, three-term hi/lo split, FP32 accumulation): its value,
    and its error against the FP64 oracle after 10 and 50 iterations (relative L2 and max-abs of
    the output volume, psi)."""
    import torch

    from spim_registration_gb300 import FLAG_TENSOR_DFT, Deconvolution

    V, n_vox = len(prob.views), prob.n_voxels
    dec = Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, local, flags | FLAG_TENSOR_DFT)
    stream = torch.cuda.ExternalStream(dec.stream(), device=local)
    for _ in range(3):
        dec.run_iteration()
    dec.synchronize()
    ms, launches, _ = time_iterations(dec, stream, steps)
    dec.synchronize()  # reports any tensor-core stage whose bounded wait gave up
    value = n_vox * V * steps / (ms / 1e3)
    prof = dec.profile_iteration()
    res = {"value": value, "unit": "voxel-updates/s", "ms_per_step": ms / steps, "steps": steps,
           "value_over_fp32_simt": value / simt_value, "zpass_ms": prof["zpass"][0],
           "plans": [dec.plan(v) for v in range(V)]}
    if not args.no_accuracy:
        from oracle import fp64_torch as T

        dec.set_psi(np.full(prob.views[0].shape, np.float32(dec.initial_average()), dtype=np.float32))
        ref = T.Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, device=f"cuda:{local}")
        done = 0
        for it in (10, 50):
            dec.run(it - done)
            ref.run(it - done)
            done = it
            e = T.errors(dec.get_psi(), ref.psi)
            res[f"accuracy_vs_fp64_{it}_iterations"] = {"rel_l2": e["rel_l2"], "max_abs": e["max_abs"],
                                                        "max_abs_rel_to_max": e["max_abs_rel"]}
        dec.synchronize()
        del ref
        torch.cuda.empty_cache()
    dec.close()
    return res


def run_psf_refinement(local, steps=10):
    """PSF refinement from bead data at full size: 4 views of 192^3 with 500 point-like beads
    (sigma 0.7, peak U[500, 2000]), PSF 31x31x61 (sigma 2, 2, 7) rotated per view, every PSF
    started 20% too wide; projected gradient steps on the Poisson NLL (mvd_forward /
    mvd_backward / mvd_set_kernel) at the bead image.  Reports the NLL and the PSFs' relative
    L2 distance to the true PSFs before and after, and the time of the gradient (mvd_backward)
    and of a whole step (gradient plus the line searches' NLL evaluations)."""
    import torch

    from spim_registration_gb300 import synthetic as S
    from spim_registration_gb300.psf_refine import PSFRefinement

    prob = S.make_problem(5)
    sigma = (2.0, 2.0, 7.0)
    angles = (0, 45, 90, 135)
    wide = [S.gaussian_psf(tuple(1.2 * x for x in sigma), (31, 31, 61), a) for a in angles]
    true = [q.astype(np.float64) / q.sum() for q in prob.psfs]
    with PSFRefinement(prob.views, prob.weights, wide, prob.ground_truth, local) as r:
        dist0 = [float(np.linalg.norm(q - t) / np.linalg.norm(t)) for q, t in zip(r.psfs, true)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.dec.backward()
        t_grad = time.perf_counter() - t0
        t0 = time.perf_counter()
        r.run(steps)
        t_steps = time.perf_counter() - t0
        dist1 = [float(np.linalg.norm(q - t) / np.linalg.norm(t)) for q, t in zip(r.psfs, true)]
        nll = [h.nll for h in r.history]
        backtracks = sum(h.backtracks for h in r.history)
    return {"workload": "4 views of 192^3, 500 beads, PSF 31x31x61 started 20% too wide",
            "steps": steps, "nll_start": nll[0], "nll_end": nll[-1],
            "nll_monotone": all(b <= a for a, b in zip(nll, nll[1:])),
            "psf_rel_l2_to_truth_start": dist0, "psf_rel_l2_to_truth_end": dist1,
            "gradient_ms": t_grad * 1e3, "ms_per_step": t_steps / steps * 1e3, "line_search_backtracks": backtracks,
            "note": "gradient = mvd_backward over all views with each blur recomputed tile by tile, including the "
                    "host copies of the gradients; a step adds the NLL evaluations of the line search"}


def run_secondary(workload, local, args):
    """Another workload (15x15x41 PSFs, the reference's 128^3 blocks for the plain form): the
    4-view 256x256x192 one, or six views cropped to random boxes in a 256^3 volume (uneven tile
    grids per view); fused value with autotuned plans, the plain form's value and the FP64
    error."""
    import torch

    from spim_registration_gb300 import FLAG_AUTOTUNE, Deconvolution

    prob = make_problem(workload)
    V, n_vox = len(prob.views), prob.n_voxels
    dec = Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, local,
                        0 if args.no_autotune else FLAG_AUTOTUNE)
    stream = torch.cuda.ExternalStream(dec.stream(), device=local)
    for _ in range(5):
        dec.run_iteration()
    dec.synchronize()
    steps = 100
    ms, launches, _ = time_iterations(dec, stream, steps)
    value = n_vox * V * steps / (ms / 1e3)
    res = {"value": value, "unit": "voxel-updates/s", "ms_per_step": ms / steps, "steps": steps,
           "gpu_launches": launches, "plans": [dec.plan(v) for v in range(V)]}
    if not args.no_accuracy:
        res["accuracy_vs_fp64"] = accuracy_vs_fp64(dec, prob, local, iterations=10)
    dec.close()
    if not args.no_plain:
        block = WORKLOADS[workload][3]
        pms, _, _ = plain_form(prob, block, local, 3)
        res["plain_fp32_form"] = {"value": n_vox * V / (pms / 1e3), "ms_per_step": pms, "block_xyz": block,
                                  "speedup_of_value": value / (n_vox * V / (pms / 1e3))}
    return res


def run_e2e(prob, device, steps=5):
    """Whole job through the C ABI with host buffers: upload (pinned), kernel preparation,
    all iterations, masked psi back to the host; autotuned plans (from the process's cache).
    `steps` jobs after one untimed job; the value is from the median job.  The host-device
    copies of a job (2.15 GB in, 268 MB out on the 512x512x256 workload) usually run at about
    210 / 190 GB/s, but now and then a copy window runs at 15-30 GB/s, for plain torch copies of
    the same pinned buffers as well; every job's time is listed."""
    import torch

    from spim_registration_gb300 import FLAG_AUTOTUNE, Deconvolution

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    views = [pinned(v) for v in prob.views]
    weights = [pinned(w) for w in prob.weights]
    psfs = [np.ascontiguousarray(p) for p in prob.psfs]
    h2d = sum(v.nbytes for v in views) + sum(w.nbytes for w in weights) + sum(p.nbytes for p in psfs)
    d2h = prob.views[0].nbytes
    out = pinned(np.zeros(prob.views[0].shape, dtype=np.float32))  # the result lands in pinned memory too
    times = []
    for i in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d = Deconvolution(views, weights, psfs, prob.psftype, prob.lam, device, FLAG_AUTOTUNE)
        d.run(prob.iterations)
        psi = d.get_psi(masked=True, out=out)
        t1 = time.perf_counter()
        d.close()
        if i > 0:  # the first job pays the one-time CUDA context / module load
            times.append(t1 - t0)
        del psi
    t = float(np.median(times))
    return {"value": prob.n_voxels * len(prob.views) * prob.iterations / t, "unit": "voxel-updates/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "seconds_per_job": t,
            "job_ms": [round(1e3 * x, 2) for x in times], "value_from": f"median of {len(times)} jobs",
            "step": f"one whole job: upload + kernel prep + {prob.iterations} iterations + masked psi download",
            "host_buffers": "pinned (inputs and the result)",
            "plans": "autotuned; the choice is cached per geometry in the process, so only the first "
                     "(untimed) job of a geometry pays for the timing runs"}


def run_inputs(prob, device, hbm_peak, reps=5):
    """Input preparation on the device at the workload's size: every view (raw stack of the
    fused box's size, rotated about y by 180 v / V degrees with a fractional shift) resampled
    with its blending weight, the overlap statistics and the VIRTUAL normalisation with the
    average-overlap OSEM factor.  Algorithmic bytes: resample 4 (view) + 8 (image, weight)
    per voxel and view; overlap 4 per voxel and view; normalisation 8 per voxel and view.
    The resample and normalisation launches queue behind a short device-side sleep, so their
    events time the kernels, not the host's launch overhead."""
    import math

    import torch

    from spim_registration_gb300 import WeightNormalizer, transform_input

    nz, ny, nx = prob.views[0].shape
    V = len(prob.views)
    n = nx * ny * nz
    raw = [torch.from_numpy(np.ascontiguousarray(v)).to(f"cuda:{device}") for v in prob.views]
    cx, cy, cz = (nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2
    affines = []
    for v in range(V):
        t = math.radians(180.0 * v / V)
        c, s_ = math.cos(t), math.sin(t)
        shift = (cx - (c * cx + s_ * cz) + 0.25, 0.375, cz - (-s_ * cx + c * cz) + 0.125)
        affines.append([c, 0, s_, shift[0], 0, 1, 0, shift[1], -s_, 0, c, shift[2]])
    border, blend = (0.0, 0.0, 0.0), (20.0, 20.0, 20.0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    ms = np.zeros(3)
    for r in range(reps + 1):
        torch.cuda.synchronize()
        torch.cuda._sleep(4_000_000)  # about 2 ms: the host queues the launches meanwhile
        ev[0].record()
        outs = [transform_input(raw[v], affines[v], (0, 0, 0), (nz, ny, nx), border, blend, device) for v in range(V)]
        ev[1].record()
        wn = WeightNormalizer([o[1] for o in outs], num_portions=32)
        wn.process()  # waits for the stream: returns the statistics to the host
        ev[2].record()
        torch.cuda._sleep(1_000_000)
        ev[3].record()
        wn.apply(wn.osem_speedup(2))
        ev[4].record()
        torch.cuda.synchronize()
        if r:
            ms += [ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]), ev[3].elapsed_time(ev[4])]
        del outs, wn
    ms /= reps
    algo = [12.0 * n * V, 4.0 * n * V, 8.0 * n * V]
    names = ["transform_view", "weight_overlap", "normalize_weights"]
    res = {k: {"ms": round(float(t), 4), "gbs": round(b / (t / 1e3) / 1e9, 1),
               "frac_of_measured_hbm": round(b / (t / 1e3) / 1e9 / hbm_peak, 3)} for k, t, b in zip(names, ms, algo)}
    res["views"] = V
    res["box_xyz"] = [nx, ny, nz]
    res["total_ms"] = round(float(ms.sum()), 4)
    res["note"] = "weight_overlap includes its device-to-host read of the statistics"
    return res


def run_separable(prob, device, hbm_peak, reps=10):
    """The difference-of-Gaussian detector's separable convolution at the workload's volume
    size: x, y and z passes with K-tap kernels, device-resident (algorithmic bytes: 8 per voxel
    and pass), and the JNA call convolve_K on a host array (copies in and out included)."""
    import torch

    from spim_registration_gb300 import native
    from spim_registration_gb300.separable import CUDASeparableConvolution

    nz, ny, nx = prob.views[0].shape
    n = nx * ny * nz
    lib = native.load()
    a = torch.from_numpy(np.ascontiguousarray(prob.views[0])).to(f"cuda:{device}")
    b = torch.empty_like(a)
    stream = torch.cuda.current_stream(device)
    res = {"volume_xyz": [nx, ny, nz], "passes": 3}
    for K in (15, 127):
        ks = [np.exp(-0.5 * ((np.arange(K) - K // 2) / (K / 6.0)) ** 2).astype(np.float32) for _ in range(3)]
        kp = (native._F * 3)(*[native.fptr(k) for k in ks])
        out = native.ctypes.c_void_p()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def run():
            native.check(lib.mvd_separable_convolve_device(a.data_ptr(), b.data_ptr(), kp, native.iarr([K, K, K]),
                                                           native.iarr([nx, ny, nz]), 2, 0.0, device,
                                                           native.ctypes.c_void_p(stream.cuda_stream),
                                                           native.ctypes.byref(out)))
        run()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        gbs = 24.0 * n / (ms / 1e3) / 1e9
        host = np.ascontiguousarray(prob.views[0]).reshape(-1).copy()
        cuda = CUDASeparableConvolution()
        getattr(cuda, f"convolve_{K}")(host, *ks, nx, ny, nz, True, True, True, 2, 0.0, device)
        t0 = time.perf_counter()
        for _ in range(3):
            getattr(cuda, f"convolve_{K}")(host, *ks, nx, ny, nz, True, True, True, 2, 0.0, device)
        t_host = (time.perf_counter() - t0) / 3
        res[f"K{K}"] = {"device_ms": round(ms, 4), "gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / hbm_peak, 3),
                        "voxels_per_s": n / (ms / 1e3), "jna_call_ms": round(t_host * 1e3, 3),
                        "jna_voxels_per_s": n / t_host}
    res["note"] = "device: 3 passes, 8 B per voxel and pass; jna_call: pageable host array in and out"
    return res


def cpu_view_stage_time(prob, min_seconds=10.0, max_stages=64):
    """Mean time of the reference algorithm's view stages on the host cores (oracle port,
    float32): after one warm-up stage, stages over the views in turn until at least
    ``min_seconds`` of work (at most ``max_stages`` stages).  Returns (seconds per stage,
    stages, total seconds)."""
    from oracle import mvdecon_oracle as O

    d = O.Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, arith="f32")
    V = len(prob.views)
    d.run_view(0)  # warm (FFT plans, page-in)
    n, t0 = 0, time.perf_counter()
    while True:
        d.run_view((1 + n) % V)
        n += 1
        t = time.perf_counter() - t0
        if t >= min_seconds or n >= max_stages:
            return t / n, n, t


def host_cores():
    """Cores this process may run on (the GPU machine's host cores visible to it)."""
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count()


def cpu_baseline(prob):
    per, n, total = cpu_view_stage_time(prob)
    return {"value": prob.n_voxels / per, "unit": "voxel-updates/s", "cores": host_cores(), "kind": "port",
            "sample": f"{n} view stages (conv1, quotient, conv2, update) of the same workload, each convolution "
                      f"over one whole-image block (the reference's single-block structure for this workload), "
                      f"float32, scipy.fft with {_workers_note()}; {total:.1f} s"}


def _workers_note():
    return f"{os.cpu_count()} workers on the {host_cores()} host cores visible to this process"


def run_reference(args, rank, world):
    if rank != 0:
        return None
    prob = make_problem(args.workload)
    from oracle import mvdecon_oracle as O

    d = O.Deconvolution(prob.views, prob.weights, prob.psfs, prob.psftype, prob.lam, arith="f32")
    V = len(prob.views)
    for i in range(args.warmup):
        d.run_view(i % V)
    # the timed region stops early once it has run REFERENCE_MAX_SECONDS, so a large --steps
    # still ends within a few minutes; the line reports the steps that ran
    steps, t0 = 0, time.perf_counter()
    while steps < args.steps:
        d.run_view(steps % V)
        steps += 1
        if time.perf_counter() - t0 >= REFERENCE_MAX_SECONDS:
            break
    t = time.perf_counter() - t0
    value = prob.n_voxels * steps / t
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "voxel-updates/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": t / steps * 1e3 if steps else 0.0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded blobs, Poisson noise, rotated Gaussian PSFs)",
        "config": {"workload": args.workload, "views": V, "volume_xyz": list(prob.dims_xyz),
                   "step": "one view stage (conv1, quotient, conv2, update) on the host cores"},
        "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": host_cores(), "kind": "port",
                         "sample": f"{steps} view stages of the workload ({args.steps} asked, at most "
                                   f"{REFERENCE_MAX_SECONDS:.0f} s timed), CPU restatement of the Java "
                                   "MVDeconvolution/MVDeconFFT loop (float32, one whole-image block per "
                                   f"convolution, scipy.fft with {_workers_note()}); the Java "
                                   "reference needs a JDK and its Maven jars, absent on this machine"},
        "e2e": {"value": value, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.steps > 0 and args.warmup < 0:
        raise SystemExit("bad warmup")
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
