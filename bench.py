"""Benchmark of the fused sequential raytrace on one GB300 (or N replicas).

Workload (default): the precision form -- the Newtonian telescope (parabolic
primary R = -800 mm behind a 12 mm obscuration, 45 degree fold, 1024^2 sensor
of 13.5 um pixels) with both mirrors Al-coated (substrate Fresnel from a
seeded 3-point complex index table), 1e8 rays per GPU: field uniform in the
+-0.15 deg square, pupil uniform on the 12-50 mm annulus, wavelength uniform
on 400-700 nm.  One step = ``rayfunction`` with sensor binning: every ray
through the 5 surfaces (object, obscuration, primary, fold, sensor), outputs
position, direction, intensity, OPL and mask in the sensor frame, plus the
count and flux images.  Metric: rays*surfaces/s.

``value`` times the kernel with inputs resident in HBM; ``e2e`` times the
public ``SequentialSystem.rayfunction`` call from pinned host arrays, whose
zero-copy launch reads the inputs and writes every output over NVLink-C2C
inside the timed region, with the images copied to the host.
``--impl reference`` times the CPU path (the float64 NumPy restatement of
the reference's trace, all host cores) on a bounded sample.

The same line carries ``error``: every output of the first 1e6 of the
timed rays against the float64 oracle (the exact solution of the
reference's equations, and the reference's closed forms as written), and
``workloads``: the batched, multilayer and learned forms at their
configured sizes (``--workload <name>`` runs one of them alone).

Multi-GPU: rays are independent, so each rank traces its own 1e8 rays with
no collective on the data path (weak scaling); value = all ranks' work over
the slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import pathlib
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "rays*surfaces/s (fused FP32 sequential raytrace, precision form)"
UNIT = "rays*surfaces/s"
NUM_SURFACES = 5

# Algorithmic bytes of one ray of this workload: the kernel reads the five
# float32 inputs (wavelength, field x/y, pupil x/y: 20 B) and writes the
# float32 position and direction (24 B), float32 intensity (4 B), float64
# optical path length (8 B) and the uint8 mask (1 B); the sensor images
# (8 MB) are L2-resident atomics.  Its algorithmic arithmetic per ray is
# counted by oracle/flops.py over the reference's own formulas (non-trivial
# real operations only) and frozen in profiles/trace_precision_1e8.json.
BYTES_PER_RAY = 5 * 4 + 6 * 4 + 4 + 8 + 1
ERROR_RAYS = 1_000_000


def _cpu_worker(args):
    """One bounded chunk of the CPU baseline (float64 NumPy restatement)."""
    n, seed = args
    sys.path.insert(0, str(ROOT))
    from optika_gb300 import configs
    from oracle import trace as O

    system = configs.newtonian(coated=True)
    g = configs.precision_grid(n, seed=seed)
    t0 = time.perf_counter()
    r = O.rayfunction(system, g["wavelength"], g["field_x"], g["field_y"], g["pupil_x"],
                      g["pupil_y"])
    O.collect(system.sensor, r)
    return n, time.perf_counter() - t0


def _error_worker(args):
    """Oracle outputs of one interleaved chunk of the error sample."""
    grid, exact = args
    sys.path.insert(0, str(ROOT))
    from optika_gb300 import configs
    from oracle import trace as O

    system = configs.newtonian(coated=True)
    r = O.rayfunction(system, grid["wavelength"], grid["field_x"], grid["field_y"],
                      grid["pupil_x"], grid["pupil_y"], exact=exact)
    return {k: r[k] for k in ("px", "py", "dx", "dy", "dz", "intensity", "opl", "unvignetted")}


def precision_errors(grid: dict, out: dict, cores: int) -> dict:
    """Per-output errors of the GPU's rays ``out`` against the float64
    oracle on the same (float32) inputs ``grid``: the exact solution of the
    reference's equations and, for position, its closed forms as written."""
    import concurrent.futures
    import multiprocessing as mp

    from optika_gb300 import configs
    from oracle import trace as O

    n = len(grid["wavelength"])
    parts = [{k: v[i::cores] for k, v in grid.items()} for i in range(cores)]
    refs = {}
    ctx = mp.get_context("spawn")
    with concurrent.futures.ProcessPoolExecutor(max_workers=cores, mp_context=ctx) as ex:
        for exact in (True, False):
            res = list(ex.map(_error_worker, [(p, exact) for p in parts]))
            ref = {}
            for k in res[0]:
                a = np.empty(n, res[0][k].dtype)
                for i in range(cores):
                    a[i::cores] = res[i][k]
                ref[k] = a
            refs[exact] = ref
    ex_, lit = refs[True], refs[False]
    m = ex_["unvignetted"]
    pix = 0.0135
    e = np.hypot(out["px"][m] - ex_["px"][m], out["py"][m] - ex_["py"][m])
    e_lit = np.hypot(out["px"][m] - lit["px"][m], out["py"][m] - lit["py"][m])
    d_opl = np.abs(out["opl"][m] - ex_["opl"][m])
    ex_edges, ey_edges = O.histogram_edges(configs.newtonian(coated=True).sensor)
    fx = (ex_["px"][m] - ex_edges[0]) / pix
    fy = (ex_["py"][m] - ey_edges[0]) / pix
    far = (np.abs(fx - np.round(fx)) > 1e-3) & (np.abs(fy - np.round(fy)) > 1e-3)
    pix_mis = np.count_nonzero(
        (O.bin_index(ex_edges, out["px"][m][far]) != O.bin_index(ex_edges, ex_["px"][m][far]))
        | (O.bin_index(ey_edges, out["py"][m][far]) != O.bin_index(ey_edges, ex_["py"][m][far])))
    return {
        "rays": n, "reference": "float64 oracle, exact solution of the reference's equations",
        "mask_mismatches": int(np.count_nonzero(out["unvignetted"] != m)),
        "position_max_mm": float(e.max()), "position_max_px": float(e.max() / pix),
        "position_rms_mm": float(np.sqrt(np.mean(e**2))),
        "position_max_mm_vs_literal_formulas": float(e_lit.max()),
        "pixel_mismatches_beyond_1e-3_px_of_an_edge": int(pix_mis),
        "direction_max": float(max(np.abs(out[k][m] - ex_[k][m]).max()
                                   for k in ("dx", "dy", "dz"))),
        "opl_max_mm": float(d_opl.max()), "opl_rms_mm": float(np.sqrt(np.mean(d_opl**2))),
        "intensity_rel_max": float((np.abs(out["intensity"][m] - ex_["intensity"][m])
                                    / ex_["intensity"][m]).max()),
    }


def cpu_baseline(total_rays: int, cores: int) -> tuple[float, float]:
    """Throughput (rays*surfaces/s) of the CPU path over `cores` processes."""
    import concurrent.futures
    import multiprocessing as mp

    chunk = max(1, total_rays // cores)
    ctx = mp.get_context("spawn")
    with concurrent.futures.ProcessPoolExecutor(max_workers=cores, mp_context=ctx) as ex:
        list(ex.map(_cpu_worker, [(1000, 7)] * cores))  # warm the workers
        t0 = time.perf_counter()
        res = list(ex.map(_cpu_worker, [(chunk, 100 + i) for i in range(cores)]))
        wall = time.perf_counter() - t0
    rays = sum(r[0] for r in res)
    return rays * NUM_SURFACES / wall, wall


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        import tempfile

        try:
            fd, name = tempfile.mkstemp(prefix=f"optika_clocks_{self.index}_", suffix=".csv")
            os.close(fd)
            self.path = pathlib.Path(name)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL,
            )
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        text = self.path.read_text()
        self.path.unlink(missing_ok=True)
        for line in text.splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> tuple[dict, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp32_roofline(workload: str, units: int, ms: float, pk: dict) -> dict | None:
    """The FP32 roofline of a workload from its frozen algorithmic counts
    (profiles/algorithmic_counts.json, made by oracle/freeze_counts.py):
    algorithmic flops per unit x units over the kernel's time, against the
    FP32 pipe's nominal peak at the measured maximum SM clock (152 SMs x 128
    lanes x 2 flops per FMA)."""
    p = ROOT / "profiles" / "algorithmic_counts.json"
    if not p.exists():
        return None
    c = json.loads(p.read_text()).get(workload)
    if not c:
        return None
    peak = 152 * 128 * 2 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    ach = c["flops"] * units / (ms * 1e-3) / 1e12
    return {"achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "algorithmic_flops_per_unit": c["flops"], "algorithmic_div_per_unit": c["div"],
            "algorithmic_special_per_unit": c["special"], "per": c["unit"],
            "counted_by": "oracle/flops.py via oracle/freeze_counts.py",
            "peak_kind": "nominal at the measured maximum SM clock"}


def issue_roofline(profile: str, units: int, ms: float, pk: dict, fp32: dict | None) -> dict | None:
    """The instruction-issue roofline of a kernel: the warp instructions per
    unit that ncu counted (profiles/<profile>.json) x units over the kernel's
    time, against 152 SMs x 4 schedulers x one warp instruction per cycle at
    the measured maximum SM clock."""
    p = ROOT / "profiles" / f"{profile}.json"
    if not p.exists():
        return None
    wi = float(json.loads(p.read_text())["warp_instructions_per_unit"])
    peak = 152 * 4 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    ach = wi * units / (ms * 1e-3) / 1e12
    out = {"achieved": ach, "peak": peak, "unit": "T warp-instructions/s", "frac": ach / peak,
           "warp_instructions_per_unit_ncu": wi, "counted_in": f"profiles/{profile}.json",
           "peak_kind": "nominal at the measured maximum SM clock"}
    if fp32:
        out["note"] = ("the binding resource: at full issue this instruction count would put "
                       f"roofline.fp32 at {fp32['frac'] / (ach / peak):.2f}")
    return out


def _ncu_traffic(profile: str, units: int) -> float | None:
    """DRAM bytes per launch of `units` units from a profile's ncu capture."""
    p = ROOT / "profiles" / f"{profile}.json"
    if not p.exists():
        return None
    return float(json.loads(p.read_text())["dram_bytes_per_unit"]) * units


def run_reference(args, rank: int, world: int) -> None:
    if rank != 0:
        return
    cores = len(os.sched_getaffinity(0))
    # each step: a bounded sample of the workload spread over all host cores
    per_step = args.ref_rays
    vals = []
    for i in range(args.warmup + args.steps):
        v, wall = cpu_baseline(per_step, cores)
        if i >= args.warmup:
            vals.append((v, wall))
    value = float(np.mean([v for v, _ in vals]))
    wall = float(np.mean([w for _, w in vals]))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded numpy)",
        "config": {"workload": "newtonian-precision (Al-coated mirrors, 400-700 nm)",
                   "rays_per_step": per_step, "surfaces": NUM_SURFACES},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{per_step} rays per step over {cores} processes"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_surrogate(args, rank: int, world: int, emit: bool = True) -> dict:
    """The learned form: a 9-256x4-3 BF16 MLP surrogate of the batched
    spectrograph's ray map over 64 configurations, trained on 5e7 rays the
    plain batched kernel traces, evaluated on 1e6 held-out rays, then used to
    simulate the sensor images of 1e9 rays with plain-trace fallback.  The
    same 1e9 rays through the plain batched kernel give the comparison.
    Single GPU (replicas under torchrun)."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from optika_gb300 import configs
    from optika_gb300.surrogate import RayMapSurrogate

    n_cfg = 64
    systems, _, params = configs.spectrograph_batch(n_cfg, seed=5)
    sg = RayMapSurrogate(systems, params, wavelength=configs.SPEC_WAVELENGTH,
                         field_half=configs.SPEC_FIELD_HALF, pupil_half=configs.SPEC_PUPIL_HALF,
                         seed=5)
    t0 = time.perf_counter()
    train = sg.traced(np.full(n_cfg, 50_000_000 // n_cfg), seed=5 + 1000 * rank)
    sg.fit_baseline(train)
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    t0 = time.perf_counter()
    hist = sg.train(train, steps=args.train_steps, batch=65536, lr=2e-3, log_every=500)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del train
    torch.cuda.empty_cache()
    held = sg.traced(np.full(n_cfg, 1_000_000 // n_cfg), seed=6 + 1000 * rank)
    ev = sg.evaluate(held)
    n_trusted = sg.set_trust(ev["per_config_rms_px"], 0.05)
    ev_t = sg.evaluate(held)  # with untrusted configurations routed to the trace
    del held

    per_cfg = args.image_rays // n_cfg
    img = sg.traced(np.full(n_cfg, per_cfg), seed=7 + 1000 * rank, image=True, outputs=())
    total = img.total
    for _ in range(max(1, args.warmup)):
        sg.image(img, chunk=args.image_chunk or None, fused=args.image_path == "fused")
        img.run()
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    _, stats = sg.image(img, chunk=args.image_chunk or None, fused=args.image_path == "fused")
    e1.record()
    sim = img.images.clone()
    e2.record()
    torch.cuda.synchronize()
    ms_sur = e0.elapsed_time(e1)
    st = stats.cpu().numpy()
    p0, p1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    p0.record()
    img.run()
    p1.record()
    torch.cuda.synchronize()
    ms_plain = p0.elapsed_time(p1)
    ref = img.images
    flux_err = abs(float(sim.sum()) - float(ref.sum())) / float(ref.sum())
    l1 = float((sim.double() - ref.double()).abs().sum()) / float(ref.sum())
    surfaces = 4
    # the network's algorithmic work per ray: 2 (9 x 256 + 3 x 256^2 + 256 x 3)
    flops_per_ray = 2 * (9 * 256 + 3 * 256 * 256 + 256 * 3)
    pk, pk_kind = peaks()
    ach = flops_per_ray * total / (ms_sur * 1e-3) / 1e12
    roofline = {
        "bound": "tensor", "achieved": ach, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
        "frac": ach / pk["bf16_tflops"], "traffic": None, "peak_kind": pk_kind + " bf16 burst",
        "kernel": "k_surrogate_fused (+ k_surrogate_fallback for the traced rays, one call)",
        "kernel_ms": ms_sur, "flops_per_ray": flops_per_ray,
        "l2_weight_bytes_per_ray": 1550,
    }
    line = {
        "metric": "rays*surfaces/s (image simulation: MLP surrogate + traced fallback vs plain "
                  "FP32 trace)",
        "value": total * surfaces / (ms_sur * 1e-3),
        "unit": "rays*surfaces/s",
        "n_gpus": world,
        "higher_is_better": True,
        "dtype": "bf16 (network), f32 (trace)",
        "data": "synthetic (seeded Philox rays on the device)",
        "config": {"workload": "spectrograph-surrogate", "configs": n_cfg,
                   "image_path": args.image_path,
                   "train_rays": 50_000_000, "held_out_rays": 1_000_000, "image_rays": total,
                   "network": "9-256-256-256-256-3 SiLU, BF16 weights, FP32 accumulation"},
        "plain_trace": {"value": total * surfaces / (ms_plain * 1e-3), "ms": ms_plain},
        "surrogate_ms": ms_sur,
        "speedup_vs_plain": ms_plain / ms_sur,
        "roofline": roofline,
        "gpu_launches": 2,
        "held_out": {k: ev[k] for k in ("rms_px", "p999_px", "max_px", "baseline_rms_px",
                                        "baseline_p999_px", "fallback_fraction",
                                        "efficiency_rel_error", "false_pass", "false_block")},
        "held_out_after_trust": {k: ev_t[k] for k in ("rms_px", "p999_px", "fallback_fraction",
                                                      "efficiency_rel_error")},
        "trusted_configs": n_trusted,
        "image": {"rays": int(st[0]), "traced": int(st[1]), "binned_by_network": int(st[2]),
                  "binned_by_trace": int(st[3]), "flux_rel_error_vs_plain": flux_err,
                  "l1_rel_diff_vs_plain": l1},
        "training": {"steps": args.train_steps, "batch": 65536, "seconds": t_train,
                     "fit_seconds": t_fit, "last": hist[-1]},
    }
    if emit and rank == 0:
        print(json.dumps(line), flush=True)
    return line


_BATCH_PARAMS = None


def _cpu_batched_worker(args):
    """One bounded chunk of the batched workload's CPU baseline: n rays of
    configuration c through the float64 oracle, binned."""
    c, n, seed = args
    sys.path.insert(0, str(ROOT))
    from optika_gb300 import configs
    from oracle import batch as OB
    from oracle import trace as O

    global _BATCH_PARAMS
    if _BATCH_PARAMS is None:  # the 4096 configurations the GPU traces
        _BATCH_PARAMS = configs.spectrograph_batch(4096, seed=seed)[2]
    s = configs.spectrograph(*_BATCH_PARAMS[c])
    g = OB.batch_inputs(seed, c, n, *configs.SPEC_WAVELENGTH, *configs.SPEC_FIELD_HALF,
                        configs.SPEC_PUPIL_HALF)
    t0 = time.perf_counter()
    r = O.rayfunction(s, *(g[k].astype(np.float64) for k in ("wavelength", "field_x", "field_y",
                                                             "pupil_x", "pupil_y")))
    O.collect(s.sensor, r)
    return n, time.perf_counter() - t0


def _cpu_pool(worker, jobs, cores):
    import concurrent.futures
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with concurrent.futures.ProcessPoolExecutor(max_workers=cores, mp_context=ctx) as ex:
        list(ex.map(worker, jobs[:cores]))  # warm the workers
        t0 = time.perf_counter()
        res = list(ex.map(worker, jobs))
        wall = time.perf_counter() - t0
    return sum(r[0] for r in res), wall


def run_batched(args, rank: int, world: int, emit: bool = True) -> dict:
    """The batched form: 4096 spectrograph configurations (spherical primary,
    toroidal VLS grating, 2048 x 1024 sensor), log-uniform 1e3-1e6 rays each,
    generated on the device and traced in one persistent launch with
    per-configuration sensor images; tile and rays-per-thread from the
    autotuner; one step replayed as a CUDA graph.  Replicas under torchrun."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from optika_gb300 import batch, configs

    n_cfg = args.configs
    systems, counts, _ = configs.spectrograph_batch(n_cfg, seed=3)
    bt = batch.BatchedTrace(systems, overrides=[2, 3], ray_counts=counts, seed=3 + 1000 * rank,
                            wavelength=configs.SPEC_WAVELENGTH,
                            field_half=configs.SPEC_FIELD_HALF,
                            pupil_half=configs.SPEC_PUPIL_HALF, image=True,
                            outputs=("px", "py", "unvignetted"))
    choice = bt.tune()
    graph = bt.graph()
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0.record()
    for _ in range(args.steps):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    total = int(bt.total)
    surfaces = 4
    value = world * total * surfaces / (ms * 1e-3)
    # bytes per ray: 9 B of outputs (px, py, mask) and one 4-byte image
    # count; no input traffic (rays generated on the device)
    bpr = 13
    pk, pk_kind = peaks()
    ach = bpr * total / (ms * 1e-3) / 1e9
    fp32 = fp32_roofline("batched-spectrograph", total, ms, pk)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        jobs = [(c, 400000, 3) for c in range(0, 4 * cores)]
        n, wall = _cpu_pool(_cpu_batched_worker, jobs, cores)
        cpu = {"value": n * surfaces / wall, "unit": "rays*surfaces/s", "cores": cores,
               "kind": "port", "sample": f"{len(jobs)} configurations x 400000 rays ({wall:.1f} s)"}
    line = {
            "metric": "rays*surfaces/s (batched spectrograph configurations, one persistent "
                      "launch)",
            "value": value, "unit": "rays*surfaces/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Philox rays on the device)",
            "config": {"workload": "spectrograph-batched", "configs": n_cfg, "rays": total,
                       "surfaces": surfaces, "sensor": "2048x1024 x 13.5um per configuration",
                       "schedule": {"tile": choice[0], "rays_per_thread": choice[1]},
                       "cuda_graph": True},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": ach / pk["hbm_gbs"],
                         "traffic": _ncu_traffic("trace_batch_spectrograph_256cfg", total),
                         "peak_kind": pk_kind,
                         "bytes_per_ray": bpr, "kernel": "k_trace_batch (spectrograph shape)",
                         "kernel_ms": ms, "fp32": fp32, "issue": issue_roofline(
                             "trace_batch_spectrograph_256cfg", total, ms, pk, fp32),
                         "note": "compute-bound (instruction issue): the byte roofline is "
                                 "shown for completeness; traffic scaled from the 256-"
                                 "configuration capture by rays"},
            "cpu_baseline": cpu, "gpu_launches": 3, "clocks": clk,
    }
    if emit and rank == 0:
        print(json.dumps(line), flush=True)
    return line


def _cpu_multilayer_worker(args):
    c, n, seed = args
    sys.path.insert(0, str(ROOT))
    from oracle import trace as O

    mirrors = _mirrors(seed, c + 1)
    rng = np.random.default_rng(1000 + c)
    wl = rng.uniform(12.0, 15.0, n)
    cos = np.cos(rng.uniform(0.0, 20.0 * math.pi / 180.0, n))
    m = mirrors[c]
    t0 = time.perf_counter()
    O.multilayer_efficiency(wl, cos, 1.0, m.layers, m.substrate)
    return n, time.perf_counter() - t0


def _mirrors(seed: int, count: int):
    """Periodic bilayer mirrors of the multilayer workload: period U(9.5,
    10.5) nm, thickness ratio 0.4, indices 1 - delta + i beta with delta
    log-uniform in [1e-3, 1e-1] and beta in [1e-4, 1e-2]."""
    import optika_gb300 as ok

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = rng.uniform(9.5, 10.5)

        def idx():
            delta = 10 ** rng.uniform(-3, -1)
            beta = 10 ** rng.uniform(-4, -2)
            z = 1 - delta + 1j * beta
            return complex(np.float32(z.real), np.float32(z.imag))

        out.append(ok.materials.PeriodicMirror(
            a=ok.materials.Layer(idx(), float(np.float32(0.4 * d))),
            b=ok.materials.Layer(idx(), float(np.float32(0.6 * d))),
            num_periods=40, substrate=ok.materials.Layer(idx())))
    return out


def run_multilayer(args, rank: int, world: int, emit: bool = True) -> dict:
    """The multilayer form: 256 periodic 40-bilayer mirrors, 1e7 samples
    (wavelength U(12, 15) nm, incidence U(0, 20) deg, a mirror each), R and
    T for s and p from float-float transfer matrices.  Inputs resident in
    HBM.  Replicas under torchrun."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from optika_gb300 import _api
    from optika_gb300 import _lib as L

    n = args.samples
    mirrors = _mirrors(4, 256)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device=dev).manual_seed(4 + 1000 * rank)
    wl = 12.0 + 3.0 * torch.rand(n, device=dev, generator=g)
    cos = torch.cos(torch.rand(n, device=dev, generator=g) * (20.0 * math.pi / 180.0))
    index = torch.randint(0, 256, (n,), device=dev, generator=g, dtype=torch.int32)
    table = _api.periodic_table(mirrors, dev)
    outs = [torch.empty(n, device=dev) for _ in range(4)]
    lib = L.load()

    def step():
        st = lib.otx_multilayer_periodic(
            _api.ptr(table), len(mirrors), n, _api.ptr(wl), 1, _api.ptr(cos), 1,
            _api.ptr(index), 1.0, 0.0, *(_api.ptr(o) for o in outs), _api.stream_handle())
        L.check(st, "otx_multilayer_periodic")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    value = world * n / (ms * 1e-3)
    bps = 12 + 16  # wavelength, cosine, mirror index in; R_s, R_p, T_s, T_p out
    pk, pk_kind = peaks()
    ach = bps * n / (ms * 1e-3) / 1e9
    fp32 = fp32_roofline("multilayer-periodic", n, ms, pk)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        jobs = [(c, 30000, 4) for c in range(0, 4 * cores)]
        m, wall = _cpu_pool(_cpu_multilayer_worker, jobs, cores)
        cpu = {"value": m / wall, "unit": "samples/s (s and p)", "cores": cores, "kind": "port",
               "sample": f"{len(jobs)} mirrors x 30000 samples, complex128 ({wall:.1f} s)"}
    line = {
            "metric": "multilayer samples/s (R and T, s and p, 40-bilayer periodic mirrors)",
            "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float products)",
            "data": "synthetic (seeded)",
            "config": {"workload": "multilayer-periodic", "mirrors": 256, "samples": n,
                       "bilayers": 40, "l2": "inputs and outputs 280 MB, larger than L2"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": ach / pk["hbm_gbs"],
                         "traffic": _ncu_traffic("multilayer_periodic_1e7", n),
                         "peak_kind": pk_kind,
                         "bytes_per_sample": bps, "kernel": "k_multilayer_periodic",
                         "kernel_ms": ms, "fp32": fp32, "issue": issue_roofline(
                             "multilayer_periodic_1e7", n, ms, pk, fp32),
                         "note": "compute-bound (instruction issue): the byte roofline is "
                                 "shown for completeness"},
            "cpu_baseline": cpu, "gpu_launches": args.steps, "clocks": clk,
    }
    if emit and rank == 0:
        print(json.dumps(line), flush=True)
    return line


_IMAGE_SURFACES = 5  # object, obscuration, primary, fold, sensor


def _image_scene(seed: int = 6):
    """The forward-model workload: 8 wavelength cells over 400-700 nm,
    128 x 128 field cells over +-0.15 deg of seeded radiance, 32 x 32 pupil
    cells over +-50 mm: 1.34e8 cells (rays) per image."""
    from optika_gb300.vectors import (Cartesian2dVectorArray, FunctionArray,
                                      SpectralPositionalVectorArray)

    rng = np.random.default_rng(seed)
    w = np.linspace(400.0, 700.0, 9)
    f = np.linspace(-0.15, 0.15, 129) * math.pi / 180
    rad = rng.uniform(0.5, 1.5, (8, 128, 128))
    v = np.linspace(-50.0, 50.0, 33)
    scene = FunctionArray(inputs=SpectralPositionalVectorArray(
        wavelength=w, position=Cartesian2dVectorArray(f, f)), outputs=rad)
    return scene, Cartesian2dVectorArray(v, v)


_IMAGE_TABLES = {}


def _cpu_image_worker(args):
    first, count, seed = args
    from optika_gb300 import configs
    from oracle import image as OI

    if "t" not in _IMAGE_TABLES:
        system = configs.newtonian(coated=True)
        scene, pupil = _image_scene()
        _IMAGE_TABLES["s"] = system
        _IMAGE_TABLES["t"] = OI.cell_tables(system, scene.inputs.wavelength,
                                            scene.inputs.position.x, scene.inputs.position.y,
                                            scene.outputs, pupil.x, pupil.y, False, False)
    inputs = OI.cell_inputs(_IMAGE_TABLES["t"], True, seed, first, count)
    OI.photon_image(_IMAGE_TABLES["s"], inputs, (400.0, 700.0, 1))
    return (count,)


def run_image(args, rank: int, world: int) -> None:
    """SequentialSystem.image of the Al-coated Newtonian: cell rays drawn on
    the device, the fused trace with sensor binning, exposure with shot and
    read noise, 1.34e8 cells per image in chunks of 2^24.  Replicas under
    torchrun (each rank its own seed)."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from optika_gb300 import configs
    from optika_gb300.imaging import ImagePlan

    system = configs.newtonian(coated=True)
    system.sensor.read_noise = 2.0
    scene, pupil = _image_scene()
    seed = 6 + 1000 * rank
    plan = ImagePlan(system, scene, pupil, normalized_field=False, normalized_pupil=False,
                     integrate=True, random=True, seed=seed)
    n = plan.count

    def step():
        return plan.run(noise=True, timedelta=1.0)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    value = world * n * _IMAGE_SURFACES / (ms * 1e-3)
    # end to end: the public call, host tables included, electrons to the host
    e2e_ms = []
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = system.image(scene, pupil=pupil, normalized_field=False, normalized_pupil=False,
                           noise=True, seed=seed, timedelta=1.0)
        host = res.outputs.cpu()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = sorted(e2e_ms)[len(e2e_ms) // 2]
    tables = sum(np.asarray(a).nbytes // 2 for a in (
        plan.tables.wavelength, plan.tables.field_x, plan.tables.field_y, plan.tables.pupil_x,
        plan.tables.pupil_y, plan.tables.weight, plan.tables.weight_pupil))  # float32 copies
    bpr = 48  # cell rays: 24 B written; trace: the same 24 B read
    pk, pk_kind = peaks()
    ach = bpr * n / (ms * 1e-3) / 1e9
    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        per = 250_000
        jobs = [(k * 7_919_993 % (n - per), per, seed) for k in range(cores)]
        rays, wall = _cpu_pool(_cpu_image_worker, jobs, cores)
        cpu = {"value": rays * _IMAGE_SURFACES / wall, "unit": "rays*surfaces/s",
               "cores": cores, "kind": "port",
               "sample": f"{len(jobs)} x {per} cells of the same image, float64 ({wall:.1f} s)"}
    if rank == 0:
        print(json.dumps({
            "metric": "rays*surfaces/s (SequentialSystem.image forward model)",
            "value": value, "unit": "rays*surfaces/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "newtonian-image (Al-coated)", "cells": n,
                       "grid": "8 wavelengths x 128^2 field x 32^2 pupil", "surfaces": 5,
                       "sensor": "1024x1024 x 13.5um", "chunk": plan.chunk,
                       "l2": "per-chunk ray inputs 400 MB, larger than L2"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": ach / pk["hbm_gbs"], "traffic": None, "peak_kind": pk_kind,
                         "bytes_per_ray": bpr, "kernel": "k_cell_rays + k_trace_fixed",
                         "kernel_ms": ms,
                         "note": "the trace is FP32-issue-bound: the byte roofline is shown "
                                 "for completeness"},
            "e2e": {"value": world * n * _IMAGE_SURFACES / (e2e * 1e-3), "unit": "rays*surfaces/s",
                    "ms_per_step": e2e, "h2d_bytes_per_step": int(tables),
                    "d2h_bytes_per_step": int(host.numel() * host.element_size())},
            "cpu_baseline": cpu, "gpu_launches": plan.launches * args.steps, "clocks": clk,
        }), flush=True)


def _cpu_stops_worker(args):
    w0, w1, count = args
    from optika_gb300 import configs
    from oracle import stops as OS

    system = configs.stop_grazing()
    for w in np.linspace(w0, w1, count):
        OS.extents(system, float(w))
    return (count,)


def run_stops(args, rank: int, world: int) -> None:
    """The stop solver: field and pupil extents of the grazing-incidence
    spectrograph at --stop-wavelengths wavelengths (default 64; 21 x 21
    boundary ray pairs each), all wavelengths in one batched solve: the
    Newton iterations in one kernel launch (otx_stop_newton), then the
    backward trace and the extents.  A step is the public call
    ``extents_many`` with the extents cleared (the lowered descriptors stay
    cached on the system, as in repeated use); replicas under torchrun."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from optika_gb300 import configs
    from optika_gb300.stops import extents_many

    from optika_gb300 import stops as stops_mod

    system = configs.stop_grazing()
    wls = np.linspace(500.0, 600.0, args.stop_wavelengths)
    launches = [0]
    trace = stops_mod._trace

    def counted(*a, **k):  # each call is one otx_trace_rays launch
        launches[0] += 1
        return trace(*a, **k)

    stops_mod._trace = counted

    def step():
        system.__dict__.pop("_stop_extents", None)
        return extents_many(system, wls)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    launches[0] = 0
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    value = world * len(wls) / (ms * 1e-3)
    traces = launches[0]
    pk, pk_kind = peaks()
    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        # 16 jobs of 64 wavelengths per core (each a float64 solve)
        edges = np.linspace(500.0, 600.0, 16 * cores + 1)
        jobs = [(float(a), float(b), 64) for a, b in zip(edges[:-1], edges[1:])]
        solves, wall = _cpu_pool(_cpu_stops_worker, jobs, cores)
        cpu = {"value": solves / wall, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"{solves} wavelengths in {len(jobs)} jobs of 64, one float64 solve "
                         f"each ({wall:.1f} s)"}
    if rank == 0:
        print(json.dumps({
            "metric": "stop solves/s (field and pupil extents per wavelength)",
            "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 trace, f64 Newton updates",
            "data": "synthetic (the grazing spectrograph test system)",
            "config": {"workload": "stop-solver", "wavelengths": len(wls),
                       "boundary_pairs": 441, "system": "grazing spectrograph"},
            "roofline": {"bound": "hbm", "achieved": None, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": None, "traffic": None, "peak_kind": pk_kind,
                         "note": "latency-bound: one Newton launch of a few thousand rays, the "
                                 "backward trace and the host setup around them"},
            "e2e": {"value": value, "unit": "solves/s", "ms_per_step": ms,
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 16 * len(wls) * 8},
            "cpu_baseline": cpu, "gpu_launches": traces, "clocks": clk,
        }), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rays", type=int, default=100_000_000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-rays", type=int, default=8_000_000)
    ap.add_argument("--ref-rays", type=int, default=2_000_000,
                    help="rays per step of the reference (CPU) arm")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--stop-wavelengths", type=int, default=64,
                    help="wavelengths per stop solve (--workload stops)")
    ap.add_argument("--no-workloads", action="store_true",
                    help="time the precision form only (no batched, multilayer, surrogate)")
    ap.add_argument("--workload", default="precision",
                    choices=["precision", "surrogate", "batched", "multilayer", "image",
                             "stops"])
    ap.add_argument("--configs", type=int, default=4096, help="batched workload configurations")
    ap.add_argument("--samples", type=int, default=10_000_000,
                    help="multilayer workload samples per step")
    ap.add_argument("--train-steps", type=int, default=6000)
    ap.add_argument("--image-rays", type=int, default=1_000_000_000)
    ap.add_argument("--image-chunk", type=int, default=0,
                    help="rays per call of the image simulation (0: the path's default)")
    ap.add_argument("--image-path", default="fused", choices=["fused", "layers"],
                    help="fused tensor-core kernel, or the network layer by layer")
    ap.add_argument("--rays-per-thread", type=int, default=0)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "surrogate":
        run_surrogate(args, rank, world)
        return
    if args.workload == "batched":
        run_batched(args, rank, world)
        return
    if args.workload == "multilayer":
        run_multilayer(args, rank, world)
        return
    if args.workload == "image":
        run_image(args, rank, world)
        return
    if args.workload == "stops":
        run_stops(args, rank, world)
        return

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    import optika_gb300 as ok
    from optika_gb300 import _api, _lib, configs

    V = ok.vectors.Cartesian2dVectorArray
    system = configs.newtonian(coated=True)
    n = args.rays
    g = configs.precision_grid(n, seed=2 + 7919 * rank)
    dev = torch.device("cuda", local)
    host = {k: torch.from_numpy(v.astype(np.float32)).pin_memory() for k, v in g.items()}
    inp = {k: v.to(dev) for k, v in host.items()}
    launch = _lib.Launch()
    launch.rays_per_thread = args.rays_per_thread
    outputs = ("px", "py", "pz", "dx", "dy", "dz", "intensity", "unvignetted", "opl")
    prep = _api.PreparedTrace(
        system, wavelength=inp["wavelength"], field=V(inp["field_x"], inp["field_y"]),
        pupil=V(inp["pupil_x"], inp["pupil_y"]), final_local=True, image=True, launch=launch,
        outputs=outputs,
    )
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        prep.run()
    torch.cuda.synchronize()
    barrier()

    clocks = Clocks(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    start.record(stream)
    for i in range(args.steps):
        prep.counts.zero_()
        prep.flux.zero_()
        ev[i][0].record(stream)
        st = prep.lib.otx_trace_grid(
            _api.ctypes.byref(prep.lowering.sys), _api.ctypes.byref(prep.grid),
            _api.ctypes.byref(prep.out), _api.ctypes.byref(prep.img),
            _api.ctypes.byref(prep.launch_desc), _api.stream_handle(),
        )
        _lib.check(st, "otx_trace_grid")
        ev[i][1].record(stream)
    stop.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    total_ms = start.elapsed_time(stop)
    kernel_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    ms_step = total_ms / args.steps
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    value = world * n * NUM_SURFACES / (ms_step * 1e-3)

    # end to end: the public API called with pinned host arrays, as a caller
    # of the reference passes NumPy arrays; it streams the rays through the
    # GPU in overlapping chunks (otx_trace_grid_host) and returns host
    # outputs and images, complete on return
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    d2h = 0
    e2e_ms = []
    for i in range(args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = system.rayfunction(
            wavelength=host["wavelength"], field=V(host["field_x"], host["field_y"]),
            pupil=V(host["pupil_x"], host["pupil_y"]), normalized_field=False,
            normalized_pupil=False, image=True, launch=launch, outputs=outputs,
        )
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_ms.append(dt * 1e3)
        o = res.outputs
        tensors = [o.position.x, o.position.y, o.position.z, o.direction.x, o.direction.y,
                   o.direction.z, o.intensity, o.opl, o.unvignetted, res.image[0], res.image[1]]
        assert all(t.device.type == "cpu" for t in tensors)
        d2h = sum(t.numel() * t.element_size() for t in tensors)
        del res, o, tensors
    e2e_ms_step = float(np.median(e2e_ms))
    e2e_value = world * n * NUM_SURFACES / (e2e_ms_step * 1e-3)

    pk, pk_kind = peaks()
    achieved = BYTES_PER_RAY * n / (kernel_ms * 1e-3) / 1e9
    roofline = {
        "bound": "hbm",
        "achieved": achieved,
        "peak": pk["hbm_gbs"],
        "unit": "GB/s",
        "frac": achieved / pk["hbm_gbs"],
        "traffic": None,
        "peak_kind": pk_kind,
        "kernel": "k_trace_fixed<1, Object, Stop, ConicCoated, FlatCoated, Detector>",
        "kernel_ms": kernel_ms,
        "bytes_per_ray": BYTES_PER_RAY,
    }
    # per-ray DRAM traffic of this kernel from one ncu capture of the same
    # workload at 8e6 rays (scaled by the ray count), and the algorithmic
    # arithmetic per ray counted by oracle/flops.py
    prof = ROOT / "profiles" / "trace_precision_1e8.json"
    if prof.exists():
        pj = json.loads(prof.read_text())
        if pj.get("dram_bytes_per_ray"):
            roofline["traffic"] = pj["dram_bytes_per_ray"] * n
        if pj.get("algorithmic_flops_per_ray"):
            # the kernel is bound by FP32 instruction issue, not by HBM: the
            # reference algorithm's FP32 work per ray at the kernel's rate,
            # against the FP32 pipe's peak at the maximum SM clock (152 SMs x
            # 128 lanes x 2 flops per FMA; nominal, no measured FP32 peak
            # exists for this pool); divisions and special functions are
            # listed beside it, not added to it
            fl = pj["algorithmic_flops_per_ray"]
            fp32_peak = 152 * 128 * 2 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
            ach = fl * n / (kernel_ms * 1e-3) / 1e12
            roofline["fp32"] = {
                "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                "algorithmic_flops_per_ray": fl,
                "algorithmic_div_per_ray": pj.get("algorithmic_div_per_ray"),
                "algorithmic_special_per_ray": pj.get("algorithmic_special_per_ray"),
                "counted_by": "oracle/flops.py (non-trivial real operations of the "
                              "reference's formulas)",
                "peak_kind": "nominal at the measured maximum SM clock",
                "executed_fp32_flops_per_ray_ncu": pj.get("flops_per_ray"),
                "fma_pipe_active_pct_ncu": pj.get("fma_pipe_active_pct")}
        if pj.get("warp_instructions_per_32_rays"):
            # the resource the kernel is bound by: instruction issue, one warp
            # instruction per cycle per scheduler (152 SMs x 4) at the
            # measured maximum clock, against the ncu-counted instructions
            # of this kernel per ray at its measured rate
            wi = pj["warp_instructions_per_32_rays"] / 32.0
            issue_peak = 152 * 4 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
            ach_i = wi * n / (kernel_ms * 1e-3) / 1e12
            roofline["issue"] = {
                "achieved": ach_i, "peak": issue_peak, "unit": "T warp-instructions/s",
                "frac": ach_i / issue_peak, "warp_instructions_per_ray_ncu": wi,
                "peak_kind": "nominal at the measured maximum SM clock",
                "note": "the binding resource: at full issue this instruction count "
                        "would put roofline.fp32 at " +
                        f"{roofline['fp32']['frac'] / (ach_i / issue_peak):.2f}"
                        if "fp32" in roofline else ""}

    cpu = None
    errors = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        v, wall = cpu_baseline(args.cpu_rays, cores)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_rays} rays of the same workload over {cores} processes "
                         f"({wall:.1f} s)"}
        # the oracle as the checker of the timed run's first rays
        k = min(ERROR_RAYS, n)
        sub = {key: host[key][:k].numpy().astype(np.float64) for key in g}
        got = {key: prep.bufs[key][:k].cpu().numpy() for key in
               ("px", "py", "dx", "dy", "dz", "intensity", "opl", "unvignetted")}
        got["unvignetted"] = got["unvignetted"] != 0
        errors = precision_errors(sub, got, cores)

    workloads = None
    if not args.no_workloads:
        del prep, inp
        torch.cuda.empty_cache()
        sub_args = argparse.Namespace(**vars(args))
        sub_args.steps = min(args.steps, 20)
        workloads = {}
        for name, fn in (("batched", run_batched), ("multilayer", run_multilayer),
                         ("surrogate", run_surrogate)):
            w = fn(sub_args, rank, world, emit=False)
            keep = ("metric", "value", "unit", "ms_per_step", "dtype", "config", "roofline",
                    "cpu_baseline", "gpu_launches", "clocks", "plain_trace", "surrogate_ms",
                    "speedup_vs_plain", "held_out", "image")
            workloads[name] = {key: w[key] for key in keep if key in w}
            torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded numpy)",
            "config": {
                "workload": "newtonian-precision (Al-coated mirrors, 400-700 nm)",
                "rays_per_gpu": n,
                "surfaces": NUM_SURFACES,
                "sensor": "1024x1024 x 13.5um, uint32 counts + float flux",
                "l2": "inputs (2 GB) and outputs larger than L2; no flush",
            },
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_ms_step,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "error": errors,
            "gpu_launches": args.steps,
            "clocks": clk,
            "workloads": workloads,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
