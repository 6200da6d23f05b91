"""Benchmark of the GB300 likelihood engine.

Headline workload (N=1): batched emission forward model + Gaussian log-likelihood,
512 live points per launch drawn uniformly over the priors; 80 levels, 6 line
species + 2 CIA tables on 10 log-p x 20 T, 2000-12000 cm^-1 at 1 cm^-1
(10257 model points), three observations of 120, 40 and 8 bins (the 8 are
top-hat / Gaussian bandpass filters). Synthetic seeded tables in the
reference's on-disk format.

One step = one batch of B likelihood evaluations. ``value`` = evaluations per
second over the timed steps with parameters resident in HBM (the autotuned
captured graph); ``e2e`` = the same through the host API with the parameter
upload and the log-likelihood download inside the timed region; ``plain_path`` =
one evaluation per bear_loglike call (host in, host out). The adjoint gradient
of the same batch is timed as well (``gradient``: evals/s and the ratio of its
time to the forward batch). L2 is flushed between timed steps
(a 512 MiB write) outside the per-step event pair.

The default run (no --workload) adds ``configs``: the same record for the other
benchmark shapes, each with its own clocks, roofline and CPU baseline:
0 plain emission (one evaluation per call), 1 plain transmission (B = 64) and its
10-annuli variant, 3 the emission adjoint (B = 256, 17 parameters incl. the grey
cloud), 4 the joint emission + transmission workload (B = 1024, forward + gradient).

Roofs of the dominant kernel: ``roofline`` (HBM: algorithmic bytes / event time
against the measured copy rate; ``traffic`` = DRAM bytes per launch from the
committed ncu capture), ``fp64`` (emission: FP64-pipe instructions counted from the
source / event time against the DFMA rate implied by the committed DGEMM
measurement) and ``issue`` (warp instructions per launch from the committed ncu
capture / event time against 4 per SM per clock).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload emission_batched|emission_adjoint|emission_plain|transmission_plain|
                                transmission_annuli|joint_large] [--no-configs]
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from bear_gb300 import synthetic as syn  # noqa: E402
from bear_gb300.config import observation_arrays, render_config  # noqa: E402
from bear_gb300.replicas import max_over_ranks  # noqa: E402

WORKLOADS = {
    "emission_batched": ("emission_batched", "emission"),
    "emission_adjoint": ("emission_adjoint", "emission"),
    "emission_plain": ("emission_plain", "emission"),
    "transmission_plain": ("transmission_plain", "transmission"),
    "transmission_annuli": ("transmission_plain", "transmission"),
    "joint_large": ("joint_large", "joint"),
}
# impact parameters per layer of the transit integral (1: the reference's tangent rays)
ANNULI = {"transmission_annuli": 10}
HEADLINE = "emission_batched"
# sub-records of the default run: (key, workload, batch, timed steps; None = --config-steps);
# one evaluation takes ~0.5 ms, so config 0 times 1000 of them (about half a second, long
# enough for the clock sampler and for the clocks to settle)
CONFIG_RECORDS = (
    ("0_emission_plain", "emission_plain", 1, 1000),
    ("1_transmission_plain", "transmission_plain", 64, None),
    ("1_transmission_annuli", "transmission_annuli", 64, None),
    ("3_emission_adjoint", "emission_adjoint", 256, None),
    ("4_joint_large", "joint_large", 1024, None),
)
# FP64-pipe instructions per wavenumber and layer of the emission kernels' recurrence
# (emission_layer), counted from the source: the conversion add of u = (B - B') / tau (formed
# in double-float; the float -> double steps run on the integer pipe), and per Gauss angle
# the conversion add and FMA of exp_neg_df, (a - 1) u as one FMA and the update FMA.
EMISSION_FP64_OPS_PER_POINT_LAYER = 1 + 2 * (2 + 1 + 1)
FLUSH_BYTES = 512 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 20; 4 for joint_large)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default=None, choices=sorted(WORKLOADS),
                    help=f"one workload only (default: {HEADLINE} with the other configurations as sub-records)")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--no-configs", action="store_true", help="headline workload only")
    ap.add_argument("--config-steps", type=int, default=5, help="timed steps of each sub-record")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-gradient", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0, help="evaluations in the CPU baseline sample")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def synth_dir():
    return os.environ.get("BEAR_SYNTH_DIR", "/tmp/bear_gb300_synth")


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    return ln.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except OSError:
        pass
    return platform.processor() or platform.machine()


def build_case(workload: str):
    """Tables, config text and observations (data attached later)."""
    name, kind = WORKLOADS[workload]
    spec = syn.CONFIGS[name]
    root = syn.write_tables(spec, synth_dir())
    text = render_config(syn.global_config(spec, root, kind), syn.model_config(spec, kind))
    if workload in ANNULI:
        text += f"transmission_annuli {ANNULI[workload]}\n"
    obs = syn.observations(spec, kind)
    return spec, kind, text, obs


def attach_engine_data(spec, kind, text, obs, device):
    """Observation data = the engine's model at the seeded truth parameters plus noise."""
    from bear_gb300.retrieval import Engine

    e0 = Engine(text, [observation_arrays(o) for o in obs], device=device)
    _, m, _ = e0.compute_model(syn.truth_parameters(spec, kind))
    e0.close()
    parts, off = [], 0
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, kind, spec.seed)
    return [observation_arrays(o) for o in obs]


def live_points(spec, kind, batch, rank):
    pr = syn.priors(spec, kind)
    cube = np.random.default_rng(spec.seed + 31 + 1000 * rank).uniform(size=(batch, len(pr)))
    return syn.cube_to_physical(pr, cube)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp64_peak():
    """DGEMM rate of this GPU model (TFLOP/s) from the committed measurement
    (profiles/fp64_peak.json, cuBLAS through torch.matmul on float64), and its source."""
    with open(os.path.join(REPO, "profiles", "fp64_peak.json")) as f:
        rec = json.load(f)
    return float(rec["dgemm_tflops"]), f"measured DGEMM {rec['shape']} (profiles/fp64_peak.json)"


def kernel_counters(workload, batch):
    """ncu counters per launch of the dominant kernel (DRAM bytes, warp instructions)
    from the committed capture of this workload and batch (profiles/kernel_counters.json),
    or None."""
    try:
        with open(os.path.join(REPO, "profiles", "kernel_counters.json")) as f:
            rec = json.load(f)[workload]
    except (OSError, KeyError, ValueError):
        return None
    return rec if rec.get("batch") == batch else None


def captured_traffic(workload, batch):
    """DRAM bytes per launch of the dominant kernel at this workload and batch, or None."""
    rec = kernel_counters(workload, batch)
    return rec["dram_bytes_per_launch"] if rec else None


def issue_roof(workload, batch, kern_ms, torch, device, clocks):
    """Warp instructions issued per second by the dominant kernel (ncu's executed
    instruction count per launch / the event time) against the SM issue rate
    (4 warp instructions per SM per clock at the sampled median SM clock)."""
    rec = kernel_counters(workload, batch)
    if not rec or "warp_instructions_per_launch" not in rec:
        return None
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    peak = 4.0 * sms * mhz * 1e6
    ach = rec["warp_instructions_per_launch"] / (kern_ms * 1e-3)
    return {"bound": "issue", "unit": "warp inst/s", "achieved": ach, "peak": peak, "frac": ach / peak,
            "warp_instructions_per_launch": rec["warp_instructions_per_launch"],
            "peak_source": f"4 x {sms} SMs x {mhz:.0f} MHz (sampled)", "counts_source": "profiles/kernel_counters.json"}


def cpu_baseline(text, arrays, params, sample, threads, budget_s):
    """The FP64 C restatement of the reference path (a port) on the host cores:
    sequential evaluations of the batch's live points until ``budget_s`` seconds
    have passed (or ``sample`` evaluations, when given)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    oracle.set_threads(threads)
    om = oracle.OracleModel(text, arrays)
    om.loglike(params[0])  # warm-up
    n = 0
    t0 = time.perf_counter()
    while (sample and n < sample) or (not sample and time.perf_counter() - t0 < budget_s):
        om.loglike(params[n % len(params)])
        n += 1
    dt = time.perf_counter() - t0
    om.close()
    return {"value": n / dt, "unit": "evals/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "sample": f"{n} sequential evaluations of this batch's live points ({dt:.1f} s), "
                      f"FP64 C oracle with OpenMP"}


class Ctx:
    """Process-wide state of one bench run."""

    def __init__(self, torch, rank, world, device, dist):
        self.torch, self.rank, self.world, self.device, self.dist = torch, rank, world, device, dist
        self.stream = torch.cuda.current_stream(device)
        self.flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=device)

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()
        self.torch.cuda.synchronize(self.device)

    def max_ms(self, ms):
        return max_over_ranks(ms, self.dist, self.device) if self.dist is not None else ms

    def timed(self, fn, steps):
        """Total device time (ms) of ``steps`` calls of fn on the stream, each bracketed by
        CUDA events, L2 flushed before each; the max over ranks."""
        torch = self.torch
        ev = []
        self.barrier()
        for _ in range(steps):
            self.flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(self.stream)
            fn()
            e.record(self.stream)
            ev.append((s, e))
        self.barrier()
        return self.max_ms(sum(s.elapsed_time(e) for s, e in ev))


def measure_engine(ctx, workload, batch, steps, warmup, args, cpu_budget_s):
    """One workload: batched (graph replay), end-to-end, plain path, gradient, stage
    times, roofs, clocks and the CPU baseline. Returns the record."""
    torch = ctx.torch
    from bear_gb300.retrieval import BatchEvaluator, Engine

    spec, kind, text, obs = build_case(workload)
    arrays = attach_engine_data(spec, kind, text, obs, ctx.device)
    eng = Engine(text, arrays, device=ctx.device)
    B = batch
    params_host = live_points(spec, kind, B, ctx.rank)
    P = torch.tensor(params_host, dtype=torch.float64, device=ctx.device)
    stream = ctx.stream
    # the batched path: launch shape picked by the autotuner, kernels replayed from a captured graph
    ev = BatchEvaluator(eng, P, autotune=True)
    ll, ng = ev.loglike, ev.neglect

    def step():
        ev.launch(stream.cuda_stream)

    for _ in range(max(warmup, 3)):
        step()
    with ClockSampler(ctx.device) as clocks:
        total_ms = ctx.timed(step, steps)
    clk = clocks.summary()
    value = ctx.world * B * steps / (total_ms * 1e-3)

    # end-to-end through the host API: pinned params in, log-likelihoods out
    p_pin = torch.tensor(params_host, dtype=torch.float64).pin_memory()
    ll_pin = torch.empty(B, dtype=torch.float64).pin_memory()

    def e2e_step():
        ev.params.copy_(p_pin, non_blocking=True)
        ev.launch(stream.cuda_stream)
        ll_pin.copy_(ll, non_blocking=True)

    for _ in range(2):
        e2e_step()
    e2e_ms = ctx.timed(e2e_step, steps)
    e2e_value = ctx.world * B * steps / (e2e_ms * 1e-3)

    # plain single-evaluation path (bear_loglike, one host call per evaluation)
    for _ in range(3):
        eng.loglike(params_host[0])
    n_plain = 50
    torch.cuda.synchronize(ctx.device)
    t0 = time.perf_counter()
    for i in range(n_plain):
        eng.loglike(params_host[i % B])
    plain_s = (time.perf_counter() - t0) / n_plain

    # adjoint gradient: log L and d log L / d params for the batch
    grad = None
    if not args.no_gradient:
        G = torch.empty(B, eng.P, dtype=torch.float64, device=ctx.device)

        def grad_step():
            eng.grad_batch_ptr(P.data_ptr(), B, ll.data_ptr(), G.data_ptr(), ng.data_ptr(), stream.cuda_stream)

        for _ in range(2):
            grad_step()
        n_grad = max(3, min(steps, 10))
        grad_ms = ctx.timed(grad_step, n_grad) / n_grad
        fwd_ms = total_ms / steps
        grad = {"evals_per_s": B / (grad_ms * 1e-3), "ms_per_batch": grad_ms, "forward_ms_per_batch": fwd_ms,
                "grad_over_forward": grad_ms / fwd_ms, "parameters": eng.P, "steps": n_grad,
                "kernels_per_batch": 6 if kind == "emission" else 9 if workload in ANNULI else 10,
                "api": "bear_loglike_grad_batch (adjoint; forward pass included in the time)"}
        del G

    # dominant kernel timing for the roofs (CUDA events on the launching stream)
    stages = eng.stage_times(P.data_ptr(), B, ll.data_ptr(), stream.cuda_stream, repeats=5)
    kern_ms = stages[1]
    rows = eng.stencil_row_count(B)
    N, M, L, S = eng.N, eng.M, spec.nb_levels, eng.table_species
    # algorithmic bytes of one radiative-transfer launch: every distinct level-table row the
    # batch's stencils touch (8 B per point), read once; the 32-byte per-level stencil
    # records; the spectrum write
    alg_bytes = rows * N * 8 + B * L * S * 32 + B * N * 8
    peaks, peak_kind = measured_peaks()
    achieved_gbs = alg_bytes / (kern_ms * 1e-3) / 1e9
    rec_k = kernel_counters(workload, B)
    if rec_k:
        kernel = rec_k["kernel"].split(" grid")[0]
    elif kind == "emission":
        kernel = "emission_kernel_x2<0>" if B >= 2 else "emission_kernel<0, 0>"
    else:
        kernel = "transmission_annuli_kernel" if workload in ANNULI else "transmission_kernel_x2<16, 8, 8, 2, 0>"

    rec = {
        "workload": workload, "batch": B, "levels": L, "spectral_points": N, "bins": M, "table_species": S,
        "annuli_per_layer": ANNULI.get(workload, 1), "steps": steps, "ms_per_step": total_ms / steps,
        "value": value, "unit": "evals/s",
        "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": int(P.numel() * 8),
                "d2h_bytes_per_step": int(B * 8)},
        "plain_path": {"evals_per_s": 1.0 / plain_s, "ms_per_eval": plain_s * 1e3,
                       "api": "bear_loglike (host params in, host log L out)"},
        "batched_over_plain": value * plain_s,
        # atmosphere + radiative transfer (+ geometry for transmission) + observation/likelihood,
        # replayed from one captured graph per step
        "gpu_launches": (3 if kind == "emission" else 4) * steps,
        "batched_path": {"api": "bear_batch_graph_launch (CUDA graph of the batched kernels)",
                         "autotuned_rt_threads": ev.rt_threads},
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved_gbs, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved_gbs / peaks["hbm_gbs"],
                     "traffic": captured_traffic(workload, B),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of the "
                                       "tuned shape (profiles/kernel_counters.json; null where not captured)",
                     "peak_source": peak_kind, "kernel_ms": kern_ms, "algorithmic_bytes": alg_bytes,
                     "distinct_table_rows": rows},
        "stage_ms": {"atmosphere": stages[0], "radiative_transfer": stages[1], "observation_loglike": stages[2]},
        "clocks": clk,
    }
    if kind == "emission":
        tf, src = fp64_peak()
        peak = tf / 2 * 1e3
        ops = B * (L - 1) * N * EMISSION_FP64_OPS_PER_POINT_LAYER
        ach = ops / (kern_ms * 1e-3) / 1e9
        rec["fp64"] = {"bound": "fp64", "unit": "Gop/s", "peak": peak, "peak_source": src + " / 2 flops per DFMA",
                       "dgemm_tflops_measured": tf, "achieved": ach, "frac": ach / peak, "ops_per_launch": ops,
                       "ops_per_point_layer": EMISSION_FP64_OPS_PER_POINT_LAYER}
    rec["issue"] = issue_roof(workload, B, kern_ms, torch, ctx.device, clk)
    if grad is not None:
        rec["gradient"] = grad
    if ctx.rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(text, arrays, params_host, args.cpu_sample, os.cpu_count() or 1, cpu_budget_s)
        rec["cpu_baseline"] = cb
        if grad is not None and "evals_per_s" in grad:
            # the reference has no derivatives: a central-difference gradient costs 2P + 1 evaluations
            grad["cpu_central_difference_evals_per_s"] = cb["value"] / (2 * eng.P + 1)
    ev.close()
    eng.close()
    return rec


def joint_parts(spec, data_from):
    """Config texts and observation arrays of the joint workload's two models, data
    attached from ``data_from(kind, text, obs)`` (the model at the seeded truth)."""
    root = syn.write_tables(spec, synth_dir())
    out = {}
    for kind in ("emission", "transmission"):
        text = render_config(syn.global_config(spec, root, kind), syn.model_config(spec, kind))
        obs = syn.observations(spec, kind)
        out[kind] = (text, data_from(kind, text, obs))
    return out


def joint_params(spec, B, rank):
    return np.concatenate([live_points(spec, "emission", B, rank), live_points(spec, "transmission", B, rank)], axis=1)


def measure_joint(ctx, batch, steps, warmup, args, cpu_budget_s):
    """Large joint workload: emission + transmission models on one spectral grid
    with shared device tables, joint log L = log L_emission + log L_transmission."""
    torch = ctx.torch
    from bear_gb300.joint import JointBatchEvaluator, JointEngine

    spec = syn.CONFIGS["joint_large"]
    parts = joint_parts(spec, lambda kind, text, obs: attach_engine_data(spec, kind, text, obs, ctx.device))
    (te, oe), (tt, ot) = parts["emission"], parts["transmission"]
    joint = JointEngine(te, oe, tt, ot, device=ctx.device)
    B = batch
    params_host = joint_params(spec, B, ctx.rank)
    P = torch.tensor(params_host, dtype=torch.float64, device=ctx.device)
    stream = ctx.stream
    ev = JointBatchEvaluator(joint, P, autotune=True)

    for _ in range(max(warmup, 3)):
        ev()
    with ClockSampler(ctx.device) as clocks:
        total_ms = ctx.timed(ev, steps)
    clk = clocks.summary()
    value = ctx.world * B * steps / (total_ms * 1e-3)

    # end to end: pinned host parameters in, joint log-likelihoods out
    p_pin = torch.tensor(params_host, dtype=torch.float64).pin_memory()
    ll_pin = torch.empty(B, dtype=torch.float64).pin_memory()
    P2 = torch.empty_like(P)

    def e2e_step():
        P2.copy_(p_pin, non_blocking=True)
        l, _ = ev(P2)
        ll_pin.copy_(l, non_blocking=True)

    e2e_step()
    e2e_ms = ctx.timed(e2e_step, steps)
    e2e_value = ctx.world * B * steps / (e2e_ms * 1e-3)

    # plain path: one host call per model per evaluation
    n_plain = 6
    for i in range(2):
        joint.emission.loglike(params_host[i, :joint.Pe])
        joint.transmission.loglike(params_host[i, joint.Pe:])
    torch.cuda.synchronize(ctx.device)
    t0 = time.perf_counter()
    for i in range(n_plain):
        joint.emission.loglike(params_host[i, :joint.Pe])
        joint.transmission.loglike(params_host[i, joint.Pe:])
    plain_s = (time.perf_counter() - t0) / n_plain

    # gradient of the joint batch (both adjoints)
    grad = None
    if not args.no_gradient:
        joint.grad_batch(P[:2])
        gms = ctx.timed(lambda: joint.grad_batch(P), 1)
        grad = {"evals_per_s": B / (gms * 1e-3), "ms_per_batch": gms, "forward_ms_per_batch": total_ms / steps,
                "grad_over_forward": gms / (total_ms / steps), "parameters": joint.P, "steps": 1,
                "api": "bear_loglike_grad_batch per model (adjoints; forward passes included in the time)"}

    # roofs of the two radiative-transfer kernels (CUDA events)
    peaks, peak_kind = measured_peaks()
    tf, src = fp64_peak()
    pe, pt = joint._split(P)
    ll1 = torch.empty(B, dtype=torch.float64, device=ctx.device)
    se = joint.emission.stage_times(pe.data_ptr(), B, ll1.data_ptr(), stream.cuda_stream, repeats=2)
    rows_e = joint.emission.stencil_row_count(B)
    st_ = joint.transmission.stage_times(pt.data_ptr(), B, ll1.data_ptr(), stream.cuda_stream, repeats=2)
    rows_t = joint.transmission.stencil_row_count(B)
    N, L, S = joint.N, spec.nb_levels, joint.emission.table_species
    alg = (rows_e + rows_t) * N * 8 + 2 * B * L * S * 32 + 2 * B * N * 8
    kern_ms = se[1] + st_[1]
    achieved = alg / (kern_ms * 1e-3) / 1e9
    em_ops = B * (L - 1) * N * EMISSION_FP64_OPS_PER_POINT_LAYER
    shared, table_bytes = joint.transmission.table_sharing()
    rec = {
        "workload": "joint_large", "batch": B, "levels": L, "spectral_points": N,
        "bins": joint.emission.M // 2 + joint.transmission.M // 2, "observations": joint.n_em_obs + joint.n_tr_obs,
        "table_species": S, "tables_shared": shared, "table_bytes": table_bytes, "steps": steps,
        "ms_per_step": total_ms / steps, "value": value, "unit": "evals/s",
        "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": int(P.numel() * 8),
                "d2h_bytes_per_step": int(B * 8)},
        "plain_path": {"evals_per_s": 1.0 / plain_s, "ms_per_eval": plain_s * 1e3,
                       "api": "bear_loglike per model (host params in, host log L out)"},
        "batched_over_plain": value * plain_s,
        "gpu_launches": 7 * steps,
        "batched_path": {"api": "two bear_batch_graph_launch per step", "autotuned_rt_threads":
                         [ev.em.rt_threads, ev.tr.rt_threads]},
        "roofline": {"bound": "hbm", "kernel": "emission_kernel_x2<0> + transmission_kernel_x2<16, 8, 8, 2, 0>", "achieved": achieved,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                     "peak_source": peak_kind, "kernel_ms": kern_ms, "algorithmic_bytes": alg,
                     "distinct_table_rows": rows_e + rows_t},
        "stage_ms": {"emission": {"atmosphere": se[0], "radiative_transfer": se[1], "observation_loglike": se[2]},
                     "transmission": {"atmosphere": st_[0], "radiative_transfer": st_[1],
                                      "observation_loglike": st_[2]}},
        "fp64": {"bound": "fp64", "unit": "Gop/s", "peak": tf / 2 * 1e3, "peak_source": src + " / 2 flops per DFMA",
                 "dgemm_tflops_measured": tf, "emission_achieved": em_ops / (se[1] * 1e-3) / 1e9,
                 "emission_frac": em_ops / (se[1] * 1e-3) / 1e9 / (tf / 2 * 1e3)},
        "clocks": clk,
    }
    if grad is not None:
        rec["gradient"] = grad
    if ctx.rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        from bear_gb300.joint import joint_observation_sets

        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        em, tr = joint_observation_sets(oe, ot)
        ome, omt = oracle.OracleModel(te, em), oracle.OracleModel(tt, tr)
        ome.loglike(params_host[0, :joint.Pe])
        n, t0 = 0, time.perf_counter()
        while (args.cpu_sample and n < args.cpu_sample) or (not args.cpu_sample and time.perf_counter() - t0 < cpu_budget_s):
            ome.loglike(params_host[n % B, :joint.Pe])
            omt.loglike(params_host[n % B, joint.Pe:])
            n += 1
        dt = time.perf_counter() - t0
        ome.close()
        omt.close()
        rec["cpu_baseline"] = {"value": n / dt, "unit": "evals/s", "cores": threads, "kind": "port",
                               "cpu_model": cpu_model(),
                               "sample": f"{n} sequential joint evaluations ({dt:.1f} s), FP64 C oracle with OpenMP"}
    ev.close()
    joint.close()
    return rec


def headline_line(rec, args, ctx):
    """The contract's JSON line around a workload record."""
    B = rec["batch"]
    config = {"workload": rec["workload"], "batch_per_gpu": B, "global_batch": B * ctx.world,
              "levels": rec["levels"], "spectral_points": rec["spectral_points"], "bins": rec["bins"],
              "table_species": rec["table_species"],
              "parallelism": f"replicas x{ctx.world}" if ctx.world > 1 else "single GPU",
              "l2": "flushed between timed steps (512 MiB write)"}
    for k in ("annuli_per_layer", "observations", "tables_shared", "table_bytes"):
        if k in rec:
            config[k] = rec[k]
    line = {"metric": "likelihood evals/s", "value": rec["value"], "unit": "evals/s", "n_gpus": ctx.world,
            "steps": rec["steps"], "warmup": args.warmup, "ms_per_step": rec["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded tables in the reference's on-disk format)", "config": config}
    for k, v in rec.items():
        if k not in ("workload", "batch", "levels", "spectral_points", "bins", "table_species", "annuli_per_layer",
                     "observations", "tables_shared", "table_bytes", "steps", "ms_per_step", "value", "unit"):
            line[k] = v
    return line


def measure(ctx, workload, batch, steps, warmup, args, cpu_budget_s):
    if workload == "joint_large":
        return measure_joint(ctx, batch, steps, warmup, args, cpu_budget_s)
    return measure_engine(ctx, workload, batch, steps, warmup, args, cpu_budget_s)


# ------------------------------------------------------------------ reference arm

def run_reference_joint(args, oracle, threads):
    """Reference arm of the joint workload: the FP64 oracle of both models
    (the same observation sets and grid as the engine arm)."""
    from bear_gb300.joint import joint_observation_sets

    spec = syn.CONFIGS["joint_large"]

    def oracle_data(kind, text, obs):
        om0 = oracle.OracleModel(text, [observation_arrays(o) for o in obs])
        _, m, _ = om0.forward(syn.truth_parameters(spec, kind))
        om0.close()
        parts, off = [], 0
        for o in obs:
            parts.append(m[off:off + len(o.data)])
            off += len(o.data)
        syn.attach_data(obs, parts, kind, spec.seed)
        return [observation_arrays(o) for o in obs]

    parts = joint_parts(spec, oracle_data)
    (te, oe), (tt, ot) = parts["emission"], parts["transmission"]
    em, tr = joint_observation_sets(oe, ot)
    ome, omt = oracle.OracleModel(te, em), oracle.OracleModel(tt, tr)
    Pe = ome.P
    B = args.batch or spec.batch
    params = joint_params(spec, B, 0)
    per_step = max(1, int(os.environ.get("BEAR_REF_EVALS_PER_STEP", "2")))
    for i in range(args.warmup):
        ome.loglike(params[i % B, :Pe])
        omt.loglike(params[i % B, Pe:])
    times, idx = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for _ in range(per_step):
            ome.loglike(params[idx % B, :Pe])
            omt.loglike(params[idx % B, Pe:])
            idx += 1
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps * per_step / total
    print(json.dumps({
        "impl": "reference", "metric": "likelihood evals/s", "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded tables in the reference format)",
        "config": {"workload": "joint_large", "batch": B, "levels": spec.nb_levels, "spectral_points": ome.N,
                   "bins": ome.M // 2 + omt.M // 2, "evals_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                         "sample": f"{args.steps * per_step} sequential joint evaluations of the workload's live points"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "host": platform.machine(),
    }))
    return 0


def run_reference(args):
    """The reference's CPU path for the same workload: the FP64 C port of it (pinned bit
    for bit to the reference binary's outputs), OpenMP on all host cores; rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    workload = args.workload or HEADLINE
    if workload == "joint_large":
        return run_reference_joint(args, oracle, threads)
    spec, kind, text, obs = build_case(workload)
    # observation data from the oracle itself (same recipe as the engine arm)
    arrays0 = [observation_arrays(o) for o in obs]
    om0 = oracle.OracleModel(text, arrays0)
    _, m, _ = om0.forward(syn.truth_parameters(spec, kind))
    om0.close()
    parts, off = [], 0
    for o in obs:
        parts.append(m[off:off + len(o.data)])
        off += len(o.data)
    syn.attach_data(obs, parts, kind, spec.seed)
    arrays = [observation_arrays(o) for o in obs]
    om = oracle.OracleModel(text, arrays)
    B = args.batch or spec.batch
    params = live_points(spec, kind, B, 0)
    per_step = max(1, int(os.environ.get("BEAR_REF_EVALS_PER_STEP", "16")))
    for i in range(args.warmup):
        om.loglike(params[i % B])
    times = []
    idx = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for _ in range(per_step):
            om.loglike(params[idx % B])
            idx += 1
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps * per_step / total
    line = {
        "impl": "reference", "metric": "likelihood evals/s", "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tables in the reference format)",
        "config": {"workload": workload, "batch": B, "levels": spec.nb_levels, "spectral_points": om.N,
                   "bins": om.M, "evals_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                         "sample": f"{args.steps * per_step} sequential evaluations of the workload's live points"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "host": platform.machine(),
    }
    om.close()
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    workload = args.workload or HEADLINE
    if args.steps is None:
        args.steps = 4 if workload == "joint_large" else 20
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local = dist_env()
    device = local
    torch.cuda.set_device(device)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", device))
    ctx = Ctx(torch, rank, world, device, dist)
    spec = syn.CONFIGS[WORKLOADS[workload][0]]
    rec = measure(ctx, workload, args.batch or spec.batch, args.steps, args.warmup, args, 12.0)
    line = headline_line(rec, args, ctx)
    if args.workload is None and not args.no_configs and world == 1:
        # the other benchmark shapes, each measured the same way on this GPU
        line["configs"] = {}
        for key, wl, b, n in CONFIG_RECORDS:
            steps = n or (args.config_steps if wl != "joint_large" else min(args.config_steps, 4))
            line["configs"][key] = measure(ctx, wl, b, steps, args.warmup, args, 8.0)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
