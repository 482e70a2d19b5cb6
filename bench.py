"""Benchmark: hits/s of the GB300 tracer (FP32 traversal + FP64 recheck) and of the plain FP64 kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload c2|c1]

A step traces one batch of desorptions to absorption on the workload's geometry.
`value` = hits (Sum nbMCHit, src/MolflowCLI.cpp:61-68) per second of device time
over K timed steps, max over ranks; `e2e` = the same through the public API
(SimulationMCStep + UpdateHitsAndLog) over K steps, with the tallies read back to host memory
and added into a host GlobalSimuState every step, after one untimed step that allocates the
host buffers.  One JSON line on rank 0.
Under torchrun each rank traces its own particle range (no data-path collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c1": dict(name="config1_tube_L10cm_R1cm_64gon_tex64x64_maxwell_N2_293K", step=100_000_000),
    "c2": dict(name="config2_beam_chamber_200k_triangles", step=10_000_000),
    "c3": dict(name="config3_tube_1ms_pulse_100_logspaced_moments", step=20_000_000),
    "c4": dict(name="config4_batch_256_instances_1k-50k_facets", step=1_000_000),
    "c5": dict(name="config5_neg_tube_1000_sticking_parameters_8_gauges", step=20_000_000),
}


# The metric each workload reports; the CPU reference arm prints the same string for the same
# workload, so that the two lines divide.
HEADLINE = "hits/s per GB300: FP32+FP64-recheck vs plain FP64 kernel at same 3\u03c3 transmission"
METRIC = {"c1": HEADLINE, "c2": HEADLINE, "c3": HEADLINE,
          "c4": "hits/s per GB300, 256-instance batch in one persistent launch",
          "c5": "hits/s per GB300 with sticking and outgassing gradients (score function)"}


def make_model(workload):
    from molflow_sources_gb300 import workloads
    if workload == "c1":
        return workloads.config1_tube()
    if workload == "c3":
        return workloads.config3_transient()
    if workload == "c5":
        from molflow_sources_gb300.sensitivity import config5_neg_tube
        return config5_neg_tube()
    return workloads.config2_beam_chamber()


def pumped_fraction(model, st):
    """(absorbed on the sinks) / desorbed, the transmission of the workload: the outlet of the
    tubes (facet 1), the four ports of the beam chamber."""
    ports = np.where(np.asarray(getattr(model, "kind", [])) >= 3)[0] if hasattr(model, "kind") else np.array([1])
    from molflow_sources_gb300 import _abi as A
    return float(st.facet_counts[0, ports, A.FC_NBABSORBED].sum()) / max(st.n_desorbed, 1.0)


def transmission_gate(model, st32, st64):
    """FP32R against FP64 kernel: difference of the transmissions in units of the combined
    binomial standard error (independent particles: the two runs use disjoint particle ids)."""
    p32, n32 = pumped_fraction(model, st32), st32.n_desorbed
    p64, n64 = pumped_fraction(model, st64), st64.n_desorbed
    sig = ((p32 * (1 - p32) / n32) + (p64 * (1 - p64) / n64)) ** 0.5
    z = (p32 - p64) / sig if sig > 0 else 0.0
    return {"quantity": "absorbed on the sinks / desorbed", "fp32r": p32, "fp32r_desorbed": int(n32),
            "fp64": p64, "fp64_desorbed": int(n64), "difference": p32 - p64, "sigma": sig, "z": z,
            "pass": bool(abs(z) < 3.0)}


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def oracle_visit_counts(model, n=2000):
    """Mean BVH nodes visited and facets tested per ray, counted by the instrumented CPU oracle."""
    from oracle.oracle import Oracle
    st, s = Oracle(model).run(n, seed=7, threads=0)
    return s["node_visits"] / s["rays"], s["prim_tests"] / s["rays"], s


def bytes_per_hit(model, nodes, prims):
    """Algorithmic bytes per hit: node and facet records visited (FP32 layout), the FP64
    hit-facet record, and the tally read-modify-writes (counters 4x8 B, texture 3x8 B when textured)."""
    L = model.layout()
    textured = float(np.mean(L["tex_off"] >= 0))
    return nodes * 32 + prims * 64 + 160 + 2 * (4 * 8 + textured * 3 * 8)


def calibrate(orc, seed, min_s=0.5):
    """Desorptions per second of the oracle on all host threads, from a run of at least min_s."""
    n = 2000
    while True:
        st, s = orc.run(n, seed=seed)
        if s["seconds"] >= min_s or n >= 10 ** 8:
            return s["desorbed"] / max(s["seconds"], 1e-6)
        n *= 4


def cpu_baseline(model, target_s=12.0):
    from oracle.oracle import Oracle
    orc = Oracle(model)
    rate_des = calibrate(orc, 11)
    n = int(max(1000, min(rate_des * target_s, 5e8)))
    st, s = orc.run(n, seed=12, first_particle=10 ** 12)
    return {"value": s["hits"] / s["seconds"], "unit": "hits/s", "cores": s["threads"], "kind": "port",
            "sample": "%d desorptions (%d hits) of the same workload, %.1f s" % (n, s["hits"], s["seconds"]),
            "seconds": s["seconds"]}


def other_workloads(torch, local, steps=2):
    """Short device-time measurements of configs 1, 3, 4 and 5 beside the headline (each at its own
    autotuned launch shape, the full step sizes of their own bench lines, `steps` timed steps after
    one warm-up, L2 not flushed): hits/s, and for config 5 the gradient run's cost over the forward
    run.  `python bench.py --workload cN` gives each one's full line."""
    from molflow_sources_gb300 import _abi as A
    from molflow_sources_gb300.simulation import GpuBatch, GpuSimulation
    seed = 0x4D6F6C66
    out = {}

    def timed(run, n):
        run(max(n // 10, 1000))
        torch.cuda.synchronize()
        ms = hits = 0.0
        for _ in range(steps):
            st = run(n)
            ms += st["kernel_ms"]
            hits += st["hits"]
        return hits / (ms / 1e3), ms / steps

    for wl in ("c1", "c3", "c5"):
        try:
            m = make_model(wl)
            sim = GpuSimulation(m, device=local)
            n = WORKLOADS[wl]["step"]
            # the sensitivity kernel is compiled for 256-thread blocks: its forward comparison runs
            # at the same shape (2 resident blocks), the other workloads at their autotuned one
            shape = (dict(block_size=256, blocks_per_sm=2) if wl == "c5"
                     else sim.autotune(max(n // 4, 10000), precision=A.PREC_FP32R, seed=seed))   # as the main line

            def fwd(k):
                sim.SimulationMCStep(k, precision=A.PREC_FP32R, seed=seed, **shape)
                return sim.last_stats
            rate, ms = timed(fwd, n)
            out[wl] = {"workload": WORKLOADS[wl]["name"], "hits_per_s": rate, "ms_per_step": ms,
                       "desorptions_per_step": n, "launch_shape": shape}
            if wl == "c5":
                from molflow_sources_gb300.sensitivity import SensitivityFunction
                sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)

                def grad(k):
                    sf.forward(k, seed=seed, **shape)
                    return sf.last_stats
                srate, sms = timed(grad, n)
                out[wl].update({"hits_per_s": srate, "ms_per_step": sms, "forward_hits_per_s": rate,
                                "gradient_cost_over_forward": rate / srate})
            sim.close()
        except Exception as e:   # a side measurement never breaks the headline line
            out[wl] = {"error": str(e)[:200]}
    try:
        from molflow_sources_gb300 import batch_workloads as BW
        batch = GpuBatch(BW.config4_batch(), device=local)
        n = WORKLOADS["c4"]["step"]
        shape = batch.autotune(max(n // 20, 1000), precision=A.PREC_FP32R, seed=seed)

        def brun(k):
            return batch.run(k, precision=A.PREC_FP32R, seed=seed, use_graph=True, **shape)
        rate, ms = timed(brun, n)
        out["c4"] = {"workload": WORKLOADS["c4"]["name"], "hits_per_s": rate, "ms_per_step": ms,
                     "desorptions_per_instance_per_step": n, "launch_shape": shape}
        batch.close()
    except Exception as e:
        out["c4"] = {"error": str(e)[:200]}
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    t0 = time.time()
    steps = []
    hits_total = 0
    secs_total = 0.0
    from oracle.oracle import Oracle
    if args.workload == "c4":
        # one oracle per instance; a step traces n particles in each, one instance after another
        from molflow_sources_gb300 import batch_workloads as BW
        orcs = [Oracle(m) for m in BW.config4_batch()]
    else:
        orcs = [Oracle(make_model(args.workload))]
    for _ in range(args.warmup):
        for orc in orcs:
            orc.run(50, seed=3)
    rate_des = calibrate(orcs[0], 4) if len(orcs) == 1 else 50.0 * len(orcs) / max(
        sum(o.run(50, seed=4)[1]["seconds"] for o in orcs), 1e-6)
    n = int(max(20, min(rate_des * args.ref_step_s / len(orcs), 5e8)))
    s = {"threads": 0}
    for k in range(args.steps):
        for i, orc in enumerate(orcs):
            st, s = orc.run(n, seed=5, first_particle=k * n, instance=i if len(orcs) > 1 else 0)
            steps.append(s["seconds"])
            hits_total += s["hits"]
            secs_total += s["seconds"]
    n = n * len(orcs)
    v = hits_total / secs_total
    line = {"metric": METRIC[args.workload], "value": v, "unit": "hits/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs_total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOADS[args.workload]["name"], "desorptions_per_step": n},
            "cpu_baseline": {"value": v, "unit": "hits/s", "cores": s["threads"], "kind": "port",
                             "sample": "%d desorptions per step x %d steps" % (n, args.steps)},
            "e2e": {"value": v, "unit": "hits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU reference arm: the reference tracer cannot be built (src_shared submodule absent), so the "
                    "arm runs the FP64 CPU restatement of ParticleTracer in oracle/ on all host cores, on the same "
                    "workload; each step is a bounded sample of desorptions (hits/s is a rate)",
            "wall_s": time.time() - t0}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args, torch, dist, rank, world, local, W, n_step):
    """Config 4: 256 instances in one persistent launch (graph-captured) vs 256 separate launches."""
    from molflow_sources_gb300 import _abi as A
    from molflow_sources_gb300 import batch_workloads as BW
    from molflow_sources_gb300.simulation import GpuBatch, GpuSimulation
    models = BW.config4_batch()
    t0 = time.time()
    batch = GpuBatch(models, device=local)
    batch.set_particle_offset(rank * (1 << 48))
    load_s = time.time() - t0
    seed = 0x4D6F6C66
    tuned = batch.autotune(max(n_step // 20, 1000), precision=A.PREC_FP32R, seed=seed)
    for _ in range(args.warmup):
        batch.run(n_step // 10, precision=A.PREC_FP32R, seed=seed, use_graph=True, **tuned)
    batch.reset()
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    ms, hits, des, launches = 0.0, 0, 0, 0
    for k in range(args.steps):
        st = batch.run(n_step, precision=A.PREC_FP32R, seed=seed, use_graph=True, **tuned)
        ms += st["kernel_ms"]
        hits += st["hits"]
        des += st["desorbed"]
        launches += st["kernel_launches"]
    clocks = sampler.stop()
    # end to end: the public batch call with its per-instance particle counts from host memory, then
    # every instance's GlobalSimuState read back to host memory (mfg_fetch_instance), every step
    e2e_hits, d2h = 0, 0
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for k in range(args.steps):
        st = batch.run(n_step, precision=A.PREC_FP32R, seed=seed, use_graph=True, **tuned)
        e2e_hits += st["hits"]
        d2h = 0
        for i in range(len(models)):
            si = batch.fetch_instance(i)
            d2h += sum(getattr(si, a).nbytes for a in ("global_", "facet_counts", "facet_sums", "texture", "profile",
                                                       "direction", "anglemap", "histogram"))
    torch.cuda.synchronize()
    e2e_rate = e2e_hits / (time.perf_counter() - t2)
    # separate launches: one simulation per instance, each stepped on its own with the same
    # desorptions per instance as the batch step, through a captured graph as well (the first
    # step of each captures it), at the launch shape the batch uses
    sims = [GpuSimulation(m, device=local) for m in models]
    sep_ms, sep_hits = 0.0, 0
    for s_ in sims:
        s_.set_particle_offset(rank * (1 << 48))
        s_.SimulationMCStep(max(n_step // 100, 1000), precision=A.PREC_FP32R, seed=seed, use_graph=True, **tuned)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for s_ in sims:
        s_.SimulationMCStep(n_step, precision=A.PREC_FP32R, seed=seed, use_graph=True, **tuned)
        sep_hits += s_.last_stats["hits"]
        sep_ms += s_.last_stats["kernel_ms"]
    sep_wall = time.perf_counter() - t1
    rate = hits / (ms / 1e3)
    line = {"metric": METRIC["c4"], "value": rate, "unit": "hits/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": W["name"], "instances": len(models), "facets_total": int(sum(m.n_facets for m in models)),
                       "desorptions_per_instance_per_step": n_step, "launch": "CUDA graph, one persistent kernel",
                       "launch_shape": tuned},
            "separate_launches": {"hits_per_s_device": sep_hits / (sep_ms / 1e3), "hits_per_s_wall": sep_hits / sep_wall,
                                  "desorptions_per_instance": n_step, "launches": len(models),
                                  "launch": "CUDA graph per instance"},
            "gpu_launches": launches, "model_load_s": load_s, "clocks": clocks,
            "e2e": {"value": e2e_rate, "unit": "hits/s", "h2d_bytes_per_step": 8 * len(models) + 96,
                    "d2h_bytes_per_step": int(d2h), "api": "mfg_run_batch + mfg_fetch_instance of every instance"},
            "cpu_baseline": None}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_sensitivity(args, torch, dist, rank, world, local, W, n_step):
    """Config 5: forward run with score-function gradients of 9 outputs with respect to 1000
    sticking coefficients and every source's outgassing, against the plain forward run."""
    from molflow_sources_gb300 import _abi as A
    from molflow_sources_gb300.sensitivity import SensitivityFunction, config5_neg_tube
    from molflow_sources_gb300.simulation import GpuSimulation
    m = config5_neg_tube()
    sim = GpuSimulation(m, device=local)
    sim.set_particle_offset(rank * (1 << 48))
    sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
    seed = 0x4D6F6C66
    for _ in range(args.warmup):
        sim.SimulationMCStep(n_step // 10, precision=A.PREC_FP32R, seed=seed)
        sf.forward(n_step // 10, seed=seed)
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    f_ms = f_hits = s_ms = s_hits = 0.0
    launches = 0
    for k in range(args.steps):
        sim.SimulationMCStep(n_step, precision=A.PREC_FP32R, seed=seed)
        f_ms += sim.last_stats["kernel_ms"]
        f_hits += sim.last_stats["hits"]
        sf.forward(n_step, seed=seed)
        s_ms += sf.last_stats["kernel_ms"]
        s_hits += sf.last_stats["hits"]
        launches += sim.last_stats["kernel_launches"] + sf.last_stats["kernel_launches"]
    clocks = sampler.stop()
    # end to end: forward with gradients, then the Jacobian read back to host memory
    t1 = time.perf_counter()
    sf.forward(n_step, seed=seed)
    js, jq, src = sf.jacobian()
    e2e_s = time.perf_counter() - t1
    rate = s_hits / (s_ms / 1e3)
    line = {"metric": METRIC["c5"], "value": rate,
            "unit": "hits/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": s_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": W["name"], "desorptions_per_step": n_step, "parameters": int(len(m.neg)),
                       "outputs": 9, "facets": int(m.n_facets)},
            "forward_hits_per_s": f_hits / (f_ms / 1e3), "gradient_cost_over_forward": (s_ms / s_hits) / (f_ms / f_hits),
            "gpu_launches": launches, "clocks": clocks,
            "e2e": {"value": sf.last_stats["hits"] / e2e_s, "unit": "hits/s", "h2d_bytes_per_step": 96,
                    "d2h_bytes_per_step": int(js.nbytes + jq.nbytes + src.nbytes)},
            "cpu_baseline": None}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("MFG_BENCH_WORKLOAD", "c2"), choices=list(WORKLOADS))
    ap.add_argument("--step-desorptions", type=int, default=0)
    ap.add_argument("--fp64-step", type=int, default=0, help="desorptions per FP64 step (default: the FP32R step)")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--ref-step-s", type=float, default=6.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--launch", default="",
                    help="fixed FP32R launch shape BLOCK,BLOCKS_PER_SM[,SMEM_BVH_LEVELS] instead of the autotuner's choice")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the short measurements of configs 1, 3, 4 and 5 in the config-2 line")
    ap.add_argument("--profile-steps", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from molflow_sources_gb300 import _abi as A
    from molflow_sources_gb300.simulation import GpuSimulation

    W = WORKLOADS[args.workload]
    n_step = args.step_desorptions or W["step"]
    if args.workload == "c4":
        return run_batch(args, torch, dist, rank, world, local, W, n_step)
    if args.workload == "c5":
        return run_sensitivity(args, torch, dist, rank, world, local, W, n_step)
    model = make_model(args.workload)
    t0 = time.time()
    sim = GpuSimulation(model, device=local)
    load_s = time.time() - t0
    sim.set_particle_offset(rank * (1 << 48))
    seed = 0x4D6F6C66
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # plain FP64 kernel on the same workload and step size, at the launch shape its own autotuner
    # picks (register budgets of 2, 3 and 4 resident blocks); its tallies are the FP64 side of the
    # transmission gate
    fp64_step = args.fp64_step or n_step
    sim.SimulationMCStep(max(1, fp64_step // 20), precision=A.PREC_FP64, seed=seed)
    tuned64 = sim.autotune(max(fp64_step // 10, 10000), precision=A.PREC_FP64, seed=seed)
    f64_ms = 0.0
    f64_hits = 0
    for _ in range(args.fp64_steps):
        sim.SimulationMCStep(fp64_step, precision=A.PREC_FP64, seed=seed)
        f64_ms += sim.last_stats["kernel_ms"]
        f64_hits += sim.last_stats["hits"]
    fp64_rate = f64_hits / (f64_ms / 1e3)
    st64 = sim.fetch()
    sim.ResetSimulation()

    if args.launch:
        v_ = [int(x) for x in args.launch.split(",")]
        tuned = {"block_size": v_[0], "blocks_per_sm": v_[1], "smem_bvh_levels": v_[2] if len(v_) > 2 else -1}
    else:
        # launch shape: trial runs of a quarter step, so that each of the up to 2048 resident
        # threads of an SM traces several particles and the tail of a launch does not decide
        tuned = sim.autotune(max(n_step // 4, 10000), precision=A.PREC_FP32R, seed=seed)
    shape = dict(tuned) if args.launch else {}
    for _ in range(args.warmup):
        sim.SimulationMCStep(n_step, precision=A.PREC_FP32R, seed=seed, **shape)
    sim.ResetSimulation()
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    kernel_ms = []
    hits = 0
    rechecks = 0
    launches = 0
    des = 0
    if args.profile_steps:
        torch.cuda.profiler.start()
    for k in range(args.steps):
        flush.fill_(k & 0xFF)   # L2 flush between steps (outside the kernel's event pair)
        sim.SimulationMCStep(n_step, precision=A.PREC_FP32R, seed=seed, **shape)
        st = sim.last_stats
        kernel_ms.append(st["kernel_ms"])
        hits += st["hits"]
        rechecks += st["rechecks"]
        launches += st["kernel_launches"]
        des += st["desorbed"]
    if args.profile_steps:
        torch.cuda.profiler.stop()
    barrier()
    gate = transmission_gate(model, sim.fetch(), st64)
    # end to end: public API call + tallies copied to host memory every step
    from molflow_sources_gb300.model import SimuState
    gstate = SimuState(model)
    # one untimed end-to-end step: host buffers are allocated and first touched here, once
    sim.SimulationMCStep(n_step, precision=A.PREC_FP32R, seed=seed, **shape)
    sim.UpdateHitsAndLog(gstate)
    e2e_hits = 0
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for k in range(max(1, args.steps)):
        sim.SimulationMCStep(n_step, precision=A.PREC_FP32R, seed=seed, **shape)
        e2e_hits += sim.last_stats["hits"]
        sim.UpdateHitsAndLog(gstate)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t1
    clocks = sampler.stop()
    # end of the job: every rank's GlobalSimuState summed to rank 0, the reference's MPI gather
    # (MolflowCLI.cpp:165-196); integer tallies exactly, untimed
    final = None
    if dist is not None:
        from molflow_sources_gb300.replicas import reduce_state
        t2 = time.perf_counter()
        reduce_state(gstate, dst=0)
        final = {"seconds": time.perf_counter() - t2,
                 "desorbed_all_ranks": int(gstate.global_[A.G_NBDESORBED]) if rank == 0 else None}
    dev_s = sum(kernel_ms) / 1e3
    rate = hits / dev_s
    e2e_rate = e2e_hits / e2e_s
    if dist is not None:
        t = torch.tensor([dev_s, e2e_s, float(hits), float(e2e_hits)], dtype=torch.float64, device="cuda")
        mx = t.clone()
        dist.all_reduce(mx[:2], op=dist.ReduceOp.MAX)
        tot = t.clone()
        dist.all_reduce(tot[2:], op=dist.ReduceOp.SUM)
        rate = float(tot[2]) / float(mx[0])
        e2e_rate = float(tot[3]) / float(mx[1])
        dev_s = float(mx[0])
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    nodes, prims, _ = oracle_visit_counts(model)
    bph = bytes_per_hit(model, nodes, prims)
    peak, peak_kind = measured_peaks()
    mean_launch_s = dev_s / args.steps
    achieved = (hits / args.steps) * bph / mean_launch_s / 1e9
    traffic = None
    l2 = None
    warp_eff = None
    tp = os.path.join(ROOT, "profiles", "traffic_%s.json" % args.workload)
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        traffic = tj.get("dram_bytes_per_hit", 0) * hits / args.steps
        if tj.get("l2_bytes_per_hit") and tj.get("l2_throughput_pct") and tj.get("capture_ms"):
            # L2 side of the roofline: the kernel's L2 bytes per hit (ncu lts__t_sectors x 32 B) at this
            # run's hit rate, against the L2 peak implied by the same capture (its L2 bytes per second
            # divided by its lts__throughput fraction of peak)
            cap_gbs = tj["l2_bytes_per_hit"] * tj["hits_in_capture"] / (tj["capture_ms"] * 1e-3) / 1e9
            l2_peak = cap_gbs / (tj["l2_throughput_pct"] / 100.0)
            l2_ach = tj["l2_bytes_per_hit"] * (hits / args.steps) / mean_launch_s / 1e9
            l2 = {"achieved": l2_ach, "peak": l2_peak, "unit": "GB/s", "frac": l2_ach / l2_peak,
                  "bytes_per_hit": tj["l2_bytes_per_hit"],
                  "peak_kind": "ncu: the capture's L2 bytes per second over its lts__throughput fraction",
                  "ncu_l2_throughput_pct_of_peak": tj["l2_throughput_pct"],
                  "ncu_l1_throughput_pct_of_peak": tj.get("l1_throughput_pct")}
        if tj.get("threads_per_warp_instruction"):
            # warp execution efficiency of the captured launch: active threads per issued warp instruction
            warp_eff = {"threads_per_instruction": tj["threads_per_warp_instruction"],
                        "efficiency": tj["threads_per_warp_instruction"] / 32.0,
                        "source": "ncu smsp__thread_inst_executed_per_inst_executed.ratio"}
    cpu = None if args.no_cpu_baseline else cpu_baseline(model)
    others = other_workloads(torch, local) if (args.workload == "c2" and world == 1 and not args.no_others) else None
    L = model.layout()
    d2h = 8 * (A.G_N + L["blocks"] * model.n_facets * (A.FC_N + A.FS_N) + L["blocks"] * L["texture_cells"] * 3 +
               L["blocks"] * L["profile_facets"] * 300 + L["anglemap_cells"])
    line = {
        "metric": METRIC[args.workload],
        "value": rate, "unit": "hits/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": W["name"], "desorptions_per_step": n_step, "facets": model.n_facets,
                   "precision": "FP32 traversal + FP64 recheck", "l2": "256 MiB write between timed steps",
                   "parallelism": "particle ranges per rank" if world > 1 else "single GPU"},
        "fp64_kernel_hits_per_s": fp64_rate, "fp32r_over_fp64": rate / fp64_rate,
        "fp64_launch_shape": tuned64, "fp64_desorptions_per_step": fp64_step,
        "transmission_gate": gate,
        "desorptions_per_s": des / dev_s * (world if dist is None else 1),
        "recheck_fraction": rechecks / max(hits + des, 1),
        "final_reduce": final,
        "e2e": {"value": e2e_rate, "unit": "hits/s", "h2d_bytes_per_step": int(A.RunOptions.__basicsize__ if hasattr(A.RunOptions, "__basicsize__") else 48),
                "d2h_bytes_per_step": int(d2h), "api": "SimulationMCStep + UpdateHitsAndLog (C ABI mfg_run + mfg_fetch)"},
        "gpu_launches": launches,
        "launch_shape": tuned,
        "model_load_s": load_s,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "bytes_per_hit": bph, "nodes_per_ray": nodes, "facets_per_ray": prims,
                     "peak_kind": peak_kind, "l2": l2, "warp_execution": warp_eff,
                     "limiter": "L1/TEX throughput and load latency: the L1 is the busiest unit (67 % of its peak "
                                "on the beam chamber, with 3.2 local-memory requests, stack and spills, per global one), "
                                "issue slots 52 %, L2 40 %, DRAM about 22 % of their peaks"},
        "clocks": clocks,
        "cpu_baseline": cpu,
        "other_workloads": others,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    if not gate["pass"]:
        # the metric is defined at the same 3-sigma transmission: a run that misses it is not a result
        sys.stderr.write("transmission gate failed: FP32R %.6g against FP64 %.6g (z = %.2f)\n"
                         % (gate["fp32r"], gate["fp64"], gate["z"]))
        return 3
    return 0


if __name__ == "__main__":
    sys.exit(main())
