#!/usr/bin/env python
"""Benchmark: batched energy + force evaluation (atom-steps/s) on GB300.

Default workload: 256 open H/C/N/O molecules with 10-120 atoms each
(about 16.5k atoms, seeded; the reference ships no dataset), seed-0
StudentForceField weights (hidden 128, 3 blocks, 20 RBF, 5 A cutoff).  One
step = one full evaluation of the batch: radius graph, model, hand-written
force adjoint.  ``value`` is device-timed with inputs resident in HBM; the
e2e figure goes through the public module API with host buffers (H2D of
positions and numbers; D2H of energies, forces and the status word) inside
the timed region.  An L2-sized buffer is rewritten between timed steps.

Beside the headline the line carries, measured in the same run:
  * ``vs_plain_fp32``: the tensor-core path against the plain FP32 CUDA path
    on the 256-molecule batch and on the 3,000-atom periodic water box, both
    paths timed the same way (CUDA-graph replays of one step, L2 flushed);
  * ``accuracy``: energy and force errors of the timed path against the
    float64 oracle (a checker, run after the timed regions);
  * ``roofline``: the dominant kernel's algorithmic filter-MLP FLOPs over its
    CUDA-event launch time against the measured bf16 burst peak, and the
    whole step's GEMM FLOPs over the step time.

  python bench.py [--gpus N --steps K --warmup W] [--workload batch256]
                  [--path fp16x3|tuned_fp32|fp32] [--impl ours|reference]

Under torchrun (N>1) every rank evaluates its own copy of the workload
(independent batches, no collective on the data path): weak scaling.
``--impl reference`` times the oracle port of the reference's CPU path
(float32 torch, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mlff-distiller_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "atom-steps/s E+F on 1 GB300: tuned vs plain FP32, force err <=1e-3 eV/A vs FP64"
UNIT = "atom-steps/s"
GEMM_FLOP_PER_EDGE = 2 * (20 * 128 + 128 * 384)      # filter MLP, per directed edge and layer
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch256")
    ap.add_argument("--path", default="fp16x3", choices=["fp16x3", "tuned_fp32", "fp32"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--graph", type=int, default=1, help="time replays of a CUDA graph of one step (1) or eager calls (0)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--md-steps", type=int, default=0,
                    help="MD workloads: further untimed steps for the energy drift (20000 = 10 ps)")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-FP32 / water-box comparison")
    ap.add_argument("--compare-steps", type=int, default=10)
    ap.add_argument("--no-accuracy", action="store_true", help="skip the float64 oracle accuracy check")
    ap.add_argument("--no-training", action="store_true", help="skip the training-step timing")
    ap.add_argument("--training-structures", type=int, default=64,
                    help="structures of a multi-structure workload in the timed training batch")
    ap.add_argument("--accuracy-structures", type=int, default=64,
                    help="structures of a multi-structure workload checked against the float64 oracle")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.path = None
        try:
            uuid = str(torch.cuda.get_device_properties(device_index).uuid)
            self.id = uuid if uuid.startswith("GPU-") else f"GPU-{uuid}"
        except Exception:
            self.id = str(device_index)

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.id, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        loaded = [s for s in sm if mx and s >= 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# -------------------------------------------------------------- workload
def seed_model(precision):
    from mlff_gb300.student_model import StudentForceField
    torch.manual_seed(0)
    return StudentForceField(precision=precision)


def _port_rate(W, sub, seconds):
    """atom-steps/s of the oracle port (float32 torch autograd) on `sub`."""
    from oracle import painn
    pos = sub.pos.astype(np.float32).astype(np.float64)
    painn.energy_forces(W, sub.Z, pos, sub.mol_ptr, box=sub.box, pbc=sub.pbc, dtype=torch.float32)
    reps, t0 = 0, time.perf_counter()
    while True:
        painn.energy_forces(W, sub.Z, pos, sub.mol_ptr, box=sub.box, pbc=sub.pbc, dtype=torch.float32)
        reps += 1
        el = time.perf_counter() - t0
        if (el >= seconds and reps >= 3) or el >= 4 * seconds:
            break
    return sub.n_atoms * reps / el, reps


def cpu_baseline(sysm, seconds, n_threads=None, one_thread_seconds=3.0):
    """Oracle port of the reference CPU path (float32 torch autograd, C
    radius graph) on a bounded sample of the workload's molecules, with all
    host threads and (value_1thread) with one."""
    if n_threads:
        torch.set_num_threads(n_threads)
    W = W_SEED0()
    n_take = min(sysm.n_mol, 16)
    sub = sysm.subset(list(range(n_take))) if sysm.n_mol > 1 else sysm
    v, reps = _port_rate(W, sub, seconds)
    cores = torch.get_num_threads()
    v1 = None
    if one_thread_seconds > 0:
        n1 = min(sysm.n_mol, 4)
        sub1 = sysm.subset(list(range(n1))) if sysm.n_mol > 1 else sysm
        torch.set_num_threads(1)
        v1, _ = _port_rate(W, sub1, one_thread_seconds)
        torch.set_num_threads(cores)
    return {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
            "value_1thread": v1,
            "sample": f"{n_take} of {sysm.n_mol} structures ({sub.n_atoms} atoms), {reps} E+F evaluations, "
                      f"float32 torch autograd on the host CPU"
                      + (f"; value_1thread on the first {min(sysm.n_mol, 4)} structures" if v1 else "")}


def read_traffic(kernel_kind, workload):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel_kind}_{workload}.md")
    if not os.path.exists(path):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def measured_peaks():
    """bf16 burst TFLOP/s (the kernels are timed inside a few-ms step, not a
    seconds-long loop) and HBM GB/s: measured on this GPU model if the
    measurement file is present, else the fallback figures."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


def step_gemm_flop(n_atoms, n_edges, n_layers=3):
    """Algorithmic GEMM FLOPs of one E+F evaluation: forward plus the
    input-gradient pass of the filter MLP per directed edge, the update MLP
    per atom and layer, and the readout per atom."""
    return 2 * (n_layers * (n_edges * GEMM_FLOP_PER_EDGE + n_atoms * 163_840) + n_atoms * 20_544)


def accuracy_vs_oracle(sysm, E, F, max_structures):
    """Checker, outside every timed region: energies [B] and forces [N,3] of
    the timed path against the float64 oracle evaluated on the same float32
    positions, on the first max_structures structures (structures are
    independent, so a subset's results are exactly the full batch's)."""
    from oracle import painn
    take = min(sysm.n_mol, max_structures)
    sub = sysm.subset(list(range(take))) if take < sysm.n_mol else sysm
    n_sub = sub.n_atoms
    t0 = time.perf_counter()
    E0, F0 = painn.energy_forces(W_SEED0(), sub.Z, sub.pos.astype(np.float32).astype(np.float64), sub.mol_ptr,
                                 box=sub.box, pbc=sub.pbc)
    el = time.perf_counter() - t0
    E0, F0 = E0.numpy(), F0.numpy()
    Eg = np.asarray(E, dtype=np.float64)[:take]
    Fg = np.asarray(F, dtype=np.float64)[:n_sub]
    per_atom = np.abs(Eg - E0) / np.diff(sub.mol_ptr)
    dF = Fg - F0
    return {"reference": "float64 oracle (CPU) on the same float32 positions",
            "structures": f"{take} of {sysm.n_mol}", "atoms": int(n_sub),
            "energy_err_mev_per_atom_max": float(1000 * per_atom.max()),
            "energy_err_mev_per_atom_mean": float(1000 * per_atom.mean()),
            "force_err_max_ev_per_a": float(np.abs(dF).max()),
            "force_err_rms_ev_per_a": float(np.sqrt((dF ** 2).mean())),
            "force_rms_ev_per_a": float(np.sqrt((F0 ** 2).mean())),
            "force_tol_ev_per_a": 1e-3, "within_tol": bool(np.abs(dF).max() <= 1e-3),
            "oracle_seconds": round(el, 1)}


_W0 = {}


def W_SEED0():
    """The seed-0 weights (the model every bench workload evaluates)."""
    if not _W0:
        _W0.update({k: v.numpy() for k, v in seed_model("tuned_fp32").state_dict().items()})
    return _W0


def run_reference(args, world, rank):
    from mlff_gb300 import systems
    if rank != 0:
        return
    sysm = systems.workload(args.workload)
    n_thr = os.cpu_count() or 1
    torch.set_num_threads(n_thr)
    step_s = max(1.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_baseline(sysm, 0.0, n_thr, one_thread_seconds=0)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(sysm, step_s, n_thr, one_thread_seconds=0))
    total = time.perf_counter() - t0
    v = statistics.mean(x["value"] for x in vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded), seed-0 weights",
            "config": {"workload": args.workload, "structures_sampled": min(16, sysm.n_mol)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": n_thr, "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MD_BLOCK = 50        # MD steps per CUDA-graph replay in the drift run
MD_TIME_BLOCK = 10   # MD steps per timed replay (from the initial state)


def run_md(args, world, rank, local):
    """MD replicas: velocity-Verlet NVE at 0.5 fs from Maxwell-Boltzmann
    velocities at 300 K, whole blocks of steps replayed from one CUDA graph.
    A bench step is one replay of MD_TIME_BLOCK steps of every replica, each
    replay started from the same initial state (restored outside the timed
    region): the seed-initialised potential is strongly repulsive and the
    replicas expand (about 8 % of the initial edges are left after 600
    steps), so timing later steps would measure a sparser system."""
    from mlff_gb300 import _lib, systems
    from mlff_gb300.md import VelocityVerletGPU, kinetic_energy, replica_drift
    from mlff_gb300.replicas import aggregate_throughput
    sysm = systems.workload(args.workload)
    model = seed_model(args.path).cuda().eval()
    drv = VelocityVerletGPU(model, sysm.Z, sysm.pos, sysm.mol_ptr, timestep_fs=0.5)
    drv.initialize_velocities(300.0, seed=rank)
    E0, _ = drv.compute_forces()
    K0 = kinetic_energy(drv.velocities(), drv.masses, sysm.mol_ptr)
    edges_start = drv.engine.status()[1]
    init = drv.snapshot()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(max(3, args.warmup)):
        drv.restore(init)
        drv.run(MD_TIME_BLOCK, graph=True, block=MD_TIME_BLOCK, record=False)
    g = drv._graph(MD_TIME_BLOCK, drv._capacity(), False)["graph"]
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    for i in range(args.steps):
        drv.restore(init)
        flush.fill_(float(i))
        starts[i].record()
        g.replay()
        ends[i].record()
    torch.cuda.synchronize()
    ck = clocks.stop()
    code, edges_end, _ = drv.engine.status()
    if code != _lib.OK:
        raise RuntimeError(f"device status {code} during the timed MD region")
    blk_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    n_md = args.steps * MD_TIME_BLOCK
    # atom-steps of all ranks / the slowest rank's timed region
    _, total_s, value = aggregate_throughput(sysm.n_atoms * n_md, sum(blk_ms) / 1000.0, device="cuda")
    # energy drift over --md-steps steps from the initial state (not timed)
    drift = None
    if args.md_steps > 0:
        from mlff_gb300.energy_metrics import replica_energy_stats
        drv.restore(init)
        trd = drv.run(args.md_steps, graph=True, block=MD_BLOCK, to_host=False)
        dst = replica_energy_stats(trd["potential_energy"], trd["kinetic_energy"], 0.5e-3,
                                   mol_ptr=torch.as_tensor(sysm.mol_ptr), epot0=torch.as_tensor(E0),
                                   ekin0=torch.as_tensor(K0))
        tr = {k: v.cpu().numpy() for k, v in trd.items()}
        rel, ab = replica_drift(tr["potential_energy"], tr["kinetic_energy"], E0, K0)
        n_per = np.diff(sysm.mol_ptr)
        mev = 1000.0 * ab / n_per
        et = tr["potential_energy"] + tr["kinetic_energy"]
        drift = {"steps": args.md_steps, "time_ps": args.md_steps * 0.5e-3,
                 "rel_drift_pct_median": float(np.median(rel)), "rel_drift_pct_max_abs": float(np.abs(rel).max()),
                 "abs_drift_mev_per_atom_median": float(np.median(mev)),
                 "abs_drift_mev_per_atom_max_abs": float(np.abs(mev).max()),
                 "max_excursion_mev_per_atom": float(1000.0 * (np.abs(et - (E0 + K0)[None, :]) / n_per).max()),
                 "edges_at_end": int(drv.engine.status()[1]),
                 "device_stats_median": {k: float(dst[k].median()) for k in (
                     "conservation_ratio", "drift_rate", "r_squared", "avg_temperature", "std_temperature")}}
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "fp16x3 filters, f32 model, f64 Verlet state" if args.path == "fp16x3" else "f32, f64 Verlet state",
            "data": "synthetic (seeded), seed-0 weights",
            "config": {"workload": args.workload, "atoms": sysm.n_atoms, "replicas": sysm.n_mol,
                       "md_steps_per_bench_step": MD_TIME_BLOCK, "dt_fs": 0.5, "temperature_K": 300.0,
                       "path": args.path, "graph": f"one CUDA graph per {MD_TIME_BLOCK} MD steps",
                       "start": "every timed replay starts from the initial state (steps 1-%d)" % MD_TIME_BLOCK,
                       "edges_initial": int(edges_start), "edges_after_block": int(edges_end),
                       "l2": "256 MiB buffer rewritten between timed graph replays"},
            "md_step_latency_ms_p50": statistics.median(blk_ms) / MD_TIME_BLOCK,
            "drift": drift, "clocks": ck}
    print(json.dumps(line), flush=True)


def training_throughput(sysm, n_structures, steps=5, warmup=2):
    """One optimisation step of the GPU trainer (ForceFieldTrainer with the
    reference's loss defaults: energy weight 1, force weight 100): forward
    and forces on the plain FP32 path, the loss derivatives, the parameter
    gradients of the energy and force terms from the hand-written reverse
    pass and its forward-mode derivative, gradient clipping and AdamW.
    Timed (CUDA events, after warm-up) on the first n_structures structures
    of the workload, targets = the untrained network's own outputs plus
    seeded noise (the cost of a step does not depend on the values)."""
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    from mlff_gb300.training import ForceFieldTrainer
    sub = sysm.subset(list(range(min(n_structures, sysm.n_mol)))) if sysm.n_mol > 1 else sysm
    per = bool(sub.pbc.any())
    b = make_batch(sub.Z, sub.pos.astype(np.float32), sub.mol_ptr, sub.box if per else None,
                   sub.pbc if per else None)
    model = seed_model("fp32").cuda()
    tr = ForceFieldTrainer(model)
    E0, F0, _ = model.engine().energy_forces(b, _lib.PATH_PLAIN_FP32, graph=False)
    g = torch.Generator(device="cuda").manual_seed(7)
    E_ref = E0.to(torch.float64) + 0.05 * torch.randn(E0.shape, generator=g, device="cuda", dtype=torch.float64)
    F_ref = F0.to(torch.float64) + 0.1 * torch.randn(F0.shape, generator=g, device="cuda", dtype=torch.float64)
    for _ in range(warmup):
        tr.step(b, E_ref, F_ref)
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        tr.step(b, E_ref, F_ref)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    med = statistics.median(ms)
    return {"structures": sub.n_mol, "atoms": sub.n_atoms, "steps": steps, "ms_per_step": round(med, 3),
            "atom_steps_per_s": round(sub.n_atoms / (med * 1e-3), 1),
            "step": "ForceFieldTrainer.step: energy + force loss (weights 1, 100), second-order parameter "
                    "gradients on the plain FP32 path, grad-norm clip 1.0, AdamW"}


def time_replays(step, steps, flush):
    """CUDA-event times (ms) of `steps` calls of step(), an L2-sized buffer
    rewritten before each one."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(float(i))
        starts[i].record()
        step()
        ends[i].record()
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def graph_step(model, sysm, warmup):
    """A CUDA graph of one E+F evaluation of the workload on the model's
    path (edge capacity sized and, for the tensor-core path, the partition
    factor tuned first); returns (replay, E, F, n_edges)."""
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    eng = model.engine()
    batch = make_batch(sysm.Z, sysm.pos, sysm.mol_ptr, sysm.box if sysm.pbc.any() else None,
                       sysm.pbc if sysm.pbc.any() else None)
    eng.energy_forces(batch, model.path, graph=False)
    if model.path == _lib.PATH_TUNED_TC:
        eng.autotune(batch, model.path)
    _, n_edges, _ = eng.status()
    step, E, F = eng.capture(batch, model.path)
    for _ in range(max(3, warmup)):
        step()
    return step, E, F, n_edges, batch


def compare_paths(args, path, flush):
    """Tensor-core path vs plain FP32 on the 256-molecule batch and the
    3,000-atom periodic water box: both timed as CUDA-graph replays of one
    step with the L2 flushed between steps."""
    from mlff_gb300 import _lib, systems
    out = {}
    for wl in ("batch256", "water3000"):
        sysm = systems.workload(wl)
        ms = {}
        for prec in (path, "fp32"):
            m = seed_model(prec).cuda().eval()
            step, _, _, n_edges, _ = graph_step(m, sysm, args.warmup)
            t = time_replays(step, args.compare_steps, flush)
            code, _, _ = m.engine().status()
            if code != _lib.OK:
                raise RuntimeError(f"device status {code} in the {prec} comparison on {wl}")
            ms[prec] = statistics.median(t)
            del m, step
            torch.cuda.empty_cache()
        out[wl] = {"ratio": round(ms["fp32"] / ms[path], 3),
                   "tuned_ms_per_step": round(ms[path], 4), "plain_fp32_ms_per_step": round(ms["fp32"], 4),
                   "tuned_atom_steps_per_s": round(sysm.n_atoms / (ms[path] * 1e-3)),
                   "plain_fp32_atom_steps_per_s": round(sysm.n_atoms / (ms["fp32"] * 1e-3)),
                   "atoms": sysm.n_atoms, "directed_edges": int(n_edges)}
    out["launch"] = "both paths: CUDA-graph replay of one step, median of %d, L2 flushed" % args.compare_steps
    return out


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.workload.startswith("replicas"):
        run_md(args, world, rank, local)
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    from mlff_gb300 import _lib, systems
    from mlff_gb300.engine import make_batch
    from mlff_gb300.replicas import aggregate_throughput

    sysm = systems.workload(args.workload)
    model = seed_model(args.path).cuda().eval()
    eng = model.engine()
    path = model.path
    batch = make_batch(sysm.Z, sysm.pos, sysm.mol_ptr, sysm.box if sysm.pbc.any() else None,
                       sysm.pbc if sysm.pbc.any() else None)
    eng.energy_forces(batch, path, graph=False)   # sizes the edge capacity, checks status
    tune = eng.autotune(batch, path) if path == _lib.PATH_TUNED_TC else None
    _, n_edges, _ = eng.status()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(max(3, args.warmup)):
        eng.energy_forces(batch, path, check=False)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if args.graph:
        step, E_out, F_out = eng.capture(batch, path)
        for _ in range(max(3, args.warmup)):
            step()
    else:
        res = {}

        def step():
            res["E"], res["F"], _ = eng.energy_forces(batch, path, check=False)
    barrier()
    clocks.start()
    time.sleep(0.3)
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record()
        step()
        ends[i].record()
    barrier()
    ck = clocks.stop()
    code, _, _ = eng.status()
    if code != _lib.OK:
        raise RuntimeError(f"device status {code} during the timed region")
    if not args.graph:
        E_out, F_out = res["E"], res["F"]
    E_timed = E_out.cpu().numpy().copy()
    F_timed = F_out.cpu().numpy().copy()
    # kernel split and launch count: the same steps again, eagerly, under the
    # library's CUDA-event profiler (not part of the timed region)
    with _lib.Profile() as prof:
        for i in range(args.steps):
            flush.fill_(float(i))
            eng.energy_forces(batch, path, check=False)
        barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    hbm_peak = int(torch.cuda.max_memory_allocated())    # the timed workload alone
    atoms_all = sysm.n_atoms * world
    _, total_s, value = aggregate_throughput(sysm.n_atoms * args.steps, sum(step_ms) / 1000.0, device="cuda")
    ms_per_step = 1000 * total_s / args.steps

    # dominant kernel and its roofline (algorithmic GEMM FLOPs of the filter MLP)
    L = model.num_interactions
    kinds = {k: v for k, v in prof.ms.items() if prof.launches.get(k, 0) > 0}
    dom = max(kinds, key=kinds.get)
    launches = prof.launches[dom]
    avg_ms = prof.ms[dom] / max(1, launches)
    peak_tf, hbm, peak_src = measured_peaks()
    if dom == "edge_fwd":
        flop = n_edges * GEMM_FLOP_PER_EDGE
    elif dom == "edge_bwd":
        flop = 2 * n_edges * GEMM_FLOP_PER_EDGE
    else:
        flop = None
    step_flop = step_gemm_flop(sysm.n_atoms, n_edges, L)
    step_tf = step_flop / (ms_per_step * 1e-3) / 1e12
    roof = None
    if flop is not None:
        ach = flop / (avg_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "kernel": dom, "achieved": round(ach, 2), "peak": peak_tf, "unit": "TFLOP/s",
                "frac": round(ach / peak_tf, 4), "peak_source": f"{peak_src} bf16 burst",
                "traffic": read_traffic(dom, args.workload), "avg_launch_ms": round(avg_ms, 4),
                "launches_per_step": launches / args.steps, "flop_per_launch": flop,
                "mma_work_factor": (3.0 * (2 * (32 * 128 + 128 * 384)) / GEMM_FLOP_PER_EDGE
                                    if path == _lib.PATH_TUNED_TC else None),
                "step": {"gemm_flop_per_step": step_flop, "achieved": round(step_tf, 2),
                         "frac": round(step_tf / peak_tf, 4)}}
        if dom == "edge_bwd" and prof.launches.get("edge_bwd_q", 0) > 0:
            # the reverse pass's companion kernel (per-atom Q rows, launched just before each
            # reverse launch): not part of the FLOPs above, reported beside them
            roof["companion"] = {"kernel": "edge_bwd_q",
                                 "avg_launch_ms": round(prof.ms["edge_bwd_q"] / prof.launches["edge_bwd_q"], 4)}
    gpu_launches = sum(prof.launches.values())

    # e2e through the public module API with host buffers
    e2e = None
    if not args.no_e2e:
        Zh = torch.from_numpy(sysm.Z.astype(np.int64)).pin_memory()
        Ph = torch.from_numpy(sysm.pos.astype(np.float32)).pin_memory()
        # structure index, cell and pbc are host-side metadata, as the calculator passes them;
        # the model turns them into molecule offsets / boxes and copies those
        bh = torch.from_numpy(np.repeat(np.arange(sysm.n_mol), np.diff(sysm.mol_ptr)).astype(np.int64))
        cell = pbc = None
        if sysm.pbc.any():
            cell = torch.from_numpy(np.diag(sysm.box[0]).astype(np.float32))
            pbc = torch.ones(3, dtype=torch.bool)

        def e2e_step():
            # host buffers in, host results out: the module copies Z and positions straight
            # into its CUDA graph's input buffers and returns E, F (and reads the status word)
            # behind one synchronisation
            return model.energy_and_forces(Zh, Ph, batch=bh if sysm.n_mol > 1 else None, cell=cell, pbc=pbc)
        for _ in range(2):
            e2e_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        barrier()
        _, el, _ = aggregate_throughput(sysm.n_atoms * args.steps, time.perf_counter() - t0, device="cuda")
        # per step: Z and positions in; energies, forces and the 16-byte status word out (molecule
        # offsets, boxes and flags are cached on the device after the first call)
        h2d = Zh.numel() * 8 + Ph.numel() * 4
        d2h = sysm.n_mol * 8 + sysm.n_atoms * 12 + 16
        e2e = {"value": atoms_all * args.steps / el, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    del model, eng
    torch.cuda.empty_cache()
    compare = None
    if not args.no_compare and world == 1:
        compare = compare_paths(args, args.path, flush)
    acc = None
    if not args.no_accuracy:
        acc = accuracy_vs_oracle(sysm, E_timed, F_timed, args.accuracy_structures)
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(sysm, args.cpu_seconds, os.cpu_count())
    train = None
    if not args.no_training and world == 1:
        train = training_throughput(sysm, args.training_structures)
    dtype = {"fp16x3": "fp16x3 (split-fp16 operands, fp32 accumulate)", "tuned_fp32": "f32", "fp32": "f32"}[args.path]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded), seed-0 weights",
            "config": {"workload": args.workload, "atoms": sysm.n_atoms, "structures": sysm.n_mol,
                       "directed_edges": n_edges, "path": args.path, "l2": "256 MiB buffer rewritten "
                       "between timed steps", "per_rank": "independent copy of the workload",
                       "launch": "CUDA graph of one step" if args.graph else "eager library call per step",
                       "hbm_peak_bytes": hbm_peak, "autotune": tune},
            "vs_plain_fp32": compare, "accuracy": acc, "training": train,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
            "kernel_ms": {k: round(v, 3) for k, v in prof.ms.items() if v > 0},
            "kernel_launches": {k: v for k, v in prof.launches.items() if v > 0},
            "clocks": ck}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
